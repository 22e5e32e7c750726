"""Device Matrix Market reader (spai_mm_read) against the host reader of the same library (the
restatement of the reference's read_matrix_market / CsrMatrix::from_entries, src/cpu.cpp:49-161):
identical CSR bits for valid files (duplicates, symmetric mirrors, comments, blank lines, every
number spelling, tokens the device hands to the host) and the same error code and message for
invalid ones, checked in file order."""
import numpy as np
import pytest

import spai_ir
from spai_ir import matrices as M

pytestmark = pytest.mark.gpu

HOST = 1 << 62  # device_min_lines above any file: the host reader


def _both(path):
    out = []
    for lines in (0, HOST):
        try:
            out.append(spai_ir.mm_read(path, lines))
        except spai_ir.SpaiError as e:
            out.append((e.code, str(e)))
    return out


def _same(a, b):
    if isinstance(a[0], int):
        assert a == b
        return
    (sa, ca, _), (sb, cb, _) = a, b
    assert sa[0] == sb[0] and ca == cb
    for x, y in zip(sa[1:], sb[1:]):
        assert x.dtype == y.dtype and np.array_equal(x.view(np.uint8), y.view(np.uint8))


def _write(path, banner, dims, lines):
    path.write_text(banner + "\n" + dims + "\n" + "\n".join(lines) + "\n")


def _values(rng, k):
    """Value spellings: %.17g, %.6e, integers, leading/trailing zeros, signs, exponents, long
    digit strings (host-converted), hexadecimal (host-converted), values near rounding midpoints."""
    out = []
    for i in range(k):
        x = rng.standard_normal() * 10.0 ** rng.integers(-30, 30)
        f = i % 10
        if f == 0:
            out.append("%.17g" % x)
        elif f == 1:
            out.append("%.6e" % x)
        elif f == 2:
            out.append("%d" % rng.integers(-1000, 1000) or "7")
        elif f == 3:
            out.append("+00%.9fE+00" % abs(x % 7))
        elif f == 4:
            out.append(".%d" % rng.integers(1, 10 ** 9))
        elif f == 5:
            out.append("%d." % rng.integers(1, 10 ** 6))
        elif f == 6:
            out.append("%.25f" % (x % 3 + 0.1))  # more than 19 significant digits
        elif f == 7:
            out.append(float(abs(x) % 5 + 1).hex())  # hexadecimal
        elif f == 8:  # near a midpoint between two doubles
            d = abs(x) % 100 + 1.0
            mid = (d + np.nextafter(d, 200.0)) / 2
            out.append("%.20g" % mid)
        else:
            out.append("%.17g" % (x * 1e-250))
    return [v if v not in ("", "0") else "3" for v in out]


def test_device_reader_matches_host_reader(built, tmp_path):
    rng = np.random.default_rng(5)
    n = 300
    rows = rng.integers(1, n + 1, 4000)
    cols = rng.integers(1, n + 1, 4000)
    vals = _values(rng, 4000)
    lines = []
    for i, (r, c, v) in enumerate(zip(rows, cols, vals)):
        if i % 97 == 0:
            lines.append("% a comment line")
        if i % 131 == 0:
            lines.append("   \t")
        lines.append("%d %d %s" % (r, c, v))
    lines += ["%d %d 1.5" % (r, c) for r, c in zip(rows[:50], cols[:50])]  # duplicates
    for v in vals[:20]:  # exact zero sums on fresh coordinates are dropped
        r, c = rng.integers(1, n + 1, 2)
        neg = v[1:] if v.startswith("-") else "-" + v.lstrip("+")
        lines += ["%d %d %s" % (r, c, v), "%d %d %s" % (r, c, neg)]
    count = sum(1 for x in lines if x.strip() and not x.strip().startswith("%"))
    p = tmp_path / "g.mtx"
    _write(p, "%%MatrixMarket matrix coordinate real general", "%d %d %d" % (n, n, count), lines)
    dev, host = _both(p)
    _same(dev, host)
    assert dev[2] > 0  # some tokens went to the host converter

    sym = tmp_path / "s.mtx"
    slines = ["%d %d %s" % (max(r, c), min(r, c), v) for r, c, v in zip(rows, cols, vals)]
    _write(sym, "%%MatrixMarket matrix coordinate real symmetric", "%d %d %d" % (n, n, len(slines)), slines)
    _same(*_both(sym))

    ints = tmp_path / "i.mtx"
    ilines = ["%d %d %d" % (r, c, rng.integers(-9, 10)) for r, c in zip(rows, cols)]
    _write(ints, "%%MatrixMarket matrix coordinate integer general", "%d %d %d" % (n, n, len(ilines)), ilines)
    _same(*_both(ints))


def test_device_reader_large_system(built, tmp_path):
    system = M.convection_diffusion_3d(32)
    p = tmp_path / "c.mtx"
    M.write_matrix_market(str(p), system)
    (s, cols, conv) = spai_ir.mm_read(p, 0)
    assert cols == system[0]
    for x, y in zip(s, system):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    _same(*_both(p))


@pytest.mark.parametrize("case", [
    ("general", "3 3 2", ["1 1 1", "2 2"]),                 # malformed entry
    ("general", "3 3 2", ["1 1 1", "2 2 2 2"]),             # extra field
    ("general", "3 3 2", ["1 1 1", "2 x 2"]),               # index token
    ("general", "3 3 2", ["1 1 1", "2 99999999999999999999999 2"]),  # index overflow
    ("general", "3 3 2", ["1 1 1", "4 1 2"]),               # index range
    ("general", "3 3 2", ["1 1 1", "2 2 abc"]),             # invalid value (host)
    ("general", "3 3 2", ["1 1 1", "2 2 1.5x"]),            # partial value (host)
    ("general", "3 3 2", ["1 1 1", "2 2 inf"]),             # non-finite (host)
    ("general", "3 3 2", ["1 1 1", "2 2 1e400"]),           # overflow (host)
    ("general", "3 3 2", ["1 1 1", "2 2 1e-320"]),          # underflow (host)
    ("general", "3 3 3", ["1 1 1", "2 2 1"]),               # truncated
    ("general", "3 3 1", ["1 1 1", "2 2 1"]),               # trailing
    ("general", "3 3 2", ["1 1 1e308", "1 1 1e308"]),       # nonfinite duplicate sum
    ("general", "3 3 2", ["2 x 2", "4 1 2"]),               # first error in file order wins
    ("general", "3 3 2", ["2 2 abc", "4 1 2"]),
    ("general", "3 3 2", ["4 1 2", "2 2 abc"]),
])
def test_device_reader_errors_match_host(built, tmp_path, case):
    sym, dims, lines = case
    p = tmp_path / "e.mtx"
    _write(p, "%%MatrixMarket matrix coordinate real " + sym, dims, lines)
    dev, host = _both(p)
    assert isinstance(dev[0], int) and dev == host, (dev, host)


def test_device_reader_integer_field_errors(built, tmp_path):
    p = tmp_path / "e.mtx"
    _write(p, "%%MatrixMarket matrix coordinate integer general", "3 3 2", ["1 1 1", "2 2 1.5"])
    dev, host = _both(p)
    assert dev == host and dev[0] == spai_ir.ERR_FORMAT


@pytest.mark.parametrize("text", [
    "%%MatrixMarket matrix coordinate real general\r\n3 3 3\r\n1 1 2.5\r\n2 2 -1\r\n3 3 4e0\r\n",   # CRLF
    "%%MatrixMarket matrix coordinate real general\n3 3 3\n1\t1\t2.5\n 2  2  -1 \n3 3 4e0",        # tabs, no final newline
    "%%MatrixMarket matrix coordinate real general\n%c\n3 3 3\n\n1 1 2.5\n  \t \n2 2 -1\n%x\n3 3 4e0\n\n",  # blanks
    "%%MatrixMarket matrix coordinate real general\n3 3 0\n",                                      # no entries
    "%%MatrixMarket matrix coordinate real symmetric\n3 3 2\n2 1 0.1\n3 3 1E-300\n",                # small values
])
def test_device_reader_edge_spellings(built, tmp_path, text):
    p = tmp_path / "x.mtx"
    p.write_bytes(text.encode())
    dev, host = _both(p)
    _same(dev, host)
