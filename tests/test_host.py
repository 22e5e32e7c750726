"""Host-side checks that need no GPU: the C ABI library loads and exports every declared symbol,
the host build of the device hypot agrees with the oracle, the drop-in CLIs' input-error exit
codes (tests/check_solver_cli.py cases that fail before any device work), the seeded generators,
and the replica reduction of bench.py over a world_size-2 gloo group."""
import math
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O
import spai_ir
from conftest import ROOT
from spai_ir import matrices as M

TINY_MTX = """%%MatrixMarket matrix coordinate real general
% A*[1,-2,3]' = [2,-5,7]'
3 3 7
1 1 4
1 2 1
2 1 2
2 2 5
2 3 1
3 2 1
3 3 3
"""


def declared_functions():
    text = open(os.path.join(ROOT, "include", "spai_ir.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_]+)\s*\([^;{]*\)\s*;", text)) - {"if", "while"})


def test_library_exports_every_declared_symbol(built):
    lib = spai_ir.lib()
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(spai_ir.SIGNATURES), set(names) - set(spai_ir.SIGNATURES)


def test_status_names_match_reference(built):
    lib = spai_ir.lib()
    for i, s in enumerate(spai_ir.SPAI_STATUS):
        assert lib.spai_status_name(i).decode() == s
    for i, s in enumerate(spai_ir.GMRES_STATUS):
        assert lib.gmres_status_name(i).decode() == s
    for i, s in enumerate(spai_ir.IR_STATUS):
        assert lib.ir_status_name(i).decode() == s


def test_device_hypot_host_build_matches_oracle(built):
    rng = np.random.default_rng(11)
    ex = rng.integers(-300, 300, 40000)
    x = rng.uniform(1, 2, ex.size) * np.exp2(ex)
    y = rng.uniform(1, 2, ex.size) * np.exp2(ex + rng.integers(-40, 40, ex.size))
    for a, b in zip(x.tolist(), y.tolist()):
        assert spai_ir.hypot(a, b) == O.hypot(a, b)
    xf = (rng.uniform(-3, 3, 40000) * np.exp2(rng.integers(-60, 60, 40000))).astype(np.float32)
    yf = (rng.uniform(-3, 3, 40000) * np.exp2(rng.integers(-60, 60, 40000))).astype(np.float32)
    for a, b in zip(xf.tolist(), yf.tolist()):
        assert spai_ir.hypotf(a, b) == O.hypotf(a, b)


@pytest.mark.parametrize("cli", ["gpu_fp64_ir", "gpu_fp32_ir", "gpu_mixed_ir", "gpu_diag_ir"])
def test_cli_input_errors(built, tmp_path, cli):
    exe = spai_ir.cli_path(cli)
    mtx = tmp_path / "tiny.mtx"
    mtx.write_text(TINY_MTX)

    def rc(*args):
        return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=60).returncode

    assert rc() == 2
    assert rc(mtx, "nan") == 2
    assert rc(mtx, ".5", "21") == 2
    assert rc(mtx, ".5", "20", "4") == 2
    assert rc(mtx, ".5", "-1") == 2
    assert rc(mtx, "0") == 2
    assert rc(mtx, "1e400") == 2
    assert rc(tmp_path / "missing.mtx") == 2
    bad = tmp_path / "bad.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n3 3\n")
    assert rc(bad) == 1  # unsupported format: runtime_error -> solver error exit 1
    nonsq = tmp_path / "nonsq.mtx"
    nonsq.write_text("%%MatrixMarket matrix coordinate real general\n2 3 1\n1 1 1\n")
    assert rc(nonsq) == 2


def test_generators():
    n, ptr, idx, val = M.convection_diffusion_2d(64)
    assert n == 4096 and len(val) == 5 * n - 4 * 64
    n, ptr, idx, val = M.convection_diffusion_3d(20)
    assert len(val) == 7 * n - 6 * 20 * 20
    for system in (M.convection_diffusion_2d(9, 7, (0.3, -0.9), 25.0), M.irregular(5000, seed=2),
                   M.anisotropic_diffusion(16, seed=1)):
        n, ptr, idx, val = system
        assert ptr[0] == 0 and ptr[-1] == len(idx) and np.all(np.diff(ptr) >= 1)
        for r in range(0, n, max(1, n // 50)):
            row = idx[ptr[r]:ptr[r + 1]]
            assert np.all(np.diff(row) > 0) and r in row
        assert np.all(val != 0) and np.all(np.isfinite(val))
    n, ptr, idx, val = M.irregular(200000, seed=5)
    assert 11.0 < len(val) / n - 1 < 14.0  # Zipf(1.5) on [1,256]: mean ~12.3 off-diagonals
    d = M.dense(M.anisotropic_diffusion(12, seed=4))
    assert np.allclose(d, d.T) and np.all(np.linalg.eigvalsh(d) > 0)


def _replica_worker(rank, world, port, out):
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    out[rank] = bench.max_over_ranks(10.0 + rank, world)
    dist.destroy_process_group()


def test_bench_replica_max_over_ranks_gloo():
    import multiprocessing as mp
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        ps = [ctx.Process(target=_replica_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
        assert all(p.exitcode == 0 for p in ps)
        assert out[0] == out[1] == 11.0


def _py_read(text):
    """Independent restatement of read_matrix_market + from_entries (src/cpu.cpp:49-161) for
    valid inputs: one-based entries, symmetric mirrors, stable (row, col) order, duplicates summed
    in input order, exact zero sums dropped."""
    lines = [l for l in text.splitlines()[1:] if l.strip(" \t\r") and not l.strip(" \t\r").startswith("%")]
    banner = text.splitlines()[0].split()
    rows, cols, count = map(int, lines[0].split())
    ent = []
    for l in lines[1:1 + count]:
        r, c, v = l.split()
        r, c, v = int(r) - 1, int(c) - 1, float(v)
        ent.append((r, c, v))
        if banner[4] == "symmetric" and r != c:
            ent.append((c, r, v))
    ent.sort(key=lambda e: (e[0], e[1]))  # Python's sort is stable
    ptr, idx, val = [0] * (rows + 1), [], []
    i = 0
    while i < len(ent):
        r, c, s = ent[i]
        i += 1
        while i < len(ent) and ent[i][:2] == (r, c):
            s += ent[i][2]
            i += 1
        if s != 0.0:
            idx.append(c)
            val.append(s)
            ptr[r + 1] += 1
    for r in range(rows):
        ptr[r + 1] += ptr[r]
    return rows, cols, np.array(ptr), np.array(idx), np.array(val)


@pytest.mark.parametrize("sym", ["general", "symmetric"])
def test_mm_reader_host_path_matches_restatement(built, tmp_path, sym):
    rng = np.random.default_rng(3)
    n = 40
    lines = []
    for k in range(600):
        r, c = sorted(rng.integers(1, n + 1, 2), reverse=(sym == "symmetric"))
        v = rng.choice(["%.17g" % rng.standard_normal(), "%d" % rng.integers(-3, 4), "1.5e-3", "-2."])
        if k % 50 == 0:
            lines.append("% comment")
        lines.append("%d %d %s" % (r, c, v))
    count = sum(1 for l in lines if not l.startswith("%"))
    text = "%%MatrixMarket matrix coordinate real " + sym + "\n%d %d %d\n" % (n, n, count) + "\n".join(lines) + "\n"
    p = tmp_path / "m.mtx"
    p.write_text(text)
    (nn, ptr, idx, val), cols, _ = spai_ir.mm_read(p, 1 << 62)  # host path: no GPU needed
    rows, cols2, ptr2, idx2, val2 = _py_read(text)
    assert nn == rows and cols == cols2
    assert np.array_equal(ptr, ptr2) and np.array_equal(idx, idx2)
    assert np.array_equal(val.view(np.uint64), val2.view(np.uint64))


def test_mm_reader_host_path_errors(built, tmp_path):
    p = tmp_path / "e.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1\n4 1 2\n")
    with pytest.raises(spai_ir.SpaiError) as e:
        spai_ir.mm_read(p, 1 << 62)
    assert e.value.code == spai_ir.ERR_FORMAT and "outside one-based" in str(e.value)
    with pytest.raises(spai_ir.SpaiError) as e:
        spai_ir.mm_read(tmp_path / "missing.mtx", 1 << 62)
    assert e.value.code == spai_ir.ERR_ARGUMENT


BANNER = "%%MatrixMarket matrix coordinate real general\n"
MM_ERRORS = [
    ("", "Missing Matrix Market banner"),
    ("%%MatrixMarket matrix coordinate real\n3 3 0\n", "Malformed Matrix Market banner"),
    ("%%MatrixMarket matrix coordinate real general x\n3 3 0\n", "Extra field in Matrix Market line"),
    ("%%MatrixMarket matrix array real general\n3 3 0\n", "Unsupported Matrix Market format"),
    ("%%MatrixMarket matrix coordinate complex general\n3 3 0\n", "Unsupported Matrix Market format"),
    ("%%matrixmarket matrix coordinate real general\n3 3 0\n", "Unsupported Matrix Market format"),
    (BANNER, "Missing matrix dimensions"),
    (BANNER + "% only a comment\n \t\r\n", "Missing matrix dimensions"),
    (BANNER + "3 3\n", "Malformed matrix dimensions"),
    (BANNER + "3 3 0 0\n", "Extra field in Matrix Market line"),
    (BANNER + "3 x 0\n", "Expected a nonnegative integer dimension/index"),
    (BANNER + "+3 3 0\n", "Expected a nonnegative integer dimension/index"),
    (BANNER + "99999999999999999999 3 0\n", "Dimension/index exceeds size_t"),
    (BANNER + "0 3 0\n", "Matrix dimensions must be positive"),
    ("%%MatrixMarket matrix coordinate real symmetric\n3 4 0\n", "Symmetric matrix must be square"),
    (BANNER + "3 3 2\n1 1 1\n", "Truncated coordinate data"),
    (BANNER + "3 3 1\n1 1 1\n2 2 2\n", "Trailing coordinate data"),
    (BANNER + "3 3 1\n1 1\n", "Malformed coordinate entry"),
    (BANNER + "3 3 1\n\v\n", "Malformed coordinate entry"),
    (BANNER + "3 3 1\n1 1 1 1\n", "Extra field in Matrix Market line"),
    (BANNER + "3 3 1\n-1 1 1\n", "Expected a nonnegative integer dimension/index"),
    (BANNER + "3 3 1\n1 18446744073709551616 1\n", "Dimension/index exceeds size_t"),
    (BANNER + "3 3 1\n4 1 1\n", "Matrix Market index outside one-based dimensions"),
    (BANNER + "3 3 1\n1 0 1\n", "Matrix Market index outside one-based dimensions"),
    (BANNER + "3 3 1\n1 1 abc\n", "Invalid coordinate value"),
    (BANNER + "3 3 1\n1 1 1e400\n", "Invalid coordinate value"),
    (BANNER + "3 3 1\n1 1 1e-320\n", "Invalid coordinate value"),
    (BANNER + "3 3 1\n1 1 1.5x\n", "Coordinate value must be finite and numeric"),
    (BANNER + "3 3 1\n1 1 inf\n", "Coordinate value must be finite and numeric"),
    (BANNER + "3 3 1\n1 1 nan\n", "Coordinate value must be finite and numeric"),
    ("%%MatrixMarket matrix coordinate integer general\n3 3 1\n1 1 1.5\n",
     "Integer field requires integer value tokens"),
    ("%%MatrixMarket matrix coordinate integer general\n3 3 1\n1 1 1e3\n",
     "Integer field requires integer value tokens"),
]


@pytest.mark.parametrize("text,message", MM_ERRORS)
def test_mm_reader_host_path_error_contract(built, tmp_path, text, message):
    """Every malformed-input case of the reference reader (src/cpu.cpp:105-161) gives its message
    and the runtime_error class (SPAI_ERR_FORMAT, CLI exit 1) through the host reader."""
    p = tmp_path / "e.mtx"
    p.write_bytes(text.encode())
    with pytest.raises(spai_ir.SpaiError) as e:
        spai_ir.mm_read(p, 1 << 62)
    assert e.value.code == spai_ir.ERR_FORMAT, (text, str(e.value))
    assert str(e.value).endswith(": " + message), (text, str(e.value))


def test_mm_reader_host_path_invalid_entries_and_edge_cases(built, tmp_path):
    """A duplicate sum that overflows is an invalid entry (invalid_argument: SPAI_ERR_ARGUMENT, CLI
    exit 2). Valid edge cases: CRLF line ends and tabs, no final newline, comment and blank lines
    between entries, a zero duplicate sum dropped, symmetric mirrors, integer spellings."""
    p = tmp_path / "d.mtx"
    p.write_text(BANNER + "2 2 2\n1 1 1e308\n1 1 1e308\n")
    with pytest.raises(spai_ir.SpaiError) as e:
        spai_ir.mm_read(p, 1 << 62)
    assert e.value.code == spai_ir.ERR_ARGUMENT and str(e.value).endswith(": Duplicate sum is nonfinite")
    p.write_bytes(b"%%MatrixMarket matrix coordinate real symmetric\r\n% c\r\n3\t3 5\r\n"
                  b"1 1 2.5\r\n\r\n3 1 -1\r\n % indented comment\n2 2 4\n3 3 1\n3 3 -1")
    (n, ptr, idx, val), cols, _ = spai_ir.mm_read(p, 1 << 62)
    assert n == 3 and cols == 3
    assert ptr.tolist() == [0, 2, 3, 4]
    assert idx.tolist() == [0, 2, 1, 0] and val.tolist() == [2.5, -1.0, 4.0, -1.0]
    p.write_text("%%MatrixMarket matrix coordinate integer general\n2 2 3\n2 2 +7\n1 2 -3\n2 2 -07\n")
    (n, ptr, idx, val), cols, _ = spai_ir.mm_read(p, 1 << 62)
    assert ptr.tolist() == [0, 1, 1] and idx.tolist() == [1] and val.tolist() == [-3.0]


def test_snapshot_number_format_round_trips():
    """The release snapshot's numbers: C99 hex-float plus '@' and the IEEE-754 bits
    (tests/release_cpu_snapshot.cpp:38-57 of the reference), exact for every finite binary64."""
    import struct

    from spai_ir import snapshot as S

    rng = np.random.default_rng(11)
    values = [0.0, -0.0, 1.0, -1.5, 0.1, 5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
              math.ldexp(1.0, -1074), -math.ldexp(3.0, -1060)] + list(rng.standard_normal(200) * 10.0 ** rng.integers(-300, 300, 200))
    for v in values:
        text = S._hex(v)
        lit, bits = text.split("@")
        x = float.fromhex(lit)
        assert struct.pack(">d", x) == struct.pack(">d", v), text
        assert struct.unpack(">Q", struct.pack(">d", x))[0] == int(bits, 16)
    for bad in (math.inf, -math.inf, math.nan):
        with pytest.raises(ValueError):
            S._hex(bad)
    assert S._hex(1.0) == "0x1.0000000000000p0@3ff0000000000000"
    assert S._hex(-0.0) == "-0x0.0000000000000p-1022@8000000000000000"
