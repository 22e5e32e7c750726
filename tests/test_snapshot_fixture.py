"""The release snapshot (schema 2) the device solver printed on a GB300
(`spai-gmres-ir_gb300/spai_release_snapshot > tests/golden/release_snapshot_gb300.txt`), checked
on the CPU with exact rational arithmetic where the relation is exact and binary64 bounds where it
is not:

* every number is a hex float whose IEEE bits match its payload;
* status-only cases carry the reference's expected statuses;
* B = A^T D and P = N D hold entry by entry as the device's binary64 products;
* every fit history grows its pattern by its selection, and its shadow is the union of B's
  column patterns over J; the selection is the binary64 (score, index) order below the mean;
* recorded GMRES solves satisfy P A V_m = V_{m+1} H_m, keep v_0..v_{m-1} orthonormal, and the
  refinement's states satisfy r = b - A x and x_s = x_{s-1} + d_s;
* the device's fit histories and P equal the oracle's bit for bit, and its GMRES case matches
  the oracle's solve.
"""
import json
import math
import os
import struct
from fractions import Fraction

import numpy as np
import pytest

from spai_ir import SPAI_STATUS

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "release_snapshot_gb300.txt")


def _num(text):
    lit, bits = text.split("@")
    x = float.fromhex(lit)
    assert math.isfinite(x) and struct.unpack(">Q", struct.pack(">d", x))[0] == int(bits, 16), text
    return x


def _vec(items):
    return np.array([_num(t) for t in items])


def _rows(c):
    vals = _vec(c["values"])
    off, idx = c["offsets"], c["indices"]
    assert len(off) == c["rows"] + 1 and off[0] == 0 and off[-1] == len(idx) == len(vals)
    return [{idx[t]: vals[t] for t in range(off[i], off[i + 1])} for i in range(c["rows"])]


def _dense(c):
    a = np.zeros((c["rows"], c["cols"]))
    for i, row in enumerate(_rows(c)):
        for j, v in row.items():
            a[i, j] = v
    return a


@pytest.fixture(scope="module")
def items():
    out = []
    with open(FIXTURE) as f:
        for line in f:
            assert line.startswith("RELEASE_CPU_SNAPSHOT ")
            out.append(json.loads(line[len("RELEASE_CPU_SNAPSHOT "):]))
    return {it["case"]: it for it in out}


def test_cases_and_statuses(items):
    assert len(items) == 15 and all(it["schema"] == 2 for it in items.values())
    for it in items.values():
        if "expected_status" in it:
            assert it["actual_status"] == it["expected_status"], it["case"]


def test_number_payloads(items):
    def walk(v):
        if isinstance(v, str) and "@" in v:
            _num(v)
        elif isinstance(v, dict):
            for u in v.values():
                walk(u)
        elif isinstance(v, list):
            for u in v:
                walk(u)

    for it in items.values():
        walk(it)


@pytest.mark.parametrize("case", ["spai_direct_full", "spai_gmres_ir", "spai_tie_growth", "spai_near_dependent"])
def test_construction_relations(items, case):
    it = items[case]
    a = _rows(it["A"])
    con = it["construction"]
    n = len(a)
    d = _vec(con["scaling"])
    bmat = _rows(con["B"])
    for i, row in enumerate(bmat):  # B(i, j) = A(j, i) d_j, the device's binary64 product
        for j, v in row.items():
            assert v == a[j][i] * d[j]
    assert sum(len(r) for r in bmat) == sum(len(r) for r in a)
    nmat, pmat = _rows(con["N"]), _rows(con["P"])
    for k, col in enumerate(con["columns"]):
        hist = col["history"]
        assert hist and hist[0]["J"] == [k] and col["pattern"] == hist[-1]["J"]
        assert list(_vec(col["coefficients"])) == list(_vec(hist[-1]["coefficients"]))
        for f, fit in enumerate(hist):
            shadow = sorted({i for i, row in enumerate(bmat) for j in row if j in fit["J"]})
            assert fit["I"] == shadow
            assert fit["residual"] == fit["full_residual"]
            if f + 1 < len(hist):
                scores = [_num(s) for s in fit["scores"]]
                assert len(scores) == len(fit["candidates"])
                mean = sum(scores) / len(scores)  # sequential binary64 sum (src/spai.cpp:216)
                assert _num(fit["mean_score"]) == mean
                want = [c for s, c in sorted(zip(scores, fit["candidates"])) if s <= mean][: it["beta"]]
                assert fit["selected"] == want
                assert hist[f + 1]["J"] == sorted(set(fit["J"]) | set(fit["selected"]))
            else:
                assert fit["candidates"] == [] and fit["selected"] == []
        for j, m in zip(col["pattern"], _vec(col["coefficients"])):
            if m != 0:
                assert nmat[j][k] == m
                assert pmat[k][j] == m * d[j]  # P(k, j) = m_jk d_j
    assert sum(len(r) for r in pmat) == sum(len(r) for r in nmat)


def _gmres_relations(a, p, rhs, g):
    V = np.array([_vec(v) for v in g["basis"]])
    H = np.array([_vec(r) for r in g["H"]])
    m = g["iterations"]
    assert len(g["history"]) == m and V.shape[0] in (m, m + 1)
    # v_0..v_{m-1} orthonormal; a last vector normalised from a rounding-level subdiagonal (a
    # Krylov space that exhausted R^n) is noise in either implementation and enters the relation
    # below only through that subdiagonal
    assert np.abs(V[:m] @ V[:m].T - np.eye(m)).max() < 1e-13
    for j in range(m):
        w = p @ (a @ V[j])
        kmax = min(j + 2, V.shape[0])
        assert np.linalg.norm(w - H[:kmax, j] @ V[:kmax]) <= 1e-13 * max(1.0, np.linalg.norm(w))
    pr = p @ rhs
    beta = np.linalg.norm(pr)
    for h in g["history"]:
        x = _vec(h["solution"])
        rel = np.linalg.norm(pr - p @ (a @ x)) / beta
        assert abs(_num(h["recomputed"]) - rel) <= 1e-12 * max(1.0, rel)
        if h["accepted"]:
            assert h["verified"] and _num(h["recomputed"]) <= 1e-8


def test_gmres_case(items):
    it = items["gmres_identity_nonsymmetric"]
    g = it["gmres"]
    assert g["status"] == "success" and g["converged"]
    _gmres_relations(_dense(it["A"]), _dense(it["fixed_P"]), _vec(it["b"]), g)


@pytest.mark.parametrize("case", ["spai_gmres_ir", "ir_identity_preconditioner_correction", "ir_inner_iteration_limit"])
def test_refinement_relations(items, case):
    it = items[case]
    a = _dense(it["A"])
    p = _dense(it["fixed_P"]) if "fixed_P" in it else _dense(it["construction"]["P"])
    b = _vec(it["b"])
    ir = it["ir"]
    hist = ir["history"]
    # x0 = P b, exactly rounded entries of an exact rational product
    x0 = _vec(hist[0]["x"])
    exact = [sum((Fraction(v) * Fraction(b[j]) for j, v in enumerate(row) if v != 0), Fraction(0)) for row in p]
    assert all(abs(Fraction(x) - e) <= abs(e) * Fraction(1, 2 ** 50) for x, e in zip(x0, exact))
    for s, st in enumerate(hist):
        x = _vec(st["x"])
        r = _vec(st["diagnostics"]["residual"])
        assert np.abs(r - (b - a @ x)).max() <= 1e-14 * (np.abs(a).sum(1).max() * np.abs(x).max() + np.abs(b).max())
        assert _num(st["diagnostics"]["inf"]) == np.abs(r).max()
        if s:
            inner = st["inner"]
            assert inner["converged"]
            assert list(_vec(ir["rhs"][s - 1])) == list(_vec(hist[s - 1]["diagnostics"]["residual"]))
            assert list(x) == list(_vec(hist[s - 1]["x"]) + _vec(inner["solution"]))
            _gmres_relations(a, p, _vec(ir["rhs"][s - 1]), inner)
    assert len(ir["updates"]) == len(ir["inner_history"]) == ir["inner_attempts"]
    if ir["converged"]:
        assert _num(hist[-1]["diagnostics"]["nbe"]) <= 10 * 2.0 ** -53


@pytest.mark.parametrize("case", ["spai_direct_full", "spai_gmres_ir", "spai_tie_growth", "spai_near_dependent"])
def test_device_fit_histories_equal_the_oracle(items, case, built):
    """The GB300's fit log in the fixture equals the oracle's fit histories bit for bit."""
    import oracle as O

    it = items[case]
    a = it["A"]
    system = (a["rows"], np.array(a["offsets"], np.int64), np.array(a["indices"], np.int64), _vec(a["values"]))
    ref = O.Spai(system, _num(it["epsilon"]), it["alpha"], it["beta"], history=True)
    cols = it["construction"]["columns"]
    assert [c["status"] for c in cols] == [SPAI_STATUS[s] for s in ref.col_status]
    for k, col in enumerate(cols):
        assert len(col["history"]) == ref.fits[k]
        for f, fit in enumerate(col["history"]):
            r = ref.fit(k, f)
            assert fit["J"] == list(r["pattern"]) and fit["I"] == list(r["shadow"])
            assert list(_vec(fit["coefficients"])) == list(r["coefficients"])
            assert _num(fit["residual"]) == r["residual"] and _num(fit["pivot_ratio"]) == r["pivot_ratio"]
            assert fit["candidates"] == list(r["candidates"]) and fit["selected"] == list(r["selected"])
            assert list(_vec(fit["scores"])) == list(r["scores"])
            if fit["candidates"]:
                assert _num(fit["mean_score"]) == r["mean_score"]
    pd = _dense(it["construction"]["P"])
    po = np.zeros_like(pd)
    for i in range(ref.n):
        po[i, ref.p_idx[ref.p_ptr[i]:ref.p_ptr[i + 1]]] = ref.p_val[ref.p_ptr[i]:ref.p_ptr[i + 1]]
    assert np.array_equal(pd, po)


def test_device_gmres_case_matches_the_oracle(items, built):
    import oracle as O

    it = items["gmres_identity_nonsymmetric"]
    a, p = it["A"], it["fixed_P"]
    sys_a = (a["rows"], np.array(a["offsets"], np.int64), np.array(a["indices"], np.int64), _vec(a["values"]))
    sys_p = (p["rows"], np.array(p["offsets"], np.int64), np.array(p["indices"], np.int64), _vec(p["values"]))
    x, rep = O.gmres(sys_a, sys_p, _vec(it["b"]), tol=1e-8)
    g = it["gmres"]
    assert rep["iterations"] == g["iterations"] and g["status"] == "success" and rep["status"] == 0
    np.testing.assert_allclose(_vec(g["solution"]), x, rtol=1e-13, atol=1e-15)
