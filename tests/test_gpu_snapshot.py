"""Record mode and the release snapshot (schema 2).

* The device's fit log equals the oracle's fit histories bit for bit: every fit's pattern J,
  shadow I, coefficients, residual and pivot ratio, and for the fits that went on to growth the
  candidates, scores, mean score and the selection in selection order (the reference's
  SpaiColumn::history, src/spai.cpp:100-244).
* A recorded refinement solve obeys the relations the reference's Decimal audit checks
  (tests/check_release_cpu_decimal.py): x0 = P b, every residual is b - A x, every applied
  correction is the inner solution, the basis is orthonormal, P A V_m = V_{m+1} H_m, each step's
  estimate follows from the unrotated Hessenberg by Givens rotations, each step's candidate has
  the recomputed residuals recorded for it, and only a triggered check accepts. Its outcome equals
  the unrecorded solve's (three-pass against lagged orthogonalisation: equal to rounding).
* The snapshot emitter's cases, statuses and number format.
"""
import json
import math
import struct

import numpy as np
import pytest

import oracle as O
import spai_ir
from spai_ir import matrices as M
from spai_ir import snapshot as S

pytestmark = pytest.mark.gpu


def _dense(system):
    n, ptr, idx, val = system
    a = np.zeros((n, n))
    for i in range(n):
        a[i, idx[ptr[i]:ptr[i + 1]]] = val[ptr[i]:ptr[i + 1]]
    return a


FIT_SYSTEMS = {
    "tiny_nonsymmetric": (S._dense([[4, 1, 0], [2, 5, 1], [0, 1, 3]]), 1e-12, 2, 8),
    "tie": (S._dense([[1, 1, 1], [1, 1, 0], [1, 0, 1]]), 1e-12, 1, 1),
    "cd2d_16": (M.convection_diffusion_2d(16), 0.3, 32, 8),
    "irregular_400": (M.irregular(400, seed=1), 0.4, 5, 8),
}


@pytest.mark.parametrize("name", sorted(FIT_SYSTEMS))
def test_fit_log_equals_oracle_fit_histories(built, name):
    system, eps, alpha, beta = FIT_SYSTEMS[name]
    n = system[0]
    with spai_ir.Handle(system, "f64") as h:
        h.record()
        rep = h.build(spai_ir.options("f64", epsilon=eps, alpha=alpha, beta=beta))
        log = h.fit_log()
    ref = O.Spai(system, eps, alpha, beta, history=True)
    assert rep["spai_status"] == ref.status
    compared = 0
    for k in range(n):
        fits = log.get(k, [])
        assert len(fits) == ref.fits[k], k
        for f, dev in enumerate(fits):
            r = ref.fit(k, f)
            assert dev["J"] == list(r["pattern"]) and dev["I"] == list(r["shadow"]), (k, f)
            assert np.array_equal(dev["coefficients"], r["coefficients"]), (k, f)
            assert dev["residual"] == r["residual"] and dev["pivot_ratio"] == r["pivot_ratio"], (k, f)
            if "candidates" in dev:
                assert dev["candidates"] == list(r["candidates"]), (k, f)
                assert np.array_equal(dev["scores"], r["scores"]), (k, f)
                assert dev["mean_score"] == r["mean_score"], (k, f)
                assert dev.get("selected", []) == list(r["selected"]), (k, f)
            else:
                assert len(r["selected"]) == 0, (k, f)
            compared += 1
    assert compared >= n


def _givens_estimates(H, m, beta):
    """|g_{j+1}| / beta after the Givens update of each column j (src/gmres.cpp:191-214)."""
    cs, sn, out = [], [], []
    g = np.zeros(m + 1)
    g[0] = beta
    for j in range(m):
        col = H[: j + 2, j].copy()
        for r, (c, s) in enumerate(zip(cs, sn)):
            col[r], col[r + 1] = c * col[r] + s * col[r + 1], -s * col[r] + c * col[r + 1]
        rad = math.hypot(col[j], col[j + 1])
        c, s = col[j] / rad, col[j + 1] / rad
        cs.append(c)
        sn.append(s)
        g[j], g[j + 1] = c * g[j], -s * g[j]
        out.append(abs(g[j + 1]) / beta)
    return np.array(out)


def test_recorded_refinement_obeys_the_audited_relations(built):
    system = M.convection_diffusion_2d(16)
    n = system[0]
    A = _dense(system)
    b = M.equal_rhs(n)
    o = spai_ir.cli_options(n, "f64", innercap=60)
    with spai_ir.Handle(system, "f64") as h:
        h.build(o)
        x_plain, rep_plain = h.solve(b, o)
        Pd = _dense(h.preconditioner())
        h.record()
        x_rec, rep = h.solve(b, o)
        rec = h.recorded()
        outer, _, _ = h.history()
    assert rep_plain["converged"] and rep["converged"]
    assert rep["outer_steps"] == rep_plain["outer_steps"]
    assert abs(rep["inner_iterations"] - rep_plain["inner_iterations"]) <= rep["inner_attempts"]
    np.testing.assert_allclose(x_rec, x_plain, rtol=0, atol=1e-12 * np.abs(x_plain).max())
    states, inner = rec["states"], rec["inner"]
    assert len(states) == rep["outer_steps"] + 1 and len(inner) == rep["inner_attempts"]
    np.testing.assert_array_equal(states[-1][0], x_rec)
    np.testing.assert_allclose(states[0][0], Pd @ b, rtol=1e-13, atol=1e-15)
    scale = np.abs(A).sum(axis=1).max() * max(np.abs(s[0]).max() for s in states) + np.abs(b).max()
    applied = [r for r in inner if r["applied"]]
    for s, (x, r) in enumerate(states):
        np.testing.assert_allclose(r, b - A @ x, rtol=0, atol=1e-14 * scale)
        assert outer[s]["residual_inf"] == np.abs(r).max()
        if s:
            np.testing.assert_array_equal(applied[s - 1]["rhs"], states[s - 1][1])
            np.testing.assert_allclose(x, states[s - 1][0] + applied[s - 1]["solution"], rtol=1e-15, atol=0)
    tau = 1e-8
    for r in inner:
        m, V, H = r["steps"], r["basis"], r["hessenberg"]
        assert m >= 1 and V.shape[0] in (m, m + 1) and H.shape == (o.innercap + 1, o.innercap)
        np.testing.assert_allclose(V[:m] @ V[:m].T, np.eye(m), rtol=0, atol=1e-12)
        for j in range(m):
            w = Pd @ (A @ V[j])
            kmax = min(j + 2, V.shape[0])
            np.testing.assert_allclose(w, H[:kmax, j] @ V[:kmax], rtol=0, atol=1e-11 * np.linalg.norm(w))
        pr = Pd @ r["rhs"]
        beta = np.linalg.norm(pr)
        rows = r["step_rows"]
        np.testing.assert_allclose(rows[:, 1], _givens_estimates(H, m, beta), rtol=1e-7, atol=1e-15)
        for j in range(m):
            xj = r["candidates"][j]
            rel = np.linalg.norm(pr - Pd @ (A @ xj)) / beta
            orig = np.linalg.norm(r["rhs"] - A @ xj)
            assert abs(rows[j, 2] - rel) <= 1e-9 * rel + 1e-14, (j, rows[j, 2], rel)
            assert abs(rows[j, 3] - orig) <= 1e-9 * orig + 1e-14 * np.linalg.norm(r["rhs"]), (j, rows[j, 3], orig)
            assert rows[j, 4] == H[j + 1, j] and rows[j, 5] == (H[j + 1, j] == 0)
            if rows[j, 7]:
                assert rows[j, 6] and rows[j, 2] <= tau and j == m - 1
        assert r["converged"] == (rows[-1, 7] == 1)
        np.testing.assert_array_equal(r["solution"], r["candidates"][-1])


def test_identity_preconditioner_gmres_matches_oracle(built):
    a = S._dense([[4, 1, 0], [2, 5, 1], [0, 1, 3]])
    ident = S._identity(3)
    rhs = np.array([0.1, -0.7, 1.3])
    with spai_ir.Handle(a, "f64") as h:
        h.set_preconditioner(ident)
        with pytest.raises(spai_ir.SpaiError):
            h.columns()  # a caller-supplied P has no SPAI columns
        h.record()
        x, rep = h.gmres(rhs, 1e-8, 0)
        r = h.recorded()["inner"][0]
    xo, ro = O.gmres(a, ident, rhs, tol=1e-8)
    assert rep["status"] == ro["status"] == 0 and rep["iterations"] == ro["iterations"]
    np.testing.assert_allclose(x, xo, rtol=1e-13, atol=1e-15)
    np.testing.assert_array_equal(x, r["solution"])
    assert r["steps"] == rep["iterations"]


def test_snapshot_cases_statuses_and_number_format(built):
    items = S.cases()
    names = [it["case"] for it in items]
    assert names == ["gmres_identity_nonsymmetric", "spai_direct_full", "spai_gmres_ir",
                     "ir_identity_preconditioner_correction", "ir_inner_iteration_limit", "spai_tie_growth",
                     "spai_near_dependent", "spai_epsilon_equal_column0", "spai_epsilon_one_ulp_below",
                     "spai_beta_zero", "spai_rank_zero_pivot", "spai_scaling_overflow", "gmres_zero_rhs",
                     "gmres_iteration_cap", "ir_zero_rhs"]
    for it in items:
        assert it["schema"] == 2
        if "expected_status" in it:
            assert it["actual_status"] == it["expected_status"], it["case"]

    def walk(v):
        if isinstance(v, str) and "@" in v:
            lit, bits = v.split("@")
            x = float.fromhex(lit)
            assert math.isfinite(x) and struct.unpack(">Q", struct.pack(">d", x))[0] == int(bits, 16), v
        elif isinstance(v, dict):
            for u in v.values():
                walk(u)
        elif isinstance(v, list):
            for u in v:
                walk(u)

    for it in items:
        walk(it)
        json.dumps(it)
    by = {it["case"]: it for it in items}
    ir = by["spai_gmres_ir"]["ir"]
    assert ir["status"] == "success" and ir["converged"] and len(ir["history"]) == ir["outer_steps"] + 1
    fail = by["ir_inner_iteration_limit"]["ir"]
    assert fail["status"] == "inner_failure" and fail["updates"] == [False]
    assert not fail["inner_history"][0]["converged"]
    assert by["spai_direct_full"]["construction"]["columns"][0]["history"][0]["selected"] == [2]  # test_spai.cpp:167
    assert by["spai_tie_growth"]["construction"]["columns"][0]["history"][0]["selected"] == [1]  # :191-198
