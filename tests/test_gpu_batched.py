"""Batched solves (spai_ir_solve_batched): many independent systems, one SPAI build over their
block-diagonal union and one persistent refinement launch (a CTA per system).

Each system is checked against the binary32-SPAI / binary64-refinement oracle and against the
single-system solve of the same library: statuses, outer steps, the backward-error target
(10 * 2^-53) and the solution (both meet the target, so they agree to the condition number
times it). Per-system failures (invalid input, construction failure) stay local to their system.
"""
import numpy as np
import pytest

import spai_ir
from spai_ir import matrices as M

pytestmark = pytest.mark.gpu

BE64 = 10 * 2.0 ** -53


def _rhs(n, seed):
    return np.random.default_rng(seed).standard_normal(n)


def _small_batch(count=12, seed=4):
    return M.batched_convection_diffusion(count, seed=seed, side_range=(12, 48))


def test_batched_matches_oracle_and_single_solves(built):
    import oracle

    systems = _small_batch()
    bs = [_rhs(s[0], 10 + i) for i, s in enumerate(systems)]
    opts = spai_ir.options("mixed", epsilon=0.3, alpha=5, innercap=100)
    xs, reps = spai_ir.ir_solve_batched(systems, bs, opts)
    for i, (s, b, x, rep) in enumerate(zip(systems, bs, xs, reps)):
        xo, ro = oracle.ir(s, b, precision="mixed", epsilon=0.3, alpha=5, innercap=100)
        assert ro["converged"], (i, ro)
        assert rep["converged"], (i, rep)
        assert rep["spai_status"] == 0
        assert rep["backward_error"] <= BE64, (i, rep)
        assert abs(rep["outer_steps"] - ro["outer_steps"]) <= 1, (i, rep, ro)
        assert np.linalg.norm(x - xo, np.inf) <= 1e-9 * np.linalg.norm(xo, np.inf), i
        x1, r1 = spai_ir.ir_solve(s, b, opts)
        assert r1["converged"]
        assert abs(rep["outer_steps"] - r1["outer_steps"]) <= 1
        assert np.linalg.norm(x - x1, np.inf) <= 1e-9 * np.linalg.norm(x1, np.inf), i


def test_batched_preconditioner_equals_per_system_spai(built):
    """The block-diagonal build gives each system exactly its own SPAI: the batched solve with
    the reference-order SPAI reproduces the single-system iteration counts."""
    systems = _small_batch(6, seed=9)
    bs = [M.equal_rhs(s[0]) for s in systems]
    opts = spai_ir.options("mixed", epsilon=0.3, alpha=5, innercap=100)
    _, reps = spai_ir.ir_solve_batched(systems, bs, opts)
    for s, b, rep in zip(systems, bs, reps):
        with spai_ir.Handle(s, "mixed") as h:
            brep = h.build(opts)
            _, r1 = h.solve(b, opts)
        assert rep["spai_status"] == brep["spai_status"] == 0
        assert rep["inner_attempts"] == r1["inner_attempts"]
        assert abs(rep["inner_iterations"] - r1["inner_iterations"]) <= 2 * r1["inner_attempts"]


def test_batched_failures_stay_local(built):
    systems = _small_batch(5, seed=2)
    bs = [_rhs(s[0], i) for i, s in enumerate(systems)]
    bs[1] = bs[1].copy()
    bs[1][3] = np.nan  # invalid input for system 1 only
    # 60 diagonal copies of [[1, 1], [1, 1]]: every column's fit is rank deficient (n = 120 keeps
    # innercap 100 valid, so the failure is the construction's, not the options').
    blocks = 60
    ptr = np.arange(0, 4 * blocks + 1, 2)
    idx = np.repeat(np.arange(0, 2 * blocks, 2), 4) + np.tile([0, 1, 0, 1], blocks)
    singular = (2 * blocks, ptr, idx, np.ones(4 * blocks))
    systems.insert(3, singular)
    bs.insert(3, np.ones(2 * blocks))
    opts = spai_ir.options("mixed", epsilon=0.3, alpha=5, innercap=100)
    xs, reps = spai_ir.ir_solve_batched(systems, bs, opts)
    assert reps[1]["ir_status"] == spai_ir.IR_INVALID_INPUT
    assert reps[3]["ir_status"] == spai_ir.IR_CONSTRUCTION_FAILURE
    assert reps[3]["spai_status"] != 0
    for i in (0, 2, 4, 5):
        assert reps[i]["converged"], (i, reps[i])
        assert reps[i]["backward_error"] <= BE64


def test_batched_zero_rhs_and_bad_arguments(built):
    systems = _small_batch(3, seed=5)
    bs = [np.zeros(s[0]) for s in systems]
    opts = spai_ir.options("mixed", epsilon=0.3, alpha=5, innercap=50)
    xs, reps = spai_ir.ir_solve_batched(systems, bs, opts)
    for x, rep in zip(xs, reps):
        assert rep["converged"] and rep["outer_steps"] == 0
        assert not np.any(x)
    with pytest.raises(spai_ir.SpaiError) as e:
        spai_ir.ir_solve_batched(systems, bs, spai_ir.options("f64", innercap=50))
    assert e.value.code == spai_ir.ERR_UNSUPPORTED


def test_batched_workload_512_systems(built):
    """512 systems, sides log-uniform in [32, 256], Pe in [0, 50]; eps 0.3, innercap 100. With a
    cap of 100 Arnoldi steps some systems' inner GMRES cannot reach tau (the oracle fails them the
    same way: inner_failure after an iteration-limited GMRES); every converged system meets the
    binary64 target, and a sample of converged and failing systems matches the oracle."""
    import oracle

    systems = M.batched_convection_diffusion(512, seed=0)
    bs = [M.equal_rhs(s[0]) for s in systems]
    opts = spai_ir.options("mixed", epsilon=0.3, alpha=5, innercap=100)
    xs, reps = spai_ir.ir_solve_batched(systems, bs, opts)
    conv = [i for i, r in enumerate(reps) if r["converged"]]
    fail = [i for i, r in enumerate(reps) if not r["converged"]]
    assert conv
    assert max(reps[i]["backward_error"] for i in conv) <= BE64
    for i in fail:
        assert reps[i]["ir_status"] == spai_ir.IR_INNER_FAILURE, (i, reps[i])
        assert reps[i]["gmres_status"] == 6, (i, reps[i])  # iteration_limit
    order = np.argsort([s[0] for s in systems])
    sample = [i for i in order if i in conv][:4] + [i for i in order if i in fail][:3]
    for i in sample:
        xo, ro = oracle.ir(systems[i], bs[i], precision="mixed", epsilon=0.3, alpha=5, innercap=100)
        assert ro["status"] == reps[i]["ir_status"], (i, ro, reps[i])
        if ro["converged"]:
            assert abs(ro["outer_steps"] - reps[i]["outer_steps"]) <= 1
            assert np.linalg.norm(xs[i] - xo, np.inf) <= 1e-9 * np.linalg.norm(xo, np.inf)


def test_batched_workload_restart_at_cap(built):
    """With SPAI_FLAG_RESTART_AT_CAP the cap-limited systems of the 512-system workload keep
    refining (restarted GMRES(100) inside IR) and every system reaches the binary64 target."""
    systems = M.batched_convection_diffusion(512, seed=0)
    bs = [M.equal_rhs(s[0]) for s in systems]
    opts = spai_ir.options("mixed", epsilon=0.3, alpha=5, innercap=100, flags=spai_ir.FLAG_RESTART_AT_CAP)
    xs, reps = spai_ir.ir_solve_batched(systems, bs, opts)
    bad = [(i, r["ir_status"], r["outer_steps"]) for i, r in enumerate(reps) if not r["converged"]]
    assert not bad, bad
    assert max(r["backward_error"] for r in reps) <= BE64
