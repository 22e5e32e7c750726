"""Autotuner: the SPAI's first workspace tier (lanes per column group, workspace per group) is
chosen by timing candidates on a column sample, and the Krylov SpMVs' slice order by timing one
SpMV per layout. Fits and row sums are deterministic, so whatever the tuner picks, the
preconditioner and the solve are bit-identical to the untuned defaults; the tests check that, and
that the choices are reported."""
import numpy as np
import pytest

import spai_ir
from spai_ir import matrices as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "f64"])
def test_spai_first_tier_tuning_changes_speed_only(built, monkeypatch, precision):
    system = M.convection_diffusion_3d(48)  # n = 110,592: large enough to be tuned
    n = system[0]
    opts = spai_ir.cli_options(n, precision)
    out = {}
    for tune in ("1", "0"):
        monkeypatch.setenv("SPAI_TUNE", tune)
        with spai_ir.Handle(system, precision) as h:
            rep = h.build(opts)
            out[tune] = (rep, h.preconditioner(), h.columns(), h.tuning())
    (r1, p1, c1, t1), (r0, p0, c0, t0) = out["1"], out["0"]
    assert r1["spai_status"] == r0["spai_status"] == 0
    for a, b in zip(p1[1:], p0[1:]):
        assert np.array_equal(a, b)
    assert np.array_equal(c1["fits"], c0["fits"])
    assert t1["spai_tuned"] and not t0["spai_tuned"]
    assert t1["group_lanes"] in (4, 8, 16, 32) and t1["ws_bytes"] > 0
    assert t1["sample_ms"] <= t1["default_sample_ms"]  # the default is one of the candidates
    assert np.isnan(t0["sample_ms"])


def test_small_systems_keep_the_default(built):
    system = M.convection_diffusion_2d(64)  # n = 4,096: below the tuning threshold
    with spai_ir.Handle(system, "mixed") as h:
        h.build(spai_ir.cli_options(system[0], "mixed"))
        t = h.tuning()
    assert not t["spai_tuned"] and t["group_lanes"] == 8 and t["ws_bytes"] == 5120
    assert t["spmv_layout_a"] == -1  # no solve set up yet


def test_spmv_slice_order_tuning_changes_speed_only(built, monkeypatch):
    system = M.irregular(100_000, seed=2)
    n = system[0]
    b = M.equal_rhs(n)
    opts = spai_ir.cli_options(n, "mixed", epsilon=0.4, innercap=150, be_tolerance=1e-12)
    res = {}
    for order in (None, "0"):
        if order is None:
            monkeypatch.delenv("SPAI_SPMV_LAYOUT", raising=False)
        else:
            monkeypatch.setenv("SPAI_SPMV_LAYOUT", order)
        with spai_ir.Handle(system, "mixed") as h:
            h.build(opts)
            x, rep = h.solve(b, opts)
            res[order] = (x, rep, h.tuning())
    (xt, rt, tt), (x0, r0, t0) = res[None], res["0"]
    assert rt["converged"] and r0["converged"]
    assert rt["inner_iterations"] == r0["inner_iterations"]
    np.testing.assert_array_equal(xt, x0)
    assert tt["spmv_layout_a"] in (0, 1, 2) and tt["spmv_layout_p"] in (0, 1, 2)
    assert t0["spmv_layout_a"] == 0 and t0["spmv_layout_p"] == 0
