"""Layouts of the Krylov SpMVs: sliced ELLPACK over natural or length-sorted rows, and diagonals.

Heavy-tailed row lengths (the irregular Zipf family) build the slices over rows sorted by length
(SELL-C-sigma); stencils may use one dense array per occupied diagonal. Each row is summed by one
thread in column order in every layout, so a GMRES run of a fixed number of steps must give
bit-identical iterates whichever layout the tuner picks (SPAI_SPMV_LAYOUT forces one)."""
import numpy as np
import pytest

import spai_ir
from spai_ir import matrices as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["mixed", "f64"])
def test_sorted_and_natural_slices_agree_bitwise(built, monkeypatch, prec):
    system = M.irregular(20000, seed=3)
    n = system[0]
    rhs = np.random.default_rng(5).standard_normal(n)
    out = {}
    for order in ("0", "1", "-1"):
        monkeypatch.setenv("SPAI_SPMV_LAYOUT", order)
        with spai_ir.Handle(system, prec) as h:
            h.build(spai_ir.options(prec, epsilon=0.4, alpha=5))
            out[order] = h.gmres(rhs, 1e-30, 40)
    for order in ("1", "-1"):
        np.testing.assert_array_equal(out[order][0], out["0"][0])
        assert out[order][1]["iterations"] == out["0"][1]["iterations"] == 40


@pytest.mark.parametrize("prec", ["mixed", "f64"])
def test_diagonal_and_sliced_layouts_agree_bitwise(built, monkeypatch, prec):
    """3-D convection-diffusion: A has 7 diagonals and its SPAI about 19, so the diagonal layout
    is available; fixed-length GMRES iterates and a full refinement solve are bit-identical in
    every layout, and the tuner's choice is reported."""
    system = M.convection_diffusion_3d(20)
    n = system[0]
    rhs = np.random.default_rng(7).standard_normal(n)
    b = M.equal_rhs(n)
    opts = spai_ir.cli_options(n, prec, innercap=120, be_tolerance=1e-12)
    out = {}
    for layout in ("0", "2", "-1"):
        monkeypatch.setenv("SPAI_SPMV_LAYOUT", layout)
        with spai_ir.Handle(system, prec) as h:
            h.build(opts)
            xg, rg = h.gmres(rhs, 1e-30, 30)
            x, r = h.solve(b, opts)
            out[layout] = (xg, rg, x, r, h.tuning())
    assert out["2"][4]["spmv_layout_a"] == 2 and out["2"][4]["spmv_layout_p"] == 2
    assert out["0"][4]["spmv_layout_a"] == 0
    assert out["-1"][4]["spmv_layout_a"] in (0, 1, 2)
    for layout in ("2", "-1"):
        np.testing.assert_array_equal(out[layout][0], out["0"][0])
        np.testing.assert_array_equal(out[layout][2], out["0"][2])
        assert out[layout][3]["inner_iterations"] == out["0"][3]["inner_iterations"]
    assert out["0"][3]["converged"] and out["0"][3]["backward_error"] <= 1e-12
