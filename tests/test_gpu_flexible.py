"""Right-preconditioned inner GMRES (SPAI_FLAG_RIGHT_PRECONDITIONING).

Flexible GMRES builds x = x0 + Z y with z_j = M_j v_j; with this solver's one fixed SPAI every
M_j is P, so it is right-preconditioned GMRES on A P u = r with d = P u. The refinement with it
must reach the forms' backward-error targets and the same solution as the reference's
left-preconditioned inner solve, and its CUDA-graph and host-driven loops must agree bit for bit.
"""
import numpy as np
import pytest

import spai_ir
from spai_ir import matrices as M

pytestmark = pytest.mark.gpu

TARGET = {"f64": 10 * 2.0 ** -53, "mixed": 10 * 2.0 ** -53, "f32": 10 * 2.0 ** -24}


@pytest.mark.parametrize("prec", ["f64", "mixed", "f32"])
@pytest.mark.parametrize("name", ["cd2d_32", "irregular_3000"])
def test_right_preconditioned_refinement(built, prec, name):
    system = M.convection_diffusion_2d(32) if name == "cd2d_32" else M.irregular(3000, seed=4)
    n = system[0]
    b = M.equal_rhs(n)
    left = spai_ir.cli_options(n, prec)
    right = spai_ir.cli_options(n, prec, flags=spai_ir.FLAG_RIGHT_PRECONDITIONING)
    host = spai_ir.cli_options(n, prec, flags=spai_ir.FLAG_RIGHT_PRECONDITIONING | spai_ir.FLAG_NO_GRAPH)
    with spai_ir.Handle(system, prec) as h:
        h.build(left)
        xl, rl = h.solve(b, left)
        xr, rr = h.solve(b, right)
        xh, rh = h.solve(b, host)
        xl2, rl2 = h.solve(b, left)  # switching back restores the left form exactly
    assert rl["converged"] and rr["converged"], (rl, rr)
    assert rr["backward_error"] <= TARGET[prec]
    np.testing.assert_array_equal(xr, xh)
    assert rr["inner_iterations"] == rh["inner_iterations"]
    np.testing.assert_array_equal(xl, xl2)
    scale = np.abs(xl).max()
    np.testing.assert_allclose(xr, xl, rtol=0, atol=(1e-4 if prec == "f32" else 1e-10) * scale)
