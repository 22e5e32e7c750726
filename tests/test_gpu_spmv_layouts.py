"""Sliced-ELLPACK layouts of the Krylov SpMVs.

Heavy-tailed row lengths (the irregular Zipf family) build the slices over rows sorted by length
(SELL-C-sigma); stencils keep the natural order. Each row is summed by one thread in column order
in both layouts, so a GMRES run of a fixed number of steps must give bit-identical iterates with
either layout, and the chosen layout must be the sorted one for the heavy-tailed profile."""
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
        monkeypatch.setenv("SPAI_SELL_ORDER", order)
        with spai_ir.Handle(system, prec) as h:
            h.build(spai_ir.options(prec, epsilon=0.4, alpha=5))
            out[order] = h.gmres(rhs, 1e-30, 40)
    for order in ("1", "-1"):
        np.testing.assert_array_equal(out[order][0], out["0"][0])
        assert out[order][1]["iterations"] == out["0"][1]["iterations"] == 40
