"""Canonical-CSR validation of spai_create and spai_set_preconditioner (the CsrMatrix invariants,
include/bspai/cpu.hpp:17-43): the check runs on the device during the upload and, when it
fails, the host names the first violation, so the messages are those of the row-by-row scan."""
import numpy as np
import pytest

import spai_ir

pytestmark = pytest.mark.gpu

GOOD = (3, np.array([0, 2, 5, 7]), np.array([0, 1, 0, 1, 2, 1, 2]), np.array([4.0, 1, 2, 5, 1, 1, 3]))


def _bad(**change):
    n, ptr, idx, val = (GOOD[0], GOOD[1].copy(), GOOD[2].copy(), GOOD[3].copy())
    if "ptr" in change:
        ptr = np.array(change["ptr"])
    if "idx" in change:
        idx = np.array(change["idx"])
    if "val" in change:
        val = np.array(change["val"], dtype=float)
    return (n, ptr, idx, val)


CASES = [
    (_bad(ptr=[0, 2, 1, 7]), "row offsets must be nondecreasing"),
    (_bad(ptr=[0, 5, 3, 7]), "column indices must be strictly increasing within a row"),
    (_bad(idx=[0, 1, 0, 3, 2, 1, 2]), "column index outside matrix"),
    (_bad(idx=[0, 1, 0, -1, 2, 1, 2]), "column index outside matrix"),
    (_bad(idx=[1, 0, 0, 1, 2, 1, 2]), "column indices must be strictly increasing within a row"),
    (_bad(idx=[0, 1, 0, 1, 1, 1, 2]), "column indices must be strictly increasing within a row"),
    (_bad(val=[4, 1, 2, 0, 1, 1, 3]), "values must be finite and nonzero (canonical CSR)"),
    (_bad(val=[4, 1, 2, 5, np.nan, 1, 3]), "values must be finite and nonzero (canonical CSR)"),
    (_bad(val=[4, 1, 2, 5, 1, 1, np.inf]), "values must be finite and nonzero (canonical CSR)"),
    (_bad(ptr=[0, 2, 5, 6]), "row offsets must run from 0 to nnz"),
]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_create_rejects_noncanonical_csr(built, case, precision):
    system, message = CASES[case]
    with pytest.raises(spai_ir.SpaiError) as e:
        spai_ir.Handle(system, precision)
    assert e.value.code == spai_ir.ERR_ARGUMENT
    assert str(e.value).endswith("spai_create: " + message), str(e.value)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_set_preconditioner_rejects_noncanonical_csr(built, case):
    system, message = CASES[case]
    with spai_ir.Handle(GOOD, "f64") as h:
        with pytest.raises(spai_ir.SpaiError) as e:
            h.set_preconditioner(system)
        assert str(e.value).endswith("spai_set_preconditioner: " + message), str(e.value)
        h.set_preconditioner(GOOD)  # the handle stays usable
        x, rep = h.gmres(np.array([1.0, 2.0, 3.0]), 1e-10, 0)
        assert rep["status"] == 0


def test_valid_csr_accepted_and_solved(built):
    with spai_ir.Handle(GOOD, "f64") as h:
        h.build(spai_ir.options("f64", epsilon=1e-12, alpha=2, beta=8))
        x, rep = h.solve(np.array([2.0, -5.0, 7.0]), spai_ir.options("f64", epsilon=1e-12, alpha=2, beta=8))
    assert rep["converged"]
    np.testing.assert_allclose(x, [1, -2, 3], rtol=1e-13)
