"""spai_backward_error_noalloc: the allocation-free backward-error query.

It exists for callers that cannot call cudaMalloc where they need this check (their device memory
belongs to their own pool allocator, or an allocation's implicit synchronisation is too costly on
their path). The test calls it through the C ABI twice in a row on the solution returned by the
regular solve and compares each result with the backward errors that spai_solve reports for the
same x, within the tolerance used for the solve diagnostics elsewhere (1e-12 relative). It also
checks the documented size limit. This file is collected last (name order) so a failure here
stops a -x run only after every other test has run.
"""
import numpy as np
import pytest

import spai_ir
from spai_ir import matrices as M

pytestmark = pytest.mark.gpu

REL = 1e-12


def test_noalloc_backward_error_matches_solve_report(built):
    import torch

    system = M.convection_diffusion_2d(64)
    n = system[0]
    b = M.equal_rhs(n)
    opts = spai_ir.cli_options(n, "f64")
    with spai_ir.Handle(system, "f64") as h:
        h.build(opts)
        x, rep = h.solve(b, opts)
        assert rep["converged"]
        db = torch.from_numpy(b).cuda()
        dx = torch.from_numpy(x).cuda()
        out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        expected = np.array([rep["backward_error"], rep["componentwise_backward_error"], rep["residual_inf"]])
        for _ in range(2):  # two calls in a row share (and reuse) the static scratch
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            h.backward_error_noalloc(db.data_ptr(), dx.data_ptr(), out.data_ptr())
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.all(np.isfinite(got))
            assert np.allclose(got, expected, rtol=REL, atol=0), (got, expected)


@pytest.mark.parametrize("precision", ["mixed"])
def test_noalloc_mixed_handle_on_a_caller_stream(built, precision):
    """A mixed-precision handle (binary64 A kept beside the binary32 copy) and a call on a stream
    the caller owns, compared with that solve's reported backward errors."""
    import torch

    system = M.convection_diffusion_2d(48)
    n = system[0]
    b = M.equal_rhs(n)
    opts = spai_ir.cli_options(n, precision)
    with spai_ir.Handle(system, precision) as h:
        h.build(opts)
        x, rep = h.solve(b, opts)
        assert rep["converged"]
        db = torch.from_numpy(b).cuda()
        dx = torch.from_numpy(x).cuda()
        out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        side = torch.cuda.Stream()
        expected = np.array([rep["backward_error"], rep["componentwise_backward_error"], rep["residual_inf"]])
        for _ in range(2):
            h.backward_error_noalloc(db.data_ptr(), dx.data_ptr(), out.data_ptr(), side.cuda_stream)
            side.synchronize()
            got = out.cpu().numpy()
            assert np.allclose(got, expected, rtol=REL, atol=0), (got, expected)


def test_noalloc_nonfinite_x_gives_nan(built):
    """A non-finite x gives SPAI_OK with a NaN normwise backward error (the documented signal)."""
    import torch

    system = M.convection_diffusion_2d(16)
    n = system[0]
    with spai_ir.Handle(system, "f64") as h:
        db = torch.from_numpy(M.equal_rhs(n)).cuda()
        dx = torch.ones(n, dtype=torch.float64, device="cuda")
        dx[5] = float("nan")
        out = torch.zeros(3, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        h.backward_error_noalloc(db.data_ptr(), dx.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        assert np.isnan(out.cpu().numpy()[0])


def test_noalloc_rejects_systems_beyond_the_scratch_limit(built):
    import torch

    system = M.convection_diffusion_3d(81)  # n = 531441 > 524288 rows of static scratch
    with spai_ir.Handle(system, "f64") as h:
        v = torch.zeros(system[0], dtype=torch.float64, device="cuda")
        out = torch.zeros(3, dtype=torch.float64, device="cuda")
        with pytest.raises(spai_ir.SpaiError) as e:
            h.backward_error_noalloc(v.data_ptr(), v.data_ptr(), out.data_ptr())
        assert e.value.code == spai_ir.ERR_ARGUMENT
        assert "524288" in str(e.value)
