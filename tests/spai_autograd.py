"""Test-side torch.autograd.Function over the library's solve and adjoint (C ABI).

Forward: X = A^{-1} B for the stored values of A (a new handle and SPAI build per call, so a
perturbed A is solved with its own preconditioner). Backward: spai_adjoint solves
A^T Lambda = dL/dX (GMRES right-preconditioned with P^T, the same SPAI without a rebuild) and
returns dL/dB = Lambda and dL/dA on A's pattern. Nothing here computes on the CPU.
"""
import numpy as np
import torch

import spai_ir


class SpaiSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, B, structure, precision, opts):
        n, ptr, idx = structure
        system = (n, ptr, idx, values.detach().cpu().numpy().astype(np.float64))
        Bn = np.asfortranarray(B.detach().cpu().numpy().astype(np.float64))
        h = spai_ir.Handle(system, precision)
        try:
            brep = h.build(opts)
            assert brep["spai_status"] == 0, brep
            X = np.zeros_like(Bn, order="F")
            for r in range(Bn.shape[1]):
                X[:, r], rep = h.solve(Bn[:, r], opts)
                assert rep["converged"], rep
        except BaseException:
            h.close()
            raise
        ctx.handle, ctx.opts, ctx.X = h, opts, X
        return torch.from_numpy(X)

    @staticmethod
    def backward(ctx, gX):
        g = np.asfortranarray(gX.detach().cpu().numpy().astype(np.float64))
        try:
            dB, dA, rep = ctx.handle.adjoint(ctx.X, g, ctx.opts)
        finally:
            ctx.handle.close()
        assert rep["converged"], rep
        ctx.adjoint_report = rep
        return torch.from_numpy(dA), torch.from_numpy(np.asfortranarray(dB)), None, None, None


def solve(values, B, structure, precision, opts):
    return SpaiSolve.apply(values, B, structure, precision, opts)
