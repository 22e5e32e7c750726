"""Adjoint (spai_adjoint) through the C ABI and the test-side autograd shim.

* The adjoint solves the transposed system: A^T lambda = g to the form's backward-error target,
  on a nonsymmetric convection-diffusion matrix, in every form.
* dL/dA is the sampled outer product -sum_r lambda_r[i] x_r[j] on A's pattern.
* Dense FP64 reference gradient on a 32 x 32 grid (anisotropic diffusion and nonsymmetric
  convection-diffusion): L = 1/2 ||X - X*||^2, dL/dB = A^{-T}(X - X*), dL/dA_ij = -sum_r ...
* Central differences (h = 1e-6, FP64 sparse direct solves on the host as the reference) along
  random directions in (A values, B); the adjoint's directional derivative agrees within 1e-5
  relative. The full differentiation workload (256 x 256, 64 right-hand sides, 32 directions)
  runs in the plain FP64 form: its condition number (~1e8) is beyond what a binary32 inner
  solve can verify to tau = 1e-4.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import spai_ir
from spai_ir import matrices as M

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _csr(system):
    n, ptr, idx, val = system
    return sp.csr_matrix((val, idx, ptr), shape=(n, n))


def _rows(system):
    return np.repeat(np.arange(system[0]), np.diff(system[1]))


def _sampled(system, lam, X):
    rows, cols = _rows(system), system[2]
    return -np.einsum("er,er->e", lam[rows], X[cols])


@pytest.mark.parametrize("prec", ["f64", "mixed", "f32"])
def test_adjoint_solves_the_transposed_system(built, prec):
    system = M.convection_diffusion_2d(32)
    n = system[0]
    A = _csr(system)
    rng = np.random.default_rng(3)
    X = np.asfortranarray(rng.standard_normal((n, 3)))
    G = np.asfortranarray(rng.standard_normal((n, 3)))
    opts = spai_ir.options(prec, epsilon=0.3, alpha=(n + 7) // 8)
    with spai_ir.Handle(system, prec) as h:
        assert h.build(opts)["spai_status"] == 0
        lam, dA, rep = h.adjoint(X, G, opts)
        lam2, dA2, _ = h.adjoint(X, G, opts)  # reuses the transposes and the graph
    assert rep["converged"], rep
    assert rep["inner_attempts"] >= 3
    np.testing.assert_array_equal(lam, lam2)
    np.testing.assert_array_equal(dA, dA2)
    bound = 1e-6 if prec == "f32" else 1e-14
    at_inf = abs(A).sum(axis=0).max()
    for r in range(3):
        res = G[:, r] - A.T @ lam[:, r]
        be = abs(res).max() / (at_inf * abs(lam[:, r]).max() + abs(G[:, r]).max())
        assert be <= bound, (r, be)
    expect = _sampled(system, lam, X)
    assert np.allclose(dA, expect, rtol=1e-12, atol=1e-13 * abs(expect).max())


def _dense_gradient(system, B, Xstar):
    Ad = M.dense(system)
    X = np.linalg.solve(Ad, B)
    lam = np.linalg.solve(Ad.T, X - Xstar)
    return X, lam, _sampled(system, lam, X)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("family", ["anisotropic", "convection"])
def test_adjoint_matches_dense_fp64_gradient_32x32(built, family):
    import spai_autograd

    if family == "anisotropic":
        system, B, star = M.differentiation_problem(32, nrhs=64, seed=11)
    else:
        system = M.convection_diffusion_2d(32, velocity=(0.8, -0.6), peclet=20.0)
        star = M.convection_diffusion_2d(32, velocity=(0.6, -0.8), peclet=20.0)
        B = np.asfortranarray(np.random.default_rng(12).standard_normal((system[0], 64)))
    n, ptr, idx, val = system
    Xstar = np.linalg.solve(M.dense(star), B)
    X_ref, gB_ref, gA_ref = _dense_gradient(system, B, Xstar)
    opts = spai_ir.options("f64", epsilon=0.3, alpha=(n + 7) // 8)
    values = torch.tensor(val, dtype=torch.float64, requires_grad=True)
    Bt = torch.tensor(B, dtype=torch.float64, requires_grad=True)
    X = spai_autograd.solve(values, Bt, (n, ptr, idx), "f64", opts)
    assert _rel(X.detach().numpy(), X_ref) <= 1e-10
    L = 0.5 * ((X - torch.from_numpy(Xstar)) ** 2).sum()
    L.backward()
    assert _rel(Bt.grad.numpy(), gB_ref) <= 1e-9
    assert _rel(values.grad.numpy(), gA_ref) <= 1e-9


def _loss_direct(system, values, B, Xstar):
    n, ptr, idx, _ = system
    lu = spla.splu(sp.csc_matrix(sp.csr_matrix((values, idx, ptr), shape=(n, n))))
    X = lu.solve(np.ascontiguousarray(B))
    return 0.5 * np.sum((X - Xstar) ** 2)


def _fd_check(N, nrhs, ndir, prec, innercap, seed=0):
    import spai_autograd

    system, B, star = M.differentiation_problem(N, nrhs=nrhs, seed=seed)
    n, ptr, idx, val = system
    Xstar = spla.splu(sp.csc_matrix(_csr(star))).solve(np.ascontiguousarray(B))
    opts = spai_ir.options(prec, epsilon=0.3, alpha=5, innercap=innercap)
    values = torch.tensor(val, dtype=torch.float64, requires_grad=True)
    Bt = torch.tensor(B, dtype=torch.float64, requires_grad=True)
    X = spai_autograd.solve(values, Bt, (n, ptr, idx), prec, opts)
    L = 0.5 * ((X - torch.from_numpy(Xstar)) ** 2).sum()
    L.backward()
    gA, gB = values.grad.numpy(), Bt.grad.numpy()
    # Binary64 sparse-direct reference gradient (the dense reference at this size).
    lu = spla.splu(sp.csc_matrix(_csr(system)))
    X_ref = lu.solve(np.ascontiguousarray(B))
    lam_ref = lu.solve(X_ref - Xstar, trans="T")
    assert _rel(gB, lam_ref) <= 1e-6
    assert _rel(gA, _sampled(system, lam_ref, X_ref)) <= 1e-6
    rng = np.random.default_rng(seed + 100)
    h = 1e-6
    worst = 0.0
    for d in range(ndir):
        # Alternate directions in A's values and in B, so that each gradient is checked on its
        # own. A directions perturb every stored value by a random multiple of 1e-3 of itself:
        # with kappa(A) ~ 1e8, a relative step of h alone would move the smallest eigenvalue by
        # about its own size and the central difference would leave the linear regime.
        if d % 2 == 0:
            dv = 1e-3 * val * rng.standard_normal(len(val))
            dB = np.zeros_like(B)
        else:
            dv = np.zeros_like(val)
            dB = rng.standard_normal(B.shape)
        fd = (_loss_direct(system, val + h * dv, B + h * dB, Xstar) -
              _loss_direct(system, val - h * dv, B - h * dB, Xstar)) / (2 * h)
        ad = float(np.dot(gA, dv) + np.sum(gB * dB))
        worst = max(worst, abs(fd - ad) / abs(ad))
    return worst


def test_adjoint_central_differences_small(built):
    assert _fd_check(32, nrhs=8, ndir=8, prec="f64", innercap=0) <= 1e-5


def test_adjoint_central_differences_differentiation_workload(built):
    """256 x 256 anisotropic diffusion, 64 right-hand sides, 32 random directions."""
    assert _fd_check(256, nrhs=64, ndir=32, prec="f64", innercap=4000) <= 1e-5
