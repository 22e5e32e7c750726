"""Seeded synthetic systems with the shapes, sizes and value distributions of the benchmark
configurations (no external dataset exists for them). All matrices are returned as canonical CSR
(int64 row offsets, int64 sorted column indices, float64 values, no stored zeros), the layout the
reference's CsrMatrix::from_entries produces (src/cpu.cpp:49-78).

Discretisation choices (not fixed by the configuration text, stated here):
  * convection-diffusion: -nu*Laplace(u) + v.grad(u) on the unit square/cube, Dirichlet boundary
    (boundary nodes eliminated), h = 1/(N+1), first-order upwind convection, cell Peclet number
    Pe = |v|_inf * h / (2 nu); rows are scaled by h^2 so entries are O(nu). Row-major node order
    (x fastest). 2-D nnz = 5N^2 - 4N, 3-D nnz = 7N^3 - 6N^2.
  * irregular: off-diagonal count per row ~ Zipf(s) restricted to [1, 256] (mean ~12 for s=1.5),
    distinct uniform columns,
    N(0,1) values, diagonal = +-1.1 * sum|off-diagonal| with a random sign.
  * anisotropic diffusion: cell-centred 5-point finite volumes of -div(K grad u), K = diag(r*k, k),
    k log-normal with a Gaussian-correlated log field, harmonic face averages, Dirichlet walls.
"""
import numpy as np


def _canonical(n, rows, cols, vals):
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    keep = vals != 0
    rows, cols, vals = rows[keep], cols[keep], vals[keep]
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, rows + 1, 1)
    np.cumsum(ptr, out=ptr)
    return ptr, cols.astype(np.int64), vals.astype(np.float64)


def convection_diffusion_2d(nx, ny=None, velocity=(1.0, 0.5), peclet=10.0):
    """5-point first-order upwind convection-diffusion on an nx x ny interior grid."""
    ny = nx if ny is None else ny
    h = 1.0 / (max(nx, ny) + 1)
    vx, vy = float(velocity[0]), float(velocity[1])
    vinf = max(abs(vx), abs(vy))
    nu = vinf * h / (2.0 * peclet) if peclet > 0 and vinf > 0 else 1.0
    n = nx * ny
    idx = np.arange(n, dtype=np.int64)
    i, j = idx % nx, idx // nx
    # h^2-scaled stencil: diffusion nu*(4, -1 x4), upwind convection h*|v| on the diagonal.
    diag = np.full(n, 4 * nu + h * (abs(vx) + abs(vy)))
    west = -nu - h * max(vx, 0.0)
    east = -nu - h * max(-vx, 0.0)
    south = -nu - h * max(vy, 0.0)
    north = -nu - h * max(-vy, 0.0)
    R, C, V = [idx], [idx], [diag]
    for mask, off, val in ((i > 0, -1, west), (i < nx - 1, 1, east),
                           (j > 0, -nx, south), (j < ny - 1, nx, north)):
        r = idx[mask]
        R.append(r); C.append(r + off); V.append(np.full(r.size, val))
    return (n,) + _canonical(n, np.concatenate(R), np.concatenate(C), np.concatenate(V))


def convection_diffusion_3d(N, velocity=None, peclet=5.0):
    """7-point first-order upwind convection-diffusion on an N^3 interior grid."""
    if velocity is None:
        velocity = (1 / np.sqrt(3),) * 3
    h = 1.0 / (N + 1)
    v = [float(c) for c in velocity]
    vinf = max(abs(c) for c in v)
    nu = vinf * h / (2.0 * peclet)
    n = N ** 3
    idx = np.arange(n, dtype=np.int64)
    i, j, k = idx % N, (idx // N) % N, idx // (N * N)
    diag = np.full(n, 6 * nu + h * sum(abs(c) for c in v))
    R, C, V = [idx], [idx], [diag]
    for axis, (coord, stride) in enumerate(((i, 1), (j, N), (k, N * N))):
        c = v[axis]
        for mask, off, val in ((coord > 0, -stride, -nu - h * max(c, 0.0)),
                               (coord < N - 1, stride, -nu - h * max(-c, 0.0))):
            r = idx[mask]
            R.append(r); C.append(r + off); V.append(np.full(r.size, val))
    return (n,) + _canonical(n, np.concatenate(R), np.concatenate(C), np.concatenate(V))


def irregular(n, seed=0, zipf_s=1.5, max_offdiag=256, diag_factor=1.1):
    """Random nonsymmetric matrix with Zipf-distributed off-diagonal counts."""
    rng = np.random.default_rng(seed)
    # Zipf law restricted to [1, max_offdiag] (renormalised): mean ~12.3 for s=1.5, 256.
    support = np.arange(1, max_offdiag + 1, dtype=np.float64)
    cdf = np.cumsum(support ** -zipf_s)
    cdf /= cdf[-1]
    counts = (np.searchsorted(cdf, rng.random(n), side="right") + 1).astype(np.int64)
    counts = np.minimum(counts, max_offdiag)
    counts = np.minimum(counts, n - 1)
    rows = np.repeat(np.arange(n, dtype=np.int64), counts)
    cols = rng.integers(0, n - 1, rows.size, dtype=np.int64)
    cols = cols + (cols >= rows)  # skip the diagonal
    for _ in range(64):
        key = rows * n + cols
        order = np.argsort(key, kind="stable")
        key_sorted = key[order]
        dup = np.zeros(key.size, dtype=bool)
        dup[order[1:]] = key_sorted[1:] == key_sorted[:-1]
        if not dup.any():
            break
        redraw = rng.integers(0, n - 1, int(dup.sum()), dtype=np.int64)
        cols[dup] = redraw + (redraw >= rows[dup])
    vals = rng.standard_normal(rows.size)
    absum = np.zeros(n)
    np.add.at(absum, rows, np.abs(vals))
    sign = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    diag = sign * diag_factor * absum
    diag[diag == 0] = 1.0
    idx = np.arange(n, dtype=np.int64)
    return (n,) + _canonical(n, np.concatenate([rows, idx]), np.concatenate([cols, idx]),
                             np.concatenate([vals, diag]))


def batched_convection_diffusion(count=512, seed=0, side_range=(32, 256), peclet_range=(0.0, 50.0)):
    """Independent 2-D upwind systems: sides log-uniform, Pe uniform, random unit velocity."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(side_range[0]), np.log(side_range[1])
    out = []
    for _ in range(count):
        nx = int(round(np.exp(rng.uniform(lo, hi))))
        ny = int(round(np.exp(rng.uniform(lo, hi))))
        pe = float(rng.uniform(*peclet_range))
        theta = float(rng.uniform(0, 2 * np.pi))
        out.append(convection_diffusion_2d(nx, ny, (np.cos(theta), np.sin(theta)), pe))
    return out


def _correlated_field(N, seed, sigma=1.0, corr_len=8.0):
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((N, N))
    k = np.fft.fftfreq(N)
    kx, ky = np.meshgrid(k, k, indexing="ij")
    spectrum = np.exp(-0.5 * (2 * np.pi * corr_len) ** 2 * (kx ** 2 + ky ** 2))
    field = np.real(np.fft.ifft2(np.fft.fft2(white) * np.sqrt(spectrum)))
    field *= sigma / max(field.std(), 1e-300)
    return np.exp(field)


def anisotropic_diffusion(N=256, seed=0, sigma=1.0, corr_len=8.0, anisotropy=10.0, field=None):
    """Cell-centred FV diffusion with a log-normal coefficient; returns (n, ptr, idx, val)."""
    kappa = _correlated_field(N, seed, sigma, corr_len) if field is None else field
    kxx, kyy = anisotropy * kappa, kappa
    n = N * N
    idx = np.arange(n, dtype=np.int64)
    i, j = idx % N, idx // N
    K1 = kxx.T.ravel()
    K2 = kyy.T.ravel()
    diag = np.zeros(n)
    R, C, V = [], [], []

    def harm(a, b):
        return 2 * a * b / (a + b)

    for mask, off, K in ((i > 0, -1, K1), (i < N - 1, 1, K1), (j > 0, -N, K2), (j < N - 1, N, K2)):
        r = idx[mask]
        t = harm(K[r], K[r + off])
        R.append(r); C.append(r + off); V.append(-t)
        np.add.at(diag, r, t)
    # Dirichlet walls: half-cell transmissibility 2K.
    for mask, K in ((i == 0, K1), (i == N - 1, K1), (j == 0, K2), (j == N - 1, K2)):
        r = idx[mask]
        np.add.at(diag, r, 2 * K[r])
    R.append(idx); C.append(idx); V.append(diag)
    return (n,) + _canonical(n, np.concatenate(R), np.concatenate(C), np.concatenate(V))


def differentiation_problem(N=256, nrhs=64, seed=0, perturbation=0.1):
    """The differentiation workload: anisotropic diffusion on an N x N grid (log-normal coefficient,
    sigma 1, correlation length 8 cells, anisotropy 10), nrhs N(0,1) right-hand sides (n x nrhs)
    and the system whose solutions are the targets x* (coefficient field multiplied by a second
    seeded log-normal field of log-standard-deviation `perturbation`)."""
    field = _correlated_field(N, seed)
    system = anisotropic_diffusion(N, field=field)
    star = anisotropic_diffusion(N, field=field * _correlated_field(N, seed + 1, sigma=perturbation))
    B = np.random.default_rng(seed + 2).standard_normal((N * N, nrhs))
    return system, np.asfortranarray(B), star


def equal_rhs(n):
    """Equal components with unit 2-norm, the CLI right-hand side (src/solver_main.cpp:94)."""
    return np.full(n, 1.0 / np.sqrt(n))


def dense(system):
    n, ptr, idx, val = system
    d = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(ptr))
    d[rows, idx] = val
    return d


def from_dense(d):
    d = np.asarray(d, dtype=np.float64)
    n = d.shape[0]
    rows, cols = np.nonzero(d)
    return (n,) + _canonical(n, rows.astype(np.int64), cols.astype(np.int64), d[rows, cols])


def write_matrix_market(path, system):
    n, ptr, idx, val = system
    rows = np.repeat(np.arange(n), np.diff(ptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{n} {n} {len(val)}\n")
        for r, c, v in zip(rows.tolist(), idx.tolist(), val.tolist()):
            f.write(f"{r + 1} {c + 1} {v!r}\n")
