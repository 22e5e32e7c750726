// GMRES (Arnoldi with classical Gram-Schmidt twice, Givens on the device) and the
// iterative-refinement outer loop, all resident on the device.
//
// Reference path replaced:
//   * CudaCsrSpmv / Matrix::apply (src/cuda_spmv.cu:177-203, src/cuda_gmres.cu:321-336):
//     cuSPARSE CSR_ALG2 plus a memset and a finite-flag round trip per product.
//   * Engine dot/axpy/norm (src/cuda_gmres.cu:238-280): one cuBLAS call and one host sync per
//     modified Gram-Schmidt coefficient, a one-thread LASSQ norm kernel.
//   * solve (src/cuda_gmres.cu:398-522): Givens, Hessenberg and the candidate solve on the host,
//     a candidate formed and verified every iteration.
//   * cuda_refine_with_preconditioner (src/cuda_ir.cpp:31-116): host residual, host update.
// Here every step keeps its scalars on the device: the Hessenberg column, rotations and the
// acceptance decision are computed by the last block of the final orthogonalisation pass, and the
// candidate x0 + V y is formed and verified only when verification is triggered (estimate <= tau,
// breakdown or the cap), which is the binary64 acceptance rule of src/gmres.cpp:238-241.
// Orthogonalisation is CGS2 (two classical passes) instead of one modified pass: same Hessenberg
// in exact arithmetic, O(1) grid synchronisations per step instead of O(k).
// Reductions are deterministic: fixed grid, fixed per-thread row assignment, fixed tree order.
#include "common.cuh"
#include "exact_math.cuh"
#pragma once
#include "krylov.cuh"
#include "cgs_tiles.cuh"
#include "sell.cuh"
#include "dia.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

namespace spai {

inline namespace kdetail {
constexpr int kBlock = 256;

template <class T> __device__ __forceinline__ T block_reduce_sum(T v, T *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0)
        sh[w] = v;
    __syncthreads();
    T r = 0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : T(0);
        for (int o = 16; o > 0; o >>= 1)
            r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r; // valid in thread 0
}
template <class T> __device__ __forceinline__ T block_reduce_max(T v, T *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1)
        v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0)
        sh[w] = v;
    __syncthreads();
    T r = 0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : T(0);
        for (int o = 16; o > 0; o >>= 1)
            r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    }
    return r;
}

// Last-block ticket: returns true in exactly one block, after every block has published.
__device__ __forceinline__ bool last_block(int *counter) {
    __shared__ int is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const int t = atomicAdd(counter, 1);
        is_last = (t == static_cast<int>(gridDim.x) - 1);
        if (is_last)
            *counter = 0; // ready for the next launch
    }
    __syncthreads();
    if (is_last)
        __threadfence();
    return is_last != 0;
}

// Overflow-safe 2-norm partial: (exponent, scaled sum of squares) with a power-of-two scale.
struct NormPart {
    int e;
    double s;
};
template <class T> __device__ __forceinline__ int exp_of(T m) {
    return m > T(0) ? ilogb(m) : INT_MIN;
}

// Resolve a vector that lives at base + index*stride where index is read on the device.
template <class T> struct VecRef {
    T *base;
    long long stride;
    const int *index; // nullptr: offset 0
    int add;          // added to *index
    __device__ __forceinline__ T *get() const {
        return index ? base + static_cast<long long>(*index + add) * stride : base;
    }
};

enum Slot : int {
    kSlotDots = 0,
    kSlotUpdNorm,
    kSlotNormA,
    kSlotNormB,
    kSlotDiag,
    kSlotCand,
    kSlotMisc
};

// ------------------------------------------------------------------------------------------
// SpMV: G lanes per row, row-per-group grid stride; accumulate in the output type.
// ------------------------------------------------------------------------------------------
template <class TA, class TX, class TY, int G>
__global__ void __launch_bounds__(kBlock) spmv_kernel(int n, const int *__restrict__ rp,
                                                      const int *__restrict__ ci,
                                                      const TA *__restrict__ av, VecRef<TX> xr,
                                                      VecRef<TY> yr, const int *gate) {
    if (gate && !*gate)
        return;
    const TX *__restrict__ x = xr.get();
    TY *__restrict__ y = yr.get();
    const int lane = threadIdx.x & (G - 1);
    const int groups = (gridDim.x * blockDim.x) / G;
    // Warp-uniform loop: every lane of a warp runs the same trip count, so the group shuffles
    // always see all 32 lanes.
    const int warp_first = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / G;
    const int sub = (threadIdx.x & 31) / G;
    for (int base = warp_first; base < n; base += groups) {
        const int row = base + sub;
        TY acc = 0;
        if (row < n) {
            const int b = rp[row], e = rp[row + 1];
            for (int t = b + lane; t < e; t += G)
                acc += static_cast<TY>(av[t]) * static_cast<TY>(__ldg(&x[ci[t]]));
        }
        for (int o = G / 2; o > 0; o >>= 1)
            acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (lane == 0 && row < n)
            y[row] = acc;
    }
}

// ------------------------------------------------------------------------------------------
// Norm of a vector (or of a - b) with a last-block finish; result written to *out.
// ------------------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(kBlock) norm_kernel(int n, VecRef<T> ar, const T *bsub,
                                                      NormPart *part, int *counter, T *out,
                                                      const int *gate) {
    if (gate && !*gate)
        return;
    __shared__ T sh[32];
    __shared__ double shd[32];
    const T *a = ar.get();
    const int stride = gridDim.x * blockDim.x;
    T mx = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T v = bsub ? a[i] - bsub[i] : a[i];
        mx = fmax(mx, fabs(v));
    }
    const T bmax = block_reduce_max(mx, sh);
    __shared__ int be;
    if (threadIdx.x == 0)
        be = exp_of(bmax);
    __syncthreads();
    double s = 0;
    if (be != INT_MIN) {
        const T scale = ldexp(T(1), -be);
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const T v = (bsub ? a[i] - bsub[i] : a[i]) * scale;
            s += static_cast<double>(v) * static_cast<double>(v);
        }
    }
    // The per-element scaled square is accumulated in binary64 only here, in a reduction over
    // at most a few thousand elements per thread pair of sweeps; the vector work stays in T.
    const double bs = block_reduce_sum(s, shd);
    if (threadIdx.x == 0)
        part[blockIdx.x] = NormPart{be, bs};
    if (!last_block(counter))
        return;
    if (threadIdx.x == 0) {
        int E = INT_MIN;
        bool nonfinite = false;
        for (int b = 0; b < static_cast<int>(gridDim.x); ++b) {
            E = max(E, part[b].e);
            nonfinite |= !isfinite(part[b].s);
        }
        double S = 0;
        if (E != INT_MIN)
            for (int b = 0; b < static_cast<int>(gridDim.x); ++b)
                if (part[b].e != INT_MIN)
                    S += ldexp(part[b].s, 2 * (part[b].e - E));
        T r = E == INT_MIN ? T(0) : static_cast<T>(ldexp(sqrt(S), E));
        if (nonfinite)
            r = T(INFINITY);
        *out = r;
    }
}
} // namespace kdetail

// Back substitution y = R^{-1} g over `count` columns (src/gmres.cpp:47-55); count = k+1, or k
// when the zero-pivot branch re-verifies the previous candidate. One block, blocked by 32 columns
// from the bottom: warp 0 solves the 32 x 32 diagonal block (lane per row, column sweep), then
// every thread removes the block's contribution from the rows above it (coalesced over R's
// column-major storage). O(count / 32) barriers instead of an O(count^2) serial loop; this runs
// at every step once the recursive estimate has dropped below tau on systems whose recomputed
// residual stays above it.
template <class T>
__global__ void __launch_bounds__(256) solve_y_kernel(Ctl *ctl, const T *H, int hld, const T *g, T *y,
                                                      const T *Ui = nullptr, T *yc = nullptr) {
    if (!ctl->active || !ctl->vgate)
        return;
    const int k = ctl->k;
    const int count = ctl->triggered == 2 ? k : k + 1;
    for (int r = threadIdx.x; r < count; r += blockDim.x)
        y[r] = g[r];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int bad = 0;
    for (int hi = count; hi > 0; hi -= 32) {
        const int lo = hi > 32 ? hi - 32 : 0;
        if (warp == 0) {
            const int row = lo + lane;
            T yr = row < hi ? y[row] : T(0);
            for (int c = hi - 1; c >= lo; --c) {
                const T *hc = H + static_cast<long long>(c) * hld;
                const T yc = __shfl_sync(0xffffffffu, yr, c - lo) / hc[c];
                if (row == c)
                    yr = yc;
                else if (row < c)
                    yr -= hc[row] * yc;
            }
            if (row < hi) {
                y[row] = yr;
                bad |= !isfinite(yr);
            }
        }
        __syncthreads();
        for (int r = threadIdx.x; r < lo; r += blockDim.x) {
            T acc = 0;
            for (int c = lo; c < hi; ++c)
                acc += H[static_cast<long long>(c) * hld + r] * y[c];
            y[r] -= acc;
        }
        __syncthreads();
    }
    bad = __syncthreads_or(bad);
    // Lagged Gram-Schmidt: the candidate combines the stored vectors, V y = S (Ui y).
    if (Ui && !bad)
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            T c = 0;
            for (int j = i; j < count; ++j)
                c += Ui[i + static_cast<long long>(j) * hld] * y[j];
            yc[i] = c;
        }
    if (threadIdx.x == 0) {
        ctl->formed = count;
        if (bad) {
            ctl->status = 8;
            ctl->active = 0;
        }
    }
}

// Acceptance (src/gmres.cpp:235-253): accepted iff verification triggered and the recomputed
// preconditioned residual <= tau; breakdown ends the solve either way; otherwise advance k.
template <class T>
__global__ void decide_kernel(Ctl *ctl, const T *orig, const T *relnum) {
    if (threadIdx.x != 0 || !ctl->active)
        return;
    const int accept_every = ctl->accept_every;
    const bool verified = ctl->vgate != 0;
    ctl->vgate = 0;
    ctl->verifications += verified ? 1 : 0;
    if (verified) {
        const double rel = static_cast<double>(*relnum) / ctl->den;
        ctl->rel = rel;
        ctl->orig = static_cast<double>(*orig);
        // Record mode checks every candidate; only a triggered check decides (gmres.cpp:235-240).
        const bool decides = ctl->triggered != 0 || !ctl->record_every;
        if (ctl->h_iter) {
            const int idx = ctl->h_iter_base + ctl->k;
            if (idx < ctl->h_cap_iter) {
                ctl->h_iter[idx].recomputed_relative = rel;
                ctl->h_iter[idx].accepted = decides && isfinite(rel) && rel <= ctl->tol_inner &&
                                            !(ctl->triggered == 2 && ctl->accept_every);
            }
        }
        if (!isfinite(rel) || !isfinite(ctl->orig)) {
            ctl->status = 8;
            ctl->active = 0;
            return;
        }
        const bool ok = rel <= ctl->tol_inner;
        if (decides && ctl->triggered == 2) { // zero Givens pivot
            ctl->converged = ok && !accept_every;
            ctl->status = ctl->converged ? 0 : 5;
            ctl->active = 0;
            return;
        }
        if (decides && ok) {
            ctl->converged = 1;
            ctl->status = 0;
            ctl->active = 0;
            return;
        }
        if (decides && ctl->breakdown) {
            ctl->status = 5;
            ctl->active = 0;
            return;
        }
    }
    if (ctl->k + 1 >= ctl->cap) {
        ctl->status = ctl->cap < ctl->nrows ? 6 : 7; // iteration_limit / nonconvergence
        ctl->active = 0;
        return;
    }
    // Device-side loop bound: at most cap steps per inner solve and (outer_cap + 1) solves.
    if (++ctl->guard > (ctl->cap + 1) * (ctl->outer_cap + 2)) {
        ctl->status = 8;
        ctl->active = 0;
        ctl->outer_active = 0;
        ctl->ir_status = 6;
        return;
    }
    ctl->k += 1;
    ctl->triggered = 0;
}

// Copies a device flag into a graph conditional handle (loop / branch condition).
__global__ void set_cond_kernel(cudaGraphConditionalHandle h, const int *flag) {
    if (threadIdx.x == 0)
        cudaGraphSetConditional(h, *flag ? 1u : 0u);
}

// ------------------------------------------------------------------------------------------
// GMRES start: r0 = rhs (x0 = 0). Zero RHS -> converged with d = 0. Then Pb, its norm and v0.
// ------------------------------------------------------------------------------------------
template <class T> __global__ void gmres_start_kernel(Ctl *ctl, const T *orig, int accept_every) {
    if (threadIdx.x != 0 || !ctl->outer_active)
        return;
    ctl->k = 0;
    ctl->lag_pending = 0;
    ctl->triggered = 0;
    ctl->breakdown = 0;
    ctl->converged = 0;
    ctl->iterations = 0;
    ctl->formed = 0;
    ctl->active = 1;
    ctl->status = 7;
    ctl->rel = NAN;
    const double r0 = static_cast<double>(*orig);
    ctl->orig = r0;
    if (!isfinite(r0)) {
        ctl->status = 8;
        ctl->active = 0;
        return;
    }
    if (r0 == 0) {
        ctl->status = accept_every ? 2 : 1; // exact_initial_solution (binary32) / zero_rhs
        ctl->converged = 1;
        ctl->active = 0;
        ctl->formed = -1; // correction is exactly zero
    }
}
template <class T>
__global__ void gmres_den_kernel(Ctl *ctl, const T *den, T *g, int accept_every) {
    if (threadIdx.x != 0 || !ctl->active)
        return;
    const double d = static_cast<double>(*den);
    ctl->den = d;
    if (!isfinite(d)) {
        ctl->status = 8;
        ctl->active = 0;
        return;
    }
    if (d == 0) {
        ctl->status = 4; // zero_preconditioned_rhs
        ctl->active = 0;
        return;
    }
    ctl->beta = d;
    if (1.0 <= ctl->tol_inner) { // initial relative residual beta/den = 1
        ctl->status = 0;
        ctl->converged = 1;
        ctl->active = 0;
        ctl->formed = -1;
        return;
    }
    g[0] = static_cast<T>(d);
}
// ------------------------------------------------------------------------------------------
// Iterative refinement in TO (binary64 for F64/MIXED, binary32 for F32).
// ------------------------------------------------------------------------------------------
struct DiagPart {
    double rinf, xinf, cbe, r2;
    int nonfinite;
};

// r = b - A x with the normwise and componentwise backward errors (src/ir.cpp:83-133).
template <class TO, int G>
__global__ void __launch_bounds__(kBlock) ir_residual_kernel(int n, const int *__restrict__ rp,
                                                             const int *__restrict__ ci,
                                                             const TO *__restrict__ av,
                                                             const TO *__restrict__ x,
                                                             const TO *__restrict__ b, TO *r,
                                                             DiagPart *part, Ctl *ctl,
                                                             int *counter) {
    if (!ctl->outer_active)
        return;
    __shared__ double sh[32];
    const int lane = threadIdx.x & (G - 1);
    const int groups = (gridDim.x * blockDim.x) / G;
    double rinf = 0, xinf = 0, cbe = 0, r2 = 0;
    int bad = 0;
    const int warp_first = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / G;
    const int sub = (threadIdx.x & 31) / G;
    for (int base = warp_first; base < n; base += groups) {
        const int row = base + sub;
        TO acc = 0, absacc = 0;
        if (row < n) {
            const int s = rp[row], e = rp[row + 1];
            for (int t = s + lane; t < e; t += G) {
                const TO xv = x[ci[t]];
                acc += av[t] * xv;
                absacc += fabs(av[t]) * fabs(xv);
            }
        }
        for (int o = G / 2; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
            absacc += __shfl_xor_sync(0xffffffffu, absacc, o, G);
        }
        if (lane == 0 && row < n) {
            const TO res = b[row] - acc;
            r[row] = res;
            bad |= !isfinite(res) || !isfinite(absacc);
            rinf = fmax(rinf, static_cast<double>(fabs(res)));
            r2 += static_cast<double>(res) * static_cast<double>(res);
            xinf = fmax(xinf, static_cast<double>(fabs(x[row])));
            const double cden = static_cast<double>(fabs(b[row]) + absacc);
            const double ares = static_cast<double>(fabs(res));
            // Divide only when this row's ratio can exceed the running maximum (the guard errs
            // low by 2^-50, so the result is the maximum of the rounded ratios exactly); the
            // binary64 division is the expensive part of this kernel on GB300's binary64 pipe.
            if (cden == 0)
                cbe = fmax(cbe, res == TO(0) ? 0.0 : INFINITY);
            else if (ares >= cbe * cden * 0.99999999999999911182)
                cbe = fmax(cbe, ares / cden);
        }
    }
    rinf = block_reduce_max(rinf, sh);
    __syncthreads();
    xinf = block_reduce_max(xinf, sh);
    __syncthreads();
    cbe = block_reduce_max(cbe, sh);
    __syncthreads();
    r2 = ctl->h_outer ? block_reduce_sum(r2, sh) : 0.0;
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0)
        part[blockIdx.x] = DiagPart{rinf, xinf, cbe, r2, bad};
    if (!last_block(counter))
        return;
    if (threadIdx.x != 0)
        return;
    double R = 0, X = 0, C = 0, S2 = 0;
    int nonfinite = 0;
    for (int i = 0; i < static_cast<int>(gridDim.x); ++i) {
        R = fmax(R, part[i].rinf);
        X = fmax(X, part[i].xinf);
        C = fmax(C, part[i].cbe);
        S2 += part[i].r2;
        nonfinite |= part[i].nonfinite;
    }
    ctl->rinf = R;
    ctl->xinf = X;
    ctl->cbe = C;
    const TO den = static_cast<TO>(ctl->anorm_inf) * static_cast<TO>(X) + static_cast<TO>(ctl->binf);
    if (nonfinite || !isfinite(den)) {
        ctl->ir_status = 6; // numerical_failure
        ctl->outer_active = 0;
        return;
    }
    const double be = den == TO(0) ? (R == 0 ? 0.0 : INFINITY) : static_cast<double>(static_cast<TO>(R) / den);
    ctl->be = be;
    if (ctl->h_outer) { // IrResult::history entry of this iterate (src/ir.cpp:149-152, 177-183)
        const int idx = ctl->outer_steps;
        if (idx < ctl->h_cap_outer)
            ctl->h_outer[idx] = spai_outer_record{idx, R, sqrt(S2), be, C};
        ctl->h_n_outer = max(ctl->h_n_outer, idx + 1);
    }
    if (be <= ctl->be_tol) {
        ctl->ir_status = 0;
        ctl->outer_active = 0;
        return;
    }
    if (ctl->ir_started && !ctl->changed) {
        ctl->ir_status = 4; // stagnation
        ctl->outer_active = 0;
        return;
    }
    if (ctl->outer_steps >= ctl->outer_cap) {
        ctl->ir_status = 5; // iteration_limit
        ctl->outer_active = 0;
        return;
    }
    // Power-of-two scale for the correction right-hand side (mixed form), exact in binary64.
    ctl->inner_scale = ctl->bscale > 0 ? ldexp(1.0, -ilogb(R)) : 1.0;
    ctl->ir_started = 1;
    ctl->changed = 0;
}

template <class TO, class T>
__global__ void __launch_bounds__(kBlock) make_rhs_kernel(int n, const TO *r, T *rhs, const Ctl *ctl) {
    if (!ctl->outer_active)
        return;
    const TO s = static_cast<TO>(ctl->inner_scale);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        rhs[i] = static_cast<T>(r[i] * s);
}

// x += d (d = correction / scale); records whether any component changed.
template <class TO, class T>
__global__ void __launch_bounds__(kBlock) ir_update_kernel(int n, const TO *x, TO *xn, const T *d,
                                                           Ctl *ctl) {
    if (!ctl->outer_active)
        return;
    __shared__ int any;
    if (threadIdx.x == 0)
        any = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        ctl->pending = 1;
    __syncthreads();
    const bool zero = ctl->formed < 0;
    const TO inv = static_cast<TO>(1.0 / ctl->inner_scale); // exact: power of two
    int changed = 0, bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const TO old = x[i];
        const TO nw = zero ? old : old + static_cast<TO>(d[i]) * inv;
        xn[i] = nw;
        changed |= nw != old;
        bad |= !isfinite(nw);
    }
    if (changed)
        any = 1;
    if (bad)
        atomicOr(&ctl->nonfinite, 1);
    __syncthreads();
    if (threadIdx.x == 0 && any)
        atomicOr(&ctl->changed, 1);
}

// Commit x <- x_new unless the new iterate's diagnostics failed (src/ir.cpp:176-186: a
// converged correction is not committed after failed outer diagnostics).
template <class TO>
__global__ void __launch_bounds__(kBlock) ir_commit_kernel(int n, TO *x, const TO *xn, const Ctl *ctl) {
    if (!ctl->pending || ctl->ir_status == 6)
        return;
    if (blockIdx.x == 0 && threadIdx.x == 0 && ctl->h_inner && ctl->inner_attempts - 1 < ctl->h_cap_inner)
        ctl->h_inner[ctl->inner_attempts - 1].update_applied = 1; // src/ir.cpp:184
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = xn[i];
}

// After an inner solve: failure ends the loop with inner_failure; otherwise count the step.
__global__ void ir_after_inner_kernel(Ctl *ctl) {
    if (threadIdx.x != 0)
        return;
    ctl->pending = 0;
    if (!ctl->outer_active)
        return;
    ctl->inner_attempts += 1;
    ctl->inner_iterations_total += ctl->iterations;
    ctl->last_gmres_status = ctl->status;
    if (ctl->h_inner) { // IrResult::inner_history entry (src/ir.cpp:158-164)
        const int idx = ctl->inner_attempts - 1;
        if (idx < ctl->h_cap_inner)
            ctl->h_inner[idx] = spai_inner_record{ctl->status, 0, ctl->iterations, ctl->rel};
        ctl->h_n_inner = max(ctl->h_n_inner, idx + 1);
        ctl->h_iter_base += ctl->iterations;
    }
    // With SPAI_FLAG_RESTART_AT_CAP a cap-limited solve whose verified candidate reduced the
    // preconditioned residual still supplies the correction (restart from the new residual).
    const bool partial = ctl->accept_partial && ctl->status == 6 && ctl->formed > 0 && ctl->rel < 1.0;
    if (!ctl->converged && !partial) {
        ctl->ir_status = 3; // inner_failure
        ctl->outer_active = 0;
    }
}
__global__ void ir_after_update_kernel(Ctl *ctl) {
    if (threadIdx.x != 0 || !ctl->outer_active)
        return;
    if (ctl->nonfinite) {
        ctl->ir_status = 6;
        ctl->outer_active = 0;
        return;
    }
    ctl->outer_steps += 1;
}

// x0 = P b with P in T and b, x in TO.
template <class T, class TO>
__global__ void __launch_bounds__(kBlock) ir_x0_kernel(int n, const int *__restrict__ rp,
                                                       const int *__restrict__ ci,
                                                       const T *__restrict__ pv,
                                                       const TO *__restrict__ b, TO *x) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        TO acc = 0;
        for (int t = rp[row]; t < rp[row + 1]; ++t)
            acc += static_cast<TO>(pv[t]) * b[ci[t]];
        x[row] = acc;
    }
}

// ||A||_inf and ||b||_inf (constant over the solve).
template <class TO>
__global__ void __launch_bounds__(kBlock) norms_inf_kernel(int n, const int *__restrict__ rp,
                                                           const TO *__restrict__ av,
                                                           const TO *__restrict__ b,
                                                           DiagPart *part, Ctl *ctl, int *counter) {
    __shared__ double sh[32];
    double an = 0, bn = 0;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        TO s = 0;
        for (int t = rp[row]; t < rp[row + 1]; ++t)
            s += fabs(av[t]);
        an = fmax(an, static_cast<double>(s));
        bn = fmax(bn, static_cast<double>(fabs(b[row])));
    }
    an = block_reduce_max(an, sh);
    __syncthreads();
    bn = block_reduce_max(bn, sh);
    if (threadIdx.x == 0)
        part[blockIdx.x] = DiagPart{an, bn, 0, 0};
    if (!last_block(counter))
        return;
    if (threadIdx.x == 0) {
        double A = 0, B = 0;
        for (int i = 0; i < static_cast<int>(gridDim.x); ++i) {
            A = fmax(A, part[i].rinf);
            B = fmax(B, part[i].xinf);
        }
        ctl->anorm_inf = A;
        ctl->binf = B;
    }
}

// ------------------------------------------------------------------------------------------
// Host orchestration.
// ------------------------------------------------------------------------------------------
template <class T> int pick_group(const DeviceCsr<T> &m) {
    const double avg = m.n ? static_cast<double>(m.nnz) / m.n : 1.0;
    if (avg <= 2.5)
        return 2;
    if (avg <= 6)
        return 4;
    if (avg <= 12)
        return 8;
    if (avg <= 24)
        return 16;
    return 32;
}

template <class TA, class TX, class TY>
void launch_spmv(const DeviceCsr<TA> &m, VecRef<TX> x, VecRef<TY> y, const int *gate, int sms,
                 cudaStream_t st) {
    const int G = pick_group(m);
    const long long threads = static_cast<long long>(m.n) * G;
    const unsigned blocks = grid_for(threads, kBlock, sms * 16);
    switch (G) {
    case 2:
        spmv_kernel<TA, TX, TY, 2><<<blocks, kBlock, 0, st>>>(m.n, m.rp, m.ci, m.val, x, y, gate);
        break;
    case 4:
        spmv_kernel<TA, TX, TY, 4><<<blocks, kBlock, 0, st>>>(m.n, m.rp, m.ci, m.val, x, y, gate);
        break;
    case 8:
        spmv_kernel<TA, TX, TY, 8><<<blocks, kBlock, 0, st>>>(m.n, m.rp, m.ci, m.val, x, y, gate);
        break;
    case 16:
        spmv_kernel<TA, TX, TY, 16><<<blocks, kBlock, 0, st>>>(m.n, m.rp, m.ci, m.val, x, y, gate);
        break;
    default:
        spmv_kernel<TA, TX, TY, 32><<<blocks, kBlock, 0, st>>>(m.n, m.rp, m.ci, m.val, x, y, gate);
    }
    SPAI_LAUNCH("spmv_kernel");
}

// Sliced-ELLPACK SpMVs (one warp per 32-row slice) for the Krylov operators.
template <class T>
__global__ void __launch_bounds__(kBlock) sell_spmv_kernel(DeviceSell<T> m, VecRef<T> x, VecRef<T> y,
                                                           const int *gate) {
    if (gate && !*gate)
        return;
    const T *xv = x.get();
    sell_rows(m, [&](int c) { return xv[c]; }, T(1), y.get());
}
// t = s_k A W_k with W_k gathered from the tile-major basis.
template <class T>
__global__ void __launch_bounds__(kBlock) sell_spmv_basis_kernel(DeviceSell<T> m, Basis<T> V, T *y,
                                                                 const Ctl *ctl) {
    constexpr int R = TileGeom<T>::R;
    if (!ctl->active)
        return;
    const int k = ctl->k;
    const T *base = V.base + static_cast<long long>(k) * R;
    const long long tstride = static_cast<long long>(V.cap1) * R;
    sell_rows(m, [&](int c) { return base[(c / R) * tstride + (c % R)]; }, V.scale[k], y);
}
template <class T>
void launch_sell(const DeviceSell<T> &m, VecRef<T> x, VecRef<T> y, const int *gate, int sms, cudaStream_t st) {
    const unsigned blocks = grid_for(static_cast<long long>(m.nslices) * 32, kBlock, sms * 8);
    sell_spmv_kernel<T><<<blocks, kBlock, 0, st>>>(m, x, y, gate);
    SPAI_LAUNCH("sell_spmv_kernel");
}

template <class T> __global__ void fill_kernel(int n, T *x, T v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = v;
}

// Autotuned slice order of a Krylov SpMV operand. With order < 0 (no override) the natural
// layout is built first; when it pads the matrix by more than 5 % (uneven row lengths), the
// length-sorted layout is built too and both are timed on one SpMV each (best of three, CUDA
// events, on a vector of ones), and the faster is kept. Both layouts sum every row in the same
// order, so the choice changes speed only. The discarded layout stays in the arena (the next
// setup of the same shape reuses its buffers).
template <class T>
DeviceSell<T> tuned_sell(DeviceArena &arena, const DeviceCsr<T> &m, int sms, cudaStream_t st, int order) {
    if (order >= 0)
        return build_sell(arena, m, sms, st, order);
    DeviceSell<T> nat = build_sell(arena, m, sms, st, 0);
    SPAI_CUDA(cudaStreamSynchronize(st));
    if (nat.entries * 20 <= static_cast<long long>(m.nnz) * 21 + 20LL * 32 || m.n < 4096)
        return nat;
    DeviceSell<T> srt = build_sell(arena, m, sms, st, 1);
    T *x = arena.alloc<T>(m.n);
    T *y = arena.alloc<T>(m.n);
    fill_kernel<T><<<grid_for(m.n, kBlock, sms * 8), kBlock, 0, st>>>(m.n, x, T(1));
    SPAI_LAUNCH("fill_kernel");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SPAI_CUDA(cudaEventCreate(&e0));
    SPAI_CUDA(cudaEventCreate(&e1));
    auto time_one = [&](const DeviceSell<T> &sm) {
        float best = INFINITY;
        for (int r = 0; r < 3; ++r) {
            SPAI_CUDA(cudaEventRecord(e0, st));
            launch_sell<T>(sm, VecRef<T>{x, 0, nullptr, 0}, VecRef<T>{y, 0, nullptr, 0}, nullptr, sms, st);
            SPAI_CUDA(cudaEventRecord(e1, st));
            SPAI_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            SPAI_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        return best;
    };
    const float t_nat = time_one(nat), t_srt = time_one(srt);
    SPAI_CUDA(cudaEventDestroy(e0));
    SPAI_CUDA(cudaEventDestroy(e1));
    if (std::getenv("SPAI_TRACE"))
        std::fprintf(stderr, "sell tune: n=%d nnz=%d natural %lld entries %.3f ms, sorted %lld entries %.3f ms\n", m.n,
                     m.nnz, nat.entries, t_nat, srt.entries, t_srt);
    return t_srt < t_nat ? srt : nat;
}

// Diagonal-layout SpMVs (stencil-like profiles, dia.cuh); MAXD: diagonals rounded up to 8.
template <class T, int MAXD>
__global__ void __launch_bounds__(kBlock) dia_spmv_kernel(DeviceDia<T> m, VecRef<T> x, VecRef<T> y, const int *gate) {
    if (gate && !*gate)
        return;
    const T *xv = x.get();
    dia_rows<MAXD>(m, [&](int c) { return __ldg(xv + c); }, T(1), y.get());
}
template <class T, int MAXD>
__global__ void __launch_bounds__(kBlock) dia_spmv_basis_kernel(DeviceDia<T> m, Basis<T> V, T *y, const Ctl *ctl) {
    constexpr int R = TileGeom<T>::R;
    if (!ctl->active)
        return;
    const int k = ctl->k;
    const T *base = V.base + static_cast<long long>(k) * R;
    const long long tstride = static_cast<long long>(V.cap1) * R;
    dia_rows<MAXD>(m, [&](int c) { return base[(c / R) * tstride + (c % R)]; }, V.scale[k], y);
}
template <class T, class F> void dia_dispatch(int ndiag, F &&launch) {
    if (ndiag <= 8)
        launch(std::integral_constant<int, 8>{});
    else if (ndiag <= 16)
        launch(std::integral_constant<int, 16>{});
    else if (ndiag <= 24)
        launch(std::integral_constant<int, 24>{});
    else
        launch(std::integral_constant<int, 32>{});
}

// A Krylov SpMV operand in the layout the tuner chose: sliced ELLPACK (natural or length-sorted
// rows) or diagonals.
template <class T> struct KrylovOp {
    DeviceSell<T> sell;
    DeviceDia<T> dia;
    int layout = 0; // 0 sliced, natural rows; 1 sliced, rows sorted by length; 2 diagonals
    // Algorithmic bytes of one SpMV: stored entries (+ indices) and row data, x and y once.
    double bytes(int n, long long nnz) const {
        if (layout == 2)
            return static_cast<double>(dia.ndiag) * n * sizeof(T) + 4.0 * n + 2.0 * n * sizeof(T);
        return static_cast<double>(nnz) * (4 + sizeof(T)) + 4.0 * (n + 1) + 2.0 * n * sizeof(T);
    }
};
template <class T>
void launch_op(const KrylovOp<T> &op, VecRef<T> x, VecRef<T> y, const int *gate, int sms, cudaStream_t st) {
    if (op.layout == 2) {
        dia_dispatch<T>(op.dia.ndiag, [&](auto md) {
            dia_spmv_kernel<T, decltype(md)::value><<<grid_for(op.dia.n, kBlock, sms * 8), kBlock, 0, st>>>(op.dia, x, y, gate);
        });
        SPAI_LAUNCH("dia_spmv_kernel");
        return;
    }
    launch_sell<T>(op.sell, x, y, gate, sms, st);
}
template <class T> void launch_op_basis(const KrylovOp<T> &op, Basis<T> V, T *y, const Ctl *ctl, int sms, cudaStream_t st) {
    if (op.layout == 2) {
        dia_dispatch<T>(op.dia.ndiag, [&](auto md) {
            dia_spmv_basis_kernel<T, decltype(md)::value><<<grid_for(op.dia.n, kBlock, sms * 8), kBlock, 0, st>>>(op.dia, V, y, ctl);
        });
        SPAI_LAUNCH("dia_spmv_basis_kernel");
        return;
    }
    const unsigned blocks = grid_for(static_cast<long long>(op.sell.nslices) * 32, kBlock, sms * 8);
    sell_spmv_basis_kernel<T><<<blocks, kBlock, 0, st>>>(op.sell, V, y, ctl);
    SPAI_LAUNCH("sell_spmv_basis_kernel");
}

// Autotuned layout of a Krylov SpMV operand: the slice order (tuned_sell), then, for profiles
// with at most kDiaMax column offsets whose diagonals move fewer bytes than the slices, the
// diagonal layout, timed against the sliced one on one SpMV each (best of three) and kept when
// faster. Every layout sums each row in CSR order (bit-identical results). layout: -1 tune;
// 0 / 1 / 2 force natural slices / sorted slices / diagonals (when the matrix allows them).
// probe / pctl: time the basis-gather kernel (the Arnoldi step's first SpMV) on this basis
// instead of the plain-vector kernel.
template <class T>
KrylovOp<T> tuned_op(DeviceArena &arena, const DeviceCsr<T> &m, int sms, cudaStream_t st, int layout,
                     const Basis<T> *probe = nullptr, const Ctl *pctl = nullptr) {
    KrylovOp<T> op;
    op.sell = tuned_sell(arena, m, sms, st, layout == 0 || layout == 1 ? layout : -1);
    op.layout = op.sell.sorted() ? 1 : 0;
    if (layout == 0 || layout == 1 || m.n < 4096)
        return op;
    const double sell_bytes = static_cast<double>(op.sell.entries) * (4 + sizeof(T));
    op.dia = build_dia(arena, m, sms, st, layout == 2 ? INFINITY : sell_bytes);
    if (!op.dia.ok())
        return op;
    if (layout == 2) {
        op.layout = 2;
        return op;
    }
    T *x = arena.alloc<T>(m.n);
    T *y = arena.alloc<T>(m.n);
    fill_kernel<T><<<grid_for(m.n, kBlock, sms * 8), kBlock, 0, st>>>(m.n, x, T(1));
    SPAI_LAUNCH("fill_kernel");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SPAI_CUDA(cudaEventCreate(&e0));
    SPAI_CUDA(cudaEventCreate(&e1));
    auto time_one = [&](int lay) {
        KrylovOp<T> o = op;
        o.layout = lay;
        float best = INFINITY;
        for (int r = 0; r < 3; ++r) {
            SPAI_CUDA(cudaEventRecord(e0, st));
            if (probe)
                launch_op_basis<T>(o, *probe, y, pctl, sms, st);
            else
                launch_op<T>(o, VecRef<T>{x, 0, nullptr, 0}, VecRef<T>{y, 0, nullptr, 0}, nullptr, sms, st);
            SPAI_CUDA(cudaEventRecord(e1, st));
            SPAI_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            SPAI_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        return best;
    };
    const float t_sell = time_one(op.layout), t_dia = time_one(2);
    SPAI_CUDA(cudaEventDestroy(e0));
    SPAI_CUDA(cudaEventDestroy(e1));
    if (std::getenv("SPAI_TRACE"))
        std::fprintf(stderr, "spmv tune: n=%d nnz=%d sliced (%s) %.3f ms, %d diagonals %.3f ms\n", m.n, m.nnz,
                     op.layout ? "sorted" : "natural", t_sell, op.dia.ndiag, t_dia);
    if (t_dia < t_sell)
        op.layout = 2;
    return op;
}

// Optional per-kernel-class timing: CUDA events recorded on the solve stream around each
// launch of the Arnoldi kernels. Launch records of speculative steps past the end of a GMRES
// solve are discarded using the solve's iteration count.
enum KernelClass : int { kClsSpmvA = 0, kClsSpmvP, kClsDots, kClsUpdate, kClsNormalize, kClsCount };
struct KernelProfile {
    bool on = false;
    std::vector<cudaEvent_t> ev;
    size_t next = 0;
    struct Rec {
        int cls, k, solve;
        size_t e0, e1;
        double bytes;
    };
    std::vector<Rec> recs;
    std::vector<int> solve_iters;
    double ms[kClsCount] = {0, 0, 0, 0, 0};
    double bytes[kClsCount] = {0, 0, 0, 0, 0};
    long long launches[kClsCount] = {0, 0, 0, 0, 0};
    ~KernelProfile() {
        for (auto e : ev)
            cudaEventDestroy(e);
    }
    size_t mark(cudaStream_t st) {
        if (next == ev.size()) {
            cudaEvent_t e;
            SPAI_CUDA(cudaEventCreate(&e));
            ev.push_back(e);
        }
        SPAI_CUDA(cudaEventRecord(ev[next], st));
        return next++;
    }
    void reset() {
        next = 0;
        recs.clear();
        solve_iters.clear();
        for (int c = 0; c < kClsCount; ++c) {
            ms[c] = 0;
            bytes[c] = 0;
            launches[c] = 0;
        }
    }
    // Accumulate the records of finished solves (all work up to the last event has completed).
    void collect() {
        for (const Rec &r : recs) {
            if (r.solve >= static_cast<int>(solve_iters.size()) || r.k >= solve_iters[r.solve])
                continue;
            float t = 0;
            SPAI_CUDA(cudaEventElapsedTime(&t, ev[r.e0], ev[r.e1]));
            ms[r.cls] += t;
            bytes[r.cls] += r.bytes;
            launches[r.cls] += 1;
        }
        recs.clear();
        next = 0;
    }
};

// Buffers and launch sequence of one refinement solve with inner type T and outer type TO.
template <class T, class TO> struct IrEngine {
    int n = 0, cap = 0, sms = 0;
    long long ld = 0;
    int hld = 0;
    const DeviceCsr<TO> *a_outer = nullptr;
    const DeviceCsr<T> *a_inner = nullptr;
    const DeviceCsr<T> *p = nullptr;
    KrylovOp<T> sa, sp; // SpMV layouts of the inner matrix and of P
    Ctl *ctl = nullptr;
    T *V = nullptr, *sc = nullptr, *w = nullptr, *t = nullptr, *rhs = nullptr, *pb = nullptr, *cand = nullptr,
      *ax = nullptr, *pax = nullptr, *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr,
      *y = nullptr, *h1 = nullptr, *h2 = nullptr, *part = nullptr, *scal = nullptr;
    // Lagged second projection: projections, pending correction, its Hessenberg image and the
    // unrotated Hessenberg (see cgs_tiles.cuh).
    T *dl = nullptr, *fco = nullptr, *ecorr = nullptr, *Hu = nullptr, *Ui = nullptr, *yc = nullptr;
    bool lag = false; // two basis reads per Arnoldi step (every step of the solve streams)
    T *Hraw = nullptr;          // record mode: Hessenberg columns before their rotations
    KrylovRecord *rec = nullptr; // record mode: host record of the running solve
    TO *r = nullptr, *xn = nullptr;
    NormPart *npart = nullptr;
    DiagPart *dpart = nullptr;
    int *counters = nullptr;
    int nblk_vec = 0, nblk_dots = 0, ntiles = 0;
    int stage_segs = 0;   // Gram-Schmidt pipeline stage size (segments)
    size_t cgs_dyn = 0;   // dynamic shared memory of a pass
    void *cgs_dots = nullptr, *cgs_norms = nullptr;
    T *cgs_gacc = nullptr, *cgs_gcf = nullptr; // long caps: accumulators in global memory
    bool always_reorth = false;
    int *pinned_host = nullptr; // host flag for profile-mode reads
    long long launches = 0;
    KernelProfile *prof = nullptr;
    int host_k = 0, solve_index = 0;
    TO *bbuf = nullptr, *xbuf = nullptr; // fixed graph-side copies of b and x
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graph_f32_accept = false;
    bool graph_mode = false;
    // Right preconditioning (adjoint solves): the operator is (inner matrix)·P, GMRES starts from
    // rhs itself, the candidate is d = P·(V y) and its only check is the true residual.
    bool right = false;
    // History buffers (SPAI_FLAG_HISTORY), in their own arena so enabling them never disturbs the
    // solve workspace.
    DeviceArena hist_mem;
    spai_outer_record *hist_outer = nullptr;
    spai_inner_record *hist_inner = nullptr;
    spai_iteration_record *hist_iter = nullptr;
    int hist_cap_outer = 0, hist_cap_inner = 0, hist_cap_iter = 0;
    void arm_history(Ctl &h, const SolveSettings &s) {
        if (!s.history)
            return;
        hist_mem.reset();
        hist_cap_outer = s.outer_cap + 2;
        hist_cap_inner = s.outer_cap + 1;
        hist_cap_iter = static_cast<int>(std::min<long long>(static_cast<long long>(cap) * (s.outer_cap + 1), 1 << 20));
        hist_outer = hist_mem.alloc<spai_outer_record>(hist_cap_outer);
        hist_inner = hist_mem.alloc<spai_inner_record>(hist_cap_inner);
        hist_iter = hist_mem.alloc<spai_iteration_record>(hist_cap_iter);
        h.h_outer = hist_outer;
        h.h_inner = hist_inner;
        h.h_iter = hist_iter;
        h.h_cap_outer = hist_cap_outer;
        h.h_cap_inner = hist_cap_inner;
        h.h_cap_iter = hist_cap_iter;
    }

    // Kernel nodes executed by the last graph solve, from the device loop counters: 4 init
    // nodes; per GMRES solve 8 start nodes (7 with right preconditioning) and 6 update/residual
    // nodes; per Arnoldi step 7 passes (6 with the lagged Gram-Schmidt), 2 condition sets and
    // the decision; per candidate verification 6 (5 with right preconditioning).
    long long graph_kernels(const Ctl &c) const {
        const long long steps = static_cast<long long>(c.guard) + c.inner_attempts;
        return 4 + (right ? 13LL : 14LL) * c.inner_attempts + (lag ? 9LL : 10LL) * steps +
               (right ? 5LL : 6LL) * c.verifications;
    }

    ~IrEngine() {
        release_graph();
    }
    void release_graph() {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }

    // Capture the launches of `f` into graph g after `deps`; returns the new leaf set.
    template <class F>
    std::vector<cudaGraphNode_t> capture_into(cudaStream_t st, cudaGraph_t g,
                                              const std::vector<cudaGraphNode_t> &deps, F &&f) {
        SPAI_CUDA(cudaStreamBeginCaptureToGraph(st, g, deps.empty() ? nullptr : deps.data(), nullptr,
                                                deps.size(), cudaStreamCaptureModeRelaxed));
        f();
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t *d = nullptr;
        size_t nd = 0;
        SPAI_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &d, nullptr, &nd));
        std::vector<cudaGraphNode_t> out(d, d + nd);
        cudaGraph_t tmp = nullptr;
        SPAI_CUDA(cudaStreamEndCapture(st, &tmp));
        return out;
    }
    cudaGraphNode_t add_conditional(cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps,
                                    cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                                    cudaGraph_t *body) {
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = type;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        SPAI_CUDA(cudaGraphAddNode(&node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &p));
        *body = p.conditional.phGraph_out[0];
        return node;
    }

    // The whole refinement solve as one graph: init, then WHILE(outer) { rhs, GMRES start,
    // WHILE(inner) { Arnoldi step, IF(verify) { candidate check }, decide }, update, residual }.
    void build_graph(cudaStream_t st, bool accept_every) {
        release_graph();
        SPAI_CUDA(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle h_outer;
        SPAI_CUDA(cudaGraphConditionalHandleCreate(&h_outer, graph, 0, 0));
        auto d0 = capture_into(st, graph, {}, [&] {
            norms_inf_kernel<TO><<<nblk_vec, kBlock, 0, st>>>(n, a_outer->rp, a_outer->val, bbuf, dpart,
                                                              ctl, counters + kSlotMisc);
            ir_x0_kernel<T, TO><<<nblk_vec, kBlock, 0, st>>>(n, p->rp, p->ci, p->val, bbuf, xbuf);
            residual(st, bbuf, xbuf);
            set_cond_kernel<<<1, 32, 0, st>>>(h_outer, &ctl->outer_active);
        });
        cudaGraph_t body_outer;
        const auto n_outer = add_conditional(graph, d0, h_outer, cudaGraphCondTypeWhile, &body_outer);
        (void)n_outer;
        cudaGraphConditionalHandle h_inner;
        SPAI_CUDA(cudaGraphConditionalHandleCreate(&h_inner, body_outer, 0, 0));
        auto d1 = capture_into(st, body_outer, {}, [&] {
            make_rhs_kernel<TO, T><<<nblk_vec, kBlock, 0, st>>>(n, r, rhs, ctl);
            gmres_start(st, accept_every);
            set_cond_kernel<<<1, 32, 0, st>>>(h_inner, &ctl->active);
        });
        cudaGraph_t body_inner;
        const auto n_inner = add_conditional(body_outer, d1, h_inner, cudaGraphCondTypeWhile, &body_inner);
        cudaGraphConditionalHandle h_verify;
        SPAI_CUDA(cudaGraphConditionalHandleCreate(&h_verify, body_inner, 0, 0));
        auto e1 = capture_into(st, body_inner, {}, [&] {
            arnoldi_passes(st);
            set_cond_kernel<<<1, 32, 0, st>>>(h_verify, &ctl->vgate);
        });
        cudaGraph_t body_verify;
        const auto n_verify = add_conditional(body_inner, e1, h_verify, cudaGraphCondTypeIf, &body_verify);
        capture_into(st, body_verify, {}, [&] { verify_checks(st); });
        capture_into(st, body_inner, {n_verify}, [&] {
            decide_kernel<T><<<1, 32, 0, st>>>(ctl, scal + 0, relnum());
            set_cond_kernel<<<1, 32, 0, st>>>(h_inner, &ctl->active);
        });
        capture_into(st, body_outer, {n_inner}, [&] {
            ir_after_inner_kernel<<<1, 32, 0, st>>>(ctl);
            ir_update_kernel<TO, T><<<nblk_vec, kBlock, 0, st>>>(n, xbuf, xn, cand, ctl);
            ir_after_update_kernel<<<1, 32, 0, st>>>(ctl);
            residual(st, bbuf, xn);
            ir_commit_kernel<TO><<<nblk_vec, kBlock, 0, st>>>(n, xbuf, xn, ctl);
            set_cond_kernel<<<1, 32, 0, st>>>(h_outer, &ctl->outer_active);
        });
        SPAI_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        graph_f32_accept = accept_every;
    }

    // Launch `f` between two profile events when profiling is on.
    template <class F> void timed(cudaStream_t st, int cls, double bytes_, F &&f) {
        if (!prof || !prof->on) {
            f();
            return;
        }
        const size_t e0 = prof->mark(st);
        f();
        const size_t e1 = prof->mark(st);
        prof->recs.push_back(KernelProfile::Rec{cls, host_k, solve_index, e0, e1, bytes_});
    }

    void setup(DeviceArena &arena, const DeviceCsr<TO> &ao, const DeviceCsr<T> &ai,
               const DeviceCsr<T> &pp, int cap_, int sms_, bool right_ = false) {
        right = right_;
        a_outer = &ao;
        a_inner = &ai;
        p = &pp;
        n = ai.n;
        cap = cap_;
        sms = sms_;
        // Vectors are padded to whole basis tiles: the streamed Gram-Schmidt passes read the
        // source vector tile by tile (pad rows of w are zero and never written).
        ld = ((static_cast<long long>(n) + TileGeom<T>::R - 1) / TileGeom<T>::R) * TileGeom<T>::R;
        hld = cap + 2;
        nblk_vec = static_cast<int>(grid_for(n, kBlock, sms * 8));
        constexpr int R = TileGeom<T>::R;
        ntiles = (n + R - 1) / R;
        // One block per SM: the pipeline stages take most of the shared memory, all of it that
        // the largest static footprint of the pass kernels (about 8 KiB) leaves.
        {
            int dev = 0, optin = 0;
            SPAI_CUDA(cudaGetDevice(&dev));
            SPAI_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
            size_t stat = 0;
            cudaFuncAttributes fa{};
            SPAI_CUDA(cudaFuncGetAttributes(&fa, cgs_pass_kernel<T, 1>));
            stat = std::max(stat, fa.sharedSizeBytes);
            SPAI_CUDA(cudaFuncGetAttributes(&fa, cgs_pass_kernel<T, 2>));
            stat = std::max(stat, fa.sharedSizeBytes);
            SPAI_CUDA(cudaFuncGetAttributes(&fa, cgs_pass_kernel<T, 3>));
            stat = std::max(stat, fa.sharedSizeBytes);
            SPAI_CUDA(cudaFuncGetAttributes(&fa, cgs_pass_kernel<T, 4>));
            stat = std::max(stat, fa.sharedSizeBytes);
            SPAI_CUDA(cudaFuncGetAttributes(&fa, cgs_pass_kernel<T, 5>));
            stat = std::max(stat, fa.sharedSizeBytes);
            const size_t budget = static_cast<size_t>(optin) > stat + 1024 ? static_cast<size_t>(optin) - stat - 256 : 0;
            stage_segs = cgs_stage_segs<T>(cap, budget);
        }
        if (stage_segs < 2)
            throw std::runtime_error("Gram-Schmidt staging does not fit in shared memory");
        cgs_dyn = cgs_dyn_smem<T>(cap, stage_segs);
        nblk_dots = std::min(ntiles, sms);
        ctl = arena.alloc<Ctl>(1);
        cudaStream_t setup_st = nullptr;
        // SpMV layout timed per operand (tuned_op); SPAI_SPMV_LAYOUT=0/1/2 forces natural slices,
        // sorted slices or diagonals (equivalence checks and tuning sweeps).
        int layout = -1;
        if (const char *e = std::getenv("SPAI_SPMV_LAYOUT"))
            layout = std::atoi(e);
        const size_t vcount = static_cast<size_t>(ntiles) * (cap + 1) * R;
        {
            size_t free_b = 0, total_b = 0;
            SPAI_CUDA(cudaMemGetInfo(&free_b, &total_b));
            if (vcount * sizeof(T) > free_b) { // cached blocks of earlier handles count as free
                block_cache().release();
                SPAI_CUDA(cudaMemGetInfo(&free_b, &total_b));
            }
            if (vcount * sizeof(T) > free_b)
                throw WorkspaceError("Krylov basis of " + std::to_string(cap + 1) + " vectors of " +
                                     std::to_string(n) + " rows needs " +
                                     std::to_string(vcount * sizeof(T) >> 20) + " MiB, more than the " +
                                     std::to_string(free_b >> 20) + " MiB free on the device; lower innercap");
        }
        V = arena.alloc<T>(vcount);
        SPAI_CUDA(cudaMemset(V, 0, vcount * sizeof(T))); // pad rows of the last tile stay zero
        sc = arena.alloc<T>(cap + 2);
        {
            // The operand that gathers the basis vector is timed in its Arnoldi form (basis
            // gather from this basis; the control block is rewritten at the start of a solve).
            fill_kernel<T><<<1, 256, 0, setup_st>>>(cap + 2, sc, T(1));
            SPAI_LAUNCH("fill_kernel");
            Ctl hc{};
            hc.active = 1;
            hc.k = 0;
            SPAI_CUDA(cudaMemcpyAsync(ctl, &hc, sizeof(Ctl), cudaMemcpyHostToDevice, setup_st));
            const Basis<T> probe{V, cap + 1, ntiles, sc};
            sa = tuned_op(arena, ai, sms, setup_st, layout, right ? nullptr : &probe, ctl);
            sp = tuned_op(arena, pp, sms, setup_st, layout, right ? &probe : nullptr, ctl);
            SPAI_CUDA(cudaStreamSynchronize(setup_st));
        }
        cgs_dots = arena.alloc<T>(static_cast<size_t>(nblk_dots) * (cap + 2));
        cgs_gacc = cgs_gcf = nullptr;
        if (cgs_acc_global<T>(cap)) {
            cgs_gacc = arena.alloc<T>(static_cast<size_t>(nblk_dots) * (cap + 2));
            cgs_gcf = arena.alloc<T>(static_cast<size_t>(nblk_dots) * (cap + 2));
        }
        cgs_norms = arena.alloc<Ssq<T>>(nblk_dots);
        const int smem = static_cast<int>(cgs_dyn);
        SPAI_CUDA(cudaFuncSetAttribute(cgs_pass_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        SPAI_CUDA(cudaFuncSetAttribute(cgs_pass_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        SPAI_CUDA(cudaFuncSetAttribute(cgs_pass_kernel<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        SPAI_CUDA(cudaFuncSetAttribute(cgs_pass_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        SPAI_CUDA(cudaFuncSetAttribute(cgs_pass_kernel<T, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        // The lagged passes need every step to stream whole tiles (k + 2 <= stage_segs for
        // k < cap); SPAI_CGS_LAG=0 keeps the three-pass form (comparisons).
        // (and the packed triangular factors of the finishing blocks fit in the staging region).
        lag = cap + 1 <= stage_segs && !cgs_acc_global<T>(cap) &&
              static_cast<size_t>(cap) * (cap + 3) / 2 * sizeof(T) <= static_cast<size_t>(kCgsStages) * stage_segs * 512;
        if (const char *e = std::getenv("SPAI_CGS_LAG"))
            lag = lag && std::atoi(e) != 0;
        w = arena.alloc<T>(ld);
        SPAI_CUDA(cudaMemset(w, 0, sizeof(T) * ld));
        t = arena.alloc<T>(ld);
        rhs = arena.alloc<T>(ld);
        pb = arena.alloc<T>(ld);
        cand = arena.alloc<T>(ld);
        ax = arena.alloc<T>(ld);
        pax = arena.alloc<T>(ld);
        r = arena.alloc<TO>(ld);
        xn = arena.alloc<TO>(ld);
        bbuf = arena.alloc<TO>(ld);
        xbuf = arena.alloc<TO>(ld);
        release_graph();
        H = arena.alloc<T>(static_cast<size_t>(hld) * (cap + 1));
        cs = arena.alloc<T>(cap + 1);
        sn = arena.alloc<T>(cap + 1);
        g = arena.alloc<T>(cap + 2);
        y = arena.alloc<T>(cap + 1);
        h1 = arena.alloc<T>(cap + 2);
        h2 = arena.alloc<T>(cap + 2);
        dl = arena.alloc<T>(cap + 2);
        fco = arena.alloc<T>(cap + 2);
        ecorr = arena.alloc<T>(cap + 2);
        yc = arena.alloc<T>(cap + 2);
        Hu = arena.alloc<T>(static_cast<size_t>(hld) * (cap + 1));
        Hraw = arena.alloc<T>(static_cast<size_t>(hld) * (cap + 1));
        Ui = arena.alloc<T>(static_cast<size_t>(hld) * (cap + 2));
        part = arena.alloc<T>(static_cast<size_t>(std::max(nblk_dots, nblk_vec)) * (cap + 2));
        npart = arena.alloc<NormPart>(std::max(nblk_dots, nblk_vec));
        dpart = arena.alloc<DiagPart>(std::max(nblk_dots, nblk_vec));
        scal = arena.alloc<T>(8);
        counters = arena.alloc<int>(16);
    }

    VecRef<T> fixed(T *p_) const {
        return VecRef<T>{p_, 0, nullptr, 0};
    }
    Basis<T> basis() const {
        return Basis<T>{V, cap + 1, ntiles, sc};
    }
    CgsArgs<T> cgs_args() const {
        return CgsArgs<T>{n, basis(), w, h1, h2, H, cs, sn, g, sc, hld, ctl,
                          CgsScratch{cgs_dots, cgs_norms, counters + kSlotDots}, always_reorth ? 1 : 0,
                          stage_segs, cgs_gacc, cgs_gcf, dl, fco, ecorr, Hu, Ui};
    }
    size_t cgs_smem() const {
        return cgs_dyn;
    }

    void norm(cudaStream_t st, VecRef<T> a, const T *bsub, T *out, int slot, const int *gate) {
        norm_kernel<T><<<nblk_vec, kBlock, 0, st>>>(n, a, bsub, npart, counters + slot, out, gate);
        SPAI_LAUNCH("norm_kernel");
        ++launches;
    }

    // One Arnoldi step plus (when triggered) candidate verification.
    // Algorithmic bytes of one launch (each stored element read or written once).
    double spmv_bytes(const DeviceCsr<T> &m) const {
        return static_cast<double>(m.nnz) * (4 + sizeof(T)) + 4.0 * (m.n + 1) +
               2.0 * m.n * sizeof(T);
    }
    double vec_bytes(double vectors) const {
        return vectors * static_cast<double>(n) * sizeof(T);
    }

    void arnoldi_step(cudaStream_t st) {
        arnoldi_passes(st);
        verify(st);
        ++host_k;
    }

    // Vector the candidate check compares with (P·rhs, or rhs itself with right preconditioning)
    // and the numerator of the relative residual the decision uses.
    const T *pbv() const {
        return right ? rhs : pb;
    }
    const T *relnum() const {
        return right ? scal + 0 : scal + 1;
    }

    void arnoldi_passes(cudaStream_t st) {
        const double kk = host_k;
        // w = P·(A v) (left) or w = A·(P v) (right): the first matrix gathers the basis vector.
        const DeviceCsr<T> &m1 = right ? *p : *a_inner;
        const DeviceCsr<T> &m2 = right ? *a_inner : *p;
        const KrylovOp<T> &s1 = right ? sp : sa;
        const KrylovOp<T> &s2 = right ? sa : sp;
        timed(st, kClsSpmvA, s1.bytes(m1.n, m1.nnz), [&] { launch_op_basis<T>(s1, basis(), t, ctl, sms, st); });
        timed(st, kClsSpmvP, s2.bytes(m2.n, m2.nnz), [&] { launch_op<T>(s2, fixed(t), fixed(w), &ctl->active, sms, st); });
        const size_t smem = cgs_smem();
        const CgsArgs<T> args = cgs_args();
        if (lag) {
            // Dots (reads W_0..W_k and z), then update and second dots (reads the same, writes
            // W_{k+1}); the second projection stays implicit in the basis' triangular factor.
            timed(st, kClsDots, vec_bytes(kk + 2), [&] {
                cgs_pass_kernel<T, 4><<<nblk_dots, kCgsThreads, smem, st>>>(args);
                SPAI_LAUNCH("cgs_pass_kernel<4>");
            });
            timed(st, kClsUpdate, vec_bytes(kk + 3), [&] {
                cgs_pass_kernel<T, 5><<<nblk_dots, kCgsThreads, smem, st>>>(args);
                SPAI_LAUNCH("cgs_pass_kernel<5>");
            });
            launches += 4;
            return;
        }
        timed(st, kClsDots, vec_bytes(kk + 2), [&] {
            cgs_pass_kernel<T, 1><<<nblk_dots, kCgsThreads, smem, st>>>(args);
            SPAI_LAUNCH("cgs_pass_kernel<1>");
        });
        timed(st, kClsUpdate, vec_bytes(kk + 3), [&] {
            cgs_pass_kernel<T, 2><<<nblk_dots, kCgsThreads, smem, st>>>(args);
            SPAI_LAUNCH("cgs_pass_kernel<2>");
        });
        if (prof && prof->on && pinned_host) {
            // Profile mode only: learn whether the DGKS pass runs, so that only real launches of
            // the third pass are timed (it returns at once otherwise).
            SPAI_CUDA(cudaMemcpyAsync(pinned_host, &ctl->reorth, sizeof(int), cudaMemcpyDeviceToHost, st));
            SPAI_CUDA(cudaStreamSynchronize(st));
            if (!*pinned_host)
                return;
        }
        timed(st, kClsNormalize, vec_bytes(kk + 3), [&] {
            cgs_pass_kernel<T, 3><<<nblk_dots, kCgsThreads, smem, st>>>(args);
            SPAI_LAUNCH("cgs_pass_kernel<3>");
        });
        launches += 5;
    }

    void verify(cudaStream_t st) {
        verify_checks(st);
        decide_kernel<T><<<1, 32, 0, st>>>(ctl, scal + 0, relnum());
        SPAI_LAUNCH("decide_kernel");
        ++launches;
    }

    void verify_checks(cudaStream_t st) {
        solve_y_kernel<T><<<1, 256, 0, st>>>(ctl, H, hld, g, y, lag ? Ui : nullptr, yc);
        SPAI_LAUNCH("solve_y_kernel");
        // Candidate coefficients: y_j s_j on the normalised basis, or Ui y on the stored vectors.
        const T *cy = lag ? yc : y;
        const int unit = lag ? 1 : 0;
        const int *g2 = &ctl->vgate;
        if (right) {
            // d = P·(V y); recomputed residual ||rhs - A d|| (right preconditioning leaves the
            // residual unpreconditioned, so it is also the decision's numerator).
            form_candidate_tiles_kernel<T><<<nblk_vec, kBlock, 0, st>>>(n, basis(), cy, unit, pax, ctl);
            SPAI_LAUNCH("form_candidate_tiles_kernel");
            launch_op<T>(sp, fixed(pax), fixed(cand), g2, sms, st);
            launch_op<T>(sa, fixed(cand), fixed(ax), g2, sms, st);
            norm(st, fixed(rhs), ax, scal + 0, kSlotNormA, g2);
            launches += 3;
            return;
        }
        form_candidate_tiles_kernel<T><<<nblk_vec, kBlock, 0, st>>>(n, basis(), cy, unit, cand, ctl);
        SPAI_LAUNCH("form_candidate_tiles_kernel");
        launch_op<T>(sa, fixed(cand), fixed(ax), g2, sms, st);
        norm(st, fixed(rhs), ax, scal + 0, kSlotNormA, g2);
        launch_op<T>(sp, fixed(ax), fixed(pax), g2, sms, st);
        norm(st, fixed(pb), pax, scal + 1, kSlotNormB, g2);
        launches += 4;
    }

    // GMRES start for the current rhs (x0 = 0): ||rhs||, Pb, ||Pb||, v0 = Pb/||Pb||; with right
    // preconditioning v0 = rhs/||rhs|| and the estimate is relative to ||rhs||.
    void gmres_start(cudaStream_t st, bool accept_every) {
        norm(st, fixed(rhs), nullptr, scal + 2, kSlotNormA, &ctl->outer_active);
        gmres_start_kernel<T><<<1, 32, 0, st>>>(ctl, scal + 2, accept_every ? 1 : 0);
        SPAI_LAUNCH("gmres_start_kernel");
        if (!right) {
            launch_op<T>(sp, fixed(rhs), fixed(pb), &ctl->active, sms, st);
            ++launches;
        }
        norm(st, fixed(const_cast<T *>(pbv())), nullptr, scal + 3, kSlotNormB, &ctl->active);
        gmres_den_kernel<T><<<1, 32, 0, st>>>(ctl, scal + 3, g, accept_every ? 1 : 0);
        SPAI_LAUNCH("gmres_den_kernel");
        basis_start_kernel<T><<<nblk_vec, kBlock, 0, st>>>(n, basis(), pbv(), sc, ctl);
        SPAI_LAUNCH("basis_start_kernel");
        launches += 3;
    }

    int read_flag(cudaStream_t st, int *host_flag, const int *dev_flag) {
        SPAI_CUDA(cudaMemcpyAsync(host_flag, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
        return *host_flag;
    }

    // ---- Record mode: every step's candidate and the solve's basis and Hessenberg, read back ----
    template <class U> std::vector<double> fetch(cudaStream_t st, const U *src, size_t count) {
        std::vector<U> tmp(count);
        if (count)
            SPAI_CUDA(cudaMemcpyAsync(tmp.data(), src, count * sizeof(U), cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
        return std::vector<double>(tmp.begin(), tmp.end());
    }
    Ctl fetch_ctl(cudaStream_t st) {
        Ctl c;
        SPAI_CUDA(cudaMemcpyAsync(&c, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
        return c;
    }
    void arm_record(Ctl &h, const SolveSettings &s) {
        rec = s.record;
        h.record_every = rec ? 1 : 0;
        h.h_raw = rec ? static_cast<void *>(Hraw) : nullptr;
        h.h_raw_ld = hld;
    }
    // After gmres_start: the correction right-hand side and its norm.
    void record_inner_begin(cudaStream_t st) {
        KrylovInner in;
        in.rhs = fetch(st, rhs, n);
        in.initial_original = fetch(st, scal + 2, 1)[0];
        rec->inner.push_back(std::move(in));
    }
    // One step at a time, so that exactly the executed steps are recorded.
    void gmres_loop_record(cudaStream_t st, int *pinned) {
        pinned_host = pinned + 1;
        host_k = 0;
        for (int it = 0; it < cap; ++it) {
            if (!read_flag(st, pinned, &ctl->active))
                break;
            arnoldi_step(st);
            KrylovStep sr;
            sr.candidate = fetch(st, cand, n);
            sr.original = fetch(st, scal + 0, 1)[0];
            rec->inner.back().steps.push_back(std::move(sr));
        }
    }
    // After the inner loop (before the refinement advances the history base): status, norms,
    // the step records, the unrotated Hessenberg and the normalised basis v_j = s_j W_j.
    void record_inner_end(cudaStream_t st) {
        KrylovInner &in = rec->inner.back();
        const Ctl c = fetch_ctl(st);
        in.status = c.status;
        in.converged = c.converged;
        in.iterations = c.iterations;
        in.final_original = c.orig;
        in.final_preconditioned = c.rel;
        const int m = static_cast<int>(in.steps.size());
        in.records.assign(m, spai_iteration_record{});
        if (m > 0 && hist_iter && c.h_iter_base + m <= hist_cap_iter)
            SPAI_CUDA(cudaMemcpyAsync(in.records.data(), hist_iter + c.h_iter_base, sizeof(spai_iteration_record) * m,
                                      cudaMemcpyDeviceToHost, st));
        const std::vector<double> raw = fetch(st, Hraw, static_cast<size_t>(hld) * (cap + 1));
        in.hcap = cap;
        in.hessenberg.assign(static_cast<size_t>(cap + 1) * cap, 0.0);
        for (int k = 0; k < m; ++k)
            for (int r = 0; r <= k + 1; ++r)
                in.hessenberg[static_cast<size_t>(r) * cap + k] = raw[static_cast<size_t>(k) * hld + r];
        // v_0, and v_{k+1} after every step whose subdiagonal is nonzero (gmres.cpp:184-190).
        in.nbasis = m == 0 ? 0 : m + (raw[static_cast<size_t>(m - 1) * hld + m] != 0 ? 1 : 0);
        in.nbasis = std::min(in.nbasis, cap + 1);
        if (in.nbasis > 0) {
            constexpr int R = TileGeom<T>::R;
            const std::vector<double> tiles = fetch(st, V, static_cast<size_t>(ntiles) * (cap + 1) * R);
            const std::vector<double> scl = fetch(st, sc, cap + 2);
            in.basis.assign(static_cast<size_t>(in.nbasis) * n, 0.0);
            for (int j = 0; j < in.nbasis; ++j)
                for (int i = 0; i < n; ++i)
                    in.basis[static_cast<size_t>(j) * n + i] =
                        static_cast<double>(static_cast<T>(scl[j]) *
                                            static_cast<T>(tiles[(static_cast<size_t>(i / R) * (cap + 1) + j) * R + i % R]));
        }
        in.solution = m > 0 ? in.steps.back().candidate : std::vector<double>(n, 0.0);
    }
    void record_state(cudaStream_t st, const TO *x) {
        KrylovState sr;
        sr.x = fetch(st, x, n);
        sr.residual = fetch(st, r, n);
        rec->states.push_back(std::move(sr));
    }
    struct LagOff { // record mode keeps the three-pass form: its basis is explicit
        bool &lag;
        bool saved;
        LagOff(bool &l, bool off) : lag(l), saved(l) {
            if (off)
                lag = false;
        }
        ~LagOff() {
            lag = saved;
        }
    };

    // Inner GMRES loop driven from the host in batches of speculative steps (steps after the
    // solve ends are no-ops gated on ctl->active).
    void gmres_loop(cudaStream_t st, bool accept_every, int *pinned) {
        (void)accept_every;
        if (rec) {
            gmres_loop_record(st, pinned);
            return;
        }
        pinned_host = pinned + 1;
        const int batch = 8;
        host_k = 0;
        for (int it = 0; it < cap; it += batch) {
            for (int s = 0; s < batch && it + s < cap; ++s)
                arnoldi_step(st);
            if (!read_flag(st, pinned, &ctl->active))
                break;
        }
        if (prof && prof->on) {
            SPAI_CUDA(cudaMemcpyAsync(pinned, &ctl->iterations, sizeof(int), cudaMemcpyDeviceToHost, st));
            SPAI_CUDA(cudaStreamSynchronize(st));
            prof->solve_iters.push_back(*pinned);
            ++solve_index;
            prof->collect();
            prof->solve_iters.clear();
            solve_index = 0;
        }
    }

    // One GMRES solve of P A d = P rhs (x0 = 0) on the current contents of `rhs`.
    void gmres_only(cudaStream_t st, const SolveSettings &s, int *pinned) {
        launches = 0;
        Ctl h{};
        h.cap = cap;
        h.outer_cap = 0;
        h.tol_inner = s.tau;
        h.outer_active = 1;
        h.ir_status = -1;
        h.last_gmres_status = -1;
        h.inner_scale = 1.0;
        h.nrows = n;
        h.accept_every = s.accept_every ? 1 : 0;
        if (s.record) { // the step records carry each step's estimate, check and trigger
            SolveSettings hs = s;
            hs.outer_cap = 0;
            hs.history = true;
            arm_history(h, hs);
        }
        arm_record(h, s);
        LagOff lag_off(lag, rec != nullptr);
        SPAI_CUDA(cudaMemcpyAsync(ctl, &h, sizeof(Ctl), cudaMemcpyHostToDevice, st));
        SPAI_CUDA(cudaMemsetAsync(counters, 0, 16 * sizeof(int), st));
        gmres_start(st, s.accept_every);
        if (rec)
            record_inner_begin(st);
        gmres_loop(st, s.accept_every, pinned);
        if (rec)
            record_inner_end(st);
        rec = nullptr;
    }

    // Full refinement solve; b, x are device vectors in TO.
    void solve(cudaStream_t st, const TO *b, TO *x, const SolveSettings &s, int *pinned) {
        launches = 0;
        graph_mode = false;
        Ctl h{};
        h.cap = cap;
        h.outer_cap = s.outer_cap;
        h.tol_inner = s.tau;
        h.be_tol = s.be_tol;
        h.bscale = s.scale_rhs ? 1.0 : 0.0;
        h.outer_active = 1;
        h.ir_status = -1;
        h.last_gmres_status = -1;
        h.inner_scale = 1.0;
        h.nrows = n;
        h.accept_every = s.accept_every ? 1 : 0;
        h.accept_partial = s.restart_at_cap ? 1 : 0;
        arm_history(h, s);
        arm_record(h, s);
        LagOff lag_off(lag, rec != nullptr);
        SPAI_CUDA(cudaMemcpyAsync(ctl, &h, sizeof(Ctl), cudaMemcpyHostToDevice, st));
        SPAI_CUDA(cudaMemsetAsync(counters, 0, 16 * sizeof(int), st));
        if (s.use_graph && !(prof && prof->on) && !rec) {
            if (!exec || graph_f32_accept != s.accept_every)
                build_graph(st, s.accept_every);
            SPAI_CUDA(cudaMemcpyAsync(bbuf, b, sizeof(TO) * n, cudaMemcpyDeviceToDevice, st));
            SPAI_CUDA(cudaGraphLaunch(exec, st));
            SPAI_CUDA(cudaMemcpyAsync(x, xbuf, sizeof(TO) * n, cudaMemcpyDeviceToDevice, st));
            graph_mode = true;
            return;
        }
        norms_inf_kernel<TO><<<nblk_vec, kBlock, 0, st>>>(n, a_outer->rp, a_outer->val, b, dpart,
                                                          ctl, counters + kSlotMisc);
        SPAI_LAUNCH("norms_inf_kernel");
        ir_x0_kernel<T, TO><<<nblk_vec, kBlock, 0, st>>>(n, p->rp, p->ci, p->val, b, x);
        SPAI_LAUNCH("ir_x0_kernel");
        residual(st, b, x);
        launches += 2;
        if (rec)
            record_state(st, x);
        int applied = 0;
        for (int step = 0; step <= s.outer_cap; ++step) {
            if (!read_flag(st, pinned, &ctl->outer_active))
                break;
            make_rhs_kernel<TO, T><<<nblk_vec, kBlock, 0, st>>>(n, r, rhs, ctl);
            SPAI_LAUNCH("make_rhs_kernel");
            gmres_start(st, s.accept_every);
            if (rec)
                record_inner_begin(st);
            gmres_loop(st, s.accept_every, pinned);
            if (rec)
                record_inner_end(st);
            ir_after_inner_kernel<<<1, 32, 0, st>>>(ctl);
            SPAI_LAUNCH("ir_after_inner_kernel");
            ir_update_kernel<TO, T><<<nblk_vec, kBlock, 0, st>>>(n, x, xn, cand, ctl);
            SPAI_LAUNCH("ir_update_kernel");
            ir_after_update_kernel<<<1, 32, 0, st>>>(ctl);
            SPAI_LAUNCH("ir_after_update_kernel");
            residual(st, b, xn);
            ir_commit_kernel<TO><<<nblk_vec, kBlock, 0, st>>>(n, x, xn, ctl);
            SPAI_LAUNCH("ir_commit_kernel");
            launches += 5;
            if (rec) {
                const Ctl c = fetch_ctl(st);
                if (c.outer_steps > applied && c.ir_status != 6) { // a correction was applied
                    applied = c.outer_steps;
                    rec->inner.back().applied = 1;
                    record_state(st, x);
                }
            }
        }
        rec = nullptr;
    }

    void residual(cudaStream_t st, const TO *b, TO *x) {
        const int G = pick_group(*a_outer);
        const unsigned blocks = nblk_vec;
        switch (G) {
        case 2:
            ir_residual_kernel<TO, 2><<<blocks, kBlock, 0, st>>>(n, a_outer->rp, a_outer->ci, a_outer->val, x, b, r, dpart, ctl, counters + kSlotDiag);
            break;
        case 4:
            ir_residual_kernel<TO, 4><<<blocks, kBlock, 0, st>>>(n, a_outer->rp, a_outer->ci, a_outer->val, x, b, r, dpart, ctl, counters + kSlotDiag);
            break;
        case 8:
            ir_residual_kernel<TO, 8><<<blocks, kBlock, 0, st>>>(n, a_outer->rp, a_outer->ci, a_outer->val, x, b, r, dpart, ctl, counters + kSlotDiag);
            break;
        case 16:
            ir_residual_kernel<TO, 16><<<blocks, kBlock, 0, st>>>(n, a_outer->rp, a_outer->ci, a_outer->val, x, b, r, dpart, ctl, counters + kSlotDiag);
            break;
        default:
            ir_residual_kernel<TO, 32><<<blocks, kBlock, 0, st>>>(n, a_outer->rp, a_outer->ci, a_outer->val, x, b, r, dpart, ctl, counters + kSlotDiag);
        }
        SPAI_LAUNCH("ir_residual_kernel");
        ++launches;
    }
};

} // namespace spai
