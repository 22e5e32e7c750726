// Batched SPAI-GMRES-IR (spai_ir_solve_batched): many independent systems of different sizes.
//
// The SPAI of all systems is one build over their block-diagonal union (columns are independent
// and every shadow/candidate set stays inside its block, so each block equals the system's own
// SPAI). The refinement solves then run in ONE persistent launch: each CTA takes a whole system
// from a largest-first queue and runs its complete mixed-precision refinement — x0 = P b, the
// binary64 residual and backward errors, the binary32 GMRES with SpMVs, tiled classical
// Gram-Schmidt with the DGKS second pass, Givens rotations, candidate checks, and the outer loop —
// synchronising only within the block. No system waits on another.
//
// Semantics follow the single-system solve (src/ir.cpp:138-204, src/gmres.cpp:108-262 with the
// binary64 acceptance rule): statuses, precedence, stagnation, inner failure, uncommitted updates
// after failed diagnostics, exact zero right-hand sides. Summation orders differ from the
// single-system kernels (block-local trees), so results agree to rounding, not bit for bit.
#include "exact_math.cuh"
#include "spai_internal.hpp"
#include "spai_ir.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

namespace spai_api {
std::string canonical_error(const spai_csr *a);
void clear_report(spai_report *r);
double inner_tau(const spai_options &o);
double be_tol(const spai_options &o);
} // namespace spai_api

namespace spai {
inline namespace batched_detail {

constexpr int kBT = 1024;      // threads per CTA (one CTA per SM)
constexpr int kBW = kBT / 32;  // warps per CTA
constexpr int kTR = 128;       // rows per basis tile (one float4 per lane)
constexpr unsigned kFull = 0xffffffffu;

struct BatchSys {
    int row0;       // first row in the block-diagonal union
    int n;          // rows
    int ntiles;     // ceil(n / kTR)
    int cap;        // GMRES basis capacity
    long long pad0; // first element of the system's padded vectors (multiple of kTR)
    long long vbase;// first element of its basis slab: ntiles * (cap + 1) * kTR floats
    int skip;       // 1: not solved (construction failure or invalid input), status preset
    int preset;     // IR status when skipped
};

struct BatchOut {
    int ir_status, converged, outer_steps, inner_attempts, inner_iterations, gmres_status,
        verifications, reorth;
    double be, cbe, rinf;
};

struct BatchArgs {
    int count, outer_cap;
    double tau, be_tol;
    const int *order;
    int *queue;
    const BatchSys *sys;
    const int *arp, *aci;
    const double *a64;
    const float *a32;
    const int *prp, *pci;
    const float *pv;
    int ga, gp; // lanes per row for A and P
    int restart; // SPAI_FLAG_RESTART_AT_CAP
    const double *b;
    double *x, *r, *xn;
    float *w, *t, *rhs, *pb, *cand, *ax;
    float *V;
    float *H; // per CTA: (hcap + 1) columns of (hcap + 2)
    int hcap;
    BatchOut *out;
};

// Per-CTA solve state (shared memory; thread 0 decides, everyone reads after a barrier).
struct St {
    // GMRES
    int k, active, status, converged, triggered, breakdown, iterations, formed, vgate, reorth;
    int verifications, reorth_count;
    double den, orig, wnorm, hnext, rel;
    // refinement
    int ir_status, outer_active, outer_steps, inner_attempts, inner_total, last_gmres, ir_started,
        changed, nonfinite;
    double inner_scale, anorm, binf, be, cbe, rinf, xinf;
};

__device__ __forceinline__ int lane_id() {
    return threadIdx.x & 31;
}

// Fixed-order block sum / max / or (every thread gets the result).
__device__ double cta_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(kFull, v, o);
    __syncthreads();
    if (lane_id() == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int i = 0; i < kBW; ++i)
        s += red[i];
    return s;
}
__device__ double cta_max(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1)
        v = fmax(v, __shfl_xor_sync(kFull, v, o));
    __syncthreads();
    if (lane_id() == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int i = 0; i < kBW; ++i)
        s = fmax(s, red[i]);
    return s;
}

// 32 partial sums per lane -> lane l holds the warp total of entry l (31 shuffles, fixed tree).
__device__ __forceinline__ float reduce_scatter32(float (&p)[32]) {
    const int lane = lane_id();
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        const bool up = (lane & m) != 0;
#pragma unroll
        for (int i = 0; i < m; ++i) {
            const float send = up ? p[i] : p[i + m];
            const float keep = up ? p[i + m] : p[i];
            p[i] = keep + __shfl_xor_sync(kFull, send, m);
        }
    }
    return p[0];
}

__device__ __forceinline__ float dot4(float4 a, float4 b) {
    return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}
__device__ __forceinline__ double sq4(float4 a) {
    return static_cast<double>(a.x) * a.x + static_cast<double>(a.y) * a.y +
           static_cast<double>(a.z) * a.z + static_cast<double>(a.w) * a.w;
}

// y[row] = scale * sum_e av[e] x(ci[e] - row0) over the system's rows, G lanes per row.
template <class XF>
__device__ void cta_spmv(int n, int row0, int G, const int *__restrict__ rp, const int *__restrict__ ci,
                         const float *__restrict__ av, XF xget, float scale, float *__restrict__ y) {
    const int lane = threadIdx.x & (G - 1);
    const int rpw = 32 / G;
    const int sub = (threadIdx.x & 31) / G;
    for (int base = (threadIdx.x >> 5) * rpw; base < n; base += kBW * rpw) {
        const int row = base + sub;
        float acc = 0;
        if (row < n) {
            const int gr = row0 + row;
            const int e1 = rp[gr + 1];
            for (int e = rp[gr] + lane; e < e1; e += G)
                acc += av[e] * xget(ci[e] - row0);
        }
        for (int o = G / 2; o > 0; o >>= 1)
            acc += __shfl_xor_sync(kFull, acc, o, G);
        if (lane == 0 && row < n)
            y[row] = acc * scale;
    }
}

// ||a - b|| (b may be null) of binary32 vectors, squares accumulated in binary64.
__device__ float cta_norm(int n, const float *a, const float *b, double *red, bool &nonfinite) {
    double s = 0;
    int bad = 0;
    for (int i = threadIdx.x; i < n; i += kBT) {
        const float v = b ? a[i] - b[i] : a[i];
        bad |= !isfinite(v);
        s += static_cast<double>(v) * v;
    }
    nonfinite = __syncthreads_or(bad) != 0;
    const double tot = cta_sum(s, red);
    return static_cast<float>(sqrt(tot));
}

struct Smem {
    float *acc;  // [kBW][cs] per-warp dot accumulators
    float *h1, *h2, *cf, *sc, *col, *cs, *sn, *g, *y; // [cs] each
    int cs_len;
};

// One tiled Gram-Schmidt pass over the system's basis (warp per tile, one float4 per lane):
// MODE 1: dots of w with W_0..W_k and ||w||^2;
// MODE 2: w' = w - sum cf_j W_j stored as W_{k+1}, ||w'||^2 and dots of w';
// MODE 3: W_{k+1} -= sum cf_j W_j and its ||.||^2.
template <int MODE>
__device__ double tile_pass(const float *__restrict__ w, float *__restrict__ V, int ntiles, int cap1,
                            int k, const Smem &sm, bool &bad) {
    const int lane = lane_id(), warp = threadIdx.x >> 5;
    const int kk = k + 1;
    float *accw = sm.acc + warp * sm.cs_len;
    double sq = 0;
    int nf = 0;
    for (int t = warp; t < ntiles; t += kBW) {
        const float *tile = V + static_cast<long long>(t) * cap1 * kTR + lane * 4;
        float4 wv = MODE == 3 ? *reinterpret_cast<const float4 *>(tile + static_cast<long long>(kk) * kTR)
                              : *reinterpret_cast<const float4 *>(w + t * kTR + lane * 4);
        if (MODE >= 2) {
            int j = 0;
            for (; j + 8 <= kk; j += 8) { // eight segment loads in flight per lane
                float4 v[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    v[q] = *reinterpret_cast<const float4 *>(tile + static_cast<long long>(j + q) * kTR);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float c = sm.cf[j + q];
                    wv.x -= c * v[q].x;
                    wv.y -= c * v[q].y;
                    wv.z -= c * v[q].z;
                    wv.w -= c * v[q].w;
                }
            }
            for (; j < kk; ++j) {
                const float4 v = *reinterpret_cast<const float4 *>(tile + static_cast<long long>(j) * kTR);
                const float c = sm.cf[j];
                wv.x -= c * v.x;
                wv.y -= c * v.y;
                wv.z -= c * v.z;
                wv.w -= c * v.w;
            }
            *reinterpret_cast<float4 *>(const_cast<float *>(tile) + static_cast<long long>(kk) * kTR) = wv;
        }
        nf |= !isfinite(wv.x) || !isfinite(wv.y) || !isfinite(wv.z) || !isfinite(wv.w);
        sq += sq4(wv);
        if (MODE <= 2) {
            for (int c0 = 0; c0 < kk; c0 += 32) {
                float p[32];
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) {
                    const int j = c0 + jj;
                    p[jj] = j < kk ? dot4(*reinterpret_cast<const float4 *>(tile + static_cast<long long>(j) * kTR), wv)
                                   : 0.f;
                }
                const float s = reduce_scatter32(p);
                if (c0 + lane < kk)
                    accw[c0 + lane] += s;
            }
        }
    }
    bad = bad || __syncthreads_or(nf);
    return sq;
}

// Per-warp accumulators -> h[j] = s_j * sum over warps (fixed order), then clear them.
__device__ void combine_dots(int kk, const Smem &sm, float *h) {
    __syncthreads();
    for (int j = threadIdx.x; j < kk; j += kBT) {
        float s = 0;
        for (int wq = 0; wq < kBW; ++wq)
            s += sm.acc[wq * sm.cs_len + j];
        h[j] = s * sm.sc[j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBW * sm.cs_len; i += kBT)
        sm.acc[i] = 0;
    __syncthreads();
}

// Hessenberg column k: rotate, new Givens rotation, estimate and triggers (thread 0;
// src/gmres.cpp:191-214).
__device__ void finish_col(St &s, const Smem &sm, float hnext, bool nonfinite, int cap, float tau) {
    const int k = s.k;
    float *col = sm.col;
    col[k + 1] = hnext;
    nonfinite |= !isfinite(hnext);
    s.hnext = hnext;
    s.breakdown = hnext == 0.f;
    sm.sc[k + 1] = hnext == 0.f ? 0.f : 1.f / hnext;
    float carry = col[0];
    for (int r = 0; r < k; ++r) {
        const float lo = col[r + 1];
        col[r] = sm.cs[r] * carry + sm.sn[r] * lo;
        carry = -sm.sn[r] * carry + sm.cs[r] * lo;
    }
    col[k] = carry;
    const float upper = col[k];
    const float radius = cr_hypot<float>(upper, col[k + 1]);
    s.iterations = k + 1;
    if (nonfinite || !isfinite(radius)) {
        s.status = 8;
        s.active = 0;
        s.triggered = 0;
        s.vgate = 0;
        return;
    }
    if (radius == 0.f) {
        s.triggered = 2;
        s.vgate = 1;
        return;
    }
    sm.cs[k] = upper / radius;
    sm.sn[k] = col[k + 1] / radius;
    col[k] = radius;
    col[k + 1] = 0;
    const float old = sm.g[k];
    sm.g[k] = sm.cs[k] * old;
    sm.g[k + 1] = -sm.sn[k] * old;
    const float est = fabsf(sm.g[k + 1]) / static_cast<float>(s.den);
    const bool trig = s.breakdown || est <= tau || k + 1 == cap;
    s.triggered = trig ? 1 : 0;
    s.vgate = trig ? 1 : 0;
}

// Binary64 residual r = b - A x with the diagnostics and the refinement decision
// (src/ir.cpp:83-133, 149-175).
__device__ void ir_residual(const BatchArgs &a, const BatchSys &d, St &s, const double *b, const double *x,
                            double *r, double *red) {
    const int n = d.n, G = a.ga;
    const int lane = threadIdx.x & (G - 1);
    const int rpw = 32 / G, sub = (threadIdx.x & 31) / G;
    double rinf = 0, xinf = 0, cbe = 0;
    int bad = 0;
    for (int base = (threadIdx.x >> 5) * rpw; base < n; base += kBW * rpw) {
        const int row = base + sub;
        double acc = 0, absacc = 0;
        if (row < n) {
            const int gr = d.row0 + row;
            const int e1 = a.arp[gr + 1];
            for (int e = a.arp[gr] + lane; e < e1; e += G) {
                const double xv = x[a.aci[e] - d.row0];
                acc += a.a64[e] * xv;
                absacc += fabs(a.a64[e]) * fabs(xv);
            }
        }
        for (int o = G / 2; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(kFull, acc, o, G);
            absacc += __shfl_xor_sync(kFull, absacc, o, G);
        }
        if (lane == 0 && row < n) {
            const double res = b[row] - acc;
            r[row] = res;
            bad |= !isfinite(res) || !isfinite(absacc);
            rinf = fmax(rinf, fabs(res));
            xinf = fmax(xinf, fabs(x[row]));
            const double cden = fabs(b[row]) + absacc;
            if (cden == 0)
                cbe = fmax(cbe, res == 0 ? 0.0 : INFINITY);
            else if (fabs(res) >= cbe * cden * 0.99999999999999911182) // divide only when it can win
                cbe = fmax(cbe, fabs(res) / cden);
        }
    }
    bad = __syncthreads_or(bad);
    rinf = cta_max(rinf, red);
    xinf = cta_max(xinf, red);
    cbe = cta_max(cbe, red);
    if (threadIdx.x == 0) {
        s.rinf = rinf;
        s.xinf = xinf;
        s.cbe = cbe;
        const double den = s.anorm * xinf + s.binf;
        if (bad || !isfinite(den)) {
            s.ir_status = 6;
            s.outer_active = 0;
        } else {
            const double be = den == 0 ? (rinf == 0 ? 0.0 : INFINITY) : rinf / den;
            s.be = be;
            if (be <= a.be_tol) {
                s.ir_status = 0;
                s.outer_active = 0;
            } else if (s.ir_started && !s.changed) {
                s.ir_status = 4;
                s.outer_active = 0;
            } else if (s.outer_steps >= a.outer_cap) {
                s.ir_status = 5;
                s.outer_active = 0;
            } else {
                s.inner_scale = ldexp(1.0, -ilogb(rinf));
                s.ir_started = 1;
                s.changed = 0;
            }
        }
    }
    __syncthreads();
}

// Inner GMRES on P A d = P rhs (x0 = 0) for one system; leaves the accepted correction in cand
// (s.formed > 0) or a zero correction (s.formed < 0).
__device__ void gmres(const BatchArgs &a, const BatchSys &d, St &s, const Smem &sm, double *red, float *w,
                      float *t, const float *rhs, float *pb, float *cand, float *ax, float *V, float *H) {
    const int n = d.n, cap = d.cap, cap1 = cap + 1, hld = a.hcap + 2;
    const float tau = static_cast<float>(a.tau);
    bool nf = false;
    const float r0 = cta_norm(n, rhs, nullptr, red, nf);
    if (threadIdx.x == 0) {
        s.k = 0;
        s.triggered = s.breakdown = s.converged = s.iterations = s.formed = 0;
        s.rel = NAN;
        s.active = 1;
        s.status = 7;
        s.orig = r0;
        if (nf || !isfinite(r0)) {
            s.status = 8;
            s.active = 0;
        } else if (r0 == 0.f) {
            s.status = 1; // zero_rhs
            s.converged = 1;
            s.active = 0;
            s.formed = -1;
        }
    }
    __syncthreads();
    if (!s.active)
        return;
    cta_spmv(n, d.row0, a.gp, a.prp, a.pci, a.pv, [&](int j) { return rhs[j]; }, 1.f, pb);
    __syncthreads();
    const float den = cta_norm(n, pb, nullptr, red, nf);
    if (threadIdx.x == 0) {
        s.den = den;
        if (nf || !isfinite(den)) {
            s.status = 8;
            s.active = 0;
        } else if (den == 0.f) {
            s.status = 4; // zero_preconditioned_rhs
            s.active = 0;
        } else if (1.0f <= tau) {
            s.status = 0;
            s.converged = 1;
            s.active = 0;
            s.formed = -1;
        } else {
            sm.g[0] = den;
            sm.sc[0] = 1.f;
        }
    }
    __syncthreads();
    if (!s.active)
        return;
    // W_0 = Pb / ||Pb|| (pad rows zero).
    for (int i = threadIdx.x; i < d.ntiles * kTR; i += kBT)
        V[static_cast<long long>(i / kTR) * cap1 * kTR + (i % kTR)] = i < n ? pb[i] / den : 0.f;
    __syncthreads();
    for (int step = 0; step < cap && s.active; ++step) {
        const int k = s.k;
        const int kk = k + 1;
        // t = s_k A W_k ; w = P t
        const float sk = sm.sc[k];
        cta_spmv(n, d.row0, a.ga, a.arp, a.aci, a.a32,
                 [&](int j) { return V[static_cast<long long>(j / kTR) * cap1 * kTR + static_cast<long long>(k) * kTR + (j % kTR)]; },
                 sk, t);
        __syncthreads();
        cta_spmv(n, d.row0, a.gp, a.prp, a.pci, a.pv, [&](int j) { return t[j]; }, 1.f, w);
        __syncthreads();
        bool bad = false;
        double sq = tile_pass<1>(w, V, d.ntiles, cap1, k, sm, bad);
        const float wnorm = static_cast<float>(sqrt(cta_sum(sq, red)));
        combine_dots(kk, sm, sm.h1);
        for (int j = threadIdx.x; j < kk; j += kBT)
            sm.cf[j] = sm.h1[j] * sm.sc[j];
        __syncthreads();
        sq = tile_pass<2>(w, V, d.ntiles, cap1, k, sm, bad);
        const float n2 = static_cast<float>(sqrt(cta_sum(sq, red)));
        combine_dots(kk, sm, sm.h2);
        // DGKS: a second projection only when the first cancelled more than 1 - 1/sqrt(2).
        const bool reorth = !bad && !(n2 >= 0.70710678118654752f * wnorm);
        float hn = n2;
        if (reorth) {
            for (int j = threadIdx.x; j < kk; j += kBT)
                sm.cf[j] = sm.h2[j] * sm.sc[j];
            __syncthreads();
            sq = tile_pass<3>(w, V, d.ntiles, cap1, k, sm, bad);
            hn = static_cast<float>(sqrt(cta_sum(sq, red)));
        }
        for (int j = threadIdx.x; j < kk; j += kBT)
            sm.col[j] = reorth ? sm.h1[j] + sm.h2[j] : sm.h1[j];
        __syncthreads();
        if (threadIdx.x == 0) {
            bool nonfinite = bad || !isfinite(wnorm);
            for (int j = 0; j < kk; ++j)
                nonfinite |= !isfinite(sm.col[j]);
            s.reorth_count += reorth ? 1 : 0;
            finish_col(s, sm, hn, nonfinite, cap, tau);
        }
        __syncthreads();
        // Keep the rotated column for the back substitution.
        float *hc = H + static_cast<long long>(k) * hld;
        for (int j = threadIdx.x; j <= k + 1; j += kBT)
            hc[j] = sm.col[j];
        __syncthreads();
        if (s.vgate && s.active) {
            // y = R^{-1} g over `count` columns (one warp, column sweep).
            const int count = s.triggered == 2 ? k : k + 1;
            if (threadIdx.x < 32) {
                const int lane = lane_id();
                for (int r = lane; r < count; r += 32)
                    sm.y[r] = sm.g[r];
                __syncwarp();
                int ybad = 0;
                for (int c = count - 1; c >= 0; --c) {
                    const float *hcol = H + static_cast<long long>(c) * hld;
                    float yc = 0;
                    if (lane == 0) {
                        yc = sm.y[c] / hcol[c];
                        sm.y[c] = yc;
                    }
                    yc = __shfl_sync(kFull, yc, 0);
                    ybad |= !isfinite(yc);
                    for (int r = lane; r < c; r += 32)
                        sm.y[r] -= hcol[r] * yc;
                    __syncwarp();
                }
                if (lane == 0) {
                    s.formed = count;
                    if (ybad) {
                        s.status = 8;
                        s.active = 0;
                    }
                }
            }
            __syncthreads();
            if (s.active) {
                for (int j = threadIdx.x; j < count; j += kBT)
                    sm.cf[j] = sm.y[j] * sm.sc[j];
                __syncthreads();
                // cand = sum_j (y_j s_j) W_j, warp per tile.
                const int lane = lane_id(), warp = threadIdx.x >> 5;
                for (int tt = warp; tt < d.ntiles; tt += kBW) {
                    const float *tile = V + static_cast<long long>(tt) * cap1 * kTR + lane * 4;
                    float4 acc = make_float4(0, 0, 0, 0);
                    for (int j = 0; j < count; ++j) {
                        const float4 v = *reinterpret_cast<const float4 *>(tile + static_cast<long long>(j) * kTR);
                        const float c = sm.cf[j];
                        acc.x += c * v.x;
                        acc.y += c * v.y;
                        acc.z += c * v.z;
                        acc.w += c * v.w;
                    }
                    *reinterpret_cast<float4 *>(cand + tt * kTR + lane * 4) = acc;
                }
                __syncthreads();
                cta_spmv(n, d.row0, a.ga, a.arp, a.aci, a.a32, [&](int j) { return cand[j]; }, 1.f, ax);
                __syncthreads();
                bool nf1 = false, nf2 = false;
                const float orig = cta_norm(n, rhs, ax, red, nf1);
                // pax = P (A cand) into t (free until the next step)
                cta_spmv(n, d.row0, a.gp, a.prp, a.pci, a.pv, [&](int j) { return ax[j]; }, 1.f, t);
                __syncthreads();
                const float relnum = cta_norm(n, pb, t, red, nf2);
                if (threadIdx.x == 0) {
                    // Acceptance (src/gmres.cpp:235-253).
                    s.verifications += 1;
                    const double rel = static_cast<double>(relnum) / s.den;
                    s.orig = orig;
                    s.rel = rel;
                    if (nf1 || nf2 || !isfinite(rel) || !isfinite(static_cast<double>(orig))) {
                        s.status = 8;
                        s.active = 0;
                    } else {
                        const bool ok = rel <= a.tau;
                        if (s.triggered == 2) {
                            s.converged = ok;
                            s.status = ok ? 0 : 5;
                            s.active = 0;
                        } else if (ok) {
                            s.converged = 1;
                            s.status = 0;
                            s.active = 0;
                        } else if (s.breakdown) {
                            s.status = 5;
                            s.active = 0;
                        }
                    }
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0 && s.active) {
            s.vgate = 0;
            if (s.k + 1 >= cap) {
                s.status = cap < n ? 6 : 7;
                s.active = 0;
            } else {
                s.k += 1;
                s.triggered = 0;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kBT, 1) batched_ir_kernel(BatchArgs a) {
    extern __shared__ __align__(16) float dyn[];
    __shared__ St s;
    __shared__ double red[kBW];
    __shared__ int q_sh;
    Smem sm;
    sm.cs_len = a.hcap + 2;
    sm.acc = dyn;
    float *p = dyn + kBW * sm.cs_len;
    float **arrays[] = {&sm.h1, &sm.h2, &sm.cf, &sm.sc, &sm.col, &sm.cs, &sm.sn, &sm.g, &sm.y};
    for (float **q : arrays) {
        *q = p;
        p += sm.cs_len;
    }
    for (int i = threadIdx.x; i < kBW * sm.cs_len; i += kBT)
        sm.acc[i] = 0;
    float *H = a.H + static_cast<long long>(blockIdx.x) * (a.hcap + 1) * (a.hcap + 2);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0)
            q_sh = atomicAdd(a.queue, 1);
        __syncthreads();
        const int q = q_sh;
        if (q >= a.count)
            return;
        const int id = a.order[q];
        const BatchSys d = a.sys[id];
        BatchOut o{};
        if (d.skip) {
            if (threadIdx.x == 0) {
                o.ir_status = d.preset;
                o.gmres_status = -1;
                o.be = o.cbe = o.rinf = NAN;
                a.out[id] = o;
            }
            continue;
        }
        const long long off = d.pad0;
        const double *b = a.b + off;
        double *x = a.x + off, *r = a.r + off, *xn = a.xn + off;
        float *w = a.w + off, *t = a.t + off, *rhs = a.rhs + off, *pb = a.pb + off, *cand = a.cand + off,
              *ax = a.ax + off;
        float *V = a.V + d.vbase;
        const int n = d.n;
        if (threadIdx.x == 0) {
            memset(&s, 0, sizeof(St));
            s.ir_status = -1;
            s.last_gmres = -1;
            s.outer_active = 1;
            s.inner_scale = 1.0;
        }
        // ||A||_inf, ||b||_inf and x0 = P b (binary64 accumulation of the binary32 P).
        double an = 0, bn = 0;
        for (int i = threadIdx.x; i < n; i += kBT) {
            const int gr = d.row0 + i;
            double rs = 0;
            for (int e = a.arp[gr]; e < a.arp[gr + 1]; ++e)
                rs += fabs(a.a64[e]);
            an = fmax(an, rs);
            bn = fmax(bn, fabs(b[i]));
            double acc = 0;
            for (int e = a.prp[gr]; e < a.prp[gr + 1]; ++e)
                acc += static_cast<double>(a.pv[e]) * b[a.pci[e] - d.row0];
            x[i] = acc;
        }
        an = cta_max(an, red);
        bn = cta_max(bn, red);
        if (threadIdx.x == 0) {
            s.anorm = an;
            s.binf = bn;
        }
        __syncthreads();
        ir_residual(a, d, s, b, x, r, red);
        for (int outer = 0; outer <= a.outer_cap && s.outer_active; ++outer) {
            const double sc = s.inner_scale;
            for (int i = threadIdx.x; i < n; i += kBT)
                rhs[i] = static_cast<float>(r[i] * sc);
            __syncthreads();
            gmres(a, d, s, sm, red, w, t, rhs, pb, cand, ax, V, H);
            if (threadIdx.x == 0) {
                s.inner_attempts += 1;
                s.inner_total += s.iterations;
                s.last_gmres = s.status;
                // SPAI_FLAG_RESTART_AT_CAP: a cap-limited solve whose verified candidate reduced
                // the preconditioned residual still supplies the correction.
                const bool partial = a.restart && s.status == 6 && s.formed > 0 && s.rel < 1.0;
                if (!s.converged && !partial) {
                    s.ir_status = 3; // inner_failure
                    s.outer_active = 0;
                }
            }
            __syncthreads();
            if (!s.outer_active)
                break;
            // x_new = x + d / scale (exact power-of-two unscaling).
            const bool zero = s.formed < 0;
            const double inv = 1.0 / sc;
            int changed = 0, bad = 0;
            for (int i = threadIdx.x; i < n; i += kBT) {
                const double old = x[i];
                const double nw = zero ? old : old + static_cast<double>(cand[i]) * inv;
                xn[i] = nw;
                changed |= nw != old;
                bad |= !isfinite(nw);
            }
            changed = __syncthreads_or(changed);
            bad = __syncthreads_or(bad);
            if (threadIdx.x == 0) {
                s.changed = changed;
                if (bad) {
                    s.ir_status = 6;
                    s.outer_active = 0;
                } else {
                    s.outer_steps += 1;
                }
            }
            __syncthreads();
            if (s.ir_status == 6)
                break;
            ir_residual(a, d, s, b, xn, r, red);
            // Commit unless the new iterate's diagnostics failed (src/ir.cpp:176-186).
            if (s.ir_status != 6)
                for (int i = threadIdx.x; i < n; i += kBT)
                    x[i] = xn[i];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            o.ir_status = s.ir_status < 0 ? 5 : s.ir_status;
            o.converged = s.ir_status == 0;
            o.outer_steps = s.outer_steps;
            o.inner_attempts = s.inner_attempts;
            o.inner_iterations = s.inner_total;
            o.gmres_status = s.last_gmres;
            o.verifications = s.verifications;
            o.reorth = s.reorth_count;
            o.be = s.be;
            o.cbe = s.cbe;
            o.rinf = s.rinf;
            a.out[id] = o;
        }
    }
}

// Block-diagonal assembly: one block per system converts its int64 CSR (staged on the device)
// to the union's int32 offsets and global column indices, and rounds the values to binary32.
__global__ void assemble_kernel(int count, const long long *__restrict__ sys_row0,
                                const long long *__restrict__ sys_nnz0, const long long *__restrict__ stage_rp,
                                const long long *__restrict__ stage_ci, const double *__restrict__ val,
                                int *rp, int *ci, float *v32) {
    for (int s = blockIdx.x; s < count; s += gridDim.x) {
        const long long r0 = sys_row0[s], r1 = sys_row0[s + 1];
        const long long z0 = sys_nnz0[s], z1 = sys_nnz0[s + 1];
        const long long *srp = stage_rp + r0 + s; // each system staged n_s + 1 offsets
        for (long long i = threadIdx.x; i <= r1 - r0; i += blockDim.x)
            if (i < r1 - r0 || s == count - 1)
                rp[r0 + i] = static_cast<int>(z0 + srp[i]);
        for (long long e = z0 + threadIdx.x; e < z1; e += blockDim.x) {
            ci[e] = static_cast<int>(r0 + stage_ci[e]);
            v32[e] = static_cast<float>(val[e]);
        }
    }
}

// Per-system SPAI status: the first failing column inside the system's block.
__global__ void system_status_kernel(int count, const long long *__restrict__ sys_row0,
                                     const int *__restrict__ col_status, int *first) {
    for (int s = blockIdx.x; s < count; s += gridDim.x) {
        int f = INT_MAX;
        for (long long c = sys_row0[s] + threadIdx.x; c < sys_row0[s + 1]; c += blockDim.x)
            if (col_status[c] != 0)
                f = min(f, static_cast<int>(c));
        for (int o = 16; o > 0; o >>= 1)
            f = min(f, __shfl_xor_sync(kFull, f, o));
        __shared__ int sh[32];
        if ((threadIdx.x & 31) == 0)
            sh[threadIdx.x >> 5] = f;
        __syncthreads();
        if (threadIdx.x == 0) {
            int m = INT_MAX;
            for (int i = 0; i < static_cast<int>(blockDim.x >> 5); ++i)
                m = min(m, sh[i]);
            first[s] = m;
        }
        __syncthreads();
    }
}

int lanes_for(int max_row) {
    return max_row <= 4 ? 4 : (max_row <= 16 ? 8 : (max_row <= 64 ? 16 : 32));
}

struct Batch {
    DeviceArena mem, build;
};

} // namespace batched_detail
} // namespace spai

using namespace spai;

extern "C" int spai_ir_solve_batched(int64_t count, const spai_csr *systems, const double *const *b,
                                     double *const *x, const spai_options *opt, spai_report *reports,
                                     void *stream) {
    try {
        if (count < 1 || count > INT_MAX / 2 || !systems || !b || !x || !opt || !reports)
            return spai_api_fail(SPAI_ERR_ARGUMENT, "spai_ir_solve_batched: bad arguments");
        if (opt->precision != SPAI_PREC_MIXED)
            return spai_api_fail(SPAI_ERR_UNSUPPORTED,
                                 "spai_ir_solve_batched: batched solves run the mixed form (SPAI_PREC_MIXED)");
        const int nsys = static_cast<int>(count);
        long long rows = 0, nnz = 0;
        int max_row_a = 0;
        for (int s = 0; s < nsys; ++s) {
            const std::string why = spai_api::canonical_error(&systems[s]);
            if (!why.empty())
                return spai_api_fail(SPAI_ERR_ARGUMENT,
                                     "spai_ir_solve_batched: system " + std::to_string(s) + ": " + why);
            if (!b[s] || !x[s])
                return spai_api_fail(SPAI_ERR_ARGUMENT, "spai_ir_solve_batched: null vector");
            rows += systems[s].n;
            nnz += systems[s].nnz;
            for (int64_t r = 0; r < systems[s].n; ++r)
                max_row_a = std::max<int>(max_row_a, static_cast<int>(systems[s].row_offsets[r + 1] - systems[s].row_offsets[r]));
        }
        if (rows > INT_MAX - 1 || nnz > INT_MAX - 1)
            return spai_api_fail(SPAI_ERR_ARGUMENT, "spai_ir_solve_batched: union exceeds 32-bit indices");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        int device = 0, sms = 0;
        SPAI_CUDA(cudaGetDevice(&device));
        SPAI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));

        // Per-system layout and validation of the options (src/ir.cpp:41-55).
        const double tau = spai_api::inner_tau(*opt);
        std::vector<BatchSys> hs(nsys);
        std::vector<long long> row0(nsys + 1), nnz0(nsys + 1);
        long long pad = 0, vtot = 0;
        int hcap = 1;
        for (int s = 0; s < nsys; ++s) {
            spai_api::clear_report(&reports[s]);
            const spai_csr &c = systems[s];
            row0[s + 1] = row0[s] + c.n;
            nnz0[s + 1] = nnz0[s] + c.nnz;
            BatchSys &d = hs[s];
            d.row0 = static_cast<int>(row0[s]);
            d.n = static_cast<int>(c.n);
            d.ntiles = (d.n + kTR - 1) / kTR;
            d.cap = opt->innercap == 0 ? d.n : static_cast<int>(std::min<int64_t>(opt->innercap, c.n));
            d.pad0 = pad;
            d.vbase = vtot;
            pad += static_cast<long long>(d.ntiles) * kTR;
            d.skip = 0;
            d.preset = 0;
            const bool valid = opt->outercap >= 0 && opt->outercap <= 20 && opt->innercap >= 0 &&
                               opt->innercap <= c.n && std::isfinite(tau) && tau > 0 && opt->alpha >= 0 &&
                               opt->beta >= 0;
            bool finite = true;
            for (int64_t i = 0; i < c.n && finite; ++i)
                finite = std::isfinite(b[s][i]);
            if (!valid || !finite) {
                d.skip = 1;
                d.preset = IR_INVALID_INPUT;
                d.cap = 1;
            }
            vtot += static_cast<long long>(d.ntiles) * (d.cap + 1) * kTR;
            hcap = std::max(hcap, d.cap);
        }
        const size_t smem = sizeof(float) * static_cast<size_t>(kBW + 9) * (hcap + 2);
        if (smem > 200 * 1024)
            return spai_api_fail(SPAI_ERR_ARGUMENT, "spai_ir_solve_batched: innercap too large for the "
                                                    "per-CTA Hessenberg workspace (at most 1936)");

        Batch bt;
        DeviceArena &m = bt.mem;
        // Upload: int64 offsets/indices staged, values binary64.
        long long *srp = m.alloc<long long>(rows + nsys);
        long long *sci = m.alloc<long long>(std::max<long long>(nnz, 1));
        long long *d_row0 = m.alloc<long long>(nsys + 1);
        long long *d_nnz0 = m.alloc<long long>(nsys + 1);
        DeviceCsr<double> a64;
        DeviceCsr<float> a32;
        a64.n = a32.n = static_cast<int>(rows);
        a64.nnz = a32.nnz = static_cast<int>(nnz);
        a64.max_row = a32.max_row = max_row_a;
        a64.rp = a32.rp = m.alloc<int>(rows + 1);
        a64.ci = a32.ci = m.alloc<int>(std::max<long long>(nnz, 1));
        a64.val = m.alloc<double>(std::max<long long>(nnz, 1));
        a32.val = m.alloc<float>(std::max<long long>(nnz, 1));
        double *db = m.alloc<double>(pad);
        SPAI_CUDA(cudaMemsetAsync(db, 0, sizeof(double) * pad, st));
        for (int s = 0; s < nsys; ++s) {
            const spai_csr &c = systems[s];
            SPAI_CUDA(cudaMemcpyAsync(srp + row0[s] + s, c.row_offsets, sizeof(long long) * (c.n + 1),
                                      cudaMemcpyHostToDevice, st));
            if (c.nnz > 0) {
                SPAI_CUDA(cudaMemcpyAsync(sci + nnz0[s], c.col_indices, sizeof(long long) * c.nnz,
                                          cudaMemcpyHostToDevice, st));
                SPAI_CUDA(cudaMemcpyAsync(a64.val + nnz0[s], c.values, sizeof(double) * c.nnz,
                                          cudaMemcpyHostToDevice, st));
            }
            SPAI_CUDA(cudaMemcpyAsync(db + hs[s].pad0, b[s], sizeof(double) * c.n, cudaMemcpyHostToDevice, st));
        }
        SPAI_CUDA(cudaMemcpyAsync(d_row0, row0.data(), sizeof(long long) * (nsys + 1), cudaMemcpyHostToDevice, st));
        SPAI_CUDA(cudaMemcpyAsync(d_nnz0, nnz0.data(), sizeof(long long) * (nsys + 1), cudaMemcpyHostToDevice, st));
        assemble_kernel<<<std::min(nsys, sms * 8), 256, 0, st>>>(nsys, d_row0, d_nnz0, srp, sci, a64.val, a64.rp,
                                                                a64.ci, a32.val);
        SPAI_LAUNCH("assemble_kernel");

        // One SPAI build over the block-diagonal union (binary32, the reference's arithmetic).
        SpaiParams prm;
        prm.epsilon = opt->epsilon;
        prm.alpha = opt->alpha;
        prm.beta = static_cast<int>(std::min<int64_t>(opt->beta, INT_MAX));
        prm.fast = (opt->flags & SPAI_FLAG_FAST_SPAI) != 0;
        SpaiOutput<float> sp;
        cudaEvent_t e0, e1, e2;
        SPAI_CUDA(cudaEventCreate(&e0));
        SPAI_CUDA(cudaEventCreate(&e1));
        SPAI_CUDA(cudaEventCreate(&e2));
        SPAI_CUDA(cudaEventRecord(e0, st));
        SpaiBuilder<float>::construct(a32, prm, st, sp, bt.build);
        SPAI_CUDA(cudaEventRecord(e1, st));
        int *first = m.alloc<int>(nsys);
        system_status_kernel<<<std::min(nsys, sms * 8), 256, 0, st>>>(nsys, d_row0, sp.col_status, first);
        SPAI_LAUNCH("system_status_kernel");
        std::vector<int> hfirst(nsys);
        SPAI_CUDA(cudaMemcpyAsync(hfirst.data(), first, sizeof(int) * nsys, cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
        std::vector<int> spai_status(nsys, SPAI_SUCCESS), spai_first(nsys, -1);
        for (int s = 0; s < nsys; ++s) {
            if (hfirst[s] != INT_MAX) {
                int cst = 0;
                SPAI_CUDA(cudaMemcpy(&cst, sp.col_status + hfirst[s], sizeof(int), cudaMemcpyDeviceToHost));
                spai_status[s] = cst;
                spai_first[s] = static_cast<int>(hfirst[s] - row0[s]);
            }
        }
        if (sp.status == SPAI_NUMERICAL_FAILURE && sp.first_failed >= 0) {
            // Assembly outside the binary range ends that system's construction.
            const int s = static_cast<int>(std::upper_bound(row0.begin(), row0.end(), sp.first_failed) - row0.begin()) - 1;
            if (s >= 0 && s < nsys && spai_status[s] == SPAI_SUCCESS) {
                spai_status[s] = SPAI_NUMERICAL_FAILURE;
                spai_first[s] = static_cast<int>(sp.first_failed - row0[s]);
            }
        }
        for (int s = 0; s < nsys; ++s)
            if (!hs[s].skip && spai_status[s] != SPAI_SUCCESS) {
                hs[s].skip = 1;
                hs[s].preset = IR_CONSTRUCTION_FAILURE;
            }

        // Refinement workspace.
        BatchSys *dsys = m.alloc<BatchSys>(nsys);
        SPAI_CUDA(cudaMemcpyAsync(dsys, hs.data(), sizeof(BatchSys) * nsys, cudaMemcpyHostToDevice, st));
        std::vector<int> order(nsys);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
            return static_cast<long long>(hs[p].n) * hs[p].cap > static_cast<long long>(hs[q].n) * hs[q].cap;
        });
        int *dorder = m.alloc<int>(nsys);
        SPAI_CUDA(cudaMemcpyAsync(dorder, order.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice, st));
        int *queue = m.alloc<int>(1);
        SPAI_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), st));
        BatchArgs a{};
        a.count = nsys;
        a.outer_cap = static_cast<int>(opt->outercap);
        a.tau = tau;
        a.be_tol = spai_api::be_tol(*opt);
        a.restart = (opt->flags & SPAI_FLAG_RESTART_AT_CAP) != 0 ? 1 : 0;
        a.order = dorder;
        a.queue = queue;
        a.sys = dsys;
        a.arp = a64.rp;
        a.aci = a64.ci;
        a.a64 = a64.val;
        a.a32 = a32.val;
        a.prp = sp.p.rp;
        a.pci = sp.p.ci;
        a.pv = sp.p.val;
        a.ga = lanes_for(max_row_a);
        a.gp = lanes_for(sp.p.max_row > 0 ? sp.p.max_row : 1);
        a.b = db;
        a.x = m.alloc<double>(pad);
        a.r = m.alloc<double>(pad);
        a.xn = m.alloc<double>(pad);
        float **fv[] = {&a.w, &a.t, &a.rhs, &a.pb, &a.cand, &a.ax};
        for (float **q : fv) {
            *q = m.alloc<float>(pad);
            SPAI_CUDA(cudaMemsetAsync(*q, 0, sizeof(float) * pad, st)); // pad rows stay zero
        }
        a.V = m.alloc<float>(std::max<long long>(vtot, 1));
        a.hcap = hcap;
        SPAI_CUDA(cudaFuncSetAttribute(batched_ir_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem)));
        int per_sm = 0;
        SPAI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_ir_kernel, kBT, smem));
        const int grid = std::max(1, std::min(nsys, sms * std::max(per_sm, 1)));
        a.H = m.alloc<float>(static_cast<size_t>(grid) * (hcap + 1) * (hcap + 2));
        a.out = m.alloc<BatchOut>(nsys);
        batched_ir_kernel<<<grid, kBT, smem, st>>>(a);
        SPAI_LAUNCH("batched_ir_kernel");
        SPAI_CUDA(cudaEventRecord(e2, st));
        std::vector<BatchOut> ho(nsys);
        SPAI_CUDA(cudaMemcpyAsync(ho.data(), a.out, sizeof(BatchOut) * nsys, cudaMemcpyDeviceToHost, st));
        for (int s = 0; s < nsys; ++s)
            if (!hs[s].skip)
                SPAI_CUDA(cudaMemcpyAsync(x[s], a.x + hs[s].pad0, sizeof(double) * hs[s].n,
                                          cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
        float spai_ms = 0, solve_ms = 0;
        SPAI_CUDA(cudaEventElapsedTime(&spai_ms, e0, e1));
        SPAI_CUDA(cudaEventElapsedTime(&solve_ms, e1, e2));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
        for (int s = 0; s < nsys; ++s) {
            spai_report &rp = reports[s];
            rp.spai_status = spai_status[s];
            rp.first_failed_column = spai_first[s];
            rp.spai_ms = spai_ms;
            rp.solve_ms = solve_ms;
            rp.kernel_launches = 2;
            const BatchOut &o = ho[s];
            rp.ir_status = o.ir_status;
            rp.converged = o.converged;
            rp.outer_steps = o.outer_steps;
            rp.inner_attempts = o.inner_attempts;
            rp.inner_iterations = o.inner_iterations;
            rp.gmres_status = o.gmres_status;
            rp.backward_error = o.be;
            rp.componentwise_backward_error = o.cbe;
            rp.residual_inf = o.rinf;
        }
        return SPAI_OK;
    } catch (const spai::ArgumentError &e) {
        return spai_api_fail(SPAI_ERR_ARGUMENT, e.what());
    } catch (const spai::WorkspaceError &e) {
        return spai_api_fail(SPAI_ERR_WORKSPACE, e.what());
    } catch (const std::exception &e) {
        return spai_api_fail(SPAI_ERR_CUDA, e.what());
    }
}
