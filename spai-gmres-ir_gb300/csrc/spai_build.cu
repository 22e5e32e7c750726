// Adaptive SPAI construction on the device: one persistent kernel in which a warp owns a column.
//
// Reference path replaced: cuda_construct_spai (src/cuda_spai.cu:519-956), whose host loop
// builds shadows/candidates, uploads them, runs cuSOLVER geqrf/ormqr, one-thread guard and
// residual kernels and downloads scores for every fit; and the CPU definition it follows,
// construct_column / least_squares / evaluate_spai_score (src/spai.cpp:30-306).
//
// Here the whole adaptive loop of a column (shadow, reduced gather, Householder QR, triangular
// solve, fitted residual, candidate scoring, mean, (score,index) selection, pattern growth) runs
// inside one warp with its working set in shared memory; warps pull columns from an atomic
// queue. A column whose working set does not fit is handed to a second pass that gives each
// warp a large global-memory workspace. Every floating-point operation follows the reference's
// order (sequential sums, hypot chains, normalised reflectors); this file is compiled with
// --fmad=false and the hypot is correctly rounded, so a column fit is bit-identical to the CPU
// restatement. Parallelism is across the independent columns of the reduced matrix (one lane per
// column in the QR step) and across candidates (one lane per candidate in the scoring step).
#include "common.cuh"
#include "exact_math.cuh"
#include "spai_internal.hpp"

#include <cooperative_groups.h>
#include <cub/device/device_scan.cuh>

#include <chrono>
#include <cstdio>
#include <cstdlib>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace spai {

enum : int {
    kSuccess = 0,
    kNotAttempted = 1,
    kInvalidInput = 2,
    kRankDeficient = 3,
    kNumericalFailure = 4,
    kEmptyCandidates = 5,
    kZeroDenominator = 6,
    kInvalidScore = 7,
    kNoGrowth = 8,
    kIterationLimit = 9,
    kOverflow = 100
};

template <class T> struct Unit;
template <> struct Unit<double> {
    static __device__ __forceinline__ double u() {
        return 0x1p-53;
    }
};
template <> struct Unit<float> {
    static __device__ __forceinline__ float u() {
        return 0x1p-24f;
    }
};

// ------------------------------------------------------------------------------------------
// Row scaling D (src/spai.cpp:322-348, src/cuda_spai.cu:247-278): warp per row.
// status: 0 ok, 1 zero diagonal, 2 reciprocal out of range, 3 scaled entry zero/nonfinite.
// ------------------------------------------------------------------------------------------
template <class T>
__global__ void scale_rows_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                  const T *__restrict__ av, T *__restrict__ d,
                                  int *__restrict__ bad_row) {
    const int lane = lane_id();
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += warps) {
        const int b = rp[row], e = rp[row + 1];
        T mx = 0;
        int diag = 0;
        for (int t = b + lane; t < e; t += 32) {
            mx = fmax(mx, fabs(av[t]));
            diag |= (ci[t] == row && av[t] != T(0));
        }
        for (int o = 16; o > 0; o >>= 1)
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        diag = __any_sync(0xffffffffu, diag);
        int status = 0;
        T scale = 0;
        if (!diag) {
            status = 1;
        } else {
            scale = T(1) / mx;
            if (!isfinite(scale) || scale == T(0))
                status = 2;
        }
        if (status == 0) {
            int bad = 0;
            for (int t = b + lane; t < e; t += 32) {
                const T v = av[t] * scale;
                bad |= (!isfinite(v) || v == T(0));
            }
            if (__any_sync(0xffffffffu, bad))
                status = 3;
        }
        if (lane == 0) {
            d[row] = scale;
            if (status)
                atomicMin(bad_row, row);
        }
    }
}

// Column structure of A (row i of B = (DA)^T): counts, then an unordered fill. Only the set of
// rows per column is used (candidate unions are sorted afterwards), so fill order is irrelevant.
__global__ void column_count_kernel(int nnz, const int *__restrict__ ci, int *__restrict__ cnt) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nnz; t += gridDim.x * blockDim.x)
        atomicAdd(&cnt[ci[t] + 1], 1);
}
__global__ void column_fill_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                   const int *__restrict__ tp, int *__restrict__ fill,
                                   int *__restrict__ ti) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += gridDim.x * blockDim.x)
        for (int t = rp[row]; t < rp[row + 1]; ++t) {
            const int c = ci[t];
            ti[tp[c] + atomicAdd(&fill[c], 1)] = row;
        }
}

// ------------------------------------------------------------------------------------------
// Group-cooperative building blocks: a group of G lanes (a thread_block_tile<G>) owns a column;
// 32/G columns run in each warp. Every function is called by all lanes of the group together.
// ------------------------------------------------------------------------------------------
namespace cg = cooperative_groups;

struct Bump {
    char *base;
    size_t cap, top;
    template <class U> __device__ U *take(long long count) {
        size_t a = (top + 15) & ~size_t(15);
        const size_t bytes = static_cast<size_t>(count < 1 ? 1 : count) * sizeof(U);
        if (a + bytes > cap)
            return nullptr;
        top = a + bytes;
        return reinterpret_cast<U *>(base + a);
    }
    __device__ size_t mark() const {
        return top;
    }
    __device__ void reset(size_t m) {
        top = m;
    }
};

__device__ __forceinline__ int pow2_at_least(int x) {
    int p = 1;
    while (p < x)
        p <<= 1;
    return p;
}

template <class Grp> __device__ __forceinline__ int grp_sum(const Grp &g, int v) {
    for (int o = Grp::size() / 2; o > 0; o >>= 1)
        v += g.shfl_xor(v, o);
    return v;
}
template <class Grp> __device__ __forceinline__ int grp_min(const Grp &g, int v) {
    for (int o = Grp::size() / 2; o > 0; o >>= 1)
        v = min(v, g.shfl_xor(v, o));
    return v;
}
template <class Grp, class T> __device__ __forceinline__ T grp_fmax(const Grp &g, T v) {
    for (int o = Grp::size() / 2; o > 0; o >>= 1)
        v = fmax(v, g.shfl_xor(v, o));
    return v;
}
template <class Grp> __device__ __forceinline__ int grp_inclusive_scan(const Grp &g, int v) {
    const int r = g.thread_rank();
    for (int o = 1; o < static_cast<int>(Grp::size()); o <<= 1) {
        const int t = g.shfl_up(v, o);
        if (r >= o)
            v += t;
    }
    return v;
}

// Ascending bitonic sort of a[0..N), N a power of two.
template <class Grp> __device__ void grp_bitonic_sort(const Grp &g, int *a, int N) {
    const int r = g.thread_rank();
    constexpr int GS = Grp::size();
    for (int size = 2; size <= N; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = r; t < (N >> 1); t += GS) {
                const int i = 2 * t - (t & (stride - 1));
                const int j = i + stride;
                const bool asc = (i & size) == 0;
                const int x = a[i], y = a[j];
                if ((x > y) == asc) {
                    a[i] = y;
                    a[j] = x;
                }
            }
            g.sync();
        }
    }
}

// In-place unique of sorted a[0..L) also dropping members of sorted ex[0..ne). Returns count.
template <class Grp> __device__ int grp_unique_except(const Grp &g, int *a, int L, const int *ex, int ne) {
    const int r = g.thread_rank();
    constexpr int GS = Grp::size();
    int out = 0;
    int prev_carry = INT_MIN;
    for (int base = 0; base < L; base += GS) {
        const int t = base + r;
        int val = 0;
        bool keep = false;
        if (t < L) {
            val = a[t];
            const int prev = t == 0 ? INT_MIN : (r == 0 ? prev_carry : a[t - 1]);
            keep = (t == 0 || val != prev);
            if (keep && ne > 0) {
                int lo = 0, hi = ne;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (ex[mid] < val)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                keep = !(lo < ne && ex[lo] == val);
            }
        }
        const int last_in_chunk = min(L, base + GS) - 1;
        prev_carry = a[last_in_chunk];
        g.sync();
        const unsigned bal = g.ballot(keep);
        if (keep)
            a[out + __popc(bal & ((1u << r) - 1))] = val;
        out += __popc(bal);
        g.sync();
    }
    return out;
}

__device__ __forceinline__ int lower_bound_int(const int *a, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Record of every fit (the per-fit history of the reference's SpaiColumn,
// include/bspai/spai.hpp:37-55) for diagnostics on small systems: two append-only streams, ints
// and binary64 values, written by the column kernel when `ints` is set. Every record starts with
// 8 ints: kind, column k, workspace tier, fit ordinal (0-based), a, b, c, offset of its values.
//   kind 1 (fit):    a = |J|, b = |I|; ints J, I; values residual, pivot ratio, coefficients (|J|)
//   kind 2 (scores): a = candidates; ints candidates (in the fit's order: ascending in exact
//                    mode); values mean score, scores (one per candidate)
//   kind 3 (selection): a = selected; ints the selection in selection order
// A column refitted from scratch in a larger tier logs again with the higher tier number; records
// of earlier tiers belong to abandoned attempts.
struct FitLog {
    int *ints;
    double *vals;
    unsigned long long *top; // [0] ints, [1] values appended (may exceed the capacities)
    long long int_cap, val_cap;
    int tier;
};

template <class T> struct ColumnArgs {
    int n;
    const int *rp, *ci;
    const T *av;
    const int *tp, *ti;
    const T *d;
    T eps;
    long long alpha;
    int beta;
    // per-column outputs
    int *status, *fits, *growths, *clamps, *qsize;
    T *residual;
    long long *out_off;
    int *packed_idx;
    T *packed_val;
    unsigned long long *packed_top;
    unsigned long long packed_cap;
    int *error;        // bit0 packed output full, bit1 column exceeded the largest workspace
    unsigned long long *phase; // optional cycle counters per fit phase (tuning aid), nullptr = off
    int dyn_scores;            // hand candidates out dynamically (heavy-tailed row lengths)
    FitLog log;                // optional record of every fit (ints == nullptr: off)
};

// Appends one record to the fit log (lane 0): reserves `nints` ints (header included) and `nvals`
// values; io / vo are their offsets, -1 when the log is full (the host sees top > capacity).
__device__ __forceinline__ void fit_log_reserve(const FitLog &L, int nints, int nvals, long long &io,
                                                long long &vo) {
    io = static_cast<long long>(atomicAdd(&L.top[0], static_cast<unsigned long long>(nints)));
    vo = static_cast<long long>(atomicAdd(&L.top[1], static_cast<unsigned long long>(nvals)));
    if (io + nints > L.int_cap || vo + nvals > L.val_cap)
        io = vo = -1;
}

// Cycle accounting of a fit by phase (lane 0's clock; only when ColumnArgs::phase is set).
enum FitPhase : int {
    kPhShadow = 0, kPhQr, kPhResidual, kPhCandidates, kPhScores, kPhSelect, kPhQrNorms, kPhQrUpdate, kPhCount
};
struct PhaseClock {
    unsigned long long *out;
    long long t = 0;
    unsigned long long acc[kPhCount] = {0, 0, 0, 0, 0, 0, 0, 0};
    __device__ explicit PhaseClock(unsigned long long *o) : out(o) {
        if (out)
            t = clock64();
    }
    __device__ void mark(int ph) {
        if (out) {
            const long long now = clock64();
            acc[ph] += static_cast<unsigned long long>(now - t);
            t = now;
        }
    }
    __device__ void commit(int lane) {
        if (out && lane == 0)
            for (int i = 0; i < kPhCount; ++i)
                atomicAdd(out + i, acc[i]);
    }
};

// Columns one launch of the column kernel takes, and where its misfits go. Workspace tiers form a
// chain: the first launch takes every column; each later launch takes the previous launch's
// misfits with a larger workspace per group; the last (global-memory) tier has no out list, so a
// misfit there is an error.
struct TierIo {
    const int *in_list;  // nullptr: columns 0..n-1
    const int *in_count; // size of in_list (device)
    int *next;           // take counter
    int *out_list;       // misfits (nullptr: error)
    int *out_count;
};

// Gather the dense reduced matrix R = B(I, J) (row-major m x q): R[i*q+jj] = A(J[jj], I[i]) d_J.
template <class Grp, class T>
__device__ void gather_reduced(const Grp &g, const ColumnArgs<T> &A, const int *J, int q,
                               const int *I, int m, T *R) {
    const int r = g.thread_rank();
    constexpr int GS = Grp::size();
    for (long long t = r; t < static_cast<long long>(m) * q; t += GS)
        R[t] = T(0);
    g.sync();
    for (int jj = 0; jj < q; ++jj) {
        const int j = J[jj];
        const int b = A.rp[j], e = A.rp[j + 1];
        const T dj = A.d[j];
        for (int t = b + r; t < e; t += GS) {
            const int pos = lower_bound_int(I, m, A.ci[t]);
            R[static_cast<long long>(pos) * q + jj] = A.av[t] * dj;
        }
    }
    g.sync();
}

// Fast-mode 2-norm of x[0..m) (stride st): power-of-two scaling by the group max, then a group
// sum of squares. Overflow-safe; the summation order is a tree, not the reference's chain.
template <class Grp, class T>
__device__ T grp_norm(const Grp &g, const T *x, int m, long long stride) {
    constexpr int GS = Grp::size();
    T mx = 0;
    for (int i = g.thread_rank(); i < m; i += GS)
        mx = fmax(mx, fabs(x[i * stride]));
    mx = grp_fmax(g, mx);
    if (!(mx > T(0)) || !isfinite(mx))
        return mx > T(0) ? mx : T(0);
    const int e = ilogb(mx);
    T acc = 0;
    for (int i = g.thread_rank(); i < m; i += GS) {
        const T v = ldexp(x[i * stride], -e);
        acc += v * v;
    }
    for (int o = GS / 2; o > 0; o >>= 1)
        acc += g.shfl_xor(acc, o);
    return ldexp(sqrt(acc), e);
}

// Householder least squares with normalised reflectors, src/spai.cpp:30-98. R is destroyed,
// rhs is transformed, coef receives the solution. Returns a SpaiStatus code.
// The reference's left-to-right hypot chain over count elements (stride apart), one correctly
// rounded hypot per step, each step carrying the running value's exact square forward
// (norm_chain_step: bit-identical to cr_hypot). Measured alternatives on the 128^3 system, all
// slower: speculative and software-pipelined variants with the exactness test moved off the
// dependency path (465-541 ms against 388-401 ms for the whole SPAI), chains over the column's
// compacted nonzeros (443 ms: after the first reflectors the reduced columns are mostly filled
// in, so the ballot/compaction costs more than the skipped zero steps save), and an explicit
// one-ahead load of the next element (453 ms).
template <class T> __device__ __forceinline__ T norm_chain(const T *x, int count, int stride) {
    NormChain<T> st;
    for (int i = 0; i < count; ++i)
        norm_chain_step(st, x[static_cast<long long>(i) * stride]);
    return st.c;
}

template <bool FAST, class Grp, class T>
__device__ int grp_least_squares(const Grp &g, T *R, T *rhs, int m, int q, T *coef, T *v,
                                 T &pivot_ratio, PhaseClock *clk = nullptr) {
    const int lane = g.thread_rank();
    constexpr int GS = Grp::size();
    if (m < q)
        return kRankDeficient;
    // Infinity norm: sequential row sums, max over rows (max is order independent).
    T inf_norm = 0;
    for (int i = lane; i < m; i += GS) {
        T sum = 0;
        for (int j = 0; j < q; ++j)
            sum += fabs(R[static_cast<long long>(i) * q + j]);
        inf_norm = fmax(inf_norm, sum);
    }
    inf_norm = grp_fmax(g, inf_norm);
    T min_pivot = T(INFINITY);
    for (int j = 0; j < q; ++j) {
        T length = 0;
        if (FAST) {
            length = grp_norm(g, R + static_cast<long long>(j) * q + j, m - j, q);
        } else {
            if (lane == 0)
                length = norm_chain(R + static_cast<long long>(j) * q + j, m - j, q);
            length = g.shfl(length, 0);
        }
        if (!isfinite(length))
            return kNumericalFailure;
        if (length == T(0))
            return kRankDeficient;
        const T x0 = R[static_cast<long long>(j) * q + j];
        const T diagonal = -copysign(length, x0);
        for (int i = j + lane; i < m; i += GS)
            v[i - j] = R[static_cast<long long>(i) * q + j] / length;
        g.sync();
        T vnorm = 0;
        if (FAST) {
            // |v|^2 = sum (x_i/L)^2 + 2|x_0|/L + 1 = 2 (1 + |x_0|/L) for the shifted reflector.
            if (lane == 0)
                v[0] += copysign(T(1), v[0]);
            vnorm = sqrt(T(2) * (T(1) + fabs(x0) / length));
        } else {
            if (lane == 0) {
                v[0] += copysign(T(1), v[0]);
                vnorm = norm_chain(v, m - j, 1);
            }
            vnorm = g.shfl(vnorm, 0);
        }
        g.sync();
        for (int i = lane; i < m - j; i += GS)
            v[i] /= vnorm;
        g.sync();
        if (clk)
            clk->mark(kPhQrNorms);
        // Columns j..q-1 of R and the right-hand side (as column q) in parallel, one per lane.
        int bad = 0;
        for (int col = j + lane; col <= q; col += GS) {
            T dot = 0;
            if (col < q) {
                for (int i = j; i < m; ++i)
                    dot += v[i - j] * R[static_cast<long long>(i) * q + col];
                for (int i = j; i < m; ++i) {
                    T &rr = R[static_cast<long long>(i) * q + col];
                    rr -= 2 * v[i - j] * dot;
                    bad |= !isfinite(rr);
                }
            } else {
                for (int i = j; i < m; ++i)
                    dot += v[i - j] * rhs[i];
                for (int i = j; i < m; ++i) {
                    rhs[i] -= 2 * v[i - j] * dot;
                    bad |= !isfinite(rhs[i]);
                }
            }
        }
        if (g.any(bad))
            return kNumericalFailure;
        g.sync();
        if (clk)
            clk->mark(kPhQrUpdate);
        if (lane == 0)
            R[static_cast<long long>(j) * q + j] = diagonal;
        g.sync();
        min_pivot = fmin(min_pivot, fabs(diagonal));
    }
    pivot_ratio = inf_norm == T(0) ? T(0) : min_pivot / inf_norm;
    int st = kSuccess;
    if (lane == 0) {
        for (int j = q - 1; j >= 0; --j) {
            T value = rhs[j];
            for (int k = j + 1; k < q; ++k)
                value -= R[static_cast<long long>(j) * q + k] * coef[k];
            const T diagonal = R[static_cast<long long>(j) * q + j];
            if (!isfinite(diagonal)) {
                st = kNumericalFailure;
                break;
            }
            if (diagonal == T(0)) {
                st = kRankDeficient;
                break;
            }
            coef[j] = value / diagonal;
            if (!isfinite(coef[j])) {
                st = kNumericalFailure;
                break;
            }
        }
    }
    st = g.shfl(st, 0);
    g.sync();
    return st;
}

// Score guard, src/spai.cpp:273-306 (u = 2^-53) and its float instantiation (u = 2^-24).
template <class T> __device__ int score_value(T rsq, T dot, T den, T &score, int &clamped) {
    clamped = 0;
    score = 0;
    if (!isfinite(rsq) || !isfinite(dot) || !isfinite(den))
        return kNumericalFailure;
    if (den == T(0))
        return kZeroDenominator;
    if (rsq < T(0) || den < T(0))
        return kInvalidScore;
    const T quotient = dot * dot / den;
    T delta = rsq - quotient;
    const T bound = T(32) * Unit<T>::u() * (rsq + fabs(quotient));
    if (!isfinite(quotient) || !isfinite(delta) || !isfinite(bound))
        return kNumericalFailure;
    if (delta < T(0)) {
        if (-delta > bound)
            return kInvalidScore;
        delta = 0;
        clamped = 1;
    }
    score = sqrt(delta);
    return kSuccess;
}

template <class T>
__global__ void score_kat_kernel(T rsq, T dot, T den, double *out) {
    T s;
    int c;
    const int st = score_value<T>(rsq, dot, den, s, c);
    out[0] = st;
    out[1] = static_cast<double>(s);
    out[2] = c;
}

// One adaptive column (src/spai.cpp:100-244). Returns a final SpaiStatus or kOverflow when the
// workspace (ws, cap bytes; J capacity qcap) is too small for this column.
template <bool FAST, bool LOG, class Grp, class T>
__device__ int fit_column(const Grp &g, const ColumnArgs<T> &A, int k, char *ws, size_t cap, int qcap) {
    const int lane = g.thread_rank();
    constexpr int GS = Grp::size();
    int *J = reinterpret_cast<int *>(ws);
    int *lastJ = J + qcap;
    T *lastC = reinterpret_cast<T *>(ws + ((static_cast<size_t>(2 * qcap) * 4 + 15) & ~size_t(15)));
    size_t head = ((static_cast<size_t>(2 * qcap) * 4 + 15) & ~size_t(15)) +
                  ((static_cast<size_t>(qcap) * sizeof(T) + 15) & ~size_t(15));
    if (head >= cap)
        return kOverflow;
    Bump bump{ws + head, cap - head, 0};
    int q = 1;
    if (lane == 0)
        J[0] = k;
    g.sync();
    int fits = 0, growths = 0, clamps = 0, lastq = 0;
    T last_res = T(NAN);
    int status = kNotAttempted;
    const T eps = A.eps;
    PhaseClock clk(A.phase);
    for (;;) {
        bump.reset(0);
        // ---- shadow I: union of the row patterns of A over J ----
        int L1 = 0;
        for (int t = lane; t < q; t += GS)
            L1 += A.rp[J[t] + 1] - A.rp[J[t]];
        L1 = grp_sum(g, L1);
        const int P1 = pow2_at_least(max(L1, 1));
        int *I = bump.take<int>(P1);
        if (!I)
            return kOverflow;
        {
            int off = 0;
            for (int jj = 0; jj < q; ++jj) {
                const int j = J[jj];
                const int b = A.rp[j], len = A.rp[j + 1] - b;
                for (int t = lane; t < len; t += GS)
                    I[off + t] = A.ci[b + t];
                off += len;
            }
            for (int t = L1 + lane; t < P1; t += GS)
                I[t] = INT_MAX;
            g.sync();
        }
        grp_bitonic_sort(g, I, P1);
        const int m = grp_unique_except(g, I, L1, static_cast<const int *>(nullptr), 0);
        bump.reset(static_cast<size_t>(m) * 4);
        clk.mark(kPhShadow);
        if (m < q) {
            status = kRankDeficient;
            break;
        }
        // Workspace of the fit: [I][R][rhs][v][coef]. The fitted residual s, which the candidate
        // phase needs, is moved next to I once R is consumed, so it does not add to the peak of the
        // least-squares phase (a column's last fit then fits a smaller workspace).
        const size_t ls_mark = bump.mark();
        T *R = bump.take<T>(static_cast<long long>(m) * q);
        T *rhs = bump.take<T>(m);
        T *v = bump.take<T>(m);
        T *coef = bump.take<T>(q);
        if (!R || !rhs || !v || !coef)
            return kOverflow;
        gather_reduced(g, A, J, q, I, m, R);
        for (int i = lane; i < m; i += GS)
            rhs[i] = I[i] == k ? T(1) : T(0);
        g.sync();
        T pivot_ratio = 0;
        clk.mark(kPhQr); // gather
        const int ls = grp_least_squares<FAST>(g, R, rhs, m, q, coef, v, pivot_ratio, &clk);
        clk.mark(kPhQr);
        if (ls != kSuccess) {
            status = ls;
            break;
        }
        // Fitted residual with the original reduced matrix (into v, free after the fit), then moved
        // to s right after I (over R's first rows: R is no longer needed; v lies beyond them).
        gather_reduced(g, A, J, q, I, m, R);
        int bad = 0;
        for (int i = lane; i < m; i += GS) {
            T acc = 0;
            for (int jj = 0; jj < q; ++jj)
                acc += R[static_cast<long long>(i) * q + jj] * coef[jj];
            acc -= (I[i] == k ? T(1) : T(0));
            v[i] = acc;
            bad |= !isfinite(acc);
        }
        if (g.any(bad)) {
            status = kNumericalFailure;
            break;
        }
        g.sync();
        bump.reset(ls_mark);
        T *s = bump.take<T>(m);
        const size_t keep_mark = bump.mark();
        for (int i = lane; i < m; i += GS)
            s[i] = v[i];
        g.sync();
        T res = 0;
        if (FAST) {
            res = grp_norm(g, s, m, 1);
        } else {
            if (lane == 0)
                res = norm_chain(s, m, 1);
            res = g.shfl(res, 0);
        }
        clk.mark(kPhResidual);
        if (!isfinite(res)) {
            status = kNumericalFailure;
            break;
        }
        if (fits != 0)
            ++growths;
        ++fits;
        lastq = q;
        last_res = res;
        for (int t = lane; t < q; t += GS) {
            lastJ[t] = J[t];
            lastC[t] = coef[t];
        }
        g.sync();
        if (LOG) {
            long long io = 0, vo = 0;
            if (lane == 0) {
                fit_log_reserve(A.log, 8 + q + m, 2 + q, io, vo);
                if (io >= 0) {
                    int *h = A.log.ints + io;
                    h[0] = 1, h[1] = k, h[2] = A.log.tier, h[3] = fits - 1;
                    h[4] = q, h[5] = m, h[6] = 0, h[7] = static_cast<int>(vo);
                    A.log.vals[vo] = static_cast<double>(res);
                    A.log.vals[vo + 1] = static_cast<double>(pivot_ratio);
                }
            }
            io = g.shfl(io, 0);
            vo = g.shfl(vo, 0);
            if (io >= 0) {
                for (int t = lane; t < q; t += GS) {
                    A.log.ints[io + 8 + t] = lastJ[t];
                    A.log.vals[vo + 2 + t] = static_cast<double>(lastC[t]);
                }
                for (int t = lane; t < m; t += GS)
                    A.log.ints[io + 8 + q + t] = I[t];
            }
        }
        if (res <= eps) {
            status = kSuccess;
            break;
        }
        if (static_cast<long long>(growths) == A.alpha) {
            status = kIterationLimit;
            break;
        }
        // ---- candidates: column patterns over I and k, minus J ----
        bump.reset(keep_mark);
        int L2 = 0;
        for (int t = lane; t < m; t += GS)
            L2 += A.tp[I[t] + 1] - A.tp[I[t]];
        L2 = grp_sum(g, L2) + (A.tp[k + 1] - A.tp[k]);
        int c = 0;
        int *C = nullptr;
        if (FAST) {
            // Unique candidates through an open-addressing set (load factor <= 2/3); the order of
            // the compacted list is irrelevant in this mode (parallel mean, index tie-break).
            const int P2 = pow2_at_least(max(3 * L2 / 2 + 1, 2));
            C = bump.take<int>(P2);
            if (!C)
                return kOverflow;
            for (int t = lane; t < P2; t += GS)
                C[t] = -1;
            g.sync();
            auto insert = [&](int x) {
                unsigned h = (static_cast<unsigned>(x) * 2654435761u) & static_cast<unsigned>(P2 - 1);
                for (int probe = 0; probe < P2; ++probe) {
                    const int prev = atomicCAS(&C[h], -1, x);
                    if (prev == -1 || prev == x)
                        return;
                    h = (h + 1) & static_cast<unsigned>(P2 - 1);
                }
            };
            for (int t = 0; t < m; ++t) {
                const int b = A.tp[I[t]], e = A.tp[I[t] + 1];
                for (int x = b + lane; x < e; x += GS)
                    insert(A.ti[x]);
            }
            for (int x = A.tp[k] + lane; x < A.tp[k + 1]; x += GS)
                insert(A.ti[x]);
            g.sync();
            // Compact in place, dropping empty slots and members of J.
            int out = 0;
            for (int base = 0; base < P2; base += GS) {
                const int t = base + lane;
                int val = t < P2 ? C[t] : -1;
                bool keep = val >= 0;
                if (keep) {
                    const int pos = lower_bound_int(J, q, val);
                    keep = !(pos < q && J[pos] == val);
                }
                g.sync();
                const unsigned bal = g.ballot(keep);
                if (keep)
                    C[out + __popc(bal & ((1u << lane) - 1))] = val;
                out += __popc(bal);
                g.sync();
            }
            c = out;
        } else {
        const int P2 = pow2_at_least(max(L2, 1));
        C = bump.take<int>(P2);
        if (!C)
            return kOverflow;
        {
            int base_off = 0;
            for (int base = 0; base < m; base += GS) {
                const int t = base + lane;
                int len = 0, b = 0;
                if (t < m) {
                    b = A.tp[I[t]];
                    len = A.tp[I[t] + 1] - b;
                }
                const int incl = grp_inclusive_scan(g, len);
                const int start = base_off + incl - len;
                for (int x = 0; x < len; ++x)
                    C[start + x] = A.ti[b + x];
                base_off += g.shfl(incl, GS - 1);
            }
            const int b = A.tp[k], len = A.tp[k + 1] - b;
            for (int x = lane; x < len; x += GS)
                C[base_off + x] = A.ti[b + x];
            for (int t = L2 + lane; t < P2; t += GS)
                C[t] = INT_MAX;
            g.sync();
        }
        grp_bitonic_sort(g, C, P2);
        c = grp_unique_except(g, C, L2, J, q);
        }
        clk.mark(kPhCandidates);
        if (c == 0) {
            status = kEmptyCandidates;
            break;
        }
        bump.reset(keep_mark + ((static_cast<size_t>(c) * 4 + 15) & ~size_t(15)));
        T *sc = bump.take<T>(c);
        const int nsel_cap = min(A.beta, c);
        int *sel = bump.take<int>(max(nsel_cap, 1));
        if (!sc || !sel)
            return kOverflow;
        // ---- scores: each candidate's dot/den by one lane in row (ascending shadow) order ----
        // Short uniform rows (stencils): lanes take candidates round-robin. Heavy-tailed rows
        // (dyn_scores): candidates are handed out dynamically, a lane that finishes a row taking
        // the next unassigned one, so long rows do not leave the group's other lanes idle (rows
        // are walked 16 entries per round). The arithmetic per candidate is the same either way.
        const T rsq = res * res;
        int first_fail = INT_MAX, my_status = kSuccess, my_clamps = 0;
        for (int t = lane; t < c && !A.dyn_scores; t += GS) {
            const int j = C[t];
            const int b = A.rp[j], e = A.rp[j + 1];
            const T dj = A.d[j];
            T dot = 0, den = 0;
            for (int x = b; x < e; ++x) {
                const int col = A.ci[x];
                const int pos = lower_bound_int(I, m, col);
                if (pos < m && I[pos] == col) {
                    const T value = A.av[x] * dj;
                    dot += s[pos] * value;
                    den += value * value;
                }
            }
            T score;
            int clamped;
            const int st = score_value<T>(rsq, dot, den, score, clamped);
            sc[t] = score;
            if (st != kSuccess && (FAST ? j : t) < first_fail) {
                first_fail = FAST ? j : t;
                my_status = st;
            }
            if (st == kSuccess && clamped)
                my_clamps += 1;
        }
        int next = 0; // first unassigned candidate (the same in every lane)
        int t = -1, x = 0, xe = 0, j = 0;
        T dj = 0, dot = 0, den = 0;
        for (; A.dyn_scores;) {
            const unsigned want = g.ballot(t < 0);
            if (t < 0) {
                const int cand = next + __popc(want & ((1u << lane) - 1u));
                if (cand < c) {
                    t = cand;
                    j = C[t];
                    x = A.rp[j];
                    xe = A.rp[j + 1];
                    dj = A.d[j];
                    dot = 0;
                    den = 0;
                }
            }
            next += __popc(want);
            if (!g.any(t >= 0))
                break;
            if (t < 0)
                continue;
            const int stop = min(xe, x + 16);
            for (; x < stop; ++x) {
                const int col = A.ci[x];
                const int pos = lower_bound_int(I, m, col);
                if (pos < m && I[pos] == col) {
                    const T value = A.av[x] * dj;
                    dot += s[pos] * value;
                    den += value * value;
                }
            }
            if (x < xe)
                continue;
            T score;
            int clamped;
            const int st = score_value<T>(rsq, dot, den, score, clamped);
            sc[t] = score;
            if (st != kSuccess && (FAST ? j : t) < first_fail) {
                first_fail = FAST ? j : t;
                my_status = st;
            }
            if (st == kSuccess && clamped)
                my_clamps += 1;
            t = -1;
        }
        const int ff = grp_min(g, first_fail);
        if (ff != INT_MAX) {
            const unsigned owner = g.ballot(first_fail == ff);
            status = g.shfl(my_status, __ffs(owner) - 1);
            break;
        }
        clamps += grp_sum(g, my_clamps);
        g.sync();
        T mean = 0;
        if (FAST) {
            for (int t = lane; t < c; t += GS)
                mean += sc[t];
            for (int o = GS / 2; o > 0; o >>= 1)
                mean += g.shfl_xor(mean, o);
            mean = mean / static_cast<T>(c);
        } else {
            if (lane == 0) {
                for (int t = 0; t < c; ++t)
                    mean += sc[t];
                mean = mean / static_cast<T>(c);
            }
            mean = g.shfl(mean, 0);
        }
        clk.mark(kPhScores);
        if (!isfinite(mean)) {
            status = kNumericalFailure;
            break;
        }
        if (LOG) {
            long long io = 0, vo = 0;
            if (lane == 0) {
                fit_log_reserve(A.log, 8 + c, 1 + c, io, vo);
                if (io >= 0) {
                    int *h = A.log.ints + io;
                    h[0] = 2, h[1] = k, h[2] = A.log.tier, h[3] = fits - 1;
                    h[4] = c, h[5] = 0, h[6] = 0, h[7] = static_cast<int>(vo);
                    A.log.vals[vo] = static_cast<double>(mean);
                }
            }
            io = g.shfl(io, 0);
            vo = g.shfl(vo, 0);
            if (io >= 0)
                for (int t = lane; t < c; t += GS) {
                    A.log.ints[io + 8 + t] = C[t];
                    A.log.vals[vo + 1 + t] = static_cast<double>(sc[t]);
                }
            g.sync();
        }
        // ---- selection: up to beta smallest (score, index) with score <= mean ----
        int nsel = 0;
        for (; nsel < nsel_cap; ++nsel) {
            T best = T(INFINITY);
            int best_t = INT_MAX;
            // Ties go to the smaller candidate index (C is sorted in exact mode, so this is the
            // reference's stable (score, index) order; in fast mode C is unordered).
            int best_c = INT_MAX;
            for (int t = lane; t < c; t += GS) {
                const T x = sc[t];
                if (x <= mean && (x < best || (x == best && C[t] < best_c))) {
                    best = x;
                    best_t = t;
                    best_c = C[t];
                }
            }
            for (int o = GS / 2; o > 0; o >>= 1) {
                const T ob = g.shfl_xor(best, o);
                const int ot = g.shfl_xor(best_t, o);
                const int oc = g.shfl_xor(best_c, o);
                if (ob < best || (ob == best && oc < best_c)) {
                    best = ob;
                    best_t = ot;
                    best_c = oc;
                }
            }
            if (best_t == INT_MAX)
                break;
            if (lane == 0) {
                sel[nsel] = C[best_t];
                sc[best_t] = T(INFINITY); // consumed
            }
            g.sync();
        }
        if (LOG && lane == 0) {
            long long io = 0, vo = 0;
            fit_log_reserve(A.log, 8 + nsel, 0, io, vo);
            if (io >= 0) {
                int *h = A.log.ints + io;
                h[0] = 3, h[1] = k, h[2] = A.log.tier, h[3] = fits - 1;
                h[4] = nsel, h[5] = 0, h[6] = 0, h[7] = static_cast<int>(vo);
                for (int t = 0; t < nsel; ++t)
                    h[8 + t] = sel[t];
            }
        }
        if (nsel == 0) {
            status = kNoGrowth;
            break;
        }
        if (q + nsel > qcap)
            return kOverflow;
        // J <- sort(J u selected): merge two sorted lists (selected are distinct from J).
        if (lane == 0) {
            for (int a = 1; a < nsel; ++a) { // insertion sort of the few selected indices
                const int x = sel[a];
                int b = a - 1;
                while (b >= 0 && sel[b] > x) {
                    sel[b + 1] = sel[b];
                    --b;
                }
                sel[b + 1] = x;
            }
            int a = q - 1, b = nsel - 1, w = q + nsel - 1;
            while (b >= 0) {
                if (a >= 0 && J[a] > sel[b])
                    J[w--] = J[a--];
                else
                    J[w--] = sel[b--];
            }
        }
        q += nsel;
        g.sync();
        clk.mark(kPhSelect);
    }
    clk.commit(lane);
    // ---- publish the last completed fit (column.pattern/coefficients) ----
    long long off = 0;
    if (lane == 0) {
        off = static_cast<long long>(atomicAdd(A.packed_top, static_cast<unsigned long long>(lastq)));
        if (static_cast<unsigned long long>(off) + lastq > A.packed_cap) {
            atomicOr(A.error, 1);
            off = -1;
        }
        A.status[k] = status;
        A.fits[k] = fits;
        A.growths[k] = growths;
        A.clamps[k] = clamps;
        A.qsize[k] = lastq;
        A.residual[k] = last_res;
        A.out_off[k] = off;
    }
    off = g.shfl(off, 0);
    if (off >= 0)
        for (int t = lane; t < lastq; t += GS) {
            A.packed_idx[off + t] = lastJ[t];
            A.packed_val[off + t] = lastC[t];
        }
    return status;
}

// Persistent column kernel with G lanes per column (32/G columns per warp): groups take columns
// from io (all columns, or the previous tier's misfits) with a workspace of ws_bytes per group in
// shared memory (gws == nullptr) or in global memory (gws + group * ws_bytes).
// LOG: the build records every fit (FitLog); a separate instantiation, so the production kernels
// carry no logging code.
template <class T, int G, bool FAST, bool LOG>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 512 : 768)
    spai_columns_kernel(ColumnArgs<T> A, TierIo io, size_t ws_bytes, int qcap, char *gws) {
    extern __shared__ __align__(16) char smem[];
    const auto g = cg::tiled_partition<G>(cg::this_thread_block());
    const int grp = threadIdx.x / G;
    const int ggrp = (blockIdx.x * blockDim.x + threadIdx.x) / G;
    char *ws = gws ? gws + static_cast<size_t>(ggrp) * ws_bytes : smem + static_cast<size_t>(grp) * ws_bytes;
    const int lane = g.thread_rank();
    const int total = io.in_list ? *io.in_count : A.n;
    for (;;) {
        int slot = 0;
        if (lane == 0)
            slot = atomicAdd(io.next, 1);
        slot = g.shfl(slot, 0);
        if (slot >= total)
            break;
        const int k = io.in_list ? io.in_list[slot] : slot;
        const int r = fit_column<FAST, LOG>(g, A, k, ws, ws_bytes, qcap);
        if (r == kOverflow && lane == 0) {
            if (io.out_list)
                io.out_list[atomicAdd(io.out_count, 1)] = k;
            else
                atomicOr(A.error, 2);
        }
        g.sync();
    }
}

// Assembly: P(k, j) = m_jk d_j (src/spai.cpp:351-373, src/cuda_spai.cu:417-427); exact zero
// coefficients are not stored (CsrMatrix::from_entries drops zero sums).
template <class T>
__global__ void count_p_kernel(int n, const int *__restrict__ qsize,
                               const long long *__restrict__ off, const T *__restrict__ pv,
                               int *__restrict__ cnt) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int c = 0;
        const long long o = off[k];
        if (o >= 0)
            for (int t = 0; t < qsize[k]; ++t)
                c += pv[o + t] != T(0);
        cnt[k + 1] = c;
    }
}
template <class T>
__global__ void fill_p_kernel(int n, const int *__restrict__ qsize, const long long *__restrict__ off,
                              const int *__restrict__ pidx, const T *__restrict__ pv,
                              const T *__restrict__ d, const int *__restrict__ prow,
                              int *__restrict__ pcol, T *__restrict__ pval, int *__restrict__ bad) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const long long o = off[k];
        if (o < 0)
            continue;
        int w = prow[k];
        for (int t = 0; t < qsize[k]; ++t) {
            const T coef = pv[o + t];
            if (coef == T(0))
                continue;
            const int j = pidx[o + t];
            const T value = coef * d[j];
            if (!isfinite(value) || value == T(0))
                atomicMin(bad, k);
            pcol[w] = j;
            pval[w] = value;
            ++w;
        }
    }
}
// First failing column (overall status is that column's status, src/spai.cpp:331-335).
__global__ void first_failure_kernel(int n, const int *__restrict__ status, int *__restrict__ out) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        if (status[k] != kSuccess)
            atomicMin(out, k);
}
template <class T>
__global__ void stats_kernel(int n, const int *__restrict__ fits, const int *__restrict__ growths,
                             unsigned long long *__restrict__ out) {
    unsigned long long f = 0, g = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        f += fits[k];
        g += growths[k];
    }
    atomicAdd(&out[0], f);
    atomicAdd(&out[1], g);
}

// ------------------------------------------------------------------------------------------
// Host driver.
// ------------------------------------------------------------------------------------------
// Launch the column kernel for a group width G with `threads` per block: persistent over the
// SMs (shared-memory workspace, at most max_blocks blocks) or exactly max_blocks blocks (global).
template <class T, int G, bool FAST, bool LOG>
void launch_columns_g(ColumnArgs<T> args, TierIo io, size_t ws, int qcap, char *gws, int threads,
                      long long max_blocks, int sms, cudaStream_t st) {
    long long blocks = max_blocks;
    size_t smem = 0;
    if (!gws) {
        smem = ws * static_cast<size_t>(threads / G);
        SPAI_CUDA(cudaFuncSetAttribute(spai_columns_kernel<T, G, FAST, LOG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem)));
        int per_sm = 0;
        SPAI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spai_columns_kernel<T, G, FAST, LOG>, threads, smem));
        blocks = std::min<long long>(max_blocks, static_cast<long long>(sms) * std::max(per_sm, 1));
    }
    spai_columns_kernel<T, G, FAST, LOG><<<static_cast<unsigned>(std::max<long long>(blocks, 1)), threads, smem, st>>>(
        args, io, ws, qcap, gws);
    SPAI_LAUNCH("spai_columns_kernel");
}
template <class T, bool FAST, bool LOG>
void launch_columns_f(int G, ColumnArgs<T> args, TierIo io, size_t ws, int qcap, char *gws, int threads,
                      long long max_blocks, int sms, cudaStream_t st) {
    switch (G) {
    case 4:
        launch_columns_g<T, 4, FAST, LOG>(args, io, ws, qcap, gws, threads, max_blocks, sms, st);
        break;
    case 8:
        launch_columns_g<T, 8, FAST, LOG>(args, io, ws, qcap, gws, threads, max_blocks, sms, st);
        break;
    case 16:
        launch_columns_g<T, 16, FAST, LOG>(args, io, ws, qcap, gws, threads, max_blocks, sms, st);
        break;
    default:
        launch_columns_g<T, 32, FAST, LOG>(args, io, ws, qcap, gws, threads, max_blocks, sms, st);
    }
}
template <class T>
void launch_columns(bool fast, int G, ColumnArgs<T> args, TierIo io, size_t ws, int qcap, char *gws, int threads,
                    long long max_blocks, int sms, cudaStream_t st) {
    if (fast)
        launch_columns_f<T, true, false>(G, args, io, ws, qcap, gws, threads, max_blocks, sms, st);
    else if (args.log.ints)
        launch_columns_f<T, false, true>(G, args, io, ws, qcap, gws, threads, max_blocks, sms, st);
    else
        launch_columns_f<T, false, false>(G, args, io, ws, qcap, gws, threads, max_blocks, sms, st);
}

// One workspace tier: group width, bytes per group, groups per block, pattern capacity, and
// whether the workspace is in global memory.
struct TierPlan {
    int G;
    size_t ws;
    int groups_per_block;
    int qcap;
    bool global;
};

// Tier chain from the sparsity profile: shared-memory workspaces doubling from the profile's
// first size while at least four groups still fit on an SM, then global-memory workspaces (1 MiB
// for 16 groups per SM, then 32 MiB). Keeping many groups resident matters more than where the
// workspace lives: a fit is a chain of dependent shared/global accesses, and with one group per
// SM every latency is exposed (measured on the 10^6 irregular system: a 224 KiB shared tier fitted
// about 1,300 columns/s, the 1 MiB global tier about 2,900 columns/s on larger columns). Columns
// that do not fit move up the chain and are fitted again from the start (fits are deterministic,
// so the result does not depend on the tier that completes a column).
inline std::vector<TierPlan> plan_tiers(size_t first_ws, int first_G, int max_threads, size_t smem_budget,
                                        int first_qcap, size_t elem = 4) {
    std::vector<TierPlan> tiers;
    // Pattern capacity by workspace: up to 1,536 values (6 KiB of binary32, 12 KiB of binary64)
    // the fits are small (a 3-D stencil column ends near 17-25 pattern entries), so 32 entries
    // keep the per-group header (J, last J, last coefficients) small; a column that outgrows it
    // moves up a tier.
    auto qcap_for = [elem](size_t ws) {
        const size_t vals = ws / elem;
        return vals <= 1536 ? 32 : (vals <= 4096 ? 64 : (vals <= 16384 ? 256 : 1024));
    };
    const size_t last_shared = smem_budget / 4;
    size_t ws = first_ws;
    int G = first_G;
    while (ws <= std::max(last_shared, first_ws)) {
        const int per_warp = 32 / G;
        int groups = static_cast<int>(std::min<size_t>(smem_budget / ws, static_cast<size_t>(max_threads / G)));
        groups = std::max(per_warp, (groups / per_warp) * per_warp);
        if (static_cast<size_t>(groups) * ws > smem_budget)
            break;
        tiers.push_back(TierPlan{G, ws, groups, tiers.empty() && first_qcap > 0 ? first_qcap : qcap_for(ws), false});
        ws *= 2;
        if (ws > 16384)
            G = std::max(G, 16);
    }
    tiers.push_back(TierPlan{32, size_t(1) << 20, 4, 4096, true});   // 1 MiB, 24 groups per SM (register limit)
    tiers.push_back(TierPlan{32, size_t(32) << 20, 1, 65536, true}); // 32 MiB, at most 512 groups
    return tiers;
}

// First-tier choice of the autotuner and its timings on the sample.
struct TuneChoice {
    int G = 0;          // 0: not tuned
    size_t ws = 0;
    double ms = 0, default_ms = 0;
};

// Autotuner for the SPAI's first workspace tier (lanes per column group, workspace bytes per
// group). Which pair is fastest depends on the sparsity profile: the workspace bounds how many
// groups stay resident, a column whose fit outgrows it is refitted from the start in the next
// tier, and wider groups shorten the parallel phases of a fit but leave more lanes idle in its
// sequential norm chains. The tuner runs the whole tier chain on an evenly spaced column sample
// for each candidate pair of the profile (the default first), times it with CUDA events and
// keeps the fastest; the choice is cached per profile (value type, size, row-length profile and
// the construction parameters) for the life of the process. Fits are deterministic, so the
// choice changes the speed of construction only, never its result. Samples: 49,152 columns for
// short rows, 8,192 for heavy-tailed rows (their fits cost about 200 times more), a quarter of
// the columns at most; matrices with fewer than 16,384 columns keep the default.
template <class T, class RunChain>
TuneChoice tune_first_tier(const DeviceCsr<T> &a, const SpaiParams &prm, bool heavy, int G_def, size_t ws_def,
                           int max_threads, size_t smem_budget, int sms, cudaStream_t st, ColumnArgs<T> args,
                           int *queue, int *err, unsigned long long *top, bool verbose, RunChain &run_chain) {
    (void)sms;
    const int n = a.n;
    const int S = std::min(heavy ? 8192 : 49152, n / 4);
    if (S < 4096)
        return TuneChoice{};
    using Key = std::tuple<int, int, int, int, int, double, long long, int>;
    static std::mutex mu;
    static std::map<Key, TuneChoice> cache;
    const Key key{static_cast<int>(sizeof(T)), prm.fast ? 1 : 0, n, a.nnz, a.max_row, prm.epsilon, prm.alpha,
                  prm.beta};
    {
        std::lock_guard<std::mutex> lock(mu);
        const auto it = cache.find(key);
        if (it != cache.end())
            return it->second;
    }
    std::vector<std::pair<int, size_t>> cands;
    if (heavy)
        cands = {{G_def, ws_def}, {32, 28672}, {16, 14336}, {32, 57344}, {8, 14336}};
    else if (sizeof(T) == 4)
        cands = {{G_def, ws_def}, {8, 4800}, {8, 4352}, {8, 4096}, {8, 3072}, {4, 3072}, {8, 6144}, {16, 10240}};
    else
        cands = {{G_def, ws_def}, {8, 10240}, {8, 9216}, {8, 8704}, {8, 8192}, {4, 8192}, {16, 12288}};
    args.phase = nullptr;
    DeviceArena mem; // sample list and global workspaces of the sample runs (freed on return)
    int *list = mem.alloc<int>(S);
    std::vector<int> h(S);
    for (int i = 0; i < S; ++i)
        h[i] = static_cast<int>(static_cast<long long>(i) * n / S);
    SPAI_CUDA(cudaMemcpyAsync(list, h.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SPAI_CUDA(cudaEventCreate(&e0));
    SPAI_CUDA(cudaEventCreate(&e1));
    TuneChoice best;
    double best_ms = INFINITY;
    for (size_t c = 0; c < cands.size(); ++c) {
        const int G = cands[c].first;
        const size_t ws = cands[c].second;
        if (ws > smem_budget || G * 4 > max_threads)
            continue;
        const std::vector<TierPlan> tiers = plan_tiers(ws, G, max_threads, smem_budget, 0, sizeof(T));
        SPAI_CUDA(cudaMemsetAsync(queue, 0, sizeof(int) * 64, st));
        SPAI_CUDA(cudaMemcpyAsync(&queue[62], &S, sizeof(int), cudaMemcpyHostToDevice, st));
        SPAI_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        SPAI_CUDA(cudaMemsetAsync(top, 0, sizeof(unsigned long long), st));
        SPAI_CUDA(cudaEventRecord(e0, st));
        int m0 = 0, gc = 0;
        run_chain(tiers, args, list, S, mem, false, m0, gc);
        SPAI_CUDA(cudaEventRecord(e1, st));
        SPAI_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        SPAI_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (verbose)
            std::fprintf(stderr, "spai tune: G=%d ws=%zu sample=%d  %.2f ms (first-tier misfits %d)\n", G, ws, S, ms, m0);
        if (c == 0)
            best.default_ms = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best.G = G;
            best.ws = ws;
            best.ms = ms;
        }
    }
    SPAI_CUDA(cudaEventDestroy(e0));
    SPAI_CUDA(cudaEventDestroy(e1));
    // The sample runs wrote per-column outputs and packed entries: the full run rewrites every
    // column, and the counters start again from zero.
    SPAI_CUDA(cudaMemsetAsync(queue, 0, sizeof(int) * 64, st));
    SPAI_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    SPAI_CUDA(cudaMemsetAsync(top, 0, sizeof(unsigned long long), st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = best;
    return best;
}

template <class T>
void SpaiBuilder<T>::construct(const DeviceCsr<T> &a, const SpaiParams &prm, cudaStream_t st,
                               SpaiOutput<T> &out, DeviceArena &arena) {
    const int n = a.n;
    const int nnz = a.nnz;
    out.n = n;
    out.status = kInvalidInput;
    out.first_failed = -1;
    out.launches = 0;
    if (n <= 0 || !(prm.epsilon > 0) || !std::isfinite(prm.epsilon) ||
        !(static_cast<T>(prm.epsilon) > T(0)))
        return;
    // Scaling.
    T *d = arena.alloc<T>(n);
    int *bad_row = arena.alloc<int>(1);
    const int big = INT_MAX;
    SPAI_CUDA(cudaMemcpyAsync(bad_row, &big, sizeof(int), cudaMemcpyHostToDevice, st));
    scale_rows_kernel<T><<<grid_for(n, 8, 152 * 64), 256, 0, st>>>(n, a.rp, a.ci, a.val, d, bad_row);
    SPAI_LAUNCH("scale_rows_kernel");
    ++out.launches;
    int h_bad = 0;
    SPAI_CUDA(cudaMemcpyAsync(&h_bad, bad_row, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    out.d = d;
    if (h_bad != INT_MAX)
        return; // invalid_input (zero diagonal / scaling range)
    // Column structure of A.
    int *tp = arena.alloc<int>(n + 1);
    int *ti = arena.alloc<int>(nnz > 0 ? nnz : 1);
    int *fill = arena.alloc<int>(n);
    SPAI_CUDA(cudaMemsetAsync(tp, 0, sizeof(int) * (n + 1), st));
    SPAI_CUDA(cudaMemsetAsync(fill, 0, sizeof(int) * n, st));
    column_count_kernel<<<grid_for(nnz, 256, 152 * 16), 256, 0, st>>>(nnz, a.ci, tp);
    SPAI_LAUNCH("column_count_kernel");
    size_t scan_bytes = 0;
    cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, tp, tp, n + 1, st);
    void *scan_tmp = arena.alloc<char>(scan_bytes + 16);
    cub::DeviceScan::InclusiveSum(scan_tmp, scan_bytes, tp, tp, n + 1, st);
    column_fill_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(n, a.rp, a.ci, tp, fill, ti);
    SPAI_LAUNCH("column_fill_kernel");
    out.launches += 3;
    // Outputs and queues.
    out.col_status = arena.alloc<int>(n);
    out.col_fits = arena.alloc<int>(n);
    out.col_growths = arena.alloc<int>(n);
    out.col_clamps = arena.alloc<int>(n);
    out.col_q = arena.alloc<int>(n);
    out.col_residual = arena.alloc<T>(n);
    long long *off = arena.alloc<long long>(n);
    int *queue = arena.alloc<int>(64);
    int *err = arena.alloc<int>(1);
    unsigned long long *top = arena.alloc<unsigned long long>(1);
    int *ovl = arena.alloc<int>(n);
    int *ovl2 = arena.alloc<int>(n);
    unsigned long long cap = std::max<unsigned long long>(static_cast<unsigned long long>(n) * 24ull, 1ull << 16);
    int *pidx = nullptr;
    T *pv = nullptr;
    // First workspace tier: an explicit override, else the autotuner's choice for this sparsity
    // profile (timed on a column sample, see tune_first_tier), else the profile default: short-row
    // matrices (stencils) use many small workspaces, heavy-tailed rows fewer, larger ones.
    const bool heavy = a.max_row > 48 || static_cast<double>(nnz) > 12.0 * n;
    const int G_def = heavy ? 16 : 8;
    const size_t ws_def = heavy ? 28672 : (sizeof(T) == 8 ? 12288 : 5120);
    int G0 = prm.group_lanes > 0 ? prm.group_lanes : G_def;
    size_t ws0 = prm.ws_bytes_per_warp > 0 ? static_cast<size_t>(prm.ws_bytes_per_warp) : ws_def;
    // Shared memory of one block: the device's per-block maximum (the kernel has no static shared
    // memory), less a small margin.
    size_t smem_budget = 225 * 1024;
    {
        int dev0 = 0, optin = 0;
        SPAI_CUDA(cudaGetDevice(&dev0));
        SPAI_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev0));
        if (optin > 64 * 1024)
            smem_budget = static_cast<size_t>(optin) - 256;
    }
    // Threads per block within the register budget of one block (124 registers/thread for
    // binary64, 77 for binary32 -> at most 512 / 768 threads).
    const int max_threads = sizeof(T) == 8 ? 512 : 768;
    if (ws0 > smem_budget)
        throw ArgumentError("SPAI workspace per group too large for one block's shared memory");
    out.tuned = false;
    out.tune_sample_ms = out.tune_default_ms = 0;
    int sms = 0, dev = 0;
    SPAI_CUDA(cudaGetDevice(&dev));
    SPAI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // SPAI_TRACE=1 prints the wall time and misfit count of each workspace tier to stderr.
    const bool trace = std::getenv("SPAI_TRACE") != nullptr;
    auto clock_ms = [] {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
    };
    // Runs a tier chain over a column list (in_list == nullptr: every column; otherwise `count`
    // columns listed in device memory, their count at queue[62]). Global-memory workspaces come
    // from ws_arena. Returns the misfits of the first tier and the columns that reached a global
    // tier.
    auto run_chain = [&](const std::vector<TierPlan> &tiers, ColumnArgs<T> args, const int *in_list, int count,
                         DeviceArena &ws_arena, bool verbose, int &misfits0, int &global_cols) {
        misfits0 = 0;
        global_cols = 0;
        int pending = count;
        int *lists[2] = {ovl, ovl2};
        for (size_t ti_ = 0; ti_ < tiers.size() && pending > 0; ++ti_) {
            const TierPlan &tp_ = tiers[ti_];
            const bool last = ti_ + 1 == tiers.size();
            int *out_list = last ? nullptr : lists[ti_ & 1];
            TierIo io{in_list, ti_ == 0 ? (in_list ? &queue[62] : nullptr) : &queue[2 * ti_ - 1], &queue[2 * ti_],
                      out_list, &queue[2 * ti_ + 1]};
            const double t0 = verbose ? clock_ms() : 0.0;
            const int threads = ((tp_.groups_per_block * tp_.G + 31) / 32) * 32;
            char *gws = nullptr;
            long long blocks = (static_cast<long long>(pending) + tp_.groups_per_block - 1) / tp_.groups_per_block;
            if (tp_.global) {
                const long long groups = std::min<long long>(pending, ti_ + 2 == tiers.size() ? sms * 24LL : 512LL);
                blocks = (groups + tp_.groups_per_block - 1) / tp_.groups_per_block;
                // one workspace for every launched group (blocks * groups_per_block >= groups)
                gws = ws_arena.alloc<char>(tp_.ws * static_cast<size_t>(blocks * tp_.groups_per_block));
                if (global_cols == 0)
                    global_cols = pending;
            }
            args.log.tier = static_cast<int>(ti_);
            launch_columns<T>(prm.fast, tp_.G, args, io, tp_.ws, tp_.qcap, gws, threads, blocks, sms, st);
            ++out.launches;
            int h_next = 0;
            if (!last) {
                SPAI_CUDA(cudaMemcpyAsync(&h_next, &queue[2 * ti_ + 1], sizeof(int), cudaMemcpyDeviceToHost, st));
            }
            SPAI_CUDA(cudaStreamSynchronize(st));
            if (verbose)
                std::fprintf(stderr, "spai tier %zu: G=%d ws=%zu%s groups/block=%d columns=%d  %.1f ms, misfits %d\n", ti_,
                             tp_.G, tp_.ws, tp_.global ? " (global)" : "", tp_.groups_per_block, pending,
                             clock_ms() - t0, h_next);
            if (ti_ == 0)
                misfits0 = h_next;
            pending = h_next;
            in_list = out_list;
        }
    };
    const bool want_tune = prm.tune && !prm.record && prm.group_lanes <= 0 && prm.ws_bytes_per_warp <= 0 &&
                           prm.first_qcap <= 0;
    out.log_ints = nullptr;
    out.log_vals = nullptr;
    out.log_top = nullptr;
    out.log_int_cap = out.log_val_cap = 0;
    if (prm.record && !prm.fast) { // the log follows the exact mode's fits
        const long long want = std::min<long long>(1LL << 28, std::max<long long>(1LL << 20, 64LL * (n + nnz)));
        out.log_int_cap = out.log_val_cap = want;
        out.log_ints = arena.alloc<int>(want);
        out.log_vals = arena.alloc<double>(want);
        out.log_top = arena.alloc<unsigned long long>(2);
    }
    for (int attempt = 0;; ++attempt) {
        pidx = arena.alloc<int>(cap);
        pv = arena.alloc<T>(cap);
        SPAI_CUDA(cudaMemsetAsync(queue, 0, sizeof(int) * 64, st));
        SPAI_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        SPAI_CUDA(cudaMemsetAsync(top, 0, sizeof(unsigned long long), st));
        unsigned long long *phase = nullptr;
        if (trace) {
            phase = arena.alloc<unsigned long long>(kPhCount);
            SPAI_CUDA(cudaMemsetAsync(phase, 0, sizeof(unsigned long long) * kPhCount, st));
        }
        ColumnArgs<T> args{n, a.rp, a.ci, a.val, tp, ti, d, static_cast<T>(prm.epsilon), prm.alpha,
                           prm.beta, out.col_status, out.col_fits, out.col_growths, out.col_clamps,
                           out.col_q, out.col_residual, off, pidx, pv, top, cap, err, phase, heavy ? 1 : 0};
        if (out.log_top)
            SPAI_CUDA(cudaMemsetAsync(out.log_top, 0, 2 * sizeof(unsigned long long), st));
        if (attempt == 0 && want_tune) {
            const TuneChoice c = tune_first_tier<T>(a, prm, heavy, G_def, ws_def, max_threads, smem_budget, sms, st,
                                                    args, queue, err, top, trace, run_chain);
            if (c.G > 0) {
                G0 = c.G;
                ws0 = c.ws;
                out.tuned = true;
                out.tune_sample_ms = c.ms;
                out.tune_default_ms = c.default_ms;
            }
        }
        args.log = FitLog{out.log_ints, out.log_vals, out.log_top, out.log_int_cap, out.log_val_cap, 0};
        const std::vector<TierPlan> tiers = plan_tiers(ws0, G0, max_threads, smem_budget, prm.first_qcap, sizeof(T));
        out.group_lanes = tiers[0].G;
        out.ws_bytes = static_cast<int>(tiers[0].ws);
        run_chain(tiers, args, nullptr, n, arena, trace, out.overflow_columns, out.overflow_columns_global);
        if (trace && phase) {
            unsigned long long hp[kPhCount];
            SPAI_CUDA(cudaMemcpy(hp, phase, sizeof(hp), cudaMemcpyDeviceToHost));
            double tot = 0;
            for (unsigned long long v : hp)
                tot += static_cast<double>(v);
            static const char *names[kPhCount] = {"shadow", "qr_other", "residual", "candidates",
                                                  "scores", "select", "qr_norms", "qr_update"};
            std::fprintf(stderr, "spai fit phases (lane-0 cycles, all tiers):");
            for (int i = 0; i < kPhCount; ++i)
                std::fprintf(stderr, " %s %.1f%%", names[i], tot > 0 ? 100.0 * hp[i] / tot : 0.0);
            std::fprintf(stderr, "\n");
        }
        int h_err = 0;
        SPAI_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
        if (h_err & 2)
            throw WorkspaceError("SPAI column exceeded the large fit workspace");
        if ((h_err & 1) == 0)
            break;
        if (attempt > 4)
            throw WorkspaceError("SPAI packed output capacity exhausted");
        cap *= 4; // packed pattern storage too small: rerun (deterministic) with more room
    }
    // Overall status: first failing column.
    int *first = arena.alloc<int>(1);
    SPAI_CUDA(cudaMemcpyAsync(first, &big, sizeof(int), cudaMemcpyHostToDevice, st));
    first_failure_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(n, out.col_status, first);
    SPAI_LAUNCH("first_failure_kernel");
    unsigned long long *stats = arena.alloc<unsigned long long>(2);
    SPAI_CUDA(cudaMemsetAsync(stats, 0, sizeof(unsigned long long) * 2, st));
    stats_kernel<T><<<grid_for(n, 256, 152 * 4), 256, 0, st>>>(n, out.col_fits, out.col_growths, stats);
    SPAI_LAUNCH("stats_kernel");
    // Assemble P.
    int *prow = arena.alloc<int>(n + 1);
    SPAI_CUDA(cudaMemsetAsync(prow, 0, sizeof(int) * (n + 1), st));
    count_p_kernel<T><<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(n, out.col_q, off, pv, prow);
    SPAI_LAUNCH("count_p_kernel");
    cub::DeviceScan::InclusiveSum(scan_tmp, scan_bytes, prow, prow, n + 1, st);
    out.launches += 4;
    int h_first = INT_MAX;
    int pnnz = 0;
    unsigned long long h_stats[2];
    SPAI_CUDA(cudaMemcpyAsync(&h_first, first, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaMemcpyAsync(&pnnz, prow + n, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaMemcpyAsync(h_stats, stats, sizeof(h_stats), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    out.fits = h_stats[0];
    out.growths = h_stats[1];
    out.p.n = n;
    out.p.nnz = pnnz;
    out.p.rp = prow;
    out.p.ci = arena.alloc<int>(pnnz > 0 ? pnnz : 1);
    out.p.val = arena.alloc<T>(pnnz > 0 ? pnnz : 1);
    int *pbad = arena.alloc<int>(1);
    SPAI_CUDA(cudaMemcpyAsync(pbad, &big, sizeof(int), cudaMemcpyHostToDevice, st));
    fill_p_kernel<T><<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(n, out.col_q, off, pidx, pv, d, prow,
                                                                 out.p.ci, out.p.val, pbad);
    SPAI_LAUNCH("fill_p_kernel");
    ++out.launches;
    int h_pbad = INT_MAX;
    SPAI_CUDA(cudaMemcpyAsync(&h_pbad, pbad, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    out.packed_idx = pidx;
    out.packed_val = pv;
    out.packed_off = off;
    if (h_first != INT_MAX) {
        int s = 0;
        SPAI_CUDA(cudaMemcpy(&s, out.col_status + h_first, sizeof(int), cudaMemcpyDeviceToHost));
        out.status = s;
        out.first_failed = h_first;
    } else {
        out.status = kSuccess;
    }
    if (h_pbad != INT_MAX) {
        // Assembly outside the binary range (spai.cpp:362-367) ends construction with
        // numerical_failure whatever any earlier column reported.
        out.status = kNumericalFailure;
        out.first_failed = h_pbad;
    }
}

template <class T> void score_kat(T rsq, T dot, T den, double *out) {
    double *dv = nullptr;
    SPAI_CUDA(cudaMalloc(&dv, 3 * sizeof(double)));
    score_kat_kernel<T><<<1, 1>>>(rsq, dot, den, dv);
    SPAI_LAUNCH("score_kat_kernel");
    SPAI_CUDA(cudaMemcpy(out, dv, 3 * sizeof(double), cudaMemcpyDeviceToHost));
    SPAI_CUDA(cudaFree(dv));
}

template struct SpaiBuilder<double>;
template struct SpaiBuilder<float>;
template void score_kat<double>(double, double, double, double *);
template void score_kat<float>(float, float, float, double *);

} // namespace spai

namespace spai {
__global__ void hypot_eval_kernel(int precision, long long count, const double *a, const double *b, double *out) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float af = static_cast<float>(a[i]), bf = static_cast<float>(b[i]);
        switch (precision) {
        case 0: out[i] = cr_hypot<double>(a[i], b[i]); break;
        case 1: out[i] = static_cast<double>(cr_hypot<float>(af, bf)); break;
        case 2: out[i] = norm_chain_step_from<double>(fabs(a[i]), b[i]); break;
        default: out[i] = static_cast<double>(norm_chain_step_from<float>(fabsf(af), bf)); break;
        }
    }
}
} // namespace spai

// The device hypot on host arrays (precision 0: binary64; 1: binary32 on the operands rounded to
// binary32, returned widened; 2 / 3: the binary64 / binary32 norm-chain step from the running
// norm |a|, which must return the same bits as 0 / 1). Check hook for the SPAI norm chains.
extern "C" int spai_hypot_device(int32_t precision, int64_t count, const double *a, const double *b, double *out) {
    if (count < 0 || (count > 0 && (!a || !b || !out)))
        return spai_api_fail(-1, "spai_hypot_device: bad arguments");
    if (count == 0)
        return 0;
    try {
        double *d = nullptr;
        const size_t bytes = sizeof(double) * static_cast<size_t>(count);
        SPAI_CUDA(cudaMalloc(&d, 3 * bytes));
        SPAI_CUDA(cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice));
        SPAI_CUDA(cudaMemcpy(d + count, b, bytes, cudaMemcpyHostToDevice));
        spai::hypot_eval_kernel<<<spai::grid_for(count, 256, 152 * 8), 256>>>(precision, count, d, d + count, d + 2 * count);
        const cudaError_t e = cudaGetLastError();
        SPAI_CUDA(cudaMemcpy(out, d + 2 * count, bytes, cudaMemcpyDeviceToHost));
        cudaFree(d);
        SPAI_CUDA(e);
    } catch (const std::exception &e) {
        return spai_api_fail(-2, e.what());
    }
    return 0;
}

extern "C" double spai_hypot(double a, double b) {
    return spai::cr_hypot<double>(a, b);
}
extern "C" float spai_hypotf(float a, float b) {
    return spai::cr_hypot<float>(a, b);
}
