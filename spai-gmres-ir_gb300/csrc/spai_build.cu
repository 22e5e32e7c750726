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

#include <cub/device/device_scan.cuh>

#include <algorithm>
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
// Warp-cooperative building blocks (all lanes of the warp call them together).
// ------------------------------------------------------------------------------------------
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

// Ascending bitonic sort of a[0..N), N a power of two.
__device__ void warp_bitonic_sort(int *a, int N) {
    const int lane = lane_id();
    for (int size = 2; size <= N; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < (N >> 1); t += 32) {
                const int i = 2 * t - (t & (stride - 1));
                const int j = i + stride;
                const bool asc = (i & size) == 0;
                const int x = a[i], y = a[j];
                if ((x > y) == asc) {
                    a[i] = y;
                    a[j] = x;
                }
            }
            __syncwarp();
        }
    }
}

// In-place unique of sorted a[0..L) also dropping members of sorted ex[0..ne). Returns count.
__device__ int warp_unique_except(int *a, int L, const int *ex, int ne) {
    const int lane = lane_id();
    int out = 0;
    int prev_carry = INT_MIN;
    for (int base = 0; base < L; base += 32) {
        const int t = base + lane;
        int val = 0;
        bool keep = false;
        if (t < L) {
            val = a[t];
            const int prev = t == 0 ? INT_MIN : (lane == 0 ? prev_carry : a[t - 1]);
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
        const int last_in_chunk = min(L, base + 32) - 1;
        prev_carry = a[last_in_chunk];
        __syncwarp();
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (keep)
            a[out + __popc(bal & ((1u << lane) - 1))] = val;
        out += __popc(bal);
        __syncwarp();
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
    int *queue;        // [0] next column (main pass), [1] overflow count, [2] next overflow
    int *overflow_list;
    int *error;        // bit0 packed output full, bit1 column exceeded the largest workspace
};

// Gather the dense reduced matrix R = B(I, J) (row-major m x q): R[i*q+jj] = A(J[jj], I[i]) d_J.
template <class T>
__device__ void gather_reduced(const ColumnArgs<T> &A, const int *J, int q, const int *I, int m,
                               T *R) {
    const int lane = lane_id();
    for (long long t = lane; t < static_cast<long long>(m) * q; t += 32)
        R[t] = T(0);
    __syncwarp();
    for (int jj = 0; jj < q; ++jj) {
        const int j = J[jj];
        const int b = A.rp[j], e = A.rp[j + 1];
        const T dj = A.d[j];
        for (int t = b + lane; t < e; t += 32) {
            const int pos = lower_bound_int(I, m, A.ci[t]);
            R[static_cast<long long>(pos) * q + jj] = A.av[t] * dj;
        }
    }
    __syncwarp();
}

// Householder least squares with normalised reflectors, src/spai.cpp:30-98. R is destroyed,
// rhs is transformed, coef receives the solution. Returns a SpaiStatus code.
template <class T>
__device__ int warp_least_squares(T *R, T *rhs, int m, int q, T *coef, T *v, T &pivot_ratio) {
    const int lane = lane_id();
    if (m < q)
        return kRankDeficient;
    // Infinity norm: sequential row sums, max over rows (max is order independent).
    T inf_norm = 0;
    for (int i = lane; i < m; i += 32) {
        T sum = 0;
        for (int j = 0; j < q; ++j)
            sum += fabs(R[static_cast<long long>(i) * q + j]);
        inf_norm = fmax(inf_norm, sum);
    }
    for (int o = 16; o > 0; o >>= 1)
        inf_norm = fmax(inf_norm, __shfl_xor_sync(0xffffffffu, inf_norm, o));
    T min_pivot = T(INFINITY);
    for (int j = 0; j < q; ++j) {
        T length = 0;
        if (lane == 0)
            for (int i = j; i < m; ++i)
                length = cr_hypot(length, R[static_cast<long long>(i) * q + j]);
        length = shfl(length, 0);
        if (!isfinite(length))
            return kNumericalFailure;
        if (length == T(0))
            return kRankDeficient;
        const T x0 = R[static_cast<long long>(j) * q + j];
        const T diagonal = -copysign(length, x0);
        for (int i = j + lane; i < m; i += 32)
            v[i - j] = R[static_cast<long long>(i) * q + j] / length;
        __syncwarp();
        T vnorm = 0;
        if (lane == 0) {
            v[0] += copysign(T(1), v[0]);
            for (int i = 0; i < m - j; ++i)
                vnorm = cr_hypot(vnorm, v[i]);
        }
        vnorm = shfl(vnorm, 0);
        __syncwarp();
        for (int i = lane; i < m - j; i += 32)
            v[i] /= vnorm;
        __syncwarp();
        // Columns j..q-1 of R and the right-hand side (as column q) in parallel, one per lane.
        int bad = 0;
        for (int col = j + lane; col <= q; col += 32) {
            T dot = 0;
            if (col < q) {
                for (int i = j; i < m; ++i)
                    dot += v[i - j] * R[static_cast<long long>(i) * q + col];
                for (int i = j; i < m; ++i) {
                    T &r = R[static_cast<long long>(i) * q + col];
                    r -= 2 * v[i - j] * dot;
                    bad |= !isfinite(r);
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
        if (__any_sync(0xffffffffu, bad))
            return kNumericalFailure;
        __syncwarp();
        if (lane == 0)
            R[static_cast<long long>(j) * q + j] = diagonal;
        __syncwarp();
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
    st = shfl(st, 0);
    __syncwarp();
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
template <class T>
__device__ int fit_column(const ColumnArgs<T> &A, int k, char *ws, size_t cap, int qcap) {
    const int lane = lane_id();
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
    __syncwarp();
    int fits = 0, growths = 0, clamps = 0, lastq = 0;
    T last_res = T(NAN);
    int status = kNotAttempted;
    const T eps = A.eps;
    for (;;) {
        bump.reset(0);
        // ---- shadow I: union of the row patterns of A over J ----
        int L1 = 0;
        for (int t = lane; t < q; t += 32)
            L1 += A.rp[J[t] + 1] - A.rp[J[t]];
        L1 = warp_sum_int(L1);
        const int P1 = pow2_at_least(max(L1, 1));
        int *I = bump.take<int>(P1);
        if (!I)
            return kOverflow;
        {
            int off = 0;
            for (int jj = 0; jj < q; ++jj) {
                const int j = J[jj];
                const int b = A.rp[j], len = A.rp[j + 1] - b;
                for (int t = lane; t < len; t += 32)
                    I[off + t] = A.ci[b + t];
                off += len;
            }
            for (int t = L1 + lane; t < P1; t += 32)
                I[t] = INT_MAX;
            __syncwarp();
        }
        warp_bitonic_sort(I, P1);
        const int m = warp_unique_except(I, L1, nullptr, 0);
        bump.reset(static_cast<size_t>(m) * 4);
        if (m < q) {
            status = kRankDeficient;
            break;
        }
        T *s = bump.take<T>(m);
        const size_t keep_mark = bump.mark();
        T *R = bump.take<T>(static_cast<long long>(m) * q);
        T *rhs = bump.take<T>(m);
        T *v = bump.take<T>(m);
        T *coef = bump.take<T>(q);
        if (!s || !R || !rhs || !v || !coef)
            return kOverflow;
        gather_reduced(A, J, q, I, m, R);
        for (int i = lane; i < m; i += 32)
            rhs[i] = I[i] == k ? T(1) : T(0);
        __syncwarp();
        T pivot_ratio = 0;
        const int ls = warp_least_squares(R, rhs, m, q, coef, v, pivot_ratio);
        if (ls != kSuccess) {
            status = ls;
            break;
        }
        // Fitted residual with the original reduced matrix.
        gather_reduced(A, J, q, I, m, R);
        int bad = 0;
        for (int i = lane; i < m; i += 32) {
            T acc = 0;
            for (int jj = 0; jj < q; ++jj)
                acc += R[static_cast<long long>(i) * q + jj] * coef[jj];
            acc -= (I[i] == k ? T(1) : T(0));
            s[i] = acc;
            bad |= !isfinite(acc);
        }
        if (__any_sync(0xffffffffu, bad)) {
            status = kNumericalFailure;
            break;
        }
        __syncwarp();
        T res = 0;
        if (lane == 0)
            for (int i = 0; i < m; ++i)
                res = cr_hypot(res, s[i]);
        res = shfl(res, 0);
        if (!isfinite(res)) {
            status = kNumericalFailure;
            break;
        }
        if (fits != 0)
            ++growths;
        ++fits;
        lastq = q;
        last_res = res;
        for (int t = lane; t < q; t += 32) {
            lastJ[t] = J[t];
            lastC[t] = coef[t];
        }
        __syncwarp();
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
        for (int t = lane; t < m; t += 32)
            L2 += A.tp[I[t] + 1] - A.tp[I[t]];
        L2 = warp_sum_int(L2) + (A.tp[k + 1] - A.tp[k]);
        const int P2 = pow2_at_least(max(L2, 1));
        int *C = bump.take<int>(P2);
        if (!C)
            return kOverflow;
        {
            int base_off = 0;
            for (int base = 0; base < m; base += 32) {
                const int t = base + lane;
                int len = 0, b = 0;
                if (t < m) {
                    b = A.tp[I[t]];
                    len = A.tp[I[t] + 1] - b;
                }
                const int incl = warp_inclusive_scan(len);
                const int start = base_off + incl - len;
                for (int x = 0; x < len; ++x)
                    C[start + x] = A.ti[b + x];
                base_off += shfl(incl, 31);
            }
            const int b = A.tp[k], len = A.tp[k + 1] - b;
            for (int x = lane; x < len; x += 32)
                C[base_off + x] = A.ti[b + x];
            for (int t = L2 + lane; t < P2; t += 32)
                C[t] = INT_MAX;
            __syncwarp();
        }
        warp_bitonic_sort(C, P2);
        const int c = warp_unique_except(C, L2, J, q);
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
        // ---- scores: one lane per candidate, ascending shadow order ----
        const T rsq = res * res;
        int first_fail = INT_MAX, my_status = kSuccess, my_clamps = 0;
        for (int t = lane; t < c; t += 32) {
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
            if (st != kSuccess && t < first_fail) {
                first_fail = t;
                my_status = st;
            }
            if (st == kSuccess && clamped)
                my_clamps += 1;
        }
        const int ff = warp_min_int(first_fail);
        if (ff != INT_MAX) {
            const unsigned owner = __ballot_sync(0xffffffffu, first_fail == ff);
            status = shfl(my_status, __ffs(owner) - 1);
            break;
        }
        clamps += warp_sum_int(my_clamps);
        __syncwarp();
        T mean = 0;
        if (lane == 0) {
            for (int t = 0; t < c; ++t)
                mean += sc[t];
            mean = mean / static_cast<T>(c);
        }
        mean = shfl(mean, 0);
        if (!isfinite(mean)) {
            status = kNumericalFailure;
            break;
        }
        // ---- selection: up to beta smallest (score, index) with score <= mean ----
        int nsel = 0;
        for (; nsel < nsel_cap; ++nsel) {
            T best = T(INFINITY);
            int best_t = INT_MAX;
            for (int t = lane; t < c; t += 32) {
                const T x = sc[t];
                if (x <= mean && (x < best || (x == best && t < best_t))) {
                    best = x;
                    best_t = t;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const T ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int ot = __shfl_xor_sync(0xffffffffu, best_t, o);
                if (ob < best || (ob == best && ot < best_t)) {
                    best = ob;
                    best_t = ot;
                }
            }
            if (best_t == INT_MAX)
                break;
            if (lane == 0) {
                sel[nsel] = C[best_t];
                sc[best_t] = T(INFINITY); // consumed
            }
            __syncwarp();
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
        __syncwarp();
    }
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
    off = shfl(off, 0);
    if (off >= 0)
        for (int t = lane; t < lastq; t += 32) {
            A.packed_idx[off + t] = lastJ[t];
            A.packed_val[off + t] = lastC[t];
        }
    return status;
}

// Persistent column kernel. mode 0: all columns via the atomic queue, shared-memory workspace
// of ws_bytes per warp; columns that do not fit go to the overflow list. mode 1: the overflow
// list, global workspace gws of ws_bytes per warp.
template <class T>
__global__ void spai_columns_kernel(ColumnArgs<T> A, int mode, size_t ws_bytes, int qcap,
                                    char *gws) {
    extern __shared__ __align__(16) char smem[];
    const int warp = threadIdx.x >> 5;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    char *ws = mode == 0 ? smem + static_cast<size_t>(warp) * ws_bytes
                         : gws + static_cast<size_t>(gwarp) * ws_bytes;
    const int lane = lane_id();
    for (;;) {
        int slot = 0;
        if (lane == 0)
            slot = atomicAdd(mode == 0 ? &A.queue[0] : &A.queue[2], 1);
        slot = shfl(slot, 0);
        int k;
        if (mode == 0) {
            if (slot >= A.n)
                break;
            k = slot;
        } else {
            if (slot >= A.queue[1])
                break;
            k = A.overflow_list[slot];
        }
        const int r = fit_column(A, k, ws, ws_bytes, qcap);
        if (r == kOverflow && lane == 0) {
            if (mode == 0)
                A.overflow_list[atomicAdd(&A.queue[1], 1)] = k;
            else
                atomicOr(A.error, 2);
        }
        __syncwarp();
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
    int *queue = arena.alloc<int>(4);
    int *err = arena.alloc<int>(1);
    unsigned long long *top = arena.alloc<unsigned long long>(1);
    int *ovl = arena.alloc<int>(n);
    unsigned long long cap = std::max<unsigned long long>(static_cast<unsigned long long>(n) * 24ull, 1ull << 16);
    int *pidx = nullptr;
    T *pv = nullptr;
    int ws_bytes = prm.ws_bytes_per_warp > 0 ? prm.ws_bytes_per_warp
                                             : (sizeof(T) == 8 ? 16384 : 8192);
    const int warps = prm.warps_per_block > 0 ? prm.warps_per_block : (sizeof(T) == 8 ? 12 : 24);
    const int qcap_main = 64;
    for (int attempt = 0;; ++attempt) {
        pidx = arena.alloc<int>(cap);
        pv = arena.alloc<T>(cap);
        SPAI_CUDA(cudaMemsetAsync(queue, 0, sizeof(int) * 4, st));
        SPAI_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        SPAI_CUDA(cudaMemsetAsync(top, 0, sizeof(unsigned long long), st));
        ColumnArgs<T> args{n, a.rp, a.ci, a.val, tp, ti, d, static_cast<T>(prm.epsilon), prm.alpha,
                           prm.beta, out.col_status, out.col_fits, out.col_growths, out.col_clamps,
                           out.col_q, out.col_residual, off, pidx, pv, top, cap, queue, ovl, err};
        const size_t smem = static_cast<size_t>(ws_bytes) * warps;
        SPAI_CUDA(cudaFuncSetAttribute(spai_columns_kernel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem)));
        int sms = 0, dev = 0;
        SPAI_CUDA(cudaGetDevice(&dev));
        SPAI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int per_sm = 0;
        SPAI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spai_columns_kernel<T>,
                                                                warps * 32, smem));
        if (per_sm < 1)
            per_sm = 1;
        const long long blocks_needed = (static_cast<long long>(n) + warps - 1) / warps;
        const unsigned blocks =
            static_cast<unsigned>(std::max<long long>(1, std::min<long long>(blocks_needed, static_cast<long long>(sms) * per_sm)));
        spai_columns_kernel<T><<<blocks, warps * 32, smem, st>>>(args, 0, ws_bytes, qcap_main, nullptr);
        SPAI_LAUNCH("spai_columns_kernel(main)");
        ++out.launches;
        int h_queue[4];
        SPAI_CUDA(cudaMemcpyAsync(h_queue, queue, sizeof(h_queue), cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
        out.overflow_columns = h_queue[1];
        if (h_queue[1] > 0) {
            const size_t gws_bytes = prm.overflow_ws_bytes > 0 ? prm.overflow_ws_bytes : (size_t(8) << 20);
            const int ow = std::min(h_queue[1], 1024);
            char *gws = arena.alloc<char>(gws_bytes * ow);
            spai_columns_kernel<T><<<ow, 32, 0, st>>>(args, 1, gws_bytes, 8192, gws);
            SPAI_LAUNCH("spai_columns_kernel(overflow)");
            ++out.launches;
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

extern "C" double spai_hypot(double a, double b) {
    return spai::cr_hypot<double>(a, b);
}
extern "C" float spai_hypotf(float a, float b) {
    return spai::cr_hypot<float>(a, b);
}
