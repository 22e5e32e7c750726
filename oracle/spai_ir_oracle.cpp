// CPU oracle for the SPAI-GMRES-IR hot path. TEST INFRASTRUCTURE ONLY: the product library never
// links, loads or calls this file; tests, smoke() and bench.py's cpu_baseline leg use it as the
// checker. It restates the reference algorithm (anirudhtheexe/spai-gmres-ir) function by
// function, each citing the reference file:line it follows:
//   * SPAI  : src/spai.cpp:100-244 (construct_column), :30-98 (least_squares),
//             :273-306 (evaluate_spai_score), :314-374 (construct_spai).
//             Shadow and candidate sets come from the column structure of A as in
//             src/cuda_spai.cu:607-639; they equal the CPU's O(n) row scans (spai.cpp:110-117,
//             :180-191) because B = (DA)^T has no scaling-induced zeros (spai.cpp:341-345).
//   * GMRES : src/gmres.cpp:108-262 (binary64 acceptance: verify only when triggered) and
//             src/fp32_cuda_gmres.cu:237-432 (binary32: accept on the recomputed residual).
//   * IR    : src/ir.cpp:83-133 (diagnostics), :138-204 (refinement), :206-227 (pipeline);
//             src/fp32_cuda_gmres.cu:468-533 (binary32 refinement).
// Templated on the value type: T=double is the FP64 drop-in, T=float follows the reference's
// float instantiation of the same SPAI code (src/fp32_cuda_spai.cu:89-135). Every 2-norm uses a
// correctly rounded hypot (oracle_hypot.hpp) so results are bit-reproducible on any IEEE machine.
// Build with -ffp-contract=off: no operation may be fused.
#include "oracle_hypot.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <chrono>
#include <numeric>
#include <stdexcept>
#include <thread>
#include <vector>

namespace orc {

// Status codes: the reference enums' declaration order (spai.hpp:10-21, gmres.hpp:10-20,
// ir.hpp:9-17).
enum SpaiStatus {
    S_SUCCESS, S_NOT_ATTEMPTED, S_INVALID_INPUT, S_RANK_DEFICIENT, S_NUMERICAL_FAILURE,
    S_EMPTY_CANDIDATES, S_ZERO_DENOMINATOR, S_INVALID_SCORE, S_NO_GROWTH, S_ITERATION_LIMIT
};
enum GmresStatus {
    G_SUCCESS, G_ZERO_RHS, G_EXACT_INITIAL, G_INVALID_INPUT, G_ZERO_PRECONDITIONED_RHS,
    G_BREAKDOWN, G_ITERATION_LIMIT, G_NONCONVERGENCE, G_NUMERICAL_FAILURE
};
enum IrStatus {
    I_SUCCESS, I_INVALID_INPUT, I_CONSTRUCTION_FAILURE, I_INNER_FAILURE, I_STAGNATION,
    I_ITERATION_LIMIT, I_NUMERICAL_FAILURE
};

struct Overflow {};

template <class T> struct Csr {
    int64_t n = 0;
    std::vector<int64_t> ptr, idx;
    std::vector<T> val;
    int64_t nnz() const {
        return static_cast<int64_t>(idx.size());
    }
};

template <class T> T unit_roundoff();
template <> double unit_roundoff<double>() {
    return std::ldexp(1.0, -53);
}
template <> float unit_roundoff<float>() {
    return std::ldexp(1.0f, -24);
}

template <class T> T finite(T v) {
    if (!std::isfinite(v))
        throw Overflow();
    return v;
}

template <class T> T norm2(const std::vector<T> &v) {
    T r = 0;
    for (T x : v)
        r = o_hypot(r, x);
    return r;
}
template <class T> T norm2_checked(const std::vector<T> &v) {
    T r = 0;
    for (T x : v)
        r = finite(o_hypot(r, x));
    return r;
}

// y = A x, sequential row sums in stored order (src/cpu.cpp:80-94). Throws on nonfinite rows.
template <class T, class X> std::vector<T> spmv(const Csr<T> &a, const std::vector<X> &x) {
    std::vector<T> y(a.n, 0);
    for (int64_t r = 0; r < a.n; ++r) {
        T s = 0;
        for (int64_t e = a.ptr[r]; e < a.ptr[r + 1]; ++e)
            s += a.val[e] * static_cast<T>(x[a.idx[e]]);
        if (!std::isfinite(s))
            throw Overflow();
        y[r] = s;
    }
    return y;
}

// ------------------------------------------------------------------------------------------
// SPAI
// ------------------------------------------------------------------------------------------
struct SpaiOptions {
    double epsilon = 0.3;
    int64_t alpha = 5, beta = 8;
};

template <class T> struct Fit {
    std::vector<int64_t> pattern, shadow, candidates, selected;
    std::vector<T> coefficients, scores;
    T residual = 0, mean_score = 0, pivot_ratio = 0;
};

template <class T> struct Column {
    int status = S_NOT_ATTEMPTED;
    std::vector<int64_t> pattern;
    std::vector<T> coefficients;
    int64_t fits = 0, growths = 0, fit_attempts = 0, growth_attempts = 0, score_clamps = 0;
    T residual = std::numeric_limits<T>::quiet_NaN();
    T pivot_ratio = std::numeric_limits<T>::quiet_NaN();
    std::vector<Fit<T>> history;
};

template <class T> struct ScoreResult {
    int status = S_NOT_ATTEMPTED;
    T score = 0;
    bool clamped = false;
};

// src/spai.cpp:273-306 (binary64) and the float instantiation src/cuda_spai.cu:348-380 with
// BSPAI_SPAI_SCORE_UNIT_ROUNDOFF = 2^-24 (src/fp32_cuda_spai.cu:110).
template <class T> ScoreResult<T> evaluate_score(T rsq, T dot, T den) {
    ScoreResult<T> r;
    if (!std::isfinite(rsq) || !std::isfinite(dot) || !std::isfinite(den)) {
        r.status = S_NUMERICAL_FAILURE;
        return r;
    }
    if (den == 0) {
        r.status = S_ZERO_DENOMINATOR;
        return r;
    }
    if (rsq < 0 || den < 0) {
        r.status = S_INVALID_SCORE;
        return r;
    }
    const T quotient = dot * dot / den;
    T delta = rsq - quotient;
    const T bound = T(32) * unit_roundoff<T>() * (rsq + std::fabs(quotient));
    if (!std::isfinite(quotient) || !std::isfinite(delta) || !std::isfinite(bound)) {
        r.status = S_NUMERICAL_FAILURE;
        return r;
    }
    if (delta < 0) {
        if (-delta > bound) {
            r.status = S_INVALID_SCORE;
            return r;
        }
        delta = 0;
        r.clamped = true;
    }
    r.score = std::sqrt(delta);
    r.status = S_SUCCESS;
    return r;
}

// Economy Householder least squares with normalised reflectors, src/spai.cpp:30-98.
// r is row-major rows x cols.
template <class T>
int least_squares(std::vector<T> r, std::vector<T> rhs, int64_t rows, int64_t cols,
                  std::vector<T> &solution, T &pivot_ratio) {
    if (rows < cols)
        return S_RANK_DEFICIENT;
    T inf_norm = 0;
    for (int64_t i = 0; i < rows; ++i) {
        T sum = 0;
        for (int64_t j = 0; j < cols; ++j)
            sum += std::fabs(r[i * cols + j]);
        inf_norm = std::max(inf_norm, sum);
    }
    T min_pivot = std::numeric_limits<T>::infinity();
    std::vector<T> v;
    for (int64_t j = 0; j < cols; ++j) {
        v.assign(rows - j, 0);
        for (int64_t i = j; i < rows; ++i)
            v[i - j] = r[i * cols + j];
        const T length = norm2(v);
        if (!std::isfinite(length))
            return S_NUMERICAL_FAILURE;
        if (length == 0)
            return S_RANK_DEFICIENT;
        const T diagonal = -std::copysign(length, v[0]);
        for (T &value : v)
            value /= length;
        v[0] += std::copysign(T(1), v[0]);
        const T vnorm = norm2(v);
        for (T &value : v)
            value /= vnorm;
        for (int64_t col = j; col < cols; ++col) {
            T dot = 0;
            for (int64_t i = j; i < rows; ++i)
                dot += v[i - j] * r[i * cols + col];
            for (int64_t i = j; i < rows; ++i) {
                r[i * cols + col] -= 2 * v[i - j] * dot;
                if (!std::isfinite(r[i * cols + col]))
                    return S_NUMERICAL_FAILURE;
            }
        }
        T dot = 0;
        for (int64_t i = j; i < rows; ++i)
            dot += v[i - j] * rhs[i];
        for (int64_t i = j; i < rows; ++i) {
            rhs[i] -= 2 * v[i - j] * dot;
            if (!std::isfinite(rhs[i]))
                return S_NUMERICAL_FAILURE;
        }
        r[j * cols + j] = diagonal;
        for (int64_t i = j + 1; i < rows; ++i)
            r[i * cols + j] = 0;
        min_pivot = std::min(min_pivot, std::fabs(diagonal));
    }
    pivot_ratio = inf_norm == 0 ? T(0) : min_pivot / inf_norm;
    solution.assign(cols, 0);
    for (int64_t j = cols; j-- > 0;) {
        T value = rhs[j];
        for (int64_t k = j + 1; k < cols; ++k)
            value -= r[j * cols + k] * solution[k];
        const T diagonal = r[j * cols + j];
        if (!std::isfinite(diagonal))
            return S_NUMERICAL_FAILURE;
        if (diagonal == 0)
            return S_RANK_DEFICIENT;
        solution[j] = value / diagonal;
        if (!std::isfinite(solution[j]))
            return S_NUMERICAL_FAILURE;
    }
    return S_SUCCESS;
}

// Row/column structure of A plus the row scaling D; B(i,j) = A(j,i) * d_j (src/spai.cpp:341-348).
template <class T> struct SpaiInput {
    const Csr<T> *a;
    std::vector<int64_t> tptr, tidx; // column structure of A (row i of B)
    std::vector<T> d;
};

template <class T> T b_value(const SpaiInput<T> &in, int64_t i, int64_t j) {
    const Csr<T> &a = *in.a;
    const auto first = a.idx.begin() + a.ptr[j], last = a.idx.begin() + a.ptr[j + 1];
    const auto it = std::lower_bound(first, last, i);
    if (it == last || *it != i)
        return 0;
    return a.val[it - a.idx.begin()] * in.d[j];
}

// Adaptive column fit, src/spai.cpp:100-244.
template <class T>
Column<T> construct_column(const SpaiInput<T> &in, int64_t k, const SpaiOptions &o,
                           bool keep_history) {
    const Csr<T> &a = *in.a;
    const T epsilon = static_cast<T>(o.epsilon);
    Column<T> column;
    std::vector<int64_t> pattern(1, k);
    for (;;) {
        ++column.fit_attempts;
        if (column.fits != 0)
            ++column.growth_attempts;
        Fit<T> fit;
        fit.pattern = pattern;
        // Shadow: rows i with B(i,j) != 0 for some j in J = union of A's row patterns.
        for (int64_t j : pattern)
            for (int64_t e = a.ptr[j]; e < a.ptr[j + 1]; ++e)
                fit.shadow.push_back(a.idx[e]);
        std::sort(fit.shadow.begin(), fit.shadow.end());
        fit.shadow.erase(std::unique(fit.shadow.begin(), fit.shadow.end()), fit.shadow.end());
        const int64_t rows = static_cast<int64_t>(fit.shadow.size());
        const int64_t cols = static_cast<int64_t>(pattern.size());
        std::vector<T> reduced(rows * cols, 0), rhs(rows, 0);
        for (int64_t i = 0; i < rows; ++i)
            rhs[i] = fit.shadow[i] == k ? T(1) : T(0);
        for (int64_t jj = 0; jj < cols; ++jj) {
            const int64_t j = pattern[jj];
            for (int64_t e = a.ptr[j]; e < a.ptr[j + 1]; ++e) {
                const int64_t pos =
                    std::lower_bound(fit.shadow.begin(), fit.shadow.end(), a.idx[e]) -
                    fit.shadow.begin();
                reduced[pos * cols + jj] = a.val[e] * in.d[j];
            }
        }
        const int st = least_squares(reduced, rhs, rows, cols, fit.coefficients, fit.pivot_ratio);
        if (st != S_SUCCESS) {
            column.status = st;
            return column;
        }
        std::vector<T> residual(rows, 0);
        for (int64_t i = 0; i < rows; ++i) {
            for (int64_t j = 0; j < cols; ++j)
                residual[i] += reduced[i * cols + j] * fit.coefficients[j];
            residual[i] -= rhs[i];
            // B*m row sums; the full product equals the reduced one outside rounding of zeros.
            if (!std::isfinite(residual[i])) {
                column.status = S_NUMERICAL_FAILURE;
                return column;
            }
        }
        fit.residual = norm2(residual);
        if (!std::isfinite(fit.residual)) {
            column.status = S_NUMERICAL_FAILURE;
            return column;
        }
        if (column.fits != 0)
            ++column.growths;
        ++column.fits;
        column.pattern = pattern;
        column.coefficients = fit.coefficients;
        column.residual = fit.residual;
        column.pivot_ratio = fit.pivot_ratio;
        if (keep_history)
            column.history.push_back(fit);
        if (fit.residual <= epsilon) {
            column.status = S_SUCCESS;
            return column;
        }
        if (column.growths == o.alpha) {
            column.status = S_ITERATION_LIMIT;
            return column;
        }
        // Candidates: columns of B in the shadow rows and in row k, minus J (spai.cpp:180-191).
        std::vector<int64_t> cand;
        for (int64_t i : fit.shadow)
            for (int64_t e = in.tptr[i]; e < in.tptr[i + 1]; ++e)
                cand.push_back(in.tidx[e]);
        for (int64_t e = in.tptr[k]; e < in.tptr[k + 1]; ++e)
            cand.push_back(in.tidx[e]);
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        std::vector<int64_t> filtered;
        std::set_difference(cand.begin(), cand.end(), pattern.begin(), pattern.end(),
                            std::back_inserter(filtered));
        fit.candidates.swap(filtered);
        if (fit.candidates.empty()) {
            column.status = S_EMPTY_CANDIDATES;
            if (keep_history)
                column.history.back() = fit;
            return column;
        }
        const T rsq = fit.residual * fit.residual;
        for (int64_t j : fit.candidates) {
            // dot/den in ascending shadow order; zero entries of B add +-0 and are skipped.
            T dot = 0, den = 0;
            int64_t e = a.ptr[j];
            const int64_t end = a.ptr[j + 1];
            for (int64_t i = 0; i < rows && e < end; ++i) {
                while (e < end && a.idx[e] < fit.shadow[i])
                    ++e;
                if (e < end && a.idx[e] == fit.shadow[i]) {
                    const T value = a.val[e] * in.d[j];
                    dot += residual[i] * value;
                    den += value * value;
                }
            }
            const ScoreResult<T> s = evaluate_score(rsq, dot, den);
            if (s.status != S_SUCCESS) {
                column.status = s.status;
                if (keep_history)
                    column.history.back() = fit;
                return column;
            }
            if (s.clamped)
                ++column.score_clamps;
            fit.scores.push_back(s.score);
        }
        T mean = 0;
        for (T s : fit.scores)
            mean += s;
        mean = mean / static_cast<T>(fit.scores.size());
        fit.mean_score = mean;
        if (!std::isfinite(mean)) {
            column.status = S_NUMERICAL_FAILURE;
            if (keep_history)
                column.history.back() = fit;
            return column;
        }
        std::vector<int64_t> order(fit.candidates.size());
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
            return fit.scores[x] < fit.scores[y] ||
                   (fit.scores[x] == fit.scores[y] && fit.candidates[x] < fit.candidates[y]);
        });
        for (int64_t i : order) {
            if (static_cast<int64_t>(fit.selected.size()) == o.beta)
                break;
            if (fit.scores[i] <= mean)
                fit.selected.push_back(fit.candidates[i]);
        }
        if (keep_history)
            column.history.back() = fit;
        if (fit.selected.empty()) {
            column.status = S_NO_GROWTH;
            return column;
        }
        pattern.insert(pattern.end(), fit.selected.begin(), fit.selected.end());
        std::sort(pattern.begin(), pattern.end());
    }
}

template <class T> struct SpaiResult {
    int status = S_INVALID_INPUT;
    int64_t first_failed_column = -1;
    std::vector<T> scaling;
    std::vector<Column<T>> columns;
    Csr<T> p; // P = N^T D, canonical CSR (zeros dropped, src/cpu.cpp:49-78)
};

// Threads for the column fits of construct_spai (oracle_set_threads); 1 = sequential.
static int g_threads = 1;

// src/spai.cpp:314-374.
template <class T>
SpaiResult<T> construct_spai(const Csr<T> &a, const SpaiOptions &o, bool keep_history) {
    SpaiResult<T> result;
    const int64_t n = a.n;
    if (n == 0 || !std::isfinite(o.epsilon) || o.epsilon <= 0 ||
        !(static_cast<T>(o.epsilon) > 0))
        return result;
    SpaiInput<T> in;
    in.a = &a;
    in.d.resize(n);
    for (int64_t row = 0; row < n; ++row) {
        bool diagonal = false;
        T maximum = 0;
        for (int64_t e = a.ptr[row]; e < a.ptr[row + 1]; ++e) {
            maximum = std::max(maximum, std::fabs(a.val[e]));
            if (a.idx[e] == row && a.val[e] != 0)
                diagonal = true;
        }
        if (!diagonal)
            return result;
        const T scale = T(1) / maximum;
        if (!std::isfinite(scale) || scale == 0)
            return result;
        in.d[row] = scale;
        for (int64_t e = a.ptr[row]; e < a.ptr[row + 1]; ++e) {
            const T v = a.val[e] * scale;
            if (!std::isfinite(v) || v == 0)
                return result;
        }
    }
    // Column structure of A.
    in.tptr.assign(n + 1, 0);
    for (int64_t e = 0; e < a.nnz(); ++e)
        ++in.tptr[a.idx[e] + 1];
    for (int64_t i = 0; i < n; ++i)
        in.tptr[i + 1] += in.tptr[i];
    in.tidx.resize(a.nnz());
    {
        std::vector<int64_t> fill(in.tptr.begin(), in.tptr.end() - 1);
        for (int64_t r = 0; r < n; ++r)
            for (int64_t e = a.ptr[r]; e < a.ptr[r + 1]; ++e)
                in.tidx[fill[a.idx[e]]++] = r;
    }
    result.scaling = in.d;
    result.status = S_SUCCESS;
    result.columns.resize(n);
    // Columns are independent (each fit reads only A, d and the column structure): they are
    // fitted on g_threads threads in interleaved order; the overall status is then taken in
    // column order, as the sequential loop of src/spai.cpp:329-336 does.
    const int nthreads = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(g_threads, n / 256)));
    if (nthreads > 1) {
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t)
            pool.emplace_back([&, t] {
                for (int64_t k = t; k < n; k += nthreads)
                    result.columns[k] = construct_column(in, k, o, keep_history);
            });
        for (auto &th : pool)
            th.join();
    } else {
        for (int64_t k = 0; k < n; ++k)
            result.columns[k] = construct_column(in, k, o, keep_history);
    }
    for (int64_t k = 0; k < n; ++k) {
        if (result.columns[k].status != S_SUCCESS && result.status == S_SUCCESS) {
            result.status = result.columns[k].status;
            result.first_failed_column = k;
        }
    }
    // P(k, j) = m_jk * d_j; CSR row k of P is column k of N (spai.cpp:351-373).
    Csr<T> &p = result.p;
    p.n = n;
    p.ptr.assign(n + 1, 0);
    for (int64_t k = 0; k < n; ++k) {
        const Column<T> &c = result.columns[k];
        for (size_t i = 0; i < c.pattern.size(); ++i) {
            const int64_t j = c.pattern[i];
            const T value = c.coefficients[i] * in.d[j];
            if (!std::isfinite(value) || (c.coefficients[i] != 0 && value == 0)) {
                result.status = S_NUMERICAL_FAILURE;
                p.ptr.assign(n + 1, 0);
                p.idx.clear();
                p.val.clear();
                return result;
            }
            if (value != 0) {
                p.idx.push_back(j);
                p.val.push_back(value);
            }
        }
        p.ptr[k + 1] = static_cast<int64_t>(p.idx.size());
    }
    return result;
}

// ------------------------------------------------------------------------------------------
// GMRES
// ------------------------------------------------------------------------------------------
struct GmresOptions {
    double tolerance = 1e-8;
    int64_t max_iterations = 0; // 0 = n
    int accept_every_iteration = 0; // 1 = binary32 drop-in semantics (fp32_cuda_gmres.cu:409)
    int lazy_candidates = 1;        // form x0 + V y only when verification is triggered
    // Binary32 dot products and 2-norms: 0 = sequential binary32 sums (the reference's CPU FP32
    // solver, src/fp32_cpu.cpp:12-23); 1 = accumulated in binary64 and rounded once, a model of
    // the reference's FP32 GPU solver, whose dots and norms are cuBLAS reductions
    // (cublasSdot_64 / cublasSnrm2_64, src/fp32_cuda_gmres.cu:158-167) with tree-order error
    // O(log n) ulps rather than the O(n) ulps of a sequential sum over n entries.
    int wide_reductions = 0;
};
struct GmresReport {
    int status = G_INVALID_INPUT;
    bool converged = false;
    int64_t iterations = 0;
    double final_original = NAN, final_relative = NAN, initial_relative = NAN;
};

// Left-preconditioned GMRES on P A d = P b, src/gmres.cpp:108-262 (and the binary32 acceptance
// variant of src/fp32_cuda_gmres.cu:237-432). Vectors, dots and Givens work in T.
template <class T>
GmresReport gmres(const Csr<T> &a, const Csr<T> &p, const std::vector<T> &rhs,
                  const GmresOptions &o, std::vector<T> &solution) {
    GmresReport rep;
    const int64_t n = a.n;
    const T tol = static_cast<T>(o.tolerance);
    if (n == 0 || !std::isfinite(o.tolerance) || o.tolerance <= 0 || o.max_iterations > n ||
        static_cast<int64_t>(rhs.size()) != n)
        return rep;
    for (T v : rhs)
        if (!std::isfinite(v))
            return rep;
    const int64_t cap = o.max_iterations == 0 ? n : o.max_iterations;
    solution.assign(n, 0);
    const bool wide = o.wide_reductions && sizeof(T) == 4;
    auto vnorm = [&](const std::vector<T> &v) -> T {
        if (!wide)
            return norm2_checked(v);
        double s2 = 0;
        for (T x : v)
            s2 += static_cast<double>(x) * static_cast<double>(x);
        return finite(static_cast<T>(std::sqrt(s2)));
    };
    auto vdot = [&](const std::vector<T> &a_, const std::vector<T> &b_) -> T {
        T dot = 0;
        if (!wide) {
            for (int64_t i = 0; i < n; ++i)
                dot = finite(dot + finite(a_[i] * b_[i]));
            return dot;
        }
        double acc = 0;
        for (int64_t i = 0; i < n; ++i)
            acc += static_cast<double>(a_[i]) * static_cast<double>(b_[i]);
        return finite(static_cast<T>(acc));
    };
    try {
        // x0 = 0: A x0 = 0, original residual = rhs.
        const T r0 = vnorm(rhs);
        rep.final_original = r0;
        if (r0 == 0) {
            const bool zero = std::all_of(rhs.begin(), rhs.end(), [](T v) { return v == 0; });
            rep.status = (zero && !o.accept_every_iteration) ? G_ZERO_RHS : G_EXACT_INITIAL;
            rep.converged = true;
            rep.final_relative = rep.initial_relative = 0;
            return rep;
        }
        const std::vector<T> pb = spmv(p, rhs);
        const T den = vnorm(pb);
        if (den == 0) {
            rep.status = G_ZERO_PRECONDITIONED_RHS;
            return rep;
        }
        const T beta = den; // residual = Pb - P A 0 = Pb
        rep.initial_relative = rep.final_relative = finite(beta / den);
        if (rep.initial_relative <= tol) {
            rep.status = G_SUCCESS;
            rep.converged = true;
            return rep;
        }
        std::vector<std::vector<T>> basis;
        basis.emplace_back(n);
        for (int64_t i = 0; i < n; ++i)
            basis[0][i] = finite(pb[i] / beta);
        std::vector<std::vector<T>> rot(cap + 1, std::vector<T>(cap, 0));
        std::vector<T> cs(cap, 0), sn(cap, 0), g(cap + 1, 0);
        g[0] = beta;
        auto check = [&](const std::vector<T> &x, T &orig, T &rel) {
            const std::vector<T> ax = spmv(a, x);
            std::vector<T> r(n);
            for (int64_t i = 0; i < n; ++i)
                r[i] = finite(rhs[i] - ax[i]);
            orig = vnorm(r);
            const std::vector<T> pax = spmv(p, ax);
            for (int64_t i = 0; i < n; ++i)
                r[i] = finite(pb[i] - pax[i]);
            rel = finite(vnorm(r) / den);
        };
        int64_t formed_count = 0;
        // Candidate x0 + V y from the first count Givens-rotated columns (gmres.cpp:47-65).
        auto form = [&](int64_t count) {
            std::vector<T> y(count, 0);
            for (int64_t r = count; r-- > 0;) {
                T v = g[r];
                for (int64_t c = r + 1; c < count; ++c)
                    v = finite(v - finite(rot[r][c] * y[c]));
                y[r] = finite(v / rot[r][r]);
            }
            std::vector<T> cand(n, 0);
            for (int64_t c = 0; c < count; ++c)
                for (int64_t i = 0; i < n; ++i)
                    cand[i] = finite(cand[i] + finite(basis[c][i] * y[c]));
            formed_count = count;
            return cand;
        };
        for (int64_t k = 0; k < cap; ++k) {
            rep.iterations = k + 1;
            std::vector<T> w = spmv(p, spmv(a, basis[k]));
            std::vector<T> hcol(k + 2, 0);
            for (int64_t j = 0; j <= k; ++j) {
                const T dot = vdot(basis[j], w);
                hcol[j] = dot;
                for (int64_t i = 0; i < n; ++i)
                    w[i] = finite(w[i] - finite(dot * basis[j][i]));
            }
            const T hnext = vnorm(w);
            hcol[k + 1] = hnext;
            const bool breakdown = hnext == 0;
            if (!breakdown) {
                for (T &v : w)
                    v = finite(v / hnext);
                basis.push_back(std::move(w));
            }
            for (int64_t r = 0; r <= k + 1; ++r)
                rot[r][k] = hcol[r];
            for (int64_t r = 0; r < k; ++r) {
                const T up = rot[r][k], lo = rot[r + 1][k];
                rot[r][k] = finite(cs[r] * up + sn[r] * lo);
                rot[r + 1][k] = finite(-sn[r] * up + cs[r] * lo);
            }
            const T upper = rot[k][k];
            const T radius = finite(o_hypot(upper, rot[k + 1][k]));
            if (radius == 0) {
                // Zero Givens pivot: re-verify the previous candidate (gmres.cpp:218-234).
                // Under lazy formation the previous candidate may not exist yet; its
                // coefficients (columns 0..k-1) are unchanged, so form it now.
                if (o.lazy_candidates && !o.accept_every_iteration && k > 0 &&
                    formed_count != k)
                    solution = form(k);
                T orig, rel;
                check(solution, orig, rel);
                rep.final_original = orig;
                rep.final_relative = rel;
                const bool ok = !o.accept_every_iteration && rel <= tol;
                rep.converged = ok;
                rep.status = ok ? G_SUCCESS : G_BREAKDOWN;
                return rep;
            }
            cs[k] = finite(upper / radius);
            sn[k] = finite(rot[k + 1][k] / radius);
            rot[k][k] = radius;
            rot[k + 1][k] = 0;
            const T old = g[k];
            g[k] = finite(cs[k] * old);
            g[k + 1] = finite(-sn[k] * old);
            const T est = finite(std::fabs(g[k + 1]) / den);
            const bool triggered = breakdown || est <= tol || k + 1 == cap;
            if (o.lazy_candidates && !triggered && !o.accept_every_iteration)
                continue;
            std::vector<T> cand = form(k + 1);
            T orig, rel;
            check(cand, orig, rel);
            rep.final_original = orig;
            rep.final_relative = rel;
            solution = cand;
            const bool accepted =
                o.accept_every_iteration ? rel <= tol : (triggered && rel <= tol);
            if (accepted) {
                rep.status = G_SUCCESS;
                rep.converged = true;
                return rep;
            }
            if (breakdown) {
                rep.status = G_BREAKDOWN;
                return rep;
            }
        }
        rep.status = cap < n ? G_ITERATION_LIMIT : G_NONCONVERGENCE;
    } catch (const Overflow &) {
        rep.status = G_NUMERICAL_FAILURE;
    }
    return rep;
}

// ------------------------------------------------------------------------------------------
// Iterative refinement
// ------------------------------------------------------------------------------------------
struct Diagnostics {
    std::vector<double> residual;
    double residual_inf = 0, residual_2 = 0, nbe = 0, cbe = 0, forward = NAN;
};
double ratio(double num, double den) {
    if (den == 0)
        return num == 0 ? 0 : INFINITY;
    return num / den;
}
// src/ir.cpp:83-133 in binary64 (A given in binary64).
Diagnostics diagnostics(const Csr<double> &a, const std::vector<double> &rhs,
                        const std::vector<double> &x, const double *reference) {
    Diagnostics d;
    const int64_t n = a.n;
    const std::vector<double> ax = spmv(a, x);
    d.residual.resize(n);
    double minf = 0, xinf = 0, binf = 0;
    for (double v : x)
        xinf = std::max(xinf, std::fabs(v));
    for (int64_t r = 0; r < n; ++r) {
        const double res = finite(rhs[r] - ax[r]);
        d.residual[r] = res;
        d.residual_inf = std::max(d.residual_inf, std::fabs(res));
        d.residual_2 = finite(cr_hypot(d.residual_2, res));
        binf = std::max(binf, std::fabs(rhs[r]));
        double row_sum = 0, cden = std::fabs(rhs[r]);
        for (int64_t e = a.ptr[r]; e < a.ptr[r + 1]; ++e) {
            const double v = std::fabs(a.val[e]);
            row_sum = finite(row_sum + v);
            cden = finite(cden + finite(v * std::fabs(x[a.idx[e]])));
        }
        minf = std::max(minf, row_sum);
        d.cbe = std::max(d.cbe, ratio(std::fabs(res), cden));
    }
    d.nbe = ratio(d.residual_inf, finite(finite(minf * xinf) + binf));
    if (reference) {
        double rinf = 0, einf = 0;
        for (int64_t i = 0; i < n; ++i) {
            rinf = std::max(rinf, std::fabs(reference[i]));
            einf = std::max(einf, std::fabs(x[i] - reference[i]));
        }
        d.forward = rinf == 0 ? einf : einf / rinf;
    }
    return d;
}
// src/fp32_cpu.cpp:509-531 (binary32 diagnostics used by the binary32 drop-in IR).
Diagnostics diagnostics32(const Csr<float> &a, const std::vector<float> &b,
                          const std::vector<float> &x) {
    Diagnostics d;
    const std::vector<float> ax = spmv(a, x);
    std::vector<float> r(a.n);
    for (int64_t i = 0; i < a.n; ++i)
        r[i] = finite(b[i] - ax[i]);
    d.residual.assign(r.begin(), r.end());
    float r2 = 0;
    for (float v : r)
        r2 = finite(cr_hypotf(r2, v));
    d.residual_2 = r2;
    float an = 0, xn = 0, bn = 0, rinf = 0;
    for (int64_t i = 0; i < a.n; ++i) {
        float rs = 0;
        for (int64_t e = a.ptr[i]; e < a.ptr[i + 1]; ++e)
            rs = finite(rs + std::fabs(a.val[e]));
        an = std::max(an, rs);
        rinf = std::max(rinf, std::fabs(r[i]));
        xn = std::max(xn, std::fabs(x[i]));
        bn = std::max(bn, std::fabs(b[i]));
    }
    d.residual_inf = rinf;
    const float den = finite(an * xn + bn);
    d.nbe = den == 0 ? (rinf == 0 ? 0.0 : INFINITY) : static_cast<double>(finite(rinf / den));
    return d;
}

struct IrOptions {
    SpaiOptions spai;
    GmresOptions gmres;
    int64_t max_outer = 20;
    double be_tolerance = 0; // 0 = the precision's 10u (ir.cpp:79-81, fp32_cpu.cpp:506-508)
};
struct IrReport {
    int status = I_INVALID_INPUT;
    bool converged = false;
    int64_t outer_steps = 0, inner_attempts = 0, inner_iterations = 0;
    int spai_status = S_NOT_ATTEMPTED, last_inner_status = -1;
    double nbe = NAN, cbe = NAN, residual_inf = NAN, forward = NAN;
    int64_t nnz_p = 0;
};

// src/ir.cpp:138-204 in binary64, with the inner solve in binary64 (precision 0) or in
// binary32 with a power-of-two scaled right-hand side (precision 2: the mixed form).
template <class TI>
IrReport refine64(const Csr<double> &a, const Csr<TI> &a_inner, const Csr<TI> &p,
                  const std::vector<double> &b, const IrOptions &o, const double *reference,
                  std::vector<double> &x) {
    IrReport rep;
    const int64_t n = a.n;
    const double tol = o.be_tolerance > 0 ? o.be_tolerance : 10 * std::ldexp(1.0, -53);
    try {
        // x0 = P b with P's values promoted to binary64.
        x.assign(n, 0);
        for (int64_t r = 0; r < n; ++r) {
            double s = 0;
            for (int64_t e = p.ptr[r]; e < p.ptr[r + 1]; ++e)
                s += static_cast<double>(p.val[e]) * b[p.idx[e]];
            x[r] = finite(s);
        }
        Diagnostics d = diagnostics(a, b, x, reference);
        rep.nbe = d.nbe;
        rep.cbe = d.cbe;
        rep.residual_inf = d.residual_inf;
        rep.forward = d.forward;
        if (d.nbe <= tol) {
            rep.status = I_SUCCESS;
            rep.converged = true;
            return rep;
        }
        for (int64_t step = 0; step < o.max_outer; ++step) {
            std::vector<TI> rhs(n);
            double scale = 1;
            if (sizeof(TI) == 4) {
                double rinf = 0;
                for (double v : d.residual)
                    rinf = std::max(rinf, std::fabs(v));
                scale = rinf > 0 ? std::ldexp(1.0, -std::ilogb(rinf)) : 1.0;
            }
            for (int64_t i = 0; i < n; ++i)
                rhs[i] = static_cast<TI>(d.residual[i] * scale);
            std::vector<TI> corr;
            const GmresReport g = gmres(a_inner, p, rhs, o.gmres, corr);
            ++rep.inner_attempts;
            rep.inner_iterations += g.iterations;
            rep.last_inner_status = g.status;
            if (!g.converged) {
                rep.status = I_INNER_FAILURE;
                return rep;
            }
            std::vector<double> next(x);
            bool changed = false;
            for (int64_t i = 0; i < n; ++i) {
                next[i] = finite(next[i] + static_cast<double>(corr[i]) / scale);
                changed = changed || next[i] != x[i];
            }
            Diagnostics dn = diagnostics(a, b, next, reference);
            x.swap(next);
            d.residual.swap(dn.residual);
            rep.nbe = dn.nbe;
            rep.cbe = dn.cbe;
            rep.residual_inf = dn.residual_inf;
            rep.forward = dn.forward;
            ++rep.outer_steps;
            if (dn.nbe <= tol) {
                rep.status = I_SUCCESS;
                rep.converged = true;
                return rep;
            }
            if (!changed) {
                rep.status = I_STAGNATION;
                return rep;
            }
        }
        rep.status = I_ITERATION_LIMIT;
    } catch (const Overflow &) {
        rep.status = I_NUMERICAL_FAILURE;
    }
    return rep;
}

// Binary32 drop-in refinement, src/fp32_cuda_gmres.cu:468-533.
IrReport refine32(const Csr<float> &a, const Csr<float> &p, const std::vector<float> &b,
                  const IrOptions &o, std::vector<float> &x) {
    IrReport rep;
    const double tol = o.be_tolerance > 0 ? o.be_tolerance : 10 * std::ldexp(1.0, -24);
    try {
        x = spmv(p, b);
        for (int64_t s = 0; s <= o.max_outer; ++s) {
            Diagnostics d = diagnostics32(a, b, x);
            rep.nbe = d.nbe;
            rep.residual_inf = d.residual_inf;
            if (d.nbe <= tol) {
                rep.status = I_SUCCESS;
                rep.converged = true;
                return rep;
            }
            if (s == o.max_outer)
                break;
            std::vector<float> rhs(d.residual.begin(), d.residual.end()), corr;
            const GmresReport g = gmres(a, p, rhs, o.gmres, corr);
            ++rep.inner_attempts;
            rep.inner_iterations += g.iterations;
            rep.last_inner_status = g.status;
            if (!g.converged) {
                rep.status = I_INNER_FAILURE;
                return rep;
            }
            const std::vector<float> prev = x;
            for (int64_t i = 0; i < a.n; ++i)
                x[i] = finite(x[i] + corr[i]);
            ++rep.outer_steps;
            Diagnostics after = diagnostics32(a, b, x);
            rep.nbe = after.nbe;
            rep.residual_inf = after.residual_inf;
            if (after.nbe <= tol) {
                rep.status = I_SUCCESS;
                rep.converged = true;
                return rep;
            }
            if (x == prev) {
                rep.status = I_STAGNATION;
                return rep;
            }
        }
        rep.status = I_ITERATION_LIMIT;
    } catch (const Overflow &) {
        rep.status = I_NUMERICAL_FAILURE;
    }
    return rep;
}

Csr<double> make_csr(int64_t n, const int64_t *ptr, const int64_t *idx, const double *val) {
    Csr<double> a;
    a.n = n;
    a.ptr.assign(ptr, ptr + n + 1);
    a.idx.assign(idx, idx + ptr[n]);
    a.val.assign(val, val + ptr[n]);
    return a;
}
Csr<float> to_float(const Csr<double> &a) {
    Csr<float> f;
    f.n = a.n;
    f.ptr = a.ptr;
    f.idx = a.idx;
    f.val.resize(a.val.size());
    for (size_t i = 0; i < a.val.size(); ++i)
        f.val[i] = static_cast<float>(a.val[i]);
    return f;
}

} // namespace orc

// CPU-baseline sample: time the adaptive fits of the listed columns (construct_column), split
// over nthreads threads (columns are independent). Returns wall seconds of the fits only;
// fits_out receives the summed fit count.
namespace orc {
template <class T>
double spai_sample(const Csr<T> &a, const SpaiOptions &o, const int64_t *cols, int64_t ncols,
                   int nthreads, int64_t *fits_out) {
    SpaiInput<T> in;
    in.a = &a;
    const int64_t n = a.n;
    in.d.resize(n);
    for (int64_t r = 0; r < n; ++r) {
        T mx = 0;
        for (int64_t e = a.ptr[r]; e < a.ptr[r + 1]; ++e)
            mx = std::max(mx, std::fabs(a.val[e]));
        in.d[r] = T(1) / mx;
    }
    in.tptr.assign(n + 1, 0);
    for (int64_t e = 0; e < a.nnz(); ++e)
        ++in.tptr[a.idx[e] + 1];
    for (int64_t i = 0; i < n; ++i)
        in.tptr[i + 1] += in.tptr[i];
    in.tidx.resize(a.nnz());
    std::vector<int64_t> fill(in.tptr.begin(), in.tptr.end() - 1);
    for (int64_t r = 0; r < n; ++r)
        for (int64_t e = a.ptr[r]; e < a.ptr[r + 1]; ++e)
            in.tidx[fill[a.idx[e]]++] = r;
    if (nthreads < 1)
        nthreads = 1;
    std::vector<int64_t> fits(nthreads, 0);
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t] {
            for (int64_t i = t; i < ncols; i += nthreads)
                fits[t] += construct_column(in, cols[i], o, false).fits;
        });
    for (auto &th : pool)
        th.join();
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    int64_t f = 0;
    for (int64_t x : fits)
        f += x;
    *fits_out = f;
    return sec;
}

// Sampled-column parity: the adaptive fits of the listed columns (construct_column, columns
// split over nthreads threads) and their rows of P = N^T D as the full construction assembles
// them (src/spai.cpp:351-373: value = m_jk d_j, exact zeros dropped). Per listed column i:
// status/fits/growths/clamps/residual[i], P row in p_idx/p_val[p_ptr[i] .. p_ptr[i+1]).
// Returns the total number of stored P entries; nothing is written to p_idx/p_val when that
// exceeds cap (call again with room). assembly_bad[i] = 1 when the row's assembly leaves the
// binary range (the full construction then reports numerical_failure).
template <class T>
int64_t spai_columns_sample(const Csr<T> &a, const SpaiOptions &o, const int64_t *cols, int64_t ncols,
                            int nthreads, int32_t *status, int32_t *fits, int32_t *growths,
                            int32_t *clamps, double *residual, int32_t *assembly_bad, int64_t *p_ptr,
                            int64_t *p_idx, double *p_val, int64_t cap) {
    SpaiInput<T> in;
    in.a = &a;
    const int64_t n = a.n;
    in.d.resize(n);
    for (int64_t r = 0; r < n; ++r) {
        T mx = 0;
        for (int64_t e = a.ptr[r]; e < a.ptr[r + 1]; ++e)
            mx = std::max(mx, std::fabs(a.val[e]));
        in.d[r] = T(1) / mx;
    }
    in.tptr.assign(n + 1, 0);
    for (int64_t e = 0; e < a.nnz(); ++e)
        ++in.tptr[a.idx[e] + 1];
    for (int64_t i = 0; i < n; ++i)
        in.tptr[i + 1] += in.tptr[i];
    in.tidx.resize(a.nnz());
    std::vector<int64_t> fill(in.tptr.begin(), in.tptr.end() - 1);
    for (int64_t r = 0; r < n; ++r)
        for (int64_t e = a.ptr[r]; e < a.ptr[r + 1]; ++e)
            in.tidx[fill[a.idx[e]]++] = r;
    if (nthreads < 1)
        nthreads = 1;
    std::vector<std::vector<int64_t>> rows_idx(ncols);
    std::vector<std::vector<double>> rows_val(ncols);
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t] {
            for (int64_t i = t; i < ncols; i += nthreads) {
                const Column<T> c = construct_column(in, cols[i], o, false);
                status[i] = c.status;
                fits[i] = static_cast<int32_t>(c.fits);
                growths[i] = static_cast<int32_t>(c.growths);
                clamps[i] = static_cast<int32_t>(c.score_clamps);
                residual[i] = static_cast<double>(c.residual);
                assembly_bad[i] = 0;
                for (size_t e = 0; e < c.pattern.size(); ++e) {
                    const int64_t j = c.pattern[e];
                    const T value = c.coefficients[e] * in.d[j];
                    if (!std::isfinite(value) || (c.coefficients[e] != 0 && value == 0))
                        assembly_bad[i] = 1;
                    if (value != 0) {
                        rows_idx[i].push_back(j);
                        rows_val[i].push_back(static_cast<double>(value));
                    }
                }
            }
        });
    for (auto &th : pool)
        th.join();
    int64_t total = 0;
    p_ptr[0] = 0;
    for (int64_t i = 0; i < ncols; ++i) {
        total += static_cast<int64_t>(rows_idx[i].size());
        p_ptr[i + 1] = total;
    }
    if (total > cap)
        return total;
    for (int64_t i = 0; i < ncols; ++i) {
        std::copy(rows_idx[i].begin(), rows_idx[i].end(), p_idx + p_ptr[i]);
        std::copy(rows_val[i].begin(), rows_val[i].end(), p_val + p_ptr[i]);
    }
    return total;
}

} // namespace orc

// ------------------------------------------------------------------------------------------
// C interface for the Python test harness (ctypes).
// ------------------------------------------------------------------------------------------
using namespace orc;

struct OracleSpai {
    int precision;
    SpaiResult<double> r64;
    SpaiResult<float> r32;
};

extern "C" {

// Threads used by the SPAI construction's column fits (results do not depend on it).
void oracle_set_threads(int threads) {
    g_threads = threads < 1 ? 1 : threads;
}

double oracle_hypot(double a, double b) {
    return cr_hypot(a, b);
}
float oracle_hypotf(float a, float b) {
    return cr_hypotf(a, b);
}

// Score guard KAT entry (spai.cpp:273-306). out = {status, score, clamped}.
void oracle_score(int precision, double rsq, double dot, double den, double *out) {
    if (precision == 1) {
        const auto s = evaluate_score<float>(static_cast<float>(rsq), static_cast<float>(dot),
                                             static_cast<float>(den));
        out[0] = s.status;
        out[1] = s.score;
        out[2] = s.clamped;
    } else {
        const auto s = evaluate_score<double>(rsq, dot, den);
        out[0] = s.status;
        out[1] = s.score;
        out[2] = s.clamped;
    }
}

// precision 0 = binary64 SPAI of A; 1 = binary32 SPAI of A rounded to binary32.
void *oracle_spai(int precision, int64_t n, const int64_t *ptr, const int64_t *idx,
                  const double *val, double epsilon, int64_t alpha, int64_t beta,
                  int keep_history) {
    auto *h = new OracleSpai();
    h->precision = precision;
    SpaiOptions o;
    o.epsilon = epsilon;
    o.alpha = alpha;
    o.beta = beta;
    const Csr<double> a = make_csr(n, ptr, idx, val);
    if (precision == 1)
        h->r32 = construct_spai(to_float(a), o, keep_history != 0);
    else
        h->r64 = construct_spai(a, o, keep_history != 0);
    return h;
}
// info = {status, first_failed_column, nnz(P)}
void oracle_spai_info(void *hp, int64_t *info) {
    auto *h = static_cast<OracleSpai *>(hp);
    if (h->precision == 1) {
        info[0] = h->r32.status;
        info[1] = h->r32.first_failed_column;
        info[2] = h->r32.p.nnz();
    } else {
        info[0] = h->r64.status;
        info[1] = h->r64.first_failed_column;
        info[2] = h->r64.p.nnz();
    }
}
void oracle_spai_p(void *hp, int64_t *ptr, int64_t *idx, double *val) {
    auto *h = static_cast<OracleSpai *>(hp);
    auto copy = [&](const auto &p) {
        std::copy(p.ptr.begin(), p.ptr.end(), ptr);
        std::copy(p.idx.begin(), p.idx.end(), idx);
        for (size_t i = 0; i < p.val.size(); ++i)
            val[i] = p.val[i];
    };
    if (h->precision == 1)
        copy(h->r32.p);
    else
        copy(h->r64.p);
}
// Per column: status, fits, growths, score_clamps, pattern size; residual; scaling.
void oracle_spai_columns(void *hp, int32_t *status, int32_t *fits, int32_t *growths,
                         int32_t *clamps, int32_t *qsize, double *residual, double *scaling) {
    auto *h = static_cast<OracleSpai *>(hp);
    auto fill = [&](const auto &r) {
        for (size_t k = 0; k < r.columns.size(); ++k) {
            const auto &c = r.columns[k];
            status[k] = c.status;
            fits[k] = static_cast<int32_t>(c.fits);
            growths[k] = static_cast<int32_t>(c.growths);
            clamps[k] = static_cast<int32_t>(c.score_clamps);
            qsize[k] = static_cast<int32_t>(c.pattern.size());
            residual[k] = c.residual;
            scaling[k] = r.scaling.empty() ? NAN : static_cast<double>(r.scaling[k]);
        }
    };
    if (h->precision == 1)
        fill(h->r32);
    else
        fill(h->r64);
}
// Solved pattern and coefficients of column k (binary64 view).
int64_t oracle_spai_column(void *hp, int64_t k, int64_t *pattern, double *coef) {
    auto *h = static_cast<OracleSpai *>(hp);
    auto get = [&](const auto &r) -> int64_t {
        const auto &c = r.columns[k];
        for (size_t i = 0; i < c.pattern.size(); ++i) {
            if (pattern)
                pattern[i] = c.pattern[i];
            if (coef)
                coef[i] = c.coefficients[i];
        }
        return static_cast<int64_t>(c.pattern.size());
    };
    return h->precision == 1 ? get(h->r32) : get(h->r64);
}
// History of column k, fit f: sizes {q, m, c, selected} then arrays if non-null.
int oracle_spai_fit(void *hp, int64_t k, int64_t f, int64_t *sizes, int64_t *pattern,
                    int64_t *shadow, int64_t *candidates, int64_t *selected, double *scores,
                    double *coef, double *scalars) {
    auto *h = static_cast<OracleSpai *>(hp);
    auto get = [&](const auto &r) -> int {
        const auto &c = r.columns[k];
        if (f >= static_cast<int64_t>(c.history.size()))
            return -1;
        const auto &fit = c.history[f];
        sizes[0] = fit.pattern.size();
        sizes[1] = fit.shadow.size();
        sizes[2] = fit.candidates.size();
        sizes[3] = fit.selected.size();
        sizes[4] = fit.scores.size();
        if (pattern)
            std::copy(fit.pattern.begin(), fit.pattern.end(), pattern);
        if (shadow)
            std::copy(fit.shadow.begin(), fit.shadow.end(), shadow);
        if (candidates)
            std::copy(fit.candidates.begin(), fit.candidates.end(), candidates);
        if (selected)
            std::copy(fit.selected.begin(), fit.selected.end(), selected);
        if (scores)
            for (size_t i = 0; i < fit.scores.size(); ++i)
                scores[i] = fit.scores[i];
        if (coef)
            for (size_t i = 0; i < fit.coefficients.size(); ++i)
                coef[i] = fit.coefficients[i];
        if (scalars) {
            scalars[0] = fit.residual;
            scalars[1] = fit.mean_score;
            scalars[2] = fit.pivot_ratio;
        }
        return 0;
    };
    return h->precision == 1 ? get(h->r32) : get(h->r64);
}
void oracle_spai_free(void *hp) {
    delete static_cast<OracleSpai *>(hp);
}

// GMRES with an explicit preconditioner P (binary64 or binary32 arithmetic).
// rep = {status, converged, iterations, final_original, final_relative}
void oracle_gmres(int precision, int64_t n, const int64_t *aptr, const int64_t *aidx,
                  const double *aval, const int64_t *pptr, const int64_t *pidx, const double *pval,
                  const double *rhs, double tolerance, int64_t cap, int accept_every,
                  int lazy, int wide, double *x_out, double *rep) {
    GmresOptions o;
    o.wide_reductions = wide;
    o.tolerance = tolerance;
    o.max_iterations = cap;
    o.accept_every_iteration = accept_every;
    o.lazy_candidates = lazy;
    const Csr<double> a = make_csr(n, aptr, aidx, aval), p = make_csr(n, pptr, pidx, pval);
    GmresReport g;
    if (precision == 1) {
        std::vector<float> b(rhs, rhs + n), x;
        g = gmres(to_float(a), to_float(p), b, o, x);
        for (int64_t i = 0; i < n && i < static_cast<int64_t>(x.size()); ++i)
            x_out[i] = x[i];
    } else {
        std::vector<double> b(rhs, rhs + n), x;
        g = gmres(a, p, b, o, x);
        for (int64_t i = 0; i < n && i < static_cast<int64_t>(x.size()); ++i)
            x_out[i] = x[i];
    }
    rep[0] = g.status;
    rep[1] = g.converged;
    rep[2] = static_cast<double>(g.iterations);
    rep[3] = g.final_original;
    rep[4] = g.final_relative;
}

// Full SPAI-GMRES-IR pipeline. precision: 0 = FP64 (cuda_gpu_spai_gmres_ir semantics),
// 1 = FP32 (fp32_cuda_spai_gmres_ir semantics), 2 = mixed (FP32 SPAI/GMRES, FP64 IR).
// opts = {epsilon, alpha, beta, tau, innercap, outercap, be_tolerance, lazy, wide}; wide < 0 =
// by precision (binary64-accumulated binary32 reductions for the mixed form, sequential binary32
// sums for the FP32 form, whose goldens come from the reference's CPU FP32 solver).
// rep  = {status, converged, outer_steps, inner_attempts, inner_iterations, nbe, cbe,
//         residual_inf, forward, spai_status, nnz_p, last_inner_status, spai_seconds,
//         refine_seconds}
int oracle_ir(int precision, int64_t n, const int64_t *ptr, const int64_t *idx, const double *val,
              const double *b, const double *reference, const double *opts, double *x_out,
              double *rep) {
    IrOptions o;
    o.spai.epsilon = opts[0];
    o.spai.alpha = static_cast<int64_t>(opts[1]);
    o.spai.beta = static_cast<int64_t>(opts[2]);
    o.gmres.tolerance = opts[3];
    o.gmres.max_iterations = static_cast<int64_t>(opts[4]);
    o.max_outer = static_cast<int64_t>(opts[5]);
    o.be_tolerance = opts[6];
    o.gmres.lazy_candidates = static_cast<int>(opts[7]);
    o.gmres.accept_every_iteration = precision == 1;
    o.gmres.wide_reductions = opts[8] < 0 ? (precision == 2 ? 1 : 0) : static_cast<int>(opts[8]);
    IrReport r;
    const Csr<double> a = make_csr(n, ptr, idx, val);
    bool finite_rhs = true;
    for (int64_t i = 0; i < n; ++i)
        finite_rhs = finite_rhs && std::isfinite(b[i]);
    if (o.max_outer > 20 || o.gmres.max_iterations > n || !finite_rhs ||
        !std::isfinite(o.gmres.tolerance) || o.gmres.tolerance <= 0) {
        rep[0] = I_INVALID_INPUT;
        return I_INVALID_INPUT;
    }
    using clk = std::chrono::steady_clock;
    const auto t_start = clk::now();
    auto t_spai = t_start;
    if (precision == 0) {
        const auto s = construct_spai(a, o.spai, false);
        t_spai = clk::now();
        r.spai_status = s.status;
        r.nnz_p = s.p.nnz();
        if (s.status != S_SUCCESS) {
            r.status = I_CONSTRUCTION_FAILURE;
        } else {
            std::vector<double> rhs(b, b + n), x;
            r = refine64(a, a, s.p, rhs, o, reference, x);
            r.spai_status = s.status;
            r.nnz_p = s.p.nnz();
            std::copy(x.begin(), x.end(), x_out);
        }
    } else {
        const Csr<float> af = to_float(a);
        const auto s = construct_spai(af, o.spai, false);
        t_spai = clk::now();
        r.spai_status = s.status;
        r.nnz_p = s.p.nnz();
        if (s.status != S_SUCCESS) {
            r.status = I_CONSTRUCTION_FAILURE;
        } else if (precision == 1) {
            std::vector<float> rhs(n), x;
            for (int64_t i = 0; i < n; ++i)
                rhs[i] = static_cast<float>(b[i]);
            r = refine32(af, s.p, rhs, o, x);
            for (int64_t i = 0; i < n && i < static_cast<int64_t>(x.size()); ++i)
                x_out[i] = x[i];
        } else {
            std::vector<double> rhs(b, b + n), x;
            r = refine64(a, af, s.p, rhs, o, reference, x);
            std::copy(x.begin(), x.end(), x_out);
        }
        r.spai_status = s.status;
        r.nnz_p = s.p.nnz();
    }
    rep[0] = r.status;
    rep[1] = r.converged;
    rep[2] = static_cast<double>(r.outer_steps);
    rep[3] = static_cast<double>(r.inner_attempts);
    rep[4] = static_cast<double>(r.inner_iterations);
    rep[5] = r.nbe;
    rep[6] = r.cbe;
    rep[7] = r.residual_inf;
    rep[8] = r.forward;
    rep[9] = r.spai_status;
    rep[10] = static_cast<double>(r.nnz_p);
    rep[11] = r.last_inner_status;
    rep[12] = std::chrono::duration<double>(t_spai - t_start).count();
    rep[13] = std::chrono::duration<double>(clk::now() - t_spai).count();
    return r.status;
}

double oracle_spai_sample(int precision, int64_t n, const int64_t *ptr, const int64_t *idx,
                          const double *val, double epsilon, int64_t alpha, int64_t beta,
                          const int64_t *cols, int64_t ncols, int nthreads, int64_t *fits_out) {
    SpaiOptions o;
    o.epsilon = epsilon;
    o.alpha = alpha;
    o.beta = beta;
    const Csr<double> a = make_csr(n, ptr, idx, val);
    if (precision == 1)
        return spai_sample(to_float(a), o, cols, ncols, nthreads, fits_out);
    return spai_sample(a, o, cols, ncols, nthreads, fits_out);
}

// precision 0 = binary64 SPAI of A, 1 = binary32 SPAI of A rounded to binary32.
int64_t oracle_spai_columns_sample(int precision, int64_t n, const int64_t *ptr, const int64_t *idx,
                                   const double *val, double epsilon, int64_t alpha, int64_t beta,
                                   const int64_t *cols, int64_t ncols, int nthreads, int32_t *status,
                                   int32_t *fits, int32_t *growths, int32_t *clamps, double *residual,
                                   int32_t *assembly_bad, int64_t *p_ptr, int64_t *p_idx, double *p_val,
                                   int64_t cap) {
    SpaiOptions o;
    o.epsilon = epsilon;
    o.alpha = alpha;
    o.beta = beta;
    const Csr<double> a = make_csr(n, ptr, idx, val);
    if (precision == 1)
        return spai_columns_sample(to_float(a), o, cols, ncols, nthreads, status, fits, growths, clamps,
                                   residual, assembly_bad, p_ptr, p_idx, p_val, cap);
    return spai_columns_sample(a, o, cols, ncols, nthreads, status, fits, growths, clamps, residual,
                               assembly_bad, p_ptr, p_idx, p_val, cap);
}

// IR with a given preconditioner (refine_with_preconditioner, ir.cpp:138-204), binary64.
int oracle_refine(int64_t n, const int64_t *ptr, const int64_t *idx, const double *val,
                  const int64_t *pptr, const int64_t *pidx, const double *pval, const double *b,
                  const double *reference, const double *opts, double *x_out, double *rep) {
    IrOptions o;
    o.gmres.tolerance = opts[3];
    o.gmres.max_iterations = static_cast<int64_t>(opts[4]);
    o.max_outer = static_cast<int64_t>(opts[5]);
    o.be_tolerance = opts[6];
    o.gmres.lazy_candidates = static_cast<int>(opts[7]);
    const Csr<double> a = make_csr(n, ptr, idx, val), p = make_csr(n, pptr, pidx, pval);
    std::vector<double> rhs(b, b + n), x;
    IrReport r;
    if (o.max_outer > 20 || o.gmres.max_iterations > n)
        r.status = I_INVALID_INPUT;
    else
        r = refine64(a, a, p, rhs, o, reference, x);
    std::copy(x.begin(), x.end(), x_out);
    rep[0] = r.status;
    rep[1] = r.converged;
    rep[2] = static_cast<double>(r.outer_steps);
    rep[3] = static_cast<double>(r.inner_attempts);
    rep[4] = static_cast<double>(r.inner_iterations);
    rep[5] = r.nbe;
    rep[6] = r.cbe;
    rep[7] = r.residual_inf;
    rep[8] = r.forward;
    rep[9] = S_SUCCESS;
    rep[10] = static_cast<double>(p.nnz());
    rep[11] = r.last_inner_status;
    return r.status;
}

} // extern "C"
