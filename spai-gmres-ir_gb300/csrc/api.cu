// C ABI of libspai_ir.so: handle management, uploads, SPAI build, refinement solves.
// The entry points and their reference counterparts are listed in include/spai_ir.h.
#include "adjoint.cuh"
#include "krylov_kernels.cuh"
#include "spai_ir.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <type_traits>
#include <string>
#include <vector>

using namespace spai;

namespace spai_api {
thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

template <class TD, class TS>
__global__ void convert_kernel(long long count, const TS *src, TD *dst) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        dst[i] = static_cast<TD>(src[i]);
}

// Device form of the canonical CSR check below, fused with the int64 -> int32 narrowing of the
// upload: offsets within [0, nnz] and nondecreasing, columns in range and strictly increasing per
// row, values finite and nonzero. Offsets are clamped into [0, nnz] before use and a row whose
// offsets decrease is skipped, so no read leaves the arrays whatever the input; *bad != 0 means
// canonical_error (host) names the first violation.
// bad[1] receives the longest row (the sparsity profile's max_row) of a valid matrix.
__global__ void csr_offsets_kernel(long long n, long long nnz, const long long *rp64, int *rp32, int *bad) {
    int longest = 0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i <= n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long v = rp64[i];
        if (v < 0 || v > nnz || (i < n && rp64[i + 1] < v))
            bad[0] = 1;
        else if (i < n && rp64[i + 1] - v > longest)
            longest = static_cast<int>(min(rp64[i + 1] - v, nnz));
        rp32[i] = static_cast<int>(v < 0 ? 0 : (v > nnz ? nnz : v));
    }
    if (longest > 0)
        atomicMax(bad + 1, longest);
}
__global__ void csr_entries_kernel(int n, const int *rp32, const long long *ci64, const double *val, int *ci32,
                                   int *bad) {
    int flag = 0;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        const int b = rp32[row], e = rp32[row + 1];
        long long prev = -1;
        for (int t = b; t < e; ++t) {
            const long long c = ci64[t];
            const double v = val[t];
            flag |= c < 0 || c >= n || c <= prev || !isfinite(v) || v == 0.0;
            ci32[t] = static_cast<int>(c < 0 || c >= n ? 0 : c);
            prev = c;
        }
    }
    if (flag)
        *bad = 1;
}

// Canonical CSR check (src/cuda_spai.cu:452-470): offsets monotone from 0 to nnz, columns in
// range and strictly increasing per row, values finite and nonzero.
// The O(1) part: pointers, sizes, first and last offset (checked before any upload).
std::string canonical_header_error(const spai_csr *a) {
    if (!a || a->n <= 0 || a->nnz < 0 || !a->row_offsets || (a->nnz > 0 && (!a->col_indices || !a->values)))
        return "CSR pointers/sizes invalid";
    if (a->n > INT_MAX - 1 || a->nnz > INT_MAX - 1)
        return "matrix exceeds 32-bit device index range";
    if (a->row_offsets[0] != 0 || a->row_offsets[a->n] != a->nnz)
        return "row offsets must run from 0 to nnz";
    return "";
}
std::string canonical_error(const spai_csr *a) {
    const std::string head = canonical_header_error(a);
    if (!head.empty())
        return head;
    for (int64_t r = 0; r < a->n; ++r) {
        const int64_t b = a->row_offsets[r], e = a->row_offsets[r + 1];
        if (b > e)
            return "row offsets must be nondecreasing";
        for (int64_t t = b; t < e; ++t) {
            const int64_t c = a->col_indices[t];
            if (c < 0 || c >= a->n)
                return "column index outside matrix";
            if (t > b && a->col_indices[t - 1] >= c)
                return "column indices must be strictly increasing within a row";
            if (!std::isfinite(a->values[t]) || a->values[t] == 0)
                return "values must be finite and nonzero (canonical CSR)";
        }
    }
    return "";
}

int sm_count(int device) {
    int sms = 0;
    SPAI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    return sms;
}

struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t st;
    explicit EventTimer(cudaStream_t s) : st(s) {
        SPAI_CUDA(cudaEventCreate(&a));
        SPAI_CUDA(cudaEventCreate(&b));
        SPAI_CUDA(cudaEventRecord(a, st));
    }
    double stop() {
        SPAI_CUDA(cudaEventRecord(b, st));
        SPAI_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        SPAI_CUDA(cudaEventElapsedTime(&ms, a, b));
        return ms;
    }
    ~EventTimer() {
        if (a)
            cudaEventDestroy(a);
        if (b)
            cudaEventDestroy(b);
    }
};
} // namespace spai_api
using namespace spai_api;

struct spai_handle_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int precision = SPAI_PREC_F64;
    int n = 0, nnz = 0, sms = 0;
    DeviceArena mat, build, solve, scratch;
    DeviceCsr<double> a64;
    DeviceCsr<float> a32;
    SpaiOutput<double> s64;
    SpaiOutput<float> s32;
    bool built = false;
    int spai_status = SPAI_NOT_ATTEMPTED;
    int *pinned = nullptr;
    IrEngine<double, double> e64;
    IrEngine<float, double> emix;
    IrEngine<float, float> e32;
    int engine_cap = -1;
    bool engine_right = false; // the engine runs right-preconditioned GMRES
    // Adjoint solves A^T lambda = g: transposes of A and P built on first use after a build, and
    // engines in right-preconditioned mode over them.
    DeviceArena adj, adj_solve, conv;
    DeviceCsr<double> at64, pt64;
    DeviceCsr<float> at32, pt32;
    bool adj_ready = false;
    IrEngine<double, double> j64;
    IrEngine<float, double> jmix;
    IrEngine<float, float> j32;
    int adj_cap = -1;
    // History of the last solve run with SPAI_FLAG_HISTORY (device records + counts).
    const spai_outer_record *hist_outer = nullptr;
    const spai_inner_record *hist_inner = nullptr;
    const spai_iteration_record *hist_iter = nullptr;
    int hist_n_outer = 0, hist_n_inner = 0, hist_n_iter = 0;
    int hist_cap_outer = 0, hist_cap_inner = 0, hist_cap_iter = 0;
    KernelProfile prof;
    // Record mode (spai_record): fit log of the next builds, step records of the next solves.
    bool recording = false;
    KrylovRecord krec;
    bool p_supplied = false; // P came from spai_set_preconditioner (no SPAI columns)
    double spai_ms = 0;
    long long spai_launches = 0;

    bool inner_f32() const {
        return precision != SPAI_PREC_F64;
    }
    ~spai_handle_s() {
        if (stream)
            cudaStreamSynchronize(stream);
        if (pinned)
            cudaFreeHost(pinned);
        if (own_stream && stream)
            cudaStreamDestroy(stream);
    }
};

void handle_view(spai_handle_s *h, spai::HandleView &v) {
    v.precision = h->precision;
    v.device = h->device;
    v.sms = h->sms;
    v.stream = h->stream;
    v.a64 = &h->a64;
}
int spai_api_fail(int code, const std::string &msg) {
    return spai_api::fail(code, msg);
}

namespace spai_api {

void fill_defaults(spai_options *o, int32_t precision) {
    o->epsilon = 0.3;
    o->alpha = 5;
    o->beta = 8;
    o->tau = 0;
    o->innercap = 0;
    o->outercap = 20;
    o->be_tolerance = 0;
    o->precision = precision;
    o->flags = 0;
}

double inner_tau(const spai_options &o) {
    if (o.tau > 0)
        return o.tau;
    return o.precision == SPAI_PREC_F64 ? 1e-8 : 1e-4;
}
double be_tol(const spai_options &o) {
    if (o.be_tolerance > 0)
        return o.be_tolerance;
    return o.precision == SPAI_PREC_F32 ? 10 * std::ldexp(1.0, -24) : 10 * std::ldexp(1.0, -53);
}

void clear_report(spai_report *r) {
    std::memset(r, 0, sizeof(*r));
    r->ir_status = IR_INVALID_INPUT;
    r->spai_status = SPAI_NOT_ATTEMPTED;
    r->gmres_status = -1;
    r->first_failed_column = -1;
    r->backward_error = NAN;
    r->componentwise_backward_error = NAN;
    r->residual_inf = NAN;
    r->forward_error = NAN;
}

// Solve engine for `cap` inner steps; right: GMRES on A P d = rhs with x = P d (the form flexible
// GMRES takes with one fixed preconditioner), else the reference's left-preconditioned P A.
void ensure_engine(spai_handle *h, int cap, bool right = false) {
    if (h->engine_cap == cap && h->engine_right == right)
        return;
    h->solve.reset();
    const int sms = h->sms;
    if (h->precision == SPAI_PREC_F64)
        h->e64.setup(h->solve, h->a64, h->a64, h->s64.p, cap, sms, right);
    else if (h->precision == SPAI_PREC_MIXED)
        h->emix.setup(h->solve, h->a64, h->a32, h->s32.p, cap, sms, right);
    else
        h->e32.setup(h->solve, h->a32, h->a32, h->s32.p, cap, sms, right);
    h->e64.prof = h->emix.prof = h->e32.prof = &h->prof;
    h->engine_cap = cap;
    h->engine_right = right;
}

template <class E> void read_ctl(spai_handle *h, E &e, Ctl &c) {
    SPAI_CUDA(cudaMemcpyAsync(&c, e.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->stream));
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
}

void fill_from_ctl(const Ctl &c, spai_report *rep) {
    rep->ir_status = c.ir_status < 0 ? IR_ITERATION_LIMIT : c.ir_status;
    rep->converged = c.ir_status == IR_SUCCESS;
    rep->outer_steps = c.outer_steps;
    rep->inner_attempts = c.inner_attempts;
    rep->inner_iterations = c.inner_iterations_total;
    rep->gmres_status = c.last_gmres_status;
    rep->backward_error = c.be;
    rep->componentwise_backward_error = c.cbe;
    rep->residual_inf = c.rinf;
}

// Validation of IrOptions against the matrix (src/ir.cpp:41-55): failures are reported as
// IrStatus::invalid_input, not as API errors.
bool options_valid(const spai_handle *h, const spai_options &o) {
    return o.outercap >= 0 && o.outercap <= 20 && o.innercap >= 0 && o.innercap <= h->n &&
           std::isfinite(inner_tau(o)) && inner_tau(o) > 0 && o.alpha >= 0 && o.beta >= 0;
}

// Build the transposes of A and P once per build, and the right-preconditioned engines for `cap`.
void ensure_adjoint(spai_handle *h, int cap) {
    cudaStream_t st = h->stream;
    if (!h->adj_ready) {
        h->adj.reset();
        const TransposePlan ta = transpose_plan(h->adj, h->a64, h->sms, st);
        h->at64 = transpose_values(h->adj, ta, h->a64.val, h->sms, st);
        if (h->inner_f32()) {
            h->at32 = transpose_values(h->adj, ta, h->a32.val, h->sms, st);
            const TransposePlan tp = transpose_plan(h->adj, h->s32.p, h->sms, st);
            h->pt32 = transpose_values(h->adj, tp, h->s32.p.val, h->sms, st);
        } else {
            const TransposePlan tp = transpose_plan(h->adj, h->s64.p, h->sms, st);
            h->pt64 = transpose_values(h->adj, tp, h->s64.p.val, h->sms, st);
        }
        SPAI_CUDA(cudaStreamSynchronize(st));
        h->adj_ready = true;
        h->adj_cap = -1;
    }
    if (h->adj_cap == cap)
        return;
    h->adj_solve.reset();
    if (h->precision == SPAI_PREC_F64)
        h->j64.setup(h->adj_solve, h->at64, h->at64, h->pt64, cap, h->sms, true);
    else if (h->precision == SPAI_PREC_MIXED)
        h->jmix.setup(h->adj_solve, h->at64, h->at32, h->pt32, cap, h->sms, true);
    else
        h->j32.setup(h->adj_solve, h->at32, h->at32, h->pt32, cap, h->sms, true);
    h->adj_cap = cap;
}

// One refinement solve on the engine of the handle's precision; b, x device binary64 vectors.
template <class E> void keep_history(spai_handle *h, const E &e, const Ctl &c, const SolveSettings &s) {
    if (!s.history)
        return;
    h->hist_outer = e.hist_outer;
    h->hist_inner = e.hist_inner;
    h->hist_iter = e.hist_iter;
    h->hist_cap_outer = e.hist_cap_outer;
    h->hist_cap_inner = e.hist_cap_inner;
    h->hist_cap_iter = e.hist_cap_iter;
    h->hist_n_outer = c.h_n_outer;
    h->hist_n_inner = c.h_n_inner;
    h->hist_n_iter = c.h_n_iter;
}

template <class E64, class EMX, class E32>
void run_solve(spai_handle *h, E64 &e64, EMX &emix, E32 &e32, const double *d_b, double *d_x,
               const SolveSettings &s, spai_report *rep) {
    EventTimer timer(h->stream);
    Ctl c{};
    if (h->precision == SPAI_PREC_F64) {
        e64.solve(h->stream, d_b, d_x, s, h->pinned);
        rep->solve_ms = timer.stop();
        read_ctl(h, e64, c);
        keep_history(h, e64, c, s);
        rep->kernel_launches = e64.graph_mode ? e64.graph_kernels(c) : e64.launches;
    } else if (h->precision == SPAI_PREC_MIXED) {
        emix.solve(h->stream, d_b, d_x, s, h->pinned);
        rep->solve_ms = timer.stop();
        read_ctl(h, emix, c);
        keep_history(h, emix, c, s);
        rep->kernel_launches = emix.graph_mode ? emix.graph_kernels(c) : emix.launches;
    } else {
        // binary32 drop-in: b rounded to binary32, refinement in binary32.
        h->conv.reset();
        float *bf = h->conv.alloc<float>(h->n);
        float *xf = h->conv.alloc<float>(h->n);
        convert_kernel<float, double><<<grid_for(h->n, 256, h->sms * 8), 256, 0, h->stream>>>(h->n, d_b, bf);
        SPAI_LAUNCH("convert_kernel");
        e32.solve(h->stream, bf, xf, s, h->pinned);
        convert_kernel<double, float><<<grid_for(h->n, 256, h->sms * 8), 256, 0, h->stream>>>(h->n, xf, d_x);
        SPAI_LAUNCH("convert_kernel");
        rep->solve_ms = timer.stop();
        read_ctl(h, e32, c);
        keep_history(h, e32, c, s);
        rep->kernel_launches = (e32.graph_mode ? e32.graph_kernels(c) : e32.launches) + 2;
    }
    fill_from_ctl(c, rep);
}

SolveSettings settings_for(const spai_handle *h, const spai_options &o, int cap) {
    SolveSettings s;
    s.cap = cap;
    s.outer_cap = static_cast<int>(o.outercap);
    s.tau = inner_tau(o);
    s.be_tol = be_tol(o);
    s.scale_rhs = h->precision == SPAI_PREC_MIXED;
    s.accept_every = h->precision == SPAI_PREC_F32;
    s.use_graph = (o.flags & SPAI_FLAG_NO_GRAPH) == 0;
    s.history = (o.flags & SPAI_FLAG_HISTORY) != 0;
    s.restart_at_cap = (o.flags & SPAI_FLAG_RESTART_AT_CAP) != 0;
    return s;
}

// Solve with device vectors b, x (binary64). Returns SPAI_OK and fills rep.
int solve_device_impl(spai_handle *h, const double *d_b, double *d_x, const spai_options &o,
                      spai_report *rep) {
    if (!h->built)
        return fail(SPAI_ERR_NOT_BUILT, "spai_solve before a successful spai_build");
    rep->spai_status = h->spai_status;
    rep->spai_ms = h->spai_ms;
    if (h->spai_status != SPAI_SUCCESS) {
        rep->ir_status = IR_CONSTRUCTION_FAILURE;
        return SPAI_OK;
    }
    if (!options_valid(h, o)) {
        rep->ir_status = IR_INVALID_INPUT;
        return SPAI_OK;
    }
    const int cap = o.innercap == 0 ? h->n : static_cast<int>(o.innercap);
    ensure_engine(h, cap, (o.flags & SPAI_FLAG_RIGHT_PRECONDITIONING) != 0);
    SolveSettings s = settings_for(h, o, cap);
    if (h->recording) { // record mode: host-driven loop, every step read back (binary64 handles)
        if (static_cast<double>(h->n) * (cap + 1) * (o.outercap + 1) > static_cast<double>(1 << 28))
            return fail(SPAI_ERR_ARGUMENT, "record mode keeps every step's candidate in host memory: "
                                           "n * (innercap + 1) * (outercap + 1) must stay below 2^28");
        h->krec.clear();
        s.record = &h->krec;
        s.history = true;
        s.use_graph = false;
    }
    run_solve(h, h->e64, h->emix, h->e32, d_b, d_x, s, rep);
    rep->nnz_p = h->precision == SPAI_PREC_F64 ? h->s64.p.nnz : h->s32.p.nnz;
    return SPAI_OK;
}

// Adjoint of x_r = A^{-1} b_r for r < nrhs (device, column-major n x nrhs): lambda_r solves
// A^T lambda_r = g_r by refinement whose inner GMRES is right-preconditioned with P^T; then
// dLdb = lambda and dLdA[e] = -sum_r lambda_r[i] x_r[j]. The report aggregates the solves:
// converged iff all converged, the first non-success status, the largest backward error and
// outer step count, summed inner iterations, launches and solve time.
int adjoint_device_impl(spai_handle *h, int nrhs, const double *d_x, const double *d_g, double *d_lambda,
                        double *d_dlda, const spai_options &o, spai_report *rep) {
    if (!h->built)
        return fail(SPAI_ERR_NOT_BUILT, "spai_adjoint before a successful spai_build");
    rep->spai_status = h->spai_status;
    rep->spai_ms = h->spai_ms;
    if (h->spai_status != SPAI_SUCCESS) {
        rep->ir_status = IR_CONSTRUCTION_FAILURE;
        return SPAI_OK;
    }
    if (!options_valid(h, o)) {
        rep->ir_status = IR_INVALID_INPUT;
        return SPAI_OK;
    }
    const int n = h->n;
    const int cap = o.innercap == 0 ? n : static_cast<int>(o.innercap);
    ensure_adjoint(h, cap);
    const SolveSettings s = settings_for(h, o, cap);
    spai_report agg = *rep;
    agg.ir_status = IR_SUCCESS;
    agg.converged = 1;
    agg.backward_error = 0;
    agg.componentwise_backward_error = 0;
    agg.residual_inf = 0;
    agg.solve_ms = 0;
    agg.kernel_launches = 0;
    for (int r = 0; r < nrhs; ++r) {
        const size_t off = static_cast<size_t>(r) * n;
        spai_report one = *rep;
        run_solve(h, h->j64, h->jmix, h->j32, d_g + off, d_lambda + off, s, &one);
        if (!one.converged && agg.converged) {
            agg.converged = 0;
            agg.ir_status = one.ir_status;
            agg.gmres_status = one.gmres_status;
        }
        if (agg.converged)
            agg.gmres_status = one.gmres_status;
        agg.outer_steps = std::max(agg.outer_steps, one.outer_steps);
        agg.inner_attempts += one.inner_attempts;
        agg.inner_iterations += one.inner_iterations;
        agg.backward_error = std::max(agg.backward_error, one.backward_error);
        agg.componentwise_backward_error = std::max(agg.componentwise_backward_error, one.componentwise_backward_error);
        agg.residual_inf = std::max(agg.residual_inf, one.residual_inf);
        agg.solve_ms += one.solve_ms;
        agg.kernel_launches += one.kernel_launches;
    }
    EventTimer timer(h->stream);
    sampled_outer_kernel<<<grid_for(n, 256, h->sms * 8), 256, 0, h->stream>>>(n, nrhs, h->a64.rp, h->a64.ci,
                                                                           d_lambda, d_x, d_dlda);
    SPAI_LAUNCH("sampled_outer_kernel");
    agg.solve_ms += timer.stop();
    agg.kernel_launches += 1;
    agg.nnz_p = h->precision == SPAI_PREC_F64 ? h->s64.p.nnz : h->s32.p.nnz;
    *rep = agg;
    return SPAI_OK;
}

#define API_BEGIN try {
#define API_END                                                                                    \
    }                                                                                              \
    catch (const spai::ArgumentError &e) {                                                         \
        return fail(SPAI_ERR_ARGUMENT, e.what());                                                  \
    }                                                                                              \
    catch (const spai::WorkspaceError &e) {                                                        \
        return fail(SPAI_ERR_WORKSPACE, e.what());                                                 \
    }                                                                                              \
    catch (const std::exception &e) {                                                              \
        return fail(SPAI_ERR_CUDA, e.what());                                                      \
    }

} // namespace spai_api

namespace spai_api {
// Host CSR -> device CSR in `dst` (64-bit indices narrowed on the device through the handle's
// scratch arena), checked on the device for the canonical form on the way; stream-ordered. The
// caller synchronises and, when bad[0] is set, reports canonical_error's message; bad[1] is then
// the longest row. `a` must pass canonical_header_error.
DeviceCsr<double> upload_csr(spai_handle *h, DeviceArena &dst, const spai_csr *a, int *bad) {
    const int n = static_cast<int>(a->n), nnz = static_cast<int>(a->nnz);
    DeviceCsr<double> m;
    m.n = n;
    m.nnz = nnz;
    m.max_row = 0; // bad[1] after the caller's synchronisation
    m.rp = dst.alloc<int>(n + 1);
    m.ci = dst.alloc<int>(nnz > 0 ? nnz : 1);
    m.val = dst.alloc<double>(nnz > 0 ? nnz : 1);
    long long *tmp = h->scratch.alloc<long long>(std::max(n + 1, nnz));
    cudaStream_t st = h->stream;
    SPAI_CUDA(cudaMemsetAsync(bad, 0, 2 * sizeof(int), st));
    SPAI_CUDA(cudaMemcpyAsync(tmp, a->row_offsets, sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, st));
    csr_offsets_kernel<<<grid_for(n + 1, 256, h->sms * 8), 256, 0, st>>>(n, nnz, tmp, m.rp, bad);
    SPAI_LAUNCH("csr_offsets_kernel");
    if (nnz > 0) {
        // The index copy reuses tmp after the row offsets are narrowed (stream order).
        SPAI_CUDA(cudaMemcpyAsync(m.val, a->values, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
        SPAI_CUDA(cudaMemcpyAsync(tmp, a->col_indices, sizeof(long long) * nnz, cudaMemcpyHostToDevice, st));
        csr_entries_kernel<<<grid_for(n, 256, h->sms * 8), 256, 0, st>>>(n, m.rp, tmp, m.val, m.ci, bad);
        SPAI_LAUNCH("csr_entries_kernel");
    }
    return m;
}
} // namespace spai_api

namespace spai_api {
// Branch-free scans (the compiler vectorises them): an exponent field of all ones is Inf or NaN.
bool all_finite(int64_t n, const double *v) {
    uint64_t bad = 0;
    for (int64_t i = 0; i < n; ++i) {
        uint64_t u;
        std::memcpy(&u, v + i, sizeof u);
        bad |= static_cast<uint64_t>(((u >> 52) & 0x7ff) == 0x7ff);
    }
    return bad == 0;
}
bool finite_inputs(int64_t n, const double *b, const double *reference) {
    return all_finite(n, b) && (!reference || all_finite(n, reference));
}
// spai_solve once b and reference are known to be finite.
int solve_host_impl(spai_handle *h, const double *b, double *x, const double *reference,
                    const spai_options *opt, spai_report *rep) {
    API_BEGIN
    const int n = h->n;
    h->scratch.reset();
    double *db = h->scratch.alloc<double>(n);
    double *dx = h->scratch.alloc<double>(n);
    SPAI_CUDA(cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    const int rc = solve_device_impl(h, db, dx, *opt, rep);
    if (rc != SPAI_OK)
        return rc;
    if (rep->ir_status != IR_CONSTRUCTION_FAILURE && rep->ir_status != IR_INVALID_INPUT) {
        SPAI_CUDA(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
        SPAI_CUDA(cudaStreamSynchronize(h->stream));
        if (reference) {
            double rinf = 0, einf = 0;
            bool overflow = false;
            for (int i = 0; i < n; ++i) {
                rinf = std::max(rinf, std::fabs(reference[i]));
                const double e = std::fabs(x[i] - reference[i]);
                overflow |= !std::isfinite(e);
                einf = std::max(einf, e);
            }
            rep->forward_error = rinf == 0 ? einf : einf / rinf;
            if (overflow || !std::isfinite(rep->forward_error))
                rep->forward_error = INFINITY;
        }
    }
    return SPAI_OK;
    API_END
}
} // namespace spai_api

extern "C" {

int spai_default_options(spai_options *opt, int32_t precision) {
    if (!opt || precision < 0 || precision > 2)
        return fail(SPAI_ERR_ARGUMENT, "spai_default_options: bad arguments");
    fill_defaults(opt, precision);
    return SPAI_OK;
}

const char *spai_status_name(int32_t s) {
    static const char *names[] = {"success",          "not_attempted",     "invalid_input",
                                  "rank_deficient",   "numerical_failure", "empty_candidates",
                                  "zero_denominator", "invalid_score",     "no_growth",
                                  "iteration_limit"};
    return (s >= 0 && s < 10) ? names[s] : "unknown";
}
const char *gmres_status_name(int32_t s) {
    static const char *names[] = {"success",         "zero_rhs",       "exact_initial_solution",
                                  "invalid_input",   "zero_preconditioned_rhs",
                                  "breakdown",       "iteration_limit", "nonconvergence",
                                  "numerical_failure"};
    return (s >= 0 && s < 9) ? names[s] : "unknown";
}
const char *ir_status_name(int32_t s) {
    static const char *names[] = {"success",    "invalid_input",   "construction_failure",
                                  "inner_failure", "stagnation",   "iteration_limit",
                                  "numerical_failure"};
    return (s >= 0 && s < 7) ? names[s] : "unknown";
}
const char *spai_last_error(void) {
    return g_last_error.c_str();
}


int spai_create(const spai_csr *a, int32_t precision, int device, void *stream, spai_handle **out) {
    API_BEGIN
    if (!out || precision < 0 || precision > 2)
        return fail(SPAI_ERR_ARGUMENT, "spai_create: bad arguments");
    *out = nullptr;
    const std::string why = canonical_header_error(a);
    if (!why.empty())
        return fail(SPAI_ERR_ARGUMENT, "spai_create: " + why);
    SPAI_CUDA(cudaSetDevice(device));
    std::unique_ptr<spai_handle> h(new spai_handle());
    h->device = device;
    h->precision = precision;
    h->n = static_cast<int>(a->n);
    h->nnz = static_cast<int>(a->nnz);
    h->sms = sm_count(device);
    if (stream) {
        h->stream = static_cast<cudaStream_t>(stream);
    } else {
        SPAI_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    SPAI_CUDA(cudaMallocHost(&h->pinned, 64));
    const int n = h->n, nnz = h->nnz;
    cudaStream_t st = h->stream;
    h->scratch.reset();
    int *bad = h->scratch.alloc<int>(2);
    h->a64 = upload_csr(h.get(), h->mat, a, bad);
    if (precision != SPAI_PREC_F64) {
        h->a32.n = n;
        h->a32.nnz = nnz;
        h->a32.rp = h->a64.rp;
        h->a32.ci = h->a64.ci;
        h->a32.val = h->mat.alloc<float>(nnz);
        convert_kernel<float, double><<<grid_for(nnz, 256, h->sms * 8), 256, 0, st>>>(nnz, h->a64.val, h->a32.val);
        SPAI_LAUNCH("convert_kernel");
    }
    int h_bad[2] = {0, 0};
    SPAI_CUDA(cudaMemcpyAsync(h_bad, bad, sizeof(h_bad), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    if (h_bad[0]) { // the host check names the first violation
        const std::string full = canonical_error(a);
        return fail(SPAI_ERR_ARGUMENT, "spai_create: " + (full.empty() ? std::string("CSR is not canonical") : full));
    }
    h->a64.max_row = h->a32.max_row = h_bad[1];
    *out = h.release();
    return SPAI_OK;
    API_END
}

int spai_destroy(spai_handle *h) {
    API_BEGIN
    if (!h)
        return SPAI_OK;
    SPAI_CUDA(cudaSetDevice(h->device));
    delete h;
    return SPAI_OK;
    API_END
}

int spai_build(spai_handle *h, const spai_options *opt, spai_report *rep) {
    API_BEGIN
    if (!h || !opt)
        return fail(SPAI_ERR_ARGUMENT, "spai_build: null argument");
    spai_report local;
    if (!rep)
        rep = &local;
    clear_report(rep);
    SPAI_CUDA(cudaSetDevice(h->device));
    h->built = false;
    h->p_supplied = false;
    h->engine_cap = -1;
    h->adj_ready = false;
    h->adj_cap = -1;
    h->build.reset();
    SpaiParams prm;
    // Tuning overrides (group width, per-group workspace) for profiling sweeps.
    if (const char *e = std::getenv("SPAI_GROUP_LANES"))
        prm.group_lanes = std::atoi(e);
    if (const char *e = std::getenv("SPAI_WS_BYTES"))
        prm.ws_bytes_per_warp = std::atoi(e);
    if (const char *e = std::getenv("SPAI_QCAP"))
        prm.first_qcap = std::atoi(e);
    if (const char *e = std::getenv("SPAI_TUNE"))
        prm.tune = std::atoi(e) != 0;
    prm.record = h->recording;
    prm.epsilon = opt->epsilon;
    // Every form follows the reference's sequential arithmetic bit for bit by default; the
    // group-parallel variant (parallel norms and mean, hashed candidate sets) is opt-in.
    prm.fast = (opt->flags & SPAI_FLAG_FAST_SPAI) != 0;
    prm.alpha = opt->alpha;
    prm.beta = static_cast<int>(std::min<int64_t>(opt->beta, INT_MAX));
    if (opt->alpha < 0 || opt->beta < 0)
        return fail(SPAI_ERR_ARGUMENT, "spai_build: alpha and beta must be nonnegative");
    EventTimer timer(h->stream);
    int status, first, overflow;
    long long fits, growths, launches, nnzp;
    if (h->precision == SPAI_PREC_F64) {
        SpaiBuilder<double>::construct(h->a64, prm, h->stream, h->s64, h->build);
        status = h->s64.status;
        first = h->s64.first_failed;
        fits = h->s64.fits;
        growths = h->s64.growths;
        overflow = h->s64.overflow_columns;
        launches = h->s64.launches;
        nnzp = h->s64.p.nnz;
    } else {
        SpaiBuilder<float>::construct(h->a32, prm, h->stream, h->s32, h->build);
        status = h->s32.status;
        first = h->s32.first_failed;
        fits = h->s32.fits;
        growths = h->s32.growths;
        overflow = h->s32.overflow_columns;
        launches = h->s32.launches;
        nnzp = h->s32.p.nnz;
    }
    h->spai_ms = timer.stop();
    h->spai_status = status;
    h->built = true;
    rep->spai_status = status;
    rep->first_failed_column = first;
    rep->spai_fits = fits;
    rep->spai_growths = growths;
    rep->spai_overflow_columns = overflow;
    rep->nnz_p = nnzp;
    rep->spai_ms = h->spai_ms;
    rep->kernel_launches = launches;
    rep->ir_status = status == SPAI_SUCCESS ? IR_INVALID_INPUT : IR_CONSTRUCTION_FAILURE;
    return SPAI_OK;
    API_END
}

int spai_solve_device(spai_handle *h, const double *d_b, double *d_x, const spai_options *opt,
                      spai_report *rep) {
    API_BEGIN
    if (!h || !d_b || !d_x || !opt)
        return fail(SPAI_ERR_ARGUMENT, "spai_solve_device: null argument");
    spai_report local;
    if (!rep)
        rep = &local;
    clear_report(rep);
    SPAI_CUDA(cudaSetDevice(h->device));
    return solve_device_impl(h, d_b, d_x, *opt, rep);
    API_END
}


int spai_solve(spai_handle *h, const double *b, double *x, const double *reference,
               const spai_options *opt, spai_report *rep) {
    API_BEGIN
    if (!h || !b || !x || !opt)
        return fail(SPAI_ERR_ARGUMENT, "spai_solve: null argument");
    spai_report local;
    if (!rep)
        rep = &local;
    clear_report(rep);
    SPAI_CUDA(cudaSetDevice(h->device));
    if (!finite_inputs(h->n, b, reference)) {
        rep->ir_status = IR_INVALID_INPUT; // src/ir.cpp:48-53
        rep->spai_status = h->spai_status;
        return SPAI_OK;
    }
    return solve_host_impl(h, b, x, reference, opt, rep);
    API_END
}


int spai_ir_solve(const spai_csr *a, const double *b, double *x, const double *reference,
                  const spai_options *opt, spai_report *rep, void *stream) {
    API_BEGIN
    if (!opt || !b || !x)
        return fail(SPAI_ERR_ARGUMENT, "spai_ir_solve: null argument");
    spai_report local;
    if (!rep)
        rep = &local;
    clear_report(rep);
    spai_handle *h = nullptr;
    int rc = spai_create(a, opt->precision, 0, stream, &h);
    if (rc != SPAI_OK)
        return rc;
    std::unique_ptr<spai_handle, int (*)(spai_handle *)> guard(h, spai_destroy);
    if (!options_valid(h, *opt)) {
        rep->ir_status = IR_INVALID_INPUT;
        return SPAI_OK;
    }
    if (!finite_inputs(a->n, b, reference)) {
        rep->ir_status = IR_INVALID_INPUT;
        return SPAI_OK;
    }
    spai_report brep;
    rc = spai_build(h, opt, &brep);
    if (rc != SPAI_OK)
        return rc;
    clear_report(rep);
    rc = solve_host_impl(h, b, x, reference, opt, rep);
    rep->spai_fits = brep.spai_fits;
    rep->spai_growths = brep.spai_growths;
    rep->spai_overflow_columns = brep.spai_overflow_columns;
    rep->first_failed_column = brep.first_failed_column;
    rep->kernel_launches += brep.kernel_launches;
    return rc;
    API_END
}

int spai_get_preconditioner(spai_handle *h, int64_t *nnz, int64_t *row_offsets,
                            int64_t *col_indices, double *values) {
    API_BEGIN
    if (!h || !nnz)
        return fail(SPAI_ERR_ARGUMENT, "spai_get_preconditioner: null argument");
    if (!h->built)
        return fail(SPAI_ERR_NOT_BUILT, "no preconditioner built");
    const bool f64 = h->precision == SPAI_PREC_F64;
    const int n = h->n;
    const int pn = f64 ? h->s64.p.nnz : h->s32.p.nnz;
    *nnz = pn;
    if (!row_offsets && !col_indices && !values)
        return SPAI_OK;
    std::vector<int> rp(n + 1), ci(pn);
    const int *drp = f64 ? h->s64.p.rp : h->s32.p.rp;
    const int *dci = f64 ? h->s64.p.ci : h->s32.p.ci;
    if (!drp) {
        std::fill(rp.begin(), rp.end(), 0);
    } else {
        SPAI_CUDA(cudaMemcpy(rp.data(), drp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
        if (pn)
            SPAI_CUDA(cudaMemcpy(ci.data(), dci, sizeof(int) * pn, cudaMemcpyDeviceToHost));
    }
    if (row_offsets)
        for (int i = 0; i <= n; ++i)
            row_offsets[i] = rp[i];
    if (col_indices)
        for (int i = 0; i < pn; ++i)
            col_indices[i] = ci[i];
    if (values && pn) {
        if (f64) {
            SPAI_CUDA(cudaMemcpy(values, h->s64.p.val, sizeof(double) * pn, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> v(pn);
            SPAI_CUDA(cudaMemcpy(v.data(), h->s32.p.val, sizeof(float) * pn, cudaMemcpyDeviceToHost));
            for (int i = 0; i < pn; ++i)
                values[i] = v[i];
        }
    }
    return SPAI_OK;
    API_END
}

int spai_get_columns(spai_handle *h, int32_t *status, int32_t *fits, int32_t *growths,
                     int32_t *score_clamps, double *residual, double *scaling) {
    API_BEGIN
    if (!h)
        return fail(SPAI_ERR_ARGUMENT, "spai_get_columns: null handle");
    if (!h->built)
        return fail(SPAI_ERR_NOT_BUILT, "no preconditioner built");
    const int n = h->n;
    const bool f64 = h->precision == SPAI_PREC_F64;
    if (h->p_supplied)
        return fail(SPAI_ERR_NOT_BUILT, "no SPAI columns (the preconditioner was supplied by the caller)");
    auto get_i = [&](int32_t *dst, const int *src) {
        if (dst && src)
            SPAI_CUDA(cudaMemcpy(dst, src, sizeof(int) * n, cudaMemcpyDeviceToHost));
    };
    if (f64) {
        get_i(status, h->s64.col_status);
        get_i(fits, h->s64.col_fits);
        get_i(growths, h->s64.col_growths);
        get_i(score_clamps, h->s64.col_clamps);
        if (residual && h->s64.col_residual)
            SPAI_CUDA(cudaMemcpy(residual, h->s64.col_residual, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (scaling && h->s64.d)
            SPAI_CUDA(cudaMemcpy(scaling, h->s64.d, sizeof(double) * n, cudaMemcpyDeviceToHost));
    } else {
        get_i(status, h->s32.col_status);
        get_i(fits, h->s32.col_fits);
        get_i(growths, h->s32.col_growths);
        get_i(score_clamps, h->s32.col_clamps);
        std::vector<float> v(n);
        if (residual && h->s32.col_residual) {
            SPAI_CUDA(cudaMemcpy(v.data(), h->s32.col_residual, sizeof(float) * n, cudaMemcpyDeviceToHost));
            for (int i = 0; i < n; ++i)
                residual[i] = v[i];
        }
        if (scaling && h->s32.d) {
            SPAI_CUDA(cudaMemcpy(v.data(), h->s32.d, sizeof(float) * n, cudaMemcpyDeviceToHost));
            for (int i = 0; i < n; ++i)
                scaling[i] = v[i];
        }
    }
    return SPAI_OK;
    API_END
}

int spai_get_column(spai_handle *h, int64_t k, int64_t *q, int64_t *pattern, double *coefficients) {
    API_BEGIN
    if (!h || !q || k < 0 || k >= h->n)
        return fail(SPAI_ERR_ARGUMENT, "spai_get_column: bad arguments");
    if (!h->built)
        return fail(SPAI_ERR_NOT_BUILT, "no preconditioner built");
    const bool f64 = h->precision == SPAI_PREC_F64;
    int qs = 0;
    long long off = -1;
    const int *cq = f64 ? h->s64.col_q : h->s32.col_q;
    const long long *co = f64 ? h->s64.packed_off : h->s32.packed_off;
    if (h->p_supplied)
        return fail(SPAI_ERR_NOT_BUILT, "no SPAI columns (the preconditioner was supplied by the caller)");
    if (!cq) {
        *q = 0;
        return SPAI_OK;
    }
    SPAI_CUDA(cudaMemcpy(&qs, cq + k, sizeof(int), cudaMemcpyDeviceToHost));
    SPAI_CUDA(cudaMemcpy(&off, co + k, sizeof(long long), cudaMemcpyDeviceToHost));
    *q = qs;
    if (off < 0 || qs == 0)
        return SPAI_OK;
    std::vector<int> idx(qs);
    SPAI_CUDA(cudaMemcpy(idx.data(), (f64 ? h->s64.packed_idx : h->s32.packed_idx) + off, sizeof(int) * qs, cudaMemcpyDeviceToHost));
    if (pattern)
        for (int i = 0; i < qs; ++i)
            pattern[i] = idx[i];
    if (coefficients) {
        if (f64) {
            SPAI_CUDA(cudaMemcpy(coefficients, h->s64.packed_val + off, sizeof(double) * qs, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> v(qs);
            SPAI_CUDA(cudaMemcpy(v.data(), h->s32.packed_val + off, sizeof(float) * qs, cudaMemcpyDeviceToHost));
            for (int i = 0; i < qs; ++i)
                coefficients[i] = v[i];
        }
    }
    return SPAI_OK;
    API_END
}

int spai_spmv(spai_handle *h, int32_t which, const double *x, double *y) {
    API_BEGIN
    if (!h || !x || !y || which < 0 || which > 1)
        return fail(SPAI_ERR_ARGUMENT, "spai_spmv: bad arguments");
    if (which == 1 && !h->built)
        return fail(SPAI_ERR_NOT_BUILT, "no preconditioner built");
    SPAI_CUDA(cudaSetDevice(h->device));
    const int n = h->n;
    h->scratch.reset();
    double *dx = h->scratch.alloc<double>(n);
    double *dy = h->scratch.alloc<double>(n);
    SPAI_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    const VecRef<double> xr{dx, 0, nullptr, 0}, yr{dy, 0, nullptr, 0};
    if (h->precision == SPAI_PREC_F64) {
        launch_spmv<double, double, double>(which ? h->s64.p : h->a64, xr, yr, nullptr, h->sms, h->stream);
    } else {
        float *fx = h->scratch.alloc<float>(n);
        float *fy = h->scratch.alloc<float>(n);
        convert_kernel<float, double><<<grid_for(n, 256, h->sms * 8), 256, 0, h->stream>>>(n, dx, fx);
        const VecRef<float> fxr{fx, 0, nullptr, 0}, fyr{fy, 0, nullptr, 0};
        launch_spmv<float, float, float>(which ? h->s32.p : h->a32, fxr, fyr, nullptr, h->sms, h->stream);
        convert_kernel<double, float><<<grid_for(n, 256, h->sms * 8), 256, 0, h->stream>>>(n, fy, dy);
        SPAI_LAUNCH("convert_kernel");
    }
    SPAI_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
    return SPAI_OK;
    API_END
}

int spai_score(int32_t precision, double rsq, double dot, double den, double *out) {
    API_BEGIN
    if (!out)
        return fail(SPAI_ERR_ARGUMENT, "spai_score: null output");
    if (precision == SPAI_PREC_F64)
        score_kat<double>(rsq, dot, den, out);
    else
        score_kat<float>(static_cast<float>(rsq), static_cast<float>(dot), static_cast<float>(den), out);
    return SPAI_OK;
    API_END
}

int spai_gmres(spai_handle *h, const double *rhs, double *x, double tau, int64_t cap,
               int32_t *out_status, int64_t *out_iterations, double *out_relative) {
    API_BEGIN
    if (!h || !rhs || !x)
        return fail(SPAI_ERR_ARGUMENT, "spai_gmres: null argument");
    if (!h->built || h->spai_status != SPAI_SUCCESS)
        return fail(SPAI_ERR_NOT_BUILT, "spai_gmres needs a successfully built preconditioner");
    const int n = h->n;
    if (cap < 0 || cap > n || !(tau > 0) || !std::isfinite(tau)) {
        if (out_status)
            *out_status = GMRES_INVALID_INPUT;
        return SPAI_OK;
    }
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(rhs[i])) {
            if (out_status)
                *out_status = GMRES_INVALID_INPUT;
            return SPAI_OK;
        }
    SPAI_CUDA(cudaSetDevice(h->device));
    const int c = cap == 0 ? n : static_cast<int>(cap);
    ensure_engine(h, c);
    SolveSettings s;
    s.cap = c;
    s.tau = tau;
    s.accept_every = h->precision == SPAI_PREC_F32;
    if (h->recording) {
        if (static_cast<double>(n) * (c + 1) > static_cast<double>(1 << 28))
            return fail(SPAI_ERR_ARGUMENT, "record mode keeps every step's candidate in host memory: "
                                           "n * (cap + 1) must stay below 2^28");
        h->krec.clear();
        s.record = &h->krec;
    }
    h->scratch.reset();
    double *dr = h->scratch.alloc<double>(n);
    double *dx = h->scratch.alloc<double>(n);
    SPAI_CUDA(cudaMemcpyAsync(dr, rhs, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    Ctl ctl{};
    auto run = [&](auto &e) {
        using T = std::remove_pointer_t<decltype(e.rhs)>;
        convert_kernel<T, double><<<grid_for(n, 256, h->sms * 8), 256, 0, h->stream>>>(n, dr, e.rhs);
        SPAI_LAUNCH("convert_kernel");
        e.gmres_only(h->stream, s, h->pinned);
        read_ctl(h, e, ctl);
        if (ctl.formed > 0) {
            convert_kernel<double, T><<<grid_for(n, 256, h->sms * 8), 256, 0, h->stream>>>(n, e.cand, dx);
            SPAI_LAUNCH("convert_kernel");
        } else {
            SPAI_CUDA(cudaMemsetAsync(dx, 0, sizeof(double) * n, h->stream));
        }
    };
    if (h->precision == SPAI_PREC_F64)
        run(h->e64);
    else if (h->precision == SPAI_PREC_MIXED)
        run(h->emix);
    else
        run(h->e32);
    SPAI_CUDA(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
    if (out_status)
        *out_status = ctl.status;
    if (out_iterations)
        *out_iterations = ctl.iterations;
    if (out_relative)
        *out_relative = ctl.rel;
    return SPAI_OK;
    API_END
}

int spai_history(spai_handle *h, spai_outer_record *outer, int64_t max_outer, int64_t *n_outer,
                 spai_inner_record *inner, int64_t max_inner, int64_t *n_inner,
                 spai_iteration_record *iterations, int64_t max_iterations, int64_t *n_iterations) {
    API_BEGIN
    if (!h || max_outer < 0 || max_inner < 0 || max_iterations < 0)
        return fail(SPAI_ERR_ARGUMENT, "spai_history: bad arguments");
    if (!h->hist_outer)
        return fail(SPAI_ERR_NOT_BUILT, "spai_history: no solve with SPAI_FLAG_HISTORY on this handle");
    SPAI_CUDA(cudaSetDevice(h->device));
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
    auto copy = [&](auto *dst, const auto *src, int64_t maxc, int recorded, int cap) {
        const int64_t cnt = std::min<int64_t>(maxc, std::min(recorded, cap));
        if (dst && cnt > 0)
            SPAI_CUDA(cudaMemcpy(dst, src, sizeof(*dst) * cnt, cudaMemcpyDeviceToHost));
    };
    copy(outer, h->hist_outer, max_outer, h->hist_n_outer, h->hist_cap_outer);
    copy(inner, h->hist_inner, max_inner, h->hist_n_inner, h->hist_cap_inner);
    copy(iterations, h->hist_iter, max_iterations, h->hist_n_iter, h->hist_cap_iter);
    if (n_outer)
        *n_outer = h->hist_n_outer;
    if (n_inner)
        *n_inner = h->hist_n_inner;
    if (n_iterations)
        *n_iterations = h->hist_n_iter;
    return SPAI_OK;
    API_END
}

int spai_set_preconditioner(spai_handle *h, const spai_csr *p) {
    API_BEGIN
    if (!h || !p)
        return fail(SPAI_ERR_ARGUMENT, "spai_set_preconditioner: null argument");
    const std::string why = canonical_header_error(p);
    if (!why.empty())
        return fail(SPAI_ERR_ARGUMENT, "spai_set_preconditioner: " + why);
    if (p->n != h->n)
        return fail(SPAI_ERR_ARGUMENT, "spai_set_preconditioner: P and A differ in dimension");
    SPAI_CUDA(cudaSetDevice(h->device));
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
    h->built = false;
    h->engine_cap = -1;
    h->adj_ready = false;
    h->adj_cap = -1;
    h->build.reset();
    h->scratch.reset();
    int *bad = h->scratch.alloc<int>(2);
    DeviceCsr<double> p64 = upload_csr(h, h->build, p, bad);
    int h_bad[2] = {0, 0};
    SPAI_CUDA(cudaMemcpyAsync(h_bad, bad, sizeof(h_bad), cudaMemcpyDeviceToHost, h->stream));
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
    p64.max_row = h_bad[1];
    if (h_bad[0]) {
        const std::string full = canonical_error(p);
        return fail(SPAI_ERR_ARGUMENT, "spai_set_preconditioner: " + (full.empty() ? std::string("CSR is not canonical") : full));
    }
    if (h->precision == SPAI_PREC_F64) {
        h->s64 = SpaiOutput<double>{};
        h->s64.n = h->n;
        h->s64.status = SPAI_SUCCESS;
        h->s64.p = p64;
    } else {
        h->s32 = SpaiOutput<float>{};
        h->s32.n = h->n;
        h->s32.status = SPAI_SUCCESS;
        h->s32.p.n = p64.n;
        h->s32.p.nnz = p64.nnz;
        h->s32.p.max_row = p64.max_row;
        h->s32.p.rp = p64.rp;
        h->s32.p.ci = p64.ci;
        h->s32.p.val = h->build.alloc<float>(p64.nnz > 0 ? p64.nnz : 1);
        if (p64.nnz > 0) {
            convert_kernel<float, double><<<grid_for(p64.nnz, 256, h->sms * 8), 256, 0, h->stream>>>(p64.nnz, p64.val,
                                                                                               h->s32.p.val);
            SPAI_LAUNCH("convert_kernel");
        }
    }
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
    h->spai_status = SPAI_SUCCESS;
    h->spai_ms = 0;
    h->built = true;
    h->p_supplied = true;
    return SPAI_OK;
    API_END
}

int spai_record(spai_handle *h, int32_t enable) {
    API_BEGIN
    if (!h)
        return fail(SPAI_ERR_ARGUMENT, "spai_record: null handle");
    if (enable && h->precision != SPAI_PREC_F64)
        return fail(SPAI_ERR_ARGUMENT, "spai_record: record mode is binary64 only");
    h->recording = enable != 0;
    h->krec.clear();
    return SPAI_OK;
    API_END
}

int spai_fit_log(spai_handle *h, int32_t *ints, int64_t max_ints, int64_t *n_ints, double *vals,
                 int64_t max_vals, int64_t *n_vals) {
    API_BEGIN
    if (!h)
        return fail(SPAI_ERR_ARGUMENT, "spai_fit_log: null handle");
    if (!h->built || !h->s64.log_top)
        return fail(SPAI_ERR_NOT_BUILT, "no fit log: the last build did not run in record mode");
    unsigned long long top[2] = {0, 0};
    SPAI_CUDA(cudaMemcpy(top, h->s64.log_top, sizeof(top), cudaMemcpyDeviceToHost));
    if (static_cast<long long>(top[0]) > h->s64.log_int_cap || static_cast<long long>(top[1]) > h->s64.log_val_cap)
        return fail(SPAI_ERR_WORKSPACE, "the fit log overflowed its capacity");
    if (n_ints)
        *n_ints = static_cast<int64_t>(top[0]);
    if (n_vals)
        *n_vals = static_cast<int64_t>(top[1]);
    if (ints && max_ints > 0)
        SPAI_CUDA(cudaMemcpy(ints, h->s64.log_ints, sizeof(int32_t) * std::min<int64_t>(max_ints, top[0]),
                             cudaMemcpyDeviceToHost));
    if (vals && max_vals > 0)
        SPAI_CUDA(cudaMemcpy(vals, h->s64.log_vals, sizeof(double) * std::min<int64_t>(max_vals, top[1]),
                             cudaMemcpyDeviceToHost));
    return SPAI_OK;
    API_END
}

int spai_record_counts(spai_handle *h, int64_t *n_states, int64_t *n_inner) {
    if (!h)
        return fail(SPAI_ERR_ARGUMENT, "spai_record_counts: null handle");
    if (n_states)
        *n_states = static_cast<int64_t>(h->krec.states.size());
    if (n_inner)
        *n_inner = static_cast<int64_t>(h->krec.inner.size());
    return SPAI_OK;
}

int spai_record_state(spai_handle *h, int64_t s, double *x, double *residual) {
    if (!h || s < 0 || s >= static_cast<int64_t>(h->krec.states.size()))
        return fail(SPAI_ERR_ARGUMENT, "spai_record_state: no such state");
    const KrylovState &st = h->krec.states[static_cast<size_t>(s)];
    if (x)
        std::copy(st.x.begin(), st.x.end(), x);
    if (residual)
        std::copy(st.residual.begin(), st.residual.end(), residual);
    return SPAI_OK;
}

int spai_record_inner(spai_handle *h, int64_t i, double *summary, double *rhs, double *solution, double *basis,
                      double *hessenberg, double *steps, double *candidates) {
    if (!h || i < 0 || i >= static_cast<int64_t>(h->krec.inner.size()))
        return fail(SPAI_ERR_ARGUMENT, "spai_record_inner: no such inner solve");
    const KrylovInner &in = h->krec.inner[static_cast<size_t>(i)];
    const int m = static_cast<int>(in.steps.size());
    if (summary) {
        const double sm[12] = {static_cast<double>(in.status), static_cast<double>(in.converged),
                               static_cast<double>(m),         static_cast<double>(in.applied),
                               in.initial_original,            1.0,
                               in.final_original,              in.final_preconditioned,
                               static_cast<double>(in.nbasis), static_cast<double>(in.hcap + 1),
                               static_cast<double>(in.hcap),   static_cast<double>(in.iterations)};
        std::copy(sm, sm + 12, summary);
    }
    if (rhs)
        std::copy(in.rhs.begin(), in.rhs.end(), rhs);
    if (solution)
        std::copy(in.solution.begin(), in.solution.end(), solution);
    if (basis)
        std::copy(in.basis.begin(), in.basis.end(), basis);
    if (hessenberg)
        std::copy(in.hessenberg.begin(), in.hessenberg.end(), hessenberg);
    for (int k = 0; k < m; ++k) {
        const spai_iteration_record &r = in.records[static_cast<size_t>(k)];
        const double sub = in.hessenberg[static_cast<size_t>(k + 1) * in.hcap + k];
        if (steps) {
            const double row[8] = {static_cast<double>(k + 1), r.estimated_relative, r.recomputed_relative,
                                   in.steps[static_cast<size_t>(k)].original, sub, sub == 0 ? 1.0 : 0.0,
                                   static_cast<double>(r.triggered), static_cast<double>(r.accepted)};
            std::copy(row, row + 8, steps + static_cast<size_t>(k) * 8);
        }
        if (candidates)
            std::copy(in.steps[static_cast<size_t>(k)].candidate.begin(), in.steps[static_cast<size_t>(k)].candidate.end(),
                      candidates + static_cast<size_t>(k) * h->n);
    }
    return SPAI_OK;
}

int spai_profile(spai_handle *h, int32_t enable) {
    API_BEGIN
    if (!h)
        return fail(SPAI_ERR_ARGUMENT, "spai_profile: null handle");
    SPAI_CUDA(cudaSetDevice(h->device));
    SPAI_CUDA(cudaStreamSynchronize(h->stream));
    h->prof.reset();
    h->prof.on = enable != 0;
    return SPAI_OK;
    API_END
}

int spai_profile_read(spai_handle *h, int32_t cls, double *ms, int64_t *launches, double *bytes) {
    API_BEGIN
    if (!h || cls < 0 || cls >= kClsCount)
        return fail(SPAI_ERR_ARGUMENT, "spai_profile_read: bad arguments");
    if (ms)
        *ms = h->prof.ms[cls];
    if (launches)
        *launches = h->prof.launches[cls];
    if (bytes)
        *bytes = h->prof.bytes[cls];
    return SPAI_OK;
    API_END
}

int spai_tuning(spai_handle *h, int32_t *out, double *ms) {
    API_BEGIN
    if (!h || !out)
        return fail(SPAI_ERR_ARGUMENT, "spai_tuning: null argument");
    const bool f64 = h->precision == SPAI_PREC_F64;
    const int G = f64 ? h->s64.group_lanes : h->s32.group_lanes;
    const int ws = f64 ? h->s64.ws_bytes : h->s32.ws_bytes;
    const bool tuned = f64 ? h->s64.tuned : h->s32.tuned;
    int oa = -1, op = -1;
    auto orders = [&](const auto &e) {
        if (e.n > 0) {
            oa = e.sa.layout;
            op = e.sp.layout;
        }
    };
    if (h->engine_cap >= 0) {
        if (h->precision == SPAI_PREC_F64)
            orders(h->e64);
        else if (h->precision == SPAI_PREC_MIXED)
            orders(h->emix);
        else
            orders(h->e32);
    }
    out[0] = G;
    out[1] = ws;
    out[2] = tuned ? 1 : 0;
    out[3] = oa;
    out[4] = op;
    if (ms) {
        ms[0] = tuned ? (f64 ? h->s64.tune_sample_ms : h->s32.tune_sample_ms) : NAN;
        ms[1] = tuned ? (f64 ? h->s64.tune_default_ms : h->s32.tune_default_ms) : NAN;
    }
    return SPAI_OK;
    API_END
}

int spai_adjoint_device(spai_handle *h, int64_t nrhs, const double *d_x, const double *d_dLdx,
                        double *d_dLdb, double *d_dLdA_values, const spai_options *opt, spai_report *rep) {
    API_BEGIN
    if (!h || !opt || nrhs < 1 || nrhs > INT_MAX || !d_x || !d_dLdx || !d_dLdb || !d_dLdA_values)
        return fail(SPAI_ERR_ARGUMENT, "spai_adjoint_device: bad arguments");
    spai_report local;
    if (!rep)
        rep = &local;
    clear_report(rep);
    SPAI_CUDA(cudaSetDevice(h->device));
    return adjoint_device_impl(h, static_cast<int>(nrhs), d_x, d_dLdx, d_dLdb, d_dLdA_values, *opt, rep);
    API_END
}

int spai_adjoint(spai_handle *h, int64_t nrhs, const double *x, const double *dLdx, double *dLdb,
                 double *dLdA_values, const spai_options *opt, spai_report *rep) {
    API_BEGIN
    if (!h || !opt || nrhs < 1 || nrhs > INT_MAX || !x || !dLdx || !dLdb || !dLdA_values)
        return fail(SPAI_ERR_ARGUMENT, "spai_adjoint: bad arguments");
    spai_report local;
    if (!rep)
        rep = &local;
    clear_report(rep);
    SPAI_CUDA(cudaSetDevice(h->device));
    const size_t total = static_cast<size_t>(nrhs) * h->n;
    for (size_t i = 0; i < total; ++i)
        if (!std::isfinite(x[i]) || !std::isfinite(dLdx[i])) {
            rep->ir_status = IR_INVALID_INPUT;
            rep->spai_status = h->spai_status;
            return SPAI_OK;
        }
    h->scratch.reset();
    double *dx = h->scratch.alloc<double>(total);
    double *dg = h->scratch.alloc<double>(total);
    double *dl = h->scratch.alloc<double>(total);
    double *da = h->scratch.alloc<double>(h->nnz);
    SPAI_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * total, cudaMemcpyHostToDevice, h->stream));
    SPAI_CUDA(cudaMemcpyAsync(dg, dLdx, sizeof(double) * total, cudaMemcpyHostToDevice, h->stream));
    const int rc = adjoint_device_impl(h, static_cast<int>(nrhs), dx, dg, dl, da, *opt, rep);
    if (rc != SPAI_OK)
        return rc;
    if (rep->ir_status != IR_CONSTRUCTION_FAILURE && rep->ir_status != IR_INVALID_INPUT) {
        SPAI_CUDA(cudaMemcpyAsync(dLdb, dl, sizeof(double) * total, cudaMemcpyDeviceToHost, h->stream));
        SPAI_CUDA(cudaMemcpyAsync(dLdA_values, da, sizeof(double) * h->nnz, cudaMemcpyDeviceToHost, h->stream));
        SPAI_CUDA(cudaStreamSynchronize(h->stream));
    }
    return SPAI_OK;
    API_END
}

} // extern "C"
