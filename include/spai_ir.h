/* GB300-native SPAI-GMRES-IR: C ABI of libspai_ir.so.
 *
 * Drop-in boundary for the reference's GPU solver path (anirudhtheexe/spai-gmres-ir). Plain
 * pointers and sizes only; no exceptions cross the boundary; every entry point returns an int
 * (SPAI_OK or a negative SPAI_ERR_*). Numerical outcomes are reported as the reference's status
 * enums inside spai_report, never as errors.
 *
 *   reference entry point (file:line)                          replaced by
 *   cuda_gpu_spai_gmres_ir      include/bspai/cuda_ir.hpp:26-28       spai_ir_solve (F64)
 *   fp32_cuda_spai_gmres_ir     include/bspai/fp32_cuda_spai.hpp:57-58 spai_ir_solve (F32)
 *   cuda_construct_spai         include/bspai/cuda_spai.hpp:47        spai_create + spai_build
 *   CudaGmresContext            include/bspai/cuda_gmres.hpp:21-36    spai_handle + spai_gmres
 *   cuda_refine_with_preconditioner include/bspai/cuda_ir.hpp:18-22   spai_build + spai_solve
 *   CudaCsrSpmv::multiply       include/bspai/cuda_spmv.hpp:8-20      spai_spmv
 *   cuda_evaluate_spai_score    include/bspai/cuda_spai.hpp:48-49     spai_score
 *   spai_status_name / gmres_status_name / ir_status_name (spai.hpp:22, gmres.hpp:21, ir.hpp:18)
 *
 * Ownership: the caller owns every host buffer; a handle owns all device memory it allocates.
 * Threading: one handle per host thread; calls on a handle are stream ordered and synchronous
 * with respect to host buffers (as the reference's "synchronous, not thread-safe" contexts).
 */
#ifndef SPAI_IR_H
#define SPAI_IR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* SpaiStatus, include/bspai/spai.hpp:10-21 (same order). */
enum {
    SPAI_SUCCESS = 0,
    SPAI_NOT_ATTEMPTED = 1,
    SPAI_INVALID_INPUT = 2,
    SPAI_RANK_DEFICIENT = 3,
    SPAI_NUMERICAL_FAILURE = 4,
    SPAI_EMPTY_CANDIDATES = 5,
    SPAI_ZERO_DENOMINATOR = 6,
    SPAI_INVALID_SCORE = 7,
    SPAI_NO_GROWTH = 8,
    SPAI_ITERATION_LIMIT = 9
};
/* GmresStatus, include/bspai/gmres.hpp:10-20 (same order). */
enum {
    GMRES_SUCCESS = 0,
    GMRES_ZERO_RHS = 1,
    GMRES_EXACT_INITIAL_SOLUTION = 2,
    GMRES_INVALID_INPUT = 3,
    GMRES_ZERO_PRECONDITIONED_RHS = 4,
    GMRES_BREAKDOWN = 5,
    GMRES_ITERATION_LIMIT = 6,
    GMRES_NONCONVERGENCE = 7,
    GMRES_NUMERICAL_FAILURE = 8
};
/* IrStatus, include/bspai/ir.hpp:9-17 (same order). */
enum {
    IR_SUCCESS = 0,
    IR_INVALID_INPUT = 1,
    IR_CONSTRUCTION_FAILURE = 2,
    IR_INNER_FAILURE = 3,
    IR_STAGNATION = 4,
    IR_ITERATION_LIMIT = 5,
    IR_NUMERICAL_FAILURE = 6
};

/* API return codes (the reference throws std::runtime_error / std::invalid_argument). */
enum {
    SPAI_OK = 0,
    SPAI_ERR_ARGUMENT = -1,  /* invalid_argument: bad sizes, non-canonical CSR, bad options */
    SPAI_ERR_CUDA = -2,      /* runtime_error from the CUDA runtime (message: spai_last_error) */
    SPAI_ERR_WORKSPACE = -3, /* a SPAI column exceeded the largest fit workspace */
    SPAI_ERR_TIMEOUT = -4,   /* a bounded device wait gave up */
    SPAI_ERR_NOT_BUILT = -5, /* spai_solve before a successful spai_build */
    SPAI_ERR_UNSUPPORTED = -6,
    SPAI_ERR_FORMAT = -7     /* malformed input file (runtime_error of the reference's reader) */
};

/* Precision forms. F64 is the drop-in for gpu_fp64_ir; F32 for gpu_fp32_ir; MIXED builds the
 * SPAI and runs GMRES in binary32 with binary64 refinement residual, update and norms. */
enum { SPAI_PREC_F64 = 0, SPAI_PREC_F32 = 1, SPAI_PREC_MIXED = 2 };

/* Option flags. */
enum {
    SPAI_FLAG_NO_GRAPH = 1,  /* run the refinement loop with host launches instead of one graph */
    SPAI_FLAG_FAST_SPAI = 2, /* build the SPAI with group-parallel norms, a parallel mean and hashed
                                candidate sets instead of the reference's sequential arithmetic
                                (patterns may differ on near-tied scores; not bit-reproducible) */
    SPAI_FLAG_HISTORY = 4,   /* record the refinement history of the solve (spai_history) */
    SPAI_FLAG_RESTART_AT_CAP = 8, /* an inner GMRES that reaches its cap with a verified candidate
                                    that reduces the preconditioned residual (relative < 1) supplies
                                    the correction anyway: the refinement restarts GMRES from the new
                                    binary64 residual, i.e. restarted GMRES(innercap) inside IR
                                    (the reference stops with inner_failure; off by default) */
    SPAI_FLAG_RIGHT_PRECONDITIONING = 16 /* inner GMRES on A P u = r with correction d = P u: the
                                    form flexible GMRES takes with this solver's one fixed SPAI;
                                    its estimate and acceptance test are relative to ||r||, the
                                    unpreconditioned residual (the reference's inner solve is
                                    left-preconditioned; off by default) */
};

/* Refinement history of one solve (IrResult::history / inner_history / update_applied and
 * GmresResult::history, ir.hpp:26-56, gmres.hpp:28-50), recorded on the device when the solve
 * ran with SPAI_FLAG_HISTORY. */
typedef struct {
    int64_t step;               /* 0 = x0 = P b, then one record per applied correction */
    double residual_inf, residual_2;
    double normwise_backward_error, componentwise_backward_error;
} spai_outer_record;
typedef struct {
    int32_t status;             /* GMRES_* */
    int32_t update_applied;     /* the correction was added and its iterate evaluated */
    int64_t iterations;
    double final_relative;      /* last recomputed preconditioned relative residual (NaN: none) */
} spai_inner_record;
typedef struct {
    int64_t inner;              /* 1-based inner solve */
    int64_t iteration;          /* 1-based Arnoldi step */
    double estimated_relative;  /* |g_{k+1}| / ||P rhs|| after the Givens update */
    double recomputed_relative; /* verified candidate's relative residual; NaN when the step was
                                   not verified (candidates are formed only when the acceptance
                                   rule can accept them) */
    int32_t accepted;
    int32_t triggered;          /* the acceptance rule's check was due at this step (estimate <= tau,
                                   breakdown or the cap; GmresIteration::verification_triggered) */
} spai_iteration_record;

/* Canonical CSR on the host (row_offsets[n+1], sorted col_indices[nnz], no stored zeros), the
 * layout of CsrMatrix (include/bspai/cpu.hpp:17-43) with 64-bit indices. */
typedef struct {
    int64_t n;
    int64_t nnz;
    const int64_t *row_offsets;
    const int64_t *col_indices;
    const double *values;
} spai_csr;

/* SpaiOptions + GmresOptions + IrOptions (spai.hpp:24-28, gmres.hpp:23-26, ir.hpp:20-24). */
typedef struct {
    double epsilon;       /* SPAI column residual target (reference default 0.3) */
    int64_t alpha;        /* growth budget per column (default 5; the CLI uses ceil(n/8)) */
    int64_t beta;         /* maximum candidates added per growth (default 8) */
    double tau;           /* inner GMRES tolerance; 0 = 1e-8 (F64) or 1e-4 (F32, MIXED) */
    int64_t innercap;     /* GMRES iteration cap; 0 = n */
    int64_t outercap;     /* refinement correction cap, <= 20 */
    double be_tolerance;  /* outer stop on normwise backward error; 0 = 10u (2^-53 or 2^-24) */
    int32_t precision;    /* SPAI_PREC_* */
    int32_t flags;        /* SPAI_FLAG_* */
} spai_options;

/* Result summary (IrResult/IrDiagnostics/SpaiResult fields, ir.hpp:26-56). */
typedef struct {
    int32_t ir_status;         /* IR_* */
    int32_t spai_status;       /* SPAI_* (overall construction status) */
    int32_t gmres_status;      /* GMRES_* of the last inner solve, -1 if none */
    int32_t converged;
    int64_t outer_steps;
    int64_t inner_attempts;
    int64_t inner_iterations;  /* summed over inner solves */
    int64_t nnz_p;
    int64_t first_failed_column; /* -1 when every column succeeded */
    double backward_error;     /* normwise ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) */
    double componentwise_backward_error;
    double residual_inf;
    double forward_error;      /* ||x - reference||_inf / ||reference||_inf, NaN without one */
    double spai_ms;            /* device time of the SPAI construction */
    double solve_ms;           /* device time of the refinement loop */
    int64_t spai_fits;
    int64_t spai_growths;
    int64_t spai_overflow_columns; /* columns refit in the large-workspace pass */
    int64_t kernel_launches;   /* kernels launched by the last build/solve call */
} spai_report;

typedef struct spai_handle_s spai_handle;

/* Fill *opt with the reference defaults for a precision (alpha 5, beta 8, epsilon 0.3,
 * outercap 20, innercap 0, tau and be_tolerance 0 = precision defaults). */
int spai_default_options(spai_options *opt, int32_t precision);

const char *spai_status_name(int32_t status);  /* spai.cpp:247-270 names */
const char *gmres_status_name(int32_t status); /* gmres.cpp:64-85 names */
const char *ir_status_name(int32_t status);    /* ir.cpp:59-76 names */
const char *spai_last_error(void);             /* message of the last SPAI_ERR_* on this thread */

/* Upload A (host CSR, canonical) to `device`, on `stream` (cudaStream_t, may be NULL). */
int spai_create(const spai_csr *a, int32_t precision, int device, void *stream, spai_handle **out);
int spai_destroy(spai_handle *h);

/* Adaptive SPAI construction on the device (cuda_construct_spai). rep may be NULL. */
int spai_build(spai_handle *h, const spai_options *opt, spai_report *rep);

/* Refinement solve with the built preconditioner; host b, host x (cuda_refine_with_preconditioner
 * semantics; x0 = P b). reference may be NULL. */
int spai_solve(spai_handle *h, const double *b, double *x, const double *reference,
               const spai_options *opt, spai_report *rep);
/* Same with device pointers (b, x resident in HBM; no host copies). */
int spai_solve_device(spai_handle *h, const double *d_b, double *d_x, const spai_options *opt,
                      spai_report *rep);

/* One call: create, build, solve, destroy (cuda_gpu_spai_gmres_ir / fp32_cuda_spai_gmres_ir). */
int spai_ir_solve(const spai_csr *a, const double *b, double *x, const double *reference,
                  const spai_options *opt, spai_report *rep, void *stream);

/* Built preconditioner P (CSR). Pass NULL arrays to query nnz only. */
int spai_get_preconditioner(spai_handle *h, int64_t *nnz, int64_t *row_offsets,
                            int64_t *col_indices, double *values);
/* Per-column construction metadata (SpaiColumn, spai.hpp:44-55); arrays of length n, any NULL. */
int spai_get_columns(spai_handle *h, int32_t *status, int32_t *fits, int32_t *growths,
                     int32_t *score_clamps, double *residual, double *scaling);
/* Solved pattern/coefficients of column k (N(:,k)); returns the pattern size via *q. */
int spai_get_column(spai_handle *h, int64_t k, int64_t *q, int64_t *pattern, double *coefficients);

/* y = M x on the device in the handle's inner precision; which: 0 = A, 1 = P (CudaCsrSpmv). */
int spai_spmv(spai_handle *h, int32_t which, const double *x, double *y);

/* One left-preconditioned GMRES solve P A d = P rhs with x0 = 0 (CudaGmresContext::solve).
 * out_status = GMRES_*, out_iterations, out_relative = recomputed preconditioned residual. */
int spai_gmres(spai_handle *h, const double *rhs, double *x, double tau, int64_t cap,
               int32_t *out_status, int64_t *out_iterations, double *out_relative);

/* Caller-supplied preconditioner (canonical CSR, n x n) in place of a SPAI build: the handle then
 * solves with P as refine_with_preconditioner and left_preconditioned_gmres do with a fixed P
 * (include/bspai/ir.hpp:63-65, include/bspai/gmres.hpp:55-57). P is kept in the handle's working
 * precision; the SPAI column queries (spai_get_columns, spai_get_column) then return
 * SPAI_ERR_NOT_BUILT. */
int spai_set_preconditioner(spai_handle *h, const spai_csr *p);

/* Record mode of a binary64 handle (enable != 0; SPAI_ERR_ARGUMENT for other precisions): the
 * next spai_build logs every fit of every column (spai_fit_log), and every later spai_solve and
 * spai_gmres runs its refinement loop from the host one Arnoldi step at a time in the three-pass
 * Gram-Schmidt form, forms and checks every step's candidate (only a triggered check may accept
 * it, gmres.cpp:235-240, so results equal the unrecorded solve's up to the three-pass
 * orthogonalisation) and keeps what the reference's GmresResult and IrResult histories hold
 * (include/bspai/gmres.hpp:28-50, ir.hpp:36-56): every step's candidate, the basis, the
 * unrotated Hessenberg, every iterate and residual. Diagnostics for small systems: a recorded solve
 * needs n * (innercap + 1) * (outercap + 1) below 2^28 (SPAI_ERR_ARGUMENT otherwise); the records
 * live in host memory of the handle until the next recorded solve. No reference counterpart
 * beyond those result structures (the reference's release snapshot prints them,
 * tests/release_cpu_snapshot.cpp:281-398). */
int spai_record(spai_handle *h, int32_t enable);
/* Fit log of the last build in record mode: an int stream and a binary64 stream of records, each
 * with an 8-int header (kind, column, workspace tier, fit ordinal, a, b, c, offset of its values):
 * kind 1 (fit): a = |J|, b = |I|; ints J then I; values residual, pivot ratio, coefficients;
 * kind 2 (candidate scores): a = candidates; ints candidates; values mean score, then one score
 * per candidate; kind 3 (selection): a = selected; ints the selection in selection order.
 * A column refitted from scratch in a larger workspace tier logs again under the higher tier;
 * only its highest tier's records are its history. n_ints / n_vals give the stream lengths;
 * SPAI_ERR_WORKSPACE when the log overflowed. */
int spai_fit_log(spai_handle *h, int32_t *ints, int64_t max_ints, int64_t *n_ints, double *vals,
                 int64_t max_vals, int64_t *n_vals);
/* Counts of the last recorded solve: iterates kept (x0 = P b and one per applied correction) and
 * inner GMRES solves (one for spai_gmres). */
int spai_record_counts(spai_handle *h, int64_t *n_states, int64_t *n_inner);
/* Iterate s of the last recorded solve and its residual b - A x (n each; either may be NULL). */
int spai_record_state(spai_handle *h, int64_t s, double *x, double *residual);
/* Inner solve i of the last recorded solve; any output may be NULL.
 * summary[12]: gmres status, converged, steps m, correction applied, ||rhs||, initial relative
 *   residual (1: zero initial guess), final original residual, final preconditioned relative
 *   residual, basis vectors kept nb, Hessenberg rows (cap + 1), columns (cap), iterations;
 * rhs[n], solution[n] (the last candidate, zero without steps), basis[nb * n] (normalised
 * v_j = s_j W_j, row j = vector j), hessenberg[(cap + 1) * cap] (unrotated, row-major),
 * steps[m * 8] (iteration, estimate, recomputed relative, original residual, subdiagonal,
 * breakdown, verification triggered, accepted), candidates[m * n] (each step's candidate). */
int spai_record_inner(spai_handle *h, int64_t i, double *summary, double *rhs, double *solution, double *basis,
                      double *hessenberg, double *steps, double *candidates);

/* Score guard KAT on the device (cuda_evaluate_spai_score). out = {status, score, clamped}. */
int spai_score(int32_t precision, double rsq, double dot, double den, double *out);

/* Batched: `count` independent systems of any sizes, each with its own SPAI, in the mixed form
 * (opt->precision must be SPAI_PREC_MIXED, else SPAI_ERR_UNSUPPORTED). One SPAI build over the
 * block-diagonal union (identical to each system's own SPAI), then one persistent launch in which
 * each CTA runs one system's whole refinement. b[i], x[i] are host vectors of systems[i].n;
 * reports[i] is system i's IrResult summary (spai_ms/solve_ms are the whole batch's). Failures
 * stay per system (invalid_input, construction_failure). innercap = 0 means cap = n per system;
 * caps above 1936 are rejected (per-CTA Hessenberg workspace). No reference counterpart (the
 * reference solves one system per call). */
int spai_ir_solve_batched(int64_t count, const spai_csr *systems, const double *const *b,
                          double *const *x, const spai_options *opt, spai_report *reports,
                          void *stream);

/* Adjoint of x = A^{-1} b for nrhs right-hand sides (column-major n x nrhs): solves
 * A^T lambda = dLdx by GMRES right-preconditioned with P^T (same SPAI, no rebuild), then
 * dLdb = lambda and dLdA[e] = -sum_r lambda_r[i] x_r[j] over A's pattern (e = (i, j)). */
int spai_adjoint(spai_handle *h, int64_t nrhs, const double *x, const double *dLdx,
                 double *dLdb, double *dLdA_values, const spai_options *opt, spai_report *rep);
/* Same with device pointers (stream-ordered on the handle's stream, synchronous on return). The
 * report aggregates the nrhs solves: converged iff all converged, the first failing status,
 * the largest backward error, summed inner iterations and device time. dLdA follows the order
 * of the stored entries of the CSR given to spai_create. No reference counterpart (the
 * reference has no adjoint). */
int spai_adjoint_device(spai_handle *h, int64_t nrhs, const double *d_x, const double *d_dLdx,
                        double *d_dLdb, double *d_dLdA_values, const spai_options *opt,
                        spai_report *rep);

/* Matrix Market reader on the device (read_matrix_market + CsrMatrix::from_entries,
 * src/cpu.cpp:49-161): the host reads the file and its banner and size line; the GPU finds the
 * lines, parses every entry, mirrors symmetric off-diagonals, stably sorts by (row, col), sums
 * duplicates in input order and drops exact zeros. Accepted format, checks and results are the
 * reference reader's: "%%MatrixMarket matrix coordinate real|integer general|symmetric",
 * comment and blank lines skipped, one-based indices, finite values. Value tokens the device
 * cannot convert with a certified correctly rounded result (more than 19 significant digits,
 * hexadecimal or special tokens, results near a rounding midpoint, outside the normal range) are
 * converted on the host by the C library's strtod, so the values are the same bits.
 * Returns SPAI_ERR_FORMAT for malformed input, SPAI_ERR_ARGUMENT for invalid entries (the
 * reference's invalid_argument), SPAI_ERR_CUDA for runtime failures. The CSR stays valid until
 * spai_mm_free. No reference counterpart beyond the host reader it replaces. */
typedef struct spai_mm_matrix_s spai_mm_matrix;
/* device_min_lines: data sections with fewer lines are parsed on the host by the same rules
 * (the transfer and launch overheads exceed the parse time; the CLIs pass 65536); 0 = always
 * parse on the device. */
int spai_mm_read(const char *path, int64_t device_min_lines, spai_mm_matrix **out);
int spai_mm_csr(const spai_mm_matrix *m, spai_csr *csr, int64_t *cols, int64_t *host_converted_values);
int spai_mm_free(spai_mm_matrix *m);

/* History of the handle's last solve that ran with SPAI_FLAG_HISTORY: copies at most max_* records
 * of each kind and reports the recorded counts (n_* may exceed max_*; iteration records stop at
 * 1,048,576). Any output pointer may be NULL. No counterpart in the reference's C++ API beyond
 * the IrResult/GmresResult histories it returns (ir.hpp:44-56). */
int spai_history(spai_handle *h, spai_outer_record *outer, int64_t max_outer, int64_t *n_outer,
                 spai_inner_record *inner, int64_t max_inner, int64_t *n_inner,
                 spai_iteration_record *iterations, int64_t max_iterations, int64_t *n_iterations);

/* Per-kernel-class timing of refinement solves (CUDA events on the handle's stream around each
 * launch). Classes: 0 SpMV with A (basis vector gathered), 1 SpMV with P, 2 Gram-Schmidt pass 1
 * (dots), 3 pass 2 (update + dots; with the lagged second projection also the correction of the
 * previous vector), 4 pass 3 (reorthogonalisation; only in the three-pass form and only when it
 * runs). enable != 0 resets and starts recording; read returns the accumulated
 * device milliseconds, launch count and algorithmic bytes of one class. No reference
 * counterpart (the reference only kept host wall-clock telemetry, src/cuda_spai.cu:19-38). */
int spai_profile(spai_handle *h, int32_t enable);
int spai_profile_read(spai_handle *h, int32_t cls, double *ms, int64_t *launches, double *bytes);

/* Choices of the autotuner for the handle's last build and solve set-up (no reference
 * counterpart: the reference's launch policy is fixed, e.g. 8 slot streams in
 * src/cuda_spai.cu:575-577). out[0] lanes per column group and out[1] workspace bytes per group
 * of the SPAI's first workspace tier; out[2] = 1 when the autotuner chose them (first-tier
 * candidates timed on a column sample, cached per sparsity profile for the process), 0 for the
 * profile default or an override; out[3] / out[4] layout of the Krylov SpMV with the inner A /
 * with P (0 sliced ELLPACK over natural rows, 1 over rows sorted by length, 2 one array per
 * occupied diagonal; -1 no solve set up yet).
 * ms (optional, 2 doubles): the chosen pair's and the default pair's time on the sample (NaN
 * when not tuned). Returns SPAI_OK or an error code. */
int spai_tuning(spai_handle *h, int32_t *out, double *ms);

/* Backward error of a given x with no device allocation (no counterpart in the reference).
 * For callers that cannot call cudaMalloc where they need this check: applications whose device
 * memory is owned by their own pool/caching allocator, and latency-critical loops that cannot
 * afford an allocation's implicit synchronisation. d_b, d_x: binary64 device vectors of the
 * handle's n; d_out: device array of 3 doubles receiving {normwise backward error,
 * componentwise backward error, ||b - A x||_inf}. The handle must hold A in binary64
 * (SPAI_PREC_F64 or SPAI_PREC_MIXED). Scratch (the residual and per-block partials) is a fixed
 * file-scope device array of 4 MiB + 33,024 bytes that every GPU loading the library keeps until exit;
 * systems with n > 524288 rows are rejected with SPAI_ERR_ARGUMENT. The first call on a device
 * looks up that array's address (once per device); make this first call before any stream
 * capture. All calls share the array and it keeps the last call's contents; calls that overlap
 * on the GPU race. stream: cudaStream_t to launch on, NULL = the handle's stream. The call is
 * asynchronous; synchronise the stream before reading d_out. When x, b, A x or the norms are not
 * finite, the call still returns SPAI_OK and d_out[0] (normwise) is NaN; d_out[1] and d_out[2]
 * then hold whatever the non-finite values give (Inf or NaN). A caller treats a NaN in d_out[0]
 * as the solve's numerical_failure. */
int spai_backward_error_noalloc(spai_handle *h, const double *d_b, const double *d_x,
                                double *d_out, void *stream);

/* The device's correctly rounded hypot on host arrays, exposed so that it can be checked against
 * an independent implementation. precision 0: binary64 hypot; 1: binary32 hypot on the operands
 * rounded to binary32 (widened on return); 2 / 3: the binary64 / binary32 step of the SPAI norm
 * chains from the running norm |a|, which must give the same bits as 0 / 1.
 * Returns SPAI_OK or an error code. No reference counterpart. */
int spai_hypot_device(int32_t precision, int64_t count, const double *a, const double *b, double *out);

/* Host builds of the device hypot used by the SPAI fits (parity tests). */
double spai_hypot(double a, double b);
float spai_hypotf(float a, float b);

#ifdef __cplusplus
}
#endif
#endif
