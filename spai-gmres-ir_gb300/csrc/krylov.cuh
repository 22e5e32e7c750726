// Device-side GMRES / iterative-refinement state shared by krylov.cu and the API layer.
#pragma once
#include "spai_internal.hpp"
#include "spai_ir.h"

#include <cmath>
#include <vector>

namespace spai {

// Control block in device memory. Every kernel of the Arnoldi step and the refinement loop
// reads its loop state here, so the same launch sequence can be replayed by a CUDA graph.
struct Ctl {
    // GMRES
    int k;           // current Arnoldi column
    int cap;         // iteration cap
    int active;      // GMRES loop still running
    int status;      // GmresStatus of the current inner solve
    int converged;
    int triggered;   // candidate verification requested for column k
    int breakdown;   // h(k+1,k) == 0
    int iterations;
    int formed;      // columns in the last formed candidate
    int norm_rescale;
    // IR
    int outer_active;
    int ir_status;
    int outer_steps;
    int inner_attempts;
    int inner_iterations_total;
    int changed;     // x + d != x somewhere (stagnation test)
    int nonfinite;   // a refinement quantity overflowed
    int last_gmres_status;
    int ir_started;
    int nrows;        // n: GMRES cap < n -> iteration_limit, else nonconvergence
    int accept_every; // binary32 drop-in acceptance (verify every step)
    int accept_partial; // SPAI_FLAG_RESTART_AT_CAP
    int vgate;        // verification kernels of this step run
    int pending;      // an update x_new = x + d awaits its diagnostics
    int guard;        // Arnoldi steps run in this solve (bounds every device-side loop)
    int verifications; // candidate checks run in this solve
    int reorth;        // this step needs the second Gram-Schmidt pass (DGKS criterion)
    int reorth_count;  // second passes run in this solve
    int lag_pending;   // lagged Gram-Schmidt: the newest basis vector awaits its second projection
    double wnorm;      // ||P A v_k|| before orthogonalisation
    double be, cbe, rinf, xinf, bscale, anorm_inf, binf;
    double inner_scale; // power of two applied to the correction right-hand side
    double tol_inner;
    double be_tol;
    double den, beta, est, hnext, rel, orig;
    int outer_cap;
    int counters[16];   // spare
    // Refinement history (SPAI_FLAG_HISTORY): records written by the decision kernels; null
    // pointers when not requested.
    spai_outer_record *h_outer;
    spai_inner_record *h_inner;
    spai_iteration_record *h_iter;
    int h_cap_outer, h_cap_inner, h_cap_iter;
    int h_n_outer, h_n_inner, h_n_iter;
    int h_iter_base;
    // Record mode (SPAI_FLAG_RECORD): every step's candidate is formed and verified for the
    // record, only a triggered check may accept it; h_raw (element type of the engine, leading
    // dimension h_raw_ld) receives each Hessenberg column before its rotations.
    int record_every;
    int h_raw_ld;
    void *h_raw;
};

struct GmresBuffers; // defined in krylov.cu

// Host record of a solve run in record mode: what the reference's GmresResult and IrResult keep
// (include/bspai/gmres.hpp:28-50, include/bspai/ir.hpp:36-56), as the device computed it, read
// back after every Arnoldi step. Diagnostics for small systems.
struct KrylovStep {
    double original = NAN;          // ||rhs - A x_j|| of the step's candidate
    std::vector<double> candidate;  // x_j = V_j y_j (zero initial guess)
};
struct KrylovInner {
    int status = -1, converged = 0, iterations = 0, applied = 0;
    double initial_original = NAN, final_original = NAN, final_preconditioned = NAN;
    std::vector<double> rhs, solution;
    std::vector<double> basis;       // nbasis normalised vectors of n entries
    int nbasis = 0;
    std::vector<double> hessenberg;  // unrotated, (cap + 1) x cap row-major
    int hcap = 0;
    std::vector<KrylovStep> steps;
    std::vector<spai_iteration_record> records; // estimate, recomputed, trigger, acceptance
};
struct KrylovState {
    std::vector<double> x, residual; // iterate and b - A x (binary64)
};
struct KrylovRecord {
    std::vector<KrylovState> states;
    std::vector<KrylovInner> inner;
    void clear() {
        states.clear();
        inner.clear();
    }
};

// Settings of one solve.
struct SolveSettings {
    int cap = 0;
    int outer_cap = 20;
    double tau = 1e-8;
    double be_tol = 0;
    bool scale_rhs = false; // mixed form: power-of-two scaled binary32 correction RHS
    bool accept_every = false; // binary32 drop-in acceptance (recomputed residual each step)
    bool use_graph = true;
    bool history = false;      // record the refinement history (SPAI_FLAG_HISTORY)
    bool restart_at_cap = false; // SPAI_FLAG_RESTART_AT_CAP
    struct KrylovRecord *record = nullptr; // SPAI_FLAG_RECORD: host record of every step
};

} // namespace spai
