// Drop-in solver CLIs: gpu_fp64_ir (SOLVER_F64), gpu_fp32_ir (SOLVER_F32), gpu_mixed_ir
// (SOLVER_MIXED). Argument, output and exit-code contract of the reference adapter
// src/solver_main.cpp:60-144:
//   MATRIX.mtx [epsilon=0.3] [outercap=20] [innercap=0 (= n)]
//   alpha = ceil(n/8), beta = 8, RHS b_i = 1/sqrt(n) in the solver precision,
//   exit 0 converged / 1 not converged or runtime error / 2 input error.
// The solve runs on the device end to end (SPAI build, GMRES, refinement), so the banner says
// cpu_outer=false where the reference printed cpu_outer=true.
#include "cli_read.hpp"
#include "spai_ir.h"

#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#if defined(SOLVER_F32)
using Scalar = float;
static const int kPrecision = SPAI_PREC_F32;
static const char *kBanner = "precision=FP32 backend=GPU cpu_outer=false";
#elif defined(SOLVER_MIXED)
using Scalar = double;
static const int kPrecision = SPAI_PREC_MIXED;
static const char *kBanner = "precision=MIXED backend=GPU cpu_outer=false";
#else
using Scalar = double;
static const int kPrecision = SPAI_PREC_F64;
static const char *kBanner = "precision=FP64 backend=GPU cpu_outer=false";
#endif

namespace {
uint64_t parse_count(const char *text) {
    const std::string v(text);
    if (v.empty() || v.find_first_not_of("0123456789") != std::string::npos)
        throw std::invalid_argument("Expected an unsigned integer cap");
    const unsigned long long c = std::stoull(v); // out_of_range for oversized values
    return static_cast<uint64_t>(c);
}

struct RuntimeFailure : std::runtime_error {
    using std::runtime_error::runtime_error;
};
} // namespace

int main(int argc, char **argv) {
    if (argc < 2 || argc > 5) {
        std::cerr << "Usage: " << argv[0]
                  << " MATRIX.mtx [epsilon=0.3] [outercap=20] [innercap=0(default n)]\n";
        return 2;
    }
    try {
        spai_mm::HostCsr a = spai_cli::read_matrix(argv[1]);
        if (!a.rows || a.rows != a.cols)
            throw std::invalid_argument("Solver requires a nonempty square matrix");
        const uint64_t n = a.rows;
#if defined(SOLVER_F32) || defined(SOLVER_MIXED)
        // Binary32 input rounding with range checks (src/solver_main.cpp:36-50); the mixed form
        // keeps A in binary64 for the refinement residual, so only the binary32 drop-in rounds.
        for (double &v : a.val) {
            if (std::fabs(v) > std::numeric_limits<float>::max())
                throw std::invalid_argument("Matrix entry exceeds FP32 range");
            const float r = static_cast<float>(v);
            if (v != 0 && r == 0)
                throw std::invalid_argument("Matrix entry underflows FP32 range");
#if defined(SOLVER_F32)
            v = r;
#endif
        }
#endif
        spai_options opt;
        spai_default_options(&opt, kPrecision);
        opt.alpha = static_cast<int64_t>(n / 8 + (n % 8 != 0));
        opt.beta = 8;
        Scalar epsilon = static_cast<Scalar>(0.3);
        if (argc >= 3) {
            const std::string text(argv[2]);
            size_t used = 0;
            const double e = std::stod(text, &used);
            if (used != text.size() || !std::isfinite(e) || e <= 0 ||
                e > std::numeric_limits<Scalar>::max())
                throw std::invalid_argument("Require a finite positive epsilon in precision range");
            epsilon = static_cast<Scalar>(e);
            if (epsilon == 0)
                throw std::invalid_argument("Epsilon underflows precision");
        }
        opt.epsilon = epsilon;
        uint64_t outercap = 20, innercap = 0;
        if (argc >= 4)
            outercap = parse_count(argv[3]);
        if (argc >= 5)
            innercap = parse_count(argv[4]);
        if (outercap > 20 || innercap > n)
            throw std::invalid_argument("Require outercap<=20 and innercap<=n");
        opt.outercap = static_cast<int64_t>(outercap);
        opt.innercap = static_cast<int64_t>(innercap);
        const Scalar bval = Scalar(1) / std::sqrt(Scalar(n));
        const std::vector<double> b(n, static_cast<double>(bval));
        std::vector<double> x(n, 0.0);
        spai_csr csr{static_cast<int64_t>(n), static_cast<int64_t>(a.val.size()), a.ptr.data(),
                     a.idx.data(), a.val.data()};
        spai_report rep;
        const int rc = spai_ir_solve(&csr, b.data(), x.data(), nullptr, &opt, &rep, nullptr);
        if (rc == SPAI_ERR_ARGUMENT)
            throw std::invalid_argument(spai_last_error());
        if (rc != SPAI_OK)
            throw RuntimeFailure(spai_last_error());
        const Scalar tau = static_cast<Scalar>(kPrecision == SPAI_PREC_F64 ? 1e-8 : 1e-4);
        std::string message;
        if (rep.ir_status == IR_CONSTRUCTION_FAILURE)
            message = std::string("GPU SPAI failed: ") + spai_status_name(rep.spai_status) +
                      ": Column " + std::to_string(rep.first_failed_column);
        else if (rep.ir_status == IR_INNER_FAILURE)
            message = std::string("Correction GPU GMRES failed: ") + gmres_status_name(rep.gmres_status);
        else if (rep.ir_status == IR_STAGNATION)
            message = "Unchanged outer iterate above original backward-error tolerance";
        else if (rep.ir_status == IR_ITERATION_LIMIT)
            message = "Outer correction cap reached above original backward-error tolerance";
        else if (rep.ir_status == IR_NUMERICAL_FAILURE)
            message = "Nonfinite outer residual/backward-error arithmetic";
        else if (rep.ir_status == IR_INVALID_INPUT)
            message = "Invalid dimensions, finite inputs, inner options, or outer cap";
        std::cout << std::setprecision(std::numeric_limits<Scalar>::max_digits10) << kBanner << '\n'
                  << "n=" << n << " nnz=" << a.val.size() << " epsilon=" << epsilon
                  << " tau=" << tau << '\n'
                  << "status=" << ir_status_name(rep.ir_status) << " converged=" << rep.converged
                  << " outer_steps=" << rep.outer_steps << '\n'
                  << "message=" << message << '\n';
        if (rep.converged)
            std::cout << "residual_inf=" << static_cast<Scalar>(rep.residual_inf)
                      << " backward_error=" << static_cast<Scalar>(rep.backward_error) << '\n';
        const bool has_solution =
            rep.ir_status != IR_CONSTRUCTION_FAILURE && rep.ir_status != IR_INVALID_INPUT;
        if (has_solution)
            for (uint64_t i = 0; i < n; ++i)
                std::cout << "x[" << i << "]=" << static_cast<Scalar>(x[i]) << '\n';
        return rep.converged ? 0 : 1;
    } catch (const std::invalid_argument &e) {
        std::cerr << "Input error: " << e.what() << '\n';
        return 2;
    } catch (const std::out_of_range &e) {
        std::cerr << "Input error: " << e.what() << '\n';
        return 2;
    } catch (const std::exception &e) {
        std::cerr << "Solver error: " << e.what() << '\n';
        return 1;
    }
}
