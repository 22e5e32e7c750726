// gpu_diag_ir: the verbose diagnostic CLI of the binary64 solve (reference adapter
// src/cuda_hybrid_main.cpp:21-140): same argv (MATRIX.mtx [epsilon=0.3] [outercap=20]
// [innercap=0 (= n)]), alpha = ceil(n/8), beta = 8, RHS b_i = 1/sqrt(n), exit codes 0 converged /
// 1 not converged or runtime error / 2 input error, and the same report lines: the solve banner,
// options, status, per-outer diagnostics (residual_inf, residual_2, eta_n, eta_c), per-inner GMRES
// summaries and per-iteration estimates, then x. Telemetry lines describe this implementation
// (device-resident solve: no per-step host transfers) instead of the reference's transfer counters.
// Recomputed relative residuals exist only for the steps where the acceptance rule verified a
// candidate; the others print nan.
#include "cli_read.hpp"
#include "spai_ir.h"

#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace {
uint64_t count(const char *text) {
    const std::string s(text);
    if (s.empty() || s.find_first_not_of("0123456789") != std::string::npos)
        throw std::invalid_argument("Expected unsigned integer cap");
    size_t used = 0;
    const unsigned long long v = std::stoull(s, &used);
    if (used != s.size())
        throw std::invalid_argument("Invalid cap");
    return static_cast<uint64_t>(v);
}
struct RuntimeFailure : std::runtime_error {
    using std::runtime_error::runtime_error;
};
void check(int rc) {
    if (rc == SPAI_ERR_ARGUMENT)
        throw std::invalid_argument(spai_last_error());
    if (rc != SPAI_OK)
        throw RuntimeFailure(spai_last_error());
}
} // namespace

int main(int argc, char **argv) {
    if (argc < 2 || argc > 5) {
        std::cerr << "Usage: gpu_diag_ir matrix.mtx [epsilon=0.3] [outercap=20] [innercap=0(default n)]\n";
        return 2;
    }
    try {
        spai_mm::HostCsr a = spai_cli::read_matrix(argv[1]);
        if (!a.rows || a.rows != a.cols)
            throw std::invalid_argument("Hybrid IR requires a nonempty square matrix");
        const uint64_t n = a.rows;
        spai_options opt;
        spai_default_options(&opt, SPAI_PREC_F64);
        opt.epsilon = 0.3;
        opt.beta = 8;
        opt.alpha = static_cast<int64_t>(n / 8 + (n % 8 != 0));
        if (argc >= 3) {
            size_t used = 0;
            const std::string s(argv[2]);
            opt.epsilon = std::stod(s, &used);
            if (used != s.size())
                throw std::invalid_argument("Invalid epsilon");
        }
        uint64_t outercap = 20, innercap = 0;
        if (argc >= 4)
            outercap = count(argv[3]);
        if (argc >= 5)
            innercap = count(argv[4]);
        if (!std::isfinite(opt.epsilon) || opt.epsilon <= 0 || outercap > 20 || innercap > n)
            throw std::invalid_argument("Require finite positive epsilon, outercap<=20, innercap<=n");
        opt.outercap = static_cast<int64_t>(outercap);
        opt.innercap = static_cast<int64_t>(innercap);
        opt.flags |= SPAI_FLAG_HISTORY;
        const std::vector<double> rhs(n, 1 / std::sqrt(static_cast<double>(n)));
        std::vector<double> x(n, 0.0);
        spai_csr csr{static_cast<int64_t>(n), static_cast<int64_t>(a.val.size()), a.ptr.data(), a.idx.data(),
                     a.val.data()};
        spai_handle *raw = nullptr;
        check(spai_create(&csr, SPAI_PREC_F64, 0, nullptr, &raw));
        std::unique_ptr<spai_handle, int (*)(spai_handle *)> h(raw, spai_destroy);
        spai_report brep, rep;
        check(spai_build(h.get(), &opt, &brep));
        check(spai_solve(h.get(), rhs.data(), x.data(), nullptr, &opt, &rep));
        const double tau = 1e-8, backward_tolerance = 10 * std::ldexp(1.0, -53);
        std::string message;
        if (rep.ir_status == IR_CONSTRUCTION_FAILURE)
            message = std::string("GPU SPAI failed: ") + spai_status_name(rep.spai_status) + ": Column " +
                      std::to_string(brep.first_failed_column);
        else if (rep.ir_status == IR_INNER_FAILURE)
            message = std::string("Correction GMRES failed: ") + gmres_status_name(rep.gmres_status);
        else if (rep.ir_status == IR_STAGNATION)
            message = "Unchanged outer iterate above original backward-error tolerance";
        else if (rep.ir_status == IR_ITERATION_LIMIT)
            message = "Outer correction cap reached above original backward-error tolerance";
        else if (rep.ir_status == IR_NUMERICAL_FAILURE)
            message = "Nonfinite outer residual/backward-error arithmetic";
        else if (rep.ir_status == IR_INVALID_INPUT)
            message = "Invalid dimensions, finite inputs, inner options, or outer cap";
        std::cout << std::setprecision(17) << "matrix=" << argv[1] << " n=" << n << " nnz=" << a.val.size()
                  << "\n"
                  << "precision=binary64 cpu_spai=false cpu_outer=false gpu_gmres=true rhs=equal_unit2 "
                     "gpu_spai=true\n"
                  << "epsilon=" << opt.epsilon << " beta=" << opt.beta << " alpha=" << opt.alpha << " tau=" << tau
                  << " innercap=" << opt.innercap << " outercap=" << opt.outercap
                  << " backward_tolerance=" << backward_tolerance << "\n"
                  << "status=" << ir_status_name(rep.ir_status) << " converged=" << rep.converged
                  << " outer_steps=" << rep.outer_steps << " inner_attempts=" << rep.inner_attempts << "\n"
                  << "message=" << message << "\n"
                  << "device_resident=true kernel_launches=" << brep.kernel_launches + rep.kernel_launches
                  << " spai_ms=" << brep.spai_ms << " solve_ms=" << rep.solve_ms << "\n";
        if (rep.spai_status != SPAI_NOT_ATTEMPTED)
            std::cout << "spai_status=" << spai_status_name(rep.spai_status) << " nnz_P=" << brep.nnz_p << "\n";
        std::cout << "construction_fits=" << brep.spai_fits << " growths=" << brep.spai_growths
                  << " workspace_overflow_columns=" << brep.spai_overflow_columns << "\n";
        int64_t no = 0, ni = 0, nit = 0;
        if (spai_history(h.get(), nullptr, 0, &no, nullptr, 0, &ni, nullptr, 0, &nit) == SPAI_OK) {
            std::vector<spai_outer_record> outer(static_cast<size_t>(no));
            std::vector<spai_inner_record> inner(static_cast<size_t>(ni));
            std::vector<spai_iteration_record> its(static_cast<size_t>(nit));
            check(spai_history(h.get(), outer.data(), no, &no, inner.data(), ni, &ni, its.data(), nit, &nit));
            for (const auto &o : outer)
                std::cout << "outer=" << o.step << " residual_inf=" << o.residual_inf
                          << " residual_2=" << o.residual_2 << " eta_n=" << o.normwise_backward_error
                          << " eta_c=" << o.componentwise_backward_error << "\n";
            size_t t = 0;
            for (int64_t j = 0; j < ni; ++j) {
                const auto &r = inner[static_cast<size_t>(j)];
                std::cout << "inner=" << j + 1 << " status=" << gmres_status_name(r.status)
                          << " iterations=" << r.iterations << " true_relative=" << r.final_relative
                          << " update_applied=" << r.update_applied << "\n";
                for (; t < its.size() && its[t].inner == j + 1; ++t)
                    std::cout << "inner_iteration=" << its[t].iteration << " estimate=" << its[t].estimated_relative
                              << " true_relative=" << its[t].recomputed_relative
                              << " accepted=" << its[t].accepted << "\n";
            }
        }
        if (rep.ir_status != IR_CONSTRUCTION_FAILURE && rep.ir_status != IR_INVALID_INPUT)
            for (uint64_t j = 0; j < n; ++j)
                std::cout << "x[" << j << "]=" << x[j] << "\n";
        return rep.converged ? 0 : (rep.ir_status == IR_INVALID_INPUT ? 2 : 1);
    } catch (const std::invalid_argument &e) {
        std::cerr << "Input error: " << e.what() << "\n";
        return 2;
    } catch (const std::out_of_range &e) {
        std::cerr << "Input range error: " << e.what() << "\n";
        return 2;
    } catch (const std::exception &e) {
        std::cerr << "Checked runtime error: " << e.what() << "\n";
        return 1;
    }
}
