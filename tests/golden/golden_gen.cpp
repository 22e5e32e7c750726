// Golden-vector generator: runs the reference's own CPU FP64/FP32 solvers (compiled from the
// reference sources by oracle/Makefile `ref`) on a Matrix Market file and writes their outputs
// as little-endian binary records for make_golden.py. Only used to (re)generate tests/golden;
// nothing at test or bench time runs it.
//
// usage: golden_gen spai   A.mtx eps alpha beta out.bin   (FP64 construct_spai, spai.cpp:314)
//        golden_gen ir     A.mtx eps alpha beta tau innercap outercap out.bin
//                                         (FP64 spai_gmres_ir, ir.cpp:206; RHS 1/sqrt(n))
//        golden_gen ir32   A.mtx eps alpha beta tau innercap outercap out.bin
//                                         (FP32 fp32_spai_gmres_ir, fp32_cpu.cpp:746)
#include "bspai/cpu.hpp"
#include "bspai/fp32.hpp"
#include "bspai/ir.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {
struct Out {
    FILE *f;
    void i64(int64_t v) {
        std::fwrite(&v, 8, 1, f);
    }
    void f64(double v) {
        std::fwrite(&v, 8, 1, f);
    }
    void vi(const std::vector<std::size_t> &v) {
        i64(static_cast<int64_t>(v.size()));
        for (auto x : v)
            i64(static_cast<int64_t>(x));
    }
    template <class T> void vf(const std::vector<T> &v) {
        i64(static_cast<int64_t>(v.size()));
        for (auto x : v)
            f64(static_cast<double>(x));
    }
};
bspai::CsrMatrix load(const char *path) {
    std::ifstream s(path);
    if (!s)
        throw std::runtime_error("cannot open matrix");
    return bspai::read_matrix_market(s);
}
} // namespace

int main(int argc, char **argv) {
    try {
        if (argc < 7)
            throw std::runtime_error("usage");
        const std::string mode = argv[1];
        const auto a = load(argv[2]);
        const std::size_t n = a.rows();
        Out o{nullptr};
        if (mode == "spai") {
            bspai::SpaiOptions opt;
            opt.epsilon = std::stod(argv[3]);
            opt.alpha = std::stoull(argv[4]);
            opt.beta = std::stoull(argv[5]);
            const auto r = bspai::construct_spai(a, opt);
            o.f = std::fopen(argv[6], "wb");
            o.i64(static_cast<int64_t>(r.status));
            o.i64(static_cast<int64_t>(n));
            o.vf(r.scaling);
            for (std::size_t k = 0; k < r.columns.size(); ++k) {
                const auto &c = r.columns[k];
                o.i64(static_cast<int64_t>(c.status));
                o.i64(static_cast<int64_t>(c.fits));
                o.i64(static_cast<int64_t>(c.growths));
                o.i64(static_cast<int64_t>(c.score_clamps));
                o.f64(c.reduced_residual);
                o.vi(c.pattern);
                o.vf(c.coefficients);
            }
            o.vi(r.preconditioner.row_offsets());
            o.vi(r.preconditioner.column_indices());
            o.vf(r.preconditioner.values());
        } else if (mode == "ir" || mode == "ir32") {
            if (argc < 10)
                throw std::runtime_error("usage");
            const double eps = std::stod(argv[3]), tau = std::stod(argv[6]);
            const std::size_t alpha = std::stoull(argv[4]), beta = std::stoull(argv[5]);
            const std::size_t inner = std::stoull(argv[7]), outer = std::stoull(argv[8]);
            o.f = std::fopen(argv[9], "wb");
            if (mode == "ir") {
                bspai::IrOptions opt;
                opt.spai.epsilon = eps;
                opt.spai.alpha = alpha;
                opt.spai.beta = beta;
                opt.gmres.tolerance = tau;
                opt.gmres.max_iterations = inner;
                opt.max_outer_steps = outer;
                const std::vector<double> rhs(n, 1.0 / std::sqrt(static_cast<double>(n)));
                const auto r = bspai::spai_gmres_ir(a, rhs, opt);
                o.i64(static_cast<int64_t>(r.status));
                o.i64(r.converged);
                o.i64(static_cast<int64_t>(r.outer_steps));
                o.i64(static_cast<int64_t>(r.construction.preconditioner.values().size()));
                std::size_t inner_total = 0;
                for (const auto &g : r.inner_history)
                    inner_total += g.iterations;
                o.i64(static_cast<int64_t>(inner_total));
                const auto &d = r.history.empty() ? bspai::IrDiagnostics() : r.history.back().diagnostics;
                o.f64(d.normwise_backward_error);
                o.f64(d.residual_inf);
                o.vf(r.solution);
            } else {
                std::vector<bspai::Fp32Entry> e;
                for (std::size_t row = 0; row < n; ++row)
                    for (auto q = a.row_offsets()[row]; q < a.row_offsets()[row + 1]; ++q)
                        e.push_back({row, a.column_indices()[q], static_cast<float>(a.values()[q])});
                const auto af = bspai::Fp32CsrMatrix::from_entries(n, n, e);
                bspai::Fp32IrOptions opt;
                opt.spai.epsilon = static_cast<float>(eps);
                opt.spai.alpha = alpha;
                opt.spai.beta = beta;
                opt.gmres.tolerance = static_cast<float>(tau);
                opt.gmres.max_iterations = inner;
                opt.max_outer_steps = outer;
                const std::vector<float> rhs(n, 1.0f / std::sqrt(static_cast<float>(n)));
                const auto r = bspai::fp32_spai_gmres_ir(af, rhs, opt);
                o.i64(static_cast<int64_t>(r.status));
                o.i64(r.converged);
                o.i64(static_cast<int64_t>(r.outer_steps));
                o.i64(static_cast<int64_t>(r.construction.preconditioner_nnz));
                std::size_t inner_total = 0;
                for (const auto &g : r.inner_history)
                    inner_total += g.iterations;
                o.i64(static_cast<int64_t>(inner_total));
                const auto d = r.outer_history.empty() ? bspai::Fp32IrDiagnostics() : r.outer_history.back();
                o.f64(d.normwise_backward_error);
                o.f64(d.residual_inf);
                o.vf(r.solution);
            }
        } else {
            throw std::runtime_error("unknown mode");
        }
        std::fclose(o.f);
        return 0;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "golden_gen: %s\n", e.what());
        return 1;
    }
}
