// Matrix Market input of the CLIs through spai_mm_read (device parse for large files), with the
// reference reader's exception classes: invalid_argument for invalid entries and unopenable
// files (exit 2), runtime_error for malformed input (exit 1), as src/solver_main.cpp maps them.
#pragma once
#include "mm_text.hpp"
#include "spai_ir.h"

#include <memory>
#include <stdexcept>
#include <string>

namespace spai_cli {
inline spai_mm::HostCsr read_matrix(const char *path) {
    spai_mm_matrix *raw = nullptr;
    const int rc = spai_mm_read(path, 65536, &raw);
    if (rc == SPAI_ERR_ARGUMENT)
        throw std::invalid_argument(spai_last_error());
    if (rc != SPAI_OK)
        throw std::runtime_error(spai_last_error());
    std::unique_ptr<spai_mm_matrix, int (*)(spai_mm_matrix *)> m(raw, spai_mm_free);
    spai_csr c;
    int64_t cols = 0;
    spai_mm_csr(m.get(), &c, &cols, nullptr);
    spai_mm::HostCsr a;
    a.rows = static_cast<uint64_t>(c.n);
    a.cols = static_cast<uint64_t>(cols);
    a.ptr.assign(c.row_offsets, c.row_offsets + c.n + 1);
    a.idx.assign(c.col_indices, c.col_indices + c.nnz);
    a.val.assign(c.values, c.values + c.nnz);
    return a;
}
} // namespace spai_cli
