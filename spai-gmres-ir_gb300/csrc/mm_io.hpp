// Host Matrix Market reader and canonical CSR builder.
//
// Same accepted format and the same canonicalisation as the reference's read_matrix_market /
// CsrMatrix::from_entries (src/cpu.cpp:49-161): "%%MatrixMarket matrix coordinate" with field
// real|integer and symmetry general|symmetric; comment and blank lines skipped; one-based
// indices; finite values; symmetric off-diagonals mirrored; entries stably sorted by (row, col),
// duplicates summed in input order, exact zero sums dropped. Malformed input throws
// std::runtime_error and invalid entries std::invalid_argument, as the reference does, so the CLI
// keeps the reference's exit codes.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <istream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace spai_io {

struct Entry {
    uint64_t row, col;
    double value;
};

struct HostCsr {
    uint64_t rows = 0, cols = 0;
    std::vector<int64_t> ptr, idx;
    std::vector<double> val;
};

inline HostCsr from_entries(uint64_t rows, uint64_t cols, std::vector<Entry> e) {
    for (const Entry &x : e) {
        if (x.row >= rows || x.col >= cols)
            throw std::invalid_argument("Entry index outside matrix dimensions");
        if (!std::isfinite(x.value))
            throw std::invalid_argument("Matrix entries must be finite");
    }
    std::stable_sort(e.begin(), e.end(), [](const Entry &a, const Entry &b) {
        return a.row < b.row || (a.row == b.row && a.col < b.col);
    });
    HostCsr m;
    m.rows = rows;
    m.cols = cols;
    m.ptr.assign(rows + 1, 0);
    for (size_t i = 0; i < e.size();) {
        const Entry first = e[i++];
        double sum = first.value;
        while (i < e.size() && e[i].row == first.row && e[i].col == first.col) {
            sum += e[i++].value;
            if (!std::isfinite(sum))
                throw std::invalid_argument("Duplicate sum is nonfinite");
        }
        if (sum != 0.0) {
            m.idx.push_back(static_cast<int64_t>(first.col));
            m.val.push_back(sum);
            ++m.ptr[first.row + 1];
        }
    }
    for (uint64_t r = 0; r < rows; ++r)
        m.ptr[r + 1] += m.ptr[r];
    return m;
}

namespace detail {
inline bool next_data_line(std::istream &in, std::string &line) {
    while (std::getline(in, line)) {
        const size_t b = line.find_first_not_of(" \t\r");
        if (b != std::string::npos && line[b] != '%')
            return true;
    }
    return false;
}
inline uint64_t parse_size(const std::string &t) {
    if (t.empty() || t.find_first_not_of("0123456789") != std::string::npos)
        throw std::runtime_error("Expected a nonnegative integer dimension/index");
    uint64_t r = 0;
    for (char c : t) {
        const uint64_t d = static_cast<uint64_t>(c - '0');
        if (r > (std::numeric_limits<uint64_t>::max() - d) / 10)
            throw std::runtime_error("Dimension/index exceeds size_t");
        r = r * 10 + d;
    }
    return r;
}
inline void require_end(std::istringstream &s) {
    std::string extra;
    if (s >> extra)
        throw std::runtime_error("Extra field in Matrix Market line");
}
} // namespace detail

inline HostCsr read_matrix_market(std::istream &in) {
    using namespace detail;
    std::string text, magic, object, format, field, symmetry;
    if (!std::getline(in, text))
        throw std::runtime_error("Missing Matrix Market banner");
    std::istringstream banner(text);
    if (!(banner >> magic >> object >> format >> field >> symmetry))
        throw std::runtime_error("Malformed Matrix Market banner");
    require_end(banner);
    if (magic != "%%MatrixMarket" || object != "matrix" || format != "coordinate" ||
        (field != "real" && field != "integer") ||
        (symmetry != "general" && symmetry != "symmetric"))
        throw std::runtime_error("Unsupported Matrix Market format");
    if (!next_data_line(in, text))
        throw std::runtime_error("Missing matrix dimensions");
    std::string rt, ct, nt;
    std::istringstream dims(text);
    if (!(dims >> rt >> ct >> nt))
        throw std::runtime_error("Malformed matrix dimensions");
    require_end(dims);
    const uint64_t rows = parse_size(rt), cols = parse_size(ct), count = parse_size(nt);
    if (rows == 0 || cols == 0)
        throw std::runtime_error("Matrix dimensions must be positive");
    if (symmetry == "symmetric" && rows != cols)
        throw std::runtime_error("Symmetric matrix must be square");
    std::vector<Entry> entries;
    entries.reserve(count < (1ull << 28) ? count : 0);
    for (uint64_t i = 0; i < count; ++i) {
        if (!next_data_line(in, text))
            throw std::runtime_error("Truncated coordinate data");
        std::istringstream coord(text);
        std::string vt;
        if (!(coord >> rt >> ct >> vt))
            throw std::runtime_error("Malformed coordinate entry");
        require_end(coord);
        const uint64_t r = parse_size(rt), c = parse_size(ct);
        if (r == 0 || c == 0 || r > rows || c > cols)
            throw std::runtime_error("Matrix Market index outside one-based dimensions");
        size_t used = 0;
        double v;
        try {
            v = std::stod(vt, &used);
        } catch (const std::exception &) {
            throw std::runtime_error("Invalid coordinate value");
        }
        if (used != vt.size() || !std::isfinite(v))
            throw std::runtime_error("Coordinate value must be finite and numeric");
        if (field == "integer" && vt.find_first_not_of("+-0123456789") != std::string::npos)
            throw std::runtime_error("Integer field requires integer value tokens");
        entries.push_back(Entry{r - 1, c - 1, v});
        if (symmetry == "symmetric" && r != c)
            entries.push_back(Entry{c - 1, r - 1, v});
    }
    if (next_data_line(in, text))
        throw std::runtime_error("Trailing coordinate data");
    return from_entries(rows, cols, std::move(entries));
}

} // namespace spai_io
