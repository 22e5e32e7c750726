// Matrix Market text rules, shared by the host reader and the device reader.
//
// The accepted input is the reference's (src/cpu.cpp:105-161, read_matrix_market): a banner
// "%%MatrixMarket matrix coordinate <real|integer> <general|symmetric>", a size line
// "rows cols count", then `count` data lines "row col value" with one-based indices; lines whose
// first character other than space, tab or carriage return is '%' (or that have none) are
// skipped; fields are separated by the C locale's white space; a symmetric file lists one
// triangle and each off-diagonal entry also stands for its mirror. The canonical matrix is CSR
// in (row, col) order where each position's duplicates are added in file order and an exact zero
// sum leaves no entry (src/cpu.cpp:49-78, CsrMatrix::from_entries).
//
// Errors keep the reference's messages and check order, and its exception classes, because the
// drop-in CLIs turn them into exit codes: std::runtime_error (exit 1) for malformed text and
// std::invalid_argument (exit 2) for invalid entries.
//
// Layout of this file: the per-line rules (field splitting, index tokens, one data line) are
// __host__ __device__ so the device reader's one-thread-per-line kernel and the host reader apply
// literally the same code; the value token's conversion is the one step that differs (the device
// certifies a fast decimal conversion and hands everything else to host_value below). The host
// reader walks a memory buffer line by line and builds the CSR by bucketing entries per row (in
// file order) and ordering each row's bucket by column with a stable merge sort.
#pragma once

#ifdef __CUDACC__
#define MM_HD __host__ __device__ __forceinline__
#else
#define MM_HD inline
#endif

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace spai_mm {

// ---- per-line rules (host and device) ----

// Outcome of one data line; negative codes are errors, numbered in the order they are checked.
enum LineCode : int {
    kLineData = 0,
    kLineSkip = 1,
    kLineTooFewFields = -1, // "Malformed coordinate entry"
    kLineExtraField = -2,   // "Extra field in Matrix Market line"
    kLineIndexToken = -3,   // "Expected a nonnegative integer dimension/index"
    kLineIndexTooBig = -4,  // "Dimension/index exceeds size_t"
    kLineIndexRange = -5,   // "Matrix Market index outside one-based dimensions"
    kLineIntegerField = -6  // "Integer field requires integer value tokens"
};

inline const char *line_message(int code) {
    switch (code) {
    case kLineTooFewFields: return "Malformed coordinate entry";
    case kLineExtraField: return "Extra field in Matrix Market line";
    case kLineIndexToken: return "Expected a nonnegative integer dimension/index";
    case kLineIndexTooBig: return "Dimension/index exceeds size_t";
    case kLineIndexRange: return "Matrix Market index outside one-based dimensions";
    default: return "Integer field requires integer value tokens";
    }
}

// Field separators: the C locale's white space (what formatted stream extraction skips).
MM_HD bool is_field_space(unsigned char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// A line is skipped when it holds nothing but spaces, tabs and carriage returns, or when its
// first other character is '%'. (Only those three count as blank here, unlike the separators.)
MM_HD bool line_is_skipped(const unsigned char *s, long long len) {
    for (long long i = 0; i < len; ++i) {
        const unsigned char c = s[i];
        if (c != ' ' && c != '\t' && c != '\r')
            return c == '%';
    }
    return true;
}

// Fields of a line as [begin, end) offsets. Stops after `limit` fields; the return value is the
// number found, so limit + 1 tells a caller that wants `limit` fields that there are more.
MM_HD int split_fields(const unsigned char *s, long long len, long long *begin, long long *end, int limit) {
    int count = 0;
    long long p = 0;
    while (count < limit) {
        while (p < len && is_field_space(s[p]))
            ++p;
        if (p >= len)
            break;
        begin[count] = p;
        while (p < len && !is_field_space(s[p]))
            ++p;
        end[count++] = p;
    }
    return count;
}

// Unsigned decimal token of digits only; values that do not fit 64 bits are an error.
MM_HD int parse_index_token(const unsigned char *s, long long len, unsigned long long &value) {
    value = 0;
    if (len <= 0)
        return kLineIndexToken;
    for (long long i = 0; i < len; ++i)
        if (s[i] < '0' || s[i] > '9')
            return kLineIndexToken;
    for (long long i = 0; i < len; ++i) {
        const unsigned long long digit = static_cast<unsigned long long>(s[i] - '0');
        if (value > (~0ull - digit) / 10)
            return kLineIndexTooBig;
        value = value * 10 + digit;
    }
    return kLineData;
}

// The integer field's extra condition on a value token: only signs and digits.
MM_HD bool integer_token(const unsigned char *s, long long len) {
    for (long long i = 0; i < len; ++i)
        if (!(s[i] == '+' || s[i] == '-' || (s[i] >= '0' && s[i] <= '9')))
            return false;
    return true;
}

// One line of the data section: skipped, or "row col value" checked up to the value token,
// whose [vb, ve) range is returned for the caller's conversion (which applies its own checks
// and then the integer-field rule).
MM_HD int classify_data_line(const unsigned char *s, long long len, unsigned long long rows,
                             unsigned long long cols, unsigned long long &row, unsigned long long &col,
                             long long &vb, long long &ve) {
    if (line_is_skipped(s, len))
        return kLineSkip;
    long long b[4], e[4];
    const int nf = split_fields(s, len, b, e, 4);
    if (nf < 3)
        return kLineTooFewFields;
    if (nf > 3)
        return kLineExtraField;
    int code = parse_index_token(s + b[0], e[0] - b[0], row);
    if (code == kLineData)
        code = parse_index_token(s + b[1], e[1] - b[1], col);
    if (code != kLineData)
        return code;
    if (row == 0 || col == 0 || row > rows || col > cols)
        return kLineIndexRange;
    vb = b[2];
    ve = e[2];
    return kLineData;
}

// ---- host side ----

struct HostCsr {
    uint64_t rows = 0, cols = 0;
    std::vector<int64_t> ptr, idx;
    std::vector<double> val;
};

struct Header {
    uint64_t rows = 0, cols = 0, count = 0;
    bool symmetric = false, integer_field = false;
};

// Line cursor over a memory buffer: lines end at '\n' (not included); a last line without a
// newline still counts, an empty remainder after the final newline does not.
class LineCursor {
  public:
    LineCursor(const char *data, size_t size) : p_(data), n_(size) {}
    bool next(const unsigned char *&s, long long &len) {
        if (pos_ >= n_)
            return false;
        const void *nl = std::memchr(p_ + pos_, '\n', n_ - pos_);
        const size_t end = nl ? static_cast<size_t>(static_cast<const char *>(nl) - p_) : n_;
        s = reinterpret_cast<const unsigned char *>(p_ + pos_);
        len = static_cast<long long>(end - pos_);
        pos_ = nl ? end + 1 : n_;
        return true;
    }
    // Next line that is not skipped (blank or comment).
    bool next_data(const unsigned char *&s, long long &len) {
        while (next(s, len))
            if (!line_is_skipped(s, len))
                return true;
        return false;
    }
    size_t position() const {
        return pos_;
    }

  private:
    const char *p_;
    size_t n_;
    size_t pos_ = 0;
};

inline std::string field_text(const unsigned char *s, long long b, long long e) {
    return std::string(reinterpret_cast<const char *>(s + b), static_cast<size_t>(e - b));
}

inline uint64_t header_index(const std::string &t) {
    unsigned long long v = 0;
    const int code = parse_index_token(reinterpret_cast<const unsigned char *>(t.data()),
                                       static_cast<long long>(t.size()), v);
    if (code != kLineData)
        throw std::runtime_error(line_message(code));
    return v;
}

// Banner and size line; on return the cursor stands at the first line after the size line.
inline Header read_header(LineCursor &cur) {
    const unsigned char *s = nullptr;
    long long len = 0;
    if (!cur.next(s, len))
        throw std::runtime_error("Missing Matrix Market banner");
    long long b[6], e[6];
    const int nb = split_fields(s, len, b, e, 6);
    if (nb < 5)
        throw std::runtime_error("Malformed Matrix Market banner");
    if (nb > 5)
        throw std::runtime_error("Extra field in Matrix Market line");
    const std::string magic = field_text(s, b[0], e[0]), object = field_text(s, b[1], e[1]),
                      format = field_text(s, b[2], e[2]), field = field_text(s, b[3], e[3]),
                      symmetry = field_text(s, b[4], e[4]);
    const bool field_ok = field == "real" || field == "integer";
    const bool symmetry_ok = symmetry == "general" || symmetry == "symmetric";
    if (magic != "%%MatrixMarket" || object != "matrix" || format != "coordinate" || !field_ok || !symmetry_ok)
        throw std::runtime_error("Unsupported Matrix Market format");
    Header h;
    h.symmetric = symmetry == "symmetric";
    h.integer_field = field == "integer";
    if (!cur.next_data(s, len))
        throw std::runtime_error("Missing matrix dimensions");
    const int nd = split_fields(s, len, b, e, 4);
    if (nd < 3)
        throw std::runtime_error("Malformed matrix dimensions");
    if (nd > 3)
        throw std::runtime_error("Extra field in Matrix Market line");
    h.rows = header_index(field_text(s, b[0], e[0]));
    h.cols = header_index(field_text(s, b[1], e[1]));
    h.count = header_index(field_text(s, b[2], e[2]));
    if (h.rows == 0 || h.cols == 0)
        throw std::runtime_error("Matrix dimensions must be positive");
    if (h.symmetric && h.rows != h.cols)
        throw std::runtime_error("Symmetric matrix must be square");
    return h;
}

// Value token with the C library's correctly rounded strtod: no conversion or a range error
// (overflow, or a nonzero value that rounds into the subnormal range or to zero) is "Invalid
// coordinate value"; unconsumed characters or a non-finite result (inf, nan spellings) is
// "Coordinate value must be finite and numeric"; then the integer field's character rule.
inline double host_value(const std::string &token, bool integer_field) {
    const char *c = token.c_str(); // a NUL inside the token ends the conversion early
    char *stop = nullptr;
    errno = 0;
    const double v = std::strtod(c, &stop);
    if (stop == c || errno == ERANGE)
        throw std::runtime_error("Invalid coordinate value");
    if (static_cast<size_t>(stop - c) != token.size() || !std::isfinite(v))
        throw std::runtime_error("Coordinate value must be finite and numeric");
    if (integer_field && !integer_token(reinterpret_cast<const unsigned char *>(token.data()),
                                        static_cast<long long>(token.size())))
        throw std::runtime_error("Integer field requires integer value tokens");
    return v;
}

// Canonical CSR from entries in file order (mirrors already placed after their entry): a
// counting pass buckets entries by row keeping file order, each row's bucket is ordered by column
// with a stable merge sort (equal columns keep file order), and each run of equal columns is
// added left to right; a run whose sum is zero leaves no entry.
inline HostCsr assemble(uint64_t rows, uint64_t cols, const std::vector<uint64_t> &erow,
                        const std::vector<uint64_t> &ecol, const std::vector<double> &evalue) {
    const size_t m = erow.size();
    std::vector<size_t> start(rows + 1, 0);
    for (size_t i = 0; i < m; ++i)
        ++start[erow[i] + 1];
    for (uint64_t r = 0; r < rows; ++r)
        start[r + 1] += start[r];
    std::vector<size_t> order(m), fill(start.begin(), start.end() - 1), tmp;
    for (size_t i = 0; i < m; ++i)
        order[fill[erow[i]]++] = i;
    HostCsr out;
    out.rows = rows;
    out.cols = cols;
    out.ptr.assign(rows + 1, 0);
    for (uint64_t r = 0; r < rows; ++r) {
        size_t *row = order.data() + start[r];
        const size_t len = start[r + 1] - start[r];
        // bottom-up stable merge sort of the row's entries by column
        tmp.resize(len);
        for (size_t width = 1; width < len; width *= 2) {
            for (size_t lo = 0; lo < len; lo += 2 * width) {
                const size_t mid = std::min(lo + width, len), hi = std::min(lo + 2 * width, len);
                size_t a = lo, b = mid, w = lo;
                while (a < mid && b < hi)
                    tmp[w++] = ecol[row[b]] < ecol[row[a]] ? row[b++] : row[a++];
                while (a < mid)
                    tmp[w++] = row[a++];
                while (b < hi)
                    tmp[w++] = row[b++];
            }
            std::copy(tmp.begin(), tmp.begin() + static_cast<long>(len), row);
        }
        for (size_t t = 0; t < len;) {
            const uint64_t c = ecol[row[t]];
            double sum = evalue[row[t]];
            for (++t; t < len && ecol[row[t]] == c; ++t) {
                sum += evalue[row[t]];
                if (!std::isfinite(sum))
                    throw std::invalid_argument("Duplicate sum is nonfinite");
            }
            if (sum != 0.0) {
                out.idx.push_back(static_cast<int64_t>(c));
                out.val.push_back(sum);
            }
        }
        out.ptr[r + 1] = static_cast<int64_t>(out.idx.size());
    }
    return out;
}

// The whole reader on a memory buffer holding the file.
inline HostCsr read_buffer(const char *data, size_t size) {
    LineCursor cur(data, size);
    const Header h = read_header(cur);
    std::vector<uint64_t> erow, ecol;
    std::vector<double> evalue;
    const size_t reserve = h.count < (1ull << 26) ? static_cast<size_t>(h.count) : 0;
    erow.reserve(reserve);
    ecol.reserve(reserve);
    evalue.reserve(reserve);
    const unsigned char *s = nullptr;
    long long len = 0;
    for (uint64_t k = 0; k < h.count; ++k) {
        if (!cur.next_data(s, len))
            throw std::runtime_error("Truncated coordinate data");
        unsigned long long r = 0, c = 0;
        long long vb = 0, ve = 0;
        const int code = classify_data_line(s, len, h.rows, h.cols, r, c, vb, ve);
        if (code != kLineData)
            throw std::runtime_error(line_message(code));
        const double v = host_value(field_text(s, vb, ve), h.integer_field);
        erow.push_back(r - 1);
        ecol.push_back(c - 1);
        evalue.push_back(v);
        if (h.symmetric && r != c) {
            erow.push_back(c - 1);
            ecol.push_back(r - 1);
            evalue.push_back(v);
        }
    }
    if (cur.next_data(s, len))
        throw std::runtime_error("Trailing coordinate data");
    return assemble(h.rows, h.cols, erow, ecol, evalue);
}

} // namespace spai_mm
