// Matrix Market reader on the device (spai_mm_read): the reference's read_matrix_market and
// CsrMatrix::from_entries (src/cpu.cpp:49-161) with the same accepted format, checks, error
// precedence and results as the host reader in mm_text.hpp, which it replaces for large files.
// Both readers apply the same per-line rules (mm_text.hpp: skipped lines, field splitting, index
// tokens, the data-line checks): the kernel below calls them once per line.
//
// Host: read the file, parse the banner and the size line (a few bytes), upload the data section.
// Device: newline positions (one select pass), one thread per line classifies it (blank, comment,
// data) and parses "row col value"; a scan numbers the data lines and places each entry and its
// symmetric mirror; a stable radix sort by (row, col) keeps input order among duplicates, which
// one thread per run sums in that order (the reference's summation order); exact zero sums are
// dropped and the rows counted into CSR offsets.
//
// Values: a plain decimal token with at most 19 significant digits becomes w * 10^q. If w fits
// 53 bits and |q| <= 22 the quotient/product of two exact doubles is the correctly rounded value
// (Clinger's fast path). Otherwise w times a double-double 10^q (table built once by exact-ish
// double-double arithmetic, relative error below 2^-95) gives z = zh + zl, and zh is accepted
// when |zl| plus the error bound stays below the distance to the nearer rounding midpoint; the
// rest (more digits, hexadecimal or special tokens, near-midpoint values, results outside the
// normal range, and every token that std::stod would reject) is converted on the host by the C
// library's correctly rounded strtod with the host reader's checks. Either way the value is the
// same bits as the host reader's.
#include "common.cuh"
#include "mm_text.hpp"
#include "spai_internal.hpp"
#include "spai_ir.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

struct spai_mm_matrix_s {
    int64_t rows = 0, cols = 0, host_converted = 0;
    std::vector<int64_t> ptr, idx;
    std::vector<double> val;
};

namespace spai {
inline namespace mm_detail {

constexpr int kQmin = -350, kQmax = 310;
struct Pow10 {
    double hi, lo; // (hi + lo) * 2^e = 10^q, hi in [1, 2)
    int e;
};

// Line statuses: the shared per-line codes (negative values are errors in check order).
using spai_mm::kLineData;
using spai_mm::kLineSkip;
using spai_mm::kLineIntegerField;

inline const char *status_message(int s) {
    return spai_mm::line_message(s);
}

// ---- double-double helpers (host table construction) ----
void dd_two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}
void dd_norm(Pow10 &p) {
    double s, e;
    dd_two_sum(p.hi, p.lo, s, e);
    p.hi = s;
    p.lo = e;
    while (p.hi >= 2.0) {
        p.hi *= 0.5;
        p.lo *= 0.5;
        ++p.e;
    }
    while (p.hi < 1.0) {
        p.hi *= 2.0;
        p.lo *= 2.0;
        --p.e;
    }
}
Pow10 dd_times10(Pow10 p) {
    const double h = p.hi * 10.0, he = std::fma(p.hi, 10.0, -h);
    const double l = p.lo * 10.0;
    Pow10 r{h, he + l, p.e};
    dd_norm(r);
    return r;
}
Pow10 dd_div10(Pow10 p) {
    const double q1 = p.hi / 10.0;
    const double m = q1 * 10.0, me = std::fma(q1, 10.0, -m);
    const double rem = ((p.hi - m) - me) + p.lo; // exact remainder up to the lo term's rounding
    const double q2 = rem / 10.0;
    Pow10 r{q1, q2, p.e};
    dd_norm(r);
    return r;
}
const std::vector<Pow10> &pow10_table() {
    static std::vector<Pow10> t;
    static std::once_flag once;
    std::call_once(once, [] {
        t.assign(kQmax - kQmin + 1, Pow10{});
        Pow10 one{1.0, 0.0, 0};
        t[-kQmin] = one;
        Pow10 p = one;
        for (int q = 1; q <= kQmax; ++q)
            t[q - kQmin] = p = dd_times10(p);
        p = one;
        for (int q = -1; q >= kQmin; --q)
            t[q - kQmin] = p = dd_div10(p);
    });
    return t;
}

// ---- device parse ----
// Decimal value token -> certified correctly rounded double, or false (host converts it).
__device__ bool parse_value(const unsigned char *s, int len, const Pow10 *tab, double &out) {
    int i = 0;
    bool neg = false;
    if (i < len && (s[i] == '+' || s[i] == '-')) {
        neg = s[i] == '-';
        ++i;
    }
    unsigned long long w = 0;
    int sig = 0, exp10 = 0, digits = 0;
    bool seen_point = false;
    for (; i < len; ++i) {
        const unsigned char c = s[i];
        if (c >= '0' && c <= '9') {
            ++digits;
            if (w == 0 && c == '0') {
                if (seen_point)
                    --exp10; // leading zeros after the point
                continue;
            }
            if (sig >= 19)
                return false; // more significant digits than a 64-bit significand holds
            w = w * 10 + (c - '0');
            ++sig;
            if (seen_point)
                --exp10;
        } else if (c == '.' && !seen_point) {
            seen_point = true;
        } else {
            break;
        }
    }
    if (digits == 0)
        return false;
    if (i < len) {
        if (s[i] != 'e' && s[i] != 'E')
            return false;
        ++i;
        bool eneg = false;
        if (i < len && (s[i] == '+' || s[i] == '-')) {
            eneg = s[i] == '-';
            ++i;
        }
        if (i >= len)
            return false;
        int e = 0;
        for (; i < len; ++i) {
            if (s[i] < '0' || s[i] > '9')
                return false;
            if (e < 100000)
                e = e * 10 + (s[i] - '0');
        }
        exp10 += eneg ? -e : e;
    }
    if (w == 0) {
        out = neg ? -0.0 : 0.0;
        return true;
    }
    double v;
    if (w <= (1ull << 53) && exp10 >= -22 && exp10 <= 22) {
        const Pow10 &t = tab[(exp10 < 0 ? -exp10 : exp10) - kQmin];
        const double pw = ldexp(t.hi, t.e); // 10^|q| <= 10^22: exact (lo = 0), exact scaling
        v = exp10 < 0 ? static_cast<double>(w) / pw : static_cast<double>(w) * pw; // both operands exact
    } else {
        if (exp10 < kQmin + 1 || exp10 > kQmax - 1)
            return false;
        const Pow10 p = tab[exp10 - kQmin];
        // w as an exact double-double, times p
        const double wh = static_cast<double>(w);
        const double wl = static_cast<double>(static_cast<long long>(w - static_cast<unsigned long long>(wh)));
        const double ph = wh * p.hi, pe = fma(wh, p.hi, -ph);
        const double lo = pe + (wh * p.lo + wl * p.hi);
        const double zh = ph + lo;
        const double zl = lo - (zh - ph);
        // distance from zh to the nearer rounding midpoint
        const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(zh));
        const double ulp = __longlong_as_double(static_cast<long long>((bits & 0x7ff0000000000000ull) - (52ull << 52)));
        const double half = (bits & 0x000fffffffffffffull) == 0 ? ulp * 0.25 : ulp * 0.5;
        if (!(fabs(zl) + fabs(zh) * 0x1p-90 < half))
            return false;
        v = ldexp(zh, p.e);
    }
    if (!(fabs(v) >= 2.2250738585072014e-308) || !isfinite(v))
        return false; // underflow or overflow: std::stod's range error
    out = neg ? -v : v;
    return true;
}

struct MmArgs {
    const unsigned char *buf;
    long long size;
    const long long *nl; // newline positions
    long long nlines;
    unsigned long long rows, cols;
    int integer_field, symmetric;
    const Pow10 *tab;
    int *status;
    int *fallback;
    unsigned long long *row, *col;
    double *val;
};

__global__ void __launch_bounds__(256) mm_lines_kernel(MmArgs a) {
    for (long long ln = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; ln < a.nlines;
         ln += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long b = ln == 0 ? 0 : a.nl[ln - 1] + 1;
        const long long e = ln < a.nlines - 1 || (a.nlines > 0 && a.nl[a.nlines - 1] == a.size - 1 && ln == a.nlines - 1)
                                ? a.nl[ln]
                                : a.size;
        const unsigned char *s = a.buf + b;
        const long long len = e - b;
        int fb = 0;
        unsigned long long r = 0, c = 0;
        double v = 0;
        long long vb = 0, ve = 0;
        int st = spai_mm::classify_data_line(s, len, a.rows, a.cols, r, c, vb, ve);
        if (st == kLineData) {
            if (!parse_value(s + vb, static_cast<int>(ve - vb), a.tab, v))
                fb = 1; // the host converts and checks this value token
            else if (a.integer_field && !spai_mm::integer_token(s + vb, ve - vb))
                st = kLineIntegerField;
        }
        a.status[ln] = st;
        a.fallback[ln] = fb;
        a.row[ln] = r;
        a.col[ln] = c;
        a.val[ln] = v;
    }
}

struct IsNewline {
    const unsigned char *buf;
    __device__ bool operator()(long long i) const {
        return buf[i] == '\n';
    }
};

// Entry placement: data line d (d < count) -> position d + (mirrored data lines before d).
__global__ void mm_place_kernel(long long nlines, long long count, const int *status, const long long *dataidx,
                                const long long *mirbefore, const unsigned long long *row,
                                const unsigned long long *col, const double *val, int symmetric,
                                unsigned long long cols, unsigned long long *keys, double *vals) {
    for (long long ln = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; ln < nlines;
         ln += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (status[ln] != kLineData)
            continue;
        const long long d = dataidx[ln];
        if (d >= count)
            continue;
        const long long pos = d + mirbefore[ln];
        const unsigned long long r = row[ln] - 1, c = col[ln] - 1;
        keys[pos] = r * cols + c;
        vals[pos] = val[ln];
        if (symmetric && r != c) {
            keys[pos + 1] = c * cols + r;
            vals[pos + 1] = val[ln];
        }
    }
}

__global__ void mm_flags_kernel(long long nlines, const int *status, const unsigned long long *row,
                                const unsigned long long *col, int symmetric, long long *isdata, long long *ismir) {
    for (long long ln = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; ln < nlines;
         ln += static_cast<long long>(gridDim.x) * blockDim.x) {
        const bool data = status[ln] != kLineSkip;
        isdata[ln] = data ? 1 : 0;
        ismir[ln] = data && status[ln] == kLineData && symmetric && row[ln] != col[ln] ? 1 : 0;
    }
}

// First error among the first `count` data lines (line order), and the host-converted lines.
__global__ void mm_scan_errors_kernel(long long nlines, long long count, const int *status, const int *fallback,
                                      const long long *dataidx, unsigned long long *first_err,
                                      long long *fb_lines, unsigned long long *fb_count) {
    for (long long ln = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; ln < nlines;
         ln += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (status[ln] == kLineSkip || dataidx[ln] >= count)
            continue;
        if (status[ln] < 0)
            atomicMin(first_err, static_cast<unsigned long long>(ln));
        else if (fallback[ln])
            fb_lines[atomicAdd(fb_count, 1ull)] = ln;
    }
}

__global__ void mm_set_values_kernel(long long m, const long long *lines, const double *values, double *val) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < m;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        val[lines[i]] = values[i];
}

// Duplicate runs of the sorted keys summed in input order; keep[i] = 1 for a run start with a
// nonzero sum; bad = first run whose running sum became non-finite.
__global__ void mm_runs_kernel(long long ne, const unsigned long long *keys, const double *vals, double *sums,
                               long long *keep, unsigned long long *bad) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < ne;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        keep[i] = 0;
        if (i > 0 && keys[i - 1] == keys[i])
            continue;
        double s = vals[i];
        for (long long j = i + 1; j < ne && keys[j] == keys[i]; ++j) {
            s += vals[j];
            if (!isfinite(s)) {
                atomicMin(bad, static_cast<unsigned long long>(i));
                break;
            }
        }
        sums[i] = s;
        keep[i] = s != 0.0 ? 1 : 0;
    }
}

__global__ void mm_compact_kernel(long long ne, const unsigned long long *keys, const double *sums,
                                  const long long *keep, const long long *outpos, unsigned long long cols,
                                  long long *idx, double *val, long long *rowcount) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < ne;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (!keep[i])
            continue;
        const long long o = outpos[i];
        idx[o] = static_cast<long long>(keys[i] % cols);
        val[o] = sums[i];
        atomicAdd(reinterpret_cast<unsigned long long *>(rowcount + keys[i] / cols + 1), 1ull);
    }
}

} // namespace mm_detail
} // namespace spai

using namespace spai;

namespace {
template <class T> struct DevBuf {
    T *p = nullptr;
    explicit DevBuf(size_t n) {
        SPAI_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    }
    ~DevBuf() {
        if (p)
            cudaFree(p);
    }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
};

int mm_fail(int code, const std::string &msg) {
    return spai_api_fail(code, msg);
}
} // namespace

extern "C" int spai_mm_read(const char *path, int64_t device_min_lines, spai_mm_matrix **out) {
    if (!path || !out)
        return mm_fail(SPAI_ERR_ARGUMENT, "spai_mm_read: null argument");
    *out = nullptr;
    try {
        // ---- host: file, banner, size line ----
        std::FILE *f = std::fopen(path, "rb");
        if (!f)
            return mm_fail(SPAI_ERR_ARGUMENT, "Cannot open Matrix Market input");
        std::unique_ptr<std::FILE, int (*)(std::FILE *)> fg(f, std::fclose);
        std::fseek(f, 0, SEEK_END);
        const long long fsize = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        std::vector<unsigned char> hstore(static_cast<size_t>(std::max<long long>(fsize, 1)));
        unsigned char *hbuf = hstore.data(); // pageable: the host path needs no GPU at all
        if (fsize > 0 && std::fread(hbuf, 1, static_cast<size_t>(fsize), f) != static_cast<size_t>(fsize))
            return mm_fail(SPAI_ERR_FORMAT, "Cannot read Matrix Market input");
        spai_mm::LineCursor cursor(reinterpret_cast<const char *>(hbuf), static_cast<size_t>(std::max<long long>(fsize, 0)));
        const spai_mm::Header hdr = spai_mm::read_header(cursor); // runtime_error -> SPAI_ERR_FORMAT
        const long long pos = static_cast<long long>(cursor.position());
        const uint64_t rows = hdr.rows, cols = hdr.cols, count = hdr.count;
        const bool symmetric = hdr.symmetric, integer_field = hdr.integer_field;
        const long long dsize = fsize - pos; // data section
        const long long approx_lines = dsize / 8 + 1;
        if (approx_lines < device_min_lines || dsize > INT_MAX - 1 || rows >= (1ull << 31) || cols >= (1ull << 31) ||
            count >= (1ull << 31)) {
            // host parse by the same rules (small files; or beyond the device path's 32-bit sizes)
            spai_mm::HostCsr h = spai_mm::read_buffer(reinterpret_cast<const char *>(hbuf), static_cast<size_t>(fsize));
            auto m = std::make_unique<spai_mm_matrix_s>();
            m->rows = static_cast<int64_t>(h.rows);
            m->cols = static_cast<int64_t>(h.cols);
            m->ptr = std::move(h.ptr);
            m->idx = std::move(h.idx);
            m->val = std::move(h.val);
            *out = m.release();
            return SPAI_OK;
        }
        // ---- device: lines ----
        const std::vector<Pow10> &tab = pow10_table();
        DevBuf<Pow10> dtab(tab.size());
        SPAI_CUDA(cudaMemcpy(dtab.p, tab.data(), sizeof(Pow10) * tab.size(), cudaMemcpyHostToDevice));
        DevBuf<unsigned char> dbuf(static_cast<size_t>(dsize) + 1);
        if (dsize > 0)
            SPAI_CUDA(cudaMemcpy(dbuf.p, hbuf + pos, static_cast<size_t>(dsize), cudaMemcpyHostToDevice));
        int sms = 0, dev = 0;
        SPAI_CUDA(cudaGetDevice(&dev));
        SPAI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        DevBuf<long long> dnl(static_cast<size_t>(dsize) / 2 + 2);
        DevBuf<long long> dnsel(1);
        size_t tmp_bytes = 0;
        thrust::counting_iterator<long long> it(0);
        IsNewline pred{dbuf.p};
        SPAI_CUDA(cub::DeviceSelect::If(nullptr, tmp_bytes, it, dnl.p, dnsel.p, static_cast<int>(dsize), pred));
        DevBuf<unsigned char> tmp(tmp_bytes);
        SPAI_CUDA(cub::DeviceSelect::If(tmp.p, tmp_bytes, it, dnl.p, dnsel.p, static_cast<int>(dsize), pred));
        long long nnl = 0;
        SPAI_CUDA(cudaMemcpy(&nnl, dnsel.p, sizeof(long long), cudaMemcpyDeviceToHost));
        const bool tail = dsize > 0 && hbuf[fsize - 1] != '\n';
        const long long nlines = nnl + (tail ? 1 : 0);
        if (static_cast<unsigned long long>(nnl) > static_cast<size_t>(dsize) / 2 + 2)
            throw std::runtime_error("newline count exceeds its buffer");
        DevBuf<int> dstatus(nlines), dfb(nlines);
        DevBuf<unsigned long long> drow(nlines), dcol(nlines);
        DevBuf<double> dval(nlines);
        MmArgs a{dbuf.p, dsize, dnl.p, nlines, rows, cols, integer_field ? 1 : 0, symmetric ? 1 : 0, dtab.p,
                 dstatus.p, dfb.p, drow.p, dcol.p, dval.p};
        const unsigned gl = grid_for(std::max<long long>(nlines, 1), 256, sms * 8);
        if (nlines > 0) {
            mm_lines_kernel<<<gl, 256>>>(a);
            SPAI_LAUNCH("mm_lines_kernel");
        }
        // ---- number the data lines ----
        DevBuf<long long> disdata(nlines + 1), dismir(nlines + 1), ddataidx(nlines + 1), dmirb(nlines + 1);
        if (nlines > 0) {
            mm_flags_kernel<<<gl, 256>>>(nlines, dstatus.p, drow.p, dcol.p, symmetric ? 1 : 0, disdata.p, dismir.p);
            SPAI_LAUNCH("mm_flags_kernel");
            size_t sb = 0;
            SPAI_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb, disdata.p, ddataidx.p, nlines + 1));
            DevBuf<unsigned char> st(sb);
            SPAI_CUDA(cudaMemset(disdata.p + nlines, 0, sizeof(long long)));
            SPAI_CUDA(cudaMemset(dismir.p + nlines, 0, sizeof(long long)));
            SPAI_CUDA(cub::DeviceScan::ExclusiveSum(st.p, sb, disdata.p, ddataidx.p, nlines + 1));
            SPAI_CUDA(cub::DeviceScan::ExclusiveSum(st.p, sb, dismir.p, dmirb.p, nlines + 1));
        }
        long long ndata = 0;
        if (nlines > 0)
            SPAI_CUDA(cudaMemcpy(&ndata, ddataidx.p + nlines, sizeof(long long), cudaMemcpyDeviceToHost));
        // ---- errors (line order among the first `count` data lines) and host-converted values ----
        DevBuf<unsigned long long> dfirst(2);
        DevBuf<long long> dfbl(nlines);
        const unsigned long long big = ULLONG_MAX;
        SPAI_CUDA(cudaMemcpy(dfirst.p, &big, sizeof(big), cudaMemcpyHostToDevice));
        SPAI_CUDA(cudaMemset(dfirst.p + 1, 0, sizeof(unsigned long long)));
        if (nlines > 0) {
            mm_scan_errors_kernel<<<gl, 256>>>(nlines, static_cast<long long>(count), dstatus.p, dfb.p, ddataidx.p,
                                               dfirst.p, dfbl.p, dfirst.p + 1);
            SPAI_LAUNCH("mm_scan_errors_kernel");
        }
        unsigned long long hfirst[2];
        SPAI_CUDA(cudaMemcpy(hfirst, dfirst.p, sizeof(hfirst), cudaMemcpyDeviceToHost));
        std::vector<long long> fbl(hfirst[1]);
        if (!fbl.empty())
            SPAI_CUDA(cudaMemcpy(fbl.data(), dfbl.p, sizeof(long long) * fbl.size(), cudaMemcpyDeviceToHost));
        std::sort(fbl.begin(), fbl.end());
        std::vector<long long> hnl; // newline positions, copied once when the host converts tokens
        if (!fbl.empty()) {
            hnl.resize(static_cast<size_t>(nnl));
            if (nnl > 0)
                SPAI_CUDA(cudaMemcpy(hnl.data(), dnl.p, sizeof(long long) * nnl, cudaMemcpyDeviceToHost));
        }
        auto line_text = [&](long long ln) {
            const long long b = ln == 0 ? 0 : hnl[ln - 1] + 1;
            const long long e = ln < nnl ? hnl[ln] : dsize;
            return std::string(reinterpret_cast<const char *>(hbuf + pos + b), static_cast<size_t>(e - b));
        };
        // host conversion of the flagged value tokens, in line order, up to the device's first error
        std::vector<double> fbv;
        fbv.reserve(fbl.size());
        long long host_err_line = -1;
        std::string host_err;
        std::vector<long long> fb_lines_used;
        for (long long ln : fbl) {
            if (hfirst[0] != ULLONG_MAX && static_cast<unsigned long long>(ln) > hfirst[0])
                break;
            const std::string text = line_text(ln);
            const unsigned char *ls = reinterpret_cast<const unsigned char *>(text.data());
            long long fbeg[3], fend[3];
            spai_mm::split_fields(ls, static_cast<long long>(text.size()), fbeg, fend, 3);
            try {
                fbv.push_back(spai_mm::host_value(spai_mm::field_text(ls, fbeg[2], fend[2]), integer_field));
                fb_lines_used.push_back(ln);
            } catch (const std::runtime_error &e) {
                host_err_line = ln;
                host_err = e.what();
                break;
            }
        }
        if (hfirst[0] != ULLONG_MAX && (host_err_line < 0 || static_cast<unsigned long long>(host_err_line) > hfirst[0])) {
            int s = 0;
            SPAI_CUDA(cudaMemcpy(&s, dstatus.p + hfirst[0], sizeof(int), cudaMemcpyDeviceToHost));
            return mm_fail(SPAI_ERR_FORMAT, status_message(s));
        }
        if (host_err_line >= 0)
            return mm_fail(SPAI_ERR_FORMAT, host_err);
        if (static_cast<unsigned long long>(ndata) < count)
            return mm_fail(SPAI_ERR_FORMAT, "Truncated coordinate data");
        if (static_cast<unsigned long long>(ndata) > count)
            return mm_fail(SPAI_ERR_FORMAT, "Trailing coordinate data");
        if (!fb_lines_used.empty()) {
            DevBuf<long long> dl(fb_lines_used.size());
            DevBuf<double> dv(fbv.size());
            SPAI_CUDA(cudaMemcpy(dl.p, fb_lines_used.data(), sizeof(long long) * fb_lines_used.size(), cudaMemcpyHostToDevice));
            SPAI_CUDA(cudaMemcpy(dv.p, fbv.data(), sizeof(double) * fbv.size(), cudaMemcpyHostToDevice));
            mm_set_values_kernel<<<grid_for(static_cast<long long>(fbv.size()), 256, sms * 4), 256>>>(
                static_cast<long long>(fbv.size()), dl.p, dv.p, dval.p);
            SPAI_LAUNCH("mm_set_values_kernel");
        }
        // ---- entries, stable sort by (row, col), duplicate sums, zeros dropped ----
        long long nmir = 0;
        if (nlines > 0)
            SPAI_CUDA(cudaMemcpy(&nmir, dmirb.p + nlines, sizeof(long long), cudaMemcpyDeviceToHost));
        const long long ne = static_cast<long long>(count) + nmir;
        DevBuf<unsigned long long> dkeys(ne), dkeys2(ne);
        DevBuf<double> dvals(ne), dvals2(ne), dsums(ne);
        if (nlines > 0 && ne > 0) {
            mm_place_kernel<<<gl, 256>>>(nlines, static_cast<long long>(count), dstatus.p, ddataidx.p, dmirb.p, drow.p,
                                         dcol.p, dval.p, symmetric ? 1 : 0, cols, dkeys.p, dvals.p);
            SPAI_LAUNCH("mm_place_kernel");
        }
        int end_bit = 1;
        while (end_bit < 64 && (end_bit >= 63 || (1ull << end_bit) < rows * cols))
            ++end_bit;
        if (ne > 0) {
            size_t sb = 0;
            SPAI_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, sb, dkeys.p, dkeys2.p, dvals.p, dvals2.p,
                                                      static_cast<int>(ne), 0, end_bit));
            DevBuf<unsigned char> st(sb);
            SPAI_CUDA(cub::DeviceRadixSort::SortPairs(st.p, sb, dkeys.p, dkeys2.p, dvals.p, dvals2.p,
                                                      static_cast<int>(ne), 0, end_bit));
        }
        DevBuf<long long> dkeep(ne + 1), dout(ne + 1);
        DevBuf<unsigned long long> dbad(1);
        SPAI_CUDA(cudaMemcpy(dbad.p, &big, sizeof(big), cudaMemcpyHostToDevice));
        const unsigned ge = grid_for(std::max<long long>(ne, 1), 256, sms * 8);
        long long nout = 0;
        if (ne > 0) {
            mm_runs_kernel<<<ge, 256>>>(ne, dkeys2.p, dvals2.p, dsums.p, dkeep.p, dbad.p);
            SPAI_LAUNCH("mm_runs_kernel");
            unsigned long long hbad = 0;
            SPAI_CUDA(cudaMemcpy(&hbad, dbad.p, sizeof(hbad), cudaMemcpyDeviceToHost));
            if (hbad != ULLONG_MAX)
                return mm_fail(SPAI_ERR_ARGUMENT, "Duplicate sum is nonfinite");
            SPAI_CUDA(cudaMemset(dkeep.p + ne, 0, sizeof(long long)));
            size_t sb = 0;
            SPAI_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb, dkeep.p, dout.p, ne + 1));
            DevBuf<unsigned char> st(sb);
            SPAI_CUDA(cub::DeviceScan::ExclusiveSum(st.p, sb, dkeep.p, dout.p, ne + 1));
            SPAI_CUDA(cudaMemcpy(&nout, dout.p + ne, sizeof(long long), cudaMemcpyDeviceToHost));
        }
        DevBuf<long long> didx(nout), drc(rows + 1), dptr(rows + 1);
        DevBuf<double> dv2(nout);
        SPAI_CUDA(cudaMemset(drc.p, 0, sizeof(long long) * (rows + 1)));
        if (ne > 0) {
            mm_compact_kernel<<<ge, 256>>>(ne, dkeys2.p, dsums.p, dkeep.p, dout.p, cols, didx.p, dv2.p, drc.p);
            SPAI_LAUNCH("mm_compact_kernel");
        }
        size_t sb = 0;
        SPAI_CUDA(cub::DeviceScan::InclusiveSum(nullptr, sb, drc.p, dptr.p, rows + 1));
        DevBuf<unsigned char> st(sb);
        SPAI_CUDA(cub::DeviceScan::InclusiveSum(st.p, sb, drc.p, dptr.p, rows + 1));
        auto m = std::make_unique<spai_mm_matrix_s>();
        m->rows = static_cast<int64_t>(rows);
        m->cols = static_cast<int64_t>(cols);
        m->host_converted = static_cast<int64_t>(fbv.size());
        m->ptr.resize(rows + 1);
        m->idx.resize(static_cast<size_t>(nout));
        m->val.resize(static_cast<size_t>(nout));
        SPAI_CUDA(cudaMemcpy(m->ptr.data(), dptr.p, sizeof(int64_t) * (rows + 1), cudaMemcpyDeviceToHost));
        if (nout > 0) {
            SPAI_CUDA(cudaMemcpy(m->idx.data(), didx.p, sizeof(int64_t) * nout, cudaMemcpyDeviceToHost));
            SPAI_CUDA(cudaMemcpy(m->val.data(), dv2.p, sizeof(double) * nout, cudaMemcpyDeviceToHost));
        }
        *out = m.release();
        return SPAI_OK;
    } catch (const std::invalid_argument &e) {
        return mm_fail(SPAI_ERR_ARGUMENT, e.what());
    } catch (const spai::CudaError &e) {
        return mm_fail(SPAI_ERR_CUDA, e.what());
    } catch (const std::runtime_error &e) {
        return mm_fail(SPAI_ERR_FORMAT, e.what());
    } catch (const std::exception &e) {
        return mm_fail(SPAI_ERR_CUDA, e.what());
    }
}

extern "C" int spai_mm_csr(const spai_mm_matrix *m, spai_csr *csr, int64_t *cols, int64_t *host_converted_values) {
    if (!m || !csr)
        return mm_fail(SPAI_ERR_ARGUMENT, "spai_mm_csr: null argument");
    csr->n = m->rows;
    csr->nnz = static_cast<int64_t>(m->val.size());
    csr->row_offsets = m->ptr.data();
    csr->col_indices = m->idx.data();
    csr->values = m->val.data();
    if (cols)
        *cols = m->cols;
    if (host_converted_values)
        *host_converted_values = m->host_converted;
    return SPAI_OK;
}

extern "C" int spai_mm_free(spai_mm_matrix *m) {
    delete m;
    return SPAI_OK;
}
