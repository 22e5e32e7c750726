// Sliced ELLPACK companion of a device CSR matrix for the Krylov SpMVs.
//
// Rows are grouped in slices of 32 (one warp); slice s stores its rows' entries column-major,
// padded to the slice's longest row: entry p of row 32 s + r sits at off[s] + 32 p + r. A warp
// processes one slice with one thread per row, so for every position p the values, the column
// indices and (for stencil-like patterns, whose p-th entry is the same offset in every row) the
// gathered x are contiguous across the warp. Padding is never multiplied: each thread stops at
// its row's true length, so non-finite x values cannot leak into other rows through 0 * inf.
// Within a row the products are summed in CSR (column) order, as in the CSR kernels.
//
// Heavy-tailed row lengths (the irregular Zipf family: most rows short, a few up to 256 entries)
// would pad a slice holding one long row to that row's length and leave 31 threads idle while it
// finishes. For such profiles the slices are built over the rows ordered by length (SELL-C-sigma
// with sigma = n, Kreutzer et al., SIAM J. Sci. Comput. 36(5), 2014): perm[p] is the row at slice
// position p, rows of equal length share a slice, padding nearly vanishes and every thread of a
// warp has the same trip count. Each row is still summed by one thread in column order, so the
// result is bit-identical to the unsorted layout; only y's writes are permuted (scattered within
// L2, where the 4n-byte output vector stays resident).
#pragma once
#include "common.cuh"
#include "spai_internal.hpp"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

namespace spai {

template <class T> struct DeviceSell {
    int n = 0, nslices = 0;
    long long entries = 0;       // stored entries including padding
    long long *off = nullptr;    // [nslices + 1] first entry of each slice
    int *len = nullptr;          // [n] row lengths, by slice position
    int *perm = nullptr;         // [n] row at each slice position; nullptr = identity
    int *ci = nullptr;           // [entries]
    T *val = nullptr;            // [entries]
    bool sorted() const {
        return perm != nullptr;
    }
};

inline namespace sell_detail {

// Slice widths (max row length in the slice) into width[s + 1] (width[0] = 0 for the scan).
__global__ void sell_width_kernel(int n, const int *__restrict__ rp, const int *__restrict__ perm, long long *width,
                                  int *len) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int nsl = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsl; s += warps) {
        const int pos = s * 32 + lane;
        int l = 0;
        if (pos < n) {
            const int row = perm ? perm[pos] : pos;
            l = rp[row + 1] - rp[row];
            len[pos] = l;
        }
        for (int o = 16; o > 0; o >>= 1)
            l = max(l, __shfl_xor_sync(0xffffffffu, l, o));
        if (lane == 0)
            width[s + 1] = 32LL * l;
        if (s == 0 && lane == 0)
            width[0] = 0;
    }
}

// Row lengths as sort keys (descending sort by length keeps equal lengths in row order).
__global__ void sell_len_keys_kernel(int n, const int *__restrict__ rp, int *keys, int *rows) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        keys[row] = rp[row + 1] - rp[row];
        rows[row] = row;
    }
}

template <class T>
__global__ void sell_fill_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                 const T *__restrict__ val, const long long *__restrict__ off,
                                 const int *__restrict__ perm, int *sci, T *sval) {
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < n; pos += gridDim.x * blockDim.x) {
        const int row = perm ? perm[pos] : pos;
        const int s = pos >> 5, r = pos & 31;
        const long long base = off[s] + r;
        const long long width = (off[s + 1] - off[s]) >> 5;
        const int b = rp[row], e = rp[row + 1];
        for (long long p = 0; p < width; ++p) {
            const int t = b + static_cast<int>(p);
            sci[base + 32 * p] = t < e ? ci[t] : row; // padding: a valid index, never read
            sval[base + 32 * p] = t < e ? val[t] : T(0);
        }
    }
}

} // namespace sell_detail

// Build the sliced companion of m in `arena` (stream-ordered; one host read of the total size).
// order: 0 = natural row order, 1 = rows sorted by length, -1 = choose: sorted when the natural
// layout would store more than 5/4 of nnz (padding from uneven row lengths).
template <class T>
DeviceSell<T> build_sell(DeviceArena &arena, const DeviceCsr<T> &m, int sms, cudaStream_t st, int order = -1) {
    DeviceSell<T> s;
    s.n = m.n;
    s.nslices = (m.n + 31) / 32;
    s.off = arena.alloc<long long>(static_cast<size_t>(s.nslices) + 1);
    s.len = arena.alloc<int>(m.n);
    int *perm = order != 0 ? arena.alloc<int>(m.n) : nullptr;
    size_t tmp_bytes = 0;
    SPAI_CUDA(cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, s.off, s.off, s.nslices + 1, st));
    size_t sort_bytes = 0;
    if (order != 0)
        SPAI_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, sort_bytes, s.len, s.len, perm, perm, m.n, 0,
                                                            32, st));
    void *tmp = arena.alloc<unsigned char>(std::max(tmp_bytes, sort_bytes) + 16);
    int *keys = order != 0 ? arena.alloc<int>(m.n) : nullptr;
    int *rows = order != 0 ? arena.alloc<int>(m.n) : nullptr;
    auto widths = [&](const int *pm) {
        sell_width_kernel<<<grid_for(static_cast<long long>(s.nslices) * 32, 256, sms * 8), 256, 0, st>>>(
            m.n, m.rp, pm, s.off, s.len);
        SPAI_LAUNCH("sell_width_kernel");
        SPAI_CUDA(cub::DeviceScan::InclusiveSum(tmp, tmp_bytes, s.off, s.off, s.nslices + 1, st));
        SPAI_CUDA(cudaMemcpyAsync(&s.entries, s.off + s.nslices, sizeof(long long), cudaMemcpyDeviceToHost, st));
        SPAI_CUDA(cudaStreamSynchronize(st));
    };
    bool sorted = order == 1;
    if (!sorted) {
        widths(nullptr);
        sorted = order < 0 && s.entries * 4 > static_cast<long long>(m.nnz) * 5 + 4LL * 32 * s.nslices;
    }
    if (sorted) {
        sell_len_keys_kernel<<<grid_for(m.n, 256, sms * 8), 256, 0, st>>>(m.n, m.rp, keys, rows);
        SPAI_LAUNCH("sell_len_keys_kernel");
        SPAI_CUDA(cub::DeviceRadixSort::SortPairsDescending(tmp, sort_bytes, keys, s.len, rows, perm, m.n, 0, 32,
                                                            st));
        s.perm = perm;
        widths(perm);
    }
    s.ci = arena.alloc<int>(static_cast<size_t>(std::max<long long>(s.entries, 1)));
    s.val = arena.alloc<T>(static_cast<size_t>(std::max<long long>(s.entries, 1)));
    sell_fill_kernel<T><<<grid_for(m.n, 256, sms * 8), 256, 0, st>>>(m.n, m.rp, m.ci, m.val, s.off, s.perm, s.ci,
                                                                     s.val);
    SPAI_LAUNCH("sell_fill_kernel");
    return s;
}

// y[row] = scale * sum_p val * x(ci) over one slice per warp, one thread per row.
template <class T, class XF>
__device__ __forceinline__ void sell_rows(const DeviceSell<T> &m, XF xget, T scale, T *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < m.nslices; s += warps) {
        const int pos = s * 32 + lane;
        if (pos >= m.n)
            continue;
        const int row = m.perm ? __ldg(m.perm + pos) : pos;
        const long long base = m.off[s] + lane;
        const int l = m.len[pos];
        T acc = 0;
        int p = 0;
        // Four entries in flight per thread (indices and values first, then the gathers).
        for (; p + 4 <= l; p += 4) {
            int c[4];
            T v[4], x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                c[u] = __ldg(m.ci + base + 32LL * (p + u));
                v[u] = __ldg(m.val + base + 32LL * (p + u));
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                x[u] = xget(c[u]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                acc += v[u] * x[u];
        }
        for (; p < l; ++p)
            acc += __ldg(m.val + base + 32LL * p) * xget(__ldg(m.ci + base + 32LL * p));
        y[row] = acc * scale;
    }
}

} // namespace spai
