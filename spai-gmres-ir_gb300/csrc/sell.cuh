// Sliced ELLPACK companion of a device CSR matrix for the Krylov SpMVs.
//
// Rows are grouped in slices of 32 (one warp); slice s stores its rows' entries column-major,
// padded to the slice's longest row: entry p of row 32 s + r sits at off[s] + 32 p + r. A warp
// processes one slice with one thread per row, so for every position p the values, the column
// indices and (for stencil-like patterns, whose p-th entry is the same offset in every row) the
// gathered x are contiguous across the warp. Padding is never multiplied: each thread stops at
// its row's true length, so non-finite x values cannot leak into other rows through 0 * inf.
// Within a row the products are summed in CSR (column) order, as in the CSR kernels.
#pragma once
#include "common.cuh"
#include "spai_internal.hpp"

#include <cub/device/device_scan.cuh>

namespace spai {

template <class T> struct DeviceSell {
    int n = 0, nslices = 0;
    long long entries = 0;       // stored entries including padding
    long long *off = nullptr;    // [nslices + 1] first entry of each slice
    int *len = nullptr;          // [n] row lengths
    int *ci = nullptr;           // [entries]
    T *val = nullptr;            // [entries]
};

inline namespace sell_detail {

// Slice widths (max row length in the slice) into width[s + 1] (width[0] = 0 for the scan).
__global__ void sell_width_kernel(int n, const int *__restrict__ rp, long long *width, int *len) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int nsl = (n + 31) / 32;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nsl; s += warps) {
        const int row = s * 32 + lane;
        int l = 0;
        if (row < n) {
            l = rp[row + 1] - rp[row];
            len[row] = l;
        }
        for (int o = 16; o > 0; o >>= 1)
            l = max(l, __shfl_xor_sync(0xffffffffu, l, o));
        if (lane == 0)
            width[s + 1] = 32LL * l;
        if (s == 0 && lane == 0)
            width[0] = 0;
    }
}

template <class T>
__global__ void sell_fill_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                 const T *__restrict__ val, const long long *__restrict__ off, int *sci,
                                 T *sval) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        const int s = row >> 5, r = row & 31;
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
template <class T>
DeviceSell<T> build_sell(DeviceArena &arena, const DeviceCsr<T> &m, int sms, cudaStream_t st) {
    DeviceSell<T> s;
    s.n = m.n;
    s.nslices = (m.n + 31) / 32;
    s.off = arena.alloc<long long>(static_cast<size_t>(s.nslices) + 1);
    s.len = arena.alloc<int>(m.n);
    sell_width_kernel<<<grid_for(static_cast<long long>(s.nslices) * 32, 256, sms * 8), 256, 0, st>>>(m.n, m.rp, s.off,
                                                                                                    s.len);
    SPAI_LAUNCH("sell_width_kernel");
    size_t tmp_bytes = 0;
    SPAI_CUDA(cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, s.off, s.off, s.nslices + 1, st));
    void *tmp = arena.alloc<unsigned char>(tmp_bytes + 16);
    SPAI_CUDA(cub::DeviceScan::InclusiveSum(tmp, tmp_bytes, s.off, s.off, s.nslices + 1, st));
    SPAI_CUDA(cudaMemcpyAsync(&s.entries, s.off + s.nslices, sizeof(long long), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    s.ci = arena.alloc<int>(static_cast<size_t>(std::max<long long>(s.entries, 1)));
    s.val = arena.alloc<T>(static_cast<size_t>(std::max<long long>(s.entries, 1)));
    sell_fill_kernel<T><<<grid_for(m.n, 256, sms * 8), 256, 0, st>>>(m.n, m.rp, m.ci, m.val, s.off, s.ci, s.val);
    SPAI_LAUNCH("sell_fill_kernel");
    return s;
}

// y[row] = scale * sum_p val * x(ci) over one slice per warp, one thread per row.
template <class T, class XF>
__device__ __forceinline__ void sell_rows(const DeviceSell<T> &m, XF xget, T scale, T *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < m.nslices; s += warps) {
        const int row = s * 32 + lane;
        if (row >= m.n)
            continue;
        const long long base = m.off[s] + lane;
        const int l = m.len[row];
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
