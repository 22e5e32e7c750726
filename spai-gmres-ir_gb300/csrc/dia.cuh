// Diagonal (DIA) companion of a device CSR matrix for the Krylov SpMVs of stencil-like profiles.
//
// Stencil matrices and their SPAI have few distinct column offsets (col - row): 7 for the 3-D
// 7-point operator, about 19 for its SPAI at epsilon 0.3. Storing each occupied diagonal as a
// dense length-n array drops the column indices (4 bytes per entry, a third to a half of a CSR or
// sliced-ELLPACK SpMV's traffic) and makes every load contiguous across a warp: thread `row`
// reads val[d][row] and x[row + off[d]] for each diagonal d. A per-row bit mask marks the entries
// that exist; absent positions are never multiplied, so non-finite x values cannot leak through
// 0 * inf, and each row is summed in ascending offset order, which is the CSR column order: the
// result is bit-identical to the CSR and sliced-ELLPACK kernels. Used only when the matrix has at
// most kDiaMax offsets and the diagonal arrays move fewer bytes than the sliced layout; the solve
// engine then times both and keeps the faster (tuned_op).
#pragma once
#include "common.cuh"
#include "spai_internal.hpp"

#include <algorithm>
#include <climits>
#include <vector>

namespace spai {

constexpr int kDiaMax = 32;
constexpr int kDiaTable = 2048; // open-addressing set of offsets while they are counted

template <class T> struct DeviceDia {
    int n = 0, ndiag = 0;
    int off[kDiaMax] = {};      // ascending offsets col - row (kernel parameter space)
    T *val = nullptr;           // [ndiag][n]; val[d * n + row]
    unsigned *mask = nullptr;   // [n]: bit d set when row has an entry on diagonal d
    bool ok() const {
        return ndiag > 0;
    }
};

inline namespace dia_detail {

// Distinct offsets into a hash set (INT_MIN = empty). Entries repeat the same few offsets, so a
// plain read finds the slot filled almost always and the compare-and-swap runs once per offset.
__global__ void dia_offsets_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci, int *table,
                                   int *distinct) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        for (int t = rp[row]; t < rp[row + 1]; ++t) {
            const int off = ci[t] - row;
            unsigned h = (static_cast<unsigned>(off) * 2654435761u) & (kDiaTable - 1);
            for (int probe = 0; probe < kDiaTable; ++probe) {
                const int cur = table[h];
                if (cur == off)
                    break;
                if (cur == INT_MIN) {
                    const int prev = atomicCAS(&table[h], INT_MIN, off);
                    if (prev == INT_MIN) {
                        atomicAdd(distinct, 1);
                        break;
                    }
                    if (prev == off)
                        break;
                }
                h = (h + 1) & (kDiaTable - 1);
            }
        }
    }
}

template <class T>
__global__ void dia_fill_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                const T *__restrict__ v, DeviceDia<T> m) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
        unsigned mk = 0;
        for (int t = rp[row]; t < rp[row + 1]; ++t) {
            const int off = ci[t] - row;
            int lo = 0, hi = m.ndiag - 1;
            while (lo < hi) { // offsets ascending; every entry's offset is present
                const int mid = (lo + hi) >> 1;
                if (m.off[mid] < off)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            m.val[static_cast<long long>(lo) * n + row] = v[t];
            mk |= 1u << lo;
        }
        m.mask[row] = mk;
    }
}

} // namespace dia_detail

// Diagonal companion of m in `arena`, or an empty one (ok() false) when m has more than kDiaMax
// offsets or its diagonals would store more than max_bytes. Stream-ordered, with one host read
// of the offset table.
template <class T>
DeviceDia<T> build_dia(DeviceArena &arena, const DeviceCsr<T> &m, int sms, cudaStream_t st, double max_bytes) {
    DeviceDia<T> d;
    if (m.n <= 0 || m.nnz <= 0)
        return d;
    int *table = arena.alloc<int>(kDiaTable + 1);
    std::vector<int> init(kDiaTable + 1, INT_MIN);
    init[kDiaTable] = 0;
    SPAI_CUDA(cudaMemcpyAsync(table, init.data(), sizeof(int) * (kDiaTable + 1), cudaMemcpyHostToDevice, st));
    dia_offsets_kernel<<<grid_for(m.n, 256, sms * 8), 256, 0, st>>>(m.n, m.rp, m.ci, table, table + kDiaTable);
    SPAI_LAUNCH("dia_offsets_kernel");
    std::vector<int> h(kDiaTable + 1);
    SPAI_CUDA(cudaMemcpyAsync(h.data(), table, sizeof(int) * (kDiaTable + 1), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    const int distinct = h[kDiaTable];
    if (distinct <= 0 || distinct > kDiaMax)
        return d;
    const double bytes = static_cast<double>(distinct) * m.n * sizeof(T) + 4.0 * m.n;
    if (bytes > max_bytes)
        return d;
    std::vector<int> offs;
    for (int i = 0; i < kDiaTable; ++i)
        if (h[i] != INT_MIN)
            offs.push_back(h[i]);
    std::sort(offs.begin(), offs.end());
    d.n = m.n;
    d.ndiag = static_cast<int>(offs.size());
    for (int i = 0; i < d.ndiag; ++i)
        d.off[i] = offs[i];
    d.val = arena.alloc<T>(static_cast<size_t>(d.ndiag) * m.n);
    d.mask = arena.alloc<unsigned>(m.n);
    SPAI_CUDA(cudaMemsetAsync(d.val, 0, sizeof(T) * static_cast<size_t>(d.ndiag) * m.n, st));
    dia_fill_kernel<T><<<grid_for(m.n, 256, sms * 8), 256, 0, st>>>(m.n, m.rp, m.ci, m.val, d);
    SPAI_LAUNCH("dia_fill_kernel");
    return d;
}

// y[row] = scale * sum_d val[d][row] x(row + off[d]) over the row's present diagonals, in
// ascending offset order; one thread per row. MAXD >= ndiag bounds a fully unrolled loop, so a
// row's value and x loads are all issued before its sum (every load independent of the others).
template <int MAXD, class T, class XF>
__device__ __forceinline__ void dia_rows(const DeviceDia<T> &m, XF xget, T scale, T *__restrict__ y) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < m.n; row += gridDim.x * blockDim.x) {
        const unsigned mk = __ldg(m.mask + row);
        T v[MAXD], x[MAXD];
#pragma unroll
        for (int d = 0; d < MAXD; ++d) {
            const bool on = d < m.ndiag && ((mk >> d) & 1u);
            v[d] = on ? __ldg(m.val + static_cast<long long>(d) * m.n + row) : T(0);
            x[d] = on ? xget(row + m.off[d]) : T(0);
        }
        T acc = 0;
#pragma unroll
        for (int d = 0; d < MAXD; ++d)
            if (d < m.ndiag && ((mk >> d) & 1u))
                acc += v[d] * x[d];
        y[row] = acc * scale;
    }
}

} // namespace spai
