// Adjoint support: device transposes of A and P (the same SPAI, no rebuild) and the sampled outer
// product that turns adjoint solutions into the gradient with respect to A's stored values.
#pragma once
#include "spai_internal.hpp"

#include <cub/device/device_radix_sort.cuh>

namespace spai {
inline namespace adjoint_detail {

__global__ void iota_kernel(int count, int *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[i] = i;
}

// row_of[e] = row of stored entry e.
__global__ void row_of_kernel(int n, const int *__restrict__ rp, int *row_of) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        for (int e = rp[r]; e < rp[r + 1]; ++e)
            row_of[e] = r;
}

// Row offsets of the transpose from the sorted column keys: rt[c] = first position whose key is
// >= c (every c in (key[p-1], key[p]] starts at p; columns past the last key start at nnz).
__global__ void transpose_offsets_kernel(int n, int nnz, const int *__restrict__ keys, int *rt) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= nnz; p += gridDim.x * blockDim.x) {
        const int prev = p == 0 ? -1 : keys[p - 1];
        const int cur = p == nnz ? n : keys[p];
        for (int c = prev + 1; c <= cur; ++c)
            rt[c] = p;
    }
}

__global__ void transpose_max_kernel(int n, const int *__restrict__ rt, int *max_len) {
    int m = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        m = max(m, rt[c + 1] - rt[c]);
    atomicMax(max_len, m);
}

// out[p] = val[perm[p]]: column indices (original rows) and values of the transpose.
template <class TV>
__global__ void gather_values_kernel(int nnz, const int *__restrict__ perm, const TV *__restrict__ val, TV *vt) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x)
        vt[p] = val[perm[p]];
}

// dLdA[e] = -sum_r lambda_r[i] x_r[j] for stored entry e = (i, j) of A, r = 0..nrhs-1 in order
// (vectors column-major, leading dimension n). One thread per row, entries in storage order.
__global__ void __launch_bounds__(256) sampled_outer_kernel(int n, int nrhs, const int *__restrict__ rp,
                                                            const int *__restrict__ ci,
                                                            const double *__restrict__ lambda,
                                                            const double *__restrict__ x, double *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int e = rp[i]; e < rp[i + 1]; ++e) {
            const long long j = ci[e];
            double acc = 0;
            for (int r = 0; r < nrhs; ++r) {
                const long long off = static_cast<long long>(r) * n;
                acc = fma(lambda[off + i], x[off + j], acc);
            }
            out[e] = -acc;
        }
    }
}

} // namespace adjoint_detail

// Structure of a transpose: the stable permutation (position in the transpose -> stored entry of
// the source) and the transpose's offsets and column indices. Values are gathered per type.
struct TransposePlan {
    int n = 0, nnz = 0, max_row = 0;
    int *perm = nullptr, *rp = nullptr, *ci = nullptr;
};

// Stable LSD radix sort of the column indices with the entry positions as payload: within each
// column of the source the original rows stay ascending, so the transpose is canonical CSR and the
// construction is deterministic.
template <class TV>
TransposePlan transpose_plan(DeviceArena &arena, const DeviceCsr<TV> &a, int sms, cudaStream_t st) {
    TransposePlan t;
    t.n = a.n;
    t.nnz = a.nnz;
    const int nnz = a.nnz;
    int *keys_out = arena.alloc<int>(nnz);
    int *idx_in = arena.alloc<int>(nnz);
    t.perm = arena.alloc<int>(nnz);
    t.rp = arena.alloc<int>(static_cast<size_t>(a.n) + 1);
    t.ci = arena.alloc<int>(nnz);
    int *row_of = arena.alloc<int>(nnz);
    int *max_len = arena.alloc<int>(1);
    const unsigned gb = grid_for(std::max(nnz, a.n) + 1, 256, sms * 8);
    iota_kernel<<<gb, 256, 0, st>>>(nnz, idx_in);
    SPAI_LAUNCH("iota_kernel");
    int end_bit = 1;
    while (end_bit < 31 && (1LL << end_bit) < a.n)
        ++end_bit;
    size_t tmp_bytes = 0;
    SPAI_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, a.ci, keys_out, idx_in, t.perm, nnz, 0,
                                              end_bit, st));
    void *tmp = arena.alloc<unsigned char>(tmp_bytes);
    SPAI_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, a.ci, keys_out, idx_in, t.perm, nnz, 0,
                                              end_bit, st));
    transpose_offsets_kernel<<<gb, 256, 0, st>>>(a.n, nnz, keys_out, t.rp);
    SPAI_LAUNCH("transpose_offsets_kernel");
    row_of_kernel<<<gb, 256, 0, st>>>(a.n, a.rp, row_of);
    SPAI_LAUNCH("row_of_kernel");
    gather_values_kernel<int><<<gb, 256, 0, st>>>(nnz, t.perm, row_of, t.ci);
    SPAI_LAUNCH("gather_values_kernel");
    SPAI_CUDA(cudaMemsetAsync(max_len, 0, sizeof(int), st));
    transpose_max_kernel<<<gb, 256, 0, st>>>(a.n, t.rp, max_len);
    SPAI_LAUNCH("transpose_max_kernel");
    int host_max = 0;
    SPAI_CUDA(cudaMemcpyAsync(&host_max, max_len, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPAI_CUDA(cudaStreamSynchronize(st));
    t.max_row = host_max;
    return t;
}

// The transpose of a matrix (with plan computed from its structure) in value type TV.
template <class TV>
DeviceCsr<TV> transpose_values(DeviceArena &arena, const TransposePlan &t, const TV *val, int sms,
                               cudaStream_t st) {
    DeviceCsr<TV> out;
    out.n = t.n;
    out.nnz = t.nnz;
    out.max_row = t.max_row;
    out.rp = t.rp;
    out.ci = t.ci;
    out.val = arena.alloc<TV>(t.nnz);
    gather_values_kernel<TV><<<grid_for(t.nnz, 256, sms * 8), 256, 0, st>>>(t.nnz, t.perm, val, out.val);
    SPAI_LAUNCH("gather_values_kernel");
    return out;
}

} // namespace spai
