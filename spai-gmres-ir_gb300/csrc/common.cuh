// Shared device/host helpers for the SPAI-GMRES-IR library.
#pragma once
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <stdexcept>
#include <string>

namespace spai {

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string &m) : std::runtime_error(m) {
    }
};
struct ArgumentError : std::invalid_argument {
    explicit ArgumentError(const std::string &m) : std::invalid_argument(m) {
    }
};
struct WorkspaceError : std::runtime_error {
    explicit WorkspaceError(const std::string &m) : std::runtime_error(m) {
    }
};

inline void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}
#define SPAI_CUDA(call) ::spai::cuda_check((call), #call)
#define SPAI_LAUNCH(what) ::spai::cuda_check(cudaGetLastError(), what)

constexpr int kWarp = 32;

__device__ __forceinline__ int lane_id() {
    return threadIdx.x & 31;
}
template <class V> __device__ __forceinline__ V shfl(V v, int src) {
    return __shfl_sync(0xffffffffu, v, src);
}
__device__ __forceinline__ int warp_sum_int(int v) {
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_min_int(int v) {
    for (int o = 16; o > 0; o >>= 1)
        v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max_int(int v) {
    for (int o = 16; o > 0; o >>= 1)
        v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// Inclusive prefix sum across the warp.
__device__ __forceinline__ int warp_inclusive_scan(int v) {
    const int lane = lane_id();
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o)
            v += t;
    }
    return v;
}

inline unsigned grid_for(long long work, int per_block, int max_blocks) {
    long long b = (work + per_block - 1) / per_block;
    if (b < 1)
        b = 1;
    if (b > max_blocks)
        b = max_blocks;
    return static_cast<unsigned>(b);
}

} // namespace spai
