// Allocation-free backward-error query (spai_backward_error_noalloc).
//
// Some callers cannot call cudaMalloc at the point where they need this number: applications that
// hand all device memory to their own pool or caching allocator at start-up, and latency-critical
// loops where the implicit device synchronisation of an allocation is not acceptable. For them
// this entry point computes the refinement residual r = b - A x and the normwise/componentwise
// backward errors of a given x with the handle's resident matrix, using no allocation at all: its
// scratch (the residual vector and the per-block partial results) lives in the file-scope array
// below, which every GPU that loads the library holds until the process exits.
//
// Limit: n <= kNoallocMaxRows (rows of the residual that fit in the array); larger systems are
// rejected with SPAI_ERR_ARGUMENT. Every call shares the array and leaves its contents behind;
// the ticket counter that must start at zero is cleared by each call. Calls that overlap on the
// GPU (different streams, or different host threads) race on the array.
#include "common.cuh"
#include "spai_internal.hpp"
#include "spai_ir.h"

#include <cmath>
#include <mutex>
#include <string>

namespace spai {

constexpr int kNoallocBlock = 256;
constexpr int kNoallocMaxBlocks = 1024;
constexpr size_t kNoallocHeader = 256;                      // ticket counter
// Partial records (32 bytes each), split in two halves: records [0, 512) hold each block's
// {||r||_inf, ||x||_inf, componentwise ratio, nonfinite flag}, records [512, 1024) the same
// block's {||A||_inf, ||b||_inf}. That split is why a launch has at most kNoallocMaxBlocks / 2
// blocks. Scratch total: 256 + 32,768 bytes of header and partials plus 4 MiB of residual.
constexpr size_t kNoallocPartials = kNoallocMaxBlocks * 32;
constexpr size_t kNoallocResidualBytes = size_t(4) << 20;  // 4 MiB of binary64 residual
constexpr size_t kNoallocBytes = kNoallocHeader + kNoallocPartials + kNoallocResidualBytes;
constexpr long long kNoallocMaxRows = static_cast<long long>(kNoallocResidualBytes / sizeof(double));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

struct NoallocPart {
    double rinf, xinf, cbe;
    int nonfinite;
};

// Variant of the refinement residual kernel: r = b - A x with ||r||_inf, ||x||_inf, the
// componentwise ratio, ||A||_inf and ||b||_inf in one sweep; the last block writes
// out = {normwise backward error, componentwise backward error, ||r||_inf}.
template <class TO, int G>
__global__ void __launch_bounds__(kNoallocBlock)
    noalloc_backward_error_kernel(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                  const TO *__restrict__ av, const TO *__restrict__ x,
                                  const TO *__restrict__ b, unsigned char *scratch, double *out) {
    int *counter = reinterpret_cast<int *>(scratch);
    NoallocPart *part = reinterpret_cast<NoallocPart *>(scratch + kNoallocHeader);
    TO *r = reinterpret_cast<TO *>(scratch + kNoallocHeader + kNoallocPartials);
    __shared__ double sh[5][kNoallocBlock / 32];
    __shared__ int is_last;
    const int lane = threadIdx.x & (G - 1);
    const int groups = (gridDim.x * blockDim.x) / G;
    const int warp_first = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / G;
    const int sub = (threadIdx.x & 31) / G;
    double rinf = 0, xinf = 0, cbe = 0, ainf = 0, binf = 0;
    int bad = 0;
    for (int base = warp_first; base < n; base += groups) {
        const int row = base + sub;
        TO acc = 0, absacc = 0, rowabs = 0;
        if (row < n)
            for (int t = rp[row] + lane; t < rp[row + 1]; t += G) {
                const TO xv = x[ci[t]];
                acc += av[t] * xv;
                absacc += fabs(av[t]) * fabs(xv);
                rowabs += fabs(av[t]);
            }
        for (int o = G / 2; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
            absacc += __shfl_xor_sync(0xffffffffu, absacc, o, G);
            rowabs += __shfl_xor_sync(0xffffffffu, rowabs, o, G);
        }
        if (lane == 0 && row < n) {
            const TO res = b[row] - acc;
            r[row] = res;
            bad |= !isfinite(res) || !isfinite(absacc) || !isfinite(rowabs);
            rinf = fmax(rinf, static_cast<double>(fabs(res)));
            xinf = fmax(xinf, static_cast<double>(fabs(x[row])));
            ainf = fmax(ainf, static_cast<double>(rowabs));
            binf = fmax(binf, static_cast<double>(fabs(b[row])));
            const double cden = static_cast<double>(fabs(b[row]) + absacc);
            cbe = fmax(cbe, cden == 0 ? (res == TO(0) ? 0.0 : INFINITY)
                                      : static_cast<double>(fabs(res)) / cden);
        }
    }
    double v[5] = {rinf, xinf, cbe, ainf, binf};
    for (int q = 0; q < 5; ++q)
        for (int o = 16; o > 0; o >>= 1)
            v[q] = fmax(v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
    bad = __syncthreads_or(bad);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 5; ++q)
            sh[q][threadIdx.x >> 5] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        double m[5] = {0, 0, 0, 0, 0};
        for (int w = 0; w < kNoallocBlock / 32; ++w)
            for (int q = 0; q < 5; ++q)
                m[q] = fmax(m[q], sh[q][w]);
        part[blockIdx.x] = NoallocPart{m[0], m[1], m[2], bad};
        // ||A||_inf and ||b||_inf travel in the unused slots of an extra record per block.
        part[kNoallocMaxBlocks / 2 + blockIdx.x] = NoallocPart{m[3], m[4], 0, 0};
        __threadfence();
        const int t = atomicAdd(counter, 1);
        is_last = t == static_cast<int>(gridDim.x) - 1;
    }
    __syncthreads();
    if (!is_last || threadIdx.x != 0)
        return;
    __threadfence();
    double R = 0, X = 0, C = 0, An = 0, Bn = 0;
    int nonfinite = 0;
    for (int i = 0; i < static_cast<int>(gridDim.x); ++i) {
        R = fmax(R, part[i].rinf);
        X = fmax(X, part[i].xinf);
        C = fmax(C, part[i].cbe);
        nonfinite |= part[i].nonfinite;
        An = fmax(An, part[kNoallocMaxBlocks / 2 + i].rinf);
        Bn = fmax(Bn, part[kNoallocMaxBlocks / 2 + i].xinf);
    }
    const TO den = static_cast<TO>(An) * static_cast<TO>(X) + static_cast<TO>(Bn);
    double be;
    if (nonfinite || !isfinite(den))
        be = NAN;
    else
        be = den == TO(0) ? (R == 0 ? 0.0 : INFINITY) : static_cast<double>(static_cast<TO>(R) / den);
    out[0] = be;
    out[1] = C;
    out[2] = R;
    *counter = 0;
}

namespace {
std::mutex g_setup_mutex;
unsigned char *g_scratch_ptr[64] = {};

// Device address of the scratch array on the current device, looked up once per device.
unsigned char *scratch_address(int device) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (device < 0 || device >= 64)
        throw ArgumentError("device ordinal out of range");
    if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw CudaError(std::string("cudaGetSymbolAddress(noalloc scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[device] = static_cast<unsigned char *>(p);
    }
    return g_scratch_ptr[device];
}

template <class TO>
void launch_noalloc(const DeviceCsr<TO> &a, const double *d_b, const double *d_x, double *d_out,
                    unsigned char *scratch, int sms, cudaStream_t st) {
    const double avg = a.n ? static_cast<double>(a.nnz) / a.n : 1.0;
    const int G = avg <= 2.5 ? 2 : avg <= 6 ? 4 : avg <= 12 ? 8 : avg <= 24 ? 16 : 32;
    const unsigned blocks = grid_for(static_cast<long long>(a.n) * G, kNoallocBlock,
                                     std::min(sms * 8, kNoallocMaxBlocks / 2));
    const TO *b = reinterpret_cast<const TO *>(d_b);
    const TO *x = reinterpret_cast<const TO *>(d_x);
#define SPAI_NOALLOC_CASE(g)                                                                       \
    case g:                                                                                        \
        noalloc_backward_error_kernel<TO, g><<<blocks, kNoallocBlock, 0, st>>>(a.n, a.rp, a.ci,   \
                                                                              a.val, x, b,         \
                                                                              scratch, d_out);     \
        break;
    switch (G) {
        SPAI_NOALLOC_CASE(2)
        SPAI_NOALLOC_CASE(4)
        SPAI_NOALLOC_CASE(8)
        SPAI_NOALLOC_CASE(16)
        SPAI_NOALLOC_CASE(32)
    }
#undef SPAI_NOALLOC_CASE
    SPAI_LAUNCH("noalloc_backward_error_kernel");
}
} // namespace
} // namespace spai

extern "C" int spai_backward_error_noalloc(spai_handle *h, const double *d_b, const double *d_x,
                                           double *d_out, void *stream) {
    using namespace spai;
    try {
        HandleView v;
        if (!h || !d_b || !d_x || !d_out)
            return spai_api_fail(SPAI_ERR_ARGUMENT, "spai_backward_error_noalloc: null argument");
        handle_view(h, v);
        if (v.precision == SPAI_PREC_F32)
            return spai_api_fail(SPAI_ERR_UNSUPPORTED,
                                 "spai_backward_error_noalloc: needs a handle with binary64 A "
                                 "(SPAI_PREC_F64 or SPAI_PREC_MIXED)");
        if (v.a64->n > kNoallocMaxRows)
            return spai_api_fail(SPAI_ERR_ARGUMENT,
                                 "spai_backward_error_noalloc: n = " + std::to_string(v.a64->n) +
                                     " exceeds the static scratch limit of " +
                                     std::to_string(kNoallocMaxRows) + " rows");
        SPAI_CUDA(cudaSetDevice(v.device));
        unsigned char *scratch = scratch_address(v.device);
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : v.stream;
        SPAI_CUDA(cudaMemsetAsync(scratch, 0, sizeof(int), st)); // ticket counter starts at zero
        launch_noalloc<double>(*v.a64, d_b, d_x, d_out, scratch, v.sms, st);
        return SPAI_OK;
    } catch (const ArgumentError &e) {
        return spai_api_fail(SPAI_ERR_ARGUMENT, e.what());
    } catch (const std::exception &e) {
        return spai_api_fail(SPAI_ERR_CUDA, e.what());
    }
}
