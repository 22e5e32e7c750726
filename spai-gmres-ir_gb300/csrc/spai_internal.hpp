// Internal interfaces between the library's translation units.
#pragma once
#include "common.cuh"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace spai {

// Device CSR with 32-bit indices (nnz < 2^31 is checked at upload).
template <class T> struct DeviceCsr {
    int n = 0, nnz = 0;
    int max_row = 0; // longest row (sparsity profile for tuning)
    int *rp = nullptr, *ci = nullptr;
    T *val = nullptr;
};

// Call-sequence caching allocator: the i-th alloc() after a reset() reuses the i-th buffer when
// it is large enough, so repeated builds/solves of the same shape allocate nothing.
class DeviceArena {
  public:
    DeviceArena() = default;
    DeviceArena(const DeviceArena &) = delete;
    DeviceArena &operator=(const DeviceArena &) = delete;
    ~DeviceArena() {
        for (auto &s : slots_)
            if (s.ptr)
                cudaFree(s.ptr);
    }
    void reset() {
        next_ = 0;
    }
    template <class U> U *alloc(size_t count) {
        const size_t bytes = ((count ? count : 1) * sizeof(U) + 255) & ~size_t(255);
        if (next_ == slots_.size())
            slots_.push_back(Slot{});
        Slot &s = slots_[next_++];
        if (s.bytes < bytes) {
            if (s.ptr)
                SPAI_CUDA(cudaFree(s.ptr));
            s.ptr = nullptr;
            s.bytes = 0;
            SPAI_CUDA(cudaMalloc(&s.ptr, bytes));
            s.bytes = bytes;
        }
        return static_cast<U *>(s.ptr);
    }
    size_t bytes_held() const {
        size_t b = 0;
        for (auto &s : slots_)
            b += s.bytes;
        return b;
    }

  private:
    struct Slot {
        void *ptr = nullptr;
        size_t bytes = 0;
    };
    std::vector<Slot> slots_;
    size_t next_ = 0;
};

struct SpaiParams {
    double epsilon = 0.3;
    long long alpha = 5;
    int beta = 8;
    int ws_bytes_per_warp = 0;   // workspace per column group (bytes); 0 = tuned default
    int warps_per_block = 0;     // 0 = fill the shared memory of one block per SM
    int group_lanes = 0;         // lanes per column (4, 8, 16, 32); 0 = tuned default
    bool fast = false;           // parallel norms/mean, hashed candidates (not bit-reproducing)
    size_t overflow_ws_bytes = 0;
    int first_qcap = 0;          // pattern capacity of the first workspace tier; 0 = by size
    bool tune = true;            // time first-tier candidates on a column sample (large n)
    bool record = false;         // log every fit (diagnostics; no tuning then)
};

template <class T> struct SpaiOutput {
    int n = 0;
    int status = 1;
    int first_failed = -1;
    long long fits = 0, growths = 0;
    int overflow_columns = 0;
    long long launches = 0;
    int group_lanes = 0, ws_bytes = 0;
    bool tuned = false;                             // first tier chosen by the autotuner
    double tune_sample_ms = 0, tune_default_ms = 0; // chosen / default pair's time on the sample
    int overflow_columns_global = 0;
    T *d = nullptr;
    // Fit log of a recording build (device streams and their appended counts, see FitLog).
    int *log_ints = nullptr;
    double *log_vals = nullptr;
    unsigned long long *log_top = nullptr;
    long long log_int_cap = 0, log_val_cap = 0;
    int *col_status = nullptr, *col_fits = nullptr, *col_growths = nullptr, *col_clamps = nullptr,
        *col_q = nullptr;
    T *col_residual = nullptr;
    long long *packed_off = nullptr;
    int *packed_idx = nullptr;
    T *packed_val = nullptr;
    DeviceCsr<T> p; // P = N^T D
};

template <class T> struct SpaiBuilder {
    static void construct(const DeviceCsr<T> &a, const SpaiParams &prm, cudaStream_t st,
                          SpaiOutput<T> &out, DeviceArena &arena);
};

template <class T> void score_kat(T rsq, T dot, T den, double *out);

// Read-only view of a handle's resident matrix for entry points outside the API unit.
struct HandleView {
    int precision = 0, device = 0, sms = 0;
    cudaStream_t stream = nullptr;
    const DeviceCsr<double> *a64 = nullptr;
};

} // namespace spai

struct spai_handle_s;
void handle_view(spai_handle_s *h, spai::HandleView &v);
int spai_api_fail(int code, const std::string &msg);

namespace spai {

} // namespace spai
