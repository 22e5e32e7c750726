// Internal interfaces between the library's translation units.
#pragma once
#include "common.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

namespace spai {

// Process-wide cache of the device blocks that destroyed arenas held, per device. A one-call solve
// creates and destroys a handle every call, and the cudaMalloc / cudaFree of its workspaces
// (cudaFree synchronises the device) cost milliseconds per call; later arenas take a cached block
// of at least the requested size and at most twice it. A failed cudaMalloc empties the cache and
// retries. SPAI_BLOCK_CACHE=0 turns the cache off.
class BlockCache {
  public:
    // A cached block of `bytes` to 2 * `bytes` bytes (its size in *got), or nullptr.
    void *take(size_t bytes, size_t *got) {
        if (!enabled())
            return nullptr;
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess)
            return nullptr;
        std::lock_guard<std::mutex> lock(mu_);
        auto it = free_.lower_bound({dev, bytes});
        if (it == free_.end() || it->first.first != dev || it->first.second > 2 * bytes)
            return nullptr;
        void *p = it->second;
        *got = it->first.second;
        free_.erase(it);
        return p;
    }
    // p (allocated on device dev) must be idle: no kernel or copy in flight uses it.
    void give(int dev, void *p, size_t bytes) {
        if (!enabled()) {
            cudaFree(p);
            return;
        }
        std::lock_guard<std::mutex> lock(mu_);
        free_.insert({{dev, bytes}, p});
    }
    void release() {
        std::lock_guard<std::mutex> lock(mu_);
        int dev0 = 0;
        cudaGetDevice(&dev0);
        for (auto &kv : free_) {
            cudaSetDevice(kv.first.first);
            cudaFree(kv.second);
        }
        free_.clear();
        cudaSetDevice(dev0);
    }
    static bool enabled() {
        static const bool on = [] {
            const char *e = std::getenv("SPAI_BLOCK_CACHE");
            return !(e && std::atoi(e) == 0);
        }();
        return on;
    }

  private:
    std::mutex mu_;
    std::multimap<std::pair<int, size_t>, void *> free_;
};
inline BlockCache &block_cache() {
    static BlockCache *c = new BlockCache(); // never destroyed: the driver frees device memory at exit
    return *c;
}

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
        // Every device holding a block is synchronised first: the blocks are idle before other
        // arenas may take them from the cache.
        std::vector<int> devs;
        for (auto &s : slots_)
            if (s.ptr && std::find(devs.begin(), devs.end(), s.dev) == devs.end())
                devs.push_back(s.dev);
        if (devs.empty())
            return;
        int dev0 = 0;
        cudaGetDevice(&dev0);
        for (int d : devs) {
            cudaSetDevice(d);
            cudaDeviceSynchronize();
        }
        cudaSetDevice(dev0);
        for (auto &s : slots_)
            if (s.ptr)
                block_cache().give(s.dev, s.ptr, s.bytes);
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
                SPAI_CUDA(cudaFree(s.ptr)); // synchronises: the old block may still be in use
            s.ptr = nullptr;
            s.bytes = 0;
            size_t got = bytes;
            void *p = block_cache().take(bytes, &got);
            if (!p && cudaMalloc(&p, bytes) != cudaSuccess) {
                cudaGetLastError();
                block_cache().release();
                SPAI_CUDA(cudaMalloc(&p, bytes));
            }
            s.ptr = p;
            s.bytes = got;
            SPAI_CUDA(cudaGetDevice(&s.dev));
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
        int dev = 0; // device the block belongs to
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
