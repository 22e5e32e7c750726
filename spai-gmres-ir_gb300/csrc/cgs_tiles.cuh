// Gram-Schmidt passes over a tile-major Krylov basis.
//
// Layout: the basis is stored in row tiles of R rows; tile t holds the R-row segments of all
// cap+1 vectors contiguously (segment j of tile t at base + (t*(cap+1) + j)*R). A block that owns
// tile t therefore streams one contiguous region of (k+1)*R*s bytes per pass into shared memory.
//
// Vectors are stored unnormalised: v_j = s_j W_j with the scale s_j kept on the device, so the
// Arnoldi step needs no normalisation pass (the next SpMV and every later pass apply s_j).
//
// One Arnoldi step (classical Gram-Schmidt with DGKS-criterion reorthogonalisation):
//   pass 1: d_j = W_j^T w, ||w||                           (reads V once)
//   pass 2: w' = w - sum_j h1_j v_j, written as W_{k+1}; d2_j = W_j^T w', ||w'||  (reads V once)
//   pass 3 (only if ||w'|| < eta ||w||): w'' = w' - sum_j h2_j v_j, ||w''||       (reads V once)
// The last block of the finishing pass forms the Hessenberg column (h1 [+ h2], ||w'|| or ||w''||),
// applies the Givens rotations and sets the acceptance flags, exactly as the single-pass
// version did. Reductions are deterministic (fixed tile assignment, fixed trees).
//
// Lagged second projection (MODE 4 and 5: two basis reads per step instead of three, used while
// every step streams whole tiles). The second projection h2 = V^T w' of a step is never applied
// to memory: the new vector is stored as w' = S_{k+1} with h(k+1,k) = ||w''|| =
// sqrt(||w'||^2 - ||h2||^2), and the true basis is V = S U^-1 with U upper triangular
// (U[j][k+1] = h2_j, U[k+1][k+1] = h(k+1,k)); its inverse Ui grows by one column per step
// (Ui[:, k+1] = (-Ui h2 / h(k+1,k), 1 / h(k+1,k))). With z = P A S_{k+1} / h(k+1,k) =
// P A v_{k+1} + V E, E = H_u h2 / h(k+1,k) (H_u the unrotated Hessenberg: P A V_k = V_{k+1} H_u):
//   pass 4: D = S^T z and ||z|| (a pass 1 over the stored vectors); d = Ui^T D, h1 = d - E,
//           ||P A v_{k+1}||^2 = ||z||^2 - 2 E^T d + ||E||^2, update coefficients f = Ui d;
//   pass 5: w' = z - S f (= z - V d: E cancels in the orthogonalised vector), second dots
//           E2 = S^T w', ||w'|| (a pass 2 with coefficients f); h2 = Ui^T E2, the DGKS decision,
//           the Hessenberg column h1 [+ h2], the next Ui column and E, the Givens update.
// The DGKS test, Hessenberg column, Givens rotations and acceptance flags are those of the
// three-pass form; the candidate combines the stored vectors with coefficients Ui y.
//
// Streaming: while k + 1 segments fit in a pipeline stage, each block streams its tiles through
// two shared-memory stages filled by asynchronous 16-byte copies (cp.async, one commit group per
// stage): a tile's k + 1 segments are contiguous, several tiles share a stage when k is small,
// and the next stage loads while the current one is consumed. Warps share a tile's segments
// (warp p of the P sharing a tile takes j = p mod P): dots accumulate per lane in registers and
// are reduced across lanes once, the update combines the warps' partial sums in a fixed order,
// and pass 2 takes its second dot product from the resident stage (no re-read). The source
// vector's segment travels in the same stage. Larger k streams (tile, chunk) items through the
// same stages (see the chunked path in the kernel).
#pragma once
#include "common.cuh"
#include "exact_math.cuh"
#include "krylov.cuh"

#include <algorithm>

namespace spai {

template <class T> struct TileGeom;
template <> struct TileGeom<float> {
    static constexpr int R = 128; // 512-byte segments
};
template <> struct TileGeom<double> {
    static constexpr int R = 64; // 512-byte segments
};
constexpr int kCgsThreads = 512;

template <class T> struct Basis {
    T *base;
    int cap1;     // cap + 1 segments per tile
    int ntiles;
    const T *scale; // s_j, j <= cap
    __device__ __forceinline__ T *seg(int tile, int j) const {
        return base + (static_cast<long long>(tile) * cap1 + j) * TileGeom<T>::R;
    }
    __device__ __forceinline__ T &at(int i, int j) const {
        constexpr int R = TileGeom<T>::R;
        return seg(i / R, j)[i % R];
    }
};

// Power-of-two scaled sum of squares: value = s * 2^(2e); combine is exact rescaling.
template <class T> struct Ssq {
    int e;
    T s;
};
template <class T> __device__ __forceinline__ Ssq<T> ssq_combine(Ssq<T> a, Ssq<T> b) {
    if (a.e == INT_MIN)
        return b;
    if (b.e == INT_MIN)
        return a;
    const int E = max(a.e, b.e);
    return Ssq<T>{E, ldexp(a.s, 2 * (a.e - E)) + ldexp(b.s, 2 * (b.e - E))};
}
template <class T> __device__ __forceinline__ T ssq_value(Ssq<T> a) {
    return a.e == INT_MIN ? T(0) : ldexp(sqrt(a.s), a.e);
}

struct CgsScratch {
    void *dots;     // [gridDim][cap+2] of T
    void *norms;    // [gridDim] of Ssq<T>
    int *counter;   // last-block ticket
};

template <class T> struct CgsArgs {
    int n;
    Basis<T> V;
    const T *w;         // plain vector P A v_k (pass 1 and 2 input)
    T *h1, *h2, *H, *cs, *sn, *g, *s;  // s: writable scales (s_{k+1} set by the finishing pass)
    int hld;
    Ctl *ctl;
    CgsScratch scr;
    int always_reorth;
    int stage_segs;     // segments per pipeline stage (at least 2)
    T *gacc;            // large caps: per-block dot accumulators and coefficients in global memory
    T *gcf;             //   ([gridDim][cap + 2] each); nullptr: both in shared memory
    // Lagged second projection (MODE 4 / 5): true projections d, update coefficients f on the
    // stored vectors, the correction image E, the unrotated Hessenberg H_u and the inverse Ui of
    // the basis' triangular factor (both column-major with leading dimension hld).
    T *dl, *fco, *ecorr, *Hu, *Ui;
};

constexpr int kCgsStages = 2;
constexpr int kCgsWarps = kCgsThreads / 32;

// Dynamic shared memory of a pass: accumulators, coefficients and per-warp accumulators first,
// then the staging region (kCgsStages stages of stage_segs segments).
// Accumulators and coefficients ([cap + 2] each) live in shared memory up to this size, in
// per-block global scratch beyond it (very long GMRES caps). Per-warp accumulators hold half a
// stage (stage_segs / 2 + 1 entries) each: the streamed path needs them only when several tiles
// share a stage (k + 2 <= stage_segs / 2), one tile per stage writing each dot straight to its
// single owner; the chunked path keeps them while k + 1 fits.
constexpr size_t kCgsSharedAccMax = 64 * 1024;
template <class T> __host__ __device__ inline bool cgs_acc_global(int cap) {
    return 2 * static_cast<size_t>(cap + 2) * sizeof(T) > kCgsSharedAccMax;
}
__host__ __device__ inline int cgs_warp_slots(int stage_segs) {
    return stage_segs / 2 + 1;
}
template <class T> __host__ __device__ inline size_t cgs_region_offset(int cap, int stage_segs) {
    const size_t accs = cgs_acc_global<T>(cap) ? 0 : 2 * static_cast<size_t>(cap + 2);
    return ((accs + static_cast<size_t>(kCgsWarps) * cgs_warp_slots(stage_segs)) * sizeof(T) + 127) &
           ~static_cast<size_t>(127);
}
// Largest stage (in 512-byte segments) that fits beside the accumulators; a tile at step k needs
// k + 2 segments (basis and source), so cap + 1 covers every step.
template <class T> inline int cgs_stage_segs(int cap, size_t dyn_budget) {
    const size_t fixed = ((cgs_acc_global<T>(cap) ? 0 : 2) * static_cast<size_t>(cap + 2) +
                          static_cast<size_t>(kCgsWarps)) * sizeof(T) + 256;
    if (fixed >= dyn_budget)
        return 0;
    const size_t per_seg = static_cast<size_t>(kCgsStages) * 512 + static_cast<size_t>(kCgsWarps) * sizeof(T) / 2;
    const size_t segs = (dyn_budget - fixed) / per_seg;
    return static_cast<int>(std::min<size_t>(segs, static_cast<size_t>(cap) + 1));
}
template <class T> inline size_t cgs_dyn_smem(int cap, int stage_segs) {
    return cgs_region_offset<T>(cap, stage_segs) + static_cast<size_t>(kCgsStages) * stage_segs * 512;
}

// 16-byte vector of T per lane: a warp covers one 512-byte segment.
template <class T> struct Vec16;
template <> struct Vec16<float> {
    using V = float4;
    static constexpr int E = 4;
    __device__ __forceinline__ static float dot(V a, V b) {
        return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
    }
    __device__ __forceinline__ static V axpy(float c, V x, V y) { // y + c x
        return make_float4(y.x + c * x.x, y.y + c * x.y, y.z + c * x.z, y.w + c * x.w);
    }
    __device__ __forceinline__ static V add(V a, V b) {
        return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
    }
    __device__ __forceinline__ static V sub(V a, V b) {
        return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
    }
    __device__ __forceinline__ static V zero() {
        return make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __device__ __forceinline__ static float get(V a, int i) {
        return i == 0 ? a.x : (i == 1 ? a.y : (i == 2 ? a.z : a.w));
    }
};
template <> struct Vec16<double> {
    using V = double2;
    static constexpr int E = 2;
    __device__ __forceinline__ static double dot(V a, V b) {
        return a.x * b.x + a.y * b.y;
    }
    __device__ __forceinline__ static V axpy(double c, V x, V y) {
        return make_double2(y.x + c * x.x, y.y + c * x.y);
    }
    __device__ __forceinline__ static V add(V a, V b) {
        return make_double2(a.x + b.x, a.y + b.y);
    }
    __device__ __forceinline__ static V sub(V a, V b) {
        return make_double2(a.x - b.x, a.y - b.y);
    }
    __device__ __forceinline__ static V zero() {
        return make_double2(0.0, 0.0);
    }
    __device__ __forceinline__ static double get(V a, int i) {
        return i == 0 ? a.x : a.y;
    }
};


// cp.async 16-byte copies global -> shared (no spin-wait; completion via wait_group).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
template <class T> __device__ T block_sum(T v, T *red) {
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    T r = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i)
        r += red[i];
    __syncthreads();
    return r; // every thread, same order
}
template <class T> __device__ T block_max(T v, T *red) {
    for (int o = 16; o > 0; o >>= 1)
        v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    T r = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i)
        r = fmax(r, red[i]);
    __syncthreads();
    return r;
}

// Givens update of Hessenberg column k (src/gmres.cpp:191-214) and the acceptance triggers.
// Runs in one thread after the column col[0..k+1] has been written.
// col: Hessenberg column k (any memory space); csr / snr: the previous rotations to read (a
// shared-memory copy, or cs / sn themselves); the new rotation is written to cs[k], sn[k].
template <class T> __device__ void finish_column_at(Ctl *ctl, T *col, const T *csr, const T *snr, T *cs, T *sn,
                                                    T *g, T *s, T hnext, bool nonfinite) {
    const int k = ctl->k;
    col[k + 1] = hnext;
    if (ctl->h_raw) { // record mode: the column before its rotations
        T *raw = static_cast<T *>(ctl->h_raw) + static_cast<long long>(k) * ctl->h_raw_ld;
        for (int r = 0; r <= k + 1; ++r)
            raw[r] = col[r];
    }
    nonfinite |= !isfinite(hnext);
    ctl->hnext = static_cast<double>(hnext);
    ctl->breakdown = hnext == T(0);
    s[k + 1] = hnext == T(0) ? T(0) : T(1) / hnext;
    // Previous rotations down the column; the entry carried to the next rotation stays in a
    // register (same arithmetic as rotating in place).
    T carry = k > 0 ? col[0] : T(0);
#pragma unroll 8
    for (int r = 0; r < k; ++r) {
        const T up = carry, lo = col[r + 1];
        col[r] = csr[r] * up + snr[r] * lo;
        carry = -snr[r] * up + csr[r] * lo;
    }
    if (k > 0)
        col[k] = carry;
    const T upper = col[k];
    const T radius = cr_hypot<T>(upper, col[k + 1]);
    ctl->iterations = k + 1;
    spai_iteration_record *rec = nullptr;
    if (ctl->h_iter && ctl->h_iter_base + k < ctl->h_cap_iter) { // GmresResult::history entry
        rec = ctl->h_iter + ctl->h_iter_base + k;
        *rec = spai_iteration_record{ctl->inner_attempts + 1, k + 1, NAN, NAN, 0, 0};
        ctl->h_n_iter = max(ctl->h_n_iter, ctl->h_iter_base + k + 1);
    }
    if (nonfinite || !isfinite(radius)) {
        ctl->status = 8;
        ctl->active = 0;
        ctl->triggered = 0;
        ctl->vgate = 0;
        return;
    }
    if (radius == T(0)) {
        ctl->triggered = 2; // verify the previously defined candidate (gmres.cpp:218-234)
        ctl->vgate = 1;
        if (rec)
            rec->triggered = 1;
        return;
    }
    cs[k] = upper / radius;
    sn[k] = col[k + 1] / radius;
    col[k] = radius;
    col[k + 1] = 0;
    const T old = g[k];
    g[k] = cs[k] * old;
    g[k + 1] = -sn[k] * old;
    const T est = fabs(g[k + 1]) / static_cast<T>(ctl->den);
    ctl->est = static_cast<double>(est);
    if (rec)
        rec->estimated_relative = static_cast<double>(est);
    const bool trig = ctl->breakdown || est <= static_cast<T>(ctl->tol_inner) || k + 1 == ctl->cap;
    ctl->triggered = trig ? 1 : 0;
    if (rec)
        rec->triggered = trig ? 1 : 0;
    ctl->vgate = (trig || ctl->accept_every || ctl->record_every) ? 1 : 0;
}
template <class T> __device__ void finish_column(Ctl *ctl, T *H, int hld, T *cs, T *sn, T *g, T *s,
                                                 T hnext, bool nonfinite) {
    finish_column_at(ctl, H + static_cast<long long>(ctl->k) * hld, cs, sn, cs, sn, g, s, hnext, nonfinite);
}

// One Gram-Schmidt pass (MODE 1, 2 or 3, or the lagged 4 and 5; see the file comment). Grid:
// persistent over tiles.
template <class T, int MODE>
__global__ void __launch_bounds__(kCgsThreads) cgs_pass_kernel(CgsArgs<T> a) {
    constexpr int R = TileGeom<T>::R;
    // The lagged passes stream exactly like passes 1 (dots) and 2 (update and second dots).
    constexpr bool LAGA = MODE == 4, LAGB = MODE == 5, LAG = LAGA || LAGB;
    constexpr int BM = LAGA ? 1 : (LAGB ? 2 : MODE);
    Ctl *ctl = a.ctl;
    if (!ctl->active)
        return;
    if (MODE == 3 && !ctl->reorth)
        return;
    extern __shared__ __align__(16) unsigned char dyn[];
    const bool gacc = a.gacc != nullptr;
    T *acc = gacc ? a.gacc + static_cast<size_t>(blockIdx.x) * (ctl->cap + 2)
                  : reinterpret_cast<T *>(dyn);                     // [cap + 2] dot accumulators
    T *cf = gacc ? a.gcf + static_cast<size_t>(blockIdx.x) * (ctl->cap + 2)
                 : acc + (ctl->cap + 2);                            // [cap + 2] update coefficients h_j s_j
    T *accw = gacc ? reinterpret_cast<T *>(dyn)
                   : cf + (ctl->cap + 2);                           // [warps][stage_segs / 2 + 1]
    T *region = reinterpret_cast<T *>(dyn + cgs_region_offset<T>(ctl->cap, a.stage_segs)); // staging (128-byte aligned)
    __shared__ T red[kCgsThreads / 32];
    const int k = ctl->k;
    const int kk = k + 1; // segments 0..k
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const T *coef = BM == 2 ? a.h1 : a.h2; // h_j (coefficient h_j s_j applied below)
    for (int j = threadIdx.x; j < kk; j += blockDim.x) {
        acc[j] = 0;
        if (LAGB)
            cf[j] = a.fco[j]; // f = Ui d: coefficients on the stored vectors
        else if (BM >= 2)
            cf[j] = coef[j] * a.V.scale[j];
    }
    // Per-thread power-of-two scaled sum of squares of the current vector (no block syncs):
    // value = ts * 2^(2 te); rescaling by powers of two is exact.
    int te = INT_MIN;
    T ts = 0;
    bool bad = false;
    auto ssq_add = [&](T v) {
        bad |= !isfinite(v);
        if (v != T(0) && isfinite(v)) {
            const int ev = ilogb(v);
            if (ev > te) {
                if (te != INT_MIN)
                    ts = ldexp(ts, 2 * (te - ev));
                te = ev;
            }
            const T sv = ldexp(v, -te);
            ts += sv * sv;
        }
    };
    // A tile occupies kk + 1 segments of a stage: W_0..W_k, then the source vector's segment (w
    // for passes 1 and 2, W_{k+1} for pass 3), so no tile waits on a dependent global load.
    const int tseg = kk + 1;
    const bool streamed = tseg <= a.stage_segs;
    // Partial updates of the warps (passes 2 and 3), shared by the streamed and chunked paths.
    __shared__ __align__(16) typename Vec16<T>::V wpart_all[BM >= 2 ? kCgsWarps : 1][32];
    if (LAG && !streamed) {
        // The engine runs the lagged passes only when every step of the solve streams.
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->status = 8;
            ctl->active = 0;
        }
        return;
    }
    if (streamed) {
        // ---- Streamed path: whole tiles through a ring of item slots in shared memory. ----
        using VT = Vec16<T>;
        using V16 = typename VT::V;
        constexpr int E = VT::E;
        auto &wpart = wpart_all;
        const int cs = cgs_warp_slots(a.stage_segs);
        for (int i = threadIdx.x; i < kCgsWarps * cs; i += blockDim.x)
            accw[i] = 0;
        T *stage0 = region;
        // The staging region is a ring of nslots item slots. An item fills one stage (tt_per
        // tiles) and two slots alternate: smaller items in a deeper ring measured slower (more
        // warps per tile, more combine barriers), 3.8 vs 4.6 TB/s for pass 1 on the 128^3 system.
        const int tt_per = max(1, a.stage_segs / tseg); // tiles per item
        const int item_segs = a.stage_segs;
        const int nslots = kCgsStages;
        const size_t stage_elems = static_cast<size_t>(item_segs) * R;
        // Warps per tile: P = 1 when a stage holds at least as many tiles as warps (each warp takes
        // whole tiles, no barrier); otherwise P warps share a tile, warp p taking segments
        // j = p (mod P), and combine their partial updates once per stage.
        const int P = tt_per >= kCgsWarps ? 1 : kCgsWarps / tt_per;
        const int slot = warp / P, part = warp % P;
        const int my_tiles = a.V.ntiles > static_cast<int>(blockIdx.x)
                                 ? (a.V.ntiles - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
                                 : 0;
        const int nitems = (my_tiles + tt_per - 1) / tt_per;
        const int basis_bytes = (BM == 3 ? tseg : kk) * R * static_cast<int>(sizeof(T));
        constexpr int kSegBytes = R * static_cast<int>(sizeof(T));
        // Every thread issues 16-byte asynchronous copies for an item's tiles; one commit group per
        // item (empty past the end), so "all but the newest group complete" means "item ready".
        auto issue = [&](int item) {
            if (item < nitems) {
                const int st = item % nslots;
                const int q0 = item * tt_per;
                const int q1 = min(my_tiles, q0 + tt_per);
                for (int q = q0; q < q1; ++q) {
                    const int t = static_cast<int>(blockIdx.x) + q * static_cast<int>(gridDim.x);
                    char *dst = reinterpret_cast<char *>(stage0 + st * stage_elems + static_cast<size_t>(q - q0) * tseg * R);
                    const char *src = reinterpret_cast<const char *>(a.V.seg(t, 0));
                    for (int o = threadIdx.x * 16; o < basis_bytes; o += kCgsThreads * 16)
                        cp_async16(dst + o, src + o);
                    if (BM != 3) {
                        const char *ws = reinterpret_cast<const char *>(a.w + static_cast<long long>(t) * R);
                        for (int o = threadIdx.x * 16; o < kSegBytes; o += kCgsThreads * 16)
                            cp_async16(dst + kk * kSegBytes + o, ws + o);
                    }
                }
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        };
        __syncthreads(); // coefficients and accumulators visible
        for (int i = 0; i < nslots; ++i)
            issue(i);
        double dsq = 0; // binary32 sums of squares, exact range in binary64
        // One tile per stage (P == warps): every segment has a single owning warp, which writes
        // its dot straight into acc; several tiles per stage (k + 2 <= stage_segs / 2): per-warp
        // accumulators, summed in warp order below.
        T *myacc = P == kCgsWarps ? acc : accw + warp * cs;
        // A warp owns the same segments (j = part mod P) for the whole launch: its per-lane dot
        // partials stay in registers across tiles (fixed order) and are reduced across lanes
        // once at the end. Shuffle-per-segment reduction is the fallback for longer sets.
        constexpr int kOwn = 20;
        const bool reg_dots = (kk + P - 1) / P <= kOwn;
        T racc[kOwn];
#pragma unroll
        for (int i = 0; i < kOwn; ++i)
            racc[i] = 0;
        // Pass 2 keeps a warp's segments in registers between the update and the second dot
        // products when it owns few enough of them (one shared-memory read of the tile, not two).
        constexpr int kCache = sizeof(T) == 4 ? 12 : 6;
        const bool cache = BM == 2 && (kk + P - 1) / P <= kCache;
        V16 vr[kCache];
        auto update_part = [&](const T *tile) {
            V16 acc4 = VT::zero();
            if (cache) {
#pragma unroll
                for (int i0 = 0; i0 < kCache; i0 += 2) {
                    if (part + i0 * P >= kk)
                        break;
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int i = i0 + u, j = part + i * P;
                        if (i < kCache && j < kk) {
                            vr[i] = *reinterpret_cast<const V16 *>(tile + j * R + lane * E);
                            acc4 = VT::axpy(cf[j], vr[i], acc4);
                        }
                    }
                }
            } else {
#pragma unroll 4
                for (int j = part; j < kk; j += P)
                    acc4 = VT::axpy(cf[j], *reinterpret_cast<const V16 *>(tile + j * R + lane * E), acc4);
            }
            return acc4;
        };
        auto dots = [&](const T *tile, V16 cur) {
            if (cache) {
#pragma unroll
                for (int i = 0; i < kCache; ++i) {
                    if (part + i * P >= kk)
                        break;
                    racc[i] += VT::dot(vr[i], cur);
                }
            } else if (reg_dots) {
#pragma unroll
                for (int i0 = 0; i0 < kOwn; i0 += 8) {
                    if (part + i0 * P >= kk)
                        break;
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int j = part + (i0 + u) * P;
                        if (j < kk)
                            racc[i0 + u] += VT::dot(*reinterpret_cast<const V16 *>(tile + j * R + lane * E), cur);
                    }
                }
            } else {
#pragma unroll 2
                for (int j = part; j < kk; j += P) {
                    T d = VT::dot(*reinterpret_cast<const V16 *>(tile + j * R + lane * E), cur);
                    for (int o = 16; o > 0; o >>= 1)
                        d += __shfl_xor_sync(0xffffffffu, d, o);
                    if (lane == 0)
                        myacc[j] += d;
                }
            }
        };
        // With several warps per tile, passes 2 and 3 no longer read the stage after the barrier that
        // combines their partial updates when the source segment was taken into registers and the
        // second dots use the segments cached in registers: the next item's copies into this slot
        // are issued right after that barrier, overlapping the combine, the stores and the dots.
        const bool early = P > 1 && BM >= 2 && (BM == 3 || cache);
        for (int item = 0; item < nitems; ++item) {
            const int st = item % nslots;
            // all but the newest nslots - 1 commit groups complete = this item has landed
            switch (nslots) {
            case 2: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
            case 3: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
            case 4: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
            case 5: asm volatile("cp.async.wait_group 4;\n" ::: "memory"); break;
            case 6: asm volatile("cp.async.wait_group 5;\n" ::: "memory"); break;
            case 7: asm volatile("cp.async.wait_group 6;\n" ::: "memory"); break;
            default: asm volatile("cp.async.wait_group 7;\n" ::: "memory"); break;
            }
            __syncthreads();
            const T *sbase = stage0 + st * stage_elems;
            const int q0 = item * tt_per;
            const int nq = min(my_tiles, q0 + tt_per) - q0;
            // P == 1: warp takes tiles slot, slot + 8, ...; P > 1: one round, tile `slot`.
            const int qstep = P == 1 ? kCgsWarps : nq + 1;
            V16 zsave = VT::zero(); // the tile's source segment (P > 1)
            for (int qq = slot; qq < nq; qq += qstep) {
                const int t = static_cast<int>(blockIdx.x) + (q0 + qq) * static_cast<int>(gridDim.x);
                const T *tile = sbase + static_cast<size_t>(qq) * tseg * R;
                V16 cur = *reinterpret_cast<const V16 *>(tile + kk * R + lane * E);
                if (BM >= 2) {
                    const V16 acc4 = update_part(tile);
                    if (P > 1) {
                        wpart[warp][lane] = acc4; // combined after the block barrier below
                        zsave = cur;
                        break;
                    }
                    cur = VT::sub(cur, acc4); // pad rows: every operand is zero there
                    *reinterpret_cast<V16 *>(a.V.seg(t, kk) + lane * E) = cur; // W_{k+1}
                }
                if (BM <= 2)
                    dots(tile, cur);
                if (part == 0)
                    for (int e = 0; e < E; ++e) {
                        const T v = VT::get(cur, e);
                        if (sizeof(T) == 4) {
                            bad |= !isfinite(v);
                            dsq += static_cast<double>(v) * static_cast<double>(v);
                        } else {
                            ssq_add(v);
                        }
                    }
            }
            if (P > 1 && BM >= 2) {
                // Combine the P partial updates of each tile in warp order, then finish the tile.
                // (Splitting the sums over the warps, one read of each partial plus a second
                // barrier, measured slower: 75.9 against 72.2 ms for pass 5 at 128^3.)
                __syncthreads();
                if (early)
                    issue(item + nslots);
                if (slot < nq) {
                    const int qq = slot;
                    const int t = static_cast<int>(blockIdx.x) + (q0 + qq) * static_cast<int>(gridDim.x);
                    const T *tile = sbase + static_cast<size_t>(qq) * tseg * R;
                    V16 tot = wpart[slot * P][lane];
                    for (int p2 = 1; p2 < P; ++p2)
                        tot = VT::add(tot, wpart[slot * P + p2][lane]);
                    V16 cur = VT::sub(zsave, tot);
                    if (part == 0) {
                        *reinterpret_cast<V16 *>(a.V.seg(t, kk) + lane * E) = cur; // W_{k+1}
                        for (int e = 0; e < E; ++e) {
                            const T v = VT::get(cur, e);
                            if (sizeof(T) == 4) {
                                bad |= !isfinite(v);
                                dsq += static_cast<double>(v) * static_cast<double>(v);
                            } else {
                                ssq_add(v);
                            }
                        }
                    }
                    if (BM == 2)
                        dots(tile, cur);
                }
            }
            if (!early) {
                __syncthreads(); // the slot is free
                issue(item + nslots);
            }
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        if (BM <= 2 && reg_dots) {
#pragma unroll
            for (int i = 0; i < kOwn; ++i) {
                const int j = part + i * P;
                if (part + i * P >= kk)
                    break;
                T d = racc[i];
                for (int o = 16; o > 0; o >>= 1)
                    d += __shfl_xor_sync(0xffffffffu, d, o);
                if (lane == 0)
                    myacc[j] = d;
            }
        }
        __syncthreads();
        // Per-warp accumulators -> acc in warp order (deterministic); with one tile per stage
        // the owners wrote acc directly.
        if (BM <= 2 && P != kCgsWarps)
            for (int j = threadIdx.x; j < kk; j += blockDim.x) {
                T sum = 0;
                for (int w2 = 0; w2 < kCgsWarps; ++w2)
                    sum += accw[w2 * cs + j];
                acc[j] = sum;
            }
        if (sizeof(T) == 4 && dsq > 0) {
            // binary64 sum of squares -> (te, ts) with ts in [1, 4)
            const int e2 = ilogb(dsq);
            te = e2 >= 0 ? e2 / 2 : -((1 - e2) / 2);
            ts = static_cast<T>(ldexp(dsq, -2 * te));
        }
    }
    // ---- Chunked streaming (k + 2 > stage_segs): items are (tile, chunk) pairs of at most
    // cs = stage_segs - 1 basis segments plus the source vector's segment. All warps share a
    // chunk; warp w owns the segments j = w (mod warps) and adds its warp-reduced dots straight
    // into acc[j] (one owner per j: no races, fixed order). Passes 2 and 3 accumulate their
    // partial update over a tile's chunks in registers and combine the warps once, at the tile's
    // last chunk; pass 2 then streams the tile's chunks again (L2-resident) for its second dots.
    const bool chunked = !streamed && a.stage_segs >= 2;
    if (chunked) {
        using VT = Vec16<T>;
        using V16 = typename VT::V;
        constexpr int E = VT::E;
        constexpr int kSegBytes = R * static_cast<int>(sizeof(T));
        auto &wpart_c = wpart_all;
        T *stage0 = region;
        const int cs = a.stage_segs - 1;
        const size_t stage_elems = static_cast<size_t>(a.stage_segs) * R;
        const int nch = (kk + cs - 1) / cs;
        const int per_tile = nch * (MODE == 2 ? 2 : 1);
        const int my_tiles = a.V.ntiles > static_cast<int>(blockIdx.x)
                                 ? (a.V.ntiles - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
                                 : 0;
        const long long nitems = static_cast<long long>(my_tiles) * per_tile;
        auto issue = [&](long long item) {
            if (item < nitems) {
                const int st = static_cast<int>(item % kCgsStages);
                const int q = static_cast<int>(item / per_tile), rem = static_cast<int>(item % per_tile);
                const int sweep = rem / nch, c = rem % nch;
                const int t = static_cast<int>(blockIdx.x) + q * static_cast<int>(gridDim.x);
                const int j0 = c * cs, j1 = min(kk, j0 + cs);
                char *dst = reinterpret_cast<char *>(stage0 + st * stage_elems);
                const char *src = reinterpret_cast<const char *>(a.V.seg(t, j0));
                const int bytes = (j1 - j0) * kSegBytes;
                for (int o = threadIdx.x * 16; o < bytes; o += kCgsThreads * 16)
                    cp_async16(dst + o, src + o);
                if (sweep == 0) { // the source segment goes after the chunk (slot cs)
                    const char *ws = MODE == 3 ? reinterpret_cast<const char *>(a.V.seg(t, kk))
                                               : reinterpret_cast<const char *>(a.w + static_cast<long long>(t) * R);
                    for (int o = threadIdx.x * 16; o < kSegBytes; o += kCgsThreads * 16)
                        cp_async16(dst + static_cast<size_t>(cs) * kSegBytes + o, ws + o);
                }
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        };
        __syncthreads(); // coefficients and accumulators visible
        for (int i = 0; i < kCgsStages; ++i)
            issue(i);
        V16 cur = VT::zero(), part4 = VT::zero();
        double dsq = 0;
        auto accumulate_norm = [&](V16 v) {
            for (int e = 0; e < E; ++e) {
                const T x = VT::get(v, e);
                if (sizeof(T) == 4) {
                    bad |= !isfinite(x);
                    dsq += static_cast<double>(x) * static_cast<double>(x);
                } else {
                    ssq_add(x);
                }
            }
        };
        // Dots land in per-warp shared accumulators (slot j / warps of the owning warp) while k
        // fits them; acc may be in global memory for long caps, where a read-modify-write per
        // (tile, segment) would serialise on its latency.
        const int cs_len = cgs_warp_slots(a.stage_segs);
        const bool own_smem = kk <= kCgsWarps * cs_len;
        T *myw = accw + warp * cs_len;
        for (int i = threadIdx.x; i < kCgsWarps * cs_len; i += blockDim.x)
            accw[i] = 0;
        __syncthreads();
        // A warp owns at most 16 segments of a chunk (cs <= 256): their 16 lane partials are
        // reduced together by a reduce-scatter (16 shuffles and adds in all, not 5 per segment:
        // the reductions dominated on the binary64 pipe), leaving lane u with owned segment u.
        auto chunk_dots = [&](const T *sb, int j0, int j1) {
            const int jf = j0 + ((warp - j0 % kCgsWarps) + kCgsWarps) % kCgsWarps;
            T p[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int j = jf + u * kCgsWarps;
                p[u] = j < j1 ? VT::dot(*reinterpret_cast<const V16 *>(sb + (j - j0) * R + lane * E), cur) : T(0);
            }
#pragma unroll
            for (int m = 8; m >= 1; m >>= 1) {
                const bool up = (lane & m) != 0;
#pragma unroll
                for (int i = 0; i < m; ++i) {
                    const T send = up ? p[i] : p[i + m];
                    const T keep = up ? p[i + m] : p[i];
                    p[i] = keep + __shfl_xor_sync(0xffffffffu, send, m);
                }
            }
            const T d = p[0] + __shfl_xor_sync(0xffffffffu, p[0], 16);
            const int j = jf + (lane & 15) * kCgsWarps;
            if (lane < 16 && j < j1) {
                if (own_smem)
                    myw[j / kCgsWarps] += d;
                else
                    acc[j] += d;
            }
        };
        for (long long item = 0; item < nitems; ++item) {
            const int st = static_cast<int>(item % kCgsStages);
            asm volatile("cp.async.wait_group %0;\n" ::"n"(kCgsStages - 1) : "memory");
            __syncthreads();
            const T *sb = stage0 + st * stage_elems;
            const int q = static_cast<int>(item / per_tile), rem = static_cast<int>(item % per_tile);
            const int sweep = rem / nch, c = rem % nch;
            const int t = static_cast<int>(blockIdx.x) + q * static_cast<int>(gridDim.x);
            const int j0 = c * cs, j1 = min(kk, j0 + cs);
            if (sweep == 0 && MODE == 1) {
                if (c == 0) {
                    cur = *reinterpret_cast<const V16 *>(sb + static_cast<size_t>(cs) * R + lane * E);
                    if (warp == 0)
                        accumulate_norm(cur);
                }
                chunk_dots(sb, j0, j1);
            } else if (sweep == 0) {
                if (c == 0)
                    part4 = VT::zero();
                for (int j = j0 + ((warp - j0 % kCgsWarps) + kCgsWarps) % kCgsWarps; j < j1; j += kCgsWarps)
                    part4 = VT::axpy(cf[j], *reinterpret_cast<const V16 *>(sb + (j - j0) * R + lane * E), part4);
                if (c == nch - 1) {
                    wpart_c[warp][lane] = part4;
                    __syncthreads();
                    V16 tot = wpart_c[0][lane];
                    for (int w2 = 1; w2 < kCgsWarps; ++w2)
                        tot = VT::add(tot, wpart_c[w2][lane]);
                    cur = VT::sub(*reinterpret_cast<const V16 *>(sb + static_cast<size_t>(cs) * R + lane * E), tot);
                    if (warp == 0) {
                        *reinterpret_cast<V16 *>(a.V.seg(t, kk) + lane * E) = cur; // W_{k+1}
                        accumulate_norm(cur);
                    }
                }
            } else {
                chunk_dots(sb, j0, j1); // pass 2, second sweep: dots of w'
            }
            __syncthreads(); // the slot (and wpart_c) is free
            issue(item + kCgsStages);
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        if (MODE <= 2 && own_smem) // one owner per j: a copy, not a sum
            for (int j = threadIdx.x; j < kk; j += blockDim.x)
                acc[j] = accw[(j % kCgsWarps) * cs_len + j / kCgsWarps];
        if (sizeof(T) == 4 && dsq > 0) {
            const int e2 = ilogb(dsq);
            te = e2 >= 0 ? e2 / 2 : -((1 - e2) / 2);
            ts = static_cast<T>(ldexp(dsq, -2 * te));
        }
    }
    // Block combine of the per-thread (te, ts) pairs: common exponent, then a fixed-order sum.
    int be = te;
    for (int o = 16; o > 0; o >>= 1)
        be = max(be, __shfl_xor_sync(0xffffffffu, be, o));
    __shared__ int be_sh[kCgsThreads / 32];
    if (lane == 0)
        be_sh[warp] = be;
    __syncthreads();
    be = INT_MIN;
    for (int i = 0; i < nw; ++i)
        be = max(be, be_sh[i]);
    const T scaled = (te == INT_MIN || be == INT_MIN) ? T(0) : ldexp(ts, 2 * (te - be));
    const T bsum = block_sum(scaled, red);
    const Ssq<T> nrm{be, bsum};
    // Publish block partials.
    T *dots = static_cast<T *>(a.scr.dots);
    Ssq<T> *norms = static_cast<Ssq<T> *>(a.scr.norms);
    const int ps = ctl->cap + 2;
    __syncthreads();
    if (BM <= 2)
        for (int j = threadIdx.x; j < kk; j += blockDim.x)
            dots[static_cast<long long>(blockIdx.x) * ps + j] = acc[j];
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0)
        norms[blockIdx.x] = bad ? Ssq<T>{INT_MAX, T(NAN)} : nrm;
    // Last-block ticket.
    __shared__ int is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const int tk = atomicAdd(a.scr.counter, 1);
        is_last = tk == static_cast<int>(gridDim.x) - 1;
        if (is_last)
            *a.scr.counter = 0;
    }
    __syncthreads();
    if (!is_last)
        return;
    __threadfence();
    const int nb = gridDim.x;
    // Dots: one warp per j, lanes over blocks, fixed tree.
    // The lagged passes keep the raw dots S^T z (in acc, reused) for the triangular transform.
    T *hout = LAG ? acc : (BM == 1 ? a.h1 : a.h2);
    if (BM <= 2)
        for (int j = warp; j < kk; j += nw) {
            T sdot = 0;
            for (int b = lane; b < nb; b += 32)
                sdot += dots[static_cast<long long>(b) * ps + j];
            for (int o = 16; o > 0; o >>= 1)
                sdot += __shfl_xor_sync(0xffffffffu, sdot, o);
            if (lane == 0)
                hout[j] = LAG ? sdot : sdot * a.V.scale[j]; // h_j = s_j W_j^T w
        }
    // Norm: parallel max of exponents, then rescaled sum (fixed tree).
    __shared__ int emax_sh;
    int emax = INT_MIN;
    bool nb_bad = false;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        emax = max(emax, norms[b].e == INT_MAX ? INT_MIN : norms[b].e);
        nb_bad |= norms[b].e == INT_MAX;
    }
    for (int o = 16; o > 0; o >>= 1)
        emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    if (threadIdx.x == 0)
        emax_sh = INT_MIN;
    __syncthreads();
    if (lane == 0)
        atomicMax(&emax_sh, emax);
    nb_bad = __syncthreads_or(nb_bad);
    const int E = emax_sh;
    T part_s = 0;
    if (E != INT_MIN)
        for (int b = threadIdx.x; b < nb; b += blockDim.x)
            if (norms[b].e != INT_MIN && norms[b].e != INT_MAX)
                part_s += ldexp(norms[b].s, 2 * (norms[b].e - E));
    const T S = block_sum(part_s, red);
    __syncthreads();
    if (LAG) {
        // Raw dots S^T z (pass 4) or S^T w' (pass 5) are in acc[0..k]. The O(k^2) triangular
        // products run from shared memory: the staging region is free now, and Ui's upper
        // triangle (then, in pass 5, H_u's upper Hessenberg part) is copied into it packed by
        // columns (coalesced), so the products below read shared memory instead of waiting on L2
        // loads one column at a time.
        const T nrm = nb_bad ? T(NAN) : (E == INT_MIN ? T(0) : ldexp(sqrt(S), E));
        const long long ld = a.hld;
        T *us = region;
        auto tri = [](int j) { return j * (j + 1) / 2; };      // column j of Ui: rows 0..j
        auto hes = [](int j) { return j * (j + 3) / 2; };      // column j of H_u: rows 0..j+1
        if (LAGA && k == 0 && threadIdx.x == 0)
            a.Ui[0] = a.V.scale[0]; // S_0 = W_0 is a true basis vector: U = (1 / s_0)
        __syncthreads();
        // Staging copies: every thread takes packed elements e, e + blockDim, ... (four loads in
        // flight), so the copy is one parallel sweep instead of a column after column wait on memory
        // (the factors were written by earlier launches on other SMs and may have left L2).
        auto stage = [&](const T *src, int nel, auto colof, auto start) {
            for (int e0 = threadIdx.x; e0 < nel; e0 += 4 * blockDim.x) {
                T v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = e0 + u * blockDim.x;
                    v[u] = T(0);
                    if (e < nel) {
                        const int j = colof(e);
                        v[u] = src[(e - start(j)) + static_cast<long long>(j) * ld];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = e0 + u * blockDim.x;
                    if (e < nel)
                        us[e] = v[u];
                }
            }
        };
        // column of packed element e: tri(j) <= e < tri(j + 1), resp. hes(j) <= e < hes(j + 1)
        auto tri_col = [&](int e) {
            int j = static_cast<int>((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
            while (j > 0 && tri(j) > e)
                --j;
            while (tri(j + 1) <= e)
                ++j;
            return j;
        };
        auto hes_col = [&](int e) {
            int j = static_cast<int>((sqrtf(8.0f * e + 9.0f) - 3.0f) * 0.5f);
            while (j > 0 && hes(j) > e)
                --j;
            while (hes(j + 1) <= e)
                ++j;
            return j;
        };
        stage(a.Ui, tri(k + 1), tri_col, tri);
        __syncthreads();
        // x = Ui^T v for v in acc (thread per entry j, rows of column j in order).
        auto uit = [&](int j) {
            const T *col = us + tri(j);
            T t = 0;
#pragma unroll 8
            for (int i = 0; i <= j; ++i)
                t += col[i] * acc[i];
            return t;
        };
        if (LAGA) {
            // d = Ui^T D, h1 = d - E (d also in cf, free after the streaming loop).
            const bool pa = ctl->lag_pending != 0;
            for (int j = threadIdx.x; j <= k; j += blockDim.x) {
                const T t = uit(j);
                cf[j] = t;
                a.dl[j] = t;
                a.h1[j] = t - (pa ? a.ecorr[j] : T(0));
            }
            __syncthreads();
            // f = Ui d (thread per entry i, columns j >= i in order).
            for (int i = threadIdx.x; i <= k; i += blockDim.x) {
                T f = 0;
#pragma unroll 8
                for (int j = i; j <= k; ++j)
                    f += us[tri(j) + i] * cf[j];
                a.fco[i] = f;
            }
            if (warp == 0) {
                T ed = 0, ee = 0;
                if (pa)
                    for (int j = lane; j <= k; j += 32) {
                        const T e = a.ecorr[j];
                        ed += e * cf[j];
                        ee += e * e;
                    }
                for (int o = 16; o > 0; o >>= 1) {
                    ed += __shfl_xor_sync(0xffffffffu, ed, o);
                    ee += __shfl_xor_sync(0xffffffffu, ee, o);
                }
                if (lane == 0)
                    ctl->wnorm = static_cast<double>(pa ? sqrt(fmax(nrm * nrm - T(2) * ed + ee, T(0))) : nrm);
            }
            return;
        }
        // Pass 5: h2 = Ui^T E2 (kept in cf for the products below).
        for (int j = threadIdx.x; j <= k; j += blockDim.x) {
            const T t = uit(j);
            cf[j] = t;
            a.h2[j] = t;
        }
        __syncthreads();
        // DGKS test; with a second projection, h(k+1,k) = sqrt(||w'||^2 - ||h2||^2) and h2 stays
        // the pending correction of the new stored vector.
        __shared__ T lag_sh[2];
        if (warp == 0) {
            T hh = 0;
            for (int j = lane; j <= k; j += 32)
                hh += cf[j] * cf[j];
            for (int o = 16; o > 0; o >>= 1)
                hh += __shfl_xor_sync(0xffffffffu, hh, o);
            if (lane == 0) {
                const bool ro = isfinite(nrm) && (a.always_reorth ||
                                                 !(nrm >= T(0.70710678118654752) * static_cast<T>(ctl->wnorm)));
                lag_sh[0] = ro ? T(1) : T(0);
                lag_sh[1] = ro ? sqrt(fmax(nrm * nrm - hh, T(0))) : nrm;
            }
        }
        __syncthreads();
        const bool ro = lag_sh[0] != T(0);
        const T beta = lag_sh[1];
        const T sb = beta == T(0) ? T(0) : T(1) / beta; // s_{k+1}, as finish_column sets it
        T *colh = a.H + k * ld;
        T *colu = a.Hu + k * ld;
        // The Hessenberg column goes to H_u (global) and to a shared copy in acc (the raw dots are
        // consumed), which the Givens update below rotates; finiteness is checked here, in parallel.
        bool nf = false;
        for (int j = threadIdx.x; j <= k; j += blockDim.x) {
            const T hj = a.h1[j] + (ro ? cf[j] : T(0));
            acc[j] = hj;
            colu[j] = hj;
            nf |= !isfinite(hj);
        }
        if (threadIdx.x == 0)
            colu[k + 1] = beta;
        nf = __syncthreads_or(nf);
        // Next column of Ui: (-Ui h2 / h(k+1,k), 1 / h(k+1,k)); E = H_u h2 / h(k+1,k).
        T *uin = a.Ui + (k + 1) * ld;
        T ui[2] = {T(0), T(0)}; // entries i = threadIdx.x, threadIdx.x + blockDim.x (k + 1 < 2 * blockDim.x)
        if (ro)
            for (int r = 0; r < 2; ++r) {
                const int i = threadIdx.x + r * blockDim.x;
                if (i <= k) {
                    T u = 0;
#pragma unroll 8
                    for (int j = i; j <= k; ++j)
                        u += us[tri(j) + i] * cf[j];
                    ui[r] = u;
                }
            }
        __syncthreads(); // Ui's copy is no longer read; H_u's new column is in memory
        if (ro) {
            stage(a.Hu, hes(k + 1), hes_col, hes);
            __syncthreads();
        }
        for (int r = 0; r < 2; ++r) {
            const int i = threadIdx.x + r * blockDim.x;
            if (i > k + 1)
                continue;
            T e = 0;
            if (ro) {
#pragma unroll 8
                for (int j = max(i - 1, 0); j <= k; ++j)
                    e += us[hes(j) + i] * cf[j];
            }
            uin[i] = i == k + 1 ? sb : -ui[r] * sb;
            a.ecorr[i] = e * sb;
        }
        // Givens update from shared copies of the column and of the previous rotations, then the
        // rotated column to H.
        __syncthreads(); // the staging region is free
        T *cssh = us, *snsh = us + (k + 1);
        for (int r = threadIdx.x; r < k; r += blockDim.x) {
            cssh[r] = a.cs[r];
            snsh[r] = a.sn[r];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            ctl->reorth = 0;
            ctl->lag_pending = ro ? 1 : 0;
            if (ro)
                ctl->reorth_count += 1;
            finish_column_at(ctl, acc, cssh, snsh, a.cs, a.sn, a.g, a.s, beta,
                             nf || !isfinite(nrm) || !isfinite(beta));
        }
        __syncthreads();
        for (int j = threadIdx.x; j <= k + 1; j += blockDim.x)
            colh[j] = acc[j];
        return;
    }
    if (threadIdx.x != 0)
        return;
    const T nrm_all = nb_bad ? T(NAN) : (E == INT_MIN ? T(0) : ldexp(sqrt(S), E));
    const int kcol = k;
    T *col = a.H + static_cast<long long>(kcol) * a.hld;
    if (MODE == 1) {
        ctl->wnorm = static_cast<double>(nrm_all);
        return;
    }
    if (MODE == 2) {
        bool nonfinite = !isfinite(nrm_all);
        // DGKS: one more pass only when the projection cancelled more than 1 - 1/sqrt(2).
        const bool reorth = a.always_reorth || !(nrm_all >= T(0.70710678118654752) * static_cast<T>(ctl->wnorm));
        ctl->reorth = reorth && !nonfinite ? 1 : 0;
        if (ctl->reorth)
            return;
        for (int j = 0; j <= kcol; ++j) {
            col[j] = a.h1[j];
            nonfinite |= !isfinite(col[j]);
        }
        finish_column(ctl, a.H, a.hld, a.cs, a.sn, a.g, a.s, nrm_all, nonfinite);
        return;
    }
    // MODE 3
    bool nonfinite = !isfinite(nrm_all);
    for (int j = 0; j <= kcol; ++j) {
        col[j] = a.h1[j] + a.h2[j];
        nonfinite |= !isfinite(col[j]);
    }
    ctl->reorth_count += 1;
    finish_column(ctl, a.H, a.hld, a.cs, a.sn, a.g, a.s, nrm_all, nonfinite);
}

// y = s_k * (A W_k) with W_k gathered from the tile-major basis; G lanes per row.
template <class T, int G>
__global__ void __launch_bounds__(256) spmv_basis_kernel(int n, const int *__restrict__ rp,
                                                         const int *__restrict__ ci,
                                                         const T *__restrict__ av, Basis<T> V,
                                                         T *__restrict__ y, const Ctl *ctl) {
    constexpr int R = TileGeom<T>::R;
    if (!ctl->active)
        return;
    const int k = ctl->k;
    const T sk = V.scale[k];
    const T *base = V.base + static_cast<long long>(k) * R;
    const long long tstride = static_cast<long long>(V.cap1) * R;
    const int lane = threadIdx.x & (G - 1);
    const int groups = (gridDim.x * blockDim.x) / G;
    const int warp_first = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / G;
    const int sub = (threadIdx.x & 31) / G;
    for (int b0 = warp_first; b0 < n; b0 += groups) {
        const int row = b0 + sub;
        T acc = 0;
        if (row < n)
            for (int t = rp[row] + lane; t < rp[row + 1]; t += G) {
                const int c = ci[t];
                acc += av[t] * __ldg(base + (c / R) * tstride + (c % R));
            }
        for (int o = G / 2; o > 0; o >>= 1)
            acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (lane == 0 && row < n)
            y[row] = acc * sk;
    }
}

// x = sum_{j < count} (y_j s_j) W_j (candidate correction; x0 = 0); unit != 0: y holds the
// coefficients on the stored vectors (lagged Gram-Schmidt), x = sum_j y_j W_j.
template <class T>
__global__ void __launch_bounds__(256) form_candidate_tiles_kernel(int n, Basis<T> V, const T *y, int unit,
                                                                   T *x, const Ctl *ctl) {
    constexpr int R = TileGeom<T>::R;
    if (!ctl->active || !ctl->vgate)
        return;
    const int count = ctl->formed;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const T *p = V.base + (static_cast<long long>(i / R) * V.cap1) * R + (i % R);
        T acc = 0;
#pragma unroll 8
        for (int j = 0; j < count; ++j)
            acc += (unit ? y[j] : y[j] * V.scale[j]) * p[static_cast<long long>(j) * R];
        x[i] = acc;
    }
}

// W_0 = Pb / ||Pb|| into the tile-major basis, s_0 = 1; pad rows of every segment zeroed once
// per solve so partial last tiles read zeros.
template <class T>
__global__ void __launch_bounds__(256) basis_start_kernel(int n, Basis<T> V, const T *pb, T *s,
                                                          const Ctl *ctl) {
    constexpr int R = TileGeom<T>::R;
    if (!ctl->active)
        return;
    const T d = static_cast<T>(ctl->den);
    const int padded = V.ntiles * R;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < padded; i += gridDim.x * blockDim.x) {
        V.seg(i / R, 0)[i % R] = i < n ? pb[i] / d : T(0);
        if (i == 0)
            s[0] = T(1);
    }
}
// Zero the pad rows (beyond n) of every segment of the last tile.
template <class T> __global__ void basis_pad_kernel(int n, Basis<T> V) {
    constexpr int R = TileGeom<T>::R;
    const int t = V.ntiles - 1;
    const int rows = n - t * R;
    for (int j = blockIdx.x; j < V.cap1; j += gridDim.x)
        for (int r = rows + threadIdx.x; r < R; r += blockDim.x)
            V.seg(t, j)[r] = T(0);
}

} // namespace spai
