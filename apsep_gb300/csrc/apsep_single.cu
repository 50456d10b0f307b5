// apsep_single.cu -- single-array APSE tile kernel for sm_103a.
//
// One launch, one pass over the keys.  Each CTA claims the next tile id from
// an atomic counter (launch order, so every tile it may wait on is already
// resident), and for its tile of B = NT*IPT keys:
//
//  1. TMA-loads the tile (cp.async.bulk.tensor, 128-byte swizzle) into shared
//     memory; the partial last tile and unaligned arrays use plain loads.
//  2. In-thread ANSV over IPT consecutive keys in registers (compare ladder),
//     the thread min, chunk mins (32 keys) published to global for later
//     tiles -- this replaces Phase 1's in-thread step and chunk-min publish
//     of apsepKernelSPT (src/apsep.cuh:2686-2730).
//  3. Warp prefix-min over thread mins and the thread-level ANSV chain by
//     warp-uniform pointer jumping (cf. src/apsep.cuh:2709-2752).
//  4. Publishes the tile min as a decoupled look-back aggregate; warp 0 then
//     looks back over predecessors for the exclusive prefix min P_t and
//     publishes the inclusive value.  This replaces Phase 2's min-tree,
//     prefix-min and all grid.sync()s (src/apsep.cuh:2831-2878).  Every
//     wait is bounded and reports ERR_LOOKBACK_TIMEOUT instead of hanging.
//  5. Keys unresolved in-thread walk the tile's answer chain in shared memory
//     (thread chain + in-thread answers, cross-warp via warp mins) -- the
//     spine walk and cross-warp fallback of src/apsep.cuh:2754-2801.
//  6. Keys unresolved in the tile: -1 when !lt(P_t, key) (the reference's
//     prefix-min early-out, src/apsep.cuh:2903-2926), else a warp-cooperative
//     search: nearest earlier tile by tile mins, its chunk mins, then one
//     32-key row of the input (src/apsep.cuh:2952-2996).
//  7. Writes the tile's answers once, from shared memory, with a TMA store.
//
// The reference's Phase 1/2/3 split needs the whole grid between phases; here
// a tile only ever waits on earlier tiles, so no grid-wide barrier exists and
// every output word is written exactly once, in one coalesced store.
#include "apsep_device.cuh"
#include "apsep_internal.h"

namespace apsep {

const TileConfig kTileConfigs[kNumTileConfigs] = {
    {256, 16},  // 4096 keys / tile
    {256, 8},   // 2048 keys / tile
    {512, 8},   // 4096 keys / tile
};

template <typename T, int NT, int IPT>
struct SmemLayout {
    static constexpr int B = NT * IPT;
    static constexpr int NW = NT / 32;
    static constexpr size_t kV = 0;                                 // T[B], swizzled
    static constexpr size_t kO = kV + (size_t)B * 4;                // int32[B], swizzled
    static constexpr size_t kNext = kO + (size_t)B * 4;             // int16[B] (later: deep list)
    static constexpr size_t kTmin = kNext + (size_t)B * 2;          // T[NT]
    static constexpr size_t kChain = kTmin + (size_t)NT * 4;        // int32[NT]
    static constexpr size_t kWmin = kChain + (size_t)NT * 4;        // T[NW]
    static constexpr size_t kMisc = (kWmin + (size_t)NW * 4 + 15) & ~(size_t)15;
    static constexpr size_t kEnd = kMisc + 64;
    static constexpr size_t kBytes = kEnd + 1024;  // + alignment slack
};

struct alignas(16) Misc {
    uint64_t bar;
    int tile;
    int full;
    uint32_t epoch;
    uint32_t p_bits;
    int has_p;
    int deep_count;
    int last_cta;
};

__device__ __forceinline__ uint32_t make_tag(uint32_t epoch, uint32_t flag) { return (epoch << 2) | flag; }

// ---------------------------------------------------------------------------
// Warp-cooperative search for the rightmost key before tile t that qualifies
// for q (lt(key, q)).  Precondition: lt(P_t, q), so an answer exists; every
// tile < t has published tile_min / chunk_min (guaranteed after t's
// look-back).  Reads go to L2 (ld.cg): the arrays are written by other SMs.
// ---------------------------------------------------------------------------
template <typename T, int B, bool INCL>
__device__ __noinline__ int deep_search(T q, int t, const T* __restrict__ tile_min,
                                        const T* __restrict__ chunk_min, const T* __restrict__ d_in,
                                        uint32_t* err) {
    constexpr int W = B / 32;
    const int lane = threadIdx.x & 31;
    int s = -1;
    for (int base = t - 1; base >= 0; base -= 32) {
        const int idx = base - lane;
        const T tm = idx >= 0 ? __ldcg(&tile_min[idx]) : KeyTraits<T>::pad();
        const unsigned m = __ballot_sync(0xffffffffu, idx >= 0 && lt<INCL>(tm, q));
        if (m) {
            s = base - (__ffs(m) - 1);
            break;
        }
    }
    if (s < 0) {
        if (lane == 0) atomicOr(err, ERR_INTERNAL);
        return -1;
    }
    int c = -1;
    for (int g = (W + 31) / 32 - 1; g >= 0; g--) {
        const int ci = g * 32 + lane;
        const T cm = ci < W ? __ldcg(&chunk_min[(size_t)s * W + ci]) : KeyTraits<T>::pad();
        const unsigned m = __ballot_sync(0xffffffffu, ci < W && lt<INCL>(cm, q));
        if (m) {
            c = g * 32 + 31 - __clz(m);
            break;
        }
    }
    if (c < 0) {
        if (lane == 0) atomicOr(err, ERR_INTERNAL);
        return -1;
    }
    const T x = __ldg(&d_in[(size_t)s * B + (size_t)c * 32 + lane]);
    const unsigned m = __ballot_sync(0xffffffffu, lt<INCL>(x, q));
    if (!m) {
        if (lane == 0) atomicOr(err, ERR_INTERNAL);
        return -1;
    }
    return s * B + c * 32 + 31 - __clz(m);
}

// ---------------------------------------------------------------------------
// Decoupled look-back for the exclusive prefix min of tile t (one full warp).
// Publishes tile t's inclusive value.  Returns has_p=false only for t == 0.
// ---------------------------------------------------------------------------
template <typename T, bool INCL>
__device__ __forceinline__ void lookback(int t, uint32_t epoch, T tile_min_t, const SingleArgs& a, T& p,
                                         bool& has_p) {
    const int lane = threadIdx.x & 31;
    uint64_t* state = a.s.state;
    T acc = KeyTraits<T>::pad();
    bool has = false;
    if (t > 0) {
        uint32_t spins = 0;
        int base = t - 1;
        while (true) {
            const int idx = base - lane;
            uint32_t flag = FLAG_INCL;  // before tile 0: an empty inclusive prefix
            uint32_t vbits = 0;
            if (idx >= 0) {
                const uint64_t w = ld_acquire_u64(&state[idx]);
                const uint32_t tag = (uint32_t)(w >> 32);
                flag = (tag >> 2) == epoch ? (tag & 3u) : 0u;
                vbits = (uint32_t)w;
            }
            const unsigned incl = __ballot_sync(0xffffffffu, flag == FLAG_INCL);
            const unsigned ready = __ballot_sync(0xffffffffu, flag != 0u);
            const int fi = incl ? __ffs(incl) - 1 : 32;
            const unsigned need = fi >= 31 ? 0xffffffffu : ((2u << fi) - 1u);
            if ((ready & need) != need) {
                if (++spins > a.spin_limit) {
                    if (lane == 0) atomicOr(&a.s.ctr->err, ERR_LOOKBACK_TIMEOUT);
                    break;
                }
                if (spins > 8) __nanosleep(spins < 256 ? 32 : 256);
                continue;
            }
            const bool contrib = lane <= fi && idx >= 0;
            T v = contrib ? KeyTraits<T>::from_bits(vbits) : KeyTraits<T>::pad();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v = KeyTraits<T>::vmin(v, __shfl_xor_sync(0xffffffffu, v, o));
            if (__any_sync(0xffffffffu, contrib)) {
                acc = has ? KeyTraits<T>::vmin(acc, v) : v;
                has = true;
            }
            if (fi < 32) break;
            base -= 32;
        }
        if (lane == 0 && t != a.skip_publish_tile) {
            const T incl_v = has ? KeyTraits<T>::vmin(acc, tile_min_t) : tile_min_t;
            st_release_u64(&state[t], ((uint64_t)make_tag(epoch, FLAG_INCL) << 32) |
                                          KeyTraits<T>::bits(incl_v));
        }
    }
    p = acc;
    has_p = has;
}

template <typename T, int NT, int IPT, bool INCL>
__global__ void __launch_bounds__(NT, (NT >= 512 ? 2 : 3))
apse_tile_kernel(const __grid_constant__ CUtensorMap map_in, const __grid_constant__ CUtensorMap map_out,
                 const SingleArgs a) {
    using L = SmemLayout<T, NT, IPT>;
    constexpr int B = NT * IPT;
    constexpr int NW = NT / 32;
    constexpr int W = B / 32;
    constexpr int TPC = 32 / IPT;  // threads per 32-key chunk
    constexpr int ROWS = B / 32;   // TMA box rows (128-byte rows)
    static_assert(IPT == 4 || IPT == 8 || IPT == 16, "IPT must be 4, 8 or 16");
    static_assert(ROWS <= 256, "TMA box height is at most 256 rows");
    static_assert(B <= 32768, "tile-relative indices are int16");

    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    T* sV = (T*)(sm + L::kV);
    int32_t* sO = (int32_t*)(sm + L::kO);
    int16_t* sNext = (int16_t*)(sm + L::kNext);
    int16_t* sDeep = sNext;  // reused once the in-tile walks are done
    T* sTmin = (T*)(sm + L::kTmin);
    int32_t* sChain = (int32_t*)(sm + L::kChain);
    T* sWmin = (T*)(sm + L::kWmin);
    Misc* misc = (Misc*)(sm + L::kMisc);

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const T* d_in = (const T*)a.d_in;
    const T* tile_min_g = (const T*)a.s.tile_min;
    T* tile_min_w = (T*)a.s.tile_min;
    T* chunk_min_w = (T*)a.s.chunk_min;
    uint32_t* err = &a.s.ctr->err;

    // ---- 0. claim a tile, start its TMA load --------------------------------
    if (tid == 0) {
        const int t = (int)atomicAdd(&a.s.ctr->tile_counter, 1u);
        misc->tile = t;
        misc->epoch = ld_relaxed_u32(&a.s.ctr->epoch);
        misc->deep_count = 0;
        const bool full = a.tma_rows > 0 && (t + 1) * ROWS <= a.tma_rows;
        misc->full = full;
        if (full) {
            mbar_init(&misc->bar, 1);
            fence_mbarrier_init();
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&misc->bar, (uint32_t)(B * 4));
            tma_load_2d(sV, &map_in, 0, t * ROWS, &misc->bar);
        }
    }
    __syncthreads();
    const int t = misc->tile;
    const bool full = misc->full != 0;
    const uint32_t epoch = misc->epoch;
    const int tile_base = t * B;

    // ---- 1. keys into shared memory ------------------------------------------
    if (full) {
        if (!mbar_wait_bounded(&misc->bar, 0, a.spin_limit)) {
            if (tid == 0) atomicOr(err, ERR_TMA_TIMEOUT);
        }
    } else {
#pragma unroll
        for (int i = 0; i < IPT; i++) {
            const int e = i * NT + tid;
            const int g = tile_base + e;
            sV[swz(e)] = g < a.n ? d_in[g] : KeyTraits<T>::pad();
        }
        __syncthreads();
    }

    // ---- 2. in-thread ANSV ------------------------------------------------------
    T v[IPT];
#pragma unroll
    for (int q4 = 0; q4 < IPT / 4; q4++) {
        const uint4 r = *reinterpret_cast<const uint4*>(&sV[swz(tid * IPT + 4 * q4)]);
        v[4 * q4 + 0] = KeyTraits<T>::from_bits(r.x);
        v[4 * q4 + 1] = KeyTraits<T>::from_bits(r.y);
        v[4 * q4 + 2] = KeyTraits<T>::from_bits(r.z);
        v[4 * q4 + 3] = KeyTraits<T>::from_bits(r.w);
    }
    int res[IPT];
    res[0] = -1;
#pragma unroll
    for (int k = 1; k < IPT; k++) {
        int r = -1;
#pragma unroll
        for (int j = 0; j < k; j++)
            if (lt<INCL>(v[j], v[k])) r = j;
        res[k] = r;
    }
    T tmin = v[0];
#pragma unroll
    for (int k = 1; k < IPT; k++) tmin = KeyTraits<T>::vmin(tmin, v[k]);

    // chunk mins first, so they are long performed by the time of the fence
    {
        T cm = tmin;
#pragma unroll
        for (int o = 1; o < TPC; o <<= 1) cm = KeyTraits<T>::vmin(cm, __shfl_xor_sync(0xffffffffu, cm, o));
        if ((lane & (TPC - 1)) == 0) __stcg(&chunk_min_w[(size_t)t * W + tid / TPC], cm);
    }

    const int nvalid = min(max(a.n - (tile_base + tid * IPT), 0), IPT);
    unsigned umask = 0;
#pragma unroll
    for (int k = 0; k < IPT; k++)
        if (res[k] < 0 && k < nvalid) umask |= 1u << k;

    // in-thread answers -> output staging (absolute), next-pointers (tile-relative)
#pragma unroll
    for (int q4 = 0; q4 < IPT / 4; q4++) {
        int4 o;
        o.x = res[4 * q4 + 0] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 0] : -1;
        o.y = res[4 * q4 + 1] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 1] : -1;
        o.z = res[4 * q4 + 2] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 2] : -1;
        o.w = res[4 * q4 + 3] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 3] : -1;
        *reinterpret_cast<int4*>(&sO[swz(tid * IPT + 4 * q4)]) = o;
    }
    {
        uint32_t pk[IPT / 2];
#pragma unroll
        for (int p = 0; p < IPT / 2; p++) {
            const int a0 = res[2 * p] >= 0 ? tid * IPT + res[2 * p] : -1;
            const int a1 = res[2 * p + 1] >= 0 ? tid * IPT + res[2 * p + 1] : -1;
            pk[p] = ((uint32_t)a0 & 0xffffu) | ((uint32_t)a1 << 16);
        }
        uint32_t* dst = reinterpret_cast<uint32_t*>(&sNext[tid * IPT]);
        if constexpr (IPT == 16) {
            reinterpret_cast<uint4*>(dst)[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            reinterpret_cast<uint4*>(dst)[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        } else if constexpr (IPT == 8) {
            reinterpret_cast<uint4*>(dst)[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        } else {
            reinterpret_cast<uint2*>(dst)[0] = make_uint2(pk[0], pk[1]);
        }
    }

    // ---- 3. warp prefix-min and thread-level chain ---------------------------------
    T incl_scan = tmin;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T nb = __shfl_up_sync(0xffffffffu, incl_scan, o);
        if (lane >= o) incl_scan = KeyTraits<T>::vmin(incl_scan, nb);
    }
    const T carry = __shfl_up_sync(0xffffffffu, incl_scan, 1);  // valid for lane > 0
    int g = (lane > 0 && lt<INCL>(carry, tmin)) ? lane - 1 : -1;
    // Pointer jumping: invariant "every lane strictly between g and this lane
    // fails lt(., tmin)"; g only decreases, so <= 31 rounds.
    for (int round = 0; round < 32; round++) {
        const int src = g >= 0 ? g : lane;
        const T tg = __shfl_sync(0xffffffffu, tmin, src);
        const int gg = __shfl_sync(0xffffffffu, g, src);
        const bool jump = g >= 0 && !lt<INCL>(tg, tmin);
        if (!__any_sync(0xffffffffu, jump)) break;
        if (jump) g = gg;
    }
    sTmin[tid] = tmin;
    sChain[tid] = g >= 0 ? warp * 32 + g : -1;
    if (lane == 31) sWmin[warp] = incl_scan;
    if ((lane & (TPC - 1)) == 0) __threadfence();  // chunk mins before the tile's flag
    __syncthreads();  // S1

    // ---- 4. publish the aggregate; warp 0 looks back ----------------------------
    T tile_min_t = sWmin[0];
#pragma unroll
    for (int w = 1; w < NW; w++) tile_min_t = KeyTraits<T>::vmin(tile_min_t, sWmin[w]);
    if (warp == 0) {
        if (lane == 0) {
            __stcg(&tile_min_w[t], tile_min_t);
            if (t != a.skip_publish_tile) {
                const uint32_t flag = t == 0 ? FLAG_INCL : FLAG_AGG;
                st_release_u64(&a.s.state[t],
                               ((uint64_t)make_tag(epoch, flag) << 32) | KeyTraits<T>::bits(tile_min_t));
            }
        }
        T p;
        bool has_p;
        lookback<T, INCL>(t, epoch, tile_min_t, a, p, has_p);
        if (lane == 0) {
            misc->p_bits = KeyTraits<T>::bits(p);
            misc->has_p = has_p ? 1 : 0;
        }
        __threadfence();  // acquired predecessor data -> visible to the CTA after S2
    }

    // ---- 5. keys unresolved in-thread: walk the tile's answer chain -------------------
    // x = min of all keys before this thread in the tile.
    bool has_x = lane > 0;
    T x = carry;
    for (int w = 0; w < warp; w++) {
        x = has_x ? KeyTraits<T>::vmin(x, sWmin[w]) : sWmin[w];
        has_x = true;
    }
    unsigned cu = 0;  // keys with no answer inside the tile
    unsigned Q = umask;
    if (Q && (!has_x || !lt<INCL>(x, v[0]))) {  // v[0] is the largest query
        cu = Q;
        Q = 0;
    }
    if (Q) {
        int j = tid - 1;  // candidate thread
        int c = -1;       // candidate key (tile-relative) inside thread j
        T cv = v[0];
        bool emode = false;
        int k = __ffs(Q) - 1;
        Q &= Q - 1;
        T q = v[0];
        int guard = 4 * B + 4 * NT + 64;
        while (true) {
            if (--guard < 0) {
                atomicOr(err, ERR_INTERNAL);
                cu |= (1u << k) | Q;
                break;
            }
            if (!emode) {
                if (j < 0) {
                    cu |= (1u << k) | Q;
                    break;
                }
                if (lt<INCL>(sTmin[j], q)) {
                    emode = true;
                    if (c < 0 || (c / IPT) != j) c = j * IPT + IPT - 1;
                    cv = sV[swz(c)];
                } else {
                    int cj = sChain[j];
                    if (cj < 0) {
                        for (int w = (j >> 5) - 1; w >= 0; w--)
                            if (lt<INCL>(sWmin[w], q)) {
                                cj = w * 32 + 31;
                                break;
                            }
                    }
                    j = cj;
                    c = -1;
                }
            } else {
                if (lt<INCL>(cv, q)) {
                    sO[swz(tid * IPT + k)] = tile_base + c;
                    if (!Q) break;
                    k = __ffs(Q) - 1;
                    Q &= Q - 1;
                    q = sV[swz(tid * IPT + k)];
                    emode = false;  // re-check thread j against the smaller query
                } else {
                    const int nx = sNext[c];
                    if (nx < 0) {  // cannot happen while lt(tmin_j, q); be safe
                        atomicOr(err, ERR_INTERNAL);
                        emode = false;
                        j = -1;
                    } else {
                        c = nx;
                        cv = sV[swz(c)];
                    }
                }
            }
        }
    }
    __syncthreads();  // S2: P_t known, walks done (sNext free for the deep list)

    // ---- 6. keys unresolved in the tile ------------------------------------------------
    if (cu) {
        const bool has_p = misc->has_p != 0;
        const T p = KeyTraits<T>::from_bits(misc->p_bits);
        const int k0 = __ffs(cu) - 1;
        const T qmax = sV[swz(tid * IPT + k0)];
        if (!has_p || !lt<INCL>(p, qmax)) {
            // every one answers -1 (the largest one already fails)
#pragma unroll
            for (int q4 = 0; q4 < IPT / 4; q4++) {
                const unsigned m4 = (cu >> (4 * q4)) & 0xfu;
                if (m4) {
                    int4* dst = reinterpret_cast<int4*>(&sO[swz(tid * IPT + 4 * q4)]);
                    int4 o = *dst;
                    if (m4 & 1u) o.x = -1;
                    if (m4 & 2u) o.y = -1;
                    if (m4 & 4u) o.z = -1;
                    if (m4 & 8u) o.w = -1;
                    *dst = o;
                }
            }
        } else {
            unsigned m = cu;
            while (m) {
                const int k = __ffs(m) - 1;
                m &= m - 1;
                const int e = tid * IPT + k;
                const T q = sV[swz(e)];
                if (lt<INCL>(p, q)) {
                    const int slot = atomicAdd(&misc->deep_count, 1);
                    sDeep[slot] = (int16_t)e;
                } else {
                    sO[swz(e)] = -1;
                }
            }
        }
    }
    __syncthreads();  // S3

    // ---- 7. warp-cooperative searches beyond the tile -----------------------------
    {
        const int nd = misc->deep_count;
        for (int i = warp; i < nd; i += NW) {
            const int e = sDeep[i];
            const T q = sV[swz(e)];
            const int ans = deep_search<T, B, INCL>(q, t, tile_min_g, (const T*)a.s.chunk_min, d_in, err);
            if (lane == 0) sO[swz(e)] = ans;
        }
    }

    // ---- 8. write the tile's answers once ------------------------------------------
    fence_proxy_async_smem();
    __syncthreads();  // S4
    if (full) {
        if (tid == 0) {
            tma_store_2d(&map_out, 0, t * ROWS, sO);
            bulk_commit();
        }
    } else {
#pragma unroll
        for (int i = 0; i < IPT; i++) {
            const int e = i * NT + tid;
            const int gi = tile_base + e;
            if (gi < a.n) a.d_out[gi] = sO[swz(e)];
        }
    }

    // ---- 9. run bookkeeping: the last CTA resets the control block ----------------------
    if (tid == 0) {
        if (full) bulk_wait_read0();
        __threadfence();
        const uint32_t prev = atomicAdd(&a.s.ctr->done, 1u);
        misc->last_cta = prev == gridDim.x - 1 ? 1 : 0;
        if (prev == gridDim.x - 1) {
            a.s.ctr->tile_counter = 0;
            a.s.ctr->done = 0;
            a.s.ctr->epoch = epoch >= EPOCH_LIMIT ? 1u : epoch + 1u;
            __threadfence();
        }
    }
    if (epoch >= EPOCH_LIMIT) {  // once per 2^30 runs: stale words could alias
        __syncthreads();
        if (misc->last_cta)
            for (int i = tid; i < a.s.cap_tiles; i += NT) a.s.state[i] = 0;
    }
}

// ---------------------------------------------------------------------------
// Host-side dispatch.
// ---------------------------------------------------------------------------
template <typename T, int NT, int IPT, bool INCL>
static cudaError_t launch_t(const SingleArgs& a, const CUtensorMap& mi, const CUtensorMap& mo, cudaStream_t st) {
    constexpr size_t smem = SmemLayout<T, NT, IPT>::kBytes;
    apse_tile_kernel<T, NT, IPT, INCL><<<a.num_tiles, NT, smem, st>>>(mi, mo, a);
    return cudaGetLastError();
}

template <typename T, int NT, int IPT, bool INCL>
static cudaError_t prepare_t() {
    constexpr size_t smem = SmemLayout<T, NT, IPT>::kBytes;
    return cudaFuncSetAttribute(apse_tile_kernel<T, NT, IPT, INCL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

#define APSEP_FOR_CFG(CFG, MACRO)                  \
    switch (CFG) {                                 \
    case 0: MACRO(256, 16); break;                 \
    case 1: MACRO(256, 8); break;                  \
    case 2: MACRO(512, 8); break;                  \
    default: return cudaErrorInvalidValue;         \
    }

cudaError_t launch_single(int dtype, int incl, int cfg, const SingleArgs& a, const CUtensorMap& mi,
                          const CUtensorMap& mo, cudaStream_t st) {
#define L_(NT, IPT)                                                                   \
    if (dtype == 0)                                                                   \
        return incl ? launch_t<int32_t, NT, IPT, true>(a, mi, mo, st)                 \
                    : launch_t<int32_t, NT, IPT, false>(a, mi, mo, st);               \
    else                                                                              \
        return incl ? launch_t<float, NT, IPT, true>(a, mi, mo, st)                   \
                    : launch_t<float, NT, IPT, false>(a, mi, mo, st);
    APSEP_FOR_CFG(cfg, L_)
#undef L_
    return cudaErrorInvalidValue;
}

cudaError_t single_prepare(int cfg) {
    cudaError_t e = cudaSuccess;
#define P_(NT, IPT)                                                            \
    {                                                                          \
        cudaError_t r[4] = {prepare_t<int32_t, NT, IPT, false>(), prepare_t<int32_t, NT, IPT, true>(), \
                            prepare_t<float, NT, IPT, false>(), prepare_t<float, NT, IPT, true>()};   \
        for (int i = 0; i < 4; i++)                                            \
            if (r[i] != cudaSuccess) e = r[i];                                 \
    }
    APSEP_FOR_CFG(cfg, P_)
#undef P_
    return e;
}

size_t single_smem_bytes(int cfg) {
    switch (cfg) {
    case 0: return SmemLayout<int32_t, 256, 16>::kBytes;
    case 1: return SmemLayout<int32_t, 256, 8>::kBytes;
    case 2: return SmemLayout<int32_t, 512, 8>::kBytes;
    default: return 0;
    }
}

}  // namespace apsep
