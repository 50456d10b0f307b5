// apsep_range.cu -- single-array APSE engine for sm_103a: persistent,
// warp-independent ranges.
//
// One launch.  Every WARP is an independent worker: it claims a contiguous
// RANGE of warp tiles (32 lanes x IPT keys) from an atomic counter (so every
// range it may wait on belongs to a warp that is already running), keeps its
// own ring of TMA stages, its own answer-chain buffers and its own stack in
// shared memory, and synchronises only with __syncwarp -- there is no
// CTA-wide barrier anywhere.
//
//  Phase 1, per warp tile (the next tiles' 128-byte-swizzled TMA loads stay
//  in flight in the warp's ring):
//   1. in-thread ANSV over IPT consecutive keys in registers (compare
//      ladder) -- the in-thread step of apsepKernelSPT (src/apsep.cuh:2701-2707);
//   2. warp prefix/suffix mins over lane mins (src/apsep.cuh:2709-2730) and
//      the lane chain by warp-uniform pointer jumping (src/apsep.cuh:2734-2752);
//   3. keys unresolved in-thread walk the tile's answer chain in shared
//      memory: a key's next candidate is its in-thread answer, or, for a
//      lane's minimum, the last key of its chain lane -- one pointer walk in
//      place of the reference's spine walk + cross-warp fallback
//      (src/apsep.cuh:2754-2801);
//   4. keys with no answer in the tile query the warp's RANGE STACK: the
//      strict suffix minima of the range's earlier tiles (binary search).
//      This replaces the reference's global min-tree descent
//      (src/apsep.cuh:2952-2996) for every answer inside the range;
//   5. keys with no answer in the range are "deferred" (the range's prefix
//      minima) -- only they wait for the global prefix;
//   6. the tile's answers leave shared memory in one TMA store; the stack
//      takes the tile's strict suffix minima.
//  Then the warp publishes its range minimum as a decoupled look-back
//  aggregate and looks back over earlier ranges (helping them publish their
//  inclusive values) for the exclusive prefix minimum P.  Every wait is
//  bounded and reports ERR_LOOKBACK_TIMEOUT / ERR_TMA_TIMEOUT.
//
//  Phase 2: the deferred keys are non-increasing, so those P qualifies form a
//  prefix (pass A: in order, one monotone cursor, a warp-cooperative search
//  through tile mins / chunk mins / one 32-key row); every later one answers
//  -1 (pass B: straight from the deferred bitmask, whole tiles as one TMA
//  store of -1) -- the reference's prefix-min early-out
//  (src/apsep.cuh:2903-2926).
//
// Compared with the reference's three grid-wide phases there is no
// grid.sync(); the only cross-warp waits are one look-back per range.  Every
// output word is written once (phase 1 skips deferred keys, phase 2 writes
// exactly those).
#include "apsep_device.cuh"
#include "apsep_internal.h"

namespace apsep {

const TileConfig kTileConfigs[kNumTileConfigs] = {
    {8, 16},  // 8 warps per CTA, 512-key warp tiles
    {8, 8},   // 8 warps per CTA, 256-key warp tiles
};

constexpr int kStages = 3;      // TMA ring depth per warp (tiles)
constexpr int kStackCap = 256;  // range-stack entries kept per warp

// Shared memory of one warp.
template <int IPT>
struct WLayout {
    static constexpr int WT = 32 * IPT;                              // keys per warp tile
    static constexpr size_t kV = 0;                                   // T[S][WT], swizzled (TMA dst)
    static constexpr size_t kO = kV + (size_t)kStages * WT * 4;       // int32[WT], swizzled (TMA src)
    static constexpr size_t kNext = kO + (size_t)WT * 4;              // int16[WT]
    static constexpr size_t kStkV = kNext + (size_t)WT * 2;           // T[K]
    static constexpr size_t kStkP = kStkV + (size_t)kStackCap * 4;    // int32[K]
    static constexpr size_t kBar = kStkP + (size_t)kStackCap * 4;     // uint64[S]
    static constexpr size_t kEnd = kBar + (size_t)kStages * 8;
    static constexpr size_t kBytes = (kEnd + 1023) / 1024 * 1024;     // keeps every warp 1024-aligned
    static_assert(kO % 1024 == 0 && (WT * 4) % 1024 == 0, "swizzled buffers need 1024-byte alignment");
};

template <int IPT, int WPC>
constexpr size_t kernel_smem_bytes() { return WLayout<IPT>::kBytes * WPC + 1024; }

__device__ __forceinline__ uint32_t make_tag(uint32_t epoch, uint32_t flag) { return (epoch << 2) | flag; }

// ---------------------------------------------------------------------------
// Warp-cooperative search: the rightmost position p < limit with
// lt(d_in[p], q), or -1 (-2 if the published minima contradict each other).
// Descends a five-level min hierarchy, 32 entries per ballot: groups of 32
// ranges (group_state) -> ranges (range_state) -> tiles of a range
// (tile_min) -> 32-key chunks of a tile (chunk_min) -> keys, so an answer
// any distance away costs a handful of dependent L2 reads.  Every range
// before the one holding limit-1, and every group before that range's group,
// must have published; so must the tiles and chunks below limit-1.  Reads of
// the published arrays go to L2 (ld.cg); the keys are read-only.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T state_key(const uint64_t* w) {
    return KeyTraits<T>::from_bits((uint32_t)__ldcg((const unsigned long long*)w));
}

// Rightmost index i in [lo, hi] (hi - lo < 32) whose minimum qualifies, or -1.
template <typename T, bool INCL, typename Load>
__device__ __forceinline__ int ballot_last(int lo, int hi, T q, Load load) {
    const int lane = threadIdx.x & 31;
    const int i = hi - lane;
    const bool ok = i >= lo && lt<INCL>(load(i), q);
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    return m ? hi - (__ffs(m) - 1) : -1;
}

template <typename T, int B, bool INCL>
__device__ __noinline__ int find_left(T q, int limit, const T* __restrict__ d_in, const T* __restrict__ tile_min,
                                      const T* __restrict__ chunk_min, const RangeArgs& a) {
    constexpr int W = B / 32;
    static_assert(W <= 32, "a tile's chunks must fit one ballot");
    const int lane = threadIdx.x & 31;
    if (limit <= 0) return -1;
    const int last = limit - 1;
    const int t = last / B;
    const int c = (last - t * B) >> 5;
    {  // 1. the row holding limit-1, positions below limit
        const int row = t * B + c * 32;
        const int p = row + lane;
        const bool ok = p < limit && lt<INCL>(__ldg(&d_in[p]), q);
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (m) return row + 31 - __clz(m);
    }
    auto tmin = [&](int i) { return __ldcg(&tile_min[i]); };
    const int tpr = a.tiles_per_range;
    int s = -1;  // tile holding the answer
    int cc = ballot_last<T, INCL>(0, c - 1, q, [&](int i) { return __ldcg(&chunk_min[(size_t)t * W + i]); });
    if (cc >= 0) {
        s = t;
    } else {
        const int R = t / tpr;
        // 3. earlier tiles of the same range
        for (int hi = t - 1; hi >= R * tpr && s < 0; hi -= 32) s = ballot_last<T, INCL>(R * tpr, hi, q, tmin);
        if (s < 0) {
            // 4. earlier ranges of the same group, then 5. earlier groups
            auto rmin = [&](int i) { return state_key<T>(&a.s.range_state[i]); };
            const int g = R >> 5;
            int rr = ballot_last<T, INCL>(g * 32, R - 1, q, rmin);
            if (rr < 0) {
                int gg = -1;
                for (int hi = g - 1; hi >= 0 && gg < 0; hi -= 32)
                    gg = ballot_last<T, INCL>(0, hi, q, [&](int i) { return state_key<T>(&a.s.group_state[i]); });
                if (gg < 0) return -1;
                rr = ballot_last<T, INCL>(gg * 32, min(gg * 32 + 31, a.num_ranges - 1), q, rmin);
                if (rr < 0) return -2;
            }
            const int rt1 = min((rr + 1) * tpr, a.num_tiles) - 1;
            for (int hi = rt1; hi >= rr * tpr && s < 0; hi -= 32) s = ballot_last<T, INCL>(rr * tpr, hi, q, tmin);
            if (s < 0) return -2;
        }
        cc = ballot_last<T, INCL>(0, W - 1, q, [&](int i) { return __ldcg(&chunk_min[(size_t)s * W + i]); });
        if (cc < 0) return -2;
    }
    const int row = s * B + cc * 32;
    const unsigned m = __ballot_sync(0xffffffffu, lt<INCL>(__ldg(&d_in[row + lane]), q));
    return m ? row + 31 - __clz(m) : -2;
}

// ---------------------------------------------------------------------------
// Range minima -> exclusive prefix minima.
//
// Ranges form groups of 32.  Publishing range r: one release store of its
// minimum (range_state) and one acq_rel increment of its group's counter.
// The last range of a group to finish publishes the group minimum
// (group_state) and increments the count of finished groups; the last group
// computes the exclusive prefix over groups (group_pre) and raises one ready
// flag per CTA.  Range r then needs group_pre of its group plus the minima of
// the earlier ranges of its group: two loads, no hot spot.
//
// Every range of a launch is resident when the launch fits the device (the
// grid is sized from occupancy), so the ready flag always comes.  When it
// does not come within a bound (the launch shares the device and some warps
// have not started), range r falls back to waiting only on the groups and
// ranges before it, all of which already run (ids are handed out in start
// order), so no wait depends on a warp that may not start.  Every wait is
// bounded and reports ERR_LOOKBACK_TIMEOUT when it gives up.
// ---------------------------------------------------------------------------
template <typename T>
__device__ void range_publish(int r, uint32_t epoch, T rmin, const RangeArgs& a) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int g = r >> 5;
    const uint32_t tag = (epoch << 2) | FLAG_AGG;
    int last = 0;
    if (lane == 0 && r != a.skip_publish_range) {
        // release: this range's tile words (written by all lanes, ordered by
        // the caller's __syncwarp) before the minimum
        st_release_u64(&a.s.range_state[r], ((uint64_t)tag << 32) | KeyTraits<T>::bits(rmin));
        const int members = min(32, a.num_ranges - g * 32);
        last = atom_add_acq_rel_u32(&a.s.group_cnt[g], 1u) == (uint32_t)(members - 1);
    }
    if (!__shfl_sync(FULL, last, 0)) return;
    // last of its group: every member's range_state is visible (acquire above)
    const int ri = g * 32 + lane;
    T v = ri < a.num_ranges ? state_key<T>(&a.s.range_state[ri]) : KeyTraits<T>::pad();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = KeyTraits<T>::vmin(v, __shfl_xor_sync(FULL, v, o));
    const int ngroups = (a.num_ranges + 31) >> 5;
    int glast = 0;
    if (lane == 0) {
        a.s.group_cnt[g] = 0;  // re-armed for the next run
        st_release_u64(&a.s.group_state[g], ((uint64_t)tag << 32) | KeyTraits<T>::bits(v));
        glast = atom_add_acq_rel_u32(&a.s.ctr->finished, 1u) == (uint32_t)(ngroups - 1);
    }
    if (!__shfl_sync(FULL, glast, 0)) return;
    // last group: exclusive prefix over the groups (at most 128, four per lane)
    T gv[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int gi = lane * 4 + k;
        gv[k] = gi < ngroups ? state_key<T>(&a.s.group_state[gi]) : KeyTraits<T>::pad();
    }
    T tot = KeyTraits<T>::vmin(KeyTraits<T>::vmin(gv[0], gv[1]), KeyTraits<T>::vmin(gv[2], gv[3]));
    T incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl = KeyTraits<T>::vmin(incl, u);
    }
    T run = __shfl_up_sync(FULL, incl, 1);
    if (lane == 0) run = KeyTraits<T>::pad();  // group 0 has no prefix (never read)
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int gi = lane * 4 + k;
        if (gi < ngroups) a.s.group_pre[gi] = KeyTraits<T>::bits(run);
        run = KeyTraits<T>::vmin(run, gv[k]);
    }
    __syncwarp();
    __threadfence();
    for (int c = lane; c < (int)gridDim.x; c += 32) a.s.cta_ready[(size_t)c * kReadyStride] = epoch;
}

template <typename T>
__device__ void range_prefix(int r, uint32_t epoch, const RangeArgs& a, T& p, bool& has_p) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int g = r >> 5;
    const uint32_t tag = (epoch << 2) | FLAG_AGG;
    p = KeyTraits<T>::pad();
    has_p = r > 0;
    if (r == 0) return;
    // 1. the ready flag of this CTA (one line, polled by one lane per warp)
    int ready = 0;
    if (lane == 0) {
        const uint32_t bound = min(a.spin_limit, 1u << 16);
        const uint32_t* f = &a.s.cta_ready[(size_t)blockIdx.x * kReadyStride];
        for (uint32_t s = 0;; s++) {
            if (ld_acquire_u32(f) == epoch) {
                ready = 1;
                break;
            }
            if (s >= bound) break;
            __nanosleep(s < 8 ? 64 : 256);
        }
    }
    __syncwarp();  // lane 0's acquire before the other lanes' loads
    if (__shfl_sync(FULL, ready, 0)) {
        const int ri = g * 32 + lane;
        T m = ri < r ? state_key<T>(&a.s.range_state[ri]) : KeyTraits<T>::pad();
        if (lane == 0 && g > 0) m = KeyTraits<T>::vmin(m, KeyTraits<T>::from_bits(__ldcg(&a.s.group_pre[g])));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = KeyTraits<T>::vmin(m, __shfl_xor_sync(FULL, m, o));
        p = m;
        return;
    }
    // 2. fallback: wait for the earlier groups and the earlier ranges of this group
    for (uint32_t spins = 0;; spins++) {
        bool ok = true;
        T m = KeyTraits<T>::pad();
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int gi = lane * 4 + k;
            if (gi < g) {
                const uint64_t w = ld_acquire_u64(&a.s.group_state[gi]);
                if ((uint32_t)(w >> 32) != tag) ok = false;
                m = KeyTraits<T>::vmin(m, KeyTraits<T>::from_bits((uint32_t)w));
            }
        }
        const int ri = g * 32 + lane;
        if (ri < r) {
            const uint64_t w = ld_acquire_u64(&a.s.range_state[ri]);
            if ((uint32_t)(w >> 32) != tag) ok = false;
            m = KeyTraits<T>::vmin(m, KeyTraits<T>::from_bits((uint32_t)w));
        }
        if (__all_sync(FULL, ok)) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = KeyTraits<T>::vmin(m, __shfl_xor_sync(FULL, m, o));
            p = m;
            return;
        }
        if (spins >= a.spin_limit) {
            if (lane == 0) atomicOr(&a.s.ctr->err, ERR_LOOKBACK_TIMEOUT);
            return;
        }
        __nanosleep(spins < 128 ? 64 : 256);
    }
}

template <typename T, int IPT, int WPC, bool INCL>
__global__ void __launch_bounds__(WPC * 32, (IPT >= 16 ? 2 : 3))
apse_warp_kernel(const __grid_constant__ CUtensorMap map_in, const __grid_constant__ CUtensorMap map_out,
                 const RangeArgs a) {
    using L = WLayout<IPT>;
    constexpr int WT = L::WT;      // keys per warp tile
    constexpr int W = WT / 32;     // 32-key chunks (and TMA rows) per warp tile
    constexpr int TPC = 32 / IPT;  // lanes per chunk
    constexpr int K = kStackCap;
    constexpr int MW = kMaxTileKeys / 32;  // deferred-mask words per tile in global
    static_assert(IPT == 8 || IPT == 16, "IPT must be 8 or 16");
    constexpr unsigned FULL = 0xffffffffu;

    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    unsigned char* wsm =
        (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023) + (size_t)warp * L::kBytes;
    T* sV = (T*)(wsm + L::kV);
    int32_t* O = (int32_t*)(wsm + L::kO);
    int16_t* sNext = (int16_t*)(wsm + L::kNext);
    T* sStkV = (T*)(wsm + L::kStkV);
    int32_t* sStkP = (int32_t*)(wsm + L::kStkP);
    uint64_t* bar = (uint64_t*)(wsm + L::kBar);

    const T* d_in = (const T*)a.d_in;
    T* tile_min_w = (T*)a.s.tile_min;
    T* chunk_min_w = (T*)a.s.chunk_min;
    uint32_t* err = &a.s.ctr->err;

    int r = 0;
    uint32_t epoch = 0;
    if (lane == 0) {
        r = (int)atomicAdd(&a.s.ctr->range_counter, 1u);
        epoch = ld_relaxed_u32(&a.s.ctr->epoch);
        for (int s = 0; s < kStages; s++) mbar_init(&bar[s], 1);
        fence_mbarrier_init();
        fence_proxy_async_smem();
    }
    r = __shfl_sync(FULL, r, 0);
    epoch = __shfl_sync(FULL, epoch, 0);
    __syncwarp();

    if (r < a.num_ranges) {
        const int t0 = r * a.tiles_per_range;
        const int t1 = min(t0 + a.tiles_per_range, a.num_tiles);
        const int ntr = t1 - t0;
        auto tile_full = [&](int t) { return a.tma_rows > 0 && (t + 1) * W <= a.tma_rows; };
        if (lane == 0) {
            for (int i = 0; i < kStages && i < ntr; i++)
                if (tile_full(t0 + i)) {
                    mbar_arrive_expect_tx(&bar[i], (uint32_t)(WT * 4));
                    tma_load_2d(sV + (size_t)i * WT, &map_in, 0, (t0 + i) * W, &bar[i]);
                }
        }
        // Range stack state (warp-uniform).
        int stk_top = 0, stk_lo = 0;
        bool has_rmin = false;
        T rmin = KeyTraits<T>::pad();

        // ======================= phase 1: the range's tiles =======================
        for (int i = 0; i < ntr; i++) {
            const int t = t0 + i;
            const int slot = i % kStages;
            const uint32_t par = (uint32_t)((i / kStages) & 1);
            T* V = sV + (size_t)slot * WT;
            const bool full = tile_full(t);
            const int tile_base = t * WT;
            const int valid_keys = min(WT, a.n - tile_base);
            const bool last_of_range = (i == ntr - 1);

            if (full) {
                if (!mbar_wait_bounded(&bar[slot], par, a.spin_limit) && lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
            } else {
#pragma unroll
                for (int j = 0; j < IPT; j++) {
                    const int e = j * 32 + lane;
                    const int g = tile_base + e;
                    V[swz(e)] = g < a.n ? d_in[g] : KeyTraits<T>::pad();
                }
            }
            if (lane == 0) bulk_wait_read0();  // the previous tile's store has read O
            __syncwarp();

            // ---- 1. in-thread ANSV -----------------------------------------------------
            T v[IPT];
#pragma unroll
            for (int q4 = 0; q4 < IPT / 4; q4++) {
                const uint4 rr = *reinterpret_cast<const uint4*>(&V[swz(lane * IPT + 4 * q4)]);
                v[4 * q4 + 0] = KeyTraits<T>::from_bits(rr.x);
                v[4 * q4 + 1] = KeyTraits<T>::from_bits(rr.y);
                v[4 * q4 + 2] = KeyTraits<T>::from_bits(rr.z);
                v[4 * q4 + 3] = KeyTraits<T>::from_bits(rr.w);
            }
            int res[IPT];
            res[0] = -1;
            {
                // If every lane's keys are monotone (each answers its neighbour, or
                // none does), the in-thread answers follow without the ladder.
                bool adj = true, none = true;
#pragma unroll
                for (int k = 1; k < IPT; k++) {
                    const bool l = lt<INCL>(v[k - 1], v[k]);
                    adj = adj && l;
                    none = none && !l;
                }
                if (__all_sync(FULL, adj || none)) {
#pragma unroll
                    for (int k = 1; k < IPT; k++) res[k] = adj ? k - 1 : -1;
                } else {
#pragma unroll
                    for (int k = 1; k < IPT; k++) {
                        int rk = -1;
#pragma unroll
                        for (int j = 0; j < k; j++)
                            if (lt<INCL>(v[j], v[k])) rk = j;
                        res[k] = rk;
                    }
                }
            }
            T tmin = v[0];
#pragma unroll
            for (int k = 1; k < IPT; k++) tmin = KeyTraits<T>::vmin(tmin, v[k]);
            {
                T cm = tmin;
#pragma unroll
                for (int o = 1; o < TPC; o <<= 1) cm = KeyTraits<T>::vmin(cm, __shfl_xor_sync(FULL, cm, o));
                if ((lane & (TPC - 1)) == 0) __stcg(&chunk_min_w[(size_t)t * W + lane / TPC], cm);
            }
            const int nvalid = min(max(a.n - (tile_base + lane * IPT), 0), IPT);
            unsigned umask = 0;
#pragma unroll
            for (int k = 0; k < IPT; k++)
                if (res[k] < 0 && k < nvalid) umask |= 1u << k;
            {
                const int b = tile_base + lane * IPT;
#pragma unroll
                for (int q4 = 0; q4 < IPT / 4; q4++) {
                    int4 o;
                    o.x = res[4 * q4 + 0] >= 0 ? b + res[4 * q4 + 0] : -1;
                    o.y = res[4 * q4 + 1] >= 0 ? b + res[4 * q4 + 1] : -1;
                    o.z = res[4 * q4 + 2] >= 0 ? b + res[4 * q4 + 2] : -1;
                    o.w = res[4 * q4 + 3] >= 0 ? b + res[4 * q4 + 3] : -1;
                    *reinterpret_cast<int4*>(&O[swz(lane * IPT + 4 * q4)]) = o;
                }
            }

            // ---- 2. warp prefix / suffix mins, lane chain, next-pointers ------------------
            T pre = tmin;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const T nb = __shfl_up_sync(FULL, pre, o);
                if (lane >= o) pre = KeyTraits<T>::vmin(pre, nb);
            }
            const T carry = __shfl_up_sync(FULL, pre, 1);  // min of lanes < this one (lane > 0)
            const T tile_min_t = __shfl_sync(FULL, pre, 31);
            T suf = tmin;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const T nb = __shfl_down_sync(FULL, suf, o);
                if (lane + o < 32) suf = KeyTraits<T>::vmin(suf, nb);
            }
            const T after_w = __shfl_down_sync(FULL, suf, 1);  // min of lanes > this one (lane < 31)
            // Lane chain: the nearest earlier lane whose min qualifies for this lane's
            // min (pointer jumping; invariant: every lane strictly between g and this
            // lane fails lt(., tmin); g only decreases, <= 31 rounds).
            int g = (lane > 0 && lt<INCL>(carry, tmin)) ? lane - 1 : -1;
            for (int round = 0; round < 32; round++) {
                const int src = g >= 0 ? g : lane;
                const T tg = __shfl_sync(FULL, tmin, src);
                const int gg = __shfl_sync(FULL, g, src);
                const bool jump = g >= 0 && !lt<INCL>(tg, tmin);
                if (!__any_sync(FULL, jump)) break;
                if (jump) g = gg;
            }
            {
                // Next candidate after a key that does not qualify for a query: its
                // in-thread answer; for a key with none (the lane's minimum, which then
                // bounds the whole lane) the last key of the chain lane.
                const int jump = g >= 0 ? g * IPT + IPT - 1 : -1;
                uint32_t pk[IPT / 2];
#pragma unroll
                for (int p = 0; p < IPT / 2; p++) {
                    const int a0 = res[2 * p] >= 0 ? lane * IPT + res[2 * p] : jump;
                    const int a1 = res[2 * p + 1] >= 0 ? lane * IPT + res[2 * p + 1] : jump;
                    pk[p] = ((uint32_t)a0 & 0xffffu) | ((uint32_t)a1 << 16);
                }
                uint4* dst = reinterpret_cast<uint4*>(&sNext[lane * IPT]);
                dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                if constexpr (IPT == 16) dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            }
            __syncwarp();

            // ---- 3. keys unresolved in-thread: walk the tile's answer chain -------------
            // Queries (in-thread prefix minima) come in non-increasing order, so the
            // cursor only moves left.  A query is walked only when some key of the
            // tile before this lane qualifies (lt(carry, q)), so the walk ends inside.
            unsigned cu = 0;
            if (umask) {
                unsigned Q = umask & (umask - 1);
                int k = 0;
                T q = v[0];
                if (lane == 0 || !lt<INCL>(carry, q)) {
                    cu = umask;
                } else {
                    int c = lane * IPT - 1;
                    int guard = 2 * WT + 64;
                    T cv = V[swz(c)];
                    while (true) {
                        if (lt<INCL>(cv, q)) {
                            O[swz(lane * IPT + k)] = tile_base + c;
                            if (!Q) break;
                            k = __ffs(Q) - 1;
                            Q &= Q - 1;
                            q = V[swz(lane * IPT + k)];
                            if (!lt<INCL>(carry, q)) {
                                cu = (1u << k) | Q;
                                break;
                            }
                        } else {
                            c = sNext[c];
                            if (c < 0 || --guard < 0) {  // cannot happen while lt(carry, q)
                                atomicOr(err, ERR_INTERNAL);
                                cu = (1u << k) | Q;
                                break;
                            }
                            cv = V[swz(c)];
                        }
                    }
                }
            }

            // ---- 4. keys with no answer in the tile: the range stack ----------------------
            // The stack's top 32 entries sit one per lane; a query is one ballot
            // (entries below a query form a prefix, the top qualifying lane wins).
            const int win_lo = max(stk_lo, stk_top - 32);
            const int widx = win_lo + lane;
            const bool wvalid = widx < stk_top;
            const T wv = wvalid ? sStkV[widx % K] : KeyTraits<T>::pad();
            unsigned dmask = 0;
            if (cu) {
                const T qmax = V[swz(lane * IPT + __ffs(cu) - 1)];
                if (!has_rmin || !lt<INCL>(rmin, qmax)) {
                    dmask = cu;  // nothing in the range qualifies even for the largest
                } else {
                    unsigned m = cu;
                    while (m) {
                        const int k = __ffs(m) - 1;
                        m &= m - 1;
                        const int e = lane * IPT + k;
                        const T q = V[swz(e)];
                        if (!lt<INCL>(rmin, q)) {
                            dmask |= (1u << k) | m;  // queries only shrink from here on
                            break;
                        }
                        int lo = stk_lo, hi = stk_top;  // first stored index that does not qualify
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            if (lt<INCL>(sStkV[mid % K], q)) lo = mid + 1;
                            else hi = mid;
                        }
                        if (lo > stk_lo) O[swz(e)] = sStkP[(lo - 1) % K];
                        else dmask |= 1u << k;  // below the kept part of the stack
                    }
                }
            }
            const int dc = (int)__reduce_add_sync(FULL, (unsigned)__popc(dmask));
            const bool may_cap = stk_lo > 0;

            // ---- 5. stack update ----------------------------------------------------------------
            if (!last_of_range) {
                unsigned fmask = 0;
                const bool has_aft = lane < 31;
                if (!has_aft || lt<false>(tmin, after_w)) {  // else no key here beats every later key
                    bool has_run = has_aft;
                    T run = after_w;
#pragma unroll
                    for (int k = IPT - 1; k >= 0; k--) {
                        if (!has_run || v[k] < run) fmask |= 1u << k;  // strict suffix minimum
                        run = has_run ? KeyTraits<T>::vmin(run, v[k]) : v[k];
                        has_run = true;
                    }
                }
                const int fcnt = __popc(fmask);
                const unsigned fl = __ballot_sync(FULL, fcnt != 0);
                int fpre = 0, total;
                if ((fl & (fl - 1)) == 0) {  // one lane holds every new entry
                    total = __shfl_sync(FULL, fcnt, fl ? __ffs(fl) - 1 : 0);
                } else {
                    fpre = fcnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int nb = __shfl_up_sync(FULL, fpre, o);
                        if (lane >= o) fpre += nb;
                    }
                    total = __shfl_sync(FULL, fpre, 31);
                    fpre -= fcnt;
                }
                // Stored entries below the tile min survive: a prefix of the stack.
                const unsigned below = __ballot_sync(FULL, wvalid && wv < tile_min_t);
                int keep;
                if (below == __ballot_sync(FULL, wvalid)) {
                    keep = stk_top;  // the whole window survives, so does everything under it
                } else if (below || win_lo == stk_lo) {
                    keep = win_lo + __popc(below);
                } else {  // the boundary lies under the window (rare)
                    int lo = stk_lo, hi = win_lo;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (sStkV[mid % K] < tile_min_t) lo = mid + 1;
                        else hi = mid;
                    }
                    keep = lo;
                }
                __syncwarp();  // every lane has read the old stack
                const int newtop = keep + total;
                if (fmask) {
                    int idx = keep + fpre;
#pragma unroll
                    for (int k = 0; k < IPT; k++) {
                        if ((fmask >> k) & 1u) {
                            if (idx >= newtop - K) {
                                sStkV[idx % K] = v[k];
                                sStkP[idx % K] = tile_base + lane * IPT + k;
                            }
                            idx++;
                        }
                    }
                }
                stk_top = newtop;
                stk_lo = max(stk_lo, newtop - K);
            }

            // ---- 6. publish tile data, output -------------------------------------------------
            if (lane == 0) {
                __stcg(&tile_min_w[t], tile_min_t);
                // bit 32: a range prefix exists; bit 33: the stack had dropped entries, so a
                // deferred key of this tile may have its answer inside the range
                __stcg(&a.s.tile_rpre[t], has_rmin ? ((1ull << 32) | (may_cap ? (1ull << 33) : 0ull) |
                                                      KeyTraits<T>::bits(rmin))
                                                   : 0ull);
                __stcg(&a.s.tile_defcnt[t], dc);
            }
            rmin = has_rmin ? KeyTraits<T>::vmin(rmin, tile_min_t) : tile_min_t;
            has_rmin = true;
            fence_proxy_async_smem();
            __syncwarp();
            if (dc == 0) {
                if (full) {
                    if (lane == 0) {
                        tma_store_2d(&map_out, 0, t * W, O);
                        bulk_commit();
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < IPT; j++) {
                        const int e = j * 32 + lane;
                        if (e < valid_keys) a.d_out[tile_base + e] = O[swz(e)];
                    }
                }
            } else if (dc < valid_keys) {
                // mask word w covers keys [32w, 32w + 32): lanes TPC*w .. TPC*w + TPC - 1
                uint32_t mw = 0;
#pragma unroll
                for (int j = 0; j < TPC; j++) {
                    const unsigned part = __shfl_sync(FULL, dmask, (lane % W) * TPC + j);
                    mw |= part << (j * IPT);
                }
#pragma unroll
                for (int j = 0; j < W; j++) {
                    const uint32_t wj = __shfl_sync(FULL, mw, j);
                    const int e = j * 32 + lane;
                    if (e < valid_keys && !((wj >> lane) & 1u)) a.d_out[tile_base + e] = O[swz(e)];
                }
                if (lane < W) __stcg(&a.s.tile_defmask[(size_t)t * MW + lane], mw);
            }
            __syncwarp();
            if (lane == 0 && i + kStages < ntr && tile_full(t + kStages)) {
                mbar_arrive_expect_tx(&bar[slot], (uint32_t)(WT * 4));
                tma_load_2d(V, &map_in, 0, (t + kStages) * W, &bar[slot]);
            }
        }

        // ======================= publish the range, look back =======================
        if (lane == 0) {
            bulk_wait_read0();
            __stcg(&((T*)a.s.range_min)[r], rmin);
        }
        __syncwarp();  // every lane's tile words before lane 0's release in range_publish
        range_publish<T>(r, epoch, rmin, a);
        T P;
        bool has_p;
        range_prefix<T>(r, epoch, a, P, has_p);
        __syncwarp();  // lane 0's acquire before every lane's reads of earlier ranges' words

        // ======================= phase 2: deferred keys =========================
        // "True" deferred keys have no qualifying key in the range before them:
        // the range's prefix minima, non-increasing, so the ones P qualifies form
        // a prefix (pass A, in order, one monotone cursor) and every later one is
        // -1 without reading its key (pass B).  "Capped" ones (tiles whose stack
        // had dropped entries, rpre bit 33) have their answer inside the range.
        const T* tile_min_r = (const T*)a.s.tile_min;
        const T* chunk_min_r = (const T*)a.s.chunk_min;
        const uint32_t* defmask = a.s.tile_defmask;
        int* list = (int*)sV;  // ordered deferred offsets of one tile (the ring is idle now)
        int stop = t1 * WT;    // first position pass B answers -1
        {
            int cur = -1;  // the last answer found (absolute), -1 = none yet
            bool done = !has_p;
            if (done) stop = t0 * WT;
            for (int ib = 0; ib < ntr && !done; ib += 32) {
                const int dcl = ib + lane < ntr ? __ldcg(&a.s.tile_defcnt[t0 + ib + lane]) : 0;
                unsigned nz = __ballot_sync(FULL, dcl != 0);
                while (nz && !done) {
                    const int jt = __ffs(nz) - 1;
                    nz &= nz - 1;
                    const int t = t0 + ib + jt;
                    const int dct = __shfl_sync(FULL, dcl, jt);
                    const int valid = min(WT, a.n - t * WT);
                    const uint64_t rp = __ldcg(&a.s.tile_rpre[t]);
                    const bool has_rp = ((rp >> 32) & 1ull) != 0;
                    const T rpv = KeyTraits<T>::from_bits((uint32_t)rp);
                    const bool dense = dct == valid;
                    if (!dense) {  // ordered list of the tile's deferred offsets
                        const uint32_t wv = lane < W ? __ldcg(&defmask[(size_t)t * MW + lane]) : 0u;
                        const int cnt = __popc(wv);
                        int incl = cnt;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const int nb = __shfl_up_sync(FULL, incl, o);
                            if (lane >= o) incl += nb;
                        }
                        int pos = incl - cnt;
                        uint32_t bits = wv;
                        while (bits) {
                            const int b = __ffs(bits) - 1;
                            bits &= bits - 1;
                            list[pos++] = lane * 32 + b;
                        }
                        __syncwarp();
                    }
                    for (int k0 = 0; k0 < dct && !done; k0 += 32) {
                        const int k = k0 + lane;
                        const bool act = k < dct;
                        const int e = act ? (dense ? k : list[k]) : 0;
                        const T q = act ? __ldg(&d_in[t * WT + e]) : KeyTraits<T>::pad();
                        const bool capped = act && has_rp && lt<INCL>(rpv, q);
                        const bool truedef = act && !capped;
                        const bool want = truedef && lt<INCL>(P, q);
                        unsigned wm = __ballot_sync(FULL, want);
                        const unsigned tm = __ballot_sync(FULL, truedef);
                        const unsigned rest = tm & ~wm;
                        if (rest) {  // the first true key P does not qualify: all later ones are -1
                            const int f = __ffs(rest) - 1;
                            stop = t * WT + __shfl_sync(FULL, e, f);
                            wm &= (1u << f) - 1u;
                            done = true;
                        }
                        unsigned pend = wm;
                        int ans = -1;
                        while (pend) {
                            if (cur >= 0) {
                                const T ac = __ldg(&d_in[cur]);
                                const bool mine = (pend >> lane) & 1u;
                                const unsigned ok = __ballot_sync(FULL, mine && lt<INCL>(ac, q));
                                if (mine && lt<INCL>(ac, q)) ans = cur;
                                pend &= ~ok;
                                if (!pend) break;
                            }
                            const int f = __ffs(pend) - 1;
                            const T qf = __shfl_sync(FULL, q, f);
                            const int found =
                                find_left<T, WT, INCL>(qf, cur >= 0 ? cur : t0 * WT, d_in, tile_min_r, chunk_min_r, a);
                            if (found < 0) {
                                if (lane == 0) atomicOr(err, ERR_INTERNAL);
                            } else {
                                cur = found;
                            }
                            if (lane == f) ans = found < 0 ? -1 : found;
                            pend &= pend - 1;
                        }
                        if ((wm >> lane) & 1u) a.d_out[t * WT + e] = ans;
                        __syncwarp();
                    }
                }
            }
        }
        // pass B
        bool neg_ready = false;
        int dcl = 0;
        uint64_t rpl = 0;
        for (int i = 0; i < ntr; i++) {
            if ((i & 31) == 0) {  // the next 32 tiles' counts and prefixes, one load each
                dcl = i + lane < ntr ? __ldcg(&a.s.tile_defcnt[t0 + i + lane]) : 0;
                rpl = i + lane < ntr ? __ldcg(&a.s.tile_rpre[t0 + i + lane]) : 0ull;
            }
            const int t = t0 + i;
            const int dct = __shfl_sync(FULL, dcl, i & 31);
            if (dct == 0) continue;
            const int valid = min(WT, a.n - t * WT);
            const uint64_t rp = __shfl_sync(FULL, rpl, i & 31);
            const bool may_cap_t = ((rp >> 33) & 1ull) != 0;
            const bool has_rp = ((rp >> 32) & 1ull) != 0;
            const T rpv = KeyTraits<T>::from_bits((uint32_t)rp);
            const bool dense = dct == valid;
            if (!may_cap_t) {
                if (t * WT + valid <= stop) continue;  // pass A answered every key here
                if (dense && t * WT >= stop) {
                    if (tile_full(t)) {
                        if (!neg_ready) {  // O as a -1 source buffer
#pragma unroll
                            for (int j = 0; j < IPT; j++) O[j * 32 + lane] = -1;
                            fence_proxy_async_smem();
                            __syncwarp();
                            neg_ready = true;
                        }
                        if (lane == 0) {
                            tma_store_2d(&map_out, 0, t * W, O);
                            bulk_commit();
                        }
                    } else {
                        for (int e = lane; e < valid; e += 32) a.d_out[t * WT + e] = -1;
                    }
                    continue;
                }
                // -1 at the deferred offsets >= stop, straight from the mask
                if (lane < W) {
                    uint32_t bits = dense ? 0xffffffffu : __ldcg(&defmask[(size_t)t * MW + lane]);
                    const int w0 = lane * 32;
                    if (w0 + 32 > valid) bits &= valid > w0 ? (0xffffffffu >> (32 - (valid - w0))) : 0u;
                    while (bits) {
                        const int b = __ffs(bits) - 1;
                        bits &= bits - 1;
                        const int pos = t * WT + w0 + b;
                        if (pos >= stop) a.d_out[pos] = -1;
                    }
                }
                continue;
            }
            // A tile that may hold capped keys: read every deferred key (rare).
            for (int j0 = 0; j0 < valid; j0 += 32) {
                const int e = j0 + lane;
                bool isdef = false;
                if (e < valid) isdef = dense || ((__ldcg(&defmask[(size_t)t * MW + (e >> 5)]) >> (e & 31)) & 1u);
                const T q = isdef ? __ldg(&d_in[t * WT + e]) : KeyTraits<T>::pad();
                const bool capped = isdef && has_rp && lt<INCL>(rpv, q);
                if (isdef && !capped && t * WT + e >= stop) a.d_out[t * WT + e] = -1;
                unsigned cm = __ballot_sync(FULL, capped);
                while (cm) {
                    const int f = __ffs(cm) - 1;
                    cm &= cm - 1;
                    const T qf = __shfl_sync(FULL, q, f);
                    const int found = find_left<T, WT, INCL>(qf, t * WT, d_in, tile_min_r, chunk_min_r, a);
                    if (found < 0 && lane == 0) atomicOr(err, ERR_INTERNAL);
                    if (lane == f) a.d_out[t * WT + e] = found < 0 ? -1 : found;
                }
            }
        }
        if (lane == 0) bulk_wait_read0();
    }

    // ---- run bookkeeping: the last warp resets the control block --------------------------
    __syncwarp();
    int last = 0;
    if (lane == 0) {
        __threadfence();
        const uint32_t prev = atomicAdd(&a.s.ctr->done, 1u);
        last = prev == gridDim.x * WPC - 1;
        if (last) {
            a.s.ctr->range_counter = 0;
            a.s.ctr->done = 0;
            a.s.ctr->finished = 0;
            a.s.ctr->epoch = epoch >= EPOCH_LIMIT ? 1u : epoch + 1u;
            __threadfence();
        }
    }
    last = __shfl_sync(FULL, last, 0);
    if (last && epoch >= EPOCH_LIMIT) {  // once per 2^30 runs: stale words could alias
        for (int i = lane; i < a.s.max_ranges; i += 32) a.s.range_state[i] = 0;
        for (int i = lane; i < a.s.max_ranges / 32; i += 32) a.s.group_state[i] = 0;
        for (int i = lane; i < kMaxCtas; i += 32) a.s.cta_ready[(size_t)i * kReadyStride] = 0;
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
size_t carve_scratch(void* base, int64_t capacity, RangeScratch* s) {
    const ScratchOffsets o = scratch_offsets(capacity);
    if (base && s) {
        char* b = (char*)base;
        s->ctr = (Counters*)b;
        s->group_cnt = (uint32_t*)(b + o.gcnt);
        s->group_state = (uint64_t*)(b + o.gstate);
        s->group_pre = (uint32_t*)(b + o.gpre);
        s->cta_ready = (uint32_t*)(b + o.ready);
        s->range_state = (uint64_t*)(b + o.state);
        s->range_min = b + o.rmin;
        s->tile_min = b + o.tmin;
        s->tile_rpre = (uint64_t*)(b + o.rpre);
        s->chunk_min = b + o.cmin;
        s->tile_defcnt = (int32_t*)(b + o.dcnt);
        s->tile_defmask = (uint32_t*)(b + o.dmask);
        s->cap_tiles = (int)o.cap_tiles;
        s->max_ranges = kMaxRanges;
    }
    return o.total;
}

namespace {
constexpr int kMaxDev = 64;
int g_warps[kMaxDev][kNumTileConfigs];  // resident warps per device and configuration
}

template <typename T, int IPT, int WPC, bool INCL>
static cudaError_t launch_t(RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo, cudaStream_t st,
                            int max_warps) {
    constexpr size_t smem = kernel_smem_bytes<IPT, WPC>();
    int tpr = (a.num_tiles + max_warps - 1) / max_warps;
    if (tpr < 1) tpr = 1;
    a.tiles_per_range = tpr;
    a.num_ranges = (a.num_tiles + tpr - 1) / tpr;
    const int ctas = (a.num_ranges + WPC - 1) / WPC;
    apse_warp_kernel<T, IPT, WPC, INCL><<<ctas, WPC * 32, smem, st>>>(mi, mo, a);
    return cudaGetLastError();
}

template <typename T, int IPT, int WPC, bool INCL>
static cudaError_t prepare_t(int* ctas_per_sm) {
    constexpr size_t smem = kernel_smem_bytes<IPT, WPC>();
    auto k = apse_warp_kernel<T, IPT, WPC, INCL>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, WPC * 32, smem);
    if (e != cudaSuccess) return e;
    if (*ctas_per_sm == 0 || n < *ctas_per_sm) *ctas_per_sm = n;
    return cudaSuccess;
}

cudaError_t range_prepare(int cfg) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev || cfg < 0 || cfg >= kNumTileConfigs) return cudaErrorInvalidValue;
    int per_sm = 0;
#define P_(IPT, WPC)                                                                   \
    {                                                                                  \
        cudaError_t rr[4] = {prepare_t<int32_t, IPT, WPC, false>(&per_sm),             \
                             prepare_t<int32_t, IPT, WPC, true>(&per_sm),              \
                             prepare_t<float, IPT, WPC, false>(&per_sm),               \
                             prepare_t<float, IPT, WPC, true>(&per_sm)};               \
        for (int q = 0; q < 4; q++)                                                    \
            if (rr[q] != cudaSuccess) return rr[q];                                    \
    }
    switch (cfg) {
    case 0: P_(16, 8); break;
    case 1: P_(8, 8); break;
    }
#undef P_
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int warps = per_sm * sms * kTileConfigs[cfg].wpc;
    if (warps > kMaxRanges) warps = kMaxRanges;
    g_warps[dev][cfg] = warps;
    return cudaSuccess;
}

cudaError_t launch_range(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo,
                         cudaStream_t st) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev || cfg < 0 || cfg >= kNumTileConfigs) return cudaErrorInvalidValue;
    if (g_warps[dev][cfg] == 0) {
        e = range_prepare(cfg);
        if (e != cudaSuccess) return e;
    }
    const int max_warps = g_warps[dev][cfg];
#define L_(IPT, WPC)                                                                        \
    if (dtype == 0)                                                                         \
        return incl ? launch_t<int32_t, IPT, WPC, true>(a, mi, mo, st, max_warps)           \
                    : launch_t<int32_t, IPT, WPC, false>(a, mi, mo, st, max_warps);         \
    else                                                                                    \
        return incl ? launch_t<float, IPT, WPC, true>(a, mi, mo, st, max_warps)             \
                    : launch_t<float, IPT, WPC, false>(a, mi, mo, st, max_warps);
    switch (cfg) {
    case 0: L_(16, 8);
    case 1: L_(8, 8);
    }
#undef L_
    return cudaErrorInvalidValue;
}

}  // namespace apsep
