// apsep_range_kernel.cuh -- the APSE engine for sm_103a: persistent,
// warp-independent ranges (single arrays and batches of segments).
//
// One launch.  Every WARP is an independent worker on a contiguous RANGE of
// warp tiles (32 lanes x IPT keys; the first warp of each CTA claims the
// CTA's consecutive ranges with one atomic, in CTA start order), with its own
// ring of TMA stages, its own answer buffers and its own stack in shared
// memory.  One __syncthreads publishes the claim; after it the warps
// synchronise only with __syncwarp.
//
//  Phase 1, per warp tile (the next tiles' 128-byte-swizzled TMA loads stay
//  in flight in the warp's ring):
//   1. in-thread answers over IPT consecutive keys in registers (compare
//      ladder) -- the in-thread step of apsepKernelSPT (src/apsep.cuh:2701-2707);
//   2. warp prefix minima over lane minima (src/apsep.cuh:2709-2730);
//   3. each key without an in-thread answer is classified: answered by an
//      earlier lane of the tile (X), by an earlier tile of the range (S), or by
//      nothing in the range (deferred);
//   4. X keys, spread evenly over the lanes, find their lane by binary lifting
//      over a 5-level table of lane minima held in registers and their key by
//      binary search over that lane's suffix minima -- a fixed number of
//      steps in place of the reference's warp-uniform pointer jumping, spine
//      walk and cross-warp fallback (src/apsep.cuh:2734-2801);
//   5. S keys search the warp's RANGE STACK (strict suffix minima of the
//      range's earlier tiles; its top 32 entries one per lane, a shuffle
//      search, binary search below), in place of the reference's global
//      min-tree descent (src/apsep.cuh:2952-2996) for every answer inside the
//      range;
//   6. the whole tile leaves shared memory in one TMA store, deferred keys as
//      -1; the stack takes the tile's strict suffix minima.
//  Then the warp publishes its range minimum and the top of its stack, and
//  reads the exclusive prefix minimum P of the earlier ranges (one handshake
//  per launch, see range_publish).  Every wait is bounded and reports
//  ERR_LOOKBACK_TIMEOUT / ERR_TMA_TIMEOUT.
//
//  Phase 2 touches only the flagged keys.  Deferred keys are the range's
//  prefix minima, non-increasing, so the ones P qualifies form a prefix (the
//  reference's prefix-min early-out, src/apsep.cuh:2903-2926); each finds
//  the nearest earlier range whose minimum qualifies and its answer at the
//  top of that range's published stack, all lanes in parallel.  Everything
//  else (stacks that dropped entries, lists that overflowed) falls back to a
//  warp-cooperative search down the min hierarchy (find_left).
#pragma once
#include "apsep_device.cuh"
#include "apsep_internal.h"

namespace apsep {

constexpr int kStages = 3;      // TMA ring depth per warp (tiles)
constexpr int kStackCap = 64;   // range-stack entries kept per warp
constexpr int kXQueries = 3;    // cross-lane queries per lane and round (32 * 3 keys per round)
constexpr int kDefCap = 64;     // deferred keys listed in shared memory per range
constexpr int kCapCap = 16;     // capped keys listed in shared memory per range

// Shared memory of one warp (KB: bytes per key).
template <int IPT, int KB = 4>
struct WLayout {
    static constexpr int WT = 32 * IPT;                              // keys per warp tile
    static constexpr size_t kV = 0;                                   // T[S][WT], swizzled (TMA dst)
    static constexpr size_t kO = kV + (size_t)kStages * WT * KB;      // int32[WT], swizzled (TMA src)
    static constexpr size_t kSM = kO + (size_t)WT * 4;                // T[WT], swizzled: lane suffix minima
    static constexpr size_t kList = kSM + (size_t)WT * KB;            // int16[WT]: X keys in order
    static constexpr size_t kStkV = kList + (size_t)WT * 2;           // T[K]
    static constexpr size_t kStkP = kStkV + (size_t)kStackCap * KB;   // int32[K]
    static constexpr size_t kDefP = kStkP + (size_t)kStackCap * 4;    // int32[kDefCap]
    static constexpr size_t kDefV = kDefP + (size_t)kDefCap * 4;      // T[kDefCap]
    static constexpr size_t kCapP = kDefV + (size_t)kDefCap * KB;     // int32[kCapCap]
    static constexpr size_t kCapS = kCapP + (size_t)kCapCap * 4;      // int32[kCapCap]: segment starts
    static constexpr size_t kBar = (kCapS + (size_t)kCapCap * 4 + 7) / 8 * 8;  // uint64[S]
    static constexpr size_t kEnd = kBar + (size_t)kStages * 8;
    static constexpr size_t kBytes = (kEnd + 1023) / 1024 * 1024;     // keeps every warp 1024-aligned
    static_assert(kO % 1024 == 0 && kSM % 1024 == 0 && (WT * KB) % 1024 == 0,
                  "swizzled buffers need 1024-byte alignment");
    static_assert(kStkV % 8 == 0 && kDefV % 8 == 0, "8-byte keys need 8-byte aligned arrays");
};

template <int IPT, int WPC, int KB = 4>
constexpr size_t kernel_smem_bytes() { return WLayout<IPT, KB>::kBytes * WPC + 1024 + 64; }  // + CTA words

__device__ __forceinline__ uint32_t make_tag(uint32_t epoch, uint32_t flag) { return (epoch << 2) | flag; }

// Key of a group word (the low half of an atomic minimum over ordered keys).
template <typename T>
__device__ __forceinline__ T group_key(const uint64_t* w) {
    return KeyTraits<T>::from_ord((uint32_t)__ldcg((const unsigned long long*)w));
}

// Key of a range word (tag << 32 | key bits).
template <typename T>
__device__ __forceinline__ T state_key(const uint64_t* w) {
    return KeyTraits<T>::from_bits((uint32_t)__ldcg((const unsigned long long*)w));
}

// The published minimum of range i (8-byte keys keep it beside the tag word).
template <typename T>
__device__ __forceinline__ T range_min(const RangeArgs& a, int i) {
    if constexpr (sizeof(T) == 8)
        return KeyTraits<T>::from_bits((uint64_t)__ldcg((const unsigned long long*)&a.s.range_key[i]));
    else
        return state_key<T>(&a.s.range_state[i]);
}

// The minimum of group g (32 ranges), every range of which has published:
// its atomic word for 4-byte keys, the minimum of its ranges' words for
// 8-byte keys (no 64-bit key fits beside a tag in one atomic word).
template <typename T>
__device__ __forceinline__ T group_min_of(const RangeArgs& a, int g) {
    if constexpr (sizeof(T) == 8) {
        T m = KeyTraits<T>::pad();
        const int e = min(32 * g + 32, a.num_ranges);
        for (int i = 32 * g; i < e; i++) m = KeyTraits<T>::vmin(m, range_min<T>(a, i));
        return m;
    } else {
        return group_key<T>(&a.s.group_min[g]);
    }
}

// ---------------------------------------------------------------------------
// Warp-cooperative search: the rightmost position p < limit with
// lt(d_in[p], q), or -1 (-2 if the published minima contradict each other).
// Descends a five-level min hierarchy, 32 entries per ballot: groups of 32
// ranges (group_min) -> ranges (range_state) -> tiles of a range
// (tile_min) -> 32-key chunks of a tile (chunk_min) -> keys, so an answer
// any distance away costs a handful of dependent L2 reads.  Every range
// before the one holding limit-1, and every group before that range's group,
// must have published; so must the tiles and chunks below limit-1.  Reads of
// the published arrays go to L2 (ld.cg); the keys are read-only.
// ---------------------------------------------------------------------------
// Rightmost index i in [lo, hi] (hi - lo < 32) whose minimum qualifies, or -1.
template <typename T, bool INCL, typename Load>
__device__ __forceinline__ int ballot_last(int lo, int hi, T q, Load load) {
    const int lane = threadIdx.x & 31;
    const int i = hi - lane;
    const bool ok = i >= lo && lt<INCL>(load(i), q);
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    return m ? hi - (__ffs(m) - 1) : -1;
}

// Exclusive prefix sum over the warp's lanes of a count c, and the total.
__device__ __forceinline__ int warp_excl_sum(int c, int& total) {
    int x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int nb = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)(threadIdx.x & 31) >= o) x += nb;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - c;
}

// Segmented runs: the segment holding position pos -- the largest s < nseg
// with off[s] <= pos (off[0] = 0 <= pos).  Warp-cooperative, 32 candidates
// per step, so about log32(nseg) dependent reads.
static __device__ __noinline__ int seg_find(const int64_t* __restrict__ off, int nseg, int pos, uint32_t* err) {
    const int lane = threadIdx.x & 31;
    int lo = 0, hi = nseg;
    while (true) {
        const int step = hi - lo > 32 ? (hi - lo + 31) / 32 : 1;
        const int idx = lo + lane * step;
        const bool ok = idx < hi && __ldg(&off[idx]) <= (int64_t)pos;
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (!m) {  // offsets not as promised (off[lo] > pos); stay in bounds
            if (lane == 0) atomicOr(err, ERR_BAD_OFFSETS);
            return lo;
        }
        lo += (31 - __clz(m)) * step;
        if (step == 1) return lo;
        hi = min(lo + step, hi);
    }
}

// Answer relative to the segment start s: an answer before the segment is none.
__device__ __forceinline__ int seg_rel(int g, int s) { return g >= s ? g - s : -1; }

// The key at position pos of the run's array, through the key map; REV runs
// see the array reversed (position pos is element n - 1 - pos).
template <typename T, int KMAP, bool REV>
__device__ __forceinline__ T key_at(const T* d_in, int n, int pos) {
    return load_key<T, KMAP>(d_in + (REV ? n - 1 - pos : pos));
}

template <typename T, int B, bool INCL, int MAPF = KMAP_NONE, bool REV = false>
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
        const bool ok = p < limit && p >= a.head && lt<INCL>(key_at<T, MAPF, REV>(d_in, a.n, p), q);
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
            auto rmin = [&](int i) { return range_min<T>(a, i); };
            const int g = R >> 5;
            int rr = ballot_last<T, INCL>(g * 32, R - 1, q, rmin);
            if (rr < 0) {
                int gg = -1;
                for (int hi = g - 1; hi >= 0 && gg < 0; hi -= 32)
                    gg = ballot_last<T, INCL>(0, hi, q, [&](int i) { return group_min_of<T>(a, i); });
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
    const unsigned m =
        __ballot_sync(0xffffffffu, row + lane >= a.head && lt<INCL>(key_at<T, MAPF, REV>(d_in, a.n, row + lane), q));
    return m ? row + 31 - __clz(m) : -2;
}

// The nearest range at or below `hi` whose minimum qualifies for q, or -1:
// the ranges of hi's group, then the minima of earlier groups, 32 per step.
// Warp-cooperative; every range and group it reads has published.
template <typename T, bool INCL>
__device__ __noinline__ int nearest_range(T q, int hi, const RangeArgs& a) {
    if (hi < 0) return -1;
    auto rmin = [&](int i) { return range_min<T>(a, i); };
    const int g = hi >> 5;
    const int rr = ballot_last<T, INCL>(g * 32, hi, q, rmin);
    if (rr >= 0) return rr;
    for (int ghi = g - 1; ghi >= 0; ghi -= 32) {
        const int gg = ballot_last<T, INCL>(0, ghi, q, [&](int i) { return group_min_of<T>(a, i); });
        if (gg >= 0) return ballot_last<T, INCL>(gg * 32, gg * 32 + 31, q, rmin);
    }
    return -1;
}

// ---------------------------------------------------------------------------
// Range minima -> exclusive prefix minima.
//
// Publishing range r (lane 0): an atomic minimum into its group's word
// (groups of 32 ranges), a fence, the range's tagged minimum (range_state),
// and one relaxed increment of the count of published ranges.  The range
// that completes the count raises one ready flag per CTA.  Range r then
// needs the minima of the earlier ranges of its group plus those of the
// earlier groups: one round of loads, no hot spot, and no step of the last
// range's path waits on another range's loads.
//
// Group words: atomic minima of (EPOCH_LIMIT - epoch) << 32 | ordered key.
// The current run's tag is below every older run's, so its first minimum
// replaces an older word and the words need no reset between runs (they
// start all-ones and are cleared again when the epoch wraps).
//
// Every range of a launch is resident when the launch fits the device (the
// grid is sized from occupancy), so the ready flag always comes.  When it
// does not come within a bound (the launch shares the device and some warps
// have not started), range r falls back to waiting on the tagged minima of
// the ranges before it, all of which already run (ids are handed out in
// start order), so no wait depends on a warp that may not start.  Every wait
// is bounded and reports ERR_LOOKBACK_TIMEOUT when it gives up.
// ---------------------------------------------------------------------------
// A launch of at most kDirectRanges ranges skips the global step: range r polls
// the tagged minima of the ranges before it directly (a few words), which ends
// sooner than waiting for every range of the launch to publish.
constexpr int kDirectRanges = 256;

template <typename T>
__device__ void range_publish(int r, uint32_t epoch, T rmin, const RangeArgs& a) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t tag = (epoch << 2) | FLAG_AGG;
    const bool direct = a.num_ranges <= kDirectRanges;
    int last = 0;
    if (lane == 0 && r != a.skip_publish_range) {
        if constexpr (sizeof(T) == 8)
            __stcg((unsigned long long*)&a.s.range_key[r], (unsigned long long)KeyTraits<T>::bits(rmin));
        else
            red_min_u64(&a.s.group_min[r >> 5], ((uint64_t)(EPOCH_LIMIT - epoch) << 32) | KeyTraits<T>::ord(rmin));
        // release: this range's words (every lane's, ordered by the caller's
        // __syncwarp) and the group minimum before the range minimum and the count
        __threadfence();
        __stcg((unsigned long long*)&a.s.range_state[r],
               ((uint64_t)tag << 32) | (sizeof(T) == 8 ? 0u : (uint32_t)KeyTraits<T>::bits(rmin)));
        if (!direct) {
            last = atomicAdd(&a.s.ctr->finished, 1u) == (uint32_t)(a.num_ranges - 1);
            if (last) __threadfence();  // acquire: every range's publication
        }
    }
    if (!__shfl_sync(FULL, last, 0)) return;
    __syncwarp();
    __threadfence();  // release to the flags' readers
    for (int c = lane; c < (int)gridDim.x; c += 32) a.s.cta_ready[(size_t)c * kReadyStride] = epoch;
}

// p: the minimum over ranges [0, r); win (lane i): the minimum of range r-1-i
// (pad below range 0), the window phase 2 searches first.
template <typename T>
__device__ void range_prefix(int r, uint32_t epoch, const RangeArgs& a, T& p, bool& has_p, T& win) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int g = r >> 5;
    const uint32_t tag = (epoch << 2) | FLAG_AGG;
    p = KeyTraits<T>::pad();
    win = KeyTraits<T>::pad();
    has_p = r > 0;
    if (r == 0) return;
    const uint32_t* flag = &a.s.cta_ready[(size_t)blockIdx.x * kReadyStride];
    // every range has published: the window (it holds the group's earlier
    // ranges) and the earlier groups, in one round of loads
    auto from_ready = [&]() {
        const int wi = r - 1 - lane;
        win = wi >= 0 ? range_min<T>(a, wi) : KeyTraits<T>::pad();
        T m = wi >= g * 32 ? win : KeyTraits<T>::pad();
        if constexpr (sizeof(T) == 8) {  // the ranges of the earlier groups, one by one
            for (int i = lane; i < g * 32; i += 32) m = KeyTraits<T>::vmin(m, range_min<T>(a, i));
        } else {
            const uint32_t gtag = EPOCH_LIMIT - epoch;
            bool bad = false;
#pragma unroll
            for (int k = 0; k < kMaxRanges / 32 / 32; k++) {
                const int gi = lane + 32 * k;
                if (gi < g) {
                    const uint64_t w = __ldcg((const unsigned long long*)&a.s.group_min[gi]);
                    bad = bad || (uint32_t)(w >> 32) != gtag;
                    m = KeyTraits<T>::vmin(m, KeyTraits<T>::from_ord((uint32_t)w));
                }
            }
            if (bad) atomicOr(&a.s.ctr->err, ERR_INTERNAL);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = KeyTraits<T>::vmin(m, __shfl_xor_sync(FULL, m, o));
        p = m;
    };
    // 1. the ready flag of this CTA (one line, polled by one lane per warp); a
    //    launch of few ranges raises none: its ranges wait on their predecessors
    int ready = 0;
    if (lane == 0 && a.num_ranges > kDirectRanges) {
        const uint32_t bound = min(a.spin_limit, 1u << 16);
        for (uint32_t s = 0;; s++) {
            if (ld_acquire_u32(flag) == epoch) {
                ready = 1;
                break;
            }
            if (s >= bound) break;
            __nanosleep(s < 8 ? 64 : 256);
        }
    }
    __syncwarp();  // lane 0's acquire before the other lanes' loads
    if (__shfl_sync(FULL, ready, 0)) {
        from_ready();
        return;
    }
    // 2. fallback: wait for the tagged minima of the earlier ranges (or the flag)
    for (uint32_t spins = 0;; spins++) {
        bool ok = true;
        T m = KeyTraits<T>::pad();
        for (int ri = lane; ri < r; ri += 32) {
            const uint64_t w = ld_acquire_u64(&a.s.range_state[ri]);
            if ((uint32_t)(w >> 32) != tag) ok = false;
            m = KeyTraits<T>::vmin(m, sizeof(T) == 8 ? range_min<T>(a, ri) : KeyTraits<T>::from_bits((uint32_t)w));
        }
        if (__all_sync(FULL, ok)) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = KeyTraits<T>::vmin(m, __shfl_xor_sync(FULL, m, o));
            p = m;
            const int wi = r - 1 - lane;
            win = wi >= 0 ? range_min<T>(a, wi) : KeyTraits<T>::pad();
            return;
        }
        if (__shfl_sync(FULL, lane == 0 ? (int)(ld_acquire_u32(flag) == epoch) : 0, 0)) {
            __syncwarp();
            from_ready();
            return;
        }
        if (spins >= a.spin_limit) {
            if (lane == 0) atomicOr(&a.s.ctr->err, ERR_LOOKBACK_TIMEOUT);
            return;
        }
        __nanosleep(spins < 128 ? 64 : 256);
    }
}

// MAPF: the key map (KMAP_*): keys pass through it as they enter shared memory
// or registers -- float64 bit patterns in int64 slots compared through
// f64_order, or the order-reversing flip for previous-greater queries.
// OUTM (single arrays, no view head, except OUT_I32): OUT_I64 -- answers as
// int64, a.out_base + answer, into a.d_out64, for the int64-position path: a
// flagged key gets UNRESOLVED64 (phase 2 overwrites the ones it answers), and a
// tile whose keys are all deferred is not written at all (its flag word says
// so); the int64-position path answers what is left.  OUT_SPAN -- int32
// position - answer (position + 1 for none): the stock span, with the flip.
// REV (single arrays, no view head, 4-byte keys): the run sees the array
// reversed -- tile t holds elements n - 1 - (t * WT + e), its TMA rows counted
// from the end (n a multiple of 32) and reversed in shared memory as they
// land -- and writes each answer mirrored back, n - 1 - answer (-1 for none)
// at element n - 1 - position: the next smaller key, in one run.

template <typename T, int IPT, int WPC, bool INCL, bool SEG, bool EP, int MAPF = KMAP_NONE, int OUTM = OUT_I32,
          bool REV = false>
__global__ void __launch_bounds__(WPC * 32, (WPC >= 16 && sizeof(T) == 4 ? 1 : 2))
apse_warp_kernel(const __grid_constant__ CUtensorMap map_in, const __grid_constant__ CUtensorMap map_out,
                 const RangeArgs a) {
    constexpr int KB = (int)sizeof(T);  // bytes per key
    using L = WLayout<IPT, KB>;
    constexpr int WT = L::WT;      // keys per warp tile
    constexpr int W = WT / 32;     // 32-key chunks (and answer TMA rows) per warp tile
    constexpr int RPT = W * KB / 4;  // key TMA rows (128 bytes) per warp tile
    static_assert(KB == 4 || (KB == 8 && IPT == 8), "8-byte keys run with 8 keys per lane");
    constexpr int TPC = 32 / IPT;  // lanes per chunk
    constexpr int K = kStackCap;
    constexpr int MW = kMaxTileKeys / 32;  // flag-mask words per tile in global
    static_assert(IPT == 8 || IPT == 16, "IPT must be 8 or 16");
    auto ks = [](int e) { return kswz<KB>(e); };  // swizzled index of key e in V / sSM
    static_assert((K & (K - 1)) == 0, "the stack ring needs a power-of-two size");
    static_assert(K % 32 == 0 && K <= WT, "a whole-tile push copies the tile's last K keys, 32 per step");
    constexpr unsigned FULL = 0xffffffffu;

    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    unsigned char* cta_sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* wsm = cta_sm + (size_t)warp * L::kBytes;
    // CTA words: [0] the CTA's first range, [1] warps of the CTA finished
    int* sCta = (int*)(cta_sm + (size_t)WPC * L::kBytes);
    T* sV = (T*)(wsm + L::kV);
    int32_t* O = (int32_t*)(wsm + L::kO);
    T* sSM = (T*)(wsm + L::kSM);
    int16_t* sList = (int16_t*)(wsm + L::kList);
    T* sStkV = (T*)(wsm + L::kStkV);
    int32_t* sStkP = (int32_t*)(wsm + L::kStkP);
    int32_t* sDefP = (int32_t*)(wsm + L::kDefP);
    T* sDefV = (T*)(wsm + L::kDefV);
    int32_t* sCapP = (int32_t*)(wsm + L::kCapP);
    int32_t* sCapS = (int32_t*)(wsm + L::kCapS);
    uint64_t* bar = (uint64_t*)(wsm + L::kBar);

    const T* d_in = (const T*)a.d_in;
    T* tile_min_w = (T*)a.s.tile_min;
    T* chunk_min_w = (T*)a.s.chunk_min;
    uint32_t* err = &a.s.ctr->err;
    // The view's virtual keys: only the segmented instantiations have them (a
    // batch off a 16-byte boundary; a single array off one runs as one implicit
    // segment with the whole-tile early paths, EP).
    const int head = SEG ? a.head : 0;
    // Segment offsets (positions in the array); with no offsets array, one segment.
    auto seg_off = [&](int i) -> int64_t {
        return a.offsets ? (int64_t)__ldg(&a.offsets[i]) : (i == 0 ? (int64_t)0 : (int64_t)(a.n - head));
    };
    auto seg_idx = [&](int pos) { return a.offsets ? seg_find(a.offsets, a.nseg, pos, err) : 0; };
    static_assert(OUTM == OUT_I32 || (!SEG && EP), "int64 and span answers: single arrays only");
    static_assert(!REV || (!SEG && EP && OUTM == OUT_I32 && KB == 4), "reversed runs: single arrays of 4-byte keys");
    constexpr bool OUT64 = OUTM == OUT_I64;
    // a final answer v of position pos (phase 2); int64 answers: out_base + v, and
    // UNRESOLVED64 for none (the key is left to the int64-position path); spans:
    // pos - v
    auto put = [&](int pos, int v) {
        if constexpr (OUT64) a.d_out64[pos] = v >= 0 ? (int64_t)v + a.out_base : UNRESOLVED64;
        else if constexpr (REV) a.d_out[a.n - 1 - pos] = v >= 0 ? a.n - 1 - v : -1;
        else if constexpr (OUTM == OUT_SPAN) a.d_out[pos] = pos - v;
        else a.d_out[pos] = v;
    };

    // One claim per CTA: its warps take WPC consecutive range ids, in the order
    // the CTAs start (so every range a warp may wait on belongs to a started CTA).
    if (threadIdx.x == 0) {
        sCta[0] = (int)atomicAdd(&a.s.ctr->range_counter, (unsigned)WPC);
        sCta[1] = 0;
    }
    uint32_t epoch = 0;
    if (lane == 0) {
        epoch = ld_relaxed_u32(&a.s.ctr->epoch);
        for (int s = 0; s < kStages; s++) mbar_init(&bar[s], 1);
        fence_mbarrier_init();
        fence_proxy_async_smem();
    }
    __syncthreads();  // the CTA's claim is in shared memory
    const int r = sCta[0] + warp;
    epoch = __shfl_sync(FULL, epoch, 0);
    __syncwarp();

    if (r < a.num_ranges) {
        const int t0 = r * a.tiles_per_range;
        const int t1 = min(t0 + a.tiles_per_range, a.num_tiles);
        const int ntr = t1 - t0;
        auto tile_full = [&](int t) { return a.tma_rows > 0 && (t + 1) * RPT <= a.tma_rows && (t > 0 || head == 0); };
        // the first TMA row of tile t (reversed runs: counted from the end)
        auto tile_row = [&](int t) { return REV ? a.tma_rows - (t + 1) * RPT : t * RPT; };
        if (lane == 0) {
            for (int i = 0; i < kStages && i < ntr; i++)
                if (tile_full(t0 + i)) {
                    mbar_arrive_expect_tx(&bar[i], (uint32_t)(WT * KB));
                    tma_load_2d(sV + (size_t)i * WT, &map_in, 0, tile_row(t0 + i), &bar[i]);
                }
        }
        // Range state (warp-uniform): the stack ring [stk_lo, stk_hi) of strict
        // suffix minima, values increasing from bottom to top; whether entries were
        // ever dropped from its bottom; the range minimum so far; flagged-key counts.
        int stk_lo = 0, stk_hi = 0;
        bool dropped = false;
        bool has_rmin = false;
        T rmin = KeyTraits<T>::pad();
        int def_total = 0, cap_total = 0;
        // Segmented runs (warp-uniform): the segment at the cursor, its start and
        // the next segment start.
        int seg_cur = 0, cur_start = 0, next_b = INT_MAX;
        int first_start = 0, first_end = INT_MAX;  // the segment holding the range's first key
        if constexpr (SEG) {
            if (r == 0 && lane == 0 && a.offsets && (a.offsets[0] != 0 || a.offsets[a.nseg] != (int64_t)(a.n - head)))
                atomicOr(err, ERR_BAD_OFFSETS);
            // offsets are positions in the array; the view adds `head` virtual keys in
            // front (they fall in segment 0, and no answer of theirs is written)
            seg_cur = seg_idx(max(t0 * WT - head, 0));
            cur_start = (int)min(max(seg_off(seg_cur), (int64_t)0) + head, (int64_t)INT_MAX);
            next_b = (int)min(max(seg_off(seg_cur + 1), (int64_t)0) + head, (int64_t)INT_MAX);
            first_start = cur_start;
            first_end = next_b;
        }

        // ======================= phase 1: the range's tiles =======================
        for (int i = 0; i < ntr; i++) {
            const int t = t0 + i;
            const int slot = i % kStages;
            const uint32_t par = (uint32_t)((i / kStages) & 1);
            T* V = sV + (size_t)slot * WT;
            const bool full = tile_full(t);
            const int tile_base = t * WT;
            const int valid_keys = min(WT, a.n - tile_base);

            if (full) {
                if (!mbar_wait_bounded(&bar[slot], par, a.spin_limit) && lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
                if constexpr (REV) {  // the tile arrived in element order: reverse it in place
                    T rv[IPT];
#pragma unroll
                    for (int j = 0; j < IPT; j++) rv[j] = V[ks(WT - 1 - (j * 32 + lane))];
                    __syncwarp();
#pragma unroll
                    for (int j = 0; j < IPT; j++) V[ks(j * 32 + lane)] = rv[j];
                    __syncwarp();
                }
                if constexpr (MAPF != KMAP_NONE) {  // the tile's keys through the key map, in place
#pragma unroll
                    for (int j = 0; j < IPT; j++) {
                        const int e = j * 32 + lane;
                        V[ks(e)] = map_key<T, MAPF>(V[ks(e)]);
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < IPT; j++) {
                    const int e = j * 32 + lane;
                    const int g = tile_base + e;
                    V[ks(e)] = g < a.n && (!head || g >= head) ? (MAPF != KMAP_NONE || REV ? key_at<T, MAPF, REV>(d_in, a.n, g) : d_in[g])
                                                                : KeyTraits<T>::pad();
                }
                // A view head makes tile 0 plain while tile kStages streams into its
                // slot: the plain tile completes the slot barrier's phase by itself.
                // (Any other plain tile is the array's last: its slot is not reused.)
                if (head && lane == 0 && a.tma_rows > 0) mbar_arrive(&bar[slot]);
            }
            if (lane == 0) bulk_wait_read0();  // the previous tile's store has read O
            __syncwarp();

            // ---- 0. segmented runs: where segments start among the tile's keys ----------
            unsigned bword = 0;  // segment starts among this lane's keys (bit k: key k)
            int lane_s = 0;      // start of the segment holding this lane's first key
            if constexpr (SEG) {
                const int tile_end = tile_base + WT;
                const int in_start = cur_start;
                if (next_b < tile_end) {
                    uint32_t* bm = (uint32_t*)sList;  // 512 bits; the X list is built later
                    if (lane < MW) bm[lane] = 0u;
                    __syncwarp();
                    for (int it = 0; it <= a.nseg / 32 + 1; it++) {  // ends once past off[nseg]
                        const int idx = seg_cur + 1 + lane;
                        const int64_t b = idx <= a.nseg ? seg_off(idx) + head : (int64_t)INT_MAX;
                        const bool in = b >= tile_base && b < tile_end;
                        if (in) atomicOr(&bm[(int)(b - tile_base) >> 5], 1u << ((int)(b - tile_base) & 31));
                        const int cnt = __popc(__ballot_sync(FULL, b < tile_end));
                        if (cnt) cur_start = (int)max((int64_t)0, __shfl_sync(FULL, b, cnt - 1));
                        seg_cur += cnt;
                        if (cnt < 32) {
                            next_b = (int)min((int64_t)INT_MAX, __shfl_sync(FULL, b, cnt));
                            break;
                        }
                    }
                    __syncwarp();
                    bword = (bm[(lane * IPT) >> 5] >> ((lane * IPT) & 31)) & (IPT == 32 ? 0xffffffffu : ((1u << IPT) - 1u));
                    int mx = bword ? tile_base + lane * IPT + 31 - __clz(bword) : -1;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int nb = __shfl_up_sync(FULL, mx, o);
                        if (lane >= o) mx = max(mx, nb);
                    }
                    const int before_b = __shfl_up_sync(FULL, mx, 1);
                    lane_s = max(in_start, lane > 0 ? before_b : -1);
                } else {
                    lane_s = in_start;
                }
            }
            // start of the segment holding key k of this lane
            auto seg_of = [&](int k) {
                const unsigned bb = bword & ((2u << k) - 1u);
                return bb ? tile_base + lane * IPT + 31 - __clz(bb) : lane_s;
            };

            // ---- 1. in-thread answers: compare ladder over IPT keys in registers --------
            T v[IPT];
            if constexpr (KB == 4) {
#pragma unroll
                for (int q4 = 0; q4 < IPT / 4; q4++) {
                    const uint4 rr = *reinterpret_cast<const uint4*>(&V[swz(lane * IPT + 4 * q4)]);
                    v[4 * q4 + 0] = KeyTraits<T>::from_bits(rr.x);
                    v[4 * q4 + 1] = KeyTraits<T>::from_bits(rr.y);
                    v[4 * q4 + 2] = KeyTraits<T>::from_bits(rr.z);
                    v[4 * q4 + 3] = KeyTraits<T>::from_bits(rr.w);
                }
            } else {  // two 8-byte keys per 16-byte chunk
#pragma unroll
                for (int q2 = 0; q2 < IPT / 2; q2++) {
                    const ulonglong2 rr = *reinterpret_cast<const ulonglong2*>(&V[ks(lane * IPT + 2 * q2)]);
                    v[2 * q2 + 0] = KeyTraits<T>::from_bits((uint64_t)rr.x);
                    v[2 * q2 + 1] = KeyTraits<T>::from_bits((uint64_t)rr.y);
                }
            }
            const int lb = tile_base + lane * IPT;  // position of this lane's first key
            const int nvalid = min(max(a.n - lb, 0), IPT);
            // Flagged keys, deferred (dm) and capped (cm), keep -1 in O.  The first kDefCap
            // deferred and kCapCap capped keys of the range go to in-order lists in shared
            // memory for phase 2; every tile also leaves its flags in global memory for the
            // lists' overflow.
            auto flag_keys = [&](const unsigned dm, const unsigned cm) {
                {
                    const unsigned fm = dm | cm;
                    const int nd = __popc(dm), nc = __popc(cm);
                    const unsigned anyf = __ballot_sync(FULL, fm != 0);
                    int dtot = 0, ctot = 0;
                    if (anyf) {
                        const int doff = warp_excl_sum(nd, dtot);
                        const int coff = warp_excl_sum(nc, ctot);
                        {
                            int idx = def_total + doff;
                            unsigned m = dm;
                            while (m && idx < kDefCap) {
                                const int k = __ffs(m) - 1;
                                m &= m - 1;
                                sDefP[idx] = lb + k;
                                sDefV[idx] = V[ks(lane * IPT + k)];
                                idx++;
                            }
                        }
                        {
                            int idx = cap_total + coff;
                            unsigned m = cm;
                            while (m && idx < kCapCap) {
                                const int k = __ffs(m) - 1;
                                m &= m - 1;
                                if constexpr (SEG) sCapS[idx] = seg_of(k);
                                sCapP[idx++] = lb + k;
                            }
                        }
                        // mask word w covers keys [32w, 32w + 32): lanes TPC*w .. TPC*w + TPC - 1
                        uint32_t mw = 0;
    #pragma unroll
                        for (int j = 0; j < TPC; j++) {
                            const unsigned part = __shfl_sync(FULL, fm, (lane % W) * TPC + j);
                            mw |= part << (j * IPT);
                        }
                        if (lane < W) __stcg(&a.s.tile_mask[(size_t)t * MW + lane], mw);
                        def_total += dtot;
                        cap_total += ctot;
                    }
                    if (lane == 0) __stcg(&a.s.tile_flag[t], (uint32_t)(dtot + ctot) | (ctot ? 0x80000000u : 0u));
                }
            };
            // The whole tile leaves O, flagged keys as -1 (segmented runs: answers made
            // relative to their segment's start).
            auto store_tile = [&]() {
                if constexpr (OUT64) {  // int64 answers, 32 consecutive keys per store
                    __syncwarp();       // every lane's answers are in O
#pragma unroll
                    for (int j = 0; j < IPT; j++) {
                        const int e = j * 32 + lane;
                        if (e < valid_keys) {
                            const int o = O[swz(e)];
                            a.d_out64[tile_base + e] = o >= 0 ? (int64_t)o + a.out_base : UNRESOLVED64;
                        }
                    }
                    return;
                }
                if constexpr (REV) {  // mirrored answers at the mirrored positions, in element order
                    __syncwarp();     // every lane's answers are in O
                    if (full) {
                        int ro[IPT];
#pragma unroll
                        for (int j = 0; j < IPT; j++) {
                            const int o = O[swz(WT - 1 - (j * 32 + lane))];
                            ro[j] = o >= 0 ? a.n - 1 - o : -1;
                        }
                        __syncwarp();
#pragma unroll
                        for (int j = 0; j < IPT; j++) O[swz(j * 32 + lane)] = ro[j];
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            tma_store_2d(&map_out, 0, tile_row(t), O);
                            bulk_commit();
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < IPT; j++) {
                            const int e = j * 32 + lane;
                            if (e < valid_keys) {
                                const int o = O[swz(e)];
                                a.d_out[a.n - 1 - (tile_base + e)] = o >= 0 ? a.n - 1 - o : -1;
                            }
                        }
                    }
                    return;
                }
                if constexpr (OUTM == OUT_SPAN) {  // spans: position - answer
                    __syncwarp();                   // every lane's answers are in O
    #pragma unroll
                    for (int q4 = 0; q4 < IPT / 4; q4++) {
                        int4* po = reinterpret_cast<int4*>(&O[swz(lane * IPT + 4 * q4)]);
                        int4 o = *po;
                        const int p0 = tile_base + lane * IPT + 4 * q4;
                        o.x = p0 - o.x;
                        o.y = p0 + 1 - o.y;
                        o.z = p0 + 2 - o.z;
                        o.w = p0 + 3 - o.w;
                        *po = o;
                    }
                }
                if constexpr (SEG) {  // answers relative to their segment's start
                    __syncwarp();     // every lane's answers are in O
    #pragma unroll
                    for (int q4 = 0; q4 < IPT / 4; q4++) {
                        int4* po = reinterpret_cast<int4*>(&O[swz(lane * IPT + 4 * q4)]);
                        int4 o = *po;
                        o.x = seg_rel(o.x, seg_of(4 * q4 + 0));
                        o.y = seg_rel(o.y, seg_of(4 * q4 + 1));
                        o.z = seg_rel(o.z, seg_of(4 * q4 + 2));
                        o.w = seg_rel(o.w, seg_of(4 * q4 + 3));
                        *po = o;
                    }
                }
                fence_proxy_async_smem();
                __syncwarp();
                if (full) {
                    if (lane == 0) {
                        tma_store_2d(&map_out, 0, t * W, O);
                        bulk_commit();
                    }
                } else {
    #pragma unroll
                    for (int j = 0; j < IPT; j++) {
                        const int e = j * 32 + lane;
                        if (e < valid_keys && (!head || tile_base + e >= head)) a.d_out[tile_base + e] = O[swz(e)];
                    }
                }
            };

            // Monotone lanes: each key answers its neighbour (adj), or no key answers
            // any later one (none); across the lane boundary likewise (b_adj, b_none).
            // A few neighbour pairs first: on almost every tile of unordered keys some
            // lane is already neither increasing nor non-increasing there, and the
            // full check (15 compares a lane) is skipped.
            bool adj = false, none = false;
            unsigned mono = 0u;
            {
                bool qa = true, qn = true;
#pragma unroll
                for (int k = IPT / 4; k < IPT; k += IPT / 4) {
                    const bool l = lt<INCL>(v[k - 1], v[k]);
                    qa = qa && l;
                    qn = qn && !l;
                }
                if (__all_sync(FULL, qa || qn)) {
                    adj = true;
                    none = true;
#pragma unroll
                    for (int k = 1; k < IPT; k++) {
                        const bool l = lt<INCL>(v[k - 1], v[k]);
                        adj = adj && l;
                        none = none && !l;
                    }
                    mono = __ballot_sync(FULL, adj || none);
                }
            }
            const T prev_last = __shfl_up_sync(FULL, v[IPT - 1], 1);
            const bool b_adj = lane == 0 || lt<INCL>(prev_last, v[0]);

            // ---- a whole tile below the range so far --------------------------------------
            // A tile that never increases (under the comparator, lane boundaries
            // included) and whose first key has no qualifying key earlier in the
            // range has no answer for any key inside the range: every key is deferred,
            // every stack entry (>= the range minimum >= the first key) is popped and
            // the tile's last key is its only strict suffix minimum.  (Single arrays,
            // also a single array behind a view head in the segmented kernel.)
            if constexpr (EP) {
                const T first = __shfl_sync(FULL, v[0], 0);
                if (mono == FULL && valid_keys == WT && __all_sync(FULL, none && (lane == 0 || !b_adj)) &&
                    (!has_rmin || !lt<INCL>(rmin, first))) {
                    const int4 m1 = make_int4(-1, -1, -1, -1);
#pragma unroll
                    for (int q4 = 0; q4 < IPT / 4; q4++) *reinterpret_cast<int4*>(&O[swz(lane * IPT + 4 * q4)]) = m1;
                    if (((lane + 1) & (TPC - 1)) == 0) __stcg(&chunk_min_w[(size_t)t * W + lane / TPC], v[IPT - 1]);
                    const T tmin = __shfl_sync(FULL, v[IPT - 1], 31);
                    for (int e = lane; e < WT && def_total + e < kDefCap; e += 32) {
                        sDefP[def_total + e] = tile_base + e;
                        sDefV[def_total + e] = V[ks(e)];
                    }
                    if (lane < W) __stcg(&a.s.tile_mask[(size_t)t * MW + lane], 0xffffffffu);
                    if (lane == 0) {
                        __stcg(&a.s.tile_flag[t], (uint32_t)WT | (OUT64 ? TILE_NOT_STORED : 0u));
                        __stcg(&tile_min_w[t], tmin);
                    }
                    def_total += WT;
                    if constexpr (OUTM == OUT_SPAN || REV) {
                        store_tile();
                    } else if constexpr (!OUT64) {  // (int64 answers: the tile is left to the int64-position path)
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (full) {
                            if (lane == 0) {
                                tma_store_2d(&map_out, 0, t * W, O);
                                bulk_commit();
                            }
                        } else {
#pragma unroll
                            for (int j = 0; j < IPT; j++)
                                if (!head || tile_base + j * 32 + lane >= head) a.d_out[tile_base + j * 32 + lane] = -1;
                        }
                    }
                    if (lane == 31) {
                        sStkV[stk_lo & (K - 1)] = v[IPT - 1];
                        sStkP[stk_lo & (K - 1)] = tile_base + WT - 1;
                    }
                    stk_hi = stk_lo + 1;
                    rmin = tmin;
                    has_rmin = true;
                    __syncwarp();
                    if (lane == 0 && i + kStages < ntr && tile_full(t + kStages)) {
                        mbar_arrive_expect_tx(&bar[slot], (uint32_t)(WT * KB));
                        tma_load_2d(V, &map_in, 0, tile_row(t + kStages), &bar[slot]);
                    }
                    continue;
                }
            }

            // ---- a whole tile above the stack top ---------------------------------------------
            // A strictly increasing tile whose first key is above the stack's top entry
            // (the range's last key): every key answers its predecessor under either
            // comparator, every key is a strict suffix minimum, and the ring keeps the
            // tile's last K keys.
            if constexpr (EP) {
                const T first = __shfl_sync(FULL, v[0], 0);
                bool up = mono == FULL && valid_keys == WT && __all_sync(FULL, adj && b_adj) && stk_hi > stk_lo &&
                          sStkV[(stk_hi - 1) & (K - 1)] < first;
                if constexpr (INCL) {
                    // adj means non-decreasing here: ties would not all be strict suffix
                    // minima, so check strict increase (only on such tiles)
                    if (up) {
                        bool inc = lane == 0 || prev_last < v[0];
#pragma unroll
                        for (int k = 1; k < IPT; k++) inc = inc && v[k - 1] < v[k];
                        up = __all_sync(FULL, inc);
                    }
                }
                if (up) {
                    // answers relative to the array (a view head's pads are never the
                    // stack top here: a pad does not lie below the tile's first key)
                    const int top_pos = sStkP[(stk_hi - 1) & (K - 1)] - head;
                    const int hb = lb - head;
#pragma unroll
                    for (int q4 = 0; q4 < IPT / 4; q4++)
                        *reinterpret_cast<int4*>(&O[swz(lane * IPT + 4 * q4)]) =
                            make_int4(lane == 0 && q4 == 0 ? top_pos : hb + 4 * q4 - 1, hb + 4 * q4, hb + 4 * q4 + 1,
                                      hb + 4 * q4 + 2);
                    if ((lane & (TPC - 1)) == 0) __stcg(&chunk_min_w[(size_t)t * W + lane / TPC], v[0]);
                    if (lane == 0) {
                        __stcg(&a.s.tile_flag[t], 0u);
                        __stcg(&tile_min_w[t], first);
                    }
                    if constexpr (OUTM != OUT_I32 || REV) {
                        store_tile();
                    } else {
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (full) {
                            if (lane == 0) {
                                tma_store_2d(&map_out, 0, t * W, O);
                                bulk_commit();
                            }
                        } else {
#pragma unroll
                            for (int j = 0; j < IPT; j++)
                                if (!head || tile_base + j * 32 + lane >= head)
                                    a.d_out[tile_base + j * 32 + lane] = O[swz(j * 32 + lane)];
                        }
                    }
                    const int base_idx = stk_hi;  // entry of tile key e: base_idx + e
#pragma unroll
                    for (int h = 0; h < K / 32; h++) {  // the tile's last K keys, one per lane and step
                        const int e = WT - K + h * 32 + lane;
                        sStkV[(base_idx + e) & (K - 1)] = V[ks(e)];
                        sStkP[(base_idx + e) & (K - 1)] = tile_base + e;
                    }
                    stk_hi = base_idx + WT;
                    stk_lo = stk_hi - K;
                    dropped = true;  // WT > K: the older entries are gone
                    rmin = KeyTraits<T>::vmin(rmin, first);
                    __syncwarp();
                    if (lane == 0 && i + kStages < ntr && tile_full(t + kStages)) {
                        mbar_arrive_expect_tx(&bar[slot], (uint32_t)(WT * KB));
                        tma_load_2d(V, &map_in, 0, tile_row(t + kStages), &bar[slot]);
                    }
                    continue;
                }
            }

            // Filled by the path below that handles the tile (steps 1-5, or a tile that never
            // increases) and used by steps 6-9.
            unsigned dm = 0u, cm = 0u;
            T lmin = KeyTraits<T>::pad(), suf = KeyTraits<T>::pad(), tile_min_t = KeyTraits<T>::pad();
            T wv = KeyTraits<T>::pad();
            int win_lo = 0, dkeep = 0;
            bool wvalid = false;
            // ---- a whole tile that never increases, above something earlier in the range -----
            // No key answers another, so every key's answer is the topmost qualifying entry
            // of the range stack (else it is capped or deferred), and as the keys do not
            // increase those entries only move down the stack: each lane searches the
            // stack for its first key, then walks down for the others.  The stack keeps
            // its entries below the tile's last key and takes that key.  Segmented
            // instantiations only (descending runs in batches of segments are made of
            // such tiles): in the single-array kernel the extra branch cost 5 us on
            // random keys at 2^25.
            const bool dtile =
                SEG && mono == FULL && valid_keys == WT && __all_sync(FULL, none && (lane == 0 || !b_adj));
            if (dtile) {
                const int dwin = max(stk_lo, stk_hi - 32);
                const int wcnt = stk_hi - dwin;
                const T dwv = dwin + lane < stk_hi ? sStkV[(dwin + lane) & (K - 1)] : KeyTraits<T>::pad();
                int lo = -1;  // topmost qualifying window entry for the lane's first key
#pragma unroll
                for (int s2 = 32; s2 > 0; s2 >>= 1) {
                    const int cand = lo + s2;
                    const T wc = __shfl_sync(FULL, dwv, cand & 31);
                    if (cand < wcnt && lt<INCL>(wc, v[0])) lo = cand;
                }
                int si = lo >= 0 ? dwin + lo : stk_lo - 1;  // stack index of the current answer
                if (lo < 0 && dwin > stk_lo) {  // below the window (values increase upwards)
                    int l2 = stk_lo, h2 = dwin;
                    while (l2 < h2) {
                        const int mid = (l2 + h2) >> 1;
                        if (lt<INCL>(sStkV[mid & (K - 1)], v[0])) l2 = mid + 1;
                        else h2 = mid;
                    }
                    si = l2 - 1;
                }
                // One rolled loop over the lane's keys, read back from the tile in shared
                // memory: with the loop unrolled over registers this path's code, beside
                // the general path's, overflowed the instruction cache when an SM's warps
                // ran both (a batch mixing descending runs with other keys: cache hit rate
                // 78 % -> 89 %, that batch 2.07 -> 1.93 ms; a batch of one long descending
                // run pays for the rolled loop instead, 0.88 -> 1.10 ms).
#pragma unroll 1
                for (int k = 0; k < IPT; k++) {
                    const T vk = V[ks(lane * IPT + k)];
                    if (k > 0)
                        while (si >= stk_lo && !lt<INCL>(sStkV[si & (K - 1)], vk)) si--;
                    int rk = -1;
                    if (si >= stk_lo) {
                        rk = sStkP[si & (K - 1)];
                    } else {
                        if (has_rmin && lt<INCL>(rmin, vk)) cm |= 1u << k;  // below the kept entries
                        else dm |= 1u << k;
                    }
                    O[swz(lane * IPT + k)] = rk;
                }
                if constexpr (SEG) {  // deferred keys outside the range's first segment are final (-1)
                    if (lb + IPT > first_end) dm &= lb >= first_end ? 0u : ((1u << (first_end - lb)) - 1u);
                }
                if (cm && !dropped) atomicOr(err, ERR_INTERNAL);
                if (((lane + 1) & (TPC - 1)) == 0) __stcg(&chunk_min_w[(size_t)t * W + lane / TPC], v[IPT - 1]);
                tile_min_t = __shfl_sync(FULL, v[IPT - 1], 31);
                // the stack keeps its entries below the tile minimum (values >= it go; the
                // search's entry may equal it under <=) and takes the tile minimum
                int kp = __shfl_sync(FULL, si, 31);
                while (kp >= stk_lo && !(sStkV[kp & (K - 1)] < tile_min_t)) kp--;
                dkeep = kp + 1;
            } else {
            unsigned umask = 0;     // keys without an in-thread answer
            bool all_inc = false;   // the whole tile increases: every key answers its predecessor
            {
                int res[IPT];  // absolute answers, -1 = none in the thread
                res[0] = -1;
                // Monotone lanes need no ladder.
                if (mono == FULL) {
#pragma unroll
                    for (int k = 1; k < IPT; k++) res[k] = adj ? lb + k - 1 : -1;
                    // every key answers its predecessor across lane boundaries too
                    all_inc = __all_sync(FULL, adj && b_adj) && valid_keys == WT;
                    if (all_inc && lane > 0) res[0] = lb - 1;
                } else {
#pragma unroll
                    for (int k = 1; k < IPT; k++) {
                        int rk = -1;
#pragma unroll
                        for (int j = 0; j < k; j++)
                            if (lt<INCL>(v[j], v[k])) rk = lb + j;
                        res[k] = rk;
                    }
                    // the first key answers the previous lane's last key when that qualifies
                    if (lane > 0 && b_adj) res[0] = lb - 1;
                }
#pragma unroll
                for (int k = 0; k < IPT; k++)
                    if (res[k] < 0) umask |= 1u << k;
                if (nvalid < IPT) umask &= (1u << nvalid) - 1u;  // (the tail tile's pads)
                // in-thread answers; every other key holds -1 until resolved below
#pragma unroll
                for (int q4 = 0; q4 < IPT / 4; q4++)
                    *reinterpret_cast<int4*>(&O[swz(lane * IPT + 4 * q4)]) =
                        make_int4(res[4 * q4], res[4 * q4 + 1], res[4 * q4 + 2], res[4 * q4 + 3]);
            }
            {  // suffix minima of the lane's keys (for the key search of X keys)
                T sfx[IPT];
                sfx[IPT - 1] = v[IPT - 1];
#pragma unroll
                for (int k = IPT - 2; k >= 0; k--) sfx[k] = KeyTraits<T>::vmin(v[k], sfx[k + 1]);
                lmin = sfx[0];
                if constexpr (KB == 4) {
#pragma unroll
                    for (int q4 = 0; q4 < IPT / 4; q4++)
                        *reinterpret_cast<uint4*>(&sSM[swz(lane * IPT + 4 * q4)]) =
                            make_uint4(KeyTraits<T>::bits(sfx[4 * q4]), KeyTraits<T>::bits(sfx[4 * q4 + 1]),
                                       KeyTraits<T>::bits(sfx[4 * q4 + 2]), KeyTraits<T>::bits(sfx[4 * q4 + 3]));
                } else {
#pragma unroll
                    for (int q2 = 0; q2 < IPT / 2; q2++)
                        *reinterpret_cast<ulonglong2*>(&sSM[ks(lane * IPT + 2 * q2)]) =
                            make_ulonglong2((unsigned long long)KeyTraits<T>::bits(sfx[2 * q2]),
                                            (unsigned long long)KeyTraits<T>::bits(sfx[2 * q2 + 1]));
                }
            }
            {
                T cmn = lmin;
#pragma unroll
                for (int o = 1; o < TPC; o <<= 1) cmn = KeyTraits<T>::vmin(cmn, __shfl_xor_sync(FULL, cmn, o));
                if ((lane & (TPC - 1)) == 0) __stcg(&chunk_min_w[(size_t)t * W + lane / TPC], cmn);
            }

            // ---- 2. warp prefix minima over lane minima ---------------------------------
            T pre = lmin;  // inclusive prefix / suffix minima over lanes, side by side
            suf = lmin;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const T nb = __shfl_up_sync(FULL, pre, o);
                const T na = __shfl_down_sync(FULL, suf, o);
                if (lane >= o) pre = KeyTraits<T>::vmin(pre, nb);
                if (lane + o < 32) suf = KeyTraits<T>::vmin(suf, na);
            }
            const T before = __shfl_up_sync(FULL, pre, 1);  // min of the lanes before (lane > 0)
            tile_min_t = __shfl_sync(FULL, pre, 31);

            // ---- 3. classify the keys without an in-thread answer ------------------------
            // X: answered by an earlier lane of the tile; S: by an earlier tile of the
            // range (the stack); D: by nothing in the range (deferred to phase 2).
            unsigned gtb = 0, gtr = ~0u;
#pragma unroll
            for (int k = 0; k < IPT; k++) gtb |= (unsigned)lt<INCL>(before, v[k]) << k;
            // Every key of a lane is >= the lane minimum: when the range minimum
            // qualifies for every lane's minimum (most tiles after a range's first),
            // it qualifies for every key and the per-key compares are skipped.
            if (!__all_sync(FULL, lt<INCL>(rmin, lmin))) {
                gtr = 0u;
#pragma unroll
                for (int k = 0; k < IPT; k++) gtr |= (unsigned)lt<INCL>(rmin, v[k]) << k;
            }
            const unsigned xm = lane > 0 ? (umask & gtb) : 0u;
            const unsigned sm = has_rmin ? (umask & ~xm & gtr) : 0u;
            dm = umask & ~xm & ~sm;
            if constexpr (SEG) {
                // Nothing in the range qualifies for a deferred key; if its segment
                // starts inside the range, -1 is its final answer.  Only keys of the
                // segment holding the range's first key stay deferred.
                if (lb + IPT > first_end) dm &= lb >= first_end ? 0u : ((1u << (first_end - lb)) - 1u);
            }
            __syncwarp();  // the in-thread answers and suffix minima are in shared memory

            // ---- 4. X keys: lane by binary lifting, then key by binary search ------------
            const int cx = __popc(xm);
            const int xtot = (int)__reduce_add_sync(FULL, (unsigned)cx);
            if (xtot) {
                // lane table: tab[k] = min of lane minima over lanes (lane - 2^k, lane]
                T tab[5];
                tab[0] = lmin;
#pragma unroll
                for (int k = 1; k < 5; k++) {
                    const T u = __shfl_up_sync(FULL, tab[k - 1], 1 << (k - 1));
                    tab[k] = lane >= (1 << (k - 1)) ? KeyTraits<T>::vmin(tab[k - 1], u) : tab[k - 1];
                }
                // Up to NQ queries per lane and round.  A key e of lane ql = e / IPT is an X key
                // only when some lane before ql qualifies, so the lifting below never
                // passes lane 0: it ends on the nearest qualifying lane p (invariant: the
                // answer lane is <= p and after each step p - answer < 2^k).  In lane p,
                // the suffix minima qualify on a prefix [0, j] and key j is the answer.
                constexpr int NQ = kXQueries;
                auto resolve = [&](const int (&e)[NQ], const bool (&act)[NQ]) {
                    T q[NQ];
                    int p[NQ];
#pragma unroll
                    for (int i2 = 0; i2 < NQ; i2++) {
                        q[i2] = act[i2] ? V[ks(e[i2])] : KeyTraits<T>::pad();
                        p[i2] = act[i2] ? e[i2] / IPT - 1 : 0;
                    }
#pragma unroll
                    for (int k = 4; k >= 0; k--) {
#pragma unroll
                        for (int i2 = 0; i2 < NQ; i2++) {
                            const T m = __shfl_sync(FULL, tab[k], p[i2]);  // p stays in [0, 31]
                            if (act[i2] && !lt<INCL>(m, q[i2])) p[i2] -= 1 << k;
                        }
                    }
                    int j[NQ];
#pragma unroll
                    for (int i2 = 0; i2 < NQ; i2++) j[i2] = 0;
#pragma unroll
                    for (int i2 = 0; i2 < NQ; i2++)
                        if (act[i2] && p[i2] < 0) {  // cannot happen (see the invariant); stay in bounds
                            atomicOr(err, ERR_INTERNAL);
                            p[i2] = 0;
                        }
                    // lane p's entries share one swizzle: word (p*IPT | j) ^ x
                    int pb[NQ], px[NQ];
#pragma unroll
                    for (int i2 = 0; i2 < NQ; i2++) {
                        pb[i2] = p[i2] * IPT;
                        px[i2] = (pb[i2] >> 3) & (KB == 4 ? 0x1C : 0x0E);
                    }
#pragma unroll
                    for (int s2 = IPT / 2; s2 > 0; s2 >>= 1) {
#pragma unroll
                        for (int i2 = 0; i2 < NQ; i2++)
                            if (act[i2] && lt<INCL>(sSM[(pb[i2] | (j[i2] + s2)) ^ px[i2]], q[i2])) j[i2] += s2;
                    }
#pragma unroll
                    for (int i2 = 0; i2 < NQ; i2++)
                        if (act[i2]) O[swz(e[i2])] = tile_base + p[i2] * IPT + j[i2];
                };
                const int xmax = (int)__reduce_max_sync(FULL, (unsigned)cx);
                const int rounds = (xtot + 32 * NQ - 1) / (32 * NQ);
                if (xmax > NQ * rounds + 1) {
                    // spread the queries evenly: an ordered list of X keys
                    int tot_unused;
                    int off = warp_excl_sum(cx, tot_unused);
                    unsigned m = xm;
                    while (m) {
                        const int k = __ffs(m) - 1;
                        m &= m - 1;
                        sList[off++] = (int16_t)(lane * IPT + k);
                    }
                    __syncwarp();
                    for (int b0 = 0; b0 < xtot; b0 += 32 * NQ) {
                        int e[NQ];
                        bool act[NQ];
#pragma unroll
                        for (int i2 = 0; i2 < NQ; i2++) {
                            act[i2] = b0 + 32 * i2 + lane < xtot;
                            e[i2] = act[i2] ? (int)sList[b0 + 32 * i2 + lane] : 0;
                        }
                        resolve(e, act);
                    }
                } else {
                    unsigned m = xm;
                    for (int rd = 0; rd < xmax; rd += NQ) {
                        int e[NQ];
                        bool act[NQ];
#pragma unroll
                        for (int i2 = 0; i2 < NQ; i2++) {
                            act[i2] = m != 0;
                            e[i2] = lane * IPT + (act[i2] ? __ffs(m) - 1 : 0);
                            m &= m - 1;
                        }
                        resolve(e, act);
                    }
                }
            }

            // ---- 5. S keys: search of the range stack -------------------------------------
            // Entries are strict suffix minima: values increase from bottom to top and
            // the ones that qualify form a bottom part; the topmost of them answers.
            // The top 32 entries sit one per lane (the window), so a query is one
            // ballot.  With nothing ever dropped the bottom entry is the range minimum,
            // which qualifies; otherwise a miss is "capped": the answer lies in the
            // range below the kept entries and phase 2 finds it.
            win_lo = max(stk_lo, stk_hi - 32);
            const int widx = win_lo + lane;
            wvalid = widx < stk_hi;
            wv = wvalid ? sStkV[widx & (K - 1)] : KeyTraits<T>::pad();
            cm = 0;
            if (__any_sync(FULL, sm != 0)) {
                const int wcnt = stk_hi - win_lo;  // window entries (uniform)
                const int wp = wvalid ? sStkP[widx & (K - 1)] : -1;
                // the answer of q: the topmost qualifying window entry (by a 6-step
                // shuffle search), else a binary search below the window; -1 = miss
                auto search = [&](T q, bool act) {
                    int lo = -1;
#pragma unroll
                    for (int s2 = 32; s2 > 0; s2 >>= 1) {
                        const int cand = lo + s2;
                        const T wc = __shfl_sync(FULL, wv, cand & 31);
                        if (act && cand < wcnt && lt<INCL>(wc, q)) lo = cand;
                    }
                    const int ap = __shfl_sync(FULL, wp, lo & 31);
                    int ans = -1;
                    if (act) {
                        ans = lo >= 0 ? ap : -1;
                        if (lo < 0 && win_lo > stk_lo) {
                            int l2 = stk_lo, h2 = win_lo;
                            while (l2 < h2) {
                                const int mid = (l2 + h2) >> 1;
                                if (lt<INCL>(sStkV[mid & (K - 1)], q)) l2 = mid + 1;
                                else h2 = mid;
                            }
                            if (l2 > stk_lo) ans = sStkP[(l2 - 1) & (K - 1)];
                        }
                    }
                    return ans;
                };
                const int cs = __popc(sm);
                int stot;
                const int soff = warp_excl_sum(cs, stot);
                const int smax = (int)__reduce_max_sync(FULL, (unsigned)cs);
                if (smax > 1 && stot <= 32) {
                    // The tile's S keys sit mostly in its first lanes: spread them, one per
                    // lane, over a single round (the X list is consumed, its space is free).
                    __syncwarp();
                    {
                        int o = soff;
                        unsigned m = sm;
                        while (m) {
                            const int k = __ffs(m) - 1;
                            m &= m - 1;
                            sList[o++] = (int16_t)(lane * IPT + k);
                        }
                    }
                    __syncwarp();
                    const bool act = lane < stot;
                    const int e = act ? (int)sList[lane] : 0;
                    const int ans = search(act ? V[ks(e)] : KeyTraits<T>::pad(), act);
                    if (act) O[swz(e)] = ans >= 0 ? ans : -2;  // -2: a miss, flagged by the key's lane
                    if (__any_sync(FULL, act && ans < 0)) {      // (only once the stack has dropped entries)
                        __syncwarp();
                        unsigned m = sm;
                        while (m) {
                            const int k = __ffs(m) - 1;
                            m &= m - 1;
                            if (O[swz(lane * IPT + k)] == -2) {
                                O[swz(lane * IPT + k)] = -1;
                                cm |= 1u << k;
                            }
                        }
                    }
                } else {
                    unsigned m = sm;
                    for (int rd = 0; rd < smax; rd++) {
                        const bool act = m != 0;
                        const int k = act ? __ffs(m) - 1 : 0;
                        m &= m - 1;
                        const int ans = search(act ? V[ks(lane * IPT + k)] : KeyTraits<T>::pad(), act);
                        if (act) {
                            if (ans >= 0) O[swz(lane * IPT + k)] = ans;
                            else cm |= 1u << k;
                        }
                    }
                }
                if (cm && !dropped) atomicOr(err, ERR_INTERNAL);
            }
            }  // steps 1-5

            // ---- 6. flagged keys: deferred (D) and capped (C) -----------------------------
            flag_keys(dm, cm);

            // ---- 7. output: the whole tile, flagged keys as -1 ----------------------------
            store_tile();

            // ---- 8. stack update: pop what the tile dominates, push its suffix minima ----
            if (dtile) {  // (the tile that never increases) push its minimum
                __syncwarp();  // every lane has read the stack
                if (lane == 31) {
                    sStkV[dkeep & (K - 1)] = v[IPT - 1];
                    sStkP[dkeep & (K - 1)] = tile_base + WT - 1;
                }
                stk_hi = dkeep + 1;
                if (stk_hi - K > stk_lo) {
                    stk_lo = stk_hi - K;
                    dropped = true;
                }
            } else {
                const T after_w = __shfl_down_sync(FULL, suf, 1);  // min of the lanes after (lane < 31)
                unsigned fmask = 0;
                const bool has_aft = lane < 31;
                if (!has_aft || lt<false>(lmin, after_w)) {  // else no key here beats every later key
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
                int total;
                const int fpre = warp_excl_sum(fcnt, total);
                // Entries below the tile minimum survive: a bottom part of the stack.
                const unsigned below = __ballot_sync(FULL, wvalid && wv < tile_min_t);
                int keep;
                if (below == __ballot_sync(FULL, wvalid)) {
                    keep = stk_hi;  // the whole window survives, so does everything under it
                } else if (below || win_lo == stk_lo) {
                    keep = win_lo + __popc(below);
                } else {  // the boundary lies under the window (rare)
                    int lo = stk_lo, hi = win_lo;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (sStkV[mid & (K - 1)] < tile_min_t) lo = mid + 1;
                        else hi = mid;
                    }
                    keep = lo;
                }
                __syncwarp();  // every lane has read the old stack
                const int newtop = keep + total;
                {
                    int idx = keep + fpre;
                    unsigned m = fmask;
                    if (idx + fcnt <= newtop - K) m = 0;  // all of this lane's entries drop at once
                    while (m) {
                        const int k = __ffs(m) - 1;
                        m &= m - 1;
                        if (idx >= newtop - K) {
                            sStkV[idx & (K - 1)] = V[ks(lane * IPT + k)];
                            sStkP[idx & (K - 1)] = lb + k;
                        }
                        idx++;
                    }
                }
                stk_hi = newtop;
                if (newtop - K > stk_lo) {
                    stk_lo = newtop - K;
                    dropped = true;
                }
            }

            // ---- 9. tile minimum, range minimum, next load ------------------------------
            if (lane == 0) __stcg(&tile_min_w[t], tile_min_t);
            rmin = has_rmin ? KeyTraits<T>::vmin(rmin, tile_min_t) : tile_min_t;
            has_rmin = true;
            __syncwarp();
            if (lane == 0 && i + kStages < ntr && tile_full(t + kStages)) {
                mbar_arrive_expect_tx(&bar[slot], (uint32_t)(WT * KB));
                tma_load_2d(V, &map_in, 0, tile_row(t + kStages), &bar[slot]);
            }
        }

        // ======================= publish the range, its prefix ======================
        {  // the top of the final stack, for later ranges' deferred keys
            const int tb = max(stk_lo, stk_hi - kTopEntries);
            const int tc = stk_hi - tb;
            T* top_key = (T*)a.s.top_key + (size_t)r * kTopEntries;
            int32_t* top_pos = a.s.top_pos + (size_t)r * kTopEntries;
            if (lane < tc) {
                __stcg(&top_key[lane], sStkV[(tb + lane) & (K - 1)]);
                __stcg(&top_pos[lane], sStkP[(tb + lane) & (K - 1)]);
            }
            if (lane == 0) __stcg(&a.s.top_cnt[r], (uint32_t)tc | ((!dropped && tb == stk_lo) ? 0x80000000u : 0u));
        }
        __syncwarp();  // every lane's words before lane 0's release in range_publish
        range_publish<T>(r, epoch, rmin, a);
        T P, win;
        bool has_p;
        range_prefix<T>(r, epoch, a, P, has_p, win);
        if (lane == 0) {
            bulk_wait0();       // this range's tile stores have landed ...
            fence_proxy_async();  // ... before phase 2 overwrites flagged keys
        }
        __syncwarp();  // lane 0's acquire and wait before every lane's reads and writes

        // ======================= phase 2: flagged keys ===============================
        const T* tile_min_r = (const T*)a.s.tile_min;
        const T* chunk_min_r = (const T*)a.s.chunk_min;
        const int range_begin = t0 * WT;
        auto range_end = [&](int rr) { return min(min((rr + 1) * a.tiles_per_range, a.num_tiles) * WT, a.n); };

        // A. deferred keys: the range's prefix minima, non-increasing, so the ones P
        //    qualifies form a prefix of the list and the rest keep -1.  Each answer is
        //    in the nearest earlier range whose minimum qualifies, at the top of its
        //    published stack (lane-parallel searches), else found by find_left.
        bool a_done = !has_p;
        const int nlist = min(def_total, kDefCap);
        for (int b0 = 0; b0 < nlist && !a_done; b0 += 32) {
            const int j = b0 + lane;
            const bool in = j < nlist;
            const T q = in ? sDefV[j] : KeyTraits<T>::pad();
            const int pos = in ? sDefP[j] : 0;
            const bool want = in && lt<INCL>(P, q);  // (segmented: all of the range's first segment)
            if (__ballot_sync(FULL, want) != __ballot_sync(FULL, in)) a_done = true;
            if (!__any_sync(FULL, want)) break;
            int rp = -1;
#pragma unroll 4
            for (int i2 = 0; i2 < 32; i2++) {
                const T m = __shfl_sync(FULL, win, i2);
                if (want && rp < 0 && r - 1 - i2 >= 0 && lt<INCL>(m, q)) rp = r - 1 - i2;
            }
            {  // no range of the window qualifies: the nearest one below it, key by key
                unsigned nw = __ballot_sync(FULL, want && rp < 0);
                while (nw) {
                    const int f = __ffs(nw) - 1;
                    nw &= nw - 1;
                    const int found = nearest_range<T, INCL>(__shfl_sync(FULL, q, f), r - 33, a);
                    if (lane == f) rp = found;
                }
            }
            int ans = -2;  // -2: not found yet
            if (want && rp >= 0) {
                // rp's published stack top, keys and positions in one round of loads:
                // entries increase from the bottom, so the qualifying ones form a
                // bottom part and the topmost of them answers
                const int cnt = (int)(__ldcg(&a.s.top_cnt[rp]) & 0xffu);
                const uint4* tk = reinterpret_cast<const uint4*>((const T*)a.s.top_key + (size_t)rp * kTopEntries);
                const uint4* tp = reinterpret_cast<const uint4*>(a.s.top_pos + (size_t)rp * kTopEntries);
                if constexpr (KB == 4) {
                    uint4 tw[kTopEntries / 4], pw[kTopEntries / 4];
#pragma unroll
                    for (int k = 0; k < kTopEntries / 4; k++) {
                        tw[k] = __ldcg(&tk[k]);
                        pw[k] = __ldcg(&tp[k]);
                    }
#pragma unroll
                    for (int k = 0; k < kTopEntries / 4; k++) {
                        const uint32_t wb[4] = {tw[k].x, tw[k].y, tw[k].z, tw[k].w};
                        const int pb[4] = {(int)pw[k].x, (int)pw[k].y, (int)pw[k].z, (int)pw[k].w};
#pragma unroll
                        for (int c = 0; c < 4; c++)
                            if (4 * k + c < cnt && lt<INCL>(KeyTraits<T>::from_bits(wb[c]), q)) ans = pb[c];
                    }
                } else {  // two 8-byte keys per 16-byte load
                    uint4 tw[kTopEntries / 2], pw[kTopEntries / 4];
#pragma unroll
                    for (int k = 0; k < kTopEntries / 2; k++) tw[k] = __ldcg(&tk[k]);
#pragma unroll
                    for (int k = 0; k < kTopEntries / 4; k++) pw[k] = __ldcg(&tp[k]);
#pragma unroll
                    for (int k = 0; k < kTopEntries / 2; k++) {
                        const uint64_t kb2[2] = {((uint64_t)tw[k].y << 32) | tw[k].x, ((uint64_t)tw[k].w << 32) | tw[k].z};
                        const uint4 p4 = pw[k / 2];
                        const int pb2[2] = {(int)(k % 2 ? p4.z : p4.x), (int)(k % 2 ? p4.w : p4.y)};
#pragma unroll
                        for (int c = 0; c < 2; c++)
                            if (2 * k + c < cnt && lt<INCL>(KeyTraits<T>::from_bits(kb2[c]), q)) ans = pb2[c];
                    }
                }
            }
            unsigned fb = __ballot_sync(FULL, want && ans == -2);
            while (fb) {
                const int f = __ffs(fb) - 1;
                fb &= fb - 1;
                const T qf = __shfl_sync(FULL, q, f);
                const int rpf = __shfl_sync(FULL, rp, f);
                const int lim = rpf >= 0 ? range_end(rpf) : range_begin;
                const int found = find_left<T, WT, INCL, MAPF, REV>(qf, lim, d_in, tile_min_r, chunk_min_r, a);
                if (lane == f) ans = found;
            }
            if (want) {
                if (ans < 0) atomicOr(err, ERR_INTERNAL);
                else if (!head || pos >= head) put(pos, SEG ? seg_rel(ans, first_start) : ans);
            }
        }
        if (!a_done && def_total > kDefCap) {
            // A'. the list overflowed and P qualified every listed key: continue over
            //     the tile flags after the last listed key, with a monotone cursor
            //     (answers of non-increasing queries only move left).
            //     Flag words 32 tiles per load (lane i: tile tb + i), a tile's mask
            //     words in one load (lane w: word w): the scan pays one L2 round
            //     trip per 32 tiles and one per flagged tile, not one per tile and word.
            const int from = sDefP[kDefCap - 1] + 1;
            int cur = -1;
            T cv = KeyTraits<T>::pad();
            static_assert(W <= 16, "two tiles' mask words per load");
            for (int tb = from / WT; tb < t1 && !a_done; tb += 32) {
              const bool tin = tb + lane < t1;
              const uint32_t tfl = tin ? __ldcg(&a.s.tile_flag[tb + lane]) : 0u;
              const T tmn = tin ? __ldcg(&tile_min_r[tb + lane]) : KeyTraits<T>::pad();
              unsigned fl = __ballot_sync(FULL, (tfl & 0x7fffffffu) != 0);
              while (fl && !a_done) {
                // Flagged tiles whose pending keys all take the cursor: not mixed, and
                // P and the cursor's key both qualify for the tile's minimum (<= every
                // pending key).  Pending keys do not increase, so these form a prefix
                // of the flagged tiles; their keys are not read, and the mask words of
                // two tiles come in one load (lanes 0-15 and 16-31).
                const unsigned fast = __ballot_sync(
                    FULL, ((fl >> lane) & 1u) && (tfl >> 31) == 0 && cur >= 0 && lt<INCL>(P, tmn) && lt<INCL>(cv, tmn));
                const unsigned slow = fl & ~fast;
                unsigned take = slow ? fl & ((slow & (0u - slow)) - 1u) : fl;
                fl &= ~take;
                while (take) {
                    const int ta = __ffs(take) - 1;
                    take &= take - 1;
                    const int tb2 = take ? __ffs(take) - 1 : -1;
                    if (take) take &= take - 1;
                    const int mine = lane < 16 ? ta : tb2;
                    const uint32_t mw2 =
                        mine >= 0 && (lane & 15) < W ? __ldcg(&a.s.tile_mask[(size_t)(tb + mine) * MW + (lane & 15)]) : 0u;
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int tt = h ? tb2 : ta;
                        if (tt < 0) break;
#pragma unroll
                        for (int w = 0; w < W; w++) {
                            const uint32_t mw = __shfl_sync(FULL, mw2, 16 * h + w);
                            const int pos = (tb + tt) * WT + w * 32 + lane;
                            if (((mw >> lane) & 1u) && pos >= from && (!head || pos >= head))
                                put(pos, SEG ? seg_rel(cur, first_start) : cur);
                        }
                    }
                }
                if (!fl) break;
                // the first other flagged tile, key by key
                const int fsrc = __ffs(fl) - 1;
                fl &= fl - 1;
                const int t = tb + fsrc;
                const bool mixed = (__shfl_sync(FULL, tfl, fsrc) >> 31) != 0;
                const uint32_t mwl = lane < W ? __ldcg(&a.s.tile_mask[(size_t)t * MW + lane]) : 0u;
                // The tile's pending keys, every word's loads in flight together, staged
                // in the idle TMA ring (each lane reads back only its own slots).
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const uint32_t mw = __shfl_sync(FULL, mwl, w);
                    const int pos = t * WT + w * 32 + lane;
                    const bool pk = ((mw >> lane) & 1u) && pos >= from && (!head || pos >= head);
                    sV[w * 32 + lane] = pk ? key_at<T, MAPF, REV>(d_in, a.n, pos) : KeyTraits<T>::pad();
                }
                for (int w = 0; w < W && !a_done; w++) {
                    const uint32_t mw = __shfl_sync(FULL, mwl, w);
                    const int pos = t * WT + w * 32 + lane;
                    unsigned pend = __ballot_sync(FULL, ((mw >> lane) & 1u) && pos >= from && (!head || pos >= head));
                    if (!pend) continue;
                    const T q = ((pend >> lane) & 1u) ? sV[w * 32 + lane] : KeyTraits<T>::pad();
                    if (mixed) {  // deferred and capped keys: a full search each
                        while (pend) {
                            const int f = __ffs(pend) - 1;
                            pend &= pend - 1;
                            const int pf = t * WT + w * 32 + f;
                            const int found = find_left<T, WT, INCL, MAPF, REV>(__shfl_sync(FULL, q, f), pf, d_in, tile_min_r,
                                                                     chunk_min_r, a);
                            int sf = 0;
                            if constexpr (SEG) sf = (int)seg_off(seg_idx(pf - head)) + head;
                            if (lane == f) {
                                if (found < -1) atomicOr(err, ERR_INTERNAL);
                                else put(pos, SEG ? seg_rel(found, sf) : found);
                            }
                        }
                        continue;
                    }
                    const unsigned wq = __ballot_sync(FULL, ((pend >> lane) & 1u) && lt<INCL>(P, q));
                    if (wq != pend) {
                        a_done = true;
                        pend = wq;
                    }
                    while (pend) {
                        // the pending keys, in order, up to the first one the cursor's
                        // key does not qualify for, take the cursor
                        const unsigned ok = __ballot_sync(FULL, ((pend >> lane) & 1u) && cur >= 0 && lt<INCL>(cv, q));
                        const unsigned fail = pend & ~ok;
                        const unsigned tk = fail ? (pend & ((fail & (0u - fail)) - 1u)) : pend;
                        if ((tk >> lane) & 1u) put(pos, SEG ? seg_rel(cur, first_start) : cur);
                        pend &= ~tk;
                        if (!pend) break;
                        const int f = __ffs(pend) - 1;
                        const T qf = __shfl_sync(FULL, q, f);
                        // qf's answer lies before the range: in the nearest earlier range
                        // whose minimum qualifies (the window, else the group minima), at
                        // the topmost qualifying entry of that range's final stack (every
                        // key after it there is >= qf); find_left when the published top
                        // part does not reach it
                        int found = -2;
                        {
                            const unsigned wm = __ballot_sync(FULL, r - 1 - lane >= 0 && lt<INCL>(win, qf));
                            const int rpf = wm ? r - 1 - (__ffs(wm) - 1) : nearest_range<T, INCL>(qf, r - 33, a);
                            if (rpf >= 0) {
                                const int cnt = (int)(__ldcg(&a.s.top_cnt[rpf]) & 0xffu);
                                const T tkey = lane < cnt ? __ldcg(&((const T*)a.s.top_key)[(size_t)rpf * kTopEntries + lane])
                                                          : KeyTraits<T>::pad();
                                const unsigned m = __ballot_sync(FULL, lane < cnt && lt<INCL>(tkey, qf));
                                found = m ? __ldcg(&a.s.top_pos[(size_t)rpf * kTopEntries + 31 - __clz(m)])
                                          : find_left<T, WT, INCL, MAPF, REV>(qf, range_end(rpf), d_in, tile_min_r, chunk_min_r, a);
                            }
                        }
                        if (found < 0) {
                            if (lane == 0) atomicOr(err, ERR_INTERNAL);
                            pend = 0;
                            a_done = true;
                        } else {
                            cur = found;
                            cv = key_at<T, MAPF, REV>(d_in, a.n, cur);
                        }
                    }
                }
              }
            }
        }

        // B. capped keys: the answer is in the range, below the stack's kept part.
        const int ncap = min(cap_total, kCapCap);
        for (int j = 0; j < ncap; j++) {
            const int pos = sCapP[j];
            const int found = find_left<T, WT, INCL, MAPF, REV>(key_at<T, MAPF, REV>(d_in, a.n, pos), pos, d_in, tile_min_r,
                                                           chunk_min_r, a);
            if (lane == 0) {
                if (found < 0) atomicOr(err, ERR_INTERNAL);
                else if (!head || pos >= head) put(pos, SEG ? seg_rel(found, sCapS[j]) : found);
            }
        }
        if (cap_total > kCapCap) {
            // B'. the capped list overflowed: every flagged key of the mixed tiles after it
            //     (flag and mask words loaded 32 at a time, as in A')
            const int from = sCapP[kCapCap - 1] + 1;
            for (int tb = from / WT; tb < t1; tb += 32) {
              const uint32_t tfl = tb + lane < t1 ? __ldcg(&a.s.tile_flag[tb + lane]) : 0u;
              unsigned fl = __ballot_sync(FULL, (tfl >> 31) != 0);
              while (fl) {
                const int t = tb + __ffs(fl) - 1;
                fl &= fl - 1;
                const uint32_t mwl = lane < W ? __ldcg(&a.s.tile_mask[(size_t)t * MW + lane]) : 0u;
                for (int w = 0; w < W; w++) {
                    const uint32_t mw = __shfl_sync(FULL, mwl, w);
                    const int pos = t * WT + w * 32 + lane;
                    unsigned pend = __ballot_sync(FULL, ((mw >> lane) & 1u) && pos >= from && (!head || pos >= head));
                    while (pend) {
                        const int f = __ffs(pend) - 1;
                        pend &= pend - 1;
                        const int pf = t * WT + w * 32 + f;
                        const int found =
                            find_left<T, WT, INCL, MAPF, REV>(key_at<T, MAPF, REV>(d_in, a.n, pf), pf, d_in, tile_min_r, chunk_min_r, a);
                        int sf = 0;
                        if constexpr (SEG) sf = (int)seg_off(seg_idx(pf - head)) + head;
                        if (lane == f) {
                            if (found < -1) atomicOr(err, ERR_INTERNAL);
                            else put(pf, SEG ? seg_rel(found, sf) : found);
                        }
                    }
                }
              }
            }
        }
    }

    // ---- run bookkeeping: the last warp resets the control block --------------------------
    // (the last warp of each CTA counts the CTA in; the last CTA resets)
    __syncwarp();
    int last = 0;
    if (lane == 0 && atomicAdd(&sCta[1], 1) == WPC - 1) {
        __threadfence();
        const uint32_t prev = atomicAdd(&a.s.ctr->done, 1u);
        last = prev == gridDim.x - 1;
        if (last) {
            a.s.ctr->range_counter = 0;
            a.s.ctr->done = 0;
            a.s.ctr->finished = 0;
            a.s.ctr->epoch = epoch >= EPOCH_LIMIT ? 1u : epoch + 1u;  // (the launch's end publishes these)
        }
    }
    last = __shfl_sync(FULL, last, 0);
    if (last && epoch >= EPOCH_LIMIT) {  // once per 2^30 runs: stale words could alias
        for (int i = lane; i < a.s.max_ranges; i += 32) a.s.range_state[i] = 0;
        for (int i = lane; i < a.s.max_ranges / 32; i += 32) a.s.group_min[i] = ~0ull;
        for (int i = lane; i < kMaxCtas; i += 32) a.s.cta_ready[(size_t)i * kReadyStride] = 0;
    }
}

// ---------------------------------------------------------------------------
// Launch plumbing shared by the single-array and segmented translation units.
// ---------------------------------------------------------------------------
template <typename T, int IPT, int WPC, bool INCL, bool SEG, bool EP, int MAPF = KMAP_NONE, int OUTM = OUT_I32,
          bool REV = false>
inline cudaError_t launch_t(RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo, cudaStream_t st,
                            int max_warps) {
    constexpr size_t smem = kernel_smem_bytes<IPT, WPC, (int)sizeof(T)>();
    int tpr = (a.num_tiles + max_warps - 1) / max_warps;
    if (tpr < 1) tpr = 1;
    a.tiles_per_range = tpr;
    a.num_ranges = (a.num_tiles + tpr - 1) / tpr;
    const int ctas = (a.num_ranges + WPC - 1) / WPC;
    apse_warp_kernel<T, IPT, WPC, INCL, SEG, EP, MAPF, OUTM, REV><<<ctas, WPC * 32, smem, st>>>(mi, mo, a);
    return cudaGetLastError();
}

template <typename T, int IPT, int WPC, bool INCL, bool SEG, bool EP, int MAPF = KMAP_NONE, int OUTM = OUT_I32,
          bool REV = false>
inline cudaError_t prepare_t(int* ctas_per_sm) {
    constexpr size_t smem = kernel_smem_bytes<IPT, WPC, (int)sizeof(T)>();
    auto k = apse_warp_kernel<T, IPT, WPC, INCL, SEG, EP, MAPF, OUTM, REV>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, WPC * 32, smem);
    if (e != cudaSuccess) return e;
    if (*ctas_per_sm == 0 || n < *ctas_per_sm) *ctas_per_sm = n;
    return cudaSuccess;
}

// Shared-memory attributes and occupancy of every kernel of one mode and
// configuration (the smallest CTAs-per-SM over the four key/comparison types).
template <bool SEG, bool EP>
inline cudaError_t prepare_mode(int cfg, int* per_sm) {
#define P_(IPT, WPC)                                                                   \
    {                                                                                  \
        cudaError_t rr[4] = {prepare_t<int32_t, IPT, WPC, false, SEG, EP>(per_sm),     \
                             prepare_t<int32_t, IPT, WPC, true, SEG, EP>(per_sm),      \
                             prepare_t<float, IPT, WPC, false, SEG, EP>(per_sm),       \
                             prepare_t<float, IPT, WPC, true, SEG, EP>(per_sm)};       \
        for (int q = 0; q < 4; q++)                                                    \
            if (rr[q] != cudaSuccess) return rr[q];                                    \
    }
    switch (cfg) {
    case 0: P_(16, 16); break;
    case 1: P_(8, 8); break;
    case 2: P_(16, 8); break;
    case 3: P_(8, 16); break;
    case 4: P_(16, 4); break;
    case 5: P_(8, 4); break;
    default: return cudaErrorInvalidValue;
    }
#undef P_
    return cudaSuccess;
}

template <bool SEG, bool EP>
inline cudaError_t launch_mode(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& mi,
                               const CUtensorMap& mo, cudaStream_t st, int max_warps) {
#define L_(IPT, WPC)                                                                        \
    if (dtype == 0)                                                                         \
        return incl ? launch_t<int32_t, IPT, WPC, true, SEG, EP>(a, mi, mo, st, max_warps)  \
                    : launch_t<int32_t, IPT, WPC, false, SEG, EP>(a, mi, mo, st, max_warps); \
    else                                                                                    \
        return incl ? launch_t<float, IPT, WPC, true, SEG, EP>(a, mi, mo, st, max_warps)    \
                    : launch_t<float, IPT, WPC, false, SEG, EP>(a, mi, mo, st, max_warps);
    switch (cfg) {
    case 0: L_(16, 16);
    case 1: L_(8, 8);
    case 2: L_(16, 8);
    case 3: L_(8, 16);
    case 4: L_(16, 4);
    case 5: L_(8, 4);
    }
#undef L_
    return cudaErrorInvalidValue;
}

}  // namespace apsep
