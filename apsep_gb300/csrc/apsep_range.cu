// apsep_range.cu -- single-array APSE engine for sm_103a (persistent ranges).
//
// One launch.  Each persistent CTA claims a contiguous RANGE of tiles
// (dynamic range ids, so every range a CTA may wait on belongs to a CTA that
// is already running) and sweeps it left to right:
//
//  Phase 1, per tile of B = NT*IPT keys (a ring of S TMA stages keeps the
//  next tiles' 128-byte-swizzled loads in flight):
//   1. in-thread ANSV over IPT consecutive keys in registers (compare
//      ladder) -- the in-thread step of apsepKernelSPT (src/apsep.cuh:2701-2707);
//   2. warp prefix/suffix mins over thread mins (src/apsep.cuh:2709-2730);
//   3. keys unresolved in-thread walk the tile's answer chain in shared
//      memory: each key's next candidate is its in-thread answer, or, for a
//      thread's minimum, the previous thread's last key -- one pointer walk
//      that replaces the reference's pointer-jumping chain plus spine walk
//      plus cross-warp fallback (src/apsep.cuh:2734-2801);
//   4. keys with no answer in the tile query the RANGE STACK: the strict
//      suffix minima of the range's earlier tiles, kept in shared memory
//      (binary search).  This replaces the reference's global min-tree
//      descent (src/apsep.cuh:2952-2996) for every answer inside the range;
//   5. keys with no answer in the range are "deferred" (they are the range's
//      prefix minima) -- only these wait for the global prefix;
//   6. the tile's answers leave shared memory in one TMA store; the stack is
//      updated with the tile's strict suffix minima.
//  Then the range publishes its minimum as a decoupled look-back aggregate
//  and warp 0 looks back over earlier ranges (helping them publish their
//  inclusive values) for the exclusive prefix minimum P.  Every wait is
//  bounded and reports ERR_LOOKBACK_TIMEOUT / ERR_TMA_TIMEOUT.
//
//  Phase 2: deferred keys answer -1 when P does not qualify (the reference's
//  prefix-min early-out, src/apsep.cuh:2903-2926: whole tiles become one TMA
//  store of -1), otherwise a warp-cooperative search left through tile mins,
//  chunk mins and one 32-key row of the input; deferred keys are
//  non-increasing, so one monotone cursor serves them all.
//
// Compared with the reference's three grid-wide phases there is no
// grid.sync(); the only cross-CTA waits are one look-back per range.  Every
// output word is written once (phase 1 skips deferred keys, phase 2 writes
// exactly those).
#include "apsep_device.cuh"
#include "apsep_internal.h"

namespace apsep {

const TileConfig kTileConfigs[kNumTileConfigs] = {
    {256, 16},  // 4096 keys / tile
    {512, 8},   // 4096 keys / tile
};

constexpr int kStages = 3;      // TMA ring depth (tiles)
constexpr int kStackCap = 1024;  // range-stack entries kept in shared memory

template <int NT, int IPT>
struct RLayout {
    static constexpr int B = NT * IPT;
    static constexpr int NW = NT / 32;
    static constexpr int W = B / 32;
    static constexpr size_t kV = 0;                                   // T[S][B], swizzled (TMA dst)
    static constexpr size_t kO = kV + (size_t)kStages * B * 4;         // int32[2][B], swizzled (TMA src)
    static constexpr size_t kNext = kO + (size_t)2 * B * 4;            // int16[B]
    static constexpr size_t kWmin = kNext + (size_t)B * 2;             // T[NW]
    static constexpr size_t kWcnt = kWmin + (size_t)NW * 4;            // int32[NW]
    static constexpr size_t kDef = (kWcnt + (size_t)NW * 4 + 15) & ~(size_t)15;  // uint32[2][W]
    static constexpr size_t kStkV = kDef + (size_t)2 * W * 4;          // T[K]
    static constexpr size_t kStkP = kStkV + (size_t)kStackCap * 4;     // int32[K]
    static constexpr size_t kMisc = (kStkP + (size_t)kStackCap * 4 + 15) & ~(size_t)15;
    static constexpr size_t kEnd = kMisc + 256;
    static constexpr size_t kBytes = kEnd + 1024;  // + alignment slack
};

struct alignas(16) RMisc {
    uint64_t full_bar[kStages];
    int range;
    uint32_t epoch;
    int stk_top;  // logical size of the range stack
    int stk_lo;   // lowest logical index still stored
    uint32_t rmin_bits;
    int has_rmin;
    int keep;
    int def_cnt;
    int def_saved;
    uint32_t p_bits;
    int has_p;
    int last_cta;
    int stop;  // phase 2: deferred keys at or after this position answer -1
};
static_assert(sizeof(RMisc) <= 256, "misc block");

__device__ __forceinline__ uint32_t make_tag(uint32_t epoch, uint32_t flag) { return (epoch << 2) | flag; }

// ---------------------------------------------------------------------------
// Warp-cooperative search: the rightmost position p < limit (limit > 0) with
// lt(d_in[p], q), or -1.  Every tile below tile(limit-1) and every chunk of
// it must have published tile_min / chunk_min.  Reads of the published
// arrays go to L2 (ld.cg); the keys are read-only.
// ---------------------------------------------------------------------------
template <typename T, int B, bool INCL>
__device__ __noinline__ int find_left(T q, int limit, const T* __restrict__ d_in, const T* __restrict__ tile_min,
                                      const T* __restrict__ chunk_min) {
    constexpr int W = B / 32;
    const int lane = threadIdx.x & 31;
    if (limit <= 0) return -1;
    const int last = limit - 1;
    const int t = last / B;
    const int c = (last - t * B) >> 5;
    // 1. the row holding limit-1, positions below limit
    {
        const int row = t * B + c * 32;
        const int p = row + lane;
        const bool ok = p < limit && lt<INCL>(__ldg(&d_in[p]), q);
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (m) return row + 31 - __clz(m);
    }
    // 2. earlier chunks of that tile
    int s = t, cc = -1;
    for (int g = (c - 1) >> 5; g >= 0 && cc < 0; g--) {
        const int ci = g * 32 + lane;
        const bool ok = ci < c && lt<INCL>(__ldcg(&chunk_min[(size_t)t * W + ci]), q);
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (m) cc = g * 32 + 31 - __clz(m);
    }
    // 3. earlier tiles
    if (cc < 0) {
        s = -1;
        for (int base = t - 1; base >= 0 && s < 0; base -= 32) {
            const int idx = base - lane;
            const bool ok = idx >= 0 && lt<INCL>(__ldcg(&tile_min[idx]), q);
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (m) s = base - (__ffs(m) - 1);
        }
        if (s < 0) return -1;
        for (int g = (W + 31) / 32 - 1; g >= 0 && cc < 0; g--) {
            const int ci = g * 32 + lane;
            const bool ok = ci < W && lt<INCL>(__ldcg(&chunk_min[(size_t)s * W + ci]), q);
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (m) cc = g * 32 + 31 - __clz(m);
        }
        if (cc < 0) return -2;  // tile min qualified but no chunk did: invariant broken
    }
    const int row = s * B + cc * 32;
    const unsigned m = __ballot_sync(0xffffffffu, lt<INCL>(__ldg(&d_in[row + lane]), q));
    return m ? row + 31 - __clz(m) : -2;
}

// ---------------------------------------------------------------------------
// Decoupled look-back over ranges (one full warp).  Returns the exclusive
// prefix min of range r, publishes r's inclusive value, and publishes the
// inclusive values of the ranges it passed in the final window ("helping"),
// so the inclusive frontier jumps forward instead of crawling.
// ---------------------------------------------------------------------------
template <typename T, bool INCL>
__device__ void range_lookback(int r, uint32_t epoch, T rmin, const RangeArgs& a, T& p, bool& has_p) {
    const int lane = threadIdx.x & 31;
    uint64_t* state = a.s.range_state;
    T acc = KeyTraits<T>::pad();
    bool has = false;
    if (r > 0) {
        uint32_t spins = 0;
        int base = r - 1;
        while (true) {
            const int idx = base - lane;
            uint32_t flag = FLAG_INCL;  // before range 0: an empty inclusive prefix
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
                if (spins > 8) __nanosleep(spins < 256 ? 64 : 512);
                continue;
            }
            const bool contrib = lane <= fi && idx >= 0;
            const T mine = contrib ? KeyTraits<T>::from_bits(vbits) : KeyTraits<T>::pad();
            // Suffix scan from lane fi down to lane: s(lane) = min(mine[lane..fi]).
            T sfx = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const T nb = __shfl_down_sync(0xffffffffu, sfx, o);
                if (lane + o <= fi && lane + o < 32) sfx = KeyTraits<T>::vmin(sfx, nb);
            }
            const T win = __shfl_sync(0xffffffffu, sfx, 0);  // min over the window's contributors
            const bool any = __any_sync(0xffffffffu, contrib);
            if (fi < 32 && lane < fi && idx >= 0 && flag == FLAG_AGG && idx != a.skip_publish_range) {
                // Range idx's inclusive prefix covers ranges <= idx only: the INCL
                // at lane fi plus the aggregates of lanes fi-1..lane, i.e. sfx.
                st_release_u64(&state[idx], ((uint64_t)make_tag(epoch, FLAG_INCL) << 32) | KeyTraits<T>::bits(sfx));
            }
            if (any) {
                acc = has ? KeyTraits<T>::vmin(acc, win) : win;
                has = true;
            }
            if (fi < 32) break;
            base -= 32;
        }
    }
    if (lane == 0 && r != a.skip_publish_range) {
        const T incl_v = has ? KeyTraits<T>::vmin(acc, rmin) : rmin;
        st_release_u64(&state[r], ((uint64_t)make_tag(epoch, FLAG_INCL) << 32) | KeyTraits<T>::bits(incl_v));
    }
    p = acc;
    has_p = has;
}

template <typename T, int NT, int IPT, bool INCL>
__global__ void __launch_bounds__(NT, 2)
apse_range_kernel(const __grid_constant__ CUtensorMap map_in, const __grid_constant__ CUtensorMap map_out,
                  const RangeArgs a) {
    using L = RLayout<NT, IPT>;
    constexpr int B = NT * IPT;
    constexpr int NW = NT / 32;
    constexpr int W = B / 32;
    constexpr int TPC = 32 / IPT;  // threads per 32-key chunk
    constexpr int ROWS = B / 32;   // TMA box rows (128-byte rows)
    constexpr int K = kStackCap;
    static_assert(IPT == 4 || IPT == 8 || IPT == 16, "IPT must be 4, 8 or 16");
    static_assert(ROWS <= 256 && B <= kMaxTileKeys, "tile too large");

    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    T* sVall = (T*)(sm + L::kV);
    int32_t* sOall = (int32_t*)(sm + L::kO);
    int16_t* sNext = (int16_t*)(sm + L::kNext);
    T* sWmin = (T*)(sm + L::kWmin);
    int32_t* sWcnt = (int32_t*)(sm + L::kWcnt);
    uint32_t* sDefAll = (uint32_t*)(sm + L::kDef);
    T* sStkV = (T*)(sm + L::kStkV);
    int32_t* sStkP = (int32_t*)(sm + L::kStkP);
    RMisc* misc = (RMisc*)(sm + L::kMisc);

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const T* d_in = (const T*)a.d_in;
    T* tile_min_w = (T*)a.s.tile_min;
    T* chunk_min_w = (T*)a.s.chunk_min;
    uint32_t* err = &a.s.ctr->err;
    const unsigned FULL = 0xffffffffu;

    // ---- claim a range, start its first loads ------------------------------------------
    if (tid == 0) {
        misc->range = (int)atomicAdd(&a.s.ctr->range_counter, 1u);
        misc->epoch = ld_relaxed_u32(&a.s.ctr->epoch);
        misc->stk_top = 0;
        misc->stk_lo = 0;
        misc->has_rmin = 0;
        misc->def_cnt = 0;
        for (int s = 0; s < kStages; s++) mbar_init(&misc->full_bar[s], 1);
        fence_mbarrier_init();
        fence_proxy_async_smem();
    }
    for (int i = tid; i < 2 * W; i += NT) sDefAll[i] = 0;
    __syncthreads();
    const int r = misc->range;
    const uint32_t epoch = misc->epoch;
    if (r >= a.num_ranges) {  // a stale range counter: report, never index past the arrays
        if (tid == 0) atomicOr(err, ERR_INTERNAL);
        return;
    }
    const int t0 = r * a.tiles_per_range;
    const int t1 = min(t0 + a.tiles_per_range, a.num_tiles);
    const int ntr = t1 - t0;
    auto tile_full = [&](int t) { return a.tma_rows > 0 && (t + 1) * ROWS <= a.tma_rows; };
    if (tid == 0) {
        for (int i = 0; i < kStages && i < ntr; i++)
            if (tile_full(t0 + i)) {
                mbar_arrive_expect_tx(&misc->full_bar[i], (uint32_t)(B * 4));
                tma_load_2d(sVall + (size_t)i * B, &map_in, 0, (t0 + i) * ROWS, &misc->full_bar[i]);
            }
    }

    // =========================== phase 1: the range's tiles ===========================
    for (int i = 0; i < ntr; i++) {
        const int t = t0 + i;
        const int slot = i % kStages;
        const uint32_t par = (uint32_t)((i / kStages) & 1);
        T* V = sVall + (size_t)slot * B;
        int32_t* O = sOall + (size_t)(i & 1) * B;
        uint32_t* sDef = sDefAll + (size_t)(i & 1) * W;
        const bool full = tile_full(t);
        const bool last_of_range = (i == ntr - 1);
        const int tile_base = t * B;
        const int valid_keys = min(B, a.n - tile_base);

        if (full) {
            if (!mbar_wait_bounded(&misc->full_bar[slot], par, a.spin_limit)) {
                if (tid == 0) atomicOr(err, ERR_TMA_TIMEOUT);
            }
        } else {
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const int e = j * NT + tid;
                const int g = tile_base + e;
                V[swz(e)] = g < a.n ? d_in[g] : KeyTraits<T>::pad();
            }
            __syncthreads();
        }

        // ---- 1. in-thread ANSV ------------------------------------------------------
        T v[IPT];
#pragma unroll
        for (int q4 = 0; q4 < IPT / 4; q4++) {
            const uint4 rr = *reinterpret_cast<const uint4*>(&V[swz(tid * IPT + 4 * q4)]);
            v[4 * q4 + 0] = KeyTraits<T>::from_bits(rr.x);
            v[4 * q4 + 1] = KeyTraits<T>::from_bits(rr.y);
            v[4 * q4 + 2] = KeyTraits<T>::from_bits(rr.z);
            v[4 * q4 + 3] = KeyTraits<T>::from_bits(rr.w);
        }
        int res[IPT];
        res[0] = -1;
#pragma unroll
        for (int k = 1; k < IPT; k++) {
            int rk = -1;
#pragma unroll
            for (int j = 0; j < k; j++)
                if (lt<INCL>(v[j], v[k])) rk = j;
            res[k] = rk;
        }
        T tmin = v[0];
#pragma unroll
        for (int k = 1; k < IPT; k++) tmin = KeyTraits<T>::vmin(tmin, v[k]);
        {
            T cm = tmin;
#pragma unroll
            for (int o = 1; o < TPC; o <<= 1) cm = KeyTraits<T>::vmin(cm, __shfl_xor_sync(FULL, cm, o));
            if ((lane & (TPC - 1)) == 0) __stcg(&chunk_min_w[(size_t)t * W + tid / TPC], cm);
        }
        const int nvalid = min(max(a.n - (tile_base + tid * IPT), 0), IPT);
        unsigned umask = 0;
#pragma unroll
        for (int k = 0; k < IPT; k++)
            if (res[k] < 0 && k < nvalid) umask |= 1u << k;
#pragma unroll
        for (int q4 = 0; q4 < IPT / 4; q4++) {
            int4 o;
            o.x = res[4 * q4 + 0] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 0] : -1;
            o.y = res[4 * q4 + 1] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 1] : -1;
            o.z = res[4 * q4 + 2] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 2] : -1;
            o.w = res[4 * q4 + 3] >= 0 ? tile_base + tid * IPT + res[4 * q4 + 3] : -1;
            *reinterpret_cast<int4*>(&O[swz(tid * IPT + 4 * q4)]) = o;
        }
        // ---- 2. warp prefix / suffix mins ----------------------------------------------
        T pre = tmin;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T nb = __shfl_up_sync(FULL, pre, o);
            if (lane >= o) pre = KeyTraits<T>::vmin(pre, nb);
        }
        const T carry = __shfl_up_sync(FULL, pre, 1);  // lanes < this one (lane > 0)
        T suf = tmin;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T nb = __shfl_down_sync(FULL, suf, o);
            if (lane + o < 32) suf = KeyTraits<T>::vmin(suf, nb);
        }
        const T after_w = __shfl_down_sync(FULL, suf, 1);  // lanes > this one (lane < 31)
        // Thread chain: the nearest earlier lane whose min qualifies for this
        // thread's min (pointer jumping; invariant: every lane strictly between
        // g and this lane fails lt(., tmin); g only decreases, <= 31 rounds).
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
            // Next candidate after a key that does not qualify for the query: its
            // in-thread answer; for a key with none (the thread's minimum, which
            // then bounds the whole thread) the last key of the chain thread; when
            // no thread of this warp qualifies, -2 - warp (look in earlier warps).
            const int jump = g >= 0 ? (warp * 32 + g) * IPT + IPT - 1 : (warp > 0 ? -2 - warp : -1);
            uint32_t pk[IPT / 2];
#pragma unroll
            for (int p = 0; p < IPT / 2; p++) {
                const int a0 = res[2 * p] >= 0 ? tid * IPT + res[2 * p] : jump;
                const int a1 = res[2 * p + 1] >= 0 ? tid * IPT + res[2 * p + 1] : jump;
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

        if (lane == 31) sWmin[warp] = pre;
        __syncthreads();  // B1

        // ---- 3. CTA-level prefix/suffix, stack-push flags -----------------------------
        bool has_x = lane > 0;
        T x = carry;
        for (int w = 0; w < warp; w++) {
            x = has_x ? KeyTraits<T>::vmin(x, sWmin[w]) : sWmin[w];
            has_x = true;
        }
        unsigned fmask = 0;
        int fcnt = 0;
        if (!last_of_range) {
            bool has_run = lane < 31;
            T run = after_w;
            for (int w = warp + 1; w < NW; w++) {
                run = has_run ? KeyTraits<T>::vmin(run, sWmin[w]) : sWmin[w];
                has_run = true;
            }
#pragma unroll
            for (int k = IPT - 1; k >= 0; k--) {
                if (!has_run || v[k] < run) fmask |= 1u << k;  // strict suffix minimum
                run = has_run ? KeyTraits<T>::vmin(run, v[k]) : v[k];
                has_run = true;
            }
            fcnt = __popc(fmask);
        }
        int fpre = fcnt;  // warp inclusive prefix of counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int nb = __shfl_up_sync(FULL, fpre, o);
            if (lane >= o) fpre += nb;
        }
        if (lane == 31) sWcnt[warp] = fpre;
        fpre -= fcnt;  // exclusive
        T tile_min_t = sWmin[0];
        if (tid == 0) {
#pragma unroll
            for (int w = 1; w < NW; w++) tile_min_t = KeyTraits<T>::vmin(tile_min_t, sWmin[w]);
            __stcg(&tile_min_w[t], tile_min_t);
            // bit 32: a range prefix exists; bit 33: the stack had dropped entries, so a
            // deferred key of this tile may have its answer inside the range
            __stcg(&a.s.tile_rpre[t], misc->has_rmin ? ((1ull << 32) | (misc->stk_lo > 0 ? (1ull << 33) : 0ull) |
                                                         misc->rmin_bits)
                                                      : 0ull);
            int keep = misc->stk_lo;
            if (!last_of_range) {
                int lo = misc->stk_lo, hi = misc->stk_top;  // count stored entries < tile min
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (sStkV[mid % K] < tile_min_t) lo = mid + 1;
                    else hi = mid;
                }
                keep = lo;
            }
            misc->keep = keep;
        }

        // ---- 4. keys unresolved in-thread: walk the tile's answer chain ------------------
        // Queries (in-thread prefix minima) come in non-increasing order, so
        // the cursor c only moves left.  A query is walked only when some key
        // of the tile before this thread qualifies (lt(x, q)), so the walk
        // always ends inside the tile.
        unsigned cu = 0;
        unsigned Q = umask;
        if (Q) {
            int k = __ffs(Q) - 1;  // k == 0
            Q &= Q - 1;
            T q = v[0];
            int c = tid * IPT - 1;
            if (!has_x || !lt<INCL>(x, q)) {
                cu = umask;
            } else {
                int guard = 2 * B + 64;
                T cv = V[swz(c)];
                while (true) {
                    if (lt<INCL>(cv, q)) {
                        O[swz(tid * IPT + k)] = tile_base + c;
                        if (!Q) break;
                        k = __ffs(Q) - 1;
                        Q &= Q - 1;
                        q = V[swz(tid * IPT + k)];
                        if (!lt<INCL>(x, q)) {
                            cu = (1u << k) | Q;
                            break;
                        }
                    } else {
                        c = sNext[c];
                        if (c <= -2) {  // leave this warp: the nearest earlier warp that can answer
                            int w = -2 - c;
                            c = -1;
                            while (--w >= 0)
                                if (lt<INCL>(sWmin[w], q)) {
                                    c = (w * 32 + 31) * IPT + IPT - 1;
                                    break;
                                }
                        }
                        if (c < 0 || --guard < 0) {  // cannot happen while lt(x, q)
                            atomicOr(err, ERR_INTERNAL);
                            cu = (1u << k) | Q;
                            break;
                        }
                        cv = V[swz(c)];
                    }
                }
            }
        }

        // ---- 5. keys with no answer in the tile: the range stack -------------------------
        if (cu) {
            const bool has_rmin = misc->has_rmin != 0;
            const T rmin = KeyTraits<T>::from_bits(misc->rmin_bits);
            unsigned dmask = 0;
            const T qmax = V[swz(tid * IPT + __ffs(cu) - 1)];
            if (!has_rmin || !lt<INCL>(rmin, qmax)) {
                dmask = cu;  // nothing in the range qualifies even for the largest
            } else {
                const int lo0 = misc->stk_lo, top = misc->stk_top;
                unsigned m = cu;
                while (m) {
                    const int k = __ffs(m) - 1;
                    m &= m - 1;
                    const int e = tid * IPT + k;
                    const T q = V[swz(e)];
                    if (!lt<INCL>(rmin, q)) {
                        dmask |= (1u << k) | m;  // queries only shrink from here on
                        break;
                    }
                    int lo = lo0, hi = top;  // first stored index that does not qualify
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (lt<INCL>(sStkV[mid % K], q)) lo = mid + 1;
                        else hi = mid;
                    }
                    if (lo > lo0) O[swz(e)] = sStkP[(lo - 1) % K];
                    else dmask |= 1u << k;  // below the kept part of the stack
                }
            }
            if (dmask) {
                const int bit = tid * IPT;  // this thread's keys as bits of the tile mask
                atomicOr(&sDef[bit >> 5], dmask << (bit & 31));
                atomicAdd(&misc->def_cnt, __popc(dmask));
            }
        }
        __syncthreads();  // B2: old stack, V and sNext no longer read

        // ---- 6. stack update, output, next load ----------------------------------------------
        if (tid < W) sDefAll[(size_t)((i + 1) & 1) * W + tid] = 0;  // next tile's mask
        if (!last_of_range) {
            const int keep = misc->keep;
            int base = keep + fpre, total = 0;
            for (int w = 0; w < NW; w++) {
                const int cw = sWcnt[w];
                if (w < warp) base += cw;
                total += cw;
            }
            const int newtop = keep + total;
            if (fmask) {
                int idx = base;
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    if ((fmask >> k) & 1u) {
                        if (idx >= newtop - K) {
                            sStkV[idx % K] = v[k];
                            sStkP[idx % K] = tile_base + tid * IPT + k;
                        }
                        idx++;
                    }
                }
            }
            if (tid == 0) {
                misc->stk_top = newtop;
                misc->stk_lo = max(misc->stk_lo, newtop - K);
            }
        }
        if (tid == 0) {
            misc->rmin_bits = KeyTraits<T>::bits(misc->has_rmin ? KeyTraits<T>::vmin(KeyTraits<T>::from_bits(
                                                                      misc->rmin_bits), tile_min_t)
                                                                : tile_min_t);
            misc->has_rmin = 1;
            bulk_wait_read0();  // the store of tile i-1 has read its buffer (tile i+1 reuses it)
            const int dc = misc->def_cnt;
            misc->def_saved = dc;
            misc->def_cnt = 0;
            __stcg(&a.s.tile_defcnt[t], dc);
        }
        fence_proxy_async_smem();
        __syncthreads();  // B3: nothing reads this stage any more
        if (tid == 0 && i + kStages < ntr && tile_full(t + kStages)) {
            mbar_arrive_expect_tx(&misc->full_bar[slot], (uint32_t)(B * 4));
            tma_load_2d(V, &map_in, 0, (t + kStages) * ROWS, &misc->full_bar[slot]);
        }
        const int dc = misc->def_saved;
        if (dc == 0) {
            if (full) {
                if (tid == 0) {
                    tma_store_2d(&map_out, 0, t * ROWS, O);
                    bulk_commit();
                }
            } else {
#pragma unroll
                for (int j = 0; j < IPT; j++) {
                    const int e = j * NT + tid;
                    if (e < valid_keys) a.d_out[tile_base + e] = O[swz(e)];
                }
            }
        } else if (dc < valid_keys) {
#pragma unroll
            for (int j = 0; j < IPT; j++) {
                const int e = j * NT + tid;
                if (e < valid_keys && !((sDef[e >> 5] >> (e & 31)) & 1u)) a.d_out[tile_base + e] = O[swz(e)];
            }
            if (tid < W) __stcg(&a.s.tile_defmask[(size_t)t * (kMaxTileKeys / 32) + tid], sDef[tid]);
        }
    }

    // =========================== publish the range, look back ===========================
    if (tid == 0) bulk_wait_read0();
    __threadfence();  // tile mins, chunk mins, prefixes, deferred masks -> visible
    __syncthreads();
    const T rmin_r = KeyTraits<T>::from_bits(misc->rmin_bits);
    if (warp == 0) {
        if (lane == 0) {
            __stcg(&((T*)a.s.range_min)[r], rmin_r);
            if (r != a.skip_publish_range) {
                const uint32_t flag = r == 0 ? FLAG_INCL : FLAG_AGG;
                st_release_u64(&a.s.range_state[r],
                               ((uint64_t)make_tag(epoch, flag) << 32) | KeyTraits<T>::bits(rmin_r));
            }
        }
        T p;
        bool has_p;
        range_lookback<T, INCL>(r, epoch, rmin_r, a, p, has_p);
        if (lane == 0) {
            misc->p_bits = KeyTraits<T>::bits(p);
            misc->has_p = has_p ? 1 : 0;
        }
        __threadfence();
    }
    // -1 source buffer for whole-tile stores
    int32_t* sNeg = sOall;
#pragma unroll 4
    for (int e = tid; e < B; e += NT) sNeg[e] = -1;
    fence_proxy_async_smem();
    __syncthreads();

    // =========================== phase 2: deferred keys ===============================
    // Deferred keys have no qualifying key in the range before their tile's
    // stack search.  "True" ones have none in the range at all; they are the
    // range's prefix minima, so they are non-increasing: the ones P
    // qualifies form a prefix (pass A, in order, one monotone cursor) and all
    // later ones answer -1 without reading their keys (pass B).  "Capped"
    // ones (only in tiles whose stack had dropped entries, rpre bit 33) have
    // their answer inside the range: pass B searches for them.
    const bool has_p = misc->has_p != 0;
    const T P = KeyTraits<T>::from_bits(misc->p_bits);
    const T* tile_min_r = (const T*)a.s.tile_min;
    const T* chunk_min_r = (const T*)a.s.chunk_min;
    const uint32_t* defmask = a.s.tile_defmask;
    constexpr int MW = kMaxTileKeys / 32;  // mask words per tile in global
    if (warp == 0) {
        int* list = (int*)sVall;  // ordered deferred offsets of one tile (the ring is free now)
        int cur = -1;             // the last answer found (absolute), -1 = none yet
        int stop = t1 * B;        // first position pass B answers -1
        bool done = !has_p;
        if (done) stop = t0 * B;
        for (int ib = 0; ib < ntr && !done; ib += 32) {
            const int dcl = ib + lane < ntr ? __ldcg(&a.s.tile_defcnt[t0 + ib + lane]) : 0;
            unsigned nz = __ballot_sync(FULL, dcl != 0);
            while (nz && !done) {
                const int jt = __ffs(nz) - 1;
                nz &= nz - 1;
                const int t = t0 + ib + jt;
                const int dct = __shfl_sync(FULL, dcl, jt);
                const int valid = min(B, a.n - t * B);
                const uint64_t rp = __ldcg(&a.s.tile_rpre[t]);
                const bool has_rp = ((rp >> 32) & 1ull) != 0;
                const T rpv = KeyTraits<T>::from_bits((uint32_t)rp);
                const bool dense = dct == valid;
                if (!dense) {  // ordered list of the tile's deferred offsets
                    uint32_t wv[4];
                    int base = 0;
#pragma unroll
                    for (int m = 0; m < 4; m++) {
                        const int w = m * 32 + lane;
                        wv[m] = w < W ? __ldcg(&defmask[(size_t)t * MW + w]) : 0u;
                    }
#pragma unroll
                    for (int m = 0; m < 4; m++) {
                        const int c = __popc(wv[m]);
                        int incl = c;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const int nb = __shfl_up_sync(FULL, incl, o);
                            if (lane >= o) incl += nb;
                        }
                        int pos = base + incl - c;
                        uint32_t bits = wv[m];
                        while (bits) {
                            const int b = __ffs(bits) - 1;
                            bits &= bits - 1;
                            list[pos++] = (m * 32 + lane) * 32 + b;
                        }
                        base += __shfl_sync(FULL, incl, 31);
                    }
                    __syncwarp();
                }
                for (int k0 = 0; k0 < dct && !done; k0 += 32) {
                    const int k = k0 + lane;
                    const bool act = k < dct;
                    const int e = act ? (dense ? k : list[k]) : 0;
                    const T q = act ? __ldg(&d_in[t * B + e]) : KeyTraits<T>::pad();
                    const bool capped = act && has_rp && lt<INCL>(rpv, q);
                    const bool truedef = act && !capped;
                    const bool want = truedef && lt<INCL>(P, q);
                    unsigned wm = __ballot_sync(FULL, want);
                    const unsigned tm = __ballot_sync(FULL, truedef);
                    const unsigned rest = tm & ~wm;
                    if (rest) {  // the first true key P does not qualify: all later ones are -1
                        const int f = __ffs(rest) - 1;
                        stop = t * B + __shfl_sync(FULL, e, f);
                        wm &= (1u << f) - 1u;  // wanted keys sit before it (non-increasing keys)
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
                            find_left<T, B, INCL>(qf, cur >= 0 ? cur : t0 * B, d_in, tile_min_r, chunk_min_r);
                        if (found < 0) {
                            if (lane == 0) atomicOr(err, ERR_INTERNAL);
                        } else {
                            cur = found;
                        }
                        if (lane == f) ans = found < 0 ? -1 : found;
                        pend &= pend - 1;
                    }
                    if ((wm >> lane) & 1u) a.d_out[t * B + e] = ans;
                }
            }
        }
        if (lane == 0) misc->stop = stop;
    }
    __syncthreads();
    const int stop = misc->stop;
    for (int i = warp; i < ntr; i += NW) {
        const int t = t0 + i;
        const int dct = __ldcg(&a.s.tile_defcnt[t]);
        if (dct == 0) continue;
        const int valid = min(B, a.n - t * B);
        const uint64_t rp = __ldcg(&a.s.tile_rpre[t]);
        const bool may_cap = ((rp >> 33) & 1ull) != 0;
        const bool has_rp = ((rp >> 32) & 1ull) != 0;
        const T rpv = KeyTraits<T>::from_bits((uint32_t)rp);
        const bool dense = dct == valid;
        if (!may_cap) {
            if (t * B + valid <= stop) continue;  // pass A answered every key here
            if (dense && t * B >= stop) {
                if (tile_full(t)) {
                    if (lane == 0) {
                        tma_store_2d(&map_out, 0, t * ROWS, sOall);  // the -1 buffer
                        bulk_commit();
                        bulk_wait_read0();
                    }
                } else {
                    for (int e = lane; e < valid; e += 32) a.d_out[t * B + e] = -1;
                }
                continue;
            }
            // -1 at the deferred offsets >= stop, straight from the mask
            for (int m = 0; m < 4; m++) {
                const int w = m * 32 + lane;
                if (w >= W) continue;
                uint32_t bits = dense ? 0xffffffffu : __ldcg(&defmask[(size_t)t * MW + w]);
                if (w * 32 + 32 > valid) bits &= valid > w * 32 ? (0xffffffffu >> (32 - (valid - w * 32))) : 0u;
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const int pos = t * B + w * 32 + b;
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
            const T q = isdef ? __ldg(&d_in[t * B + e]) : KeyTraits<T>::pad();
            const bool capped = isdef && has_rp && lt<INCL>(rpv, q);
            if (isdef && !capped && t * B + e >= stop) a.d_out[t * B + e] = -1;
            unsigned cm = __ballot_sync(FULL, capped);
            while (cm) {
                const int f = __ffs(cm) - 1;
                cm &= cm - 1;
                const T qf = __shfl_sync(FULL, q, f);
                const int found = find_left<T, B, INCL>(qf, t * B, d_in, tile_min_r, chunk_min_r);
                if (found < 0 && lane == 0) atomicOr(err, ERR_INTERNAL);
                if (lane == f) a.d_out[t * B + e] = found < 0 ? -1 : found;
            }
        }
    }

    // ---- run bookkeeping: the last CTA resets the control block ----------------------------
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const uint32_t prev = atomicAdd(&a.s.ctr->done, 1u);
        misc->last_cta = prev == gridDim.x - 1 ? 1 : 0;
        if (prev == gridDim.x - 1) {
            a.s.ctr->range_counter = 0;
            a.s.ctr->done = 0;
            a.s.ctr->epoch = epoch >= EPOCH_LIMIT ? 1u : epoch + 1u;
            __threadfence();
        }
    }
    if (epoch >= EPOCH_LIMIT) {  // once per 2^30 runs: stale words could alias
        __syncthreads();
        if (misc->last_cta)
            for (int i = tid; i < a.s.max_ranges; i += NT) a.s.range_state[i] = 0;
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

template <typename T, int NT, int IPT, bool INCL>
static cudaError_t launch_t(RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo, cudaStream_t st,
                            int max_ctas) {
    constexpr size_t smem = RLayout<NT, IPT>::kBytes;
    int tpr = (a.num_tiles + max_ctas - 1) / max_ctas;
    if (tpr < 1) tpr = 1;
    a.tiles_per_range = tpr;
    a.num_ranges = (a.num_tiles + tpr - 1) / tpr;
    apse_range_kernel<T, NT, IPT, INCL><<<a.num_ranges, NT, smem, st>>>(mi, mo, a);
    return cudaGetLastError();
}

namespace {
constexpr int kMaxDev = 64;
int g_ctas[kMaxDev][kNumTileConfigs];  // resident CTAs per device and configuration
}

template <typename T, int NT, int IPT, bool INCL>
static cudaError_t prepare_t(int* ctas_per_sm) {
    constexpr size_t smem = RLayout<NT, IPT>::kBytes;
    auto k = apse_range_kernel<T, NT, IPT, INCL>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NT, smem);
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
#define P_(NT, IPT)                                                          \
    {                                                                        \
        cudaError_t rr[4] = {prepare_t<int32_t, NT, IPT, false>(&per_sm),    \
                             prepare_t<int32_t, NT, IPT, true>(&per_sm),     \
                             prepare_t<float, NT, IPT, false>(&per_sm),      \
                             prepare_t<float, NT, IPT, true>(&per_sm)};      \
        for (int q = 0; q < 4; q++)                                          \
            if (rr[q] != cudaSuccess) return rr[q];                          \
    }
    switch (cfg) {
    case 0: P_(256, 16); break;
    case 1: P_(512, 8); break;
    }
#undef P_
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int ctas = per_sm * sms;
    if (ctas > kMaxRanges) ctas = kMaxRanges;
    g_ctas[dev][cfg] = ctas;
    return cudaSuccess;
}

cudaError_t launch_range(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo,
                         cudaStream_t st) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev || cfg < 0 || cfg >= kNumTileConfigs) return cudaErrorInvalidValue;
    if (g_ctas[dev][cfg] == 0) {
        e = range_prepare(cfg);
        if (e != cudaSuccess) return e;
    }
    const int max_ctas = g_ctas[dev][cfg];
#define L_(NT, IPT)                                                                      \
    if (dtype == 0)                                                                      \
        return incl ? launch_t<int32_t, NT, IPT, true>(a, mi, mo, st, max_ctas)          \
                    : launch_t<int32_t, NT, IPT, false>(a, mi, mo, st, max_ctas);        \
    else                                                                                 \
        return incl ? launch_t<float, NT, IPT, true>(a, mi, mo, st, max_ctas)            \
                    : launch_t<float, NT, IPT, false>(a, mi, mo, st, max_ctas);
    switch (cfg) {
    case 0: L_(256, 16);
    case 1: L_(512, 8);
    }
#undef L_
    return cudaErrorInvalidValue;
}

}  // namespace apsep
