// apsep_long.cu -- 64-bit positions: APSE over arrays of any length.
//
// The engine's positions are int32, like the reference's (every entry point
// takes `int n`, src/apsep.cuh:3052-3076, while its key types already reach
// 8-byte keys, src/apsep.cuh:62-70).  apsep_run64 answers arrays of up to
// APSEP_MAX_KEYS64 keys with int64 positions:
//
//   * the array runs as consecutive pieces [b0, b1) of at most the plan's
//     capacity (a multiple of 32 keys), each one engine run that writes
//     b0 + answer straight into the int64 output for every key its piece
//     answers (the engine's int64-answer instantiation: 4 bytes read and 8
//     written per key, nothing in between);
//   * a key without an answer in its piece (a prefix minimum of the piece)
//     looks before b0.  The engine leaves such keys as UNRESOLVED64, and a tile
//     of them whose keys are all prefix minima of their range unwritten
//     (TILE_NOT_STORED): the fix-up pass tells those apart from the keys that
//     the engine's phase 2 answered by the exclusive prefix minimum of the range
//     minima, and skips reading the keys of a 32-key chunk whose upper bound
//     (the previous chunk's minimum: such a tile never increases) already
//     says that nothing before it qualifies;
//   * before b0 there is a hierarchy of minima over the keys so far: level l
//     holds the minimum of every aligned run of 32^l keys (level 0 = the keys),
//     level 1 written by the engine runs themselves (their minima of every 32
//     keys go straight into it), the levels above built piece by piece as their
//     entries complete.  The "frontier" of b0 at level l is the run of level-l
//     entries from the last multiple of 32 up to b0's own entry; the frontiers
//     of all levels tile [0, b0) from near to far (level 0 holds the keys just
//     before b0, the top level the oldest).  So a key q is answered by the
//     nearest frontier whose minimum qualifies (none: -1), a ballot over that
//     frontier's entries (the last qualifying one) and a descent, one ballot
//     over 32 entries per level, to the key.
//
// The frontier minima of a piece and the prefix minima of its ranges come from
// one small prologue kernel; the fix-up's queries are warp-cooperative (one at
// a time per warp, every lane on one entry).  Keys that need a query are the
// prefix minima of their piece that something before the piece qualifies for:
// a few dozen per piece on random keys, none on descending keys; an input whose
// every piece descends while the pieces rise makes every key a query (a few
// dependent L2 reads each, one query at a time per warp), the slow case of
// this path.
#include <stdint.h>

#include <type_traits>

#include "apsep.h"
#include "apsep_device.cuh"
#include "apsep_internal.h"

using namespace apsep;

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kLevels = 9;  // levels 0..8: 32^8 = 2^40 >= APSEP_MAX_KEYS64
constexpr int kThreads = 256;

size_t align16(size_t x) { return (x + 15) / 16 * 16; }
int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// The hierarchy: p[l] holds size[l] = ceil(n / 32^l) minima (l >= 1); size[0] = n.
template <typename K>
struct Levels {
    K* p[kLevels];
    int64_t size[kLevels];
    int top;  // the first level with at most 31 entries
};

// Frontier minima of one piece start: u[l] is valid when bit l of has is set.
template <typename K>
struct Frontier {
    K u[kLevels];
    uint32_t has;
};

int top_level(int64_t n) {
    int l = 1;
    int64_t s = ceil_div(n, 32);
    while (s > 31) {
        s = ceil_div(s, 32);
        l++;
    }
    return l;
}

// Keys per piece: the whole array when it fits the plan, else the capacity
// rounded down to whole 32-key groups (0: the plan is too small to split).
int64_t piece_keys(int64_t capacity, int64_t n) { return n <= capacity ? n : capacity / 32 * 32; }

template <typename K>
__device__ __forceinline__ K warp_min(K v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = KeyTraits<K>::vmin(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// An entry of level lev: a key (mapped when MAPF) or a stored minimum.
template <typename K, bool MAPF>
__device__ __forceinline__ K entry(const K* keys, const Levels<K>& lv, int lev, int64_t e) {
    return lev == 0 ? load_key<K, MAPF>(keys + e) : lv.p[lev][e];
}

// Level-l entries [e_lo, e_hi) from level l-1: one warp per entry.
template <typename K>
__global__ void __launch_bounds__(kThreads) level_kernel(const K* __restrict__ src, int64_t src_size,
                                                         K* __restrict__ dst, int64_t e_lo, int64_t e_hi) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = e_lo + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); e < e_hi; e += nw) {
        const int64_t j = (e << 5) + lane;
        const K m = warp_min(j < src_size ? src[j] : KeyTraits<K>::pad());
        if (lane == 0) dst[e] = m;
    }
}

// The answer of q from the frontier of b0 at level l, whose minimum
// qualifies: the last qualifying entry there, then the last qualifying entry
// of each 32-entry group below it.  Warp-cooperative; q and l are uniform.
template <typename K, bool MAPF, bool INCL>
__device__ int64_t answer_before(const K* keys, const Levels<K>& lv, K q, int l, int64_t b0, uint32_t* err) {
    const int lane = threadIdx.x & 31;
    const int64_t idx = b0 >> (5 * l);
    const int64_t g0 = (idx >> 5) << 5;
    bool ok = g0 + lane < idx && lt<INCL>(entry<K, MAPF>(keys, lv, l, g0 + lane), q);
    unsigned b = __ballot_sync(FULL, ok);
    int64_t f = g0 + 31 - __clz(b);
    for (int lev = l; lev > 0 && b; lev--) {
        const int64_t e = (f << 5) + lane;
        ok = e < lv.size[lev - 1] && lt<INCL>(entry<K, MAPF>(keys, lv, lev - 1, e), q);
        b = __ballot_sync(FULL, ok);
        f = (f << 5) + 31 - __clz(b);
    }
    if (!b) {  // a minimum qualified but none of its entries did: cannot happen
        if (lane == 0) atomicOr(err, ERR_INTERNAL);
        return -1;
    }
    return f;
}

// The prologue of piece [b0, b1), after its engine run: rpre[r] = the minimum
// of the piece's ranges before r (range minima from the run's range words), and,
// with look_before, the frontier minima of b0 (warp 0; every entry it reads lies
// wholly before b0, so it is complete).  One block of kPrologue threads.
constexpr int kPrologue = 1024;
static_assert(kMaxRanges <= 4 * kPrologue, "four range minima per thread");

template <typename K, bool MAPF>
__global__ void __launch_bounds__(kPrologue)
    prologue_kernel(const K* __restrict__ keys, Levels<K> lv, int64_t b0, bool look_before, RangeScratch rs,
                    int num_ranges, K* __restrict__ rpre, Frontier<K>* fr) {
    __shared__ K wsum[kPrologue / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0 && look_before) {
        int64_t idx = b0;
        uint32_t has = 0;
        for (int l = 0; l <= lv.top; l++) {
            const int64_t g = idx >> 5;
            const int cnt = (int)(idx & 31);
            const K v = lane < cnt ? entry<K, MAPF>(keys, lv, l, (g << 5) + lane) : KeyTraits<K>::pad();
            const K m = warp_min(v);
            if (lane == 0) fr->u[l] = m;
            if (cnt) has |= 1u << l;
            idx = g;  // (at the top level g is 0: at most 31 entries)
        }
        if (lane == 0) fr->has = has;
    }
    // four consecutive range minima per thread, then an exclusive scan (min)
    K v[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int r = 4 * threadIdx.x + j;
        v[j] = KeyTraits<K>::pad();
        if (r < num_ranges) {
            if constexpr (sizeof(K) == 8)
                v[j] = KeyTraits<K>::from_bits((uint64_t)__ldcg((const unsigned long long*)&rs.range_key[r]));
            else
                v[j] = KeyTraits<K>::from_bits((uint32_t)__ldcg((const unsigned long long*)&rs.range_state[r]));
        }
    }
    const K tot = KeyTraits<K>::vmin(KeyTraits<K>::vmin(v[0], v[1]), KeyTraits<K>::vmin(v[2], v[3]));
    K inc = tot;  // inclusive scan over the warp's threads
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const K u = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc = KeyTraits<K>::vmin(inc, u);
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        K w = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const K u = __shfl_up_sync(FULL, w, o);
            if (lane >= o) w = KeyTraits<K>::vmin(w, u);
        }
        wsum[lane] = w;  // inclusive over warps 0..lane
    }
    __syncthreads();
    K run = warp > 0 ? wsum[warp - 1] : KeyTraits<K>::pad();
    const K before = __shfl_up_sync(FULL, inc, 1);
    if (lane > 0) run = KeyTraits<K>::vmin(run, before);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int r = 4 * threadIdx.x + j;
        if (r < num_ranges) rpre[r] = run;
        run = KeyTraits<K>::vmin(run, v[j]);
    }
}

// The fix-up of piece [b0, b1) after its engine run (int64 answers): every key
// the run left unanswered gets its answer before b0, or -1.  One warp per 32
// tiles of the run at a time: a ballot over their flag words, then each flagged
// tile in turn.  A tile written by the engine names its unanswered keys by its
// mask words and UNRESOLVED64; a tile left unwritten (TILE_NOT_STORED: its keys
// are all prefix minima of their range, and never increase) has its keys
// answered by phase 2 exactly when the range's prefix minimum qualifies.
template <typename K, bool MAPF, bool INCL>
__global__ void __launch_bounds__(kThreads)
    fixup_kernel(const K* __restrict__ keys, int64_t* __restrict__ out, int64_t b0, int64_t b1, Levels<K> lv,
                 const Frontier<K>* __restrict__ fr, bool look_before, const K* __restrict__ rpre, RangeScratch rs,
                 const K* __restrict__ cmin, int num_tiles, int tiles_per_range, uint32_t* err) {
    constexpr int WT = sizeof(K) == 8 ? kWideTileKeys : 512;  // keys per engine tile
    constexpr int W = WT / 32;                                 // 32-key chunks per tile
    constexpr int MW = kMaxTileKeys / 32;                      // mask words per tile
    __shared__ K su[kLevels];
    __shared__ K spm;  // the minimum of everything before b0
    __shared__ uint32_t shas;
    if (threadIdx.x < kLevels) su[threadIdx.x] = look_before ? fr->u[threadIdx.x] : KeyTraits<K>::pad();
    if (threadIdx.x == 0) {
        const uint32_t h = look_before ? fr->has : 0u;
        K m = KeyTraits<K>::pad();
        for (int l = 0; l < kLevels; l++)
            if ((h >> l) & 1u) m = KeyTraits<K>::vmin(m, fr->u[l]);
        spm = m;
        shas = h;
    }
    __syncthreads();
    const uint32_t has = shas;
    const K pm = spm;
    const K* tmin = (const K*)rs.tile_min;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    // the answer before b0 of the keys `need` marks (uniform call), written
    auto resolve = [&](bool need, K q, int64_t i) {
        int64_t o = -1;
        int lvl = -1;  // the nearest frontier whose minimum qualifies
        if (need && has && lt<INCL>(pm, q)) {
            for (int l = 0; l < kLevels; l++)
                if (((has >> l) & 1u) && lt<INCL>(su[l], q)) {
                    lvl = l;
                    break;
                }
        }
        unsigned qm = __ballot_sync(FULL, lvl >= 0);
        while (qm) {
            const int src = __ffs(qm) - 1;
            qm &= qm - 1;
            const K qs = __shfl_sync(FULL, q, src);
            const int l = __shfl_sync(FULL, lvl, src);
            const int64_t ans = answer_before<K, MAPF, INCL>(keys, lv, qs, l, b0, err);
            if (lane == src) o = ans;
        }
        if (need) __stcs(reinterpret_cast<long long*>(out) + i, (long long)o);
    };
    const int ngroups = (num_tiles + 31) >> 5;
    for (int tg = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); tg < ngroups; tg += nw) {
        const int tl = (tg << 5) + lane;
        const uint32_t myf = tl < num_tiles ? __ldcg(&rs.tile_flag[tl]) : 0u;
        unsigned fm = __ballot_sync(FULL, (myf & 0x3fffffffu) != 0);
        while (fm) {
            const int src = __ffs(fm) - 1;
            fm &= fm - 1;
            const int t = (tg << 5) + src;
            const uint32_t tf = __shfl_sync(FULL, myf, src);
            const int r = t / tiles_per_range;
            const bool has_p = r > 0;  // the piece's ranges before r
            const K P = has_p ? rpre[r] : KeyTraits<K>::pad();
            const int64_t tb = b0 + (int64_t)t * WT;  // the tile's first position
            if (tf & TILE_NOT_STORED) {
                // chunk c's keys are at most the minimum of chunk c - 1, and chunk
                // 0's at most the previous tile's minimum (the range's minimum
                // before the tile is >= its first key); lane c holds chunk c's bound
                bool dec = false;
                if (lane < W && (lane > 0 || t % tiles_per_range != 0)) {
                    const K ub = lane > 0 ? __ldcg(&cmin[(size_t)t * W + lane - 1]) : __ldcg(&tmin[t - 1]);
                    dec = !(has_p && lt<INCL>(P, ub)) && !(has && lt<INCL>(pm, ub));
                }
                const unsigned decm = __ballot_sync(FULL, dec);
#pragma unroll 1
                for (int c = 0; c < W; c++) {
                    const int64_t i = tb + 32 * c + lane;
                    const bool valid = i < b1;
                    if ((decm >> c) & 1u) {  // no key of the chunk has an answer
                        if (valid) __stcs(reinterpret_cast<long long*>(out) + i, -1ll);
                        continue;
                    }
                    const K q = valid ? load_key<K, MAPF>(keys + i) : KeyTraits<K>::pad();
                    resolve(valid && !(has_p && lt<INCL>(P, q)), q, i);
                }
            } else {
                const uint32_t mw = lane < W ? __ldcg(&rs.tile_mask[(size_t)t * MW + lane]) : 0u;
#pragma unroll 1
                for (int c = 0; c < W; c++) {
                    const uint32_t m = __shfl_sync(FULL, mw, c);
                    if (!m) continue;
                    const int64_t i = tb + 32 * c + lane;
                    const bool need = ((m >> lane) & 1u) && i < b1 &&
                                      __ldcg(reinterpret_cast<const long long*>(out) + i) == (long long)UNRESOLVED64;
                    const K q = need ? load_key<K, MAPF>(keys + i) : KeyTraits<K>::pad();
                    resolve(need, q, i);
                }
            }
        }
    }
}

// Workspace: the frontier slot, the range prefix minima, the hierarchy (level 1
// with room for the engine's minima up to the end of its last tile).
constexpr size_t kFrontBytes = 256;
constexpr size_t kRpreBytes = (size_t)kMaxRanges * 8;
constexpr int64_t kLevel1Slack = kMaxTileKeys / 32;
struct Work {
    void* front;
    void* rpre;
    char* levels;
};
Work carve(void* d_work) {
    char* w = (char*)d_work;
    return {w, w + kFrontBytes, w + kFrontBytes + kRpreBytes};
}
static_assert(sizeof(Frontier<int64_t>) <= kFrontBytes, "frontier slot");

template <typename K>
Levels<K> make_levels(const Work& w, int64_t n, bool with_levels) {
    Levels<K> lv{};
    lv.size[0] = n;
    lv.top = top_level(n);
    char* p = w.levels;
    int64_t s = n;
    for (int l = 1; l < kLevels; l++) {
        s = ceil_div(s, 32);
        lv.size[l] = s;
        if (l <= lv.top && with_levels) {
            lv.p[l] = (K*)p;
            p += align16((size_t)(s + (l == 1 ? kLevel1Slack : 0)) * sizeof(K));
        }
    }
    return lv;
}

template <typename K, bool MAPF>
apsep_status run_long(apsep_plan* plan, const K* keys, int64_t* out, int64_t n, apsep_cmp cmp, int64_t piece,
                      void* d_work, cudaStream_t st) {
    const Work w = carve(d_work);
    const bool pieces = n > piece;
    const Levels<K> lv = make_levels<K>(w, n, pieces);
    Frontier<K>* fr = (Frontier<K>*)w.front;
    K* rpre = (K*)w.rpre;
    auto fix = cmp == APSEP_LE ? fixup_kernel<K, MAPF, true> : fixup_kernel<K, MAPF, false>;
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fix, kThreads, 0) != cudaSuccess)
        return APSEP_ECUDA;
    for (int64_t b0 = 0; b0 < n; b0 += piece) {
        const int64_t b1 = std::min(n, b0 + piece);
        RangeArgs ra;
        // the run's minima of every 32 keys are level 1 of the hierarchy
        void* cdst = pieces ? (void*)(lv.p[1] + (b0 >> 5)) : nullptr;
        apsep_status s = plan_run_out64(plan, keys + b0, out + b0, b1 - b0, b0, cmp, cdst, st, &ra);
        if (s != APSEP_OK) return s;
        const bool look = b0 > 0;
        prologue_kernel<K, MAPF><<<1, kPrologue, 0, st>>>(keys, lv, b0, look, ra.s, ra.num_ranges, rpre, fr);
        const int groups = (ra.num_tiles + 31) / 32;  // 32 tiles per warp and step
        const int grid = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(groups, kThreads / 32), 1),
                                                (int64_t)sms * std::max(per_sm, 1));
        fix<<<grid, kThreads, 0, st>>>(keys, out, b0, b1, lv, fr, look, rpre, ra.s, (const K*)ra.s.chunk_min,
                                       ra.num_tiles, ra.tiles_per_range, &ra.s.ctr->err);
        if (cudaGetLastError() != cudaSuccess) return APSEP_ECUDA;
        if (!pieces || b1 == n) continue;
        // level entries that complete inside this piece (level 1 came with the run)
        int64_t span = 32;
        for (int l = 2; l <= lv.top; l++) {
            span *= 32;
            const int64_t e_lo = b0 / span, e_hi = b1 / span;
            if (e_hi > e_lo) {
                const int g = (int)std::min<int64_t>(ceil_div(e_hi - e_lo, kThreads / 32), (int64_t)sms * 8);
                level_kernel<K><<<g, kThreads, 0, st>>>(lv.p[l - 1], lv.size[l - 1], lv.p[l], e_lo, e_hi);
            }
        }
        if (cudaGetLastError() != cudaSuccess) return APSEP_ECUDA;
    }
    return APSEP_OK;
}

bool overlaps(const void* a, size_t an, const void* b, size_t bn) {
    const uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
    return a0 < b0 + bn && b0 < a0 + an;
}

}  // namespace

extern "C" {

int64_t apsep_run64_workspace_bytes(const apsep_plan* plan, int64_t n) {
    apsep_plan_info info;
    if (!plan || n < 0 || n > APSEP_MAX_KEYS64 || apsep_plan_get_info(plan, &info) != APSEP_OK) return -1;
    const int64_t piece = piece_keys(info.capacity, n);
    if (n > 0 && piece == 0) return -1;
    size_t bytes = kFrontBytes + kRpreBytes;
    if (n > piece) {
        const size_t kb = info.dtype == APSEP_INT64 || info.dtype == APSEP_FLOAT64 ? 8 : 4;
        int64_t s = n;
        for (int l = 1, top = top_level(n); l <= top; l++) {
            s = ceil_div(s, 32);
            bytes += align16((size_t)(s + (l == 1 ? kLevel1Slack : 0)) * kb);
        }
    }
    return (int64_t)bytes;
}

apsep_status apsep_run64(apsep_plan* plan, const void* d_in, int64_t* d_out, int64_t n, apsep_cmp cmp,
                         void* d_work, void* stream) {
    apsep_plan_info info;
    if (!plan || apsep_plan_get_info(plan, &info) != APSEP_OK) return APSEP_EINVAL;
    if (n < 0 || n > APSEP_MAX_KEYS64 || (cmp != APSEP_LT && cmp != APSEP_LE)) return APSEP_EINVAL;
    if (n == 0) return APSEP_OK;
    const int64_t wb = apsep_run64_workspace_bytes(plan, n);
    if (wb < 0 || !d_in || !d_out || !d_work) return APSEP_EINVAL;
    const size_t kb = info.dtype == APSEP_INT64 || info.dtype == APSEP_FLOAT64 ? 8 : 4;
    if ((uintptr_t)d_in % kb || (uintptr_t)d_out % 8 || (uintptr_t)d_work % 16) return APSEP_EINVAL;
    if (overlaps(d_work, (size_t)wb, d_in, (size_t)n * kb) || overlaps(d_work, (size_t)wb, d_out, (size_t)n * 8) ||
        overlaps(d_in, (size_t)n * kb, d_out, (size_t)n * 8))
        return APSEP_EINVAL;
    const int64_t piece = piece_keys(info.capacity, n);
    const cudaStream_t st = (cudaStream_t)stream;
    // the whole call on the plan's device (the engine runs there; so must the
    // fix-up and level passes, sized from that device's SMs), the caller's
    // device restored afterwards
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return APSEP_ECUDA;
    if (prev != info.device && cudaSetDevice(info.device) != cudaSuccess) return APSEP_ECUDA;
    struct Restore {
        int dev;
        ~Restore() {
            int cur = -1;
            if (cudaGetDevice(&cur) == cudaSuccess && cur != dev) cudaSetDevice(dev);
        }
    } restore{prev};
    switch (info.dtype) {
    case APSEP_INT32: return run_long<int32_t, false>(plan, (const int32_t*)d_in, d_out, n, cmp, piece, d_work, st);
    case APSEP_FLOAT32: return run_long<float, false>(plan, (const float*)d_in, d_out, n, cmp, piece, d_work, st);
    case APSEP_INT64: return run_long<int64_t, false>(plan, (const int64_t*)d_in, d_out, n, cmp, piece, d_work, st);
    default:  // float64 keys compare as their order-preserving int64 map
        return run_long<int64_t, true>(plan, (const int64_t*)d_in, d_out, n, cmp, piece, d_work, st);
    }
}

}  // extern "C"
