// apsep_long.cu -- 64-bit positions: APSE over arrays of any length.
//
// The engine's positions are int32, like the reference's (every entry point
// takes `int n`, src/apsep.cuh:3052-3076, while its key types already reach
// 8-byte keys, src/apsep.cuh:62-70).  apsep_run64 answers arrays of up to
// APSEP_MAX_KEYS64 keys with int64 positions:
//
//   * the array runs as consecutive pieces [b0, b1) of at most the plan's
//     capacity (a multiple of 32 keys), each one engine run into an int32
//     scratch of answers relative to the piece;
//   * a widening pass writes b0 + answer for every key answered inside its
//     piece; a key without one (a prefix minimum of its piece) looks before b0;
//   * before b0 there is a hierarchy of minima over the keys so far: level l
//     holds the minimum of every aligned run of 32^l keys (level 0 = the keys),
//     built piece by piece as its entries complete.  The "frontier" of b0 at
//     level l is the run of level-l entries from the last multiple of 32 up to
//     b0's own entry; the frontiers of all levels tile [0, b0) from near to far
//     (level 0 holds the keys just before b0, the top level the oldest).  So a
//     key q is answered by the nearest frontier whose minimum qualifies (none:
//     -1), a ballot over that frontier's entries (the last qualifying one) and a
//     descent, one ballot over 32 entries per level, to the key.
//
// The frontier minima of a piece are computed once, by one warp, before its
// widening pass; the queries are warp-cooperative (one at a time per warp,
// every lane on one entry).  Keys that need a query are the prefix minima of
// their piece that something before the piece qualifies for: a few dozen per
// piece on random keys, none on descending keys; an input whose every piece
// descends while the pieces rise makes every key a query (a few dependent L2
// reads each, one query at a time per warp: 4.2 million such keys take about
// 2 ms on GB300), the slow case of this path.
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
constexpr int kU = 4;  // 32-key groups per warp and step of the widening pass

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

// The frontier minima of piece start b0 (one warp).  Every entry read lies
// wholly before b0, so it is complete.
template <typename K, bool MAPF>
__global__ void frontier_kernel(const K* __restrict__ keys, Levels<K> lv, int64_t b0, Frontier<K>* f) {
    const int lane = threadIdx.x;
    int64_t idx = b0;
    uint32_t has = 0;
    for (int l = 0; l <= lv.top; l++) {
        const int64_t g = idx >> 5;
        const int cnt = (int)(idx & 31);
        const K v = lane < cnt ? entry<K, MAPF>(keys, lv, l, (g << 5) + lane) : KeyTraits<K>::pad();
        const K m = warp_min(v);
        if (lane == 0) f->u[l] = m;
        if (cnt) has |= 1u << l;
        idx = g;  // (at the top level g is 0: at most 31 entries)
    }
    if (lane == 0) f->has = has;
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

// Piece [b0, b1): out[i] = b0 + t32[i - b0] when the piece answers key i,
// else the answer before b0 (or -1).  With build_l1, also the level-1 minima
// of the piece's 32-key groups: copied from the engine run's own chunk
// minima (cmin) when it has them in key order, else taken over the keys.
template <typename K, bool MAPF, bool INCL>
__global__ void __launch_bounds__(kThreads)
    widen_kernel(const K* __restrict__ keys, const int32_t* __restrict__ t32, int64_t* __restrict__ out, int64_t b0,
                 int64_t b1, Levels<K> lv, const Frontier<K>* __restrict__ fr, bool look_before, bool build_l1,
                 const K* __restrict__ cmin, uint32_t* err) {
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
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t ngroups = (b1 - b0 + 31) >> 5;
    const bool all_keys = build_l1 && !cmin;  // every key, for the level-1 minima
    // kU groups of 32 keys per warp and step, their loads issued together
    for (int64_t g0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kU; g0 < ngroups; g0 += nw * kU) {
        int32_t t[kU];
        K k[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int64_t i = b0 + ((g0 + u) << 5) + lane;
            t[u] = i < b1 ? __ldcs(t32 + (i - b0)) : 0;
        }
        // a key is read for the level-1 minima, or when the piece does not answer it
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int64_t i = b0 + ((g0 + u) << 5) + lane;
            k[u] = i < b1 && (all_keys || (has && t[u] < 0)) ? load_key<K, MAPF>(keys + i) : KeyTraits<K>::pad();
        }
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int64_t g = g0 + u;
            if (g >= ngroups) break;
            const int64_t i = b0 + (g << 5) + lane;
            const bool valid = i < b1;
            if (all_keys) {
                const K m = warp_min(k[u]);
                if (lane == 0) lv.p[1][(b0 >> 5) + g] = m;
            } else if (build_l1 && lane == 0) {
                lv.p[1][(b0 >> 5) + g] = __ldcs(cmin + g);
            }
            int64_t o = t[u] >= 0 ? b0 + t[u] : -1;
            int lvl = -1;  // the nearest frontier whose minimum qualifies
            if (valid && t[u] < 0 && has && lt<INCL>(pm, k[u])) {
                for (int l = 0; l < kLevels; l++)
                    if (((has >> l) & 1u) && lt<INCL>(su[l], k[u])) {
                        lvl = l;
                        break;
                    }
            }
            unsigned qm = __ballot_sync(FULL, lvl >= 0);
            while (qm) {
                const int src = __ffs(qm) - 1;
                qm &= qm - 1;
                const K q = __shfl_sync(FULL, k[u], src);
                const int l = __shfl_sync(FULL, lvl, src);
                const int64_t ans = answer_before<K, MAPF, INCL>(keys, lv, q, l, b0, err);
                if (lane == src) o = ans;
            }
            if (valid) __stcs(reinterpret_cast<long long*>(out) + i, (long long)o);
        }
    }
}

struct Work {
    int32_t* t32;
    void* front;
    char* levels;
};
Work carve(void* d_work, int64_t piece) {
    char* w = (char*)d_work;
    const size_t tb = align16((size_t)piece * 4);
    return {(int32_t*)w, w + tb, w + tb + 256};
}
static_assert(sizeof(Frontier<int64_t>) <= 256, "frontier slot");

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
            p += align16((size_t)s * sizeof(K));
        }
    }
    return lv;
}

template <typename K, bool MAPF>
apsep_status run_long(apsep_plan* plan, const K* keys, int64_t* out, int64_t n, apsep_cmp cmp, int64_t piece,
                      void* d_work, cudaStream_t st) {
    const Work w = carve(d_work, piece);
    const bool pieces = n > piece;
    const Levels<K> lv = make_levels<K>(w, n, pieces);
    Frontier<K>* fr = (Frontier<K>*)w.front;
    uint32_t* err = plan_error_word(plan);
    // one wave of resident blocks at most (the pass strides over its groups)
    auto widen = cmp == APSEP_LE ? widen_kernel<K, MAPF, true> : widen_kernel<K, MAPF, false>;
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, widen, kThreads, 0) != cudaSuccess)
        return APSEP_ECUDA;
    const int64_t keys_per_block = (int64_t)kThreads * kU;  // per step
    const int grid = (int)std::min<int64_t>(std::max<int64_t>(ceil_div(piece, keys_per_block), 1),
                                            (int64_t)sms * std::max(per_sm, 1));
    for (int64_t b0 = 0; b0 < n; b0 += piece) {
        const int64_t b1 = std::min(n, b0 + piece);
        apsep_status s = apsep_run_cmp(plan, keys + b0, w.t32, b1 - b0, cmp, st);
        if (s != APSEP_OK) return s;
        const bool look = b0 > 0;
        if (look) frontier_kernel<K, MAPF><<<1, 32, 0, st>>>(keys, lv, b0, fr);
        const K* cmin = (const K*)plan_chunk_minima(plan);  // this piece's, when in key order
        widen<<<grid, kThreads, 0, st>>>(keys, w.t32, out, b0, b1, lv, fr, look, pieces, cmin, err);
        if (cudaGetLastError() != cudaSuccess) return APSEP_ECUDA;
        if (!pieces || b1 == n) continue;
        // level entries that complete inside this piece (level 1 came with the pass)
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
    size_t bytes = align16((size_t)piece * 4) + 256;
    if (n > piece) {
        const size_t kb = info.dtype == APSEP_INT64 || info.dtype == APSEP_FLOAT64 ? 8 : 4;
        int64_t s = n;
        for (int l = 1, top = top_level(n); l <= top; l++) {
            s = ceil_div(s, 32);
            bytes += align16((size_t)s * kb);
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
    // widening and level passes, sized from that device's SMs), the caller's
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
