// apsep_device.cuh -- device-side building blocks of the GB300 APSE engine.
//
// Inline-PTX wrappers for the sm_100-family async machinery the tile kernels
// use (mbarrier, TMA tensor loads/stores, async-proxy fences, gpu-scope
// acquire/release), the key traits, the comparator, and the shared-memory
// 128-byte swizzle index map that matches CU_TENSOR_MAP_SWIZZLE_128B.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include <limits.h>

namespace apsep {

// ---------------------------------------------------------------------------
// Keys.  Padding value for positions >= n (the reference pads its tail block
// with ApsepInfinity<T>, src/apsep.cuh:53-70).  Padded positions lie to the
// right of every real element, so they are never an answer and never query.
// ---------------------------------------------------------------------------
template <typename T> struct KeyTraits;
template <> struct KeyTraits<int32_t> {
    __device__ __forceinline__ static int32_t pad() { return INT_MAX; }
    __device__ __forceinline__ static int32_t vmin(int32_t a, int32_t b) { return min(a, b); }
    __device__ __forceinline__ static uint32_t bits(int32_t a) { return (uint32_t)a; }
    __device__ __forceinline__ static int32_t from_bits(uint32_t b) { return (int32_t)b; }
    // order-preserving map to unsigned (for unsigned atomic minima) and back
    __device__ __forceinline__ static uint32_t ord(int32_t a) { return (uint32_t)a ^ 0x80000000u; }
    __device__ __forceinline__ static int32_t from_ord(uint32_t o) { return (int32_t)(o ^ 0x80000000u); }
};
template <> struct KeyTraits<float> {
    __device__ __forceinline__ static float pad() { return __int_as_float(0x7f800000); }  // +inf
    // fminf: for the two zeros (equal under <, <=) either may be returned;
    // no comparison outcome depends on which.
    __device__ __forceinline__ static float vmin(float a, float b) { return fminf(a, b); }
    __device__ __forceinline__ static uint32_t bits(float a) { return __float_as_uint(a); }
    __device__ __forceinline__ static float from_bits(uint32_t b) { return __uint_as_float(b); }
    // order-preserving map to unsigned: negatives reversed below the positives
    __device__ __forceinline__ static uint32_t ord(float a) {
        const uint32_t b = __float_as_uint(a);
        return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    }
    __device__ __forceinline__ static float from_ord(uint32_t o) {
        return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
    }
};

// 8-byte keys (int64, and float64 through f64_order below), with int32
// positions: bits are the raw 64-bit pattern; their status words keep the
// key apart from the tag.
template <> struct KeyTraits<int64_t> {
    __device__ __forceinline__ static int64_t pad() { return LLONG_MAX; }
    __device__ __forceinline__ static int64_t vmin(int64_t a, int64_t b) { return a < b ? a : b; }
    __device__ __forceinline__ static uint64_t bits(int64_t a) { return (uint64_t)a; }
    __device__ __forceinline__ static int64_t from_bits(uint64_t b) { return (int64_t)b; }
};

// float64 keys compare as int64 (the FP64 pipe is slow on this part): the
// order-preserving map of a float64 bit pattern to int64, both zeros to 0,
// so a < b as doubles <=> f64_order(a) < f64_order(b) for every non-NaN pair.
__device__ __forceinline__ int64_t f64_order(int64_t b) {
    return (b << 1) == 0 ? 0 : (b ^ ((b >> 63) & 0x7fffffffffffffffLL));
}
// Key maps, applied as keys enter registers or shared memory (the engine's
// KMAP template parameter): KMAP_F64 -- int64 slots holding float64 bit
// patterns, compared through f64_order; KMAP_FLIP -- the order-reversing map
// (integers ~x = -x - 1, floats -x; the two zeros stay equal), so that a
// previous-smaller run answers previous-greater queries.
constexpr int KMAP_NONE = 0, KMAP_F64 = 1, KMAP_FLIP = 2;
__device__ __forceinline__ int32_t flip_key(int32_t x) { return ~x; }
__device__ __forceinline__ float flip_key(float x) { return -x; }
__device__ __forceinline__ int64_t flip_key(int64_t x) { return ~x; }
template <typename T, int KMAP>
__device__ __forceinline__ T map_key(T x) {
    if constexpr (KMAP == KMAP_F64) return (T)f64_order((int64_t)x);
    else if constexpr (KMAP == KMAP_FLIP) return flip_key(x);
    else return x;
}
// A key from global memory, through the key map.
template <typename T, int KMAP>
__device__ __forceinline__ T load_key(const T* p) {
    return map_key<T, KMAP>(__ldg(p));
}

// lt(a, b): "a qualifies as the answer for query b".  INCL=false is the
// strict previous-smaller (APSEP), INCL=true previous-smaller-or-equal; the
// reference routes every comparison through the same predicate
// (src/apsep.cuh:2669-2673).
template <bool INCL, typename T>
__device__ __forceinline__ bool lt(T a, T b) { return INCL ? (a <= b) : (a < b); }

// ---------------------------------------------------------------------------
// 128-byte swizzle.  A TMA tile with CU_TENSOR_MAP_SWIZZLE_128B and a 128-byte
// inner box row stores 16-byte chunk c of row r at chunk c ^ (r % 8) (smem
// buffer 1024-byte aligned).  In 4-byte word units: word e -> e ^ ((e>>3)&0x1C).
// The map keeps 4-word groups contiguous, so int4 accesses stay legal, and a
// thread reading 16/8/4 consecutive keys with 128-bit loads is bank-conflict
// free.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int swz(int e) { return e ^ ((e >> 3) & 0x1C); }
// The same map in 8-byte element units: element e -> e ^ ((e>>3)&0x0E)
// (chunk (e>>1)&7 of row e>>4); pairs stay contiguous.
__device__ __forceinline__ int swz8(int e) { return e ^ ((e >> 3) & 0x0E); }
// Swizzled index of key e in a key array of KB-byte keys.
template <int KB>
__device__ __forceinline__ int kswz(int e) { return KB == 8 ? swz8(e) : swz(e); }

// ---------------------------------------------------------------------------
// mbarrier
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbarrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// A plain arrival (no transaction bytes): completes the phase of a count-1 barrier.
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false when `limit` polls passed without completion.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++) {
        if (mbar_try_wait(bar, phase)) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

// ---------------------------------------------------------------------------
// TMA (tensor) copies, 2-D, tile mode.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* smem_src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     (uint64_t)map),
                 "r"(x), "r"(y), "r"(smem_u32(smem_src))
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() {
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Generic-proxy smem writes -> visible to the async proxy (before a TMA store).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Completed bulk (async-proxy) writes to global -> ordered before later generic accesses.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// ---------------------------------------------------------------------------
// gpu-scope acquire / release on 64-bit status words, L2-only loads.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Atomic add with acquire + release semantics at gpu scope; returns the old value.
__device__ __forceinline__ uint32_t atom_add_acq_rel_u32(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
// Fire-and-forget atomic minimum (relaxed, gpu scope).
__device__ __forceinline__ void red_min_u64(uint64_t* p, uint64_t v) {
    asm volatile("red.relaxed.gpu.global.min.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

}  // namespace apsep
