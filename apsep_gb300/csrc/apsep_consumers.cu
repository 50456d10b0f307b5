// apsep_consumers.cu -- the classic callers of APSE, built on the engine.
//
// Previous greater, next smaller, stock span, largest rectangle in a
// histogram and Cartesian-tree parents are all nearest-smaller queries in
// disguise (the reference names them as the consumers of its output,
// README.md:3, src/bench_spt_le.cu:1-3):
//   previous greater  = APSE of the order-reversed keys (int: ~x, float: -x)
//   next smaller      = APSE of the reversed array, answers mirrored back
//   stock span        = i - previous strictly greater
//   largest rectangle = max over i of h[i] * (next smaller - previous smaller - 1)
//   Cartesian parent  = of previous smaller-or-equal and next smaller, the one
//                       with the larger key (ties: the next one)
// With 4-byte keys on a 16-byte boundary the engine does the flips and
// reversals itself (apsep_mapped.cu): previous greater and the stock span are
// one run each with the keys flipped as they load (and position - answer as
// the answers leave), next smaller one run over the reversed array with its
// answers mirrored as they leave (n a multiple of 32), and the histogram and
// Cartesian tree take that run for their next-smaller half.  Otherwise each is
// a few memory-bound passes (flip / reverse / mirror / epilogue, grid-stride,
// coalesced) around one or two engine runs.  All run on the caller's plan and
// stream with a caller-provided workspace: no allocation, no synchronisation,
// graph-capturable like apsep_run.
#include <stdint.h>

#include <type_traits>

#include "apsep.h"
#include "apsep_internal.h"

namespace {

constexpr int kThreads = 256;

int grid_for(int64_t n) {
    const int64_t b = (n + kThreads * 4 - 1) / (kThreads * 4);  // ~4 elements per thread
    return (int)(b < 1 ? 1 : b > 152 * 16 ? 152 * 16 : b);
}

size_t align16(size_t x) { return (x + 15) / 16 * 16; }

// Order-reversing map: a < b  <=>  flip(a) > flip(b), exactly (int: ~x = -x-1;
// float: -x, the two zeros stay equal).
__device__ __forceinline__ int32_t flip(int32_t x) { return ~x; }
__device__ __forceinline__ float flip(float x) { return -x; }
__device__ __forceinline__ int64_t flip(int64_t x) { return ~x; }
__device__ __forceinline__ double flip(double x) { return -x; }

int key_bytes(int dtype) { return dtype == APSEP_INT64 || dtype == APSEP_FLOAT64 ? 8 : 4; }

// Calls f(T*) with a null pointer of the plan's key type.
template <typename F>
void for_key_type(int dtype, F&& f) {
    switch (dtype) {
    case APSEP_INT32: f((int32_t*)nullptr); break;
    case APSEP_FLOAT32: f((float*)nullptr); break;
    case APSEP_INT64: f((int64_t*)nullptr); break;
    default: f((double*)nullptr); break;
    }
}

// Workspace: the keys (n of the plan's type), then two answer arrays.
struct Work {
    void* keys;
    int32_t* a;
    int32_t* b;
};
Work carve(void* d_work, int64_t n, int dtype) {
    char* w = (char*)d_work;
    const size_t kb = align16((size_t)n * key_bytes(dtype)), ab = align16((size_t)n * 4);
    return {w, (int32_t*)(w + kb), (int32_t*)(w + kb + ab)};
}

template <typename T>
__global__ void flip_keys(const T* __restrict__ in, T* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = flip(in[i]);
}

template <typename T>
__global__ void reverse_keys(const T* __restrict__ in, T* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = in[n - 1 - i];
}

// next[i] from the previous-smaller answers ar of the reversed array (-1: none).
__device__ __forceinline__ int64_t next_from_reversed(const int32_t* __restrict__ ar, int64_t n, int64_t i) {
    const int32_t a = ar[n - 1 - i];
    return a >= 0 ? n - 1 - a : -1;
}
// next[i] from R: the next-smaller answers themselves (direct, a reversed run
// of the engine), or the reversed array's previous-smaller answers.
__device__ __forceinline__ int64_t next_of(const int32_t* __restrict__ R, bool direct, int64_t n, int64_t i) {
    return direct ? (int64_t)R[i] : next_from_reversed(R, n, i);
}

__global__ void mirror_answers(const int32_t* __restrict__ ar, int32_t* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)next_from_reversed(ar, n, i);
}

__global__ void span_from_previous(int32_t* __restrict__ a, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (int32_t)(i - a[i]);
}

// max over i of h[i] * (R - L - 1): L previous strictly smaller (-1: none), R
// next strictly smaller (n: none).  Only positive areas compete (heights are
// non-negative by contract; a negative height contributes nothing).
__global__ void rect_area(const int32_t* __restrict__ h, const int32_t* __restrict__ L,
                          const int32_t* __restrict__ ar, bool direct, int64_t n, unsigned long long* __restrict__ best) {
    __shared__ long long warp_best[kThreads / 32];
    long long m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = next_of(ar, direct, n, i);
        const int64_t w = (r < 0 ? n : r) - (int64_t)L[i] - 1;
        const long long area = (long long)h[i] * w;
        m = area > m ? area : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(0xffffffffu, m, o);
        m = u > m ? u : m;
    }
    if ((threadIdx.x & 31) == 0) warp_best[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long b = 0;
        for (int w = 0; w < kThreads / 32; w++) b = warp_best[w] > b ? warp_best[w] : b;
        if (b > 0) atomicMax(best, (unsigned long long)b);
    }
}

// Min-rooted Cartesian tree, ties as the stack construction makes them (a
// later equal key is the right child of an earlier one): L previous
// smaller-or-equal, R next strictly smaller; the parent is the one with the
// larger key, R on a tie; -1 for the root.
template <typename T>
__global__ void cartesian_parent(const T* __restrict__ a, const int32_t* __restrict__ L,
                                 const int32_t* __restrict__ ar, bool direct, int32_t* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = L[i], r = next_of(ar, direct, n, i);
        int64_t p;
        if (r < 0) p = l;
        else if (l < 0) p = r;
        else p = a[r] >= a[l] ? r : l;
        out[i] = (int32_t)p;
    }
}

bool overlaps(const void* a, size_t an, const void* b, size_t bn) {
    const uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
    return a0 < b0 + bn && b0 < a0 + an;
}

// Common argument checks; fills the plan's key type.
apsep_status check_args(apsep_plan* plan, const void* d_in, const void* d_out, size_t out_bytes, int64_t n,
                        void* d_work, int* dtype) {
    if (!plan || n < 0) return APSEP_EINVAL;
    apsep_plan_info info;
    const apsep_status s = apsep_plan_get_info(plan, &info);
    if (s != APSEP_OK) return s;
    *dtype = info.dtype;
    if (n == 0) return APSEP_OK;
    if (n > info.capacity || !d_in || !d_out || !d_work) return APSEP_EINVAL;
    const size_t kb = (size_t)n * key_bytes(info.dtype);
    if ((uintptr_t)d_work % 16 != 0 || (uintptr_t)d_in % key_bytes(info.dtype) != 0) return APSEP_EINVAL;
    const size_t wb = (size_t)apsep_consumer_workspace_bytes(n);
    if (overlaps(d_work, wb, d_in, kb) || overlaps(d_work, wb, d_out, out_bytes)) return APSEP_EINVAL;
    return APSEP_OK;
}

apsep_status launched() { return cudaGetLastError() == cudaSuccess ? APSEP_OK : APSEP_ECUDA; }

}  // namespace

extern "C" {

int64_t apsep_consumer_workspace_bytes(int64_t n) {
    if (n < 0) return 0;
    return (int64_t)(align16((size_t)n * 8) + 2 * align16((size_t)n * 4));  // any key type
}

apsep_status apsep_run_prev_greater(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                                    void* d_work, void* stream) {
    int dtype = 0;
    apsep_status s = check_args(plan, d_in, d_out, (size_t)n * 4, n, d_work, &dtype);
    if (s != APSEP_OK || n == 0) return s;
    // one engine run that flips the keys as it loads them (4-byte keys on a
    // 16-byte boundary), else a flip pass into the workspace and a plain run
    if ((s = plan_run_flipped(plan, d_in, d_out, n, cmp, 0, stream)) != APSEP_ENOTSUP) return s;
    const cudaStream_t st = (cudaStream_t)stream;
    for_key_type(dtype, [&](auto tag) {
        using T = std::remove_pointer_t<decltype(tag)>;
        flip_keys<T><<<grid_for(n), kThreads, 0, st>>>((const T*)d_in, (T*)d_work, n);
    });
    if ((s = launched()) != APSEP_OK) return s;
    return apsep_run_cmp(plan, d_work, d_out, n, cmp, stream);
}

apsep_status apsep_run_next_smaller(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                                    void* d_work, void* stream) {
    int dtype = 0;
    apsep_status s = check_args(plan, d_in, d_out, (size_t)n * 4, n, d_work, &dtype);
    if (s != APSEP_OK || n == 0) return s;
    // one engine run over the reversed array, answers mirrored as they leave,
    // when it has that form for the call; else reverse, run, mirror
    if ((s = plan_run_reversed(plan, d_in, d_out, n, cmp, stream)) != APSEP_ENOTSUP) return s;
    const cudaStream_t st = (cudaStream_t)stream;
    const Work w = carve(d_work, n, dtype);
    for_key_type(dtype, [&](auto tag) {
        using T = std::remove_pointer_t<decltype(tag)>;
        reverse_keys<T><<<grid_for(n), kThreads, 0, st>>>((const T*)d_in, (T*)w.keys, n);
    });
    if ((s = launched()) != APSEP_OK) return s;
    if ((s = apsep_run_cmp(plan, w.keys, w.a, n, cmp, stream)) != APSEP_OK) return s;
    mirror_answers<<<grid_for(n), kThreads, 0, st>>>(w.a, d_out, n);
    return launched();
}

apsep_status apsep_stock_span(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, void* d_work,
                              void* stream) {
    int dtype = 0;
    apsep_status s = check_args(plan, d_in, d_out, (size_t)n * 4, n, d_work, &dtype);
    if (s != APSEP_OK || n == 0) return s;
    // one engine run that flips the keys as it loads them and writes
    // position - answer, when it has that form for the call
    if ((s = plan_run_flipped(plan, d_in, d_out, n, APSEP_LT, 1, stream)) != APSEP_ENOTSUP) return s;
    s = apsep_run_prev_greater(plan, d_in, d_out, n, APSEP_LT, d_work, stream);
    if (s != APSEP_OK || n == 0) return s;
    span_from_previous<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(d_out, n);
    return launched();
}

apsep_status apsep_largest_rectangle(apsep_plan* plan, const int32_t* d_heights, int64_t n, int64_t* d_area,
                                     void* d_work, void* stream) {
    int dtype = 0;
    apsep_status s = check_args(plan, d_heights, d_area, 8, n, d_work, &dtype);
    if (s != APSEP_OK) return s;
    if (dtype != APSEP_INT32) return APSEP_ENOTSUP;
    if (!d_area || (uintptr_t)d_area % 8 != 0) return APSEP_EINVAL;
    const cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(d_area, 0, 8, st) != cudaSuccess) return APSEP_ECUDA;
    if (n == 0) return APSEP_OK;
    const Work w = carve(d_work, n, dtype);
    if ((s = apsep_run_cmp(plan, d_heights, w.b, n, APSEP_LT, stream)) != APSEP_OK) return s;
    // next smaller: one reversed run when the engine has that form, else
    // reverse the heights and run (the answers then come mirrored)
    bool direct = true;
    if ((s = plan_run_reversed(plan, d_heights, w.a, n, APSEP_LT, stream)) == APSEP_ENOTSUP) {
        direct = false;
        reverse_keys<int32_t><<<grid_for(n), kThreads, 0, st>>>(d_heights, (int32_t*)w.keys, n);
        if ((s = launched()) != APSEP_OK) return s;
        s = apsep_run_cmp(plan, w.keys, w.a, n, APSEP_LT, stream);
    }
    if (s != APSEP_OK) return s;
    rect_area<<<grid_for(n), kThreads, 0, st>>>(d_heights, w.b, w.a, direct, n, (unsigned long long*)d_area);
    return launched();
}

apsep_status apsep_cartesian_parents(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, void* d_work,
                                     void* stream) {
    int dtype = 0;
    apsep_status s = check_args(plan, d_in, d_out, (size_t)n * 4, n, d_work, &dtype);
    if (s != APSEP_OK || n == 0) return s;
    const cudaStream_t st = (cudaStream_t)stream;
    const Work w = carve(d_work, n, dtype);
    if ((s = apsep_run_cmp(plan, d_in, w.b, n, APSEP_LE, stream)) != APSEP_OK) return s;
    bool direct = true;  // next smaller straight from a reversed run, else mirrored
    if ((s = plan_run_reversed(plan, d_in, w.a, n, APSEP_LT, stream)) == APSEP_ENOTSUP) {
        direct = false;
        for_key_type(dtype, [&](auto tag) {
            using T = std::remove_pointer_t<decltype(tag)>;
            reverse_keys<T><<<grid_for(n), kThreads, 0, st>>>((const T*)d_in, (T*)w.keys, n);
        });
        if ((s = launched()) != APSEP_OK) return s;
        s = apsep_run_cmp(plan, w.keys, w.a, n, APSEP_LT, stream);
    }
    if (s != APSEP_OK) return s;
    for_key_type(dtype, [&](auto tag) {
        using T = std::remove_pointer_t<decltype(tag)>;
        cartesian_parent<T><<<grid_for(n), kThreads, 0, st>>>((const T*)d_in, w.b, w.a, direct, d_out, n);
    });
    return launched();
}

}  // extern "C"
