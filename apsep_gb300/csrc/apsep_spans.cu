// apsep_spans.cu -- apsep_copy_spans: many byte spans copied in one launch.
//
// The serving layer gathers the keys of every request it admits into its
// device pool, and scatters answers back out, many spans at a time; one
// cudaMemcpyAsync per span would cost the host several microseconds each.
// Here the span descriptors travel as kernel parameters (up to kMaxSpans
// per launch), the work is cut into 16 KB pieces, and every CTA copies whole
// pieces.  Where both ends are 16-byte aligned a piece goes through shared
// memory: all of it in flight at once by asynchronous 16-byte copies, then
// stored back.  The CTAs are small (two warps, 16 KB of shared memory, few
// registers) so that one fits on an SM beside a running engine CTA: a gather
// issued on another stream overlaps the engine instead of waiting for its
// SMs.
#include <string.h>

#include <mutex>

#include "apsep.h"

namespace {

constexpr int kMaxSpans = 256;
constexpr int64_t kPiece = 16384;  // bytes per work item
constexpr int kThreads = 64;

struct SpanBatch {
    int n;
    int64_t piece_start[kMaxSpans + 1];  // exclusive prefix sum of each span's pieces
    const char* src[kMaxSpans];
    char* dst[kMaxSpans];
    int64_t bytes[kMaxSpans];
};

// 16-byte global -> shared copy that completes asynchronously (cp.async):
// the in-flight data sits in shared memory, not in registers.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

constexpr int kDepth = (int)(kPiece / 16 / kThreads);  // 16-byte copies per thread per piece

__global__ void __launch_bounds__(kThreads, 16) copy_spans_kernel(const __grid_constant__ SpanBatch b) {
    __shared__ __align__(16) uint4 stage[kThreads * kDepth];  // one piece (16 KB)
    const int64_t total = b.piece_start[b.n];
    for (int64_t pc = blockIdx.x; pc < total; pc += gridDim.x) {
        // the span holding piece pc: the last s with piece_start[s] <= pc (empty spans are skipped)
        int lo = 0, hi = b.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (b.piece_start[mid] <= pc) lo = mid;
            else hi = mid - 1;
        }
        const int64_t off = (pc - b.piece_start[lo]) * kPiece;
        const int64_t len = min(kPiece, b.bytes[lo] - off);
        const char* src = b.src[lo] + off;
        char* dst = b.dst[lo] + off;
        const uintptr_t al = (uintptr_t)src | (uintptr_t)dst;
        int64_t done = 0;
        if ((al & 15) == 0) {
            // the whole piece in flight at once through shared memory; each thread
            // stores back only the 16-byte words it loaded itself
            const int nv = (int)(len >> 4);
            const uint4* s4 = reinterpret_cast<const uint4*>(src);
            uint4* d4 = reinterpret_cast<uint4*>(dst);
#pragma unroll
            for (int j = 0; j < kDepth; j++) {
                const int i = j * kThreads + threadIdx.x;
                if (i < nv) cp_async16(&stage[i], s4 + i);
            }
            cp_async_wait_all();
#pragma unroll
            for (int j = 0; j < kDepth; j++) {
                const int i = j * kThreads + threadIdx.x;
                if (i < nv) d4[i] = stage[i];
            }
            done = (int64_t)nv << 4;
        } else if ((al & 3) == 0) {
            const int64_t nw = len >> 2;
            for (int64_t i = threadIdx.x; i < nw; i += kThreads)
                reinterpret_cast<uint32_t*>(dst)[i] = __ldg(reinterpret_cast<const uint32_t*>(src) + i);
            done = nw << 2;
        }
        for (int64_t i = done + threadIdx.x; i < len; i += kThreads) dst[i] = src[i];
    }
}

int ctas_for_device() {
    static int ctas[64] = {};
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    std::lock_guard<std::mutex> lock(mu);
    if (!ctas[dev]) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
        // the same shared-memory carveout as the engine's kernels, so that an SM
        // running an engine CTA can take a copy CTA beside it
        if (cudaFuncSetAttribute(copy_spans_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return 0;
        ctas[dev] = sms * 16;
    }
    return ctas[dev];
}

}  // namespace

extern "C" apsep_status apsep_copy_spans(const void* const* src, void* const* dst, const int64_t* bytes,
                                         int32_t nspans, void* stream) {
    if (nspans < 0 || (nspans > 0 && (!src || !dst || !bytes))) return APSEP_EINVAL;
    for (int32_t i = 0; i < nspans; i++)
        if (bytes[i] < 0 || (bytes[i] > 0 && (!src[i] || !dst[i]))) return APSEP_EINVAL;
    const int ctas = ctas_for_device();
    if (ctas <= 0) return APSEP_ECUDA;
    SpanBatch b;
    for (int32_t i0 = 0; i0 < nspans; i0 += kMaxSpans) {
        const int m = nspans - i0 < kMaxSpans ? nspans - i0 : kMaxSpans;
        b.n = m;
        b.piece_start[0] = 0;
        for (int j = 0; j < m; j++) {
            b.src[j] = (const char*)src[i0 + j];
            b.dst[j] = (char*)dst[i0 + j];
            b.bytes[j] = bytes[i0 + j];
            b.piece_start[j + 1] = b.piece_start[j] + (bytes[i0 + j] + kPiece - 1) / kPiece;
        }
        const int64_t pieces = b.piece_start[m];
        if (pieces == 0) continue;
        const int grid = (int)(pieces < ctas ? pieces : ctas);
        copy_spans_kernel<<<grid, kThreads, 0, (cudaStream_t)stream>>>(b);
        if (cudaGetLastError() != cudaSuccess) return APSEP_ECUDA;
    }
    return APSEP_OK;
}
