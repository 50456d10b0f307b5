// apsep_noalloc.cu -- apsep_run_noalloc: the single-array run without any
// device allocation.
//
// Some callers cannot allocate device memory when they need an answer: a
// host process that reserved the whole device heap up front for its own pool
// allocator, or a latency-critical path where cudaMalloc/cudaFree (and the
// device-wide synchronisation cudaFree implies) are not allowed.  For them
// the scratch this engine needs (control block, look-back words, tile and
// chunk minima) lives in one file-scope __device__ array below, sized for at
// most APSEP_NOALLOC_MAX_KEYS keys.  Every GPU that loads this library holds
// that array (2,869,504 bytes) until the process exits.
//
// Host code must not pass the array's name to a kernel: on the host it is
// only a stand-in symbol.  The first call on each device looks up the
// array's device address with cudaGetSymbolAddress (with that device
// current) and initialises its control block; later calls reuse the
// address.  All calls share the one array, so calls whose kernels overlap on
// the GPU race and must be serialised by the caller (e.g. one stream).
#include <cudaTypedefs.h>
#include <string.h>

#include <mutex>

#include "apsep.h"
#include "apsep_internal.h"

using namespace apsep;

namespace {

constexpr int64_t kMaxKeys = APSEP_NOALLOC_MAX_KEYS;
constexpr size_t kBytes = scratch_offsets(kMaxKeys).total;  // the same layout a plan uses
static_assert(kBytes == 2869504, "the size stated in include/apsep.h changed: update it there");

constexpr int kConfig = 0;                 // 16 warps per CTA, 512-key warp tiles
constexpr uint32_t kSpinLimit = 1u << 22;  // bound on every device-side wait
constexpr int kMaxDevices = 64;

// The scratch itself.  Zero-initialised at module load; set up per device below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

bool encode(CUtensorMap* map, const void* base, int rows, int tile_rows, int dtype) {
    auto enc = encoder();
    if (!enc) return false;
    cuuint64_t dims[2] = {32, (cuuint64_t)rows};
    cuuint64_t strides[1] = {128};
    cuuint32_t box[2] = {32, (cuuint32_t)tile_rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, dtype == APSEP_FLOAT32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_INT32, 2,
               const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Device address of the static scratch on the current device; the first
// call per device resolves it and writes the initial control block.
apsep_status scratch_for_current_device(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return APSEP_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return APSEP_ENOTSUP;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return APSEP_ECUDA;
        }
        Counters c0;
        memset(&c0, 0, sizeof(c0));
        c0.epoch = 1;
        if (cudaMemcpy(p, &c0, sizeof(c0), cudaMemcpyHostToDevice) != cudaSuccess) return APSEP_ECUDA;
        RangeScratch rs0;
        carve_scratch(p, kMaxKeys, &rs0);
        if (cudaMemset(rs0.group_min, 0xff, group_min_bytes()) != cudaSuccess) return APSEP_ECUDA;
        if (range_prepare(kConfig) != cudaSuccess) return APSEP_ECUDA;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return APSEP_OK;
}

}  // namespace

extern "C" apsep_status apsep_run_noalloc(const void* d_in, int32_t* d_out, int64_t n, apsep_dtype dtype,
                                          apsep_cmp cmp, void* stream) {
    if (n < 0 || (dtype != APSEP_INT32 && dtype != APSEP_FLOAT32) || (cmp != APSEP_LT && cmp != APSEP_LE))
        return APSEP_EINVAL;
    if (n > kMaxKeys) return APSEP_EINVAL;  // beyond the static scratch: use a plan
    if (n == 0) return APSEP_OK;
    if (!d_in || !d_out) return APSEP_EINVAL;
    if ((uintptr_t)d_in % 4 != 0 || (uintptr_t)d_out % 4 != 0) return APSEP_EINVAL;
    const uintptr_t a0 = (uintptr_t)d_in, b0 = (uintptr_t)d_out, bytes = (uintptr_t)n * 4;
    if (a0 < b0 + bytes && b0 < a0 + bytes) return APSEP_EINVAL;

    void* base = nullptr;
    apsep_status st = scratch_for_current_device(&base);
    if (st != APSEP_OK) return st;

    RangeScratch rs;
    carve_scratch(base, kMaxKeys, &rs);
    // The range counters must start at zero; a completed run leaves them so,
    // this also covers a run that never completed.
    if (cudaMemsetAsync(rs.ctr, 0, 2 * sizeof(uint32_t), (cudaStream_t)stream) != cudaSuccess ||
        cudaMemsetAsync(&rs.ctr->finished, 0, sizeof(uint32_t), (cudaStream_t)stream) != cudaSuccess)
        return APSEP_ECUDA;

    const TileConfig tc = kTileConfigs[kConfig];
    const int B = 32 * tc.ipt;  // keys per warp tile
    const int tile_rows = B / 32;
    // the view: `head` virtual keys in front put it on a 16-byte boundary
    const int vh = view_head(d_in, d_out);
    const int head = vh > 0 ? vh : 0;
    const int64_t nv = n + head;
    const void* v_in = (const char*)d_in - 4 * head;
    int32_t* v_out = d_out - head;
    int rows = (int)(nv / 32);
    CUtensorMap mi, mo;
    memset(&mi, 0, sizeof(mi));
    memset(&mo, 0, sizeof(mo));
    if (vh < 0 || rows < tile_rows) rows = 0;
    if (rows > 0 && (!encode(&mi, v_in, rows, tile_rows, dtype) || !encode(&mo, v_out, rows, tile_rows, 0)))
        return APSEP_ECUDA;

    RangeArgs a;
    a.d_in = v_in;
    a.d_out = v_out;
    a.n = (int)nv;
    a.head = head;
    a.num_tiles = (int)((nv + B - 1) / B);
    a.tiles_per_range = 0;
    a.num_ranges = 0;
    a.tma_rows = rows;
    a.spin_limit = kSpinLimit;
    a.skip_publish_range = -1;
    a.s = rs;
    const int incl = cmp == APSEP_LE ? 1 : 0;
    cudaError_t e = head ? launch_range_view(dtype, incl, kConfig, a, mi, mo, (cudaStream_t)stream)
                         : launch_range(dtype, incl, kConfig, a, mi, mo, (cudaStream_t)stream);
    return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
}
