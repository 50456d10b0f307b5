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
// that array (2,902,272 bytes) until the process exits.
//
// Host code must not pass the array's name to a kernel: on the host it is
// only a stand-in symbol.  Every call looks up the array's device address
// with cudaGetSymbolAddress (with the caller's device current; the lookup
// allocates nothing).  The first call in each CUDA context on a device -- the
// first of the process, or the first after cudaDeviceReset or a switch to
// another context, each of which loads the module afresh -- clears the array
// and writes its initial control block.  All calls share the one array, so
// calls whose kernels overlap on the GPU race and must be serialised by the
// caller (e.g. one stream).  Device-side errors (a wait that gave up, a
// broken search invariant) are sticky in the array's control block until
// apsep_noalloc_check reads and clears them.
#include <cudaTypedefs.h>
#include <string.h>

#include <mutex>

#include "apsep.h"
#include "apsep_internal.h"

using namespace apsep;

namespace {

constexpr int64_t kMaxKeys = APSEP_NOALLOC_MAX_KEYS;
constexpr size_t kBytes = scratch_offsets(kMaxKeys).total;  // the same layout a plan uses
static_assert(kBytes == 2902272, "the size stated in include/apsep.h changed: update it there");

constexpr int kConfig = 0;                 // 16 warps per CTA, 512-key warp tiles
constexpr uint32_t kSpinLimit = 1u << 22;  // bound on every device-side wait
constexpr int kMaxDevices = 64;

// The scratch itself.  Zero-initialised at module load; set up per device below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

std::mutex g_mu;
// Per device: the context whose copy of the array was last set up, and its address.
unsigned long long g_ctx[kMaxDevices] = {};
void* g_addr[kMaxDevices] = {};
// One-shot fault injection for the next run (apsep_debug_inject with no plan).
int g_dbg_skip_range = -1;
uint32_t g_dbg_spin_limit = 0;

using PFN_ctxGetCurrent = CUresult (*)(CUcontext*);
using PFN_ctxGetId = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the caller's current CUDA context (0 if none can be read).
unsigned long long current_context_id() {
    static PFN_ctxGetCurrent get_cur = nullptr;
    static PFN_ctxGetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = (PFN_ctxGetCurrent)p;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (PFN_ctxGetId)p;
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_cur || !get_id || get_cur(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

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

// Device address of the static scratch on the current device and context.
// The address is looked up on every call; the array is set up when the
// context (or the address) differs from the one set up last on this device.
apsep_status scratch_for_current_device(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return APSEP_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return APSEP_ENOTSUP;
    std::lock_guard<std::mutex> lock(g_mu);
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return APSEP_ECUDA;
    }
    const unsigned long long ctx = current_context_id();
    if (g_addr[dev] != p || g_ctx[dev] != ctx) {
        int major = 0;
        if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess)
            return APSEP_ECUDA;
        if (major < 10) return APSEP_ENOTSUP;  // the engine is built for sm_103a
        // Stale tags from runs in an earlier context could alias the restarted
        // epochs: clear the whole array, then write the initial control block.
        if (cudaMemset(p, 0, kBytes) != cudaSuccess) return APSEP_ECUDA;
        Counters c0;
        memset(&c0, 0, sizeof(c0));
        c0.epoch = 1;
        if (cudaMemcpy(p, &c0, sizeof(c0), cudaMemcpyHostToDevice) != cudaSuccess) return APSEP_ECUDA;
        RangeScratch rs0;
        carve_scratch(p, kMaxKeys, &rs0);
        if (cudaMemset(rs0.group_min, 0xff, group_min_bytes()) != cudaSuccess) return APSEP_ECUDA;
        if (range_prepare(kConfig) != cudaSuccess) return APSEP_ECUDA;
        g_addr[dev] = p;
        g_ctx[dev] = ctx;
    }
    *out = p;
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
    {
        std::lock_guard<std::mutex> lock(g_mu);
        a.spin_limit = g_dbg_spin_limit ? g_dbg_spin_limit : kSpinLimit;
        a.skip_publish_range = g_dbg_skip_range;
        g_dbg_skip_range = -1;  // one-shot
        g_dbg_spin_limit = 0;
    }
    a.s = rs;
    const int incl = cmp == APSEP_LE ? 1 : 0;
    cudaError_t e = head ? launch_range_view(dtype, incl, kConfig, a, mi, mo, (cudaStream_t)stream)
                         : launch_range(dtype, incl, kConfig, a, mi, mo, (cudaStream_t)stream);
    return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
}

extern "C" apsep_status apsep_noalloc_check(void* stream) {
    void* base = nullptr;
    apsep_status st = scratch_for_current_device(&base);
    if (st != APSEP_OK) return st;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return APSEP_ECUDA;
    Counters c0;
    if (cudaMemcpy(&c0, base, sizeof(c0), cudaMemcpyDeviceToHost) != cudaSuccess) return APSEP_ECUDA;
    const uint32_t err = c0.err;
    if (!err) return APSEP_OK;
    // A run that gave up may have left its counters half-way: re-arm the
    // control block, keeping the epoch.
    const uint32_t epoch = c0.epoch;
    memset(&c0, 0, sizeof(c0));
    c0.epoch = epoch;
    if (cudaMemcpy(base, &c0, sizeof(c0), cudaMemcpyHostToDevice) != cudaSuccess) return APSEP_ECUDA;
    if (err & (ERR_LOOKBACK_TIMEOUT | ERR_TMA_TIMEOUT)) return APSEP_ETIMEOUT;
    return APSEP_EINTERNAL;
}

namespace apsep {
void noalloc_debug_inject(int32_t range, uint32_t spin_limit) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_dbg_skip_range = range;
    g_dbg_spin_limit = spin_limit;
}
}  // namespace apsep
