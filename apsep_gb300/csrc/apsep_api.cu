// apsep_api.cu -- the C ABI (include/apsep.h): plans, runs, status codes.
//
// A plan owns one device allocation of scratch (control block, look-back
// status words, tile mins, chunk mins) sized for its capacity; runs only
// enqueue kernels.  Errors are status codes, never exit() (the reference's
// gpuAssert exits, src/apsep.cuh:39-47).
#include <cudaTypedefs.h>
#include <string.h>

#include <mutex>

#include "apsep.h"
#include "apsep_internal.h"

using namespace apsep;

struct apsep_plan {
    int device = 0;
    int dtype = 0;
    int cmp = 0;
    int cfg = 0;
    int64_t capacity = 0;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    RangeScratch rs{};
    int dbg_skip_range = -1;
    uint32_t dbg_spin_limit = 0;
};

namespace {

constexpr uint32_t kDefaultSpinLimit = 1u << 22;  // ~1 s of polling with back-off
constexpr int64_t kMaxKeysPerRun = (int64_t)INT32_MAX - 4095;  // APSEP_MAX_KEYS

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    std::call_once(g_encode_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    return g_encode;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

bool wide(int dtype) { return dtype == APSEP_INT64 || dtype == APSEP_FLOAT64; }
int key_bytes(int dtype) { return wide(dtype) ? 8 : 4; }

// 2-D view of an array as 128-byte rows (32 4-byte or 16 8-byte elements),
// box = one tile (tile_rows rows).
bool encode_rows(CUtensorMap* map, const void* base, int rows, int tile_rows, int dtype) {
    auto enc = encoder();
    if (!enc) return false;
    const cuuint64_t per_row = (cuuint64_t)(128 / key_bytes(dtype));
    cuuint64_t dims[2] = {per_row, (cuuint64_t)rows};
    cuuint64_t strides[1] = {128};
    cuuint32_t box[2] = {(cuuint32_t)per_row, (cuuint32_t)tile_rows};
    cuuint32_t estr[2] = {1, 1};
    const CUtensorMapDataType t = dtype == APSEP_FLOAT32   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                  : dtype == APSEP_INT64   ? CU_TENSOR_MAP_DATA_TYPE_INT64
                                  : dtype == APSEP_FLOAT64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                                           : CU_TENSOR_MAP_DATA_TYPE_INT32;
    CUresult r = enc(map, t, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            ok = false;
            return;
        }
        if (prev != dev && cudaSetDevice(dev) != cudaSuccess) ok = false;
    }
    ~DeviceGuard() {
        int cur;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

bool ranges_overlap(const void* a, size_t an, const void* b, size_t bn) {
    uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
    return a0 < b0 + bn && b0 < a0 + an;
}

}  // namespace


extern "C" {

int apsep_version(void) { return 10000; }

const char* apsep_status_string(apsep_status s) {
    switch (s) {
    case APSEP_OK: return "ok";
    case APSEP_EINVAL: return "invalid argument";
    case APSEP_ENOMEM: return "out of device memory";
    case APSEP_ECUDA: return "CUDA error";
    case APSEP_ETIMEOUT: return "device-side wait timed out";
    case APSEP_EINTERNAL: return "device-side invariant failed";
    case APSEP_ENOTSUP: return "not supported";
    }
    return "unknown status";
}

int32_t apsep_num_configs(void) { return kNumTileConfigs; }

apsep_status apsep_config_shape(int32_t config, int32_t* threads, int32_t* keys_per_thread) {
    if (config < 0 || config >= kNumTileConfigs) return APSEP_EINVAL;
    if (threads) *threads = kTileConfigs[config].wpc * 32;
    if (keys_per_thread) *keys_per_thread = kTileConfigs[config].ipt;
    return APSEP_OK;
}

apsep_status apsep_plan_create(apsep_plan** out, apsep_dtype dtype, apsep_cmp cmp, int64_t capacity) {
    if (!out) return APSEP_EINVAL;
    *out = nullptr;
    if ((dtype != APSEP_INT32 && dtype != APSEP_FLOAT32 && !wide(dtype)) || (cmp != APSEP_LT && cmp != APSEP_LE))
        return APSEP_EINVAL;
    // int32 positions; the last tile's end (up to n rounded up to whole tiles)
    // must stay below 2^31 as well
    if (capacity < 0 || capacity > kMaxKeysPerRun) return APSEP_EINVAL;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return APSEP_ECUDA;
    int major = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return APSEP_ECUDA;
    if (major < 10) return APSEP_ENOTSUP;  // TMA tensor path + sm_103a build

    apsep_plan* p = new apsep_plan();
    p->device = dev;
    p->dtype = dtype;
    p->cmp = cmp;
    p->capacity = capacity;
    p->cfg = wide(dtype) ? 1 : 0;  // 8-byte keys: the one configuration their kernels have (8 keys per lane)
    const size_t total = carve_scratch(nullptr, capacity, nullptr, key_bytes(dtype));
    if (cudaMalloc(&p->scratch, total) != cudaSuccess) {
        cudaGetLastError();
        delete p;
        return APSEP_ENOMEM;
    }
    p->scratch_bytes = total;
    carve_scratch(p->scratch, capacity, &p->rs, key_bytes(dtype));
    Counters c0;
    memset(&c0, 0, sizeof(c0));
    c0.epoch = 1;
    if (cudaMemset(p->scratch, 0, total) != cudaSuccess ||
        cudaMemset(p->rs.group_min, 0xff, group_min_bytes()) != cudaSuccess ||
        cudaMemcpy(p->rs.ctr, &c0, sizeof(c0), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(p->scratch);
        delete p;
        return APSEP_ECUDA;
    }
    for (int cfg = 0; cfg < kNumTileConfigs; cfg++)
        if (range_prepare(cfg) != cudaSuccess || (wide(dtype) && prepare_wide() != cudaSuccess)) {
            cudaGetLastError();
            cudaFree(p->scratch);
            delete p;
            return APSEP_ECUDA;
        }
    *out = p;
    return APSEP_OK;
}

apsep_status apsep_plan_destroy(apsep_plan* p) {
    if (!p) return APSEP_OK;
    DeviceGuard g(p->device);
    cudaError_t e = cudaFree(p->scratch);
    delete p;
    return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
}

apsep_status apsep_plan_get_info(const apsep_plan* p, apsep_plan_info* info) {
    if (!p || !info) return APSEP_EINVAL;
    memset(info, 0, sizeof(*info));
    info->capacity = p->capacity;
    info->scratch_bytes = (int64_t)p->scratch_bytes;
    info->tile_keys = 32 * kTileConfigs[p->cfg].ipt;  // one warp's tile
    info->config = p->cfg;
    info->device = p->device;
    info->dtype = p->dtype;
    info->cmp = p->cmp;
    return APSEP_OK;
}

apsep_status apsep_plan_set_config(apsep_plan* p, int32_t config) {
    if (!p || config < 0 || config >= kNumTileConfigs) return APSEP_EINVAL;
    if (wide(p->dtype) && config != 1) return APSEP_ENOTSUP;  // 8-byte keys: 8 keys per lane only
    p->cfg = config;
    return APSEP_OK;
}

}  // extern "C"

namespace {

// One run of the range engine: a single array, or (offsets != nullptr) a batch
// of nseg segments stored back to back.
apsep_status run_impl(apsep_plan* p, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                      const int64_t* offsets, int32_t nseg, void* stream) {
    if (!p || n < 0 || (cmp != APSEP_LT && cmp != APSEP_LE)) return APSEP_EINVAL;
    if (offsets && (nseg < 1 || (uintptr_t)offsets % 8 != 0)) return APSEP_EINVAL;
    if (n == 0) return APSEP_OK;
    if (n > p->capacity || !d_in || !d_out) return APSEP_EINVAL;
    const size_t kb = (size_t)key_bytes(p->dtype);
    if ((uintptr_t)d_in % kb != 0 || (uintptr_t)d_out % 4 != 0) return APSEP_EINVAL;  // keys, answers aligned
    if (ranges_overlap(d_in, (size_t)n * kb, d_out, (size_t)n * 4)) return APSEP_EINVAL;
    if (offsets && (ranges_overlap(offsets, (size_t)(nseg + 1) * 8, d_out, (size_t)n * 4) ||
                    ranges_overlap(offsets, (size_t)(nseg + 1) * 8, d_in, (size_t)n * kb)))
        return APSEP_EINVAL;
    DeviceGuard g(p->device);
    if (!g.ok) return APSEP_ECUDA;
    if (wide(p->dtype)) {  // 8-byte keys: TMA when both arrays are 16-byte aligned
        const int B = kWideTileKeys, key_rows_per_tile = B * 8 / 128;
        int rows = (int)(n / 16);  // 128-byte rows of keys
        CUtensorMap mi, mo;
        memset(&mi, 0, sizeof(mi));
        memset(&mo, 0, sizeof(mo));
        if ((uintptr_t)d_in % 16 != 0 || (uintptr_t)d_out % 16 != 0 || rows < key_rows_per_tile) rows = 0;
        if (rows > 0) {
            if (!encode_rows(&mi, d_in, rows, key_rows_per_tile, p->dtype) ||
                !encode_rows(&mo, d_out, (int)(n / 32), B / 32, APSEP_INT32))
                return APSEP_ECUDA;
        }
        RangeArgs a;
        a.d_in = d_in;
        a.d_out = d_out;
        a.n = (int)n;
        a.head = 0;
        a.num_tiles = (int)((n + B - 1) / B);
        a.tiles_per_range = 0;
        a.num_ranges = 0;
        a.tma_rows = rows;
        a.spin_limit = p->dbg_spin_limit ? p->dbg_spin_limit : kDefaultSpinLimit;
        a.skip_publish_range = p->dbg_skip_range;
        a.offsets = offsets;
        a.nseg = offsets ? nseg : 0;
        a.s = p->rs;
        p->dbg_skip_range = -1;
        p->dbg_spin_limit = 0;
        const cudaError_t e = launch_range_wide(p->dtype, cmp == APSEP_LE ? 1 : 0, a, mi, mo, (cudaStream_t)stream);
        return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
    }

    const TileConfig tc = kTileConfigs[p->cfg];
    const int B = 32 * tc.ipt;  // keys per warp tile
    const int tile_rows = B / 32;
    // the view: `head` virtual keys in front put it on a 16-byte boundary
    const int vh = view_head(d_in, d_out);
    const int head = vh > 0 ? vh : 0;
    const int64_t nv = n + head;
    const void* v_in = (const char*)d_in - 4 * head;
    int32_t* v_out = d_out - head;
    const int64_t num_tiles = (nv + B - 1) / B;
    int rows = (int)(nv / 32);
    CUtensorMap mi, mo;
    memset(&mi, 0, sizeof(mi));
    memset(&mo, 0, sizeof(mo));
    if (vh < 0 || rows < tile_rows) rows = 0;
    if (rows > 0) {
        if (!encode_rows(&mi, v_in, rows, tile_rows, p->dtype) || !encode_rows(&mo, v_out, rows, tile_rows, 0))
            return APSEP_ECUDA;
    }
    RangeArgs a;
    a.d_in = v_in;
    a.d_out = v_out;
    a.n = (int)nv;
    a.head = head;
    a.num_tiles = (int)num_tiles;
    a.tiles_per_range = 0;
    a.num_ranges = 0;
    a.tma_rows = rows;
    a.spin_limit = p->dbg_spin_limit ? p->dbg_spin_limit : kDefaultSpinLimit;
    a.skip_publish_range = p->dbg_skip_range;
    // (a single array behind a view head runs in the view kernel: one implicit
    //  segment; the plain single-array kernel has no view head)
    a.offsets = offsets;
    a.nseg = offsets ? nseg : 1;
    a.s = p->rs;
    p->dbg_skip_range = -1;  // one-shot
    p->dbg_spin_limit = 0;
    const int incl = cmp == APSEP_LE ? 1 : 0;
    cudaError_t e = offsets ? launch_range_segmented(p->dtype, incl, p->cfg, a, mi, mo, (cudaStream_t)stream)
                    : head  ? launch_range_view(p->dtype, incl, p->cfg, a, mi, mo, (cudaStream_t)stream)
                            : launch_range(p->dtype, incl, p->cfg, a, mi, mo, (cudaStream_t)stream);
    return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
}

}  // namespace

apsep_status plan_run_flipped(apsep_plan* p, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp, int span,
                              void* stream) {
    if (!p || n <= 0 || n > p->capacity || !d_in || !d_out || (cmp != APSEP_LT && cmp != APSEP_LE)) return APSEP_EINVAL;
    if (wide(p->dtype) || (span && cmp != APSEP_LT)) return APSEP_ENOTSUP;
    if ((uintptr_t)d_in % 4 != 0 || (uintptr_t)d_out % 4 != 0) return APSEP_EINVAL;
    // answers over the keys themselves (in place) take the general route, which
    // reads the keys into the workspace first
    if (ranges_overlap(d_in, (size_t)n * 4, d_out, (size_t)n * 4)) return APSEP_ENOTSUP;
    // a view head would need the view instantiation: those runs take the general route
    if ((uintptr_t)d_in % 16 != (uintptr_t)d_out % 16 || (uintptr_t)d_in % 16 != 0) return APSEP_ENOTSUP;
    DeviceGuard g(p->device);
    if (!g.ok) return APSEP_ECUDA;
    const int B = 32 * kTileConfigs[0].ipt;  // keys per warp tile
    const int tile_rows = B / 32;
    int rows = (int)(n / 32);
    CUtensorMap mi, mo;
    memset(&mi, 0, sizeof(mi));
    memset(&mo, 0, sizeof(mo));
    if (rows < tile_rows) rows = 0;
    if (rows > 0 && (!encode_rows(&mi, d_in, rows, tile_rows, p->dtype) || !encode_rows(&mo, d_out, rows, tile_rows, 0)))
        return APSEP_ECUDA;
    RangeArgs a;
    a.d_in = d_in;
    a.d_out = d_out;
    a.n = (int)n;
    a.head = 0;
    a.num_tiles = (int)((n + B - 1) / B);
    a.tiles_per_range = 0;
    a.num_ranges = 0;
    a.tma_rows = rows;
    a.spin_limit = p->dbg_spin_limit ? p->dbg_spin_limit : kDefaultSpinLimit;
    a.skip_publish_range = p->dbg_skip_range;
    a.offsets = nullptr;
    a.nseg = 1;
    a.s = p->rs;
    p->dbg_skip_range = -1;
    p->dbg_spin_limit = 0;
    const cudaError_t e =
        launch_range_flipped(p->dtype, cmp == APSEP_LE ? 1 : 0, span, a, mi, mo, (cudaStream_t)stream);
    return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
}

apsep_status plan_run_reversed(apsep_plan* p, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                               void* stream) {
    if (!p || n <= 0 || n > p->capacity || !d_in || !d_out || (cmp != APSEP_LT && cmp != APSEP_LE)) return APSEP_EINVAL;
    if (wide(p->dtype) || n % 32 != 0) return APSEP_ENOTSUP;
    if ((uintptr_t)d_in % 16 != 0 || (uintptr_t)d_out % 16 != 0) return APSEP_ENOTSUP;
    if (ranges_overlap(d_in, (size_t)n * 4, d_out, (size_t)n * 4)) return APSEP_ENOTSUP;  // in place: general route
    DeviceGuard g(p->device);
    if (!g.ok) return APSEP_ECUDA;
    const int B = 32 * kTileConfigs[0].ipt;  // keys per warp tile
    const int tile_rows = B / 32;
    int rows = (int)(n / 32);
    CUtensorMap mi, mo;
    memset(&mi, 0, sizeof(mi));
    memset(&mo, 0, sizeof(mo));
    if (rows < tile_rows) rows = 0;
    if (rows > 0 && (!encode_rows(&mi, d_in, rows, tile_rows, p->dtype) || !encode_rows(&mo, d_out, rows, tile_rows, 0)))
        return APSEP_ECUDA;
    RangeArgs a;
    a.d_in = d_in;
    a.d_out = d_out;
    a.n = (int)n;
    a.head = 0;
    a.num_tiles = (int)((n + B - 1) / B);
    a.tiles_per_range = 0;
    a.num_ranges = 0;
    a.tma_rows = rows;
    a.spin_limit = p->dbg_spin_limit ? p->dbg_spin_limit : kDefaultSpinLimit;
    a.skip_publish_range = p->dbg_skip_range;
    a.offsets = nullptr;
    a.nseg = 1;
    a.s = p->rs;
    p->dbg_skip_range = -1;
    p->dbg_spin_limit = 0;
    const cudaError_t e = launch_range_reversed(p->dtype, cmp == APSEP_LE ? 1 : 0, a, mi, mo, (cudaStream_t)stream);
    return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
}

apsep_status plan_run_out64(apsep_plan* p, const void* d_in, int64_t* d_out, int64_t n, int64_t out_base,
                            apsep_cmp cmp, void* chunk_min, void* stream, RangeArgs* layout) {
    if (!p || !layout || n <= 0 || n > p->capacity || !d_in || !d_out || (cmp != APSEP_LT && cmp != APSEP_LE))
        return APSEP_EINVAL;
    const int kb = key_bytes(p->dtype);
    if ((uintptr_t)d_in % kb != 0 || (uintptr_t)d_out % 8 != 0 || (chunk_min && (uintptr_t)chunk_min % kb != 0))
        return APSEP_EINVAL;
    DeviceGuard g(p->device);
    if (!g.ok) return APSEP_ECUDA;
    const int B = wide(p->dtype) ? kWideTileKeys : 32 * kTileConfigs[0].ipt;  // keys per warp tile
    const int tile_rows = B * kb / 128;                                         // 128-byte rows per tile
    int rows = (int)(n * kb / 128);
    CUtensorMap mi;
    memset(&mi, 0, sizeof(mi));
    if ((uintptr_t)d_in % 16 != 0 || rows < tile_rows) rows = 0;
    if (rows > 0 && !encode_rows(&mi, d_in, rows, tile_rows, p->dtype)) return APSEP_ECUDA;
    RangeArgs a;
    a.d_in = d_in;
    a.d_out = nullptr;
    a.n = (int)n;
    a.head = 0;
    a.num_tiles = (int)((n + B - 1) / B);
    a.tiles_per_range = 0;
    a.num_ranges = 0;
    a.tma_rows = rows;
    a.spin_limit = p->dbg_spin_limit ? p->dbg_spin_limit : kDefaultSpinLimit;
    a.skip_publish_range = p->dbg_skip_range;
    a.offsets = nullptr;
    a.nseg = 1;
    a.s = p->rs;
    if (chunk_min) a.s.chunk_min = chunk_min;
    a.d_out64 = d_out;
    a.out_base = out_base;
    p->dbg_skip_range = -1;
    p->dbg_spin_limit = 0;
    const cudaError_t e = launch_range_out64(p->dtype, cmp == APSEP_LE ? 1 : 0, a, mi, (cudaStream_t)stream);
    *layout = a;
    return e == cudaSuccess ? APSEP_OK : APSEP_ECUDA;
}

extern "C" {

apsep_status apsep_run_cmp(apsep_plan* p, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                           void* stream) {
    return run_impl(p, d_in, d_out, n, cmp, nullptr, 0, stream);
}

apsep_status apsep_run_segmented(apsep_plan* p, const void* d_in, int32_t* d_out, int64_t n,
                                 const int64_t* d_offsets, int32_t nseg, void* stream) {
    if (!p || !d_offsets) return APSEP_EINVAL;
    return run_impl(p, d_in, d_out, n, (apsep_cmp)p->cmp, d_offsets, nseg, stream);
}

apsep_status apsep_run(apsep_plan* p, const void* d_in, int32_t* d_out, int64_t n, void* stream) {
    if (!p) return APSEP_EINVAL;
    return apsep_run_cmp(p, d_in, d_out, n, (apsep_cmp)p->cmp, stream);
}

apsep_status apsep_plan_check(apsep_plan* p, void* stream) {
    if (!p) return APSEP_EINVAL;
    DeviceGuard g(p->device);
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return APSEP_ECUDA;
    uint32_t err = 0;
    if (cudaMemcpy(&err, &p->rs.ctr->err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return APSEP_ECUDA;
    if (!err) return APSEP_OK;
    // A run that gave up may have left counters half-way: re-arm the control
    // region (counters, group counters) keeping the epoch.
    Counters c0;
    if (cudaMemcpy(&c0, p->rs.ctr, sizeof(c0), cudaMemcpyDeviceToHost) != cudaSuccess) return APSEP_ECUDA;
    const uint32_t epoch = c0.epoch;
    memset(&c0, 0, sizeof(c0));
    c0.epoch = epoch;
    if (cudaMemset(p->scratch, 0, control_bytes()) != cudaSuccess ||
        cudaMemcpy(p->rs.ctr, &c0, sizeof(c0), cudaMemcpyHostToDevice) != cudaSuccess)
        return APSEP_ECUDA;
    if (err & ERR_BAD_OFFSETS) return APSEP_EINVAL;
    if (err & (ERR_LOOKBACK_TIMEOUT | ERR_TMA_TIMEOUT)) return APSEP_ETIMEOUT;
    return APSEP_EINTERNAL;
}

apsep_status apsep_plan_error_async(apsep_plan* p, uint32_t* host_word, void* stream) {
    if (!p || !host_word) return APSEP_EINVAL;
    DeviceGuard g(p->device);
    if (!g.ok) return APSEP_ECUDA;
    return cudaMemcpyAsync(host_word, &p->rs.ctr->err, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           (cudaStream_t)stream) == cudaSuccess
               ? APSEP_OK
               : APSEP_ECUDA;
}

apsep_status apsep_launch(const void* d_in, int32_t* d_out, int64_t n, apsep_dtype dtype, apsep_cmp cmp) {
    if (n == 0) return APSEP_OK;
    apsep_plan* p = nullptr;
    apsep_status s = apsep_plan_create(&p, dtype, cmp, n);
    if (s != APSEP_OK) return s;
    s = apsep_run(p, d_in, d_out, n, nullptr);
    apsep_status c = apsep_plan_check(p, nullptr);
    apsep_plan_destroy(p);
    return s != APSEP_OK ? s : c;
}

apsep_status apsep_debug_inject(apsep_plan* p, int32_t range, uint32_t spin_limit) {
    if (range < -1) return APSEP_EINVAL;
    if (!p) {  // the next apsep_run_noalloc call
        noalloc_debug_inject(range, spin_limit);
        return APSEP_OK;
    }
    p->dbg_skip_range = range;
    p->dbg_spin_limit = spin_limit;
    return APSEP_OK;
}

}  // extern "C"
