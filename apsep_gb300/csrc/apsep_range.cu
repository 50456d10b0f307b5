// apsep_range.cu -- host side of the range engine: scratch layout, occupancy,
// launches of the single-array kernels (the kernel itself is in
// apsep_range_kernel.cuh; the segmented instantiations are in
// apsep_segmented.cu).
#include "apsep_range_kernel.cuh"

namespace apsep {

const TileConfig kTileConfigs[kNumTileConfigs] = {
    {16, 16},  // 16 warps per CTA (one CTA per SM), 512-key warp tiles
    {8, 8},    // 8 warps per CTA, 256-key warp tiles
    {8, 16},   // 8 warps per CTA, 512-key warp tiles
    {16, 8},   // 16 warps per CTA, 256-key warp tiles
    {4, 16},   // 4 warps per CTA: a small array spreads over more SMs
    {4, 8},
};

size_t carve_scratch(void* base, int64_t capacity, RangeScratch* s, int kb) {
    const ScratchOffsets o = scratch_offsets(capacity, kb);
    if (base && s) {
        char* b = (char*)base;
        s->ctr = (Counters*)b;
        s->group_min = (uint64_t*)(b + o.gmin);
        s->cta_ready = (uint32_t*)(b + o.ready);
        s->range_state = (uint64_t*)(b + o.state);
        s->range_key = (uint64_t*)(b + o.rkey);
        s->top_key = b + o.topk;
        s->top_pos = (int32_t*)(b + o.topp);
        s->top_cnt = (uint32_t*)(b + o.topc);
        s->tile_min = b + o.tmin;
        s->chunk_min = b + o.cmin;
        s->tile_flag = (uint32_t*)(b + o.flag);
        s->tile_mask = (uint32_t*)(b + o.mask);
        s->cap_tiles = (int)o.cap_tiles;
        s->max_ranges = kMaxRanges;
    }
    return o.total;
}

namespace {
constexpr int kMaxDev = 64;
int g_warps[kMaxDev][kNumTileConfigs];  // resident warps per device and configuration
}

cudaError_t range_prepare(int cfg) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev || cfg < 0 || cfg >= kNumTileConfigs) return cudaErrorInvalidValue;
    int per_sm = 0;  // the smallest over the three modes, so every run fits
    e = prepare_mode<false, true>(cfg, &per_sm);
    if (e != cudaSuccess) return e;
    e = prepare_segmented(cfg, &per_sm);
    if (e != cudaSuccess) return e;
    e = prepare_view(cfg, &per_sm);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int warps = per_sm * sms * kTileConfigs[cfg].wpc;
    if (warps > kMaxRanges) warps = kMaxRanges;
    g_warps[dev][cfg] = warps;
    return cudaSuccess;
}

cudaError_t range_max_warps(int cfg, int* warps) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev || cfg < 0 || cfg >= kNumTileConfigs) return cudaErrorInvalidValue;
    if (g_warps[dev][cfg] == 0) {
        e = range_prepare(cfg);
        if (e != cudaSuccess) return e;
    }
    *warps = g_warps[dev][cfg];
    return cudaSuccess;
}

cudaError_t launch_range(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo,
                         cudaStream_t st) {
    int max_warps = 0;
    const cudaError_t e = range_max_warps(cfg, &max_warps);
    if (e != cudaSuccess) return e;
    a.offsets = nullptr;
    a.nseg = 0;
    return launch_mode<false, true>(dtype, incl, cfg, a, mi, mo, st, max_warps);
}

}  // namespace apsep
