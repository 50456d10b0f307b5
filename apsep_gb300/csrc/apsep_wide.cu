// apsep_wide.cu -- the range engine for 8-byte keys (int64 / float64).
//
// The same kernel template with 8-byte keys: 8 keys per lane (256-key warp
// tiles, 12 KB of shared memory per warp), 8 warps per CTA, keys streamed as
// 128-byte TMA rows of 16 keys, answers as int32 positions (n < 2^31).
// Range minima sit beside their tag words (no 64-bit key fits beside a tag
// in one atomic word), and group minima are read from the ranges' words.
// float64 keys run as int64 through an order-preserving map of their bits
// (applied as keys enter shared memory or registers): the FP64 compare rate
// of this part would make every comparison the bottleneck.
// Single arrays and segmented batches; one configuration; no view head
// (arrays off a 16-byte boundary take plain loads and stores).
#include "apsep_range_kernel.cuh"

namespace apsep {

namespace {
constexpr int kWideIpt = 8;
constexpr int kWideWpc = 8;
constexpr int kMaxDevW = 64;
int g_wide_warps[kMaxDevW];  // resident warps per device
}  // namespace

cudaError_t prepare_wide() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevW) return cudaErrorInvalidValue;
    if (g_wide_warps[dev]) return cudaSuccess;
    int per_sm = 0;
    cudaError_t rr[8] = {prepare_t<int64_t, kWideIpt, kWideWpc, false, false, true>(&per_sm),
                         prepare_t<int64_t, kWideIpt, kWideWpc, true, false, true>(&per_sm),
                         prepare_t<int64_t, kWideIpt, kWideWpc, false, false, true, KMAP_F64>(&per_sm),
                         prepare_t<int64_t, kWideIpt, kWideWpc, true, false, true, KMAP_F64>(&per_sm),
                         prepare_t<int64_t, kWideIpt, kWideWpc, false, true, false>(&per_sm),
                         prepare_t<int64_t, kWideIpt, kWideWpc, true, true, false>(&per_sm),
                         prepare_t<int64_t, kWideIpt, kWideWpc, false, true, false, KMAP_F64>(&per_sm),
                         prepare_t<int64_t, kWideIpt, kWideWpc, true, true, false, KMAP_F64>(&per_sm)};
    for (int q = 0; q < 8; q++)
        if (rr[q] != cudaSuccess) return rr[q];
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int warps = per_sm * sms * kWideWpc;
    if (warps > kMaxRanges) warps = kMaxRanges;
    g_wide_warps[dev] = warps;
    return cudaSuccess;
}

cudaError_t launch_range_wide(int dtype, int incl, RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo,
                              cudaStream_t st) {
    cudaError_t e = prepare_wide();
    if (e != cudaSuccess) return e;
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    const int max_warps = g_wide_warps[dev];
    a.head = 0;
    if (a.offsets) {  // a segmented batch
        if (a.nseg < 1) return cudaErrorInvalidValue;
        if (dtype == 2)
            return incl ? launch_t<int64_t, kWideIpt, kWideWpc, true, true, false>(a, mi, mo, st, max_warps)
                        : launch_t<int64_t, kWideIpt, kWideWpc, false, true, false>(a, mi, mo, st, max_warps);
        return incl ? launch_t<int64_t, kWideIpt, kWideWpc, true, true, false, KMAP_F64>(a, mi, mo, st, max_warps)
                    : launch_t<int64_t, kWideIpt, kWideWpc, false, true, false, KMAP_F64>(a, mi, mo, st, max_warps);
    }
    a.nseg = 0;
    if (dtype == 2)
        return incl ? launch_t<int64_t, kWideIpt, kWideWpc, true, false, true>(a, mi, mo, st, max_warps)
                    : launch_t<int64_t, kWideIpt, kWideWpc, false, false, true>(a, mi, mo, st, max_warps);
    // float64: int64 slots compared through the order map (no FP64 compares)
    return incl ? launch_t<int64_t, kWideIpt, kWideWpc, true, false, true, KMAP_F64>(a, mi, mo, st, max_warps)
                : launch_t<int64_t, kWideIpt, kWideWpc, false, false, true, KMAP_F64>(a, mi, mo, st, max_warps);
}

}  // namespace apsep
