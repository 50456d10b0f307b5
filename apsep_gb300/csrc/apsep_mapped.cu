// apsep_mapped.cu -- the range engine in the forms the consumers ask for:
//   * the order-reversing key map: keys are flipped as they enter shared
//     memory or registers (integers ~x, floats -x), so one run of the
//     previous-smaller engine over the unchanged input answers previous
//     greater (or greater-or-equal under <=), and with the span output form
//     it writes the stock span (position - previous strictly greater);
//   * the reversed array: tiles counted from the end and reversed as they
//     land, answers mirrored as they leave, so one run answers next smaller
//     (or smaller-or-equal).
// Single arrays on a 16-byte boundary (keys and answers), 4-byte keys,
// configuration 0 (16 warps per CTA, 512-key warp tiles).
#include "apsep_range_kernel.cuh"

namespace apsep {

namespace {
constexpr int kMaxDevM = 64;
int g_warps_m[kMaxDevM];  // resident warps per device

template <typename T>
cudaError_t prep(int* per_sm) {
    cudaError_t rr[5] = {prepare_t<T, 16, 16, false, false, true, KMAP_FLIP, OUT_I32>(per_sm),
                         prepare_t<T, 16, 16, true, false, true, KMAP_FLIP, OUT_I32>(per_sm),
                         prepare_t<T, 16, 16, false, false, true, KMAP_FLIP, OUT_SPAN>(per_sm),
                         prepare_t<T, 16, 16, false, false, true, KMAP_NONE, OUT_I32, true>(per_sm),
                         prepare_t<T, 16, 16, true, false, true, KMAP_NONE, OUT_I32, true>(per_sm)};
    for (int q = 0; q < 5; q++)
        if (rr[q] != cudaSuccess) return rr[q];
    return cudaSuccess;
}

cudaError_t warps_for(int* warps) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevM) return cudaErrorInvalidValue;
    if (!g_warps_m[dev]) {
        int per_sm = 0, sms = 0;
        if ((e = prep<int32_t>(&per_sm)) != cudaSuccess) return e;
        if ((e = prep<float>(&per_sm)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        const int w = per_sm * sms * 16;
        g_warps_m[dev] = w > kMaxRanges ? kMaxRanges : w;
    }
    *warps = g_warps_m[dev];
    return cudaSuccess;
}
}  // namespace

cudaError_t launch_range_flipped(int dtype, int incl, int span, RangeArgs& a, const CUtensorMap& mi,
                                 const CUtensorMap& mo, cudaStream_t st) {
    int max_warps = 0;
    const cudaError_t e = warps_for(&max_warps);
    if (e != cudaSuccess) return e;
    if (a.head != 0 || dtype > 1 || (span && incl)) return cudaErrorInvalidValue;
    a.offsets = nullptr;
    a.nseg = 1;
    if (span)
        return dtype == 0 ? launch_t<int32_t, 16, 16, false, false, true, KMAP_FLIP, OUT_SPAN>(a, mi, mo, st, max_warps)
                          : launch_t<float, 16, 16, false, false, true, KMAP_FLIP, OUT_SPAN>(a, mi, mo, st, max_warps);
    if (dtype == 0)
        return incl ? launch_t<int32_t, 16, 16, true, false, true, KMAP_FLIP, OUT_I32>(a, mi, mo, st, max_warps)
                    : launch_t<int32_t, 16, 16, false, false, true, KMAP_FLIP, OUT_I32>(a, mi, mo, st, max_warps);
    return incl ? launch_t<float, 16, 16, true, false, true, KMAP_FLIP, OUT_I32>(a, mi, mo, st, max_warps)
                : launch_t<float, 16, 16, false, false, true, KMAP_FLIP, OUT_I32>(a, mi, mo, st, max_warps);
}

cudaError_t launch_range_reversed(int dtype, int incl, RangeArgs& a, const CUtensorMap& mi, const CUtensorMap& mo,
                                  cudaStream_t st) {
    int max_warps = 0;
    const cudaError_t e = warps_for(&max_warps);
    if (e != cudaSuccess) return e;
    if (a.head != 0 || dtype > 1 || (a.tma_rows > 0 && (int64_t)a.tma_rows * 32 != (int64_t)a.n))
        return cudaErrorInvalidValue;
    a.offsets = nullptr;
    a.nseg = 1;
    if (dtype == 0)
        return incl ? launch_t<int32_t, 16, 16, true, false, true, KMAP_NONE, OUT_I32, true>(a, mi, mo, st, max_warps)
                    : launch_t<int32_t, 16, 16, false, false, true, KMAP_NONE, OUT_I32, true>(a, mi, mo, st, max_warps);
    return incl ? launch_t<float, 16, 16, true, false, true, KMAP_NONE, OUT_I32, true>(a, mi, mo, st, max_warps)
                : launch_t<float, 16, 16, false, false, true, KMAP_NONE, OUT_I32, true>(a, mi, mo, st, max_warps);
}

}  // namespace apsep
