// apsep_out64.cu -- the range engine with int64 answers, for the
// int64-position path (apsep_run64): single arrays on a 16-byte boundary,
// 4-byte keys in configuration 0 (16 warps per CTA, 512-key warp tiles),
// 8-byte keys in their one configuration (8 warps per CTA, 256-key tiles).
// Each piece of a long array writes out_base + answer straight into the
// int64 output, so no int32 scratch is written and read back; keys the piece
// leaves unanswered are marked (UNRESOLVED64, or a tile flagged as not
// stored) for the int64-position path's fix-up.
#include "apsep_range_kernel.cuh"

namespace apsep {

namespace {
constexpr int kMaxDevO = 64;
int g_warps64[kMaxDevO][2];  // resident warps per device: [0] 4-byte keys, [1] 8-byte keys

template <typename T, int IPT, int WPC, int KMAP>
cudaError_t prep(int* per_sm) {
    cudaError_t rr[2] = {prepare_t<T, IPT, WPC, false, false, true, KMAP, OUT_I64>(per_sm),
                         prepare_t<T, IPT, WPC, true, false, true, KMAP, OUT_I64>(per_sm)};
    return rr[0] != cudaSuccess ? rr[0] : rr[1];
}

cudaError_t warps_for(int wide, int* warps) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevO) return cudaErrorInvalidValue;
    if (!g_warps64[dev][wide]) {
        int per_sm = 0;
        if (wide) {
            if ((e = prep<int64_t, 8, 8, KMAP_NONE>(&per_sm)) != cudaSuccess) return e;
            if ((e = prep<int64_t, 8, 8, KMAP_F64>(&per_sm)) != cudaSuccess) return e;
        } else {
            if ((e = prep<int32_t, 16, 16, KMAP_NONE>(&per_sm)) != cudaSuccess) return e;
            if ((e = prep<float, 16, 16, KMAP_NONE>(&per_sm)) != cudaSuccess) return e;
        }
        int sms = 0;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        int w = per_sm * sms * (wide ? 8 : 16);
        g_warps64[dev][wide] = w > kMaxRanges ? kMaxRanges : w;
    }
    *warps = g_warps64[dev][wide];
    return cudaSuccess;
}
}  // namespace

cudaError_t launch_range_out64(int dtype, int incl, RangeArgs& a, const CUtensorMap& mi, cudaStream_t st) {
    const int wide = dtype >= 2;
    int max_warps = 0;
    const cudaError_t e = warps_for(wide, &max_warps);
    if (e != cudaSuccess) return e;
    if (a.head != 0 || !a.d_out64) return cudaErrorInvalidValue;
    a.offsets = nullptr;
    a.nseg = 1;
    const CUtensorMap& mo = mi;  // (no tensor store: answers leave as int64 from registers)
    switch (dtype) {
    case 0:
        return incl ? launch_t<int32_t, 16, 16, true, false, true, KMAP_NONE, OUT_I64>(a, mi, mo, st, max_warps)
                    : launch_t<int32_t, 16, 16, false, false, true, KMAP_NONE, OUT_I64>(a, mi, mo, st, max_warps);
    case 1:
        return incl ? launch_t<float, 16, 16, true, false, true, KMAP_NONE, OUT_I64>(a, mi, mo, st, max_warps)
                    : launch_t<float, 16, 16, false, false, true, KMAP_NONE, OUT_I64>(a, mi, mo, st, max_warps);
    case 2:
        return incl ? launch_t<int64_t, 8, 8, true, false, true, KMAP_NONE, OUT_I64>(a, mi, mo, st, max_warps)
                    : launch_t<int64_t, 8, 8, false, false, true, KMAP_NONE, OUT_I64>(a, mi, mo, st, max_warps);
    default:  // float64 keys compare as their order-preserving int64 map
        return incl ? launch_t<int64_t, 8, 8, true, false, true, KMAP_F64, OUT_I64>(a, mi, mo, st, max_warps)
                    : launch_t<int64_t, 8, 8, false, false, true, KMAP_F64, OUT_I64>(a, mi, mo, st, max_warps);
    }
}

}  // namespace apsep
