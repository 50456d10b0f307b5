// apsep_segmented.cu -- the segmented instantiations of the range engine.
//
// A batch of arrays stored back to back (segment s is d_in[off[s],
// off[s+1])) runs as one launch over the concatenation: every key's answer is
// the nearest earlier key that qualifies in the whole concatenation, turned
// relative to its own segment start -- and -1 when that key lies before the
// segment, since then nothing in the segment qualifies.  The kernel follows
// the segment starts tile by tile (apsep_range_kernel.cuh, step 0), converts
// the tile's answers before its store, and skips the cross-range search for
// any deferred key whose segment starts inside its own range.
#include "apsep_range_kernel.cuh"

namespace apsep {

cudaError_t prepare_segmented(int cfg, int* ctas_per_sm) { return prepare_mode<true, false>(cfg, ctas_per_sm); }

cudaError_t launch_range_segmented(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& mi,
                                   const CUtensorMap& mo, cudaStream_t st) {
    int max_warps = 0;
    const cudaError_t e = range_max_warps(cfg, &max_warps);
    if (e != cudaSuccess) return e;
    if (!a.offsets || a.nseg < 1) return cudaErrorInvalidValue;
    return launch_mode<true, false>(dtype, incl, cfg, a, mi, mo, st, max_warps);
}

}  // namespace apsep
