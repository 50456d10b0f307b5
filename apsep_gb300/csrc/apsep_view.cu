// apsep_view.cu -- single arrays off a 16-byte boundary.
//
// A single array whose keys and answers sit at the same offset within 16
// bytes streams through a TMA view that starts 1-3 virtual keys before it
// (RangeArgs::head).  That view needs the segmented kernel's machinery (an
// answer relative to a start, plain loads and stores for tile 0), with one
// implicit segment and the single-array kernel's whole-tile early paths: a
// third instantiation of the range engine, so neither of the other two pays
// for it.
#include "apsep_range_kernel.cuh"

namespace apsep {

cudaError_t prepare_view(int cfg, int* ctas_per_sm) { return prepare_mode<true, true>(cfg, ctas_per_sm); }

cudaError_t launch_range_view(int dtype, int incl, int cfg, RangeArgs& a, const CUtensorMap& mi,
                              const CUtensorMap& mo, cudaStream_t st) {
    int max_warps = 0;
    const cudaError_t e = range_max_warps(cfg, &max_warps);
    if (e != cudaSuccess) return e;
    a.offsets = nullptr;  // one segment: [0, n)
    a.nseg = 1;
    return launch_mode<true, true>(dtype, incl, cfg, a, mi, mo, st, max_warps);
}

}  // namespace apsep
