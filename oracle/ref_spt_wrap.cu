// ref_spt_wrap.cu -- TEST INFRASTRUCTURE ONLY (a second parity leg).
//
// Instantiates the reference's own single-pass GPU kernel, unmodified:
// apsepKernelSPT (src/apsep.cuh:2634-2998, launched by runSPT,
// src/apsep.cuh:3052-3067) for int32 keys in its default shape
// <int, BLOCK_SIZE = 128, IPT = 4>, with both comparators (INCL false / true,
// src/apsep.cuh:2669-2673).  oracle/build_ref.py compiles this file with the
// reference's src/ on the include path into device code only (PTX for
// compute_103a, written to oracle/_ref/); tests/test_gpu_ref_kernel.py loads
// that module through the CUDA driver API and launches the kernel the way
// runSPT does: one cooperative launch of occupancy x SM-count blocks of 128
// threads over the five scratch arrays of allocSPTScratch
// (src/apsep.cuh:3014-3040).  Its float path converts keys by value
// (src/apsep.cuh:2689-2690), so only int32 keys are instantiated.
#include "apsep.cuh"

template __global__ void apsepKernelSPT<int, 128, 4, false>(const int*, int*, int, int, int, int, unsigned*, int*,
                                                            int*, int*, int*);
template __global__ void apsepKernelSPT<int, 128, 4, true>(const int*, int*, int, int, int, int, unsigned*, int*,
                                                           int*, int*, int*);
