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
//
// Also the reference's generic multi-kernel path, WSTL (strict comparator,
// src/apsep.cuh:2296-2500, driven by runWSTL, src/apsep.cuh:2548-2596): its
// four kernels for int32 and float32 keys, the reference's own GPU oracle for
// float keys.
#include "apsep.cuh"

template __global__ void apsepKernelSPT<int, 128, 4, false>(const int*, int*, int, int, int, int, unsigned*, int*,
                                                            int*, int*, int*);
template __global__ void apsepKernelSPT<int, 128, 4, true>(const int*, int*, int, int, int, int, unsigned*, int*,
                                                           int*, int*, int*);

#define APSEP_REF_WSTL(T)                                                                                      \
    template __global__ void wstlPass1Kernel<T, 128, 4>(const T*, int*, int, int, T*, T*, T*);                \
    template __global__ void wstlFillLeavesKernel<T>(const T*, T*, int, int, int);                            \
    template __global__ void wstlReduceLevelKernel<T>(T*, int, int);                                          \
    template __global__ void wstlPass3Kernel<T, 128, 4>(const T*, int*, int, int, const T*, const T*, const T*, \
                                                        const T*, int);
APSEP_REF_WSTL(int)
APSEP_REF_WSTL(float)
