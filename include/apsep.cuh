// apsep.cuh -- drop-in C++ shim: the reference's host API on the GB300 engine.
//
// Code written against CoderDue/APSEP's src/apsep.cuh keeps compiling and
// behaving the same: include this header instead, link libapsep.so.
//
//   SPTScratch<T,BS,IPT>             src/apsep.cuh:3001-3012
//   allocSPTScratch<T,BS,IPT,INCL>   src/apsep.cuh:3014-3040
//   freeSPTScratch<T,BS,IPT>         src/apsep.cuh:3042-3050
//   runSPT<T,BS,IPT,INCL>            src/apsep.cuh:3052-3067
//   launchSPT<T,BS,IPT,INCL>         src/apsep.cuh:3069-3076
//   WSTLScratch / allocWSTLScratch / freeWSTLScratch / runWSTL / launchWSTL
//                                    src/apsep.cuh:2509-2605
//   gpuAssert                        src/apsep.cuh:39-47
//
// Same argument meaning: device pointers, int n, answers are global indices
// or -1, INCL selects "<=".  Same sync semantics: run* enqueue on the legacy
// default stream and return, launch* synchronise.  Same error behaviour by
// default: a failure prints "APSEP error ..." and exits like gpuAssert; define
// APSEP_SHIM_THROW before including to get a std::runtime_error instead.
// The BLOCK_SIZE / IPT template arguments are accepted for source
// compatibility; the engine's tile shape comes from its own configuration.
// Keys: int, float, long long and double (the reference's ApsepInfinity
// also lists unsigned, which the engine does not support: it fails to
// compile here).
#pragma once

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>

#include "apsep.h"

#ifdef APSEP_SHIM_THROW
#include <stdexcept>
#include <string>
#endif

#ifndef gpuAssert
#define gpuAssert(x) _gpuAssert((x), __FILE__, __LINE__)
static inline void _gpuAssert(cudaError_t code, const char* file, int line) {
    if (code != cudaSuccess) {
        fprintf(stderr, "CUDA error %s:%d: %s\n", file, line, cudaGetErrorString(code));
        exit(EXIT_FAILURE);
    }
}
#endif

namespace apsep_shim {

static inline void fail(apsep_status s, const char* what, const char* file, int line) {
#ifdef APSEP_SHIM_THROW
    throw std::runtime_error(std::string("APSEP error in ") + what + ": " + apsep_status_string(s));
#else
    fprintf(stderr, "APSEP error %s:%d: %s: %s\n", file, line, what, apsep_status_string(s));
    exit(EXIT_FAILURE);
#endif
}

template <typename T> struct Dtype;
template <> struct Dtype<int> { static constexpr apsep_dtype value = APSEP_INT32; };
template <> struct Dtype<float> { static constexpr apsep_dtype value = APSEP_FLOAT32; };
template <> struct Dtype<long long> { static constexpr apsep_dtype value = APSEP_INT64; };
template <> struct Dtype<double> { static constexpr apsep_dtype value = APSEP_FLOAT64; };

}  // namespace apsep_shim

#define APSEP_SHIM_CHECK(call)                                                   \
    do {                                                                         \
        apsep_status _s = (call);                                                \
        if (_s != APSEP_OK) apsep_shim::fail(_s, #call, __FILE__, __LINE__);     \
    } while (0)

// ---------------------------------------------------------------------------
// SPT names
// ---------------------------------------------------------------------------
template <typename T, int BLOCK_SIZE = 128, int IPT = 4>
struct SPTScratch {
    apsep_plan* plan = nullptr;
    int num_blocks = 0;   // tiles of the engine's configuration
    int M = 0;            // next power of two >= num_blocks (kept for source compatibility)
    int leaf_offset = 0;  // M - 1
    int num_phys = 0;     // CTAs one run launches (one per tile)
};

template <typename T, int BLOCK_SIZE = 128, int IPT = 4, bool INCL = false>
SPTScratch<T, BLOCK_SIZE, IPT> allocSPTScratch(int n) {
    SPTScratch<T, BLOCK_SIZE, IPT> s;
    APSEP_SHIM_CHECK(apsep_plan_create(&s.plan, apsep_shim::Dtype<T>::value, INCL ? APSEP_LE : APSEP_LT,
                                       n > 0 ? (int64_t)n : 1));
    apsep_plan_info info;
    APSEP_SHIM_CHECK(apsep_plan_get_info(s.plan, &info));
    s.num_blocks = n > 0 ? (int)((n + info.tile_keys - 1) / info.tile_keys) : 0;
    s.M = 1;
    while (s.M < s.num_blocks) s.M <<= 1;
    s.leaf_offset = s.M - 1;
    s.num_phys = s.num_blocks;
    return s;
}

template <typename T, int BLOCK_SIZE = 128, int IPT = 4>
void freeSPTScratch(SPTScratch<T, BLOCK_SIZE, IPT>& s) {
    apsep_plan_destroy(s.plan);
    s = SPTScratch<T, BLOCK_SIZE, IPT>{};
}

template <typename T, int BLOCK_SIZE = 128, int IPT = 4, bool INCL = false>
void runSPT(const T* d_in, int* d_out, int n, SPTScratch<T, BLOCK_SIZE, IPT>& s) {
    if (n <= 0) return;
    APSEP_SHIM_CHECK(apsep_run_cmp(s.plan, d_in, d_out, n, INCL ? APSEP_LE : APSEP_LT, nullptr));
}

template <typename T, int BLOCK_SIZE = 128, int IPT = 4, bool INCL = false>
void launchSPT(const T* d_in, int* d_out, int n) {
    if (n <= 0) return;
    auto s = allocSPTScratch<T, BLOCK_SIZE, IPT, INCL>(n);
    runSPT<T, BLOCK_SIZE, IPT, INCL>(d_in, d_out, n, s);
    gpuAssert(cudaDeviceSynchronize());
    APSEP_SHIM_CHECK(apsep_plan_check(s.plan, nullptr));
    freeSPTScratch<T, BLOCK_SIZE, IPT>(s);
}

// ---------------------------------------------------------------------------
// WSTL names: the same engine (one launch instead of 3 + log2 M).
// ---------------------------------------------------------------------------
template <typename T, int BLOCK_SIZE = 128, int IPT = 4>
struct WSTLScratch {
    apsep_plan* plan = nullptr;
    int num_blocks = 0;
    int M = 0;
    int leaf_offset = 0;
    int tree_size = 0;
};

template <typename T, int BLOCK_SIZE = 128, int IPT = 4>
WSTLScratch<T, BLOCK_SIZE, IPT> allocWSTLScratch(int n) {
    auto sp = allocSPTScratch<T, BLOCK_SIZE, IPT, false>(n);
    WSTLScratch<T, BLOCK_SIZE, IPT> s;
    s.plan = sp.plan;
    s.num_blocks = sp.num_blocks;
    s.M = sp.M;
    s.leaf_offset = sp.leaf_offset;
    s.tree_size = 2 * sp.M - 1;
    return s;
}

template <typename T, int BLOCK_SIZE = 128, int IPT = 4>
void freeWSTLScratch(WSTLScratch<T, BLOCK_SIZE, IPT>& s) {
    apsep_plan_destroy(s.plan);
    s = WSTLScratch<T, BLOCK_SIZE, IPT>{};
}

template <typename T, int BLOCK_SIZE = 128, int IPT = 4>
void runWSTL(const T* d_in, int* d_out, int n, WSTLScratch<T, BLOCK_SIZE, IPT>& s) {
    if (n <= 0) return;
    APSEP_SHIM_CHECK(apsep_run_cmp(s.plan, d_in, d_out, n, APSEP_LT, nullptr));
}

template <typename T, int BLOCK_SIZE = 128, int IPT = 4>
void launchWSTL(const T* d_in, int* d_out, int n) {
    if (n <= 0) return;
    auto s = allocWSTLScratch<T, BLOCK_SIZE, IPT>(n);
    runWSTL<T, BLOCK_SIZE, IPT>(d_in, d_out, n, s);
    gpuAssert(cudaDeviceSynchronize());
    APSEP_SHIM_CHECK(apsep_plan_check(s.plan, nullptr));
    freeWSTLScratch<T, BLOCK_SIZE, IPT>(s);
}
