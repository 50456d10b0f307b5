// ref_cpu_wrap.cu -- TEST INFRASTRUCTURE ONLY (oracle pinning).
//
// Compiles the reference's OWN sequential CPU oracles, unmodified, straight
// from the reference sources, and exports them with a C ABI so the tests can
// pin the oracle restatement (apsep_oracle.c) against them:
//   cpuApsep  src/main.cu:102-113           -> ref_cpu_apsep
//   cpuPSE    src/bench_spt_le.cu:24-35     -> ref_cpu_pse
// Also exports the reference harnesses' own input generators re-expressed as
// plain functions over the same PRNGs (std::mt19937 as in main.cu:145-175,
// glibc srand/rand as in bench_spt_le.cu:93-127), so golden inputs are the
// exact inputs the reference tests use.
//
// Built by oracle/build_ref.py with include path <reference>/src; the output
// goes to oracle/_ref/ only.  The reference's main() functions are renamed by
// the preprocessor and never called.  main.cu reads
// cudaDeviceProp::memoryClockRate, a field CUDA 13 removed; the recipe maps
// that one name onto an existing int field at compile time so the file
// compiles as shipped (that code path is never executed here).

#include <cstring>
#include <random>
#include <vector>
#include <cstdlib>

#define main apsep_reference_main_cu_unused
#include "main.cu"
#undef main

#define main apsep_reference_bench_spt_le_unused
#include "bench_spt_le.cu"
#undef main

extern "C" {

int ref_cpu_apsep(const int* a, int n, int* out) {
    std::vector<int> v(a, a + n);
    std::vector<int> r = cpuApsep(v);
    std::memcpy(out, r.data(), (size_t)n * sizeof(int));
    return 0;
}

int ref_cpu_pse(const int* a, int n, int le, int* out) {
    std::vector<int> v(a, a + n), r(n);
    cpuPSE(v, n, le != 0, r);
    std::memcpy(out, r.data(), (size_t)n * sizeof(int));
    return 0;
}

// Raw std::mt19937 stream (the generator main.cu's stressKernel draws from).
void ref_mt19937_raw(unsigned seed, unsigned* out, long long count) {
    std::mt19937 rng(seed);
    for (long long i = 0; i < count; i++) out[i] = (unsigned)rng();
}

// glibc srand/rand stream (the generator bench_spt_le.cu's cases draw from).
void ref_glibc_rand(unsigned seed, int* out, long long count) {
    srand(seed);
    for (long long i = 0; i < count; i++) out[i] = rand();
}

}  // extern "C"
