// apsep_main.cu -- correctness + benchmark harness in the reference's style,
// written against the drop-in shim (include/apsep.cuh) exactly as code using
// CoderDue/APSEP's src/apsep.cuh would be.  TEST INFRASTRUCTURE: it links the
// CPU oracle (oracle/apsep_oracle.c) to verify every answer.
//
// Same checks as the reference harnesses:
//   * structured small cases            (src/main.cu:181-222)
//   * random stress, std::mt19937 seeds  (src/main.cu:145-175, 246-252)
//   * SPT "<" and "<=" cases on poisoned outputs (src/bench_spt_le.cu:65-127)
// then a benchmark table at N = 2^25 (random / descending / ascending) and an
// N sweep, timed like src/main.cu:125-142 (median of events around runSPT).
//
//   apsep_main [--quick]      --quick: correctness only, smaller stress
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "apsep.cuh"

extern "C" int oracle_apse_i32(const int32_t* a, int64_t n, int le, int32_t* out);
extern "C" int oracle_gen_spt_le_case(int which, int64_t full_n, int64_t n, int32_t* out);
extern "C" int oracle_apse_i64(const int64_t* a, int64_t n, int le, int32_t* out);
extern "C" int oracle_apse_f64(const double* a, int64_t n, int le, int32_t* out);

// 8-byte keys through the same names: launchSPT<long long> / <double>.
static bool wideKeys() {
    std::mt19937_64 rng(64);
    bool ok = true;
    for (int n : {1, 511, 100003}) {
        std::vector<long long> a(n);
        std::vector<double> b(n);
        for (int i = 0; i < n; i++) {
            a[i] = (long long)rng();
            b[i] = (double)(long long)(rng() % 1000) * 1e-300;
        }
        std::vector<int> ra(n), rb(n), ga(n), gb(n);
        oracle_apse_i64((const int64_t*)a.data(), n, 0, ra.data());
        oracle_apse_f64(b.data(), n, 0, rb.data());
        long long* da;
        double* db;
        int* dout;
        gpuAssert(cudaMalloc(&da, n * sizeof(long long)));
        gpuAssert(cudaMalloc(&db, n * sizeof(double)));
        gpuAssert(cudaMalloc(&dout, n * sizeof(int)));
        gpuAssert(cudaMemcpy(da, a.data(), n * sizeof(long long), cudaMemcpyHostToDevice));
        gpuAssert(cudaMemcpy(db, b.data(), n * sizeof(double), cudaMemcpyHostToDevice));
        launchSPT<long long>(da, dout, n);
        gpuAssert(cudaMemcpy(ga.data(), dout, n * sizeof(int), cudaMemcpyDeviceToHost));
        launchSPT<double>(db, dout, n);
        gpuAssert(cudaMemcpy(gb.data(), dout, n * sizeof(int), cudaMemcpyDeviceToHost));
        gpuAssert(cudaFree(da));
        gpuAssert(cudaFree(db));
        gpuAssert(cudaFree(dout));
        ok = ok && ga == ra && gb == rb;
    }
    printf("  8-byte keys (long long, double): %s\n", ok ? "PASSED" : "FAILED");
    return ok;
}

static std::vector<int> cpuRef(const std::vector<int>& a, bool le = false) {
    std::vector<int> r(a.size());
    oracle_apse_i32(a.data(), (int64_t)a.size(), le ? 1 : 0, r.data());
    return r;
}

template <typename Launch>
static bool checkOne(Launch launch, const std::vector<int>& h, const char* name, const char* label) {
    int n = (int)h.size();
    int *d_in, *d_out;
    gpuAssert(cudaMalloc(&d_in, n * sizeof(int)));
    gpuAssert(cudaMalloc(&d_out, n * sizeof(int)));
    gpuAssert(cudaMemcpy(d_in, h.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    gpuAssert(cudaMemset(d_out, 0xAB, n * sizeof(int)));
    launch(d_in, d_out, n);
    gpuAssert(cudaDeviceSynchronize());
    std::vector<int> got(n);
    gpuAssert(cudaMemcpy(got.data(), d_out, n * sizeof(int), cudaMemcpyDeviceToHost));
    cudaFree(d_in);
    cudaFree(d_out);
    auto exp = cpuRef(h);
    for (int i = 0; i < n; i++)
        if (got[i] != exp[i]) {
            printf("  [%s] %-24s FAIL n=%d i=%d val=%d got=%d exp=%d\n", name, label, n, i, h[i], got[i], exp[i]);
            return false;
        }
    return true;
}

template <typename Launch>
static bool smallCases(Launch launch, const char* name) {
    const int B = 512;
    std::vector<std::pair<const char*, std::vector<int>>> cases = {
        {"single element", {42}},
        {"two ascending", {1, 2}},
        {"two descending", {2, 1}},
        {"all equal", {5, 5, 5, 5, 5}},
        {"ascending", {1, 2, 3, 4, 5, 6, 7, 8}},
        {"descending", {8, 7, 6, 5, 4, 3, 2, 1}},
        {"alternating", {3, 1, 4, 1, 5, 9, 2, 6}},
        {"exact block (B=512)", std::vector<int>(B)},
        {"two full blocks", std::vector<int>(2 * B)},
        {"non-power-of-two", std::vector<int>(B + 13)},
    };
    std::iota(cases[7].second.begin(), cases[7].second.end(), 0);
    for (int i = 0; i < 2 * B; i++) cases[8].second[i] = (i % 7) * 13;
    for (int i = 0; i < B + 13; i++) cases[9].second[i] = i % 17;
    bool ok = true;
    for (auto& c : cases) {
        bool r = checkOne(launch, c.second, name, c.first);
        printf("  [%s] %-24s %s\n", name, c.first, r ? "PASS" : "FAIL");
        ok = ok && r;
    }
    return ok;
}

template <typename Launch>
static bool stress(Launch launch, const char* name, int trials, int maxN, unsigned seed) {
    std::mt19937 rng(seed);
    for (int t = 0; t < trials; t++) {
        int n = 1 + (int)(rng() % (unsigned)maxN);
        std::vector<int> h(n);
        for (auto& v : h) v = (int)(rng() % 1000000u);
        if (!checkOne(launch, h, name, "stress")) return false;
    }
    return true;
}

static bool sptLeCases() {
    const int FULL = 32 * 1024 * 1024;
    const int sizes[] = {1000003, 513, 512, 511, 1};
    const char* names[] = {"random", "dup16", "dup2", "all-equal", "descending", "ascending", "intmax"};
    std::vector<int> h(1000003), ref(1000003), got(1000003);
    int *d_in, *d_out;
    gpuAssert(cudaMalloc(&d_in, 1000003 * sizeof(int)));
    gpuAssert(cudaMalloc(&d_out, 1000003 * sizeof(int)));
    auto s_lt = allocSPTScratch<int, 128, 4, false>(1000003);
    auto s_le = allocSPTScratch<int, 128, 4, true>(1000003);
    bool ok = true;
    for (int c = 0; c < 7; c++) {
        oracle_gen_spt_le_case(c, FULL, 1000003, h.data());
        gpuAssert(cudaMemcpy(d_in, h.data(), 1000003 * sizeof(int), cudaMemcpyHostToDevice));
        for (int n : sizes)
            for (int le = 0; le < 2; le++) {
                gpuAssert(cudaMemset(d_out, 0xAB, (size_t)n * sizeof(int)));
                if (le) runSPT<int, 128, 4, true>(d_in, d_out, n, s_le);
                else runSPT<int, 128, 4, false>(d_in, d_out, n, s_lt);
                gpuAssert(cudaDeviceSynchronize());
                gpuAssert(cudaMemcpy(got.data(), d_out, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost));
                oracle_apse_i32(h.data(), n, le, ref.data());
                int bad = -1;
                for (int i = 0; i < n && bad < 0; i++)
                    if (ref[i] != got[i]) bad = i;
                printf("  [%-2s %-10s n=%8d] %s\n", le ? "<=" : "<", names[c], n, bad < 0 ? "PASS" : "MISMATCH");
                ok = ok && bad < 0;
            }
    }
    freeSPTScratch<int, 128, 4>(s_lt);
    freeSPTScratch<int, 128, 4>(s_le);
    cudaFree(d_in);
    cudaFree(d_out);
    return ok;
}

template <typename Fn>
static double medianMs(Fn fn, int warmup, int iters) {
    for (int i = 0; i < warmup; i++) {
        fn();
        gpuAssert(cudaDeviceSynchronize());
    }
    cudaEvent_t t0, t1;
    gpuAssert(cudaEventCreate(&t0));
    gpuAssert(cudaEventCreate(&t1));
    std::vector<float> ms(iters);
    for (int i = 0; i < iters; i++) {
        gpuAssert(cudaEventRecord(t0));
        fn();
        gpuAssert(cudaEventRecord(t1));
        gpuAssert(cudaEventSynchronize(t1));
        gpuAssert(cudaEventElapsedTime(&ms[i], t0, t1));
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    std::sort(ms.begin(), ms.end());
    return ms[iters / 2];
}

static void benchmark() {
    const int N = 32 * 1024 * 1024;
    std::vector<int> h(N);
    int *d_in, *d_out;
    gpuAssert(cudaMalloc(&d_in, (size_t)N * sizeof(int)));
    gpuAssert(cudaMalloc(&d_out, (size_t)N * sizeof(int)));
    auto s = allocSPTScratch<int>(N);
    printf("\n=== Benchmark N=%d (useful GB/s = 2*N*4 B / median time) ===\n", N);
    const char* labels[] = {"random", "descending", "ascending"};
    std::mt19937_64 rng(20250325);
    for (int c = 0; c < 3; c++) {
        for (int i = 0; i < N; i++) h[i] = c == 0 ? (int)(rng() >> 33) : c == 1 ? N - 1 - i : i;
        gpuAssert(cudaMemcpy(d_in, h.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice));
        double ms = medianMs([&] { runSPT<int>(d_in, d_out, N, s); }, 2, 9);
        printf("  %-11s %8.1f us  %8.1f GB/s\n", labels[c], ms * 1e3, 2.0 * N * 4 / (ms * 1e-3) / 1e9);
    }
    printf("\n=== N sweep (random / descending) ===\n");
    for (int lg = 14; lg <= 25; lg += 1) {
        int n = 1 << lg;
        double r[2];
        for (int c = 0; c < 2; c++) {
            for (int i = 0; i < n; i++) h[i] = c == 0 ? (int)(rng() >> 33) : n - 1 - i;
            gpuAssert(cudaMemcpy(d_in, h.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice));
            double ms = medianMs([&] { runSPT<int>(d_in, d_out, n, s); }, 2, 7);
            r[c] = 2.0 * n * 4 / (ms * 1e-3) / 1e9;
        }
        printf("  2^%-2d %10d  %9.1f  %9.1f\n", lg, n, r[0], r[1]);
    }
    freeSPTScratch<int>(s);
    cudaFree(d_in);
    cudaFree(d_out);
}

int main(int argc, char** argv) {
    bool quick = argc > 1 && strcmp(argv[1], "--quick") == 0;
    cudaDeviceProp prop;
    gpuAssert(cudaGetDeviceProperties(&prop, 0));
    printf("Device: %s  (SM %d.%d, %d SMs)\n\n", prop.name, prop.major, prop.minor, prop.multiProcessorCount);
    auto spt = [](int* di, int* dout, int n) { launchSPT<int, 128, 4>(di, dout, n); };
    auto wstl = [](int* di, int* dout, int n) { launchWSTL<int, 128, 4>(di, dout, n); };
    printf("=== Correctness ===\n");
    bool ok_w = smallCases(wstl, "WSTL");
    bool ok_s = smallCases(spt, "SPT");
    int t1 = quick ? 100 : 500, t2 = quick ? 20 : 200;
    ok_w = ok_w && stress(wstl, "WSTL", t1, 4096, 42);
    ok_s = ok_s && stress(spt, "SPT", t1, 4096, 43);
    ok_w = ok_w && stress(wstl, "WSTL", t2, 131072, 100);
    ok_s = ok_s && stress(spt, "SPT", t2, 131072, 101);
    printf("  stress WSTL: %s  SPT: %s\n", ok_w ? "PASSED" : "FAILED", ok_s ? "PASSED" : "FAILED");
    bool ok_le = sptLeCases();
    bool ok_wide = wideKeys();
    bool ok = ok_w && ok_s && ok_le && ok_wide;
    printf("%s\n", ok ? "ALL PASSED" : "CORRECTNESS FAILED");
    if (!ok) return 1;
    if (!quick) benchmark();
    return 0;
}
