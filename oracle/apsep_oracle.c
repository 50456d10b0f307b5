/*
 * apsep_oracle.c -- CPU ORACLE for the All Previous Smaller Element problem.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the apsep_gb300 package,
 * libapsep.so, the C ABI) links, loads or calls this file.  The tests and
 * __graft_entry__.smoke() compare the engine's answers with it, and bench.py
 * times it as the CPU baseline ("cpu_baseline", "--impl reference").
 *
 * It restates, in plain C, the reference's sequential monotone-stack oracles:
 *   - cpuApsep  (src/main.cu:102-113): strict "<", int only;
 *   - cpuPSE    (src/bench_spt_le.cu:24-35): "<" or "<=" ("le" flag), which
 *     pops while the stack top does NOT qualify as the answer.
 * Both are the same algorithm: scan left to right, keep a stack of indices
 * whose values are candidates, pop every top that does not qualify, the
 * surviving top (or -1) is the answer, push i.  cpuPSE's pop test
 * "!(a[top] < a[i])" equals cpuApsep's "a[top] >= a[i]" for integers and for
 * finite floats, so one routine covers both.
 *
 * Generic over the key type (int32, float32, int64, float64) through a macro, plus a
 * segmented form (answers relative to each segment's start, never crossing a
 * segment's left edge) for the batched API.
 *
 * Parity pin: tests/test_oracle.py checks these routines bit-exactly against
 * outputs of the reference's own cpuApsep / cpuPSE (compiled from the
 * reference sources by oracle/build_ref.py, fixtures in tests/golden/).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define APSE_BODY(T)                                                          \
    int32_t* stk = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t)); \
    if (!stk) return -1;                                                      \
    int64_t sp = 0;                                                           \
    for (int64_t i = 0; i < n; i++) {                                         \
        const T x = a[i];                                                     \
        if (le) {                                                             \
            while (sp > 0 && !(a[stk[sp - 1]] <= x)) sp--;                    \
        } else {                                                              \
            while (sp > 0 && !(a[stk[sp - 1]] < x)) sp--;                     \
        }                                                                     \
        out[i] = sp > 0 ? stk[sp - 1] : -1;                                   \
        stk[sp++] = (int32_t)i;                                               \
    }                                                                         \
    free(stk);                                                                \
    return 0;

/* out[i] = max{ j < i : a[j] < a[i] } (or <= when le != 0), else -1. */
int oracle_apse_i32(const int32_t* a, int64_t n, int le, int32_t* out) {
    if (n < 0 || n > INT32_MAX) return -2;
    APSE_BODY(int32_t)
}

int oracle_apse_f32(const float* a, int64_t n, int le, int32_t* out) {
    if (n < 0 || n > INT32_MAX) return -2;
    APSE_BODY(float)
}

/* 8-byte keys (the reference's ApsepInfinity<long long / double>,
 * src/apsep.cuh:62-70): the same stack, int32 positions. */
int oracle_apse_i64(const int64_t* a, int64_t n, int le, int32_t* out) {
    if (n < 0 || n > INT32_MAX) return -2;
    APSE_BODY(int64_t)
}

int oracle_apse_f64(const double* a, int64_t n, int le, int32_t* out) {
    if (n < 0 || n > INT32_MAX) return -2;
    APSE_BODY(double)
}

/* Segmented form: segment s covers [offsets[s], offsets[s+1]); each answer is
 * relative to the segment start and never looks left of it.  offsets has
 * nseg+1 entries, non-decreasing, offsets[0] == 0 is not required. */
#define SEG_BODY(FN, T)                                                       \
    for (int64_t s = 0; s < nseg; s++) {                                      \
        int64_t lo = offsets[s], hi = offsets[s + 1];                         \
        if (hi < lo) return -2;                                               \
        int rc = FN(a + lo, hi - lo, le, out + lo);                           \
        if (rc) return rc;                                                    \
    }                                                                         \
    return 0;

int oracle_apse_segmented_i32(const int32_t* a, const int64_t* offsets,
                              int64_t nseg, int le, int32_t* out) {
    SEG_BODY(oracle_apse_i32, int32_t)
}

int oracle_apse_segmented_f32(const float* a, const int64_t* offsets,
                              int64_t nseg, int le, int32_t* out) {
    SEG_BODY(oracle_apse_f32, float)
}

/*
 * Inputs of the reference's SPT "<" / "<=" correctness cases
 * (src/bench_spt_le.cu:93-127), regenerated with the same glibc srand/rand
 * draws so their outputs can be compared with golden hashes:
 *   0 random      srand(1234), rand()
 *   1 dup16       srand(99),   rand() % 16
 *   2 dup2        srand(7),    rand() % 2
 *   3 all-equal   42
 *   4 descending  N - i   (N = the full array length the harness fills)
 *   5 ascending   i
 *   6 intmax      srand(5), (rand() % 4 == 0) ? INT_MAX : rand()
 * The harness fills N = 2^25 values and checks prefixes of length n; this
 * writes the first n of them.  Returns 0, or -2 for an unknown case.
 */
int oracle_gen_spt_le_case(int which, int64_t full_n, int64_t n, int32_t* out) {
    switch (which) {
    case 0: srand(1234); for (int64_t i = 0; i < n; i++) out[i] = rand(); break;
    case 1: srand(99);   for (int64_t i = 0; i < n; i++) out[i] = rand() % 16; break;
    case 2: srand(7);    for (int64_t i = 0; i < n; i++) out[i] = rand() % 2; break;
    case 3: for (int64_t i = 0; i < n; i++) out[i] = 42; break;
    case 4: for (int64_t i = 0; i < n; i++) out[i] = (int32_t)(full_n - i); break;
    case 5: for (int64_t i = 0; i < n; i++) out[i] = (int32_t)i; break;
    case 6:
        srand(5);
        for (int64_t i = 0; i < n; i++) out[i] = (rand() % 4 == 0) ? 2147483647 : rand();
        break;
    default: return -2;
    }
    return 0;
}
