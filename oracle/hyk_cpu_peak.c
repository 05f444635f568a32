/* FP64 fused multiply-add throughput of the host cores (TEST
 * INFRASTRUCTURE: the denominator of the compiled CPU baseline's roofline).
 *
 * Every thread runs 24 independent chains a = a * b + c on 2-lane double
 * vectors (compiled with -ffp-contract=fast, so each is one vector fused
 * multiply-add), enough independent work to cover the latency of every FMA
 * pipe of a core.  Result: flop/s over all threads (2 flops per lane-FMA). */
#include <omp.h>
#include <stdint.h>

typedef double v2d __attribute__((vector_size(16)));

static double chains(uint64_t iters, double seed) {
    v2d a[24];
    const v2d b = {0.999999999, 0.999999998}, c = {1e-9, 2e-9};
    for (int k = 0; k < 24; ++k) a[k] = (v2d){seed + k, seed - k};
    for (uint64_t it = 0; it < iters; ++it) {
#pragma GCC unroll 24
        for (int k = 0; k < 24; ++k) a[k] = a[k] * b + c;
    }
    v2d s = {0.0, 0.0};
    for (int k = 0; k < 24; ++k) s += a[k];
    return s[0] + s[1];
}

/* Runs `iters` iterations per thread on n_threads threads (0: all); returns
 * the flop/s and stores the elapsed seconds and a checksum (keeps the work). */
double hyk_cpu_fma_peak(int n_threads, uint64_t iters, double *seconds, double *checksum) {
    const int nt = n_threads > 0 ? n_threads : omp_get_max_threads();
    double sum = 0.0;
    const double t0 = omp_get_wtime();
#pragma omp parallel num_threads(nt) reduction(+ : sum)
    sum += chains(iters, 1.0 + omp_get_thread_num());
    const double dt = omp_get_wtime() - t0;
    if (seconds) *seconds = dt;
    if (checksum) *checksum = sum;
    return (double)nt * (double)iters * 24.0 * 2.0 * 2.0 / dt;
}
