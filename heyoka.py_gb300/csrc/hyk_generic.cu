// System-independent kernels of libhyk, compiled ahead of time by nvcc for
// sm_103a: dense-output evaluation, the finished-lane counter of the
// one-launch-per-step propagation, and the FP64 FMA throughput probe used as
// the roofline denominator.

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "hyk_dmath.h"

namespace {

// out[i][l] = sum_n tc[i][n][l] dt[l]^n, Horner with fused multiply-adds (the
// same operation sequence as the generated kernels' dense output), in double
// or in float.
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <typename R>
__global__ void dense_eval_kernel(const R *__restrict__ tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes,
                                  uint64_t ld, const R *__restrict__ dt, R *__restrict__ out) {
    const uint64_t lane = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (lane >= n_lanes) return;
    const R t = dt[lane];
    for (uint32_t i = 0; i < n_eq; ++i) {
        const R *c = tc + (uint64_t)i * (order + 1) * ld + lane;
        R acc = c[(uint64_t)order * ld];
        for (int n = (int)order - 1; n >= 0; --n) acc = fma_rn(acc, t, c[(uint64_t)n * ld]);
        out[(uint64_t)i * ld + lane] = acc;
    }
}

__global__ void count_finished_kernel(const uint32_t *__restrict__ status, uint64_t n_lanes, uint32_t *finished) {
    uint32_t c = 0;
    for (uint64_t l = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l < n_lanes; l += (uint64_t)gridDim.x * blockDim.x)
        c += (status[l] & 3u) != 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(finished, c);
}

__global__ void zero_u32(uint32_t *p) { *p = 0; }

__global__ void dmath_kernel(int fn, const double *__restrict__ x, const double *__restrict__ a, double *__restrict__ out,
                             uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s, c;
    switch (fn) {
    case 0: out[i] = hyk_dm_exp(x[i]); break;
    case 1: out[i] = hyk_dm_log(x[i]); break;
    case 2: hyk_dm_sincos(x[i], &s, &c); out[i] = s; break;
    case 3: hyk_dm_sincos(x[i], &s, &c); out[i] = c; break;
    case 4: out[i] = hyk_dm_pow(x[i], a[i]); break;
    case 5: out[i] = hyk_dm_rho(x[i], a[i], 1.0, 1.0 / 20, 1.0 / 19); break;
    default: {
        // single precision: the inputs rounded to float, the result widened
        const float xf = (float)x[i], af = a ? (float)a[i] : 0.0f;
        float fs, fc;
        switch (fn) {
        case 6: out[i] = hyk_dmf_exp(xf); break;
        case 7: out[i] = hyk_dmf_log(xf); break;
        case 8: hyk_dmf_sincos(xf, &fs, &fc); out[i] = fs; break;
        case 9: hyk_dmf_sincos(xf, &fs, &fc); out[i] = fc; break;
        case 10: out[i] = hyk_dmf_pow(xf, af); break;
        default: out[i] = hyk_dmf_rho(xf, af, 1.0f, 1.0f / 9, 1.0f / 8); break;
        }
    }
    }
}

// FMA throughput (FP64, or FP32 for the float integrator's roofline): each
// thread runs 8 independent dependency chains of `iters` fused multiply-adds.
// The values stay bounded (a*x + b with a < 1).
template <typename R>
__global__ void fma_probe_kernel(R *sink, uint64_t iters, R a, R b) {
    R x0 = (R)threadIdx.x * (R)1e-3, x1 = x0 + (R)0.1, x2 = x0 + (R)0.2, x3 = x0 + (R)0.3;
    R x4 = x0 + (R)0.4, x5 = x0 + (R)0.5, x6 = x0 + (R)0.6, x7 = x0 + (R)0.7;
    for (uint64_t i = 0; i < iters; ++i) {
        x0 = fma_rn(x0, a, b);
        x1 = fma_rn(x1, a, b);
        x2 = fma_rn(x2, a, b);
        x3 = fma_rn(x3, a, b);
        x4 = fma_rn(x4, a, b);
        x5 = fma_rn(x5, a, b);
        x6 = fma_rn(x6, a, b);
        x7 = fma_rn(x7, a, b);
    }
    const R s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (R)1234.5678) sink[blockIdx.x] = s;  // keeps the chains alive
}

}  // namespace

extern "C" int hyk_generic_dense_eval(const double *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes, uint64_t ld,
                                      const double *dt, double *out, void *stream) {
    const unsigned blk = 128;
    const uint64_t grid = (n_lanes + blk - 1) / blk;
    dense_eval_kernel<double><<<(unsigned)grid, blk, 0, (cudaStream_t)stream>>>(tc, n_eq, order, n_lanes, ld, dt, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int hyk_generic_dense_eval_f32(const float *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes,
                                          uint64_t ld, const float *dt, float *out, void *stream) {
    const unsigned blk = 128;
    const uint64_t grid = (n_lanes + blk - 1) / blk;
    dense_eval_kernel<float><<<(unsigned)grid, blk, 0, (cudaStream_t)stream>>>(tc, n_eq, order, n_lanes, ld, dt, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int hyk_generic_dmath(int fn, const double *x, const double *a, double *out, uint64_t n, void *stream) {
    if (n == 0) return 0;
    dmath_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(fn, x, a, out, n);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int hyk_generic_count_finished(const uint32_t *status, uint64_t n_lanes, uint32_t *finished, void *stream) {
    zero_u32<<<1, 1, 0, (cudaStream_t)stream>>>(finished);
    uint64_t grid = (n_lanes + 255) / 256;
    if (grid > 4096) grid = 4096;
    if (grid == 0) grid = 1;
    count_finished_kernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(status, n_lanes, finished);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

template <typename R>
static int fma_peak(int device, double millis, double *flops_per_s, char *err, size_t errlen) {
    auto bad = [&](cudaError_t e, const char *what) {
        std::snprintf(err, errlen, "%s: %s", what, cudaGetErrorString(e));
        return -2;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return bad(e, "cudaSetDevice");
    int n_sm = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device);
    R *sink = nullptr;
    const int blocks_per_sm = 4, threads = 256;
    const int grid = n_sm * blocks_per_sm;
    e = cudaMalloc(&sink, sizeof(R) * grid);
    if (e != cudaSuccess) return bad(e, "cudaMalloc");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    // Calibrate the iteration count on a short run, then time the real one.
    uint64_t iters = 1 << 12;
    float ms = 0.f;
    for (int pass = 0; pass < 2; ++pass) {
        fma_probe_kernel<R><<<grid, threads>>>(sink, iters, (R)0.999999, (R)1e-6);  // warm-up
        cudaEventRecord(a);
        fma_probe_kernel<R><<<grid, threads>>>(sink, iters, (R)0.999999, (R)1e-6);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        if (e != cudaSuccess) {
            cudaFree(sink);
            return bad(e, "FMA probe");
        }
        cudaEventElapsedTime(&ms, a, b);
        if (pass == 0 && ms > 0.f) {
            double scale = millis / ms;
            if (scale < 1.0) scale = 1.0;
            if (scale > 65536.0) scale = 65536.0;
            iters = (uint64_t)(iters * scale);
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    const double fmas = (double)grid * threads * 8.0 * (double)iters;
    *flops_per_s = 2.0 * fmas / (ms * 1e-3);
    return 0;
}

extern "C" int hyk_generic_fp64_peak(int device, double millis, double *flops_per_s, char *err, size_t errlen) {
    return fma_peak<double>(device, millis, flops_per_s, err, errlen);
}

extern "C" int hyk_generic_fp32_peak(int device, double millis, double *flops_per_s, char *err, size_t errlen) {
    return fma_peak<float>(device, millis, flops_per_s, err, errlen);
}
