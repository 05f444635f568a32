/*
 * hyk_dmath.h - deterministic double-precision elementary functions.
 *
 * One source, compiled three ways: into the NVRTC-generated step kernels,
 * into libhyk's nvcc kernels, and into the CPU oracle.  Every function uses
 * only IEEE-754 operations that are correctly rounded on both the GPU and
 * the host (+, -, *, /, sqrt, fused multiply-add) plus bit manipulation, in
 * a fixed order, so a GPU kernel and the oracle that both use these functions
 * produce bit-identical results.  The host build must not contract or
 * reassociate floating-point expressions (-ffp-contract=off, no fast-math);
 * the device build uses --fmad=false.
 *
 * Methods (written for this project from the textbook mathematics):
 *  exp:  x = k ln2 + r, k = nearest integer to x / ln2 (two-constant
 *        Cody-Waite reduction, |r| <= ln2/2); e^r by its Taylor series to
 *        degree 13 (truncation < 5e-18); scaling by 2^k through the exponent bits.
 *  log:  x = 2^e m with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
 *        s = (m - 1) / (m + 1), by the odd series to s^23 (|s| <= 0.1716);
 *        e ln2 added with a two-part ln2.
 *  sin/cos: x = k pi/2 + r with a three-part pi/2 for |x| < 2^30; for
 *        larger |x| the reduction of Payne and Hanek ("Radian reduction for
 *        trigonometric functions", SIGNUM Newsletter 18(1), 1983): the
 *        fraction of x 2/pi from the bits of 2/pi that matter at x's
 *        exponent, in 128-bit integer arithmetic, exact for every double;
 *        then the Taylor series to r^17 (sine) and r^18 (cosine) on
 *        |r| <= pi/4, quadrant selection from k mod 4.
 *  pow with a constant exponent: integer and half-integer exponents by
 *        products, one square root and one division; other exponents as
 *        exp(alpha log x).
 * Accuracy (checked against 300-bit references in the test suite): exp, log,
 * sin, cos within 2 ulp on their reduced-argument ranges of use.
 */
#ifndef HYK_DMATH_H
#define HYK_DMATH_H

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define HYK_DM_FN static __device__ __forceinline__
#define HYK_DM_FMA(a, b, c) __fma_rn((a), (b), (c))
#define HYK_DM_SQRT(x) __dsqrt_rn(x)
#define HYK_DM_BITS(x) ((unsigned long long)__double_as_longlong(x))
#define HYK_DM_FROM(u) __longlong_as_double((long long)(u))
#define HYK_DM_FMAF(a, b, c) __fmaf_rn((a), (b), (c))
#define HYK_DM_SQRTF(x) __fsqrt_rn(x)
#define HYK_DM_FBITS(x) ((unsigned)__float_as_uint(x))
#define HYK_DM_FFROM(u) __uint_as_float((unsigned)(u))
#else
#include <cmath>
#include <cstring>
#define HYK_DM_FN static inline
#define HYK_DM_FMA(a, b, c) std::fma((a), (b), (c))
#define HYK_DM_SQRT(x) std::sqrt(x)
static inline unsigned long long hyk_dm_bits_(double x) {
    unsigned long long u;
    std::memcpy(&u, &x, sizeof u);
    return u;
}
static inline double hyk_dm_from_(unsigned long long u) {
    double x;
    std::memcpy(&x, &u, sizeof x);
    return x;
}
#define HYK_DM_BITS(x) hyk_dm_bits_(x)
#define HYK_DM_FROM(u) hyk_dm_from_(u)
static inline unsigned hyk_dm_fbits_(float x) {
    unsigned u;
    std::memcpy(&u, &x, sizeof u);
    return u;
}
static inline float hyk_dm_ffrom_(unsigned u) {
    float x;
    std::memcpy(&x, &u, sizeof x);
    return x;
}
#define HYK_DM_FMAF(a, b, c) std::fma((float)(a), (float)(b), (float)(c))
#define HYK_DM_SQRTF(x) std::sqrt((float)(x))
#define HYK_DM_FBITS(x) hyk_dm_fbits_(x)
#define HYK_DM_FFROM(u) hyk_dm_ffrom_(u)
#endif

#define HYK_DM_NAN HYK_DM_FROM(0x7ff8000000000000ULL)
#define HYK_DM_INF HYK_DM_FROM(0x7ff0000000000000ULL)
/* 1.5 * 2^52: adding it rounds a double of magnitude < 2^51 to an integer
 * held in the low mantissa bits. */
#define HYK_DM_RND 6755399441055744.0

HYK_DM_FN int hyk_dm_isnan(double x) { return (HYK_DM_BITS(x) & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL; }

/* 2^k for integer k in [-1022, 1023]. */
HYK_DM_FN double hyk_dm_pow2i(int k) { return HYK_DM_FROM((unsigned long long)(long long)(k + 1023) << 52); }

HYK_DM_FN double hyk_dm_exp(double x) {
    if (hyk_dm_isnan(x)) return x;
    if (x > 709.782712893384) return HYK_DM_INF;
    if (x < -745.1332191019412) return 0.0;
    const double t = HYK_DM_FMA(x, 1.4426950408889634, HYK_DM_RND);
    const double kd = t - HYK_DM_RND;
    const int k = (int)((long long)(HYK_DM_BITS(t) << 32) >> 32); /* low 32 bits, signed */
    double r = HYK_DM_FMA(-kd, 0.6931471805599453, x);
    r = HYK_DM_FMA(-kd, 2.3190468138462996e-17, r);
    double p = 1.6059043836821613e-10;  // 1/13!
    p = HYK_DM_FMA(p, r, 2.08767569878681e-09);
    p = HYK_DM_FMA(p, r, 2.505210838544172e-08);
    p = HYK_DM_FMA(p, r, 2.755731922398589e-07);
    p = HYK_DM_FMA(p, r, 2.7557319223985893e-06);
    p = HYK_DM_FMA(p, r, 2.48015873015873e-05);
    p = HYK_DM_FMA(p, r, 0.0001984126984126984);
    p = HYK_DM_FMA(p, r, 0.001388888888888889);
    p = HYK_DM_FMA(p, r, 0.008333333333333333);
    p = HYK_DM_FMA(p, r, 0.041666666666666664);
    p = HYK_DM_FMA(p, r, 0.16666666666666666);
    p = HYK_DM_FMA(p, r, 0.5);
    p = HYK_DM_FMA(p, r, 1.0);
    p = HYK_DM_FMA(p, r, 1.0);
    if (k >= -1022 && k <= 1023) return p * hyk_dm_pow2i(k);
    /* Results near the overflow or underflow limits: scale in two factors. */
    const int k1 = k / 2, k2 = k - k1;
    return (p * hyk_dm_pow2i(k1)) * hyk_dm_pow2i(k2);
}

HYK_DM_FN double hyk_dm_log(double x) {
    unsigned long long u = HYK_DM_BITS(x);
    if (hyk_dm_isnan(x)) return x;
    if (u >> 63) return (u << 1) == 0 ? -HYK_DM_INF : HYK_DM_NAN; /* -0 or negative */
    if (u == 0) return -HYK_DM_INF;
    if (u == 0x7ff0000000000000ULL) return x;
    int e = 0;
    if ((u >> 52) == 0) { /* subnormal: scale by 2^54 */
        x = x * 18014398509481984.0;
        u = HYK_DM_BITS(x);
        e = -54;
    }
    e += (int)(u >> 52) - 1023;
    double m = HYK_DM_FROM((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL); /* [1, 2) */
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    const double f = m - 1.0; /* exact */
    const double s = f / (2.0 + f);
    const double t = s * s;
    double q = 0.043478260869565216;  // 1/23
    q = HYK_DM_FMA(q, t, 0.047619047619047616);
    q = HYK_DM_FMA(q, t, 0.05263157894736842);
    q = HYK_DM_FMA(q, t, 0.058823529411764705);
    q = HYK_DM_FMA(q, t, 0.06666666666666667);
    q = HYK_DM_FMA(q, t, 0.07692307692307693);
    q = HYK_DM_FMA(q, t, 0.09090909090909091);
    q = HYK_DM_FMA(q, t, 0.1111111111111111);
    q = HYK_DM_FMA(q, t, 0.14285714285714285);
    q = HYK_DM_FMA(q, t, 0.2);
    q = HYK_DM_FMA(q, t, 0.3333333333333333);
    const double a = s + s;
    const double lm = HYK_DM_FMA(a * t, q, a); /* 2 atanh(s) */
    const double ed = (double)e;
    return HYK_DM_FMA(ed, 0.6931471805599453, HYK_DM_FMA(ed, 2.3190468138462996e-17, lm));
}

/* The binary digits of 2/pi, 64 per word, most significant first, after one
 * word of zeros (the digits of weight 2^0 and above): word j >= 1 holds the
 * digits of weight 2^-(64(j-1)+1) .. 2^-64j.  The 19 words after the zero
 * word are floor(2/pi 2^1216) (computed with mpmath at 1536 bits), enough
 * for the largest double exponent. */
#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
static __device__ const unsigned long long hyk_dm_2opi[20] = {
#else
static const unsigned long long hyk_dm_2opi[20] = {
#endif
    0x0000000000000000ULL, 0xa2f9836e4e441529ULL, 0xfc2757d1f534ddc0ULL, 0xdb6295993c439041ULL,
    0xfe5163abdebbc561ULL, 0xb7246e3a424dd2e0ULL, 0x06492eea09d1921cULL, 0xfe1deb1cb129a73eULL,
    0xe88235f52ebb4484ULL, 0xe99c7026b45f7e41ULL, 0x3991d639835339f4ULL, 0x9c845f8bbdf9283bULL,
    0x1ff897ffde05980fULL, 0xef2f118b5a0a6d1fULL, 0x6d367ecf27cb09b7ULL, 0x4f463f669e5fea2dULL,
    0x7527bac7ebe5f17bULL, 0x3d0739f78a5292eaULL, 0x6bfb5fb11f8d5d08ULL, 0x56033046fc7b6babULL,
};

/* High 64 bits of the 128-bit product of two 64-bit integers, and the
 * leading zeros of a non-zero 64-bit integer. */
#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
HYK_DM_FN unsigned long long hyk_dm_mulhi(unsigned long long a, unsigned long long b) { return __umul64hi(a, b); }
HYK_DM_FN int hyk_dm_clz(unsigned long long a) { return __clzll((long long)a); }
#else
HYK_DM_FN unsigned long long hyk_dm_mulhi(unsigned long long a, unsigned long long b) {
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
HYK_DM_FN int hyk_dm_clz(unsigned long long a) { return __builtin_clzll(a); }
#endif

/* 2^e as a double, -1022 <= e <= 1023. */
HYK_DM_FN double hyk_dm_pow2(int e) { return HYK_DM_FROM((unsigned long long)(1023 + e) << 52); }

/* Reduction of a finite |x| >= 2^30: r = x - k pi/2 with |r| <= pi/4 and
 * q = k mod 4.  With x = m 2^E (m the 53-bit integer significand) and
 * 2/pi = sum_i b_i 2^-i, the terms of x 2/pi with i < E - 1 are multiples of
 * 4, so x 2/pi = 4 frac(m W) (mod 4) where W = 0.b_(E-1) b_E ... is read
 * from the table (192 digits: the error of the fraction is below 2^-128).
 * The nearest quarter of 4 frac(m W) gives q, the signed remainder y times
 * pi/2 (as two doubles) gives r. */
HYK_DM_FN double hyk_dm_reduce_big(double x, unsigned *qp) {
    const unsigned long long u = HYK_DM_BITS(x);
    const int E = (int)((u >> 52) & 0x7ffULL) - 1075;
    const unsigned long long m = (u & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const int P0 = E + 62; /* table digit (from the start of word 0) of b_(E-1) */
    const int k = P0 >> 6, sh = P0 & 63;
    const unsigned long long t0 = hyk_dm_2opi[k], t1 = hyk_dm_2opi[k + 1], t2 = hyk_dm_2opi[k + 2],
                             t3 = hyk_dm_2opi[k + 3];
    const unsigned long long w0 = sh ? (t0 << sh) | (t1 >> (64 - sh)) : t0;
    const unsigned long long w1 = sh ? (t1 << sh) | (t2 >> (64 - sh)) : t1;
    const unsigned long long w2 = sh ? (t2 << sh) | (t3 >> (64 - sh)) : t2;
    /* frac(m W) = 0.f1 f2 (the integer part of m W is dropped) */
    const unsigned long long l0 = m * w0, h1 = hyk_dm_mulhi(m, w1), l1 = m * w1, h2 = hyk_dm_mulhi(m, w2);
    const unsigned long long f2 = l1 + h2;
    const unsigned long long f1 = l0 + h1 + (f2 < l1 ? 1ULL : 0ULL);
    /* 4 frac(m W) = q0 + g, g = 0.g1 g2 in [0, 1) */
    unsigned q = (unsigned)(f1 >> 62);
    unsigned long long g1 = (f1 << 2) | (f2 >> 62), g2 = f2 << 2;
    bool neg = false;
    if (g1 >> 63) { /* g >= 1/2: the nearest integer is q0 + 1 and y = g - 1 */
        q += 1;
        neg = true;
        g2 = ~g2 + 1ULL;
        g1 = ~g1 + (g2 == 0 ? 1ULL : 0ULL);
    }
    double r = 0.0;
    if (g1 | g2) {
        /* |y| = 0.g1 g2 normalised: its top 64 digits n1, then n2 */
        const int lz = g1 ? hyk_dm_clz(g1) : 64 + hyk_dm_clz(g2);
        unsigned long long n1, n2;
        if (lz >= 64) {
            n1 = g2 << (lz - 64);
            n2 = 0;
        } else if (lz > 0) {
            n1 = (g1 << lz) | (g2 >> (64 - lz));
            n2 = g2 << lz;
        } else {
            n1 = g1;
            n2 = g2;
        }
        /* |y| = (n1 + n2 2^-64) 2^(-64 - lz) = yh + yl */
        const double sc = hyk_dm_pow2(-64 - lz);
        const double yh = (double)(n1 >> 11) * (2048.0 * sc);
        const double yl = ((double)(n1 & 0x7ffULL) + (double)(n2 >> 11) * 1.1102230246251565e-16) * sc;
        /* r = |y| pi/2 with pi/2 = 1.5707963267948966 + 6.123233995736766e-17 */
        const double p = yh * 1.5707963267948966;
        const double pe = HYK_DM_FMA(yh, 1.5707963267948966, -p);
        r = p + (pe + HYK_DM_FMA(yh, 6.123233995736766e-17, yl * 1.5707963267948966));
        if (neg) r = -r;
    }
    if (x < 0.0) {
        r = -r;
        q = 0u - q;
    }
    *qp = q & 3u;
    return r;
}

/* sin and cos of x together. */
HYK_DM_FN void hyk_dm_sincos(double x, double *sp, double *cp) {
    const unsigned long long u = HYK_DM_BITS(x);
    if ((u & 0x7ff0000000000000ULL) == 0x7ff0000000000000ULL) { /* inf or nan */
        *sp = HYK_DM_NAN;
        *cp = HYK_DM_NAN;
        return;
    }
    unsigned q;
    double r;
    if ((u & 0x7fffffffffffffffULL) < 0x41d0000000000000ULL) { /* |x| < 2^30 */
        const double t = HYK_DM_FMA(x, 0.6366197723675814, HYK_DM_RND);
        const double kd = t - HYK_DM_RND;
        q = (unsigned)(HYK_DM_BITS(t) & 3ULL);
        r = HYK_DM_FMA(-kd, 1.5707963267948966, x);
        r = HYK_DM_FMA(-kd, 6.123233995736766e-17, r);
        r = HYK_DM_FMA(-kd, -1.4973849048591698e-33, r);
    } else {
        r = hyk_dm_reduce_big(x, &q);
    }
    const double z = r * r;
    double ps = 2.8114572543455206e-15;  // 1/17!
    ps = HYK_DM_FMA(ps, z, -7.647163731819816e-13);
    ps = HYK_DM_FMA(ps, z, 1.6059043836821613e-10);
    ps = HYK_DM_FMA(ps, z, -2.505210838544172e-08);
    ps = HYK_DM_FMA(ps, z, 2.7557319223985893e-06);
    ps = HYK_DM_FMA(ps, z, -0.0001984126984126984);
    ps = HYK_DM_FMA(ps, z, 0.008333333333333333);
    ps = HYK_DM_FMA(ps, z, -0.16666666666666666);
    const double s = HYK_DM_FMA(r * z, ps, r);
    double pc = -1.5619206968586225e-16;  // -1/18!
    pc = HYK_DM_FMA(pc, z, 4.779477332387385e-14);
    pc = HYK_DM_FMA(pc, z, -1.1470745597729725e-11);
    pc = HYK_DM_FMA(pc, z, 2.08767569878681e-09);
    pc = HYK_DM_FMA(pc, z, -2.755731922398589e-07);
    pc = HYK_DM_FMA(pc, z, 2.48015873015873e-05);
    pc = HYK_DM_FMA(pc, z, -0.001388888888888889);
    pc = HYK_DM_FMA(pc, z, 0.041666666666666664);
    pc = HYK_DM_FMA(pc, z, -0.5);
    const double c = HYK_DM_FMA(z, pc, 1.0);
    switch (q) {
    case 0:
        *sp = s;
        *cp = c;
        break;
    case 1:
        *sp = c;
        *cp = -s;
        break;
    case 2:
        *sp = -s;
        *cp = -c;
        break;
    default:
        *sp = -c;
        *cp = s;
        break;
    }
}

/* x^n for a non-negative integer n by binary powering (fixed product order). */
HYK_DM_FN double hyk_dm_powi(double x, unsigned n) {
    double r = 1.0, b = x;
    bool first = true;
    while (n) {
        if (n & 1u) {
            r = first ? b : r * b;
            first = false;
        }
        n >>= 1;
        if (n) b = b * b;
    }
    return r;
}

/* x^alpha for a constant alpha. */
HYK_DM_FN double hyk_dm_pow(double x, double alpha) {
    const double a2 = alpha + alpha;
    const bool integral = alpha <= 64.0 && alpha >= -64.0 && alpha == (double)(long long)alpha;
    const bool half = !integral && a2 <= 129.0 && a2 >= -129.0 && a2 == (double)(long long)a2;
    if (integral) {
        const long long n = (long long)alpha;
        if (n >= 0) return hyk_dm_powi(x, (unsigned)n);
        return 1.0 / hyk_dm_powi(x, (unsigned)(-n));
    }
    if (half) {
        const long long n2 = (long long)a2; /* odd */
        const double sq = HYK_DM_SQRT(x);
        if (n2 > 0) {
            const unsigned m = (unsigned)((n2 - 1) / 2);
            return m == 0 ? sq : hyk_dm_powi(x, m) * sq;
        }
        const unsigned m = (unsigned)((-n2 - 1) / 2);
        return 1.0 / (m == 0 ? sq : hyk_dm_powi(x, m) * sq);
    }
    if (x < 0.0) return HYK_DM_NAN;
    if (x == 0.0) return alpha > 0.0 ? 0.0 : HYK_DM_INF;
    return hyk_dm_exp(alpha * hyk_dm_log(x));
}

/* Jorba-Zou rho from the infinity norms: min over o in {p-1, p} of
 * (num / m_o)^(1/o), evaluated as exp(-max(log(m_o / num) / o)). */
HYK_DM_FN double hyk_dm_rho(double m_p, double m_pm1, double num, double inv_p, double inv_pm1) {
    const double e1 = hyk_dm_log(m_p / num) * inv_p;
    const double e2 = hyk_dm_log(m_pm1 / num) * inv_pm1;
    const double e = e2 > e1 ? e2 : e1;
    return hyk_dm_exp(-e);
}

/* ------------------------------------------------------------------ float
 * The same methods in single precision (the float32 batch integrator), with
 * float splits of ln 2 and pi/2 (leading parts with 12 and 9 significant bits,
 * so their products with the reduction's integer k are exact) and series
 * truncated for float accuracy (exp to r^7, log's atanh to s^11, sine to
 * r^9, cosine to r^10; truncation below 0.1 ulp). */
#define HYK_DMF_RND 12582912.0f /* 1.5 * 2^23 */

HYK_DM_FN int hyk_dmf_isnan(float x) { return (HYK_DM_FBITS(x) & 0x7fffffffu) > 0x7f800000u; }
HYK_DM_FN float hyk_dmf_pow2i(int k) { return HYK_DM_FFROM((unsigned)(k + 127) << 23); }

HYK_DM_FN float hyk_dmf_exp(float x) {
    if (hyk_dmf_isnan(x)) return x;
    if (x > 88.72283f) return HYK_DM_FFROM(0x7f800000u);
    if (x < -103.97208f) return 0.0f;
    const float t = HYK_DM_FMAF(x, 1.44269502f, HYK_DMF_RND);
    const float kf = t - HYK_DMF_RND;
    const int k = (int)(HYK_DM_FBITS(t) & 0x7fffffu) - 0x400000; /* the mantissa holds k + 2^22 */
    float r = HYK_DM_FMAF(-kf, 0.693115234375f, x);
    r = HYK_DM_FMAF(-kf, 3.19461833e-05f, r);
    float p = 1.98412698e-04f;  // 1/7!
    p = HYK_DM_FMAF(p, r, 1.38888889e-03f);
    p = HYK_DM_FMAF(p, r, 8.33333333e-03f);
    p = HYK_DM_FMAF(p, r, 4.16666667e-02f);
    p = HYK_DM_FMAF(p, r, 0.166666667f);
    p = HYK_DM_FMAF(p, r, 0.5f);
    p = HYK_DM_FMAF(p, r, 1.0f);
    p = HYK_DM_FMAF(p, r, 1.0f);
    if (k >= -126 && k <= 127) return p * hyk_dmf_pow2i(k);
    const int k1 = k / 2, k2 = k - k1;
    return (p * hyk_dmf_pow2i(k1)) * hyk_dmf_pow2i(k2);
}

HYK_DM_FN float hyk_dmf_log(float x) {
    unsigned u = HYK_DM_FBITS(x);
    if (hyk_dmf_isnan(x)) return x;
    if (u >> 31) return (u << 1) == 0 ? -HYK_DM_FFROM(0x7f800000u) : HYK_DM_FFROM(0x7fc00000u);
    if (u == 0) return -HYK_DM_FFROM(0x7f800000u);
    if (u == 0x7f800000u) return x;
    int e = 0;
    if ((u >> 23) == 0) { /* subnormal: scale by 2^25 */
        x = x * 33554432.0f;
        u = HYK_DM_FBITS(x);
        e = -25;
    }
    e += (int)(u >> 23) - 127;
    float m = HYK_DM_FFROM((u & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float t = s * s;
    float q = 9.09090909e-02f;  // 1/11
    q = HYK_DM_FMAF(q, t, 0.111111111f);
    q = HYK_DM_FMAF(q, t, 0.142857143f);
    q = HYK_DM_FMAF(q, t, 0.2f);
    q = HYK_DM_FMAF(q, t, 0.333333333f);
    const float a = s + s;
    const float lm = HYK_DM_FMAF(a * t, q, a);
    const float ef = (float)e;
    return HYK_DM_FMAF(ef, 0.693115234375f, HYK_DM_FMAF(ef, 3.19461833e-05f, lm));
}

HYK_DM_FN void hyk_dmf_sincos(float x, float *sp, float *cp) {
    const unsigned u = HYK_DM_FBITS(x);
    if ((u & 0x7f800000u) == 0x7f800000u) {
        *sp = HYK_DM_FFROM(0x7fc00000u);
        *cp = HYK_DM_FFROM(0x7fc00000u);
        return;
    }
    if ((u & 0x7fffffffu) >= 0x47800000u) {
        /* |x| >= 2^16: the float reduction's k pi/2 is no longer exact; the
         * double functions (exact reduction), rounded to float */
        double sd, cd;
        hyk_dm_sincos((double)x, &sd, &cd);
        *sp = (float)sd;
        *cp = (float)cd;
        return;
    }
    const float t = HYK_DM_FMAF(x, 0.636619747f, HYK_DMF_RND);
    const float kf = t - HYK_DMF_RND;
    const unsigned q = HYK_DM_FBITS(t) & 3u;
    float r = HYK_DM_FMAF(-kf, 1.5703125f, x);
    r = HYK_DM_FMAF(-kf, 4.83512878e-04f, r);
    r = HYK_DM_FMAF(-kf, 3.13916473e-07f, r);
    const float z = r * r;
    float ps = 2.75573192e-06f;  // 1/9!
    ps = HYK_DM_FMAF(ps, z, -1.98412698e-04f);
    ps = HYK_DM_FMAF(ps, z, 8.33333333e-03f);
    ps = HYK_DM_FMAF(ps, z, -0.166666667f);
    const float s = HYK_DM_FMAF(r * z, ps, r);
    float pc = -2.75573192e-07f;  // -1/10!
    pc = HYK_DM_FMAF(pc, z, 2.48015873e-05f);
    pc = HYK_DM_FMAF(pc, z, -1.38888889e-03f);
    pc = HYK_DM_FMAF(pc, z, 4.16666667e-02f);
    pc = HYK_DM_FMAF(pc, z, -0.5f);
    const float c = HYK_DM_FMAF(z, pc, 1.0f);
    switch (q) {
    case 0: *sp = s; *cp = c; break;
    case 1: *sp = c; *cp = -s; break;
    case 2: *sp = -s; *cp = -c; break;
    default: *sp = -c; *cp = s; break;
    }
}

HYK_DM_FN float hyk_dmf_powi(float x, unsigned n) {
    float r = 1.0f, b = x;
    bool first = true;
    while (n) {
        if (n & 1u) {
            r = first ? b : r * b;
            first = false;
        }
        n >>= 1;
        if (n) b = b * b;
    }
    return r;
}

HYK_DM_FN float hyk_dmf_pow(float x, float alpha) {
    const float a2 = alpha + alpha;
    const bool integral = alpha <= 64.0f && alpha >= -64.0f && alpha == (float)(int)alpha;
    const bool half = !integral && a2 <= 129.0f && a2 >= -129.0f && a2 == (float)(int)a2;
    if (integral) {
        const int n = (int)alpha;
        if (n >= 0) return hyk_dmf_powi(x, (unsigned)n);
        return 1.0f / hyk_dmf_powi(x, (unsigned)(-n));
    }
    if (half) {
        const int n2 = (int)a2;
        const float sq = HYK_DM_SQRTF(x);
        if (n2 > 0) {
            const unsigned m = (unsigned)((n2 - 1) / 2);
            return m == 0 ? sq : hyk_dmf_powi(x, m) * sq;
        }
        const unsigned m = (unsigned)((-n2 - 1) / 2);
        return 1.0f / (m == 0 ? sq : hyk_dmf_powi(x, m) * sq);
    }
    if (x < 0.0f) return HYK_DM_FFROM(0x7fc00000u);
    if (x == 0.0f) return alpha > 0.0f ? 0.0f : HYK_DM_FFROM(0x7f800000u);
    /* other exponents: alpha log x loses |alpha log x| ulps in float, so
     * through the double functions (rounded once at the end) */
    return (float)hyk_dm_exp((double)alpha * hyk_dm_log((double)x));
}

HYK_DM_FN float hyk_dmf_rho(float m_p, float m_pm1, float num, float inv_p, float inv_pm1) {
    const float e1 = hyk_dmf_log(m_p / num) * inv_p;
    const float e2 = hyk_dmf_log(m_pm1 / num) * inv_pm1;
    const float e = e2 > e1 ? e2 : e1;
    return hyk_dmf_exp(-e);
}

#endif /* HYK_DMATH_H */
