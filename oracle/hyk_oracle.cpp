// hyk_oracle.cpp - CPU oracle for the batch Taylor integrator.
//
// TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
// and the CPU-baseline leg of bench.py load this library, and only as the
// checker or as the timed CPU restatement; the CUDA library never calls it.
//
// This is a restatement of the algorithm of the reference's batch integrator
// (heyoka::taylor_adaptive_batch<double>, heyoka C++ 7.11.0, called from
// heyoka/expose_batch_integrators.cpp).  The reference's arithmetic lives in
// the un-vendored heyoka C++ library, so every rule below is restated from the
// published method and pinned by the reference's own known-answer outputs:
//
//  * Taylor recurrences of the elementary u-variables (doc/tut_taylor_method.rst:10-81),
//    evaluated in decomposition order for orders 0..p; state coefficients
//    x^[n+1] = f^[n] / (n+1).
//  * Order rule p = ceil(-ln(tol)/2 + 1) (computed by the caller).
//  * Step size (Jorba-Zou with heyoka's safety factor): absolute mode when
//    max|x_i| < 1, relative otherwise; rho = min over o in {p-1, p} of
//    1 / pow(max_i|x_i^[o]| / num, 1/o); h = rho * exp(-2) * exp(-0.7/(p-1)),
//    clamped to |max_delta_t|.  Pinned bit-exactly by the first step of
//    doc/notebooks/The adaptive integrator.ipynb (h = 0.21605277478009474) and
//    by the four step_res values of doc/notebooks/Batch mode overview.ipynb.
//  * Horner state update, double-length (hi, lo) time with Knuth/Dekker
//    error-free additions (heyoka/expose_batch_integrators.cpp:394-449 expose it).
//  * Batch propagate semantics (doc/notebooks/Batch mode overview.ipynb):
//    remaining time kept in double-length, step limit = min(max_delta_t,
//    remaining), lanes that reached their final time take zero steps (not
//    counted), remaining time forced to zero when the step equals it,
//    propagate_res = (outcome, min |h|, max |h|, nonzero steps); a non-finite
//    state stops the batch with err_nf_state; max_steps gives step_limit.
//  * propagate_grid: dense output (Horner at the offset from the step start)
//    for every grid point inside each step, NaN rows on early exit
//    (heyoka/expose_batch_integrators.cpp:315-392).
//  * continuous output: per-iteration Taylor coefficients and end times
//    (heyoka/taylor_expose_c_output.cpp:259-523).
//  * events (t_event_batch / nt_event_batch, heyoka/taylor_expose_events.cpp:202-311):
//    the event functions' Taylor coefficients up to order p, roots of their
//    step polynomials by hyk_events.h, a terminal event ending its lane's
//    step at the first root, non-terminal roots recorded in order
//    (hyko_propagate_ev, gpu arithmetic, per-lane stopping like the kernels).
//
// Two arithmetic modes:
//  mode 0 ("pin"): sums of products with separate multiply and add, division
//         by n and by order-0 denominators.  This is the mode pinned to the
//         reference's notebook outputs.
//  mode 1 ("gpu"): the same operation sequence with every product-accumulate
//         as a fused multiply-add, divisions by n replaced by multiplication
//         with the double nearest 1/n, and divisions by an order-0 value b0 at
//         orders n >= 1 replaced by multiplication with 1/b0 (one division per
//         step), and exp, log, sin, cos, pow and the step-size exponentials
//         evaluated by the deterministic functions of hyk_dmath.h.  This is,
//         operation for operation, what the CUDA kernels compute (they are
//         compiled with --fmad=false, explicit FMAs and the same hyk_dmath.h),
//         so the GPU and the oracle in this mode agree bit for bit.
//
// Precision: double, or binary128 (__float128 on x86-64, long double on
// aarch64) for the high-precision error reference.
//
// Build: oracle/build.py (g++ -O3 -fopenmp -ffp-contract=off, no -march flags).

#include "hyk.h"
#include "hyk_dmath.h"   // the deterministic elementary functions of the CUDA kernels
#include "hyk_events.h"  // the event root finder of the CUDA kernels
#include "hyk_fuse.h"    // the kernels' fusion of sums with a square (gpu arithmetic)

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#if defined(_OPENMP)
#include <omp.h>
#endif

#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
typedef __float128 qreal;
#define HYKO_QUADMATH 1
#else
typedef long double qreal;  // IEEE binary128 on aarch64 Linux
#define HYKO_QUADMATH 0
#endif

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------- math shims
template <typename T> struct M;
template <> struct M<double> {
    static double sin(double x) { return std::sin(x); }
    static double cos(double x) { return std::cos(x); }
    static double exp(double x) { return std::exp(x); }
    static double log(double x) { return std::log(x); }
    static double sqrt(double x) { return std::sqrt(x); }
    static double pow(double x, double y) { return std::pow(x, y); }
    static double fma(double a, double b, double c) { return std::fma(a, b, c); }
    static double abs(double x) { return std::fabs(x); }
    static bool isfinite(double x) { return std::isfinite(x); }
    static double inf() { return std::numeric_limits<double>::infinity(); }
    static double nan() { return std::numeric_limits<double>::quiet_NaN(); }
};
template <> struct M<float> {
    static float sin(float x) { return std::sin(x); }
    static float cos(float x) { return std::cos(x); }
    static float exp(float x) { return std::exp(x); }
    static float log(float x) { return std::log(x); }
    static float sqrt(float x) { return std::sqrt(x); }
    static float pow(float x, float y) { return std::pow(x, y); }
    static float fma(float a, float b, float c) { return std::fma(a, b, c); }
    static float abs(float x) { return std::fabs(x); }
    static bool isfinite(float x) { return std::isfinite(x); }
    static float inf() { return std::numeric_limits<float>::infinity(); }
    static float nan() { return std::numeric_limits<float>::quiet_NaN(); }
};
template <> struct M<qreal> {
#if HYKO_QUADMATH
    static qreal sin(qreal x) { return sinq(x); }
    static qreal cos(qreal x) { return cosq(x); }
    static qreal exp(qreal x) { return expq(x); }
    static qreal log(qreal x) { return logq(x); }
    static qreal sqrt(qreal x) { return sqrtq(x); }
    static qreal pow(qreal x, qreal y) { return powq(x, y); }
    static qreal fma(qreal a, qreal b, qreal c) { return fmaq(a, b, c); }
    static qreal abs(qreal x) { return fabsq(x); }
    static bool isfinite(qreal x) { return finiteq(x) != 0; }
#else
    static qreal sin(qreal x) { return sinl(x); }
    static qreal cos(qreal x) { return cosl(x); }
    static qreal exp(qreal x) { return expl(x); }
    static qreal log(qreal x) { return logl(x); }
    static qreal sqrt(qreal x) { return sqrtl(x); }
    static qreal pow(qreal x, qreal y) { return powl(x, y); }
    static qreal fma(qreal a, qreal b, qreal c) { return fmal(a, b, c); }
    static qreal abs(qreal x) { return fabsl(x); }
    static bool isfinite(qreal x) { return std::isfinite(x); }
#endif
    static qreal inf() { return (qreal)std::numeric_limits<double>::infinity(); }
    static qreal nan() { return (qreal)std::numeric_limits<double>::quiet_NaN(); }
};

// Transcendental functions per arithmetic mode: "pin" uses the C library
// (the reference's arithmetic), "gpu" the deterministic functions shared with
// the CUDA kernels.  binary128 always uses the quad-precision library.
template <typename T> struct F {
    static T exp(T x, int) { return M<T>::exp(x); }
    static T log(T x, int) { return M<T>::log(x); }
    static T pow(T x, T a, int) { return M<T>::pow(x, a); }
    static void sincos(T x, T &s, T &c, int) {
        s = M<T>::sin(x);
        c = M<T>::cos(x);
    }
    static bool rho(T, T, T, T, T, int, T &) { return false; }
};
template <> struct F<double> {
    static double exp(double x, int m) { return m ? hyk_dm_exp(x) : std::exp(x); }
    static double log(double x, int m) { return m ? hyk_dm_log(x) : std::log(x); }
    static double pow(double x, double a, int m) { return m ? hyk_dm_pow(x, a) : std::pow(x, a); }
    static void sincos(double x, double &s, double &c, int m) {
        if (m) {
            hyk_dm_sincos(x, &s, &c);
        } else {
            s = std::sin(x);
            c = std::cos(x);
        }
    }
    static bool rho(double mp, double mq, double num, double ip, double iq, int m, double &out) {
        if (!m) return false;
        out = hyk_dm_rho(mp, mq, num, ip, iq);
        return true;
    }
};

// Single precision (heyoka's float integrator): "gpu" arithmetic only, with
// the float functions of the kernels.
template <> struct F<float> {
    static float exp(float x, int m) { return m ? hyk_dmf_exp(x) : std::exp(x); }
    static float log(float x, int m) { return m ? hyk_dmf_log(x) : std::log(x); }
    static float pow(float x, float a, int m) { return m ? hyk_dmf_pow(x, a) : std::pow(x, a); }
    static void sincos(float x, float &s, float &c, int m) {
        if (m) {
            hyk_dmf_sincos(x, &s, &c);
        } else {
            s = std::sin(x);
            c = std::cos(x);
        }
    }
    static bool rho(float mp, float mq, float num, float ip, float iq, int m, float &out) {
        if (!m) return false;
        out = hyk_dmf_rho(mp, mq, num, ip, iq);
        return true;
    }
};

// ------------------------------------------------------ double-length time
template <typename T> struct dfl {
    T hi, lo;
};
// Knuth's branch-free error-free sum.
template <typename T> inline void two_sum(T a, T b, T &s, T &e) {
    s = a + b;
    const T bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// Dekker's error-free sum, |a| >= |b|.
template <typename T> inline void fast_two_sum(T a, T b, T &s, T &e) {
    s = a + b;
    e = b - (s - a);
}
template <typename T> inline dfl<T> dadd(dfl<T> x, dfl<T> y) {
    T s, e;
    two_sum(x.hi, y.hi, s, e);
    e = e + (x.lo + y.lo);
    dfl<T> r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
template <typename T> inline dfl<T> dneg(dfl<T> x) { return {-x.hi, -x.lo}; }
template <typename T> inline dfl<T> dsub(dfl<T> x, dfl<T> y) { return dadd(x, dneg(y)); }
template <typename T> inline dfl<T> dnorm(T hi, T lo) {
    dfl<T> r;
    two_sum(hi, lo, r.hi, r.lo);
    return r;
}
template <typename T> inline bool dle(dfl<T> x, dfl<T> y) { return x.hi < y.hi || (x.hi == y.hi && x.lo <= y.lo); }
template <typename T> inline bool dge(dfl<T> x, dfl<T> y) { return x.hi > y.hi || (x.hi == y.hi && x.lo >= y.lo); }

// ---------------------------------------------------------- decomposition
struct Dec {
    uint32_t n_eq = 0, n_ops = 0, n_pars = 0;
    std::vector<hyk_uop_t> ops;
    std::vector<hyk_arg_t> rhs;
    std::vector<hyk_event_t> ev;
    uint32_t n_u() const { return n_eq + n_ops; }
};

bool load_dec(const hyk_decomp_t *d, Dec &out) {
    if (!d || d->n_eq == 0) {
        g_err = "invalid decomposition";
        return false;
    }
    out.n_eq = d->n_eq;
    out.n_ops = d->n_ops;
    out.n_pars = d->n_pars;
    out.ops.assign(d->ops, d->ops + d->n_ops);
    out.rhs.assign(d->rhs, d->rhs + d->n_eq);
    const uint32_t nu = out.n_u();
    auto chk = [&](const hyk_arg_t &a, uint32_t self) {
        switch (a.kind) {
        case HYK_ARG_NONE:
        case HYK_ARG_NUM:
        case HYK_ARG_TIME:
            return true;
        case HYK_ARG_U:
            return a.idx >= 0 && (uint32_t)a.idx < self;
        case HYK_ARG_PAR:
            return a.idx >= 0 && (uint32_t)a.idx < out.n_pars;
        default:
            return false;
        }
    };
    for (uint32_t k = 0; k < out.n_ops; ++k) {
        const auto &o = out.ops[k];
        const uint32_t self = out.n_eq + k;
        if (o.op < HYK_OP_ADD || o.op > HYK_OP_COS || !chk(o.a, self) || !chk(o.b, self)) {
            g_err = "invalid u-variable definition at index " + std::to_string(self);
            return false;
        }
        if ((o.op == HYK_OP_SIN || o.op == HYK_OP_COS) && (o.aux < (int)out.n_eq || (uint32_t)o.aux >= nu)) {
            g_err = "invalid sin/cos partner";
            return false;
        }
    }
    for (const auto &r : out.rhs)
        if (!chk(r, nu) || r.kind == HYK_ARG_NONE) {
            g_err = "invalid right-hand side";
            return false;
        }
    if (d->n_ev > 0 && d->ev) out.ev.assign(d->ev, d->ev + d->n_ev);
    for (const auto &e : out.ev)
        if (!chk(e.g, nu) || e.g.kind == HYK_ARG_NONE) {
            g_err = "invalid event";
            return false;
        }
    return true;
}

// ------------------------------------------------------------ the batch
template <typename T> struct Batch {
    const Dec &d;
    uint32_t p, B, nu;
    int mode;  // 0 pin, 1 gpu
    std::vector<T> J, KA, I0;  // jets [nu][p+1][B], j*a_j [nu][p+1][B], per-u order-0 inverses [nu][B]
    std::vector<char> need_ka;
    std::vector<T> pars, state, thi, tlo, ones, inv;
    std::vector<T> numrows;             // constant rows for NUM arguments
    std::vector<int64_t> numrow_of;     // (op*2 + which) -> row index, -1
    std::vector<int64_t> rhs_numrow;    // per rhs
    std::vector<T> s_acc, s_num, s_tmp, s_den;  // per-lane scratch rows
    T rhofac;

    int ha = 0;  // high accuracy: compensated summation in the state update
    // gpu arithmetic: time-constant operations (every argument a number, a
    // parameter or such an operation) have only an order-0 value, their
    // higher orders are known zeros (the kernels' code generator does the same).
    std::vector<char> cst;
    // gpu arithmetic: sums of squares and sums of scaled terms computed as
    // one chain where the kernels' code generator does so (hyk_fuse.h); the
    // absorbed squares, products, negations and sums are not computed.
    HykFusePlan fz;

    // md: bit 0 = gpu arithmetic, bit 1 = high accuracy.
    Batch(const Dec &dd, uint32_t order, uint32_t b, int md)
        : d(dd), p(order), B(b), nu(dd.n_u()), mode(md & 1), ha((md >> 1) & 1) {
        J.assign((size_t)nu * (p + 1) * B, T(0));
        KA.assign((size_t)nu * (p + 1) * B, T(0));
        I0.assign((size_t)nu * B, T(0));
        need_ka.assign(nu, 0);
        pars.assign((size_t)d.n_pars * B, T(0));
        state.assign((size_t)d.n_eq * B, T(0));
        thi.assign(B, T(0));
        tlo.assign(B, T(0));
        ones.assign(B, T(1));
        inv.assign(p + 2, T(0));
        for (uint32_t n = 1; n <= p + 1; ++n) inv[n] = T(1) / T(n);
        s_acc.assign(B, T(0));
        s_num.assign(B, T(0));
        s_tmp.assign(B, T(0));
        s_den.assign(B, T(0));
        numrow_of.assign((size_t)d.n_ops * 2, -1);
        rhs_numrow.assign(d.n_eq, -1);
        auto add_row = [&](double v) {
            const int64_t r = (int64_t)(numrows.size() / B);
            numrows.insert(numrows.end(), B, T(v));
            return r;
        };
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const auto &o = d.ops[k];
            if (o.a.kind == HYK_ARG_NUM) numrow_of[2 * k] = add_row(o.a.num);
            if (o.b.kind == HYK_ARG_NUM && o.op != HYK_OP_POW) numrow_of[2 * k + 1] = add_row(o.b.num);
            // j*a_j is needed for the argument of exp, sin, cos, and for the
            // result of log (the log recurrence runs over j*l_j).
            if (o.op == HYK_OP_EXP || o.op == HYK_OP_SIN || o.op == HYK_OP_COS)
                if (o.a.kind == HYK_ARG_U) need_ka[o.a.idx] = 1;
            if (o.op == HYK_OP_LOG) need_ka[d.n_eq + k] = 1;
        }
        for (uint32_t i = 0; i < d.n_eq; ++i)
            if (d.rhs[i].kind == HYK_ARG_NUM) rhs_numrow[i] = add_row(d.rhs[i].num);
        cst.assign(nu, 0);
        if (mode == 1)
            for (uint32_t k = 0; k < d.n_ops; ++k) {
                const auto &o = d.ops[k];
                auto kc = [&](const hyk_arg_t &a) {
                    return a.kind == HYK_ARG_NONE || a.kind == HYK_ARG_NUM || a.kind == HYK_ARG_PAR ||
                           (a.kind == HYK_ARG_U && cst[a.idx]);
                };
                cst[d.n_eq + k] = kc(o.a) && kc(o.b);
            }
        if (mode == 1)
            fz = hyk_fuse_plan(d.n_eq, d.n_ops, d.ops.data(), d.rhs.data(), (uint32_t)d.ev.size(), d.ev.data());
        // rho factor exp(-2) * exp(-0.7/(p-1)), written as 1/(e*e) * exp((-7/10)/(p-1)).
        const T e1 = M<T>::exp(T(1));
        rhofac = T(1) / (e1 * e1) * M<T>::exp((T(-7) / T(10)) / T(p - 1));
    }

    T *jr(uint32_t u, uint32_t n) { return &J[((size_t)u * (p + 1) + n) * B]; }
    T *kr(uint32_t u, uint32_t n) { return &KA[((size_t)u * (p + 1) + n) * B]; }

    // Row of order-j coefficients of an argument, or nullptr when identically 0.
    const T *row(const hyk_arg_t &a, int64_t nr, uint32_t j) {
        switch (a.kind) {
        case HYK_ARG_U:
            return (cst[a.idx] && j >= 1) ? nullptr : jr(a.idx, j);
        case HYK_ARG_NUM:
            return j == 0 ? &numrows[(size_t)nr * B] : nullptr;
        case HYK_ARG_PAR:
            return j == 0 ? &pars[(size_t)a.idx * B] : nullptr;
        case HYK_ARG_TIME:
            return j == 0 ? thi.data() : (j == 1 ? ones.data() : nullptr);
        }
        return nullptr;
    }
    // Row of j * a_j (j >= 1), or nullptr when identically 0.
    const T *karow(const hyk_arg_t &a, uint32_t j) {
        switch (a.kind) {
        case HYK_ARG_U:
            return cst[a.idx] ? nullptr : kr(a.idx, j);
        case HYK_ARG_TIME:
            return j == 1 ? ones.data() : nullptr;
        default:
            return nullptr;
        }
    }

    // acc (+)= x*y over lanes; `first` initialises with a plain product.
    void term(T *acc, const T *x, const T *y, bool &first) {
        if (!x || !y) return;
        if (first) {
            for (uint32_t l = 0; l < B; ++l) acc[l] = x[l] * y[l];
            first = false;
        } else if (mode) {
            for (uint32_t l = 0; l < B; ++l) acc[l] = M<T>::fma(x[l], y[l], acc[l]);
        } else {
            for (uint32_t l = 0; l < B; ++l) acc[l] = acc[l] + x[l] * y[l];
        }
    }
    // out = acc / n (pin) or acc * (1/n) (gpu)
    void divn(T *out, const T *acc, uint32_t n) {
        if (mode) {
            const T c = inv[n];
            for (uint32_t l = 0; l < B; ++l) out[l] = acc[l] * c;
        } else {
            const T c = T(n);
            for (uint32_t l = 0; l < B; ++l) out[l] = acc[l] / c;
        }
    }
    // out = num / den0 (pin) or num * inv0 (gpu), den0 the order-0 denominator of u.
    void div0(T *out, const T *num, const T *den0, uint32_t u) {
        if (mode) {
            const T *iv = &I0[(size_t)u * B];
            for (uint32_t l = 0; l < B; ++l) out[l] = num[l] * iv[l];
        } else {
            for (uint32_t l = 0; l < B; ++l) out[l] = num[l] / den0[l];
        }
    }

    void set_ka(uint32_t u, uint32_t n) {
        if (!need_ka[u] || n == 0) return;
        T *o = kr(u, n);
        const T *a = jr(u, n);
        const T c = T(n);
        for (uint32_t l = 0; l < B; ++l) o[l] = c * a[l];
    }

    // Coefficient n of op k (u = n_eq + k).
    void op_coef(uint32_t k, uint32_t n) {
        const hyk_uop_t &o = d.ops[k];
        const uint32_t u = d.n_eq + k;
        if (cst[u] && n >= 1) return;  // known zero
        T *c = jr(u, n);
        const int64_t ra = numrow_of[2 * k], rb = numrow_of[2 * k + 1];
        std::vector<T> &acc = s_acc;
        bool first = true;
        if (!fz.dead.empty() && fz.dead[k]) return;  // absorbed by a fused sum
        if (!fz.fuse.empty() && fz.fuse[k] == HYK_FUSE_SC) {
            // c_n = a_n + sum_i k_i t_i,n (hyk_fuse.h): c = a_n (k_1 t_1,n
            // without a), then c = fma(k_i, t_i,n, c) leaf by leaf
            const bool ha = fz.addend[k] >= 0;
            const T *a = ha ? jr((uint32_t)fz.addend[k], n) : nullptr;
            for (size_t i = 0; i < fz.leaves[k].size(); ++i) {
                const T kk = T(fz.scales[k][i]);
                const T *x = jr((uint32_t)fz.leaves[k][i], n);
                for (uint32_t l = 0; l < B; ++l)
                    c[l] = i == 0 ? (ha ? M<T>::fma(kk, x[l], a[l]) : kk * x[l]) : M<T>::fma(kk, x[l], c[l]);
            }
            set_ka(u, n);
            return;
        }
        if (!fz.fuse.empty() && fz.fuse[k]) {
            // c_n = a_n + sum_i (x_i^2)_n (hyk_fuse.h): s = sum_i sum_{j < n/2}
            // x_i,j x_i,n-j, c = fma(2, s, a_n) (s + s without a), then
            // fma(x_i,n/2, x_i,n/2, c) for every leaf at even n
            const bool ha = fz.addend[k] >= 0;
            const T *a = ha ? jr((uint32_t)fz.addend[k], n) : nullptr;
            for (int32_t x : fz.leaves[k])
                for (uint32_t j = 0; 2 * j < n; ++j) term(acc.data(), jr((uint32_t)x, j), jr((uint32_t)x, n - j), first);
            bool have = true;
            if (!first) {
                for (uint32_t l = 0; l < B; ++l) c[l] = ha ? M<T>::fma(T(2), acc[l], a[l]) : acc[l] + acc[l];
            } else if (ha) {
                for (uint32_t l = 0; l < B; ++l) c[l] = a[l];
            } else {
                have = false;
            }
            if (n % 2 == 0)
                for (int32_t x : fz.leaves[k]) {
                    const T *xm = jr((uint32_t)x, n / 2);
                    for (uint32_t l = 0; l < B; ++l) c[l] = have ? M<T>::fma(xm[l], xm[l], c[l]) : xm[l] * xm[l];
                    have = true;
                }
            if (!have)
                for (uint32_t l = 0; l < B; ++l) c[l] = T(0);
            set_ka(u, n);
            return;
        }
        switch (o.op) {
        case HYK_OP_ADD:
        case HYK_OP_SUB: {
            const T *a = row(o.a, ra, n), *b = row(o.b, rb, n);
            for (uint32_t l = 0; l < B; ++l) {
                if (a && b)
                    c[l] = o.op == HYK_OP_ADD ? a[l] + b[l] : a[l] - b[l];
                else if (a)
                    c[l] = a[l];
                else if (b)
                    c[l] = o.op == HYK_OP_ADD ? b[l] : -b[l];
                else
                    c[l] = T(0);
            }
            break;
        }
        case HYK_OP_NEG: {
            const T *a = row(o.a, ra, n);
            for (uint32_t l = 0; l < B; ++l) c[l] = a ? -a[l] : T(0);
            break;
        }
        case HYK_OP_MUL: {
            for (uint32_t j = 0; j <= n; ++j) term(acc.data(), row(o.a, ra, j), row(o.b, rb, n - j), first);
            for (uint32_t l = 0; l < B; ++l) c[l] = first ? T(0) : acc[l];
            break;
        }
        case HYK_OP_DIV: {
            const T *b0 = row(o.b, rb, 0);
            const T *an = row(o.a, ra, n);
            if (n == 0) {
                for (uint32_t l = 0; l < B; ++l) c[l] = an[l] / b0[l];
                T *iv = &I0[(size_t)u * B];
                for (uint32_t l = 0; l < B; ++l) iv[l] = T(1) / b0[l];
                break;
            }
            for (uint32_t j = 1; j <= n; ++j) term(acc.data(), row(o.b, rb, j), jr(u, n - j), first);
            std::vector<T> &num = s_num;
            for (uint32_t l = 0; l < B; ++l) {
                const T av = an ? an[l] : T(0);
                num[l] = first ? av : av - acc[l];
            }
            div0(c, num.data(), b0, u);
            break;
        }
        case HYK_OP_SQUARE: {
            // c_n = 2 * sum_{j < n-j} a_j a_{n-j} + (n even ? a_{n/2}^2 : 0)
            for (uint32_t j = 0; 2 * j < n; ++j) term(acc.data(), row(o.a, ra, j), row(o.a, ra, n - j), first);
            if (!first)
                for (uint32_t l = 0; l < B; ++l) acc[l] = acc[l] + acc[l];
            if (n % 2 == 0) term(acc.data(), row(o.a, ra, n / 2), row(o.a, ra, n / 2), first);
            for (uint32_t l = 0; l < B; ++l) c[l] = first ? T(0) : acc[l];
            break;
        }
        case HYK_OP_SQRT: {
            const T *an = row(o.a, ra, n);
            if (n == 0) {
                T *iv = &I0[(size_t)u * B];
                for (uint32_t l = 0; l < B; ++l) {
                    c[l] = M<T>::sqrt(an[l]);
                    iv[l] = T(1) / (T(2) * c[l]);
                }
                break;
            }
            for (uint32_t j = 1; 2 * j < n; ++j) term(acc.data(), jr(u, j), jr(u, n - j), first);
            if (!first)
                for (uint32_t l = 0; l < B; ++l) acc[l] = acc[l] + acc[l];
            if (n % 2 == 0) term(acc.data(), jr(u, n / 2), jr(u, n / 2), first);
            std::vector<T> &num = s_num, &den = s_den;
            const T *c0 = jr(u, 0);
            for (uint32_t l = 0; l < B; ++l) {
                const T av = an ? an[l] : T(0);
                num[l] = first ? av : av - acc[l];
                den[l] = T(2) * c0[l];
            }
            div0(c, num.data(), den.data(), u);
            break;
        }
        case HYK_OP_POW: {
            const T alpha = T(o.b.num);
            const T *a0 = row(o.a, ra, 0);
            if (n == 0) {
                T *iv = &I0[(size_t)u * B];
                for (uint32_t l = 0; l < B; ++l) {
                    c[l] = F<T>::pow(a0[l], alpha, mode);
                    iv[l] = T(1) / a0[l];
                }
                break;
            }
            // c_n = (1/(n a_0)) sum_{j=0}^{n-1} (n*alpha - j*(alpha+1)) a_{n-j} c_j
            std::vector<T> &tmp = s_tmp;
            for (uint32_t j = 0; j < n; ++j) {
                const T *an_j = row(o.a, ra, n - j);
                if (!an_j) continue;
                const T coef = T(n) * alpha - T(j) * (alpha + T(1));
                for (uint32_t l = 0; l < B; ++l) tmp[l] = coef * an_j[l];
                term(acc.data(), tmp.data(), jr(u, j), first);
            }
            if (first) {
                for (uint32_t l = 0; l < B; ++l) c[l] = T(0);
                break;
            }
            if (mode) {
                std::vector<T> &t2 = s_num;
                divn(t2.data(), acc.data(), n);
                div0(c, t2.data(), a0, u);
            } else {
                const T nn = T(n);
                for (uint32_t l = 0; l < B; ++l) c[l] = acc[l] / (nn * a0[l]);
            }
            break;
        }
        case HYK_OP_EXP: {
            if (n == 0) {
                const T *a0 = row(o.a, ra, 0);
                for (uint32_t l = 0; l < B; ++l) c[l] = F<T>::exp(a0[l], mode);
                break;
            }
            for (uint32_t j = 1; j <= n; ++j) term(acc.data(), karow(o.a, j), jr(u, n - j), first);
            if (first) {
                for (uint32_t l = 0; l < B; ++l) c[l] = T(0);
                break;
            }
            divn(c, acc.data(), n);
            break;
        }
        case HYK_OP_LOG: {
            const T *a0 = row(o.a, ra, 0), *an = row(o.a, ra, n);
            if (n == 0) {
                T *iv = &I0[(size_t)u * B];
                for (uint32_t l = 0; l < B; ++l) {
                    c[l] = F<T>::log(a0[l], mode);
                    iv[l] = T(1) / a0[l];
                }
                break;
            }
            // l_n = (a_n - (1/n) sum_{j=1}^{n-1} (j l_j) a_{n-j}) / a_0
            for (uint32_t j = 1; j < n; ++j) term(acc.data(), kr(u, j), row(o.a, ra, n - j), first);
            std::vector<T> &num = s_num;
            if (!first) divn(acc.data(), acc.data(), n);
            for (uint32_t l = 0; l < B; ++l) {
                const T av = an ? an[l] : T(0);
                num[l] = first ? av : av - acc[l];
            }
            div0(c, num.data(), a0, u);
            break;
        }
        case HYK_OP_SIN:
        case HYK_OP_COS: {
            const uint32_t partner = (uint32_t)o.aux;
            if (n == 0) {
                const T *a0 = row(o.a, ra, 0);
                for (uint32_t l = 0; l < B; ++l) {
                    T sv, cv;
                    F<T>::sincos(a0[l], sv, cv, mode);
                    c[l] = o.op == HYK_OP_SIN ? sv : cv;
                }
                break;
            }
            // s_n = (1/n) sum_{j=1}^n j a_j c_{n-j};  c_n = -(1/n) sum_{j=1}^n j a_j s_{n-j}
            for (uint32_t j = 1; j <= n; ++j) term(acc.data(), karow(o.a, j), jr(partner, n - j), first);
            if (first) {
                for (uint32_t l = 0; l < B; ++l) c[l] = T(0);
                break;
            }
            divn(c, acc.data(), n);
            if (o.op == HYK_OP_COS)
                for (uint32_t l = 0; l < B; ++l) c[l] = -c[l];
            break;
        }
        }
        set_ka(u, n);
    }

    // State coefficient of order n+1 from the right-hand side at order n.
    void state_next(uint32_t n) {
        for (uint32_t i = 0; i < d.n_eq; ++i) {
            const T *f = row(d.rhs[i], rhs_numrow[i], n);
            T *x = jr(i, n + 1);
            if (!f) {
                for (uint32_t l = 0; l < B; ++l) x[l] = T(0);
            } else {
                divn(x, f, n + 1);
            }
            set_ka(i, n + 1);
        }
    }

    void jets() {
        for (uint32_t i = 0; i < d.n_eq; ++i) std::memcpy(jr(i, 0), &state[(size_t)i * B], sizeof(T) * B);
        // sin/cos pairs: the partner of a u-variable at order n must exist
        // before it is used at order n+1 only, so plain decomposition order works.
        // Intermediate u-variables are needed up to order p-1 only (the
        // state's order p comes from the right-hand sides at order p-1).
        for (uint32_t n = 0; n < p; ++n) {
            for (uint32_t k = 0; k < d.n_ops; ++k) op_coef(k, n);
            state_next(n);
        }
        // Event functions need every order up to p.
        if (!d.ev.empty())
            for (uint32_t k = 0; k < d.n_ops; ++k) op_coef(k, p);
    }

    // Order-n coefficient of an argument (event functions), lane l.
    T arg_coef(const hyk_arg_t &a, uint32_t n, uint32_t l) {
        switch (a.kind) {
        case HYK_ARG_U: return jr((uint32_t)a.idx, n)[l];
        case HYK_ARG_NUM: return n == 0 ? T(a.num) : T(0);
        case HYK_ARG_PAR: return n == 0 ? pars[(size_t)a.idx * B + l] : T(0);
        case HYK_ARG_TIME: return n == 0 ? thi[l] : (n == 1 ? T(1) : T(0));
        }
        return T(0);
    }

    // Step size per lane from the jets (unclamped, positive).
    void step_size(std::vector<T> &h) {
        for (uint32_t l = 0; l < B; ++l) {
            T ms = T(0), mp = T(0), mpm1 = T(0);
            for (uint32_t i = 0; i < d.n_eq; ++i) {
                const T a0 = M<T>::abs(jr(i, 0)[l]);
                const T ap = M<T>::abs(jr(i, p)[l]);
                const T apm1 = M<T>::abs(jr(i, p - 1)[l]);
                if (!(a0 <= ms)) ms = a0;
                if (!(ap <= mp)) mp = ap;
                if (!(apm1 <= mpm1)) mpm1 = apm1;
            }
            const T num = ms < T(1) ? T(1) : ms;
            T rho_m;
            if (!F<T>::rho(mp, mpm1, num, inv[p], inv[p - 1], mode, rho_m)) {
                const T rho_o = T(1) / M<T>::pow(mp / num, T(1) / T(p));
                const T rho_om1 = T(1) / M<T>::pow(mpm1 / num, T(1) / T(p - 1));
                rho_m = rho_om1 < rho_o ? rho_om1 : rho_o;
            }
            h[l] = rho_m * rhofac;
        }
    }

    // State polynomials at offsets dt (per lane): Horner's rule, or in
    // high-accuracy mode the terms x_n dt^n (powers by repeated
    // multiplication) summed from n = p down to 0 with Kahan's compensation.
    void horner(const T *dt, T *out /*[n_eq][B]*/) {
        if (ha) {
            std::vector<T> t(p + 1);
            for (uint32_t i = 0; i < d.n_eq; ++i)
                for (uint32_t l = 0; l < B; ++l) {
                    T hp = T(1);
                    for (uint32_t n = 0; n <= p; ++n) {
                        t[n] = jr(i, n)[l] * hp;
                        hp = hp * dt[l];
                    }
                    T sm = T(0), c = T(0);
                    for (uint32_t n = p + 1; n-- > 0;) {
                        const T y = t[n] - c;
                        const T u = sm + y;
                        c = (u - sm) - y;
                        sm = u;
                    }
                    out[(size_t)i * B + l] = sm;
                }
            return;
        }
        for (uint32_t i = 0; i < d.n_eq; ++i)
            for (uint32_t l = 0; l < B; ++l) {
                T acc = jr(i, p)[l];
                for (uint32_t n = p; n-- > 0;) acc = mode ? M<T>::fma(acc, dt[l], jr(i, n)[l]) : acc * dt[l] + jr(i, n)[l];
                out[(size_t)i * B + l] = acc;
            }
    }

    // One step with signed limits lim[l] (+-inf allowed).  Returns per-lane
    // outcome and h; the jets stay in J (the step's Taylor coefficients).
    void step(const T *lim, std::vector<int64_t> &oc, std::vector<T> &h) {
        jets();
        step_size(h);
        for (uint32_t l = 0; l < B; ++l) {
            T hh = lim[l] < T(0) ? -h[l] : h[l];
            if (M<T>::abs(lim[l]) < M<T>::abs(hh)) hh = lim[l];
            h[l] = hh;
            oc[l] = (hh == lim[l]) ? HYK_OUTCOME_TIME_LIMIT : HYK_OUTCOME_SUCCESS;
        }
        std::vector<T> ns((size_t)d.n_eq * B);
        horner(h.data(), ns.data());
        state.swap(ns);
        for (uint32_t l = 0; l < B; ++l) {
            const dfl<T> t = dadd(dfl<T>{thi[l], tlo[l]}, dfl<T>{h[l], T(0)});
            thi[l] = t.hi;
            tlo[l] = t.lo;
            bool fin = M<T>::isfinite(t.hi);
            for (uint32_t i = 0; i < d.n_eq && fin; ++i) fin = M<T>::isfinite(state[(size_t)i * B + l]);
            if (!fin) oc[l] = HYK_OUTCOME_ERR_NF_STATE;
        }
    }

    void copy_tc(double *tc) {
        for (uint32_t i = 0; i < d.n_eq; ++i)
            for (uint32_t n = 0; n <= p; ++n)
                for (uint32_t l = 0; l < B; ++l) tc[((size_t)i * (p + 1) + n) * B + l] = (double)jr(i, n)[l];
    }
};

template <typename T> void load(std::vector<T> &dst, const double *src, size_t n) {
    for (size_t i = 0; i < n; ++i) dst[i] = src ? T(src[i]) : T(0);
}
template <typename T> void store(double *dst, const std::vector<T> &src, size_t n) {
    for (size_t i = 0; i < n; ++i) dst[i] = (double)src[i];
}

struct PropIO {
    double *state;
    const double *pars;
    double *t_hi, *t_lo;
    const double *tf_hi, *tf_lo;
    uint64_t max_steps;
    const double *max_dt;
    const double *grid;
    uint64_t n_grid;
    double *grid_out;
    int c_output;
    std::vector<double> *c_tcs, *c_thi, *c_tlo;
    int64_t *outcome;
    double *min_h, *max_h;
    uint64_t *n_steps;
    double *last_h, *last_tc;
    uint64_t *n_iter;
};

// Batch propagate loop of the reference (restated; see the file header).
template <typename T>
int propagate(const Dec &d, uint32_t p, int mode, uint32_t B, const PropIO &io) {
    Batch<T> bt(d, p, B, mode);
    load(bt.state, io.state, (size_t)d.n_eq * B);
    load(bt.pars, io.pars, (size_t)d.n_pars * B);
    load(bt.thi, io.t_hi, B);
    load(bt.tlo, io.t_lo, B);

    std::vector<dfl<T>> rem(B);
    std::vector<char> dir(B);
    std::vector<T> maxdt(B), mn(B, M<T>::inf()), mx(B, T(0)), lim(B), h(B), lasth(B, T(0));
    std::vector<uint64_t> cnt(B, 0), gidx(B, 0);
    std::vector<int64_t> oc(B);
    for (uint32_t l = 0; l < B; ++l) {
        const dfl<T> tf = dnorm(T(io.tf_hi[l]), io.tf_lo ? T(io.tf_lo[l]) : T(0));
        rem[l] = dsub(tf, dfl<T>{bt.thi[l], bt.tlo[l]});
        dir[l] = dge(rem[l], dfl<T>{T(0), T(0)});
        maxdt[l] = io.max_dt ? T(io.max_dt[l]) : M<T>::inf();
    }
    const uint32_t ne = d.n_eq;
    // Grid: row 0 is the current state.
    if (io.grid && io.n_grid) {
        for (size_t k = 0; k < (size_t)io.n_grid * ne * B; ++k) io.grid_out[k] = std::numeric_limits<double>::quiet_NaN();
        for (uint32_t l = 0; l < B; ++l) {
            for (uint32_t i = 0; i < ne; ++i) io.grid_out[(size_t)i * B + l] = (double)bt.state[(size_t)i * B + l];
            gidx[l] = 1;
        }
    }
    if (io.c_output) {
        io.c_thi->clear();
        io.c_tlo->clear();
        io.c_tcs->clear();
        for (uint32_t l = 0; l < B; ++l) {
            io.c_thi->push_back((double)bt.thi[l]);
            io.c_tlo->push_back((double)bt.tlo[l]);
        }
    }
    uint64_t iter = 0;
    int64_t final_oc = HYK_OUTCOME_TIME_LIMIT;
    bool all_zero = true;
    for (uint32_t l = 0; l < B; ++l) all_zero = all_zero && rem[l].hi == T(0) && rem[l].lo == T(0);
    if (!all_zero) {
        std::vector<double> tcbuf;
        for (;;) {
            for (uint32_t l = 0; l < B; ++l) {
                const T tl = rem[l].hi;
                lim[l] = dir[l] ? std::min(maxdt[l], tl) : std::max(-maxdt[l], tl);
            }
            std::vector<T> t0hi = bt.thi, t0lo = bt.tlo;
            bt.step(lim.data(), oc, h);
            bool err = false;
            for (uint32_t l = 0; l < B; ++l)
                err = err || (oc[l] != HYK_OUTCOME_SUCCESS && oc[l] != HYK_OUTCOME_TIME_LIMIT);
            if (err) {
                for (uint32_t l = 0; l < B; ++l) {
                    io.outcome[l] = oc[l];
                    lasth[l] = h[l];
                }
                final_oc = 0;
                ++iter;
                break;
            }
            ++iter;
            // Grid output inside this step.  A step that ends the lane's
            // propagation (its size equals the remaining time) also takes
            // every grid row left, so rounding in the tracked remaining time
            // can never leave the last row unwritten.
            if (io.grid && io.n_grid) {
                for (uint32_t l = 0; l < B; ++l) {
                    const bool last = h[l] != T(0) && h[l] == rem[l].hi;
                    while (gidx[l] < io.n_grid) {
                        const dfl<T> g{T(io.grid[gidx[l] * B + l]), T(0)};
                        const T dt = dsub(g, dfl<T>{t0hi[l], t0lo[l]}).hi;
                        if (!(last || (dir[l] ? dt <= h[l] : dt >= h[l]))) break;
                        for (uint32_t i = 0; i < ne; ++i) {
                            T acc = bt.jr(i, p)[l];
                            for (uint32_t n = p; n-- > 0;) acc = mode ? M<T>::fma(acc, dt, bt.jr(i, n)[l]) : acc * dt + bt.jr(i, n)[l];
                            io.grid_out[(gidx[l] * ne + i) * B + l] = (double)acc;
                        }
                        ++gidx[l];
                    }
                }
            }
            for (uint32_t l = 0; l < B; ++l) {
                const T hh = h[l];
                cnt[l] += hh != T(0);
                rem[l] = (hh == rem[l].hi) ? dfl<T>{T(0), T(0)} : dsub(rem[l], dfl<T>{hh, T(0)});
                // min/max |h| only over steps whose outcome is success: a
                // step clamped by the time limit or max_delta_t is not an
                // adaptive step (the reference's pinned min_h values exclude
                // the final clamped step).
                if (hh != T(0) && oc[l] == HYK_OUTCOME_SUCCESS) {
                    const T ah = M<T>::abs(hh);
                    mn[l] = std::min(mn[l], ah);
                    mx[l] = std::max(mx[l], ah);
                }
                lasth[l] = hh;
            }
            if (io.c_output) {
                tcbuf.assign((size_t)ne * (p + 1) * B, 0.0);
                bt.copy_tc(tcbuf.data());
                io.c_tcs->insert(io.c_tcs->end(), tcbuf.begin(), tcbuf.end());
                for (uint32_t l = 0; l < B; ++l) {
                    io.c_thi->push_back((double)bt.thi[l]);
                    io.c_tlo->push_back((double)bt.tlo[l]);
                }
            }
            bool done = true;
            for (uint32_t l = 0; l < B; ++l) done = done && rem[l].hi == T(0) && rem[l].lo == T(0);
            if (done) {
                final_oc = HYK_OUTCOME_TIME_LIMIT;
                break;
            }
            if (io.max_steps != 0 && iter == io.max_steps) {
                final_oc = HYK_OUTCOME_STEP_LIMIT;
                break;
            }
        }
    }
    for (uint32_t l = 0; l < B; ++l) {
        if (final_oc != 0) io.outcome[l] = final_oc;
        io.min_h[l] = (double)mn[l];
        io.max_h[l] = (double)mx[l];
        io.n_steps[l] = cnt[l];
        if (io.last_h) io.last_h[l] = (double)lasth[l];
    }
    if (io.n_iter) *io.n_iter = iter;
    if (io.last_tc && iter > 0) bt.copy_tc(io.last_tc);
    store(io.state, bt.state, (size_t)ne * B);
    store(io.t_hi, bt.thi, B);
    store(io.t_lo, bt.tlo, B);
    return 0;
}

template <typename T>
int step_one(const Dec &d, uint32_t p, int mode, uint32_t B, double *state, const double *pars, double *t_hi,
             double *t_lo, const double *max_dt, int backward, int64_t *outcome, double *h, double *tc) {
    Batch<T> bt(d, p, B, mode);
    load(bt.state, state, (size_t)d.n_eq * B);
    load(bt.pars, pars, (size_t)d.n_pars * B);
    load(bt.thi, t_hi, B);
    load(bt.tlo, t_lo, B);
    std::vector<T> lim(B), hh(B);
    std::vector<int64_t> oc(B);
    for (uint32_t l = 0; l < B; ++l) lim[l] = max_dt ? T(max_dt[l]) : (backward ? -M<T>::inf() : M<T>::inf());
    bt.step(lim.data(), oc, hh);
    for (uint32_t l = 0; l < B; ++l) {
        outcome[l] = oc[l];
        h[l] = (double)hh[l];
    }
    if (tc) bt.copy_tc(tc);
    store(state, bt.state, (size_t)d.n_eq * B);
    store(t_hi, bt.thi, B);
    store(t_lo, bt.tlo, B);
    return 0;
}

// Per-lane propagation with events, gpu arithmetic (double, or float for the
// float32 integrator): every lane is its own batch of one, stepped exactly as
// the kernels step it (events after the step size, a terminal event ending
// the lane at its root).
struct EvRec {
    std::vector<double> t_hi, t_lo;
    std::vector<int32_t> info;
    std::vector<uint32_t> lane;
};

template <typename T>
int propagate_ev(const Dec &d, uint32_t p, uint32_t B, double *state, const double *pars, double *t_hi,
                 double *t_lo, const double *tf_hi, uint64_t max_steps, int64_t *outcome, uint64_t *n_steps,
                 uint32_t *status, double *ev_last, int32_t *ev_sign, EvRec &rec) {
    const uint32_t ne = d.n_eq, np = d.n_pars;
    std::vector<double> btd((size_t)(p + 1) * (p + 1));
    hyk_ev_btab((int)p, btd.data());
    std::vector<T> bt(btd.begin(), btd.end()), work(3 * (p + 1)), g(p + 1);
    const T cool_rel = sizeof(T) == sizeof(float) ? T(HYK_EV_COOL_REL_F) : T(HYK_EV_COOL_REL_D);
    uint32_t n_term = 0;
    std::vector<int> idx(d.ev.size());
    {
        uint32_t nn = 0;
        for (size_t k = 0; k < d.ev.size(); ++k) idx[k] = d.ev[k].terminal ? (int)n_term++ : (int)nn++;
    }
    for (uint32_t l = 0; l < B; ++l) {
        Batch<T> bq(d, p, 1, 1);
        for (uint32_t i = 0; i < ne; ++i) bq.state[i] = T(state[(size_t)i * B + l]);
        for (uint32_t i = 0; i < np; ++i) bq.pars[i] = pars ? T(pars[(size_t)i * B + l]) : T(0);
        bq.thi[0] = T(t_hi[l]);
        bq.tlo[0] = t_lo ? T(t_lo[l]) : T(0);
        dfl<T> rem = dsub(dnorm(T(tf_hi[l]), T(0)), dfl<T>{bq.thi[0], bq.tlo[0]});
        const bool dir = dge(rem, dfl<T>{T(0), T(0)});
        uint64_t nit = 0, nst = 0;
        int64_t oc = HYK_OUTCOME_TIME_LIMIT;
        uint32_t st = (rem.hi == T(0) && rem.lo == T(0)) ? HYK_LANE_DONE : 0u;
        std::vector<T> h(1);
        while (!st) {
            const T lim = dir ? std::min(M<T>::inf(), rem.hi) : std::max(-M<T>::inf(), rem.hi);
            bq.jets();
            bq.step_size(h);
            T hh = lim < T(0) ? -h[0] : h[0];
            if (std::fabs(lim) < std::fabs(hh)) hh = lim;
            int64_t soc = (hh == lim) ? HYK_OUTCOME_TIME_LIMIT : HYK_OUTCOME_SUCCESS;
            // events of the step
            const T th = bq.thi[0], tl = bq.tlo[0];
            int kt = -1, sgt = 0;
            T stt = 2;
            size_t rec0 = rec.t_hi.size();
            if (hh != T(0)) {
                const T ah = std::fabs(hh);
                for (size_t k = 0; k < d.ev.size(); ++k) {
                    if (!d.ev[k].terminal) continue;
                    const int j = idx[k];
                    T slo = 0;
                    const T last = T(ev_last[(size_t)j * B + l]);
                    if (last == last) {
                        const T cool = T(d.ev[k].cooldown);
                        const T cd = cool >= T(0) ? cool : cool_rel * (std::fabs(last) > T(1) ? std::fabs(last) : T(1));
                        const T r = cd - std::fabs(th - last);
                        if (r > T(0)) slo = r / ah;
                    }
                    if (slo >= T(1)) continue;
                    for (uint32_t n = 0; n <= p; ++n) g[n] = bq.arg_coef(d.ev[k].g, n, 0);
                    T rs = 0;
                    int rsg = 0;
                    const int nf = hyk_ev_find<T>(g.data(), 1, (int)p, hh, bt.data(), slo, T(1), d.ev[k].direction, 1,
                                                  &rs, &rsg, 1, 1, work.data());
                    if (nf > 0 && rs < stt) {
                        stt = rs;
                        kt = j;
                        sgt = rsg;
                    }
                }
                const T shi = kt >= 0 ? stt : T(1);
                for (size_t k = 0; k < d.ev.size(); ++k) {
                    if (d.ev[k].terminal) continue;
                    for (uint32_t n = 0; n <= p; ++n) g[n] = bq.arg_coef(d.ev[k].g, n, 0);
                    std::vector<T> rs(4096);
                    std::vector<int> rsg(4096);
                    const int nf = hyk_ev_find<T>(g.data(), 1, (int)p, hh, bt.data(), T(0), shi, d.ev[k].direction, 0,
                                                  rs.data(), rsg.data(), 1, 4096, work.data());
                    for (int r = 0; r < std::min(nf, 4096); ++r) {
                        const dfl<T> t = dadd(dfl<T>{th, tl}, dfl<T>{rs[r] * hh, T(0)});
                        rec.t_hi.push_back((double)t.hi);
                        rec.t_lo.push_back((double)t.lo);
                        rec.info.push_back(4 * idx[k] + rsg[r] + 1);
                        rec.lane.push_back(l);
                    }
                }
                if (kt >= 0) {
                    hh = stt * hh;
                    soc = kt;
                }
            }
            std::vector<T> ns(ne);
            bq.horner(&hh, ns.data());
            const dfl<T> t = dadd(dfl<T>{th, tl}, dfl<T>{hh, T(0)});
            bool fin = std::isfinite(t.hi);
            for (uint32_t i = 0; i < ne; ++i) fin = fin && std::isfinite(ns[i]);
            bq.state.assign(ns.begin(), ns.end());
            bq.thi[0] = t.hi;
            bq.tlo[0] = t.lo;
            ++nit;
            if (!fin) {
                rec.t_hi.resize(rec0);
                rec.t_lo.resize(rec0);
                rec.info.resize(rec0);
                rec.lane.resize(rec0);
                oc = HYK_OUTCOME_ERR_NF_STATE;
                st = HYK_LANE_STOPPED;
                break;
            }
            nst += hh != T(0);
            rem = (hh == rem.hi) ? dfl<T>{T(0), T(0)} : dsub(rem, dfl<T>{hh, T(0)});
            oc = soc;
            if (kt >= 0) {
                ev_last[(size_t)kt * B + l] = (double)t.hi;
                ev_sign[l] = sgt;
                oc = -(int64_t)kt - 1;
                st = HYK_LANE_STOPPED | HYK_LANE_EVENT;
                break;
            }
            if (rem.hi == T(0) && rem.lo == T(0)) {
                oc = HYK_OUTCOME_TIME_LIMIT;
                st = HYK_LANE_DONE;
                break;
            }
            if (max_steps != 0 && nit >= max_steps) {
                oc = HYK_OUTCOME_STEP_LIMIT;
                st = HYK_LANE_STOPPED;
                break;
            }
        }
        for (uint32_t i = 0; i < ne; ++i) state[(size_t)i * B + l] = (double)bq.state[i];
        t_hi[l] = (double)bq.thi[0];
        if (t_lo) t_lo[l] = (double)bq.tlo[0];
        outcome[l] = oc;
        n_steps[l] = nst;
        status[l] = st;
    }
    return 0;
}

}  // namespace

extern "C" {

const char *hyko_last_error(void) { return g_err.c_str(); }

// Per-lane propagation to tf_hi with events (gpu arithmetic; prec 0 double,
// 2 float).  The
// non-terminal roots come back in malloc'ed arrays (free with hyko_free) in
// the order the kernels record them per lane: (time hi, time lo, info =
// 4 * event index + direction + 1, lane).  ev_last (n_terminal, B) and ev_sign
// (B) are in/out like the kernels' buffers.
int hyko_propagate_ev(const hyk_decomp_t *dd, uint32_t order, uint32_t B, double *state, const double *pars,
                      double *t_hi, double *t_lo, const double *tf_hi, uint64_t max_steps, int64_t *outcome,
                      uint64_t *n_steps, uint32_t *status, double *ev_last, int32_t *ev_sign, uint64_t *n_rec,
                      double **rec_t_hi, double **rec_t_lo, int32_t **rec_info, uint32_t **rec_lane, int prec) {
    Dec d;
    if (!load_dec(dd, d)) return HYK_ERR_INVALID;
    if (order < 2 || B == 0) {
        g_err = "invalid order or batch size";
        return HYK_ERR_INVALID;
    }
    EvRec rec;
    const int r = prec == 2 ? propagate_ev<float>(d, order, B, state, pars, t_hi, t_lo, tf_hi, max_steps, outcome,
                                                  n_steps, status, ev_last, ev_sign, rec)
                            : propagate_ev<double>(d, order, B, state, pars, t_hi, t_lo, tf_hi, max_steps, outcome,
                                                   n_steps, status, ev_last, ev_sign, rec);
    auto dup = [](const void *src, size_t bytes) {
        void *q = std::malloc(std::max<size_t>(bytes, 8));
        if (bytes) std::memcpy(q, src, bytes);
        return q;
    };
    *n_rec = rec.t_hi.size();
    *rec_t_hi = (double *)dup(rec.t_hi.data(), rec.t_hi.size() * sizeof(double));
    *rec_t_lo = (double *)dup(rec.t_lo.data(), rec.t_lo.size() * sizeof(double));
    *rec_info = (int32_t *)dup(rec.info.data(), rec.info.size() * sizeof(int32_t));
    *rec_lane = (uint32_t *)dup(rec.lane.data(), rec.lane.size() * sizeof(uint32_t));
    return r;
}

// The kernels' root finder on one polynomial (tests of hyk_events.h on the host).
int hyko_ev_find(const double *g, uint32_t p, double h, double s_lo, double s_hi, int dir, int first_only, double *rs,
                 int32_t *rsg, int maxr) {
    std::vector<double> bt((size_t)(p + 1) * (p + 1)), work(3 * (p + 1));
    hyk_ev_btab((int)p, bt.data());
    std::vector<int> sg(std::max(maxr, 1));
    const int n = hyk_ev_find<double>(g, 1, (int)p, h, bt.data(), s_lo, s_hi, dir, first_only, rs, sg.data(), 1, maxr,
                                      work.data());
    for (int i = 0; i < std::min(n, maxr); ++i) rsg[i] = sg[i];
    return n;
}

// One step of a batch of B lanes (host arrays, [var][lane]).  prec: 0 double,
// 1 binary128, 2 float (the values are converted from and to double exactly).
int hyko_step(const hyk_decomp_t *dd, uint32_t order, int prec, int mode, uint32_t B, double *state,
              const double *pars, double *t_hi, double *t_lo, const double *max_dt, int backward,
              int64_t *outcome, double *h, double *tc) {
    Dec d;
    if (!load_dec(dd, d)) return HYK_ERR_INVALID;
    if (order < 2 || B == 0) {
        g_err = "invalid order or batch size";
        return HYK_ERR_INVALID;
    }
    if (prec == 0) return step_one<double>(d, order, mode, B, state, pars, t_hi, t_lo, max_dt, backward, outcome, h, tc);
    if (prec == 2) return step_one<float>(d, order, mode, B, state, pars, t_hi, t_lo, max_dt, backward, outcome, h, tc);
    return step_one<qreal>(d, order, mode, B, state, pars, t_hi, t_lo, max_dt, backward, outcome, h, tc);
}

// Batch propagation (until/for/grid) of B lanes.  With c_output != 0 the
// per-iteration Taylor coefficients (c_n, n_eq, order+1, B) and end times
// (c_n+1, B) are returned in malloc'ed buffers (free with hyko_free); c_n is
// n_iter, or n_iter - 1 when a non-finite state stopped the batch (the
// failing iteration is not recorded).
int hyko_propagate(const hyk_decomp_t *dd, uint32_t order, int prec, int mode, uint32_t B, double *state,
                   const double *pars, double *t_hi, double *t_lo, const double *tf_hi, const double *tf_lo,
                   uint64_t max_steps, const double *max_dt, const double *grid, uint64_t n_grid,
                   double *grid_out, int c_output, double **c_tcs, double **c_thi, double **c_tlo,
                   uint64_t *n_iter, int64_t *outcome, double *min_h, double *max_h, uint64_t *n_steps,
                   double *last_h, double *last_tc, uint64_t *c_n) {
    Dec d;
    if (!load_dec(dd, d)) return HYK_ERR_INVALID;
    if (order < 2 || B == 0) {
        g_err = "invalid order or batch size";
        return HYK_ERR_INVALID;
    }
    std::vector<double> vt, vh, vl;
    PropIO io{state,  pars,     t_hi,   t_lo,  tf_hi, tf_lo, max_steps, max_dt, grid,    n_grid,  grid_out,
              c_output, &vt, &vh, &vl, outcome, min_h, max_h, n_steps, last_h, last_tc, n_iter};
    const int r = prec == 0   ? propagate<double>(d, order, mode, B, io)
                  : prec == 2 ? propagate<float>(d, order, mode, B, io)
                              : propagate<qreal>(d, order, mode, B, io);
    if (c_output) {
        auto dup = [](const std::vector<double> &v) {
            double *p = (double *)std::malloc(sizeof(double) * std::max<size_t>(v.size(), 1));
            if (!v.empty()) std::memcpy(p, v.data(), sizeof(double) * v.size());
            return p;
        };
        *c_tcs = dup(vt);
        *c_thi = dup(vh);
        *c_tlo = dup(vl);
        if (c_n) *c_n = vh.size() / B - 1;
    }
    return r;
}

void hyko_free(void *p) { std::free(p); }

// Evaluate one of the deterministic elementary functions on the host:
// fn 0 exp, 1 log, 2 sin, 3 cos, 4 pow(x, a[i]), 5 rho(x, a, num=1, 1/20, 1/19).
void hyko_dm_eval(int fn, const double *x, const double *a, double *out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) {
        double s, c;
        switch (fn) {
        case 0: out[i] = hyk_dm_exp(x[i]); break;
        case 1: out[i] = hyk_dm_log(x[i]); break;
        case 2: hyk_dm_sincos(x[i], &s, &c); out[i] = s; break;
        case 3: hyk_dm_sincos(x[i], &s, &c); out[i] = c; break;
        case 4: out[i] = hyk_dm_pow(x[i], a[i]); break;
        case 5: out[i] = hyk_dm_rho(x[i], a[i], 1.0, 1.0 / 20, 1.0 / 19); break;
        default: {
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
}

// Ensemble propagate_until over n_lanes lanes split into batches of B lanes
// (the reference's ensemble of batch integrators, heyoka/_ensemble_impl.py:23-68),
// run on `n_threads` OpenMP threads.  Arrays are (var, n_lanes) with row
// stride n_lanes.  Returns the total number of non-zero steps in *total_steps.
int hyko_ensemble_until(const hyk_decomp_t *dd, uint32_t order, int mode, uint32_t B, uint64_t n_lanes,
                        double *state, const double *pars, double *t_hi, double *t_lo, const double *tf,
                        int n_threads, int64_t *outcome, double *min_h, double *max_h, uint64_t *n_steps,
                        int prec) {
    Dec d;
    if (!load_dec(dd, d)) return HYK_ERR_INVALID;
    if (order < 2 || B == 0) {
        g_err = "invalid order or batch size";
        return HYK_ERR_INVALID;
    }
    const uint64_t nb = (n_lanes + B - 1) / B;
    const uint32_t ne = d.n_eq, np = d.n_pars;
    int rc = 0;
#if defined(_OPENMP)
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t b = 0; b < (int64_t)nb; ++b) {
        const uint64_t l0 = (uint64_t)b * B;
        const uint32_t bl = (uint32_t)std::min<uint64_t>(B, n_lanes - l0);
        std::vector<double> st((size_t)ne * bl), pa((size_t)np * bl), th(bl), tl(bl), tfh(bl);
        for (uint32_t i = 0; i < ne; ++i)
            for (uint32_t l = 0; l < bl; ++l) st[(size_t)i * bl + l] = state[(size_t)i * n_lanes + l0 + l];
        for (uint32_t i = 0; i < np; ++i)
            for (uint32_t l = 0; l < bl; ++l) pa[(size_t)i * bl + l] = pars[(size_t)i * n_lanes + l0 + l];
        for (uint32_t l = 0; l < bl; ++l) {
            th[l] = t_hi[l0 + l];
            tl[l] = t_lo ? t_lo[l0 + l] : 0.0;
            tfh[l] = tf[l0 + l];
        }
        std::vector<int64_t> oc(bl);
        std::vector<double> mn(bl), mx(bl);
        std::vector<uint64_t> ns(bl);
        std::vector<double> vt, vh, vl;
        PropIO io{st.data(), pa.data(), th.data(), tl.data(), tfh.data(), nullptr, 0, nullptr, nullptr, 0, nullptr,
                  0, &vt, &vh, &vl, oc.data(), mn.data(), mx.data(), ns.data(), nullptr, nullptr, nullptr};
        if (prec == 2)
            propagate<float>(d, order, mode, bl, io);
        else
            propagate<double>(d, order, mode, bl, io);
        for (uint32_t i = 0; i < ne; ++i)
            for (uint32_t l = 0; l < bl; ++l) state[(size_t)i * n_lanes + l0 + l] = st[(size_t)i * bl + l];
        for (uint32_t l = 0; l < bl; ++l) {
            t_hi[l0 + l] = th[l];
            if (t_lo) t_lo[l0 + l] = tl[l];
            outcome[l0 + l] = oc[l];
            min_h[l0 + l] = mn[l];
            max_h[l0 + l] = mx[l];
            n_steps[l0 + l] = ns[l];
        }
    }
    return rc;
}

int hyko_max_threads(void) {
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
