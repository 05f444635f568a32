// Compiled CPU batch stepper: the timed CPU baseline (TEST INFRASTRUCTURE).
//
// Only bench.py's CPU-baseline leg and tests/ use this file; the GPU product
// path never does.  The reference integrates ensembles with heyoka's
// LLVM-compiled batch stepper: taylor_adaptive_batch<double>::propagate_until
// (reached from heyoka/expose_batch_integrators.cpp:279-314) on batches of
// SIMD width, fanned out over host threads by ensemble_propagate_until
// (heyoka/_ensemble_impl.py:23-68).  That library cannot be built here, so
// this file stands in for it with the same structure:
//  * the Taylor recurrences of the system are generated code (libhyk's code
//    generator, hyk_codegen_check with verbose = 4: straight-line code, every
//    index a compile-time constant, the reference's arithmetic: no fused
//    multiply-adds, true divisions, the C library's elementary functions),
//    included below as HYK_JETS_INC and compiled with -O3;
//  * the element type is a batch of HYK_B lanes (GCC vector extension), so
//    every operation of the recurrences acts on HYK_B trajectories at once;
//  * the propagate loop is the oracle's restatement of the reference's batch
//    loop (hyk_oracle.cpp, propagate<T>): finished lanes take zero steps until
//    every lane of the batch is done, a non-finite state stops the batch;
//  * OpenMP spreads batches over the host threads (dynamic schedule).
// Built with -ffp-contract=off, so it computes the oracle's "pin" arithmetic.

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef HYK_B
#define HYK_B 8
#endif

typedef double hyk_vd __attribute__((vector_size(8 * HYK_B)));

// A batch of HYK_B doubles with the arithmetic operators; a double converts
// to the batch with every lane equal to it.
struct hyk_v {
    hyk_vd v;
    hyk_v() = default;
    hyk_v(double x) : v(hyk_vd{} + x) {}
    hyk_v(hyk_vd x) : v(x) {}
};
static inline hyk_v operator+(hyk_v a, hyk_v b) { return a.v + b.v; }
static inline hyk_v operator-(hyk_v a, hyk_v b) { return a.v - b.v; }
static inline hyk_v operator*(hyk_v a, hyk_v b) { return a.v * b.v; }
static inline hyk_v operator/(hyk_v a, hyk_v b) { return a.v / b.v; }
static inline hyk_v operator-(hyk_v a) { return -a.v; }
// Element-wise C library functions (the reference arithmetic's elementary functions).
static inline hyk_v pow(hyk_v x, double a) {
    hyk_v r;
    for (int l = 0; l < HYK_B; ++l) r.v[l] = std::pow(x.v[l], a);
    return r;
}
static inline hyk_v exp(hyk_v x) {
    hyk_v r;
    for (int l = 0; l < HYK_B; ++l) r.v[l] = std::exp(x.v[l]);
    return r;
}
static inline hyk_v log(hyk_v x) {
    hyk_v r;
    for (int l = 0; l < HYK_B; ++l) r.v[l] = std::log(x.v[l]);
    return r;
}
static inline hyk_v sqrt(hyk_v x) {
    hyk_v r;
    for (int l = 0; l < HYK_B; ++l) r.v[l] = std::sqrt(x.v[l]);
    return r;
}
static inline void sincos(hyk_v x, hyk_v *s, hyk_v *c) {
    for (int l = 0; l < HYK_B; ++l) {
        s->v[l] = std::sin(x.v[l]);
        c->v[l] = std::cos(x.v[l]);
    }
}

typedef hyk_v hyk_real;
#define __device__
#define __noinline__
#define __forceinline__ inline
#define __restrict__ __restrict
static inline void __syncwarp() {}
#define HYK_WARP_SYNC()
static inline double hyk_inf() { return HUGE_VAL; }

#define HYK_STR2(x) #x
#define HYK_STR(x) HYK_STR2(x)
#include HYK_STR(HYK_JETS_INC)

namespace {

struct dfl {
    double hi, lo;
};
inline void two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
inline void fast_two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    e = b - (s - a);
}
inline dfl dadd(dfl x, dfl y) {
    double s, e;
    two_sum(x.hi, y.hi, s, e);
    e = e + (x.lo + y.lo);
    dfl r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
inline dfl dsub(dfl x, dfl y) { return dadd(x, dfl{-y.hi, -y.lo}); }

constexpr int64_t OC_SUCCESS = -4294967297LL;
constexpr int64_t OC_TIME_LIMIT = -4294967299LL;
constexpr int64_t OC_ERR_NF_STATE = -4294967300LL;

struct Args {
    uint64_t n, ld;
    const double *state_in, *pars;
    double t0;
    const double *tf;
    double *state_out;
    int64_t *outcome;
    double *min_h, *max_h;
    uint64_t *n_steps;
};

// propagate_until(tf[lane]) of the lanes l0 .. l0 + HYK_B - 1 (the last
// batch is padded with copies of the last lane), from time t0 (low part zero).
void run_batch(const Args &a, uint64_t l0) {
    constexpr int B = HYK_B, NE = HYK_NEQ, P = HYK_ORDER;
    alignas(64) hyk_v S[HYK_NSLOT];
    uint64_t lane[B];
    for (int l = 0; l < B; ++l) lane[l] = std::min<uint64_t>(l0 + l, a.n - 1);
    for (int i = 0; i < NE; ++i)
        for (int l = 0; l < B; ++l) HYK_SX(i, 0).v[l] = a.state_in[(uint64_t)i * a.ld + lane[l]];
    for (int k = 0; k < HYK_NPARS; ++k)
        for (int l = 0; l < B; ++l) HYK_PAR(k).v[l] = a.pars[(uint64_t)k * a.ld + lane[l]];
    const double e1 = std::exp(1.0);
    const double rhofac = 1.0 / (e1 * e1) * std::exp((-7.0 / 10.0) / (P - 1.0));
    double thi[B], tlo[B], mn[B], mx[B], h[B], lim[B];
    dfl rem[B];
    bool dir[B];
    uint64_t cnt[B];
    int64_t oc[B];
    bool any = false;
    for (int l = 0; l < B; ++l) {
        thi[l] = a.t0;
        tlo[l] = 0.0;
        dfl tf;
        two_sum(a.tf[lane[l]], 0.0, tf.hi, tf.lo);
        rem[l] = dsub(tf, dfl{thi[l], tlo[l]});
        dir[l] = rem[l].hi > 0.0 || (rem[l].hi == 0.0 && rem[l].lo >= 0.0);
        mn[l] = HUGE_VAL;
        mx[l] = 0.0;
        cnt[l] = 0;
        oc[l] = OC_TIME_LIMIT;
        any = any || rem[l].hi != 0.0 || rem[l].lo != 0.0;
    }
    int64_t final_oc = OC_TIME_LIMIT;
    while (any) {
        for (int l = 0; l < B; ++l) lim[l] = dir[l] ? std::min(HUGE_VAL, rem[l].hi) : std::max(-HUGE_VAL, rem[l].hi);
        hyk_v t0;
        for (int l = 0; l < B; ++l) t0.v[l] = thi[l];
        hyk_jets(S, t0);
        for (int l = 0; l < B; ++l) {
            double ms = 0.0, mp = 0.0, mq = 0.0;
            for (int i = 0; i < NE; ++i) {
                const double x0 = std::fabs(HYK_SX(i, 0).v[l]);
                const double xp = std::fabs(HYK_SX(i, P).v[l]);
                const double xq = std::fabs(HYK_SX(i, P - 1).v[l]);
                if (!(x0 <= ms)) ms = x0;
                if (!(xp <= mp)) mp = xp;
                if (!(xq <= mq)) mq = xq;
            }
            const double num = ms < 1.0 ? 1.0 : ms;
            const double rho_o = 1.0 / std::pow(mp / num, 1.0 / (double)P);
            const double rho_om1 = 1.0 / std::pow(mq / num, 1.0 / (double)(P - 1));
            const double rho_m = rho_om1 < rho_o ? rho_om1 : rho_o;
            double hh = rho_m * rhofac;
            hh = lim[l] < 0.0 ? -hh : hh;
            if (std::fabs(lim[l]) < std::fabs(hh)) hh = lim[l];
            h[l] = hh;
            oc[l] = (hh == lim[l]) ? OC_TIME_LIMIT : OC_SUCCESS;
        }
        // Horner update of all lanes at once.
        hyk_v hv;
        for (int l = 0; l < B; ++l) hv.v[l] = h[l];
        hyk_v xn[NE];
        for (int i = 0; i < NE; ++i) {
            hyk_v acc = HYK_SX(i, P);
            for (int n = P; n-- > 0;) acc = acc * hv + HYK_SX(i, n);
            xn[i] = acc;
        }
        bool err = false;
        for (int l = 0; l < B; ++l) {
            const dfl t = dadd(dfl{thi[l], tlo[l]}, dfl{h[l], 0.0});
            thi[l] = t.hi;
            tlo[l] = t.lo;
            bool fin = std::isfinite(t.hi);
            for (int i = 0; i < NE && fin; ++i) fin = std::isfinite(xn[i].v[l]);
            if (!fin) oc[l] = OC_ERR_NF_STATE;
            err = err || (oc[l] != OC_SUCCESS && oc[l] != OC_TIME_LIMIT);
        }
        for (int i = 0; i < NE; ++i) HYK_SX(i, 0) = xn[i];
        if (err) {
            final_oc = 0;
            break;
        }
        bool done = true;
        for (int l = 0; l < B; ++l) {
            const double hh = h[l];
            cnt[l] += hh != 0.0;
            rem[l] = (hh == rem[l].hi) ? dfl{0.0, 0.0} : dsub(rem[l], dfl{hh, 0.0});
            if (hh != 0.0 && oc[l] == OC_SUCCESS) {
                const double ah = std::fabs(hh);
                mn[l] = std::min(mn[l], ah);
                mx[l] = std::max(mx[l], ah);
            }
            done = done && rem[l].hi == 0.0 && rem[l].lo == 0.0;
        }
        if (done) break;
    }
    for (int l = 0; l < B && l0 + l < a.n; ++l) {
        const uint64_t j = l0 + l;
        for (int i = 0; i < NE; ++i) a.state_out[(uint64_t)i * a.ld + j] = HYK_SX(i, 0).v[l];
        a.outcome[j] = final_oc != 0 ? final_oc : oc[l];
        a.min_h[j] = mn[l];
        a.max_h[j] = mx[l];
        a.n_steps[j] = cnt[l];
    }
}

}  // namespace

// propagate_until(tf[lane]) of n lanes ([var][lane] arrays with leading
// dimension ld) from time t0, batches of HYK_B lanes over n_threads host
// threads (0: all).  Returns the number of threads used.
extern "C" int hyk_cpu_until(uint64_t n, uint64_t ld, const double *state_in, const double *pars, double t0, const double *tf,
                             int n_threads, double *state_out, int64_t *outcome, double *min_h, double *max_h,
                             uint64_t *n_steps) {
    if (n == 0) return 0;
    const Args a{n, ld, state_in, pars, t0, tf, state_out, outcome, min_h, max_h, n_steps};
    const int nt = n_threads > 0 ? n_threads : omp_get_max_threads();
    const int64_t nb = (int64_t)((n + HYK_B - 1) / HYK_B);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t b = 0; b < nb; ++b) run_batch(a, (uint64_t)b * HYK_B);
    return nt;
}

extern "C" int hyk_cpu_batch_width(void) { return HYK_B; }
