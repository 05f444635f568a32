/*
 * hyk_events.h - roots of an event function's Taylor polynomial over a step.
 *
 * One source for the generated GPU kernels and the CPU oracle (included after
 * hyk_dmath.h, whose HYK_DM_* macros it uses), so both find the same roots
 * bit for bit.
 *
 * Problem.  At the start of a step of signed size h the integrator has the
 * Taylor coefficients g_0..g_p of an event function g(t).  With t = t0 + h s,
 * q(s) = sum_n a_n s^n, a_n = g_n h^n, is g over the step for s in [0, 1].
 * The roots of q in (s_lo, s_hi] are wanted in increasing order, with the
 * sign of dg/dt at each root (the direction of the event).
 *
 * Method (the event detection of the reference, heyoka's t_event/nt_event,
 * restated from its published description: root isolation on the step's
 * Taylor polynomial with Descartes' rule of signs, then refinement):
 *  - quick exclusion: |a_0| > sum_{n>=1} |a_n| means q has no root in [0, 1];
 *  - otherwise a depth-first walk over the dyadic intervals [i 2^-d,
 *    (i+1) 2^-d] of [0, 1]: the Bernstein coefficients of q on the interval
 *    (Taylor shift by its left end, scaling by its width, conversion with the
 *    ratios C(k,i)/C(p,i)) have V sign changes; V = 0 means no root, V = 1
 *    one root, V >= 2 a split into the two halves (up to HYK_EV_DEPTH levels);
 *  - an interval with V = 1 (or at the deepest level) whose end values have
 *    opposite signs is refined by bisection to adjacent numbers; a zero value
 *    at the right end is a root there.
 * Every operation is an IEEE add, multiply or fused multiply-add in a fixed
 * order, in the integrator's precision R (double, or float for the float32
 * integrator, whose dyadic walk stops at depth 22 so that the interval ends
 * i 2^-d stay exact).
 */
#ifndef HYK_EVENTS_H
#define HYK_EVENTS_H

#define HYK_EV_DEPTH 40

/* Automatic cooldown of a terminal event that triggered at time t:
 * REL * max(1, |t|), about 4500 units in the last place of t in either
 * precision (a root found again this close after the trigger is the same root). */
#define HYK_EV_COOL_REL_D 1e-12
#define HYK_EV_COOL_REL_F 5e-4f

#if !defined(__CUDACC_RTC__)
/* C(k, i) / C(p, i) for 0 <= i <= k <= p, row-major (p + 1) x (p + 1);
 * entries with i > k are zero.  Host code (the code generator prints the
 * table into the kernel source; the oracle calls it directly). */
static inline void hyk_ev_btab(int p, double *bt) {
    for (int k = 0; k <= p; ++k)
        for (int i = 0; i <= p; ++i) {
            double r = 0.0;
            if (i <= k) {
                r = 1.0;
                for (int j = 0; j < i; ++j) r = r * ((double)(k - j) / (double)(p - j));
            }
            bt[k * (p + 1) + i] = r;
        }
}
#endif

HYK_DM_FN double hyk_ev_fma(double a, double b, double c) { return HYK_DM_FMA(a, b, c); }
HYK_DM_FN float hyk_ev_fma(float a, float b, float c) { return HYK_DM_FMAF(a, b, c); }
HYK_DM_FN int hyk_ev_finite(double x) { return (HYK_DM_BITS(x) & 0x7ff0000000000000ULL) != 0x7ff0000000000000ULL; }
HYK_DM_FN int hyk_ev_finite(float x) { return (HYK_DM_FBITS(x) & 0x7f800000u) != 0x7f800000u; }

template <typename R> HYK_DM_FN R hyk_ev_q(const R *a, int p, R s) {
    R r = a[p];
    for (int n = p - 1; n >= 0; --n) r = hyk_ev_fma(r, s, a[n]);
    return r;
}

template <typename R> HYK_DM_FN R hyk_ev_dq(const R *a, int p, R s) {
    R r = (R)p * a[p];
    for (int n = p - 1; n >= 1; --n) r = hyk_ev_fma(r, s, (R)n * a[n]);
    return r;
}

/* Sign changes of the Bernstein coefficients of q on [lo, lo + w]
 * (c and b are work arrays of p + 1 numbers). */
template <typename R>
HYK_DM_FN int hyk_ev_changes(const R *a, int p, R lo, R w, const R *bt, R *c, R *b) {
    for (int k = 0; k <= p; ++k) c[k] = a[k];
    for (int k = 0; k < p; ++k)
        for (int j = p - 1; j >= k; --j) c[j] = hyk_ev_fma(c[j + 1], lo, c[j]);
    R wk = 1;
    for (int k = 0; k <= p; ++k) {
        c[k] = c[k] * wk;
        wk = wk * w;
    }
    for (int k = 0; k <= p; ++k) {
        R acc = c[0] * bt[k * (p + 1)];
        for (int i = 1; i <= k; ++i) acc = hyk_ev_fma(bt[k * (p + 1) + i], c[i], acc);
        b[k] = acc;
    }
    int v = 0, last = 0;
    for (int k = 0; k <= p; ++k) {
        const int sg = b[k] > 0 ? 1 : (b[k] < 0 ? -1 : 0);
        if (sg == 0) continue;
        if (last != 0 && sg != last) ++v;
        last = sg;
    }
    return v;
}

/* Roots of q in (s_lo, s_hi] with direction dir (0: any, +1: dg/dt > 0,
 * -1: dg/dt < 0), in increasing order.  g: coefficients g_0..g_p at stride
 * gs; work: 3 (p + 1) numbers.  Stores at most maxr roots (rs[k * rstride]:
 * s, rsg[k * rstride]: direction) and returns how many roots it found, which
 * exceeds maxr when some were not stored; with first_only the walk stops at
 * the first root. */
template <typename R>
HYK_DM_FN int hyk_ev_find(const R *g, long gs, int p, R h, const R *bt, R s_lo, R s_hi, int dir, int first_only, R *rs,
                          int *rsg, long rstride, int maxr, R *work) {
    R *a = work, *c = work + (p + 1), *b = work + 2 * (p + 1);
    const int depth = sizeof(R) == sizeof(float) ? 22 : HYK_EV_DEPTH;
    R hp = 1;
    for (int n = 0; n <= p; ++n) {
        a[n] = g[(long)n * gs] * hp;
        hp = hp * h;
    }
    R sum = 0;
    for (int n = 1; n <= p; ++n) sum = sum + (a[n] < 0 ? -a[n] : a[n]);
    const R a0 = a[0] < 0 ? -a[0] : a[0];
    if (!hyk_ev_finite(sum) || !hyk_ev_finite(a0)) return 0;
    if (a0 > sum) return 0;
    const int hs = h > 0 ? 1 : (h < 0 ? -1 : 0);
    int nr = 0, d = 0;
    long long i = 0;
    R scale = 1; /* 2^-d */
    for (;;) {
        const R lo = (R)i * scale, hi = (R)(i + 1) * scale;
        if (lo >= s_hi) break; /* intervals come in increasing order */
        if (hi > s_lo) {
            const int v = hyk_ev_changes(a, p, lo, scale, bt, c, b);
            if (v >= 2 && d < depth) {
                ++d;
                i = 2 * i;
                scale = scale * (R)0.5;
                continue;
            }
            if (v >= 1) {
                R l = lo, r = hi, root = -1;
                R fl = hyk_ev_q(a, p, l), fr = hyk_ev_q(a, p, r);
                if (fr == 0) {
                    root = r;
                } else if (fl != 0 && ((fl < 0) != (fr < 0))) {
                    for (int it = 0; it < 200; ++it) {
                        const R m = l + (R)0.5 * (r - l);
                        if (!(m > l && m < r)) break;
                        const R fm = hyk_ev_q(a, p, m);
                        if (fm == 0) {
                            l = m;
                            r = m;
                            break;
                        }
                        if ((fm < 0) == (fl < 0)) {
                            l = m;
                            fl = fm;
                        } else {
                            r = m;
                        }
                    }
                    root = l + (R)0.5 * (r - l);
                }
                if (root > s_lo && root <= s_hi) {
                    const R dq = hyk_ev_dq(a, p, root);
                    const int sg = (dq > 0 ? 1 : (dq < 0 ? -1 : 0)) * hs;
                    if (dir == 0 || sg == dir) {
                        if (nr < maxr) {
                            rs[(long)nr * rstride] = root;
                            rsg[(long)nr * rstride] = sg;
                        }
                        ++nr;
                        if (first_only) return nr;
                    }
                }
            }
        }
        while (d > 0 && (i & 1)) {
            i >>= 1;
            --d;
            scale = scale * (R)2;
        }
        if (d == 0) break;
        ++i;
    }
    return nr;
}

#endif
