/*
 * hyk_fuse.h - sums of squares and sums of scaled terms fused into one
 * recurrence.
 *
 * Shared by the code generator (both kernel forms) and the CPU oracle's GPU
 * arithmetic, so that both make the same choice.  The reference's
 * decomposition writes x^2 + y^2 + z^2 as squares and sums, each its own
 * u-variable; at order n every square costs a product that starts its
 * convolution and a doubling, and every sum one more operation, none of them
 * a fused multiply-add.  A tree of ADDs whose leaves are squares, every inner
 * node read by nothing else, plus at most one other operand a at the root, is
 * computed at its root as
 *     c_n = a_n + sum_i (x_i^2)_n
 * in one chain: s = sum_i sum_{j < n/2} x_i,j x_i,n-j (leaf by leaf, j
 * ascending: a product, then fused multiply-adds), c = fma(2, s, a_n) (s + s
 * without a), then c = fma(x_i,n/2, x_i,n/2, c) for every leaf at even n
 * (at order 0: c = a_0, then the same fused multiply-adds); the inner squares
 * and sums are computed nowhere.  Only where the leaves' operands and a are
 * u-variables that vary in time and are not negations (whose signs the
 * generator folds into their readers), and with at most HYK_FUSE_MAX leaves.
 * The reference's arithmetic (pin mode) keeps the squares and sums as they
 * are.
 *
 * Sums of scaled terms likewise (the N-body accelerations: sum_j m_j t_j):
 * a tree of ADDs and SUBs whose leaves are products of a number and a
 * u-variable, possibly negated, every inner node read by nothing else, plus
 * at most one other operand a at the root (added, never subtracted), is
 * computed at its root as c_n = a_n + sum_i k_i t_i,n in one chain: c = a_n
 * (k_1 t_1,n without a), then c = fma(k_i, t_i,n, c) leaf by leaf, with at
 * most HYK_FUSE_MAX leaves; the signs of the subtrahends and negations are
 * folded into the numbers k_i, and the products, negations and inner sums
 * are computed nowhere.  A root is one kind or the other, never both.
 */
#ifndef HYK_FUSE_H
#define HYK_FUSE_H

#include <stdint.h>

#include <functional>
#include <vector>

#include "hyk.h"

#define HYK_FUSE_MAX 4

#define HYK_FUSE_SQ 1 /* a sum of squares */
#define HYK_FUSE_SC 2 /* a sum of scaled terms */

struct HykFusePlan {
    std::vector<uint8_t> fuse;                 // per operation: HYK_FUSE_SQ or HYK_FUSE_SC at a root, else 0
    std::vector<uint8_t> dead;                 // per operation: a square, product, negation or sum absorbed
    std::vector<int32_t> addend;               // per root: the u-variable a (-1: none)
    std::vector<std::vector<int32_t>> leaves;  // per root: the u-variables squared or scaled, in order
    std::vector<std::vector<double>> scales;   // per HYK_FUSE_SC root: each leaf's number
};

static inline HykFusePlan hyk_fuse_plan(uint32_t n_eq, uint32_t n_ops, const hyk_uop_t *ops, const hyk_arg_t *rhs,
                                        uint32_t n_ev, const hyk_event_t *ev) {
    HykFusePlan pl;
    pl.fuse.assign(n_ops, 0);
    pl.dead.assign(n_ops, 0);
    pl.addend.assign(n_ops, -1);
    pl.leaves.assign(n_ops, {});
    pl.scales.assign(n_ops, {});
    const uint32_t nu = n_eq + n_ops;
    std::vector<uint32_t> uses(nu, 0);
    auto use = [&](const hyk_arg_t &a) {
        if (a.kind == HYK_ARG_U && a.idx >= 0 && (uint32_t)a.idx < nu) ++uses[(uint32_t)a.idx];
    };
    for (uint32_t k = 0; k < n_ops; ++k) {
        use(ops[k].a);
        use(ops[k].b);
    }
    for (uint32_t i = 0; i < n_eq; ++i) use(rhs[i]);
    for (uint32_t e = 0; e < n_ev; ++e) use(ev[e].g);
    // constant in time: every operand a number, a parameter or a constant operation
    std::vector<uint8_t> cst(nu, 0);
    for (uint32_t k = 0; k < n_ops; ++k) {
        auto kc = [&](const hyk_arg_t &a) {
            return a.kind == HYK_ARG_NONE || a.kind == HYK_ARG_NUM || a.kind == HYK_ARG_PAR ||
                   (a.kind == HYK_ARG_U && cst[(uint32_t)a.idx]);
        };
        cst[n_eq + k] = kc(ops[k].a) && kc(ops[k].b);
    }
    // a u-variable that varies in time and is not a negation
    auto plainvar = [&](const hyk_arg_t &a) {
        if (a.kind != HYK_ARG_U) return false;
        const uint32_t u = (uint32_t)a.idx;
        return u < n_eq || (ops[u - n_eq].op != HYK_OP_NEG && !cst[u]);
    };
    // The leaves an operand contributes when absorbed: a square read only
    // here (its operand), or a sum of squares without an addend read only
    // here (its leaves); none otherwise.
    auto absorbable = [&](const hyk_arg_t &a, std::vector<int32_t> &lv) {
        if (a.kind != HYK_ARG_U || (uint32_t)a.idx < n_eq || uses[(uint32_t)a.idx] != 1) return false;
        const uint32_t k = (uint32_t)a.idx - n_eq;
        if (ops[k].op == HYK_OP_SQUARE && plainvar(ops[k].a)) {
            lv.assign(1, ops[k].a.idx);
            return true;
        }
        if (ops[k].op == HYK_OP_ADD && pl.fuse[k] == HYK_FUSE_SQ && pl.addend[k] < 0) {
            lv = pl.leaves[k];
            return true;
        }
        return false;
    };
    // The scaled leaves an operand contributes when absorbed (its number in
    // sc, times sign): a product of a number and a plain variable read only
    // here, the negation (read only here) of such a product, or a sum of
    // scaled terms without an addend read only here; none otherwise.  The
    // operations it absorbs go to `gone`.
    std::function<bool(const hyk_arg_t &, double, std::vector<int32_t> &, std::vector<double> &,
                       std::vector<uint32_t> &)>
        scaled = [&](const hyk_arg_t &a, double sign, std::vector<int32_t> &lv, std::vector<double> &sc,
                     std::vector<uint32_t> &gone) {
        if (a.kind != HYK_ARG_U || (uint32_t)a.idx < n_eq || uses[(uint32_t)a.idx] != 1) return false;
        const uint32_t k = (uint32_t)a.idx - n_eq;
        const hyk_uop_t &o = ops[k];
        if (o.op == HYK_OP_MUL && ((o.a.kind == HYK_ARG_NUM && plainvar(o.b)) || (o.b.kind == HYK_ARG_NUM && plainvar(o.a)))) {
            const bool na = o.a.kind == HYK_ARG_NUM;
            lv.assign(1, na ? o.b.idx : o.a.idx);
            sc.assign(1, sign * (na ? o.a.num : o.b.num));
            gone.assign(1, k);
            return true;
        }
        if (o.op == HYK_OP_NEG && scaled(o.a, -sign, lv, sc, gone)) {
            gone.push_back(k);
            return true;
        }
        if ((o.op == HYK_OP_ADD || o.op == HYK_OP_SUB) && pl.fuse[k] == HYK_FUSE_SC && pl.addend[k] < 0) {
            lv = pl.leaves[k];
            sc = pl.scales[k];
            for (double &x : sc) x *= sign;
            gone.assign(1, k);
            return true;
        }
        return false;
    };
    for (uint32_t k = 0; k < n_ops; ++k) {
        const int op = ops[k].op;
        if (op != HYK_OP_ADD && op != HYK_OP_SUB) continue;
        std::vector<int32_t> lv;
        std::vector<double> sc;
        std::vector<uint32_t> gone;
        int32_t add = -1;
        uint8_t kind = 0;
        if (op == HYK_OP_ADD) {
            std::vector<int32_t> la, lb;
            const bool aa = absorbable(ops[k].a, la), ab = absorbable(ops[k].b, lb);
            if (aa && ab && la.size() + lb.size() <= HYK_FUSE_MAX) {
                lv = la;
                lv.insert(lv.end(), lb.begin(), lb.end());
                kind = HYK_FUSE_SQ;
            } else if (ab && plainvar(ops[k].a)) {
                lv = lb;
                add = ops[k].a.idx;
                kind = HYK_FUSE_SQ;
            } else if (aa && plainvar(ops[k].b)) {
                lv = la;
                add = ops[k].b.idx;
                kind = HYK_FUSE_SQ;
            }
        }
        if (!kind) {
            // sums of scaled terms: a + b, or a - b (b's numbers negated; b
            // never the addend of a difference)
            std::vector<int32_t> la, lb;
            std::vector<double> sa, sb;
            std::vector<uint32_t> ga, gb;
            const bool sub = op == HYK_OP_SUB;
            const bool aa = scaled(ops[k].a, 1.0, la, sa, ga);
            const bool ab = scaled(ops[k].b, sub ? -1.0 : 1.0, lb, sb, gb);
            if (aa && ab && la.size() + lb.size() <= HYK_FUSE_MAX) {
                lv = la;
                lv.insert(lv.end(), lb.begin(), lb.end());
                sc = sa;
                sc.insert(sc.end(), sb.begin(), sb.end());
                gone = ga;
                gone.insert(gone.end(), gb.begin(), gb.end());
                kind = HYK_FUSE_SC;
            } else if (ab && lb.size() <= HYK_FUSE_MAX && plainvar(ops[k].a)) {
                lv = lb;
                sc = sb;
                gone = gb;
                add = ops[k].a.idx;
                kind = HYK_FUSE_SC;
            } else if (!sub && aa && la.size() <= HYK_FUSE_MAX && plainvar(ops[k].b)) {
                lv = la;
                sc = sa;
                gone = ga;
                add = ops[k].b.idx;
                kind = HYK_FUSE_SC;
            }
            if (kind) {
                pl.fuse[k] = kind;
                pl.addend[k] = add;
                pl.leaves[k] = lv;
                pl.scales[k] = sc;
                for (uint32_t c : gone) {
                    pl.dead[c] = 1;
                    pl.fuse[c] = 0;
                }
            }
            continue;
        }
        pl.fuse[k] = kind;
        pl.addend[k] = add;
        pl.leaves[k] = lv;
        for (const hyk_arg_t *a : {&ops[k].a, &ops[k].b}) {
            if (a->kind != HYK_ARG_U || a->idx == add) continue;
            const uint32_t c = (uint32_t)a->idx - n_eq;
            pl.dead[c] = 1;
            pl.fuse[c] = 0;
        }
    }
    return pl;
}

#endif
