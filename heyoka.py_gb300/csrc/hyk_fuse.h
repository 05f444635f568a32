/*
 * hyk_fuse.h - sums of squares fused into one recurrence.
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
 */
#ifndef HYK_FUSE_H
#define HYK_FUSE_H

#include <stdint.h>

#include <vector>

#include "hyk.h"

#define HYK_FUSE_MAX 4

struct HykFusePlan {
    std::vector<uint8_t> fuse;                 // per operation: the root of a fused sum of squares
    std::vector<uint8_t> dead;                 // per operation: a square or sum absorbed by a root
    std::vector<int32_t> addend;               // per root: the u-variable a (-1: none)
    std::vector<std::vector<int32_t>> leaves;  // per root: the u-variables squared, in order
};

static inline HykFusePlan hyk_fuse_plan(uint32_t n_eq, uint32_t n_ops, const hyk_uop_t *ops, const hyk_arg_t *rhs,
                                        uint32_t n_ev, const hyk_event_t *ev) {
    HykFusePlan pl;
    pl.fuse.assign(n_ops, 0);
    pl.dead.assign(n_ops, 0);
    pl.addend.assign(n_ops, -1);
    pl.leaves.assign(n_ops, {});
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
        if (ops[k].op == HYK_OP_ADD && pl.fuse[k] && pl.addend[k] < 0) {
            lv = pl.leaves[k];
            return true;
        }
        return false;
    };
    for (uint32_t k = 0; k < n_ops; ++k) {
        if (ops[k].op != HYK_OP_ADD) continue;
        std::vector<int32_t> la, lb;
        const bool aa = absorbable(ops[k].a, la), ab = absorbable(ops[k].b, lb);
        std::vector<int32_t> lv;
        int32_t add = -1;
        if (aa && ab && la.size() + lb.size() <= HYK_FUSE_MAX) {
            lv = la;
            lv.insert(lv.end(), lb.begin(), lb.end());
        } else if (ab && plainvar(ops[k].a) && lb.size() < HYK_FUSE_MAX + 1) {
            lv = lb;
            add = ops[k].a.idx;
        } else if (aa && plainvar(ops[k].b) && la.size() < HYK_FUSE_MAX + 1) {
            lv = la;
            add = ops[k].b.idx;
        } else {
            continue;
        }
        pl.fuse[k] = 1;
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
