// Code generator: Taylor decomposition -> fused FP64 CUDA step kernel.
//
// The reference JIT-compiles the Taylor recurrences of each ODE system with
// LLVM for the host CPU (inside the heyoka C++ library, reached from
// heyoka/expose_batch_integrators.cpp:166-208).  Here the same recurrences
// are emitted as straight-line CUDA C++, one block per Taylor order, and
// compiled with NVRTC for sm_103a.  Every index is a compile-time constant:
// jets that later orders read live in shared memory at fixed slots, values
// used only within their own order stay in registers, a NEG node is folded
// into its readers as a sign, and the order-p coefficients of the
// intermediate u-variables are skipped (only the state's order p is used).
//
// Recurrences (normalised derivatives, restated from doc/tut_taylor_method.rst):
//   add/sub  c_n = a_n +- b_n
//   mul      c_n = sum_{j=0}^{n} a_j b_{n-j}
//   div      c_n = (a_n - sum_{j=1}^{n} b_j c_{n-j}) / b_0
//   square   c_n = 2 sum_{j<n-j} a_j a_{n-j} (+ a_{n/2}^2)
//   sqrt     c_n = (a_n - 2 sum_{0<j<n-j} c_j c_{n-j} (- c_{n/2}^2)) / (2 c_0)
//   pow      c_n = sum_{j=0}^{n-1} (n alpha - j (alpha + 1)) a_{n-j} c_j / (n a_0)
//   exp      c_n = (1/n) sum_{j=1}^{n} (j a_j) c_{n-j}
//   log      c_n = (a_n - (1/n) sum_{j=1}^{n-1} (j c_j) a_{n-j}) / a_0
//   sin/cos  s_n = (1/n) sum (j a_j) c_{n-j},  c_n = -(1/n) sum (j a_j) s_{n-j}
//   state    x_{n+1} = f_n / (n + 1)
// Sums run over increasing j, skip identically-zero terms, start with a
// product and accumulate with fused multiply-adds; "/ n" is a multiplication
// by the double nearest 1/n and "/ b_0" (n >= 1) a multiplication by 1/b_0
// computed once per step.  The CPU oracle's "gpu" mode performs the same
// operations in the same order.  With pin arithmetic (HYK_CFG_PIN_ARITH)
// the generator emits plain multiply + add and true divisions instead, the
// oracle's "pin" mode.

#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <algorithm>
#include <sstream>

#include "hyk_fuse.h"
#include "hyk_internal.hpp"

// hyk_ev_btab (the Bernstein conversion table printed into event kernels)
#define HYK_DM_FN static inline
#define HYK_DM_FMA(a, b, c) std::fma((a), (b), (c))
#define HYK_DM_BITS(x) hyk_host_bits_(x)
#define HYK_DM_FMAF(a, b, c) std::fma((a), (b), (c))
#define HYK_DM_FBITS(x) hyk_host_fbits_(x)
static inline unsigned long long hyk_host_bits_(double x) {
    unsigned long long u;
    std::memcpy(&u, &x, sizeof u);
    return u;
}
static inline unsigned hyk_host_fbits_(float x) {
    unsigned u;
    std::memcpy(&u, &x, sizeof u);
    return u;
}
#include "hyk_events.h"
#undef HYK_DM_FN
#undef HYK_DM_FMA
#undef HYK_DM_BITS
#undef HYK_DM_FMAF
#undef HYK_DM_FBITS

namespace hyk {

bool load_dec(const hyk_decomp_t *d, Dec &out, std::string &err) {
    if (!d || d->n_eq == 0) {
        err = "invalid decomposition: no state variables";
        return false;
    }
    if (d->n_ops > 0 && !d->ops) {
        err = "invalid decomposition: null ops";
        return false;
    }
    if (!d->rhs) {
        err = "invalid decomposition: null right-hand sides";
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
        case HYK_ARG_TIME:
            return true;
        case HYK_ARG_NUM:
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
        if (o.op < HYK_OP_ADD || o.op > HYK_OP_COS || !chk(o.a, self) || o.a.kind == HYK_ARG_NONE ||
            !chk(o.b, self)) {
            err = "invalid u-variable definition at index " + std::to_string(self);
            return false;
        }
        const bool binary = o.op == HYK_OP_ADD || o.op == HYK_OP_SUB || o.op == HYK_OP_MUL || o.op == HYK_OP_DIV;
        if (binary && o.b.kind == HYK_ARG_NONE) {
            err = "missing second argument at index " + std::to_string(self);
            return false;
        }
        if (o.op == HYK_OP_POW && o.b.kind != HYK_ARG_NUM) {
            err = "pow() needs a numerical exponent (index " + std::to_string(self) + ")";
            return false;
        }
        if (o.op == HYK_OP_SIN || o.op == HYK_OP_COS) {
            if (o.aux < (int)out.n_eq || (uint32_t)o.aux >= nu) {
                err = "invalid sin/cos partner at index " + std::to_string(self);
                return false;
            }
            const auto &pt = out.ops[o.aux - out.n_eq];
            const int want = o.op == HYK_OP_SIN ? HYK_OP_COS : HYK_OP_SIN;
            if (pt.op != want || pt.aux != (int)self || pt.a.kind != o.a.kind || pt.a.idx != o.a.idx) {
                err = "inconsistent sin/cos pair at index " + std::to_string(self);
                return false;
            }
        }
    }
    for (const auto &r : out.rhs)
        if (!chk(r, nu) || r.kind == HYK_ARG_NONE) {
            err = "invalid right-hand side";
            return false;
        }
    out.ev.clear();
    if (d->n_ev > 0) {
        if (!d->ev) {
            err = "invalid decomposition: null events";
            return false;
        }
        out.ev.assign(d->ev, d->ev + d->n_ev);
        for (const auto &e : out.ev)
            if (!chk(e.g, nu) || e.g.kind == HYK_ARG_NONE || (e.terminal != 0 && e.terminal != 1) || e.direction < -1 ||
                e.direction > 1 || !(e.cooldown == e.cooldown)) {
                err = "invalid event";
                return false;
            }
    }
    return true;
}

namespace {

// Precision of the code being generated: float for the float32 integrator.
// Literals are then the float nearest to the value (with an f suffix), and
// the generator's own constants (1/n, pow coefficients, the step-size
// factor) are computed in float arithmetic, as the oracle's float mode does.
thread_local bool g_f32 = false;

std::string lit(double v) {
    if (g_f32) {
        const float f = (float)v;
        if (std::isnan(f)) return "HYK_FROM_BITS(HYK_NAN_BITS)";
        if (std::isinf(f)) return f > 0 ? "hyk_inf()" : "(-hyk_inf())";
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.9g", (double)f);
        std::string s(buf);
        if (s.find_first_of(".eE") == std::string::npos) s += ".0";
        s += "f";
        if (f < 0 || (f == 0 && std::signbit(f))) s = "(" + s + ")";
        return s;
    }
    if (std::isnan(v)) return "__longlong_as_double(0x7ff8000000000000LL)";
    if (std::isinf(v)) return v > 0 ? "hyk_inf()" : "(-hyk_inf())";
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.17g", v);
    std::string s(buf);
    if (s.find_first_of(".eE") == std::string::npos) s += ".0";
    if (v < 0 || (v == 0 && std::signbit(v))) s = "(" + s + ")";
    return s;
}

// The nearest number of the generated precision to 1/n.
double recip(double n) { return g_f32 ? (double)(1.0f / (float)n) : 1.0 / n; }

// The pow recurrence's coefficient n alpha - j (alpha + 1), in the generated precision.
double powcoef(uint32_t n, uint32_t j, double alpha) {
    if (g_f32) {
        const float a = (float)alpha;
        return (double)((float)n * a - (float)j * (a + 1.0f));
    }
    return (double)n * alpha - (double)j * (alpha + 1.0);
}

// The step-size safety factor exp(-2) exp(-0.7 / (p - 1)), as 1/(e e) exp((-7/10)/(p-1)).
double rhofac_of(uint32_t p) {
    if (g_f32) {
        const float e1 = std::exp(1.0f);
        return (double)(1.0f / (e1 * e1) * std::exp((-7.0f / 10.0f) / (float)(p - 1)));
    }
    const double e1 = std::exp(1.0);
    return 1.0 / (e1 * e1) * std::exp((-7.0 / 10.0) / (p - 1.0));
}

// Precision-dependent part of a generated module's header.
std::string precision_header(bool pin) {
    std::string h;
    if (g_f32) {
        h += "#define HYK_F32 1\n";
        h += "#define HYK_FMA(a, b, c) __fmaf_rn((a), (b), (c))\n";
        h += "#define HYK_FMAOPS_CONSTS\n#define HYK_MUL(a, b) ((a) * (b))\n#define HYK_ADD(a, b) ((a) + (b))\n"
             "#define HYK_SUB(a, b) ((a) - (b))\n";
        h += "#define HYK_DM_EXP hyk_dmf_exp\n#define HYK_DM_LOG hyk_dmf_log\n#define HYK_DM_SINCOS hyk_dmf_sincos\n"
             "#define HYK_DM_POW hyk_dmf_pow\n#define HYK_DM_RHO hyk_dmf_rho\n";
    } else {
        h += "#define HYK_F32 0\n";
        h += "#define HYK_FMA(a, b, c) __fma_rn((a), (b), (c))\n";
        // x * y, x + y and x - y as fused multiply-adds (same bits); the
        // constants -0 and 1 come from volatile loads of module globals, so
        // that the compiler cannot turn the fused operations back into plain ones.
        h += "__device__ double hyk_nz_g = -0.0, hyk_one_g = 1.0;\n";
        h += "#define HYK_FMAOPS_CONSTS const double hyk_nz = *(volatile double *)&hyk_nz_g, "
             "hyk_one = *(volatile double *)&hyk_one_g;\n";
        h += "#define HYK_MUL(a, b) __fma_rn((a), (b), hyk_nz)\n";
        h += "#define HYK_ADD(a, b) __fma_rn((a), hyk_one, (b))\n";
        h += "#define HYK_SUB(a, b) __fma_rn((b), -hyk_one, (a))\n";
        h += "#define HYK_DM_EXP hyk_dm_exp\n#define HYK_DM_LOG hyk_dm_log\n#define HYK_DM_SINCOS hyk_dm_sincos\n"
             "#define HYK_DM_POW hyk_dm_pow\n#define HYK_DM_RHO hyk_dm_rho\n";
    }
    (void)pin;
    return h;
}

struct Ref {
    int kind = HYK_ARG_NONE;  // after NEG folding
    int u = -1;
    bool neg = false;
    double num = 0;
    int par = -1;
};

struct Gen {
    const Dec &d;
    uint32_t p, N, NU;
    bool pin;
    std::vector<int> base;
    std::vector<char> negf, alias, hist, needka;
    std::vector<int> slot, kslot;
    uint32_t nslot = 0, par_slot = 0;
    std::ostringstream o;
    double flops = 0;

    bool adj = false;  // also emit the reverse sweep (adjoint module)
    std::vector<int> aslot, akslot;
    uint32_t abase = 0;

    // Large systems: one function per Taylor order (a single straight-line
    // function of tens of thousands of operations takes ptxas many minutes).
    // Order n then reloads the state's order-n coefficients from the jet
    // store and the 1/b_0 factors from slots of their own.
    bool split = false;
    std::vector<int> islot;

    // Events: every order's coefficient of each event function in its own
    // slots (evslot + k (p+1) + n), the histories kept up to order p-1 (as
    // for the adjoint), and an extra order-p pass over the operations the
    // event functions depend on.
    bool evx = false;
    uint32_t evslot = 0;
    std::vector<char> cone;

    // Operations whose arguments are all time-constant (numbers, parameters,
    // other such operations) are constant in time: only their order-0 value
    // exists (one slot, like a parameter) and their higher orders are known
    // zeros, so products with them are single terms.  Gpu arithmetic only;
    // the pinned arithmetic and the adjoint keep the full recurrences.
    std::vector<char> cst;

    // Cold state rows (coldrows mode): a state variable whose coefficients no
    // recurrence reads at a later order (it enters the right-hand sides only
    // through sums and differences, or not at all: the velocities of
    // Kepler, N-body and CR3BP) is read again only by the step size, the
    // state update and the coefficient outputs.  Its orders 1..p then live
    // in a global buffer of the module (row crow[i], slot crow[i] * p + n - 1,
    // slot stride HYK_CSTRIDE), and only its order 0 in shared memory, so
    // that more lanes fit the shared memory of an SM.
    bool coldrows = false;
    std::vector<int> crow;
    std::vector<char> hread;
    uint32_t ncold = 0;

    // Sums of squares and sums of scaled terms fused into one recurrence
    // (hyk_fuse.h; GPU arithmetic only): fz.fuse[k] marks the root, fz.dead
    // the squares, products, negations and sums it absorbs (skipped like
    // aliases).
    HykFusePlan fz;
    bool fused(uint32_t u) const { return u >= N && !fz.fuse.empty() && fz.fuse[u - N]; }
    bool fused_sq(uint32_t u) const { return fused(u) && fz.fuse[u - N] == HYK_FUSE_SQ; }
    bool fused_sc(uint32_t u) const { return fused(u) && fz.fuse[u - N] == HYK_FUSE_SC; }
    const std::vector<double> &fz_k(uint32_t u) const { return fz.scales[u - N]; }
    Ref uref(int32_t v) const {
        hyk_arg_t a{};
        a.kind = HYK_ARG_U;
        a.idx = v;
        return res(a);
    }
    // The fused root's addend (kind HYK_ARG_NONE when it has none) and leaves.
    Ref fz_a(uint32_t u) const { return fz.addend[u - N] >= 0 ? uref(fz.addend[u - N]) : Ref{}; }
    std::vector<Ref> fz_x(uint32_t u) const {
        std::vector<Ref> v;
        for (int32_t x : fz.leaves[u - N]) v.push_back(uref(x));
        return v;
    }

    // split: one __noinline__ function per order.  Forced for large systems
    // (ptxas time), for the adjoint module and for coefficients in global
    // memory: there a single function of all orders spills (the compiler
    // keeps values of many operations live across the order's long FMA
    // chains), and the per-order functions do not.
    Gen(const Dec &dd, uint32_t order, bool pin_arith, bool adjoint = false, bool cold_rows = false,
        bool force_split = false)
        : d(dd), p(order), N(dd.n_eq), NU(dd.n_u()), pin(pin_arith), adj(adjoint),
          split((uint64_t)dd.n_ops * order > 3000 || adjoint || force_split), evx(!dd.ev.empty()) {
        coldrows = cold_rows && !adjoint && !evx;
        base.resize(NU);
        negf.assign(NU, 0);
        alias.assign(NU, 0);
        cst.assign(NU, 0);
        for (uint32_t u = 0; u < NU; ++u) base[u] = (int)u;
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const auto &op = d.ops[k];
            const uint32_t u = N + k;
            if (op.op == HYK_OP_NEG && op.a.kind == HYK_ARG_U) {
                alias[u] = 1;
                base[u] = base[op.a.idx];
                negf[u] = !negf[op.a.idx];
            }
            if (!pin && !adj) {
                auto kconst = [&](const hyk_arg_t &a) {
                    return a.kind == HYK_ARG_NONE || a.kind == HYK_ARG_NUM || a.kind == HYK_ARG_PAR ||
                           (a.kind == HYK_ARG_U && cst[base[a.idx]]);
                };
                cst[u] = kconst(op.a) && kconst(op.b);
            }
        }
        if (!pin) {
            fz = hyk_fuse_plan(N, d.n_ops, d.ops.data(), d.rhs.data(), (uint32_t)d.ev.size(), d.ev.data());
            for (uint32_t k = 0; k < d.n_ops; ++k)
                if (fz.dead[k]) alias[N + k] = 1;  // computed nowhere
        }
        analyse();
    }

    Ref res(const hyk_arg_t &a) const {
        Ref r;
        r.kind = a.kind;
        if (a.kind == HYK_ARG_U) {
            r.u = base[a.idx];
            r.neg = negf[a.idx];
        } else if (a.kind == HYK_ARG_NUM) {
            r.num = a.num;
        } else if (a.kind == HYK_ARG_PAR) {
            r.par = a.idx;
        }
        return r;
    }
    bool varying(const Ref &r) const { return (r.kind == HYK_ARG_U && !cst[r.u]) || r.kind == HYK_ARG_TIME; }

    void analyse() {
        hist.assign(NU, 0);
        needka.assign(NU, 0);
        hread.assign(NU, 0);
        for (uint32_t i = 0; i < N; ++i) hist[i] = 1;
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const uint32_t u = N + k;
            if (alias[u]) continue;
            const auto &op = d.ops[k];
            const Ref A = res(op.a), B = res(op.b);
            auto H = [&](const Ref &r) {
                if (r.kind == HYK_ARG_U) hist[r.u] = hread[r.u] = 1;
            };
            auto K = [&](const Ref &r) {
                if (r.kind == HYK_ARG_U && !cst[r.u]) needka[r.u] = 1;
            };
            if (fused(u)) {
                if (fused_sq(u))
                    for (const Ref &x : fz_x(u)) H(x);
                continue;  // a sum of scaled terms reads order n only
            }
            switch (op.op) {
            case HYK_OP_MUL:
                if (varying(B)) H(A);
                if (varying(A)) H(B);
                break;
            case HYK_OP_DIV:
                H(B);
                if (varying(B)) hist[u] = 1;
                break;
            case HYK_OP_SQUARE:
                H(A);
                break;
            case HYK_OP_SQRT:
                if (varying(A)) hist[u] = 1;
                break;
            case HYK_OP_POW:
                H(A);
                if (varying(A)) hist[u] = 1;
                break;
            case HYK_OP_EXP:
                K(A);
                if (varying(A)) hist[u] = 1;
                break;
            case HYK_OP_LOG:
                H(A);
                if (varying(A)) needka[u] = 1;
                break;
            case HYK_OP_SIN:
            case HYK_OP_COS:
                K(A);
                if (varying(A)) {
                    hist[u] = 1;
                    hist[op.aux] = 1;
                }
                break;
            default:
                break;
            }
        }
        if (adj) {
            // The reverse sweep reads every operation's coefficients.
            for (uint32_t u = N; u < NU; ++u)
                if (!alias[u]) hist[u] = 1;
            // Values the reverse sweep reads besides the forward histories:
            // the factor multiplied by a parameter (for the parameter's
            // adjoint), the quotient by a parameter, and the logarithm.
            for (uint32_t k = 0; k < d.n_ops; ++k) {
                const uint32_t u = N + k;
                if (alias[u]) continue;
                const auto &op = d.ops[k];
                const Ref A = res(op.a), B = res(op.b);
                if (op.op == HYK_OP_MUL) {
                    if (A.kind == HYK_ARG_PAR && B.kind == HYK_ARG_U) hist[B.u] = 1;
                    if (B.kind == HYK_ARG_PAR && A.kind == HYK_ARG_U) hist[A.u] = 1;
                }
                if (op.op == HYK_OP_DIV && B.kind == HYK_ARG_PAR) hist[u] = 1;
                if (op.op == HYK_OP_LOG) hist[u] = 1;
            }
        }
        // Slots: state variables (orders 0..p), other histories (orders
        // 0..p-2: order p-1 is only read within its own block and order p of
        // intermediates is never computed), j*a_j histories (orders 1..p-2),
        // then the parameters.
        slot.assign(NU, -1);
        kslot.assign(NU, -1);
        crow.assign(N, -1);
        ncold = 0;
        uint32_t s = 0;
        for (uint32_t i = 0; i < N; ++i) {
            slot[i] = (int)s;
            if (coldrows && !hread[i]) {
                crow[i] = (int)ncold++;
                s += 1;  // order 0 only
            } else {
                s += p + 1;
            }
        }
        // The adjoint module keeps every history up to order p-1.
        const bool ext = adj || evx;
        const uint32_t hl = ext ? p : (p >= 2 ? p - 1 : 1), kl = ext ? p - 1 : (p >= 3 ? p - 2 : 0);
        for (uint32_t u = N; u < NU; ++u)
            if (!alias[u] && cst[u]) {
                hist[u] = 1;  // the order-0 value, read at every order
                needka[u] = 0;
                slot[u] = (int)s;
                s += 1;
            } else if (hist[u] && !alias[u]) {
                slot[u] = (int)s;
                s += hl;
            }
        for (uint32_t u = 0; u < NU; ++u)
            if (needka[u] && !alias[u] && kl > 0) {
                kslot[u] = (int)s;
                s += kl;
            }
        islot.assign(NU, -1);
        if (split)
            for (uint32_t k = 0; k < d.n_ops; ++k) {
                const int o = d.ops[k].op;
                if (!alias[N + k] && (o == HYK_OP_DIV || o == HYK_OP_SQRT || o == HYK_OP_POW || o == HYK_OP_LOG))
                    islot[N + k] = (int)s++;
            }
        par_slot = s;
        s += d.n_pars;
        if (evx) {
            evslot = s;
            s += (uint32_t)d.ev.size() * (p + 1);
            // The operations the event functions depend on (through u-variable
            // arguments, aliases resolved), for the order-p pass.
            cone.assign(NU, 0);
            std::vector<uint32_t> stack;
            for (const auto &e : d.ev)
                if (e.g.kind == HYK_ARG_U) stack.push_back((uint32_t)base[e.g.idx]);
            while (!stack.empty()) {
                const uint32_t u = stack.back();
                stack.pop_back();
                if (u < N || cone[u]) continue;
                cone[u] = 1;
                const auto &op = d.ops[u - N];
                for (const hyk_arg_t *a : {&op.a, &op.b})
                    if (a->kind == HYK_ARG_U) stack.push_back((uint32_t)base[a->idx]);
            }
        }
        if (adj) {
            // Reverse sweep (gather form): per operation the history of its
            // adjoint factor at orders 1..p-1 (slot hslot[u] + n - 1), and one
            // slot per state variable for its adjoint at the order above.
            abase = s;
            aslot.assign(NU, -1);
            akslot.assign(NU, -1);
            for (uint32_t k = 0; k < d.n_ops; ++k) {
                const uint32_t u = N + k;
                const int o = d.ops[k].op;
                if (alias[u] || p < 2 || ((o == HYK_OP_ADD || o == HYK_OP_SUB || o == HYK_OP_NEG) && !fused_sq(u)))
                    continue;
                aslot[u] = (int)s;
                s += p - 1;
            }
            for (uint32_t i = 0; i < N; ++i) akslot[i] = (int)s++;
        }
        nslot = s;
    }

    std::string vname(uint32_t u, uint32_t n) const { return "v" + std::to_string(u) + "_" + std::to_string(n); }
    std::string kname(uint32_t u, uint32_t n) const { return "k" + std::to_string(u) + "_" + std::to_string(n); }
    std::string smem(uint32_t s) const { return "S[" + std::to_string(s) + " * HYK_STRIDE]"; }

    // Coefficient of order j of u-variable u (not an alias) while emitting block n.
    std::string ucoef(uint32_t u, uint32_t j, uint32_t n) const {
        if (j == n) return vname(u, j);
        if (!hist[u] || slot[u] < 0 || (u < N && crow[u] >= 0 && j > 0)) {
            std::fprintf(stderr, "hyk codegen: missing history for u%u\n", u);
            std::abort();
        }
        return smem((uint32_t)slot[u] + j);
    }
    // Coefficient expression, or "" when identically zero.
    std::string cf(const Ref &r, uint32_t j, uint32_t n) const {
        switch (r.kind) {
        case HYK_ARG_U: {
            if (cst[r.u] && j >= 1) return "";
            const std::string s = ucoef((uint32_t)r.u, j, n);
            return r.neg ? "(-" + s + ")" : s;
        }
        case HYK_ARG_NUM:
            return j == 0 ? lit(r.num) : "";
        case HYK_ARG_PAR:
            return j == 0 ? "HYK_PAR(" + std::to_string(r.par) + ")" : "";
        case HYK_ARG_TIME:
            return j == 0 ? "t0" : (j == 1 ? lit(1.0) : "");
        }
        return "";
    }
    // j * a_j (j >= 1), or "" when identically zero.
    std::string kcf(const Ref &r, uint32_t j, uint32_t n) const {
        switch (r.kind) {
        case HYK_ARG_U: {
            if (cst[r.u]) return "";
            const uint32_t u = (uint32_t)r.u;
            std::string s;
            if (j == n)
                s = kname(u, j);
            else {
                if (kslot[u] < 0) {
                    std::fprintf(stderr, "hyk codegen: missing j*a_j history for u%u\n", u);
                    std::abort();
                }
                s = smem((uint32_t)kslot[u] + j - 1);
            }
            return r.neg ? "(-" + s + ")" : s;
        }
        case HYK_ARG_TIME:
            return j == 1 ? lit(1.0) : "";
        default:
            return "";
        }
    }

    // Whether the order-j coefficient (or j * a_j) of an argument can be
    // non-zero; checked before building an expression, so that no history is
    // requested for a term that vanishes.
    bool nz(const Ref &r, uint32_t j) const {
        switch (r.kind) {
        case HYK_ARG_U:
            return !cst[r.u] || j == 0;
        case HYK_ARG_TIME:
            return j <= 1;
        case HYK_ARG_NUM:
        case HYK_ARG_PAR:
            return j == 0;
        }
        return false;
    }
    bool knz(const Ref &r, uint32_t j) const {
        return (r.kind == HYK_ARG_U && !cst[r.u] && j >= 1) || (r.kind == HYK_ARG_TIME && j == 1);
    }

    std::string fma(const std::string &x, const std::string &y, const std::string &c) const {
        if (pin) return "(" + c + " + " + x + " * " + y + ")";
        return "HYK_FMA(" + x + ", " + y + ", " + c + ")";
    }
    // Products, sums and differences of the gpu arithmetic in double
    // precision: fused multiply-adds with an addend of -0 (x * y) or a factor
    // of 1 (x + y, x - y).  They give exactly the bits of the plain
    // operations, and the FP64 pipe of this GPU issues fused multiply-adds
    // faster than plain multiplications and additions.
    bool fmaops() const { return !pin && !g_f32; }
    std::string mul(const std::string &x, const std::string &y) const {
        return fmaops() ? "HYK_MUL(" + x + ", " + y + ")" : "(" + x + " * " + y + ")";
    }
    std::string add(const std::string &x, const std::string &y) const {
        return fmaops() ? "HYK_ADD(" + x + ", " + y + ")" : "(" + x + " + " + y + ")";
    }
    std::string sub(const std::string &x, const std::string &y) const {
        return fmaops() ? "HYK_SUB(" + x + ", " + y + ")" : "(" + x + " - " + y + ")";
    }

    struct Acc {
        std::string name;
        bool first = true;
    };
    void term(Acc &a, const std::string &x, const std::string &y) {
        if (x.empty() || y.empty()) return;
        if (a.first) {
            o << "    hyk_real " << a.name << " = " << mul(x, y) << ";\n";
            a.first = false;
            flops += 1;
        } else {
            o << "    " << a.name << " = " << fma(x, y, a.name) << ";\n";
            flops += 2;
        }
    }
    std::string divn(const std::string &x, uint32_t n) {
        flops += 1;
        if (pin) return "(" + x + " / " + lit((double)n) + ")";
        return mul(x, lit(recip((double)n)));
    }
    std::string inv0(uint32_t u) const { return "i" + std::to_string(u); }
    // After defining 1/b_0 at order 0: keep it for the later order functions.
    void keep_inv0(uint32_t u) {
        if (split && !pin && islot[u] >= 0) o << "    " << smem((uint32_t)islot[u]) << " = " << inv0(u) << ";\n";
    }

    void def(uint32_t u, uint32_t n, const std::string &expr) { o << "    const hyk_real " << vname(u, n) << " = " << expr << ";\n"; }

    void store_hist(uint32_t u, uint32_t n) {
        if (u >= N && cst[u]) {
            if (n == 0) o << "    " << smem((uint32_t)slot[u]) << " = " << vname(u, 0) << ";\n";
            return;
        }
        const uint32_t lim = (adj || evx) ? p : p - 1;  // stored orders: 0..lim-1
        if (u >= N && hist[u] && n + 1 <= lim) o << "    " << smem((uint32_t)slot[u] + n) << " = " << vname(u, n) << ";\n";
        if (needka[u] && n >= 1) {
            o << "    const hyk_real " << kname(u, n) << " = " << mul(lit((double)n), vname(u, n)) << ";\n";
            flops += 1;
            if (kslot[u] >= 0 && n + 1 <= lim) o << "    " << smem((uint32_t)kslot[u] + n - 1) << " = " << kname(u, n) << ";\n";
        }
    }

    void emit_op(uint32_t k, uint32_t n) {
        const auto &op = d.ops[k];
        const uint32_t u = N + k;
        if (alias[u]) return;
        if (cst[u] && n >= 1) return;  // known zero
        const Ref A = res(op.a), B = res(op.b);
        const std::string acc = "a" + std::to_string(u) + "_" + std::to_string(n);
        const std::string z = lit(0.0);
        if (fused_sc(u)) {
            // a + sum_i k_i t_i in one chain (hyk_fuse.h)
            const Ref FA = fz_a(u);
            const std::vector<Ref> FX = fz_x(u);
            const std::vector<double> &FK = fz_k(u);
            std::string r = FA.kind == HYK_ARG_U ? cf(FA, n, n) : "";
            for (size_t i = 0; i < FX.size(); ++i) {
                flops += r.empty() ? 1 : 2;
                r = r.empty() ? mul(lit(FK[i]), cf(FX[i], n, n)) : fma(lit(FK[i]), cf(FX[i], n, n), r);
            }
            def(u, n, r);
            return;
        }
        if (fused(u)) {
            // a + sum_i x_i^2 in one chain (hyk_fuse.h)
            const Ref FA = fz_a(u);
            const std::vector<Ref> FX = fz_x(u);
            const bool ha = FA.kind == HYK_ARG_U;
            Acc s{acc};
            for (const Ref &x : FX)
                for (uint32_t j = 0; 2 * j < n; ++j) term(s, cf(x, j, n), cf(x, n - j, n));
            std::string r = ha ? cf(FA, n, n) : "";
            if (!s.first) {
                r = ha ? fma(lit(2.0), acc, r) : add(acc, acc);
                flops += ha ? 2 : 1;
            }
            if (n % 2 == 0)
                for (const Ref &x : FX) {
                    const std::string xm = cf(x, n / 2, n);
                    flops += r.empty() ? 1 : 2;
                    r = r.empty() ? mul(xm, xm) : fma(xm, xm, r);
                }
            def(u, n, r);
            return;
        }
        switch (op.op) {
        case HYK_OP_ADD:
        case HYK_OP_SUB: {
            const std::string a = cf(A, n, n), b = cf(B, n, n);
            const bool add = op.op == HYK_OP_ADD;
            if (!a.empty() && !b.empty()) {
                def(u, n, add ? this->add(a, b) : sub(a, b));
                flops += 1;
            } else if (!a.empty())
                def(u, n, a);
            else if (!b.empty())
                def(u, n, add ? b : "(-" + b + ")");
            else
                def(u, n, z);
            break;
        }
        case HYK_OP_NEG: {
            const std::string a = cf(A, n, n);
            def(u, n, a.empty() ? z : "(-" + a + ")");
            break;
        }
        case HYK_OP_MUL: {
            Acc s{acc};
            for (uint32_t j = 0; j <= n; ++j)
                if (nz(A, j) && nz(B, n - j)) term(s, cf(A, j, n), cf(B, n - j, n));
            def(u, n, s.first ? z : acc);
            break;
        }
        case HYK_OP_DIV: {
            const std::string b0 = cf(B, 0, n), an = cf(A, n, n);
            if (n == 0) {
                def(u, 0, "(" + an + " / " + b0 + ")");
                if (!pin) o << "    const hyk_real " << inv0(u) << " = " << lit(1.0) << " / " << b0 << ";\n";
                flops += 2;
                keep_inv0(u);
                break;
            }
            Acc s{acc};
            for (uint32_t j = 1; j <= n; ++j)
                if (nz(B, j)) term(s, cf(B, j, n), ucoef(u, n - j, n));
            const std::string av = an.empty() ? z : an;
            const std::string num = s.first ? av : sub(av, acc);
            if (!s.first) flops += 1;
            flops += 1;
            def(u, n, pin ? "(" + num + " / " + b0 + ")" : mul(num, inv0(u)));
            break;
        }
        case HYK_OP_SQUARE: {
            Acc s{acc};
            for (uint32_t j = 0; 2 * j < n; ++j)
                if (nz(A, j) && nz(A, n - j)) term(s, cf(A, j, n), cf(A, n - j, n));
            if (!s.first) {
                o << "    " << acc << " = " << add(acc, acc) << ";\n";
                flops += 1;
            }
            if (n % 2 == 0 && nz(A, n / 2)) term(s, cf(A, n / 2, n), cf(A, n / 2, n));
            def(u, n, s.first ? z : acc);
            break;
        }
        case HYK_OP_SQRT: {
            const std::string an = cf(A, n, n);
            if (n == 0) {
                def(u, 0, "sqrt(" + an + ")");  // IEEE square root in both arithmetics
                if (!pin) o << "    const hyk_real " << inv0(u) << " = " << lit(1.0) << " / (" << lit(2.0) << " * " << vname(u, 0) << ");\n";
                flops += 3;
                keep_inv0(u);
                break;
            }
            Acc s{acc};
            for (uint32_t j = 1; 2 * j < n; ++j) term(s, ucoef(u, j, n), ucoef(u, n - j, n));
            if (!s.first) {
                o << "    " << acc << " = " << add(acc, acc) << ";\n";
                flops += 1;
            }
            if (n % 2 == 0) term(s, ucoef(u, n / 2, n), ucoef(u, n / 2, n));
            const std::string av = an.empty() ? z : an;
            const std::string num = s.first ? av : sub(av, acc);
            flops += s.first ? 1 : 2;
            def(u, n, pin ? "(" + num + " / (2.0 * " + ucoef(u, 0, n) + "))" : mul(num, inv0(u)));
            break;
        }
        case HYK_OP_POW: {
            const double alpha = op.b.num;
            const std::string a0 = cf(A, 0, n);
            if (n == 0) {
                def(u, 0, (pin ? "pow(" : "HYK_DM_POW(") + a0 + ", " + lit(alpha) + ")");
                if (!pin) o << "    const hyk_real " << inv0(u) << " = " << lit(1.0) << " / " << a0 << ";\n";
                flops += 21;
                keep_inv0(u);
                break;
            }
            Acc s{acc};
            for (uint32_t j = 0; j < n; ++j) {
                const std::string anj = cf(A, n - j, n);
                if (anj.empty()) continue;
                const double coef = powcoef(n, j, alpha);
                const std::string t = "t" + std::to_string(u) + "_" + std::to_string(n) + "_" + std::to_string(j);
                o << "    const hyk_real " << t << " = " << mul(lit(coef), anj) << ";\n";
                flops += 1;
                term(s, t, ucoef(u, j, n));
            }
            if (s.first) {
                def(u, n, z);
                break;
            }
            flops += 2;
            if (pin)
                def(u, n, "(" + acc + " / (" + lit((double)n) + " * " + a0 + "))");
            else
                def(u, n, mul(mul(acc, lit(recip((double)n))), inv0(u)));
            break;
        }
        case HYK_OP_EXP: {
            if (n == 0) {
                def(u, 0, (pin ? "exp(" : "HYK_DM_EXP(") + cf(A, 0, n) + ")");
                flops += 20;
                break;
            }
            Acc s{acc};
            for (uint32_t j = 1; j <= n; ++j)
                if (knz(A, j)) term(s, kcf(A, j, n), ucoef(u, n - j, n));
            def(u, n, s.first ? z : divn(acc, n));
            break;
        }
        case HYK_OP_LOG: {
            const std::string a0 = cf(A, 0, n), an = cf(A, n, n);
            if (n == 0) {
                def(u, 0, (pin ? "log(" : "HYK_DM_LOG(") + a0 + ")");
                if (!pin) o << "    const hyk_real " << inv0(u) << " = " << lit(1.0) << " / " << a0 << ";\n";
                flops += 21;
                keep_inv0(u);
                break;
            }
            Acc s{acc};
            if (varying(A))
                for (uint32_t j = 1; j < n; ++j) {
                    const Ref self{HYK_ARG_U, (int)u, false, 0, -1};
                    if (nz(A, n - j)) term(s, kcf(self, j, n), cf(A, n - j, n));
                }
            const std::string av = an.empty() ? z : an;
            std::string num = av;
            if (!s.first) {
                num = sub(av, divn(acc, n));
                flops += 1;
            }
            flops += 1;
            def(u, n, pin ? "(" + num + " / " + a0 + ")" : mul(num, inv0(u)));
            break;
        }
        case HYK_OP_SIN:
        case HYK_OP_COS: {
            const uint32_t partner = (uint32_t)op.aux;
            const bool is_sin = op.op == HYK_OP_SIN;
            if (n == 0) {
                // The pair is evaluated together at its first member.
                if (u < partner) {
                    const uint32_t su = is_sin ? u : partner, cu = is_sin ? partner : u;
                    o << "    hyk_real " << vname(su, 0) << "_m, " << vname(cu, 0) << "_m;\n";
                    o << "    " << (pin ? "sincos(" : "HYK_DM_SINCOS(") << cf(A, 0, n) << ", &" << vname(su, 0) << "_m, &"
                      << vname(cu, 0) << "_m);\n";
                    o << "    const hyk_real " << vname(su, 0) << " = " << vname(su, 0) << "_m;\n";
                    o << "    const hyk_real " << vname(cu, 0) << " = " << vname(cu, 0) << "_m;\n";
                    flops += 40;
                }
                break;
            }
            Acc s{acc};
            for (uint32_t j = 1; j <= n; ++j)
                if (knz(A, j)) term(s, kcf(A, j, n), ucoef(partner, n - j, n));
            if (s.first)
                def(u, n, z);
            else
                def(u, n, is_sin ? divn(acc, n) : "(-" + divn(acc, n) + ")");
            break;
        }
        default:
            break;
        }
    }

    // State variable i, order n in the jets code: shared memory, or for a
    // cold row (n >= 1) the module's global buffer.
    std::string sx(uint32_t i, uint32_t n) const {
        if (coldrows && crow[i] >= 0 && n > 0)
            return "HYK_CX(" + std::to_string(crow[i] * p + n - 1) + ")";
        return "HYK_SX(" + std::to_string(i) + ", " + std::to_string(n) + ")";
    }

    // The template's access to state coefficients (HYK_SX): a function of
    // the variable and the order that knows each variable's place.
    void emit_sx_access(std::ostream &h) const {
        if (!coldrows) return;
        h << "#define HYK_COLDROWS 1\n#define HYK_NCOLD " << ncold << "\n";
        h << "extern \"C\" { __constant__ hyk_real *hyk_cold_base; }\n";
        h << "#define HYK_CX(k) hyk_cold_g[(hyk_u64)(k) * HYK_CSTRIDE]\n";
        h << "static __device__ __forceinline__ hyk_real *hyk_cold_ptr() {\n"
             "    return hyk_cold_base + ((hyk_u64)blockIdx.x * HYK_TPB + threadIdx.x);\n}\n";
        h << "template <typename R>\nstatic __device__ __forceinline__ R *hyk_sxp(R *S, int i, int n) {\n    switch (i) {\n";
        for (uint32_t i = 0; i < N; ++i) {
            h << "    case " << i << ": return ";
            if (crow[i] >= 0)
                h << "n == 0 ? S + " << slot[i] << " * HYK_STRIDE : hyk_cold_ptr() + (hyk_u64)(" << crow[i] * p
                  << " + n - 1) * HYK_CSTRIDE;\n";
            else
                h << "S + (" << slot[i] << " + n) * HYK_STRIDE;\n";
        }
        h << "    default: return S;\n    }\n}\n";
        h << "#define HYK_SX(i, n) (*hyk_sxp(S, (i), (n)))\n";
    }

    void emit_jets() {
        std::string coldg = coldrows ? "    hyk_real *__restrict__ hyk_cold_g = hyk_cold_ptr();\n" : "";
        if (fmaops()) coldg += "    HYK_FMAOPS_CONSTS\n";
        if (!split) {
            o << "static __device__ __noinline__ void hyk_jets(hyk_real *__restrict__ S, const hyk_real t0, "
                 "const unsigned hyk_wm = 0xffffffffu) {\n" << coldg;
            for (uint32_t i = 0; i < N; ++i) o << "    const hyk_real " << vname(i, 0) << " = HYK_SX(" << i << ", 0);\n";
        }
        const uint32_t last = evx ? p : p - 1;  // order p: the event functions' cone only
        for (uint32_t n = 0; n <= last; ++n) {
            if (split) {
                o << "static __device__ __noinline__ void hyk_jets_o" << n
                  << "(hyk_real *__restrict__ S, const hyk_real t0, const unsigned hyk_wm) {\n" << coldg;
                for (uint32_t i = 0; i < N; ++i) {
                    o << "    const hyk_real " << vname(i, n) << " = " << sx(i, n) << ";\n";
                    // The same product the previous order formed (k_i_0 is never read).
                    if (needka[i] && n >= 1)
                        o << "    const hyk_real " << kname(i, n) << " = " << mul(lit((double)n), vname(i, n)) << ";\n";
                }
                if (!pin && n >= 1)
                    for (uint32_t u = N; u < NU; ++u)
                        if (islot[u] >= 0) o << "    const hyk_real " << inv0(u) << " = " << smem((uint32_t)islot[u]) << ";\n";
            }
            o << "    // ---- order " << n << "\n";
            for (uint32_t k = 0; k < d.n_ops; ++k) {
                const uint32_t u = N + k;
                if (n == p && !cone[u]) continue;
                emit_op(k, n);
                if (!alias[u]) store_hist(u, n);
            }
            for (size_t k = 0; k < d.ev.size(); ++k) {
                const std::string f = cf(res(d.ev[k].g), n, n);
                o << "    " << smem(evslot + (uint32_t)k * (p + 1) + n) << " = " << (f.empty() ? lit(0.0) : f) << ";\n";
            }
            if (n == p) {
                if (split) o << "}\n";
                continue;
            }
            for (uint32_t i = 0; i < N; ++i) {
                const Ref r = res(d.rhs[i]);
                const std::string f = cf(r, n, n);
                def(i, n + 1, f.empty() ? lit(0.0) : divn(f, n + 1));
                o << "    " << sx(i, n + 1) << " = " << vname(i, n + 1) << ";\n";
                if (needka[i]) {
                    o << "    const hyk_real " << kname(i, n + 1) << " = " << mul(lit((double)(n + 1)), vname(i, n + 1))
                      << ";\n";
                    flops += 1;
                    if (kslot[i] >= 0 && n + 1 + ((adj || evx) ? 1u : 2u) <= p)
                        o << "    " << smem((uint32_t)kslot[i] + n) << " = " << kname(i, n + 1) << ";\n";
                }
            }
            // Values of earlier orders are re-read from shared memory: the
            // warp barrier keeps the compiler from carrying them in registers.
            // It also reconverges the warp's threads at every order (they run
            // different lanes and may have diverged since the last step):
            // hyk_wm names the whole warp, except in the serving kernel, whose
            // idle threads wait elsewhere (hyk_wm 0: the active threads).
            o << "    HYK_WARP_SYNC();\n";
            if (split) o << "}\n";
        }
        if (split) {
            o << "static __device__ __noinline__ void hyk_jets(hyk_real *__restrict__ S, const hyk_real t0, "
                 "const unsigned hyk_wm = 0xffffffffu) {\n";
            for (uint32_t n = 0; n <= last; ++n) o << "    hyk_jets_o" << n << "(S, t0, hyk_wm);\n";
        }
        o << "}\n";
    }

    // Constants of the events for the kernel template.
    void emit_events(std::ostream &h) const {
        const size_t m = d.ev.size();
        uint32_t nt = 0;
        for (const auto &e : d.ev) nt += e.terminal ? 1u : 0u;
        h << "#define HYK_NEV " << m << "\n#define HYK_NTEV " << nt << "\n#define HYK_EV_SLOT " << evslot << "\n";
        if (!m) return;
        h << "#define HYK_EVC(k, n) S[(HYK_EV_SLOT + (k) * (HYK_ORDER + 1) + (n)) * HYK_STRIDE]\n";
        std::vector<int> idx(m);
        uint32_t it = 0, in = 0;
        for (size_t k = 0; k < m; ++k) idx[k] = d.ev[k].terminal ? (int)it++ : (int)in++;
        auto arr = [&](const char *type, const char *name, auto f) {
            h << "static __constant__ " << type << " " << name << "[" << m << "] = {";
            for (size_t k = 0; k < m; ++k) h << (k ? ", " : "") << f(k);
            h << "};\n";
        };
        arr("int", "hyk_ev_term", [&](size_t k) { return std::to_string(d.ev[k].terminal); });
        arr("int", "hyk_ev_dir", [&](size_t k) { return std::to_string(d.ev[k].direction); });
        arr("int", "hyk_ev_idx", [&](size_t k) { return std::to_string(idx[k]); });
        arr("hyk_real", "hyk_ev_cool", [&](size_t k) { return lit(d.ev[k].cooldown); });
        std::vector<double> bt((size_t)(p + 1) * (p + 1));
        hyk_ev_btab((int)p, bt.data());
        h << "static __constant__ hyk_real hyk_ev_bt[" << bt.size() << "] = {";
        for (size_t k = 0; k < bt.size(); ++k) h << (k ? ", " : "") << lit(bt[k]);
        h << "};\n";
    }

    // ------------------------------------------------------------------
    // Reverse sweep (adjoint module).  Reads the forward coefficients from
    // shared memory only, accumulates the adjoint of every stored
    // coefficient in its own slot and of same-order temporaries in
    // registers, and walks the orders and the operations backwards.  The
    // step size is held fixed: the derivative is that of the Taylor map
    // x_{k+1} = sum_n x^[n](x_k, p, t_k) h_k^n at the taped h_k.
    std::string val(const Ref &r, uint32_t j) const {
        switch (r.kind) {
        case HYK_ARG_U: {
            const std::string s = smem((uint32_t)slot[r.u] + j);
            return r.neg ? "(-" + s + ")" : s;
        }
        case HYK_ARG_NUM:
            return j == 0 ? lit(r.num) : "0.0";
        case HYK_ARG_PAR:
            return j == 0 ? "HYK_PAR(" + std::to_string(r.par) + ")" : "0.0";
        case HYK_ARG_TIME:
            return j == 0 ? "t0" : (j == 1 ? "1.0" : "0.0");
        }
        return "0.0";
    }
    std::string kval(const Ref &r, uint32_t j) const {
        if (r.kind == HYK_ARG_U) {
            const std::string s = smem((uint32_t)kslot[r.u] + j - 1);
            return r.neg ? "(-" + s + ")" : s;
        }
        return (r.kind == HYK_ARG_TIME && j == 1) ? "1.0" : "0.0";
    }
    // ------------------------------------------------------------------
    // Reverse sweep in gather form.  The orders are walked downwards; at
    // order m the operations are walked in reverse.  ub<u> (a register of the
    // order's function) collects the adjoint of coefficient m of u: every
    // consumer of u adds its whole contribution to order m at once, as a sum
    // over the orders n >= m of the consumer's adjoint factor (its history,
    // aslot, read back from memory; order m itself from the register) times a
    // forward coefficient.  An operation whose recurrence reads its own lower
    // orders gathers those terms the same way before its adjoint is complete.
    // Nothing is accumulated in memory: every slot is written once.
    std::string ub(uint32_t u) const { return "ub" + std::to_string(u); }
    std::string hfac(uint32_t u) const { return "hf" + std::to_string(u); }
    // The adjoint factor of u at order n while emitting order m (n >= m).
    std::string hval(uint32_t u, uint32_t n, uint32_t m) const {
        if (n == m) return hfac(u);
        return smem((uint32_t)aslot[u] + n - 1);
    }
    // ub(r) += e (r a variable, or a parameter at order 0).
    // (as fused multiply-adds, which the FP64 pipe issues fastest; scale:
    // ub(r) += scale * e).
    void contrib(const Ref &r, uint32_t m, const std::string &e, const std::string &scale = "") {
        std::string f = scale.empty() ? "hyk_one" : scale;
        if (r.neg) f = "(-" + f + ")";
        if (r.kind == HYK_ARG_U) {
            o << "    " << ub((uint32_t)r.u) << " = __fma_rn(" << f << ", " << e << ", " << ub((uint32_t)r.u) << ");\n";
        } else if (r.kind == HYK_ARG_PAR && m == 0) {
            o << "    pb[" << r.par << "] = __fma_rn(" << f << ", " << e << ", pb[" << r.par << "]);\n";
        }
    }
    // A sum of products as one fused multiply-add chain; "" when empty.
    int gcount = 0;
    std::string gsum(const std::vector<std::pair<std::string, std::string>> &t) {
        if (t.empty()) return "";
        const std::string a = "gs" + std::to_string(gcount++);
        o << "    double " << a << " = __fma_rn(" << t[0].first << ", " << t[0].second << ", hyk_nz);\n";
        for (size_t k = 1; k < t.size(); ++k)
            o << "    " << a << " = __fma_rn(" << t[k].first << ", " << t[k].second << ", " << a << ");\n";
        return a;
    }
    // The adjoint factor at order m is final: keep it for the lower orders.
    void keep(uint32_t u, uint32_t m) {
        if (m >= 1) o << "    " << smem((uint32_t)aslot[u] + m - 1) << " = " << hfac(u) << ";\n";
    }
    // Whether an argument receives an adjoint at order m (a variable, or a
    // parameter at order 0).
    static bool wants(const Ref &r, uint32_t m) { return r.kind == HYK_ARG_U || (r.kind == HYK_ARG_PAR && m == 0); }

    void emit_op_bw(uint32_t k, uint32_t m) {
        const auto &op = d.ops[k];
        const uint32_t u = N + k;
        if (alias[u]) return;
        const Ref A = res(op.a), B = res(op.b);
        const Ref self{HYK_ARG_U, (int)u, false, 0, -1};
        const bool unary_fn = op.op == HYK_OP_SQRT || op.op == HYK_OP_POW || op.op == HYK_OP_EXP ||
                              op.op == HYK_OP_LOG || op.op == HYK_OP_SIN || op.op == HYK_OP_COS;
        // A function of a constant is constant: nothing flows back above order 0.
        if (unary_fn && m >= 1 && !varying(A)) return;
        const std::string G = ub(u), H = hfac(u), inv = "i" + std::to_string(u);
        std::vector<std::pair<std::string, std::string>> t;
        if (fused_sc(u)) {
            // c_n = a_n + sum_i k_i t_i,n: abar_m += cbar_m, tbar_i,m += k_i cbar_m
            const Ref FA = fz_a(u);
            const std::vector<Ref> FX = fz_x(u);
            if (FA.kind == HYK_ARG_U) contrib(FA, m, G);
            for (size_t i = 0; i < FX.size(); ++i) contrib(FX[i], m, G, lit(fz_k(u)[i]));
            return;
        }
        if (fused(u)) {
            // c_n = a_n + sum_i sum_j x_i,j x_i,n-j: abar_m += cbar_m,
            // xbar_i,m += 2 sum_{n>=m} cbar_n x_i,n-m
            const Ref FA = fz_a(u);
            o << "    const double " << H << " = " << G << ";\n";
            keep(u, m);
            if (FA.kind == HYK_ARG_U) contrib(FA, m, H);
            for (const Ref &x : fz_x(u)) {
                t.clear();
                if (wants(x, m))
                    for (uint32_t n = m; n < p; ++n) t.push_back({hval(u, n, m), val(x, n - m)});
                const std::string sx = gsum(t);
                if (!sx.empty()) contrib(x, m, sx, "2.0");
            }
            return;
        }
        switch (op.op) {
        case HYK_OP_ADD:
            if (nz(A, m)) contrib(A, m, G);
            if (nz(B, m)) contrib(B, m, G);
            break;
        case HYK_OP_SUB:
            if (nz(A, m)) contrib(A, m, G);
            if (nz(B, m)) contrib(B, m, G, "(-hyk_one)");
            break;
        case HYK_OP_NEG:
            if (nz(A, m)) contrib(A, m, G, "(-hyk_one)");
            break;
        case HYK_OP_MUL: {
            // c_n = sum_j a_j b_{n-j}: abar_m += sum_{n>=m} cbar_n b_{n-m}, and symmetrically.
            o << "    const double " << H << " = " << G << ";\n";
            keep(u, m);
            if (nz(A, m) && wants(A, m))
                for (uint32_t n = m; n < p; ++n)
                    if (nz(B, n - m)) t.push_back({hval(u, n, m), val(B, n - m)});
            const std::string sa = gsum(t);
            if (!sa.empty()) contrib(A, m, sa);
            t.clear();
            if (nz(B, m) && wants(B, m))
                for (uint32_t n = m; n < p; ++n)
                    if (nz(A, n - m)) t.push_back({hval(u, n, m), val(A, n - m)});
            const std::string sb = gsum(t);
            if (!sb.empty()) contrib(B, m, sb);
            break;
        }
        case HYK_OP_DIV: {
            // c_n = (a_n - sum_{j>=1} b_j c_{n-j}) / b_0, w_n = cbar_n / b_0:
            // cbar_m -= sum_{n>m} w_n b_{n-m}; abar_m += w_m; bbar_m -= sum_{n>=m} w_n c_{n-m}.
            for (uint32_t n = m + 1; n < p; ++n)
                if (nz(B, n - m)) t.push_back({hval(u, n, m), val(B, n - m)});
            const std::string ss = gsum(t);
            if (!ss.empty()) o << "    " << G << " = " << G << " - " << ss << ";\n";
            o << "    const double " << H << " = __fma_rn(" << G << ", " << inv << ", hyk_nz);\n";
            keep(u, m);
            if (nz(A, m)) contrib(A, m, H);
            t.clear();
            if (nz(B, m) && wants(B, m))
                for (uint32_t n = m; n < p; ++n) t.push_back({hval(u, n, m), val(self, n - m)});
            const std::string sb = gsum(t);
            if (!sb.empty()) contrib(B, m, sb, "(-hyk_one)");
            break;
        }
        case HYK_OP_SQUARE: {
            o << "    const double " << H << " = " << G << ";\n";
            keep(u, m);
            if (nz(A, m) && wants(A, m))
                for (uint32_t n = m; n < p; ++n)
                    if (nz(A, n - m)) t.push_back({hval(u, n, m), val(A, n - m)});
            const std::string sa = gsum(t);
            if (!sa.empty()) contrib(A, m, sa, "2.0");
            break;
        }
        case HYK_OP_SQRT: {
            // c_n = (a_n - sum_{0<j<n} c_j c_{n-j}) / (2 c_0), w_n = cbar_n / (2 c_0):
            // cbar_m -= 2 sum_{n>m} w_n c_{n-m}; abar_m += w_m.
            for (uint32_t n = m + 1; n < p; ++n) t.push_back({hval(u, n, m), val(self, n - m)});
            const std::string ss = gsum(t);
            if (!ss.empty()) o << "    " << G << " = __fma_rn(-2.0, " << ss << ", " << G << ");\n";
            o << "    const double " << H << " = __fma_rn(" << G << ", " << inv << ", hyk_nz);\n";
            keep(u, m);
            if (nz(A, m)) contrib(A, m, H);
            break;
        }
        case HYK_OP_POW: {
            // c_n = (1/(n a_0)) sum_{j<n} (n al - j (al+1)) a_{n-j} c_j, w_n = cbar_n / (n a_0):
            // cbar_m += sum_{n>m} w_n coef(n, m) a_{n-m};
            // abar_m += sum_{n>=m} w_n coef(n, n-m) c_{n-m} (m >= 1);
            // abar_0 += al cbar_0 c_0 / a_0 - sum_{n>=1} n w_n c_n.
            const double alpha = op.b.num;
            for (uint32_t n = m + 1; n < p; ++n)
                if (nz(A, n - m)) {
                    const double coef = (double)n * alpha - (double)m * (alpha + 1.0);
                    t.push_back({hval(u, n, m), "__fma_rn(" + lit(coef) + ", " + val(A, n - m) + ", hyk_nz)"});
                }
            const std::string ss = gsum(t);
            if (!ss.empty()) o << "    " << G << " = " << G << " + " << ss << ";\n";
            t.clear();
            if (m == 0) {
                for (uint32_t n = 1; n < p; ++n) t.push_back({hval(u, n, m), "__fma_rn(" + lit(-(double)n) + ", " + val(self, n) + ", hyk_nz)"});
                const std::string s0 = gsum(t);
                std::string e = "(" + G + " * " + lit(alpha) + ") * (" + val(self, 0) + " * " + inv + ")";
                if (!s0.empty()) e = "(" + e + " + " + s0 + ")";
                contrib(A, 0, e);
                break;
            }
            o << "    const double " << H << " = (" << G << " * " << inv << ") * " << lit(1.0 / (double)m) << ";\n";
            keep(u, m);
            for (uint32_t n = m; n < p; ++n) {
                const double coef = (double)n * alpha - (double)(n - m) * (alpha + 1.0);
                t.push_back({hval(u, n, m), "__fma_rn(" + lit(coef) + ", " + val(self, n - m) + ", hyk_nz)"});
            }
            const std::string sa = gsum(t);
            if (!sa.empty()) contrib(A, m, sa);
            break;
        }
        case HYK_OP_EXP: {
            // c_n = (1/n) sum_{j=1}^{n} (j a_j) c_{n-j}, w_n = cbar_n / n:
            // cbar_m += sum_{n>m} w_n (n-m) a_{n-m}; abar_m += m sum_{n>=m} w_n c_{n-m} (m >= 1);
            // abar_0 += cbar_0 c_0.
            for (uint32_t n = m + 1; n < p; ++n)
                if (knz(A, n - m)) t.push_back({hval(u, n, m), kval(A, n - m)});
            const std::string ss = gsum(t);
            if (!ss.empty()) o << "    " << G << " = " << G << " + " << ss << ";\n";
            t.clear();
            if (m == 0) {
                contrib(A, 0, "(" + G + " * " + val(self, 0) + ")");
                break;
            }
            o << "    const double " << H << " = __fma_rn(" << G << ", " << lit(1.0 / (double)m) << ", hyk_nz);\n";
            keep(u, m);
            if (knz(A, m))
                for (uint32_t n = m; n < p; ++n) t.push_back({hval(u, n, m), val(self, n - m)});
            const std::string sa = gsum(t);
            if (!sa.empty()) contrib(A, m, sa, lit((double)m));
            break;
        }
        case HYK_OP_LOG: {
            // c_n = (a_n - (1/n) sum_{0<j<n} (j c_j) a_{n-j}) / a_0, w_n = cbar_n / a_0:
            // cbar_m -= m sum_{n>m} (w_n / n) a_{n-m};
            // abar_m += w_m - sum_{n>m} (w_n / n) (n-m) c_{n-m} (m >= 1);
            // abar_0 += cbar_0 / a_0 - sum_{n>=1} w_n c_n.
            if (m >= 1 && varying(A))
                for (uint32_t n = m + 1; n < p; ++n)
                    if (nz(A, n - m)) t.push_back({hval(u, n, m), "__fma_rn(" + lit(1.0 / (double)n) + ", " + val(A, n - m) + ", hyk_nz)"});
            const std::string ss = gsum(t);
            if (!ss.empty()) o << "    " << G << " = __fma_rn(" << lit(-(double)m) << ", " << ss << ", " << G << ");\n";
            t.clear();
            if (m == 0) {
                for (uint32_t n = 1; n < p; ++n) t.push_back({hval(u, n, m), val(self, n)});
                const std::string s0 = gsum(t);
                std::string e = "(" + G + " * " + inv + ")";
                if (!s0.empty()) e = "(" + e + " - " + s0 + ")";
                contrib(A, 0, e);
                break;
            }
            o << "    const double " << H << " = __fma_rn(" << G << ", " << inv << ", hyk_nz);\n";
            keep(u, m);
            std::string e = H;
            if (varying(A)) {
                for (uint32_t n = m + 1; n < p; ++n)
                    t.push_back({hval(u, n, m), "__fma_rn(" + lit(1.0 / (double)n) + ", " + kval(self, n - m) + ", hyk_nz)"});
                const std::string sa = gsum(t);
                if (!sa.empty()) e = "(" + H + " - " + sa + ")";
            }
            if (nz(A, m)) contrib(A, m, e);
            break;
        }
        case HYK_OP_SIN:
        case HYK_OP_COS: {
            // s_n = (1/n) sum (j a_j) c_{n-j}, c_n = -(1/n) sum (j a_j) s_{n-j};
            // w_n = sigma ubar_n / n (sigma = +1 sin, -1 cos):
            // ubar_m += sum_{n>m} wP_n (n-m) a_{n-m} (wP the partner's factors);
            // abar_m += m sum_{n>=m} w_n P_{n-m} (m >= 1); abar_0 += sigma ubar_0 P_0.
            const uint32_t partner = (uint32_t)op.aux;
            const bool is_sin = op.op == HYK_OP_SIN;
            const Ref P{HYK_ARG_U, (int)partner, false, 0, -1};
            for (uint32_t n = m + 1; n < p; ++n)
                if (knz(A, n - m)) t.push_back({hval(partner, n, m), kval(A, n - m)});
            const std::string ss = gsum(t);
            if (!ss.empty()) o << "    " << G << " = " << G << " + " << ss << ";\n";
            t.clear();
            if (m == 0) {
                contrib(A, 0, "(" + std::string(is_sin ? "" : "-") + G + " * " + val(P, 0) + ")");
                break;
            }
            o << "    const double " << H << " = __fma_rn(" << G << ", " << lit((is_sin ? 1.0 : -1.0) / (double)m) << ", hyk_nz);\n";
            keep(u, m);
            if (knz(A, m))
                for (uint32_t n = m; n < p; ++n) t.push_back({hval(u, n, m), val(P, n - m)});
            const std::string sa = gsum(t);
            if (!sa.empty()) contrib(A, m, sa, lit((double)m));
            break;
        }
        default:
            break;
        }
    }

    void emit_inverses(bool only_used) {
        (void)only_used;
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const auto &op = d.ops[k];
            const uint32_t u = N + k;
            if (alias[u]) continue;
            const Ref A = res(op.a), B = res(op.b);
            const std::string inv = "i" + std::to_string(u);
            if (op.op == HYK_OP_DIV) o << "    const double " << inv << " = 1.0 / " << val(B, 0) << ";\n";
            if (op.op == HYK_OP_POW || op.op == HYK_OP_LOG) o << "    const double " << inv << " = 1.0 / " << val(A, 0) << ";\n";
            if (op.op == HYK_OP_SQRT) o << "    const double " << inv << " = 1.0 / (2.0 * sqrt(" << val(A, 0) << "));\n";
        }
    }

    // One function per order keeps each compiled block small (compile time
    // grows faster than linearly with the size of a straight-line block).
    // Order m: the state variables' adjoints start from the Horner update
    // (lam_i h^m); the right-hand sides receive x̄_{m+1} / (m+1) (x̄_{m+1} kept
    // in slot akslot[i] by order m+1); then the operations in reverse order.
    void emit_bw() {
        for (uint32_t m = 0; m < p; ++m) {
            gcount = 0;
            o << "static __device__ __noinline__ void hyk_bw_o" << m
              << "(double *__restrict__ S, const double t0, const double h, double *__restrict__ lam, "
                 "double *__restrict__ pb) {\n";
            o << "    (void)t0;\n    HYK_FMAOPS_CONSTS\n    (void)hyk_nz;\n";
            emit_inverses(true);
            o << "    double hm = 1.0;\n";
            for (uint32_t q = 0; q < m; ++q) o << "    hm = hm * h;\n";
            for (uint32_t i = 0; i < N; ++i) o << "    double " << ub(i) << " = lam[" << i << "] * hm;\n";
            for (uint32_t k = 0; k < d.n_ops; ++k)
                if (!alias[N + k]) o << "    double " << ub(N + k) << " = 0.0;\n";
            for (uint32_t ii = N; ii-- > 0;) {
                const Ref r = res(d.rhs[ii]);
                if (nz(r, m)) contrib(r, m, smem((uint32_t)akslot[ii]), lit(1.0 / (double)(m + 1)));
            }
            for (uint32_t kk = d.n_ops; kk-- > 0;) emit_op_bw(kk, m);
            for (uint32_t i = 0; i < N; ++i) {
                if (m > 0)
                    o << "    " << smem((uint32_t)akslot[i]) << " = " << ub(i) << ";\n";
                else
                    o << "    lam[" << i << "] = " << ub(i) << ";\n";
            }
            o << "}\n";
        }
        o << "static __device__ __noinline__ void hyk_jets_bw(double *__restrict__ S, const double t0, const double h, "
             "double *__restrict__ lam, double *__restrict__ pb) {\n";
        // x̄_p comes from the Horner update only
        o << "    double hp = 1.0;\n";
        for (uint32_t q = 0; q < p; ++q) o << "    hp = hp * h;\n";
        for (uint32_t i = 0; i < N; ++i) o << "    " << smem((uint32_t)akslot[i]) << " = lam[" << i << "] * hp;\n";
        for (uint32_t mm = p; mm-- > 0;) o << "    hyk_bw_o" << mm << "(S, t0, h, lam, pb);\n";
        o << "}\n";
    }
};

// ---------------------------------------------------------------------------
// Team form.  HYK_TEAM consecutive threads of a warp integrate one trajectory
// together: the u-operations of one dependency level are spread over the
// team, one operation per thread and round, and every coefficient lives in
// the trajectory's own shared-memory region (stride 1), so that a system too
// large for 32 lanes of shared memory still runs from shared memory with
// enough warps per SM.  The orders 1..p-1 are a runtime loop over per-level
// code whose operand slots come from a table of per-operation descriptors;
// each operation performs the same terms in the same order as the lane form
// (Gen::emit_op), so both forms give the same bits.
struct TeamGen {
    Gen g;  // alias folding, histories and j*a_j needs (gpu arithmetic, no adjoint)
    const Dec &d;
    uint32_t p, N, NU;
    // Cold state rows (when every state variable is read by the recurrences
    // at the current order only, as in the N-body problem): each state
    // variable keeps two shared-memory slots, order n in slot n & 1 (order 0
    // is copied in at the start of the step; the update of order n writes
    // order n + 1 into the other slot, so that the updates that read a state
    // variable, x' = v, still find its order n), and all its orders 0..p live
    // in the team's region of the module's global buffer, order-major
    // (HYK_CROW(i, n)), where the step size, the state update and the
    // outputs read them.
    bool cold = false;
    bool coldvar(uint32_t u) const { return cold && u < N; }
    // Whether u's history is in shared memory (slot + n) rather than its current order only.
    bool th(uint32_t u) const { return g.hist[u] && !(cold && u < N); }
    uint32_t XS, HS, KS;  // strides of state rows, operation histories, j*a_j histories (odd)
    std::vector<int> tslot, tkslot, tislot, level;
    uint32_t nslot = 0, par_slot = 0;
    int max_level = 0;
    struct Desc {
        int a = 0, b = 0, c = 0, ka = 0, kc = 0, inv = 0, prt = 0, x3 = 0;
        double num = 0;
    };
    std::vector<Desc> descs;
    struct Group {
        std::string key;
        std::vector<uint32_t> members;  // u-variables (operations) or state indices (updates)
        uint32_t off = 0;               // first descriptor
    };
    std::vector<std::vector<Group>> levels;  // [level - 1]
    std::vector<Group> supd;                 // state updates
    std::vector<double> alphas;              // distinct pow exponents
    std::vector<double> scales;              // the leaves' numbers of the sums of scaled terms
    std::string err;
    std::ostringstream o;
    // Unrolling of the convolution loops over j (the same sequence of fused
    // multiply-adds, with the operand loads of later terms hoisted; 4 measured
    // best on the 6-body problem against 1, 2 and 8).
    int ju = 4;

    TeamGen(const Dec &dd, uint32_t order, bool cold_rows = false)
        : g(dd, order, false, false), d(dd), p(order), N(dd.n_eq), NU(dd.n_u()) {
        cold = cold_rows;
        for (uint32_t i = 0; i < N; ++i) cold = cold && !g.hread[i];
        XS = cold ? 2u : (p + 1) | 1u;
        HS = p | 1u;
        KS = (p >= 2 ? p - 1 : 1) | 1u;
        tslot.assign(NU, -1);
        tkslot.assign(NU, -1);
        tislot.assign(NU, -1);
        level.assign(NU, 0);
        uint32_t s = 0;
        for (uint32_t i = 0; i < N; ++i) {
            tslot[i] = (int)s;
            s += XS;
        }
        for (uint32_t u = N; u < NU; ++u)
            if (!g.alias[u]) {
                tslot[u] = (int)s;
                s += (g.hist[u] && !g.cst[u]) ? HS : 1;
            }
        for (uint32_t u = 0; u < NU; ++u)
            if (g.needka[u] && !g.alias[u]) {
                tkslot[u] = (int)s;
                s += KS;
            }
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const int op = d.ops[k].op;
            if (!g.alias[N + k] && (op == HYK_OP_DIV || op == HYK_OP_SQRT || op == HYK_OP_POW || op == HYK_OP_LOG))
                tislot[N + k] = (int)s++;
        }
        par_slot = s;
        s += d.n_pars;
        nslot = s;
    }

    // The operands as the recurrence reads them: a fused a + x^2 (hyk_fuse.h)
    // reads a and x (in the descriptor's a and b).
    std::pair<Ref, Ref> opnds(uint32_t u) const {
        if (g.fused(u)) return {g.fz_a(u), g.fz_x(u)[0]};
        const auto &op = d.ops[u - N];
        return {g.res(op.a), g.res(op.b)};
    }

    // A time-constant operation (Gen::cst) reads like a parameter: its value in
    // its slot at order 0, zero above.
    bool isK(const Ref &r) const {
        return r.kind == HYK_ARG_NUM || r.kind == HYK_ARG_PAR || (r.kind == HYK_ARG_U && g.cst[r.u]);
    }
    bool isU(const Ref &r) const { return r.kind == HYK_ARG_U && !g.cst[r.u]; }
    static bool isT(const Ref &r) { return r.kind == HYK_ARG_TIME; }

    // Whether the team form covers an operation (operand kinds per operation).
    bool supported(uint32_t u, std::string &why) const {
        const auto &op = d.ops[u - N];
        const Ref A = g.res(op.a), B = g.res(op.b);
        auto bad = [&](const char *m) {
            why = std::string(m) + " at u" + std::to_string(u);
            return false;
        };
        if (g.cst[u]) return true;  // order 0 only
        if (g.fused(u)) return true;  // two time-varying u-variables (hyk_fuse.h)
        switch (op.op) {
        case HYK_OP_ADD:
        case HYK_OP_SUB:
            if (isT(A) && isT(B)) return bad("time +- time");
            if (A.kind == HYK_ARG_NUM && B.kind == HYK_ARG_NUM) return bad("number +- number");
            return true;
        case HYK_OP_MUL:
            if (isT(A) && isT(B)) return bad("time * time");
            if (A.kind == HYK_ARG_NUM && B.kind == HYK_ARG_NUM) return bad("number * number");
            return true;
        case HYK_OP_DIV:
            if (!((isU(A) && isU(B)) || (isU(A) && isK(B)) || (isK(A) && isU(B)))) return bad("division operands");
            return true;
        case HYK_OP_EXP:
        case HYK_OP_SIN:
        case HYK_OP_COS:
            if (!isU(A) && !isT(A)) return bad("constant argument");
            return true;
        case HYK_OP_SQUARE:
        case HYK_OP_SQRT:
        case HYK_OP_POW:
        case HYK_OP_LOG:
            if (!isU(A)) return bad("non-variable argument");
            return true;
        default:
            return bad("operation");
        }
    }

    std::string rkey(const Ref &r) const {
        if (r.kind == HYK_ARG_U && g.cst[r.u]) return std::string("3") + (r.neg ? "n" : "p");
        std::string k = std::to_string(r.kind);
        if (isU(r)) k += std::string(r.neg ? "n" : "p") + (coldvar(r.u) ? "d" : th(r.u) ? "h" : "c");
        return k;
    }

    bool analyse() {
        if (!d.ev.empty()) {
            err = "events are handled by the lane form";
            return false;
        }
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const uint32_t u = N + k;
            if (g.alias[u]) continue;
            if (!supported(u, err)) return false;
            const auto AB = opnds(u);
            const Ref A = AB.first, B = AB.second;
            int lv = 0;  // after every u-variable argument (time-constant ones included: order 0 reads them)
            if (A.kind == HYK_ARG_U) lv = std::max(lv, level[A.u]);
            if (B.kind == HYK_ARG_U) lv = std::max(lv, level[B.u]);
            if (g.fused(u))
                for (const Ref &x : g.fz_x(u)) lv = std::max(lv, level[x.u]);
            level[u] = lv + 1;
            max_level = std::max(max_level, lv + 1);
        }
        levels.assign(max_level, {});
        std::vector<std::map<std::string, size_t>> index(max_level);
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const uint32_t u = N + k;
            if (g.alias[u]) continue;
            const auto &op = d.ops[k];
            const auto AB = opnds(u);
            const Ref A = AB.first, B = AB.second;
            std::string key = "op" + std::to_string(op.op) + "_" + rkey(A) + "_" + rkey(B) + "_c" +
                              (g.cst[u] ? "K" : (g.hist[u] ? "h" : "c")) + (g.needka[u] ? "k" : "");
            if (g.fused(u)) {  // a fused sum: its leaves' kinds (the first is B)
                if (g.fused_sc(u)) key = "op" + std::to_string(HYK_OP_ADD) + "_" + rkey(A) + "_" + rkey(B) + "_S";
                else key += "_F";
                for (const Ref &x : g.fz_x(u)) key += rkey(x);
            }
            if (op.op == HYK_OP_POW) {
                char buf[40];
                std::snprintf(buf, sizeof buf, "_a%a", op.b.num);
                key += buf;
            }
            if (op.op == HYK_OP_SIN || op.op == HYK_OP_COS) key += (u < (uint32_t)op.aux) ? "_lead" : "_follow";
            auto &lv = levels[level[u] - 1];
            auto &ix = index[level[u] - 1];
            auto it = ix.find(key);
            if (it == ix.end()) {
                ix[key] = lv.size();
                lv.push_back(Group{key, {u}, 0});
            } else {
                lv[it->second].members.push_back(u);
            }
        }
        for (auto &lv : levels)
            std::sort(lv.begin(), lv.end(), [](const Group &x, const Group &y) { return x.key < y.key; });
        std::map<std::string, size_t> sx;
        for (uint32_t i = 0; i < N; ++i) {
            const Ref R = g.res(d.rhs[i]);
            const std::string key = "upd_" + rkey(R) + (g.needka[i] ? "k" : "");
            auto it = sx.find(key);
            if (it == sx.end()) {
                sx[key] = supd.size();
                supd.push_back(Group{key, {i}, 0});
            } else {
                supd[it->second].members.push_back(i);
            }
        }
        std::sort(supd.begin(), supd.end(), [](const Group &x, const Group &y) { return x.key < y.key; });
        // Slots of the operations in group order (the layout of the
        // constructor, reordered): the members of a group take consecutive
        // regions of odd stride, so that the threads of a round (consecutive
        // members) find their coefficients in distinct shared-memory banks,
        // and so do the groups that read them in the same member order.
        {
            uint32_t s = N * XS;
            for (auto &lv : levels)
                for (auto &gr : lv)
                    for (uint32_t u : gr.members) {
                        tslot[u] = (int)s;
                        s += (g.hist[u] && !g.cst[u]) ? HS : 1;
                    }
            for (uint32_t i = 0; i < N; ++i)
                if (g.needka[i]) {
                    tkslot[i] = (int)s;
                    s += KS;
                }
            for (auto &lv : levels)
                for (auto &gr : lv)
                    for (uint32_t u : gr.members)
                        if (g.needka[u]) {
                            tkslot[u] = (int)s;
                            s += KS;
                        }
            for (auto &lv : levels)
                for (auto &gr : lv)
                    for (uint32_t u : gr.members)
                        if (tislot[u] >= 0) tislot[u] = (int)s++;
            if (s != par_slot) {
                err = "internal: team slot layout";
                return false;
            }
        }
        // Descriptors, group by group.
        auto slot_of = [&](const Ref &r) {
            if (r.kind == HYK_ARG_U) return tslot[r.u];
            if (r.kind == HYK_ARG_PAR) return (int)par_slot + r.par;
            return 0;
        };
        for (auto &lv : levels)
            for (auto &gr : lv) {
                gr.off = (uint32_t)descs.size();
                for (uint32_t u : gr.members) {
                    const auto &op = d.ops[u - N];
                    const auto AB = opnds(u);
                    const Ref A = AB.first, B = AB.second;
                    Desc D;
                    D.a = slot_of(A);
                    D.b = slot_of(B);
                    D.c = tslot[u];
                    D.ka = isU(A) ? tkslot[A.u] : 0;
                    D.kc = tkslot[u];
                    D.inv = tislot[u];
                    if (op.op == HYK_OP_SIN || op.op == HYK_OP_COS) D.prt = tslot[op.aux];
                    if (A.kind == HYK_ARG_NUM) D.num = A.num;
                    if (B.kind == HYK_ARG_NUM && op.op != HYK_OP_POW) D.num = B.num;
                    if (g.fused(u)) {
                        // a fused sum: the leaves' slots in b, inv, prt, x3; a
                        // sum of scaled terms the offset of its leaves' numbers
                        // in hyk_tsc in ka
                        const std::vector<Ref> X = g.fz_x(u);
                        int *f[HYK_FUSE_MAX] = {&D.b, &D.inv, &D.prt, &D.x3};
                        for (size_t i = 0; i < X.size(); ++i) *f[i] = tslot[X[i].u];
                        if (g.fused_sc(u)) {
                            D.ka = (int)scales.size();
                            for (double k : g.fz_k(u)) scales.push_back(k);
                        }
                    }
                    descs.push_back(D);
                }
                if (d.ops[gr.members[0] - N].op == HYK_OP_POW) {
                    const double al = d.ops[gr.members[0] - N].b.num;
                    bool seen = false;
                    for (double x : alphas) seen = seen || std::memcmp(&x, &al, sizeof al) == 0;
                    if (!seen) alphas.push_back(al);
                }
            }
        for (auto &gr : supd) {
            gr.off = (uint32_t)descs.size();
            for (uint32_t i : gr.members) {
                const Ref R = g.res(d.rhs[i]);
                Desc D;
                D.a = slot_of(R);
                D.b = (int)i;  // (cold rows: the state index)
                D.c = tslot[i];
                D.kc = tkslot[i];
                if (R.kind == HYK_ARG_NUM) D.num = R.num;
                descs.push_back(D);
            }
        }
        return true;
    }

    // Weighted share of busy threads over all rounds of one order for a team of T threads.
    double util(uint32_t T) const {
        double work = 0, busy = 0;
        auto add = [&](const Group &gr, double w) {
            const double m = (double)gr.members.size();
            work += m * w;
            busy += std::ceil(m / T) * T * w;
        };
        for (auto &lv : levels)
            for (auto &gr : lv) {
                const auto &op = d.ops[gr.members[0] - N];
                const Ref A = g.res(op.a), B = g.res(op.b);
                bool conv = false;
                if (g.fused(gr.members[0])) {
                    add(gr, g.fused_sq(gr.members[0]) ? 0.5 * p : 1.0);
                    continue;
                }
                switch (op.op) {
                case HYK_OP_MUL: conv = isU(A) && isU(B); break;
                case HYK_OP_DIV: conv = isU(B); break;
                case HYK_OP_ADD: case HYK_OP_SUB: conv = false; break;
                default: conv = true;
                }
                add(gr, conv ? 0.5 * p : 1.0);
            }
        for (auto &gr : supd) add(gr, 1.0);
        return busy > 0 ? work / busy : 0.0;
    }

    // ---- expressions (D = the thread's descriptor, n = the order)
    static std::string wrap(const Ref &r, const std::string &s) { return r.neg ? "(-" + s + ")" : s; }
    // The current order of u-variable u (not time-constant) whose slot is in
    // the expression fld: its history's order n, its only slot, or (a cold
    // state variable) slot n & 1.
    std::string now(uint32_t u, const std::string &fld, bool n0) const {
        if (n0 || (!th(u) && !coldvar(u))) return "S[" + fld + "]";
        return coldvar(u) ? "S[" + fld + " + (n & 1)]" : "S[" + fld + " + n]";
    }
    // Operand coefficient at the current order n (runtime) or at order 0.
    std::string cur(const Ref &r, char f, bool n0) const {
        const std::string fld = std::string("D.") + f;
        switch (r.kind) {
        case HYK_ARG_U:
            if (g.cst[r.u]) return n0 ? wrap(r, "S[" + fld + "]") : "";
            return wrap(r, now(r.u, fld, n0));
        case HYK_ARG_PAR:
            return n0 ? "S[" + fld + "]" : "";
        case HYK_ARG_NUM:
            return n0 ? "D.num" : "";
        case HYK_ARG_TIME:
            return n0 ? "t0" : "";  // order n >= 2; order 1 handled by the caller
        }
        return "";
    }
    // Operand coefficient at order J (expression, a past order: needs the history).
    std::string at(const Ref &r, char f, const std::string &J) const {
        return wrap(r, std::string("S[D.") + f + " + " + J + "]");
    }
    std::string K(const Ref &r, char f) const {
        return r.kind == HYK_ARG_NUM ? "D.num" : wrap(r, std::string("S[D.") + f + "]");
    }

    void out(uint32_t u, bool n0, const std::string &v) {
        o << "            const hyk_real v = " << v << ";\n";
        o << "            S[D.c" << ((!n0 && g.hist[u]) ? " + n" : "") << "] = v;\n";
        if (!n0 && g.needka[u]) o << "            S[D.kc + n - 1] = HYK_MUL((hyk_real)n, v);\n";
    }

    void addsub(const std::string &a, const std::string &b, bool add, uint32_t u, bool n0) {
        std::string v;
        if (!a.empty() && !b.empty())
            v = add ? "HYK_ADD(" + a + ", " + b + ")" : "HYK_SUB(" + a + ", " + b + ")";
        else if (!a.empty())
            v = a;
        else if (!b.empty())
            v = add ? b : "(-" + b + ")";
        else
            v = lit(0.0);
        out(u, n0, v);
    }

    void emit_group_op(const Group &gr, bool n0) {
        const uint32_t u = gr.members[0];
        if (!n0 && g.cst[u]) return;  // time-constant: order 0 only
        const auto &op = d.ops[u - N];
        const auto AB = opnds(u);
        const Ref A = AB.first, B = AB.second;
        const std::string fma_ = "HYK_FMA";
        o << "        // " << gr.key << "\n";
        o << "#pragma unroll 1\n";
        o << "        for (int q = r; q < " << gr.members.size() << "; q += HYK_TEAM) {\n";
        o << "            const hyk_tdesc &D = hyk_td[" << gr.off << " + q];\n";
        if (g.fused_sc(u)) {
            // a + sum_i k_i t_i in one chain (hyk_fuse.h), the lane form's
            // arithmetic; the leaves' slots are in D.b, D.inv, D.prt, D.x3,
            // their numbers in hyk_tsc from D.ka
            const std::vector<Ref> X = g.fz_x(u);
            const char *lf[HYK_FUSE_MAX] = {"D.b", "D.inv", "D.prt", "D.x3"};
            std::string r = A.kind == HYK_ARG_U ? cur(A, 'a', n0) : "";
            for (size_t i = 0; i < X.size(); ++i) {
                const std::string x = now(X[i].u, lf[i], n0);
                const std::string k = "hyk_tsc[D.ka + " + std::to_string(i) + "]";
                r = r.empty() ? "HYK_MUL(" + k + ", " + x + ")" : fma_ + "(" + k + ", " + x + ", " + r + ")";
            }
            out(u, n0, r);
            o << "        }\n";
            return;
        }
        if (g.fused(u)) {
            // a + sum_i x_i^2 in one chain (hyk_fuse.h), the lane form's arithmetic;
            // the leaves' slots are in D.b, D.inv, D.prt, D.x3
            const std::vector<Ref> X = g.fz_x(u);
            const char *lf[HYK_FUSE_MAX] = {"D.b", "D.inv", "D.prt", "D.x3"};
            auto lx = [&](size_t i, const std::string &J) { return "S[" + std::string(lf[i]) + " + " + J + "]"; };
            const bool ha = A.kind == HYK_ARG_U;
            if (n0) {
                std::string r = ha ? cur(A, 'a', true) : "";
                for (size_t i = 0; i < X.size(); ++i)
                    r = r.empty() ? "HYK_MUL(" + lx(i, "0") + ", " + lx(i, "0") + ")"
                                  : fma_ + "(" + lx(i, "0") + ", " + lx(i, "0") + ", " + r + ")";
                out(u, true, r);
            } else {
                for (size_t i = 0; i < X.size(); ++i) {
                    if (i == 0)
                        o << "            hyk_real acc = HYK_MUL(" << lx(0, "0") << ", " << lx(0, "n") << ");\n";
                    else
                        o << "            acc = " << fma_ << "(" << lx(i, "0") << ", " << lx(i, "n") << ", acc);\n";
                    o << "#pragma unroll " << ju << "\n";
                    o << "            for (int j = 1; 2 * j < n; ++j) acc = " << fma_ << "(" << lx(i, "j") << ", "
                      << lx(i, "n - j") << ", acc);\n";
                }
                if (ha)
                    o << "            acc = " << fma_ << "(" << lit(2.0) << ", acc, " << cur(A, 'a', false) << ");\n";
                else
                    o << "            acc = HYK_ADD(acc, acc);\n";
                o << "            if ((n & 1) == 0) {\n";
                for (size_t i = 0; i < X.size(); ++i)
                    o << "                acc = " << fma_ << "(" << lx(i, "n / 2") << ", " << lx(i, "n / 2") << ", acc);\n";
                o << "            }\n";
                out(u, false, "acc");
            }
            o << "        }\n";
            return;
        }
        if (n0) {
            const std::string a = cur(A, 'a', true), b = cur(B, 'b', true);
            switch (op.op) {
            case HYK_OP_ADD: out(u, true, "(" + a + " + " + b + ")"); break;
            case HYK_OP_SUB: out(u, true, "(" + a + " - " + b + ")"); break;
            case HYK_OP_NEG: out(u, true, "(-" + a + ")"); break;  // of a constant (a NEG of a u-variable is folded)
            case HYK_OP_MUL: out(u, true, a + " * " + b); break;
            case HYK_OP_DIV:
                out(u, true, "(" + a + " / " + b + ")");
                o << "            S[D.inv] = " << lit(1.0) << " / " << b << ";\n";
                break;
            case HYK_OP_SQUARE: out(u, true, a + " * " + a); break;
            case HYK_OP_SQRT:
                out(u, true, "sqrt(" + a + ")");
                o << "            S[D.inv] = " << lit(1.0) << " / (" << lit(2.0) << " * v);\n";
                break;
            case HYK_OP_POW:
                out(u, true, "HYK_DM_POW(" + a + ", " + lit(op.b.num) + ")");
                o << "            S[D.inv] = " << lit(1.0) << " / " << a << ";\n";
                break;
            case HYK_OP_EXP: out(u, true, "HYK_DM_EXP(" + a + ")"); break;
            case HYK_OP_LOG:
                out(u, true, "HYK_DM_LOG(" + a + ")");
                o << "            S[D.inv] = " << lit(1.0) << " / " << a << ";\n";
                break;
            case HYK_OP_SIN:
            case HYK_OP_COS:
                if (u < (uint32_t)op.aux) {
                    o << "            hyk_real sv, cv;\n";
                    o << "            HYK_DM_SINCOS(" << a << ", &sv, &cv);\n";
                    o << "            S[D.c] = " << (op.op == HYK_OP_SIN ? "sv" : "cv") << ";\n";
                    o << "            S[D.prt] = " << (op.op == HYK_OP_SIN ? "cv" : "sv") << ";\n";
                }
                break;
            }
            o << "        }\n";
            return;
        }
        switch (op.op) {
        case HYK_OP_ADD:
        case HYK_OP_SUB: {
            const bool add = op.op == HYK_OP_ADD;
            const std::string a = cur(A, 'a', false), b = cur(B, 'b', false);
            if (isT(A) || isT(B)) {
                o << "            if (n == 1) {\n";
                addsub(isT(A) ? lit(1.0) : a, isT(B) ? lit(1.0) : b, add, u, false);
                o << "            } else {\n";
                addsub(a, b, add, u, false);
                o << "            }\n";
            } else {
                addsub(a, b, add, u, false);
            }
            break;
        }
        case HYK_OP_MUL:
            if (isU(A) && isU(B)) {
                o << "            hyk_real acc = HYK_MUL(" << at(A, 'a', "0") << ", " << at(B, 'b', "n") << ");\n";
                o << "#pragma unroll " << ju << "\n";
                o << "            for (int j = 1; j <= n; ++j) acc = " << fma_ << "(" << at(A, 'a', "j") << ", "
                  << at(B, 'b', "n - j") << ", acc);\n";
                out(u, false, "acc");
            } else if (isU(A) && isK(B)) {
                out(u, false, "HYK_MUL(" + cur(A, 'a', false) + ", " + K(B, 'b') + ")");
            } else if (isK(A) && isU(B)) {
                out(u, false, "HYK_MUL(" + K(A, 'a') + ", " + cur(B, 'b', false) + ")");
            } else if (isU(A) && isT(B)) {
                o << "            hyk_real acc = " << at(A, 'a', "n - 1") << " * " << lit(1.0) << ";\n";
                o << "            acc = " << fma_ << "(" << at(A, 'a', "n") << ", t0, acc);\n";
                out(u, false, "acc");
            } else if (isT(A) && isU(B)) {
                o << "            hyk_real acc = t0 * " << at(B, 'b', "n") << ";\n";
                o << "            acc = " << fma_ << "(" << lit(1.0) << ", " << at(B, 'b', "n - 1") << ", acc);\n";
                out(u, false, "acc");
            } else if (isK(A) && isK(B)) {
                out(u, false, lit(0.0));
            } else if (isK(A) && isT(B)) {
                out(u, false, "(n == 1 ? " + K(A, 'a') + " * " + lit(1.0) + " : " + lit(0.0) + ")");
            } else {  // time * constant
                out(u, false, "(n == 1 ? " + lit(1.0) + " * " + K(B, 'b') + " : " + lit(0.0) + ")");
            }
            break;
        case HYK_OP_DIV:
            if (isU(B)) {
                o << "            hyk_real acc = HYK_MUL(" << at(B, 'b', "1") << ", S[D.c + n - 1]);\n";
                o << "#pragma unroll " << ju << "\n";
                o << "            for (int j = 2; j <= n; ++j) acc = " << fma_ << "(" << at(B, 'b', "j")
                  << ", S[D.c + n - j], acc);\n";
                const std::string a = isU(A) ? cur(A, 'a', false) : lit(0.0);
                out(u, false, "HYK_MUL(HYK_SUB(" + a + ", acc), S[D.inv])");
            } else {
                out(u, false, "HYK_MUL(" + cur(A, 'a', false) + ", S[D.inv])");
            }
            break;
        case HYK_OP_SQUARE:
            o << "            hyk_real acc = HYK_MUL(" << at(A, 'a', "0") << ", " << at(A, 'a', "n") << ");\n";
            o << "#pragma unroll " << ju << "\n";
            o << "            for (int j = 1; 2 * j < n; ++j) acc = " << fma_ << "(" << at(A, 'a', "j") << ", "
              << at(A, 'a', "n - j") << ", acc);\n";
            o << "            acc = HYK_ADD(acc, acc);\n";
            o << "            if ((n & 1) == 0) acc = " << fma_ << "(" << at(A, 'a', "n / 2") << ", "
              << at(A, 'a', "n / 2") << ", acc);\n";
            out(u, false, "acc");
            break;
        case HYK_OP_SQRT:
            o << "            hyk_real acc = " << lit(0.0) << ";\n";
            o << "            if (n == 2) {\n";
            o << "                acc = HYK_MUL(S[D.c + 1], S[D.c + 1]);\n";
            o << "            } else if (n > 2) {\n";
            o << "                acc = HYK_MUL(S[D.c + 1], S[D.c + n - 1]);\n";
            o << "#pragma unroll " << ju << "\n";
            o << "                for (int j = 2; 2 * j < n; ++j) acc = " << fma_ << "(S[D.c + j], S[D.c + n - j], acc);\n";
            o << "                acc = HYK_ADD(acc, acc);\n";
            o << "                if ((n & 1) == 0) acc = " << fma_ << "(S[D.c + n / 2], S[D.c + n / 2], acc);\n";
            o << "            }\n";
            out(u, false, "(n == 1 ? HYK_MUL(" + cur(A, 'a', false) + ", S[D.inv]) : HYK_MUL(HYK_SUB(" +
                              cur(A, 'a', false) + ", acc), S[D.inv]))");
            break;
        case HYK_OP_POW: {
            size_t ai = 0;
            for (; ai < alphas.size(); ++ai)
                if (std::memcmp(&alphas[ai], &op.b.num, sizeof(double)) == 0) break;
            const std::string pc = "hyk_pc" + std::to_string(ai) + "[n * (HYK_ORDER + 1)";
            o << "            hyk_real acc = HYK_MUL(HYK_MUL(" << pc << "], " << at(A, 'a', "n") << "), S[D.c]);\n";
            o << "#pragma unroll " << ju << "\n";
            o << "            for (int j = 1; j < n; ++j) acc = " << fma_ << "(HYK_MUL(" << pc << " + j], "
              << at(A, 'a', "n - j") << "), S[D.c + j], acc);\n";
            out(u, false, "HYK_MUL(HYK_MUL(acc, hyk_invn[n]), S[D.inv])");
            break;
        }
        case HYK_OP_EXP:
            if (isT(A)) {  // d(t)/dt = 1: the single term j = 1
                o << "            const hyk_real acc = " << lit(1.0) << " * S[D.c + n - 1];\n";
                out(u, false, "HYK_MUL(acc, hyk_invn[n])");
                break;
            }
            o << "            hyk_real acc = HYK_MUL(" << wrap(A, "S[D.ka]") << ", S[D.c + n - 1]);\n";
            o << "#pragma unroll " << ju << "\n";
            o << "            for (int j = 2; j <= n; ++j) acc = " << fma_ << "(" << wrap(A, "S[D.ka + j - 1]")
              << ", S[D.c + n - j], acc);\n";
            out(u, false, "HYK_MUL(acc, hyk_invn[n])");
            break;
        case HYK_OP_LOG:
            o << "            hyk_real acc = " << lit(0.0) << ";\n";
            o << "            if (n >= 2) {\n";
            o << "                acc = HYK_MUL(S[D.kc], " << at(A, 'a', "n - 1") << ");\n";
            o << "#pragma unroll " << ju << "\n";
            o << "                for (int j = 2; j < n; ++j) acc = " << fma_ << "(S[D.kc + j - 1], " << at(A, 'a', "n - j")
              << ", acc);\n";
            o << "            }\n";
            out(u, false, "(n == 1 ? HYK_MUL(" + cur(A, 'a', false) + ", S[D.inv]) : HYK_MUL(HYK_SUB(" +
                              cur(A, 'a', false) + ", HYK_MUL(acc, hyk_invn[n])), S[D.inv]))");
            break;
        case HYK_OP_SIN:
        case HYK_OP_COS:
            if (isT(A)) {
                o << "            const hyk_real acc = " << lit(1.0) << " * S[D.prt + n - 1];\n";
            } else {
                o << "            hyk_real acc = HYK_MUL(" << wrap(A, "S[D.ka]") << ", S[D.prt + n - 1]);\n";
                o << "#pragma unroll " << ju << "\n";
                o << "            for (int j = 2; j <= n; ++j) acc = " << fma_ << "(" << wrap(A, "S[D.ka + j - 1]")
                  << ", S[D.prt + n - j], acc);\n";
            }
            out(u, false, op.op == HYK_OP_SIN ? "HYK_MUL(acc, hyk_invn[n])" : "(-HYK_MUL(acc, hyk_invn[n]))");
            break;
        }
        o << "        }\n";
    }

    void emit_group_upd(const Group &gr, bool n0) {
        const uint32_t i = gr.members[0];
        const Ref R = g.res(d.rhs[i]);
        o << "        // " << gr.key << "\n";
        o << "#pragma unroll 1\n";
        o << "        for (int q = r; q < " << gr.members.size() << "; q += HYK_TEAM) {\n";
        o << "            const hyk_tdesc &D = hyk_td[" << gr.off << " + q];\n";
        std::string f;
        if (n0) {
            f = cur(R, 'a', true);
        } else if (isU(R)) {
            f = cur(R, 'a', false);
        } else if (isT(R)) {
            f = "(n == 1 ? " + lit(1.0) + " : " + lit(0.0) + ")";
        }
        const std::string nn = n0 ? "1" : "n + 1";
        std::string v;
        if (f.empty())
            v = lit(0.0);
        else if (isT(R) && !n0)
            v = "(n == 1 ? (" + lit(1.0) + " * hyk_invn[2]) : " + lit(0.0) + ")";
        else
            v = "HYK_MUL(" + f + ", hyk_invn[" + nn + "])";
        o << "            const hyk_real v = " << v << ";\n";
        if (cold) {
            o << "            S[D.c + " << (n0 ? "1" : "((n + 1) & 1)") << "] = v;\n";
            o << "            HYK_CROW(D.b, " << nn << ") = v;\n";
        } else {
            o << "            S[D.c + " << nn << "] = v;\n";
        }
        if (g.needka[i]) {
            if (n0)
                o << "            if (1 < HYK_ORDER) S[D.kc] = " << lit(1.0) << " * v;\n";
            else
                o << "            if (n + 1 < HYK_ORDER) S[D.kc + n] = HYK_MUL((hyk_real)(n + 1), v);\n";
        }
        o << "        }\n";
    }

    void emit_order(bool n0) {
        for (auto &lv : levels) {
            for (auto &gr : lv) emit_group_op(gr, n0);
            o << "        __syncwarp();\n";
        }
        for (auto &gr : supd) emit_group_upd(gr, n0);
        o << "        __syncwarp();\n";
    }

    void emit() {
        // (a fused sum keeps its leaves' slots in b, inv, prt, x3)
        o << "struct hyk_tdesc {\n    int a, b, c, ka, kc, inv, prt, x3;\n    hyk_real num;\n};\n";
        o << "static __device__ const hyk_tdesc hyk_td[" << std::max<size_t>(descs.size(), 1) << "] = {\n";
        for (const auto &D : descs)
            o << "    {" << D.a << ", " << D.b << ", " << D.c << ", " << D.ka << ", " << D.kc << ", " << D.inv << ", "
              << D.prt << ", " << D.x3 << ", " << lit(D.num) << "},\n";
        if (descs.empty()) o << "    {0, 0, 0, 0, 0, 0, 0, 0, " << lit(0.0) << "},\n";
        o << "};\n";
        o << "static __device__ const hyk_real hyk_tsc[" << std::max<size_t>(scales.size(), 1) << "] = {";
        for (size_t i = 0; i < scales.size(); ++i) o << (i ? ", " : "") << lit(scales[i]);
        if (scales.empty()) o << lit(0.0);
        o << "};\n";
        o << "static __constant__ hyk_real hyk_invn[" << (p + 2) << "] = {" << lit(0.0);
        for (uint32_t k = 1; k <= p + 1; ++k) o << ", " << lit(recip((double)k));
        o << "};\n";
        for (size_t ai = 0; ai < alphas.size(); ++ai) {
            const double alpha = alphas[ai];
            o << "static __device__ const hyk_real hyk_pc" << ai << "[" << (p + 1) * (p + 1) << "] = {\n";
            for (uint32_t n = 0; n <= p; ++n) {
                o << "   ";
                for (uint32_t j = 0; j <= p; ++j) {
                    const double coef = (j < n) ? powcoef(n, j, alpha) : 0.0;
                    o << " " << lit(coef) << ",";
                }
                o << "\n";
            }
            o << "};\n";
        }
        // (C: the team's cold rows, HYK_CROW(i, n) = C[n * HYK_NEQ + i]; unused without them)
        o << "#define HYK_CROW(i, n) C[(n) * HYK_NEQ + (i)]\n";
        o << "static __device__ __noinline__ void hyk_tjets(hyk_real *__restrict__ S, hyk_real *__restrict__ C, "
             "const hyk_real t0, const int r) {\n";
        o << "    HYK_FMAOPS_CONSTS\n";
        o << "    __syncwarp();\n";
        if (cold) {
            o << "    for (int i = r; i < HYK_NEQ; i += HYK_TEAM) S[i * HYK_XS] = HYK_CROW(i, 0);\n";
            o << "    __syncwarp();\n";
        }
        o << "    {\n        // ---- order 0\n";
        emit_order(true);
        o << "    }\n";
        o << "#pragma unroll 1\n";
        o << "    for (int n = 1; n < HYK_ORDER; ++n) {\n";
        emit_order(false);
        o << "    }\n";
        o << "}\n";
    }
};

const char *kCommon =
#include "kernel_common.inc"
    ;

const char *kTemplate =
#include "kernel_template.inc"
    ;

const char *kTeam =
#include "kernel_team.inc"
    ;

// hyk_dmath.h and hyk_events.h as strings (generated at build time from the headers).
const char *kDmath =
#include "hyk_dmath.inc"
    ;

const char *kEvents =
#include "hyk_events.inc"
    ;

}  // namespace

uint32_t count_slots(const Dec &d, uint32_t order, bool adjoint, bool pin, bool cold_rows, uint32_t *n_cold,
                     bool split) {
    Gen g(d, order, pin, adjoint, cold_rows, split);
    if (n_cold) *n_cold = g.ncold;
    return g.nslot;
}

struct PrecisionScope {
    explicit PrecisionScope(bool f32) { g_f32 = f32; }
    ~PrecisionScope() { g_f32 = false; }
};

bool generate(const Dec &d, uint32_t order, bool pin_arith, uint32_t blk, size_t kparams_size, GenOut &out,
              std::string &err, bool adjoint, uint64_t gmem_stride, bool high_acc, bool f32, uint64_t cold_stride,
              bool split) {
    if (order < 2) {
        err = "the Taylor order must be at least 2";
        return false;
    }
    if (f32 && (pin_arith || adjoint)) {
        err = "single precision supports neither pin arithmetic nor the adjoint";
        return false;
    }
    PrecisionScope prec(f32);
    Gen g(d, order, pin_arith, adjoint, cold_stride != 0 && gmem_stride == 0, split);
    const double p = (double)order;
    const double rhofac = rhofac_of(order);
    std::ostringstream h;
    h << "// Generated by libhyk: " << d.n_eq << " equations, " << d.n_ops << " u-operations, order " << order
      << (pin_arith ? ", pin arithmetic" : "") << "\n";
    h << "#define HYK_NEQ " << d.n_eq << "\n#define HYK_NPARS " << d.n_pars << "\n#define HYK_ORDER " << order
      << "\n#define HYK_BLK " << blk << "\n#define HYK_TPB " << blk << "\n#define HYK_GMEM " << (gmem_stride ? 1 : 0)
      << "\n#define HYK_STRIDE " << (gmem_stride ? std::to_string(gmem_stride) + "ULL" : std::to_string(blk))
      << "\n#define HYK_NSLOT " << g.nslot << "\n#define HYK_PAR_SLOT " << g.par_slot
      << "\n#define HYK_RHOFAC " << lit(rhofac) << "\n#define HYK_INV_P " << lit(recip(p)) << "\n#define HYK_INV_PM1 "
      << lit(recip(p - 1.0)) << "\n";
    h << precision_header(pin_arith);
    if (pin_arith) {
        h << "#define HYK_FMA_ACC(a, b, c) ((a) * (b) + (c))\n";
        h << "#define HYK_RHO(mp, mq, num) (1.0 / pow((mq) / (num), HYK_INV_PM1) < 1.0 / pow((mp) / (num), HYK_INV_P) "
             "? 1.0 / pow((mq) / (num), HYK_INV_PM1) : 1.0 / pow((mp) / (num), HYK_INV_P))\n";
    } else {
        h << "#define HYK_FMA_ACC(a, b, c) HYK_FMA((a), (b), (c))\n";
        h << "#define HYK_RHO(mp, mq, num) HYK_DM_RHO((mp), (mq), (num), HYK_INV_P, HYK_INV_PM1)\n";
    }
    if (adjoint) h << "#define HYK_ADJOINT 1\n";
    h << "#define HYK_HIGH_ACC " << (high_acc ? 1 : 0) << "\n";
    if (g.coldrows) h << "#define HYK_CSTRIDE " << cold_stride << "ULL\n";
    h << kDmath << "\n";
    h << kCommon << "\n";
    g.emit_sx_access(h);
    g.emit_events(h);
    if (!d.ev.empty()) h << kEvents << "\n";
    h << kTemplate << "\n";
    h << "static_assert(sizeof(hyk_kparams) == " << kparams_size << ", \"hyk_kparams layout mismatch\");\n";
    g.emit_jets();
    if (adjoint) g.emit_bw();
    // The template's kernels call hyk_jets(); declare-before-use ordering is
    // satisfied by emitting the jets function first.
    std::string body = g.o.str();
    std::string full = h.str();
    // Insert the jets definition before the first kernel of the template.
    const std::string marker = "// One Taylor step per lane";
    const size_t pos = full.find(marker);
    if (pos == std::string::npos) {
        err = "internal: template marker not found";
        return false;
    }
    full.insert(pos, body + "\n");
    out.src = std::move(full);
    out.n_slot = g.nslot;
    out.n_cold = g.coldrows ? g.ncold : 0;
    out.par_slot = g.par_slot;
    // Per-step flops: recurrences + Horner (2 per coefficient) + step size
    // (two pow and the norm arithmetic) + double-length time update.
    out.flops = g.flops + 2.0 * d.n_eq * order + 46.0 + 10.0;
    return true;
}


bool team_layout(const Dec &d, uint32_t order, TeamInfo &info, std::string &err) {
    TeamGen tg(d, order);
    if (!tg.analyse()) {
        err = tg.err;
        return false;
    }
    info.n_slot = tg.nslot | 1u;
    for (uint32_t T = 1; T <= 32; T *= 2) info.util[__builtin_ctz(T)] = tg.util(T);
    TeamGen tc(d, order, true);
    info.n_slot_cold = (tc.cold && tc.analyse()) ? (tc.nslot | 1u) : 0;
    return true;
}

bool generate_team(const Dec &d, uint32_t order, uint32_t team, uint32_t tpb, size_t kparams_size, GenOut &out,
                   std::string &err, bool high_acc, bool f32, bool gmem, bool cold) {
    if (order < 2) {
        err = "the Taylor order must be at least 2";
        return false;
    }
    if (team < 2 || team > 32 || (team & (team - 1)) || tpb % 32 || tpb == 0) {
        err = "invalid team geometry";
        return false;
    }
    PrecisionScope prec(f32);
    TeamGen tg(d, order, cold && !gmem);
    if (!tg.analyse()) {
        err = tg.err;
        return false;
    }
    tg.g.emit_jets();  // flop count of the same recurrences
    const double p = (double)order;
    const double rhofac = rhofac_of(order);
    const uint32_t nt = tg.nslot | 1u;
    std::ostringstream h;
    h << "// Generated by libhyk (team form, " << team << " threads per trajectory): " << d.n_eq << " equations, "
      << d.n_ops << " u-operations, order " << order << "\n";
    h << "#define HYK_NEQ " << d.n_eq << "\n#define HYK_NPARS " << d.n_pars << "\n#define HYK_ORDER " << order
      << "\n#define HYK_TPB " << tpb << "\n#define HYK_TEAM " << team << "\n#define HYK_GMEM " << (gmem ? 1 : 0)
      << "\n#define HYK_COLD " << (tg.cold ? 1 : 0) << "\n#define HYK_XS " << tg.XS
      << "\n#define HYK_NT " << nt << "\n#define HYK_NSLOT " << tg.nslot << "\n#define HYK_PAR_SLOT " << tg.par_slot
      << "\n#define HYK_RHOFAC " << lit(rhofac) << "\n#define HYK_INV_P " << lit(recip(p)) << "\n#define HYK_INV_PM1 "
      << lit(recip(p - 1.0)) << "\n";
    h << precision_header(false);
    h << "#define HYK_FMA_ACC(a, b, c) HYK_FMA((a), (b), (c))\n";
    h << "#define HYK_RHO(mp, mq, num) HYK_DM_RHO((mp), (mq), (num), HYK_INV_P, HYK_INV_PM1)\n";
    h << "#define HYK_NEV 0\n#define HYK_NTEV 0\n#define HYK_HIGH_ACC " << (high_acc ? 1 : 0) << "\n";
    h << kDmath << "\n";
    h << kCommon << "\n";
    h << "static_assert(sizeof(hyk_kparams) == " << kparams_size << ", \"hyk_kparams layout mismatch\");\n";
    if (tg.cold) h << "extern \"C\" { __constant__ hyk_real *hyk_cold_base; }\n";
    tg.emit();
    h << tg.o.str() << "\n";
    h << kTeam << "\n";
    out.src = h.str();
    out.n_slot = nt;
    out.n_cold = tg.cold ? d.n_eq : 0;
    out.par_slot = tg.par_slot;
    out.flops = tg.g.flops + 2.0 * d.n_eq * order + 46.0 + 10.0;
    return true;
}

// Host translation unit of the same generated recurrences (forward jets and,
// with the adjoint, the reverse sweep) for CPU checks of the generator: one
// lane, HYK_BLK = 1, the CUDA intrinsics mapped to their host equivalents.
bool generate_host(const Dec &d, uint32_t order, bool adjoint, std::string &src, std::string &err, bool team, bool f32,
                   bool cold) {
    PrecisionScope ps(f32);
    if (order < 2) {
        err = "the Taylor order must be at least 2";
        return false;
    }
    if (team) {
        // The team form's recurrences run by a team of one thread (with cold
        // state rows: in the array C of the translation unit).
        TeamGen tg(d, order, cold);
        if (!tg.analyse()) {
            err = tg.err;
            return false;
        }
        std::ostringstream h;
        h << "#include <cmath>\n#include <cstdint>\n#define __device__\n#define __constant__\n#define __noinline__\n"
             "#define __forceinline__ inline\n#define __restrict__\n"
             "static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }\n"
             "static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }\n"
             "static inline void __syncwarp() {}\n#define HYK_WARP_SYNC()\n";
        h << kDmath << "\n";
        h << (f32 ? "typedef float hyk_real;\n" : "typedef double hyk_real;\n") << precision_header(false);
        h << "#define HYK_NEQ " << d.n_eq << "\n#define HYK_NPARS " << d.n_pars << "\n#define HYK_ORDER " << order
          << "\n#define HYK_TEAM 1\n#define HYK_XS " << tg.XS << "\n#define HYK_NSLOT " << tg.nslot
          << "\n#define HYK_PAR_SLOT " << tg.par_slot << "\n";
        h << "static hyk_real C[HYK_NEQ * (HYK_ORDER + 1)];\n";
        if (tg.cold)
            h << "#define HYK_SX(i, n) C[(n) * HYK_NEQ + (i)]\n";
        else
            h << "#define HYK_SX(i, n) S[(i) * HYK_XS + (n)]\n";
        h << "#define HYK_PAR(k) S[HYK_PAR_SLOT + (k)]\n";
        tg.emit();
        h << tg.o.str();
        h << "extern \"C\" int hyk_host_nslot(void) { return HYK_NSLOT; }\n";
        h << "extern \"C\" void hyk_host_step(hyk_real *S, const hyk_real *x0, const hyk_real *pars, hyk_real t0, hyk_real h, hyk_real *x1) {\n"
             "    for (int i = 0; i < HYK_NEQ; ++i) HYK_SX(i, 0) = x0[i];\n"
             "    for (int k = 0; k < HYK_NPARS; ++k) HYK_PAR(k) = pars[k];\n"
             "    hyk_tjets(S, C, t0, 0);\n"
             "    for (int i = 0; i < HYK_NEQ; ++i) {\n"
             "        hyk_real acc = HYK_SX(i, HYK_ORDER);\n"
             "        for (int n = HYK_ORDER - 1; n >= 0; --n) acc = HYK_FMA(acc, h, HYK_SX(i, n));\n"
             "        x1[i] = acc;\n    }\n}\n";
        h << "extern \"C\" void hyk_host_tc(hyk_real *S, const hyk_real *x0, const hyk_real *pars, hyk_real t0, hyk_real *tc) {\n"
             "    for (int i = 0; i < HYK_NEQ; ++i) HYK_SX(i, 0) = x0[i];\n"
             "    for (int k = 0; k < HYK_NPARS; ++k) HYK_PAR(k) = pars[k];\n"
             "    hyk_tjets(S, C, t0, 0);\n"
             "    for (int i = 0; i < HYK_NEQ; ++i)\n"
             "        for (int n = 0; n <= HYK_ORDER; ++n) tc[i * (HYK_ORDER + 1) + n] = HYK_SX(i, n);\n}\n";
        src = h.str();
        return true;
    }
    Gen g(d, order, false, adjoint);
    const double p = (double)order;
    std::ostringstream h;
    h << "#include <cmath>\n#include <cstdint>\n#define __device__\n#define __noinline__\n"
         "#define __forceinline__ inline\n#define __restrict__\n"
         "static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }\n"
             "static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }\n"
         "static inline void __syncwarp() {}\n#define HYK_WARP_SYNC()\n";
    h << kDmath << "\n";
    h << (f32 ? "typedef float hyk_real;\n" : "typedef double hyk_real;\n") << precision_header(false);
    h << "#define HYK_NEQ " << d.n_eq << "\n#define HYK_NPARS " << d.n_pars << "\n#define HYK_ORDER " << order
      << "\n#define HYK_BLK 1\n#define HYK_STRIDE 1\n#define HYK_NSLOT " << g.nslot << "\n#define HYK_PAR_SLOT " << g.par_slot
      << "\n#define HYK_RHOFAC " << lit(rhofac_of(order)) << "\n#define HYK_INV_P " << lit(recip(p)) << "\n#define HYK_INV_PM1 "
      << lit(recip(p - 1.0)) << "\n";
    h << "#define HYK_SX(i, n) S[((i) * (HYK_ORDER + 1) + (n)) * HYK_STRIDE]\n#define HYK_PAR(k) S[(HYK_PAR_SLOT + (k)) * HYK_STRIDE]\n";
    h << "static inline hyk_real hyk_inf() { return (hyk_real)HUGE_VAL; }\n";
    g.emit_jets();
    if (adjoint) g.emit_bw();
    h << g.o.str();
    h << "extern \"C\" int hyk_host_nslot(void) { return HYK_NSLOT; }\n";
    h << "extern \"C\" void hyk_host_step(hyk_real *S, const hyk_real *x0, const hyk_real *pars, hyk_real t0, hyk_real h, hyk_real *x1) {\n"
         "    for (int i = 0; i < HYK_NEQ; ++i) HYK_SX(i, 0) = x0[i];\n"
         "    for (int k = 0; k < HYK_NPARS; ++k) HYK_PAR(k) = pars[k];\n"
         "    hyk_jets(S, t0);\n"
         "    for (int i = 0; i < HYK_NEQ; ++i) {\n"
         "        hyk_real acc = HYK_SX(i, HYK_ORDER);\n"
         "        for (int n = HYK_ORDER - 1; n >= 0; --n) acc = HYK_FMA(acc, h, HYK_SX(i, n));\n"
         "        x1[i] = acc;\n    }\n}\n";
    h << "extern \"C\" void hyk_host_tc(hyk_real *S, const hyk_real *x0, const hyk_real *pars, hyk_real t0, hyk_real *tc) {\n"
         "    for (int i = 0; i < HYK_NEQ; ++i) HYK_SX(i, 0) = x0[i];\n"
         "    for (int k = 0; k < HYK_NPARS; ++k) HYK_PAR(k) = pars[k];\n"
         "    hyk_jets(S, t0);\n"
         "    for (int i = 0; i < HYK_NEQ; ++i)\n"
         "        for (int n = 0; n <= HYK_ORDER; ++n) tc[i * (HYK_ORDER + 1) + n] = HYK_SX(i, n);\n}\n";
    if (adjoint)
        h << "extern \"C\" void hyk_host_adjoint(double *S, const double *x0, const double *pars, double t0, double h, "
             "double *lam, double *pb) {\n"
             "    for (int i = 0; i < HYK_NEQ; ++i) HYK_SX(i, 0) = x0[i];\n"
             "    for (int k = 0; k < HYK_NPARS; ++k) HYK_PAR(k) = pars[k];\n"
             "    hyk_jets(S, t0);\n    hyk_jets_bw(S, t0, h, lam, pb);\n}\n";
    src = h.str();
    return true;
}

// Recurrences of one system in the reference's arithmetic (no fused
// multiply-adds, true divisions, the C library's elementary functions) over
// an element type chosen by the including translation unit: `hyk_real` may
// be a vector of lanes (GCC vector extension), in which case every operation
// acts on a batch of trajectories at once and the includer provides the
// element-wise pow/exp/log/sqrt/sincos for that type.  This is the per-system
// part of the compiled CPU stepper that stands in for the reference's
// LLVM-compiled batch stepper in timing comparisons; nothing on the GPU path
// uses it.
bool generate_host_batch(const Dec &d, uint32_t order, std::string &src, std::string &err) {
    PrecisionScope ps(false);
    if (order < 2) {
        err = "the Taylor order must be at least 2";
        return false;
    }
    if (!d.ev.empty()) {
        err = "the compiled CPU stepper does not support events";
        return false;
    }
    Gen g(d, order, true, false);
    std::ostringstream h;
    h << "#define HYK_NEQ " << d.n_eq << "\n#define HYK_NPARS " << d.n_pars << "\n#define HYK_ORDER " << order
      << "\n#define HYK_STRIDE 1\n#define HYK_NSLOT " << g.nslot << "\n#define HYK_PAR_SLOT " << g.par_slot << "\n";
    h << "#define HYK_SX(i, n) S[((i) * (HYK_ORDER + 1) + (n)) * HYK_STRIDE]\n#define HYK_PAR(k) S[(HYK_PAR_SLOT + (k)) * HYK_STRIDE]\n";
    g.emit_jets();
    h << g.o.str();
    h << "#define HYK_FLOPS_PER_STEP " << lit(g.flops) << "\n";
    src = h.str();
    return true;
}

}  // namespace hyk
