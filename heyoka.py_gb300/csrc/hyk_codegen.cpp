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
#include <cstdio>
#include <cstring>
#include <limits>
#include <sstream>

#include "hyk_internal.hpp"

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
    return true;
}

namespace {

std::string lit(double v) {
    if (std::isnan(v)) return "__longlong_as_double(0x7ff8000000000000LL)";
    if (std::isinf(v)) return v > 0 ? "hyk_inf()" : "(-hyk_inf())";
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.17g", v);
    std::string s(buf);
    if (s.find_first_of(".eE") == std::string::npos) s += ".0";
    if (v < 0 || (v == 0 && std::signbit(v))) s = "(" + s + ")";
    return s;
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

    Gen(const Dec &dd, uint32_t order, bool pin_arith, bool adjoint = false)
        : d(dd), p(order), N(dd.n_eq), NU(dd.n_u()), pin(pin_arith), adj(adjoint),
          split((uint64_t)dd.n_ops * order > 3000) {
        base.resize(NU);
        negf.assign(NU, 0);
        alias.assign(NU, 0);
        for (uint32_t u = 0; u < NU; ++u) base[u] = (int)u;
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const auto &op = d.ops[k];
            const uint32_t u = N + k;
            if (op.op == HYK_OP_NEG && op.a.kind == HYK_ARG_U) {
                alias[u] = 1;
                base[u] = base[op.a.idx];
                negf[u] = !negf[op.a.idx];
            }
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
    static bool varying(const Ref &r) { return r.kind == HYK_ARG_U || r.kind == HYK_ARG_TIME; }

    void analyse() {
        hist.assign(NU, 0);
        needka.assign(NU, 0);
        for (uint32_t i = 0; i < N; ++i) hist[i] = 1;
        for (uint32_t k = 0; k < d.n_ops; ++k) {
            const uint32_t u = N + k;
            if (alias[u]) continue;
            const auto &op = d.ops[k];
            const Ref A = res(op.a), B = res(op.b);
            auto H = [&](const Ref &r) {
                if (r.kind == HYK_ARG_U) hist[r.u] = 1;
            };
            auto K = [&](const Ref &r) {
                if (r.kind == HYK_ARG_U) needka[r.u] = 1;
            };
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
        uint32_t s = 0;
        for (uint32_t i = 0; i < N; ++i) {
            slot[i] = (int)s;
            s += p + 1;
        }
        // The adjoint module keeps every history up to order p-1.
        const uint32_t hl = adj ? p : (p >= 2 ? p - 1 : 1), kl = adj ? p - 1 : (p >= 3 ? p - 2 : 0);
        for (uint32_t u = N; u < NU; ++u)
            if (hist[u] && !alias[u]) {
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
        if (adj) {
            // Adjoint accumulators: orders 0..p of every history, of every j*a_j.
            abase = s;
            aslot.assign(NU, -1);
            akslot.assign(NU, -1);
            for (uint32_t u = 0; u < NU; ++u)
                if (hist[u] && !alias[u]) {
                    aslot[u] = (int)s;
                    s += p + 1;
                }
            for (uint32_t u = 0; u < NU; ++u)
                if (needka[u] && !alias[u]) {
                    akslot[u] = (int)s;
                    s += p + 1;
                }
        }
        nslot = s;
    }

    std::string vname(uint32_t u, uint32_t n) const { return "v" + std::to_string(u) + "_" + std::to_string(n); }
    std::string kname(uint32_t u, uint32_t n) const { return "k" + std::to_string(u) + "_" + std::to_string(n); }
    std::string smem(uint32_t s) const { return "S[" + std::to_string(s) + " * HYK_STRIDE]"; }

    // Coefficient of order j of u-variable u (not an alias) while emitting block n.
    std::string ucoef(uint32_t u, uint32_t j, uint32_t n) const {
        if (j == n) return vname(u, j);
        if (!hist[u] || slot[u] < 0) {
            std::fprintf(stderr, "hyk codegen: missing history for u%u\n", u);
            std::abort();
        }
        return smem((uint32_t)slot[u] + j);
    }
    // Coefficient expression, or "" when identically zero.
    std::string cf(const Ref &r, uint32_t j, uint32_t n) const {
        switch (r.kind) {
        case HYK_ARG_U: {
            const std::string s = ucoef((uint32_t)r.u, j, n);
            return r.neg ? "(-" + s + ")" : s;
        }
        case HYK_ARG_NUM:
            return j == 0 ? lit(r.num) : "";
        case HYK_ARG_PAR:
            return j == 0 ? "HYK_PAR(" + std::to_string(r.par) + ")" : "";
        case HYK_ARG_TIME:
            return j == 0 ? "t0" : (j == 1 ? "1.0" : "");
        }
        return "";
    }
    // j * a_j (j >= 1), or "" when identically zero.
    std::string kcf(const Ref &r, uint32_t j, uint32_t n) const {
        switch (r.kind) {
        case HYK_ARG_U: {
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
            return j == 1 ? "1.0" : "";
        default:
            return "";
        }
    }

    // Whether the order-j coefficient (or j * a_j) of an argument can be
    // non-zero; checked before building an expression, so that no history is
    // requested for a term that vanishes.
    static bool nz(const Ref &r, uint32_t j) {
        switch (r.kind) {
        case HYK_ARG_U:
            return true;
        case HYK_ARG_TIME:
            return j <= 1;
        case HYK_ARG_NUM:
        case HYK_ARG_PAR:
            return j == 0;
        }
        return false;
    }
    static bool knz(const Ref &r, uint32_t j) {
        return (r.kind == HYK_ARG_U && j >= 1) || (r.kind == HYK_ARG_TIME && j == 1);
    }

    std::string fma(const std::string &x, const std::string &y, const std::string &c) const {
        if (pin) return "(" + c + " + " + x + " * " + y + ")";
        return "__fma_rn(" + x + ", " + y + ", " + c + ")";
    }

    struct Acc {
        std::string name;
        bool first = true;
    };
    void term(Acc &a, const std::string &x, const std::string &y) {
        if (x.empty() || y.empty()) return;
        if (a.first) {
            o << "    double " << a.name << " = " << x << " * " << y << ";\n";
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
        return "(" + x + " * " + lit(1.0 / (double)n) + ")";
    }
    std::string inv0(uint32_t u) const { return "i" + std::to_string(u); }
    // After defining 1/b_0 at order 0: keep it for the later order functions.
    void keep_inv0(uint32_t u) {
        if (split && !pin && islot[u] >= 0) o << "    " << smem((uint32_t)islot[u]) << " = " << inv0(u) << ";\n";
    }

    void def(uint32_t u, uint32_t n, const std::string &expr) { o << "    const double " << vname(u, n) << " = " << expr << ";\n"; }

    void store_hist(uint32_t u, uint32_t n) {
        const uint32_t lim = adj ? p : p - 1;  // stored orders: 0..lim-1
        if (u >= N && hist[u] && n + 1 <= lim) o << "    " << smem((uint32_t)slot[u] + n) << " = " << vname(u, n) << ";\n";
        if (needka[u] && n >= 1) {
            o << "    const double " << kname(u, n) << " = " << lit((double)n) << " * " << vname(u, n) << ";\n";
            flops += 1;
            if (kslot[u] >= 0 && n + 1 <= lim) o << "    " << smem((uint32_t)kslot[u] + n - 1) << " = " << kname(u, n) << ";\n";
        }
    }

    void emit_op(uint32_t k, uint32_t n) {
        const auto &op = d.ops[k];
        const uint32_t u = N + k;
        if (alias[u]) return;
        const Ref A = res(op.a), B = res(op.b);
        const std::string acc = "a" + std::to_string(u) + "_" + std::to_string(n);
        const std::string z = "0.0";
        switch (op.op) {
        case HYK_OP_ADD:
        case HYK_OP_SUB: {
            const std::string a = cf(A, n, n), b = cf(B, n, n);
            const bool add = op.op == HYK_OP_ADD;
            if (!a.empty() && !b.empty()) {
                def(u, n, "(" + a + (add ? " + " : " - ") + b + ")");
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
                if (!pin) o << "    const double " << inv0(u) << " = 1.0 / " << b0 << ";\n";
                flops += 2;
                keep_inv0(u);
                break;
            }
            Acc s{acc};
            for (uint32_t j = 1; j <= n; ++j)
                if (nz(B, j)) term(s, cf(B, j, n), ucoef(u, n - j, n));
            const std::string av = an.empty() ? z : an;
            const std::string num = s.first ? av : "(" + av + " - " + acc + ")";
            if (!s.first) flops += 1;
            flops += 1;
            def(u, n, pin ? "(" + num + " / " + b0 + ")" : "(" + num + " * " + inv0(u) + ")");
            break;
        }
        case HYK_OP_SQUARE: {
            Acc s{acc};
            for (uint32_t j = 0; 2 * j < n; ++j)
                if (nz(A, j) && nz(A, n - j)) term(s, cf(A, j, n), cf(A, n - j, n));
            if (!s.first) {
                o << "    " << acc << " = " << acc << " + " << acc << ";\n";
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
                if (!pin) o << "    const double " << inv0(u) << " = 1.0 / (2.0 * " << vname(u, 0) << ");\n";
                flops += 3;
                keep_inv0(u);
                break;
            }
            Acc s{acc};
            for (uint32_t j = 1; 2 * j < n; ++j) term(s, ucoef(u, j, n), ucoef(u, n - j, n));
            if (!s.first) {
                o << "    " << acc << " = " << acc << " + " << acc << ";\n";
                flops += 1;
            }
            if (n % 2 == 0) term(s, ucoef(u, n / 2, n), ucoef(u, n / 2, n));
            const std::string av = an.empty() ? z : an;
            const std::string num = s.first ? av : "(" + av + " - " + acc + ")";
            flops += s.first ? 1 : 2;
            def(u, n, pin ? "(" + num + " / (2.0 * " + ucoef(u, 0, n) + "))" : "(" + num + " * " + inv0(u) + ")");
            break;
        }
        case HYK_OP_POW: {
            const double alpha = op.b.num;
            const std::string a0 = cf(A, 0, n);
            if (n == 0) {
                def(u, 0, (pin ? "pow(" : "hyk_dm_pow(") + a0 + ", " + lit(alpha) + ")");
                if (!pin) o << "    const double " << inv0(u) << " = 1.0 / " << a0 << ";\n";
                flops += 21;
                keep_inv0(u);
                break;
            }
            Acc s{acc};
            for (uint32_t j = 0; j < n; ++j) {
                const std::string anj = cf(A, n - j, n);
                if (anj.empty()) continue;
                const double coef = (double)n * alpha - (double)j * (alpha + 1.0);
                const std::string t = "t" + std::to_string(u) + "_" + std::to_string(n) + "_" + std::to_string(j);
                o << "    const double " << t << " = " << lit(coef) << " * " << anj << ";\n";
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
                def(u, n, "((" + acc + " * " + lit(1.0 / (double)n) + ") * " + inv0(u) + ")");
            break;
        }
        case HYK_OP_EXP: {
            if (n == 0) {
                def(u, 0, (pin ? "exp(" : "hyk_dm_exp(") + cf(A, 0, n) + ")");
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
                def(u, 0, (pin ? "log(" : "hyk_dm_log(") + a0 + ")");
                if (!pin) o << "    const double " << inv0(u) << " = 1.0 / " << a0 << ";\n";
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
                num = "(" + av + " - " + divn(acc, n) + ")";
                flops += 1;
            }
            flops += 1;
            def(u, n, pin ? "(" + num + " / " + a0 + ")" : "(" + num + " * " + inv0(u) + ")");
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
                    o << "    double " << vname(su, 0) << "_m, " << vname(cu, 0) << "_m;\n";
                    o << "    " << (pin ? "sincos(" : "hyk_dm_sincos(") << cf(A, 0, n) << ", &" << vname(su, 0) << "_m, &"
                      << vname(cu, 0) << "_m);\n";
                    o << "    const double " << vname(su, 0) << " = " << vname(su, 0) << "_m;\n";
                    o << "    const double " << vname(cu, 0) << " = " << vname(cu, 0) << "_m;\n";
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

    void emit_jets() {
        if (!split) {
            o << "static __device__ __noinline__ void hyk_jets(double *__restrict__ S, const double t0) {\n";
            for (uint32_t i = 0; i < N; ++i) o << "    const double " << vname(i, 0) << " = HYK_SX(" << i << ", 0);\n";
        }
        for (uint32_t n = 0; n < p; ++n) {
            if (split) {
                o << "static __device__ __noinline__ void hyk_jets_o" << n
                  << "(double *__restrict__ S, const double t0) {\n";
                for (uint32_t i = 0; i < N; ++i) {
                    o << "    const double " << vname(i, n) << " = HYK_SX(" << i << ", " << n << ");\n";
                    // The same product the previous order formed (k_i_0 is never read).
                    if (needka[i] && n >= 1)
                        o << "    const double " << kname(i, n) << " = " << lit((double)n) << " * " << vname(i, n)
                          << ";\n";
                }
                if (!pin && n >= 1)
                    for (uint32_t u = N; u < NU; ++u)
                        if (islot[u] >= 0) o << "    const double " << inv0(u) << " = " << smem((uint32_t)islot[u]) << ";\n";
            }
            o << "    // ---- order " << n << "\n";
            for (uint32_t k = 0; k < d.n_ops; ++k) {
                emit_op(k, n);
                const uint32_t u = N + k;
                if (!alias[u]) store_hist(u, n);
            }
            for (uint32_t i = 0; i < N; ++i) {
                const Ref r = res(d.rhs[i]);
                const std::string f = cf(r, n, n);
                def(i, n + 1, f.empty() ? "0.0" : divn(f, n + 1));
                o << "    HYK_SX(" << i << ", " << (n + 1) << ") = " << vname(i, n + 1) << ";\n";
                if (needka[i]) {
                    o << "    const double " << kname(i, n + 1) << " = " << lit((double)(n + 1)) << " * "
                      << vname(i, n + 1) << ";\n";
                    flops += 1;
                    if (kslot[i] >= 0 && n + 1 + (adj ? 1u : 2u) <= p)
                        o << "    " << smem((uint32_t)kslot[i] + n) << " = " << kname(i, n + 1) << ";\n";
                }
            }
            // Values of earlier orders are re-read from shared memory: the
            // warp barrier keeps the compiler from carrying them in registers.
            o << "    __syncwarp();\n";
            if (split) o << "}\n";
        }
        if (split) {
            o << "static __device__ __noinline__ void hyk_jets(double *__restrict__ S, const double t0) {\n";
            for (uint32_t n = 0; n < p; ++n) o << "    hyk_jets_o" << n << "(S, t0);\n";
        }
        o << "}\n";
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
    std::string aref(uint32_t u, uint32_t j) const { return smem((uint32_t)aslot[u] + j); }
    std::string akref(uint32_t u, uint32_t j) const { return smem((uint32_t)akslot[u] + j); }
    std::string gname(uint32_t u, uint32_t n) const { return "g" + std::to_string(u) + "_" + std::to_string(n); }
    // adjoint(r, order j) += x * y
    void acc(const Ref &r, uint32_t j, uint32_t n, const std::string &x, const std::string &y) {
        if (r.kind == HYK_ARG_U) {
            const uint32_t u = (uint32_t)r.u;
            const std::string xx = r.neg ? "(-" + x + ")" : x;
            std::string t;
            if (hist[u])
                t = aref(u, j);
            else {
                if (j != n) {
                    std::fprintf(stderr, "hyk codegen: adjoint of a non-stored value at another order (u%u)\n", u);
                    std::abort();
                }
                t = gname(u, n);
            }
            o << "    " << t << " = __fma_rn(" << xx << ", " << y << ", " << t << ");\n";
        } else if (r.kind == HYK_ARG_PAR && j == 0) {
            o << "    pb[" << r.par << "] = __fma_rn(" << x << ", " << y << ", pb[" << r.par << "]);\n";
        }
    }
    void acck(const Ref &r, uint32_t j, const std::string &x, const std::string &y) {
        if (r.kind != HYK_ARG_U) return;
        const std::string xx = r.neg ? "(-" + x + ")" : x;
        o << "    " << akref((uint32_t)r.u, j) << " = __fma_rn(" << xx << ", " << y << ", " << akref((uint32_t)r.u, j)
          << ");\n";
    }

    void emit_op_bw(uint32_t k, uint32_t n) {
        const auto &op = d.ops[k];
        const uint32_t u = N + k;
        if (alias[u]) return;
        const Ref A = res(op.a), B = res(op.b);
        const Ref self{HYK_ARG_U, (int)u, false, 0, -1};
        // A function of a constant is constant: nothing flows back above order 0.
        const bool unary_fn = op.op == HYK_OP_SQRT || op.op == HYK_OP_POW || op.op == HYK_OP_EXP ||
                              op.op == HYK_OP_LOG || op.op == HYK_OP_SIN || op.op == HYK_OP_COS;
        if (unary_fn && n >= 1 && !varying(A)) return;
        const std::string G = "G" + std::to_string(u) + "_" + std::to_string(n);
        std::string gsrc = hist[u] ? aref(u, n) : gname(u, n);
        if (needka[u] && n >= 1) gsrc = "__fma_rn(" + lit((double)n) + ", " + akref(u, n) + ", " + gsrc + ")";
        o << "    const double " << G << " = " << gsrc << ";\n";
        const std::string W = "W" + std::to_string(u) + "_" + std::to_string(n);
        const std::string inv = "i" + std::to_string(u);
        switch (op.op) {
        case HYK_OP_ADD:
            if (nz(A, n)) acc(A, n, n, G, "1.0");
            if (nz(B, n)) acc(B, n, n, G, "1.0");
            break;
        case HYK_OP_SUB:
            if (nz(A, n)) acc(A, n, n, G, "1.0");
            if (nz(B, n)) acc(B, n, n, G, "(-1.0)");
            break;
        case HYK_OP_NEG:
            if (nz(A, n)) acc(A, n, n, G, "(-1.0)");
            break;
        case HYK_OP_MUL:
            for (uint32_t j = 0; j <= n; ++j)
                if (nz(A, j) && nz(B, n - j)) {
                    acc(A, j, n, G, val(B, n - j));
                    acc(B, n - j, n, G, val(A, j));
                }
            break;
        case HYK_OP_DIV:
            o << "    const double " << W << " = " << G << " * " << inv << ";\n";
            if (nz(A, n)) acc(A, n, n, W, "1.0");
            for (uint32_t j = 1; j <= n; ++j)
                if (nz(B, j)) {
                    acc(B, j, n, "(-" + W + ")", val(self, n - j));
                    acc(self, n - j, n, "(-" + W + ")", val(B, j));
                }
            acc(B, 0, n, "(-" + W + ")", val(self, n));
            break;
        case HYK_OP_SQUARE:
            for (uint32_t j = 0; j <= n; ++j)
                if (nz(A, j) && nz(A, n - j)) acc(A, j, n, "(2.0 * " + G + ")", val(A, n - j));
            break;
        case HYK_OP_SQRT:
            o << "    const double " << W << " = " << G << " * " << inv << ";\n";
            if (nz(A, n)) acc(A, n, n, W, "1.0");
            if (n >= 1) {
                for (uint32_t j = 1; j < n; ++j) acc(self, j, n, "(-2.0 * " + W + ")", val(self, n - j));
                acc(self, 0, n, "(-2.0 * " + W + ")", val(self, n));
            }
            break;
        case HYK_OP_POW: {
            const double alpha = op.b.num;
            if (n == 0) {
                acc(A, 0, 0, "(" + G + " * " + lit(alpha) + ")", "(" + val(self, 0) + " * " + inv + ")");
                break;
            }
            o << "    const double " << W << " = (" << G << " * " << inv << ") * " << lit(1.0 / (double)n) << ";\n";
            for (uint32_t j = 0; j < n; ++j) {
                if (!nz(A, n - j)) continue;
                const double coef = (double)n * alpha - (double)j * (alpha + 1.0);
                const std::string wc = "(" + W + " * " + lit(coef) + ")";
                acc(A, n - j, n, wc, val(self, j));
                acc(self, j, n, wc, val(A, n - j));
            }
            acc(A, 0, n, "(-" + G + " * " + inv + ")", val(self, n));
            break;
        }
        case HYK_OP_EXP:
            if (n == 0) {
                acc(A, 0, 0, G, val(self, 0));
                break;
            }
            o << "    const double " << W << " = " << G << " * " << lit(1.0 / (double)n) << ";\n";
            for (uint32_t j = 1; j <= n; ++j)
                if (knz(A, j)) {
                    acck(A, j, W, val(self, n - j));
                    acc(self, n - j, n, W, kval(A, j));
                }
            break;
        case HYK_OP_LOG:
            if (n == 0) {
                acc(A, 0, 0, G, inv);
                break;
            }
            o << "    const double " << W << " = " << G << " * " << inv << ";\n";
            if (nz(A, n)) acc(A, n, n, W, "1.0");
            if (varying(A))
                for (uint32_t j = 1; j < n; ++j) {
                    if (!nz(A, n - j)) continue;
                    const std::string t = "(-" + W + " * " + lit(1.0 / (double)n) + ")";
                    acck(self, j, t, val(A, n - j));
                    acc(A, n - j, n, t, kval(self, j));
                }
            acc(A, 0, n, "(-" + G + " * " + inv + ")", val(self, n));
            break;
        case HYK_OP_SIN:
        case HYK_OP_COS: {
            const Ref P{HYK_ARG_U, op.aux, false, 0, -1};
            const bool is_sin = op.op == HYK_OP_SIN;
            if (n == 0) {
                acc(A, 0, 0, is_sin ? G : "(-" + G + ")", val(P, 0));
                break;
            }
            o << "    const double " << W << " = " << G << " * " << lit((is_sin ? 1.0 : -1.0) / (double)n) << ";\n";
            for (uint32_t j = 1; j <= n; ++j)
                if (knz(A, j)) {
                    acck(A, j, W, val(P, n - j));
                    acc(P, n - j, n, W, kval(A, j));
                }
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
    void emit_bw() {
        for (uint32_t n = 0; n < p; ++n) {
            o << "static __device__ __noinline__ void hyk_bw_o" << n
              << "(double *__restrict__ S, const double t0, double *__restrict__ pb) {\n";
            o << "    (void)t0;\n";
            emit_inverses(true);
            for (uint32_t k = 0; k < d.n_ops; ++k) {
                const uint32_t u = N + k;
                if (!alias[u] && !hist[u]) o << "    double " << gname(u, n) << " = 0.0;\n";
            }
            for (uint32_t ii = N; ii-- > 0;) {
                const uint32_t i = ii;
                if (needka[i])
                    o << "    " << aref(i, n + 1) << " = __fma_rn(" << lit((double)(n + 1)) << ", " << akref(i, n + 1) << ", "
                      << aref(i, n + 1) << ");\n";
                const Ref r = res(d.rhs[i]);
                if (nz(r, n)) acc(r, n, n, aref(i, n + 1), lit(1.0 / (double)(n + 1)));
            }
            for (uint32_t kk = d.n_ops; kk-- > 0;) emit_op_bw(kk, n);
            o << "}\n";
        }
        o << "static __device__ __noinline__ void hyk_jets_bw(double *__restrict__ S, const double t0, const double h, "
             "double *__restrict__ lam, double *__restrict__ pb) {\n";
        o << "#pragma unroll 1\n    for (int s = " << abase << "; s < " << nslot << "; ++s) S[s * HYK_STRIDE] = 0.0;\n";
        // Horner update x_new_i = sum_n x_i^[n] h^n
        o << "    double hp = 1.0;\n";
        for (uint32_t n = 0; n <= p; ++n) {
            for (uint32_t i = 0; i < N; ++i) o << "    " << aref(i, n) << " = lam[" << i << "] * hp;\n";
            if (n < p) o << "    hp = hp * h;\n";
        }
        for (uint32_t nn = p; nn-- > 0;) o << "    hyk_bw_o" << nn << "(S, t0, pb);\n";
        for (uint32_t i = 0; i < N; ++i) o << "    lam[" << i << "] = " << aref(i, 0) << ";\n";
        o << "}\n";
    }
};

const char *kTemplate =
#include "kernel_template.inc"
    ;

// hyk_dmath.h as a string (generated at build time from the header).
const char *kDmath =
#include "hyk_dmath.inc"
    ;

}  // namespace

uint32_t count_slots(const Dec &d, uint32_t order, bool adjoint) {
    Gen g(d, order, false, adjoint);
    return g.nslot;
}

bool generate(const Dec &d, uint32_t order, bool pin_arith, uint32_t blk, size_t kparams_size, GenOut &out,
              std::string &err, bool adjoint, uint64_t gmem_stride) {
    if (order < 2) {
        err = "the Taylor order must be at least 2";
        return false;
    }
    Gen g(d, order, pin_arith, adjoint);
    const double p = (double)order;
    const double e1 = std::exp(1.0);
    const double rhofac = 1.0 / (e1 * e1) * std::exp((-7.0 / 10.0) / (p - 1.0));
    std::ostringstream h;
    h << "// Generated by libhyk: " << d.n_eq << " equations, " << d.n_ops << " u-operations, order " << order
      << (pin_arith ? ", pin arithmetic" : "") << "\n";
    h << "#define HYK_NEQ " << d.n_eq << "\n#define HYK_NPARS " << d.n_pars << "\n#define HYK_ORDER " << order
      << "\n#define HYK_BLK " << blk << "\n#define HYK_TPB " << blk << "\n#define HYK_GMEM " << (gmem_stride ? 1 : 0)
      << "\n#define HYK_STRIDE " << (gmem_stride ? std::to_string(gmem_stride) + "ULL" : std::to_string(blk))
      << "\n#define HYK_NSLOT " << g.nslot << "\n#define HYK_PAR_SLOT " << g.par_slot
      << "\n#define HYK_RHOFAC " << lit(rhofac) << "\n#define HYK_INV_P " << lit(1.0 / p) << "\n#define HYK_INV_PM1 "
      << lit(1.0 / (p - 1.0)) << "\n";
    if (pin_arith) {
        h << "#define HYK_FMA_ACC(a, b, c) ((a) * (b) + (c))\n";
        h << "#define HYK_RHO(mp, mq, num) (1.0 / pow((mq) / (num), HYK_INV_PM1) < 1.0 / pow((mp) / (num), HYK_INV_P) "
             "? 1.0 / pow((mq) / (num), HYK_INV_PM1) : 1.0 / pow((mp) / (num), HYK_INV_P))\n";
    } else {
        h << "#define HYK_FMA_ACC(a, b, c) __fma_rn((a), (b), (c))\n";
        h << "#define HYK_RHO(mp, mq, num) hyk_dm_rho((mp), (mq), (num), HYK_INV_P, HYK_INV_PM1)\n";
    }
    if (adjoint) h << "#define HYK_ADJOINT 1\n";
    h << kDmath << "\n";
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
    out.par_slot = g.par_slot;
    // Per-step flops: recurrences + Horner (2 per coefficient) + step size
    // (two pow and the norm arithmetic) + double-length time update.
    out.flops = g.flops + 2.0 * d.n_eq * order + 46.0 + 10.0;
    return true;
}


// Host translation unit of the same generated recurrences (forward jets and,
// with the adjoint, the reverse sweep) for CPU checks of the generator: one
// lane, HYK_BLK = 1, the CUDA intrinsics mapped to their host equivalents.
bool generate_host(const Dec &d, uint32_t order, bool adjoint, std::string &src, std::string &err) {
    if (order < 2) {
        err = "the Taylor order must be at least 2";
        return false;
    }
    Gen g(d, order, false, adjoint);
    const double p = (double)order;
    const double e1 = std::exp(1.0);
    const double rhofac = 1.0 / (e1 * e1) * std::exp((-7.0 / 10.0) / (p - 1.0));
    std::ostringstream h;
    h << "#include <cmath>\n#include <cstdint>\n#define __device__\n#define __noinline__\n"
         "#define __forceinline__ inline\n#define __restrict__\n"
         "static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }\n"
         "static inline void __syncwarp() {}\n";
    h << kDmath << "\n";
    h << "#define HYK_NEQ " << d.n_eq << "\n#define HYK_NPARS " << d.n_pars << "\n#define HYK_ORDER " << order
      << "\n#define HYK_BLK 1\n#define HYK_STRIDE 1\n#define HYK_NSLOT " << g.nslot << "\n#define HYK_PAR_SLOT " << g.par_slot
      << "\n#define HYK_RHOFAC " << lit(rhofac) << "\n#define HYK_INV_P " << lit(1.0 / p) << "\n#define HYK_INV_PM1 "
      << lit(1.0 / (p - 1.0)) << "\n";
    h << "#define HYK_SX(i, n) S[((i) * (HYK_ORDER + 1) + (n)) * HYK_STRIDE]\n#define HYK_PAR(k) S[(HYK_PAR_SLOT + (k)) * HYK_STRIDE]\n";
    h << "static inline double hyk_inf() { return HUGE_VAL; }\n";
    g.emit_jets();
    if (adjoint) g.emit_bw();
    h << g.o.str();
    h << "extern \"C\" int hyk_host_nslot(void) { return HYK_NSLOT; }\n";
    h << "extern \"C\" void hyk_host_step(double *S, const double *x0, const double *pars, double t0, double h, double *x1) {\n"
         "    for (int i = 0; i < HYK_NEQ; ++i) HYK_SX(i, 0) = x0[i];\n"
         "    for (int k = 0; k < HYK_NPARS; ++k) HYK_PAR(k) = pars[k];\n"
         "    hyk_jets(S, t0);\n"
         "    for (int i = 0; i < HYK_NEQ; ++i) {\n"
         "        double acc = HYK_SX(i, HYK_ORDER);\n"
         "        for (int n = HYK_ORDER - 1; n >= 0; --n) acc = __fma_rn(acc, h, HYK_SX(i, n));\n"
         "        x1[i] = acc;\n    }\n}\n";
    if (adjoint)
        h << "extern \"C\" void hyk_host_adjoint(double *S, const double *x0, const double *pars, double t0, double h, "
             "double *lam, double *pb) {\n"
             "    for (int i = 0; i < HYK_NEQ; ++i) HYK_SX(i, 0) = x0[i];\n"
             "    for (int k = 0; k < HYK_NPARS; ++k) HYK_PAR(k) = pars[k];\n"
             "    hyk_jets(S, t0);\n    hyk_jets_bw(S, t0, h, lam, pb);\n}\n";
    src = h.str();
    return true;
}

}  // namespace hyk
