"""The fusion plan (heyoka.py_gb300/csrc/hyk_fuse.h), the choice shared by
both kernel forms and the oracle's GPU arithmetic: which sums absorb which
squares, scaled terms and inner sums, on the benchmark systems and on the
cases it must leave alone (a square or product read twice, a negation, a
constant)."""

import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_SRC = r"""
#include "hyk_fuse.h"
extern "C" int plan(uint32_t n_eq, uint32_t n_ops, const hyk_uop_t *ops, const hyk_arg_t *rhs, uint32_t n_ev,
                    const hyk_event_t *ev, int32_t *out, double *sc) {
    // out per operation: -2 dead, -1 plain, else the root's addend (or n_ops + n_eq for none)
    // followed, for roots, by the leaves in out[n_ops + 4 k + i] (-1 unused), the
    // kinds in out[5 n_ops + k], and the scales in sc[4 k + i]
    const HykFusePlan p = hyk_fuse_plan(n_eq, n_ops, ops, rhs, n_ev, ev);
    for (uint32_t k = 0; k < n_ops; ++k) {
        out[k] = p.dead[k] ? -2 : (p.fuse[k] ? (p.addend[k] >= 0 ? p.addend[k] : (int32_t)(n_eq + n_ops)) : -1);
        out[5 * n_ops + k] = p.fuse[k];
        for (int i = 0; i < HYK_FUSE_MAX; ++i) {
            out[n_ops + 4 * k + i] = (p.fuse[k] && i < (int)p.leaves[k].size()) ? p.leaves[k][i] : -1;
            sc[4 * k + i] = (p.fuse[k] == HYK_FUSE_SC && i < (int)p.scales[k].size()) ? p.scales[k][i] : 0.0;
        }
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def fuse_lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("fuse")
    src = d / "fuse.cpp"
    src.write_text(_SRC)
    so = d / "libfuse.so"
    subprocess.run(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "heyoka.py_gb300", "csrc"), str(src), "-o", str(so)], check=True)
    return ctypes.CDLL(str(so))


SQ, SC = 1, 2


def plan(lib, sys_, scales=False):
    """{u: "dead" | ("root", addend or None, leaves)} (with the kind and the
    leaves' numbers appended when scales)."""
    from hyk.decompose import taylor_decompose

    dec = taylor_decompose(sys_)
    d, keep = dec.as_c()
    n = dec.n_ops
    out = (ctypes.c_int32 * (6 * n))()
    sc = (ctypes.c_double * (4 * n))()
    assert lib.plan(d.n_eq, d.n_ops, d.ops, d.rhs, d.n_ev, d.ev, out, sc) == 0
    res = {}
    for k in range(n):
        u = dec.n_eq + k
        if out[k] == -2:
            res[u] = "dead"
        elif out[k] >= 0:
            leaves = [x for x in out[n + 4 * k: n + 4 * k + 4] if x >= 0]
            r = ("root", None if out[k] == dec.n_eq + n else out[k], leaves)
            if scales:
                r = r + (out[5 * n + k], list(sc[4 * k: 4 * k + len(leaves)]))
            elif out[5 * n + k] != SQ:
                continue
            res[u] = r
    return dec, res


def test_kepler_one_chain_of_three_squares(fuse_lib):
    from hyk import workloads as W

    dec, res = plan(fuse_lib, W.kepler_sys())
    roots = [v for v in res.values() if v != "dead"]
    assert roots == [("root", None, [0, 1, 2])]  # x^2 + y^2 + z^2 at the root, no addend
    assert sum(v == "dead" for v in res.values()) == 4  # three squares and the inner sum


def test_shared_square_is_not_absorbed(fuse_lib):
    import hyk

    x, y, z = hyk.make_vars("x", "y", "z")
    y2 = y**2
    # y^2 is read by two sums: it stays; each sum absorbs only its own single-use square
    sys_ = [(x, x**2 + y2), (y, z**2 + y2), (z, x)]
    dec, res = plan(fuse_lib, sys_)
    roots = sorted((v[1], v[2]) for v in res.values() if v != "dead")
    assert len(roots) == 2 and all(len(lv) == 1 for _, lv in roots)
    assert all(a is not None for a, _ in roots)  # y^2 is each root's addend


def test_negation_and_constants_left_alone(fuse_lib):
    import hyk

    x, y = hyk.make_vars("x", "y")
    # the square of a negation, and a square of a parameter (constant in time)
    sys_ = [(x, (-x) ** 2 + y**2), (y, hyk.par[0] ** 2 + x**2)]
    dec, res = plan(fuse_lib, sys_)
    for v in res.values():
        if v != "dead":
            _, a, leaves = v
            for u in leaves + ([a] if a is not None else []):
                assert u < dec.n_eq or dec.ops[u - dec.n_eq][0] not in (4,)  # no negation operand


def test_nbody_pairs(fuse_lib):
    from hyk import workloads as W

    dec, res = plan(fuse_lib, W.oss_sys(), scales=True)
    sq = [v for v in res.values() if v != "dead" and v[3] == SQ]
    sc = [v for v in res.values() if v != "dead" and v[3] == SC]
    # 6 bodies: 15 pairs, each |r_i - r_j|^2 a chain of three squares
    assert len(sq) == 15 and all(len(v[2]) == 3 and v[1] is None for v in sq)
    # 18 acceleration components, each a sum of 5 scaled terms: 4 in one
    # chain, the fifth added to it by a second root
    four = [v for v in sc if v[1] is None]
    one = [v for v in sc if v[1] is not None]
    assert len(four) == 18 and all(len(v[2]) == 4 for v in four)
    assert len(one) == 18 and all(len(v[2]) == 1 for v in one)
    roots4 = {u for u, v in res.items() if v != "dead" and v[3] == SC and v[1] is None}
    assert {v[1] for v in one} == roots4
    # products, their negations and the inner sums: computed nowhere
    assert sum(v == "dead" for v in res.values()) == 15 * 4 + 18 * 5 + 45 + 18 * 2
    # the leaves' numbers are the masses times G, with the signs of the negations
    ms = sorted({abs(k) for v in sc for k in v[4]})
    assert len(ms) == 6 and all(k > 0 for k in ms)
    assert sum(k < 0 for v in sc for k in v[4]) == 45


def test_scaled_sums(fuse_lib):
    import hyk

    x, y, z = hyk.make_vars("x", "y", "z")
    # a - k b and -(k b) + a: the subtrahend's and the negation's signs go into
    # the numbers; a product read twice stays
    w = 5.0 * z
    sys_ = [(x, 2.0 * y - 3.0 * z), (y, -(4.0 * x) + z * x), (z, w + y + w * x)]
    dec, res = plan(fuse_lib, sys_, scales=True)
    sc = {tuple(v[2]): (v[1], v[4]) for v in res.values() if v != "dead" and v[3] == SC}
    assert sc[(1, 2)] == (None, [2.0, -3.0])
    assert any(v[1] == [-4.0] and v[0] is not None for v in sc.values())
    # w = 5 z is read twice: never a leaf
    wu = [u for u, v in res.items() if v == "dead"]
    for u in wu:
        op = dec.ops[u - dec.n_eq]
        assert not (op[0] == 2 and 5.0 in [a for a in op[1:] if isinstance(a, float)])
