"""The sum-of-squares fusion plan (heyoka.py_gb300/csrc/hyk_fuse.h), the
choice shared by both kernel forms and the oracle's GPU arithmetic: which
ADDs absorb which squares and sums, on the benchmark systems and on the
cases it must leave alone (a square read twice, a negation, a constant)."""

import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_SRC = r"""
#include "hyk_fuse.h"
extern "C" int plan(uint32_t n_eq, uint32_t n_ops, const hyk_uop_t *ops, const hyk_arg_t *rhs, uint32_t n_ev,
                    const hyk_event_t *ev, int32_t *out) {
    // out per operation: -2 dead, -1 plain, else the root's addend (or n_ops + n_eq for none)
    // followed, for roots, by the leaves in out[n_ops + 4 k + i] (-1 unused)
    const HykFusePlan p = hyk_fuse_plan(n_eq, n_ops, ops, rhs, n_ev, ev);
    for (uint32_t k = 0; k < n_ops; ++k) {
        out[k] = p.dead[k] ? -2 : (p.fuse[k] ? (p.addend[k] >= 0 ? p.addend[k] : (int32_t)(n_eq + n_ops)) : -1);
        for (int i = 0; i < HYK_FUSE_MAX; ++i)
            out[n_ops + 4 * k + i] = (p.fuse[k] && i < (int)p.leaves[k].size()) ? p.leaves[k][i] : -1;
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


def plan(lib, sys_):
    from hyk.decompose import taylor_decompose

    dec = taylor_decompose(sys_)
    d, keep = dec.as_c()
    n = dec.n_ops
    out = (ctypes.c_int32 * (5 * n))()
    assert lib.plan(d.n_eq, d.n_ops, d.ops, d.rhs, d.n_ev, d.ev, out) == 0
    res = {}
    for k in range(n):
        u = dec.n_eq + k
        if out[k] == -2:
            res[u] = "dead"
        elif out[k] >= 0:
            leaves = [x for x in out[n + 4 * k: n + 4 * k + 4] if x >= 0]
            res[u] = ("root", None if out[k] == dec.n_eq + n else out[k], leaves)
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

    dec, res = plan(fuse_lib, W.oss_sys())
    roots = [v for v in res.values() if v != "dead"]
    # 6 bodies: 15 pairs, each |r_i - r_j|^2 a chain of three squares
    assert len(roots) == 15 and all(len(v[2]) == 3 and v[1] is None for v in roots)
