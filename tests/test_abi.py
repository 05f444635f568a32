"""The C ABI library: loads without a GPU, exports every declared symbol,
and its code generator emits CUDA that NVRTC compiles for sm_103a."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "hyk.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hyk_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(libhyk):
    syms = declared_symbols()
    assert "hyk_module_create" in syms and "hyk_propagate" in syms
    for s in syms:
        assert hasattr(libhyk, s), s


def test_python_binding_covers_header(libhyk):
    from hyk import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_struct_layouts(tmp_path):
    """The ctypes mirrors have the sizes and field offsets of the C header
    (a host program compiled against include/hyk.h prints them)."""
    import subprocess

    from hyk import _lib
    from hyk.decompose import hyk_arg_t, hyk_decomp_t, hyk_event_t, hyk_uop_t

    structs = {
        "hyk_arg_t": hyk_arg_t, "hyk_uop_t": hyk_uop_t, "hyk_decomp_t": hyk_decomp_t, "hyk_event_t": hyk_event_t,
        "hyk_config_t": _lib.hyk_config_t, "hyk_module_info_t": _lib.hyk_module_info_t,
        "hyk_lanes_t": _lib.hyk_lanes_t, "hyk_prop_t": _lib.hyk_prop_t,
    }
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "hyk.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append('printf("%s %zu\\n", "{0}", sizeof({0}));'.format(name))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %zu\\n", "{0}", "{1}", offsetof({0}, {1}));'.format(name, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.splitlines())
    for name, cls in structs.items():
        assert int(out[name]) == ctypes.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(out[name + "." + f]) == getattr(cls, f).offset, (name, f)


def test_no_device_errors(libhyk):
    import hyk
    from hyk.decompose import taylor_decompose
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    d, keep = taylor_decompose(hyk.workloads.pendulum_sys()).as_c()
    h = ctypes.c_void_p()
    rc = libhyk.hyk_module_create(ctypes.byref(d), 20, None, 0, ctypes.byref(h))
    assert rc != 0 and libhyk.hyk_last_error()


@pytest.mark.parametrize("name", ["pendulum", "kepler", "forced", "cr3bp"])
def test_codegen_compiles_for_sm103a(libhyk, name):
    import hyk
    from hyk import _lib, workloads as W
    from hyk.decompose import taylor_decompose

    x, v = hyk.make_vars("x", "v")
    systems = {
        "pendulum": (W.pendulum_sys(), 20),
        "kepler": (W.kepler_sys(), 19),
        "forced": ([(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))], 20),
        "cr3bp": (W.cr3bp_sys(), 19),
    }
    sys_, order = systems[name]
    d, keep = taylor_decompose(sys_).as_c()
    for pin in (0, 1):
        cfg = _lib.hyk_config_t(128, 0, pin, 0)
        buf = ctypes.create_string_buffer(1 << 16)
        ns, fl = ctypes.c_uint32(), ctypes.c_double()
        rc = libhyk.hyk_codegen_check(ctypes.byref(d), order, ctypes.byref(cfg), 0, buf, len(buf), ctypes.byref(ns),
                                      ctypes.byref(fl))
        assert rc == 0, libhyk.hyk_last_error().decode()
        assert ns.value > 0 and fl.value > 0


def test_codegen_rejects_bad_input(libhyk):
    from hyk.decompose import hyk_arg_t, hyk_decomp_t, hyk_uop_t

    ops = (hyk_uop_t * 1)()
    ops[0].op, ops[0].aux = 2, -1
    ops[0].a.kind, ops[0].a.idx = 1, 5  # refers to a later u-variable
    ops[0].b.kind, ops[0].b.idx = 1, 0
    rhs = (hyk_arg_t * 1)()
    rhs[0].kind, rhs[0].idx = 1, 1
    d = hyk_decomp_t(1, 1, 0, 0, ctypes.cast(ops, ctypes.POINTER(hyk_uop_t)), ctypes.cast(rhs, ctypes.POINTER(hyk_arg_t)))
    rc = libhyk.hyk_codegen_check(ctypes.byref(d), 10, None, 0, None, 0, None, None)
    assert rc == -1 and b"invalid" in libhyk.hyk_last_error()


@pytest.mark.parametrize("team", [0, 4])
def test_debug_build_compiles_for_sm103a(libhyk, team):
    """HYK_CFG_DEBUG: the generated source carries the debug hooks (lane
    index checks, the non-finite coefficient record) and compiles with NVRTC
    for sm_103a, in the lane and the team form."""
    from hyk import _lib, workloads as W
    from hyk.decompose import taylor_decompose

    d, keep = taylor_decompose(W.kepler_sys()).as_c()
    cfg = _lib.hyk_config_t(128 if team == 0 else 32, 0, _lib.HYK_CFG_DEBUG, team)
    buf = ctypes.create_string_buffer(1 << 16)
    rc = libhyk.hyk_codegen_check(ctypes.byref(d), 19, ctypes.byref(cfg), 0, buf, len(buf), None, None)
    assert rc == 0, libhyk.hyk_last_error().decode()
    assert libhyk.hyk_module_debug(None, None, 0) == _lib.HYK_ERR_INVALID
