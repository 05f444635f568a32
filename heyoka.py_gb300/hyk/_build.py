"""In-tree build of libhyk.so (the CUDA library behind the C ABI of include/hyk.h).

nvcc compiles the system-independent kernels for sm_103a and the C++ runtime
and code generator with the host compiler; the per-system kernels are
generated and compiled at run time by NVRTC.  The three translation units
are compiled in parallel, then linked against the CUDA driver and NVRTC.
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)  # heyoka.py_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIB_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIB_DIR, "libhyk.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = ["hyk_generic.cu", "hyk_noalloc.cu", "hyk_runtime.cpp", "hyk_codegen.cpp"]
DEPS = SOURCES + ["kernel_template.inc", "kernel_common.inc", "kernel_team.inc", "hyk_internal.hpp", "hyk_dmath.h", "hyk_fuse.h",
                  "hyk_events.h"]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    files = [os.path.join(CSRC, f) for f in DEPS] + [os.path.join(INCLUDE, "hyk.h"), __file__]
    return any(os.path.getmtime(f) > t for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(LIB_DIR, exist_ok=True)
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    # The deterministic math header is also compiled into every generated
    # module: embed its text as a C++ raw string.
    with open(os.path.join(CSRC, "hyk_dmath.h")) as f:
        dm = f.read()
    with open(os.path.join(obj_dir, "hyk_dmath.inc"), "w") as f:
        f.write('R"HYKDM(' + dm + ')HYKDM"\n')
    with open(os.path.join(CSRC, "hyk_events.h")) as f:
        ev = f.read()
    with open(os.path.join(obj_dir, "hyk_events.inc"), "w") as f:
        f.write('R"HYKEV(' + ev + ')HYKEV"\n')
    # --fmad=false: device arithmetic exactly as written (no contraction), so
    # the shared math gives the same bits as the host build of the oracle.
    # -ffp-contract=off: the code generator's host arithmetic (the literals it
    # prints) is the same on x86-64 and on AArch64, where GCC would otherwise
    # fuse multiply-adds.
    common = [NVCC, "-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", INCLUDE, "-I", CSRC]
    common += ["-I", obj_dir]
    common += GENCODE

    def compile_one(src):
        obj = os.path.join(obj_dir, src + ".o")
        cmd = common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compilation of {} failed:\n{}\n{}".format(src, r.stdout, r.stderr))
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    link = (
        [NVCC, "-shared", "-o", tmp]
        + GENCODE
        + objs
        + [
            "-L" + os.path.join(CUDA_HOME, "lib64"),
            "-lnvrtc",
            "-ldl",
            "-Xlinker",
            "-rpath=" + os.path.join(CUDA_HOME, "lib64"),
        ]
    )
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link of libhyk.so failed:\n{}\n{}".format(r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
