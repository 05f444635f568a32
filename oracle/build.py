"""Build the CPU oracle (test infrastructure): oracle/_build/libhyk_oracle.so.

g++ -O3 -fopenmp -ffp-contract=off; no -march flags, so the same source gives
the same results on x86-64 and aarch64.  binary128 uses libquadmath on x86-64
and the IEEE-quad long double of aarch64.
"""

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhyk_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "hyk_oracle.cpp")
    hdr = os.path.join(ROOT, "include", "hyk.h")
    csrc = os.path.join(ROOT, "heyoka.py_gb300", "csrc")
    deps = [src, hdr] + [os.path.join(csrc, f) for f in ("hyk_dmath.h", "hyk_events.h", "hyk_fuse.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = [
        "g++",
        "-std=c++17",
        "-O3",
        "-fopenmp",
        "-ffp-contract=off",
        "-fno-fast-math",
        "-fPIC",
        "-shared",
        "-I",
        os.path.join(ROOT, "include"),
        "-I",
        os.path.join(ROOT, "heyoka.py_gb300", "csrc"),
        src,
        "-o",
        LIB + ".tmp",
    ]
    if platform.machine() in ("x86_64", "i686"):
        cmd.append("-lquadmath")
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
