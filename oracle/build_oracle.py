"""Build recipe for the oracle (test infrastructure; plain g++, no GPU).

Compiles ``skew_oracle.cpp`` into ``libskew_oracle.so`` next to it (-O3, no BLAS:
every loop is the restatement's own scalar code).  Floating point contraction is
switched off and no reassociation is allowed, so the FP64 restatement rounds the
same way on x86-64 and aarch64.  On x86-64 the quad type is __float128 (libquadmath); on
aarch64 it is the native binary128 long double.
"""
from __future__ import annotations

import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "skew_oracle.cpp")
OUT = os.path.join(HERE, "libskew_oracle.so")


def build_oracle(force: bool = False) -> str:
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    libs = ["-lquadmath"] if platform.machine() in ("x86_64", "AMD64") else []
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", SRC, "-o",
           OUT + ".tmp"] + libs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build_oracle(force=True))
