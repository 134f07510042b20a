"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/mibm_oracle.cpp into oracle/_build/libmibm_oracle.so with
g++ and OpenMP.  ``-ffp-contract=off`` keeps the arithmetic identical on x86
and Arm hosts (no fused multiply-add contraction), as the reference's
gfortran build on baseline x86-64 has none.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mibm_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmibm_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    hdr = os.path.join(os.path.dirname(HERE), "include", "mibm.h")
    # the written-out exp of the MLS weights, shared with the library
    mexp = os.path.join(os.path.dirname(HERE), "melt_ibm_gb300", "csrc", "mls_exp.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr), os.path.getmtime(mexp))):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
