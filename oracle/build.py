"""Build recipe for the CPU oracle (test infrastructure only).

Compiles tea_oracle_kernels.c and tea_oracle_driver.c with gcc into
oracle/_build/libtea_oracle.so.  -ffp-contract=off keeps every multiply and
add separately rounded, as the CUDA build does with --fmad=false.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtea_oracle.so")
SOURCES = ["tea_oracle_kernels.c", "tea_oracle_driver.c"]


def build(force=False, verbose=False):
    srcs = [os.path.join(HERE, s) for s in SOURCES + ["tea_oracle.h"]]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC",
           "-shared", "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"]
    cmd += [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
