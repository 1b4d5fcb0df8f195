"""Builds libtealeaf_gb300.so for sm_103a from csrc/ with nvcc.

Each translation unit is compiled in its own process (in parallel), then
linked into tealeaf_opencl_gb300/_build/libtealeaf_gb300.so.  Device code is
built with --fmad=false and host code with -ffp-contract=off so that every
floating-point operation rounds as written.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtealeaf_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
              "-Xptxas", "-warn-spills"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC)
                  if f.endswith(".cu") or f.endswith(".cpp"))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "tealeaf_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def _compile(nvcc, src, verbose):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-I", CSRC, "-I", INCLUDE, "-c", src,
                                        "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, res.stdout, res.stderr))
    return obj, res.stderr


def build(force=False, verbose=False):
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(f) for f in _deps())):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    srcs = [os.path.join(CSRC, s) for s in sources()]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    cmd = [nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcuda"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (res.stdout, res.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
