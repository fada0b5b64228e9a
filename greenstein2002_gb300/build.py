"""Build libgw_fru.so in-tree (greenstein2002_gb300/_build/).

nvcc compiles the CUDA sources for sm_103a only; gcc compiles the host C
sources.  Host code uses -ffp-contract=off so x86-64 and aarch64 builds give
identical FP64 results; the FP64 FRU kernel is built with -fmad=false so its
arithmetic matches the reference's operation by operation.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgw_fru.so")
EXE = os.path.join(OUT, "gw_caf")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-I" + CSRC, "-I" + INC]
CUDA_UNITS = {
    # source: extra flags
    "gw_fru_stage.cu": ["-fmad=false"],
    "gw_fru_stage4.cu": ["-fmad=false"],
    "gw_fru_mixed.cu": [],
    "gw_batch.cu": [],
    "gw_serve.cu": [],
    "gw_abi.cu": [],
    "gw_probe.cu": [],
    "gw_noalloc.cu": ["-fmad=false"],
    "gw_tune.cu": [],
    "gw_devdp.cu": ["-fmad=false"],
    "gw_persist.cu": ["-fmad=false"],
}
C_UNITS = ["gw_dp.c", "gw_dropin.c"]


def _nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if p and (os.path.isabs(p) and os.path.exists(p) or not os.path.isabs(p)):
            return p
    return "nvcc"


def _sources():
    return ([os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INC, "gw_fru.h")] +
            [os.path.join(HERE, "host", f) for f in os.listdir(os.path.join(HERE, "host"))])


def up_to_date():
    if not os.path.isfile(LIB) or not os.path.isfile(EXE):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src, extra in CUDA_UNITS.items():
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        jobs.append([nvcc] + NVCC_COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj])
    cc = os.environ.get("CC", "gcc")
    for src in C_UNITS:
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        jobs.append([cc, "-O2", "-std=c99", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + CSRC, "-I" + INC,
                     "-c", os.path.join(CSRC, src), "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs + ["-lm", "-lpthread"])
    # the C host driver (caf.c main loop) linked against the library
    run([cc, "-O2", "-std=c99", "-ffp-contract=off", "-Wall", "-I" + CSRC, "-I" + INC, "-o", EXE,
         os.path.join(HERE, "host", "gw_caf.c"), "-L" + OUT, "-lgw_fru", "-Wl,-rpath,$ORIGIN", "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
