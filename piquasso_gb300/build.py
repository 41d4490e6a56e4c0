"""Builds the GB300 permanent engine: piquasso_gb300/_lib/libpqperm_gb300.so.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked with a
static CUDA runtime.  Host code is plain C++17 and builds the same on x86 and
Arm.  ``nvcc`` cross-compiles without a GPU, so this runs on any machine with
the CUDA toolkit.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libpqperm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = [
    "capi.cu",
    "noalloc.cu",
    "mlp.cu",
    "mlp_tc.cu",
    "marginal.cu",
    "proposal.cu",
    "k_plain_c128_0.cu",
    "k_plain_c128_1.cu",
    "k_plain_c64_0.cu",
    "k_plain_c64_1.cu",
    "k_plain_df_0.cu",
    "k_plain_df_1.cu",
    "k_plain_c128o_0.cu",
    "k_plain_c128o_1.cu",
    "k_plain_c64o_0.cu",
    "k_plain_c64o_1.cu",
    "k_plain_dfo_0.cu",
    "k_plain_dfo_1.cu",
    "k_laplace_c128_0.cu",
    "k_laplace_c128_1.cu",
    "k_laplace_c64_0.cu",
    "k_laplace_c64_1.cu",
    "k_laplace_c64o_0.cu",
    "k_laplace_c64o_1.cu",
    "k_laplace_dfo_0.cu",
    "k_laplace_dfo_1.cu",
    "k_laplace_df_0.cu",
    "k_laplace_df_1.cu",
]
CPP_SOURCES = ["plan.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build piquasso_gb300")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".hpp"))]
    hs.append(os.path.join(INCLUDE, "pqperm_gb300.h"))
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            jobs.append([nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v", "-I", CSRC, "-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-I", CSRC, "-c", src, "-o", obj])

    def run(cmd):
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        with open(cmd[-1] + ".log", "w") as f:
            f.write(p.stdout)
        return cmd, p

    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            for cmd, p in ex.map(run, jobs):
                if p.returncode != 0:
                    sys.stderr.write(p.stdout)
                    raise RuntimeError("piquasso_gb300 build failed: " + " ".join(cmd))
                if verbose:
                    sys.stdout.write(p.stdout)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        subprocess.check_call([nvcc, "-shared", *ARCH, "-cudart", "static", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import time

    t0 = time.time()
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print("build: %.1f s" % (time.time() - t0))
