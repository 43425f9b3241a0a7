"""Build the engine's shared library and C host program with nvcc / gcc.

    python -m raptor_gb300.build            # library + host program
    python -m raptor_gb300.build --clean

Products (git-ignored, in-tree):
    raptor_gb300/_lib/libraptor_gpu.so   the C-ABI engine (include/raptor_gpu.h)
    raptor_gb300/_lib/libraptor_gpu_checked.so  the same with device-side bounds
                                          checks (-DRAPTOR_CHECKED, csrc/checked.cuh)
    raptor_gb300/_lib/libraptor_benchutil.so  FP64 peak probe and L2 flush for bench.py
    raptor_gb300/_lib/raptor_gb300       C host program, drop-in for `./RAPTOR`
Translation units compile in parallel; one -gencode (sm_103a) only.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(ROOT, "_build", "obj")
LIB = os.path.join(LIBDIR, "libraptor_gpu.so")
LIB_CHECKED = os.path.join(LIBDIR, "libraptor_gpu_checked.so")
BENCH_LIB = os.path.join(LIBDIR, "libraptor_benchutil.so")
HOST_BIN = os.path.join(LIBDIR, "raptor_gb300")

CU_SOURCES = ["raptor_gpu.cu", "tuner.cu", "vjp.cu", "noalloc.cu", "ray_kernel_df.cu", "vjp_df.cu"]
HOST_SOURCES = ["raptor_main.c", "harm_io.c", "model_io.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--ptxas-options=-O3", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _deps_newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
           [os.path.join(INCLUDE, "raptor_gpu.h")]


def _compile(src: str, verbose: bool, checked: bool = False) -> str:
    obj = os.path.join(OBJDIR + ("_checked" if checked else ""), os.path.basename(src) + ".o")
    if not _deps_newer(obj, [src] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-DRAPTOR_CHECKED"] if checked else []) + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(verbose: bool = False, checked: bool = False) -> str:
    """The engine library; checked: the bounds-checked build."""
    lib = LIB_CHECKED if checked else LIB
    os.makedirs(OBJDIR + ("_checked" if checked else ""), exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, checked), srcs))
    if _deps_newer(lib, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return lib


def build_bench_util(verbose: bool = False) -> str:
    src = os.path.join(CSRC, "bench_util.cu")
    if _deps_newer(BENCH_LIB, [src]):
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-shared", "-o", BENCH_LIB, src]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"bench_util build failed:\n{r.stdout}\n{r.stderr}")
    return BENCH_LIB


def build_host(verbose: bool = False) -> str:
    srcs = [os.path.join(HOST, s) for s in HOST_SOURCES]
    if not all(os.path.exists(s) for s in srcs):
        return ""
    deps = srcs + [LIB] + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    if _deps_newer(HOST_BIN, deps):
        cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-fopenmp", "-Wall", "-I" + INCLUDE,
               "-I" + HOST, "-o", HOST_BIN] + srcs + ["-L" + LIBDIR, "-lraptor_gpu",
                                                      "-Wl,-rpath,$ORIGIN", "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host build failed:\n{r.stdout}\n{r.stderr}")
    return HOST_BIN


def build(verbose: bool = False) -> str:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_chk = ex.submit(build_library, verbose, True)
        f_bench = ex.submit(build_bench_util, verbose)
        lib = f_lib.result()
        f_chk.result()
        f_bench.result()
    build_host(verbose)
    return lib


def clean():
    for p in (LIBDIR, OBJDIR, OBJDIR + "_checked"):
        if os.path.isdir(p):
            shutil.rmtree(p)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    if a.clean:
        clean()
        sys.exit(0)
    print(build(a.verbose))
