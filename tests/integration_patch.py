"""Builds the reference RAPTOR program with its calculate_image replaced by
the engine call that INTEGRATION.md section 1 shows - the drop-in as a
maintainer of the reference would apply it.

The patch is taken from INTEGRATION.md itself (its first C block), so what
the document shows is what is compiled.  The program is the reference's own
sources (main.c and the eleven files of the imaging path, from
oracle/_ref/src, which `make -C oracle stage` fills from a reference
checkout), with core.c's calculate_image (core.c:74-152) swapped for the
patch, compiled with the reference makefile's CPU flags (makefile:13-15,
plus -fcommon and the stub GSL/PNG headers the oracle build uses; N1, N2
and int_method set through oracle/ref_config.h as a user sets them in
parameters.h) and linked against libraptor_gpu.so.

Test infrastructure for tests/test_integration_patch.py (builds and links on
the CPU) and tests/test_gpu_integration_patch.py (runs it on the GPU).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
SOURCES = ["main.c", "core.c", "GRmath.c", "integrator.c", "metric.c", "radiative_transfer.c",
           "raptor_harm_model.c", "utilities.c", "j_nu.c", "rcarry.c", "newtonraphson.c", "grmhd.c"]
HEADERS = ["constants.h", "functions.h", "parameters.h", "raptor_harm_model.h"]
# makefile:13-15 (CPU build), with -fcommon for gcc >= 10
CFLAGS = ["-fopenmp", "-std=c99", "-Ofast", "-Wno-unused-result", "-fcommon", "-w"]


def sources_dir() -> str | None:
    from oracle import ref
    d = ref.REF_SRC_DIR
    ok = all(os.path.isfile(os.path.join(d, f)) for f in SOURCES + HEADERS)
    return d if ok else None


def patch_block() -> str:
    """The replacement calculate_image of INTEGRATION.md section 1."""
    md = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"```c\n(.*?)```", md, re.S)
    if not m or "void calculate_image(" not in m.group(1):
        raise ValueError("INTEGRATION.md holds no calculate_image patch")
    return m.group(1)


def patched_core(core: str, block: str) -> str:
    """core.c with the definition of calculate_image replaced by block."""
    start = core.index("void calculate_image(")
    i = core.index("{", start)
    depth = 0
    while True:
        if core[i] == "{":
            depth += 1
        elif core[i] == "}":
            depth -= 1
            if depth == 0:
                break
        i += 1
    return core[:start] + block + core[i + 1:]


def build(out_dir: str, n1: int = 64, n2: int = 64, rk: str = "RK4", lib_dir: str | None = None) -> str:
    """Writes the patched sources under out_dir/src and builds out_dir/RAPTOR;
    returns its path."""
    src = sources_dir()
    if src is None:
        raise FileNotFoundError("the reference's sources are not staged (make -C oracle stage REFERENCE=...)")
    from raptor_gb300 import engine
    lib_dir = lib_dir or os.path.dirname(engine.LIB_PATH)
    work = os.path.join(out_dir, "src")
    os.makedirs(work, exist_ok=True)
    for f in SOURCES + HEADERS:
        shutil.copyfile(os.path.join(src, f), os.path.join(work, f))
    core = open(os.path.join(src, "core.c")).read()
    with open(os.path.join(work, "core.c"), "w") as f:
        f.write(patched_core(core, patch_block()))
    exe = os.path.join(out_dir, "RAPTOR")
    cmd = (["gcc"] + CFLAGS +
           ["-I" + work, "-I" + os.path.join(ORACLE, "ref_stubs"), "-I" + os.path.join(ROOT, "include"),
            "-include", os.path.join(ORACLE, "ref_config.h"), f"-DREF_N1={n1}", f"-DREF_N2={n2}",
            f"-DREF_INT_METHOD={rk}"] +
           [os.path.join(work, f) for f in SOURCES] + [os.path.join(ORACLE, "ref_stubs", "gsl_hyperg_stub.c")] +
           ["-o", exe, "-L" + lib_dir, "-lraptor_gpu", "-Wl,-rpath," + lib_dir, "-lm"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"patched RAPTOR build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return exe
