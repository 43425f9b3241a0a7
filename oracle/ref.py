"""ctypes wrapper around the reference RAPTOR build (oracle test
infrastructure).

The shared library is the reference's own C sources, compiled unmodified by
oracle/Makefile with compile-time overrides (ref_config.h).  opt="ieee" (-O2,
the source's IEEE semantics) is the parity oracle; opt="stock" (-Ofast, the
reference makefile's flags) is only timed.  This module is
imported only by tests/, by tests/golden/make_golden.py and by bench.py's
CPU-baseline leg; the engine never calls it.

The reference's sources are read from oracle/_ref/src, a git-ignored copy
that `stage()` (make -C oracle stage) takes from a reference checkout, so
the same build runs wherever that directory travels; RAPTOR_REFERENCE_DIR
names another source directory.  Without sources `available()` is False
and callers fall back to the C port (oracle/port.py).
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STAGED_DIR = os.path.join(HERE, "_ref", "src")
REF_SRC_DIR = os.environ.get("RAPTOR_REFERENCE_DIR", STAGED_DIR)
_LIBS: dict = {}


def sources_present() -> bool:
    return os.path.isfile(os.path.join(REF_SRC_DIR, "integrator.c"))


def stage(reference_dir: str) -> str:
    """Copy the reference's C sources and headers from reference_dir into
    oracle/_ref/src (git-ignored).  Returns the staged directory."""
    subprocess.run(["make", "-s", "-C", HERE, "stage", f"REFERENCE={reference_dir}"], check=True)
    return STAGED_DIR


def lib_path(n1: int, n2: int, rk: str = "RK4", opt: str = "ieee", cam: str = "linear") -> str:
    suffix = "_logcam" if cam == "log" else ""
    return os.path.join(HERE, "_ref", f"libraptor_ref_{n1}x{n2}_{rk}_{opt}{suffix}.so")


def build(n1: int, n2: int, rk: str = "RK4", opt: str = "ieee", cam: str = "linear") -> str:
    """cam: "linear" (LINEAR_IMPACT_CAM, the stock camera) or "log" (LOG_IMPACT_CAM)."""
    path = lib_path(n1, n2, rk, opt, cam)
    if not os.path.exists(path):
        if not sources_present():
            raise FileNotFoundError("reference sources are not present on this machine")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"N1={n1}", f"N2={n2}", f"RK={rk}", f"OPT={opt}",
                        f"CAM={cam}", f"REFDIR={REF_SRC_DIR}"], check=True)
    return path


def available(n1: int, n2: int, rk: str = "RK4", opt: str = "ieee", cam: str = "linear") -> bool:
    """True if a reference library for this grid can be loaded here."""
    path = lib_path(n1, n2, rk, opt, cam)
    if not os.path.exists(path) and not sources_present():
        return False
    try:
        load(n1, n2, rk, opt, cam)
        return True
    except OSError:
        return False


def load(n1: int, n2: int, rk: str = "RK4", opt: str = "ieee", cam: str = "linear") -> ctypes.CDLL:
    key = (n1, n2, rk, opt, cam)
    if key in _LIBS:
        return _LIBS[key]
    lib = ctypes.CDLL(build(n1, n2, rk, opt, cam), mode=ctypes.RTLD_LOCAL)
    D = ctypes.c_double
    P = ctypes.POINTER
    lib.ref_setup.argtypes = [ctypes.c_char_p, ctypes.c_char_p, D, D, D, D, D]
    lib.ref_setup.restype = ctypes.c_int
    lib.ref_render_serial.argtypes = [D, P(D), P(D)]
    lib.ref_render_serial.restype = ctypes.c_int
    lib.ref_render_pixels.argtypes = [P(ctypes.c_int), ctypes.c_int, D, P(D), ctypes.c_int]
    lib.ref_render_pixels.restype = ctypes.c_int
    lib.ref_wtime.restype = D
    _LIBS[key] = lib
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class RefSession:
    """One reference set-up (model.in + dump + argv scalars), after which
    images are rendered serially (stock calculate_image) or over a pixel
    list with OpenMP."""

    def __init__(self, dump_path: str, model, m_unit: float, inclination: float,
                 r_high: float, r_low: float, time_init: float = 0.0, rk: str = "RK4", opt: str = "ieee",
                 n1: int | None = None, n2: int | None = None, workdir: str | None = None, cam: str = "linear"):
        from raptor_gb300.harm import read_dump
        if n1 is None:
            with open(dump_path) as f:
                head = f.readline().split()
            n1, n2 = int(head[1]), int(head[2])
        self.n1, self.n2 = n1, n2
        self.model = model
        self.lib = load(n1, n2, rk, opt, cam)
        self._tmp = tempfile.mkdtemp(prefix="rgo_", dir=workdir or "/tmp")
        self.model_path = os.path.join(self._tmp, "model.in")
        model.write(self.model_path)
        self.dump_path = dump_path
        self.args = (m_unit, inclination, r_high, r_low, time_init)
        self._setup()

    def _setup(self):
        rc = self.lib.ref_setup(self.model_path.encode(), self.dump_path.encode(), *self.args)
        if rc != 0:
            raise RuntimeError(f"ref_setup failed ({rc})")

    def render_serial(self, freq: float):
        w, h = self.model.IMG_WIDTH, self.model.IMG_HEIGHT
        out = np.zeros(w * h)
        spec = np.zeros(1)
        t0 = self.lib.ref_wtime()
        rc = self.lib.ref_render_serial(freq, _dptr(out), _dptr(spec))
        t1 = self.lib.ref_wtime()
        if rc != 0:
            raise RuntimeError(f"ref_render_serial failed ({rc})")
        self._setup()  # calculate_image frees the grid pointer (core.c:143)
        return out, float(spec[0]), t1 - t0

    def render_pixels(self, pixels, freq: float, nthreads: int = 0):
        pix = np.ascontiguousarray(pixels, dtype=np.int32)
        out = np.zeros(len(pix))
        t0 = self.lib.ref_wtime()
        rc = self.lib.ref_render_pixels(pix.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(pix),
                                        freq, _dptr(out), nthreads)
        t1 = self.lib.ref_wtime()
        if rc != 0:
            raise RuntimeError(f"ref_render_pixels failed ({rc})")
        return out, t1 - t0


def machine() -> str:
    return platform.machine()
