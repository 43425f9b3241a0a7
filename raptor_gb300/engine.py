"""Python binding of the engine's C ABI (include/raptor_gpu.h) via ctypes.

This is a thin mirror of the C interface for tests, benchmarks and Python
callers; the reference-facing host is the C program in raptor_gb300/host.
The library must be the in-tree build (raptor_gb300/_lib/libraptor_gpu.so):
there is no CPU fallback, and every call raises EngineError on a non-zero
status.
"""
from __future__ import annotations

import ctypes
import os
import warnings
from typing import Sequence

import numpy as np

from .synth import GridGeom

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libraptor_gpu.so")
# the same engine with device-side bounds checks (csrc/checked.cuh)
CHECKED_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libraptor_gpu_checked.so")

RAPTOR_MAX_FREQS = 8
RAPTOR_MAX_GRIDS = 16
PREC_FP64 = 0
PREC_MIXED = 1
PREC_MIXED_DF = 2
RK4 = 4
RK2 = 2
CAM_LINEAR = 0
CAM_LOG = 1
EMISSION_THERMAL = 0
EMISSION_KAPPA = 1
TRACE_WIDTH = 16

STATUS = {0: "OK", -1: "INVALID", -2: "CUDA", -3: "DEVICE", -4: "NOMEM", -5: "NODEVICE", -6: "NOALLOC_LIMIT",
          -7: "NONFINITE", 1: "WARN_STEPCAP"}
ERR_NONFINITE = -7
WARN_STEPCAP = 1

EXPORTED = ("raptor_gpu_init", "raptor_gpu_destroy", "raptor_gpu_last_error", "raptor_gpu_upload_grid",
            "raptor_gpu_render", "raptor_gpu_render_range", "raptor_gpu_output_size",
            "raptor_gpu_spectrum_size", "raptor_gpu_get_stats", "raptor_gpu_vjp", "raptor_gpu_trace_ray",
            "raptor_gpu_vjp_range", "raptor_gpu_render_noalloc")


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class EngineWarning(UserWarning):
    """A positive status: the call's results are complete (for example, rays
    stopped at the step cap, as the reference stops them)."""


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("block_size", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("refill_interval", ctypes.c_int), ("autotune", ctypes.c_int), ("use_graph", ctypes.c_int),
                ("no_sample_pool", ctypes.c_int), ("vjp_tape", ctypes.c_int),
                ("reserved", ctypes.c_int * 6)]


class GridGeomC(ctypes.Structure):
    _fields_ = [("n1", ctypes.c_int), ("n2", ctypes.c_int), ("startx1", ctypes.c_double),
                ("startx2", ctypes.c_double), ("dx1", ctypes.c_double), ("dx2", ctypes.c_double),
                ("a", ctypes.c_double), ("hslope", ctypes.c_double), ("R0", ctypes.c_double)]


class ImageDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("cam_size_x", ctypes.c_double),
                ("cam_size_y", ctypes.c_double), ("inclination", ctypes.c_double), ("mbh", ctypes.c_double),
                ("m_unit", ctypes.c_double), ("r_high", ctypes.c_double), ("r_low", ctypes.c_double),
                ("stepsize", ctypes.c_double), ("integrator", ctypes.c_int), ("grid", ctypes.c_int),
                ("n_freq", ctypes.c_int), ("freq", ctypes.c_double * RAPTOR_MAX_FREQS), ("camera", ctypes.c_int),
                ("emission", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("kernel_ms", ctypes.c_double), ("device_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("h2d_bytes", ctypes.c_double),
                ("d2h_bytes", ctypes.c_double), ("rays", ctypes.c_longlong), ("steps", ctypes.c_longlong),
                ("rt_calls", ctypes.c_longlong), ("rt_samples", ctypes.c_longlong),
                ("max_ray_steps", ctypes.c_longlong), ("n_stepcap", ctypes.c_longlong),
                ("n_nonfinite", ctypes.c_longlong), ("kk_max", ctypes.c_double), ("block_size", ctypes.c_int),
                ("blocks_per_sm", ctypes.c_int), ("refill_interval", ctypes.c_int),
                ("grid_blocks", ctypes.c_int), ("graph_replayed", ctypes.c_int),
                ("device_bytes", ctypes.c_longlong), ("peak_device_bytes", ctypes.c_longlong),
                ("vjp_terms", ctypes.c_longlong), ("vjp_gated_terms", ctypes.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GradC(ctypes.Structure):
    _fields_ = [("d_m_unit", ctypes.c_double), ("d_r_high", ctypes.c_double), ("d_r_low", ctypes.c_double),
                ("d_inclination", ctypes.c_double), ("d_rho", ctypes.POINTER(ctypes.c_double)),
                ("d_u", ctypes.POINTER(ctypes.c_double)), ("d_lnthetae", ctypes.POINTER(ctypes.c_double))]


_LIBS: dict = {}


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the in-tree engine library (or, with CHECKED_LIB_PATH, its
    bounds-checked build); raises if it was not built."""
    if path in _LIBS:
        return _LIBS[path]
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run `python -m raptor_gb300.build` "
                                "(the engine has no CPU fallback)")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    D = ctypes.c_double
    lib.raptor_gpu_init.argtypes = [P(Options), P(ctypes.c_void_p)]
    lib.raptor_gpu_destroy.argtypes = [ctypes.c_void_p]
    lib.raptor_gpu_destroy.restype = None
    lib.raptor_gpu_last_error.argtypes = [ctypes.c_void_p]
    lib.raptor_gpu_last_error.restype = ctypes.c_char_p
    lib.raptor_gpu_upload_grid.argtypes = [ctypes.c_void_p, P(D), P(GridGeomC), P(ctypes.c_int)]
    lib.raptor_gpu_render.argtypes = [ctypes.c_void_p, P(ImageDesc), ctypes.c_int, ctypes.c_int, P(D), P(D)]
    lib.raptor_gpu_render_range.argtypes = [ctypes.c_void_p, P(ImageDesc), ctypes.c_int, ctypes.c_int,
                                            ctypes.c_longlong, ctypes.c_longlong, P(D), P(D)]
    lib.raptor_gpu_output_size.argtypes = [P(ImageDesc), ctypes.c_int]
    lib.raptor_gpu_output_size.restype = ctypes.c_longlong
    lib.raptor_gpu_spectrum_size.argtypes = [P(ImageDesc), ctypes.c_int]
    lib.raptor_gpu_spectrum_size.restype = ctypes.c_longlong
    lib.raptor_gpu_get_stats.argtypes = [ctypes.c_void_p, P(Stats)]
    lib.raptor_gpu_vjp.argtypes = [ctypes.c_void_p, P(ImageDesc), ctypes.c_int, P(D), P(D), P(GradC)]
    lib.raptor_gpu_vjp_range.argtypes = [ctypes.c_void_p, P(ImageDesc), ctypes.c_int, ctypes.c_longlong,
                                         ctypes.c_longlong, P(D), P(D), P(GradC)]
    lib.raptor_gpu_trace_ray.argtypes = [ctypes.c_void_p, P(ImageDesc), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         P(D), P(ctypes.c_int)]
    _LIBS[path] = lib
    return lib


def _dp(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def image_desc(width, height, freqs: Sequence[float], grid: int = 0, inclination=60.0, cam_size_x=40.0,
               cam_size_y=40.0, mbh=8.9505e39, m_unit=1e19, r_high=3.0, r_low=3.0, stepsize=0.05,
               integrator=RK4, camera=0, emission=EMISSION_THERMAL) -> ImageDesc:
    """camera: CAM_LINEAR (0, the reference's default) or CAM_LOG (1);
    emission: EMISSION_THERMAL (0, the reference's) or EMISSION_KAPPA (1,
    the kappa = 3.5 fits, in every form and the adjoints)."""
    freqs = list(np.atleast_1d(freqs).astype(float))
    if not 1 <= len(freqs) <= RAPTOR_MAX_FREQS:
        raise ValueError(f"1..{RAPTOR_MAX_FREQS} frequencies per image")
    fa = (ctypes.c_double * RAPTOR_MAX_FREQS)(*(freqs + [0.0] * (RAPTOR_MAX_FREQS - len(freqs))))
    return ImageDesc(width, height, cam_size_x, cam_size_y, inclination, mbh, m_unit, r_high, r_low,
                     stepsize, integrator, grid, len(freqs), fa, camera, emission)


class Engine:
    """One engine context on one CUDA device."""

    def __init__(self, device: int = 0, block_size: int = 0, blocks_per_sm: int = 0, refill_interval: int = 0,
                 autotune: int = 0, use_graph: int = 0, no_sample_pool: int = 0, checked: bool = False,
                 vjp_tape: int = 0):
        """checked: use the bounds-checked build of the library, where a
        failed device-side index check fails the call with RAPTOR_ERR_DEVICE.
        vjp_tape: records per lane of the one-pass adjoint's tape (0: 2048;
        -1: the two-pass VJP), raptor_gpu_options.vjp_tape."""
        self.lib = load(CHECKED_LIB_PATH if checked else LIB_PATH)
        opt = Options(device, block_size, blocks_per_sm, refill_interval, autotune, use_graph, no_sample_pool,
                      vjp_tape)
        h = ctypes.c_void_p()
        rc = self.lib.raptor_gpu_init(ctypes.byref(opt), ctypes.byref(h))
        if rc != 0:
            raise EngineError(rc, "raptor_gpu_init failed (no usable sm_103 device?)")
        self.h = h
        self.grids = {}
        self.last_status = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.raptor_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        """Negative statuses raise EngineError; positive ones (warnings, the
        results complete) issue an EngineWarning.  The status is kept in
        last_status."""
        self.last_status = rc
        if rc < 0:
            raise EngineError(rc, self.lib.raptor_gpu_last_error(self.h).decode())
        if rc > 0:
            warnings.warn(EngineWarning(f"{STATUS.get(rc, rc)}: {self.lib.raptor_gpu_last_error(self.h).decode()}"),
                          stacklevel=3)

    def upload_grid(self, geom: GridGeom, prims: np.ndarray, grid_id: int = -1) -> int:
        prims = np.ascontiguousarray(prims, dtype=np.float64)
        if prims.shape != (8, geom.n1, geom.n2):
            raise ValueError(f"prims must be [8][{geom.n1}][{geom.n2}]")
        g = GridGeomC(geom.n1, geom.n2, geom.startx1, geom.startx2, geom.dx1, geom.dx2, geom.a, geom.hslope,
                      geom.R0)
        gid = ctypes.c_int(grid_id)
        self._check(self.lib.raptor_gpu_upload_grid(self.h, _dp(prims), ctypes.byref(g), ctypes.byref(gid)))
        self.grids[gid.value] = geom
        return gid.value

    def render(self, imgs, precision=PREC_FP64, ray_begin=None, ray_count=None, out=None, spectrum=None):
        """Render a batch; returns (I [sum W*H*F], spectrum [sum F])."""
        if isinstance(imgs, ImageDesc):
            imgs = [imgs]
        arr = (ImageDesc * len(imgs))(*imgs)
        n_out = self.lib.raptor_gpu_output_size(arr, len(imgs))
        n_spec = self.lib.raptor_gpu_spectrum_size(arr, len(imgs))
        if out is None:
            out = np.empty(n_out)
        if spectrum is None:
            spectrum = np.empty(n_spec)
        assert out.size >= n_out and spectrum.size >= n_spec
        if ray_begin is None:
            rc = self.lib.raptor_gpu_render(self.h, arr, len(imgs), precision, _dp(out), _dp(spectrum))
        else:
            rc = self.lib.raptor_gpu_render_range(self.h, arr, len(imgs), precision, ray_begin,
                                                  ray_count if ray_count is not None else -1, _dp(out),
                                                  _dp(spectrum))
        self._check(rc)
        return out, spectrum

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.raptor_gpu_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def trace_ray(self, img: ImageDesc, pixel: int, precision=PREC_FP64, max_records=4096) -> np.ndarray:
        """Per-step states of one ray, [n][16] (see raptor_gpu_trace_ray)."""
        rec = np.zeros((max_records, TRACE_WIDTH))
        n = ctypes.c_int(0)
        self._check(self.lib.raptor_gpu_trace_ray(self.h, ctypes.byref(img), precision, pixel, max_records,
                                                  _dp(rec), ctypes.byref(n)))
        return rec[:n.value]

    def vjp(self, img: ImageDesc, dL_dI: np.ndarray, precision=PREC_FP64, want_fields=True, ray_begin=None,
            ray_count=None):
        """Image and gradients of L given dL/dI (raptor_gpu_vjp: the image the
        one-pass adjoint renders, or the forward render in two passes); with
        ray_begin / ray_count, of those rays only (raptor_gpu_vjp_range)."""
        geom = self.grids[img.grid]
        dldi = np.ascontiguousarray(dL_dI, dtype=np.float64)
        out = np.empty(img.width * img.height * img.n_freq)
        d_rho = np.zeros(geom.n1 * geom.n2) if want_fields else None
        d_u = np.zeros(geom.n1 * geom.n2) if want_fields else None
        d_th = np.zeros(geom.n1 * geom.n2) if want_fields else None
        g = GradC(0, 0, 0, 0, _dp(d_rho), _dp(d_u), _dp(d_th))
        if ray_begin is None:
            self._check(self.lib.raptor_gpu_vjp(self.h, ctypes.byref(img), precision, _dp(dldi), _dp(out),
                                                ctypes.byref(g)))
        else:
            self._check(self.lib.raptor_gpu_vjp_range(
                self.h, ctypes.byref(img), precision, ray_begin,
                ray_count if ray_count is not None else img.width * img.height - ray_begin, _dp(dldi), _dp(out),
                ctypes.byref(g)))
        res = dict(d_m_unit=g.d_m_unit, d_r_high=g.d_r_high, d_r_low=g.d_r_low, d_inclination=g.d_inclination)
        if want_fields:
            res["d_rho"] = d_rho.reshape(geom.n1, geom.n2)
            res["d_u"] = d_u.reshape(geom.n1, geom.n2)
            res["d_lnthetae"] = d_th.reshape(geom.n1, geom.n2)
        return out, res
