"""ctypes wrapper of the C restatement (oracle/raptor_port.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker / baseline, never by the engine.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_port", "libraptor_port.so")
_LIB = None


class PortScene(ctypes.Structure):
    _fields_ = [("n1", ctypes.c_int), ("n2", ctypes.c_int),
                ("startx1", ctypes.c_double), ("startx2", ctypes.c_double),
                ("dx1", ctypes.c_double), ("dx2", ctypes.c_double),
                ("a", ctypes.c_double), ("hslope", ctypes.c_double), ("R0", ctypes.c_double),
                ("prims", ctypes.POINTER(ctypes.c_double)),
                ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("cam_size_x", ctypes.c_double), ("cam_size_y", ctypes.c_double),
                ("inclination", ctypes.c_double), ("stepsize", ctypes.c_double),
                ("mbh", ctypes.c_double), ("m_unit", ctypes.c_double),
                ("r_high", ctypes.c_double), ("r_low", ctypes.c_double),
                ("integrator", ctypes.c_int), ("camera", ctypes.c_int), ("emission", ctypes.c_int)]


class PortRayStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("rt_samples", ctypes.c_int), ("rt_calls", ctypes.c_int),
                ("reason", ctypes.c_int), ("kk", ctypes.c_double)]


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def load() -> ctypes.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "raptor_port.c")):
        build()
    lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_LOCAL)
    D = ctypes.c_double
    P = ctypes.POINTER
    S = P(PortScene)
    lib.port_render.argtypes = [S, P(ctypes.c_int), ctypes.c_int, P(D), ctypes.c_int, P(D),
                                P(PortRayStats), ctypes.c_int]
    lib.port_render.restype = ctypes.c_int
    for name in ("port_metric_dd", "port_metric_uu", "port_connection"):
        getattr(lib, name).argtypes = [S, P(D), P(D)]
        getattr(lib, name).restype = None
    lib.port_init_photon.argtypes = [S, D, D, P(D)]
    lib.port_camera_x2.argtypes = [S]
    lib.port_camera_x2.restype = D
    lib.port_j_thsynch.argtypes = [D, D, D, D, D]
    lib.port_j_thsynch.restype = D
    lib.port_a_th.argtypes = [D, D, D]
    lib.port_a_th.restype = D
    for name in ("port_j_kappa", "port_a_kappa"):
        getattr(lib, name).argtypes = [D, D, D, D, D]
        getattr(lib, name).restype = D
    lib.port_hyp2f1.argtypes = [D, D, D, D]
    lib.port_hyp2f1.restype = D
    lib.port_fluid.argtypes = [S, P(D), P(D)]
    lib.port_fluid.restype = ctypes.c_int
    lib.port_trace_ray.argtypes = [S, ctypes.c_int, P(D), ctypes.c_int, ctypes.c_int, P(D)]
    lib.port_trace_ray.restype = ctypes.c_int
    _LIB = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Scene:
    """A grid plus camera/model scalars, as one port_scene."""

    def __init__(self, geom, prims, width, height, cam_size_x=40.0, cam_size_y=40.0,
                 inclination=60.0, stepsize=0.05, mbh=8.9505e39, m_unit=1e19, r_high=3.0,
                 r_low=3.0, integrator=4, camera=0, emission=0):
        self.prims = np.ascontiguousarray(prims, dtype=np.float64)
        assert self.prims.shape == (8, geom.n1, geom.n2)
        self.c = PortScene(geom.n1, geom.n2, geom.startx1, geom.startx2, geom.dx1, geom.dx2,
                           geom.a, geom.hslope, geom.R0, _dp(self.prims), width, height,
                           cam_size_x, cam_size_y, inclination, stepsize, mbh, m_unit,
                           r_high, r_low, integrator, camera, emission)
        self.lib = load()

    def render(self, freqs, pixels=None, nthreads=0, with_stats=False):
        freqs = np.atleast_1d(np.asarray(freqs, dtype=np.float64))
        if pixels is None:
            pixels = np.arange(self.c.width * self.c.height, dtype=np.int32)
        pix = np.ascontiguousarray(pixels, dtype=np.int32)
        out = np.zeros((len(pix), len(freqs)))
        stats = (PortRayStats * max(len(pix), 1))() if with_stats else None
        t0 = time.perf_counter()
        rc = self.lib.port_render(ctypes.byref(self.c), pix.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                  len(pix), _dp(freqs), len(freqs), _dp(out), stats, nthreads)
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(f"port_render failed ({rc})")
        if with_stats:
            st = np.ctypeslib.as_array(stats)[:len(pix)]
            return out, dt, st
        return out, dt

    def trace_ray(self, pixel, freqs, cap=4096):
        freqs = np.atleast_1d(np.asarray(freqs, dtype=np.float64))
        rec = np.zeros((cap, 16))
        n = self.lib.port_trace_ray(ctypes.byref(self.c), pixel, _dp(freqs), len(freqs), cap, _dp(rec))
        if n < 0:
            raise RuntimeError("port_trace_ray failed")
        return rec[:n]

    def metric_dd(self, X):
        g = np.zeros(16)
        self.lib.port_metric_dd(ctypes.byref(self.c), _dp(np.ascontiguousarray(X, dtype=np.float64)), _dp(g))
        return g.reshape(4, 4)

    def metric_uu(self, X):
        g = np.zeros(16)
        self.lib.port_metric_uu(ctypes.byref(self.c), _dp(np.ascontiguousarray(X, dtype=np.float64)), _dp(g))
        return g.reshape(4, 4)

    def connection(self, X):
        G = np.zeros(64)
        self.lib.port_connection(ctypes.byref(self.c), _dp(np.ascontiguousarray(X, dtype=np.float64)), _dp(G))
        return G.reshape(4, 4, 4)

    def init_photon(self, alpha, beta):
        ph = np.zeros(8)
        self.lib.port_init_photon(ctypes.byref(self.c), alpha, beta, _dp(ph))
        return ph

    def camera_x2(self):
        return self.lib.port_camera_x2(ctypes.byref(self.c))

    def fluid(self, X):
        out = np.zeros(12)
        ok = self.lib.port_fluid(ctypes.byref(self.c), _dp(np.ascontiguousarray(X, dtype=np.float64)), _dp(out))
        return ok, out
