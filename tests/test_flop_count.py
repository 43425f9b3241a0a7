"""Pins the algorithmic FP64 work per unit (raptor_gb300/workload.py) by
counting operations in the oracle's restatement of the reference."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from raptor_gb300 import synth, workload

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(os.path.dirname(HERE), "oracle")


@pytest.fixture(scope="module")
def counting():
    subprocess.run(["make", "-s", "-C", ORACLE, "count"], check=True)
    lib = ctypes.CDLL(os.path.join(ORACLE, "_port", "libraptor_port_count.so"))
    lib.port_flop_buckets.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]
    return lib


def run(lib, torus, nf, rk, incl=60.0, n=12):
    from oracle import port
    sc = port.Scene(torus.geom, torus.prims, n, n, inclination=incl, integrator=rk)
    freqs = np.array([230e9, 86e9, 345e9, 140e9, 690e9, 43e9, 1e12, 5e11][:nf])
    pix = np.arange(n * n, dtype=np.int32)
    out = np.zeros((n * n, nf))
    stats = (port.PortRayStats * (n * n))()
    b = (ctypes.c_ulonglong * 8)()
    lib.port_flop_buckets(b, 1)
    lib.port_render.argtypes = port.load().port_render.argtypes
    P = ctypes.POINTER(ctypes.c_double)
    lib.port_render(ctypes.byref(sc.c), pix.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n * n,
                    freqs.ctypes.data_as(P), nf, out.ctypes.data_as(P), stats, 1)
    lib.port_flop_buckets(b, 1)
    st = np.ctypeslib.as_array(stats)
    escaped = int(np.sum(st["reason"] == 2))
    return list(b), int(st["steps"].sum()), int(st["rt_samples"].sum()), escaped, n * n


@pytest.mark.parametrize("rk,per_step", [(4, workload.FLOP_RK4_STEP), (2, workload.FLOP_RK2_STEP)])
def test_flops_per_step_and_setup(counting, torus64, rk, per_step):
    b, steps, samples, escaped, rays = run(counting, torus64, 1, rk)
    assert b[0] == workload.FLOP_RAY_SETUP * rays
    # a ray that escapes outward breaks before the two trailing exp(x1)
    assert b[1] == per_step * steps - 2 * escaped


def test_flops_per_sample(counting, torus64):
    per = {}
    for nf in (1, 3, 8):
        b, steps, samples, _, _ = run(counting, torus64, nf, 4)
        per[nf] = b[3] / samples
    slope = (per[8] - per[1]) / 7
    assert slope == pytest.approx(workload.FLOP_SAMPLE_PER_FREQ, abs=0.5)
    # a few samples return j = 0 early (j_nu.c:138-147), so the mean sits just below
    assert workload.FLOP_SAMPLE_BASE + workload.FLOP_SAMPLE_PER_FREQ - 2 < per[1] <= \
        workload.FLOP_SAMPLE_BASE + workload.FLOP_SAMPLE_PER_FREQ
