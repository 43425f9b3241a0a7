"""Parity helpers shared by the tests (tolerances are stated here)."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def pixel_errors(got, ref):
    """Per-pixel relative error; a pixel that is zero in the reference counts
    as exact only if it is zero here too."""
    got = np.asarray(got, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    err = np.zeros_like(ref)
    nz = ref != 0
    err[nz] = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])
    err[~nz] = np.where(got[~nz] == 0, 0.0, np.inf)
    return err


# FP64 parity bar: per-pixel relative error <= 1e-6 except for at most 0.1% of
# pixels (rays grazing the critical curve, where ulp differences between libm
# implementations grow through many orbits), and total flux within 1e-6.
PIXEL_RTOL = 1e-6
GRAZING_FRACTION = 1e-3
FLUX_RTOL_FP64 = 1e-6
# mixed form (FP64 geodesic, FP32 transfer): total flux within 1e-4
FLUX_RTOL_MIXED = 1e-4


def assert_fp64_parity(got, ref, label=""):
    err = pixel_errors(got, ref)
    n_bad = int(np.sum(err > PIXEL_RTOL))
    allowed = int(np.floor(GRAZING_FRACTION * err.size))
    flux_err = abs(np.sum(got) - np.sum(ref)) / abs(np.sum(ref))
    msg = (f"{label}: {n_bad}/{err.size} pixels above {PIXEL_RTOL:g} (allowed {allowed}), "
           f"max {np.max(err):.3e}, median {np.median(err):.3e}, flux err {flux_err:.3e}, "
           f"worst pixels {np.argsort(err)[-4:][::-1].tolist()}")
    out_dir = os.environ.get("RAPTOR_ARTIFACT_DIR")  # where to keep the arrays of a failed comparison
    if (n_bad > allowed or flux_err > FLUX_RTOL_FP64) and out_dir and os.path.isdir(out_dir):
        safe = "".join(ch if ch.isalnum() else "_" for ch in label)
        np.savez(os.path.join(out_dir, f"parity_fail_{safe}.npz"), got=got, ref=ref)
    assert n_bad <= allowed, msg
    assert flux_err <= FLUX_RTOL_FP64, msg
    return dict(n_bad=n_bad, max=float(np.max(err)), median=float(np.median(err)), flux=float(flux_err))
