"""Generate the golden fixtures under tests/golden/ from the reference RAPTOR
build (oracle/_ref, compiled from the reference's own C sources).

Run here, where the reference sources are mounted:

    python tests/golden/make_golden.py [--large]

Every input is the seeded synthetic torus of raptor_gb300.synth (written as
a HARM ASCII dump and read by the reference's own init_harm_data), so the
fixtures hold only parameters and reference outputs.  --large adds the
1024x1024 subsample fixture on a 512x512 torus (minutes on 8 cores).
"""
from __future__ import annotations

import argparse
import contextlib
import ctypes
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from raptor_gb300 import harm, synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# (name, torus size, width, height, inclination, freq, integrator, stepsize, m_unit, r_high, r_low)
SMALL_IMAGES = [
    ("g64_i60_rk4", 32, 32, 60.0, 230e9, "RK4", 0.05, 1e19, 3.0, 3.0),
    ("g64_i17_rk4", 24, 24, 17.0, 230e9, "RK4", 0.05, 1e19, 3.0, 3.0),
    ("g64_i120_rk4_86", 16, 16, 120.0, 86e9, "RK4", 0.05, 3e19, 4.0, 1.0),
    ("g64_i60_rk2", 16, 16, 60.0, 345e9, "RK2", 0.05, 1e19, 3.0, 3.0),
    ("g64_i35_rk4_odd", 15, 13, 35.0, 230e9, "RK4", 0.1, 1e19, 3.0, 3.0),
]


@contextlib.contextmanager
def quiet():
    """Silence the reference's stdout/stderr prints (file-descriptor level)."""
    sys.stdout.flush()
    sys.stderr.flush()
    saved = os.dup(1), os.dup(2)
    dn = os.open(os.devnull, os.O_WRONLY)
    os.dup2(dn, 1)
    os.dup2(dn, 2)
    try:
        yield
    finally:
        # flush C stdio's buffers while they still point at /dev/null
        ctypes.CDLL(None).fflush(None)
        os.dup2(saved[0], 1)
        os.dup2(saved[1], 2)
        os.close(dn)
        os.close(saved[0])
        os.close(saved[1])


# log-polar camera images on the 256x256 torus: name, W, H, inclination, frequency, integrator
LOGCAM_IMAGES = [
    ("log_i60_rk4", 64, 48, 60.0, 230e9, "RK4"),
    ("log_i17_rk2", 40, 33, 17.0, 345e9, "RK2"),
]


# one image per dump of the batched configuration: name, W, H, inclination, frequency, integrator, M_unit
BATCH_DUMP_IMAGES = [
    ("a05_i120_345", 48, 40, 120.0, 345e9, "RK4", 3e18),
    ("a09375_i25_86", 40, 48, 25.0, 86e9, "RK4", 5e19),
]


# images of the R0 = 0.3 dump: name, W, H, inclination, frequency, integrator
R0_IMAGES = [
    ("r0_i50_rk4", 32, 28, 50.0, 230e9, "RK4"),
    ("r0_i130_rk2", 24, 24, 130.0, 345e9, "RK2"),
]


def r0_dump():
    """The 64x64 torus with its header's R0 set to 0.3."""
    import dataclasses
    d = synth.make_torus(n1=64, n2=64)
    return dataclasses.replace(d, geom=dataclasses.replace(d.geom, R0=0.3))


def prim_checksum(prims):
    return np.array([np.sum(np.abs(p), dtype=np.float64) for p in prims])


def torus_and_dump(n, tmp, **kw):
    d = synth.make_torus(n1=n, n2=n, **kw)
    path = os.path.join(tmp, f"torus{n}.dump")
    harm.write_dump(path, d)
    return d, path


def ref_image(dump_path, n, w, h, incl, freq, rk, eps, m_unit, rh, rl, pixels=None, threads=0, cam="linear"):
    model = harm.ModelIn(MBH=8.9505e39, M_UNIT=m_unit, IMG_WIDTH=w, IMG_HEIGHT=h, CAM_SIZE_X=40.0,
                         CAM_SIZE_Y=40.0, FREQ_MIN=freq, FREQ_MAX=freq, STEPSIZE=eps)
    with quiet():
        s = ref.RefSession(dump_path, model, m_unit, incl, rh, rl, 0.0, rk=rk, n1=n, n2=n, cam=cam)
        if pixels is None:
            img, spec, dt = s.render_serial(freq)
            return img, spec, dt
        vals, dt = s.render_pixels(pixels, freq, threads)
        return vals, None, dt


def kats(dump_path, n):
    """Function-level known answers straight from the reference's functions."""
    lib = ref.load(n, n, "RK4")
    model = harm.ModelIn(IMG_WIDTH=16, IMG_HEIGHT=16)
    with quiet():
        ref.RefSession(dump_path, model, 1e19, 60.0, 3.0, 3.0, 0.0, n1=n, n2=n)
    D = ctypes.c_double
    P = ctypes.POINTER(D)
    for fn in ("metric_dd", "metric_uu", "connection_udd"):
        getattr(lib, fn).argtypes = [P, P]
        getattr(lib, fn).restype = None
    lib.emission_coeff_THSYNCH.argtypes = [D, D, D, D, D]
    lib.emission_coeff_THSYNCH.restype = D
    lib.absorption_coeff_TH.argtypes = [D, D, D]
    lib.absorption_coeff_TH.restype = D
    lib.get_fluid_params.argtypes = [P, P, P, P, P, P, P, P, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, P, P]
    lib.get_fluid_params.restype = ctypes.c_int
    p_grid = ctypes.c_void_p.in_dll(lib, "p")

    rng = np.random.default_rng(7)
    npt = 24
    X = np.zeros((npt, 4))
    X[:, 1] = rng.uniform(np.log(1.5), np.log(40.0), npt)
    X[:, 2] = rng.uniform(0.02, 0.98, npt)
    gdd = np.zeros((npt, 16))
    guu = np.zeros((npt, 16))
    gam = np.zeros((npt, 64))
    for k in range(npt):
        x = np.ascontiguousarray(X[k])
        out = np.zeros(16)
        lib.metric_dd(x.ctypes.data_as(P), out.ctypes.data_as(P))
        gdd[k] = out
        out = np.zeros(16)
        lib.metric_uu(x.ctypes.data_as(P), out.ctypes.data_as(P))
        guu[k] = out
        out = np.zeros(64)
        lib.connection_udd(x.ctypes.data_as(P), out.ctypes.data_as(P))
        gam[k] = out

    # emissivity / absorptivity lattice (B, cos pitch, Theta_e, nu, n_e)
    lat = []
    for B in (0.3, 10.0, 300.0):
        for cp in (-0.9, 0.1, 0.7):
            for th in (0.5, 5.0, 60.0):
                for nu in (8.6e10, 2.3e11, 3.45e12):
                    for ne in (1e4, 1e7):
                        lat.append((B, cp, th, nu, ne))
    lat = np.array(lat)
    jv = np.array([lib.emission_coeff_THSYNCH(*row) for row in lat])
    av = np.array([lib.absorption_coeff_TH(jv[i], lat[i, 3], lat[i, 2]) for i in range(len(lat))])

    # fluid parameters at grid-interior points
    fx = np.zeros((npt, 4))
    fx[:, 1] = rng.uniform(np.log(5.0), np.log(30.0), npt)
    fx[:, 2] = rng.uniform(0.2, 0.8, npt)
    fluid = np.zeros((npt, 12))
    fok = np.zeros(npt, dtype=np.int32)
    for k in range(npt):
        x = np.ascontiguousarray(fx[k])
        ne, th, B, beta, bern = (D(), D(), D(), D(), D())
        bcon = np.zeros(4)
        ucon = np.zeros(4)
        inv = ctypes.c_int()
        gc = np.zeros(16)
        gn = np.zeros(16)
        ok = lib.get_fluid_params(x.ctypes.data_as(P), ctypes.byref(ne), ctypes.byref(th), ctypes.byref(B),
                                  ctypes.byref(beta), ctypes.byref(bern), bcon.ctypes.data_as(P),
                                  ucon.ctypes.data_as(P), ctypes.byref(inv), p_grid, gc.ctypes.data_as(P),
                                  gn.ctypes.data_as(P))
        fok[k] = ok
        fluid[k] = [ne.value, th.value, B.value, beta.value, *ucon, *bcon]
    return dict(kat_X=X, kat_gdd=gdd, kat_guu=guu, kat_gamma=gam, kat_lattice=lat, kat_j=jv, kat_a=av,
                kat_fluid_X=fx, kat_fluid=fluid, kat_fluid_ok=fok)


def ref_output_files(dump, img, spec, w=32, h=32, cam="linear", dst_name="ref_output"):
    """The reference's own output_files (core.c:154-200) for a w x h image of
    the 64x64 torus, run in a scratch directory with relative file names,
    copied to tests/golden/<dst_name>/."""
    import shutil
    tmp = tempfile.mkdtemp(prefix="rgo_out_", dir="/tmp")
    harm.write_dump(os.path.join(tmp, "torus64.dump"), dump)
    model = harm.ModelIn(IMG_WIDTH=w, IMG_HEIGHT=h, FREQ_MIN=230e9, FREQ_MAX=230e9, STEPSIZE=0.05)
    cwd = os.getcwd()
    os.chdir(tmp)
    try:
        lib = ref.load(64, 64, "RK4", cam=cam)
        lib.ref_output_files.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double]
        with quiet():
            ref.RefSession("torus64.dump", model, 1e19, 60.0, 3.0, 3.0, 1.0, n1=64, n2=64, workdir=tmp, cam=cam)
            field = np.ascontiguousarray(img, dtype=np.float64)
            lib.ref_output_files(field.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), spec, 230e9)
    finally:
        os.chdir(cwd)
    dst = os.path.join(OUT, dst_name)
    os.makedirs(dst, exist_ok=True)
    for fn in os.listdir(os.path.join(tmp, "output")):
        shutil.copy(os.path.join(tmp, "output", fn), os.path.join(dst, fn))
    model.write(os.path.join(dst, "model.in"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--large", action="store_true")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--parts", default="small,256,logcam,batchdumps,r0",
                    help="comma list of fixture groups to write: small, 256, logcam, batchdumps, r0")
    a = ap.parse_args()
    parts = set(a.parts.split(","))
    tmp = tempfile.mkdtemp(prefix="rgg_", dir="/tmp")

    if "r0" in parts:
        # a non-zero MKS radial offset: the 64x64 torus's cells read under a
        # header with R0 = 0.3 (r = R0 + exp(x1) in the metric and the
        # connection, metric.c:94-137,538-638); the inputs need not be a
        # physical solution for parity, only the same on both sides
        d64 = r0_dump()
        path = os.path.join(tmp, "torus64_r0.dump")
        harm.write_dump(path, d64)
        out = dict(prim_checksum=prim_checksum(d64.prims), R0=np.array([d64.geom.R0]))
        for (name, w, h, incl, freq, rk) in R0_IMAGES:
            img, spec, dt = ref_image(path, 64, w, h, incl, freq, rk, 0.05, 1e19, 3.0, 3.0)
            out[f"{name}_img"] = img
            out[f"{name}_spec"] = np.array([spec])
            out[f"{name}_params"] = np.array([w, h, incl, freq, 4 if rk == "RK4" else 2, 0.05, 1e19, 3.0, 3.0])
            print(f"{name}: {dt:.2f} s, flux {spec:.6e}", flush=True)
        out["names"] = np.array([c[0] for c in R0_IMAGES])
        np.savez_compressed(os.path.join(OUT, "r0_g64.npz"), **out)

    if "batchdumps" in parts:
        # the two dumps of the batched configuration (a = 0.5 and a = 0.9375,
        # their own seeds), one image each with batch-like parameters
        from raptor_gb300 import workloads
        out = {}
        for k, d in enumerate(workloads.batch_dumps(256)):
            path = os.path.join(tmp, f"batch{k}.dump")
            harm.write_dump(path, d)
            name, w, h, incl, freq, rk, mu = BATCH_DUMP_IMAGES[k]
            img, spec, dt = ref_image(path, 256, w, h, incl, freq, rk, 0.05, mu, 3.0, 3.0)
            out[f"{name}_img"] = img
            out[f"{name}_spec"] = np.array([spec])
            out[f"{name}_params"] = np.array([w, h, incl, freq, 4 if rk == "RK4" else 2, 0.05, mu, 3.0, 3.0])
            out[f"{name}_prim_checksum"] = prim_checksum(d.prims)
            print(f"{name}: {dt:.2f} s, flux {spec:.6e}", flush=True)
        out["names"] = np.array([c[0] for c in BATCH_DUMP_IMAGES])
        np.savez_compressed(os.path.join(OUT, "batch_dumps_g256.npz"), **out)

    if "logcam" in parts:
        # the log-polar camera (LOG_IMPACT_CAM build): stock serial calculate_image,
        # whose post-scale (core.c:123-133) is part of what is pinned
        d256, p256 = torus_and_dump(256, tmp)
        out = dict(prim_checksum=prim_checksum(d256.prims))
        for (name, w, h, incl, freq, rk) in LOGCAM_IMAGES:
            img, spec, dt = ref_image(p256, 256, w, h, incl, freq, rk, 0.05, 1e19, 3.0, 3.0, cam="log")
            out[f"{name}_img"] = img
            out[f"{name}_spec"] = np.array([spec])
            out[f"{name}_params"] = np.array([w, h, incl, freq, 4 if rk == "RK4" else 2])
            print(f"{name}: {dt:.2f} s, flux {spec:.6e}", flush=True)
        out["names"] = np.array([c[0] for c in LOGCAM_IMAGES])
        np.savez_compressed(os.path.join(OUT, "logcam_g256.npz"), **out)
        # the reference's output files of a 32x24 log-polar image of the 64x64 torus
        d64, p64 = torus_and_dump(64, tmp)
        img, spec, _ = ref_image(p64, 64, 32, 24, 60.0, 230e9, "RK4", 0.05, 1e19, 3.0, 3.0, cam="log")
        ref_output_files(d64, img, spec, w=32, h=24, cam="log", dst_name="ref_output_logcam")
    if "small" not in parts:
        return

    # small grid: several images through the stock serial calculate_image
    d64, p64 = torus_and_dump(64, tmp)
    res = dict(torus_n=64, prim_checksum=prim_checksum(d64.prims))
    names = []
    for (name, w, h, incl, freq, rk, eps, mu, rh, rl) in SMALL_IMAGES:
        img, spec, dt = ref_image(p64, 64, w, h, incl, freq, rk, eps, mu, rh, rl)
        res[f"{name}_img"] = img
        res[f"{name}_spec"] = np.array([spec])
        res[f"{name}_params"] = np.array([w, h, incl, freq, 4 if rk == "RK4" else 2, eps, mu, rh, rl])
        names.append(name)
        print(f"{name}: {dt:.2f} s, flux {spec:.6e}", flush=True)
    res["names"] = np.array(names)
    res.update(kats(p64, 64))
    np.savez_compressed(os.path.join(OUT, "small_g64.npz"), **res)
    ref_output_files(d64, res["g64_i60_rk4_img"], res["g64_i60_rk4_spec"][0])

    if "256" not in parts:
        return
    # the 100x100 image on the 256x256 torus (RK4, eps 0.05, i = 60, 230 GHz)
    d256, p256 = torus_and_dump(256, tmp)
    img, spec, dt = ref_image(p256, 256, 100, 100, 60.0, 230e9, "RK4", 0.05, 1e19, 3.0, 3.0)
    print(f"config 100x100 on 256^2: {dt:.2f} s, flux {spec:.6e}", flush=True)
    np.savez_compressed(os.path.join(OUT, "img100_g256.npz"), img=img, spec=np.array([spec]),
                        prim_checksum=prim_checksum(d256.prims), serial_seconds=np.array([dt]),
                        params=np.array([100, 100, 60.0, 230e9, 4, 0.05, 1e19, 3.0, 3.0]))

    if a.large:
        d512, p512 = torus_and_dump(512, tmp)
        out = dict(prim_checksum=prim_checksum(d512.prims))
        W = 1024
        pix_all = np.arange(W * W, dtype=np.int32)
        sub = pix_all[::61]  # 17190 pixels, strided across every row
        for incl in (60.0, 17.0):
            full, _, dt = ref_image(p512, 512, W, W, incl, 230e9, "RK4", 0.05, 1e19, 3.0, 3.0, pixels=pix_all,
                                    threads=a.threads)
            print(f"1024^2 on 512^2, i={incl}: {dt:.1f} s (OpenMP), flux {full.sum():.6e}", flush=True)
            tag = f"i{int(incl)}"
            out[f"{tag}_sub_pixels"] = sub
            out[f"{tag}_sub_vals"] = full[sub]
            out[f"{tag}_spec"] = np.array([full.sum()])
            out[f"{tag}_omp_seconds"] = np.array([dt])
        np.savez_compressed(os.path.join(OUT, "img1024_g512_sub.npz"), **out)


if __name__ == "__main__":
    main()
