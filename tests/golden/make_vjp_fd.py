"""Finite-difference gradients of an image loss from the reference build
(oracle/_ref, IEEE semantics), for checking raptor_gpu_vjp.

    python tests/golden/make_vjp_fd.py [--threads 8] [--workload adjoint256|5freq512]

adjoint256 (the adjoint workload): 256x256 image, 230 GHz, i = 60 deg,
a = 0.9375 torus at 256x256, M_unit = 1e19, R_high = R_low = 3, RK4 eps
0.05; 32 cells.  5freq512, the large differentiable batch reduced in rays
(its five frequencies 86/140/230/345/690 GHz and its 512x512 torus, on a
128x128 image): 8 cells, written to tests/golden/vjp_fd_5freq_512.npz.
Loss L = 1/2 sum (O - O_target)^2 over the nu^3-scaled image O, the target
rendered at M_unit x 1.3, R_high = R_low = 4, i = 62 deg.  Central differences
with relative step h = 1e-4 on M_unit, R_high, R_low, the inclination, and on
rho and u of 32 seeded cells inside the torus.  For the four scalars the
differences at h and h/2 are also Richardson-extrapolated,
(4 D(h/2) - D(h)) / 3.  The inclination also gets plain central differences
at h = 1e-6 and 1e-7: the image loss is only piecewise smooth in the
inclination (clamps, min() in the step size, cell-index changes along every
ray), so its difference quotient at h = 1e-4 sits ~0.7 % from the derivative
and approaches it only as h shrinks.  Writes tests/golden/vjp_fd_256.npz;
--parts selects what to (re)compute, merged into an existing file.
"""
from __future__ import annotations

import argparse
import ctypes
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from raptor_gb300 import harm, synth  # noqa: E402
from tests.golden.make_golden import quiet  # noqa: E402

BASE = dict(m_unit=1e19, r_high=3.0, r_low=3.0, incl=60.0)
TARGET = dict(m_unit=1.3e19, r_high=4.0, r_low=4.0, incl=62.0)
REL_H = 1e-4
# workload: grid size, image size, frequencies, cells, output file
WORKLOADS = {
    "adjoint256": dict(n=256, w=256, freqs=(230e9,), n_cells=32, out="vjp_fd_256.npz"),
    "5freq512": dict(n=512, w=128, freqs=(86e9, 140e9, 230e9, 345e9, 690e9), n_cells=8, out="vjp_fd_5freq_512.npz"),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="adjoint256")
    ap.add_argument("--parts", default="scalars,cells,incl_small")
    a = ap.parse_args()
    cfg = WORKLOADS[a.workload]
    N, W, FREQS, N_CELLS = cfg["n"], cfg["w"], cfg["freqs"], cfg["n_cells"]
    H = W
    parts = set(a.parts.split(","))
    dst = os.path.join(ROOT, "tests", "golden", cfg["out"])
    res = dict(np.load(dst)) if os.path.exists(dst) else {}
    tmp = tempfile.mkdtemp(prefix="rgv_", dir="/tmp")
    d = synth.make_torus(n1=N, n2=N)
    path = os.path.join(tmp, "t.dump")
    harm.write_dump(path, d)
    model = harm.ModelIn(IMG_WIDTH=W, IMG_HEIGHT=H, FREQ_MIN=FREQS[0], FREQ_MAX=FREQS[0], STEPSIZE=0.05)
    pix = np.arange(W * H, dtype=np.int32)
    lib = ref.load(N, N, "RK4")
    lib.ref_scale_prim.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]

    def render(prm, scale=None):
        """[W*H][F] image, frequency fastest (one reference pass per
        frequency: the reference build renders one at a time)."""
        with quiet():
            s = ref.RefSession(path, model, prm["m_unit"], prm["incl"], prm["r_high"], prm["r_low"], 0.0,
                               n1=N, n2=N, workdir=tmp)
            if scale:
                assert lib.ref_scale_prim(*scale) == 0
            img = np.stack([s.render_pixels(pix, f, a.threads)[0] for f in FREQS], axis=1)
        return img if len(FREQS) > 1 else img[:, 0]

    target = render(TARGET)

    def loss(prm, scale=None):
        o = render(prm, scale)
        return 0.5 * float(np.sum((o - target) ** 2))

    L0 = loss(BASE)
    res["L0"] = np.array([L0])
    res["rel_h"] = np.array([REL_H])
    if "incl_small" in parts:
        for rel in (1e-6, 1e-7):
            h = rel * BASE["incl"]
            op = render(dict(BASE, incl=BASE["incl"] + h))
            om = render(dict(BASE, incl=BASE["incl"] - h))
            # L(+) - L(-) without subtracting two large sums
            res[f"fd_incl_{rel:g}"] = np.array([0.5 * np.sum((op - om) * (op + om - 2 * target)) / (2 * h)])
            print("incl", rel, res[f"fd_incl_{rel:g}"][0], flush=True)
    fd, rich = {}, {}
    for key in (("m_unit", "r_high", "r_low", "incl") if "scalars" in parts else ()):
        diffs = []
        for rel in (REL_H, REL_H / 2):
            h = rel * BASE[key]
            lp = loss(dict(BASE, **{key: BASE[key] + h}))
            lm = loss(dict(BASE, **{key: BASE[key] - h}))
            diffs.append((lp - lm) / (2 * h))
        fd[key] = diffs[0]
        rich[key] = (4 * diffs[1] - diffs[0]) / 3
        short = "incl" if key == "incl" else key
        res[f"fd_{short}"] = np.array([fd[key]])
        res[f"rich_{short}"] = np.array([rich[key]])
        print(key, fd[key], rich[key], flush=True)
    rng = np.random.default_rng(2024)
    cand = np.argwhere(d.prims[0] > 0.2)
    cells = cand[rng.choice(len(cand), N_CELLS, replace=False)]
    fd_rho = np.zeros(N_CELLS)
    fd_u = np.zeros(N_CELLS)
    for c, (i, j) in enumerate(cells if "cells" in parts else ()):
        for q, arr in ((0, fd_rho), (1, fd_u)):
            v = d.prims[q, i, j]
            lp = loss(BASE, (q, int(i), int(j), 1 + REL_H))
            lm = loss(BASE, (q, int(i), int(j), 1 - REL_H))
            arr[c] = (lp - lm) / (2 * REL_H * v)
        print("cell", i, j, fd_rho[c], fd_u[c], flush=True)
    if "cells" in parts:
        res.update(cells=cells, fd_rho=fd_rho, fd_u=fd_u)
    res["freqs"] = np.array(FREQS)
    res["image"] = np.array([W, H, N])
    np.savez_compressed(dst, **res)


if __name__ == "__main__":
    main()
