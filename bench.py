"""Benchmark: one 1024x1024 230 GHz image of the synthetic 512x512 torus
(a = 0.9375, inclination 60 deg, RK4, eps = 0.05) per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Engine arm: W untimed renders, then K timed renders of the FP64 form (the
headline; device time from CUDA events on the engine's stream, L2 flushed
between renders), K of the mixed form, and K end-to-end renders through the
C ABI with host buffers (grid upload from pinned memory + render + image
read-back inside the timed region).  Reference arm: the reference's CPU
algorithm (the reference build where it can be loaded, else the C port) on
all host cores, on a bounded pixel sample of the same image per step.
One JSON line on rank 0.  Under torchrun every rank renders its own image
(weak scaling, no data-path collective); times are maxed over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1024² image ms & ray-steps/s, mixed vs FP64 at ≤1e-4 flux err; VJP/fwd ratio"
W = H = 1024
GRID_N = 512
INCL = 60.0
FREQ = 230e9
EPS = 0.05
L2_FLUSH_BYTES = 512 << 20
NOMINAL_FP64_TFLOPS = 1.25
# ncu dram__bytes_read.sum + dram__bytes_write.sum of one FP64 ray-kernel
# (ray_kernel_pool<1>) launch of the 1024x1024 workload (17,052,160 + 0
# bytes; the algorithmic bytes are the 16.8 MB grid read once and the 8.4 MB
# image written once)
TRAFFIC_FP64_1024 = 17052160


# ncu smsp__sass_thread_inst_executed_op_{ffma,fadd,fmul}_pred_on.sum of one
# mixed-DF ray-kernel launch (ray_kernel_df<1>) on the 1024x1024 workload:
# the FP32 thread-instructions the double-float geodesic and the FP32 sample
# execute (8.176e11 FADD + 4.945e11 FFMA + 2.335e11 FMUL)
FP32_INST_DF_1024 = 1545619712704


def df_roofline(kernel_ms, peak_tinst):
    """The mixed-DF kernel against the FP32 pipe: FP32 thread-instructions
    per launch (ncu) over the kernel's CUDA-event time, against an FFMA
    throughput probe on the same GPU."""
    inst = FP32_INST_DF_1024 if (W, H, GRID_N) == (1024, 1024, 512) else None
    achieved = inst / (kernel_ms * 1e-3) / 1e12 if inst else None
    return {"bound": "fp32", "achieved": achieved, "peak": peak_tinst, "unit": "T FP32 thread-inst/s",
            "frac": achieved / peak_tinst if achieved and peak_tinst > 0 else None, "fp32_inst_per_launch": inst,
            "peak_source": "measured FFMA loop on this GPU (FP32 lanes: 152 SMs x 128 x clock)"}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # the samples go to RAPTOR_ARTIFACT_DIR when set, else to a scratch file
        out_dir = os.environ.get("RAPTOR_ARTIFACT_DIR") or tempfile.mkdtemp(prefix="raptor_clocks_")
        self.path = os.path.join(out_dir, f"clocks_rank{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        mx = max(r[1] for r in rows)
        load = [r for r in rows if r[0] > 0.5 * mx] or rows
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in load for i, v in enumerate(r[2]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def make_scene():
    from raptor_gb300 import synth
    return synth.make_torus(n1=GRID_N, n2=GRID_N, a=0.9375)


_REF_SESSION = {}


def _reference_session(dump):
    """The reference's stock (-Ofast, makefile:13-15) build set up on this
    dump through its own read_model / init_model / set_constants, or None
    where the reference cannot be built here (cached per process)."""
    from oracle import ref
    if "s" in _REF_SESSION:
        return _REF_SESSION["s"]
    sess = None
    if ref.available(GRID_N, GRID_N, opt="stock"):
        try:
            from raptor_gb300 import harm
            from tests.golden.make_golden import quiet
            tmp = tempfile.mkdtemp(prefix="rgb_", dir="/tmp")
            path = os.path.join(tmp, "t.dump")
            harm.write_dump(path, dump)
            model = harm.ModelIn(IMG_WIDTH=W, IMG_HEIGHT=H, FREQ_MIN=FREQ, FREQ_MAX=FREQ, STEPSIZE=EPS)
            with quiet():
                sess = ref.RefSession(path, model, 1e19, INCL, 3.0, 3.0, 0.0, n1=GRID_N, n2=GRID_N, workdir=tmp,
                                      opt="stock")
        except Exception as e:  # noqa: BLE001
            print(f"reference build unusable, timing the port: {e}", file=sys.stderr)
            sess = None
    _REF_SESSION["s"] = sess
    return sess


def cpu_sample_run(dump, n_rays_target=None, seconds_target=12.0, nthreads=0, reps=1, with_port=False):
    """Time the reference's CPU implementation of the path on a strided pixel
    sample of the 1024x1024 image with all host threads: the reference's own
    C sources in their stock build (OpenMP over the pixels, as core.c:105's
    pragma would), or the C port where the reference cannot be built.  With
    with_port, the port is also timed on the same pixels.  Returns (ms per
    full image, detail dict)."""
    from oracle import port
    threads = nthreads or os.cpu_count() or 1
    sess = _reference_session(dump)
    kind = "reference" if sess is not None else "port"
    scene = port.Scene(dump.geom, dump.prims, W, H, inclination=INCL, stepsize=EPS)

    def run(pix, which):
        if which == "reference":
            return sess.render_pixels(pix, FREQ, threads)[1]
        return scene.render([FREQ], pixels=pix, nthreads=threads)[1]

    # pilot to size the sample for ~seconds_target of wall time
    pilot = np.arange(0, W * H, 997, dtype=np.int32)
    t_pilot = run(pilot, kind)
    if n_rays_target is None:
        n_rays_target = int(len(pilot) * seconds_target / max(t_pilot, 1e-3))
    stride = max(1, int(W * H / max(n_rays_target, 1)))
    pix = np.arange(0, W * H, stride, dtype=np.int32)
    times = [run(pix, kind) for _ in range(reps)]
    t = min(times)
    ms_image = t * 1e3 * (W * H) / len(pix)
    what = ("the reference's own sources, stock -Ofast build (makefile:13-15), OpenMP pixel loop"
            if kind == "reference" else "the C port of the reference's path (reference not buildable here)")
    det = {"kind": kind, "cores": threads, "rays": int(len(pix)), "stride": stride, "seconds": t, "times": times,
           "sample": f"one pixel in {stride} of the 1024x1024 image ({len(pix)} rays), {threads} OpenMP threads, "
                     f"extrapolated to the full image; {what}"}
    if with_port and kind == "reference":
        tp = run(pix, "port")
        det["port_same_pixels_ms_per_image"] = tp * 1e3 * (W * H) / len(pix)
        det["port_over_reference_time"] = tp / t
    return ms_image, det


def run_reference(args, rank):
    if rank != 0:
        return
    dump = make_scene()
    vals = []
    detail = None
    # warm-up: one short run per requested warm-up step
    for _ in range(args.warmup):
        cpu_sample_run(dump, n_rays_target=4096)
    for k in range(args.steps):
        v, detail = cpu_sample_run(dump, seconds_target=args.ref_seconds, with_port=(k == args.steps - 1))
        vals.append(v)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "ms/image", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.gpus),
            "cpu_baseline": {"value": value, "unit": "ms/image", "cores": detail["cores"], "kind": detail["kind"],
                             "sample": detail["sample"],
                             "port_same_pixels_ms_per_image": detail.get("port_same_pixels_ms_per_image"),
                             "port_over_reference_time": detail.get("port_over_reference_time")},
            "e2e": {"value": value, "unit": "ms/image", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(n_gpus=1):
    return {"workload": "1024x1024 image at 230 GHz of a seeded 512x512 Fishbone-Moncrief torus "
                        "(a=0.9375, MKS hslope=0.3, Rout=40), inclination 60 deg, RK4 eps=0.05, "
                        "M_unit=1e19 g, R_high=R_low=3",
            "image": [W, H], "grid": [GRID_N, GRID_N], "inclination_deg": INCL, "freq_hz": FREQ, "stepsize": EPS,
            "integrator": "RK4", "l2": "flushed between timed renders (512 MiB write)",
            "parallelism": f"replicas{n_gpus}"}


def run_vjp_adjoint256(reps=3):
    """Adjoint configuration: 256x256 image of the 256x256 torus, loss = L2
    distance to a target at M_unit x 1.3, R = 4, i = 62 deg.  Reports, for
    the FP64, mixed and mixed-DF forms, the forward and VJP (the
    raptor_gpu_vjp call: that form's one-pass adjoint) device times; the
    mixed and mixed-DF gradients are compared with the FP64 ones."""
    from raptor_gb300 import engine, synth
    d = synth.make_torus(n1=256, n2=256)
    eng = engine.Engine()
    gid = eng.upload_grid(d.geom, d.prims)
    desc = engine.image_desc(256, 256, [FREQ], grid=gid, inclination=60.0)
    target, _ = eng.render(engine.image_desc(256, 256, [FREQ], grid=gid, inclination=62.0, m_unit=1.3e19,
                                             r_high=4.0, r_low=4.0), engine.PREC_FP64)
    keys = ("d_m_unit", "d_r_high", "d_r_low", "d_inclination")
    out = {"config": "256x256 image, 256x256 torus, i=60, 230 GHz; loss to target at M_unit*1.3, R=4, i=62"}
    grads = {}
    for prec, name in ((engine.PREC_FP64, "fp64"), (engine.PREC_MIXED, "mixed"), (engine.PREC_MIXED_DF, "mixed_df")):
        fwd, vjp = [], []
        for _ in range(reps):
            img, _ = eng.render(desc, prec)
            fwd.append(eng.stats()["device_ms"])
            _, grads[name] = eng.vjp(desc, img - target, prec)
            vjp.append(eng.stats()["device_ms"])
        f, v = min(fwd), min(vjp)
        out[name] = {"fwd_ms": f, "vjp_ms": v, "ratio": v / f, "grad": {k: grads[name][k] for k in keys}}
    for name in ("mixed", "mixed_df"):
        out[name]["grad_rel_diff_vs_fp64"] = {
            k: abs(grads[name][k] - grads["fp64"][k]) / abs(grads["fp64"][k]) for k in keys}
    eng.close()
    # the FP64 numbers stay at the top level
    out.update(fwd_ms=out["fp64"]["fwd_ms"], vjp_ms=out["fp64"]["vjp_ms"], ratio=out["fp64"]["ratio"])
    return out


def run_batch_64(dev):
    """Batched configuration: 64 images (32x128^2, 24x256^2, 6x512^2,
    2x1024^2) over two 256x256 dumps, seeded angles/frequencies/M_unit: one
    graph-replayed persistent launch with the autotuned shape, against 64
    sequential plain renders."""
    from raptor_gb300 import engine, workloads
    dumps = workloads.batch_dumps(256)
    g_eng = engine.Engine(device=dev, use_graph=1, autotune=1)
    gids = [g_eng.upload_grid(d.geom, d.prims) for d in dumps]
    descs = workloads.batch_images(gids)
    g_eng.render(descs, engine.PREC_FP64)  # tunes the shape and captures the graph
    t0 = time.perf_counter()
    g_eng.render(descs, engine.PREC_FP64)
    wall_batch = (time.perf_counter() - t0) * 1e3
    st = g_eng.stats()
    # the same batch in the mixed-DF form (its own tuned shape and graph)
    g_eng.render(descs, engine.PREC_MIXED_DF)
    t0 = time.perf_counter()
    g_eng.render(descs, engine.PREC_MIXED_DF)
    wall_df = (time.perf_counter() - t0) * 1e3
    st_df = g_eng.stats()
    p_eng = engine.Engine(device=dev)
    for d in dumps:
        p_eng.upload_grid(d.geom, d.prims)
    seq_dev = 0.0
    t0 = time.perf_counter()
    for d in descs:
        p_eng.render(d, engine.PREC_FP64)
        seq_dev += p_eng.stats()["device_ms"]
    wall_seq = (time.perf_counter() - t0) * 1e3
    g_eng.close()
    p_eng.close()
    return {"images": len(descs), "rays": st["rays"], "graph_replayed": st["graph_replayed"],
            "launch": [st["block_size"], st["blocks_per_sm"], st["refill_interval"]],
            "batched_device_ms": st["device_ms"], "batched_wall_ms": wall_batch,
            "sequential_device_ms": seq_dev, "sequential_wall_ms": wall_seq,
            "speedup_wall": wall_seq / wall_batch, "rays_per_s": st["rays"] / (st["device_ms"] * 1e-3),
            "mixed_df": {"batched_device_ms": st_df["device_ms"], "batched_wall_ms": wall_df,
                         "graph_replayed": st_df["graph_replayed"],
                         "launch": [st_df["block_size"], st_df["blocks_per_sm"], st_df["refill_interval"]],
                         "rays_per_s": st_df["rays"] / (st_df["device_ms"] * 1e-3)}}


def _loss_delta(op, om, target):
    """L(O+) - L(O-) for L = 1/2 sum (O - target)^2, without the cancellation
    of subtracting two large sums."""
    return 0.5 * float(np.sum((op - om) * (op + om - 2.0 * target)))


def run_differentiable(dev, n_cells=4, reps=2, incl_hs=(1e-4, 1e-6, 1e-7)):
    """Large differentiable batch: a 2048x2048 image at 86/140/230/345/690 GHz
    (with its spectrum) of the 512x512 torus, and the VJP of
    L = 1/2 |O - O_target|^2 (target at M_unit x 1.3, R = 4, i = 62 deg) with
    respect to the four scalars and the per-cell rho, u and ln Theta_e
    fields, in each form as a forward render and that form's VJP call (one
    adjoint pass that takes each ray's I from its own sums and keeps the
    ray's per-cell terms on a record tape): mixed (the workload's: FP64
    geodesic, FP32 transfer; its adjoint keeps the FP64 path with FP32
    tangents and the FP32 dual sample), FP64, and mixed-DF.  Reports
    forward, adjoint and VJP device times, the engine's
    peak device memory, and each form's gradients against central
    differences of the FP64 forward: the four scalars (h = 1e-4 relative,
    and the inclination also at the smaller incl_hs, where the piecewise
    smooth loss reaches its derivative) and rho and u of the n_cells cells
    with the largest gradient."""
    from raptor_gb300 import engine
    d = make_scene()
    freqs = [86e9, 140e9, 230e9, 345e9, 690e9]
    n = 2048
    base = dict(m_unit=1e19, r_high=3.0, r_low=3.0, inclination=60.0)
    eng = engine.Engine(device=dev)
    gid = eng.upload_grid(d.geom, d.prims)
    mk = lambda **o: engine.image_desc(n, n, freqs, grid=gid, **dict(base, **o))  # noqa: E731
    target, _ = eng.render(mk(m_unit=1.3e19, r_high=4.0, r_low=4.0, inclination=62.0), engine.PREC_MIXED)
    forms = (("mixed", engine.PREC_MIXED), ("fp64", engine.PREC_FP64), ("mixed_df", engine.PREC_MIXED_DF))
    res, grads = {}, {}
    for name, prec in forms:
        fwd_ms, adj_ms, vjp_ms = [], [], []
        for _ in range(reps):
            img, _ = eng.render(mk(), prec)
            fwd_ms.append(eng.stats()["device_ms"])
            _, g = eng.vjp(mk(), img - target, prec)
            st = eng.stats()
            adj_ms.append(st["kernel_ms"])
            vjp_ms.append(st["device_ms"])
        grads[name] = g
        f, a, v = min(fwd_ms), min(adj_ms), min(vjp_ms)
        res[name] = {"forward_ms": f, "adjoint_kernel_ms": a, "vjp_total_ms": v, "adjoint_over_forward": a / f,
                     "vjp_total_over_forward": v / f}
    res["fp64"]["adjoint"] = "FP64 geodesic with FP64 tangents, FP64 dual sample (sample pool)"
    res["mixed"]["adjoint"] = "FP64 geodesic with FP32 tangents, FP32 dual sample"
    res["mixed_df"]["adjoint"] = "double-float geodesic with FP32 tangents, FP32 dual sample"
    peak = eng.stats()["peak_device_bytes"]

    # central differences of the FP64 forward
    def fd_scalar(key, rel, richardson):
        diffs = []
        for r in ((rel, rel / 2) if richardson else (rel,)):
            h = r * base[key]
            op, _ = eng.render(mk(**{key: base[key] + h}), engine.PREC_FP64)
            om, _ = eng.render(mk(**{key: base[key] - h}), engine.PREC_FP64)
            diffs.append(_loss_delta(op, om, target) / (2 * h))
        return diffs[0] if not richardson else (4 * diffs[1] - diffs[0]) / 3

    def versus(fd, key):
        return {"fd": fd, **{f"vjp_{nm}": grads[nm][key] for nm, _ in forms},
                **{f"rel_err_{nm}": abs(grads[nm][key] - fd) / abs(fd) for nm, _ in forms}}

    t0 = time.perf_counter()
    scal = {}
    for key, gk in (("m_unit", "d_m_unit"), ("r_high", "d_r_high"), ("r_low", "d_r_low")):
        scal[key] = versus(fd_scalar(key, 1e-4, False), gk)
    # the loss is only piecewise smooth in the inclination (clamps, min() in the
    # step size, cell-index changes along every ray): its difference quotient
    # reaches the derivative only as h shrinks
    for rel in incl_hs:
        scal[f"inclination_h{rel:g}"] = versus(fd_scalar("inclination", rel, rel >= 1e-4), "d_inclination")
    cells = {}
    order = np.argsort(-np.abs(grads["mixed"]["d_rho"]).ravel())[:n_cells]
    fd_all, got_all = [], {nm: [] for nm, _ in forms}
    for flat in order:
        i, j = divmod(int(flat), d.geom.n2)
        for q, field in ((0, "d_rho"), (1, "d_u")):
            pr = d.prims.copy()
            v = pr[q, i, j]
            pr[q, i, j] = v * (1 + 1e-4)
            eng.upload_grid(d.geom, pr, grid_id=gid)
            op, _ = eng.render(mk(), engine.PREC_FP64)
            pr[q, i, j] = v * (1 - 1e-4)
            eng.upload_grid(d.geom, pr, grid_id=gid)
            om, _ = eng.render(mk(), engine.PREC_FP64)
            fd = _loss_delta(op, om, target) / (2e-4 * v)
            cells[f"{field}[{i},{j}]"] = {"fd": fd, **{f"vjp_{nm}": float(grads[nm][field][i, j]) for nm, _ in forms}}
            fd_all.append(fd)
            for nm, _ in forms:
                got_all[nm].append(float(grads[nm][field][i, j]))
    eng.upload_grid(d.geom, d.prims, grid_id=gid)
    fd_s = time.perf_counter() - t0
    scale = max(abs(x) for x in fd_all)
    for nm, _ in forms:
        res[nm]["cell_max_err_over_scale"] = max(abs(a - b) for a, b in zip(got_all[nm], fd_all)) / scale
        res[nm]["scalar_max_rel_err"] = max(
            scal[k][f"rel_err_{nm}"] for k in ("m_unit", "r_high", "r_low", f"inclination_h{min(incl_hs):g}"))
    # uniform Theta_e factor = change of T_p/T_e at R_high = R_low = R
    R = base["r_high"]
    tg = 0.5 * ((1.0 + 2.0 / 3.0 * (R + 1.0) / (R + 2.0)) + 4.0 / 3.0)
    dlnT_dR = (1.0 / 3.0) / (R + 2.0) ** 2 / (tg - 1.0) - 1.0 / (1.0 + R)
    for nm, _ in forms:
        g = grads[nm]
        th_sum = float(np.sum(g["d_lnthetae"]))
        th_want = (g["d_r_high"] + g["d_r_low"]) / dlnT_dR
        res[nm]["thetae_sum_identity_rel_err"] = abs(th_sum - th_want) / abs(th_want)
    eng.close()
    m = res["mixed"]
    return {
        "metric": "2048² x 5-frequency differentiable render: VJP/forward time, peak device memory, "
                  "finite-difference agreement",
        "config": {"workload": "2048x2048 image at 86/140/230/345/690 GHz with spectrum, 512x512 torus a=0.9375, "
                               "i=60, M_unit=1e19, R_high=R_low=3; loss to target at M_unit*1.3, R=4, i=62",
                   "forward": "mixed", "adjoint": m["adjoint"] + " (forward-mode tangents + suffix identity, "
                                                               "one pass with a per-lane record tape, "
                                                               "no checkpoints)"},
        "forward_ms": m["forward_ms"], "adjoint_kernel_ms": m["adjoint_kernel_ms"], "vjp_total_ms": m["vjp_total_ms"],
        "adjoint_over_forward": m["adjoint_over_forward"], "vjp_total_over_forward": m["vjp_total_over_forward"],
        "peak_device_bytes": peak, "forms": res,
        "grad_values": int(3 * d.geom.n1 * d.geom.n2 + 4),
        "fd": {"scalars": scal, "cells": cells, "seconds": fd_s, "h_rel": 1e-4},
    }


def pixel_error_summary(img, ref):
    """Per-pixel relative errors of a mixed form against the FP64 image: over
    the emitting pixels the median, maximum and the fractions above 1e-3 and
    1e-2; the same fractions over the pixels within six decades of the
    brightest, which carry all but ~2e-6 of the flux (most emitting pixels
    lie below that, some 30 decades down, where the FP32 emissivity's
    exp(-X^1/3) underflows and relative errors reach 1); and the summed
    absolute error over the flux."""
    nz = ref != 0
    pe = np.abs(img[nz] - ref[nz]) / np.abs(ref[nz])
    br = ref >= 1e-6 * ref.max()
    pb = np.abs(img[br] - ref[br]) / np.abs(ref[br])
    return {"pixel_err_median": float(np.median(pe)), "pixel_err_max": float(np.max(pe)),
            "frac_pixels_above_1e-3": float(np.mean(pe > 1e-3)), "frac_pixels_above_1e-2": float(np.mean(pe > 1e-2)),
            "pixels_compared": int(pe.size),
            "bright_frac_above_1e-3": float(np.mean(pb > 1e-3)), "bright_frac_above_1e-2": float(np.mean(pb > 1e-2)),
            "bright_pixel_err_max": float(np.max(pb)), "bright_pixels": int(pb.size),
            "abs_err_sum_over_flux": float(np.sum(np.abs(img - ref)) / np.sum(ref))}


def run_inclination(eng, blib, dev, gid, incl, forms, steps):
    """The headline image at another inclination (the workload's second
    angle): each form rendered `steps` times after an L2 flush (device time,
    mean), with flux / pixel / k.k errors against the FP64 form."""
    from raptor_gb300 import engine
    desc = engine.image_desc(W, H, [FREQ], grid=gid, inclination=incl, stepsize=EPS)
    got = {}
    for prec, name in forms:
        ms = []
        for _ in range(max(1, steps)):
            blib.raptor_bench_flush_l2(dev, L2_FLUSH_BYTES)
            img, spec = eng.render(desc, prec)
            ms.append(eng.stats()["device_ms"])
        st = eng.stats()
        got[name] = dict(img=img, flux=float(spec[0]), ms=float(np.mean(ms)), kk=st["kk_max"], steps=st["steps"])
    ref = got["fp64"]
    out = {"inclination_deg": incl}
    for name, g in got.items():
        row = {"ms_per_image": g["ms"], "kk_max": g["kk"], "steps": g["steps"]}
        if name != "fp64":
            row.update(speedup_vs_fp64=ref["ms"] / g["ms"], flux_err_vs_fp64=abs(g["flux"] - ref["flux"]) / ref["flux"],
                       **pixel_error_summary(g["img"], ref["img"]))
        out[name] = row
    return out


def run_engine(args, rank, world, local):
    from raptor_gb300 import engine
    dev = local
    dump = make_scene()
    eng = engine.Engine(device=dev, autotune=1 if args.autotune else 0)
    lib = eng.lib
    blib = ctypes.CDLL(os.path.join(ROOT, "raptor_gb300", "_lib", "libraptor_benchutil.so"))
    blib.raptor_bench_fp64_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    blib.raptor_bench_fp32_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    blib.raptor_bench_flush_l2.argtypes = [ctypes.c_int, ctypes.c_longlong]
    gid = eng.upload_grid(dump.geom, dump.prims)
    # each rank renders its own image (weak scaling): inclination offset per rank
    incl = INCL + 0.0 * rank
    desc = engine.image_desc(W, H, [FREQ], grid=gid, inclination=incl, stepsize=EPS)
    arr = (engine.ImageDesc * 1)(desc)

    def render_resident(prec):
        rc = lib.raptor_gpu_render(eng.h, arr, 1, prec, None, None)
        if rc != 0:
            raise engine.EngineError(rc, lib.raptor_gpu_last_error(eng.h).decode())
        return eng.stats()

    barrier = None
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("gloo")
        barrier = dist.barrier

    def maxed(x):
        if world == 1:
            return x
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    forms = ((engine.PREC_FP64, "fp64"), (engine.PREC_MIXED, "mixed"), (engine.PREC_MIXED_DF, "mixed_df"))
    for _ in range(args.warmup):
        for prec, _name in forms:
            render_resident(prec)

    results = {}
    with Clocks(dev) as clk:
        for prec, name in forms:
            if barrier:
                barrier()
            dev_ms, ker_ms, stats = [], [], None
            for _ in range(args.steps):
                blib.raptor_bench_flush_l2(dev, L2_FLUSH_BYTES)
                stats = render_resident(prec)
                dev_ms.append(stats["device_ms"])
                ker_ms.append(stats["kernel_ms"])
            if barrier:
                barrier()
            results[name] = dict(device_ms=dev_ms, kernel_ms=ker_ms, stats=stats)
    clocks = clk.summary()

    # images of both forms for the mixed-vs-FP64 error report
    img64, spec64 = eng.render(desc, engine.PREC_FP64)
    imgmx, specmx = eng.render(desc, engine.PREC_MIXED)
    imgdf, specdf = eng.render(desc, engine.PREC_MIXED_DF)
    kk_df = eng.stats()["kk_max"]
    flux_err = abs(specmx[0] - spec64[0]) / spec64[0]
    flux_err_df = abs(specdf[0] - spec64[0]) / spec64[0]

    # end to end through the C ABI with host buffers: grid upload (pinned) + render + image read-back
    try:
        import torch
        prims_pinned = torch.empty(dump.prims.shape, dtype=torch.float64, pin_memory=True).numpy()
        out_pinned = torch.empty(W * H, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        prims_pinned = np.empty_like(dump.prims)
        out_pinned = np.empty(W * H)
    prims_pinned[...] = dump.prims
    spec_out = np.empty(1)
    e2e_ms = []
    if barrier:
        barrier()
    for _ in range(0 if args.no_e2e else args.steps):
        blib.raptor_bench_flush_l2(dev, L2_FLUSH_BYTES)
        t0 = time.perf_counter()
        eng.upload_grid(dump.geom, prims_pinned, grid_id=gid)
        eng.render(desc, engine.PREC_FP64, out=out_pinned, spectrum=spec_out)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if barrier:
        barrier()
    e2e_stats = eng.stats()

    # FP64 DFMA and FP32 FFMA peaks of this GPU (roofline denominators)
    peak = ctypes.c_double(0.0)
    blib.raptor_bench_fp64_peak(dev, 5, ctypes.byref(peak))
    peak32 = ctypes.c_double(0.0)
    blib.raptor_bench_fp32_peak(dev, 5, ctypes.byref(peak32))

    st = results["fp64"]["stats"]
    t_fp64 = maxed(float(np.mean(results["fp64"]["device_ms"])))
    t_mixed = maxed(float(np.mean(results["mixed"]["device_ms"])))
    t_mixed_df = maxed(float(np.mean(results["mixed_df"]["device_ms"])))
    t_e2e = maxed(float(np.mean(e2e_ms))) if e2e_ms else None
    e2e_h2d = int(dump.prims.nbytes + e2e_stats["h2d_bytes"])  # grid upload + descriptors
    k_fp64 = float(np.mean(results["fp64"]["kernel_ms"]))
    k_df = float(np.mean(results["mixed_df"]["kernel_ms"]))
    from raptor_gb300 import workload
    flop = workload.image_flops(st["rays"], st["steps"], st["rt_samples"], 1, rk4=True)
    flop_sym = workload.image_flops_symmetric(st["steps"], st["rt_samples"], 1)
    achieved = flop / (k_fp64 * 1e-3) / 1e12

    vjp = batch = incl17 = diff = None
    if not args.no_e2e:
        incl17 = run_inclination(eng, blib, dev, gid, 17.0, forms, args.steps)
        vjp = run_vjp_adjoint256()
        batch = run_batch_64(dev)
        if not args.no_differentiable:
            diff = run_differentiable(dev, n_cells=2, reps=1, incl_hs=(1e-7,))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        ms_cpu, det = cpu_sample_run(dump, seconds_target=args.ref_seconds, with_port=True)
        cpu = {"value": ms_cpu, "unit": "ms/image", "cores": det["cores"], "kind": det["kind"],
               "sample": det["sample"], "port_same_pixels_ms_per_image": det.get("port_same_pixels_ms_per_image"),
               "port_over_reference_time": det.get("port_over_reference_time")}
    eng.close()
    if rank != 0:
        return
    n = world
    line = {
        "metric": METRIC, "value": t_fp64 / n, "unit": "ms/image", "n_gpus": n, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_fp64, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Fishbone-Moncrief torus)",
        "config": workload_config(n),
        "e2e": ({"value": t_e2e / n, "unit": "ms/image", "h2d_bytes_per_step": e2e_h2d,
                 "d2h_bytes_per_step": int(e2e_stats["d2h_bytes"]),
                 "path": "raptor_gpu_upload_grid (pinned host prims) + raptor_gpu_render (host image out)"}
                if t_e2e is not None else None),
        # timed loop, per render of each of the three forms: L2 flush, ray kernel, spectrum kernel
        "gpu_launches": 3 * 3 * args.steps,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value > 0 else None,
                     # DRAM bytes per launch of this kernel on this workload, from one ncu
                     # capture (dram__bytes_read.sum + dram__bytes_write.sum)
                     "traffic": TRAFFIC_FP64_1024 if (W, H, GRID_N) == (1024, 1024, 512) else None,
                     "traffic_unit": "bytes per launch",
                     "peak_source": "measured DFMA loop on this GPU (MEASURED_PEAKS.json has no FP64 figure); "
                                    f"nominal {NOMINAL_FP64_TFLOPS} TFLOP/s",
                     "flop_per_launch": flop, "kernel_ms": k_fp64,
                     # the same with the symmetric hand count of the algorithm
                     # (1,260 per RK4 step, 316 + 63 F per sample)
                     "flop_per_launch_symmetric": flop_sym,
                     "frac_symmetric": (flop_sym / (k_fp64 * 1e-3) / 1e12) / peak.value if peak.value > 0 else None},
        "clocks": clocks,
        "forms": {
            "fp64": {"ms_per_image": t_fp64, "kernel_ms": k_fp64, "rays_per_s": W * H / (t_fp64 * 1e-3),
                     "ray_steps_per_s": st["steps"] / (k_fp64 * 1e-3), "steps": st["steps"],
                     "rt_samples": st["rt_samples"], "max_ray_steps": st["max_ray_steps"], "kk_max": st["kk_max"],
                     "launch": [st["block_size"], st["blocks_per_sm"], st["refill_interval"]]},
            "mixed": {"ms_per_image": t_mixed, "speedup_vs_fp64": t_fp64 / t_mixed, "flux_err_vs_fp64": flux_err,
                      **pixel_error_summary(imgmx, img64)},
            "mixed_df": {"ms_per_image": t_mixed_df, "speedup_vs_fp64": t_fp64 / t_mixed_df,
                         "flux_err_vs_fp64": flux_err_df, **pixel_error_summary(imgdf, img64), "kk_max": kk_df,
                         "geodesic": "double-float (FP32 pairs, 48-bit significand)",
                         "kernel_ms": k_df,
                         # the same algorithmic FLOP count as the FP64 form, per second of the DF kernel
                         "algorithmic_tflops": flop / (k_df * 1e-3) / 1e12,
                         "roofline": df_roofline(k_df, peak32.value),
                         "launch": [results["mixed_df"]["stats"][k] for k in
                                    ("block_size", "blocks_per_sm", "refill_interval")]},
            "inclination_17": incl17,
            "vjp": vjp,
            "batch": batch,
            "differentiable": diff,
        },
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("engine", "reference"), default="engine")
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-differentiable", action="store_true",
                    help="leave out the 2048x2048 5-frequency VJP leg (about two minutes)")
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--workload", choices=("1024", "profile", "differentiable", "adjoint"), default="1024",
                    help="profile: a 256x256 image on a 256x256 torus, render timings only (for ncu captures); "
                         "differentiable: the 2048x2048 5-frequency forward + VJP with finite-difference checks; "
                         "adjoint: the 256x256 adjoint configuration alone (FP64 and mixed-DF VJP)")
    args = ap.parse_args()
    if args.workload == "differentiable":
        print(json.dumps(run_differentiable(dist_env()[2])), flush=True)
        return
    if args.workload == "adjoint":
        print(json.dumps(run_vjp_adjoint256(reps=args.steps)), flush=True)
        return
    if args.workload == "profile":
        global W, H, GRID_N
        W = H = 256
        GRID_N = 256
        args.no_cpu_baseline = True
        args.no_e2e = True
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_engine(args, rank, world, local)


if __name__ == "__main__":
    main()
