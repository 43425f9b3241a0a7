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
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{device}.csv")

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


def cpu_sample_run(dump, n_rays_target=None, seconds_target=12.0, nthreads=0, reps=1):
    """Time the reference's CPU algorithm on a strided pixel sample of the
    1024x1024 image.  Uses the reference build if one loads here, else the
    C port.  Returns (ms per full image, detail dict)."""
    from oracle import port, ref
    kind = "port"
    threads = nthreads or os.cpu_count() or 1
    sess = None
    if ref.available(GRID_N, GRID_N, opt="stock"):
        try:
            import tempfile
            from raptor_gb300 import harm
            from tests.golden.make_golden import quiet
            tmp = tempfile.mkdtemp(prefix="rgb_", dir="/tmp")
            path = os.path.join(tmp, "t.dump")
            harm.write_dump(path, dump)
            model = harm.ModelIn(IMG_WIDTH=W, IMG_HEIGHT=H, FREQ_MIN=FREQ, FREQ_MAX=FREQ, STEPSIZE=EPS)
            with quiet():
                sess = ref.RefSession(path, model, 1e19, INCL, 3.0, 3.0, 0.0, n1=GRID_N, n2=GRID_N, workdir=tmp,
                                      opt="stock")
            kind = "reference"
        except Exception:
            sess = None
            kind = "port"
    scene = port.Scene(dump.geom, dump.prims, W, H, inclination=INCL, stepsize=EPS)

    def run(pix):
        if sess is not None:
            return sess.render_pixels(pix, FREQ, threads)[1]
        return scene.render([FREQ], pixels=pix, nthreads=threads)[1]

    # pilot to size the sample for ~seconds_target of wall time
    pilot = np.arange(0, W * H, 997, dtype=np.int32)
    t_pilot = run(pilot)
    if n_rays_target is None:
        n_rays_target = int(len(pilot) * seconds_target / max(t_pilot, 1e-3))
    stride = max(1, int(W * H / max(n_rays_target, 1)))
    pix = np.arange(0, W * H, stride, dtype=np.int32)
    times = [run(pix) for _ in range(reps)]
    t = min(times)
    ms_image = t * 1e3 * (W * H) / len(pix)
    return ms_image, {"kind": kind, "cores": threads, "rays": int(len(pix)), "stride": stride,
                      "seconds": t, "times": times,
                      "sample": f"every {stride}th pixel of the 1024x1024 image ({len(pix)} rays), "
                                f"{threads} OpenMP threads, extrapolated to the full image"}


def run_reference(args, rank):
    if rank != 0:
        return
    dump = make_scene()
    vals = []
    detail = None
    # warm-up: one short run per requested warm-up step
    for _ in range(args.warmup):
        cpu_sample_run(dump, n_rays_target=4096)
    for _ in range(args.steps):
        v, detail = cpu_sample_run(dump, seconds_target=args.ref_seconds)
        vals.append(v)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "ms/image", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "ms/image", "cores": detail["cores"], "kind": detail["kind"],
                             "sample": detail["sample"]},
            "e2e": {"value": value, "unit": "ms/image", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config():
    return {"workload": "1024x1024 image at 230 GHz of a seeded 512x512 Fishbone-Moncrief torus "
                        "(a=0.9375, MKS hslope=0.3, Rout=40), inclination 60 deg, RK4 eps=0.05, "
                        "M_unit=1e19 g, R_high=R_low=3",
            "image": [W, H], "grid": [GRID_N, GRID_N], "inclination_deg": INCL, "freq_hz": FREQ, "stepsize": EPS,
            "integrator": "RK4", "l2": "flushed between timed renders (512 MiB write)"}


def run_engine(args, rank, world, local):
    from raptor_gb300 import engine
    dev = local
    dump = make_scene()
    eng = engine.Engine(device=dev, autotune=1 if args.autotune else 0)
    lib = eng.lib
    blib = ctypes.CDLL(os.path.join(ROOT, "raptor_gb300", "_lib", "libraptor_benchutil.so"))
    blib.raptor_bench_fp64_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
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

    for _ in range(args.warmup):
        render_resident(engine.PREC_FP64)
        render_resident(engine.PREC_MIXED)

    results = {}
    with Clocks(dev) as clk:
        for prec, name in ((engine.PREC_FP64, "fp64"), (engine.PREC_MIXED, "mixed")):
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
    nz = img64 != 0
    pix_err = np.abs(imgmx[nz] - img64[nz]) / np.abs(img64[nz])
    flux_err = abs(specmx[0] - spec64[0]) / spec64[0]

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

    # FP64 DFMA peak of this GPU (roofline denominator)
    peak = ctypes.c_double(0.0)
    blib.raptor_bench_fp64_peak(dev, 5, ctypes.byref(peak))

    st = results["fp64"]["stats"]
    t_fp64 = maxed(float(np.mean(results["fp64"]["device_ms"])))
    t_mixed = maxed(float(np.mean(results["mixed"]["device_ms"])))
    t_e2e = maxed(float(np.mean(e2e_ms))) if e2e_ms else None
    e2e_h2d = int(dump.prims.nbytes + e2e_stats["h2d_bytes"])  # grid upload + descriptors
    k_fp64 = float(np.mean(results["fp64"]["kernel_ms"]))
    from raptor_gb300 import workload
    flop = workload.image_flops(st["rays"], st["steps"], st["rt_samples"], 1, rk4=True)
    achieved = flop / (k_fp64 * 1e-3) / 1e12

    # VJP / forward ratio (if the adjoint is available)
    vjp = None
    try:
        if args.no_e2e:
            raise RuntimeError("skipped in the profile workload")
        dl = np.ones(W * H) * 1e-3
        t0 = time.perf_counter()
        eng.vjp(desc, dl, engine.PREC_FP64, want_fields=True)
        vjp_ms = eng.stats()["device_ms"]
        vjp = {"vjp_ms": vjp_ms, "fwd_ms": t_fp64, "ratio": vjp_ms / t_fp64,
               "wall_ms": (time.perf_counter() - t0) * 1e3}
    except Exception as ex:  # not built yet
        vjp = {"unavailable": str(ex)[:120]}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        ms_cpu, det = cpu_sample_run(dump, seconds_target=args.ref_seconds)
        cpu = {"value": ms_cpu, "unit": "ms/image", "cores": det["cores"], "kind": det["kind"],
               "sample": det["sample"]}
    eng.close()
    if rank != 0:
        return
    n = world
    line = {
        "metric": METRIC, "value": t_fp64 / n, "unit": "ms/image", "n_gpus": n, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_fp64, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Fishbone-Moncrief torus)",
        "config": dict(workload_config(), parallelism=f"replicas{n}"),
        "e2e": ({"value": t_e2e / n, "unit": "ms/image", "h2d_bytes_per_step": e2e_h2d,
                 "d2h_bytes_per_step": int(e2e_stats["d2h_bytes"]),
                 "path": "raptor_gpu_upload_grid (pinned host prims) + raptor_gpu_render (host image out)"}
                if t_e2e is not None else None),
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value > 0 else None, "traffic": None,
                     "peak_source": "measured DFMA loop on this GPU (MEASURED_PEAKS.json has no FP64 figure); "
                                    f"nominal {NOMINAL_FP64_TFLOPS} TFLOP/s",
                     "flop_per_launch": flop, "kernel_ms": k_fp64},
        "clocks": clocks,
        "forms": {
            "fp64": {"ms_per_image": t_fp64, "kernel_ms": k_fp64, "rays_per_s": W * H / (t_fp64 * 1e-3),
                     "ray_steps_per_s": st["steps"] / (k_fp64 * 1e-3), "steps": st["steps"],
                     "rt_samples": st["rt_samples"], "max_ray_steps": st["max_ray_steps"], "kk_max": st["kk_max"],
                     "launch": [st["block_size"], st["blocks_per_sm"], st["refill_interval"]]},
            "mixed": {"ms_per_image": t_mixed, "speedup_vs_fp64": t_fp64 / t_mixed, "flux_err_vs_fp64": flux_err,
                      "pixel_err_median": float(np.median(pix_err)), "pixel_err_max": float(np.max(pix_err))},
            "vjp": vjp,
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
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--workload", choices=("1024", "profile"), default="1024",
                    help="profile: a 256x256 image on a 256x256 torus, render timings only (for ncu captures)")
    args = ap.parse_args()
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
