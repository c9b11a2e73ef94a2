"""Benchmark: slices/s of CGLS to relative residual 1e-3 on the 1024^2 x 512-slice,
1200-angle cylinder (square-pixel projector), on one GB300 per rank.

One step = one complete CGLS solve of the whole volume from zero, stopped when
||A^T(b - A x_k)|| / ||A^T b|| <= 1e-3 (fixed denominator) or after 200
iterations.  Inputs: a seeded random-sphere cylinder with analytic line
integrals and Poisson noise at 5e3 photons (no public dataset exists).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line on rank 0.  With N > 1 (torchrun) every rank solves its
own replica (the path needs no exchange: replicas only, weak scaling).
`--impl reference` times the reference's CPU algorithm for the same metric on
this host's cores (the oracle's C restatement, one thread per slab of slices
like the reference's MPI ranks) on a bounded sample and extrapolates.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
os.environ.setdefault("ARECGB_QUIET", "1")

NX, NY, NA = 1024, 512, 1200
TOL, MAXIT = 1e-3, 200
PHOTONS = 5e3
METRIC = "slices/s to rel. residual 1e-3 (1024², 1200 ang): warm-start vs plain CGLS"
CONFIG = {"workload": "plain CGLS to ||A^T r||/||A^T b|| <= 1e-3 (max 200 it), square-pixel "
                      "projector, 1024^2 x 512 slices, 1200 angles over [0,180), random-sphere "
                      "cylinder r=500 px with 200 spheres, Poisson 5e3 photons",
          "nx": NX, "slices": NY, "angles": NA, "tol": TOL, "maxit": MAXIT,
          "warm_start": False,
          "l2": "inputs larger than L2 (b 2.5 GB, x 1.7 GB per solve)"}


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


def make_problem(gb, seed, device="cuda"):
    import torch

    from arec3d_gb300 import synthetic as syn

    angles = syn.uniform_angles(NA)
    plan = gb.Plan(gb.SQ, 0.5 * (NX - 1), NY, angles)
    ph = syn.sphere_cylinder_phantom(seed, NX, NY)
    b = syn.sphere_sinogram(ph, NX, NY, angles, ys=plan.ys, device=device)
    syn.poisson_log(b, PHOTONS, seed + 1, NY, device=device)
    torch.cuda.synchronize()
    return plan, b, angles


def cpu_sample(weighting_sq=True, slices=16, iters=1, threads=None):
    """Reference CGLS (oracle restatement, one thread per slab) on a slab of the
    benchmark geometry; returns seconds per slice per projector pass."""
    import oracle

    oracle.build()
    threads = threads or min(os.cpu_count() or 1, slices)
    rng = np.random.default_rng(0)
    angles = (np.arange(NA) * (np.pi / NA)).astype(np.float32)
    b = (rng.random((NA, slices, NX), dtype=np.float32) * 2.0).astype(np.float32)
    t0 = time.perf_counter()
    oracle.cgls(3, b, angles, maxit=iters, tol=0.0, nthreads=threads)
    dt = time.perf_counter() - t0
    passes = 1 + 2 * iters  # initial A^T s, then A p and A^T s per iteration
    return dt / (slices * passes), {"slices": slices, "iterations": iters, "threads": threads,
                                    "seconds": dt}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU algorithm on this host's cores."""
    if rank != 0:
        return
    it_gpu = args.ref_iters
    times = []
    info = None
    for i in range(args.warmup + args.steps):
        per, info = cpu_sample(slices=args.ref_slices, iters=1)
        if i >= args.warmup:
            times.append(per)
    per = statistics.median(times)
    solve_s = per * NY * (1 + 2 * it_gpu)
    value = NY / solve_s
    out = {
        "metric": METRIC, "value": value, "unit": "slices/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": solve_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "impl": "reference", "config": CONFIG,
        "cpu_baseline": {"value": value, "unit": "slices/s", "cores": info["threads"],
                         "kind": "port",
                         "sample": "oracle C restatement of cyl_cgls_SQ, %d slices x 1 CGLS "
                                   "iteration on the 1024^2/1200-angle geometry per step, "
                                   "extrapolated linearly to 512 slices x %d iterations"
                                   % (info["slices"], it_gpu)},
        "e2e": {"value": value, "unit": "slices/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def kernels_only(args):
    """Forward and back projector of the benchmark geometry on `--slices`
    slices, `--launches` times each (a short command for ncu)."""
    import torch

    import arec3d_gb300 as gb
    from arec3d_gb300 import synthetic as syn

    gb.build()
    angles = syn.uniform_angles(args.angles)
    plan = gb.Plan(gb.SQ, 0.5 * (NX - 1), args.slices, angles)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    x = torch.rand(plan.nrays, plan.ys, device="cuda", generator=g)
    x[:, args.slices:] = 0
    q = torch.zeros(plan.nangles, plan.nx, plan.ys, device="cuda")
    n2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(args.launches):
        plan.project(x, q, norm2=n2)
        plan.backproject(q, x, norm2=n2)
    torch.cuda.synchronize()
    print(json.dumps({"kernels_only": True, "slices": args.slices, "launches": args.launches,
                      "norm2": float(n2.item())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ref-slices", type=int, default=16)
    ap.add_argument("--ref-iters", type=int, default=60,
                    help="iterations to extrapolate the reference arm to")
    ap.add_argument("--kernels-only", action="store_true",
                    help="run only the forward and back projectors (for profiling)")
    ap.add_argument("--slices", type=int, default=NY, help="slices for --kernels-only")
    ap.add_argument("--launches", type=int, default=3, help="launches for --kernels-only")
    ap.add_argument("--angles", type=int, default=NA, help="angles for --kernels-only")
    args = ap.parse_args()
    rank, local, world = dist_env()
    if args.kernels_only:
        kernels_only(args)
        return

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch

    import arec3d_gb300 as gb

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    gb.build()
    plan, b, angles = make_problem(gb, seed=1000 + rank)
    x = torch.zeros(plan.nrays, plan.ys, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    # fixed denominator ||A^T b||
    g = torch.zeros_like(x)
    n2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    plan.backproject(b, g, norm2=n2, stream=stream)
    rnorm_ref = float(n2.item()) ** 0.5
    del g

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    iters = []
    for _ in range(args.warmup):
        hist, info = plan.cgls(b, x, MAXIT, TOL, rnorm_ref=rnorm_ref, stream=stream)
    barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        hist, info = plan.cgls(b, x, MAXIT, TOL, rnorm_ref=rnorm_ref, stream=stream)
        iters.append(info.iterations)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = world * NY / (ms_step / 1e3)
    n_it = int(statistics.median(iters))
    rel_final = float(hist[-1]) if len(hist) else None

    # Kernel roofline: forward and back projector timed alone on this stream.
    q = torch.zeros(plan.nangles, plan.nx, plan.ys, dtype=torch.float32, device="cuda")
    gg = torch.zeros_like(x)
    kt = {}
    for name, fn in (("fp", lambda: plan.project(x, q, stream=stream)),
                     ("bp", lambda: plan.backproject(b, gg, stream=stream))):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        kt[name] = e0.elapsed_time(e1) / 3 / 1e3
    del q, gg
    vol_b = plan.nrays * NY * 4
    sin_b = NA * NX * NY * 4
    fp_bytes = vol_b + sin_b           # read x, write q
    fp_flops = 2 * 3 * plan.nrays * NY * NA
    peak, peak_kind = peaks()
    dom = "fp" if kt["fp"] >= kt["bp"] else "bp"
    achieved = fp_bytes / kt[dom] / 1e9
    traffic = profiled_traffic().get(dom)
    sm = ck.get("sm_mhz") or 1900.0
    props = torch.cuda.get_device_properties(local)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm * 1e6 / 1e12
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                "peak_source": peak_kind,
                "fp32": {"achieved_tflops": fp_flops / kt[dom] / 1e12,
                         "peak_tflops_at_median_clock": fp32_peak,
                         "frac": fp_flops / kt[dom] / 1e12 / fp32_peak},
                "fp_ms": kt["fp"] * 1e3, "bp_ms": kt["bp"] * 1e3}

    # End to end through the reference-compatible entry point (host buffers).
    e2e = None
    if not args.no_e2e:
        b_host = torch.empty(NA, NY, NX, dtype=torch.float32, pin_memory=True)
        b_host.copy_(b[:, :, :NY].permute(0, 2, 1))
        x_host = torch.empty(plan.nrays, NY, dtype=torch.float32, pin_memory=True)
        L = gb.lib()
        img = gb.ArecImage()
        img.nz, img.ny, img.nx = NA, NY, NX
        img.is_cyl = 0
        img.data = C.cast(C.c_void_p(b_host.data_ptr()), C.POINTER(C.c_float))
        ang = np.ascontiguousarray(angles)

        def e2e_step():
            vol = gb.ArecImage()
            vol.data = C.cast(C.c_void_p(x_host.data_ptr()), C.POINTER(C.c_float))
            # a non-NULL data pointer warm-starts; pass zeros -> identical to a cold start
            x_host.zero_()
            vol.nx = vol.nz = NX
            vol.ny = vol.height = NY
            vol.radius = 0.5 * (NX - 1)
            vol.nrays = plan.nrays
            vol.nnz = plan.nrays * NY
            vol.is_cyl = 1
            st = L.arecgb_cyl_cgls_SQ(0, img, gb._f32p(ang), C.byref(vol), 0.0, MAXIT, TOL)
            assert st == 0, st

        e2e_step()  # plan cache
        t0 = time.perf_counter()
        n_e2e = max(1, min(args.steps, 2))
        for _ in range(n_e2e):
            e2e_step()
        dt = (time.perf_counter() - t0) / n_e2e
        e2e = {"value": world * NY / dt, "unit": "slices/s", "h2d_bytes_per_step": NA * NY * NX * 4,
               "d2h_bytes_per_step": plan.nrays * NY * 4, "ms_per_step": dt * 1e3,
               "note": "cyl_cgls_SQ over pinned host arecImage buffers; zero warm start; "
                       "reference stopping rule (equals the fixed denominator from zero)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        per, info = cpu_sample(slices=16, iters=1)
        cpu_solve = per * NY * (1 + 2 * n_it)
        cpu = {"value": NY / cpu_solve, "unit": "slices/s", "cores": info["threads"],
               "kind": "port",
               "sample": "oracle C restatement of cyl_cgls_SQ: %d slices x 1 iteration on the "
                         "benchmark geometry (%.1f s, %d threads), extrapolated linearly to 512 "
                         "slices x %d iterations" % (info["slices"], info["seconds"],
                                                    info["threads"], n_it)}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "slices/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32", "data": "synthetic (seeded sphere cylinder, analytic chords, "
                                       "Poisson 5e3)",
               "config": dict(CONFIG, iterations=n_it, rel_final=rel_final,
                              parallelism="replicas" if world > 1 else "single"),
               "clocks": ck, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": None}
        # own kernels per step: per iteration 7 vector/scalar + 2 projectors + 2 reductions
        out["gpu_launches"] = args.steps * (n_it * 11 + 4)
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
