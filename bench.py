"""Benchmark: slices/s to relative residual 1e-3 on the 1024^2 x 512-slice,
1200-angle cylinder (square-pixel projector), on one GB300 per rank:
learned-warm-start CGLS (the headline `value`) beside plain CGLS.

One step = one complete reconstruction of the whole volume: the network's
input (the filtered back projection, or the SIRT iterations the weights file
records), the BF16 U-Net warm start (arec3d_gb300/weights), then CGLS from
that guess until ||A^T(b - A x_k)|| / ||A^T b|| <= 1e-3 (the denominator
fixed at its cold-start value) or 200 iterations.  Beside it, on the same
data: `config.plain_cgls` (CGLS from zero), `config.fbp_cgls` (CGLS from the
filtered back projection, no network) and `config.sirt_net_cgls` (the network
trained on SIRT input), each with its error against the phantom.  `--plain`
(or missing weights) makes plain CGLS the headline.  Inputs: a seeded
random-sphere cylinder with analytic line integrals and Poisson noise at 5e3
photons (no public dataset exists).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line on rank 0.  With N > 1 (torchrun) every rank solves its
own replica (the path needs no exchange: replicas only, weak scaling).
`--impl reference` times the reference's CPU algorithm (plain CGLS) for the
same metric on all of this host's cores (the oracle's C restatement, one
thread per slab of slices like the reference's MPI ranks) on a bounded sample
(every slice, a uniform subset of the angles, one iteration) and extrapolates
linearly in angles and iterations.
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
SIRT_ITERS = 10
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


def max_over_ranks(ms, world, device):
    """The job's time is the slowest rank's (all-reduce MAX)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def timed_steps(fn, steps, world, stream=None):
    """Runs fn() `steps` times between a barrier and a device synchronize on
    both sides; returns (ms per step as the maximum over ranks, [fn()
    results]).  Timed with CUDA events on `stream`, or with the host clock when
    stream is None (the CPU ranks of the multi-process tests)."""
    import torch

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    out = []
    barrier()
    if stream is not None:
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            out.append(fn())
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    else:
        t0 = time.perf_counter()
        for _ in range(steps):
            out.append(fn())
        ms = (time.perf_counter() - t0) * 1e3
    barrier()
    return max_over_ranks(ms, world, "cuda" if stream is not None else "cpu") / steps, out


def job_value(world, ms_per_step):
    """Whole-job slices/s: every rank reconstructs its own NY-slice replica."""
    return world * NY / (ms_per_step / 1e3)


# Slices of the headline result whose normal-equation residual the FP64 oracle
# recomputes (slice-separable: the residual is a sum over slices).
FP64_SLICES = (137, 388)


def fp64_check(gb, plan, b_s, x_s, slices):
    """||A^T (b - A x)|| / ||A^T b|| over `slices` of the headline result,
    recomputed with the oracle's FP64 projectors (the checker), beside the same
    quantity evaluated by the GPU projectors in FP32.  b_s: [na][nx][k] and x_s:
    [nrays][k] float32 host arrays of those slices."""
    import torch

    import oracle

    radius = 0.5 * (NX - 1)
    b_ref = np.ascontiguousarray(b_s.transpose(0, 2, 1), np.float64)  # [na][k][nx]
    x64 = np.ascontiguousarray(x_s, np.float64)
    t0 = time.perf_counter()
    with oracle.op_threads():
        atb = oracle.backproject64(3, radius, b_ref, plan.angles)
        r = b_ref - oracle.project64(3, radius, x64, plan.angles)
        atr = oracle.backproject64(3, radius, r, plan.angles)
    rel64 = float(np.linalg.norm(atr) / np.linalg.norm(atb))
    secs = time.perf_counter() - t0
    # the GPU's FP32 evaluation of the same quantity (a plan of k slices)
    k = len(slices)
    old = os.environ.get("ARECGB_PLAN_TABLES")
    os.environ["ARECGB_PLAN_TABLES"] = "0"  # same results without the tables
    try:
        p2 = gb.Plan(gb.SQ, radius, k, plan.angles)
    finally:
        if old is None:
            del os.environ["ARECGB_PLAN_TABLES"]
        else:
            os.environ["ARECGB_PLAN_TABLES"] = old
    bd = torch.zeros(NA, NX, p2.ys, device="cuda")
    bd[:, :, :k] = torch.from_numpy(b_s).cuda()
    xd = torch.zeros(p2.nrays, p2.ys, device="cuda")
    xd[:, :k] = torch.from_numpy(x_s).cuda()
    q = torch.zeros_like(bd)
    p2.project(xd, q)
    g = torch.zeros_like(xd)
    gb_ = torch.zeros_like(xd)
    p2.backproject(bd - q, g)
    p2.backproject(bd, gb_)
    rel32 = float(g.double().norm() / gb_.double().norm())
    p2.close()
    return {"slices": list(slices), "rel_residual_fp64": rel64, "rel_residual_gpu_fp32": rel32,
            "abs_diff": abs(rel64 - rel32), "oracle_seconds": secs,
            "note": "normal-equation residual of the last timed solve over these slices "
                    "(numerator and denominator restricted to them), FP64 oracle projectors "
                    "vs the GPU's FP32 projectors"}


def make_problem(gb, seed, device="cuda"):
    import torch

    from arec3d_gb300 import synthetic as syn

    angles = syn.uniform_angles(NA)
    t0 = time.perf_counter()
    plan = gb.Plan(gb.SQ, 0.5 * (NX - 1), NY, angles)
    plan.create_ms = (time.perf_counter() - t0) * 1e3  # geometry tables + projector tables
    ph = syn.sphere_cylinder_phantom(seed, NX, NY)
    b = syn.sphere_sinogram(ph, NX, NY, angles, ys=plan.ys, device=device)
    syn.poisson_log(b, PHOTONS, seed + 1, NY, device=device)
    torch.cuda.synchronize()
    plan.phantom = ph
    return plan, b, angles


def host_cpu():
    """The host's CPU as the baseline reports it: cores this process may use,
    all online cores, and the model name."""
    import platform

    try:
        usable = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        usable = os.cpu_count() or 1
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as fh:
                for ln in fh:
                    if ln.lower().startswith(("model name", "cpu part")):
                        model = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"usable": usable, "nproc": os.cpu_count(), "model": model or platform.machine(),
            "machine": platform.machine()}


# Angles kept in the CPU sample: every CPU_ANGLE_STEP-th of the 1200.  The
# reference's projectors loop angle by angle with the same work per angle
# (AREC3D/AREC3D/arecproject.cpp:595-645, 698-762), so their time is linear in
# the number of angles; all 512 slices are kept so each rank holds the slab it
# would hold in the full run (the per-(ray, angle) weights are shared by the
# slab's slices, as in the reference).
CPU_ANGLE_STEP = 50


def cpu_sample(threads=None, iters=1, slices=NY, angle_step=CPU_ANGLE_STEP):
    """Reference CGLS (the oracle's C restatement of cyl_cgls_SQ, one thread
    per slab of slices like the reference's MPI ranks) on the benchmark
    geometry with every `angle_step`-th angle; returns seconds per slice per
    full-size projector pass (scaled to all 1200 angles) and the sample's
    description."""
    import oracle

    oracle.build()
    cpu = host_cpu()
    threads = threads or cpu["usable"]
    rng = np.random.default_rng(0)
    angles = (np.arange(0, NA, angle_step) * (np.pi / NA)).astype(np.float32)
    b = (rng.random((len(angles), slices, NX), dtype=np.float32) * 2.0).astype(np.float32)
    t0 = time.perf_counter()
    oracle.cgls(3, b, angles, maxit=iters, tol=0.0, nthreads=threads)
    dt = time.perf_counter() - t0
    passes = 1 + 2 * iters  # initial A^T s, then A p and A^T s per iteration
    per = dt * (NA / len(angles)) / (slices * passes)
    return per, {"slices": slices, "angles": len(angles), "iterations": iters,
                 "threads": threads, "seconds": dt, "cpu": cpu}


def cpu_sample_text(info, n_it):
    return ("oracle C restatement of cyl_cgls_SQ (bit-identical to the reference build), "
            "%d ranks (threads) x slabs of the %d slices, %d of the 1200 angles (every %dth), "
            "%d iteration: %.1f s, extrapolated linearly to 1200 angles x %d iterations "
            "(plain CGLS to 1e-3); host %s, %d usable of %s cores"
            % (info["threads"], info["slices"], info["angles"], NA // info["angles"],
               info["iterations"], info["seconds"], n_it, info["cpu"]["model"],
               info["cpu"]["usable"], info["cpu"]["nproc"]))


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU algorithm on this host's cores."""
    if rank != 0:
        return
    it_gpu = args.ref_iters
    times = []
    info = None
    for i in range(args.warmup + args.steps):
        per, info = cpu_sample(angle_step=args.ref_angle_step)
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
                         "kind": "port", "host": info["cpu"],
                         "sample": "per step: " + cpu_sample_text(info, it_gpu)},
        "e2e": {"value": value, "unit": "slices/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def extra_config(args):
    """Measurements of the other benchmark configurations (one JSON line each;
    not the headline): 1 = SIRT x50 at 256^2 x 64 slices / 180 angles;
    3 = shift search over 720 pairs of 2048^2 images; 5 = the uneven batch of
    64 cylinders (uneven_batch)."""
    import math

    import torch

    import arec3d_gb300 as gb
    from arec3d_gb300 import synthetic as syn
    from arec3d_gb300 import warmstart as ws

    gb.build()
    st = torch.cuda.current_stream()

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            out = fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, out

    if args.config == 1:
        nx, ny, na = 256, 64, 180
        angles = syn.uniform_angles(na)
        plan = gb.Plan(gb.SQ, 0.5 * (nx - 1), ny, angles)
        ph = syn.ellipse_phantom(7, nx, ny)
        b = syn.ellipse_sinogram(ph, nx, ny, angles, ys=plan.ys)
        syn.poisson_log(b, 1e4, 8, ny)
        x = torch.zeros(plan.nrays, plan.ys, device="cuda")
        ms, (hist, info) = timed(lambda: plan.sirt(b, x, 5e-6, 50, 0.0, stream=st), args.steps)
        out = {"config": 1, "workload": "SIRT x50 (lam 5e-6, tol 0), square-pixel, 256^2 x 64 "
               "slices, 180 angles, 10 ellipses per slice, Poisson 1e4",
               "value": ny / (ms / 1e3), "unit": "slices/s", "ms_per_solve": ms,
               "iterations": info.iterations, "restarts": info.restarts}
    elif args.config == 3:
        n, size = args.pairs, 2048
        g = torch.Generator(device="cuda")
        g.manual_seed(3)
        ky = torch.fft.fftfreq(size, device="cuda")[:, None]
        kx = torch.fft.fftfreq(size, device="cuda")[None, :]
        lowpass = torch.exp(-((kx ** 2 + ky ** 2) / (2 * 0.02 ** 2)))
        a = torch.empty(n, size, size, device="cuda")
        bimg = torch.empty_like(a)
        shifts = []
        rng = np.random.default_rng(3)
        for i in range(0, n, 16):
            k = min(16, n - i)
            noise = torch.randn(k, size, size, device="cuda", generator=g)
            spec = torch.fft.fft2(noise) * lowpass
            sy = rng.integers(-20, 21, k) + rng.uniform(-0.5, 0.5, k)
            sx = rng.integers(-20, 21, k) + rng.uniform(-0.5, 0.5, k)
            shifts += list(zip(sx, sy))
            ramp = torch.exp(-2j * math.pi * (ky[None] * torch.tensor(sy, device="cuda")[:, None, None]
                                             + kx[None] * torch.tensor(sx, device="cuda")[:, None, None]))
            a[i:i + k] = torch.fft.ifft2(spec).real
            img = torch.fft.ifft2(spec * ramp).real
            bimg[i:i + k] = img + 0.02 * img.std() * torch.randn(k, size, size, device="cuda",
                                                                generator=g)
        sxo = torch.zeros(n, device="cuda")
        syo = torch.zeros(n, device="cuda")
        ms, _ = timed(lambda: gb.cc_shifts(a, bimg, sxo, syo, stream=st), args.steps)
        err = np.abs(np.array(shifts) - np.stack([sxo.cpu().numpy(), syo.cpu().numpy()], 1))
        out = {"config": 3, "workload": "shift search, %d pairs of 2048^2 float images "
               "(integer shifts +-20 px plus sub-pixel +-0.5 px, 2%% noise)" % n,
               "value": n / (ms / 1e3), "unit": "pairs/s", "ms_per_stack": ms,
               "hbm_gbs": n * 2 * 4 * size * size / (ms / 1e3) / 1e9,
               "max_abs_shift_error_px": float(err.max())}
    else:
        out = uneven_batch(args, gb, syn, ws, timed)
    print(json.dumps(out))


def uneven_batch(args, gb, syn, ws, timed):
    """Config 5: 64 cylinders (radius U[128, 1024] px, detector 2 r + 16 bins,
    32-512 slices, 360-1800 angles over [0, 180), random-sphere phantoms at
    5e3 photons; problem 0 the largest instance the configuration names,
    r = 1024 with 512 slices and 1800 angles), solved together by the
    library's scheduler (arecgb_solve_uneven): waves of problems whose solver
    workspace fits the budget, each wave's problems warm-started by the
    network (one size per width class) and solved by one batched CGLS (one
    CUDA graph launch per iteration for the whole wave) to 1e-3.  Inputs and
    results stay resident in HBM."""
    import torch

    rng = np.random.default_rng(5)
    k = args.batch_problems
    specs = [(1024.0, 512, 1800)]
    for _ in range(k - 1):
        specs.append((float(rng.uniform(128, 1024)), int(rng.integers(32, 513)),
                      int(rng.integers(360, 1801))))
    scale = args.c5_scale
    problems, slices = [], 0
    t0 = time.perf_counter()
    for i, (r, ny, na) in enumerate(specs):
        r = max(16.0, r * scale)
        ny = max(8, int(ny * scale)) if scale < 1 else ny
        nx = int(2 * round(r) + 16)
        radius = 0.5 * (nx - 1)
        angles = syn.uniform_angles(na)
        _, nr, ys = gb.cylinder_info(radius, ny)
        nsph = max(8, int(round(200 * (r / 500.0) ** 2 * ny / 512)))
        ph = syn.sphere_cylinder_phantom(500 + i, nx, ny, n_spheres=nsph, cyl_radius=r - 4,
                                         r_max=min(80.0, 0.5 * (r - 4)))
        b = syn.sphere_sinogram(ph, nx, ny, angles, ys=ys)
        syn.poisson_log(b, 5e3, 700 + i, ny)
        x = torch.zeros(nr, ys, device="cuda")
        problems.append(dict(radius=radius, ny=ny, angles=angles, b=b, x=x, nx=nx, na=na))
        slices += ny
        if (i + 1) % 8 == 0:
            torch.cuda.synchronize()
            print("config 5: %d problems generated, %.1f s" % (i + 1, time.perf_counter() - t0),
                  file=sys.stderr, flush=True)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    nets = []
    if not args.plain and os.path.exists(args.weights):
        widths = sorted({p["nx"] for p in problems})
        lo = 0
        for size, batch in ((512, 16), (1024, 8), (2072, 4)):
            if any(lo < w <= size for w in widths):
                net, _ = ws.load(gb, args.weights, size, batch)
                nets.append(net)
            lo = size
    free, total = torch.cuda.mem_get_info()
    budget = int(args.c5_budget_gb * 1e9) if args.c5_budget_gb else int(0.8 * free) - (2 << 30)
    st = torch.cuda.current_stream()

    def run():
        return gb.solve_uneven(problems, budget, maxit=MAXIT, tol=TOL, nets=nets, stream=st)

    # one timed pass (a pass is minutes long at full size; no separate warm-up)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    infos, waves = run()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    seq = None
    if args.c5_sequential:
        # the same problems solved one at a time through the same scheduler (a
        # wave of one, one graph per iteration with a single branch), for the
        # batched launch's overlap
        for p in problems:
            p["x"].zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        seq_it = []
        for p in problems:
            inf1, _ = gb.solve_uneven([p], budget, maxit=MAXIT, tol=TOL, nets=nets, stream=st)
            seq_it.append(inf1[0].iterations)
        torch.cuda.synchronize()
        seq = {"ms": (time.perf_counter() - t0) * 1e3,
               "same_iterations": seq_it == [inf.iterations for inf in infos]}
    out = {"config": 5,
           "workload": "uneven batch: %d cylinders, radius 128-1024 px (problem 0: 1024, 512 "
                       "slices, 1800 angles), detector 2r+16 bins, 32-512 slices, 360-1800 "
                       "angles, random spheres, Poisson 5e3; %s CGLS to 1e-3 (max %d it), "
                       "waves under a %.0f GB workspace budget"
                       % (k, "learned warm start +" if nets else "plain", MAXIT, budget / 1e9),
           "value": slices / (ms / 1e3), "unit": "slices/s", "ms_per_batch": ms,
           "slices": slices, "waves": max(waves) + 1, "setup_s": gen_s,
           "resident_gb": sum(p["b"].numel() + p["x"].numel() for p in problems) * 4 / 1e9,
           "scale": scale,
           "sequential": seq,
           "problems": [{"nx": p["nx"], "slices": p["ny"], "angles": p["na"],
                         "iterations": inf.iterations, "rel_final": inf.rel_final, "wave": w}
                        for p, inf, w in zip(problems, infos, waves)]}
    return out


def unet_only(args):
    """U-Net inference on --launches batches of 16 images of 1024^2 (the warm
    start's network and batch), for profiling."""
    import torch

    import arec3d_gb300 as gb
    from arec3d_gb300 import warmstart as ws

    gb.build()
    net, _ = ws.load(gb, args.weights, NX, 16)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    x = torch.rand(16, NX, NX, device="cuda", generator=g)
    y = torch.empty_like(x)
    for _ in range(args.launches):
        net.forward(x, y)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.launches):
        net.forward(x, y)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.launches
    flops = 2 * 188928 * 16 * NX * NX  # multiply-adds of the 3x3 layers per pixel x 2
    print(json.dumps({"unet_only": True, "ms_per_16_images": ms,
                      "tensor_tflops": flops / (ms / 1e3) / 1e12,
                      "checksum": float(y.double().sum())}))


def kernels_only(args):
    """Forward and back projector of the benchmark geometry on `--slices`
    slices, `--launches` times each (a short command for ncu)."""
    import torch

    import arec3d_gb300 as gb
    from arec3d_gb300 import synthetic as syn

    gb.build()
    angles = syn.uniform_angles(args.angles)
    plan = gb.Plan(gb.SQ, 0.5 * (args.nx - 1), args.slices, angles)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    x = torch.rand(plan.nrays, plan.ys, device="cuda", generator=g)
    x[:, args.slices:] = 0
    q = torch.zeros(plan.nangles, plan.nx, plan.ys, device="cuda")
    n2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    tuned = None
    if args.shapes:
        plan.set_shapes(*[int(v) for v in args.shapes.split(",")])
        tuned = plan.shapes()
    if args.tune:
        plan.autotune(x, q)
        tuned = plan.shapes()
        x.uniform_(generator=g)
        x[:, args.slices:] = 0
    if not args.tune:  # one untimed pair: module loading on first launch
        plan.project(x, q, norm2=n2)
        plan.backproject(q, x, norm2=n2)
    plan.timing(1)
    for _ in range(args.launches):
        plan.project(x, q, norm2=n2)
        plan.backproject(q, x, norm2=n2)
    torch.cuda.synchronize()
    fp_ms, fp_n, bp_ms, bp_n = plan.timing(0)
    print(json.dumps({"kernels_only": True, "slices": args.slices, "launches": args.launches,
                      "fp_ms": fp_ms / max(fp_n, 1), "bp_ms": bp_ms / max(bp_n, 1),
                      "autotuned": tuned,
                      "norm2": float(n2.item())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ref-angle-step", type=int, default=CPU_ANGLE_STEP,
                    help="reference arm: keep every k-th angle in each step's CPU sample")
    ap.add_argument("--ref-iters", type=int, default=32,
                    help="iterations to extrapolate the reference arm to (plain CGLS needs 32 "
                         "on this problem)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="run only the forward and back projectors (for profiling)")
    ap.add_argument("--slices", type=int, default=NY, help="slices for --kernels-only")
    ap.add_argument("--launches", type=int, default=3, help="launches for --kernels-only")
    ap.add_argument("--tune", action="store_true", help="--kernels-only: autotune first")
    ap.add_argument("--shapes", default="", help="--kernels-only: band,fp_vec,bp_vec,chunks")
    ap.add_argument("--angles", type=int, default=NA, help="angles for --kernels-only")
    ap.add_argument("--nx", type=int, default=NX, help="detector bins for --kernels-only")
    ap.add_argument("--plain", action="store_true", help="plain CGLS only (no warm start)")
    ap.add_argument("--profile-step", action="store_true",
                    help="after the warm-up, run one headline step and exit (for ncu)")
    ap.add_argument("--config", type=int, default=0, choices=[0, 1, 3, 5],
                    help="measure another benchmark configuration instead of the headline")
    ap.add_argument("--batch-problems", type=int, default=64, help="problems for --config 5")
    ap.add_argument("--c5-scale", type=float, default=1.0,
                    help="--config 5: scale radii (and slices below 1) for a smaller test run")
    ap.add_argument("--c5-sequential", action="store_true",
                    help="--config 5: also solve the problems one at a time, for comparison")
    ap.add_argument("--c5-budget-gb", type=float, default=0.0,
                    help="--config 5: solver workspace budget (default: most of the free HBM)")
    ap.add_argument("--pairs", type=int, default=720, help="image pairs for --config 3")
    ap.add_argument("--unet-only", action="store_true",
                    help="run only the warm-start network's inference (for profiling)")
    ap.add_argument("--weights", default=os.path.join(ROOT, "arec3d_gb300", "weights",
                                                      "unet_warm_start.npz"))
    ap.add_argument("--weights-sirt", default=os.path.join(ROOT, "arec3d_gb300", "weights",
                                                           "unet_warm_start_sirt4.npz"),
                    help="the network trained on SIRT input, timed beside the headline")
    args = ap.parse_args()
    rank, local, world = dist_env()
    if args.kernels_only:
        kernels_only(args)
        return
    if args.unet_only:
        unet_only(args)
        return
    if args.config:
        extra_config(args)
        return

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch

    import math

    import arec3d_gb300 as gb
    from arec3d_gb300 import synthetic as syn
    from arec3d_gb300 import warmstart as ws

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    # the e2e leg's page-locked host buffers, allocated first: on the GPU machine's
    # virtual machine a page-locked buffer allocated after gigabytes of host
    # traffic uploaded at a fraction of the speed of one allocated early
    gb.build()
    b_host = x_host = None
    if not args.no_e2e and not args.profile_step:
        _, nr0, _ = gb.cylinder_info(0.5 * (NX - 1), NY)
        b_host = torch.empty(NA, NY, NX, dtype=torch.float32, pin_memory=True)
        x_host = torch.empty(nr0, NY, dtype=torch.float32, pin_memory=True)
    plan, b, angles = make_problem(gb, seed=1000 + rank)
    x = torch.zeros(plan.nrays, plan.ys, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    lam = ws.sirt_lambda(plan)
    # launch shapes from the library's autotuner (scratch buffers, before any timing)
    q_tmp = torch.zeros(plan.nangles, plan.nx, plan.ys, dtype=torch.float32, device="cuda")
    plan.autotune(x, q_tmp, stream=stream)
    tuned = plan.shapes()
    del q_tmp
    x.zero_()

    # the learned warm start: committed weights, inference net over 16 slices at a time
    net, meta = None, {}
    npix = 16 * plan.nx * plan.nx
    if not args.plain and os.path.exists(args.weights):
        net, meta = ws.load(gb, args.weights, plan.nx, 16)
        scratch = (torch.empty(npix, device="cuda"), torch.empty(npix, device="cuda"))
    work = torch.empty_like(b)     # the filtered sinogram
    atb2 = torch.zeros(1, dtype=torch.float64, device="cuda")

    def solve_plain():
        hist, info = plan.cgls(b, x, MAXIT, TOL, stream=stream)
        return info

    def first_reconstruction(kind, iters, lam):
        """FBP or SIRT from zero into x; returns ||A^T b|| (both compute it)."""
        if kind == "fbp":
            plan.fbp(b, x, work, atb_norm2=atb2, stream=stream)
            return math.sqrt(float(atb2.item()))
        _, sinfo = plan.sirt(b, x, lam, iters, 0.0, stream=stream)
        return sinfo.rnorm0

    def warm_pipeline(nt, stage_ev=None):
        kind = getattr(nt, "input", "fbp") if nt is not None else "fbp"
        iters = getattr(nt, "sirt_iters", SIRT_ITERS)
        lam_n = ws.sirt_lambda(plan, getattr(nt, "sirt_lam_scale", 1.0))

        def solve():
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record(stream)
            rn = first_reconstruction(kind, iters, lam_n)
            ev[1].record(stream)
            if nt is not None:
                nt.warm_start(plan, x, x, scratch[0], scratch[1], stream=stream)
            ev[2].record(stream)
            hist, info = plan.cgls(b, x, MAXIT, TOL, warm=True, rnorm_ref=rn, stream=stream)
            ev[3].record(stream)
            if stage_ev is not None:
                stage_ev.append(ev)
            return info
        return solve

    stage_ev = []  # per step: events after the input, after the U-Net, after CGLS
    solve = warm_pipeline(net, stage_ev) if net is not None else solve_plain
    sirt_iters = getattr(net, "sirt_iters", SIRT_ITERS) if net is not None else 0
    lam = ws.sirt_lambda(plan, getattr(net, "sirt_lam_scale", 1.0))

    for _ in range(args.warmup):
        solve()
    stage_ev.clear()
    if args.profile_step:  # one more step alone, for a launch list (no timing, no JSON)
        n0 = gb.launch_count()
        torch.cuda.synchronize()
        info = solve()
        torch.cuda.synchronize()
        print(json.dumps({"profile_step": True, "launches": gb.launch_count() - n0,
                          "iterations": info.iterations}))
        return
    # timed region: the headline pipeline, with projector timing and clocks
    clocks = ClockSampler(local)
    clocks.start()
    plan.timing(1)
    n0 = gb.launch_count()
    ms_step, infos = timed_steps(solve, args.steps, world, stream)
    launches = gb.launch_count() - n0
    fp_ms, fp_calls, bp_ms, bp_calls = plan.timing(0)
    ck = clocks.stop()
    value = job_value(world, ms_step)
    n_it = int(statistics.median([i.iterations for i in infos]))
    rel_final = float(infos[-1].rel_final)
    stages = None
    if stage_ev:
        stages = {k: statistics.mean(ev[j].elapsed_time(ev[j + 1]) for ev in stage_ev)
                  for j, k in enumerate(("input_ms", "unet_ms", "cgls_ms"))}
    # the headline result on a few slices, kept for the FP64 check below
    keep = list(FP64_SLICES)
    x_keep = x[:, keep].contiguous().cpu().numpy()
    b_keep = b[:, :, keep].contiguous().cpu().numpy()
    truth = syn.sphere_volume(plan.phantom, 0.5 * (NX - 1), NY, plan.ys)
    tnorm = float(truth[:, :NY].double().pow(2).sum().sqrt())

    def err_truth():
        return float((x[:, :NY].double() - truth[:, :NY].double()).pow(2).sum().sqrt()) / tnorm

    err_headline = err_truth()

    # End to end through one C-ABI call over page-locked host buffers in the
    # reference's layouts (arecgb_reconstruct_host): every step the sinogram
    # [angle][slice][bin] goes up, the warm start and CGLS run, and the
    # volume [ray][slice] comes back; host-clock time around the call.  Run
    # right after the headline: on the GPU machine's virtual machine page-locked
    # transfers slowed down after the comparison pipelines' gigabytes of traffic.
    e2e = None
    if not args.no_e2e:
        b_host.copy_(b[:, :, :NY].permute(0, 2, 1))

        def e2e_step():
            return plan.reconstruct_host(b_host, x_host, net, sirt_iters, lam, MAXIT, TOL,
                                         stream=stream)

        e2e_step()
        n_e2e = max(1, min(args.steps, 2))
        e2e_ms, e2e_infos = timed_steps(e2e_step, n_e2e, world, None)
        # the two copies alone, timed the same way, for the breakdown
        b_scr = torch.empty(NA, NY, NX, dtype=torch.float32, device="cuda")
        x_scr = torch.empty(plan.nrays, NY, dtype=torch.float32, device="cuda")
        h2d_ms, _ = timed_steps(lambda: b_scr.copy_(b_host, non_blocking=True), 3, 1, stream)
        d2h_ms, _ = timed_steps(lambda: x_host.copy_(x_scr, non_blocking=True), 3, 1, stream)
        del b_scr, x_scr
        e2e = {"value": job_value(world, e2e_ms), "unit": "slices/s",
               "h2d_bytes_per_step": NA * NY * NX * 4,
               "d2h_bytes_per_step": plan.nrays * NY * 4, "ms_per_step": e2e_ms,
               "iterations": int(statistics.median([i.iterations for i in e2e_infos])),
               "h2d_copy_ms": h2d_ms, "d2h_copy_ms": d2h_ms,
               "h2d_gbs": NA * NY * NX * 4 / (h2d_ms / 1e3) / 1e9,
               "d2h_gbs": plan.nrays * NY * 4 / (d2h_ms / 1e3) / 1e9,
               "path": "pinned host sinogram [angle][slice][bin] -> arecgb_reconstruct_host ("
                       + (("filtered back projection" if sirt_iters == 0 else "SIRT")
                          + " -> warm start -> CGLS" if net is not None else "CGLS")
                       + ") -> pinned host volume [ray][slice]"}

    # the other pipelines beside it, same data (untimed warm-up, then 1-2 steps)
    def compare(fn):
        fn()
        pm, pinfos = timed_steps(fn, max(1, min(args.steps, 2)), world, stream)
        return {"slices_per_s": job_value(world, pm), "ms_per_solve": pm,
                "iterations": int(statistics.median([i.iterations for i in pinfos])),
                "error_vs_phantom": err_truth()}

    plain = fbp_only = sirt_net = None
    if net is not None:
        plain = compare(solve_plain)
        fbp_only = compare(warm_pipeline(None))
        if os.path.exists(args.weights_sirt):
            net_s, meta_s = ws.load(gb, args.weights_sirt, plan.nx, 16)
            sirt_net = compare(warm_pipeline(net_s))
            sirt_net.update(input="SIRT-%d" % net_s.sirt_iters,
                            weights=os.path.relpath(args.weights_sirt, ROOT))
            del net_s
        for d in (plain, fbp_only, sirt_net):
            if d:
                d["speedup_vs_plain"] = d["slices_per_s"] / plain["slices_per_s"]
    del truth

    # Roofline of the dominant kernel from the projector times recorded in the
    # timed region.  Unit: one projection (the forward projector is 32 band
    # launches; per-launch figures divide both bytes and time by the same count).
    vol_b = plan.nrays * NY * 4
    sin_b = NA * NX * NY * 4
    algo_bytes = vol_b + sin_b            # compulsory: read x (s), write q (g)
    flops = 2 * 3 * plan.nrays * NY * NA  # 3 taps per (ray, angle, slice)
    fp_avg = fp_ms / max(fp_calls, 1) / 1e3
    bp_avg = bp_ms / max(bp_calls, 1) / 1e3
    dom = "fp" if fp_ms >= bp_ms else "bp"
    t_dom = fp_avg if dom == "fp" else bp_avg
    peak, peak_kind = peaks()
    achieved = algo_bytes / t_dom / 1e9
    sm = ck.get("sm_mhz") or 1900.0
    props = torch.cuda.get_device_properties(local)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm * 1e6 / 1e12
    traffic = profiled_traffic().get(dom)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "kernel": "fp_band_kernel (one forward projection)" if dom == "fp"
                else "bp_kernel (one back projection)",
                "peak_source": peak_kind,
                "algorithmic_bytes_per_projection": algo_bytes,
                "fp32": {"achieved_tflops": flops / t_dom / 1e12,
                         "peak_tflops_at_median_clock": fp32_peak,
                         "frac": flops / t_dom / 1e12 / fp32_peak},
                "fp_ms": fp_avg * 1e3, "bp_ms": bp_avg * 1e3,
                "fp_calls": fp_calls, "bp_calls": bp_calls,
                # projections per step: the timed (non-graph) calls plus one forward and
                # one back projection per CGLS iteration replayed from the CUDA graph
                # (the first iteration runs eagerly and is among the timed calls)
                "projector_ms_per_step": (fp_avg * (fp_calls / args.steps + max(n_it - 1, 0)) +
                                          bp_avg * (bp_calls / args.steps + max(n_it - 1, 0)))
                * 1e3,
                "projector_share_of_step": (fp_avg * (fp_calls / args.steps + max(n_it - 1, 0)) +
                                            bp_avg * (bp_calls / args.steps + max(n_it - 1, 0)))
                * 1e3 / ms_step}

    cpu = None
    fp64 = None
    if rank == 0 and not args.no_cpu:
        n_cpu_it = plain["iterations"] if plain else n_it
        per, cinfo = cpu_sample()
        cpu_solve = per * NY * (1 + 2 * n_cpu_it)
        cpu = {"value": NY / cpu_solve, "unit": "slices/s", "cores": cinfo["threads"],
               "kind": "port", "host": cinfo["cpu"], "sample": cpu_sample_text(cinfo, n_cpu_it)}
        # the oracle as the checker of the headline result: its FP64 projectors
        # recompute the normal-equation residual of the last timed solve on a
        # few slices (the residual is a sum over slices)
        fp64 = fp64_check(gb, plan, b_keep, x_keep, keep)

    if rank == 0:
        cfg = dict(CONFIG, iterations=n_it, rel_final=rel_final,
                   parallelism="replicas" if world > 1 else "single",
                   autotuned={"fp_band_lines": tuned[0], "fp_vec": tuned[1], "bp_vec": tuned[2],
                              "bp_slice_chunks": tuned[3]},
                   plan={"projector_tables_gb": plan.table_bytes() / 1e9,
                         "create_ms": getattr(plan, "create_ms", None),
                         "note": "created once per geometry, outside the timed region"})
        cfg["fp64_check"] = fp64
        cfg["error_vs_phantom"] = err_headline
        if net is not None:
            first = "filtered back projection" if sirt_iters == 0 else "SIRT-%d" % sirt_iters
            cfg.update(warm_start=True, network_input=first, stage_ms=stages,
                       workload="learned warm start: %s -> BF16 U-Net -> CGLS to "
                                "||A^T r||/||A^T b|| <= 1e-3 (max 200 it), square-pixel "
                                "projector, 1024^2 x 512 slices, 1200 angles over [0,180), "
                                "random-sphere cylinder r=500 px with 200 spheres, Poisson 5e3 "
                                "photons" % first,
                       plain_cgls=plain, fbp_cgls=fbp_only, sirt_net_cgls=sirt_net,
                       speedup_vs_plain=(value / plain["slices_per_s"]) if plain else None,
                       weights=os.path.relpath(args.weights, ROOT),
                       weights_meta={k: meta.get(k) for k in ("input", "sets", "steps",
                                                              "final_loss")})
        out = {"metric": METRIC, "value": value, "unit": "slices/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32", "data": "synthetic (seeded sphere cylinder, analytic chords, "
                                       "Poisson 5e3)",
               "config": cfg, "clocks": ck, "roofline": roofline, "cpu_baseline": cpu,
               "e2e": e2e, "gpu_launches": launches}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
