"""Learned warm start: training pairs made by the method itself, training of
the U-Net on the GPU, and the warm-started solve, all through the library's C
ABI (arecgb_sirt, arecgb_cgls, arecgb_unet_*, arecgb_warm_start).

A pair is one synthetic volume reconstructed twice from the same noisy data:
a cheap first reconstruction (the network input: a few SIRT iterations, or
the filtered back projection) and many CGLS iterations (the target).  Images are the cylinder's slices on a zero-padded square grid,
normalised by the RMS of the SIRT volume over the cylinder, the normalisation
arecgb_warm_start applies at inference.  Plain CGLS then continues from the
network's output to the same residual tolerance, so the solver still decides
the result (and is the fallback: a bad guess costs iterations, not accuracy).

torch is used only to hold device memory and pick training crops.

    python -m arec3d_gb300.warmstart --input fbp --out arec3d_gb300/weights/unet_warm_start.npz
"""
import argparse
import json
import math
import os
import time

import numpy as np

from . import synthetic as syn

DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights",
                               "unet_warm_start.npz")
SIRT_ITERS = 10
CGLS_ITERS = 200


def sirt_lambda(plan, scale=1.0):
    """Landweber step scale / (nangles * nx), below the stability limit
    2 / ||A||^2 for scale < 2 (||A||^2 ~ nangles * chord length)."""
    return scale / (plan.nangles * plan.nx)


def pad8(n):
    return (n + 7) // 8 * 8


def volume_rms(plan, x):
    return float(x[:, :plan.ny].double().pow(2).sum().sqrt()) / math.sqrt(plan.nrays * plan.ny)


def make_problem(gb, nx, na, slices, photons, seed, kind="sphere", device="cuda"):
    """Seeded phantom -> noisy sinogram b (device layout) and its plan."""
    angles = syn.uniform_angles(na)
    plan = gb.Plan(gb.SQ, 0.5 * (nx - 1), slices, angles)
    if kind == "sphere":
        ph = syn.sphere_cylinder_phantom(seed, nx, slices)
        b = syn.sphere_sinogram(ph, nx, slices, angles, ys=plan.ys, device=device)
    else:
        ph = syn.ellipse_phantom(seed, nx, slices, centre_radius=0.3 * nx,
                                 a_min=5.0 * nx / 512.0, a_max=60.0 * nx / 512.0)
        b = syn.ellipse_sinogram(ph, nx, slices, angles, ys=plan.ys, device=device)
    syn.poisson_log(b, photons, seed + 1, slices, device=device)
    return plan, b


def first_reconstruction(plan, b, x, inp, lam_scale=1.0, work=None):
    """The network input: inp "fbp" (filtered back projection) or an int k
    (k SIRT iterations from zero at step lam_scale / (nangles nx)).  Returns
    ||A^T b||, the cold start's CGLS denominator, which both compute."""
    import torch

    if inp == "fbp":
        n2 = torch.zeros(1, dtype=torch.float64, device="cuda")
        plan.fbp(b, x, torch.empty_like(b) if work is None else work, atb_norm2=n2)
        return math.sqrt(float(n2.item()))
    _, sinfo = plan.sirt(b, x, sirt_lambda(plan, lam_scale), int(inp), 0.0)
    return sinfo.rnorm0


def make_pairs(gb, nx, na, slices, photons, seed, kind="sphere", sirt_iters=(SIRT_ITERS,),
               cgls_iters=CGLS_ITERS, lam_scale=1.0):
    """{k: (input, target)} image stacks [slices][npad][npad] on the device, one
    pair per input k in `sirt_iters` (a SIRT depth, or "fbp"; the CGLS target
    is shared)."""
    import torch

    plan, b = make_problem(gb, nx, na, slices, photons, seed, kind)
    xc = torch.zeros(plan.nrays, plan.ys, device="cuda")
    plan.cgls(b, xc, cgls_iters, 0.0)
    xs = torch.zeros_like(xc)
    npad = pad8(plan.nx)
    out = {}
    for k in sirt_iters:
        xs.zero_()
        first_reconstruction(plan, b, xs, k, lam_scale)
        rms = volume_rms(plan, xs)
        inp = torch.empty(slices, npad, npad, device="cuda")
        tgt = torch.empty_like(inp)
        gb.images_from_volume(plan, xs, inp, npad, 0, slices, 1.0 / rms)
        gb.images_from_volume(plan, xc, tgt, npad, 0, slices, 1.0 / rms)
        out[k] = (inp, tgt)
    torch.cuda.synchronize()
    return out


def random_crops(gen, inp, tgt, batch, crop, out_in, out_tgt):
    """Random crop-aligned windows (multiples of 8) of random slices."""
    import torch

    n, h, w = inp.shape
    idx = torch.randint(0, n, (batch,), generator=gen).tolist()
    ys = torch.randint(0, (h - crop) // 8 + 1, (batch,), generator=gen).tolist()
    xs = torch.randint(0, (w - crop) // 8 + 1, (batch,), generator=gen).tolist()
    for k in range(batch):
        y0, x0 = 8 * ys[k], 8 * xs[k]
        out_in[k].copy_(inp[idx[k], y0:y0 + crop, x0:x0 + crop])
        out_tgt[k].copy_(tgt[idx[k], y0:y0 + crop, x0:x0 + crop])


def train(gb, datasets, steps=2000, batch=16, crop=256, lr=1e-3, weight_decay=1e-4, seed=0,
          log_every=100, net=None):
    """AdamW on the MSE between net(input) and target over random crops drawn
    from `datasets` (a list of (input, target) stacks, sampled in turn);
    cosine learning-rate decay.  Returns (net, loss history)."""
    import torch

    net = net or gb.UNet(crop, batch, train=True, seed=seed)
    gen = torch.Generator()
    gen.manual_seed(seed)
    xi = torch.empty(batch, crop, crop, device="cuda")
    xt = torch.empty_like(xi)
    hist = []
    t0 = time.time()
    for s in range(steps):
        inp, tgt = datasets[s % len(datasets)]
        random_crops(gen, inp, tgt, batch, crop, xi, xt)
        lr_s = lr * 0.5 * (1.0 + math.cos(math.pi * s / steps))
        loss = net.train_step(xi, xt, lr_s, weight_decay)
        hist.append(loss)
        if log_every and (s % log_every == 0 or s == steps - 1):
            print("step %5d  loss %.4e  lr %.2e  %.1fs" % (s, loss, lr_s, time.time() - t0),
                  flush=True)
    return net, hist


def save(net, path, meta=None):
    """Parameters rounded to bf16 (the precision the network computes in),
    stored as uint16 bit patterns, with the layer table and metadata."""
    import torch

    p = torch.zeros(net.nparams, device="cuda")
    net.get_params(p)
    bits = p.cpu().numpy().view(np.uint32)
    rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params_bf16=rounded, meta=json.dumps(meta or {}),
                        layers=json.dumps(net.layers))


def load(gb, path, size, max_batch):
    """An inference net of `size` x `size` images with saved parameters."""
    import torch

    z = np.load(path)
    bits = z["params_bf16"].astype(np.uint32) << 16
    params = bits.view(np.float32)
    net = gb.UNet(size, max_batch, train=False)
    if net.nparams != params.size or json.loads(str(z["layers"])) != net.layers:
        raise ValueError("%s: parameter layout does not match this library's network" % path)
    net.set_params(torch.from_numpy(params.copy()).cuda())
    meta = json.loads(str(z["meta"]))
    net.input = "fbp" if meta.get("input") == "fbp" else "sirt"
    net.sirt_iters = 0 if net.input == "fbp" else int(meta.get("sirt_iters", SIRT_ITERS))
    net.sirt_lam_scale = float(meta.get("sirt_lam_scale", 1.0))
    return net, meta


def solve(gb, plan, b, x, net=None, tol=1e-3, maxit=200, sirt_iters=None, scratch=None,
          start=None):
    """CGLS to ||A^T r|| / ||A^T b|| <= tol, warm-started by the network when
    `net` is given (first reconstruction -> U-Net -> CGLS: the network's input
    kind, SIRT or the filtered back projection, is in its metadata), from the
    filtered back projection alone with start="fbp", else from zero.  Returns
    (CGLS info, seconds of each stage: "input" for the first reconstruction)."""
    import torch

    st = {}
    t = time.perf_counter()
    rnorm_ref = 0.0
    if net is not None or start == "fbp":
        if start == "fbp" or getattr(net, "input", "sirt") == "fbp":
            inp = "fbp"
        else:
            inp = sirt_iters if sirt_iters is not None else getattr(net, "sirt_iters", SIRT_ITERS)
        rnorm_ref = first_reconstruction(plan, b, x, inp, getattr(net, "sirt_lam_scale", 1.0),
                                         work=scratch[2] if scratch and len(scratch) > 2 else None)
        torch.cuda.synchronize()
        st["input"] = time.perf_counter() - t
        t = time.perf_counter()
    if net is not None:
        if scratch is None:
            npix = net.max_batch * net.size * net.size
            scratch = (torch.empty(npix, device="cuda"), torch.empty(npix, device="cuda"))
        net.warm_start(plan, x, x, scratch[0], scratch[1])
        torch.cuda.synchronize()
        st["unet"] = time.perf_counter() - t
        t = time.perf_counter()
    _, info = plan.cgls(b, x, maxit, tol, warm=rnorm_ref > 0.0, rnorm_ref=rnorm_ref)
    torch.cuda.synchronize()
    st["cgls"] = time.perf_counter() - t
    return info, st


def main():
    import arec3d_gb300 as gb

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=DEFAULT_WEIGHTS,
                    help="weights file; with several --sirt-iters, _sirt<k> is appended")
    ap.add_argument("--input", default=str(SIRT_ITERS),
                    help="network input(s), comma separated: a SIRT depth, or fbp (the "
                         "filtered back projection)")
    ap.add_argument("--sirt-lam-scale", type=float, default=1.0,
                    help="SIRT step as a multiple of 1/(nangles*nx)")
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--crop", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--sets", default="1024:1200:256:5e3:sphere:2,512:360:128:1e4:sphere:3,"
                    "512:360:128:1e4:ellipse:3",
                    help="nx:angles:slices:photons:kind:volumes, comma separated")
    ap.add_argument("--seed", type=int, default=50000)
    args = ap.parse_args()
    gb.build()
    ks = [k if k == "fbp" else int(k) for k in args.input.split(",")]
    datasets = {k: [] for k in ks}
    desc = []
    seed = args.seed
    t0 = time.time()
    for spec in args.sets.split(","):
        nx, na, sl, ph, kind, nv = spec.split(":")
        for _ in range(int(nv)):
            pairs = make_pairs(gb, int(nx), int(na), int(sl), float(ph), seed, kind, ks,
                               lam_scale=args.sirt_lam_scale)
            for k in ks:
                datasets[k].append(pairs[k])
            seed += 7
        desc.append(spec)
        print("pairs %s done %.1fs" % (spec, time.time() - t0), flush=True)
    for k in ks:
        net, hist = train(gb, datasets[k], steps=args.steps, batch=args.batch, crop=args.crop,
                          lr=args.lr, seed=args.seed)
        meta = {"input": "fbp" if k == "fbp" else "sirt", "cgls_iters": CGLS_ITERS,
                "sets": desc, "steps": args.steps, "batch": args.batch, "crop": args.crop,
                "lr": args.lr, "final_loss": float(np.mean(hist[-50:])),
                "first_loss": float(hist[0])}
        if k != "fbp":
            meta.update(sirt_iters=k, sirt_lam_scale=args.sirt_lam_scale)
        tag = "fbp" if k == "fbp" else "sirt%d" % k
        out = args.out if len(ks) == 1 else args.out.replace(".npz", "_%s.npz" % tag)
        save(net, out, meta)
        print(json.dumps(dict(meta, out=out)), flush=True)
        del net


if __name__ == "__main__":
    main()
