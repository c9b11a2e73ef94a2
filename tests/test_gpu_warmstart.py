"""What the trained warm-start network gains over the method without it.

Seeded problems the network never saw (their own phantom seed): the
benchmark's geometry (1024^2 slices, 1200 angles, 5e3 photons) and the smaller
learned-warm-start configuration (512^2, 360 angles, 1e4 photons), 4 slices
each: plain CGLS from zero against first reconstruction -> U-Net -> CGLS,
for both shipped networks (input: the filtered back projection,
unet_warm_start.npz; SIRT-k, unet_warm_start_sirt4.npz, k and the step as the
file records), and against CGLS from the filtered back projection alone, all
to ||A^T r|| / ||A^T b|| <= 1e-3.  The gain is CGLS iterations saved.  Both GPU results of each problem are then checked in
FP64 with the oracle's projectors: their normal-equation residual, recomputed
in double, must be within the tolerance the GPU solver reported meeting
(RESID_SLACK allows for the GPU evaluating the same quantity in FP32)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-3
RESID_SLACK = 1.05
SLICES = 4


def _fp64_relative_residual(oc, radius, b_ref, x, ang):
    """||A^T (b - A x)|| / ||A^T b|| in FP64 (oracle projectors, SQ weighting)."""
    atb = oc.backproject64(3, radius, b_ref, ang)
    r = b_ref - oc.project64(3, radius, x, ang)
    return float(np.linalg.norm(oc.backproject64(3, radius, r, ang)) / np.linalg.norm(atb))


# (nx, angles, photons, the gain asked for): the benchmark's geometry must save
# iterations; a smaller, better-conditioned problem (plain CGLS needs ~10
# iterations) must not lose any.
CASES = [(1024, 1200, 5e3, "saves"), (512, 360, 1e4, "no loss")]


@pytest.mark.parametrize("weights", ["unet_warm_start.npz", "unet_warm_start_sirt4.npz"])
@pytest.mark.parametrize("nx,na,photons,want", CASES)
def test_warm_start_saves_iterations(gb, oc, nx, na, photons, want, weights):
    import torch

    from arec3d_gb300 import warmstart as ws

    path = os.path.join(os.path.dirname(ws.DEFAULT_WEIGHTS), weights)
    assert os.path.exists(path), "trained weights missing: " + path
    plan, b = ws.make_problem(gb, nx, na, SLICES, photons, 777001, "sphere")
    net, meta = ws.load(gb, path, ws.pad8(plan.nx), SLICES)
    assert net.input == ("fbp" if weights == "unet_warm_start.npz" else "sirt")

    x_plain = torch.zeros(plan.nrays, plan.ys, device="cuda")
    info_plain, _ = ws.solve(gb, plan, b, x_plain, net=None, tol=TOL)
    x_warm = torch.zeros_like(x_plain)
    info_warm, stages = ws.solve(gb, plan, b, x_warm, net=net, tol=TOL)
    saved = info_plain.iterations - info_warm.iterations
    print("warm start %dx%d, %d angles: CGLS iterations plain %d, warm %d (saved %d); "
          "input %.3fs U-Net %.3fs CGLS %.3fs" % (nx, nx, na, info_plain.iterations,
                                                info_warm.iterations, saved, stages["input"],
                                                stages["unet"], stages["cgls"]))
    assert info_plain.rel_final <= TOL and info_warm.rel_final <= TOL
    assert saved > 0 if want == "saves" else saved >= 0
    results = [("plain", x_plain, info_plain), ("warm", x_warm, info_warm)]
    if net.input == "fbp":  # the filtered back projection alone as the start
        x_fbp = torch.zeros_like(x_plain)
        info_fbp, _ = ws.solve(gb, plan, b, x_fbp, start="fbp", tol=TOL)
        print("from the filtered back projection alone: %d CGLS iterations"
              % info_fbp.iterations)
        assert info_fbp.rel_final <= TOL and info_fbp.iterations <= info_plain.iterations
        results.append(("fbp", x_fbp, info_fbp))

    # FP64 check of both results (reference layout [angle][slice][bin]); the
    # oracle's projectors run threaded (bit-identical to one thread)
    b_ref = b[:, :, :SLICES].permute(0, 2, 1).contiguous().double().cpu().numpy()
    ang = plan.angles
    radius = 0.5 * (nx - 1)
    for name, xd, info in results:
        x = xd[:, :SLICES].double().cpu().numpy()
        with oc.op_threads():
            rel = _fp64_relative_residual(oc, radius, b_ref, x, ang)
        print("%s: FP64 relative normal-equation residual %.3e (GPU reported %.3e)"
              % (name, rel, info.rel_final))
        assert rel <= TOL * RESID_SLACK
    # the two answers agree to the precision a 1e-3 residual implies
    d = (np.linalg.norm((x_warm - x_plain)[:, :SLICES].double().cpu().numpy()) /
         np.linalg.norm(x_plain[:, :SLICES].double().cpu().numpy()))
    print("warm vs plain solution: relative difference %.3e" % d)


@pytest.mark.parametrize("weights", ["unet_warm_start.npz", "unet_warm_start_sirt4.npz"])
def test_reconstruct_host_matches_device_pipeline(gb, weights):
    """arecgb_reconstruct_host (host buffers in the reference's layouts, one
    call) gives bit for bit the device pipeline's result: same first
    reconstruction, network, denominator and CGLS."""
    import torch

    from arec3d_gb300 import warmstart as ws

    ny = 8
    path = os.path.join(os.path.dirname(ws.DEFAULT_WEIGHTS), weights)
    plan, b = ws.make_problem(gb, 256, 180, ny, 1e4, 4242, "sphere")
    net, _ = ws.load(gb, path, ws.pad8(plan.nx), ny)
    x = torch.zeros(plan.nrays, plan.ys, device="cuda")
    info, _ = ws.solve(gb, plan, b, x, net=net, tol=TOL)
    b_host = b[:, :, :ny].permute(0, 2, 1).contiguous().cpu()  # [angle][slice][bin]
    x_host = torch.empty(plan.nrays, ny)
    lam = ws.sirt_lambda(plan, net.sirt_lam_scale)
    info_h = plan.reconstruct_host(b_host, x_host, net, net.sirt_iters, lam, 200, TOL)
    print("%s: %d CGLS iterations (device pipeline %d)" % (weights, info_h.iterations,
                                                           info.iterations))
    assert info_h.iterations == info.iterations
    np.testing.assert_array_equal(x_host.numpy(), x[:, :ny].cpu().numpy())
