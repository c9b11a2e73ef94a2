"""GPU SIRT / CGLS parity against the oracle (reference cyl_sirt[_KB|_SQ],
AREC3D/AREC3D/arecsirt.cpp; cyl_cgls[_KB|_SQ], AREC3D/AREC3D/areccgls.cpp)."""
import numpy as np
import pytest

from conftest import rel_l2, uniform_angles
from devutil import empty_sino, empty_vol, sino_to_dev, vol_from_dev, vol_to_dev

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2 on reconstructions (SIRT; CGLS up to 12 iterations)
# Longer CGLS solves of these ill-conditioned problems amplify float rounding:
# the reference's own float result then differs from an FP64 evaluation of the
# same algorithm (oracle cgls64) by 1e-4..1e-2.  There the GPU must reproduce
# the reference's float trajectory to within FRAC of that distance.
FRAC = 0.25
# Residual traces: the normal-equation residual ||A^T(b - A x_k)|| is, in the
# late iterations, a small difference of large quantities; a 1e-6 change of x
# moves it by several per cent while x itself agrees to 1e-5.  Traces are
# compared to RTOL_TRACE; the iteration counts (the stopping decisions) exactly.
RTOL_TRACE = 0.2


def _problem(oc, w, nx, ny, na, seed, noise=0.01):
    rng = np.random.default_rng(seed)
    ang = uniform_angles(na)
    radius = 0.5 * (nx - 1)
    _, nr, _ = oc.cyl(radius)
    xt = rng.random((nr, ny), dtype=np.float32)
    b = oc.project(w, radius, xt, ang)
    b = (b + noise * rng.standard_normal(b.shape)).astype(np.float32)
    return b, ang, radius


@pytest.mark.parametrize("w", [1, 2, 3])
def test_sirt_parity(gb, oc, w):
    b, ang, radius = _problem(oc, w, 49, 6, 30, seed=w)
    x_ref, tr = oc.sirt(w, b, ang, lam=2e-4, maxit=20, tol=0.0)
    plan = gb.Plan(w, radius, b.shape[1], ang)
    xd = empty_vol(plan)
    hist, info = plan.sirt(sino_to_dev(plan, b), xd, 2e-4, 20, 0.0)
    x = vol_from_dev(plan, xd)
    assert info.iterations == tr.iterations and info.restarts == tr.restarts
    if w == 1:
        x, x_ref = x[:-2], x_ref[:-2]
    assert rel_l2(x, x_ref) < TOL
    np.testing.assert_allclose(hist, tr.rel_history()[:len(hist)], rtol=1e-4)


def test_sirt_restarts(gb, oc):
    """A step size far above 2/||A||^2 diverges: the reference halves it and
    restarts, accumulating ||A^T b||^2 (arecsirt.cpp:273-290, 318-338)."""
    w = 3
    b, ang, radius = _problem(oc, w, 33, 4, 20, seed=5)
    x_ref, tr = oc.sirt(w, b, ang, lam=0.05, maxit=12, tol=0.0)
    assert tr.restarts > 0
    plan = gb.Plan(w, radius, b.shape[1], ang)
    xd = empty_vol(plan)
    hist, info = plan.sirt(sino_to_dev(plan, b), xd, 0.05, 12, 0.0)
    assert info.restarts == tr.restarts
    assert info.lam_final == pytest.approx(tr.lam_final, rel=0, abs=0)
    assert rel_l2(vol_from_dev(plan, xd), x_ref) < TOL


@pytest.mark.parametrize("w", [1, 2, 3])
def test_cgls_parity(gb, oc, w):
    b, ang, radius = _problem(oc, w, 49, 6, 30, seed=10 + w)
    x_ref, tr = oc.cgls(w, b, ang, maxit=12, tol=1e-7)
    plan = gb.Plan(w, radius, b.shape[1], ang)
    xd = empty_vol(plan)
    hist, info = plan.cgls(sino_to_dev(plan, b), xd, 12, 1e-7)
    x = vol_from_dev(plan, xd)
    assert info.iterations == tr.iterations
    assert info.iterbest == tr.iterbest
    if w == 1:
        x, x_ref = x[:-2], x_ref[:-2]
    assert rel_l2(x, x_ref) < TOL
    np.testing.assert_allclose(hist, tr.rel_history(), rtol=RTOL_TRACE)
    x64, _ = oc.cgls64(w, b, ang, maxit=12, tol=1e-7)
    if w == 1:
        x64 = x64[:-2]
    print("cgls w=%d: gpu-ref %.2e, ref-fp64 %.2e, gpu-fp64 %.2e"
          % (w, rel_l2(x, x_ref), rel_l2(x_ref, x64), rel_l2(x, x64)))


def test_cgls_tolerance_stop_and_warm_start(gb, oc):
    w = 3
    b, ang, radius = _problem(oc, w, 65, 8, 40, seed=21)
    x0, _ = oc.sirt(w, b, ang, lam=2e-4, maxit=5, tol=0.0)
    x_ref, tr = oc.cgls(w, b, ang, maxit=50, tol=2e-3, x0=x0)
    plan = gb.Plan(w, radius, b.shape[1], ang)
    xd = vol_to_dev(plan, x0)
    hist, info = plan.cgls(sino_to_dev(plan, b), xd, 50, 2e-3, warm=True)
    assert info.iterations == tr.iterations < 50
    x64, _ = oc.cgls64(w, b, ang, maxit=50, tol=2e-3, x0=x0)
    e_gpu, e_ref = rel_l2(vol_from_dev(plan, xd), x_ref), rel_l2(x_ref, x64)
    print("warm-started cgls (%d it): gpu-ref %.2e, ref-fp64 %.2e" % (info.iterations, e_gpu, e_ref))
    assert e_gpu < max(TOL, FRAC * e_ref)


def test_cgls_fixed_denominator(gb, oc):
    w = 3
    b, ang, radius = _problem(oc, w, 33, 4, 24, seed=3)
    ref = 1234.5
    x_ref, tr = oc.cgls(w, b, ang, maxit=8, tol=0.0, rnorm_ref=ref)
    plan = gb.Plan(w, radius, b.shape[1], ang)
    xd = empty_vol(plan)
    hist, info = plan.cgls(sino_to_dev(plan, b), xd, 8, 0.0, rnorm_ref=ref)
    np.testing.assert_allclose(hist, tr.rel_history(), rtol=RTOL_TRACE)
    x64, _ = oc.cgls64(w, b, ang, maxit=8, tol=0.0, rnorm_ref=ref)
    e_gpu, e_ref = rel_l2(vol_from_dev(plan, xd), x_ref), rel_l2(x_ref, x64)
    print("fixed-denominator cgls: gpu-ref %.2e, ref-fp64 %.2e" % (e_gpu, e_ref))
    assert e_gpu < max(TOL, FRAC * e_ref)


def test_cgls_long_solve_tracks_reference(gb, oc):
    """60 iterations: report the error against FP64 of both implementations."""
    w = 3
    b, ang, radius = _problem(oc, w, 65, 6, 48, seed=31)
    x_ref, tr = oc.cgls(w, b, ang, maxit=60, tol=0.0)
    x64, _ = oc.cgls64(w, b, ang, maxit=60, tol=0.0)
    plan = gb.Plan(w, radius, b.shape[1], ang)
    xd = empty_vol(plan)
    plan.cgls(sino_to_dev(plan, b), xd, 60, 0.0)
    x = vol_from_dev(plan, xd)
    e_gpu, e_ref, e_64 = rel_l2(x, x_ref), rel_l2(x_ref, x64), rel_l2(x, x64)
    print("cgls 60 it: gpu-ref %.2e, ref-fp64 %.2e, gpu-fp64 %.2e" % (e_gpu, e_ref, e_64))
    assert e_gpu < max(TOL, FRAC * e_ref)
    assert e_64 < 1.5 * e_ref + TOL


@pytest.mark.parametrize("w", [2, 3])
def test_projector_error_vs_fp64(gb, oc, w):
    """The GPU projectors are at least as close to FP64 as the reference's float code."""
    from devutil import empty_sino, sino_from_dev

    radius, ny, ang = 63.5, 16, uniform_angles(64)
    rng = np.random.default_rng(9)
    plan = gb.Plan(w, radius, ny, ang)
    x = rng.random((plan.nrays, ny), dtype=np.float32)
    q64 = oc.project64(w, radius, x, ang)
    q_ref = oc.project(w, radius, x, ang)
    qd = empty_sino(plan)
    plan.project(vol_to_dev(plan, x), qd)
    q = sino_from_dev(plan, qd)
    e_gpu, e_ref = rel_l2(q, q64), rel_l2(q_ref, q64)
    print("FP w=%d: gpu-fp64 %.2e, ref-fp64 %.2e, gpu-ref %.2e" % (w, e_gpu, e_ref, rel_l2(q, q_ref)))
    assert e_gpu < 2 * e_ref + 1e-7


def test_cgls_batch_matches_single_solves(gb):
    """Three uneven problems (radius, slices, angles, weighting) solved as one
    batch (one CUDA graph launch per iteration) give exactly the iterates and
    histories of three separate solves."""
    import torch

    specs = [(3, 31.5, 20, uniform_angles(40)), (2, 12.0, 8, uniform_angles(16)),
             (3, 63.5, 64, uniform_angles(90))]
    rng = np.random.default_rng(11)
    plans, bs, singles, infos = [], [], [], []
    for w, radius, ny, ang in specs:
        plan = gb.Plan(w, radius, ny, ang)
        b = rng.random((len(ang), ny, plan.nx)).astype(np.float32)
        bd = sino_to_dev(plan, b)
        xd = empty_vol(plan)
        hist, info = plan.cgls(bd, xd, 15, 1e-4)
        plans.append(plan)
        bs.append(bd)
        singles.append(vol_from_dev(plan, xd))
        infos.append(info)
    xs = [empty_vol(p) for p in plans]
    binfo = gb.cgls_batch(plans, bs, xs, 15, 1e-4)
    for i, plan in enumerate(plans):
        assert binfo[i].iterations == infos[i].iterations
        assert binfo[i].rel_final == infos[i].rel_final
        np.testing.assert_array_equal(vol_from_dev(plan, xs[i]), singles[i])


@pytest.mark.parametrize("w", [2, 3])
def test_cgls_stat_parity(gb, oc, w):
    """Statistically weighted CGLS (cyl_cgls_SQ_stat / _KB_stat,
    areccgls_stat.cpp) on the device against the oracle (pinned bit for bit to
    the reference build) and its FP64 twin; odd nx as the reference requires."""
    rng = np.random.default_rng(20 + w)
    radius, ny, na = 24, 6, 36
    nx = 2 * radius + 1
    ang = uniform_angles(na)
    _, nr, _ = oc.cyl(float(radius))
    xt = rng.random((nr, ny), dtype=np.float32) * 0.02
    b = oc.project(w, float(radius), xt, ang)
    b = (b + 0.01 * rng.standard_normal(b.shape)).astype(np.float32)
    x_ref, tr = oc.cgls_stat(w, b, ang, maxit=10, tol=1e-7)
    x64, _ = oc.cgls_stat64(w, b, ang, maxit=10, tol=1e-7)
    plan = gb.Plan(w, float(radius), ny, ang)
    assert plan.nx == nx
    xd = empty_vol(plan)
    hist, info = plan.cgls_stat(sino_to_dev(plan, b), xd, 10, 1e-7)
    x = vol_from_dev(plan, xd)
    e_gpu, e_ref = rel_l2(x, x_ref), rel_l2(x_ref, x64)
    print("cgls_stat w=%d: gpu-ref %.2e, ref-fp64 %.2e, gpu-fp64 %.2e"
          % (w, e_gpu, e_ref, rel_l2(x, x64)))
    assert info.iterations == tr.iterations
    assert e_gpu < max(TOL, FRAC * e_ref)
    np.testing.assert_allclose(hist, tr.rel_history(), rtol=RTOL_TRACE)
    # and through the reference-compatible entry point (host arecImage buffers)
    name = "cyl_cgls_SQ_stat" if w == 3 else "cyl_cgls_KB_stat"
    xc, st = getattr(gb, name)(b, ang, maxit=10, tol=1e-7)
    assert st == 0
    assert rel_l2(xc, x_ref) < max(TOL, FRAC * e_ref)


def test_solve_uneven_waves_match_single_solves(gb):
    """arecgb_solve_uneven: five cylinders of uneven radius, slices and angles
    under a budget that forces several waves give exactly the results of
    solving each alone (plans without tables compute the same values), with
    and without the learned warm start (first reconstruction -> U-Net -> CGLS
    with the cold start's denominator, as the single-problem pipeline does), for
    both shipped networks (filtered back projection input, SIRT input)."""
    import torch

    from arec3d_gb300 import synthetic as syn
    from arec3d_gb300 import warmstart as ws

    rng = np.random.default_rng(55)
    specs = [(60.5, 24, 90), (31.5, 8, 40), (90.0, 40, 120), (47.5, 16, 64), (20.0, 8, 30)]
    probs, singles = [], []
    net_fbp, _ = ws.load(gb, ws.DEFAULT_WEIGHTS, 184, 4)
    net_sirt, _ = ws.load(gb, ws.DEFAULT_WEIGHTS.replace(".npz", "_sirt4.npz"), 184, 4)
    assert (net_fbp.input, net_sirt.input) == ("fbp", "sirt")
    for radius, ny, na in specs:
        ang = syn.uniform_angles(na)
        plan = gb.Plan(gb.SQ, radius, ny, ang)
        xt = rng.random((plan.nrays, ny), dtype=np.float32)
        qd = empty_sino(plan)
        plan.project(vol_to_dev(plan, xt), qd)
        qd[:, :, :ny] += 0.02 * torch.randn(plan.nangles, plan.nx, ny, device="cuda")
        singles.append((plan, qd))
        probs.append(dict(radius=radius, ny=ny, angles=ang, b=qd, x=empty_vol(plan)))
    nxv = [gb.cylinder_info(r, ny)[:2] for r, ny, _ in specs]
    assert [(p.nx, p.nrays) for p, _ in singles] == nxv
    for net in (None, net_fbp, net_sirt):
        use_net = net is not None
        budget = 1 << 20  # 1 MiB of workspace: every problem its own wave
        infos, waves = gb.solve_uneven(probs, budget, maxit=30, tol=1e-3,
                                       nets=[net] if use_net else None)
        assert sorted(waves) == list(range(len(specs)))
        for i, (plan, qd) in enumerate(singles):
            x = empty_vol(plan)
            if use_net:
                info, _ = ws.solve(gb, plan, qd, x, net=net, tol=1e-3, maxit=30)
            else:
                _, info = plan.cgls(qd, x, 30, 1e-3)
            assert infos[i].iterations == info.iterations
            np.testing.assert_array_equal(vol_from_dev(plan, probs[i]["x"]), vol_from_dev(plan, x))
        # one wave for all of them gives the same answers too
        infos2, waves2 = gb.solve_uneven(probs, 1 << 40, maxit=30, tol=1e-3,
                                         nets=[net] if use_net else None)
        assert set(waves2) == {0}
        assert [i.iterations for i in infos2] == [i.iterations for i in infos]
        print("uneven batch (%s): iterations %s" % (net.input if use_net else "plain",
                                                    [i.iterations for i in infos]))
