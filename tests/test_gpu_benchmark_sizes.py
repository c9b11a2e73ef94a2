"""Parity at the benchmark configurations' own sizes.

The small-geometry tests (test_gpu_projectors.py, test_gpu_solvers.py) stop at
radius 100 and 60 angles.  The benchmark runs at nx = 1024 with 1200 angles,
the uneven batch reaches nx = 2064 with 1800 angles, and the ray position xb
grows with the radius: at xb ~ 1000-2000 a float xb would be off by ~1e-4 px,
which is why the GPU builds xb as an exact float pair.  These cases check that
precision where it matters, on a slab of slices so the oracle (threaded per
projector call, bit-identical to one thread) finishes in seconds:

* square-pixel forward and back projection at 1024^2 x 1200 angles (4 slices)
  and 2064^2 x 1800 angles (2 slices): <= 1e-5 relative L2 against the oracle
  (arecProject2D_SQ / arecBackProject2D_SQ, AREC3D/AREC3D/arecproject.cpp:540-765),
  with the FP64 error of both printed;
* SIRT x50 at config 1's 256^2 x 180 angles on an 8-slice slab of its ellipse
  phantom (cyl_sirt_SQ, arecsirt.cpp:193-373);
* CGLS, 3 iterations, at 1024^2 x 1200 angles on 4 slices of the benchmark's
  sphere cylinder (cyl_cgls_SQ, areccgls.cpp:245-478);
* the shift search on 8 pairs of 2048^2 projections of a sphere cylinder with
  config 3's shifts and noise: integer peaks bit-exact against the oracle's
  ccorr2d + speak (align2dstack.cpp:480-521, 1059-1105).
"""
import math

import numpy as np
import pytest

from conftest import rel_l2, uniform_angles
from devutil import empty_sino, empty_vol, sino_from_dev, sino_to_dev, vol_from_dev, vol_to_dev

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2, projections and reconstructions


@pytest.mark.parametrize("nx,na,ny", [(1024, 1200, 4), (2064, 1800, 2)])
def test_sq_projectors_at_benchmark_geometry(gb, oc, nx, na, ny):
    radius = 0.5 * (nx - 1)
    ang = uniform_angles(na)
    plan = gb.Plan(gb.SQ, radius, ny, ang)
    assert plan.nx == nx
    rng = np.random.default_rng(nx + na)
    x = rng.random((plan.nrays, ny), dtype=np.float32)
    s = rng.standard_normal((na, ny, nx)).astype(np.float32)
    with oc.op_threads():
        q_ref = oc.project(oc.SQ, radius, x, ang)
        g_ref = oc.backproject(oc.SQ, radius, s, ang)
        q64 = oc.project64(oc.SQ, radius, x, ang)
        g64 = oc.backproject64(oc.SQ, radius, s, ang)
    qd = empty_sino(plan)
    plan.project(vol_to_dev(plan, x), qd)
    q = sino_from_dev(plan, qd)
    gd = empty_vol(plan)
    plan.backproject(sino_to_dev(plan, s), gd)
    g = vol_from_dev(plan, gd)
    assert plan.check() == 0
    eq, eg = rel_l2(q, q_ref), rel_l2(g, g_ref)
    print("SQ %d^2 x %d angles, %d slices: forward gpu-ref %.2e, gpu-fp64 %.2e, ref-fp64 %.2e; "
          "back gpu-ref %.2e, gpu-fp64 %.2e, ref-fp64 %.2e"
          % (nx, na, ny, eq, rel_l2(q, q64), rel_l2(q_ref, q64), eg, rel_l2(g, g64),
             rel_l2(g_ref, g64)))
    assert eq < TOL and eg < TOL
    # the GPU is at least as close to FP64 as the reference's own float code
    assert rel_l2(q, q64) < 2 * rel_l2(q_ref, q64) + 1e-7
    assert rel_l2(g, g64) < 2 * rel_l2(g_ref, g64) + 1e-7


def test_sirt50_config1_slab(gb, oc):
    """Config 1: SIRT x50 (lam 5e-6, tol 0), 256^2, 180 angles, 10 ellipses per
    slice, Poisson 1e4 — on 8 of its 64 slices."""
    from arec3d_gb300 import synthetic as syn

    nx, ny, na = 256, 8, 180
    ang = uniform_angles(na)
    plan = gb.Plan(gb.SQ, 0.5 * (nx - 1), ny, ang)
    ph = syn.ellipse_phantom(7, nx, ny)
    bd = syn.ellipse_sinogram(ph, nx, ny, ang, ys=plan.ys)
    syn.poisson_log(bd, 1e4, 8, ny)
    b = sino_from_dev(plan, bd)
    with oc.op_threads():
        x_ref, tr = oc.sirt(oc.SQ, b, ang, lam=5e-6, maxit=50, tol=0.0)
        x64, _ = oc.sirt64(oc.SQ, b, ang, lam=5e-6, maxit=50, tol=0.0)
    xd = empty_vol(plan)
    hist, info = plan.sirt(bd, xd, 5e-6, 50, 0.0)
    x = vol_from_dev(plan, xd)
    e = rel_l2(x, x_ref)
    print("SIRT x50 256^2 x 180, 8 slices: %d iterations, %d restarts; gpu-ref %.2e, "
          "gpu-fp64 %.2e, ref-fp64 %.2e" % (info.iterations, info.restarts, e, rel_l2(x, x64),
                                            rel_l2(x_ref, x64)))
    assert info.iterations == tr.iterations == 50 and info.restarts == tr.restarts
    assert e < TOL
    np.testing.assert_allclose(hist, tr.rel_history()[:len(hist)], rtol=1e-4)


def test_cgls3_benchmark_geometry(gb, oc):
    """The benchmark's problem (1024^2, 1200 angles, sphere cylinder, Poisson
    5e3) on 4 slices, 3 CGLS iterations from zero."""
    from arec3d_gb300 import warmstart as ws

    nx, na, ny = 1024, 1200, 4
    plan, bd = ws.make_problem(gb, nx, na, ny, 5e3, 4242, "sphere")
    b = sino_from_dev(plan, bd)
    ang = plan.angles
    with oc.op_threads():
        x_ref, tr = oc.cgls(oc.SQ, b, ang, maxit=3, tol=0.0)
        x64, _ = oc.cgls64(oc.SQ, b, ang, maxit=3, tol=0.0)
    xd = empty_vol(plan)
    hist, info = plan.cgls(bd, xd, 3, 0.0)
    x = vol_from_dev(plan, xd)
    e = rel_l2(x, x_ref)
    print("CGLS x3 1024^2 x 1200, 4 slices: gpu-ref %.2e, gpu-fp64 %.2e, ref-fp64 %.2e; "
          "residual trace gpu %s ref %s" % (e, rel_l2(x, x64), rel_l2(x_ref, x64),
                                            np.array2string(np.asarray(hist), precision=6),
                                            np.array2string(tr.rel_history(), precision=6)))
    assert info.iterations == tr.iterations == 3
    assert e < TOL
    np.testing.assert_allclose(hist, tr.rel_history(), rtol=1e-4)


def _fourier_shift(img, sy, sx):
    ny, nx = img.shape
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.fftfreq(nx)[None, :]
    return np.real(np.fft.ifft2(np.fft.fft2(img) * np.exp(-2j * np.pi * (ky * sy + kx * sx))))


def test_shift_search_2048_pairs(gb, oc):
    """Config 3's images: projections (2048 slices x 2048 bins) of a
    random-sphere cylinder at 8 angles, each shifted by an integer in +-20 px
    plus a sub-pixel part in +-0.5 px, with 2 % Gaussian noise."""
    import torch

    from arec3d_gb300 import synthetic as syn

    n, nz = 2048, 8
    ang = (np.arange(nz) * (math.pi / nz)).astype(np.float32)
    ph = syn.sphere_cylinder_phantom(33, n, n, n_spheres=300, r_min=8.0, r_max=120.0)
    sino = syn.sphere_sinogram(ph, n, n, ang, ys=n)          # [angle][bin][slice]
    prj = sino.permute(0, 2, 1).contiguous().cpu().numpy()   # [angle][slice][bin]
    rng = np.random.default_rng(34)
    img = np.empty_like(prj)
    shifts = []
    for i in range(nz):
        sx = rng.integers(-20, 21) + rng.uniform(-0.5, 0.5)
        sy = rng.integers(-20, 21) + rng.uniform(-0.5, 0.5)
        sh = _fourier_shift(prj[i].astype(np.float64), sy, sx)
        img[i] = sh + 0.02 * sh.std() * rng.standard_normal(sh.shape)
        shifts.append((sx, sy))
    shifts = np.array(shifts)
    ix_ref, iy_ref = [], []
    for i in range(nz):
        _, _, ix, iy = oc.speak(oc.ccorr2d(prj[i], img[i]))
        ix_ref.append(ix)
        iy_ref.append(iy)
    sx_ref, sy_ref = oc.cc_images(prj, img, nthreads=oc.host_threads())
    sx = torch.zeros(nz, device="cuda")
    sy = torch.zeros(nz, device="cuda")
    ix = torch.zeros(nz, dtype=torch.int32, device="cuda")
    iy = torch.zeros(nz, dtype=torch.int32, device="cuda")
    gb.cc_shifts(torch.from_numpy(prj).cuda(), torch.from_numpy(img).cuda(), sx, sy, ix, iy)
    sxg, syg = sx.cpu().numpy(), sy.cpu().numpy()
    print("2048^2 shift search, 8 pairs: max |gpu-ref| %.2e / %.2e px, max |gpu-planted| %.3f px"
          % (np.abs(sxg - sx_ref).max(), np.abs(syg - sy_ref).max(),
             max(np.abs(sxg - shifts[:, 0]).max(), np.abs(syg - shifts[:, 1]).max())))
    assert ix.cpu().numpy().tolist() == ix_ref
    assert iy.cpu().numpy().tolist() == iy_ref
    assert np.abs(sxg - sx_ref).max() < 0.05 and np.abs(syg - sy_ref).max() < 0.05
    assert np.abs(sxg - shifts[:, 0]).max() < 0.25 and np.abs(syg - shifts[:, 1]).max() < 0.25
