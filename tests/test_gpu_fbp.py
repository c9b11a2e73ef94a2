"""Filtered back projection (arecgb_ramp_filter, arecgb_fbp): the ramp filter
against a float64 direct convolution, the reconstruction against the oracle's
back projector (reference arecBackProject2D[_KB|_SQ], arecproject.cpp) of the
same filtered sinogram, and the inversion formula's scale on a uniform disk.
The filter has no counterpart in the reference; it feeds the warm start."""
import math

import numpy as np
import pytest

from conftest import rel_l2, uniform_angles
from devutil import empty_sino, empty_vol, sino_from_dev, sino_to_dev, vol_from_dev

pytestmark = pytest.mark.gpu

TOL_FILTER = 1e-6  # relative L2 against float64: FP32 sums of up to nx/2 taps
TOL = 1e-5         # relative L2, the back projection of the filtered sinogram


def ramlak(nx):
    d = np.arange(-(nx - 1), nx)
    h = np.zeros(d.size)
    h[d == 0] = 0.25
    odd = d % 2 != 0
    h[odd] = -1.0 / (math.pi * d[odd]) ** 2
    return h


def filtered(q, na):
    """(pi / na) * linear convolution along bins, float64; q [na][ny][nx]."""
    nx = q.shape[2]
    h = ramlak(nx)
    out = np.empty(q.shape, np.float64)
    for a in range(q.shape[0]):
        for y in range(q.shape[1]):
            out[a, y] = np.convolve(q[a, y].astype(np.float64), h)[nx - 1:2 * nx - 1]
    return out * (math.pi / na)


@pytest.mark.parametrize("radius,ny,na", [(16.0, 3, 12), (31.5, 10, 20), (128.0, 130, 9),
                                          (200.5, 16, 7)])
def test_ramp_filter_matches_float64(gb, radius, ny, na):
    ang = uniform_angles(na)
    plan = gb.Plan(gb.SQ, radius, ny, ang)
    rng = np.random.default_rng(int(radius * 10) + ny)
    q = rng.standard_normal((na, ny, plan.nx)).astype(np.float32)
    qd, fd = sino_to_dev(plan, q), empty_sino(plan)
    fd.fill_(7.0)
    plan.ramp_filter(qd, fd)
    f = sino_from_dev(plan, fd)
    ref = filtered(q, na)
    e = rel_l2(f, ref)
    print("ramp filter nx=%d: %.2e" % (plan.nx, e))
    assert e < TOL_FILTER
    if plan.ys > ny:  # padding slices of the device layout stay zero
        assert float(fd[:, :, ny:].abs().max()) == 0.0


@pytest.mark.parametrize("w", [1, 2, 3])
def test_fbp_matches_oracle_backprojection(gb, oc, w):
    radius, ny, na = 40.5, 6, 30
    ang = uniform_angles(na)
    plan = gb.Plan(w, radius, ny, ang)
    rng = np.random.default_rng(w)
    b = rng.random((na, ny, plan.nx)).astype(np.float32)
    fr = filtered(b, na).astype(np.float32)
    x_ref = oc.backproject(w, radius, fr, ang)
    atb = oc.backproject(w, radius, b, ang)
    import torch

    bd, xd, work = sino_to_dev(plan, b), empty_vol(plan), empty_sino(plan)
    n2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    plan.fbp(bd, xd, work, atb_norm2=n2)
    x = vol_from_dev(plan, xd)
    if w == 1:  # the linear weighting's last two rays read past the reference's table
        x, x_ref, atb = x[:-2], x_ref[:-2], atb[:-2]
    e = rel_l2(x, x_ref)
    print("fbp w=%d vs oracle back projection of the filtered sinogram: %.2e" % (w, e))
    assert e < TOL
    if w != 1:  # (the linear weighting's norm includes the two rays left out above)
        ref_n2 = float((atb.astype(np.float64) ** 2).sum())
        assert float(n2.item()) == pytest.approx(ref_n2, rel=1e-5)
    assert plan.check() == 0


def test_fbp_reconstructs_a_uniform_disk(gb):
    """Line integrals of a centred disk of radius R and attenuation mu: the
    reconstruction's interior is mu to within a few percent (the inversion
    formula's weight pi / nangles and the unit bin spacing)."""
    import torch

    radius, ny, na, R, mu = 63.5, 2, 180, 40.0, 0.02
    ang = uniform_angles(na)
    plan = gb.Plan(gb.SQ, radius, ny, ang)
    t = np.arange(plan.nx) - radius
    chord = 2 * mu * np.sqrt(np.clip(R * R - t * t, 0, None))
    b = np.broadcast_to(chord[None, None, :], (na, ny, plan.nx)).astype(np.float32)
    bd, xd, work = sino_to_dev(plan, b), empty_vol(plan), empty_sino(plan)
    plan.fbp(bd, xd, work)
    x = vol_from_dev(plan, xd)
    # ray coordinates of the reference's cylinder (iz-major, truncation toward 0)
    r2 = int(radius * radius)
    cx, cz = [], []
    for iz in range(plan.nx):
        zs = int(iz - radius)
        for ix in range(plan.nx):
            xs = int(ix - radius)
            if xs * xs + zs * zs <= r2:
                cx.append(ix - radius)
                cz.append(iz - radius)
    rho = np.hypot(np.array(cx), np.array(cz))
    assert rho.size == plan.nrays
    inner = x[rho < 0.8 * R].mean()
    outer = np.abs(x[rho > 1.2 * R]).mean()
    print("disk: interior %.5f (mu %.5f), exterior |x| %.2e" % (inner, mu, outer))
    assert abs(inner - mu) < 0.03 * mu
    assert outer < 0.05 * mu
    assert torch.isfinite(xd).all()
