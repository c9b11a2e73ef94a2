"""Rotational alignment on the GPU (arecRotCCImages, arecRotateImages, _skew,
_skew_safe) against the reference's own outputs (tests/golden/
reference_rotation.npz, made by the reference) and the oracle
(oracle/rotation.py) on larger seeded stacks.

Tolerances: rotations (shears, bilinear) within 2e-6 of the image's range --
the arithmetic is the reference's operation for operation, so the results are
normally bit-identical; the slack covers a last-ulp difference of the
device's double tan / sin / cos from the C library's.  Angles of the rotation
search within 1e-3 degrees (the reference's float FFT correlation against the
device's FP64-accumulated direct sum).  Filtered correlations within 1e-12
(FP64 sums in another order)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "reference_rotation.npz")
IMG_TOL = 2e-6
ANG_TOL = 1e-3


def _close(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    d = np.abs(a - b).max() if a.size else 0.0
    scale = max(np.abs(b).max(), 1e-30)
    print("%s: max |diff| %.3e (range %.3e), bit-identical %s" % (what, d, scale,
                                                                  np.array_equal(a, b)))
    assert d <= IMG_TOL * scale, what


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def test_golden_rotation_device(gb):
    import torch

    g = np.load(GOLD)
    ref, img = _dev(torch, g["rot_ref"]), _dev(torch, g["rot_img"])
    ang = torch.zeros(ref.shape[0], device="cuda")
    gb.rot_cc_images(ref, img, int(g["rotcc_r2"]), ang)
    torch.cuda.synchronize()
    a = ang.cpu().numpy()
    print("rotation search", a, "reference", g["rotcc_angles"])
    assert np.abs(a - g["rotcc_angles"]).max() < ANG_TOL

    x = img.clone()
    sa = _dev(torch, g["skew_angles_in"])
    gb.rotate_images_skew(x, sa)
    torch.cuda.synchronize()
    _close(x.cpu().numpy(), g["skew_img"], "skew rotation")
    assert np.array_equal(sa.cpu().numpy(), g["skew_angles"])

    x = img.clone()
    gb.rotate_images(x, _dev(torch, g["skew_angles_in"]))
    torch.cuda.synchronize()
    _close(x.cpu().numpy(), g["bilinear_img"], "bilinear rotation")

    x = img.clone()
    fa = _dev(torch, g["safe_angles_in"])
    n_rot, mean_cc = gb.rotate_images_skew_safe(x, ref, fa)
    _close(x.cpu().numpy(), g["safe_img"], "guarded shear rotation")
    assert np.array_equal(fa.cpu().numpy(), g["safe_angles"])
    assert n_rot == 3

    cc = torch.zeros(ref.shape[0], dtype=torch.float64, device="cuda")
    gb.ncc_filtered(ref, img, cc)
    torch.cuda.synchronize()
    assert np.allclose(cc.cpu().numpy(), g["ncc"], rtol=1e-12, atol=0)


def test_golden_rotation_compat(gb):
    """The reference-named host entry points (arecRotCCImages, ...)."""
    g = np.load(GOLD)
    ang, st = gb.arecRotCCImages(g["rot_ref"], g["rot_img"], int(g["rotcc_r2"]))
    assert st == 0 and np.abs(ang - g["rotcc_angles"]).max() < ANG_TOL
    out, a = gb.arecRotateImages(g["rot_img"], g["skew_angles_in"], "_skew")
    _close(out, g["skew_img"], "compat skew")
    assert np.array_equal(a, g["skew_angles"])
    out, a = gb.arecRotateImages_skew_safe(g["rot_img"], g["rot_ref"], g["safe_angles_in"])
    _close(out, g["safe_img"], "compat guarded")
    assert np.array_equal(a, g["safe_angles"])


@pytest.mark.parametrize("ny,nx,r2", [(256, 256, 100), (200, 320, 64), (96, 128, 2)])
def test_rotation_against_oracle(gb, ny, nx, r2):
    import torch

    from oracle import rotation as R

    rng = np.random.default_rng(ny + nx + r2)
    yy, xx = np.mgrid[0:ny, 0:nx].astype(np.float64)
    truth = np.array([6.0, -3.5, 0.0, 12.0, -40.0])
    ref, img = [], []
    for t in truth:
        th = np.deg2rad(t)
        x, y = xx - nx / 2, yy - ny / 2
        xr, yr = x * np.cos(th) + y * np.sin(th), -x * np.sin(th) + y * np.cos(th)
        base = np.exp(-((x - nx / 8) ** 2 + (y - ny / 10) ** 2) / (nx * 2.0)) + \
            0.5 * (np.abs(x + nx / 6) < nx / 12) * (np.abs(y) < ny / 5)
        rot = np.exp(-((xr - nx / 8) ** 2 + (yr - ny / 10) ** 2) / (nx * 2.0)) + \
            0.5 * (np.abs(xr + nx / 6) < nx / 12) * (np.abs(yr) < ny / 5)
        ref.append(base + 0.02 * rng.standard_normal(base.shape))
        img.append(rot + 0.02 * rng.standard_normal(rot.shape))
    ref = np.array(ref, np.float32)
    img = np.array(img, np.float32)
    dref, dimg = _dev(torch, ref), _dev(torch, img)

    ang = torch.zeros(len(truth), device="cuda")
    gb.rot_cc_images(dref, dimg, r2, ang)
    torch.cuda.synchronize()
    a_gpu = ang.cpu().numpy()
    a_orc = R.rot_cc_angles(ref, img, r2)
    print("angles gpu", a_gpu, "oracle", a_orc, "truth", truth)
    assert np.abs(a_gpu - a_orc).max() < ANG_TOL

    angles = np.array([4.0, -9.5, 0.0, 22.0, 181.0], np.float32)
    x = dimg.clone()
    da = _dev(torch, angles)
    gb.rotate_images_skew(x, da)
    o_img, o_ang = R.rotate_images_skew(img, angles)
    torch.cuda.synchronize()
    _close(x.cpu().numpy(), o_img, "skew %dx%d" % (ny, nx))
    assert np.array_equal(da.cpu().numpy(), o_ang)

    x = dimg.clone()
    da = _dev(torch, a_orc)
    n_rot, mean_cc = gb.rotate_images_skew_safe(x, dref, da)
    o_img, o_ang, o_n, o_mean = R.rotate_images_skew_safe(img, ref, a_orc)
    _close(x.cpu().numpy(), o_img, "guarded %dx%d" % (ny, nx))
    assert np.array_equal(da.cpu().numpy(), o_ang) and n_rot == o_n
    assert abs(mean_cc - o_mean) < 1e-12


def test_rotation_edges(gb):
    import torch

    x = torch.zeros(0, 64, 64, device="cuda")
    a = torch.zeros(0, device="cuda")
    gb.rot_cc_images(x, x, 10, a)          # empty stack: nothing to do
    gb.rotate_images_skew(x, a)
    y = torch.zeros(1, 64, 64, device="cuda")
    b = torch.zeros(1, device="cuda")
    for r2 in (1, 33, 5000):                # outside [2, min(nx, ny)/2]
        with pytest.raises(RuntimeError):
            gb.rot_cc_images(y, y, r2, b)
    # a flat image pair correlates equally at every lag: first index, angle 0
    gb.rot_cc_images(y + 1.0, y + 1.0, 20, b)
    torch.cuda.synchronize()
    assert float(b[0]) == 0.0
