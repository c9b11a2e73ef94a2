"""GPU cross-correlation shift search against the oracle (reference ccorr2d +
speak + quad2dfit, AREC3D/AREC3D/align2dstack.cpp:480-521, 1059-1166, and
arecCCImages, AREC3D/AREC3D/arecImage.cpp:384-434)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def smooth_image(rng, ny, nx, nblob=12):
    yy, xx = np.mgrid[0:ny, 0:nx].astype(np.float64)
    img = np.zeros((ny, nx))
    for _ in range(nblob):
        cy, cx = rng.uniform(0, ny), rng.uniform(0, nx)
        s = rng.uniform(0.03, 0.12) * min(nx, ny)
        img += rng.uniform(0.2, 1.0) * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
    return img


def fourier_shift(img, sy, sx):
    ny, nx = img.shape
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.fftfreq(nx)[None, :]
    return np.real(np.fft.ifft2(np.fft.fft2(img) * np.exp(-2j * np.pi * (ky * sy + kx * sx))))


def make_pairs(seed, nz, ny, nx, noise=0.02):
    rng = np.random.default_rng(seed)
    a = np.zeros((nz, ny, nx), np.float32)
    b = np.zeros((nz, ny, nx), np.float32)
    shifts = []
    for i in range(nz):
        img = smooth_image(rng, ny, nx)
        sy = rng.integers(-nx // 8, nx // 8 + 1) + rng.uniform(-0.5, 0.5)
        sx = rng.integers(-nx // 8, nx // 8 + 1) + rng.uniform(-0.5, 0.5)
        a[i] = img
        b[i] = fourier_shift(img, sy, sx) + noise * rng.standard_normal((ny, nx))
        shifts.append((sx, sy))
    return a, b, np.array(shifts)


@pytest.mark.parametrize("shape", [(16, 16), (32, 64), (128, 128), (64, 256), (256, 64)])
def test_ccorr2d_image(gb, oc, shape):
    import torch

    ny, nx = shape
    a, b, _ = make_pairs(1, 1, ny, nx)
    c_ref = oc.ccorr2d(a[0], b[0])
    x, y = torch.from_numpy(a[0]).cuda(), torch.from_numpy(b[0]).cuda()
    c = torch.zeros_like(x)
    gb.ccorr2d_device(x, y, c)
    assert rel_l2(c.cpu().numpy(), c_ref) < 1e-5
    # and through the reference-compatible entry point
    assert rel_l2(gb.ccorr2d(a[0], b[0]), c_ref) < 1e-5


@pytest.mark.parametrize("shape", [(64, 64), (128, 256), (512, 512), (2048, 128), (4096, 64)])
def test_shift_search(gb, oc, shape):
    import torch

    ny, nx = shape
    nz = 6
    a, b, truth = make_pairs(7, nz, ny, nx)
    sx_ref, sy_ref = oc.cc_images(a, b)
    ix_ref, iy_ref = [], []
    for i in range(nz):
        _, _, ix, iy = oc.speak(oc.ccorr2d(a[i], b[i]))
        ix_ref.append(ix)
        iy_ref.append(iy)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    sx = torch.zeros(nz, device="cuda")
    sy = torch.zeros(nz, device="cuda")
    ix = torch.zeros(nz, dtype=torch.int32, device="cuda")
    iy = torch.zeros(nz, dtype=torch.int32, device="cuda")
    gb.cc_shifts(da, db, sx, sy, ix, iy)
    # integer peak positions bit-exact, sub-pixel within 0.05 px
    assert ix.cpu().numpy().tolist() == ix_ref
    assert iy.cpu().numpy().tolist() == iy_ref
    assert np.abs(sx.cpu().numpy() - sx_ref).max() < 0.05
    assert np.abs(sy.cpu().numpy() - sy_ref).max() < 0.05
    # the recovered shifts are the planted ones
    assert np.abs(sx.cpu().numpy() - truth[:, 0]).max() < 0.25
    # reference-compatible entry point
    sx2, sy2, st = gb.arecCCImages(a, b)
    assert st == 0
    np.testing.assert_array_equal(sx2, sx.cpu().numpy())
    np.testing.assert_array_equal(sy2, sy.cpu().numpy())


def test_speak_rules(gb, oc):
    """speak's scan order and signed-pmax quirk (align2dstack.cpp:1072-1079)."""
    rng = np.random.default_rng(3)
    cases = []
    c = rng.standard_normal((32, 32)).astype(np.float32)
    c[5, 9] = 10.0
    c[20, 3] = 10.0  # tie: the first in x-major order wins
    cases.append(c)
    c = rng.standard_normal((32, 32)).astype(np.float32)
    c[7, 11] = -12.0  # negative peak: the scan continues after it
    cases.append(c)
    c = rng.standard_normal((16, 64)).astype(np.float32)
    c[15, 63] = -9.0  # negative peak at the very end of the scan
    cases.append(c)
    c = np.abs(rng.standard_normal((16, 16))).astype(np.float32)
    c[0, 0] = 30.0  # peak at the origin, 3x3 window wraps
    cases.append(c)
    for c in cases:
        xt_ref, yt_ref, _, _ = oc.speak(c)
        xt, yt = gb.speak(c)
        assert (xt, yt) == pytest.approx((xt_ref, yt_ref), abs=1e-6)


def test_bad_sizes_rejected(gb):
    """Lengths with a prime factor above 7 are refused with ARECGB_ERR_ARG (and
    a message naming the sizes); the reference's FFTW takes any length."""
    a = np.zeros((1, 48, 97), np.float32)
    sx, sy, st = gb.arecCCImages(a, a)
    assert st == gb.ERR_ARG
    assert "97" in gb.last_error()


# Lengths that are not powers of two (prime factors 2, 3, 5, 7), as crops and
# binning of real detectors give: the mixed-radix transforms against the
# oracle's double-precision FFT (radix 2 + Bluestein), as the reference plans
# FFTW for any nx, ny (AREC3D/AREC3D/align2dstack.cpp:490-520, 577-629).
@pytest.mark.parametrize("shape", [(12, 20), (48, 60), (75, 100), (96, 210), (343, 250)])
def test_ccorr2d_image_any_size(gb, oc, shape):
    import torch

    ny, nx = shape
    a, b, _ = make_pairs(2, 1, ny, nx)
    c_ref = oc.ccorr2d(a[0], b[0])
    x, y = torch.from_numpy(a[0]).cuda(), torch.from_numpy(b[0]).cuda()
    c = torch.zeros_like(x)
    gb.ccorr2d_device(x, y, c)
    assert rel_l2(c.cpu().numpy(), c_ref) < 1e-5
    assert rel_l2(gb.ccorr2d(a[0], b[0]), c_ref) < 1e-5


@pytest.mark.parametrize("shape", [(750, 1000), (1536, 2048), (1000, 750), (90, 96)])
def test_shift_search_any_size(gb, oc, shape):
    import torch

    ny, nx = shape
    nz = 3
    a, b, truth = make_pairs(17, nz, ny, nx)
    sx_ref, sy_ref = oc.cc_images(a, b, nthreads=oc.host_threads())
    ix_ref, iy_ref = [], []
    for i in range(nz):
        _, _, ix, iy = oc.speak(oc.ccorr2d(a[i], b[i]))
        ix_ref.append(ix)
        iy_ref.append(iy)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    sx = torch.zeros(nz, device="cuda")
    sy = torch.zeros(nz, device="cuda")
    ix = torch.zeros(nz, dtype=torch.int32, device="cuda")
    iy = torch.zeros(nz, dtype=torch.int32, device="cuda")
    gb.cc_shifts(da, db, sx, sy, ix, iy)
    assert ix.cpu().numpy().tolist() == ix_ref
    assert iy.cpu().numpy().tolist() == iy_ref
    assert np.abs(sx.cpu().numpy() - sx_ref).max() < 0.05
    assert np.abs(sy.cpu().numpy() - sy_ref).max() < 0.05
    assert np.abs(sx.cpu().numpy() - truth[:, 0]).max() < 0.25
    sx2, sy2, st = gb.arecCCImages(a, b)
    assert st == 0
    np.testing.assert_array_equal(sx2, sx.cpu().numpy())


@pytest.mark.parametrize("shape", [(32, 64), (128, 128), (256, 512), (60, 90), (250, 375),
                                   (21, 35)])
def test_fshift2d_matches_oracle(gb, oc, shape):
    """Fourier shift of an image stack (fshift2d, align2dstack.cpp:566-630)
    against the oracle (pinned to the reference build), through the device
    API and the reference-compatible host entry point."""
    import torch

    ny, nx = shape
    rng = np.random.default_rng(ny + nx)
    imgs = np.stack([smooth_image(rng, ny, nx) for _ in range(3)]).astype(np.float32)
    sx = np.array([3.25, -7.5, 0.4], np.float32)
    sy = np.array([-2.0, 11.75, -0.6], np.float32)
    ref = np.stack([oc.fshift2d(imgs[i], sx[i], sy[i]) for i in range(3)])
    d = torch.from_numpy(imgs).cuda()
    out = torch.zeros_like(d)
    gb.fshift2d_device(d, out, torch.from_numpy(sx).cuda(), torch.from_numpy(sy).cuda())
    assert rel_l2(out.cpu().numpy(), ref) < 1e-5
    assert rel_l2(gb.fshift2d(imgs[1], sx[1], sy[1]), ref[1]) < 1e-5
