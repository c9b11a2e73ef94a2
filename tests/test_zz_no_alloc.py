"""arecgb_cc_shifts_static (shift search with static scratch, no allocation)
against arecgb_cc_shifts, both called through the C ABI.

Both run the same kernels with the same twiddle values, so integer peaks must
agree exactly and sub-pixel shifts within SUBPIX_TOL."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SUBPIX_TOL = 1e-6
MAX_PIXELS = 512 * 512


def _pairs(seed, nz, ny, nx):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:ny, 0:nx].astype(np.float64)
    a = np.zeros((nz, ny, nx), np.float32)
    b = np.zeros((nz, ny, nx), np.float32)
    for i in range(nz):
        img = np.zeros((ny, nx))
        for _ in range(8):
            cy, cx = rng.uniform(0, ny), rng.uniform(0, nx)
            s = rng.uniform(0.04, 0.1) * min(nx, ny)
            img += rng.uniform(0.2, 1.0) * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
        a[i] = img
        dy, dx = rng.integers(-ny // 8, ny // 8 + 1), rng.integers(-nx // 8, nx // 8 + 1)
        b[i] = np.roll(img, (dy, dx), axis=(0, 1)) + 0.02 * rng.standard_normal((ny, nx))
    return a, b


def _run(L, fn, a, b):
    import torch

    nz, ny, nx = a.shape
    sx = torch.zeros(nz, device="cuda")
    sy = torch.zeros(nz, device="cuda")
    ix = torch.zeros(nz, dtype=torch.int32, device="cuda")
    iy = torch.zeros(nz, dtype=torch.int32, device="cuda")
    rc = getattr(L, fn)(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), nz, ny, nx,
                        C.c_void_p(sx.data_ptr()), C.c_void_p(sy.data_ptr()),
                        C.c_void_p(ix.data_ptr()), C.c_void_p(iy.data_ptr()), None)
    torch.cuda.synchronize()
    return rc, sx.cpu().numpy(), sy.cpu().numpy(), ix.cpu().numpy(), iy.cpu().numpy()


# sizes mixed in this order so that the allocating and the static calls
# alternate between small and large images (the shared-memory limits the
# kernels need change with the image width)
@pytest.mark.parametrize("nz,ny,nx", [(1, 512, 512), (64, 64, 64), (16, 16, 16), (2, 128, 256)])
def test_static_matches_allocating(gb, nz, ny, nx):
    import torch

    L = gb.lib()
    for call, seed in enumerate((11, 12)):  # two calls in a row, different inputs
        a_np, b_np = _pairs(seed + nz, nz, ny, nx)
        a, b = torch.from_numpy(a_np).cuda(), torch.from_numpy(b_np).cuda()
        rc, sx, sy, ix, iy = _run(L, "arecgb_cc_shifts_static", a, b)
        assert rc == 0, gb.last_error()
        rc0, sx0, sy0, ix0, iy0 = _run(L, "arecgb_cc_shifts", a, b)
        assert rc0 == 0
        np.testing.assert_array_equal(ix, ix0)
        np.testing.assert_array_equal(iy, iy0)
        assert np.max(np.abs(sx - sx0)) <= SUBPIX_TOL, (call, sx, sx0)
        assert np.max(np.abs(sy - sy0)) <= SUBPIX_TOL, (call, sy, sy0)


def test_static_allocates_nothing(gb):
    import torch

    L = gb.lib()
    a_np, b_np = _pairs(3, 4, 128, 128)
    a, b = torch.from_numpy(a_np).cuda(), torch.from_numpy(b_np).cuda()
    assert _run(L, "arecgb_cc_shifts_static", a, b)[0] == 0  # set-up done
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert _run(L, "arecgb_cc_shifts_static", a, b)[0] == 0
    assert torch.cuda.mem_get_info()[0] == free0


def test_static_rejects_oversize(gb):
    import torch

    L = gb.lib()
    a = torch.zeros(2, 512, 512, device="cuda")
    sx = torch.zeros(2, device="cuda")
    for nz, ny, nx in [(2, 512, 512), (1, 1024, 256), (1, 48, 64), (1, 8, 512)]:
        rc = L.arecgb_cc_shifts_static(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), nz, ny,
                                       nx, C.c_void_p(sx.data_ptr()), C.c_void_p(sx.data_ptr()),
                                       None, None, None)
        assert rc == gb.ERR_ARG, (nz, ny, nx, rc)
        assert "cc_shifts_static" in gb.last_error()
    assert (2 * 512 * 512) > MAX_PIXELS
