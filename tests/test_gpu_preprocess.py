"""Preprocessing on the GPU (arecImageTakeLog, periodicDecomposition,
makePeriodicSlice) against the reference's outputs
(tests/golden/reference_preprocess.npz) and the oracle (oracle/preprocess.py)
on larger stacks.

Tolerances: take-log within one float ulp (the device's double log rounded to
float against the C library's logf); the smooth part S within 1e-5 of max |S|
(the device sums its inverse DFT in FP32 over up to nx/2 + ny terms, the
reference uses float FFTs) and the corrected images within 1e-5 of their
range."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "reference_preprocess.npz")
S_TOL = 1e-5


def test_take_log(gb):
    import torch

    g = np.load(GOLD)
    x = torch.from_numpy(g["log_in"].copy()).cuda()
    gb.take_log(x)
    torch.cuda.synchronize()
    out, ref = x.cpu().numpy(), g["log_out"]
    ulp = np.spacing(np.abs(ref).astype(np.float32))
    assert np.all(np.abs(out - ref) <= ulp)
    assert np.array_equal(gb.arecImageTakeLog(g["log_in"])[ref == 0], ref[ref == 0])


def test_golden_periodic(gb):
    import torch

    g = np.load(GOLD)
    for tag in ("even", "odd"):
        img = g["pd_%s_in" % tag]
        d = torch.from_numpy(img.copy()).cuda()
        s = torch.zeros_like(d)
        gb.periodic_decomposition(d, smooth=s)
        ref_s = g["pd_%s_smooth0" % tag]
        e = np.abs(s[0].cpu().numpy() - ref_s).max() / np.abs(ref_s).max()
        print(tag, "smooth part rel err %.2e" % e)
        assert e <= S_TOL
        gb.periodic_decomposition(d)
        out = d.cpu().numpy()
        assert np.abs(out - g["pd_%s_out" % tag]).max() <= S_TOL * np.abs(img).max()
        c = gb.periodicDecomposition(img)
        assert np.abs(c - g["pd_%s_out" % tag]).max() <= S_TOL * np.abs(img).max()
        assert np.abs(gb.makePeriodicSlice(img[0]) - ref_s).max() <= S_TOL * np.abs(ref_s).max()


@pytest.mark.parametrize("shape", [(4, 256, 256), (2, 200, 333), (1, 1024, 1024), (3, 7, 2)])
def test_periodic_against_oracle(gb, shape):
    import torch

    from oracle import preprocess as P

    rng = np.random.default_rng(sum(shape))
    nz, ny, nx = shape
    img = (rng.random(shape) + np.linspace(0, 6, nx)[None, None, :] +
           np.linspace(0, 3, ny)[None, :, None]).astype(np.float32)
    d = torch.from_numpy(img.copy()).cuda()
    s = torch.zeros_like(d)
    gb.periodic_decomposition(d, smooth=s)
    gb.periodic_decomposition(d)
    torch.cuda.synchronize()
    for z in range(nz):
        ref_s = P.make_periodic_slice(img[z])
        e = np.abs(s[z].cpu().numpy() - ref_s).max() / np.abs(ref_s).max()
        assert e <= S_TOL, (shape, z, e)
    out = P.periodic_decomposition(img)
    e = np.abs(d.cpu().numpy() - out).max() / np.abs(img).max()
    print(shape, "corrected images: max rel err %.2e" % e)
    assert e <= S_TOL
