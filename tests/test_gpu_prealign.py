"""Prealign's vertical profile alignment on the GPU (arecgb_profile_shifts:
TubeAlign::profile_gc_img / profile_cc_img's correlation loops) against the
reference's pieces (tests/golden/reference_prealign.npz) and the oracle
(oracle/prealign.py) on larger stacks.  Tolerance 1e-4 px: the device sums
the correlation directly (FP32 products, FP64 chunk sums), the reference
through a float FFT."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-4


def test_golden_prealign(gb):
    import torch

    g = np.load(os.path.join(ROOT, "tests", "golden", "reference_prealign.npz"))
    p = torch.from_numpy(g["profiles"].copy()).cuda()
    for tag, succ in (("global", False), ("successive", True)):
        s, spread = gb.profile_shifts(p, int(g["pad"]), succ)
        print(tag, s, g[tag + "_shifts"])
        assert np.abs(s - g[tag + "_shifts"]).max() < TOL
        assert abs(spread - float(g[tag + "_spread"])) < TOL


@pytest.mark.parametrize("prof_y,prof_x,pad", [(360, 1024, 50), (1200, 2048, 100), (5, 57, 3)])
def test_prealign_against_oracle(gb, prof_y, prof_x, pad):
    import torch

    from oracle import prealign as P

    rng = np.random.default_rng(prof_y + prof_x)
    t = np.arange(prof_x)
    drift = np.cumsum(rng.normal(0, 2.0, prof_y))
    w = prof_x / 12.0
    prof = np.stack([np.exp(-((t - prof_x / 2 - d) / w) ** 2) +
                     0.5 * np.exp(-((t - prof_x / 3 - d) / (w / 3)) ** 2) for d in drift])
    prof = (prof + 0.02 * rng.standard_normal(prof.shape)).astype(np.float32)
    p = torch.from_numpy(prof).cuda()
    for succ in (False, True):
        s, spread = gb.profile_shifts(p, pad, succ)
        so, spo = P.profile_shifts(prof, pad, succ)
        e = np.abs(s - so).max()
        print(prof_y, prof_x, "successive" if succ else "global", "max |diff| %.2e px" % e)
        assert e < TOL and abs(spread - spo) < TOL


def test_prealign_bad_args(gb):
    import torch

    p = torch.zeros(4, 40, device="cuda")
    for pad in (-1, 20, 25):  # segment length prof_x - 2 pad must be >= 1
        with pytest.raises(RuntimeError):
            gb.profile_shifts(p, pad)
