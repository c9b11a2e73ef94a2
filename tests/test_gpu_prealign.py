"""Prealign's vertical profile alignment on the GPU (arecgb_profile_shifts:
TubeAlign::profile_gc_img / profile_cc_img's correlation loops) against the
reference's pieces (tests/golden/reference_prealign.npz) and the oracle
(oracle/prealign.py) on larger stacks.  The device sums the correlation
directly (FP32 products, FP64 chunk sums), the reference and the oracle through
an FFT; all three round the correlation to float before the 7-point fit.  On
a broad peak (the larger cases: widths up to 85 px) the fit's curvature is
small against the values, and one float rounding of a correlation value moves
the vertex by up to ~2e-3 px: tolerance 1e-4 px on the golden profiles
(narrow peaks), 5e-3 px on the larger ones."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-4
TOL_BROAD = 5e-3


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
    # steps an integer plus at most 0.3 px: the correlation's two largest
    # values never tie, so the arg max (and the 7 points fitted) are the same
    # for every implementation
    drift = np.cumsum(np.round(rng.normal(0, 2.0, prof_y)) + rng.uniform(-0.3, 0.3, prof_y))
    w = min(prof_x / 12.0, 85.0)  # peak width (the fit's conditioning falls as 1/w^2)
    prof = np.stack([np.exp(-((t - prof_x / 2 - d) / w) ** 2) +
                     0.5 * np.exp(-((t - prof_x / 3 - d) / (w / 3)) ** 2) for d in drift])
    prof = (prof + 0.02 * rng.standard_normal(prof.shape)).astype(np.float32)
    p = torch.from_numpy(prof).cuda()
    for succ in (False, True):
        s, spread = gb.profile_shifts(p, pad, succ)
        so, spo = P.profile_shifts(prof, pad, succ)
        if succ:
            # successive shifts are a running sum of per-pair fits: compare the
            # per-pair steps; the sum's error is a random walk of them
            e = np.abs(np.diff(s) - np.diff(so)).max()
            spread_tol = 3 * TOL_BROAD * np.sqrt(prof_y)
        else:
            e = np.abs(s - so).max()
            spread_tol = TOL_BROAD
        print(prof_y, prof_x, "successive" if succ else "global", "max |diff| %.2e px" % e)
        assert e < TOL_BROAD and abs(spread - spo) < spread_tol


def test_prealign_bad_args(gb):
    import torch

    p = torch.zeros(4, 40, device="cuda")
    for pad in (-1, 20, 25):  # segment length prof_x - 2 pad must be >= 1
        with pytest.raises(RuntimeError):
            gb.profile_shifts(p, pad)
