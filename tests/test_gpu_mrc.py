"""MRC stacks straight to and from device memory (arecgb_mrc_read_device /
arecgb_mrc_write_device) against numpy and the host readers: every mode, both
distributions over several ranks, files larger than one staging buffer (32
MiB) and a single image larger than one buffer (read in row ranges)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mrc(path, data, mode):
    hdr = np.zeros(256, np.int32)
    hdr[:4] = data.shape[2], data.shape[1], data.shape[0], mode
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.ascontiguousarray(data).tobytes())


def _part(a, rank, nranks, by_y):
    n = a.shape[1] if by_y else a.shape[0]
    cnt = n // nranks + (1 if rank < n % nranks else 0)
    off = rank * (n // nranks) + min(rank, n % nranks)
    return a[:, off:off + cnt] if by_y else a[off:off + cnt]


@pytest.mark.parametrize("shape,mode", [((7, 33, 20), 2), ((5, 16, 24), 1), ((5, 16, 24), 6),
                                        ((12, 1024, 1024), 2), ((2, 3000, 3000), 2),
                                        ((1, 4100, 4100), 1)])
def test_read_device(gb, tmp_path, shape, mode):
    rng = np.random.default_rng(sum(shape) + mode)
    if mode == 2:
        a = rng.standard_normal(shape).astype(np.float32)
    else:
        a = rng.integers(-32768, 32767, size=shape).astype(np.int16)
    p = str(tmp_path / "s.mrc")
    _mrc(p, a, mode)
    assert gb.mrc_read_header(p) == (shape[2], shape[1], shape[0], mode)
    want = a.astype(np.float32)
    for nranks in (1, 3):
        for by_y in (False, True):
            for r in range(nranks):
                t = gb.mrc_read_device(p, r, nranks, by_y)
                assert np.array_equal(t.cpu().numpy(), _part(want, r, nranks, by_y)), \
                    (nranks, by_y, r)


@pytest.mark.parametrize("shape", [(3, 17, 29), (9, 1024, 1024)])
def test_write_device(gb, tmp_path, shape):
    import torch

    rng = np.random.default_rng(shape[0])
    a = (rng.standard_normal(shape) * 5 + 2).astype(np.float32)
    p, q = str(tmp_path / "d.mrc"), str(tmp_path / "h.mrc")
    gb.mrc_write_device(p, torch.from_numpy(a).cuda())
    assert gb.arecWriteImage(q, a) == 0
    hd = np.fromfile(p, np.uint8, 1024)
    hh = np.fromfile(q, np.uint8, 1024)
    # every header byte but the mean (FP64 sum in another order) agrees
    keep = np.r_[0:84, 88:1024]
    assert np.array_equal(hd[keep], hh[keep])
    md, mh = np.frombuffer(hd[84:88].tobytes(), np.float32)[0], \
        np.frombuffer(hh[84:88].tobytes(), np.float32)[0]
    assert abs(md - mh) <= 1e-6 * abs(mh)
    assert np.array_equal(np.fromfile(p, np.float32)[256:], a.ravel())
    b, st = gb.arecReadImage(p)
    assert st == 0 and np.array_equal(a, b)
