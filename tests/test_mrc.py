"""MRC stack files: the library's reference-named readers and writers
(arecReadImage, arecWriteImage, arecReadImageDistbyZ/Y, arecWriteImageMergeY/Z,
host code, no GPU) against the reference's own (built from its sources in
oracle/_ref) and against files numpy writes, and the rank split of the
device reader (a size query, no GPU)."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HAVE_REF = os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libarec_ref.so"))

# header bytes the reference leaves uninitialised (machinestamp 212-215,
# labels 224-1023); everything else must agree byte for byte
SET_BYTES = np.r_[0:212, 216:224]


def _mrc(path, data, mode):
    """A minimal MRC file: 1024-byte header (nx, ny, nz, mode) + data."""
    hdr = np.zeros(256, np.int32)
    hdr[:4] = data.shape[2], data.shape[1], data.shape[0], mode
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.ascontiguousarray(data).tobytes())


@pytest.fixture(scope="module")
def gbl():
    import arec3d_gb300 as gb

    gb.build()
    return gb


def test_roundtrip_and_modes(gbl, tmp_path):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((5, 7, 9)).astype(np.float32)
    p = str(tmp_path / "a.mrc")
    assert gbl.arecWriteImage(p, a) == 0
    assert gbl.arecReadImageHeader(p) == ((9, 7, 5), 0)
    b, st = gbl.arecReadImage(p)
    assert st == 0 and np.array_equal(a, b)
    for dist in ("Z", "Y"):
        b, _ = gbl.arecReadImage(p, dist)
        assert np.array_equal(a, b)
    hdr = np.fromfile(p, np.float32, 256)
    assert hdr[19] == np.float32(a.min()) and hdr[20] == np.float32(a.max())
    assert abs(hdr[21] - a.astype(np.float64).mean()) <= 1e-6 * max(1.0, abs(a).max())
    s = rng.integers(-32768, 32767, size=(3, 4, 6)).astype(np.int16)
    for mode in (1, 6):
        _mrc(str(tmp_path / "s.mrc"), s, mode)
        b, st = gbl.arecReadImage(str(tmp_path / "s.mrc"))
        assert st == 0 and np.array_equal(b, s.astype(np.float32))
    _mrc(str(tmp_path / "bad.mrc"), s, 0)
    b, st = gbl.arecReadImage(str(tmp_path / "bad.mrc"))
    assert st == -1 and b is None
    b, st = gbl.arecReadImage(str(tmp_path / "missing.mrc"))
    assert st == -1


def test_rank_split_matches_reference_rule(gbl, tmp_path):
    """Sizes each rank gets (the first n % nranks ranks take one more)."""
    import ctypes as C

    p = str(tmp_path / "z.mrc")
    _mrc(p, np.zeros((10, 7, 3), np.float32), 2)
    L = gbl.lib()
    for nranks in (1, 3, 4):
        for by_y, n in ((0, 10), (1, 7)):
            sizes = []
            for r in range(nranks):
                nx, nyl, nzl = C.c_int(), C.c_int(), C.c_int()
                assert L.arecgb_mrc_read_device(os.fsencode(p), r, nranks, by_y, None, 0,
                                                C.byref(nx), C.byref(nyl), C.byref(nzl),
                                                None) == 0
                sizes.append(nyl.value if by_y else nzl.value)
            want = [n // nranks + (1 if r < n % nranks else 0) for r in range(nranks)]
            assert sizes == want, (nranks, by_y, sizes)


@pytest.mark.skipif(not HAVE_REF, reason="reference not built here")
def test_against_reference_build(gbl, tmp_path):
    import oracle as O

    R = O.Reference()
    rng = np.random.default_rng(8)
    a = (rng.standard_normal((4, 6, 10)) * 3 + 1).astype(np.float32)
    for merge in ("", "Y", "Z"):
        pr, pg = str(tmp_path / "r.mrc"), str(tmp_path / "g.mrc")
        R.write_image(pr, a, merge)
        gbl.arecWriteImage(pg, a, merge)
        hr = np.fromfile(pr, np.uint8, 1024)
        hg = np.fromfile(pg, np.uint8, 1024)
        assert np.array_equal(hr[SET_BYTES], hg[SET_BYTES]), merge
        assert np.array_equal(np.fromfile(pr, np.uint8)[1024:], np.fromfile(pg, np.uint8)[1024:])
        for dist in ("", "Z", "Y"):
            x, _ = R.read_image(pg, dist)
            y, _ = gbl.arecReadImage(pr, dist)
            assert np.array_equal(x, a) and np.array_equal(y, a)
    s = rng.integers(-3000, 3000, size=(2, 5, 8)).astype(np.int16)
    _mrc(str(tmp_path / "s.mrc"), s, 1)
    x, _ = R.read_image(str(tmp_path / "s.mrc"))
    y, _ = gbl.arecReadImage(str(tmp_path / "s.mrc"))
    assert np.array_equal(x, y)
