"""Generates the golden fixtures in tests/golden/*.npz by running the reference
itself (AREC3D, compiled from its own sources into oracle/_ref by
oracle/build_ref.sh) on small seeded inputs.  Run in the container that has the
reference checkout:

    bash oracle/build_ref.sh && python tests/golden/make_golden.py \
        [--rotation|--preprocess|--prealign|--compat]

(each flag writes only its own file: reference_rotation.npz,
reference_preprocess.npz, reference_prealign.npz, reference_compat.npz.)

The reference's linear weighting (pmethod=1) reads two entries past its
coordinate table; to make those reads return zero (as they do for large tables
served by mmap), this script first lowers glibc's mmap threshold so every table
of 4 KiB or more gets its own zero-filled pages.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

M_MMAP_THRESHOLD = -3


def main():
    ctypes.CDLL("libc.so.6").mallopt(M_MMAP_THRESHOLD, 4096)
    import oracle as O

    R = O.Reference()
    rng = np.random.default_rng(20261203)
    out = {}

    # geometry (arecAllocateCylImage)
    for r in (0.5, 1.0, 1.5, 7.5, 12.0, 31.5):
        im = R._cyl(r, 1)
        nr = im.nrays
        out["cyl_%g_cord" % r] = np.ctypeslib.as_array(im.cord, shape=(nr, 2)).copy()
        out["cyl_%g_nx" % r] = np.array(im.nx)

    # solvers (nx 64, 4 slices, 24 angles), seeded noisy data
    nx, ny, na = 64, 4, 24
    ang = (np.arange(na) * np.pi / na).astype(np.float32)
    _, nr, _ = O.cyl(0.5 * (nx - 1))
    xt = rng.random((nr, ny), dtype=np.float32)
    for tag, w in (("lin", 1), ("kb", 2), ("sq", 3)):
        b = O.project(w, 0.5 * (nx - 1), xt, ang)
        b = (b + 0.01 * rng.standard_normal(b.shape)).astype(np.float32)
        out["solve_%s_b" % tag] = b
        nm = {"lin": "", "kb": "_KB", "sq": "_SQ"}[tag]
        xs, st = R.solve("cyl_sirt" + nm, b, ang, 2e-4, 12, 0.0)
        assert st == 0
        out["solve_%s_sirt" % tag] = xs
        if w == 1:
            xo, _ = O.sirt(w, b, ang, lam=2e-4, maxit=12, tol=0.0)
            assert np.array_equal(xo, xs), "reference read nonzero memory past its table"
        xc, st = R.solve("cyl_cgls" + nm, b, ang, 0.0, 10, 1e-7)
        out["solve_%s_cgls" % tag] = xc
        out["solve_%s_cgls_status" % tag] = np.array(st)
    out["solve_angles"] = ang

    # projectors (radius 31.5 -> nx 64; tables > 4 KiB so pmethod=1 reads zeros)
    radius, ny = 31.5, 3
    ang = np.array([0.0, 0.31, 0.7853982, 1.2, 1.5707964, 2.4, 3.0, 4.1, 21.123], np.float32)
    _, nr, _ = O.cyl(radius)
    x = rng.standard_normal((nr, ny)).astype(np.float32)
    s = rng.standard_normal((len(ang), ny, 64)).astype(np.float32)
    out["proj_angles"] = ang
    out["proj_x"] = x
    out["proj_s"] = s
    for tag, fp, bp in (("lin", "arecProject2D", "arecBackProject2D"),
                        ("kb", "arecProject2D_KB", "arecBackProject2D_KB"),
                        ("sq", "arecProject2D_SQ", "arecBackProject2D_SQ")):
        q, st = R.project(fp, radius, x, ang)
        assert st == 0
        g, st = R.backproject(bp, radius, s, ang)
        assert st == 0
        out["proj_%s_q" % tag] = q
        out["proj_%s_g" % tag] = g

    # cross-correlation (FFT of the FFTW-API stand-in, see oracle/shim)
    ny2, nx2 = 32, 64
    a = rng.random((3, ny2, nx2), dtype=np.float32)
    bb = np.stack([np.roll(a[0], (2, -7), axis=(0, 1)), np.roll(a[1], (-5, 11), axis=(0, 1)),
                   -np.roll(a[2], (1, 1), axis=(0, 1))]).astype(np.float32)
    bb += (0.01 * rng.standard_normal(bb.shape)).astype(np.float32)
    out["cc_a"] = a
    out["cc_b"] = bb
    out["cc_c0"] = R.ccorr2d(a[0], bb[0])
    sx, sy, st = R.cc_images(a, bb)
    out["cc_sx"], out["cc_sy"] = sx, sy
    pk = rng.standard_normal((16, 16)).astype(np.float32)
    pk[4, 9] = -20.0
    out["speak_neg_c"] = pk
    out["speak_neg_xy"] = np.array(R.speak(pk), np.float32)

    np.savez_compressed(os.path.join(HERE, "reference_small.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_small.npz"))


def blobs(ny, nx, angle_deg, rng):
    """Seeded test image: two Gaussian blobs and a bar, rotated by angle_deg about
    the centre, plus 1 % noise."""
    yy, xx = np.mgrid[0:ny, 0:nx].astype(np.float64)
    t = np.deg2rad(angle_deg)
    x, y = xx - nx / 2, yy - ny / 2
    xr, yr = x * np.cos(t) + y * np.sin(t), -x * np.sin(t) + y * np.cos(t)
    s = nx / 64.0
    img = (np.exp(-((xr - 6 * s) ** 2 / (30 * s * s) + (yr - 3 * s) ** 2 / (8 * s * s))) +
           0.6 * np.exp(-((xr + 8 * s) ** 2 / (10 * s * s) + (yr + 5 * s) ** 2 / (20 * s * s))) +
           0.3 * ((np.abs(xr) < 12 * s) & (np.abs(yr - 9 * s) < 2 * s)))
    return (img + 0.01 * rng.standard_normal(img.shape)).astype(np.float32)


def rotation():
    """Rotation search and rotations (arecRotCCImages, arecRotateImages,
    _skew, _skew_safe) on a 4-slice 48 x 64 stack."""
    import oracle as O

    R = O.Reference()
    rng = np.random.default_rng(20261204)
    ny, nx = 48, 64
    truth = [7.5, -4.0, 30.0, 0.0]
    ref = np.stack([blobs(ny, nx, 0.0, rng) for _ in truth])
    rot = np.stack([blobs(ny, nx, a, rng) for a in truth])
    out = {"rot_ref": ref, "rot_img": rot}
    ang, st = R.rot_cc_images(ref, rot, 20)
    assert st == 0
    out["rotcc_r2"] = np.array(20)
    out["rotcc_angles"] = ang
    skew_in = np.array([3.0, 25.0, -60.0, 370.0], np.float32)
    out["skew_angles_in"] = skew_in
    out["skew_img"], out["skew_angles"] = R.rotate_images(rot, skew_in, "_skew")
    out["bilinear_img"], _ = R.rotate_images(rot, skew_in, "")
    safe_in = np.array(ang, np.float32).copy()
    safe_in[3] = 5.0  # a slice the rotation makes worse
    out["safe_angles_in"] = safe_in
    out["safe_img"], out["safe_angles"] = R.rotate_images_skew_safe(rot, ref, safe_in)
    out["ncc"] = np.array([R.ncc_filtered(a, b) for a, b in zip(ref, rot)])
    np.savez_compressed(os.path.join(HERE, "reference_rotation.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_rotation.npz"))


def preprocess():
    """arecImageTakeLog and periodicDecomposition / makePeriodicSlice on seeded
    stacks (sizes 3 x 24 x 40 and 1 x 33 x 50: even and odd)."""
    import ctypes as C

    import oracle as O

    R = O.Reference()
    rng = np.random.default_rng(20261205)
    out = {}
    raw = (rng.random((3, 24, 40)) * 2.0).astype(np.float32)
    raw[0, 0, :4] = [0.0, -1.0, 1.0, 1e-30]
    out["log_in"] = raw
    a = raw.copy()
    f = R.L._Z16arecImageTakeLog5Image
    f.argtypes = [O.ArecImage]
    f.restype = None
    f(R._cb(a))
    out["log_out"] = a
    pd = R.L._Z21periodicDecomposition5Image
    pd.argtypes = [O.ArecImage]
    pd.restype = None
    mk = R.L._Z17makePeriodicSliceiiPfS_
    mk.argtypes = [C.c_int, C.c_int, O._f32p, O._f32p]
    mk.restype = None
    for tag, shape in (("even", (3, 24, 40)), ("odd", (1, 33, 50))):
        nz, ny, nx = shape
        img = (rng.random(shape) + np.linspace(0, 4, nx)[None, None, :] +
               np.linspace(0, 2, ny)[None, :, None]).astype(np.float32)
        out["pd_%s_in" % tag] = img
        s = np.zeros((ny, nx), np.float32)
        mk(nx, ny, img[0].copy(), s)
        out["pd_%s_smooth0" % tag] = s
        a = img.copy()
        pd(R._cb(a))
        out["pd_%s_out" % tag] = a
    np.savez_compressed(os.path.join(HERE, "reference_preprocess.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_preprocess.npz"))


def prealign():
    """Prealign's profile alignment: the two TubeAlign correlation loops as the
    oracle restates them, with ccorr1d and findMaxCC_fit taken from the
    reference's own TubeAlign_utils.cpp (oracle/_ref/libprealign_ref.so)."""
    import ctypes as C

    from oracle import prealign as P

    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libprealign_ref.so"))
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    cc = L._Z7ccorr1diPfS_S_
    cc.argtypes = [C.c_int, f32p, f32p, f32p]
    cc.restype = None
    fit = L._Z13findMaxCC_fitPKfi
    fit.argtypes = [f32p, C.c_int]
    fit.restype = C.c_double

    def ref_pair(x, y):
        n = len(x)
        c = np.zeros(n, np.float32)
        cc(n, np.ascontiguousarray(x, np.float32).copy(), np.ascontiguousarray(y, np.float32).copy(), c)
        return fit(c, n)

    rng = np.random.default_rng(20261206)
    prof_y, prof_x, pad = 12, 200, 20
    t = np.arange(prof_x)
    drift = np.cumsum(rng.normal(0, 1.5, prof_y))
    prof = np.stack([np.exp(-((t - 100 - d) / 18.0) ** 2) + 0.4 * np.exp(-((t - 60 - d) / 6.0) ** 2)
                     for d in drift]).astype(np.float32)
    prof += (0.01 * rng.standard_normal(prof.shape)).astype(np.float32)
    out = {"profiles": prof, "pad": np.array(pad)}
    for tag, succ in (("global", False), ("successive", True)):
        s, spread = P.profile_shifts(prof, pad, succ, fit_pair=ref_pair)
        out[tag + "_shifts"] = s
        out[tag + "_spread"] = np.array(spread)
    np.savez_compressed(os.path.join(HERE, "reference_prealign.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_prealign.npz"))


def _stdout_of(fn):
    """Runs fn() with file descriptor 1 sent to a temporary file; returns
    (fn's result, the text the C library printed)."""
    import tempfile

    sys.stdout.flush()
    libc = ctypes.CDLL(None)
    libc.fflush(None)
    with tempfile.TemporaryFile(mode="w+b") as tmp:
        saved = os.dup(1)
        os.dup2(tmp.fileno(), 1)
        try:
            res = fn()
            libc.fflush(None)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        tmp.seek(0)
        text = tmp.read().decode()
    return res, text


def compat():
    """The reference's solver entry points as a caller of the library sees
    them: warm-started CGLS from a non-NULL xvol (areccgls.cpp:323-340), the
    Kaiser-Bessel CGLS at an odd width (its integer radius nx/2 needs odd nx,
    areccgls_KB.cpp:37-48), and the log lines the solvers print on rank 0
    (areccgls.cpp:198, 358-453; arecsirt.cpp:131-156, 343-373)."""
    import oracle as O

    ctypes.CDLL("libc.so.6").mallopt(M_MMAP_THRESHOLD, 4096)
    R = O.Reference()
    small = np.load(os.path.join(HERE, "reference_small.npz"))
    rng = np.random.default_rng(20261207)
    out = {}
    ang = small["solve_angles"]
    for tag, nm in (("sq", "_SQ"), ("kb", "_KB")):
        b = small["solve_%s_b" % tag]
        if tag == "kb":  # odd width for the KB CGLS: radius 32 -> nx 65
            nx, ny = 65, 4
            _, nr, _ = O.cyl(32.0)
            xt = rng.random((nr, ny), dtype=np.float32)
            b = O.project(O.KB, 32.0, xt, ang)
            b = (b + 0.01 * rng.standard_normal(b.shape)).astype(np.float32)
            out["kb65_b"] = b
            x, st = R.solve("cyl_cgls_KB", b, ang, 0.0, 5, 1e-7)
            assert st == 0
            out["kb65_cgls"] = x
            out["kb65_maxit"] = np.array(5)
            x0 = (x * 0.5).astype(np.float32)
            maxit = 5
        else:
            x0 = small["solve_sq_sirt"]
            maxit = 6
        out["warm_%s_x0" % tag] = x0
        x, st = R.solve("cyl_cgls" + nm, b, ang, 0.0, maxit, 1e-7, x0=x0)
        assert st == 0
        out["warm_%s_cgls" % tag] = x
        out["warm_%s_maxit" % tag] = np.array(maxit)
    b = small["solve_sq_b"]
    (_, st), text = _stdout_of(lambda: R.solve("cyl_cgls_SQ", b, ang, 0.0, 10, 1e-7))
    assert st == 0
    out["log_cgls_sq"] = np.array(text)
    (_, st), text = _stdout_of(lambda: R.solve("cyl_sirt_SQ", b, ang, 2e-4, 12, 0.0))
    assert st == 0
    out["log_sirt_sq"] = np.array(text)
    np.savez_compressed(os.path.join(HERE, "reference_compat.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_compat.npz"))


if __name__ == "__main__":
    if "--compat" in sys.argv:
        compat()
    elif "--rotation" in sys.argv:
        rotation()
    elif "--preprocess" in sys.argv:
        preprocess()
    elif "--prealign" in sys.argv:
        prealign()
    else:
        main()
        rotation()
        preprocess()
        prealign()
        compat()
