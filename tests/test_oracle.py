"""The oracle (oracle/arec_oracle.c, a CPU restatement of the reference path)
pinned against the reference's own known answers (AREC3D/AREC3D_test/
AREC3D_test.cpp), against golden fixtures produced by the reference itself
(tests/golden/make_golden.py), and -- where the reference is built in this
checkout -- against the reference directly."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, rel_l2

GOLD = os.path.join(ROOT, "tests", "golden", "reference_small.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


# ---- known answers of the reference's Catch suite -------------------------------------------
def test_cylvol_odd(oc):
    nx, nr, cord = oc.cyl(1.0)  # AREC3D_test.cpp:8-40
    assert (nx, nr) == (3, 5)
    assert cord.tolist() == [[1, 0], [0, 1], [1, 1], [2, 1], [1, 2]]


def test_cylvol_even(oc):
    nx, nr, cord = oc.cyl(0.5)  # AREC3D_test.cpp:42-70
    assert (nx, nr) == (2, 4)
    assert cord.tolist() == [[0, 0], [1, 0], [0, 1], [1, 1]]


def test_projection_odd(oc):
    x = np.zeros((5, 2), np.float32)  # AREC3D_test.cpp:97-147
    x.ravel()[4], x.ravel()[5] = 1.0, 2.0
    q = oc.project(oc.SQ, 1.0, x, np.zeros(1, np.float32))
    assert q.sum() == pytest.approx(3.0)
    assert q.ravel()[1] == pytest.approx(1.0, rel=1.2e-5)
    assert q.ravel()[4] == pytest.approx(2.0, rel=1.2e-5)


def test_backprojection_odd(oc):
    q = np.zeros((1, 2, 3), np.float32)  # AREC3D_test.cpp:149-189
    q.ravel()[1], q.ravel()[4] = 1.0, 2.0
    g = oc.backproject(oc.SQ, 1.0, q, np.zeros(1, np.float32))
    assert g.sum() == pytest.approx(9.0)


@pytest.mark.parametrize("w,radius,ang,step", [
    (3, 1.0, [1.475, 21.123, 2.123], 1),  # AREC3D_test.cpp:216-243
    (3, 1.5, [0.698132, 1.22173], 3),     # :245-271
    (2, 0.5, [0.698132, 1.22173], 3),     # :298-324
])
def test_exact_adjoint(oc, w, radius, ang, step):
    ang = np.array(ang, np.float32)
    ny = 2
    nx, nr, _ = oc.cyl(radius)
    nv, ns = nr * ny, len(ang) * ny * nx
    for a in range(0, nv, step):
        x = np.zeros(nv, np.float32)
        x[a] = 1
        q = oc.project(w, radius, x.reshape(nr, ny), ang).ravel()
        for b in range(0, ns, step):
            s = np.zeros(ns, np.float32)
            s[b] = 1
            g = oc.backproject(w, radius, s.reshape(len(ang), ny, nx), ang).ravel()
            assert q[b] == g[a]


# ---- golden fixtures made by the reference ---------------------------------------------------
@pytest.mark.parametrize("r", [0.5, 1.0, 1.5, 7.5, 12.0, 31.5])
def test_golden_cylinder(oc, gold, r):
    nx, nr, cord = oc.cyl(r)
    assert nx == int(gold["cyl_%g_nx" % r])
    np.testing.assert_array_equal(cord, gold["cyl_%g_cord" % r])


@pytest.mark.parametrize("tag,w", [("lin", 1), ("kb", 2), ("sq", 3)])
def test_golden_projectors(oc, gold, tag, w):
    ang, x, s = gold["proj_angles"], gold["proj_x"], gold["proj_s"]
    q = oc.project(w, 31.5, x, ang)
    g = oc.backproject(w, 31.5, s, ang)
    np.testing.assert_array_equal(q, gold["proj_%s_q" % tag])
    np.testing.assert_array_equal(g, gold["proj_%s_g" % tag])


@pytest.mark.parametrize("tag,w", [("lin", 1), ("kb", 2), ("sq", 3)])
def test_golden_solvers(oc, gold, tag, w):
    ang, b = gold["solve_angles"], gold["solve_%s_b" % tag]
    xs, _ = oc.sirt(w, b, ang, lam=2e-4, maxit=12, tol=0.0)
    np.testing.assert_array_equal(xs, gold["solve_%s_sirt" % tag])
    if tag == "kb":
        # even nx: the reference's KB CGLS builds its volumes with radius nx/2 and
        # returns -1 (areccgls_KB.cpp:37,112-113)
        assert int(gold["solve_kb_cgls_status"]) == -1
        return
    xc, _ = oc.cgls(w, b, ang, maxit=10, tol=1e-7)
    np.testing.assert_array_equal(xc, gold["solve_%s_cgls" % tag])


def test_golden_ccorr(oc, gold):
    a, b = gold["cc_a"], gold["cc_b"]
    c = oc.ccorr2d(a[0], b[0])
    assert rel_l2(c, gold["cc_c0"]) < 1e-6
    sx, sy = oc.cc_images(a, b)
    np.testing.assert_allclose(sx, gold["cc_sx"], atol=1e-4)
    np.testing.assert_allclose(sy, gold["cc_sy"], atol=1e-4)
    xt, yt, _, _ = oc.speak(gold["speak_neg_c"])
    np.testing.assert_array_equal(np.array([xt, yt], np.float32), gold["speak_neg_xy"])


def test_fft64_matches_numpy(oc):
    rng = np.random.default_rng(0)
    for ny, nx in ((16, 16), (12, 20), (64, 32), (7, 5)):
        x = rng.standard_normal((ny, nx)).astype(np.float32)
        y = rng.standard_normal((ny, nx)).astype(np.float32)
        c = oc.ccorr2d(x, y)
        ref = np.real(np.fft.ifft2(np.conj(np.fft.fft2(x)) * np.fft.fft2(y))) * nx * ny
        assert rel_l2(c, ref) < 1e-6


def test_quad2dfit_paraboloid(oc):
    # exact paraboloid with its vertex at (+0.3, -0.2) is recovered
    z = np.zeros(9, np.float32)
    for j in (-1, 0, 1):
        for i in (-1, 0, 1):
            z[(j + 1) * 3 + (i + 1)] = 5.0 - (i - 0.3) ** 2 - 2 * (j + 0.2) ** 2
    xs, ys, pv = oc.quad2dfit(z)
    assert xs == pytest.approx(0.3, abs=1e-5) and ys == pytest.approx(-0.2, abs=1e-5)


def test_threaded_slabs_agree(oc, gold):
    """Slabs of slices on several threads (the reference's MPI ranks) give the
    single-rank result up to the order of the scalar sums."""
    ang, b = gold["solve_angles"], gold["solve_sq_b"]
    x1, t1 = oc.cgls(3, b, ang, maxit=6, tol=0.0, nthreads=1)
    x2, t2 = oc.cgls(3, b, ang, maxit=6, tol=0.0, nthreads=3)
    assert rel_l2(x2, x1) < 1e-6


# ---- the reference itself (only in a checkout where oracle/build_ref.sh ran) -----------------
@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libarec_ref.so")),
                    reason="reference not built here")
def test_against_reference_build(oc):
    code = r"""
import ctypes, sys, numpy as np
ctypes.CDLL("libc.so.6").mallopt(-3, 4096)
sys.path.insert(0, %r)
import oracle as O
R = O.Reference()
rng = np.random.default_rng(5)
for radius in (7.5, 20.0, 40.5):
    _, nr, _ = O.cyl(radius)
    ang = rng.uniform(-4, 4, 11).astype(np.float32)
    x = rng.standard_normal((nr, 5)).astype(np.float32)
    for w, fp, bp in ((1, "arecProject2D", "arecBackProject2D"), (2, "arecProject2D_KB", "arecBackProject2D_KB"), (3, "arecProject2D_SQ", "arecBackProject2D_SQ")):
        q = O.project(w, radius, x, ang); qr, _ = R.project(fp, radius, x, ang)
        g = O.backproject(w, radius, q, ang); gr, _ = R.backproject(bp, radius, q, ang)
        if w == 1:
            g, gr = g[:-2], gr[:-2]
        assert np.array_equal(q, qr) or w == 1 and np.array_equal(q[:, :, :], qr), (radius, w)
        assert np.array_equal(g, gr), (radius, w)
print("ok")
""" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-2000:]


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libarec_ref.so")),
                    reason="reference not built here")
def test_cgls_stat_against_reference_build(oc):
    """The oracle's statistically weighted CGLS against the reference's own
    cyl_cgls_SQ_stat / cyl_cgls_KB_stat (areccgls_stat.cpp), bit for bit."""
    code = r"""
import ctypes, sys, numpy as np
ctypes.CDLL("libc.so.6").mallopt(-3, 4096)
sys.path.insert(0, %r)
import oracle as O
R = O.Reference()
rng = np.random.default_rng(9)
for radius, ny, na in ((12, 4, 15), (20, 3, 24)):
    nx = 2 * radius + 1
    ang = (np.arange(na) * np.pi / na).astype(np.float32)
    b = (rng.random((na, ny, nx)) * 2.0).astype(np.float32)
    for w, name in ((3, "cyl_cgls_SQ_stat"), (2, "cyl_cgls_KB_stat")):
        xr, st = R.solve(name, b, ang, 0.0, 6, 0.0)
        x, tr = O.cgls_stat(w, b, ang, maxit=6, tol=0.0)
        assert st == 0, (name, st)
        assert np.array_equal(x, xr), (name, radius, float(np.abs(x - xr).max()))
print("ok")
""" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, (r.stdout[-1500:], r.stderr[-2000:])


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libarec_ref.so")),
                    reason="reference not built here")
def test_fshift2d_against_reference_build(oc):
    """The oracle's fshift2d against the reference's own (align2dstack.cpp:566)
    over the FFTW-API stand-in."""
    code = r"""
import ctypes, sys, numpy as np
ctypes.CDLL("libc.so.6").mallopt(-3, 4096)
sys.path.insert(0, %r)
import oracle as O
R = O.Reference()
rng = np.random.default_rng(4)
for ny, nx, sx, sy in ((32, 64, 3.25, -7.5), (64, 64, -0.4, 12.7), (48, 80, 5.0, 2.0)):
    img = rng.standard_normal((ny, nx)).astype(np.float32)
    a, b = O.fshift2d(img, sx, sy), R.fshift2d(img, sx, sy)
    e = np.linalg.norm(a - b) / np.linalg.norm(b)
    assert e < 1e-6, (ny, nx, e)
print("ok")
""" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, (r.stdout[-1500:], r.stderr[-2000:])


def test_unet_oracle_gradients_finite_differences():
    """The U-Net oracle's autograd gradients (FP64, no bf16 rounding) against
    central differences on a few parameters of every layer."""
    pytest.importorskip("torch")
    from oracle import unet_ref

    layers, n = unet_ref.layer_table()
    rng = np.random.default_rng(0)
    p = np.zeros(n)
    for l in layers:
        nw = l["cin"] if l["name"] == "out" else l["cout"] * 9 * l["cin"]
        p[l["w_off"]:l["w_off"] + nw] = rng.standard_normal(nw) * np.sqrt(2.0 / (9 * l["cin"]))
        p[l["b_off"]:l["b_off"] + l["cout"]] = 0.1 * rng.standard_normal(l["cout"])
    x = rng.standard_normal((1, 16, 16))
    dout = rng.standard_normal((1, 16, 16))
    _, g = unet_ref.forward_and_grads(p, layers, n, x, dout, bf16=False)

    def f(q):
        import torch

        t = unet_ref.unpack(q, layers)
        return float((unet_ref.forward(t, torch.as_tensor(x), bf16=False) * torch.as_tensor(dout)).sum())

    h = 1e-6
    for l in layers:
        for off in (l["w_off"], l["w_off"] + 5, l["b_off"]):
            q1, q2 = p.copy(), p.copy()
            q1[off] += h
            q2[off] -= h
            fd = (f(q1) - f(q2)) / (2 * h)
            assert abs(fd - g[off]) <= 1e-5 * max(1.0, abs(fd)), (l["name"], off, fd, g[off])


# ---- rotational alignment (arecRotCCImages, arecRotateImages*) --------------------------------
ROT_GOLD = os.path.join(ROOT, "tests", "golden", "reference_rotation.npz")


def test_golden_rotation_oracle():
    """The oracle's rotation search and rotations against the reference's own
    outputs on the golden stack: rotations bit for bit (the shears, the bilinear
    rotation, the guarded shear rotation and their angle updates), the
    rotation search within the FFT rounding of its float cross-correlation."""
    from oracle import rotation as R

    g = np.load(ROT_GOLD)
    ref, img = g["rot_ref"], g["rot_img"]
    ang = R.rot_cc_angles(ref, img, int(g["rotcc_r2"]))
    # the reference's ccorr1d output is float (FFTW-API stand-in); 1e-3 deg is
    # 0.0022 of a profile sample at r2 = 20 (125 samples per turn)
    assert np.abs(ang - g["rotcc_angles"]).max() < 1e-3, (ang, g["rotcc_angles"])
    out, a = R.rotate_images_skew(img, g["skew_angles_in"])
    assert np.array_equal(out, g["skew_img"]) and np.array_equal(a, g["skew_angles"])
    assert np.array_equal(R.rotate_images(img, g["skew_angles_in"]), g["bilinear_img"])
    out, a, n_rot, mean_cc = R.rotate_images_skew_safe(img, ref, g["safe_angles_in"])
    assert np.array_equal(out, g["safe_img"]) and np.array_equal(a, g["safe_angles"])
    assert n_rot == 3
    cc = [R.ncc_filtered(x, y) for x, y in zip(ref, img)]
    assert np.allclose(cc, g["ncc"], rtol=1e-12, atol=0)


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libarec_ref.so")),
                    reason="reference not built here")
def test_rotation_pieces_against_reference_build():
    """Each piece of the oracle's rotation path against the reference's own
    function: shearX_circ / shearY_circ, rotate2d, getRadialProfile (bit for
    bit), findPeak1d on the same correlation, the filtered NCC."""
    code = r"""
import sys, numpy as np
sys.path.insert(0, %r)
import oracle as O
from oracle import rotation as R
Ref = O.Reference()
rng = np.random.default_rng(11)
for ny, nx in ((48, 64), (33, 50)):
    img = rng.standard_normal((ny, nx)).astype(np.float32)
    # shifts stay shorter than the row / column: a longer one makes the
    # reference's circShiftX / circShiftY read outside their buffers
    for sh in (0.0, 0.031, -0.113, 0.41, -0.9):
        assert np.array_equal(Ref.shear(img, sh, "x"), R.shear_x(img, np.float32(sh))), sh
        assert np.array_equal(Ref.shear(img, sh, "y"), R.shear_y(img, np.float32(sh))), sh
    for th in (0.0, 3.3, -12.5, 44.0, -179.0, 200.0):
        assert np.array_equal(Ref.rotate2d(img, th), R.rotate2d(img, np.float32(th))), th
    for r2 in (2, 7, min(nx, ny) // 2):
        n = int(r2 * 2 * R.PI)
        assert np.array_equal(Ref.radial_profile(img, n, r2), R.radial_profile(img, n, r2)), r2
    img2 = rng.standard_normal((ny, nx)).astype(np.float32)
    assert abs(Ref.ncc_filtered(img, img2) - R.ncc_filtered(img, img2)) < 1e-13
    c = rng.standard_normal(97).astype(np.float32)
    assert Ref.find_peak_1d(c) == R.find_peak_1d(c)
print("ok")
""" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, (r.stdout[-1500:], r.stderr[-2000:])


# ---- preprocessing (arecImageTakeLog, periodicDecomposition) ---------------------------------
PRE_GOLD = os.path.join(ROOT, "tests", "golden", "reference_preprocess.npz")


def test_golden_preprocess_oracle():
    """The oracle's take-log (bit for bit) and periodic decomposition against
    the reference's outputs; the decomposition within one float rounding of
    its FFTs (the reference's spectrum passes through float)."""
    from oracle import preprocess as P

    g = np.load(PRE_GOLD)
    assert np.array_equal(P.take_log(g["log_in"]), g["log_out"])
    for tag in ("even", "odd"):
        img = g["pd_%s_in" % tag]
        s = P.make_periodic_slice(img[0])
        ref_s = g["pd_%s_smooth0" % tag]
        assert np.abs(s - ref_s).max() <= 1e-6 * np.abs(ref_s).max()
        out = P.periodic_decomposition(img)
        assert np.abs(out - g["pd_%s_out" % tag]).max() <= 1e-6 * np.abs(img).max()


# ---- Prealign profile alignment ---------------------------------------------------------------
PRE_REF = os.path.join(ROOT, "oracle", "_ref", "libprealign_ref.so")


def test_golden_prealign_oracle():
    """The oracle's TubeAlign profile loops (its own ccorr1d and findMaxCC_fit)
    against the same loops over the reference's pieces: within the float
    rounding of the correlation as the 7-point fit sees it (1e-5 px)."""
    from oracle import prealign as P

    g = np.load(os.path.join(ROOT, "tests", "golden", "reference_prealign.npz"))
    for tag, succ in (("global", False), ("successive", True)):
        s, spread = P.profile_shifts(g["profiles"], int(g["pad"]), succ)
        assert np.abs(s - g[tag + "_shifts"]).max() < 1e-5
        assert abs(spread - float(g[tag + "_spread"])) < 1e-5


@pytest.mark.skipif(not os.path.exists(PRE_REF), reason="reference not built here")
def test_prealign_pieces_against_reference_build():
    """findMaxCC_fit bit for bit on the reference's own correlation, and the
    oracle's ccorr1d within float rounding of the reference's."""
    import ctypes as C

    from oracle import prealign as P

    L = C.CDLL(PRE_REF)
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    cc = L._Z7ccorr1diPfS_S_
    cc.argtypes = [C.c_int, f32p, f32p, f32p]
    cc.restype = None
    fit = L._Z13findMaxCC_fitPKfi
    fit.argtypes = [f32p, C.c_int]
    fit.restype = C.c_double
    rng = np.random.default_rng(2)
    for n in (7, 64, 97, 300):
        x = rng.standard_normal(n).astype(np.float32)
        y = (np.roll(x, 3) + 0.1 * rng.standard_normal(n)).astype(np.float32)
        c = np.zeros(n, np.float32)
        cc(n, x.copy(), y.copy(), c)
        assert np.abs(c - P.ccorr1d(x, y)).max() <= 1e-6 * np.abs(c).max()
        assert fit(c, n) == P.find_max_cc_fit(c)
