"""GPU projector parity against the oracle (reference arecProject2D[_KB|_SQ] /
arecBackProject2D[_KB|_SQ], AREC3D/AREC3D/arecproject.cpp) and the reference's
own known answers (AREC3D/AREC3D_test/AREC3D_test.cpp)."""
import numpy as np
import pytest

from conftest import rel_l2, uniform_angles
from devutil import empty_sino, empty_vol, sino_from_dev, sino_to_dev, vol_from_dev, vol_to_dev

pytestmark = pytest.mark.gpu

# tolerance on projections (relative L2), the bar for floating-point parity
TOL = 1e-5

GEOMS = [
    (1.0, 2, uniform_angles(3)),
    (1.5, 3, np.array([0.698132, 1.22173], np.float32)),
    (12.0, 5, uniform_angles(16)),
    (31.5, 64, uniform_angles(45)),
    (63.5, 130, uniform_angles(60)),
    (40.0, 9, np.array([1.475, 21.123, 2.123, -0.3, 7.9], np.float32)),
    (100.0, 300, uniform_angles(24, 2 * np.pi)),
]


@pytest.mark.parametrize("w", [1, 2, 3])
@pytest.mark.parametrize("gi", range(len(GEOMS)))
def test_fp_bp_parity(gb, oc, w, gi):
    radius, ny, ang = GEOMS[gi]
    rng = np.random.default_rng(100 * gi + w)
    plan = gb.Plan(w, radius, ny, ang)
    x = rng.standard_normal((plan.nrays, ny)).astype(np.float32)
    if w == 1:  # the reference's linear weighting reads past its table for the last two rays
        x[-2:] = 0
    q_ref = oc.project(w, radius, x, ang)
    xd, qd = vol_to_dev(plan, x), empty_sino(plan)
    plan.project(xd, qd)
    q = sino_from_dev(plan, qd)
    assert rel_l2(q, q_ref) < TOL
    s = rng.standard_normal(q_ref.shape).astype(np.float32)
    g_ref = oc.backproject(w, radius, s, ang)
    gd = empty_vol(plan)
    plan.backproject(sino_to_dev(plan, s), gd)
    g = vol_from_dev(plan, gd)
    if w == 1:
        g, g_ref = g[:-2], g_ref[:-2]
    assert rel_l2(g, g_ref) < TOL
    assert plan.check() == 0


@pytest.mark.parametrize("w", [1, 2, 3])
def test_norm_fused(gb, w):
    import torch

    radius, ny, ang = 31.5, 20, uniform_angles(30)
    plan = gb.Plan(w, radius, ny, ang)
    rng = np.random.default_rng(w)
    x = rng.random((plan.nrays, ny), dtype=np.float32)
    xd, qd = vol_to_dev(plan, x), empty_sino(plan)
    n2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    plan.project(xd, qd, norm2=n2)
    q = qd.double()
    assert abs(n2.item() - float((q * q).sum())) <= 1e-9 * n2.item()
    gd = empty_vol(plan)
    plan.backproject(qd, gd, norm2=n2)
    g = gd.double()
    assert abs(n2.item() - float((g * g).sum())) <= 1e-9 * n2.item()


@pytest.mark.parametrize("w", [2, 3])
def test_adjoint_random(gb, w):
    radius, ny, ang = 47.5, 17, uniform_angles(33)
    plan = gb.Plan(w, radius, ny, ang)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((plan.nrays, ny)).astype(np.float32)
    s = rng.standard_normal((len(ang), ny, plan.nx)).astype(np.float32)
    qd, gd = empty_sino(plan), empty_vol(plan)
    plan.project(vol_to_dev(plan, x), qd)
    plan.backproject(sino_to_dev(plan, s), gd)
    a = float(np.dot(sino_from_dev(plan, qd).ravel().astype(np.float64), s.ravel()))
    b = float(np.dot(x.ravel().astype(np.float64), vol_from_dev(plan, gd).ravel()))
    assert abs(a - b) <= 1e-5 * abs(a)


def _coeff_tables(gb, w, radius, ny, ang, step):
    """Dense A and A^T coefficients on unit vectors, as the Catch test does."""
    plan = gb.Plan(w, radius, ny, ang)
    nv, ns = plan.nrays * ny, len(ang) * ny * plan.nx
    A = {}
    AT = {}
    for a in range(0, nv, step):
        x = np.zeros(nv, np.float32)
        x[a] = 1
        qd = empty_sino(plan)
        plan.project(vol_to_dev(plan, x.reshape(plan.nrays, ny)), qd)
        q = sino_from_dev(plan, qd).ravel()
        for b in range(0, ns, step):
            A[(a, b)] = q[b]
    for b in range(0, ns, step):
        s = np.zeros(ns, np.float32)
        s[b] = 1
        gd = empty_vol(plan)
        plan.backproject(sino_to_dev(plan, s.reshape(len(ang), ny, plan.nx)), gd)
        g = vol_from_dev(plan, gd).ravel()
        for a in range(0, nv, step):
            AT[(a, b)] = g[a]
    return A, AT


@pytest.mark.parametrize("case", [
    (3, 1.0, 2, [1.475, 21.123, 2.123], 1),   # "A vs AT, odd"  (AREC3D_test.cpp:216-243)
    (3, 1.5, 2, [0.698132, 1.22173], 3),       # "A vs AT, even" (:245-271)
    (2, 0.5, 2, [0.698132, 1.22173], 3),       # "A vs AT, even KB" (:298-324)
    (1, 7.5, 2, [0.3, 1.2, 2.9], 5),           # linear weighting, same property
])
def test_exact_adjoint_unit_vectors(gb, case):
    w, radius, ny, ang, step = case
    A, AT = _coeff_tables(gb, w, radius, ny, np.array(ang, np.float32), step)
    for k in A:
        assert A[k] == AT[k], k


def test_catch_projection_odd(gb):
    """"projection, odd" (AREC3D_test.cpp:97-147) through the reference API."""
    x = np.zeros((5, 2), np.float32)
    x.ravel()[4] = 1.0
    x.ravel()[5] = 2.0
    q, st = gb.arecProject2D_SQ(1.0, x, np.zeros(1, np.float32))
    assert st == 0
    assert x.sum() == pytest.approx(3.0)
    assert q.sum() == pytest.approx(3.0, rel=1.2e-5)
    assert q.ravel()[1] == pytest.approx(1.0, rel=1.2e-5)
    assert q.ravel()[4] == pytest.approx(2.0, rel=1.2e-5)


def test_catch_backprojection_odd(gb):
    """"backprojection, odd" (AREC3D_test.cpp:149-189)."""
    q = np.zeros((1, 2, 3), np.float32)
    q.ravel()[1] = 1.0
    q.ravel()[4] = 2.0
    g, st = gb.arecBackProject2D_SQ(1.0, q, np.zeros(1, np.float32))
    assert st == 0
    assert g.sum() == pytest.approx(9.0, rel=1.2e-5)


def test_reference_status_codes(gb):
    x = np.zeros((5, 2), np.float32)
    # projection stack of the wrong width -> 2 (arecproject.cpp:576-580)
    cyl = gb.arecAllocateCylImage(1.0, 2)
    q = np.zeros((1, 2, 4), np.float32)
    out = gb._cb_image(q)
    ang = np.zeros(1, np.float32)
    import ctypes as C

    st = gb.lib().arecgb_arecProject2D_SQ(cyl, gb._f32p(ang), 1, C.byref(out))
    assert st == 2
    # back-projection with nz != nangles -> 1 (arecproject.cpp:658-661)
    img = gb._cb_image(np.zeros((2, 2, 3), np.float32))
    st = gb.lib().arecgb_arecBackProject2D_SQ(img, gb._f32p(ang), 1, C.byref(cyl))
    assert st == 1
    gb.arecImageFree(cyl)


@pytest.mark.parametrize("w", [2, 3])
def test_autotuned_shapes_keep_parity(gb, oc, w):
    """After the autotuner has picked band heights and slices per block, the
    projectors still match the oracle (only summation order across bands may
    change)."""
    radius, ny, ang = 63.5, 300, uniform_angles(40)
    plan = gb.Plan(w, radius, ny, ang)
    band, nsc = plan.autotune(empty_vol(plan), empty_sino(plan))
    assert band in (32, 64, 128) and nsc in (1, 2)
    _, fvec, bvec, _ = plan.shapes()
    assert fvec in (4, 8) and bvec in (4, 8)
    rng = np.random.default_rng(w)
    x = rng.standard_normal((plan.nrays, ny)).astype(np.float32)
    q_ref = oc.project(w, radius, x, ang)
    qd = empty_sino(plan)
    plan.project(vol_to_dev(plan, x), qd)
    assert rel_l2(sino_from_dev(plan, qd), q_ref) < TOL
    g_ref = oc.backproject(w, radius, q_ref, ang)
    gd = empty_vol(plan)
    plan.backproject(sino_to_dev(plan, q_ref), gd)
    assert rel_l2(vol_from_dev(plan, gd), g_ref) < TOL
    assert plan.check() == 0
    print("autotune w=%d: band %d, back-projection chunks %d" % (w, band, nsc))


@pytest.mark.parametrize("w", [2, 3])
@pytest.mark.parametrize("gi", [2, 4, 5, 6])
def test_plan_tables_change_nothing(gb, w, gi, monkeypatch):
    """A plan with the projector tables (the taps of every ray and angle, the
    back projector's ring plans) and one without give bit-identical
    projections: the tables hold exactly what the kernels compute."""
    radius, ny, ang = GEOMS[gi]
    with_t = gb.Plan(w, radius, ny, ang)
    monkeypatch.setenv("ARECGB_PLAN_TABLES", "0")
    without = gb.Plan(w, radius, ny, ang)
    assert with_t.table_bytes() > 0 and without.table_bytes() == 0
    rng = np.random.default_rng(gi * 10 + w)
    x = rng.standard_normal((with_t.nrays, ny)).astype(np.float32)
    s = rng.standard_normal((len(ang), ny, with_t.nx)).astype(np.float32)
    out = []
    for plan in (with_t, without):
        qd, gd = empty_sino(plan), empty_vol(plan)
        plan.project(vol_to_dev(plan, x), qd)
        plan.backproject(sino_to_dev(plan, s), gd)
        out.append((sino_from_dev(plan, qd), vol_from_dev(plan, gd)))
        assert plan.check() == 0
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_linear_forward_projection_is_deterministic(gb, oc):
    """The linear weighting (pmethod 1, the reference parser's default,
    AREC3D/AREC3D/arec3dutil.cpp:110) gathers each bin's rays in a fixed order
    from the plan's ray index: repeated projections are bit-identical, match
    the oracle, and stay the exact transpose of the back projection."""
    radius, ny, ang = 63.5, 40, uniform_angles(50)
    plan = gb.Plan(1, radius, ny, ang)
    assert plan.table_bytes() > 0  # the ray index
    rng = np.random.default_rng(3)
    x = rng.standard_normal((plan.nrays, ny)).astype(np.float32)
    x[-2:] = 0
    xd = vol_to_dev(plan, x)
    outs = []
    for _ in range(3):
        qd = empty_sino(plan)
        plan.project(xd, qd)
        outs.append(sino_from_dev(plan, qd))
    assert all(np.array_equal(outs[0], o) for o in outs[1:])
    assert rel_l2(outs[0], oc.project(1, radius, x, ang)) < TOL
