"""The C-ABI library: it builds for sm_103a, loads without a GPU, exports
every entry point include/*.h declares plus the reference's own C++ symbols,
and its host-side data model matches the reference (no device calls here)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    import arec3d_gb300

    arec3d_gb300.build()
    return arec3d_gb300


def declared_functions():
    names = set()
    for h in ("arec_gb300.h", "arec_compat.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"^\s*(?:const\s+char\s*\*|int|void)\s+\**\s*(arecgb_\w+)\s*\(",
                                text, re.M))
    return sorted(names)


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True)
    return {ln.split()[-1] for ln in out.stdout.splitlines() if ln.strip()}


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) > 30
    syms = exported(lib.LIB_PATH)
    missing = [n for n in names if n not in syms]
    assert not missing, missing
    L = lib.lib()  # loads on a machine without a GPU
    for n in names:
        assert getattr(L, n) is not None


# The reference's C++ entry points (g++ Itanium mangling, MPICH-style int MPI_Comm).
REF_SYMBOLS = [
    "_Z13arecProject2D5ImagePfiPS_", "_Z16arecProject2D_KB5ImagePfiPS_",
    "_Z16arecProject2D_SQ5ImagePfiPS_", "_Z17arecBackProject2D5ImagePfiPS_",
    "_Z20arecBackProject2D_KB5ImagePfiPS_", "_Z20arecBackProject2D_SQ5ImagePfiPS_",
    "_Z8cyl_sirti5ImagePfPS_fif", "_Z11cyl_sirt_KBi5ImagePfPS_fif",
    "_Z11cyl_sirt_SQi5ImagePfPS_fif", "_Z8cyl_cglsi5ImagePfPS_fif",
    "_Z11cyl_cgls_KBi5ImagePfPS_fif", "_Z11cyl_cgls_SQi5ImagePfPS_fif",
    "_Z12arecCCImagesi5ImageS_PfS0_", "_Z7ccorr2diiPfS_S_", "_Z5speakiiPfS_S_",
    "_Z13cyl_cgls_stati5ImagePfPS_fif", "_Z16cyl_cgls_KB_stati5ImagePfPS_fif",
    "_Z16cyl_cgls_SQ_stati5ImagePfPS_fif", "_Z12init_weightsi5ImagePS_",
    "_Z8fshift2diiPfS_ff", "_Z15arecRotCCImagesi5ImageS_iPf", "_Z16arecRotateImagesP5ImagePf",
    "_Z21arecRotateImages_skewP5ImagePf", "_Z26arecRotateImages_skew_safeP5ImageS0_Pf",
]


def test_reference_cxx_symbols(lib):
    syms = exported(lib.LIB_PATH)
    missing = [s for s in REF_SYMBOLS if s not in syms]
    assert not missing, missing


def test_builder_targets_sm103a():
    """Every translation unit is compiled for sm_103a only (the builder's flags)."""
    from arec3d_gb300 import builder

    flags = " ".join(builder.ARCH + builder.FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags
    assert flags.count("-gencode") == 1


@pytest.mark.parametrize("r", [0.5, 1.0, 1.5, 7.5, 12.0, 31.5, 100.0])
def test_cylinder_allocation_matches_oracle(lib, oc, r):
    im = lib.arecAllocateCylImage(r, 3)
    nx, nr, cord = oc.cyl(r)
    assert (im.nx, im.nrays, im.nnz, im.is_cyl) == (nx, nr, 3 * nr, 1)
    np.testing.assert_array_equal(lib.cyl_cord(im), cord)
    lib.arecImageFree(im)


@pytest.mark.parametrize("r,ny", [(0.5, 1), (12.0, 5), (63.5, 300), (1031.5, 512)])
def test_cylinder_info_matches_oracle(lib, oc, r, ny):
    """arecgb_cylinder_info: the device layout sizes of a cylinder without a plan."""
    import arec3d_gb300 as gb

    nx, nr, _ = oc.cyl(r)
    assert gb.cylinder_info(r, ny) == (nx, nr, (ny + 7) // 8 * 8)


def test_image_cyl2cb_roundtrip(lib):
    """"ImageCyl2CB" (AREC3D_test.cpp:326-363)."""
    L = lib.lib()
    cyl = lib.arecAllocateCylImage(1.0, 2)
    d = lib.cyl_data(cyl)
    d[:] = np.arange(cyl.nnz, dtype=np.float32).reshape(d.shape)
    cube = np.zeros((cyl.nz, cyl.ny, cyl.nx), np.float32)
    cb = lib._cb_image(cube)
    assert L.arecgb_ImageCyl2CB(cyl, cb, cyl.nx, cyl.ny, cyl.nz) == 0
    assert cube.sum() == d.sum()
    cyl2 = lib.arecAllocateCylImage(1.0, 2)
    assert L.arecgb_ImageCB2Cyl(cb, cyl2, 2, 2, 2.0, 2) == 0
    np.testing.assert_array_equal(lib.cyl_data(cyl2), d)
    lib.arecImageFree(cyl)
    lib.arecImageFree(cyl2)


def test_reset_and_soft_noneg(lib):
    L = lib.lib()
    cyl = lib.arecAllocateCylImage(2.0, 2)
    d = lib.cyl_data(cyl)
    d[:] = np.linspace(-1, 1, d.size, dtype=np.float32).reshape(d.shape)
    before = d.copy()
    L.arecgb_soft_noneg(C.byref(cyl))
    np.testing.assert_array_equal(d, np.where(before < 0, before * 0.5, before))
    L.arecgb_reset(C.byref(cyl))
    assert not d.any()
    lib.arecImageFree(cyl)


def test_no_cpu_fallback(tmp_path, monkeypatch):
    """Without the built library every call raises instead of computing on the CPU."""
    import importlib

    import arec3d_gb300

    monkeypatch.setattr(arec3d_gb300, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(arec3d_gb300, "_lib", None)
    with pytest.raises(RuntimeError):
        arec3d_gb300.lib()


def test_argument_errors_before_any_device_call(lib):
    """Invalid arguments come back as ARECGB_ERR_ARG with a message, checked
    before the library touches a device (so this runs without a GPU)."""
    L = lib.lib()
    ERR_ARG = -90
    vp, fp = C.c_void_p, C.POINTER(C.c_float)
    ang = np.zeros(4, np.float32)
    angp = ang.ctypes.data_as(fp)
    plan = vp()
    for w, radius, ny, na, a in ((0, 10.0, 4, 4, angp), (4, 10.0, 4, 4, angp),
                                 (3, -1.0, 4, 4, angp), (3, 9000.0, 4, 4, angp),
                                 (3, 10.0, 0, 4, angp), (3, 10.0, 4, 0, angp),
                                 (3, 10.0, 4, 4, None)):
        assert L.arecgb_plan_create(C.byref(plan), w, radius, ny, na, a) == ERR_ARG
        assert not plan.value
        assert L.arecgb_last_error().decode().startswith("plan_create:")
    assert L.arecgb_plan_create(None, 3, 10.0, 4, 4, angp) == ERR_ARG
    ip = C.POINTER(C.c_int)
    n = C.c_int()
    assert L.arecgb_plan_info(None, C.byref(n), C.byref(n), C.byref(n)) == ERR_ARG
    assert L.arecgb_plan_shapes(None, None, None, None, None) == ERR_ARG
    assert L.arecgb_plan_set_shapes(None, 64, 8, 8, 1) == ERR_ARG
    assert L.arecgb_plan_table_bytes(None) == 0
    L.arecgb_cgls_batch.argtypes = [vp, vp, vp, ip, C.c_int, C.c_int, C.c_float, vp, vp, vp]
    assert L.arecgb_cgls_batch(None, None, None, None, 0, 10, 1e-3, None, None, None) == ERR_ARG


def test_warm_start_entry_argument_errors(lib):
    """The filtered back projection and the uneven scheduler reject bad
    arguments before any device call: null plan or buffers, a negative SIRT
    depth (0 selects the filtered back projection as the network's input)."""
    L = lib.lib()
    ERR_ARG = -90
    vp = C.c_void_p
    L.arecgb_fbp.argtypes = [vp, vp, vp, vp, vp, vp]
    L.arecgb_ramp_filter.argtypes = [vp, vp, vp, vp]
    assert L.arecgb_fbp(None, None, None, None, None, None) == ERR_ARG
    assert L.arecgb_last_error().decode().startswith("arecgb_fbp")
    assert L.arecgb_ramp_filter(None, None, None, None) == ERR_ARG
    assert L.arecgb_last_error().decode().startswith("arecgb_ramp_filter")
    prob = lib.Problem(3, 10.0, 4, 4, np.zeros(4, np.float32).ctypes.data_as(C.POINTER(C.c_float)),
                       None, None)
    info = (lib.SolveInfo * 1)()
    for sirt_iters in (-1,):
        rc = L.arecgb_solve_uneven(C.byref(prob), 1, 1 << 30, None, 0, sirt_iters, 1.0, 10,
                                   C.c_float(1e-3), info, None, None)
        assert rc == ERR_ARG
    # a problem without device buffers is rejected, with or without a network
    rc = L.arecgb_solve_uneven(C.byref(prob), 1, 1 << 30, None, 0, 0, 1.0, 10, C.c_float(1e-3),
                               info, None, None)
    assert rc == ERR_ARG and "bad problem 0" in L.arecgb_last_error().decode()


@pytest.mark.parametrize("r", [0.5, 1.0, 12.0, 31.5, 127.5, 511.5])
def test_synthetic_cylinder_coords_match_oracle(oc, r):
    """The benchmark's ground truth (synthetic.sphere_volume) samples the
    phantom at the pixel centres of the reference's cylinder in its ray order
    (arecAllocateCylImage, AREC3D/AREC3D/arecImage.cpp:29-86)."""
    from arec3d_gb300 import synthetic as syn

    nx, nr, cord = oc.cyl(r)
    cx, cz = syn.cylinder_coords(r)
    assert cx.size == nr
    np.testing.assert_array_equal(cx, cord[:, 0] - r)
    np.testing.assert_array_equal(cz, cord[:, 1] - r)
