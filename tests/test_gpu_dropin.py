"""The drop-in from the reference's side: the reference-named solvers over host
`arecImage` buffers, compared with the reference's own outputs, and a C++
program written against the reference's declarations, linked to the library.

Goldens (tests/golden/make_golden.py, produced by the reference built from its
sources):
* reference_small.npz: cyl_sirt / cyl_sirt_KB / cyl_sirt_SQ (12 iterations,
  lam 2e-4) and cyl_cgls / cyl_cgls_SQ (10 iterations) on seeded noisy data at
  nx = 64, and the status -1 of cyl_cgls_KB there (its integer radius nx/2 needs
  odd nx, AREC3D/AREC3D/areccgls_KB.cpp:37-48);
* reference_compat.npz: cyl_cgls_SQ and cyl_cgls_KB warm-started from a
  non-NULL xvol (areccgls.cpp:323-340), cyl_cgls_KB at nx = 65, and the log
  lines cyl_cgls_SQ and cyl_sirt_SQ print (areccgls.cpp:349-465,
  arecsirt.cpp:240-373).
"""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
# CGLS on these small noisy problems is ill-conditioned: after a few iterations
# the reference's own float result departs from an FP64 evaluation of the same
# algorithm (the oracle's cgls64) by up to 1e-2.  There the GPU must reproduce
# the reference's float trajectory to within FRAC of that distance (the rule of
# tests/test_gpu_solvers.py).
FRAC = 0.25
# Residual values in the logs: late-iteration residuals are small differences
# of large quantities (the tolerance of the solver tests' residual traces).
RTOL_TRACE = 0.2
GOLD = os.path.join(ROOT, "tests", "golden")


def _cgls_bar(oc, w, b, ang, maxit, x_ref, x0=None):
    """max(TOL, FRAC * |reference - FP64|) for a CGLS result."""
    x64, _ = oc.cgls64(w, b, ang, maxit=maxit, tol=1e-7, x0=x0)
    if w == 1:
        x64, x_ref = x64[:-2], x_ref[:-2]
    e64 = rel_l2(x_ref, x64)
    return max(TOL, FRAC * e64), e64


@pytest.fixture(scope="module")
def small():
    return np.load(os.path.join(GOLD, "reference_small.npz"))


@pytest.fixture(scope="module")
def compat():
    return np.load(os.path.join(GOLD, "reference_compat.npz"))


@pytest.mark.parametrize("tag,suffix", [("lin", ""), ("kb", "_KB"), ("sq", "_SQ")])
def test_sirt_matches_reference_output(gb, small, tag, suffix):
    b, ang = small["solve_%s_b" % tag], small["solve_angles"]
    x, st = getattr(gb, "cyl_sirt" + suffix)(b, ang, lam=2e-4, maxit=12, tol=0.0)
    ref = small["solve_%s_sirt" % tag]
    assert st == 0 and x.shape == ref.shape
    if tag == "lin":  # the last two rays read past the reference's coordinate table
        x, ref = x[:-2], ref[:-2]
    e = rel_l2(x, ref)
    print("cyl_sirt%s vs the reference: %.2e" % (suffix, e))
    assert e < TOL


@pytest.mark.parametrize("tag,suffix,w", [("lin", "", 1), ("sq", "_SQ", 3)])
def test_cgls_matches_reference_output(gb, oc, small, tag, suffix, w):
    b, ang = small["solve_%s_b" % tag], small["solve_angles"]
    x, st = getattr(gb, "cyl_cgls" + suffix)(b, ang, maxit=10, tol=1e-7)
    ref = small["solve_%s_cgls" % tag]
    assert st == int(small["solve_%s_cgls_status" % tag]) == 0
    bar, e64 = _cgls_bar(oc, w, b, ang, 10, ref)
    if tag == "lin":
        x, ref = x[:-2], ref[:-2]
    e = rel_l2(x, ref)
    print("cyl_cgls%s vs the reference: %.2e (reference vs FP64 %.2e)" % (suffix, e, e64))
    assert e < bar


def test_cgls_kb_even_width_fails_like_the_reference(gb, small):
    b, ang = small["solve_kb_b"], small["solve_angles"]
    assert b.shape[2] % 2 == 0
    _, st = gb.cyl_cgls_KB(b, ang, maxit=10, tol=1e-7)
    assert st == int(small["solve_kb_cgls_status"]) == -1


def test_cgls_kb_odd_width(gb, oc, compat, small):
    b, ang, maxit = compat["kb65_b"], small["solve_angles"], int(compat["kb65_maxit"])
    x, st = gb.cyl_cgls_KB(b, ang, maxit=maxit, tol=1e-7)
    assert st == 0
    bar, e64 = _cgls_bar(oc, 2, b, ang, maxit, compat["kb65_cgls"])
    e = rel_l2(x, compat["kb65_cgls"])
    print("cyl_cgls_KB nx=65 vs the reference: %.2e (reference vs FP64 %.2e)" % (e, e64))
    assert e < bar


@pytest.mark.parametrize("tag,suffix,w", [("sq", "_SQ", 3), ("kb", "_KB", 2)])
def test_cgls_warm_start_from_caller_volume(gb, oc, compat, small, tag, suffix, w):
    """xvol->data != NULL: CGLS starts from the caller's volume."""
    b = small["solve_sq_b"] if tag == "sq" else compat["kb65_b"]
    ang, maxit, x0 = small["solve_angles"], int(compat["warm_%s_maxit" % tag]), \
        compat["warm_%s_x0" % tag]
    x, st = getattr(gb, "cyl_cgls" + suffix)(b, ang, maxit=maxit, tol=1e-7, x0=x0)
    assert st == 0
    ref = compat["warm_%s_cgls" % tag]
    bar, e64 = _cgls_bar(oc, w, b, ang, maxit, ref, x0=x0)
    e = rel_l2(x, ref)
    print("cyl_cgls%s warm start vs the reference: %.2e (reference vs FP64 %.2e)"
          % (suffix, e, e64))
    assert e < bar


def test_null_xvol_is_allocated(gb, small):
    """xvol->data == NULL: the solver allocates the cylinder (calloc) with the
    reference's table; the caller frees it with arecImageFree."""
    b = np.ascontiguousarray(small["solve_sq_b"], np.float32)
    ang = np.ascontiguousarray(small["solve_angles"], np.float32)
    img = gb._cb_image(b)
    vol = gb.ArecImage()
    vol.data = C.POINTER(C.c_float)()
    st = gb.lib().arecgb_cyl_cgls_SQ(0, img, gb._f32p(ang), C.byref(vol), 0.0, 3, 1e-7)
    assert st == 0 and bool(vol.data)
    assert (vol.nx, vol.nz, vol.height, vol.is_cyl) == (64, 64, 4, 1)
    assert vol.radius == 31.5 and vol.nrays == 3252 and vol.nnz == 3252 * 4
    cord = np.ctypeslib.as_array(vol.cord, shape=(vol.nrays, 2))
    np.testing.assert_array_equal(cord, small["cyl_31.5_cord"])
    gb.arecImageFree(vol)
    assert not bool(vol.data)


_NUM = re.compile(r"[-+]?\d+\.\d+e[-+]\d+|[-+]?\d+\.\d+|[-+]?\d+")


def _compare_logs(ours, ref):
    a = [ln for ln in ours.strip().splitlines() if ln.strip()]
    r = [ln for ln in ref.strip().splitlines() if ln.strip()]
    assert len(a) == len(r), (a, r)
    for la, lr in zip(a, r):
        assert _NUM.sub("#", la) == _NUM.sub("#", lr), (la, lr)
        if la.startswith("Total time"):
            continue
        for va, vr in zip(_NUM.findall(la), _NUM.findall(lr)):
            assert float(va) == pytest.approx(float(vr), rel=RTOL_TRACE, abs=0), (la, lr)


def test_log_lines_match_the_reference(gb, compat):
    """Same lines, same formats, same iteration numbers (and so the same
    stopping decisions), residual values within RTOL_TRACE: log diffs of
    iteration counts and residuals keep working."""
    code = r'''
import sys
sys.path.insert(0, %r)
import numpy as np
import arec3d_gb300 as gb
d = np.load(%r)
b, ang = d["solve_sq_b"], d["solve_angles"]
sys.stdout.flush()
gb.cyl_cgls_SQ(b, ang, maxit=10, tol=1e-7)
gb.lib()
import ctypes
ctypes.CDLL(None).fflush(None)
print("=====", flush=True)
gb.cyl_sirt_SQ(b, ang, lam=2e-4, maxit=12, tol=0.0)
ctypes.CDLL(None).fflush(None)
''' % (ROOT, os.path.join(GOLD, "reference_small.npz"))
    env = dict(os.environ)
    env.pop("ARECGB_QUIET", None)
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    cg, sirt = out.stdout.split("=====")
    _compare_logs(cg, str(compat["log_cgls_sq"]))
    _compare_logs(sirt, str(compat["log_sirt_sq"]))


def test_cxx_program_against_reference_declarations(gb, tmp_path):
    """tests/dropin/catch_cases.cpp: the Catch suite's known answers and one
    solver per family, through the reference's C++ names, from a separately
    compiled program linked to libarec_gb300.so."""
    exe = tmp_path / "catch_cases"
    libdir = os.path.join(ROOT, "arec3d_gb300")
    subprocess.run(["g++", "-std=c++14", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "dropin", "catch_cases.cpp"), "-L", libdir,
                    "-larec_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    env = dict(os.environ, ARECGB_QUIET="1")
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300, env=env)
    print(out.stdout.strip())
    assert out.returncode == 0, out.stdout + out.stderr
    assert re.search(r"all \d+ checks passed", out.stdout)
