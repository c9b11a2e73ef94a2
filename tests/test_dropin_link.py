"""The reference's own programs link against libarec_gb300.so unchanged.

oracle/build_dropin.sh compiles the reference's driver (AREC3D.cpp) and its
Catch suite (AREC3D_test.cpp) from the reference checkout, leaves out the
translation units the library replaces (arecproject.cpp, areccgls.cpp,
areccgls_KB.cpp, arecsirt.cpp, arecsirt_KB.cpp) and links the rest against the
library.  This checks that both link, that every projector and solver symbol
they use is undefined in them and defined by the library (so the calls go to
the GPU), and that they record libarec_gb300.so as a needed library.  Running
them needs the reference's sources next to a GPU; where the checkout is absent
the test is skipped.
"""
import os
import re
import subprocess

import pytest

from conftest import ROOT

HOT = ["arecProject2D", "arecProject2D_KB", "arecProject2D_SQ", "arecBackProject2D",
       "arecBackProject2D_KB", "arecBackProject2D_SQ", "cyl_sirt", "cyl_sirt_KB",
       "cyl_sirt_SQ", "cyl_cgls", "cyl_cgls_KB", "cyl_cgls_SQ"]


_NM_LINE = re.compile(r"^\s*(?:[0-9a-fA-F]+\s+)?[A-Za-z]\s+(.+)$")


def _symbols(args):
    """Demangled names (without argument lists) that `nm args` lists."""
    out = subprocess.run(["nm", "-C"] + args, capture_output=True, text=True, check=True).stdout
    names = set()
    for ln in out.splitlines():
        m = _NM_LINE.match(ln)
        if m:
            names.add(m.group(1).split("(")[0].strip())
    return names


def test_reference_programs_link_against_library():
    import arec3d_gb300

    arec3d_gb300.build()
    script = os.path.join(ROOT, "oracle", "build_dropin.sh")
    r = subprocess.run(["bash", script], capture_output=True, text=True)
    if r.returncode == 2:
        pytest.skip("reference checkout not present: " + r.stderr.strip())
    assert r.returncode == 0, r.stdout + r.stderr
    lib = os.path.join(ROOT, "arec3d_gb300", "libarec_gb300.so")
    defined = _symbols(["-D", "--defined-only", lib])
    driver = os.path.join(ROOT, "oracle", "_ref", "arec3d_on_gb300")
    catch = os.path.join(ROOT, "oracle", "_ref", "arec_catch_on_gb300")
    for exe, used in ((driver, HOT), (catch, HOT[:6])):
        undef = _symbols(["-u", exe])
        for name in used:
            assert name in undef, (exe, name)
            assert name in defined, name
        needed = subprocess.run(["readelf", "-d", exe], capture_output=True, text=True,
                                check=True).stdout
        assert "libarec_gb300.so" in needed
