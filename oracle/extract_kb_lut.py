"""Extracts the Kaiser-Bessel blob profile table of the reference
(AREC3D/AREC3D/arecproject.cpp:192-338, `float LUT[1000]`) into
arec3d_gb300/csrc/kb_lut_table.inc.

The table is measured data (a blob convolved with a one-pixel box); it cannot be
regenerated from a formula, so the weighting `pmethod=2` is only reproducible
with these exact numbers.  Each entry is emitted as the hex-float literal of the
float the reference's compiler stores: the decimal literal is a double constant
converted to float, i.e. float(double(text)), which is what numpy computes below.

Only entries 0..511 are written: the projectors evaluate the table at
|x| <= 1.5 px, i.e. index <= 1.5 / (3/999) < 500, plus the right neighbour.

Usage: python oracle/extract_kb_lut.py REFERENCE_ROOT   (or set AREC3D_REFERENCE)
"""
import os
import re
import sys

import numpy as np

KEEP = 512


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AREC3D_REFERENCE")
    if not ref:
        raise SystemExit("usage: extract_kb_lut.py REFERENCE_ROOT (or set AREC3D_REFERENCE)")
    src = os.path.join(ref, "AREC3D", "AREC3D", "arecproject.cpp")
    text = open(src, encoding="utf-8", errors="replace").read()
    m = re.search(r"float\s+LUT\s*\[\s*LUT_SIZE\s*\]\s*=\s*\{(.*?)\};", text, re.S)
    if not m:
        raise SystemExit("LUT not found in " + src)
    vals = [v.strip() for v in m.group(1).replace("\n", " ").split(",") if v.strip()]
    if len(vals) != 1000:
        raise SystemExit("expected 1000 LUT entries, found %d" % len(vals))
    f = np.array([np.float32(float(v)) for v in vals[:KEEP]], dtype=np.float32)
    here = os.path.dirname(os.path.abspath(__file__))
    out = os.path.join(here, "..", "arec3d_gb300", "csrc", "kb_lut_table.inc")
    with open(out, "w") as fh:
        fh.write("/* Kaiser-Bessel blob profile, entries 0..%d of the reference table\n" % (KEEP - 1))
        fh.write(" * (AREC3D/AREC3D/arecproject.cpp:192-338), as the floats the reference\n")
        fh.write(" * stores.  Generated by oracle/extract_kb_lut.py; do not edit. */\n")
        for i in range(0, KEEP, 4):
            fh.write("    " + ", ".join(float(x).hex() + "f" for x in f[i:i + 4]) + ",\n")
    print("wrote", os.path.normpath(out))


if __name__ == "__main__":
    main()
