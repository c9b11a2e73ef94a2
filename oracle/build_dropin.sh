#!/usr/bin/env bash
# Links the reference's own programs against libarec_gb300.so, the way a
# maintainer would switch them over: the driver (AREC3D.cpp, with its parser and
# angle reader) and the Catch suite (AREC3D_test.cpp) are compiled unmodified
# from the read-only reference checkout, the translation units the library
# replaces (arecproject.cpp, areccgls.cpp, areccgls_KB.cpp, arecsirt.cpp,
# arecsirt_KB.cpp) are left out, and the rest of the reference is kept.
# Outputs go to oracle/_ref/ (git-ignored):
#   oracle/_ref/arec3d_on_gb300        the reference driver on the library
#   oracle/_ref/arec_catch_on_gb300    the reference Catch suite on the library
# Test infrastructure only (tests/test_dropin_link.py checks that both link with
# every projector and solver symbol resolved by the library).  MPI and FFTW come
# from the single-rank and FFTW-API stand-ins in oracle/shim/, as in
# oracle/build_ref.sh.
#
# Usage: oracle/build_dropin.sh [REFERENCE_ROOT] [LIBDIR]
#   REFERENCE_ROOT defaults to $AREC3D_REFERENCE, else /root/reference;
#   LIBDIR (holding libarec_gb300.so) defaults to arec3d_gb300/.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(dirname "$HERE")"
REF="${1:-${AREC3D_REFERENCE:-/root/reference}}"
LIBDIR="${2:-$ROOT/arec3d_gb300}"
SRC="$REF/AREC3D/AREC3D"
TST="$REF/AREC3D/AREC3D_test"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
    echo "build_dropin: reference sources not found at $SRC" >&2
    exit 2
fi
if [ ! -f "$LIBDIR/libarec_gb300.so" ]; then
    echo "build_dropin: $LIBDIR/libarec_gb300.so not built" >&2
    exit 3
fi
mkdir -p "$OUT/dropin"
CXX="${CXX:-g++}"
CC="${CC:-gcc}"
FLAGS=(-O2 -w -DNDEBUG)
KEEP=(AREC3D arec3dutil ReadAndDistAngles arecImage align2dstack imagetools arecImageIO
      arecImageIO_mpi areccgls_stat)
pids=()
for u in "${KEEP[@]}"; do
    "$CXX" -std=c++14 "${FLAGS[@]}" -I"$HERE/shim" -I"$SRC" -c "$SRC/$u.cpp" \
        -o "$OUT/dropin/$u.o" &
    pids+=($!)
done
"$CC" -std=c99 "${FLAGS[@]}" -I"$HERE/shim" -c "$HERE/shim/mpi_shim.c" -o "$OUT/dropin/mpi_shim.o" &
pids+=($!)
"$CC" -std=c99 "${FLAGS[@]}" -I"$HERE/shim" -c "$HERE/shim/fftw_shim.c" -o "$OUT/dropin/fftw_shim.o" &
pids+=($!)
"$CC" -std=c99 "${FLAGS[@]}" -c "$HERE/fft64.c" -o "$OUT/dropin/fft64.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
common=()
for u in arecImage align2dstack imagetools arecImageIO arecImageIO_mpi areccgls_stat; do
    common+=("$OUT/dropin/$u.o")
done
common+=("$OUT/dropin/mpi_shim.o" "$OUT/dropin/fftw_shim.o" "$OUT/dropin/fft64.o")
LINK=(-L"$LIBDIR" -larec_gb300 -Wl,-rpath,"$LIBDIR" -lm)
"$CXX" -o "$OUT/arec3d_on_gb300" "$OUT/dropin/AREC3D.o" "$OUT/dropin/arec3dutil.o" \
    "$OUT/dropin/ReadAndDistAngles.o" "${common[@]}" "${LINK[@]}"
if [ -f "$TST/AREC3D_test.cpp" ]; then
    iconv -f UTF-16 -t UTF-8 "$TST/AREC3D_test.cpp" > "$OUT/dropin/AREC3D_test_utf8.cpp"
    "$CXX" -std=c++14 -O1 -w -DCATCH_CONFIG_NO_POSIX_SIGNALS -I"$HERE/shim" -I"$SRC" -I"$TST" \
        "$OUT/dropin/AREC3D_test_utf8.cpp" "${common[@]}" -o "$OUT/arec_catch_on_gb300" \
        "${LINK[@]}"
fi
rm -rf "$OUT/dropin"
echo "build_dropin: linked $OUT/arec3d_on_gb300 and $OUT/arec_catch_on_gb300"
