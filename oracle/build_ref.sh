#!/usr/bin/env bash
# Builds the reference's own AREC3D sources, unmodified and read in place from
# the read-only reference checkout, into oracle/_ref/ (git-ignored):
#   oracle/_ref/libarec_ref.so   the reference path (projectors, SIRT, CGLS,
#                                cross-correlation) over the single-rank MPI and
#                                FFTW-API stand-ins in oracle/shim/
#   oracle/_ref/arec_ref_catch   the reference's own Catch unit tests
#   oracle/_ref/libprealign_ref.so  Prealign's profile correlation
#                                (TubeAlign_utils.cpp) over the same stand-ins
# Test infrastructure only: nothing in the product links these.
#
# FP contraction is switched off (-ffp-contract=off) so that the build's double
# arithmetic is the literal C++ expression order; the C restatement in
# oracle/arec_oracle.c is built the same way and must agree bit for bit.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $AREC3D_REFERENCE, else /root/reference.
#   Exit status 2 when the checkout is not there (nothing is built).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${AREC3D_REFERENCE:-/root/reference}}"
SRC="$REF/AREC3D/AREC3D"
TST="$REF/AREC3D/AREC3D_test"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
    echo "build_ref: reference sources not found at $SRC" >&2
    exit 2
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
CC="${CC:-gcc}"
FLAGS=(-O2 -fPIC -ffp-contract=off -w -DNDEBUG)
UNITS=(arecImage arecproject areccgls areccgls_KB areccgls_stat arecsirt arecsirt_KB align2dstack
       imagetools arecImageIO arecImageIO_mpi)
pids=()
for u in "${UNITS[@]}"; do
    "$CXX" -std=c++14 "${FLAGS[@]}" -I"$HERE/shim" -I"$SRC" -c "$SRC/$u.cpp" -o "$OUT/$u.o" &
    pids+=($!)
done
"$CC" -std=c99 "${FLAGS[@]}" -I"$HERE/shim" -c "$HERE/shim/mpi_shim.c" -o "$OUT/mpi_shim.o" &
pids+=($!)
"$CC" -std=c99 "${FLAGS[@]}" -I"$HERE/shim" -c "$HERE/shim/fftw_shim.c" -o "$OUT/fftw_shim.o" &
pids+=($!)
"$CC" -std=c99 "${FLAGS[@]}" -c "$HERE/fft64.c" -o "$OUT/fft64.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
objs=()
for u in "${UNITS[@]}"; do objs+=("$OUT/$u.o"); done
"$CXX" -shared -o "$OUT/libarec_ref.so" "${objs[@]}" "$OUT/mpi_shim.o" "$OUT/fftw_shim.o" \
    "$OUT/fft64.o" -lm -Wl,--no-undefined

# Prealign's profile correlation (ccorr1d, findMaxCC_fit) in its own library:
# its ccorr1d has the same C++ name as AREC3D's.
PRE="$REF/Prealign/Prealign"
if [ -f "$PRE/TubeAlign_utils.cpp" ]; then
    "$CXX" -std=c++17 "${FLAGS[@]}" -I"$HERE/shim" -I"$PRE" -c "$PRE/TubeAlign_utils.cpp" \
        -o "$OUT/TubeAlign_utils.o"
    "$CXX" -std=c++17 "${FLAGS[@]}" -I"$PRE" -c "$PRE/mpfit.cpp" -o "$OUT/mpfit.o"
    "$CC" -std=c99 "${FLAGS[@]}" -I"$HERE/shim" -c "$HERE/shim/fftw_shim.c" -o "$OUT/fftw_shim2.o"
    "$CC" -std=c99 "${FLAGS[@]}" -c "$HERE/fft64.c" -o "$OUT/fft64_2.o"
    "$CXX" -shared -o "$OUT/libprealign_ref.so" "$OUT/TubeAlign_utils.o" "$OUT/mpfit.o" \
        "$OUT/fftw_shim2.o" "$OUT/fft64_2.o" -lm -Wl,--no-undefined
fi

# The Catch suite is stored as UTF-16; convert a copy into _ref and build it.
if [ -f "$TST/AREC3D_test.cpp" ]; then
    iconv -f UTF-16 -t UTF-8 "$TST/AREC3D_test.cpp" > "$OUT/AREC3D_test_utf8.cpp"
    "$CXX" -std=c++14 -O1 -w -DCATCH_CONFIG_NO_POSIX_SIGNALS -I"$HERE/shim" -I"$SRC" -I"$TST" \
        "$OUT/AREC3D_test_utf8.cpp" -o "$OUT/arec_ref_catch" -L"$OUT" -larec_ref \
        -Wl,-rpath,"$OUT"
fi
rm -f "$OUT"/*.o
echo "build_ref: built $OUT/libarec_ref.so"
