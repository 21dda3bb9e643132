#!/bin/sh
# Build the reference's own HEALPix sources (src/Healpix_2.15a) into
# oracle/_ref/libref_healpix.so for the enumeration parity tests.
# Needs the reference tree in $RELION_REFERENCE; compiles the two .cc files
# where they lie and copies nothing into this repository.
set -e
REF=${RELION_REFERENCE:?set RELION_REFERENCE to the reference source tree}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/Healpix_2.15a/healpix_base.cc" ]; then
  echo "reference tree not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -O2 -fPIC -shared -ffp-contract=off -std=c++11 -w -I"$REF" \
    "$HERE/ref/healpix_ref_driver.cpp" \
    "$REF/src/Healpix_2.15a/healpix_base.cc" \
    "$REF/src/Healpix_2.15a/cxxutils.cc" \
    -o "$OUT/libref_healpix.so"
echo "built $OUT/libref_healpix.so"
