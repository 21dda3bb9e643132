#!/bin/sh
# Build the reference's own code for the oracle's checks (TEST INFRASTRUCTURE
# ONLY).  Needs the reference source tree in $RELION_REFERENCE; compiles its
# files where they lie (unmodified, nothing copied into this repository) into
# oracle/_ref:
#   libref_healpix.so  src/Healpix_2.15a (HEALPix enumeration)
#   ref_pin            a driver (oracle/ref/ref_pin_driver.cpp) linked with the
#                      reference's CPU sources for projection, backprojection,
#                      CTF images, HEALPix sampling, shifts, Euler matrices,
#                      reconstruction and the Fourier map of a reference, over
#                      the shims of oracle/ref/shim (FFTW API on our own FFT,
#                      TIFF / PNG declarations) and oracle/ref/stubs.cpp;
#   ref_estep          a driver (oracle/ref/ref_estep_driver.cpp) running the
#                      reference's MlOptimiser E-step (getAllSquaredDifferences,
#                      convertAllSquaredDifferencesToWeights, storeWeightedSums)
#                      with its model, sampling, particle and optics classes.
# Paths the drivers never take (helical geometry, aberrations, tomography
# I/O, atomic models, plots) stay unresolved (--unresolved-symbols=ignore-all).
set -e
REF=${RELION_REFERENCE:?set RELION_REFERENCE to the reference source tree}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/Healpix_2.15a/healpix_base.cc" ]; then
  echo "reference tree not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
g++ -O2 -fPIC -shared -ffp-contract=off -std=c++11 -w -I"$REF" \
    "$HERE/ref/healpix_ref_driver.cpp" \
    "$REF/src/Healpix_2.15a/healpix_base.cc" \
    "$REF/src/Healpix_2.15a/cxxutils.cc" \
    -o "$OUT/libref_healpix.so"
echo "built $OUT/libref_healpix.so"

FLAGS="-std=c++14 -O2 -w -fopenmp -ffp-contract=off -I$REF -I$HERE/ref/shim"
SRCS="projector backprojector ctf healpix_sampling fftw euler symmetries funcs error transformations tabfuncs mask
      filename strings metadata_table metadata_label metadata_container image numerical_recipes args time memory
      matrix1d matrix2d multidim_array complex pipeline_control"
pids=""
for f in $SRCS; do
  g++ $FLAGS -c "$REF/src/$f.cpp" -o "$OUT/obj/$f.o" &
  pids="$pids $!"
done
g++ $FLAGS -c "$REF/src/Healpix_2.15a/healpix_base.cc" -o "$OUT/obj/healpix_base.o" &
pids="$pids $!"
g++ $FLAGS -c "$REF/src/Healpix_2.15a/cxxutils.cc" -o "$OUT/obj/cxxutils.o" &
pids="$pids $!"
for f in ml_optimiser ml_model exp_model parallel helix jaz/single_particle/obs_model jaz/optics/optics_data \
         jaz/tomography/tomogram_set jaz/tomography/particle_set jaz/tomography/tomogram; do
  g++ $FLAGS -c "$REF/src/$f.cpp" -o "$OUT/obj/$(basename $f).o" &
  pids="$pids $!"
done
mkdir -p "$OUT/drv"
g++ $FLAGS -c "$HERE/ref/ref_pin_driver.cpp" -o "$OUT/drv/ref_pin_driver.o" &
pids="$pids $!"
g++ $FLAGS -c "$HERE/ref/ref_estep_driver.cpp" -o "$OUT/drv/ref_estep_driver.o" &
pids="$pids $!"
g++ -std=c++14 -O2 -w -I"$HERE/ref/shim" -c "$HERE/ref/fftw_shim.cpp" -o "$OUT/obj/fftw_shim.o" &
pids="$pids $!"
g++ -std=c++14 -O2 -w -I"$HERE/ref/shim" -c "$HERE/ref/stubs.cpp" -o "$OUT/obj/stubs.o" &
pids="$pids $!"
for p in $pids; do wait $p; done
g++ -fopenmp -o "$OUT/ref_pin" "$OUT/drv/ref_pin_driver.o" "$OUT"/obj/*.o -lpthread \
    -Wl,--unresolved-symbols=ignore-all 2>/dev/null
echo "built $OUT/ref_pin"
g++ -fopenmp -o "$OUT/ref_estep" "$OUT/drv/ref_estep_driver.o" "$OUT"/obj/*.o -lpthread \
    -Wl,--unresolved-symbols=ignore-all 2>/dev/null
echo "built $OUT/ref_estep"
