#!/bin/sh
# Builds oracle/_ref/libfvmic2d_ref.so from fvmic2d's OWN hot-path sources, compiled
# in place (read-only) from the reference tree against the single-rank petsc_lite
# stand-in.  Test infrastructure only: the library pins the project's C
# restatement (oracle/mic_oracle.c) and generates the golden vectors under
# tests/golden/.  Nothing is copied out of the reference tree.
#
# usage: oracle/build_ref.sh REFERENCE_DIR   (the fvmic2d source tree)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
if [ $# -lt 1 ]; then
  echo "usage: $0 REFERENCE_DIR" >&2
  exit 2
fi
REF=$1
OUT="$HERE/_ref"
if [ ! -f "$REF/markerProjection.c" ]; then
  echo "reference sources not found under $REF; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$OUT"
CC=${CC:-gcc}
# -ffp-contract=off: no fused multiply-add, so results do not depend on the host ISA.
CFLAGS="-O2 -fPIC -std=gnu99 -ffp-contract=off -fno-fast-math -w"
INC="-I$HERE/petsc_lite/include -I$REF -I$HERE/../include"
SRCS="markers.c markerProjection.c updateMarkerStrainPressure.c subgridStressChanges.c updateMarkerStress.c \
subgridTemperatureChanges.c viscosity.c residual.c benchmarkInitialConditions.c gridSpacing.c profile.c \
nodalStressStrain.c limitTimestep.c retrieveSolutions.c io.c restart.c vep_system.c formThermalSystem.c \
enforceThermalBC.c adiabaticHeating.c post.c"
OBJS=""
for s in $SRCS; do
  o="$OUT/$(basename "$s" .c).o"
  $CC $CFLAGS $INC -c "$REF/$s" -o "$o"
  OBJS="$OBJS $o"
done
$CC $CFLAGS $INC -c "$HERE/petsc_lite/petsc_lite.c" -o "$OUT/petsc_lite.o"
$CC $CFLAGS $INC -c "$HERE/ref_bridge.c" -o "$OUT/ref_bridge.o"
$CC -shared -o "$OUT/libfvmic2d_ref.so" $OBJS "$OUT/petsc_lite.o" "$OUT/ref_bridge.o" -lm
# the same library with the reference's compile-time JAUMANN switch (markers.c:2147-2156: the
# first-order Jaumann stress rotation in advectMarkersRK instead of the exact rotation)
$CC $CFLAGS -DJAUMANN $INC -c "$REF/markers.c" -o "$OUT/markers_jaumann.o"
$CC -shared -o "$OUT/libfvmic2d_ref_jaumann.so" $(echo $OBJS | sed "s#$OUT/markers.o#$OUT/markers_jaumann.o#") \
  "$OUT/petsc_lite.o" "$OUT/ref_bridge.o" -lm
rm -f "$OUT"/*.o
echo "built $OUT/libfvmic2d_ref.so $OUT/libfvmic2d_ref_jaumann.so"
