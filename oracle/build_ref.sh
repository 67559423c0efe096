#!/bin/sh
# Builds the reference mspms2 force layer (C part) into oracle/_ref/ as the pinning
# oracle for the CPU restatement. TEST INFRASTRUCTURE ONLY.
#
# Sources are read where they lie under the reference checkout, given as the first
# argument or as $MSPMS2_REF (no default: without one the script does nothing). The path is
# recorded in oracle/_ref/checkout for the recipes that link or run against the same
# checkout later (mspms2_gb300/shim/build_md.sh, tests/golden/gen_golden.py).
# Two documented patches are applied to transient copies under
# oracle/_ref/build/, which are deleted after compiling (nothing of the reference is
# kept in the repository):
#   1. src/frclong.c:86 - j atoms of molecule iMole+1 (the unpatched line pairs a
#      molecule with itself for iMole >= 1 and returns NaN);
#   2. src/molevars.h:6-13 - NATOM_MAX/NMOLE_MAX/NBOND_MAX/NANGLE_MAX raised so the
#      benchmark systems fit.
# Also built: tools/sfgridgen.c (the solid-fluid grid generator) as oracle/_ref/sfgridgen, and
# the reference program itself (src/mspms2.c's main) as oracle/_ref/mspms2_ref.
# Left out of mspms_ref_force: src/mspms2.c (its main() is replaced by oracle/ref_harness.c);
# left out of both: src/dftmcff.c (needs GSL). The Fortran grid library mylibtasos/ cannot be compiled
# here (no gfortran); oracle/ref_stubs.c supplies its four entry points on top of the
# C restatement in oracle/mspms_oracle.c.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-$MSPMS2_REF}
OUT="$HERE/_ref"
CC=${CC:-gcc}
if [ -z "$REF" ] || [ ! -f "$REF/src/frclong.c" ]; then
  echo "build_ref.sh: no reference checkout (argument or MSPMS2_REF); skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
printf '%s\n' "$REF" > "$OUT/checkout"
rm -rf "$OUT/build"
mkdir -p "$OUT/build/src"
for f in "$REF"/src/*.c "$REF"/src/*.h; do
  b=$(basename "$f")
  case "$b" in mspms2.c|dftmcff.c) continue ;; esac
  cp "$f" "$OUT/build/src/$b"
done
sed -i 's/jabs = jsum_atom + (jStartMole==DYNAMIC_ID ? jAtom : 0);/jabs = (jStartMole==DYNAMIC_ID ? iabs + jAtom : jsum_atom);/' "$OUT/build/src/frclong.c"
grep -q 'jabs = (jStartMole==DYNAMIC_ID ? iabs + jAtom : jsum_atom);' "$OUT/build/src/frclong.c"
sed -i -e 's/^#define NATOM_MAX.*/#define NATOM_MAX	200000/' \
       -e 's/^#define NBOND_MAX.*/#define NBOND_MAX	200000/' \
       -e 's/^#define NANGLE_MAX.*/#define NANGLE_MAX	200000/' \
       -e 's/^#define NDIH_MAX.*/#define NDIH_MAX	200000/' \
       -e 's/^#define NIMP_MAX.*/#define NIMP_MAX	200000/' \
       -e 's/^#define NNBP_MAX.*/#define NNBP_MAX	200000/' \
       -e 's/^#define NMOLE_MAX.*/#define NMOLE_MAX	70000/' "$OUT/build/src/molevars.h"
CFLAGS="-std=gnu99 -O2 -fcommon -ffp-contract=off -w"
OBJS=""
for f in "$OUT"/build/src/*.c "$HERE/ref_harness.c" "$HERE/ref_stubs.c" "$HERE/mspms_oracle.c"; do
  o="$OUT/build/$(basename "$f" .c).o"
  $CC $CFLAGS -I"$OUT/build/src" -c "$f" -o "$o"
  OBJS="$OBJS $o"
done
$CC -o "$OUT/mspms_ref_force" $OBJS -lm
echo "built $OUT/mspms_ref_force"
# the reference program itself (its main, src/mspms2.c, with the same two patches and the
# same stand-ins): the CPU side of the drop-in comparison in mspms2_gb300/shim/compare_md.py
cp "$REF/src/mspms2.c" "$OUT/build/src/mspms2.c"
$CC $CFLAGS -I"$OUT/build/src" -c "$OUT/build/src/mspms2.c" -o "$OUT/build/mspms2.o"
$CC -o "$OUT/mspms2_ref" $(echo $OBJS | tr ' ' '\n' | grep -v '/ref_harness.o$' | tr '\n' ' ') "$OUT/build/mspms2.o" -lm
echo "built $OUT/mspms2_ref"
rm -rf "$OUT/build"
# the reference's solid-fluid grid generator, unchanged, read where it lies
if [ -f "$REF/tools/sfgridgen.c" ]; then
  $CC -O2 -ffp-contract=off -w -o "$OUT/sfgridgen" "$REF/tools/sfgridgen.c" -lm
  echo "built $OUT/sfgridgen"
fi
