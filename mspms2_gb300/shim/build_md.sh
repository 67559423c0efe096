#!/bin/sh
# Links the mspms2 program with this engine as its force layer: the reference's own C
# sources, compiled where they lie under the reference checkout (first argument, else
# $MSPMS2_REF, else the checkout oracle/build_ref.sh recorded in oracle/_ref/checkout),
# without src/frclong.c and src/frcshort.c (replaced by frc_gb300.c)
# and without src/dftmcff.c (the GSL metal-cluster force field, called only from the
# replaced frclong.c). The mylibtasos Fortran entry points come from frc_gb300.c.
#
# Output: mspms2_gb300/shim/_build/mspms2_gb300_md, linked against
# mspms2_gb300/libmspms2_gb300.so (build that first: python -m mspms2_gb300.build).
# Nothing of the reference is copied into the repository; its objects stay in _build/.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
REF=${1:-$MSPMS2_REF}
if [ -z "$REF" ] && [ -f "$ROOT/oracle/_ref/checkout" ]; then
  REF=$(cat "$ROOT/oracle/_ref/checkout")
fi
OUT="$HERE/_build"
CC=${CC:-gcc}
if [ -z "$REF" ] || [ ! -f "$REF/src/frclong.c" ]; then
  echo "build_md.sh: no reference checkout (argument, MSPMS2_REF or oracle/_ref/checkout); skipping" >&2
  exit 0
fi
if [ ! -f "$ROOT/mspms2_gb300/libmspms2_gb300.so" ]; then
  echo "build_md.sh: mspms2_gb300/libmspms2_gb300.so is missing; run python -m mspms2_gb300.build" >&2
  exit 1
fi
rm -rf "$OUT"
mkdir -p "$OUT"
CFLAGS="-std=gnu99 -O2 -fcommon -w -I$REF/src"
for f in "$REF"/src/*.c; do
  b=$(basename "$f" .c)
  case "$b" in frclong|frcshort|dftmcff) continue ;; esac
  $CC $CFLAGS -c "$f" -o "$OUT/$b.o"
done
# src/misc.c:127 (deriv_inc_gamma, not on any force path) refers to GSL's incomplete
# gamma function, which is not installed here
cat > "$OUT/no_gsl.c" <<'EOF'
#include <stdio.h>
#include <stdlib.h>
double gsl_sf_gamma_inc(double a, double x) {
    (void)a; (void)x;
    fprintf(stderr, "gsl_sf_gamma_inc is not available in this build\n");
    abort();
}
EOF
$CC $CFLAGS -c "$OUT/no_gsl.c" -o "$OUT/no_gsl.o"
$CC $CFLAGS -Wall -I"$ROOT/include" -c "$HERE/frc_gb300.c" -o "$OUT/frc_gb300.o"
$CC -o "$OUT/mspms2_gb300_md" "$OUT"/*.o -L"$ROOT/mspms2_gb300" -lmspms2_gb300 \
    -Wl,-rpath,"$ROOT/mspms2_gb300" -lm
echo "$OUT/mspms2_gb300_md"
