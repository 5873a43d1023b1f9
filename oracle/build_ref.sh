#!/bin/bash
# Builds the reference's own C relaxation kernels (x2dhf src/c, pthread
# backend) unmodified into oracle/_ref/libx2dhf_refc.so, linked with
# oracle/ref_shim.c, which supplies what the Fortran program would: the
# COMMON blocks and the putinc_/putoutc_ callbacks.  TEST INFRASTRUCTURE.
#
# The sources are staged from the x2dhf tree into oracle/_ref/src (git-ignored)
# so that the same build can run where the tree is not mounted.  The
# reference passes an int* as void** to pthread_join (mcsor_pthread.c,
# coulExch_pthread.c); it is built without the stack protector, as the
# distribution compilers of its authors do by default, so that this write
# does not abort the multi-threaded runs.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${X2DHF_REF:-/root/reference}"
OUT="$HERE/_ref"
mkdir -p "$OUT/src"
FILES="sorpt.c sorpt.h params.h mcsor_pthread.c mcsor_single_colour_pthread.c coulExch_pthread.c relax_single_pot_pthread.c"
if [ -d "$REF/src/c" ]; then
  for f in $FILES; do cp "$REF/src/c/$f" "$OUT/src/$f"; done
fi
for f in $FILES; do
  if [ ! -f "$OUT/src/$f" ]; then echo "build_ref: reference source $f not available" >&2; exit 0; fi
done
CC="${CC:-gcc}"
$CC -O2 -fPIC -shared -ffp-contract=off -fno-stack-protector -pthread -w -I "$OUT/src" -o "$OUT/libx2dhf_refc.so" \
    "$OUT/src/sorpt.c" "$OUT/src/mcsor_pthread.c" "$OUT/src/mcsor_single_colour_pthread.c" \
    "$OUT/src/coulExch_pthread.c" "$OUT/src/relax_single_pot_pthread.c" "$HERE/ref_shim.c" -lm
echo "built $OUT/libx2dhf_refc.so"
