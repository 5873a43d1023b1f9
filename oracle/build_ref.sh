#!/bin/bash
# Builds the reference's own C relaxation kernels (x2dhf src/c, pthread
# backend) unmodified into oracle/_ref/libx2dhf_refc.so, linked with
# oracle/ref_shim.c, which supplies what the Fortran program would: the
# COMMON blocks and the putinc_/putoutc_ callbacks.  TEST INFRASTRUCTURE.
#
# The sources are staged from the x2dhf tree into oracle/_ref/src (git-ignored)
# so that the same build can run where the tree is not mounted.  The
# reference passes an int* as void** to pthread_join (mcsor_pthread.c,
# coulExch_pthread.c): the sources are compiled with pthread_join renamed to
# the shim's x2r_pthread_join, which discards the exit value instead of
# storing a pointer into 4 bytes of their stack.  The potential driver
# (coulExch_pthread_ / relax_single_pot_pthread_, which writes past a stack
# array at relax_single_pot_pthread.c:47) is linked but not called: the
# shim's x2r_coulexch drives sorpt_ one thread per potential.
#
# Usage: build_ref.sh [x2dhf-tree]; the tree defaults to $X2DHF_REF, else to
# the read-only mount where this build environment provides the reference.
# Without a tree the previously staged sources are compiled.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${X2DHF_REF:-/root/reference}}"
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
$CC -O2 -fPIC -shared -ffp-contract=off -fno-stack-protector -pthread -w -Dpthread_join=x2r_pthread_join \
    -I "$OUT/src" -o "$OUT/libx2dhf_refc.so" \
    "$OUT/src/sorpt.c" "$OUT/src/mcsor_pthread.c" "$OUT/src/mcsor_single_colour_pthread.c" \
    "$OUT/src/coulExch_pthread.c" "$OUT/src/relax_single_pot_pthread.c" "$HERE/ref_shim.c" -lm
echo "built $OUT/libx2dhf_refc.so"
