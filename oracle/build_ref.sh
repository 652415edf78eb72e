#!/bin/sh
# Builds the reference's own hot-path sources, unmodified and from where they
# lie, into oracle/_ref/libgasref.so for pinning the oracle (test use only).
# Usage: oracle/build_ref.sh [reference-dir]   (default /root/reference)
# Writes only under oracle/_ref/.  Needs gcc; no cmake, no reference Makefile.
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/pkd.c" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
CFLAGS="-O2 -fPIC -ffp-contract=off -fno-fast-math -w -DNOCOOLING -DGASOLINE -DM4 \
 -include stdio.h -I$HERE/shim -I$REF -I$HERE/../include"
OBJS=""
for f in pkd walk grav ewald v_sqrt1 treezip smooth smoothfcn dumpframe dffuncs; do
  gcc $CFLAGS -c "$REF/$f.c" -o "$OUT/$f.o" &
  OBJS="$OBJS $OUT/$f.o"
done
gcc $CFLAGS -c "$HERE/shim/mdl_null.c" -o "$OUT/mdl_null.o" &
gcc $CFLAGS -c "$HERE/ref_harness.c" -o "$OUT/ref_harness.o" &
wait
gcc -shared -o "$OUT/libgasref.so" $OBJS "$OUT/mdl_null.o" "$OUT/ref_harness.o" -lm
echo "built $OUT/libgasref.so"
