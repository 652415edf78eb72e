#!/bin/sh
# Builds the reference's own hot-path sources, unmodified and from where they
# lie, into oracle/_ref/libgasref.so for pinning the oracle (test use only).
# Usage: oracle/build_ref.sh [--if-present] [reference-dir]
#   reference-dir defaults to $GASOLINE_REFERENCE, else /root/reference (the
#   checkout this recipe was written against).  With --if-present a missing
#   checkout is not an error: the script says so and exits 0.
# Writes only under oracle/_ref/.  Needs gcc; no cmake, no reference Makefile.
set -e
OPTIONAL=0
if [ "$1" = "--if-present" ]; then OPTIONAL=1; shift; fi
REF=${1:-${GASOLINE_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/pkd.c" ]; then
  echo "reference sources not found at $REF" >&2
  [ $OPTIONAL = 1 ] && exit 0
  exit 1
fi
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
# The same harness with ref_grav/ref_sph going through the reference-side
# binding of libtsph (gasoline_gb300/pkd/tsph_pkd.c, compiled against the
# reference's headers as an integrator would), linked against the CPU
# stand-in of libtsph whose arithmetic is the oracle's.
PKDB="$HERE/../gasoline_gb300/pkd"
gcc $CFLAGS -DTSPH_ADAPTER -I"$PKDB" -c "$HERE/ref_harness.c" -o "$OUT/ref_harness_adapter.o" &
gcc $CFLAGS -I"$PKDB" -c "$PKDB/tsph_pkd.c" -o "$OUT/tsph_pkd.o" &
gcc -O2 -fPIC -ffp-contract=off -fno-fast-math -w -I"$HERE" -I"$HERE/../include" \
    -c "$HERE/adapter_fake_tsph.c" -o "$OUT/adapter_fake_tsph.o" &
gcc -O2 -fPIC -ffp-contract=off -fno-fast-math -w -std=gnu99 \
    -c "$HERE/tsph_oracle.c" -o "$OUT/tsph_oracle_adapter.o" &
wait
gcc -shared -o "$OUT/libgasadapt.so" $OBJS "$OUT/mdl_null.o" "$OUT/ref_harness_adapter.o" \
    "$OUT/tsph_pkd.o" "$OUT/adapter_fake_tsph.o" "$OUT/tsph_oracle_adapter.o" -lm
echo "built $OUT/libgasadapt.so"
