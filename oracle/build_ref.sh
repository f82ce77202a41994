#!/usr/bin/env bash
# Build the LPM-C reference from its own sources into oracle/_ref/ (test
# oracle only).  The sources are compiled where they lie; nothing is copied.
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Needs gcc with OpenMP.  MKL is replaced by oracle/mkl_shim (public-API shim).
# src/lpmc_project.c is compiled with its main() renamed so that its global
# definitions link while oracle/ref_driver.c provides callable load steps.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
    echo "reference sources not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT/obj"
CFLAGS="-std=gnu11 -O2 -fopenmp -ffp-contract=off -fPIC -w -I$HERE/mkl_shim -I$REF/include"
pids=()
for f in "$REF"/src/*.c; do
    b="$(basename "$f" .c)"
    extra=""
    [ "$b" = "lpmc_project" ] && extra="-Dmain=lpm_reference_main"
    gcc $CFLAGS $extra -c "$f" -o "$OUT/obj/$b.o" & pids+=($!)
done
gcc $CFLAGS -c "$HERE/mkl_shim/mkl_shim.c" -o "$OUT/obj/mkl_shim.o" & pids+=($!)
gcc $CFLAGS -c "$HERE/ref_driver.c" -o "$OUT/obj/ref_driver.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
gcc -shared -fopenmp -o "$OUT/libref_lpm.so" "$OUT"/obj/*.o -lm
echo "built $OUT/libref_lpm.so"
