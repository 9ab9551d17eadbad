#!/bin/sh
# Build the reference's own mechanics functions from the reference sources into
# oracle/_ref/libwcfe_ref_<variant>.so (test infrastructure: pins the C
# restatement and generates tests/golden/).  Compiles, per variant, exactly
#   cellBP/UL_growth_explicit.cpp + eltopo3d/nondestructivetrimesh.cpp
#   + cellBP/iomesh.cpp and common/bfstream.cpp (the VTK frame writers)
# with the reference's own release flags (-O3 -funroll-loops, cellBP/Makefile.local_defs:9)
# plus -fPIC, and links the harness (ref_harness.cpp) and the rand()/srand()
# stand-ins (ref_rng.c) with -Bsymbolic.  Does not run the reference's build system.
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: $WCFE_REF or /root/reference)
set -e
REF=${1:-${WCFE_REF:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/wholeCellFE_kMD/cellBP" ]; then
    echo "reference sources not found at $REF; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$OUT"
gcc -O2 -fPIC -c "$HERE/ref_rng.c" -o "$OUT/ref_rng.o"
for V in kMD k1 k31; do
    D="$REF/wholeCellFE_$V"
    INC="-I$D/cellBP -I$D/eltopo3d -I$D/common"
    FLAGS="-O3 -funroll-loops -fPIC -w -D__LITTLE_ENDIAN__ -DNO_GUI"
    g++ $FLAGS $INC -c "$D/cellBP/UL_growth_explicit.cpp" -o "$OUT/ul_$V.o" &
    g++ $FLAGS $INC -c "$D/eltopo3d/nondestructivetrimesh.cpp" -o "$OUT/ndtm_$V.o" &
    g++ $FLAGS $INC -c "$D/cellBP/iomesh.cpp" -o "$OUT/iomesh_$V.o" &
    g++ $FLAGS $INC -c "$D/common/bfstream.cpp" -o "$OUT/bfs_$V.o" &
    HFLAGS=""
    if [ "$V" = "kMD" ]; then HFLAGS="-DWCFE_REF_WRITER_KINT"; fi
    g++ $FLAGS $HFLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OUT/harness_$V.o" &
    wait
    g++ -shared -Wl,-Bsymbolic -o "$OUT/libwcfe_ref_$V.so" "$OUT/ul_$V.o" "$OUT/ndtm_$V.o" "$OUT/iomesh_$V.o" \
        "$OUT/bfs_$V.o" "$OUT/harness_$V.o" "$OUT/ref_rng.o" -lm
done
rm -f "$OUT"/*.o
echo "built $(ls "$OUT"/*.so | wc -l) reference libraries in $OUT"
