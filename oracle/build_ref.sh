#!/bin/sh
# Builds the reference library (libqdt, C++14) straight from its own sources
# into oracle/_ref/, for use as a checker and a CPU baseline. It needs the
# reference tree (default /root/reference, or $QDT_REFERENCE); where that tree
# is absent the script does nothing and exits 0. Outputs never leave
# oracle/_ref/ (git-ignored).
set -e
REF="${QDT_REFERENCE:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/libqdt/qdt.cpp" ]; then
    echo "build_ref: reference sources not found at $REF; skipped"
    exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-std=c++14 -O2 -pthread -fPIC -fno-fast-math -ffp-contract=off"
$CXX $FLAGS -shared -o "$OUT/libqdt_ref.so" \
    "$REF/libqdt/qdt.cpp" \
    "$REF/libqdt/GuibasStolfiDwyer_Wrapper.cpp" \
    "$REF/libqdt/GuibasStolfiDwyer_Threads.cpp"
# the reference's own correctness harness, linked against the reference
$CXX $FLAGS -I"$REF/libqdt" -o "$OUT/qdt_verify_ref" "$REF/test/qdt_verify.cpp" \
    -L"$OUT" -lqdt_ref -Wl,-rpath,"$OUT"
# bulk read-back helper for the fixture generator, bound to the reference
gcc -O2 -fPIC -shared -o "$OUT/libqdt_dump_ref.so" "$HERE/qdt_dump.c" -L"$OUT" -lqdt_ref -Wl,-rpath,"$OUT"
echo "build_ref: built $OUT/libqdt_ref.so and $OUT/qdt_verify_ref"
