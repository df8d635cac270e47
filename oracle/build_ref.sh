#!/usr/bin/env bash
# Builds the golden-vector generator oracle/_ref/refgen from the UNMODIFIED
# reference sources (jak-xyz/xpbd-fem) where they lie, plus the harness driver
# oracle/refgen.cpp. Test infrastructure only; outputs go to oracle/_ref/ only.
#
# The reference is compiled as it is, file by file, with a force-included
# prelude (oracle/prelude.h) that supplies the <cmath> float overloads MSVC and
# the wasm libc shim put in the global namespace. -ffp-contract=off keeps the
# float arithmetic unfused so results are the same on x86-64 and AArch64.
# The reference tree is XFEM_REFERENCE_DIR, by default a directory named
# "reference" beside this repository's root. Skipped (exit 0 with a note)
# where the reference tree is absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${XFEM_REFERENCE_DIR:-$HERE/../../reference}/XPBDFEM"
OUT="$HERE/_ref"
if [ ! -f "$REF/Fem.cpp" ]; then
  echo "build_ref: reference sources not found at $REF; skipping"
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-std=c++17 -O2 -ffp-contract=off -w -include $HERE/prelude.h -I$REF"
OBJS=()
for f in Fem Geo Connectivity Allocator MeshGen vectormath DebugGeo; do
  "$CXX" $FLAGS -c "$REF/$f.cpp" -o "$OUT/$f.o" &
  OBJS+=("$OUT/$f.o")
done
"$CXX" $FLAGS -c "$HERE/refgen.cpp" -o "$OUT/refgen.o" &
wait
"$CXX" -o "$OUT/refgen" "$OUT/refgen.o" "${OBJS[@]}"
echo "build_ref: built $OUT/refgen"
