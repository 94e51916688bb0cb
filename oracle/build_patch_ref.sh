#!/bin/sh
# Extracts from the reference's windows/patch/rtxgi_bench.patch (read where it lies in the
# reference checkout), unchanged:
#   the dependency-marking shader functions DepMarkPoint and DepMarkSegment -> _ref/hlsl_dep.inc
#     (the only edit: HLSL's `inout uint3 m` parameter becomes `uint3& m`);
#   the host function Pathtracer::BenchObjVoxels (an object's event zones) -> _ref/bench_obj.inc;
#   the snapshot compute shaders of BenchSnap.hlsl -> _ref/bench_snap.inc (register and semantic
#     annotations and [numthreads] removed, `out` parameters made references);
# and compiles them as C++ with oracle/patch_ref.cpp (HLSL's types from oracle/hlsl_compat.h, a
# stand-in for the members BenchObjVoxels reads) into oracle/_ref/libpatch_ref.so, without FP
# contraction.
# Usage: oracle/build_patch_ref.sh [reference checkout]; default $RC_REFERENCE_DIR, else the
# directory "reference" beside this repository
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${RC_REFERENCE_DIR:-$HERE/../../reference}}"
PATCH="$REF/windows/patch/rtxgi_bench.patch"
[ -f "$PATCH" ] || { echo "reference patch not found: $PATCH" >&2; exit 1; }
mkdir -p "$HERE/_ref"
# the added lines from "void DepMarkPoint" up to (not including) "void DepOr", '+' removed
awk '
  /^\+void DepMarkPoint\(/ { on = 1 }
  /^\+void DepOr\(/ { on = 0 }
  on && /^\+/ { print substr($0, 2) }
' "$PATCH" | sed 's/inout uint3 m/uint3\& m/' > "$HERE/_ref/hlsl_dep.inc.tmp"
grep -q "void DepMarkSegment" "$HERE/_ref/hlsl_dep.inc.tmp" || { echo "marking functions not found in $PATCH" >&2; exit 1; }
mv "$HERE/_ref/hlsl_dep.inc.tmp" "$HERE/_ref/hlsl_dep.inc"
# the added lines of BenchObjVoxels, from its definition to its closing brace
awk '
  /^\+void Pathtracer::BenchObjVoxels\(/ { on = 1 }
  on && /^\+/ { print substr($0, 2) }
  on && /^\+}/ { on = 0 }
' "$PATCH" > "$HERE/_ref/bench_obj.inc.tmp"
grep -q "BenchObjVoxels" "$HERE/_ref/bench_obj.inc.tmp" || { echo "BenchObjVoxels not found in $PATCH" >&2; exit 1; }
mv "$HERE/_ref/bench_obj.inc.tmp" "$HERE/_ref/bench_obj.inc"
# the snapshot compute shaders (the new file BenchSnap.hlsl), with HLSL's register and semantic
# annotations and its [numthreads] attributes removed and its `out` parameters made references
awk '
  /^\+\+\+ b\/Samples\/Pathtracer\/BenchSnap.hlsl/ { on = 1; next }
  on && /^diff --git/ { on = 0 }
  on && /^\+/ { print substr($0, 2) }
' "$PATCH" | sed -e 's/ *: *register([^)]*)//' -e '/^\[numthreads/d' -e 's/ *: *SV_DispatchThreadID//' \
                 -e 's/out \(uint[0-9]\) \([a-z][a-z]*\)/\1\& \2/g' > "$HERE/_ref/bench_snap.inc.tmp"
grep -q "void snapRestore" "$HERE/_ref/bench_snap.inc.tmp" || { echo "BenchSnap.hlsl not found in $PATCH" >&2; exit 1; }
mv "$HERE/_ref/bench_snap.inc.tmp" "$HERE/_ref/bench_snap.inc"
g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -fPIC -shared -I "$HERE" -I "$HERE/_ref" \
    "$HERE/patch_ref.cpp" -o "$HERE/_ref/libpatch_ref.so.tmp"
mv "$HERE/_ref/libpatch_ref.so.tmp" "$HERE/_ref/libpatch_ref.so"
