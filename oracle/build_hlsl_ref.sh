#!/bin/sh
# Extracts the bench's dependency-marking shader functions, DepMarkPoint and DepMarkSegment,
# unchanged from the reference's windows/patch/rtxgi_bench.patch (read where it lies in the
# reference checkout) into oracle/_ref/hlsl_dep.inc, and compiles them as C++ with
# oracle/hlsl_compat.h into oracle/_ref/libhlsl_dep.so (no FP contraction).  The only edit is
# HLSL's `inout uint3 m` parameter, which becomes `uint3& m`.
# Usage: oracle/build_hlsl_ref.sh [reference checkout]; default $RC_REFERENCE_DIR, else the
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
g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -fPIC -shared -I "$HERE" -I "$HERE/_ref" \
    "$HERE/hlsl_dep_ref.cpp" -o "$HERE/_ref/libhlsl_dep.so.tmp"
mv "$HERE/_ref/libhlsl_dep.so.tmp" "$HERE/_ref/libhlsl_dep.so"
