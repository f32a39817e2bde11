#!/usr/bin/env bash
# Builds oracle/_ref/libref.so from the reference's own header-only sources,
# compiled in place (include path only, nothing copied), with the small shim
# headers in oracle/ref/shim standing in for the configure-generated files.
# Test-infrastructure only; the output stays out of version control.
#
# usage: oracle/ref/build_ref.sh [REFERENCE_ROOT]
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ref="${1:-/root/reference}"
out="$here/../_ref"
if [ ! -d "$ref/include/libint2" ]; then
  echo "reference tree not found at $ref; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$out"
g++ -std=c++17 -O2 -fPIC -shared -w \
  -I"$here/shim" -I"$ref/include" -I"$ref/src/bin/test_eri" \
  -DDATADIR="\"$ref/lib\"" -DLIBINT2_DISABLE_BOOST_CONTAINER_SMALL_VECTOR \
  "$here/ref_driver.cpp" -o "$out/libref.so.tmp"
mv "$out/libref.so.tmp" "$out/libref.so"
echo "built $out/libref.so"
