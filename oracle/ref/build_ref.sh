#!/usr/bin/env bash
# Compiles the reference's host LBVH (bvh.h and the headers it includes) from
# the reference tree into oracle/_ref/libref_lbvh.so. Needs the reference
# sources (REF_ROOT, default /root/reference) and nvcc; it runs where both
# exist and is skipped elsewhere. Nothing from the reference is copied.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
OUT="$HERE/../_ref"
if [ ! -f "$REF_ROOT/src/renderer/bvh.h" ]; then
  echo "reference sources not found at $REF_ROOT; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
"$NVCC" -std=c++17 -O2 -DNDEBUG -Xcompiler -fPIC,-ffp-contract=off -shared \
  -I "$HERE/shim" -I "$REF_ROOT/src" \
  -o "$OUT/libref_lbvh.so" "$HERE/ref_lbvh.cu"
echo "built $OUT/libref_lbvh.so"
