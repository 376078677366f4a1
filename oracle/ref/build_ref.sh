#!/usr/bin/env bash
# Compiles reference code from the reference tree into oracle/_ref/ (outputs
# only; nothing from the reference is copied into this repository):
#   libref_lbvh.so         the reference's host LBVH (bvh.h and the headers it
#                          includes), for pinning the LBVH oracle;
#   ref_kernels.cubin      the reference's own device kernels (pathtracer_kernel.h:
#                          primary rays, traversal, shading, accumulation, frame
#                          finish) for sm_103a with nvcc's default device flags,
#                          as its own build compiles them;
#   ref_kernels_nofma.cubin the same with --fmad=false (every float operation
#                          rounded as written), for bit-exact pinning of the
#                          traversal restatement;
#   ref_layout.json        the byte layout of the records those kernels read;
#   libref_records.so      reference scene records (camera, environment) built
#                          by the reference's own host code, for pinning the
#                          records ref_gpu.py lays out;
#   libref_loader.so       the reference's scene loading (Scene::Scene: the
#                          Mitsuba-XML and OBJ loaders and the flattening into
#                          m_cpu_triangles), compiled by the host C++ compiler
#                          as the reference's CMake build (cuda_add_executable)
#                          compiles its .cpp files, for pinning this library's
#                          loader (ref_loader.cpp). texture.h's
#                          TextureView::operator=(TextureView&) cannot take the
#                          temporaries mitsubaloader.cpp assigns with g++, so
#                          a copy of that one header with the parameter made
#                          const is generated into _ref/patch/ and found first.
# Needs the reference sources (GR_REFERENCE_ROOT, default /root/reference) and
# nvcc; it runs where both exist and is skipped elsewhere.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${GR_REFERENCE_ROOT:-/root/reference}"
OUT="$HERE/../_ref"
if [ ! -f "$REF_ROOT/src/renderer/bvh.h" ]; then
  echo "reference sources not found at $REF_ROOT; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
"$NVCC" -std=c++17 -O2 -DNDEBUG -Xcompiler -fPIC,-ffp-contract=off -shared \
  -I "$HERE/shim" -I "$REF_ROOT/src" \
  -o "$OUT/libref_lbvh.so" "$HERE/ref_lbvh.cu" &
# Warnings the reference's headers raise (host functions redeclared host-device,
# inline __global__, missing returns, unused values) are not ours to fix.
QUIET="-diag-suppress 20040,20050,940,174,177,550"
KFLAGS="-std=c++17 -cubin -gencode arch=compute_103a,code=sm_103a $QUIET -I $HERE/shim_assert -I $HERE/shim -I $REF_ROOT/src"
"$NVCC" $KFLAGS -o "$OUT/ref_kernels.cubin" "$HERE/ref_kernels.cu" &
"$NVCC" $KFLAGS --fmad=false -o "$OUT/ref_kernels_nofma.cubin" "$HERE/ref_kernels.cu" &
HOSTINC="-I $HERE/shim_assert -I $HERE/shim -I $REF_ROOT/src"
R="$REF_ROOT/src/renderer"
"$NVCC" -std=c++17 -O1 -shared -Xcompiler -fPIC $QUIET $HOSTINC -o "$OUT/libref_records.so" \
  "$HERE/ref_records.cu" "$R/transform.cpp" "$R/environment.cpp" "$R/imageio.cpp" &
mkdir -p "$OUT/patch/renderer"
sed 's/void operator = (TextureView& t)/void operator = (const TextureView\& t)/' "$R/texture.h" \
  > "$OUT/patch/renderer/texture.h"
CUDA_INC="$(dirname "$(command -v "$NVCC")")/../include"
g++ -std=c++17 -O2 -shared -fPIC -w -I "$HERE/shim_assert" -I "$HERE/shim" -I "$OUT/patch" -I "$REF_ROOT/src" \
  -I "$REF_ROOT/src/ext/tinyobjloader" -I "$CUDA_INC" -I "$CUDA_INC/cccl" \
  -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP \
  -include memory -include cstdint -include cstring -include algorithm -include fstream \
  -o "$OUT/libref_loader.so" "$HERE/ref_loader.cpp" "$R/scene.cpp" "$R/loaders/mitsubaloader.cpp" \
  "$R/loaders/objloader.cpp" "$R/loaders/propertylist.cpp" "$R/texture.cpp" "$R/triangle.cpp" "$R/transform.cpp" \
  "$R/environment.cpp" "$R/imageio.cpp" "$R/framebuffer.cpp" "$REF_ROOT/src/ext/pugixml/pugixml.cpp" &
TMP="$(mktemp -d)"
"$NVCC" -std=c++17 -O1 $QUIET -Xcompiler -Wno-invalid-offsetof $HOSTINC \
  -o "$TMP/ref_layout" "$HERE/ref_layout.cu" "$R/transform.cpp"
"$TMP/ref_layout" > "$OUT/ref_layout.json"
rm -f "$TMP/ref_layout"
rmdir "$TMP"
for job in 1 2 3 4 5; do wait %$job; done
echo "built $OUT/libref_lbvh.so, libref_records.so, libref_loader.so, ref_kernels.cubin, ref_kernels_nofma.cubin, ref_layout.json"
