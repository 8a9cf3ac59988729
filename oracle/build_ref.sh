#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY.  Builds the reference's own code, unmodified, from
# the read-only reference tree into oracle/_ref/ (git-ignored):
#   * ref_loader      : src/graph.cpp (the SNAP loader, serialized cache and JSON
#                       writer) + oracle/ref_loader_main.cpp, host code (x86 build
#                       host only: it makes the golden fixtures under tests/golden/)
#   * ref_peel.cubin  : src/ours.cc + src/buffer.cc kernels (selectNodesAtLevel1,
#                       processNodes1) for sm_103a; oracle/ref_peel_driver.cpp loads it
#                       through the CUDA driver API on a GPU host
# Nothing here is copied into the repository.  The reference tree is taken from
# KC_REFERENCE_DIR (kcoregpu_gb300/build.py sets it to the checkout beside this
# repository when one is there).
set -euo pipefail
REF=${KC_REFERENCE_DIR:?set KC_REFERENCE_DIR to the reference checkout}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
[ -d "$REF/src" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
g++ -O2 -fopenmp -I/usr/local/cuda/include -I"$REF/inc" \
    "$REF/src/graph.cpp" "$HERE/ref_loader_main.cpp" -o "$OUT/ref_loader"
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -I"$REF/inc" -I"$REF/src" \
    -o "$OUT/ref_peel.cubin" "$HERE/ref_peel_kernels.cu"
echo "built $OUT/ref_loader $OUT/ref_peel.cubin"
