#!/usr/bin/env bash
# Builds the reference's own CPU pipeline (cudaGSEA, read-only sources) into
# oracle/_ref/ to pin the oracle and serve as the CPU baseline.  Test infrastructure only.
#
# Recipe:
#   * the reference sources are staged in a temporary directory as SYMLINKS
#     (nothing is copied); the vendored CUB 1.5 directory is left out so that
#     the quoted "cub/cub.cuh" include resolves to CUDA 13's CCCL CUB, whose
#     DeviceSegmentedRadixSort / DoubleBuffer API still matches;
#   * oracle/ref_harness.cu (ours) includes the staged headers and exports the
#     CPU stages as extern "C" functions -> oracle/_ref/libgsea_ref.so;
#   * the reference CLI (src/cudaGSEA.cu) is built the same way through a shim
#     that adds the standard headers the reference forgets ->
#     oracle/_ref/cudaGSEA_cpu (run with -cpu).
#   * -ffp-contract=off keeps the host compiler from fusing multiply-adds,
#     which is what the reference's x86-64 CPU build computes.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF_ROOT="${1:-/root/reference}"
SRC="$REF_ROOT/cudaGSEA/src"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$SRC/include" ]; then
  echo "reference sources not found under $SRC" >&2
  exit 2
fi
mkdir -p "$OUT"
STAGE="$(mktemp -d /tmp/gsea_ref_stage.XXXXXX)"
trap 'rm -rf "$STAGE"' EXIT
mkdir -p "$STAGE/include"
for f in "$SRC"/*.cu "$SRC"/*.cuh "$SRC"/*.cpp "$SRC"/HELP.txt; do
  ln -s "$f" "$STAGE/$(basename "$f")"
done
for f in "$SRC"/include/*; do
  b="$(basename "$f")"
  [ "$b" = "cub" ] && continue
  ln -s "$f" "$STAGE/include/$b"
done

ARCH="-gencode arch=compute_103a,code=sm_103a"
HOSTFLAGS="-fopenmp -ffp-contract=off -fPIC -w"
QUIET="-diag-suppress 174,177,550,20012"

# 1) harness library (stage functions)
nvcc -O3 -std=c++17 $QUIET $ARCH -I"$STAGE" -Xcompiler "$HOSTFLAGS" -shared \
     -o "$OUT/libgsea_ref.so" "$HERE/ref_harness.cu" -lgomp

# 2) the reference CLI, CPU mode usable without a GPU
cat > "$STAGE/shim.cu" <<'EOF'
#include <cstdint>
#include <numeric>
#include <climits>
#include <functional>
#include <algorithm>
#include <cuda_runtime.h>
#define cudaGetLastError() cudaSuccess
#include "cudaGSEA.cu"
EOF
nvcc -O3 -std=c++17 $QUIET $ARCH -I"$STAGE" -Xcompiler "-fopenmp -ffp-contract=off -w -DCUDA_GSEA_OPENMP_ENABLED" \
     -o "$OUT/cudaGSEA_cpu" "$STAGE/shim.cu" -lgomp
echo "built $OUT/libgsea_ref.so $OUT/cudaGSEA_cpu"
