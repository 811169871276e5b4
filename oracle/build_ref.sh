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
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $GSEA_REFERENCE_ROOT, else to the copy that
#   oracle/stage_ref.sh staged in baseline/_ref/ (git-ignored; it travels to
#   the GPU host, where this script then builds the reference natively).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${1:-${GSEA_REFERENCE_ROOT:-$(dirname "$HERE")/baseline/_ref}}"
SRC="$REF_ROOT/cudaGSEA/src"
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

# 1) harness library (stage functions), built beside the CLI below
nvcc -O3 -std=c++17 $QUIET $ARCH -I"$STAGE" -Xcompiler "$HOSTFLAGS" -shared \
     -o "$OUT/libgsea_ref.so.tmp$$" "$HERE/ref_harness.cu" -lgomp &
HARNESS=$!

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
     -o "$OUT/cudaGSEA_cpu.tmp$$" "$STAGE/shim.cu" -lgomp
wait "$HARNESS"
mv "$OUT/libgsea_ref.so.tmp$$" "$OUT/libgsea_ref.so"
mv "$OUT/cudaGSEA_cpu.tmp$$" "$OUT/cudaGSEA_cpu"
echo "built $OUT/libgsea_ref.so $OUT/cudaGSEA_cpu"
