#!/usr/bin/env bash
# Stages the reference's CPU-path sources (cudaGSEA/src without the vendored
# CUB 1.5, which CUDA 13's CCCL CUB replaces) into baseline/_ref/, the
# git-ignored folder that travels with the working tree to the GPU host, so
# that oracle/build_ref.sh can compile the reference's own CPU pipeline there
# (the GPU host is aarch64 and receives no binaries built here).  Nothing
# staged is ever committed: baseline/_ref/ is listed in .gitignore.
# Test infrastructure only.
#
# Usage: oracle/stage_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Exits 0 without staging when the reference sources are not on this machine.
set -euo pipefail
REF_ROOT="${1:-/root/reference}"
SRC="$REF_ROOT/cudaGSEA/src"
HERE="$(cd "$(dirname "$0")" && pwd)"
DEST="$(dirname "$HERE")/baseline/_ref/cudaGSEA/src"
if [ ! -d "$SRC/include" ]; then
  echo "reference sources not found under $SRC: nothing staged"
  exit 0
fi
rm -rf "$DEST.tmp$$"
mkdir -p "$DEST.tmp$$/include"
for f in "$SRC"/*.cu "$SRC"/*.cuh "$SRC"/*.cpp "$SRC"/HELP.txt; do
  cp "$f" "$DEST.tmp$$/"
done
for f in "$SRC"/include/*; do
  [ "$(basename "$f")" = "cub" ] && continue
  cp -r "$f" "$DEST.tmp$$/include/"
done
chmod -R u+w "$DEST.tmp$$"
rm -rf "$DEST"
mv "$DEST.tmp$$" "$DEST"
echo "staged $SRC -> $DEST"
