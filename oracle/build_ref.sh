#!/usr/bin/env bash
# Compile the reference's own multi-way cluster-id builder
# (src/core/cluster_id_builder.c) from the reference tree into oracle/_ref/.
# Test infrastructure only: the library is used to check the oracle and the
# CUDA cluster-id kernels bit for bit. It is built only where the reference
# tree is present; nothing in the product links it.
set -euo pipefail
REF="${FE_GPU_REFERENCE:-/root/reference}"
SRC="$REF/src/core/cluster_id_builder.c"
OUT_DIR="$(cd "$(dirname "$0")" && pwd)/_ref"
if [ ! -f "$SRC" ]; then
  echo "reference source not found: $SRC" >&2
  exit 1
fi
mkdir -p "$OUT_DIR"
gcc -O2 -fopenmp -fPIC -shared -o "$OUT_DIR/libref_cluster_ids.so.tmp" "$SRC"
mv "$OUT_DIR/libref_cluster_ids.so.tmp" "$OUT_DIR/libref_cluster_ids.so"
echo "built $OUT_DIR/libref_cluster_ids.so"
