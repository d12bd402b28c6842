#!/bin/bash
# Builds the reference's own CUDA driver (test infrastructure) into
# oracle/_ref/ref_driver from the PASIf sources: by default where they lie
# (/root/reference/src), or from REF_SRC.  Plain nvcc on the reference's
# three translation units plus oracle/ref/ref_driver.cu; reel = double as the
# reference ships it.  Output only into oracle/_ref/ (git-ignored).
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(dirname "$(dirname "$HERE")")"
REF_SRC="${REF_SRC:-/root/reference/src}"
ARCH="${REF_ARCH:-sm_103}"
mkdir -p "$ROOT/oracle/_ref"
nvcc -O3 -std=c++17 -arch="$ARCH" -w -I"$REF_SRC" \
    "$HERE/ref_driver.cu" "$REF_SRC/__GpuDriver.cu" "$REF_SRC/helpers.cu" "$REF_SRC/kernels.cu" \
    -lcublas -lcusparse -o "$ROOT/oracle/_ref/ref_driver"
echo "$ROOT/oracle/_ref/ref_driver"
