#!/usr/bin/env bash
# Compile the reference's own kernel source (MDT_OneStation_client/
# MDT_device_functions.cu, read in place from the reference checkout named by
# MDT_REFERENCE_DIR) for sm_103a into baseline/_ref/mdt_ref_kernels.fatbin.
# baseline/refseq.cu loads it on the GPU to run the reference's own FX
# sequence (its kernels plus cuFFT and cuBLAS) beside this repository's
# library.  The fatbin is git-ignored and travels to the GPU machine with the
# working tree; nothing here is product code.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${MDT_REFERENCE_DIR:-}"
if [ -z "$REF" ]; then
  echo "MDT_REFERENCE_DIR not set; skipping the GPU build of the reference kernels" >&2
  exit 0
fi
SRC="$REF/MDT_OneStation_client/MDT_device_functions.cu"
if [ ! -f "$SRC" ]; then
  echo "reference source not found at $SRC; skipping" >&2
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
"$NVCC" -fatbin -gencode arch=compute_103a,code=sm_103a -O3 \
  -I "$REF/MDT_OneStation_client" -o "$OUT/mdt_ref_kernels.fatbin.tmp" "$SRC"
mv "$OUT/mdt_ref_kernels.fatbin.tmp" "$OUT/mdt_ref_kernels.fatbin"
sha256sum "$SRC" | awk '{print "source sha256 " $1}' > "$OUT/mdt_ref_kernels.txt"
"$NVCC" --version | tail -1 >> "$OUT/mdt_ref_kernels.txt"
echo "built $OUT/mdt_ref_kernels.fatbin"
