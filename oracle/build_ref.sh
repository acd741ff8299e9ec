#!/usr/bin/env bash
# Compile the reference's own kernel source (MDT_device_functions.cu, read in
# place from the read-only reference checkout) for the CPU, with the stand-in
# CUDA headers in oracle/ref_emu/, into oracle/_ref/libmdt_ref_emu.so.
# The result pins the oracle's bit-exact restatements (PpS_Batch,
# ReorderFOutput) to the reference code itself; tests/golden/make_golden.py
# captures its outputs as committed fixtures.  Runs only where the reference
# checkout exists (the build container), named by MDT_REFERENCE_DIR; nothing
# here is product code.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${MDT_REFERENCE_DIR:-}"
if [ -z "$REF" ]; then
  echo "MDT_REFERENCE_DIR not set; skipping the CPU build of the reference kernels" >&2
  exit 0
fi
SRC="$REF/MDT_OneStation_client/MDT_device_functions.cu"
OUT="$HERE/_ref"
if [ ! -f "$SRC" ]; then
  echo "reference source not found at $SRC; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
# -ffp-contract=off: the CPU run performs exactly the roundings written in the
# source (fmaf where the kernel calls fmaf, separate multiply/add elsewhere).
"$CXX" -O1 -std=c++17 -fopenmp -ffp-contract=off -fPIC -shared \
  -I "$HERE/ref_emu" -include "$HERE/ref_emu/mdt_cuda_emu.h" \
  -x c++ "$SRC" -x c++ "$HERE/ref_emu/ref_runner.cpp" \
  -o "$OUT/libmdt_ref_emu.so"
echo "built $OUT/libmdt_ref_emu.so"
