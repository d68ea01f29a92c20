#!/usr/bin/env bash
# Compiles the reference's own CUDA kernels (RFBA Main/GradientCalc/kernel.cu,
# unmodified, default nvcc options as its Visual Studio project uses) for
# sm_103a into baseline/_ref/srrf_ref_kernel.sm_103a.cubin. Only device code
# goes into the cubin; the reference's host orchestration is restated in
# baseline/refgpu.py, which loads the cubin through the CUDA driver API.
# A cubin is GPU code, not host code, so the file built here also runs on the
# Arm GPU host. baseline/_ref/ is git-ignored: nothing built here is committed.
#
# Usage: baseline/build_refgpu.sh [REFERENCE_ROOT]
# The tree is $RFBA_REFERENCE_ROOT when set, else the argument, else the
# development container's mount point (/root/reference).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${RFBA_REFERENCE_ROOT:-${1:-/root/reference}}"
src="$ref/RFBA Main/GradientCalc"
if [ ! -f "$src/kernel.cu" ]; then
  echo "build_refgpu: reference sources not found under $ref; skipping" >&2
  exit 0
fi
out="$here/_ref"
mkdir -p "$out"
cubin="$out/srrf_ref_kernel.sm_103a.cubin"
if [ -f "$cubin" ] && [ "$cubin" -nt "$src/kernel.cu" ] && [ "$cubin" -nt "$0" ]; then
  exit 0
fi
nvcc=$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)
"$nvcc" -cubin -gencode arch=compute_103a,code=sm_103a -I "$src" "$src/kernel.cu" -o "$cubin.tmp"
mv "$cubin.tmp" "$cubin"
echo "build_refgpu: built $cubin"
