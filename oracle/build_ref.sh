#!/usr/bin/env bash
# Builds oracle/_ref/libsrrf_ref_host.so: the reference's own GradientCalc sources
# (kernel.cu + GradientCalc.cpp), compiled as host C++ against the stand-in
# headers in oracle/refshim, so the reference's exact FP32 arithmetic and its
# block split / put-back loop run on CPU cores. It pins the oracle.
#
# The only change made to the reference text is mechanical and happens in a
# temporary folder outside the repository (removed on exit): each CUDA launch
# `k << <g, b >> > (args)` becomes `REF_LAUNCH(g, b, k, args)` (a host grid
# loop). GradientCalc.cpp compiles from where it lies. Only the built library
# lands in oracle/_ref/, which is git-ignored.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The tree is $RFBA_REFERENCE_ROOT when set, else the argument, else the
# development container's mount point (/root/reference).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${RFBA_REFERENCE_ROOT:-${1:-/root/reference}}"
src="$ref/RFBA Main/GradientCalc"
if [ ! -f "$src/kernel.cu" ]; then
  echo "build_ref: reference sources not found under $ref; skipping" >&2
  exit 0
fi
out="$here/_ref"
mkdir -p "$out"
rm -f "$out/kernel_host.cpp"
tmp="$(mktemp -d)"
trap 'rm -rf "$tmp"' EXIT
sed -E 's/([A-Za-z_][A-Za-z0-9_]*) << <([A-Za-z_][A-Za-z0-9_]*), ([A-Za-z_][A-Za-z0-9_]*) >> > \(/REF_LAUNCH(\2, \3, \1, /' \
  "$src/kernel.cu" > "$tmp/kernel_host.cpp"
if grep -q '<<<\|<< <' "$tmp/kernel_host.cpp"; then
  echo "build_ref: a launch was not rewritten" >&2
  exit 1
fi
g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared -w "-D__declspec(x)=" \
  -I "$here/refshim" -I "$src" \
  "$tmp/kernel_host.cpp" "$src/GradientCalc.cpp" "$here/refshim/ref_launch.cpp" \
  -o "$out/libsrrf_ref_host.so"
echo "build_ref: built $out/libsrrf_ref_host.so"
# The 3B spot-gradient pieces (forward_algorithm.h, spot_with_background.hh,
# storm.h with the vendored TooN and CVD headers) through oracle/refshim/ref3b_harness.cpp.
main="$ref/RFBA Main"
g++ -O2 -std=c++11 -ffp-contract=off -fno-fast-math -fPIC -shared -w \
  -I "$main/include" -I "$main" "$here/refshim/ref3b_harness.cpp" -o "$out/libref3b_host.so"
echo "build_ref: built $out/libref3b_host.so"
# The 3B Gibbs sampler (sampled_multispot.h's GibbsSampler2 with MT19937 from
# mersenne.cpp) and the free-energy loop around it, through
# oracle/refshim/ref3b_gibbs_harness.cpp. image3d.h qualifies Ref3D's members
# redundantly, which g++ accepts with -fpermissive.
g++ -O2 -std=c++11 -fpermissive -ffp-contract=off -fno-fast-math -fPIC -shared -w \
  -I "$main/include" -I "$main" "$here/refshim/ref3b_gibbs_harness.cpp" "$main/mersenne.cpp" \
  -o "$out/libref3b_gibbs_host.so" -lpthread
echo "build_ref: built $out/libref3b_gibbs_host.so"
