#!/usr/bin/env bash
# Builds the reference's own CPU B-spline fitter from its sources where they lie
# (read-only) into oracle/_ref/, as the checker for the oracle restatement:
#   oracle/_ref/libref_f32.so  FP32, as shipped
#   oracle/_ref/libref_f64.so  the same sources with float promoted to double
#   oracle/_ref/libref_maxfind.so  the peak finder MultiD_fitter/shared/maximumfind2.c
#   oracle/_ref/ref_emccd.ptx  the reference's CUDA fitter kernels (PTX, sm_103a)
# Only the three fitter sources are compiled (not erf.cpp, which the reference's
# own project does not build, nor the mex driver, which needs MATLAB).
# -fno-stack-protector: the 8-parameter solver kernel_luEvaluate5D declares
# `float y[7]` and writes y[7] (CPUsplineLib.cpp:17-27); without the flag the
# canary check aborts. The stray element lands in the array's alignment padding.
# Usage: oracle/build_ref.sh <reference root>
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
if [ $# -lt 1 ]; then
  echo "usage: $0 <reference project root>" >&2
  exit 2
fi
REF="$1"
SRC="$REF/MultiD_bspline/visual code/CPUmleFit_LM"
OUT="$HERE/_ref"
if [ ! -f "$SRC/CPUmleFit_LM.cpp" ]; then
  echo "reference sources not found under $SRC; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-O2 -fPIC -ffp-contract=off -fno-stack-protector -w -I "$HERE/ref_shim" -I "$SRC" -include "$HERE/ref_shim/prelude.h")
for variant in f32 f64; do
  extra=()
  if [ "$variant" = f64 ]; then extra=(-DBSFIT_REF_PROMOTE_DOUBLE); fi
  objs=()
  for f in CPUmleFit_LM.cpp CPUsplineLib.cpp CPUgaussLib.cpp; do
    o="$OUT/${f%.cpp}_$variant.o"
    "$CXX" "${FLAGS[@]}" "${extra[@]}" -c "$SRC/$f" -o "$o" &
    objs+=("$o")
  done
  o="$OUT/ref_entry_$variant.o"
  "$CXX" "${FLAGS[@]}" "${extra[@]}" -c "$HERE/ref_shim/ref_entry.cpp" -o "$o" &
  objs+=("$o")
  wait
  "$CXX" -shared -Wl,--no-undefined -o "$OUT/libref_$variant.so" "${objs[@]}" -lm
  rm -f "${objs[@]}"
done
# The reference's peak finder (non-maximum suppression of the frame front end),
# compiled as C with a mex.h stand-in; only its NMS function is called.
PEAK="$REF/MultiD_fitter/shared/maximumfind2.c"
if [ -f "$PEAK" ]; then
  CC="${CC:-gcc}"
  "$CC" -O2 -fPIC -w -I "$HERE/ref_shim_mex" -c "$PEAK" -o "$OUT/maximumfind2.o"
  "$CC" -O2 -fPIC -w -I "$HERE/ref_shim_mex" -c "$HERE/ref_shim_mex/mex_stubs.c" -o "$OUT/mex_stubs.o"
  "$CC" -shared -Wl,--no-undefined -o "$OUT/libref_maxfind.so" "$OUT/maximumfind2.o" "$OUT/mex_stubs.o"
  rm -f "$OUT/maximumfind2.o" "$OUT/mex_stubs.o"
fi
# The reference's own CUDA kernels (VC/GPUmleFit_LM/GPUmleFit_LM_EMCCD.cu with
# the headers of VC/Lib), compiled as the reference's project does (one
# translation unit) but to PTX for compute_103a, loaded through the driver API
# by oracle/ref_gpu.py: the reference GPU kernel timed on the same device.
GPU="$REF/MultiD_bspline/visual code/GPUmleFit_LM"
if [ -f "$GPU/GPUmleFit_LM_EMCCD.cu" ] && command -v "${NVCC:-nvcc}" > /dev/null; then
  "${NVCC:-nvcc}" -arch=compute_103a -ptx -O3 -w -I "$HERE/ref_shim_mex" \
    -I "$REF/MultiD_bspline/visual code/Lib" -I "$GPU" "$GPU/GPUmleFit_LM_EMCCD.cu" \
    -o "$OUT/ref_emccd.ptx"
fi
echo "built $OUT/libref_f32.so $OUT/libref_f64.so $OUT/libref_maxfind.so $OUT/ref_emccd.ptx"
