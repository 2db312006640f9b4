#!/usr/bin/env bash
# Builds pieces of the reference (yuelingfan/fft_demo) from its own sources,
# where they lie, into oracle/_ref/. Used only to pin the oracle's
# restatements on this machine (the sources are absent on GPU hosts):
#   libref_tcfft1d.so  <- tcfft_half.cu     (gen_rev, tcfftCreate host logic)
#   libref_tcfft2d.so  <- tcfft_half_2d.cu  (gen_rev_2d)
#   ref_tcfft1d.cubin  <- oracle/ref_kernels_1d.cu (#includes tcfft_half.cu):
#                         the reference's 1D stage kernels, device code only
#   ref_tcfft2d.cubin  <- oracle/ref_kernels_2d.cu (#includes tcfft_half_2d.cu)
#   ref_conv.cubin     <- oracle/ref_kernels_conv.cu (#includes
#                         tensorcore_fft_conv2d_kernel.cu): the convolution's
#                         stage, pointwise and quantisation kernels
# The cubins hold no host code, so they run on any host with the same GPU
# (oracle/ref_launch.py loads them through the CUDA driver API).
# The two files define clashing kernel templates, so they become separate
# libraries. Nothing here is copied; nvcc reads the reference tree read-only.
# Usage: oracle/ref_build.sh [REFERENCE_DIR]   (or FFT_DEMO_REF=REFERENCE_DIR);
# without either it builds nothing.
set -euo pipefail
REF=${1:-${FFT_DEMO_REF:-}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$REF/tcfft_half.cu" ]; then
  echo "reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
NVFLAGS="-std=c++17 -O1 -shared -Xcompiler -fPIC -gencode arch=compute_103a,code=sm_103a -I$REF -I$REF/include"
nvcc $NVFLAGS "$REF/tcfft_half.cu" -o "$OUT/libref_tcfft1d.so" -lcudart &
nvcc $NVFLAGS "$REF/tcfft_half_2d.cu" -o "$OUT/libref_tcfft2d.so" -lcudart &
CUBIN="-cubin -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -I$REF -I$REF/include"
nvcc $CUBIN "$HERE/ref_kernels_1d.cu" -o "$OUT/ref_tcfft1d.cubin" &
nvcc $CUBIN "$HERE/ref_kernels_2d.cu" -o "$OUT/ref_tcfft2d.cubin" &
nvcc $CUBIN "$HERE/ref_kernels_conv.cu" -o "$OUT/ref_conv.cubin" &
wait
echo "built: $(ls "$OUT")"
