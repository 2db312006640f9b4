// Kernel table for the convolution passes (instantiated in conv_k_*.cu).
#pragma once
#include <cuda_runtime.h>

#include "conv_fused.cuh"
#include "conv_io.cuh"
#include "fft_split.cuh"
#include "fft_tile.cuh"

namespace tcfft {

constexpr int kConvMinLogP = 6;   // P >= 64
constexpr int kConvMaxLogP = 12;  // P <= 4096

// Which pass of the convolution pipeline.
enum ConvPassSel : int {
  kConvRowFwdImg = 0,   // real image rows (plan's real type) -> half-spectrum rows
  kConvRowFwdFilt = 1,  // real FP32 filter rows (optionally flipped) -> rows
  kConvColFwd = 2,      // columns, zero rows masked -> full spectrum
  kConvColInv = 3,      // columns inverse, crop rows
  kConvRowInv = 4,      // rows inverse, crop columns, real part out
  kConvColMid = 5,      // columns forward, times the filter spectrum, inverse, crop rows (one filter)
  kNumConvPass = 6
};

struct ConvKernel {
  const void* fn = nullptr;
  int smem = 0;
  int G = 0;
  int Mt = 0;
};

using ConvTable = ConvKernel[kNumConvPass][kConvMaxLogP + 1];

void register_conv_f16(ConvTable& t);
void register_conv_split(ConvTable& t);

template <int P, int Mt, bool LINE_MINOR, int SIGN, class IO>
ConvKernel conv_entry_f16() {
  constexpr int G = Mt * 16 / P;
  ConvKernel k;
  k.fn = reinterpret_cast<const void*>(&fft_pass_f16<P, G, LINE_MINOR, SIGN, IO>);
  k.smem = pass_smem_bytes<P, G>();
  k.G = G;
  k.Mt = Mt;
  return k;
}

template <int P, int Mt, bool LINE_MINOR, int SIGN, class IO>
ConvKernel conv_entry_split() {
  constexpr int G = Mt * 16 / P;
  ConvKernel k;
  k.fn = reinterpret_cast<const void*>(&fft_pass_split<P, G, LINE_MINOR, SIGN, IO>);
  k.smem = split_smem_bytes<P, G>();
  k.G = G;
  k.Mt = Mt;
  return k;
}

template <int P, int Mt>
ConvKernel conv_entry_mid_f16() {
  constexpr int G = Mt * 16 / P;
  ConvKernel k;
  k.fn = reinterpret_cast<const void*>(&conv_mid_f16<P, G, half2>);
  k.smem = mid_smem_bytes<P, G>();
  k.G = G;
  k.Mt = Mt;
  return k;
}

template <int P>
void conv_fill_f16(ConvTable& t) {
  constexpr int LOG = ilog2c(P);
  t[kConvColMid][LOG] = conv_entry_mid_f16<P, 1024>();
  t[kConvRowFwdImg][LOG] = conv_entry_f16<P, 1024, false, -1, IoRealRowIn<__half, half2>>();
  t[kConvRowFwdFilt][LOG] = conv_entry_f16<P, 1024, false, -1, IoRealRowIn<float, half2>>();
  t[kConvColFwd][LOG] = conv_entry_f16<P, 1024, true, -1, IoColMaskCrop<half2>>();
  t[kConvColInv][LOG] = conv_entry_f16<P, 1024, true, +1, IoColMaskCrop<half2>>();
  t[kConvRowInv][LOG] = conv_entry_f16<P, 1024, false, +1, IoRowCropReal<half2, __half>>();
}

template <int P>
void conv_fill_split(ConvTable& t) {
  constexpr int LOG = ilog2c(P);
  t[kConvRowFwdImg][LOG] = conv_entry_split<P, 512, false, -1, IoRealRowIn<float, float2>>();
  t[kConvRowFwdFilt][LOG] = t[kConvRowFwdImg][LOG];
  t[kConvColFwd][LOG] = conv_entry_split<P, 512, true, -1, IoColMaskCrop<float2>>();
  t[kConvColInv][LOG] = conv_entry_split<P, 512, true, +1, IoColMaskCrop<float2>>();
  t[kConvRowInv][LOG] = conv_entry_split<P, 512, false, +1, IoRowCropReal<float2, float>>();
}

}  // namespace tcfft
