// Fused middle pass of the FFT convolution with one filter (S = F = 1): per
// tile of G adjacent columns of a padded P x P plane, the forward column FFT
// (rows past the image read as zero), the product with the filter spectrum,
// and the inverse column FFT, storing only the rows of the output window.
// The forward transform's last stage multiplies by the spectrum and writes
// the product back into the planes in the natural order the inverse's first
// stage reads, so the spectrum never goes to HBM: the pipeline is row pass,
// this pass, row pass -- three launches instead of five (column forward,
// pointwise, column inverse).
//
// Two real images share each complex plane when the batch has more than one
// (Z = X_a + i X_b): since the spectrum K is that of a real filter,
// Z K = X_a K + i X_b K, so the product needs no separation of the pair.
//
// Method kept from the reference (tensorcore_fft_conv2d.cpp:250-289,
// tensorcore_fft_conv2d_kernel.cu:1101-1150): pad, forward FFT, pointwise
// product with the pre-transformed filter, inverse FFT, crop; the stage
// boundaries are fused here. For P = 16^k (256, 4096) the inverse starts with
// a radix-16 stage and the hand-off writes the products as they are; other
// lengths start the inverse with a radix-T stage (T = 2, 4, 8), whose
// butterflies take inputs that one thread already holds, so the hand-off runs
// that stage and its twiddle in registers (stage_epilogue).
#pragma once
#include "conv_io.cuh"
#include "fft_tile.cuh"

namespace tcfft {

// Forward half: loads like IoColMaskCrop; its last stage hands off on chip.
template <class E>
struct IoConvMidFwd : IoColMaskCrop<E> {
  static constexpr bool TO_PLANES = true;
  static constexpr int NEXT_SIGN = +1;  // the transform that follows on chip: inverse
  const E* K;  // [P][P] filter spectrum (row ky, column kx), forward, unscaled
  const float2* tw_next;  // W_P^e of the inverse direction (its radix-T stage's twiddles)
  // v[c] = X[ky = j + c J][kx] * K[ky][kx] * scale, kx = the line's column
  __device__ __forceinline__ void product16(long long line, int j, int J, float2 (&v)[16]) const {
    const int P = this->P;
    const long long col = line & ((1ll << this->lps_log2) - 1);
    const E* k = K + static_cast<long long>(j) * P + col;
    const float s = this->scale;
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
      const float2 k0 = from_elem(__ldg(k + static_cast<long long>(c) * J * P));
      const float2 k1 = from_elem(__ldg(k + static_cast<long long>(c + 1) * J * P));
      // two products per packed instruction, then the scale
      const TwPair w = twpair(k0, k1);
      float2 yr, yi;
      cmul_pair(make_float2(v[c].x, v[c + 1].x), make_float2(v[c].y, v[c + 1].y), w, yr, yi);
      yr = f2mul(yr, f2bcast(s));
      yi = f2mul(yi, f2bcast(s));
      v[c] = make_float2(yr.x, yi.x);
      v[c + 1] = make_float2(yr.y, yi.y);
    }
  }
};

// Shared memory: [0, 2 KiB) forward DFT16 B image, [2, 4 KiB) inverse image,
// [4 KiB, +64 B) mbarriers and the TMEM address slot, planes from 5 KiB.
constexpr uint32_t kMidPlaneOffset = 5120;

template <uint32_t TMEM_COLS>
__device__ __forceinline__ void mid_setup(PassState& st, const uint32_t* __restrict__ bfwd,
                                          const uint32_t* __restrict__ binv) {
  st.smem = aligned_dynamic_smem();
  st.bmat = st.smem;
  st.mbar = reinterpret_cast<uint64_t*>(st.smem + 4096);
  st.tma_bar = reinterpret_cast<uint64_t*>(st.smem + 4104);
  st.tslot = reinterpret_cast<uint32_t*>(st.smem + 4112);
  const int tid = threadIdx.x;
  uint32_t* b = reinterpret_cast<uint32_t*>(st.smem);
  for (int i = tid; i < 512; i += blockDim.x) {
    b[i] = __ldg(bfwd + i);
    b[512 + i] = __ldg(binv + i);
  }
  if (tid == 0) {
    mbar_init(st.mbar, 1);
    mbar_init(st.tma_bar, 1);
  }
  if ((tid >> 5) == 0) {
    tmem_alloc(st.tslot, TMEM_COLS);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  st.tbase = *st.tslot;
  st.phase = 0;
  st.tma_phase = 0;
}

template <int P, int G, class E>
__global__ void __launch_bounds__(kPassThreads, 2)
    conv_mid_f16(const IoConvMidFwd<E> fio, const IoColMaskCrop<E> iio, const PassCore cf, const PassCore ci) {
  using Tl = Tile<P, G, true>;
  constexpr uint32_t TMEM_COLS = pass_tmem_cols<P, G>();
  PassState st;
  mid_setup<TMEM_COLS>(st, cf.bmat, ci.bmat);
  uint8_t* re = st.smem + kMidPlaneOffset;
  uint8_t* im = re + Tl::PLANE;
  const long long ntiles = (fio.total_lines + G - 1) / G;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long line0 = tile * G;
    st.bmat = st.smem;
    if (!tile_load<P, G, true, -1, IoConvMidFwd<E>>(st, fio, cf, line0, re, im)) break;
    if (!run_stages<P, G, true, -1, IoConvMidFwd<E>>(st, fio, cf, line0, re, im, false)) break;
    st.bmat = st.smem + 2048;
    if (!run_stages<P, G, true, +1, IoColMaskCrop<E>>(st, iio, ci, line0, re, im, false)) break;
  }
  pass_teardown<TMEM_COLS>(st);
}

template <int P, int G>
constexpr int mid_smem_bytes() {
  return static_cast<int>(kMidPlaneOffset) + 2 * (G * P / 16) * 32 + 1024;
}

}  // namespace tcfft
