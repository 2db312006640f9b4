// 2D FFT convolution (C ABI): plan, resident filter spectra, execution.
//
// Pipeline per batch of images (P x P padded transform, P = 2^k):
//   1 row pass    real image rows (zero-padded on load) -> half-spectrum rows,
//                 only the sy rows that hold data            (scale 1/P)
//   2 column pass columns, rows >= sy read as zero -> spectrum (scale 1/P)
//   3 pointwise   Y[f] = sum_s X[s] * K[f][s] in FP32 (K resident)
//   4 column pass inverse, only the rows of the output window are stored
//   5 row pass    inverse, real part of the output window's columns
// The two forward scales make the spectra 1/P^2 of the unnormalised DFT, so
// the unnormalised inverse yields the convolution itself and FP16 spectra stay
// in range for image values up to ~1e3.
//
// Reference semantics (tensorcore_fft_conv2d.cpp:12-58, 250-289;
// tensorcore_fft_conv2d_kernel.cu:1034-1150, 1222-1285, 1373-1404):
// conv2d_forward flips each filter 180 degrees, zero-pads image and filter,
// multiplies the spectra, sums over input channels in FP32, inverse-FFTs and
// reads the window at offset (fx-1, fx-1) scaled by 1/P^2: the valid
// cross-correlation, TCFFT_CONV_VALID_CORR here. The reference quantises the
// FP32 product to FP16 with a per-filter power-of-ten scale
// (fft_cpx_point_wise_quant_p1..p3) before its FP16 inverse FFT; this library
// scales the forward transforms by 1/P instead and keeps the product in the
// plan's precision.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/tcfft_gb300.h"
#include "capi_internal.cuh"
#include "conv_kernels.cuh"
#include "qd_internal.cuh"
#include "tables.cuh"

using namespace tcfft;

namespace {

// every entry point records its status (tcfft_get_last_error) and, for an
// exec, its launch count (tcfft_last_launch_count)
tcfftStatus cret(tcfftStatus s, int launches = 0) { return record_status(s, launches); }

ConvTable g_ctab[2];  // [precision]
int g_cocc[2][kNumConvPass][kConvMaxLogP + 1];
std::once_flag g_conv_once;
cudaError_t g_conv_err = cudaSuccess;
int g_conv_sms = 0;

void conv_init() {
  register_conv_f16(g_ctab[0]);
  register_conv_split(g_ctab[1]);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_conv_sms, cudaDevAttrMultiProcessorCount, dev);
  for (int pr = 0; pr < 2 && e == cudaSuccess; ++pr)
    for (int k = 0; k < kNumConvPass && e == cudaSuccess; ++k)
      for (int l = kConvMinLogP; l <= kConvMaxLogP && e == cudaSuccess; ++l) {
        ConvKernel& ck = g_ctab[pr][k][l];
        if (!ck.fn) continue;
        e = cudaFuncSetAttribute(ck.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, ck.smem);
        if (e == cudaSuccess)
          e = cudaFuncSetAttribute(ck.fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared);
        cudaFuncAttributes fa;
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, ck.fn);
        if (e != cudaSuccess) break;
        const int regs_per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
        int occ = 65536 / (regs_per_warp * (kPassThreads / 32));
        const int by_smem = (228 * 1024) / (ck.smem + 1024);
        if (by_smem < occ) occ = by_smem;
        const int tmem = 512 / (ck.Mt / (pr == 0 ? 4 : 2));
        if (tmem < occ) occ = tmem;
        g_cocc[pr][k][l] = occ < 1 ? 1 : occ;
      }
  g_conv_err = e;
}

int ilog2i(long long v) {
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

// Y[b][f][i] = sum_s X[b][s][i] * K[f][s][i]
template <class E>
__global__ void conv_pointwise_kernel(const E* __restrict__ X, const E* __restrict__ K, E* __restrict__ Y,
                                      long long plane, int S, int F, long long total) {
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long i = t % plane;
    const long long bf = t / plane;
    const int f = static_cast<int>(bf % F);
    const long long b = bf / F;
    float2 acc = make_float2(0.f, 0.f);
    for (int s = 0; s < S; ++s) {
      const float2 x = from_elem(X[(b * S + s) * plane + i]);
      const float2 k = from_elem(K[(static_cast<long long>(f) * S + s) * plane + i]);
      acc.x += x.x * k.x - x.y * k.y;
      acc.y += x.x * k.y + x.y * k.x;
    }
    Y[t] = to_elem<E>(acc);
  }
}

// Pointwise stage on paired spectra. Input plane q (of nqp) holds
// Z = X_2q + i X_2q+1, the spectra of two real images (flattened index
// b * S + s); output plane p holds W = Y_2p + i Y_2p+1 for outputs
// o = b * F + f. Since each X is the spectrum of a real image,
// X(k) = conj X(-k), so X_2q = (Z(k) + conj Z(-k)) / 2 and
// X_2q+1 = (Z(k) - conj Z(-k)) / (2i), -k = ((P - ky) mod P, (P - kx) mod P).
// A last unpaired image or output is the plane itself.
template <class E>
__global__ void conv_pointwise_pair_kernel(const E* __restrict__ Zin, const E* __restrict__ K, E* __restrict__ W,
                                           int P, int S, int F, long long n_img, long long n_out) {
  const long long plane = static_cast<long long>(P) * P;
  const long long n_pairs_out = (n_out + 1) / 2;
  const long long total = n_pairs_out * plane;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long i = t % plane;
    const long long po = t / plane;
    const int ky = static_cast<int>(i / P), kx = static_cast<int>(i % P);
    const long long im = static_cast<long long>((P - ky) & (P - 1)) * P + ((P - kx) & (P - 1));
    float2 y[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const long long o = 2 * po + e;
      if (o >= n_out) break;
      const long long b = o / F;
      const int f = static_cast<int>(o % F);
      float2 acc = make_float2(0.f, 0.f);
      for (int sidx = 0; sidx < S; ++sidx) {
        const long long q = b * S + sidx;
        const long long zq = q / 2;
        const float2 z = from_elem(Zin[zq * plane + i]);
        float2 x;
        if (2 * zq + 1 >= n_img) {
          x = z;  // unpaired image
        } else {
          const float2 zm = from_elem(Zin[zq * plane + im]);
          x = (q & 1) ? make_float2(0.5f * (z.y + zm.y), 0.5f * (zm.x - z.x))
                      : make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
        }
        const float2 k = from_elem(K[(static_cast<long long>(f) * S + sidx) * plane + i]);
        acc.x += x.x * k.x - x.y * k.y;
        acc.y += x.x * k.y + x.y * k.x;
      }
      y[e] = acc;
    }
    // W = Y_2p + i Y_2p+1
    W[t] = to_elem<E>(make_float2(y[0].x - y[1].y, y[0].y + y[1].x));
  }
}

}  // namespace

struct tcfftConvImpl {
  int S = 0, F = 0, sy = 0, sx = 0, fy = 0, fx = 0, mode = 0, precision = 0;
  int P = 0, logP = 0;
  int oy = 0, ox = 0, r0 = 0, c0 = 0;
  long long max_batch = 0;
  size_t esz = 4;  // bytes per complex element (4 FP16, 8 split)
  void* K = nullptr;
  void* X = nullptr;
  void* Xf = nullptr;
  void* Y = nullptr;
  void* Z = nullptr;
  float2* tw[2] = {nullptr, nullptr};
  uint16_t* bmat[2] = {nullptr, nullptr};
  int* err = nullptr;
  bool filters_set = false;
  int last_launches = 0;  // launches of the last exec (tcfft_last_launch_count)
};

namespace {

void conv_free(tcfftConvImpl* c) {
  if (!c) return;
  cudaFree(c->K);
  cudaFree(c->X);
  cudaFree(c->Xf);
  cudaFree(c->Y);
  cudaFree(c->Z);
  for (int s = 0; s < 2; ++s) {
    cudaFree(c->tw[s]);
    cudaFree(c->bmat[s]);
  }
  cudaFree(c->err);
  delete c;
}

template <class IO>
tcfftStatus conv_launch(tcfftConvImpl* c, int pass, int sign_idx, const IO& io, cudaStream_t st) {
  const int pr = c->precision == TCFFT_FP16 ? 0 : 1;
  const ConvKernel& k = g_ctab[pr][pass][c->logP];
  if (!k.fn) return TCFFT_UNSUPPORTED;
  PassCore core;
  core.tw = c->tw[sign_idx];
  core.bmat = reinterpret_cast<const uint32_t*>(c->bmat[sign_idx]);
  core.err = c->err;
  const long long ntiles = (io.total_lines + k.G - 1) / k.G;
  long long grid = static_cast<long long>(g_conv_sms) * g_cocc[pr][pass][c->logP];
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) grid = 1;
  void* args[] = {const_cast<IO*>(&io), &core};
  if (cudaLaunchKernel(k.fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), args, static_cast<size_t>(k.smem),
                       st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  return TCFFT_OK;
}

template <class T>
T zero_io() {
  T t;
  std::memset(&t, 0, sizeof(t));
  return t;
}

// Row pass forward on real input rows: `count` images of rows x cols, flip
// for correlation filters.
template <class R, class E>
tcfftStatus conv_row_fwd(tcfftConvImpl* c, int pass, const R* in, E* out, long long count, int rows, int cols,
                         int flip, float scale, cudaStream_t st, bool pair = false) {
  auto io = zero_io<IoRealRowIn<R, E>>();
  io.in = in;
  io.out = out;
  io.pair = pair ? 1 : 0;
  io.n_images = count;
  io.total_lines = (pair ? (count + 1) / 2 : count) * rows;
  io.sy = rows;
  io.sx = cols;
  io.P = c->P;
  io.in_image_stride = static_cast<long long>(rows) * cols;
  io.flip = flip;
  io.scale = scale;
  return conv_launch(c, pass, 0, io, st);
}

template <class E>
tcfftStatus conv_col(tcfftConvImpl* c, int pass, int sign_idx, const E* in, E* out, long long count, int valid_rows,
                     int r0, int nr, float scale, cudaStream_t st) {
  auto io = zero_io<IoColMaskCrop<E>>();
  io.in = in;
  io.out = out;
  io.total_lines = count * c->P;
  io.P = c->P;
  io.lps_log2 = c->logP;
  io.valid_rows = valid_rows;
  io.r0 = r0;
  io.nr = nr;
  io.scale = scale;
  return conv_launch(c, pass, sign_idx, io, st);
}

// count = output images; pair: the input holds (count + 1) / 2 paired planes
template <class E, class RO>
tcfftStatus conv_row_inv(tcfftConvImpl* c, const E* in, RO* out, long long count, float scale, cudaStream_t st,
                         bool pair = false) {
  auto io = zero_io<IoRowCropReal<E, RO>>();
  io.in = in;
  io.out = out;
  io.pair = pair ? 1 : 0;
  io.rows = c->oy;
  io.n_out = count;
  io.total_lines = (pair ? (count + 1) / 2 : count) * c->oy;
  io.P = c->P;
  io.c0 = c->c0;
  io.nc = c->ox;
  io.scale = scale;
  return conv_launch(c, kConvRowInv, 1, io, st);
}

// Fused middle pass (conv_fused.cuh): forward column FFT of the row pass's
// output X (rows past the image zero), product with the one filter spectrum
// K and 1/P, inverse column FFT, output rows [r0, r0 + oy) to Z.
tcfftStatus conv_mid(tcfftConvImpl* c, const half2* X, half2* Z, long long planes, cudaStream_t st) {
  const ConvKernel& k = g_ctab[0][kConvColMid][c->logP];
  if (!k.fn) return TCFFT_UNSUPPORTED;
  auto fio = zero_io<IoConvMidFwd<half2>>();
  fio.in = X;
  fio.total_lines = planes * c->P;
  fio.P = c->P;
  fio.lps_log2 = c->logP;
  fio.valid_rows = c->sy;
  fio.r0 = 0;
  fio.nr = c->P;
  fio.scale = 1.0f / static_cast<float>(c->P);
  fio.K = static_cast<const half2*>(c->K);
  fio.tw_next = c->tw[1];
  auto iio = zero_io<IoColMaskCrop<half2>>();
  iio.out = Z;
  iio.total_lines = planes * c->P;
  iio.P = c->P;
  iio.lps_log2 = c->logP;
  iio.valid_rows = c->P;
  iio.r0 = c->r0;
  iio.nr = c->oy;
  iio.scale = 1.0f;
  PassCore cf, ci;
  cf.tw = c->tw[0];
  cf.bmat = reinterpret_cast<const uint32_t*>(c->bmat[0]);
  cf.err = c->err;
  ci.tw = c->tw[1];
  ci.bmat = reinterpret_cast<const uint32_t*>(c->bmat[1]);
  ci.err = c->err;
  const long long ntiles = (fio.total_lines + k.G - 1) / k.G;
  long long grid = static_cast<long long>(g_conv_sms) * g_cocc[0][kConvColMid][c->logP];
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) grid = 1;
  void* args[] = {&fio, &iio, &cf, &ci};
  if (cudaLaunchKernel(k.fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), args, static_cast<size_t>(k.smem),
                       st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  return TCFFT_OK;
}

template <class E, class RI>
tcfftStatus conv_run(tcfftConvImpl* c, const RI* images, RI* out, long long batch, cudaStream_t st) {
  const float inv_p = 1.0f / static_cast<float>(c->P);
  E* X = static_cast<E*>(c->X);
  E* Xf = static_cast<E*>(c->Xf);
  E* Y = static_cast<E*>(c->Y);
  E* Z = static_cast<E*>(c->Z);
  // Two real images per complex transform (real part, imaginary part) on
  // both sides whenever there are at least two: the forward passes run on
  // ceil(batch*S / 2) planes, the inverse ones on ceil(batch*F / 2).
  const long long n_img = batch * c->S, n_out = batch * c->F;
  const bool pair = n_img > 1 || n_out > 1;
  const long long n_img_planes = pair ? (n_img + 1) / 2 : n_img;
  const long long n_out_planes = pair ? (n_out + 1) / 2 : n_out;
  tcfftStatus s = conv_row_fwd<RI, E>(c, kConvRowFwdImg, images, X, n_img, c->sy, c->sx, 0, inv_p, st, pair);
  if constexpr (sizeof(E) == 4) {
    // one filter: the column passes and the product run as one pass
    // (the paired planes need no separation: Z K = X_a K + i X_b K)
    if (c->S == 1 && c->F == 1 && g_ctab[0][kConvColMid][c->logP].fn) {
      if (s == TCFFT_OK) s = conv_mid(c, X, Z, n_img_planes, st);
      if (s == TCFFT_OK) s = conv_row_inv<E, RI>(c, Z, out, n_out, 1.0f, st, pair);
      c->last_launches = 3;
      return s;
    }
  }
  c->last_launches = 5;
  if (s == TCFFT_OK) s = conv_col<E>(c, kConvColFwd, 0, X, Xf, n_img_planes, c->sy, 0, c->P, inv_p, st);
  if (s == TCFFT_OK) {
    const long long plane = static_cast<long long>(c->P) * c->P;
    if (pair) {
      conv_pointwise_pair_kernel<E><<<static_cast<unsigned>(g_conv_sms * 8), 256, 0, st>>>(
          Xf, static_cast<const E*>(c->K), Y, c->P, c->S, c->F, n_img, n_out);
    } else {
      conv_pointwise_kernel<E><<<static_cast<unsigned>(g_conv_sms * 8), 256, 0, st>>>(
          Xf, static_cast<const E*>(c->K), Y, plane, c->S, c->F, n_out * plane);
    }
    if (cudaGetLastError() != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
  }
  if (s == TCFFT_OK) s = conv_col<E>(c, kConvColInv, 1, Y, Z, n_out_planes, c->P, c->r0, c->oy, 1.0f, st);
  if (s == TCFFT_OK) s = conv_row_inv<E, RI>(c, Z, out, n_out, 1.0f, st, pair);
  return s;
}

}  // namespace

extern "C" {

tcfftStatus tcfft_conv2d_plan(tcfftConv* conv, int S, int F, int sy, int sx, int fy, int fx, int mode,
                              int precision, long long max_batch) {
  if (!conv) return cret(TCFFT_INVALID_VALUE);
  *conv = nullptr;
  if (S < 1 || F < 1 || sy < 1 || sx < 1 || fy < 1 || fx < 1 || max_batch < 1) return cret(TCFFT_INVALID_SIZE);
  if (precision != TCFFT_FP16 && precision != TCFFT_SPLIT_FP32) return cret(TCFFT_INVALID_VALUE);
  if (mode != TCFFT_CONV_VALID_CORR && mode != TCFFT_CONV_SAME && mode != TCFFT_CONV_FULL)
    return cret(TCFFT_INVALID_VALUE);
  if (mode == TCFFT_CONV_VALID_CORR && (fy > sy || fx > sx)) return cret(TCFFT_INVALID_SIZE);
  if (mode == TCFFT_CONV_SAME && ((fy % 2) == 0 || (fx % 2) == 0)) return cret(TCFFT_INVALID_SIZE);
  std::call_once(g_conv_once, conv_init);
  if (g_conv_err != cudaSuccess) return cret(TCFFT_NO_DEVICE);
  tcfftConvImpl* c = new (std::nothrow) tcfftConvImpl();
  if (!c) return cret(TCFFT_ALLOC_FAILED);
  c->S = S;
  c->F = F;
  c->sy = sy;
  c->sx = sx;
  c->fy = fy;
  c->fx = fx;
  c->mode = mode;
  c->precision = precision;
  c->max_batch = max_batch;
  c->esz = precision == TCFFT_FP16 ? 4 : 8;
  // Smallest power of two free of wrap-around inside the output window.
  long long need = 0;
  if (mode == TCFFT_CONV_VALID_CORR) {
    need = sy > sx ? sy : sx;
    c->oy = sy - fy + 1;
    c->ox = sx - fx + 1;
    c->r0 = fy - 1;
    c->c0 = fx - 1;
  } else if (mode == TCFFT_CONV_SAME) {
    const long long ny = sy + (fy - 1) / 2, nx = sx + (fx - 1) / 2;
    need = ny > nx ? ny : nx;
    c->oy = sy;
    c->ox = sx;
    c->r0 = (fy - 1) / 2;
    c->c0 = (fx - 1) / 2;
  } else {
    const long long ny = sy + fy - 1, nx = sx + fx - 1;
    need = ny > nx ? ny : nx;
    c->oy = sy + fy - 1;
    c->ox = sx + fx - 1;
    c->r0 = 0;
    c->c0 = 0;
  }
  if (need < (1 << kConvMinLogP)) need = 1 << kConvMinLogP;
  c->logP = ilog2i(need);
  c->P = 1 << c->logP;
  const int max_log = precision == TCFFT_FP16 ? kConvMaxLogP : kConvMaxLogP - 1;
  if (c->logP > max_log) {
    conv_free(c);
    return cret(TCFFT_INVALID_SIZE);
  }
  const size_t plane = static_cast<size_t>(c->P) * c->P;
  tcfftStatus s = TCFFT_OK;
  auto alloc = [&](void** p, size_t bytes) {
    if (s == TCFFT_OK && cudaMalloc(p, bytes) != cudaSuccess) s = TCFFT_ALLOC_FAILED;
  };
  const size_t filt_rows = static_cast<size_t>(F) * S * fy * c->P;
  const size_t img_rows = static_cast<size_t>(max_batch) * S * sy * c->P;
  alloc(&c->K, static_cast<size_t>(F) * S * plane * c->esz);
  alloc(&c->X, (img_rows > filt_rows ? img_rows : filt_rows) * c->esz);
  alloc(&c->Xf, static_cast<size_t>(max_batch) * S * plane * c->esz);
  alloc(&c->Y, static_cast<size_t>(max_batch) * F * plane * c->esz);
  alloc(&c->Z, static_cast<size_t>(max_batch) * F * c->oy * c->P * c->esz);
  for (int d = 0; d < 2; ++d) {
    alloc(reinterpret_cast<void**>(&c->tw[d]), sizeof(float2) * c->P);
    alloc(reinterpret_cast<void**>(&c->bmat[d]), 4096);
    if (s == TCFFT_OK && (gen_twiddles(c->tw[d], c->P, c->logP, 0, d == 0 ? -1 : 1, 0) != cudaSuccess ||
                          gen_dft16_bmat(c->bmat[d], d == 0 ? -1 : 1, 0, 0) != cudaSuccess ||
                          gen_dft16_bmat(c->bmat[d] + 1024, d == 0 ? -1 : 1, 1, 0) != cudaSuccess))
      s = TCFFT_LAUNCH_FAILED;
  }
  alloc(reinterpret_cast<void**>(&c->err), sizeof(int));
  if (s == TCFFT_OK && cudaMemset(c->err, 0, sizeof(int)) != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
  if (s == TCFFT_OK && cudaDeviceSynchronize() != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
  if (s != TCFFT_OK) {
    conv_free(c);
    return cret(s);
  }
  *conv = c;
  return cret(TCFFT_OK);
}

tcfftStatus tcfft_conv2d_set_filters(tcfftConv c, const float* filters, void* stream) {
  if (!c || !filters) return cret(TCFFT_INVALID_VALUE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int flip = c->mode == TCFFT_CONV_VALID_CORR ? 1 : 0;
  const long long count = static_cast<long long>(c->F) * c->S;
  tcfftStatus s;
  if (c->precision == TCFFT_FP16) {
    s = conv_row_fwd<float, half2>(c, kConvRowFwdFilt, filters, static_cast<half2*>(c->X), count, c->fy, c->fx, flip,
                                   1.0f, st);
    if (s == TCFFT_OK)
      s = conv_col<half2>(c, kConvColFwd, 0, static_cast<half2*>(c->X), static_cast<half2*>(c->K), count, c->fy, 0,
                          c->P, 1.0f, st);
  } else {
    s = conv_row_fwd<float, float2>(c, kConvRowFwdFilt, filters, static_cast<float2*>(c->X), count, c->fy, c->fx,
                                    flip, 1.0f, st);
    if (s == TCFFT_OK)
      s = conv_col<float2>(c, kConvColFwd, 0, static_cast<float2*>(c->X), static_cast<float2*>(c->K), count, c->fy,
                           0, c->P, 1.0f, st);
  }
  if (s == TCFFT_OK) c->filters_set = true;
  return cret(s);
}

tcfftStatus tcfft_conv2d_set_filters_qd(tcfftConv c, const float* filters, void* stream) {
  if (!c || !filters) return cret(TCFFT_INVALID_VALUE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int flip = c->mode == TCFFT_CONV_VALID_CORR ? 1 : 0;
  const long long count = static_cast<long long>(c->F) * c->S;
  tcfftQdImpl* q = nullptr;
  tcfftStatus s = qd_create(&q, c->P, (count + 1) / 2, c->fy, c->fx);
  if (s == TCFFT_OK) {
    // same spectra as the masked passes: forward sign, unnormalised
    if (c->precision == TCFFT_FP16)
      s = qd_exec_filter_pairs<half2>(q, filters, count, flip, static_cast<half2*>(c->K), TCFFT_FORWARD, st);
    else
      s = qd_exec_filter_pairs<float2>(q, filters, count, flip, static_cast<float2*>(c->K), TCFFT_FORWARD, st);
    // the projections are freed below: finish with them first (and report
    // a flagged error of their transforms)
    const tcfftStatus w = qd_check(q, st);
    if (s == TCFFT_OK) s = w;
  }
  qd_free(q);
  if (s == TCFFT_OK) c->filters_set = true;
  return cret(s);
}

tcfftStatus tcfft_conv2d_exec(tcfftConv c, const void* images, void* out, long long batch, void* stream) {
  if (!c || !images || !out) return cret(TCFFT_INVALID_VALUE);
  if (batch < 1 || batch > c->max_batch) return cret(TCFFT_CAPACITY);
  if (!c->filters_set) return cret(TCFFT_INVALID_VALUE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  tcfftStatus s;
  if (c->precision == TCFFT_FP16)
    s = conv_run<half2, __half>(c, static_cast<const __half*>(images), static_cast<__half*>(out), batch, st);
  else
    s = conv_run<float2, float>(c, static_cast<const float*>(images), static_cast<float*>(out), batch, st);
  return cret(s, s == TCFFT_OK ? c->last_launches : 0);
}

tcfftStatus tcfft_conv2d_shape(tcfftConv c, int* out_rows, int* out_cols, int* padded) {
  if (!c) return cret(TCFFT_INVALID_VALUE);
  if (out_rows) *out_rows = c->oy;
  if (out_cols) *out_cols = c->ox;
  if (padded) *padded = c->P;
  return cret(TCFFT_OK);
}

tcfftStatus tcfft_conv2d_check(tcfftConv c, void* stream) {
  if (!c) return cret(TCFFT_INVALID_VALUE);
  if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess) return cret(TCFFT_LAUNCH_FAILED);
  int h = 0;
  if (cudaMemcpy(&h, c->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return cret(TCFFT_LAUNCH_FAILED);
  if (h) {
    cudaMemset(c->err, 0, sizeof(int));
    return cret(TCFFT_TIMEOUT);
  }
  return cret(TCFFT_OK);
}

tcfftStatus tcfft_conv2d_destroy(tcfftConv c) {
  if (!c) return cret(TCFFT_INVALID_VALUE);
  conv_free(c);
  return cret(TCFFT_OK);
}

}  // extern "C"
