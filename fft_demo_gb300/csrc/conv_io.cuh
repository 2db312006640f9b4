// IO policies for the 2D FFT convolution passes (zero padding on load, crop
// on store, real input / real output), for either storage type
// (E = half2: FP16 plans, E = float2: split-precision plans).
//
// Geometry: an "image" is one channel of one input, sy x sx real values; the
// padded transform is P x P (P = 2^k >= the linear-convolution extent).
#pragma once
#include <cuda_fp16.h>

#include "fft_io.cuh"
#include "fft_tile.cuh"

namespace tcfft {

template <class E>
__device__ __forceinline__ E to_elem(float2 v);
template <>
__device__ __forceinline__ half2 to_elem<half2>(float2 v) {
  return __floats2half2_rn(v.x, v.y);
}
template <>
__device__ __forceinline__ float2 to_elem<float2>(float2 v) {
  return v;
}
__device__ __forceinline__ float2 from_elem(half2 h) { return __half22float2(h); }
__device__ __forceinline__ float2 from_elem(float2 f) { return f; }

template <class R>
__device__ __forceinline__ float real_load(const R* p);
template <>
__device__ __forceinline__ float real_load<__half>(const __half* p) {
  return __half2float(__ldg(p));
}
template <>
__device__ __forceinline__ float real_load<float>(const float* p) {
  return __ldg(p);
}
template <class R>
__device__ __forceinline__ R real_from(float v);
template <>
__device__ __forceinline__ __half real_from<__half>(float v) {
  return __float2half_rn(v);
}
template <>
__device__ __forceinline__ float real_from<float>(float v) {
  return v;
}

// four elements of a line: real parts re[], imaginary parts im[]
struct RawRI4 {
  float re[4], im[4];
};

// Forward row pass: line = (image, row < sy); reads sx reals (zero beyond),
// writes P complex values (row `row` of the image's half-spectrum buffer,
// sy rows of P). Optional filter flip (180-degree rotation) for correlation.
// pair = 1: line = (image pair, row): image 2p is the real part and image
// 2p + 1 (zero past the last of n_images) the imaginary part, so one complex
// transform carries two real images.
template <class R, class E>
struct IoRealRowIn {
  static constexpr bool IN_VEC_L = true;
  static constexpr bool OUT_VEC_L = true;
  using Raw = RawRI4;
  const R* in;
  E* out;
  long long total_lines;  // (images or image pairs) * sy
  int sy, sx, P;
  long long in_image_stride;  // elements between images of `in`
  int flip;                   // 1: read w[sy-1-row][sx-1-l] (correlation filters)
  int ld;                     // elements between rows of an image (0: sx)
  int pair;
  long long n_images;
  float scale;
  bool in_contig, out_contig;
  long long contig_len;

  __device__ __forceinline__ void load4(long long img, int row, int l0, float (&v)[4]) const {
    const R* p = in + img * in_image_stride + static_cast<long long>(row) * (ld ? ld : sx);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int l = l0 + q;
      const int col = flip ? sx - 1 - l : l;
      v[q] = (l < sx) ? real_load<R>(p + col) : 0.f;
    }
  }
  __device__ __forceinline__ Raw fetch_l(long long line, int l0, bool ok) const {
    Raw r{{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    if (!ok || line >= total_lines) return r;
    const long long item = line / sy;
    const int row0 = static_cast<int>(line % sy);
    const int row = flip ? sy - 1 - row0 : row0;
    const long long img = pair ? 2 * item : item;
    load4(img, row, l0, r.re);
    if (pair && img + 1 < n_images) load4(img + 1, row, l0, r.im);
    return r;
  }
  __device__ __forceinline__ Raw fetch_g(long long, int, bool) const { return Raw{}; }
  __device__ __forceinline__ void decode_l(const Raw& r, long long, int, float2 (&v)[4]) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = make_float2(r.re[q], r.im[q]);
  }
  __device__ __forceinline__ void decode_g(const Raw&, long long, int, float2 (&v)[4]) const {}
  __device__ __forceinline__ void store_row16(long long line, int j, int J, float2 (&v)[16]) const {
    E* p = out + line * P;
#pragma unroll
    for (int c = 0; c < 16; ++c) p[j + c * J] = to_elem<E>(make_float2(v[c].x * scale, v[c].y * scale));
  }
  __device__ __forceinline__ const half2* tile_src(long long) const { return nullptr; }
  __device__ __forceinline__ half2* tile_dst(long long) const { return nullptr; }
};

// Column pass over a [rows][P] complex buffer per image (lines = the P
// adjacent columns). Rows >= valid_rows read as zero (they were never
// stored). Output rows [r0, r0 + nr) go to out as [nr][P] per image
// (nr = P, r0 = 0 for the full spectrum).
template <class E>
struct IoColMaskCrop {
  static constexpr bool IN_VEC_L = false;
  static constexpr bool OUT_VEC_L = false;
  struct Raw {
    E e[4];
  };
  const E* in;
  E* out;
  long long total_lines;  // images * P
  int P, lps_log2;        // lines per image = P
  int valid_rows;         // rows present in `in` (stride P)
  int r0, nr;             // output row window
  float scale;
  bool in_contig, out_contig;
  long long contig_len;

  __device__ __forceinline__ Raw fetch_g(long long line0, int l, bool ok) const {
    Raw r;
#pragma unroll
    for (int q = 0; q < 4; ++q) r.e[q] = to_elem<E>(make_float2(0.f, 0.f));
    if (!ok || line0 >= total_lines || l >= valid_rows) return r;
    const long long img = line0 >> lps_log2;
    const long long col = line0 & ((1ll << lps_log2) - 1);
    const E* p = in + img * static_cast<long long>(valid_rows) * P + static_cast<long long>(l) * P + col;
    if constexpr (sizeof(E) == 4) {
      const uint4 w = ldg_nc_v4(p);
      r.e[0] = *reinterpret_cast<const E*>(&w.x);
      r.e[1] = *reinterpret_cast<const E*>(&w.y);
      r.e[2] = *reinterpret_cast<const E*>(&w.z);
      r.e[3] = *reinterpret_cast<const E*>(&w.w);
    } else {
      const uint4 w0 = ldg_nc_v4(p), w1 = ldg_nc_v4(p + 2);
      r.e[0] = make_float2(__uint_as_float(w0.x), __uint_as_float(w0.y));
      r.e[1] = make_float2(__uint_as_float(w0.z), __uint_as_float(w0.w));
      r.e[2] = make_float2(__uint_as_float(w1.x), __uint_as_float(w1.y));
      r.e[3] = make_float2(__uint_as_float(w1.z), __uint_as_float(w1.w));
    }
    return r;
  }
  __device__ __forceinline__ Raw fetch_l(long long, int, bool) const { return Raw{}; }
  __device__ __forceinline__ const void* src_g(long long line0, int l, bool& ok) const {
    ok = line0 < total_lines && l < valid_rows;
    if (!ok) return in;
    const long long img = line0 >> lps_log2;
    const long long col = line0 & ((1ll << lps_log2) - 1);
    return in + img * static_cast<long long>(valid_rows) * P + static_cast<long long>(l) * P + col;
  }
  __device__ __forceinline__ void decode_g(const Raw& r, long long, int, float2 (&v)[4]) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = from_elem(r.e[q]);
  }
  __device__ __forceinline__ void decode_l(const Raw&, long long, int, float2 (&)[4]) const {}
  __device__ __forceinline__ void store_row16(long long line, int j, int J, float2 (&v)[16]) const {
    const long long img = line >> lps_log2;
    const long long col = line & ((1ll << lps_log2) - 1);
    E* p = out + img * static_cast<long long>(nr) * P + col;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int row = j + c * J - r0;
      if (row >= 0 && row < nr)
        p[static_cast<long long>(row) * P] = to_elem<E>(make_float2(v[c].x * scale, v[c].y * scale));
    }
  }
  __device__ __forceinline__ const half2* tile_src(long long) const { return nullptr; }
  __device__ __forceinline__ half2* tile_dst(long long) const { return nullptr; }
};

// Inverse row pass: line = (output image, row) over a [rows][P] complex
// buffer; writes the real part of columns [c0, c0 + nc), times scale, to a
// real [rows][nc] output per image. pair = 1: line = (output pair, row); the
// real part goes to output image 2p and the imaginary part to 2p + 1 (when
// 2p + 1 < n_out).
template <class E, class RO>
struct IoRowCropReal {
  static constexpr bool IN_VEC_L = true;
  static constexpr bool OUT_VEC_L = true;
  struct Raw {
    E e[4];
  };
  const E* in;
  RO* out;
  long long total_lines;
  int P, c0, nc;
  int pair, rows;  // rows per output image (pair = 1)
  long long n_out;
  float scale;
  bool in_contig, out_contig;
  long long contig_len;

  __device__ __forceinline__ Raw fetch_l(long long line, int l0, bool ok) const {
    Raw r;
#pragma unroll
    for (int q = 0; q < 4; ++q) r.e[q] = to_elem<E>(make_float2(0.f, 0.f));
    if (!ok || line >= total_lines) return r;
    const E* p = in + line * P + l0;
    if constexpr (sizeof(E) == 4) {
      const uint4 w = ldg_nc_v4(p);
      r.e[0] = *reinterpret_cast<const E*>(&w.x);
      r.e[1] = *reinterpret_cast<const E*>(&w.y);
      r.e[2] = *reinterpret_cast<const E*>(&w.z);
      r.e[3] = *reinterpret_cast<const E*>(&w.w);
    } else {
      const uint4 w0 = ldg_nc_v4(p), w1 = ldg_nc_v4(p + 2);
      r.e[0] = make_float2(__uint_as_float(w0.x), __uint_as_float(w0.y));
      r.e[1] = make_float2(__uint_as_float(w0.z), __uint_as_float(w0.w));
      r.e[2] = make_float2(__uint_as_float(w1.x), __uint_as_float(w1.y));
      r.e[3] = make_float2(__uint_as_float(w1.z), __uint_as_float(w1.w));
    }
    return r;
  }
  __device__ __forceinline__ Raw fetch_g(long long, int, bool) const { return Raw{}; }
  __device__ __forceinline__ void decode_l(const Raw& r, long long, int, float2 (&v)[4]) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = from_elem(r.e[q]);
  }
  __device__ __forceinline__ void decode_g(const Raw&, long long, int, float2 (&)[4]) const {}
  __device__ __forceinline__ void store_row16(long long line, int j, int J, float2 (&v)[16]) const {
    if (pair) {
      const long long o0 = 2 * (line / rows);
      const long long row = line % rows;
      RO* p0 = out + (o0 * rows + row) * nc;
      RO* p1 = o0 + 1 < n_out ? out + ((o0 + 1) * rows + row) * nc : nullptr;
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int col = j + c * J - c0;
        if (col >= 0 && col < nc) {
          p0[col] = real_from<RO>(v[c].x * scale);
          if (p1) p1[col] = real_from<RO>(v[c].y * scale);
        }
      }
      return;
    }
    RO* p = out + line * nc;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int col = j + c * J - c0;
      if (col >= 0 && col < nc) p[col] = real_from<RO>(v[c].x * scale);
    }
  }
  __device__ __forceinline__ const half2* tile_src(long long) const { return nullptr; }
  __device__ __forceinline__ half2* tile_dst(long long) const { return nullptr; }
};

}  // namespace tcfft
