// Tensor-core FFT "pass" kernel for sm_103a.
//
// A pass transforms many independent lines of length L (power of two,
// 16 <= L <= 16384) that live in global memory with arbitrary
// (sequence, line, element) strides. One CTA owns a tile of G lines in shared
// memory and runs the whole length-L transform on it:
//
//   load   : global -> registers -> shared, 8 x 16-byte loads in flight per
//            thread. A radix-T first stage (T = L / 16^S in {1,2,4,8}) runs
//            here on the CUDA cores in FP32, followed by the twiddle of the
//            first radix-16 stage.
//   stages : S radix-16 stages (unrolled at compile time). Each is one batch
//            of tcgen05 MMAs D[m][n] = sum_k A[m][k] B[k][n] with
//              A = the tile in MN-major 128B-swizzled layout: K row r (0..15)
//                  holds input r of every butterfly m; real and imaginary
//                  parts are separate planes (two K=16 MMAs),
//              B = the 16-point DFT as a 32x32 real matrix (FP16),
//              D = FP32 accumulator in TMEM: lane m, 16 real + 16 imaginary
//                  outputs.
//            The epilogue reads D (tcgen05.ld), applies the next stage's
//            twiddle in FP32, rounds once to FP16 and scatters into the next
//            stage's positions (Stockham autosort order).
//   store  : shared -> global in natural order through the IO policy (outer
//            four-step twiddle, scale, crop, pointwise product ...).
//
// Method (radix-16 DFT stages on tensor cores, twiddles between stages,
// radix-2/4/8 tail on CUDA cores) follows tcfft_half.cu:70-1175 of
// yuelingfan/fft_demo; the data layout, autosort order, FP32 accumulation and
// TMEM staging are this library's own.
#pragma once
#include <cuda_fp16.h>
#include <cstdint>
#include <utility>

#include "tc_ptx.cuh"

namespace tcfft {

constexpr int kPassThreads = 256;

__device__ __forceinline__ void unpack_h2x4(const uint4& r, float2 (&v)[4]) {
  v[0] = __half22float2(*reinterpret_cast<const __half2*>(&r.x));
  v[1] = __half22float2(*reinterpret_cast<const __half2*>(&r.y));
  v[2] = __half22float2(*reinterpret_cast<const __half2*>(&r.z));
  v[3] = __half22float2(*reinterpret_cast<const __half2*>(&r.w));
}

// Error word bits set by kernels (read back by the host after a launch).
enum : int { kErrMmaTimeout = 1, kErrBadArgs = 2, kErrQueueTimeout = 4 };

__host__ __device__ constexpr int ilog2c(long long x) { return x <= 1 ? 0 : 1 + ilog2c(x / 2); }

template <int L>
struct LineShape {
  static constexpr int LOG = ilog2c(L);
  static constexpr int T = 1 << (LOG % 4);  // tail radix done in the loader
  static constexpr int S = LOG / 4;         // radix-16 tensor-core stages
  static constexpr int J = L / 16;          // butterflies per line per radix-16 stage
  static_assert((1 << LOG) == L, "L must be a power of two");
  static_assert(L >= 16, "L >= 16");
};

// Per-pass constants shared by every IO policy.
struct PassCore {
  const float2* tw;      // W_L^e (this direction), e in [0, L)
  const uint32_t* bmat;  // 2 KB image of B for this direction
  int* err;
};

// IO policies that can move column-layout tiles by TMA tensor maps.
template <class IO>
concept TensorMapIo = requires(const IO& io) {
  io.in_tma;
  io.out_tma;
  io.in_map;
  io.out_map;
};

// IO policies whose last stage stays on chip: the outputs, after the
// policy's product16 (e.g. a pointwise product), are written back into the
// planes in natural order -- element j + c*J of line g at K row c, column
// pos(g, j) -- which is exactly the input layout of a following transform of
// the same tile whose length is a power of 16 (no radix-T stage).
template <class IO>
concept PlanesOutIo = requires { IO::TO_PLANES; };

// Complex product with a fixed rounding sequence (one product rounded, then
// one fused multiply-add per component), so every kernel that forms the same
// product gets the same bits whatever the compiler would contract.
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)), __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}

// Packed FP32 pairs: one sm_100-family instruction does the same operation on
// two lanes of work (a float2 held in an aligned register pair), so complex
// arithmetic over two outputs at a time costs half the issue slots.
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2bcast(float v) { return make_float2(v, v); }

// Twiddles of two outputs as pairs of components: re = (w0.x, w1.x),
// im = (w0.y, w1.y), and nim = -im (kept so that no product needs a negation).
struct TwPair {
  float2 re, im, nim;
};
__device__ __forceinline__ TwPair twpair(float2 w0, float2 w1) {
  return TwPair{make_float2(w0.x, w1.x), make_float2(w0.y, w1.y), make_float2(-w0.y, -w1.y)};
}
// Multiplies both twiddles by the complex scalar s, given as broadcast pairs
// sr = (s.x, s.x), si = (s.y, s.y), nsi = -si.
__device__ __forceinline__ void twpair_step(TwPair& w, float2 sr, float2 si, float2 nsi) {
  const float2 re = f2fma(w.im, nsi, f2mul(w.re, sr));
  const float2 im = f2fma(w.im, sr, f2mul(w.re, si));
  const float2 nim = f2fma(w.nim, sr, f2mul(w.re, nsi));
  w.re = re;
  w.im = im;
  w.nim = nim;
}
// (yr, yi) = (xr + i xi) * w for two outputs: xr = (x0.x, x1.x), xi = (x0.y, x1.y).
__device__ __forceinline__ void cmul_pair(float2 xr, float2 xi, const TwPair& w, float2& yr, float2& yi) {
  yr = f2fma(xi, w.nim, f2mul(xr, w.re));
  yi = f2fma(xi, w.re, f2mul(xr, w.im));
}
// Twiddle recurrence over 16 outputs c = 0..15 as 8 pairs (c, c + 1):
// W^(e0 + c de) from w = W^e0 and step = W^de; pair k+1 = pair k * step^2.
struct TwPairSeq {
  TwPair w;
  float2 sr, si, nsi;
  __device__ __forceinline__ TwPairSeq(float2 w0, float2 step) {
    w = twpair(w0, cmulf(w0, step));
    const float2 s2 = cmulf(step, step);
    sr = f2bcast(s2.x);
    si = f2bcast(s2.y);
    nsi = f2bcast(-s2.y);
  }
  __device__ __forceinline__ void next() { twpair_step(w, sr, si, nsi); }
};

// In-register radix-T DFT (T in {1,2,4,8}), SIGN = -1 forward, +1 inverse.
template <int T, int SIGN>
__device__ __forceinline__ void small_dft(float2 (&v)[T]) {
  if constexpr (T == 1) {
    return;
  } else if constexpr (T == 2) {
    float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
  } else if constexpr (T == 4) {
    float2 s02 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
    float2 d02 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
    float2 s13 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
    float2 d13 = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
    // SIGN * i * d13
    float2 rd13 = SIGN < 0 ? make_float2(d13.y, -d13.x) : make_float2(-d13.y, d13.x);
    v[0] = make_float2(s02.x + s13.x, s02.y + s13.y);
    v[2] = make_float2(s02.x - s13.x, s02.y - s13.y);
    v[1] = make_float2(d02.x + rd13.x, d02.y + rd13.y);
    v[3] = make_float2(d02.x - rd13.x, d02.y - rd13.y);
  } else {
    static_assert(T == 8, "tail radix");
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    small_dft<4, SIGN>(e);
    small_dft<4, SIGN>(o);
    const float h = 0.70710678118654752f;
    const float2 w[4] = {make_float2(1.f, 0.f), make_float2(h, SIGN * h), make_float2(0.f, SIGN * 1.f),
                         make_float2(-h, SIGN * h)};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float2 t = cmulf(o[c], w[c]);
      v[c] = make_float2(e[c].x + t.x, e[c].y + t.y);
      v[c + 4] = make_float2(e[c].x - t.x, e[c].y - t.y);
    }
  }
}

// ---------------------------------------------------------------------------
// Tile geometry (compile time).
// ---------------------------------------------------------------------------
template <int L, int G, bool LINE_MINOR>
struct Tile {
  static constexpr int J = LineShape<L>::J;
  static constexpr int Mt = G * L / 16;
  static constexpr uint32_t PLANE = Mt * 32;
  static constexpr uint32_t KSTRIDE = (Mt / 64) * 1024;
  // column m of butterfly j of line g
  __device__ __forceinline__ static int pos(int g, int j) { return LINE_MINOR ? j * G + g : g * J + j; }
  __device__ __forceinline__ static void unpos(int m, int& g, int& j) {
    if (LINE_MINOR) {
      j = m / G;
      g = m % G;
    } else {
      g = m / J;
      j = m % J;
    }
  }
  // byte offset in a plane of logical element l of line g
  __device__ __forceinline__ static uint32_t off(int g, int l) {
    return sw128_mn_offset(static_cast<uint32_t>(l / J), static_cast<uint32_t>(pos(g, l % J)), 1024u,
                           KSTRIDE);
  }
};

__device__ __forceinline__ void st_pair(uint8_t* re, uint8_t* im, uint32_t off, float2 v) {
  *reinterpret_cast<__half*>(re + off) = __float2half_rn(v.x);
  *reinterpret_cast<__half*>(im + off) = __float2half_rn(v.y);
}

__device__ __forceinline__ float2 ld_pair(const uint8_t* re, const uint8_t* im, uint32_t off) {
  return make_float2(__half2float(*reinterpret_cast<const __half*>(re + off)),
                     __half2float(*reinterpret_cast<const __half*>(im + off)));
}

// four consecutive m (same K row, 8-byte aligned) in one store per plane
__device__ __forceinline__ void st_quad(uint8_t* re, uint8_t* im, uint32_t off, const float2 (&x)[4]) {
  __half2 r01 = __floats2half2_rn(x[0].x, x[1].x), r23 = __floats2half2_rn(x[2].x, x[3].x);
  __half2 i01 = __floats2half2_rn(x[0].y, x[1].y), i23 = __floats2half2_rn(x[2].y, x[3].y);
  uint2 rr, ii;
  rr.x = *reinterpret_cast<uint32_t*>(&r01);
  rr.y = *reinterpret_cast<uint32_t*>(&r23);
  ii.x = *reinterpret_cast<uint32_t*>(&i01);
  ii.y = *reinterpret_cast<uint32_t*>(&i23);
  *reinterpret_cast<uint2*>(re + off) = rr;
  *reinterpret_cast<uint2*>(im + off) = ii;
}

// N consecutive m in one K row (N = 2, 4, 8; offset 2N-byte aligned, inside
// one 16-byte chunk): one 2N-byte store per plane.
template <int N>
__device__ __forceinline__ void st_run(uint8_t* re, uint8_t* im, uint32_t off, const float2 (&x)[N]) {
  static_assert(N == 2 || N == 4 || N == 8, "run length");
  uint32_t rr[N / 2], ii[N / 2];
#pragma unroll
  for (int k = 0; k < N / 2; ++k) {
    const __half2 hr = __floats2half2_rn(x[2 * k].x, x[2 * k + 1].x);
    const __half2 hi = __floats2half2_rn(x[2 * k].y, x[2 * k + 1].y);
    rr[k] = *reinterpret_cast<const uint32_t*>(&hr);
    ii[k] = *reinterpret_cast<const uint32_t*>(&hi);
  }
  if constexpr (N == 2) {
    *reinterpret_cast<uint32_t*>(re + off) = rr[0];
    *reinterpret_cast<uint32_t*>(im + off) = ii[0];
  } else if constexpr (N == 4) {
    *reinterpret_cast<uint2*>(re + off) = make_uint2(rr[0], rr[1]);
    *reinterpret_cast<uint2*>(im + off) = make_uint2(ii[0], ii[1]);
  } else {
    *reinterpret_cast<uint4*>(re + off) = make_uint4(rr[0], rr[1], rr[2], rr[3]);
    *reinterpret_cast<uint4*>(im + off) = make_uint4(ii[0], ii[1], ii[2], ii[3]);
  }
}

__device__ __forceinline__ void ld_quad(const uint8_t* re, const uint8_t* im, uint32_t off, float2 (&x)[4]) {
  const uint2 rr = *reinterpret_cast<const uint2*>(re + off);
  const uint2 ii = *reinterpret_cast<const uint2*>(im + off);
  const float2 r01 = __half22float2(*reinterpret_cast<const __half2*>(&rr.x));
  const float2 r23 = __half22float2(*reinterpret_cast<const __half2*>(&rr.y));
  const float2 i01 = __half22float2(*reinterpret_cast<const __half2*>(&ii.x));
  const float2 i23 = __half22float2(*reinterpret_cast<const __half2*>(&ii.y));
  x[0] = make_float2(r01.x, i01.x);
  x[1] = make_float2(r01.y, i01.y);
  x[2] = make_float2(r23.x, i23.x);
  x[3] = make_float2(r23.y, i23.y);
}

// ---------------------------------------------------------------------------
// One radix-16 stage epilogue (compile-time stage index s).
//   intermediate stage: D -> x twiddle of the next stage -> FP16 -> next
//                       stage's positions in shared memory;
//   last stage        : D -> the IO policy's per-element store, straight to
//                       global memory (lanes hold adjacent butterflies, or
//                       adjacent lines in line-minor order, so every warp store
//                       is one contiguous segment per output index c).
// ---------------------------------------------------------------------------
template <int L, int G, bool LINE_MINOR, int s, class IO, int NT = kPassThreads>
__device__ __forceinline__ void stage_epilogue(uint8_t* re, uint8_t* im, const float2* __restrict__ tw,
                                               uint32_t tbase, int warp, int lane, const IO& io,
                                               long long line0, bool stage_out) {
  using Sh = LineShape<L>;
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr int J = Sh::J;
  constexpr int NG = Tl::Mt / 128;
  constexpr int Ns = Sh::T << (4 * s);
  constexpr bool LAST = (s == Sh::S - 1);
#pragma unroll 1
  for (int grp = warp >> 2; grp < NG; grp += NT / 128) {
    const int m = grp * 128 + 32 * (warp & 3) + lane;
    int g, j;
    Tl::unpos(m, g, j);
    // twiddle reads of the next stage issued before the TMEM load, so their
    // latency overlaps it (they depend on the row only)
    float2 w_pre = make_float2(1.f, 0.f), wstep_pre = make_float2(1.f, 0.f);
    if constexpr (!LAST) {
      const int rp_ = ((j / Ns) * 16 * Ns + j % Ns) / J;
      w_pre = __ldg(tw + rp_ * (j % Ns) * (L / (256 * Ns)));
      wstep_pre = __ldg(tw + rp_ * (L / 256));
    }
    uint32_t d[32];
    tmem_ld_x32(tbase + (static_cast<uint32_t>(32 * (warp & 3)) << 16) + grp * 32u, d);
    tmem_ld_wait();
    if constexpr (LAST && PlanesOutIo<IO>) {
      const long long line = line0 + g;
      float2 v[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) v[c] = make_float2(__uint_as_float(d[c]), __uint_as_float(d[16 + c]));
      if (line < io.total_lines) {
        io.product16(line, j, J, v);
      } else {
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] = make_float2(0.f, 0.f);
      }
      if constexpr (Sh::T == 1) {
#pragma unroll
        for (int c = 0; c < 16; ++c) st_pair(re, im, Tl::off(g, j + c * J), v[c]);
      } else {
        // The following transform starts with a radix-T stage over x[j'' +
        // r L/T]; with L/T = (16/T) J, the inputs of its butterfly j'' = j +
        // c0 J are this thread's outputs c = c0 + r 16/T. So the stage runs
        // here, in registers, with the next transform's direction and first
        // twiddle W_(16T)^(rp c'), and its outputs go to l' = j'' T + c' --
        // what that transform's load phase would have written.
        constexpr int T = Sh::T;
        constexpr int R = 16 / T;
#pragma unroll
        for (int c0 = 0; c0 < R; ++c0) {
          float2 t[T];
#pragma unroll
          for (int r = 0; r < T; ++r) t[r] = v[c0 + r * R];
          small_dft<T, IO::NEXT_SIGN>(t);
          const int jj = j + c0 * J;
          const int rp = (jj * T) / J;
#pragma unroll
          for (int cp = 0; cp < T; ++cp) {
            const float2 x = cp == 0 ? t[0] : cmulf(t[cp], __ldg(io.tw_next + rp * cp * (L / (16 * T))));
            st_pair(re, im, Tl::off(g, jj * T + cp), x);
          }
        }
      }
    } else if constexpr (LAST) {
      // final outputs X[j + c*J] of line line0 + g
      const long long line = line0 + g;
      if (line < io.total_lines) {
        float2 v[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] = make_float2(__uint_as_float(d[c]), __uint_as_float(d[16 + c]));
        bool staged = false;
        if (stage_out) {
          // natural-order half2 copy of the tile for the bulk store
          uint32_t* row = reinterpret_cast<uint32_t*>(re) + static_cast<uint32_t>(g) * L + j;
          if (io.scale != 1.0f) {
#pragma unroll
            for (int c = 0; c < 16; ++c) v[c] = make_float2(v[c].x * io.scale, v[c].y * io.scale);
          }
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            __half2 h = __floats2half2_rn(v[c].x, v[c].y);
            row[c * J] = *reinterpret_cast<uint32_t*>(&h);
          }
          staged = true;
        }
        if constexpr (TensorMapIo<IO> && LINE_MINOR) {
          if (io.out_tma) {
            // column-layout copy of the tile (element (g, l) at l * G + g)
            // for the tensor store the kernel issues after the stages
            io.prepare_row16(line, j, J, v);
            uint32_t* col = reinterpret_cast<uint32_t*>(re) + g;
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              __half2 h = __floats2half2_rn(v[c].x, v[c].y);
              col[(j + c * J) * G] = *reinterpret_cast<uint32_t*>(&h);
            }
            staged = true;
          }
        }
        if (!staged) io.store_row16(line, j, J, v);
      }
    } else {
      // output c goes to l' = (j / Ns) * 16Ns + c*Ns + (j % Ns); all 16 land in
      // the same K row r' = l' / J (16Ns divides J), columns j' = j'0 + c*Ns.
      const int a = j / Ns, b = j % Ns;
      const int lp0 = a * 16 * Ns + b;
      const int rp = lp0 / J;
      const int jp0 = lp0 % J;
      // twiddle of the next stage: W_{256 Ns}^{r' (c Ns + b)} = W_L^{e0 + c*de}
      // with e0 = r' b L / (256 Ns), de = r' L / 256 (read above as w_pre, wstep_pre)
      const uint32_t krow = (static_cast<uint32_t>(rp) >> 3) * Tl::KSTRIDE + (rp & 7) * 128u;
      if constexpr (Ns == 1 && !LINE_MINOR) {
        // 16 outputs -> 16 consecutive columns: two 16-byte stores per plane
        uint32_t pr[8], pi[8];
        // twiddles by recurrence, two outputs per packed instruction: two
        // table reads per row (FP32 error ~1e-6, far below the FP16 rounding
        // that follows)
        TwPairSeq tws(w_pre, wstep_pre);
#pragma unroll
        for (int c = 0; c < 16; c += 2) {
          float2 yr, yi;
          cmul_pair(make_float2(__uint_as_float(d[c]), __uint_as_float(d[c + 1])),
                    make_float2(__uint_as_float(d[16 + c]), __uint_as_float(d[17 + c])), tws.w, yr, yi);
          if (c + 2 < 16) tws.next();
          __half2 hr = __float22half2_rn(yr), hi = __float22half2_rn(yi);
          pr[c / 2] = *reinterpret_cast<uint32_t*>(&hr);
          pi[c / 2] = *reinterpret_cast<uint32_t*>(&hi);
        }
        const uint32_t mp = static_cast<uint32_t>(Tl::pos(g, jp0));  // multiple of 16
        // lanes with bit 2 set store the upper half first, so the 8 lanes of a
        // quarter-warp cover all 8 16-byte bank groups in each instruction
        const bool sw = (lane >> 2) & 1;
        const uint32_t m0 = mp + (sw ? 8u : 0u), m1 = mp + (sw ? 0u : 8u);
        const uint32_t off0 = krow + (m0 >> 6) * 1024u + ((((m0 & 63u) >> 3) ^ (rp & 7)) << 4);
        const uint32_t off1 = krow + (m1 >> 6) * 1024u + ((((m1 & 63u) >> 3) ^ (rp & 7)) << 4);
        const uint4 rlo = make_uint4(pr[0], pr[1], pr[2], pr[3]), rhi = make_uint4(pr[4], pr[5], pr[6], pr[7]);
        const uint4 ilo = make_uint4(pi[0], pi[1], pi[2], pi[3]), ihi = make_uint4(pi[4], pi[5], pi[6], pi[7]);
        *reinterpret_cast<uint4*>(re + off0) = sw ? rhi : rlo;
        *reinterpret_cast<uint4*>(im + off0) = sw ? ihi : ilo;
        *reinterpret_cast<uint4*>(re + off1) = sw ? rlo : rhi;
        *reinterpret_cast<uint4*>(im + off1) = sw ? ilo : ihi;
      } else {
        // the 16 twiddled outputs, two per packed instruction
        float2 y[16];
        {
          TwPairSeq tws(w_pre, wstep_pre);
#pragma unroll
          for (int c = 0; c < 16; c += 2) {
            float2 yr, yi;
            cmul_pair(make_float2(__uint_as_float(d[c]), __uint_as_float(d[c + 1])),
                      make_float2(__uint_as_float(d[16 + c]), __uint_as_float(d[17 + c])), tws.w, yr, yi);
            if (c + 2 < 16) tws.next();
            y[c] = make_float2(yr.x, yi.x);
            y[c + 1] = make_float2(yr.y, yi.y);
          }
        }
        // column step between consecutive outputs: Ns (line-major) or Ns*G
        // (line-minor); when it is a multiple of 64 (one swizzle atom) the
        // swizzled offset moves by a compile-time amount per output
        constexpr uint32_t CSTEP = LINE_MINOR ? static_cast<uint32_t>(Ns * G) : static_cast<uint32_t>(Ns);
        if constexpr (CSTEP % 64 == 0) {
          const uint32_t mp0 = static_cast<uint32_t>(Tl::pos(g, jp0));
          const uint32_t off0 =
              krow + (mp0 >> 6) * 1024u + ((((mp0 & 63u) >> 3) ^ (rp & 7)) << 4) + (mp0 & 7u) * 2u;
#pragma unroll
          for (int c = 0; c < 16; ++c) st_pair(re, im, off0 + static_cast<uint32_t>(c) * (CSTEP / 64u) * 1024u, y[c]);
        } else if constexpr (CSTEP >= 8 && (CSTEP & (CSTEP - 1)) == 0) {
          // the column moves by CSTEP < 64 per output: the swizzled offsets
          // repeat with period PER = 64 / CSTEP, shifted by one 1 KiB atom
          // per period, so PER offsets computed once serve all 16 outputs
          constexpr int PER = static_cast<int>(64u / CSTEP);
          const uint32_t mp0 = static_cast<uint32_t>(Tl::pos(g, jp0));
          uint32_t offs[PER];
#pragma unroll
          for (int k = 0; k < PER; ++k) {
            const uint32_t mp = mp0 + static_cast<uint32_t>(k) * CSTEP;
            offs[k] = krow + (mp >> 6) * 1024u + ((((mp & 63u) >> 3) ^ (rp & 7)) << 4) + (mp & 7u) * 2u;
          }
#pragma unroll
          for (int c = 0; c < 16; ++c) st_pair(re, im, offs[c % PER] + static_cast<uint32_t>(c / PER) * 1024u, y[c]);
        } else if constexpr (LINE_MINOR && Ns == 1 && G == 4) {
          // Four-line tiles, first stage: output c of butterfly (g, j) goes
          // to column (jp0 + c) * 4 + g of K row rp, jp0 a multiple of 16.
          // A warp's 8 butterflies j share rp, so one output of all of them
          // falls in the same 16-byte chunk of 8 atoms: 8 wavefronts per
          // store. Lane group k = (lane >> 2) & 7 stores its outputs in the
          // order c ^ 2k instead (slot i holds output i ^ 2k, chunk
          // (i >> 1) ^ k ^ rp), so one instruction's stores fill 8 chunks.
          // The values move as packed (re, im) halves through three
          // conditional swaps.
          const uint32_t k = (static_cast<uint32_t>(lane) >> 2) & 7u;
          uint32_t h[16];
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const __half2 p = __floats2half2_rn(y[c].x, y[c].y);
            h[c] = *reinterpret_cast<const uint32_t*>(&p);
          }
#pragma unroll
          for (int lvl = 0; lvl < 3; ++lvl) {
            const bool sw = (k >> lvl) & 1u;
            const int stride = 2 << lvl;
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              if ((c & stride) == 0) {
                const uint32_t a = h[c], b = h[c + stride];
                h[c] = sw ? b : a;
                h[c + stride] = sw ? a : b;
              }
            }
          }
          const uint32_t mp0 = static_cast<uint32_t>(Tl::pos(g, jp0));
          const uint32_t base = krow + (mp0 >> 6) * 1024u + static_cast<uint32_t>(g) * 2u;
          const uint32_t kx = k ^ static_cast<uint32_t>(rp & 7);
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const uint32_t off = base + (((static_cast<uint32_t>(i) >> 1) ^ kx) << 4) + static_cast<uint32_t>(i & 1) * 8u;
            *reinterpret_cast<uint16_t*>(re + off) = static_cast<uint16_t>(h[i] & 0xffffu);
            *reinterpret_cast<uint16_t*>(im + off) = static_cast<uint16_t>(h[i] >> 16);
          }
        } else {
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const uint32_t mp = static_cast<uint32_t>(Tl::pos(g, jp0 + c * Ns));
            const uint32_t off = krow + (mp >> 6) * 1024u + ((((mp & 63u) >> 3) ^ (rp & 7)) << 4) + (mp & 7u) * 2u;
            st_pair(re, im, off, y[c]);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Per-CTA state shared by the tiles a CTA processes. Shared-memory layout:
//   [0, 2048)      B matrix image (the 16-point DFT, this direction)
//   [2048, 2112)   mbarriers (MMA, TMA), TMEM address slot
//   [3072, ...)    tile planes (real plane, imaginary plane), 1024-aligned
// ---------------------------------------------------------------------------
constexpr uint32_t kPlaneOffset = 3072;

struct PassState {
  uint8_t* smem;
  uint8_t* bmat;
  uint64_t* mbar;
  uint64_t* tma_bar;
  uint32_t* tslot;
  uint32_t tbase;
  uint32_t phase;
  uint32_t tma_phase;
};

__device__ __forceinline__ uint8_t* aligned_dynamic_smem() {
  extern __shared__ uint8_t smem_raw[];
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                    ~static_cast<uintptr_t>(1023));
}

// B matrix, barriers, TMEM allocation (whole CTA).
template <uint32_t TMEM_COLS>
__device__ __forceinline__ void pass_setup(PassState& st, const uint32_t* __restrict__ bmat_g) {
  st.smem = aligned_dynamic_smem();
  st.bmat = st.smem;
  st.mbar = reinterpret_cast<uint64_t*>(st.smem + 2048);
  st.tma_bar = reinterpret_cast<uint64_t*>(st.smem + 2056);
  st.tslot = reinterpret_cast<uint32_t*>(st.smem + 2064);
  const int tid = threadIdx.x;
  for (int i = tid; i < 512; i += blockDim.x) reinterpret_cast<uint32_t*>(st.bmat)[i] = __ldg(bmat_g + i);
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

// Outstanding bulk stores complete, TMEM released (whole CTA).
template <uint32_t TMEM_COLS>
__device__ __forceinline__ void pass_teardown(PassState& st) {
  if (threadIdx.x == 0) bulk_wait_all();
  tc_fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tmem_dealloc(st.tbase, TMEM_COLS);
}

// The S radix-16 tensor-core stages of one tile held in the planes (MMA
// batch, commit, bounded wait, epilogue). False if a wait gave up.
template <int L, int G, bool LINE_MINOR, int SIGN, class IO, int NT = kPassThreads>
__device__ __forceinline__ bool run_stages(PassState& st, const IO& io, const PassCore& core, long long line0,
                                           uint8_t* re, uint8_t* im, bool stage_out) {
  using Sh = LineShape<L>;
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr int S = Sh::S;
  constexpr int NG = Tl::Mt / 128;
  constexpr uint32_t KSTRIDE = Tl::KSTRIDE;
  constexpr uint32_t IDESC = make_idesc_f16_f32(128, 32, true, false);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  bool timed_out = false;
    // ================= radix-16 tensor-core stages =================
    auto run_stage = [&](auto s_const) {
      constexpr int s = decltype(s_const)::value;
      if (timed_out) return;
      if (tid == 0) {
        tc_fence_after_sync();
        const uint32_t a0 = smem_u32(re), a1 = smem_u32(im), b0 = smem_u32(st.bmat);
        const uint64_t bd0 = make_sdesc(b0, 128u, 512u, kLayoutNone);
        const uint64_t bd1 = make_sdesc(b0 + 256u, 128u, 512u, kLayoutNone);
#pragma unroll
        for (int grp = 0; grp < NG; ++grp) {
          const uint64_t ad0 = make_sdesc(a0 + grp * 2048u, 1024u, KSTRIDE, kLayoutSw128);
          const uint64_t ad1 = make_sdesc(a1 + grp * 2048u, 1024u, KSTRIDE, kLayoutSw128);
          umma_f16(st.tbase + grp * 32u, ad0, bd0, IDESC, 0u);
          umma_f16(st.tbase + grp * 32u, ad1, bd1, IDESC, 1u);
        }
        umma_commit(st.mbar);
      }
      // one thread polls the MMA barrier; the others block at the CTA
      // barrier (no issue slots spent spinning), which carries the
      // completion to them
      bool to = false;
      if (tid == 0) {
        to = !mbar_wait_bounded(st.mbar, st.phase & 1u);
        if (to) atomicOr(core.err, kErrMmaTimeout);
      }
      st.phase++;
      if (__syncthreads_or(to)) {
        timed_out = true;
        return;
      }
      tc_fence_after_sync();
      stage_epilogue<L, G, LINE_MINOR, s, IO, NT>(re, im, core.tw, st.tbase, warp, lane, io, line0, stage_out);
      fence_proxy_async_smem();
      tc_fence_before_sync();
      __syncthreads();
    };
    [&]<int... Is>(std::integer_sequence<int, Is...>) {
      (run_stage(std::integral_constant<int, Is>{}), ...);
    }(std::make_integer_sequence<int, S>{});
    return !timed_out;
}

// Five lane-bit destinations for remap_lane_bits.
struct LaneBits {
  int b[5];
};

// Thread index with its five lane bits sent to bits B0..B4 (the other bits
// of the index fill the remaining positions in order): a permutation of
// [0, NT), so the items one sweep of NT threads covers stay the same.
template <int NT, int B0, int B1, int B2, int B3, int B4>
__device__ __forceinline__ int remap_lane_bits(int tid) {
  constexpr int K = ilog2c(NT);
  static_assert((1 << K) == NT && K >= 5 && K <= 10, "index range: a power of two, 32 to 1024");
  constexpr int B[5] = {B0, B1, B2, B3, B4};
  if constexpr (B0 == 0 && B1 == 1 && B2 == 2 && B3 == 3 && B4 == 4) {
    return tid;
  } else {
    static_assert(B0 < K && B1 < K && B2 < K && B3 < K && B4 < K, "lane bit in range");
    static_assert(B0 != B1 && B0 != B2 && B0 != B3 && B0 != B4 && B1 != B2 && B1 != B3 && B1 != B4 &&
                      B2 != B3 && B2 != B4 && B3 != B4,
                  "distinct destinations");
    int r = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i) r |= ((tid >> i) & 1) << B[i];
    // the higher thread-index bits, in order, into the positions left free
    int src = 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (k != B0 && k != B1 && k != B2 && k != B3 && k != B4) {
        r |= ((tid >> src) & 1) << k;
        ++src;
      }
    }
    return r;
  }
}

// Lane-bit destinations (remap_lane_bits) of tile_load's column-input items
// (four adjacent lines at one butterfly, one 8-byte store per plane and
// output), per (L, butterflies per tile), from the same shared-memory bank
// model as permute_lane_bits; lane bit 0 stays, so two lanes still read one
// 32-byte element row. E.g. L = 1024 on 512-butterfly tiles: 1024 -> 256
// store wavefronts per tile. Identity where nothing is gained.
template <int L, int Mt, bool LINE_MINOR>
constexpr LaneBits tile_load_lane_bits() {
  if constexpr (LINE_MINOR) {
    if constexpr (Mt == 128) {
      if constexpr (L == 64) return {{0, 1, 2, 5, 3}};
      if constexpr (L == 128) return {{0, 1, 3, 4, 2}};
    } else if constexpr (Mt == 512) {
      if constexpr (L == 512) return {{0, 1, 2, 7, 3}};
      if constexpr (L == 1024) return {{0, 1, 5, 6, 2}};
      if constexpr (L == 2048) return {{0, 1, 4, 5, 2}};
    } else if constexpr (Mt == 1024) {
      if constexpr (L == 1024) return {{0, 1, 2, 7, 3}};
      if constexpr (L == 2048) return {{0, 5, 6, 7, 1}};
    }
  }
  return {{0, 1, 2, 3, 4}};
}

// ---------------------------------------------------------------------------
// Load phase of one tile: G lines of length L starting at line0 from global
// memory into the planes re / im (the radix-T stage and the first radix-16
// stage's twiddle applied), ending with the CTA barrier that hands the planes
// to the tensor core. False if a bounded wait gave up (the error word is set;
// the caller stops and tears down).
//   L          line length
//   G          lines per tile (G * L / 16 must be 128, 256, 512 or 1024)
//   LINE_MINOR butterfly order in the tile (true for column passes)
//   SIGN       -1 forward, +1 inverse
//   IO         global-memory policy (see fft_io.cuh)
// ---------------------------------------------------------------------------
template <int L, int G, bool LINE_MINOR, int SIGN, class IO>
__device__ __forceinline__ bool tile_load(PassState& st, const IO& io, const PassCore& core, long long line0, uint8_t* re,
                                          uint8_t* im) {
  using Sh = LineShape<L>;
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr int T = Sh::T;
  constexpr int J = Sh::J;
  constexpr int Mt = Tl::Mt;
  static_assert(Mt % 128 == 0 && Mt <= 1024, "tile size");
  static_assert(G % 4 == 0 || IO::IN_VEC_L, "line-vectorised loads need G % 4 == 0");
  static_assert(G % 4 == 0 || IO::OUT_VEC_L, "line-vectorised stores need G % 4 == 0");
  const int tid = threadIdx.x;
  bool timed_out = false;
  // Contiguous tiles (element (line, l) at base + line*L + l) move with bulk
  // TMA copies: one 2*PLANE-byte copy in, one out, through the tile region.
  const bool tma_in = IO::IN_VEC_L && io.in_contig;
    const long long rem = io.total_lines - line0;
    const int nval = rem < G ? static_cast<int>(rem) : G;

    // ================= load (+ radix-T stage) =================
    if (tma_in) {
      if (tid == 0) {
        bulk_wait_read_all();  // the previous tile's bulk store has read the region
        const uint32_t bytes = static_cast<uint32_t>(nval) * L * 4u;
        mbar_arrive_expect_tx(st.tma_bar, bytes);
        bulk_g2s(re, io.tile_src(line0), bytes, st.tma_bar);
        // the issuing thread polls; the others wait at the CTA barrier
        if (!mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u)) {
          timed_out = true;
          atomicOr(core.err, kErrMmaTimeout);
        }
      }
      st.tma_phase++;
      if (__syncthreads_or(timed_out)) return false;
      // every thread takes its quads of the radix-T stage into registers ...
      constexpr int QPL = (L / T) / 4;
      constexpr int ITEMS = G * QPL;
      constexpr int NU = (ITEMS + kPassThreads - 1) / kPassThreads;
      uint4 raw[NU][T];
      const uint32_t* src = reinterpret_cast<const uint32_t*>(re);
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int it = tid + u * kPassThreads;
        const int g = it / QPL;
        const int j0 = (it % QPL) * 4;
#pragma unroll
        for (int r = 0; r < T; ++r)
          raw[u][r] = (it < ITEMS && g < nval)
                          ? *reinterpret_cast<const uint4*>(src + g * L + j0 + r * (L / T))
                          : make_uint4(0, 0, 0, 0);
      }
      __syncthreads();  // ... before the region is overwritten in planar form
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int it = tid + u * kPassThreads;
        if (ITEMS % kPassThreads != 0 && it >= ITEMS) continue;
        const int g = it / QPL;
        const int j0 = (it % QPL) * 4;
        if constexpr (T == 1 && !LINE_MINOR && J >= 4) {
          // de-interleave (re, im) pairs without leaving FP16
          const uint4 w = raw[u][0];
          uint2 rr, ii;
          rr.x = __byte_perm(w.x, w.y, 0x5410);
          rr.y = __byte_perm(w.z, w.w, 0x5410);
          ii.x = __byte_perm(w.x, w.y, 0x7632);
          ii.y = __byte_perm(w.z, w.w, 0x7632);
          const uint32_t off = Tl::off(g, j0);
          *reinterpret_cast<uint2*>(re + off) = rr;
          *reinterpret_cast<uint2*>(im + off) = ii;
        } else {
          float2 v[T][4];
#pragma unroll
          for (int r = 0; r < T; ++r) unpack_h2x4(raw[u][r], v[r]);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            float2 t[T];
#pragma unroll
            for (int r = 0; r < T; ++r) t[r] = v[r][q];
            small_dft<T, SIGN>(t);
            const int j = j0 + q;
#pragma unroll
            for (int c = 0; c < T; ++c) {
              const int lp = j * T + c;
              float2 x = t[c];
              if constexpr (T > 1) {
                const int rp = lp / J, jp = lp % J;
                x = cmulf(x, __ldg(core.tw + rp * (jp % T) * (L / (16 * T))));
              }
              st_pair(re, im, Tl::off(g, lp), x);
            }
          }
        }
      }
    } else if constexpr (IO::IN_VEC_L) {
      // item = (line g, butterflies j0..j0+3 of the radix-T stage); T fetches each
      constexpr int QPL = (L / T) / 4;
      constexpr int ITEMS = G * QPL;
      constexpr int U = T >= 8 ? 1 : 8 / T;
#pragma unroll 1
      for (int base = tid; base < ITEMS; base += kPassThreads * U) {
        typename IO::Raw raw[U][T];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int it = base + u * kPassThreads;
          const int g = it / QPL;
          const int j0 = (it % QPL) * 4;
#pragma unroll
          for (int r = 0; r < T; ++r)
            raw[u][r] = io.fetch_l(line0 + g, j0 + r * (L / T), it < ITEMS);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int it = base + u * kPassThreads;
          if (ITEMS % (kPassThreads * U) != 0 && it >= ITEMS) continue;
          const int g = it / QPL;
          const int j0 = (it % QPL) * 4;
          float2 v[T][4];
#pragma unroll
          for (int r = 0; r < T; ++r) io.decode_l(raw[u][r], line0 + g, j0 + r * (L / T), v[r]);
          if constexpr (T == 1) {
            if constexpr (!LINE_MINOR && J >= 4) {
              st_quad(re, im, Tl::off(g, j0), v[0]);
            } else {
#pragma unroll
              for (int q = 0; q < 4; ++q) st_pair(re, im, Tl::off(g, j0 + q), v[0][q]);
            }
          } else {
            // output c of butterfly j -> l' = j*T + c: K row rp = j*T / J for
            // every c, twiddle W_(16T)^(rp c) of the next stage (Ns = T); the
            // four butterflies of an item share rp when J / T is a multiple of
            // 4. Line-major tiles store a butterfly's T outputs as one run.
            constexpr bool SHARED_RP = ((J / T) % 4) == 0;
            float2 wt[T];
            auto load_tw = [&](int rp) {
              wt[0] = make_float2(1.f, 0.f);
#pragma unroll
              for (int c = 1; c < T; ++c) wt[c] = __ldg(core.tw + rp * c * (L / (16 * T)));
            };
            if constexpr (SHARED_RP) load_tw((j0 * T) / J);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              float2 t[T];
#pragma unroll
              for (int r = 0; r < T; ++r) t[r] = v[r][q];
              small_dft<T, SIGN>(t);
              const int j = j0 + q;
              if constexpr (!SHARED_RP) load_tw((j * T) / J);
#pragma unroll
              for (int c = 1; c < T; ++c) t[c] = cmulf(t[c], wt[c]);
              if constexpr (!LINE_MINOR) {
                st_run<T>(re, im, Tl::off(g, j * T), t);
              } else {
#pragma unroll
                for (int c = 0; c < T; ++c) st_pair(re, im, Tl::off(g, j * T + c), t[c]);
              }
            }
          }
        }
      }
    } else {
      // item = (4 adjacent lines g0..g0+3, butterfly j of the radix-T stage);
      // the lane bits of the first item are remapped so that one store
      // instruction's 8-byte plane stores spread over the banks
      constexpr int GQ = G / 4;
      constexpr int ITEMS = GQ * (L / T);
      constexpr int U = T >= 8 ? 1 : 8 / T;
      constexpr LaneBits lb = tile_load_lane_bits<L, Mt, LINE_MINOR>();
      const int first = remap_lane_bits<kPassThreads, lb.b[0], lb.b[1], lb.b[2], lb.b[3], lb.b[4]>(tid);
#pragma unroll 1
      for (int base = first; base < ITEMS; base += kPassThreads * U) {
        typename IO::Raw raw[U][T];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int it = base + u * kPassThreads;
          const int j = it / GQ;
          const int g0 = (it % GQ) * 4;
#pragma unroll
          for (int r = 0; r < T; ++r) raw[u][r] = io.fetch_g(line0 + g0, j + r * (L / T), it < ITEMS);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int it = base + u * kPassThreads;
          if (ITEMS % (kPassThreads * U) != 0 && it >= ITEMS) continue;
          const int j = it / GQ;
          const int g0 = (it % GQ) * 4;
          float2 v[T][4];
#pragma unroll
          for (int r = 0; r < T; ++r) io.decode_g(raw[u][r], line0 + g0, j + r * (L / T), v[r]);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            float2 t[T];
#pragma unroll
            for (int r = 0; r < T; ++r) t[r] = v[r][q];
            small_dft<T, SIGN>(t);
#pragma unroll
            for (int r = 0; r < T; ++r) v[r][q] = t[r];
          }
#pragma unroll
          for (int c = 0; c < T; ++c) {
            const int lp = j * T + c;
            float2 x[4] = {v[c][0], v[c][1], v[c][2], v[c][3]};
            if constexpr (T > 1) {
              const int rp = lp / J, jp = lp % J;
              const float2 w = __ldg(core.tw + rp * (jp % T) * (L / (16 * T)));
#pragma unroll
              for (int q = 0; q < 4; ++q) x[q] = cmulf(x[q], w);
            }
            if constexpr (LINE_MINOR) {
              st_quad(re, im, Tl::off(g0, lp), x);  // 4 adjacent lines -> 4 consecutive m
            } else {
#pragma unroll
              for (int q = 0; q < 4; ++q) st_pair(re, im, Tl::off(g0 + q, lp), x[q]);
            }
          }
        }
      }
    }
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();
    return true;
}

// One tile: load, the S radix-16 tensor-core stages, store (FP16 storage,
// FP32 accumulation and twiddles). False if a bounded wait gave up.
template <int L, int G, bool LINE_MINOR, int SIGN, class IO>
__device__ __forceinline__ bool pass_tile(PassState& st, const IO& io, const PassCore& core, long long line0) {
  using Tl = Tile<L, G, LINE_MINOR>;
  uint8_t* re = st.smem + kPlaneOffset;
  uint8_t* im = re + Tl::PLANE;
  if (!tile_load<L, G, LINE_MINOR, SIGN, IO>(st, io, core, line0, re, im)) return false;
  // Contiguous tiles (element (line, l) at base + line*L + l) leave by one
  // bulk TMA store from the tile region.
  const bool stage_out = IO::OUT_VEC_L && io.out_contig && !LINE_MINOR;
  const long long rem = io.total_lines - line0;
  const int nval = rem < G ? static_cast<int>(rem) : G;
  if (!run_stages<L, G, LINE_MINOR, SIGN, IO>(st, io, core, line0, re, im, stage_out)) return false;
  if (stage_out && threadIdx.x == 0) {
    // the last stage left the tile in natural order: one bulk store
    bulk_s2g(io.tile_dst(line0), re, static_cast<uint32_t>(nval) * L * 4u);
    bulk_commit();
  }
  return true;
}

template <int L, int G>
__host__ __device__ constexpr uint32_t pass_tmem_cols() {
  return static_cast<uint32_t>(G * L / 16 / 128 * 32);
}

// ---------------------------------------------------------------------------
// The pass kernel: persistent CTAs over the tiles of one pass.
// ---------------------------------------------------------------------------
template <int L, int G, bool LINE_MINOR, int SIGN, class IO, int MINB = 2>
__global__ void __launch_bounds__(kPassThreads, MINB) fft_pass_f16(const IO io, const PassCore core) {
  constexpr uint32_t TMEM_COLS = pass_tmem_cols<L, G>();
  static_assert(TMEM_COLS >= 32 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  PassState st;
  pass_setup<TMEM_COLS>(st, core.bmat);
  const long long ntiles = (io.total_lines + G - 1) / G;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    if (!pass_tile<L, G, LINE_MINOR, SIGN, IO>(st, io, core, tile * G)) break;
  pass_teardown<TMEM_COLS>(st);
}

// ---------------------------------------------------------------------------
// Prefetching pass kernel. Each CTA owns a raw input buffer beside the
// planes; tile t+1's input streams into it (one TMA bulk copy for contiguous
// tiles, 16-byte cp.async chunks otherwise) while tile t runs its
// tensor-core stages, so the load latency leaves the critical path.
//   shared memory: [B matrix, barriers][planes: 2*PLANE][raw: 2*PLANE]
//   raw layout: natural [line][l] half2 (vector-along-line inputs) or
//               line-minor [l][line] half2 (column inputs)
// ---------------------------------------------------------------------------
template <int L, int G, bool LINE_MINOR, class IO, int NT = kPassThreads>
__device__ __forceinline__ void prefetch_tile(PassState& st, const IO& io, long long line0, uint8_t* raw) {
  if (IO::IN_VEC_L && io.in_contig) {
    if (threadIdx.x == 0) {
      const long long rem = io.total_lines - line0;
      const int nval = rem < G ? static_cast<int>(rem) : G;
      const uint32_t bytes = static_cast<uint32_t>(nval) * L * 4u;
      mbar_arrive_expect_tx(st.tma_bar, bytes);
      bulk_g2s(raw, io.tile_src(line0), bytes, st.tma_bar);
    }
  } else if constexpr (!IO::IN_VEC_L) {
    if constexpr (TensorMapIo<IO>) {
      if (io.in_tma) {
        // one [L x G] box as L / 256 tensor loads (the host only sets the
        // map when tiles never straddle a sequence)
        if (threadIdx.x == 0) {
          constexpr int BY = L < 256 ? L : 256;
          mbar_arrive_expect_tx(st.tma_bar, static_cast<uint32_t>(G) * L * 4u);
          const int seq = static_cast<int>(line0 >> io.lps_log2);
          const int x0 = static_cast<int>(line0 & ((1ll << io.lps_log2) - 1));
#pragma unroll
          for (int r0 = 0; r0 < L; r0 += BY)
            tma_load_3d(raw + static_cast<uint32_t>(r0) * G * 4u, &io.in_map, x0, r0, seq, st.tma_bar);
        }
        return;
      }
    }
    constexpr int GQ = G / 4;
    constexpr int CH = L * GQ;
#pragma unroll 4
    for (int c = threadIdx.x; c < CH; c += NT) {
      const int l = c / GQ, q = c % GQ;
      bool ok;
      const void* src = io.src_g(line0 + 4 * q, l, ok);
      cp_async16(raw + (static_cast<uint32_t>(l) * G + 4u * q) * 4u, src, ok ? 16u : 0u);
    }
    cp_async_commit();
  } else {
    constexpr int QPL = L / 4;
    constexpr int CH = G * QPL;
#pragma unroll 4
    for (int c = threadIdx.x; c < CH; c += NT) {
      const int g = c / QPL, q = c % QPL;
      bool ok;
      const void* src = io.src_l(line0 + g, 4 * q, ok);
      cp_async16(raw + (static_cast<uint32_t>(g) * L + 4u * q) * 4u, src, ok ? 16u : 0u);
    }
    cp_async_commit();
  }
}

// Whether a tile's input / output moves by tensor map.
template <class IO>
__device__ __forceinline__ bool tensor_in(const IO& io) {
  if constexpr (TensorMapIo<IO>) return !IO::IN_VEC_L && io.in_tma;
  return false;
}
template <class IO>
__device__ __forceinline__ bool tensor_out(const IO& io) {
  if constexpr (TensorMapIo<IO>) return io.out_tma;
  return false;
}

// Wait for the prefetched tile (whole CTA). False if the bounded wait gave up.
template <class IO>
__device__ __forceinline__ bool wait_prefetch(PassState& st, const IO& io, const PassCore& core) {
  if ((IO::IN_VEC_L && io.in_contig) || tensor_in(io)) {
    // one thread polls the copy barrier, the others wait at the CTA barrier
    bool ok = true;
    if (threadIdx.x == 0) {
      ok = mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u);
      if (!ok) atomicOr(core.err, kErrMmaTimeout);
    }
    st.tma_phase++;
    return !__syncthreads_or(!ok);
  }
  cp_async_wait_all();
  __syncthreads();
  return true;
}

// Which item of permute_raw's loop a thread starts at. In a line-minor tile
// the 16-byte chunks of a K row are XOR-swizzled by the row, so an 8-byte
// plane store from lanes whose butterflies share a K row lands in a few banks
// (up to 8 wavefronts per half-warp where 1 would do); lanes whose butterflies
// lie in different K rows spread over all 32. The five lane bits of the
// thread index are therefore sent to other bits of the item index (the
// remaining bits keep their order), which leaves the item set of each sweep of
// the NT threads unchanged. The destinations per (input kind, L, butterflies
// per tile) were chosen by counting shared-memory wavefronts -- per phase
// (32, 16 or 8 lanes for 4-, 8- or 16-byte accesses) the largest number of
// distinct words in one bank -- of the staged-tile loads plus the plane
// stores over every assignment of the lane bits; e.g. L = 1024, 512
// butterflies: 2304 -> 1024 wavefronts per tile for row input, 1280 -> 768
// for column input. Identity where nothing is gained.
template <int L, int Mt, bool IN_VEC_L, bool LINE_MINOR>
constexpr LaneBits permute_lane_bits() {
  constexpr int G = Mt * 16 / L;  // lines per tile; the table covers G % 4 == 0
  if constexpr (G % 4 != 0) {
    return {{0, 1, 2, 3, 4}};
  } else if constexpr (LINE_MINOR && !IN_VEC_L) {
    if constexpr (Mt == 512) {
      if constexpr (L == 512) return {{0, 1, 2, 7, 3}};
      if constexpr (L == 1024) return {{0, 1, 2, 5, 3}};
      if constexpr (L == 2048) return {{0, 1, 4, 5, 2}};
    } else if constexpr (Mt == 256) {
      if constexpr (L == 128 || L == 512) return {{0, 1, 2, 5, 3}};
      if constexpr (L == 1024) return {{0, 1, 2, 4, 3}};
    }
  } else if constexpr (LINE_MINOR && IN_VEC_L) {
    if constexpr (Mt == 512) {
      if constexpr (L <= 64) return {{0, 1, 2, 4, 3}};
      if constexpr (L >= 256 && L <= 1024) return {{0, 1, 4, 5, 2}};
      if constexpr (L == 2048) return {{0, 1, 2, 4, 5}};
    } else if constexpr (Mt == 256) {
      if constexpr (L != 128) return {{0, 1, 2, 4, 3}};
    }
  }
  return {{0, 1, 2, 3, 4}};
}

template <int L, int Mt, bool IN_VEC_L, bool LINE_MINOR, int NT>
__device__ __forceinline__ int permute_first_item(int tid) {
  constexpr LaneBits lb = permute_lane_bits<L, Mt, IN_VEC_L, LINE_MINOR>();
  return remap_lane_bits<NT, lb.b[0], lb.b[1], lb.b[2], lb.b[3], lb.b[4]>(tid);
}

// raw (staged input) -> planes, with the radix-T first stage and the first
// radix-16 stage's twiddle. Lines >= nval read as zero.
template <int L, int G, bool LINE_MINOR, int SIGN, class IO, int NT = kPassThreads>
__device__ __forceinline__ void permute_raw(const uint8_t* raw, uint8_t* re, uint8_t* im, const PassCore& core,
                                            int nval) {
  using Sh = LineShape<L>;
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr int T = Sh::T;
  constexpr int J = Sh::J;
  const int tid = permute_first_item<L, Tl::Mt, IO::IN_VEC_L, LINE_MINOR, NT>(threadIdx.x);
  const uint4 zero = make_uint4(0, 0, 0, 0);
  if constexpr (IO::IN_VEC_L && LINE_MINOR && G % 4 == 0) {
    // Line-minor tile from line-major raw input: item = LPI adjacent lines
    // at one butterfly j (butterflies fastest across lanes, so the raw reads
    // are consecutive words), so every output is LPI consecutive columns:
    // one 2*LPI-byte store per plane, one twiddle read shared by the lines.
    // LPI = 2 for the radix-8 tail keeps the item's values in registers.
    constexpr int LPI = T == 8 ? 2 : 4;
    constexpr int JT = L / T;
    constexpr int ITEMS = (G / LPI) * JT;
    const uint32_t* raw32 = reinterpret_cast<const uint32_t*>(raw);
#pragma unroll 2
    for (int it = tid; it < ITEMS; it += NT) {
      const int j = it % JT;
      const int g0 = (it / JT) * LPI;
      uint32_t w[T][LPI];
#pragma unroll
      for (int r = 0; r < T; ++r)
#pragma unroll
        for (int k = 0; k < LPI; ++k)
          w[r][k] = g0 + k < nval ? raw32[static_cast<uint32_t>(g0 + k) * L + j + r * JT] : 0u;
      if constexpr (T == 1) {
        uint2 rr, ii;
        rr.x = __byte_perm(w[0][0], w[0][1], 0x5410);
        rr.y = __byte_perm(w[0][2], w[0][3], 0x5410);
        ii.x = __byte_perm(w[0][0], w[0][1], 0x7632);
        ii.y = __byte_perm(w[0][2], w[0][3], 0x7632);
        const uint32_t off = Tl::off(g0, j);
        *reinterpret_cast<uint2*>(re + off) = rr;
        *reinterpret_cast<uint2*>(im + off) = ii;
      } else {
        float2 v[T][LPI];
#pragma unroll
        for (int r = 0; r < T; ++r)
#pragma unroll
          for (int k = 0; k < LPI; ++k) v[r][k] = __half22float2(*reinterpret_cast<const __half2*>(&w[r][k]));
#pragma unroll
        for (int k = 0; k < LPI; ++k) {
          float2 t[T];
#pragma unroll
          for (int r = 0; r < T; ++r) t[r] = v[r][k];
          small_dft<T, SIGN>(t);
#pragma unroll
          for (int r = 0; r < T; ++r) v[r][k] = t[r];
        }
        // output c -> l' = j*T + c, twiddle W_(16T)^(rp c), rp = j*T / J
        const int rp = (j * T) / J;
#pragma unroll
        for (int c = 0; c < T; ++c) {
          float2 x[LPI];
#pragma unroll
          for (int k = 0; k < LPI; ++k) x[k] = v[c][k];
          if (c > 0) {
            const float2 tw = __ldg(core.tw + rp * c * (L / (16 * T)));
#pragma unroll
            for (int k = 0; k < LPI; ++k) x[k] = cmulf(x[k], tw);
          }
          if constexpr (LPI == 4) {
            st_quad(re, im, Tl::off(g0, j * T + c), x);
          } else {
            st_run<2>(re, im, Tl::off(g0, j * T + c), x);
          }
        }
      }
    }
  } else if constexpr (IO::IN_VEC_L) {
    constexpr int QPL = (L / T) / 4;
    constexpr int ITEMS = G * QPL;
#pragma unroll 2
    for (int it = tid; it < ITEMS; it += NT) {
      const int g = it / QPL;
      const int j0 = (it % QPL) * 4;
      uint4 w[T];
#pragma unroll
      for (int r = 0; r < T; ++r)
        w[r] = g < nval ? *reinterpret_cast<const uint4*>(raw + (static_cast<uint32_t>(g) * L + j0 + r * (L / T)) * 4u)
                        : zero;
      if constexpr (T == 1 && !LINE_MINOR && J >= 4) {
        uint2 rr, ii;
        rr.x = __byte_perm(w[0].x, w[0].y, 0x5410);
        rr.y = __byte_perm(w[0].z, w[0].w, 0x5410);
        ii.x = __byte_perm(w[0].x, w[0].y, 0x7632);
        ii.y = __byte_perm(w[0].z, w[0].w, 0x7632);
        const uint32_t off = Tl::off(g, j0);
        *reinterpret_cast<uint2*>(re + off) = rr;
        *reinterpret_cast<uint2*>(im + off) = ii;
      } else {
        float2 v[T][4];
#pragma unroll
        for (int r = 0; r < T; ++r) unpack_h2x4(w[r], v[r]);
        // output c of butterfly j -> l' = j*T + c: K row rp = j*T / J for
        // every c, twiddle W_(16T)^(rp c); the item's four butterflies share
        // rp when J / T is a multiple of 4
        constexpr bool SHARED_RP = ((J / T) % 4) == 0 && T <= 4;
        float2 wt[T];
        auto load_tw = [&](int rp) {
          wt[0] = make_float2(1.f, 0.f);
#pragma unroll
          for (int c = 1; c < T; ++c) wt[c] = __ldg(core.tw + rp * c * (L / (16 * T)));
        };
        if constexpr (T > 1 && SHARED_RP) load_tw((j0 * T) / J);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float2 t[T];
#pragma unroll
          for (int r = 0; r < T; ++r) t[r] = v[r][q];
          small_dft<T, SIGN>(t);
          const int j = j0 + q;
          if constexpr (T > 1 && !SHARED_RP) load_tw((j * T) / J);
#pragma unroll
          for (int c = 1; c < T; ++c) t[c] = cmulf(t[c], wt[c]);
          if constexpr (!LINE_MINOR && T > 1) {
            st_run<T>(re, im, Tl::off(g, j * T), t);  // T consecutive columns of K row rp
          } else {
#pragma unroll
            for (int c = 0; c < T; ++c) st_pair(re, im, Tl::off(g, j * T + c), t[c]);
          }
        }
      }
    }
  } else {
    constexpr int GQ = G / 4;
    constexpr int ITEMS = GQ * (L / T);
#pragma unroll 2
    for (int it = tid; it < ITEMS; it += NT) {
      const int j = it / GQ;
      const int g0 = (it % GQ) * 4;
      uint4 w[T];
#pragma unroll
      for (int r = 0; r < T; ++r)
        w[r] = *reinterpret_cast<const uint4*>(raw + (static_cast<uint32_t>(j + r * (L / T)) * G + g0) * 4u);
      if constexpr (T == 1 && LINE_MINOR) {
        uint2 rr, ii;
        rr.x = __byte_perm(w[0].x, w[0].y, 0x5410);
        rr.y = __byte_perm(w[0].z, w[0].w, 0x5410);
        ii.x = __byte_perm(w[0].x, w[0].y, 0x7632);
        ii.y = __byte_perm(w[0].z, w[0].w, 0x7632);
        const uint32_t off = Tl::off(g0, j);
        *reinterpret_cast<uint2*>(re + off) = rr;
        *reinterpret_cast<uint2*>(im + off) = ii;
      } else {
        float2 v[T][4];
#pragma unroll
        for (int r = 0; r < T; ++r) unpack_h2x4(w[r], v[r]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float2 t[T];
#pragma unroll
          for (int r = 0; r < T; ++r) t[r] = v[r][q];
          small_dft<T, SIGN>(t);
#pragma unroll
          for (int r = 0; r < T; ++r) v[r][q] = t[r];
        }
#pragma unroll
        for (int c = 0; c < T; ++c) {
          const int lp = j * T + c;
          float2 x[4] = {v[c][0], v[c][1], v[c][2], v[c][3]};
          if constexpr (T > 1) {
            const int rp = lp / J, jp = lp % J;
            const float2 tw = __ldg(core.tw + rp * (jp % T) * (L / (16 * T)));
#pragma unroll
            for (int q = 0; q < 4; ++q) x[q] = cmulf(x[q], tw);
          }
          if constexpr (LINE_MINOR) {
            st_quad(re, im, Tl::off(g0, lp), x);
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) st_pair(re, im, Tl::off(g0 + q, lp), x[q]);
          }
        }
      }
    }
  }
}

// NT: threads per CTA (256, or 128 for 256-row tiles run 6 CTAs per SM).
template <int L, int G, bool LINE_MINOR, int SIGN, class IO, int MINB = 3, int NT = kPassThreads>
__global__ void __launch_bounds__(NT, MINB) fft_pass_f16_pf(const __grid_constant__ IO io, const PassCore core) {
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr uint32_t TMEM_COLS = pass_tmem_cols<L, G>();
  static_assert(TMEM_COLS >= 32 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  static_assert(G % 4 == 0 || IO::IN_VEC_L, "line-vectorised loads need G % 4 == 0");
  PassState st;
  pass_setup<TMEM_COLS>(st, core.bmat);
  uint8_t* re = st.smem + kPlaneOffset;
  uint8_t* im = re + Tl::PLANE;
  uint8_t* raw = re + 2 * Tl::PLANE;
  const bool stage_out = IO::OUT_VEC_L && io.out_contig && !LINE_MINOR;
  const bool tma_in = (IO::IN_VEC_L && io.in_contig) || tensor_in(io);
  const bool tensor_store = LINE_MINOR && tensor_out(io);
  const long long ntiles = (io.total_lines + G - 1) / G;
  long long tile = blockIdx.x;
  bool pending = false;
  if (tile < ntiles) {
    prefetch_tile<L, G, LINE_MINOR, IO, NT>(st, io, tile * G, raw);
    pending = true;
  }
  for (; tile < ntiles; tile += gridDim.x) {
    const long long line0 = tile * G;
    const long long rem = io.total_lines - line0;
    const int nval = rem < G ? static_cast<int>(rem) : G;
    if (!wait_prefetch(st, io, core)) {
      pending = false;
      break;
    }
    pending = false;
    if ((stage_out || tensor_store) && threadIdx.x == 0) bulk_wait_read_all();  // previous store has read the planes
    __syncthreads();
    permute_raw<L, G, LINE_MINOR, SIGN, IO, NT>(raw, re, im, core, nval);
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();
    if (tile + gridDim.x < ntiles) {
      prefetch_tile<L, G, LINE_MINOR, IO, NT>(st, io, (tile + gridDim.x) * G, raw);
      pending = true;
    }
    if (!run_stages<L, G, LINE_MINOR, SIGN, IO, NT>(st, io, core, line0, re, im, stage_out)) break;
    if (stage_out && threadIdx.x == 0) {
      bulk_s2g(io.tile_dst(line0), re, static_cast<uint32_t>(nval) * L * 4u);
      bulk_commit();
    }
    if constexpr (TensorMapIo<IO> && LINE_MINOR) {
      if (tensor_store && threadIdx.x == 0) {
        constexpr int BY = L < 256 ? L : 256;
        const int seq = static_cast<int>(line0 >> io.lps_log2);
        const int x0 = static_cast<int>(line0 & ((1ll << io.lps_log2) - 1));
#pragma unroll
        for (int r0 = 0; r0 < L; r0 += BY) tma_store_3d(&io.out_map, re + static_cast<uint32_t>(r0) * G * 4u, x0, r0, seq);
        bulk_commit();
      }
    }
  }
  // an early exit may leave a prefetch in flight: let it land before the CTA ends
  if (pending) {
    if (tma_in) {
      mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u);
    } else {
      cp_async_wait_all();
    }
  }
  pass_teardown<TMEM_COLS>(st);
}

template <int L, int G>
constexpr int pass_pf_smem_bytes() {
  return static_cast<int>(kPlaneOffset) + 4 * (G * L / 16) * 32 + 1024;
}

// Dynamic shared memory bytes for a pass kernel instance (+1 KB alignment slack).
template <int L, int G>
constexpr int pass_smem_bytes() {
  return static_cast<int>(kPlaneOffset) + 2 * (G * L / 16) * 32 + 1024;
}

}  // namespace tcfft
