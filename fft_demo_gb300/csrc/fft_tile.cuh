// Tensor-core FFT "pass" kernel for sm_103a.
//
// A pass transforms many independent lines of length L (power of two,
// 16 <= L <= 16384) that live in global memory with arbitrary
// (sequence, line, element) strides. One CTA owns a tile of G lines in shared
// memory and runs the whole length-L transform on it:
//
//   load   : global -> registers -> shared. A radix-T first stage
//            (T = L / 16^S in {1,2,4,8}) runs here on the CUDA cores in FP32,
//            followed by the twiddle of the first radix-16 stage.
//   stages : S radix-16 stages. Each is one batch of tcgen05 MMAs
//            D[m][n] = sum_k A[m][k] B[k][n] with
//              A = the tile in MN-major 128B-swizzled layout: K row r (0..15)
//                  holds input r of every butterfly m; real and imaginary
//                  parts are separate planes (two K=16 MMAs),
//              B = the 16-point DFT as a 32x32 real matrix (FP16),
//              D = FP32 accumulator in TMEM: lane m, 16 real + 16 imaginary
//                  outputs.
//            The epilogue reads D (tcgen05.ld), applies the next stage's
//            twiddle in FP32, rounds once to FP16 and scatters into the next
//            stage's positions (Stockham autosort order).
//   store  : shared -> global in natural order, with an optional outer
//            twiddle (four-step) and scale.
//
// Method (radix-16 DFT stages on tensor cores, twiddles between stages,
// radix-2/4/8 tail on CUDA cores) follows tcfft_half.cu:70-1175 of
// yuelingfan/fft_demo; the data layout, autosort order, FP32 accumulation and
// TMEM staging are this library's own.
#pragma once
#include <cuda_fp16.h>
#include <cstdint>

#include "tc_ptx.cuh"

namespace tcfft {

constexpr int kPassThreads = 256;

// Error word bits set by kernels (read back by the host after a launch).
enum : int { kErrMmaTimeout = 1, kErrBadArgs = 2 };

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

struct PassArgs {
  const void* in;
  void* out;
  long long total_lines;    // lines in the whole pass
  long long lines_per_seq;  // lines per sequence (line index -> (seq, line))
  long long in_seq_stride, in_line_stride, in_elem_stride;  // in elements
  long long out_seq_stride, out_line_stride, out_elem_stride;
  const float2* tw;        // W_L^e (this direction), e in [0, L)
  const uint32_t* bmat;    // 2 KB image of B for this direction
  // Outer (four-step) twiddle applied on store: W_N^{(line % lines_per_seq) * l}
  // factored as otw_hi[e >> otw_shift] * otw_lo[e & ((1 << otw_shift) - 1)],
  // e = product mod N (N = 2^otw_logn). Null = none.
  const float2* otw_hi;
  const float2* otw_lo;
  int otw_shift;
  int otw_logn;
  float scale;  // applied on store (1.0f = none)
  int* err;
};

// Row position m (0..Mt-1) of butterfly j of line g.
template <int L, int G, bool LINE_MINOR>
__device__ __forceinline__ int bfly_pos(int g, int j) {
  return LINE_MINOR ? j * G + g : g * LineShape<L>::J + j;
}

template <int L, int G, bool LINE_MINOR>
__device__ __forceinline__ void bfly_of_pos(int m, int& g, int& j) {
  if (LINE_MINOR) {
    j = m / G;
    g = m % G;
  } else {
    g = m / LineShape<L>::J;
    j = m % LineShape<L>::J;
  }
}

// Byte offset (within a plane) of logical element l of line g.
template <int L, int G, bool LINE_MINOR>
__device__ __forceinline__ uint32_t elem_off(int g, int l) {
  constexpr int Mt = G * L / 16;
  constexpr uint32_t KSTRIDE = (Mt / 64) * 1024;
  const int k = l / LineShape<L>::J;
  const int m = bfly_pos<L, G, LINE_MINOR>(g, l % LineShape<L>::J);
  return sw128_mn_offset(k, m, 1024u, KSTRIDE);
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 h2f(__half2 h) { return __half22float2(h); }

// In-register radix-T DFT (T in {1,2,4,8}), sign = -1 forward, +1 inverse.
template <int T, int SIGN>
__device__ __forceinline__ void small_dft(float2 (&v)[T]) {
  if constexpr (T == 1) {
    return;
  } else if constexpr (T == 2) {
    float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
  } else if constexpr (T == 4) {
    // y_c = sum_r v_r * w^{rc}, w = exp(SIGN * i*pi/2)
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
    // radix-8 as 2 x radix-4 (even / odd inputs) + twiddles W8^c
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    small_dft<4, SIGN>(e);
    small_dft<4, SIGN>(o);
    const float h = 0.70710678118654752f;
    // W8^c for c = 0..3 (SIGN = -1: exp(-i*pi*c/4))
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

template <typename T>
__device__ __forceinline__ T ldg_vec(const T* p) {
  return __ldg(p);
}

// Twiddle applied to element l' (logical index written for the next
// radix-16 stage whose Ns is NSN): W_{16*NSN}^{r' * (j' mod NSN)}.
template <int L, int NSN>
__device__ __forceinline__ float2 next_twiddle(const float2* __restrict__ tw, int lp) {
  constexpr int J = LineShape<L>::J;
  const int rp = lp / J;
  const int jp = lp % J;
  const int e = rp * (jp % NSN) * (L / (16 * NSN));
  return __ldg(tw + e);
}

__device__ __forceinline__ void st_half_pair(uint8_t* re_plane, uint8_t* im_plane, uint32_t off,
                                             float2 v) {
  *reinterpret_cast<__half*>(re_plane + off) = __float2half_rn(v.x);
  *reinterpret_cast<__half*>(im_plane + off) = __float2half_rn(v.y);
}

// Outer four-step twiddle W_N^{e}, e = (a * b) mod N.
__device__ __forceinline__ float2 outer_twiddle(const PassArgs& a, long long x, long long y) {
  const unsigned long long mask = (1ull << a.otw_logn) - 1ull;
  const unsigned long long e = (static_cast<unsigned long long>(x) * static_cast<unsigned long long>(y)) & mask;
  const unsigned long long lo_mask = (1ull << a.otw_shift) - 1ull;
  float2 hi = __ldg(a.otw_hi + (e >> a.otw_shift));
  float2 lo = __ldg(a.otw_lo + (e & lo_mask));
  return cmulf(hi, lo);
}

// ---------------------------------------------------------------------------
// The pass kernel (FP16 storage; FP32 accumulation and twiddles).
//   L          line length
//   G          lines per tile (G * L / 16 must be 128, 256, 512 or 1024)
//   LINE_MINOR butterfly order in the tile (true for column passes)
//   IN_VEC_L   true: vector loads along the line (in_elem_stride == 1);
//              false: along 4 adjacent lines (in_line_stride == 1)
//   OUT_VEC_L  same for stores
//   SIGN       -1 forward, +1 inverse
// ---------------------------------------------------------------------------
template <int L, int G, bool LINE_MINOR, bool IN_VEC_L, bool OUT_VEC_L, int SIGN>
__global__ void __launch_bounds__(kPassThreads, 2) fft_pass_f16(const PassArgs a) {
  using Sh = LineShape<L>;
  constexpr int T = Sh::T;
  constexpr int S = Sh::S;
  constexpr int J = Sh::J;
  constexpr int Mt = G * L / 16;
  constexpr int NG = Mt / 128;
  constexpr uint32_t PLANE = Mt * 32;  // bytes per plane (16 rows x Mt halves)
  constexpr uint32_t KSTRIDE = (Mt / 64) * 1024;
  constexpr uint32_t TMEM_COLS = NG * 32;
  static_assert(Mt % 128 == 0 && Mt <= 1024, "tile size");
  static_assert(TMEM_COLS >= 32 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  static_assert(G % 4 == 0 || IN_VEC_L, "line-vectorised loads need G % 4 == 0");
  static_assert(G % 4 == 0 || OUT_VEC_L, "line-vectorised stores need G % 4 == 0");
  constexpr uint32_t IDESC = make_idesc_f16_f32(128, 32, true, false);

  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  uint8_t* re_plane = smem;
  uint8_t* im_plane = smem + PLANE;
  uint8_t* bmat = smem + 2 * PLANE;                               // 2 KB
  uint64_t* mbar = reinterpret_cast<uint64_t*>(bmat + 2048);      // 8 B
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bmat + 2048 + 16);
  int* sflag = reinterpret_cast<int*>(bmat + 2048 + 32);

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;

  // ---- one-time setup: B matrix, mbarrier, TMEM ----
  for (int i = tid; i < 512; i += kPassThreads)
    reinterpret_cast<uint32_t*>(bmat)[i] = __ldg(a.bmat + i);
  if (tid == 0) {
    mbar_init(mbar, 1);
    *sflag = 0;
  }
  if (warp == 0) {
    tmem_alloc(tslot, TMEM_COLS);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t tbase = *tslot;
  uint32_t phase = 0;

  const long long ntiles = (a.total_lines + G - 1) / G;
  const half2* __restrict__ gin = reinterpret_cast<const half2*>(a.in);
  half2* __restrict__ gout = reinterpret_cast<half2*>(a.out);

  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long line0 = tile * G;

    // ================= load (+ radix-T stage) =================
    if constexpr (IN_VEC_L) {
      // work item = (line g, quad of butterflies j0..j0+3 of the radix-T stage)
      constexpr int QPL = (L / T) / 4;  // quads per line
      for (int it = tid; it < G * QPL; it += kPassThreads) {
        const int g = it / QPL;
        const int j0 = (it % QPL) * 4;
        const long long line = line0 + g;
        float2 v[4][T];
        if (line < a.total_lines) {
          const long long seq = line / a.lines_per_seq;
          const long long li = line % a.lines_per_seq;
          const half2* base = gin + seq * a.in_seq_stride + li * a.in_line_stride;
#pragma unroll
          for (int r = 0; r < T; ++r) {
            const uint4 raw = *reinterpret_cast<const uint4*>(base + (j0 + r * (L / T)));
            const half2* hp = reinterpret_cast<const half2*>(&raw);
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q][r] = h2f(hp[q]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int r = 0; r < T; ++r) v[q][r] = make_float2(0.f, 0.f);
        }
        if constexpr (T == 1) {
          // four consecutive l -> four consecutive m in the same K row (J >= 4)
          const uint32_t off = elem_off<L, G, LINE_MINOR>(g, j0);
          if constexpr (!LINE_MINOR && J >= 4) {
            __half2 r01 = __floats2half2_rn(v[0][0].x, v[1][0].x);
            __half2 r23 = __floats2half2_rn(v[2][0].x, v[3][0].x);
            __half2 i01 = __floats2half2_rn(v[0][0].y, v[1][0].y);
            __half2 i23 = __floats2half2_rn(v[2][0].y, v[3][0].y);
            uint2 rr, ii;
            rr.x = *reinterpret_cast<uint32_t*>(&r01);
            rr.y = *reinterpret_cast<uint32_t*>(&r23);
            ii.x = *reinterpret_cast<uint32_t*>(&i01);
            ii.y = *reinterpret_cast<uint32_t*>(&i23);
            *reinterpret_cast<uint2*>(re_plane + off) = rr;
            *reinterpret_cast<uint2*>(im_plane + off) = ii;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              st_half_pair(re_plane, im_plane, elem_off<L, G, LINE_MINOR>(g, j0 + q), v[q][0]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            small_dft<T, SIGN>(v[q]);
#pragma unroll
            for (int c = 0; c < T; ++c) {
              const int lp = (j0 + q) * T + c;
              float2 w = next_twiddle<L, T>(a.tw, lp);
              st_half_pair(re_plane, im_plane, elem_off<L, G, LINE_MINOR>(g, lp), cmulf(v[q][c], w));
            }
          }
        }
      }
    } else {
      // work item = (quad of adjacent lines g0..g0+3, butterfly j of the radix-T stage)
      constexpr int GQ = G / 4;
      for (int it = tid; it < GQ * (L / T); it += kPassThreads) {
        const int j = it / GQ;
        const int g0 = (it % GQ) * 4;
        const long long line = line0 + g0;
        float2 v[4][T];
        if (line < a.total_lines) {
          const long long seq = line / a.lines_per_seq;
          const long long li = line % a.lines_per_seq;
          const half2* base = gin + seq * a.in_seq_stride + li * a.in_line_stride;
#pragma unroll
          for (int r = 0; r < T; ++r) {
            const uint4 raw =
                *reinterpret_cast<const uint4*>(base + static_cast<long long>(j + r * (L / T)) * a.in_elem_stride);
            const half2* hp = reinterpret_cast<const half2*>(&raw);
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q][r] = h2f(hp[q]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int r = 0; r < T; ++r) v[q][r] = make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) small_dft<T, SIGN>(v[q]);
#pragma unroll
        for (int c = 0; c < T; ++c) {
          const int lp = j * T + c;
          float2 w = make_float2(1.f, 0.f);
          if constexpr (T > 1) w = next_twiddle<L, T>(a.tw, lp);
          if constexpr (LINE_MINOR) {
            // 4 adjacent lines -> 4 consecutive m in the same K row
            const uint32_t off = elem_off<L, G, LINE_MINOR>(g0, lp);
            float2 x0 = cmulf(v[0][c], w), x1 = cmulf(v[1][c], w), x2 = cmulf(v[2][c], w),
                   x3 = cmulf(v[3][c], w);
            __half2 r01 = __floats2half2_rn(x0.x, x1.x), r23 = __floats2half2_rn(x2.x, x3.x);
            __half2 i01 = __floats2half2_rn(x0.y, x1.y), i23 = __floats2half2_rn(x2.y, x3.y);
            uint2 rr, ii;
            rr.x = *reinterpret_cast<uint32_t*>(&r01);
            rr.y = *reinterpret_cast<uint32_t*>(&r23);
            ii.x = *reinterpret_cast<uint32_t*>(&i01);
            ii.y = *reinterpret_cast<uint32_t*>(&i23);
            *reinterpret_cast<uint2*>(re_plane + off) = rr;
            *reinterpret_cast<uint2*>(im_plane + off) = ii;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              st_half_pair(re_plane, im_plane, elem_off<L, G, LINE_MINOR>(g0 + q, lp), cmulf(v[q][c], w));
          }
        }
      }
    }
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();

    // ================= radix-16 tensor-core stages =================
    bool timed_out = false;
#pragma unroll 1
    for (int s = 0; s < S; ++s) {
      if (tid == 0) {
        tc_fence_after_sync();
        const uint32_t a0 = smem_u32(re_plane), a1 = smem_u32(im_plane), b0 = smem_u32(bmat);
#pragma unroll 1
        for (int grp = 0; grp < NG; ++grp) {
          const uint64_t ad0 = make_sdesc(a0 + grp * 2048u, 1024u, KSTRIDE, kLayoutSw128);
          const uint64_t ad1 = make_sdesc(a1 + grp * 2048u, 1024u, KSTRIDE, kLayoutSw128);
          const uint64_t bd0 = make_sdesc(b0, 128u, 512u, kLayoutNone);
          const uint64_t bd1 = make_sdesc(b0 + 256u, 128u, 512u, kLayoutNone);
          umma_f16(tbase + grp * 32u, ad0, bd0, IDESC, 0u);
          umma_f16(tbase + grp * 32u, ad1, bd1, IDESC, 1u);
        }
        umma_commit(mbar);
      }
      if (!mbar_wait_bounded(mbar, phase & 1u)) {
        timed_out = true;
        if (lane == 0) atomicOr(a.err, kErrMmaTimeout);
      }
      phase++;
      if (__syncthreads_or(timed_out)) {
        timed_out = true;
        break;
      }
      tc_fence_after_sync();

      // Ns of this stage = T * 16^s ; next stage Ns' = 16 * Ns
      const int Ns = T << (4 * s);
      const bool last = (s == S - 1);
      for (int grp = warp >> 2; grp < NG; grp += kPassThreads / 128) {
        uint32_t d[32];
        tmem_ld_x32(tbase + (static_cast<uint32_t>(32 * (warp & 3)) << 16) + grp * 32u, d);
        tmem_ld_wait();
        const int m = grp * 128 + 32 * (warp & 3) + lane;
        int g, j;
        bfly_of_pos<L, G, LINE_MINOR>(m, g, j);
        if (last) {
          // final outputs l' = j + c*J: same butterfly column, K row c
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const uint32_t off = sw128_mn_offset(c, m, 1024u, KSTRIDE);
            st_half_pair(re_plane, im_plane, off,
                         make_float2(__uint_as_float(d[c]), __uint_as_float(d[16 + c])));
          }
        } else {
          const int ja = j / Ns, jb = j % Ns;
          const int NsN = Ns * 16;
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const int lp = ja * 16 * Ns + c * Ns + jb;
            const int rp = lp / J, jp = lp % J;
            const int e = rp * (jp % NsN) * (L / (16 * NsN));
            const float2 w = __ldg(a.tw + e);
            const float2 x = cmulf(make_float2(__uint_as_float(d[c]), __uint_as_float(d[16 + c])), w);
            st_half_pair(re_plane, im_plane, sw128_mn_offset(rp, bfly_pos<L, G, LINE_MINOR>(g, jp), 1024u, KSTRIDE), x);
          }
        }
      }
      fence_proxy_async_smem();
      tc_fence_before_sync();
      __syncthreads();
    }
    if (timed_out) break;

    // ================= store =================
    const bool do_otw = a.otw_hi != nullptr;
    if constexpr (OUT_VEC_L) {
      constexpr int QPL = L / 4;
      for (int it = tid; it < G * QPL; it += kPassThreads) {
        const int g = it / QPL;
        const int l0 = (it % QPL) * 4;
        const long long line = line0 + g;
        if (line >= a.total_lines) continue;
        const long long seq = line / a.lines_per_seq;
        const long long li = line % a.lines_per_seq;
        half2 o[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t off = elem_off<L, G, LINE_MINOR>(g, l0 + q);
          float2 x = make_float2(__half2float(*reinterpret_cast<const __half*>(re_plane + off)),
                                 __half2float(*reinterpret_cast<const __half*>(im_plane + off)));
          if (do_otw) x = cmulf(x, outer_twiddle(a, li, l0 + q));
          x.x *= a.scale;
          x.y *= a.scale;
          o[q] = __floats2half2_rn(x.x, x.y);
        }
        half2* dst = gout + seq * a.out_seq_stride + li * a.out_line_stride + l0;
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<uint4*>(o);
      }
    } else {
      constexpr int GQ = G / 4;
      for (int it = tid; it < GQ * L; it += kPassThreads) {
        const int l = it / GQ;
        const int g0 = (it % GQ) * 4;
        const long long line = line0 + g0;
        if (line >= a.total_lines) continue;
        const long long seq = line / a.lines_per_seq;
        const long long li = line % a.lines_per_seq;
        half2 o[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t off = elem_off<L, G, LINE_MINOR>(g0 + q, l);
          float2 x = make_float2(__half2float(*reinterpret_cast<const __half*>(re_plane + off)),
                                 __half2float(*reinterpret_cast<const __half*>(im_plane + off)));
          if (do_otw) x = cmulf(x, outer_twiddle(a, li + q, l));
          x.x *= a.scale;
          x.y *= a.scale;
          o[q] = __floats2half2_rn(x.x, x.y);
        }
        half2* dst = gout + seq * a.out_seq_stride + li * a.out_line_stride +
                     static_cast<long long>(l) * a.out_elem_stride;
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<uint4*>(o);
      }
    }
    __syncthreads();
  }

  // ---- teardown ----
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, TMEM_COLS);
}

// Dynamic shared memory bytes for a pass kernel instance (+1 KB alignment slack).
template <int L, int G>
constexpr int pass_smem_bytes() {
  return 2 * (G * L / 16) * 32 + 2048 + 64 + 1024;
}

}  // namespace tcfft
