// Global-memory IO policies for the pass kernel.
//
// A policy tells the pass kernel where line `line`, element `l` lives and how
// to convert it. Lines are numbered 0..total_lines-1; line -> (sequence,
// line-in-sequence) uses lines_per_seq = 2^lps_log2. Vector accesses move four
// complex elements: four consecutive elements of one line ("_l") or the same
// element of four adjacent lines ("_g", lines adjacent in memory).
//
// Interface used by fft_pass_f16:
//   IN_VEC_L / OUT_VEC_L, Raw, total_lines,
//   Raw  fetch_l(line, l0, ok) / fetch_g(line0, l, ok)   (issue global loads)
//   void decode_l(raw, line, l0, v[4]) / decode_g(...)   (to FP32)
//   void store_row16(line, j, J, v[16])   (outputs l = j + c*J, c = 0..15)
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>
#include <cstdint>

#include "fft_tile.cuh"

namespace tcfft {

__device__ __forceinline__ uint4 ldg_nc_v4(const void* p) {
  uint4 r;
  asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}

// L2-coherent load (skips L1): for data written earlier in the same kernel by
// other CTAs (the fused four-step workspace).
__device__ __forceinline__ uint4 ldg_cg_v4(const void* p) {
  uint4 r;
  asm volatile("ld.global.cg.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p)
               : "memory");
  return r;
}

__device__ __forceinline__ void stg_v4(void* p, uint4 v) {
  asm volatile("st.global.v4.u32 [%0], {%1,%2,%3,%4};" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

__device__ __forceinline__ uint4 pack_h2x4(const float2 (&x)[4]) {
  uint4 r;
  __half2 h0 = __floats2half2_rn(x[0].x, x[0].y), h1 = __floats2half2_rn(x[1].x, x[1].y);
  __half2 h2 = __floats2half2_rn(x[2].x, x[2].y), h3 = __floats2half2_rn(x[3].x, x[3].y);
  r.x = *reinterpret_cast<uint32_t*>(&h0);
  r.y = *reinterpret_cast<uint32_t*>(&h1);
  r.z = *reinterpret_cast<uint32_t*>(&h2);
  r.w = *reinterpret_cast<uint32_t*>(&h3);
  return r;
}

// Outer (four-step) twiddle W_N^{(x*y) mod N} from two FP32 tables:
// W_N^e = hi[e >> shift] * lo[e & (2^shift - 1)].
struct OuterTwiddle {
  const float2* hi = nullptr;
  const float2* lo = nullptr;
  int shift = 0;
  int logn = 0;
  __device__ __forceinline__ float2 operator()(long long x, long long y) const {
    const unsigned long long e =
        (static_cast<unsigned long long>(x) * static_cast<unsigned long long>(y)) & ((1ull << logn) - 1ull);
    return cmulf(__ldg(hi + (e >> shift)), __ldg(lo + (e & ((1ull << shift) - 1ull))));
  }
};

// Interleaved complex half in and out, arbitrary strides (in elements).
// COHERENT: input is read with L2-coherent loads (it is written by other CTAs
// of the same launch).
template <bool IN_L, bool OUT_L, bool COHERENT = false>
struct IoHalf {
  static constexpr bool IN_VEC_L = IN_L;
  static constexpr bool OUT_VEC_L = OUT_L;
  using Raw = uint4;

  const half2* in;
  half2* out;
  long long total_lines;
  int lps_log2;
  long long in_seq, in_line, in_elem;
  long long out_seq, out_line, out_elem;
  OuterTwiddle otw;  // applied on store when otw.hi != nullptr: W_N^{li * l}
  float scale;
  // Tile contiguity: element (line, l) at in + line * L + l (resp. out), so a
  // tile of lines moves as one bulk copy. Set by the host.
  bool in_contig, out_contig;
  long long contig_len;  // L
  // Column-layout tiles (lines adjacent in memory, in_line / out_line == 1)
  // moved by TMA through 3D tensor maps: x = line within its sequence,
  // y = element of the line, z = sequence; 4-byte elements. Set by the host
  // for the prefetching kernels only (the kernel parameter is
  // __grid_constant__, so the maps stay in parameter space).
  bool in_tma, out_tma;
  CUtensorMap in_map, out_map;

  __device__ __forceinline__ const half2* tile_src(long long line0) const { return in + line0 * contig_len; }
  __device__ __forceinline__ half2* tile_dst(long long line0) const { return out + line0 * contig_len; }

  __device__ __forceinline__ long long in_base(long long line) const {
    return (line >> lps_log2) * in_seq + (line & ((1ll << lps_log2) - 1)) * in_line;
  }
  __device__ __forceinline__ long long out_base(long long line) const {
    return (line >> lps_log2) * out_seq + (line & ((1ll << lps_log2) - 1)) * out_line;
  }
  __device__ __forceinline__ Raw fetch_l(long long line, int l0, bool ok) const {
    if (!ok || line >= total_lines) return make_uint4(0, 0, 0, 0);
    if constexpr (COHERENT) return ldg_cg_v4(in + in_base(line) + l0);
    return ldg_nc_v4(in + in_base(line) + l0);
  }
  __device__ __forceinline__ Raw fetch_g(long long line0, int l, bool ok) const {
    if (!ok || line0 >= total_lines) return make_uint4(0, 0, 0, 0);
    if constexpr (COHERENT) return ldg_cg_v4(in + in_base(line0) + static_cast<long long>(l) * in_elem);
    return ldg_nc_v4(in + in_base(line0) + static_cast<long long>(l) * in_elem);
  }
  // Source of the 16-byte chunk at element l of 4 adjacent lines / at
  // elements l0..l0+3 of one line, for asynchronous copies; ok = false when
  // the lines lie past the end (the copy then zero-fills).
  __device__ __forceinline__ const void* src_g(long long line0, int l, bool& ok) const {
    ok = line0 < total_lines;
    return ok ? static_cast<const void*>(in + in_base(line0) + static_cast<long long>(l) * in_elem)
              : static_cast<const void*>(in);
  }
  __device__ __forceinline__ const void* src_l(long long line, int l0, bool& ok) const {
    ok = line < total_lines;
    return ok ? static_cast<const void*>(in + in_base(line) + l0) : static_cast<const void*>(in);
  }
  __device__ __forceinline__ void decode_l(const Raw& r, long long, int, float2 (&v)[4]) const {
    unpack_h2x4(r, v);
  }
  __device__ __forceinline__ void decode_g(const Raw& r, long long, int, float2 (&v)[4]) const {
    unpack_h2x4(r, v);
  }
  // The outer twiddle and scale store_row16 applies, in place (for outputs
  // that go out through a staged tensor store instead).
  __device__ __forceinline__ void prepare_row16(long long line, int j, int J, float2 (&v)[16]) const {
    if (otw.hi) outer_twiddle16(line, j, J, v);
    if (scale != 1.0f) {
#pragma unroll
      for (int c = 0; c < 16; ++c) v[c] = make_float2(v[c].x * scale, v[c].y * scale);
    }
  }
  // Outputs l = j + c*J (c = 0..15) of one line. The outer twiddle
  // W_N^{li*l} is formed as W_N^{li*j} * (W_N^{li*J})^c (FP32 recurrence).
  // v[c] *= W_N^{li*(j + c*J)} for c = 0..15: W_N^{li*j} * (W_N^{li*J})^c,
  // an FP32 recurrence over pairs of outputs (packed instructions).
  __device__ __forceinline__ void outer_twiddle16(long long line, int j, int J, float2 (&v)[16]) const {
    const long long li = line & ((1ll << lps_log2) - 1);
    TwPairSeq tws(otw(li, j), otw(li, J));
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
      float2 yr, yi;
      cmul_pair(make_float2(v[c].x, v[c + 1].x), make_float2(v[c].y, v[c + 1].y), tws.w, yr, yi);
      if (c + 2 < 16) tws.next();
      v[c] = make_float2(yr.x, yi.x);
      v[c + 1] = make_float2(yr.y, yi.y);
    }
  }
  __device__ __forceinline__ void store_row16(long long line, int j, int J, float2 (&v)[16]) const {
    half2* p = out + out_base(line);
    if (otw.hi) outer_twiddle16(line, j, J, v);
    const long long step = static_cast<long long>(J) * out_elem;
    half2* q = p + static_cast<long long>(j) * out_elem;
    if (scale == 1.0f) {
#pragma unroll
      for (int c = 0; c < 16; ++c) q[c * step] = __floats2half2_rn(v[c].x, v[c].y);
    } else {
#pragma unroll
      for (int c = 0; c < 16; ++c) q[c * step] = __floats2half2_rn(v[c].x * scale, v[c].y * scale);
    }
  }
};

}  // namespace tcfft
