// Split-precision pass kernel: FP32 data, tensor-core arithmetic on FP16
// (hi, lo) pairs.
//
// Every value v held in shared memory is stored as two FP16 numbers with a
// per-tile power-of-two scale 2^sigma:
//     v * 2^sigma = hi + lo,  hi = fp16(v * 2^sigma),  lo = fp16(v * 2^sigma - hi)
// and so is the DFT matrix B = B_hi + B_lo. Each radix-16 stage runs, per
// plane (real, imaginary), two K = 16 MMAs with N = 64 against [B_hi | B_lo]:
//     D[:, 0:32]  += A_hi * B_hi + A_lo * B_hi
//     D[:, 32:64] += A_hi * B_lo + A_lo * B_lo
// (four MMAs per 128 rows) and the epilogue adds the two halves in FP32: the
// full product (A_hi + A_lo)(B_hi + B_lo). sigma is
// chosen per tile from the input's largest magnitude (largest value ->
// <= 2^14 after the radix-T stage), so lo stays in FP16's normal range for
// every value within 2^17 of the tile's maximum; each radix-16 stage scales
// its output by 2^-4 (its largest possible growth is 16), so no FP16
// operand overflows.
#pragma once
#include "fft_io.cuh"
#include "fft_tile.cuh"

namespace tcfft {

struct SplitPlanes {
  uint8_t *rh, *ih, *rl, *il;
};

__device__ __forceinline__ void split_f(float v, __half& hi, __half& lo) {
  hi = __float2half_rn(v);
  lo = __float2half_rn(v - __half2float(hi));
}

// hi / lo halves of two values at once (packed instructions): hi = rn16(y),
// lo = rn16(y - hi), the difference exact in FP32
__device__ __forceinline__ void split_pair(float2 y, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __float22half2_rn(y);
  const float2 f = __half22float2(h);
  const __half2 l = __float22half2_rn(f2fma(f, f2bcast(-1.f), y));
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

__device__ __forceinline__ void st_pair_split(const SplitPlanes& P, uint32_t off, float2 v) {
  __half a, b, c, d;
  split_f(v.x, a, b);
  split_f(v.y, c, d);
  *reinterpret_cast<__half*>(P.rh + off) = a;
  *reinterpret_cast<__half*>(P.rl + off) = b;
  *reinterpret_cast<__half*>(P.ih + off) = c;
  *reinterpret_cast<__half*>(P.il + off) = d;
}

// N consecutive m in one K row (N = 2, 4, 8; offset 2N-byte aligned, inside
// one 16-byte chunk): one 2N-byte store per plane.
template <int N>
__device__ __forceinline__ void st_run_split(const SplitPlanes& P, uint32_t off, const float2 (&x)[N]) {
  static_assert(N == 2 || N == 4 || N == 8, "run length");
  uint32_t rh[N / 2], rl[N / 2], ih[N / 2], il[N / 2];
#pragma unroll
  for (int k = 0; k < N / 2; ++k) {
    split_pair(make_float2(x[2 * k].x, x[2 * k + 1].x), rh[k], rl[k]);
    split_pair(make_float2(x[2 * k].y, x[2 * k + 1].y), ih[k], il[k]);
  }
  auto put = [&](uint8_t* plane, const uint32_t (&w)[N / 2]) {
    if constexpr (N == 2) {
      *reinterpret_cast<uint32_t*>(plane + off) = w[0];
    } else if constexpr (N == 4) {
      *reinterpret_cast<uint2*>(plane + off) = make_uint2(w[0], w[1]);
    } else {
      *reinterpret_cast<uint4*>(plane + off) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  };
  put(P.rh, rh);
  put(P.ih, ih);
  put(P.rl, rl);
  put(P.il, il);
}

// four consecutive m in one K row (8-byte aligned)
__device__ __forceinline__ void st_quad_split(const SplitPlanes& P, uint32_t off, const float2 (&x)[4]) {
  st_run_split<4>(P, off, x);
}

// Two outputs (real parts yr, imaginary parts yi, as pairs) split into the
// four planes at two 2-byte positions o0 (first output) and o1 (second).
__device__ __forceinline__ void st_two_split(const SplitPlanes& P, uint32_t o0, uint32_t o1, float2 yr, float2 yi) {
  uint32_t rh, rl, ih, il;
  split_pair(yr, rh, rl);
  split_pair(yi, ih, il);
  auto put = [&](uint8_t* plane, uint32_t w) {
    *reinterpret_cast<uint16_t*>(plane + o0) = static_cast<uint16_t>(w & 0xffffu);
    *reinterpret_cast<uint16_t*>(plane + o1) = static_cast<uint16_t>(w >> 16);
  };
  put(P.rh, rh);
  put(P.ih, ih);
  put(P.rl, rl);
  put(P.il, il);
}

__device__ __forceinline__ float max_abs4(const float2 (&v)[4]) {
  float m = 0.f;
#pragma unroll
  for (int q = 0; q < 4; ++q) m = fmaxf(m, fmaxf(fabsf(v[q].x), fabsf(v[q].y)));
  return m;
}

// IO types whose row store (and staging) take an extra factor s, applied
// with their own scale as one multiply.
template <class IO>
concept ScaledStoreIo = requires(const IO& io, float2 (&r)[16]) {
  io.store_row16(0ll, 0, 0, r, 1.0f);
  io.prepare_row16(0ll, 0, 0, r, 1.0f);
};

// Each warp waits for its own group's MMAs (mbar[grp], committed per group)
// before reading that group's accumulator, so TMEM reads (and, in the last
// stage, the global stores) overlap the MMAs of later groups. Stores into
// the planes wait for every group (mbar[NG - 1]): the planes are rewritten in
// place, and a later group's MMAs may still be reading them. Returns false if
// a bounded wait gave up (the group is then skipped).
template <int L, int G, bool LINE_MINOR, int s, class IO, int NT = kPassThreads>
__device__ __forceinline__ bool split_stage_epilogue(const SplitPlanes& P, const float2* __restrict__ tw,
                                                     uint32_t tbase, int warp, int lane, const IO& io,
                                                     long long line0, float out_scale, uint64_t* mbar,
                                                     uint32_t parity) {
  using Sh = LineShape<L>;
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr int J = Sh::J;
  constexpr int NG = Tl::Mt / 128;
  constexpr int Ns = Sh::T << (4 * s);
  constexpr bool LAST = (s == Sh::S - 1);
  bool ok = true;
  // the last stage writes shared memory only when it stages a tensor store
  bool stage_tensor = false;
  if constexpr (TensorMapIo<IO> && LINE_MINOR) stage_tensor = LAST && io.out_tma;
  bool planes_free = LAST && !stage_tensor;
#pragma unroll 1
  for (int grp = warp >> 2; grp < NG; grp += NT / 128) {
    const int m = grp * 128 + 32 * (warp & 3) + lane;
    int g, j;
    Tl::unpos(m, g, j);
    // Twiddles of the next stage, W_L^(e0 + c*de) for outputs c = 0..15 (see
    // below for e0, de); the stage's 2^-4 (exact) is applied to the products.
    // Exact table values at c = 0, 4, 8, 12 and the step W_L^de, read before
    // the wait and the TMEM load so their latency overlaps them; the three
    // values between two exact ones follow by multiplying with the step (at
    // most three FP32 products from an exact value). Five loads per row
    // instead of one per output, whose latency sat between the TMEM load and
    // the products.
    int e0_ = 0, de_ = 0;
    float2 wq[4] = {}, wstep = make_float2(1.f, 0.f);
    if constexpr (!LAST) {
      const int rp_ = ((j / Ns) * 16 * Ns + j % Ns) / J;
      e0_ = rp_ * (j % Ns) * (L / (256 * Ns));
      de_ = rp_ * (L / 256);
#pragma unroll
      for (int q = 0; q < 4; ++q) wq[q] = __ldg(tw + e0_ + 4 * q * de_);
      wstep = __ldg(tw + de_);
    }
    auto twiddle = [&](int c, float2& w) {
      w = (c & 3) == 0 ? wq[c >> 2] : cmulf(w, wstep);
      return w;
    };
    if (!mbar_wait_bounded(mbar + grp, parity)) {
      ok = false;
      continue;
    }
    tc_fence_after_sync();
    const uint32_t taddr = tbase + (static_cast<uint32_t>(32 * (warp & 3)) << 16) + grp * 64u;
    uint32_t d[32], e[32];
    tmem_ld_x32(taddr, d);
    tmem_ld_x32(taddr + 32u, e);
    tmem_ld_wait();
    // the two halves of the accumulator summed, outputs as pairs: vr[k] =
    // real parts of outputs 2k, 2k + 1, vi[k] = their imaginary parts
    float2 vr[8], vi[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      vr[k] = f2add(make_float2(__uint_as_float(d[2 * k]), __uint_as_float(d[2 * k + 1])),
                    make_float2(__uint_as_float(e[2 * k]), __uint_as_float(e[2 * k + 1])));
      vi[k] = f2add(make_float2(__uint_as_float(d[16 + 2 * k]), __uint_as_float(d[17 + 2 * k])),
                    make_float2(__uint_as_float(e[16 + 2 * k]), __uint_as_float(e[17 + 2 * k])));
    }
    if constexpr (LAST) {
      const long long line = line0 + g;
      if (line < io.total_lines) {
        // IO types that take an extra factor fold the tile scale into their
        // own scale (one multiply per value instead of two)
        constexpr bool FOLD = ScaledStoreIo<IO>;
        if constexpr (!FOLD) {
          const float2 s2 = f2bcast(out_scale);
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            vr[k] = f2mul(vr[k], s2);
            vi[k] = f2mul(vi[k], s2);
          }
        }
        float2 v[16];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          v[2 * k] = make_float2(vr[k].x, vi[k].x);
          v[2 * k + 1] = make_float2(vr[k].y, vi[k].y);
        }
        bool staged = false;
        if constexpr (TensorMapIo<IO> && LINE_MINOR) {
          if (stage_tensor) {
            // column-layout copy of the tile (element (g, l) at l * G + g) in
            // the plane region, for the tensor store issued after the stage;
            // the planes are rewritten in place, so every group's MMAs first
            if (!planes_free) {
              if (!mbar_wait_bounded(mbar + (NG - 1), parity)) {
                ok = false;
                continue;
              }
              planes_free = true;
            }
            if constexpr (FOLD) {
              io.prepare_row16(line, j, J, v, out_scale);
            } else {
              io.prepare_row16(line, j, J, v);
            }
            float2* col = reinterpret_cast<float2*>(P.rh) + g;
#pragma unroll
            for (int c = 0; c < 16; ++c) col[(j + c * J) * G] = v[c];
            staged = true;
          }
        }
        if (!staged) {
          if constexpr (FOLD) {
            io.store_row16(line, j, J, v, out_scale);
          } else {
            io.store_row16(line, j, J, v);
          }
        }
      }
    } else {
      if (!planes_free) {
        if (!mbar_wait_bounded(mbar + (NG - 1), parity)) {
          ok = false;
          continue;
        }
        planes_free = true;
      }
      const int a = j / Ns, b = j % Ns;
      const int lp0 = a * 16 * Ns + b;
      const int rp = lp0 / J;
      const int jp0 = lp0 % J;
      // next stage's twiddle exponents (read above): e0 = rp b L / (256 Ns),
      // de = rp L / 256
      const uint32_t krow = (static_cast<uint32_t>(rp) >> 3) * Tl::KSTRIDE + (rp & 7) * 128u;
      constexpr uint32_t CSTEP = LINE_MINOR ? static_cast<uint32_t>(Ns * G) : static_cast<uint32_t>(Ns);
      // outputs 2k, 2k + 1 times their twiddles and 2^-4, as pairs
      const float2 sixteenth = f2bcast(0.0625f);
      float2 w;
      auto twiddled = [&](int k, float2& yr, float2& yi) {
        const float2 w0 = twiddle(2 * k, w);
        const float2 w1 = twiddle(2 * k + 1, w);
        cmul_pair(vr[k], vi[k], twpair(w0, w1), yr, yi);
        yr = f2mul(yr, sixteenth);
        yi = f2mul(yi, sixteenth);
      };
      if constexpr (Ns == 1 && !LINE_MINOR) {
        // 16 outputs -> 16 consecutive columns: per plane two 16-byte stores
        uint32_t prh[8], pih[8], prl[8], pil[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          float2 yr, yi;
          twiddled(k, yr, yi);
          split_pair(yr, prh[k], prl[k]);
          split_pair(yi, pih[k], pil[k]);
        }
        const uint32_t mp = static_cast<uint32_t>(Tl::pos(g, jp0));  // multiple of 16
        // lanes with bit 2 set store the upper half first (bank spread)
        const bool sw = (lane >> 2) & 1;
        const uint32_t m0 = mp + (sw ? 8u : 0u), m1 = mp + (sw ? 0u : 8u);
        const uint32_t off0 = krow + (m0 >> 6) * 1024u + ((((m0 & 63u) >> 3) ^ (rp & 7)) << 4);
        const uint32_t off1 = krow + (m1 >> 6) * 1024u + ((((m1 & 63u) >> 3) ^ (rp & 7)) << 4);
        auto put = [&](uint8_t* plane, const uint32_t (&p)[8]) {
          const uint4 lo = make_uint4(p[0], p[1], p[2], p[3]), hi4 = make_uint4(p[4], p[5], p[6], p[7]);
          *reinterpret_cast<uint4*>(plane + off0) = sw ? hi4 : lo;
          *reinterpret_cast<uint4*>(plane + off1) = sw ? lo : hi4;
        };
        put(P.rh, prh);
        put(P.ih, pih);
        put(P.rl, prl);
        put(P.il, pil);
      } else if constexpr (CSTEP >= 8 && CSTEP < 64 && (CSTEP & (CSTEP - 1)) == 0) {
        // offsets repeat with period 64 / CSTEP, one 1 KiB atom further per period
        constexpr int PER = static_cast<int>(64u / CSTEP);
        const uint32_t mp0 = static_cast<uint32_t>(Tl::pos(g, jp0));
        uint32_t offs[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
          const uint32_t mp = mp0 + static_cast<uint32_t>(k) * CSTEP;
          offs[k] = krow + (mp >> 6) * 1024u + ((((mp & 63u) >> 3) ^ (rp & 7)) << 4) + (mp & 7u) * 2u;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          float2 yr, yi;
          twiddled(k, yr, yi);
          const int c0 = 2 * k, c1 = 2 * k + 1;
          st_two_split(P, offs[c0 % PER] + static_cast<uint32_t>(c0 / PER) * 1024u,
                       offs[c1 % PER] + static_cast<uint32_t>(c1 / PER) * 1024u, yr, yi);
        }
      } else {
        auto off_of = [&](int c) {
          const uint32_t mp = static_cast<uint32_t>(Tl::pos(g, jp0 + c * Ns));
          return krow + (mp >> 6) * 1024u + ((((mp & 63u) >> 3) ^ (rp & 7)) << 4) + (mp & 7u) * 2u;
        };
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          float2 yr, yi;
          twiddled(k, yr, yi);
          st_two_split(P, off_of(2 * k), off_of(2 * k + 1), yr, yi);
        }
      }
    }
  }
  return ok;
}

// ---------------------------------------------------------------------------
// Split-precision tile machinery. Shared-memory layout:
//   [0, 4096)      B matrix images (hi, lo)
//   [4096, 4160)   mbarriers (one per 128-row group), TMEM slot, tile maximum
//   [5120, ...)    four planes (re hi, im hi, re lo, im lo), 1024-aligned
// ---------------------------------------------------------------------------
constexpr uint32_t kSplitPlaneOffset = 5120;

struct SplitState {
  uint8_t* smem;
  uint8_t* bhi;
  uint8_t* blo;
  uint64_t* mbar;  // kSplitMaxGroups mbarriers: MMA completion per 128-row group
  uint64_t* tma_bar;  // tensor-map tile loads
  uint32_t* tslot;
  int* smax;
  uint32_t tbase;
  uint32_t phase;
  uint32_t tma_phase;
  bool pf_pending;  // prefetching kernel: a tile copy into the raw buffer is in flight
};

constexpr int kSplitMaxGroups = 4;  // Mt <= 512

template <uint32_t TMEM_COLS>
__device__ __forceinline__ void split_setup(SplitState& st, const uint32_t* __restrict__ bmat_g) {
  st.smem = aligned_dynamic_smem();
  st.bhi = st.smem;
  st.blo = st.smem + 2048;
  st.mbar = reinterpret_cast<uint64_t*>(st.smem + 4096);
  st.tslot = reinterpret_cast<uint32_t*>(st.smem + 4096 + 8 * kSplitMaxGroups);
  st.smax = reinterpret_cast<int*>(st.smem + 4096 + 8 * kSplitMaxGroups + 8);
  st.tma_bar = reinterpret_cast<uint64_t*>(st.smem + 4096 + 8 * kSplitMaxGroups + 16);
  const int tid = threadIdx.x;
  for (int i = tid; i < 1024; i += blockDim.x) reinterpret_cast<uint32_t*>(st.bhi)[i] = __ldg(bmat_g + i);
  if (tid == 0) {
    for (int k = 0; k < kSplitMaxGroups; ++k) mbar_init(st.mbar + k, 1);
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
  st.pf_pending = false;
}

template <uint32_t TMEM_COLS>
__device__ __forceinline__ void split_teardown(SplitState& st) {
  if (threadIdx.x == 0) bulk_wait_all();  // tensor stores complete before the CTA ends
  tc_fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tmem_dealloc(st.tbase, TMEM_COLS);
}

template <int L, int G>
__host__ __device__ constexpr uint32_t split_tmem_cols() {
  return static_cast<uint32_t>(G * L / 16 / 128 * 64);
}

// One split-precision tile: G lines of length L starting at line0. Same
// geometry rules as pass_tile, with G * L / 16 in {128, 256, 512} (4 planes
// + 64 TMEM columns per 128 rows). False if a bounded wait gave up.
// IO types that can hint the next tile's input into L2.
template <class IO>
concept L2PrefetchIo = requires(const IO& io) { io.prefetch_tile_l2(0ll, 0, 0); };

// ---------------------------------------------------------------------------
// Prefetching split kernel: the next tile's input is copied into a raw
// buffer beside the planes while the current tile runs. Raw layout: row
// input [g][L], column input [l][G], 8-byte elements. Contiguous row tiles
// move as one bulk copy and column tiles with an input map as tensor loads
// (completion on the copy barrier); otherwise 16-byte asynchronous copies
// (two lines of one column element, or two elements of one row), zero-filled
// past the last line.
// ---------------------------------------------------------------------------
template <class IO>
__device__ __forceinline__ bool split_pf_by_barrier(const IO& io) {
  if constexpr (IO::IN_VEC_L) {
    return io.in_contig;
  } else if constexpr (TensorMapIo<IO>) {
    return io.in_tma;
  }
  return false;
}

template <int L, int G, class IO, int NT>
__device__ __forceinline__ void split_prefetch(SplitState& st, const IO& io, long long line0, uint8_t* raw) {
  const int tid = threadIdx.x;
  const long long rem = io.total_lines - line0;
  const int nval = rem < G ? static_cast<int>(rem) : G;
  st.pf_pending = true;
  if constexpr (IO::IN_VEC_L) {
    if (io.in_contig) {
      if (tid == 0) {
        const uint32_t bytes = static_cast<uint32_t>(nval) * L * 8u;
        mbar_arrive_expect_tx(st.tma_bar, bytes);
        bulk_g2s(raw, io.in + io.in_base(line0), bytes, st.tma_bar);
      }
      return;
    }
    constexpr int HPL = L / 2;  // 16-byte chunks per line
#pragma unroll 4
    for (int c = tid; c < G * HPL; c += NT) {
      const int g = c / HPL, q = c % HPL;
      const bool ok = g < nval;
      const void* src = ok ? static_cast<const void*>(io.in + io.in_base(line0 + g) + 2 * q)
                           : static_cast<const void*>(io.in);
      cp_async16(raw + (static_cast<uint32_t>(g) * L + 2u * q) * 8u, src, ok ? 16u : 0u);
    }
    cp_async_commit();
  } else {
    if constexpr (TensorMapIo<IO>) {
      if (io.in_tma) {
        if (tid == 0) {
          constexpr int BY = L < 256 ? L : 256;
          mbar_arrive_expect_tx(st.tma_bar, static_cast<uint32_t>(G) * L * 8u);
          const int seq = static_cast<int>(line0 >> io.lps_log2);
          const int x0 = static_cast<int>(line0 & ((1ll << io.lps_log2) - 1));
#pragma unroll
          for (int r0 = 0; r0 < L; r0 += BY)
            tma_load_3d(raw + static_cast<uint32_t>(r0) * G * 8u, &io.in_map, x0, r0, seq, st.tma_bar);
        }
        return;
      }
    }
    // one 8-byte copy per element: lines need not be adjacent in memory
#pragma unroll 4
    for (int c = tid; c < L * G; c += NT) {
      const int l = c / G, g = c % G;
      const bool ok = g < nval;
      const void* src = ok ? static_cast<const void*>(io.in + io.in_base(line0 + g) + static_cast<long long>(l) * io.in_elem)
                           : static_cast<const void*>(io.in);
      cp_async8(raw + (static_cast<uint32_t>(l) * G + g) * 8u, src, ok ? 8u : 0u);
    }
    cp_async_commit();
  }
}

// Wait for the prefetched tile (whole CTA). False if the bounded wait gave up.
template <class IO>
__device__ __forceinline__ bool split_wait_prefetch(SplitState& st, const IO& io, const PassCore& core) {
  st.pf_pending = false;
  if (split_pf_by_barrier(io)) {
    bool ok = true;
    if (threadIdx.x == 0) {
      ok = mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u);
      if (!ok) {
        atomicOr(core.err, kErrMmaTimeout);
        mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u);  // let a late copy land before giving up
      }
    }
    st.tma_phase++;
    return !__syncthreads_or(!ok);
  }
  cp_async_wait_all();
  __syncthreads();
  return true;
}

// next_line0 >= 0: the tile this CTA processes next, whose input is
// prefetched into L2 while this one runs.
// TMA_IN: the tile arrives by tensor loads (column tiles whose IO carries an
// input map); a template parameter so each load path is compiled on its own.
// NT: threads per CTA (256, or 128 for 256-row tiles run 4 CTAs per SM).
// PF: prefetching kernel; the tile is in rawbuf (its copy is awaited here)
// and the next one's copy is issued once the planes are written.
//
// Lane-bit destinations (remap_lane_bits over the NT * U items) of the
// prefetching kernel's row-input items in line-minor tiles (the transposing
// passes), from a CPU model of the shared-memory banks counting the raw
// reads and the four planes' stores of a tile: 2560 -> 2048 wavefronts for
// every 256-row tile (L = 256 .. 2048 on 16 .. 2 lines). Identity elsewhere.
// The same for column input ([L][G] raw tiles: the four-step column
// passes): 2^20's 1024-point pass on 4-line tiles 1536 -> 1024 wavefronts,
// 65536's 128-point pass on 32-line tiles 1024 -> 768.
template <int L, int G, bool APPLY, int NITEMS>
constexpr LaneBits split_pf_col_lane_bits() {
  if constexpr (APPLY && L == 1024 && G == 4 && NITEMS == 256) return LaneBits{{0, 1, 2, 4, 3}};
  if constexpr (APPLY && ((L == 128 && G == 32) || (L == 512 && G == 8)) && NITEMS >= 64)
    return LaneBits{{0, 1, 2, 5, 3}};
  return LaneBits{{0, 1, 2, 3, 4}};
}

template <int L, int G, bool APPLY, int NITEMS>
constexpr LaneBits split_pf_row_lane_bits() {
  if constexpr (APPLY && L * G == 4096 && L >= 256 && NITEMS >= 128) return LaneBits{{0, 2, 3, 4, 6}};
  return LaneBits{{0, 1, 2, 3, 4}};
}

template <int L, int G, bool LINE_MINOR, int SIGN, class IO, bool TMA_IN = false, int NT = kPassThreads,
          bool PF = false>
__device__ __forceinline__ bool split_tile(SplitState& st, const IO& io, const PassCore& core, long long line0,
                                           long long next_line0 = -1, uint8_t* rawbuf = nullptr) {
  using Sh = LineShape<L>;
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr int T = Sh::T;
  constexpr int S = Sh::S;
  constexpr int J = Sh::J;
  constexpr int Mt = Tl::Mt;
  constexpr int NG = Mt / 128;
  constexpr uint32_t PLANE = Tl::PLANE;
  constexpr uint32_t KSTRIDE = Tl::KSTRIDE;
  static_assert(Mt % 128 == 0 && Mt / 128 <= kSplitMaxGroups, "tile size");
  static_assert(G % 4 == 0 || IO::IN_VEC_L, "line-vectorised loads need G % 4 == 0");
  // N = 64: B_hi (2 KiB) and B_lo (the next 2 KiB) side by side form one
  // K-major operand (SBO 512 B), so D = [A * B_hi | A * B_lo]
  constexpr uint32_t IDESC = make_idesc_f16_f32(128, 64, true, false);
  constexpr int U = T >= 8 ? 1 : 8 / T;
  uint8_t* pl = st.smem + kSplitPlaneOffset;
  SplitPlanes P{pl, pl + PLANE, pl + 2 * PLANE, pl + 3 * PLANE};
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  bool timed_out = false;
  static_assert(!(PF && TMA_IN), "the prefetching kernel moves column tiles into its raw buffer");
  [[maybe_unused]] int nval = G;
  if constexpr (PF) {
    const long long rem = io.total_lines - line0;
    nval = rem < G ? static_cast<int>(rem) : G;
    if (!split_wait_prefetch(st, io, core)) return false;
  } else if constexpr (L2PrefetchIo<IO>) {
    if (next_line0 >= 0) io.prefetch_tile_l2(next_line0, G, L);
  }
  // a tensor store of the previous tile reads the plane region: it must be
  // done reading before this tile's planes are written (no-op otherwise).
  // Tensor loads write the plane region, so they wait here; direct loads
  // fill registers, so they are issued first and the wait comes at the
  // barrier that precedes the first plane store (scales_from below).
  if (TMA_IN && tid == 0) bulk_wait_read_all();
  // column tiles with an input map arrive by tensor loads into the plane
  // region ([L][G] elements), read back by the threads below
  constexpr bool tma_in = TMA_IN;
  if constexpr (TMA_IN) {
    static_assert(TensorMapIo<IO> && !IO::IN_VEC_L, "tensor loads: column tiles with a map");
    if (tid == 0) {
      constexpr int BY = L < 256 ? L : 256;
      mbar_arrive_expect_tx(st.tma_bar, static_cast<uint32_t>(G) * L * 8u);
      const int seq = static_cast<int>(line0 >> io.lps_log2);
      const int x0 = static_cast<int>(line0 & ((1ll << io.lps_log2) - 1));
#pragma unroll
      for (int r0 = 0; r0 < L; r0 += BY)
        tma_load_3d(st.smem + kSplitPlaneOffset + static_cast<uint32_t>(r0) * G * 8u, &io.in_map, x0, r0, seq,
                    st.tma_bar);
    }
  }
    if (tid == 0) *st.smax = 0;
    __syncthreads();

    // ---- the tile is read once: every thread's share fits one batch of
    // loads (4 * Mt / T items of T x 4 elements, Mt <= 512), so the loaded
    // values give the tile's largest magnitude before they are scaled,
    // put through the radix-T stage and split ----
    float in_scale = 1.0f, out_scale = 1.0f;
    auto scales_from = [&](float lmax) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
      if (lane == 0) atomicMax(st.smax, __float_as_int(lmax));
      if constexpr (!TMA_IN) {
        if (tid == 0) bulk_wait_read_all();
      }
      __syncthreads();
      const float tmax = __int_as_float(*st.smax) * static_cast<float>(T);
      // sigma: largest value after the radix-T stage maps to <= 2^14
      int sigma = 0;
      if (tmax > 0.f && isfinite(tmax)) {
        int ex;
        frexpf(tmax, &ex);  // tmax = f * 2^ex, f in [0.5, 1)
        sigma = 14 - ex;
      }
      in_scale = ldexpf(1.0f, sigma);
      out_scale = ldexpf(1.0f, -(sigma - 4 * (S - 1)));
    };
    if constexpr (IO::IN_VEC_L) {
      constexpr int QPL = (L / T) / 4;
      constexpr int ITEMS = G * QPL;
      static_assert(ITEMS <= NT * U, "one load batch per tile");
      constexpr LaneBits LB = split_pf_row_lane_bits<L, G, PF && LINE_MINOR, NT * U>();
      constexpr int B0 = LB.b[0], B1 = LB.b[1], B2 = LB.b[2], B3 = LB.b[3], B4 = LB.b[4];
      constexpr bool REMAP = !(B0 == 0 && B1 == 1 && B2 == 2 && B3 == 3 && B4 == 4);
      auto row_item = [&](int u) {
        if constexpr (REMAP) {
          return remap_lane_bits<NT * U, B0, B1, B2, B3, B4>(tid + u * NT);
        } else {
          return tid + u * NT;
        }
      };
      // item -> (line g, first of four consecutive butterflies j0): a warp's
      // loads run along one line
      auto item_g = [](int it) { return it / QPL; };
      auto item_j0 = [](int it) { return (it % QPL) * 4; };
      typename IO::Raw raw[U][T];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = row_item(u);
#pragma unroll
        for (int r = 0; r < T; ++r) {
          if constexpr (PF) {
            const int g = item_g(it);
            if ((ITEMS % (NT * U) == 0 || it < ITEMS) && g < nval) {
              raw[u][r] = *reinterpret_cast<const typename IO::Raw*>(
                  rawbuf + ((static_cast<uint32_t>(g) * L + item_j0(it) + r * (L / T)) << 3));
            } else {
              raw[u][r] = typename IO::Raw{make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
            }
          } else {
            raw[u][r] = io.fetch_l(line0 + item_g(it), item_j0(it) + r * (L / T), it < ITEMS);
          }
        }
      }
      float2 v[U][T][4];
      float lmax = 0.f;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = row_item(u);
        const int g = item_g(it);
        const int j0 = item_j0(it);
#pragma unroll
        for (int r = 0; r < T; ++r) {
          io.decode_l(raw[u][r], line0 + g, j0 + r * (L / T), v[u][r]);
          lmax = fmaxf(lmax, max_abs4(v[u][r]));
        }
      }
      scales_from(lmax);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = row_item(u);
        if (ITEMS % (NT * U) != 0 && it >= ITEMS) continue;
        const int g = item_g(it);
        const int j0 = item_j0(it);
#pragma unroll
        for (int r = 0; r < T; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            v[u][r][q].x *= in_scale;
            v[u][r][q].y *= in_scale;
          }
        if constexpr (T == 1) {
          if constexpr (!LINE_MINOR && J >= 4) {
            st_quad_split(P, Tl::off(g, j0), v[u][0]);
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) st_pair_split(P, Tl::off(g, j0 + q), v[u][0][q]);
          }
        } else {
          // Output c of butterfly j goes to l' = j*T + c: K row rp = j*T / J
          // for every c (T divides J), column (j*T + c) % J, twiddle
          // W_L^(rp c L / (16T)) = W_(16T)^(rp c). When J / T is a multiple
          // of 4 the item's four butterflies share rp and its T twiddles are
          // read once.
          constexpr bool SHARED_RP = ((J / T) % 4) == 0;
          float2 wt[T];
          auto load_tw = [&](int rp) {
            wt[0] = make_float2(1.f, 0.f);
#pragma unroll
            for (int c = 1; c < T; ++c) wt[c] = __ldg(core.tw + rp * c * (L / (16 * T)));
          };
          if constexpr (SHARED_RP) load_tw((j0 * T) / J);
          if constexpr (LINE_MINOR && SHARED_RP) {
            // two butterflies at a time: output c of each goes to its own
            // column, and the products and the hi / lo split run on pairs
#pragma unroll
            for (int q = 0; q < 4; q += 2) {
              float2 t0[T], t1[T];
#pragma unroll
              for (int r = 0; r < T; ++r) {
                t0[r] = v[u][r][q];
                t1[r] = v[u][r][q + 1];
              }
              small_dft<T, SIGN>(t0);
              small_dft<T, SIGN>(t1);
              const int j = j0 + q;
#pragma unroll
              for (int c = 0; c < T; ++c) {
                float2 yr = make_float2(t0[c].x, t1[c].x), yi = make_float2(t0[c].y, t1[c].y);
                if (c > 0) cmul_pair(yr, yi, twpair(wt[c], wt[c]), yr, yi);
                st_two_split(P, Tl::off(g, j * T + c), Tl::off(g, (j + 1) * T + c), yr, yi);
              }
            }
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              float2 t[T];
#pragma unroll
              for (int r = 0; r < T; ++r) t[r] = v[u][r][q];
              small_dft<T, SIGN>(t);
              const int j = j0 + q;
              if constexpr (!SHARED_RP) load_tw((j * T) / J);
#pragma unroll
              for (int c = 1; c < T; ++c) t[c] = cmulf(t[c], wt[c]);
              if constexpr (!LINE_MINOR) {
                // T consecutive columns of one K row: one store per plane
                st_run_split<T>(P, Tl::off(g, j * T), t);
              } else {
#pragma unroll
                for (int c = 0; c < T; ++c) st_pair_split(P, Tl::off(g, j * T + c), t[c]);
              }
            }
          }
        }
      }
    } else {
      constexpr int GQ = G / 4;
      constexpr int ITEMS = GQ * (L / T);
      static_assert(ITEMS <= NT * U, "one load batch per tile");
      constexpr LaneBits CB = split_pf_col_lane_bits<L, G, PF && ITEMS == NT * U, NT * U>();
      constexpr int C0 = CB.b[0], C1 = CB.b[1], C2 = CB.b[2], C3 = CB.b[3], C4 = CB.b[4];
      constexpr bool CREMAP = !(C0 == 0 && C1 == 1 && C2 == 2 && C3 == 3 && C4 == 4);
      auto col_item = [&](int u) {
        if constexpr (CREMAP) {
          return remap_lane_bits<NT * U, C0, C1, C2, C3, C4>(tid + u * NT);
        } else {
          return tid + u * NT;
        }
      };
      typename IO::Raw raw[U][T];
      bool loaded = false;
      if constexpr (TMA_IN) {
        {
          // one thread polls the copy barrier, the others wait at the CTA barrier
          bool to = false;
          if (tid == 0) {
            to = !mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u);
            if (to) {
              atomicOr(core.err, kErrMmaTimeout);
              mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u);  // let a late copy land before giving up
            }
          }
          st.tma_phase++;
          if (__syncthreads_or(to)) return false;
          const uint8_t* src = st.smem + kSplitPlaneOffset;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int it = col_item(u);
#pragma unroll
            for (int r = 0; r < T; ++r) {
              raw[u][r] = typename IO::Raw{make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
              if (ITEMS % (NT * U) == 0 || it < ITEMS) {
                const uint8_t* p =
                    src + ((static_cast<uint32_t>(it / GQ + r * (L / T)) * G + (it % GQ) * 4u) << 3);
                raw[u][r].a = *reinterpret_cast<const uint4*>(p);
                raw[u][r].b = *reinterpret_cast<const uint4*>(p + 16);
              }
            }
          }
          loaded = true;
        }
      }
      if constexpr (PF) {
        // the prefetched [L][G] tile (past the last line: zero-filled)
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int it = col_item(u);
#pragma unroll
          for (int r = 0; r < T; ++r) {
            raw[u][r] = typename IO::Raw{make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
            if (ITEMS % (NT * U) == 0 || it < ITEMS)
              raw[u][r] = *reinterpret_cast<const typename IO::Raw*>(
                  rawbuf + ((static_cast<uint32_t>(it / GQ + r * (L / T)) * G + (it % GQ) * 4u) << 3));
          }
        }
        loaded = true;
      }
      if (!loaded) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int it = col_item(u);
#pragma unroll
          for (int r = 0; r < T; ++r)
            raw[u][r] = io.fetch_g(line0 + (it % GQ) * 4, it / GQ + r * (L / T), it < ITEMS);
        }
      }
      float2 v[U][T][4];
      float lmax = 0.f;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = col_item(u);
        const int j = it / GQ;
        const int g0 = (it % GQ) * 4;
#pragma unroll
        for (int r = 0; r < T; ++r) {
          io.decode_g(raw[u][r], line0 + g0, j + r * (L / T), v[u][r]);
          lmax = fmaxf(lmax, max_abs4(v[u][r]));
        }
      }
      scales_from(lmax);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = col_item(u);
        if (ITEMS % (NT * U) != 0 && it >= ITEMS) continue;
        const int j = it / GQ;
        const int g0 = (it % GQ) * 4;
#pragma unroll
        for (int r = 0; r < T; ++r)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            v[u][r][q].x *= in_scale;
            v[u][r][q].y *= in_scale;
          }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float2 t[T];
#pragma unroll
          for (int r = 0; r < T; ++r) t[r] = v[u][r][q];
          small_dft<T, SIGN>(t);
#pragma unroll
          for (int r = 0; r < T; ++r) v[u][r][q] = t[r];
        }
#pragma unroll
        for (int c = 0; c < T; ++c) {
          const int lp = j * T + c;
          float2 x[4] = {v[u][c][0], v[u][c][1], v[u][c][2], v[u][c][3]};
          if constexpr (T > 1) {
            const int rp = lp / J, jp = lp % J;
            const float2 w = __ldg(core.tw + rp * (jp % T) * (L / (16 * T)));
#pragma unroll
            for (int q = 0; q < 4; ++q) x[q] = cmulf(x[q], w);
          }
          if constexpr (LINE_MINOR) {
            st_quad_split(P, Tl::off(g0, lp), x);
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) st_pair_split(P, Tl::off(g0 + q, lp), x[q]);
          }
        }
      }
    }
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();
    // the raw buffer is read: the next tile's copy can go in
    if constexpr (PF) {
      if (next_line0 >= 0) split_prefetch<L, G, IO, NT>(st, io, next_line0, rawbuf);
    }

    auto run_stage = [&](auto s_const) {
      constexpr int s = decltype(s_const)::value;
      if (timed_out) return;
      if (tid == 0) {
        tc_fence_after_sync();
        const uint32_t arh = smem_u32(P.rh), aih = smem_u32(P.ih), arl = smem_u32(P.rl), ail = smem_u32(P.il);
        const uint64_t bh0 = make_sdesc(smem_u32(st.bhi), 128u, 512u, kLayoutNone);
        const uint64_t bh1 = make_sdesc(smem_u32(st.bhi) + 256u, 128u, 512u, kLayoutNone);
#pragma unroll
        for (int grp = 0; grp < NG; ++grp) {
          const uint32_t o = grp * 2048u;
          const uint64_t a_rh = make_sdesc(arh + o, 1024u, KSTRIDE, kLayoutSw128);
          const uint64_t a_ih = make_sdesc(aih + o, 1024u, KSTRIDE, kLayoutSw128);
          const uint64_t a_rl = make_sdesc(arl + o, 1024u, KSTRIDE, kLayoutSw128);
          const uint64_t a_il = make_sdesc(ail + o, 1024u, KSTRIDE, kLayoutSw128);
          const uint32_t dacc = st.tbase + grp * 64u;
          umma_f16(dacc, a_rh, bh0, IDESC, 0u);
          umma_f16(dacc, a_ih, bh1, IDESC, 1u);
          umma_f16(dacc, a_rl, bh0, IDESC, 1u);
          umma_f16(dacc, a_il, bh1, IDESC, 1u);
          umma_commit(st.mbar + grp);  // this group and every earlier one
        }
      }
      const bool to = !split_stage_epilogue<L, G, LINE_MINOR, s, IO, NT>(P, core.tw, st.tbase, warp, lane, io, line0,
                                                                     out_scale, st.mbar, st.phase & 1u);
      if (to && lane == 0) atomicOr(core.err, kErrMmaTimeout);
      st.phase++;
      fence_proxy_async_smem();
      tc_fence_before_sync();
      if (__syncthreads_or(to)) timed_out = true;
    };
    [&]<int... Is>(std::integer_sequence<int, Is...>) {
      (run_stage(std::integral_constant<int, Is>{}), ...);
    }(std::make_integer_sequence<int, S>{});
    return !timed_out;
}

// ---------------------------------------------------------------------------
// Split-precision pass kernel: persistent CTAs over the tiles of one pass.
// ---------------------------------------------------------------------------
template <int L, int G, bool LINE_MINOR, int SIGN, class IO, int NT = kPassThreads>
__global__ void __launch_bounds__(NT, 512 / NT) fft_pass_split(const __grid_constant__ IO io, const PassCore core) {
  constexpr uint32_t TMEM_COLS = split_tmem_cols<L, G>();
  static_assert(TMEM_COLS >= 32 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  SplitState st;
  split_setup<TMEM_COLS>(st, core.bmat);
  const long long ntiles = (io.total_lines + G - 1) / G;
  // column tiles with an input map take the tensor-load path (one loop per
  // path, so each is compiled on its own)
  bool tma_in = false;
  if constexpr (TensorMapIo<IO> && !IO::IN_VEC_L) tma_in = io.in_tma;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long next = tile + gridDim.x < ntiles ? (tile + gridDim.x) * G : -1;
    bool ok;
    if constexpr (TensorMapIo<IO> && !IO::IN_VEC_L) {
      ok = tma_in ? split_tile<L, G, LINE_MINOR, SIGN, IO, true, NT>(st, io, core, tile * G, next)
                  : split_tile<L, G, LINE_MINOR, SIGN, IO, false, NT>(st, io, core, tile * G, next);
    } else {
      ok = split_tile<L, G, LINE_MINOR, SIGN, IO, false, NT>(st, io, core, tile * G, next);
    }
    if (!ok) break;
    if constexpr (TensorMapIo<IO> && LINE_MINOR) {
      if (io.out_tma && threadIdx.x == 0) {
        // the staged [L][G] tile as L / 256 tensor stores (the host sets the
        // map only when tiles never straddle a sequence)
        constexpr int BY = L < 256 ? L : 256;
        const long long line0 = tile * G;
        const int seq = static_cast<int>(line0 >> io.lps_log2);
        const int x0 = static_cast<int>(line0 & ((1ll << io.lps_log2) - 1));
        const uint8_t* stage = st.smem + kSplitPlaneOffset;
#pragma unroll
        for (int r0 = 0; r0 < L; r0 += BY)
          tma_store_3d(&io.out_map, stage + static_cast<uint32_t>(r0) * G * 8u, x0, r0, seq);
        bulk_commit();
      }
    }
  }
  split_teardown<TMEM_COLS>(st);
}

template <int L, int G>
constexpr int split_smem_bytes() {
  return static_cast<int>(kSplitPlaneOffset) + 4 * (G * L / 16) * 32 + 1024;
}

// Prefetching split-precision pass kernel: the planes plus a raw buffer of
// one tile's input (G * L * 8 bytes), whose copy for the next tile runs
// while the current one goes through its stages.
template <int L, int G, bool LINE_MINOR, int SIGN, class IO, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) fft_pass_split_pf(const __grid_constant__ IO io, const PassCore core) {
  using Tl = Tile<L, G, LINE_MINOR>;
  constexpr uint32_t TMEM_COLS = split_tmem_cols<L, G>();
  static_assert(TMEM_COLS >= 32 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  SplitState st;
  split_setup<TMEM_COLS>(st, core.bmat);
  uint8_t* raw = st.smem + kSplitPlaneOffset + 4 * Tl::PLANE;
  const long long ntiles = (io.total_lines + G - 1) / G;
  if (blockIdx.x < ntiles) split_prefetch<L, G, IO, NT>(st, io, static_cast<long long>(blockIdx.x) * G, raw);
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long next = tile + gridDim.x < ntiles ? (tile + gridDim.x) * G : -1;
    if (!split_tile<L, G, LINE_MINOR, SIGN, IO, false, NT, true>(st, io, core, tile * G, next, raw)) break;
    if constexpr (TensorMapIo<IO> && LINE_MINOR) {
      if (io.out_tma && threadIdx.x == 0) {
        constexpr int BY = L < 256 ? L : 256;
        const long long line0 = tile * G;
        const int seq = static_cast<int>(line0 >> io.lps_log2);
        const int x0 = static_cast<int>(line0 & ((1ll << io.lps_log2) - 1));
        const uint8_t* stage = st.smem + kSplitPlaneOffset;
#pragma unroll
        for (int r0 = 0; r0 < L; r0 += BY)
          tma_store_3d(&io.out_map, stage + static_cast<uint32_t>(r0) * G * 8u, x0, r0, seq);
        bulk_commit();
      }
    }
  }
  // an early exit may leave a copy in flight: let it land before the CTA ends
  if (st.pf_pending) {
    if (split_pf_by_barrier(io)) {
      if (threadIdx.x == 0) mbar_wait_bounded(st.tma_bar, st.tma_phase & 1u);
    } else {
      cp_async_wait_all();
    }
  }
  split_teardown<TMEM_COLS>(st);
}

template <int L, int G>
constexpr int split_pf_smem_bytes() {
  return static_cast<int>(kSplitPlaneOffset) + 4 * (G * L / 16) * 32 + G * L * 8 + 1024;
}

// Interleaved complex float in and out, arbitrary strides (in elements).
// COHERENT: input is read with L2-coherent loads (written by other CTAs of the
// same launch).
template <bool IN_L, bool OUT_L, bool COHERENT = false>
struct IoFloat {
  static constexpr bool IN_VEC_L = IN_L;
  static constexpr bool OUT_VEC_L = OUT_L;
  struct Raw {
    uint4 a, b;
  };

  const float2* in;
  float2* out;
  long long total_lines;
  int lps_log2;
  long long in_seq, in_line, in_elem;
  long long out_seq, out_line, out_elem;
  OuterTwiddle otw;
  float scale;
  bool in_contig, out_contig;  // not used by the split kernel (direct loads / stores)
  long long contig_len;
  // Column-layout output (lines adjacent in memory, out_line == 1) stored by
  // TMA through a 3D tensor map (x = line within its sequence, y = element,
  // z = sequence; 8-byte elements), set by the host; the kernel parameter is
  // __grid_constant__. The split kernel uses the input map only for L2
  // prefetches of the next tile.
  bool in_tma, out_tma;
  CUtensorMap in_map, out_map;

  __device__ __forceinline__ long long in_base(long long line) const {
    return (line >> lps_log2) * in_seq + (line & ((1ll << lps_log2) - 1)) * in_line;
  }
  __device__ __forceinline__ long long out_base(long long line) const {
    return (line >> lps_log2) * out_seq + (line & ((1ll << lps_log2) - 1)) * out_line;
  }
  // L2 prefetch of the input of lines [line0, line0 + g) of length l:
  // contiguous lines (IN_L) one range per line; column layout (adjacent
  // lines adjacent in memory, in_line == 1) one range of g elements per line
  // element. Called by every thread of the CTA; lines past the end are left
  // out.
  __device__ __forceinline__ void prefetch_tile_l2(long long line0, int g, int l) const {
    const int tid = threadIdx.x;
    if constexpr (IN_L) {
      for (int k = tid; k < g; k += blockDim.x) {
        const long long line = line0 + k;
        if (line < total_lines) prefetch_l2_bulk(in + in_base(line), static_cast<uint32_t>(l) * 8u);
      }
    } else {
      if (in_line != 1) return;
      if (in_tma) {
        // the host set an input map (tiles never straddle a sequence): the
        // tile as L / 256 box prefetches
        if (tid == 0) {
          const int by = l < 256 ? l : 256;
          const int seq = static_cast<int>(line0 >> lps_log2);
          const int x0 = static_cast<int>(line0 & ((1ll << lps_log2) - 1));
          for (int r0 = 0; r0 < l; r0 += by) tma_prefetch_3d(&in_map, x0, r0, seq);
        }
        return;
      }
      const long long rem = total_lines - line0;
      const int lines = rem < g ? static_cast<int>(rem) : g;
      if (lines <= 0 || (lines & 1)) return;  // ranges of whole 16-byte units
      // the lines must lie in one sequence (adjacent in memory)
      if ((line0 >> lps_log2) != ((line0 + lines - 1) >> lps_log2)) return;
      const float2* base = in + in_base(line0);
      for (int e = tid; e < l; e += blockDim.x)
        prefetch_l2_bulk(base + static_cast<long long>(e) * in_elem, static_cast<uint32_t>(lines) * 8u);
    }
  }
  __device__ __forceinline__ Raw fetch_l(long long line, int l0, bool ok) const {
    Raw r{make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    if (!ok || line >= total_lines) return r;
    const float2* p = in + in_base(line) + l0;
    r.a = COHERENT ? ldg_cg_v4(p) : ldg_nc_v4(p);
    r.b = COHERENT ? ldg_cg_v4(p + 2) : ldg_nc_v4(p + 2);
    return r;
  }
  __device__ __forceinline__ Raw fetch_g(long long line0, int l, bool ok) const {
    Raw r{make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    if (!ok || line0 >= total_lines) return r;
    const float2* p = in + in_base(line0) + static_cast<long long>(l) * in_elem;
    r.a = COHERENT ? ldg_cg_v4(p) : ldg_nc_v4(p);
    r.b = COHERENT ? ldg_cg_v4(p + 2) : ldg_nc_v4(p + 2);
    return r;
  }
  __device__ __forceinline__ static void unpack(const Raw& r, float2 (&v)[4]) {
    v[0] = make_float2(__uint_as_float(r.a.x), __uint_as_float(r.a.y));
    v[1] = make_float2(__uint_as_float(r.a.z), __uint_as_float(r.a.w));
    v[2] = make_float2(__uint_as_float(r.b.x), __uint_as_float(r.b.y));
    v[3] = make_float2(__uint_as_float(r.b.z), __uint_as_float(r.b.w));
  }
  __device__ __forceinline__ void decode_l(const Raw& r, long long, int, float2 (&v)[4]) const { unpack(r, v); }
  __device__ __forceinline__ void decode_g(const Raw& r, long long, int, float2 (&v)[4]) const { unpack(r, v); }
  // v[c] *= W_N^{li (j + c J)} * k for c = 0..15 (the outer twiddle of line
  // li and the store scale k). The twiddle is exact (two-level table) at
  // c = 0, 4, 8, 12, each times k; the three values after an exact one follow
  // from the exact step W_N^{li J} (c + 1 by one product, c + 2 and c + 3 as a
  // pair times step^2), products on packed pairs.
  __device__ __forceinline__ void twiddle_scale16(long long line, int j, int J, float2 (&v)[16], float k) const {
    const long long li = line & ((1ll << lps_log2) - 1);
    const float2 step = otw(li, J);
    const float2 s2 = cmulf(step, step);
    const TwPair s2p = twpair(s2, s2);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float2 w0 = otw(li, j + 4 * q * J);
      w0 = make_float2(w0.x * k, w0.y * k);
      const float2 w1 = cmulf(w0, step);
      const TwPair p01 = twpair(w0, w1);
      float2 r23, i23;
      cmul_pair(p01.re, p01.im, s2p, r23, i23);  // (w2, w3) = (w0, w1) * step^2
      const TwPair p23 = TwPair{r23, i23, make_float2(-i23.x, -i23.y)};
      const int c = 4 * q;
      float2 yr, yi;
      cmul_pair(make_float2(v[c].x, v[c + 1].x), make_float2(v[c].y, v[c + 1].y), p01, yr, yi);
      v[c] = make_float2(yr.x, yi.x);
      v[c + 1] = make_float2(yr.y, yi.y);
      cmul_pair(make_float2(v[c + 2].x, v[c + 3].x), make_float2(v[c + 2].y, v[c + 3].y), p23, yr, yi);
      v[c + 2] = make_float2(yr.x, yi.x);
      v[c + 3] = make_float2(yr.y, yi.y);
    }
  }
  __device__ __forceinline__ static void scale16(float2 (&v)[16], float k) {
    const float2 k2 = f2bcast(k);
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
      const float2 r = f2mul(make_float2(v[c].x, v[c + 1].x), k2);
      const float2 i = f2mul(make_float2(v[c].y, v[c + 1].y), k2);
      v[c] = make_float2(r.x, i.x);
      v[c + 1] = make_float2(r.y, i.y);
    }
  }
  // Outer twiddle and scale applied in place to outputs l = j + c*J of one
  // line (same values as store_row16 writes), for the staged tensor store.
  __device__ __forceinline__ void prepare_row16(long long line, int j, int J, float2 (&v)[16],
                                                float s = 1.0f) const {
    const float k = scale * s;
    if (otw.hi) {
      twiddle_scale16(line, j, J, v, k);
    } else {
      scale16(v, k);
    }
  }
  // Outputs l = j + c*J (c = 0..15) of one line, times the outer twiddle (if
  // any) and scale * s.
  __device__ __forceinline__ void store_row16(long long line, int j, int J, float2 (&v)[16],
                                              float s = 1.0f) const {
    prepare_row16(line, j, J, v, s);
    float2* p = out + out_base(line);
#pragma unroll
    for (int c = 0; c < 16; ++c) p[static_cast<long long>(j + c * J) * out_elem] = v[c];
  }
};

}  // namespace tcfft
