// Registry of instantiated pass kernels.
#pragma once
#include <cuda_runtime.h>

#include "fft_fused.cuh"
#include "fft_io.cuh"
#include "fft_split.cuh"
#include "fft_tile.cuh"

namespace tcfft {

// Pass kinds (how lines sit in global memory and which way vectors run).
enum PassKind : int {
  kPassRow = 0,   // lines contiguous; load and store along the line
  kPassCol = 1,   // lines = adjacent columns; load and store across lines
  kPassRowT = 2,  // load along the line, store across lines (transposing)
  kNumPassKinds = 3
};

// Tile-size variants: Mt = butterflies per radix-16 stage in one tile
// (FP16: small 128, big 1024, mid 512 prefetching at 3 CTAs/SM, narrow 256
//  prefetching on 128 threads at 6 CTAs/SM;
//  split: small 128, big 512, mid 256 on 128 threads at 4 CTAs/SM, narrow
//  256 prefetching on 128 threads at 3 CTAs/SM).
enum TileSel : int { kTileSmall = 0, kTileBig = 1, kTileMid = 2, kTileNarrow = 3, kNumTileSel = 4 };

enum PrecSel : int { kPrecF16 = 0, kPrecSplit = 1, kNumPrec = 2 };

constexpr int kMinLogL = 4;
constexpr int kMaxLogL = 14;

struct PassKernel {
  const void* fn = nullptr;
  int smem = 0;
  int G = 0;   // lines per tile
  int Mt = 0;  // butterflies per stage per tile
  int threads = kPassThreads;
};

using PassTable = PassKernel[kMaxLogL + 1][kNumTileSel][2];

// Filled by the instantiation units.
void register_row_kernels(PassTable& tab);
void register_col_kernels(PassTable& tab);
void register_rowt_kernels(PassTable& tab);
void register_split_row_kernels(PassTable& tab);
void register_split_col_kernels(PassTable& tab);
void register_split_rowt_kernels(PassTable& tab);
void register_split_mid_kernels(PassTable& row, PassTable& col, PassTable& rowt);
void register_f16_narrow_kernels(PassTable& row, PassTable& col, PassTable& rowt);
void register_split_pf_kernels(PassTable& row, PassTable& col, PassTable& rowt);

template <int L, int Mt>
constexpr int tile_lines() {
  return Mt * 16 / L;
}

template <int L, int Mt, bool LINE_MINOR, bool IN_VEC_L, bool OUT_VEC_L, int MINB = 2>
void fill_entry(PassTable& tab, int tile) {
  constexpr int G = tile_lines<L, Mt>();
  constexpr int LOG = ilog2c(L);
  const int smem = pass_smem_bytes<L, G>();
  PassKernel f, i;
  using IO = IoHalf<IN_VEC_L, OUT_VEC_L>;
  f.fn = reinterpret_cast<const void*>(&fft_pass_f16<L, G, LINE_MINOR, -1, IO, MINB>);
  i.fn = reinterpret_cast<const void*>(&fft_pass_f16<L, G, LINE_MINOR, +1, IO, MINB>);
  f.smem = i.smem = smem;
  f.G = i.G = G;
  f.Mt = i.Mt = Mt;
  tab[LOG][tile][0] = f;
  tab[LOG][tile][1] = i;
}

// Prefetching variant (raw input buffer beside the planes; fft_pass_f16_pf).
template <int L, int Mt, bool LINE_MINOR, bool IN_VEC_L, bool OUT_VEC_L, int MINB = 3, int NT = kPassThreads>
void fill_pf_entry(PassTable& tab, int tile) {
  constexpr int G = tile_lines<L, Mt>();
  constexpr int LOG = ilog2c(L);
  const int smem = pass_pf_smem_bytes<L, G>();
  PassKernel f, i;
  using IO = IoHalf<IN_VEC_L, OUT_VEC_L>;
  f.fn = reinterpret_cast<const void*>(&fft_pass_f16_pf<L, G, LINE_MINOR, -1, IO, MINB, NT>);
  i.fn = reinterpret_cast<const void*>(&fft_pass_f16_pf<L, G, LINE_MINOR, +1, IO, MINB, NT>);
  f.smem = i.smem = smem;
  f.G = i.G = G;
  f.Mt = i.Mt = Mt;
  f.threads = i.threads = NT;
  tab[LOG][tile][0] = f;
  tab[LOG][tile][1] = i;
}

template <int L, int Mt, bool LINE_MINOR, bool IN_VEC_L, bool OUT_VEC_L, int NT = kPassThreads>
void fill_split_entry(PassTable& tab, int tile) {
  constexpr int G = tile_lines<L, Mt>();
  constexpr int LOG = ilog2c(L);
  const int smem = split_smem_bytes<L, G>();
  PassKernel f, i;
  using IO = IoFloat<IN_VEC_L, OUT_VEC_L>;
  f.fn = reinterpret_cast<const void*>(&fft_pass_split<L, G, LINE_MINOR, -1, IO, NT>);
  i.fn = reinterpret_cast<const void*>(&fft_pass_split<L, G, LINE_MINOR, +1, IO, NT>);
  f.smem = i.smem = smem;
  f.G = i.G = G;
  f.Mt = i.Mt = Mt;
  f.threads = i.threads = NT;
  tab[LOG][tile][0] = f;
  tab[LOG][tile][1] = i;
}

// Prefetching split-precision variant (raw input buffer beside the planes;
// fft_pass_split_pf).
template <int L, int Mt, bool LINE_MINOR, bool IN_VEC_L, bool OUT_VEC_L, int NT, int MINB>
void fill_split_pf_entry(PassTable& tab, int tile) {
  constexpr int G = tile_lines<L, Mt>();
  constexpr int LOG = ilog2c(L);
  const int smem = split_pf_smem_bytes<L, G>();
  PassKernel f, i;
  using IO = IoFloat<IN_VEC_L, OUT_VEC_L>;
  f.fn = reinterpret_cast<const void*>(&fft_pass_split_pf<L, G, LINE_MINOR, -1, IO, NT, MINB>);
  i.fn = reinterpret_cast<const void*>(&fft_pass_split_pf<L, G, LINE_MINOR, +1, IO, NT, MINB>);
  f.smem = i.smem = smem;
  f.G = i.G = G;
  f.Mt = i.Mt = Mt;
  f.threads = i.threads = NT;
  tab[LOG][tile][0] = f;
  tab[LOG][tile][1] = i;
}

// Fused four-step kernels, indexed by log2 N (15..24) and direction.
constexpr int kFusedMinLog = 15, kFusedMaxLog = 24;
struct FusedKernel {
  const void* fn = nullptr;
  int smem = 0;
  int log_n1 = 0, log_n2 = 0;
  int G1 = 0, G2 = 0;
};
using FusedTable = FusedKernel[kFusedMaxLog + 1][2];
void register_fused_kernels(FusedTable& tab);

template <int L1, int L2>
void fill_fused(FusedTable& tab) {
  constexpr int G1 = 16384 / L1, G2 = 16384 / L2;
  constexpr int LOG = ilog2c(static_cast<long long>(L1) * L2);
  FusedKernel f, i;
  f.fn = reinterpret_cast<const void*>(&fft_fourstep_fused<L1, G1, L2, G2, -1>);
  i.fn = reinterpret_cast<const void*>(&fft_fourstep_fused<L1, G1, L2, G2, +1>);
  f.smem = i.smem = fused_smem_bytes<L1, G1, L2, G2>();
  f.log_n1 = i.log_n1 = ilog2c(L1);
  f.log_n2 = i.log_n2 = ilog2c(L2);
  f.G1 = i.G1 = G1;
  f.G2 = i.G2 = G2;
  tab[LOG][0] = f;
  tab[LOG][1] = i;
}

}  // namespace tcfft
