// C ABI: plan creation, execution and destruction for the tensor-core FFT.
//
// Plan logic restates, for arbitrary powers of two, what the reference's
// tcfftCreate / tcfftExec do for a fixed list of sizes
// (tcfft_half.cu:1177-1345): choose a chain of passes over the data, build the
// DFT-matrix table, launch. Here a pass is one kernel that runs a complete
// FFT of length L <= 2^14 on tiles held in shared memory; sizes above 2^14
// use the four-step split N = N1 * N2 (column pass with outer twiddle, then a
// transposing row pass), so every transform is at most two HBM round trips.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/tcfft_gb300.h"
#include "capi_internal.cuh"
#include "passes.cuh"
#include "tables.cuh"

using namespace tcfft;

namespace {

thread_local tcfftStatus g_last = TCFFT_OK;
thread_local int g_last_launches = 0;

tcfftStatus ret(tcfftStatus s) {
  g_last = s;
  return s;
}

PassTable g_tab[kNumPrec][kNumPassKinds];
FusedTable g_fused;
int g_fused_occ[kFusedMaxLog + 1][2];
int g_occ[kNumPrec][kNumPassKinds][kMaxLogL + 1][kNumTileSel][2];
std::once_flag g_once;
cudaError_t g_init_err = cudaSuccess;
int g_num_sms = 0;
// Tile variant per (precision, pass kind, log2 length); -1 = built-in choice.
// Written by tcfft_tune_set (exact: the autotuner's timing, the tile tests)
// or tcfft_tune_prefer (a tuning file: the tuner measured on batches that
// fill the GPU, so a batch too small for the variant may take another),
// read at every launch.
int g_tune[kNumPrec][kNumPassKinds][kMaxLogL + 1];
bool g_tune_pref[kNumPrec][kNumPassKinds][kMaxLogL + 1];
// Four-step split per (precision, log2 n): log2 of the column-pass length,
// -1 = built-in choice. Written by tcfft_tune_split, read at plan creation.
constexpr int kMaxLogN = 24;
int g_split[kNumPrec][kMaxLogN + 1];
std::once_flag g_tune_once;
void tune_reset() {
  for (auto& a : g_tune)
    for (auto& b : a)
      for (int& c : b) c = -1;
  for (auto& a : g_tune_pref)
    for (auto& b : a)
      for (bool& c : b) c = false;
  for (auto& a : g_split)
    for (int& c : a) c = -1;
}

bool pass_built(int prec, int kind, int logl) {
  if (logl < 0 || logl > kMaxLogL) return false;
  for (int t = 0; t < kNumTileSel; ++t)
    if (g_tab[prec][kind][logl][t][0].fn) return true;
  return false;
}

void init_registry() {
  register_row_kernels(g_tab[kPrecF16][kPassRow]);
  register_col_kernels(g_tab[kPrecF16][kPassCol]);
  register_rowt_kernels(g_tab[kPrecF16][kPassRowT]);
  register_split_row_kernels(g_tab[kPrecSplit][kPassRow]);
  register_split_col_kernels(g_tab[kPrecSplit][kPassCol]);
  register_split_rowt_kernels(g_tab[kPrecSplit][kPassRowT]);
  register_split_mid_kernels(g_tab[kPrecSplit][kPassRow], g_tab[kPrecSplit][kPassCol], g_tab[kPrecSplit][kPassRowT]);
  register_f16_narrow_kernels(g_tab[kPrecF16][kPassRow], g_tab[kPrecF16][kPassCol], g_tab[kPrecF16][kPassRowT]);
  register_split_pf_kernels(g_tab[kPrecSplit][kPassRow], g_tab[kPrecSplit][kPassCol], g_tab[kPrecSplit][kPassRowT]);
  register_fused_kernels(g_fused);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  for (int pr = 0; pr < kNumPrec && e == cudaSuccess; ++pr)
  for (int k = 0; k < kNumPassKinds && e == cudaSuccess; ++k)
    for (int l = 0; l <= kMaxLogL && e == cudaSuccess; ++l)
      for (int t = 0; t < kNumTileSel && e == cudaSuccess; ++t)
        for (int s = 0; s < 2 && e == cudaSuccess; ++s) {
          PassKernel& pk = g_tab[pr][k][l][t][s];
          if (!pk.fn) continue;
          e = cudaFuncSetAttribute(pk.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pk.smem);
          if (e != cudaSuccess) break;
          e = cudaFuncSetAttribute(pk.fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared);
          if (e != cudaSuccess) break;
          int occ = 0;
          e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk.fn, pk.threads, pk.smem);
          if (e != cudaSuccess) break;
          // Own bound from the resources a CTA holds (registers, shared memory,
          // threads); the larger of this and the runtime's answer is used.
          cudaFuncAttributes fa;
          e = cudaFuncGetAttributes(&fa, pk.fn);
          if (e != cudaSuccess) break;
          const int regs_per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
          const int by_regs = 65536 / (regs_per_warp * (pk.threads / 32));
          const int by_smem = (228 * 1024) / (pk.smem + static_cast<int>(fa.sharedSizeBytes) + 1024);
          const int by_threads = 2048 / pk.threads;
          int own = by_regs < by_smem ? by_regs : by_smem;
          own = own < by_threads ? own : by_threads;
          if (own > occ) occ = own;
          // TMEM: 512 columns per SM; a CTA holds Mt/4 (FP16) or Mt/2 (split)
          // columns.
          const int tmem_limit = 512 / (pk.Mt / (pr == kPrecF16 ? 4 : 2));
          g_occ[pr][k][l][t][s] = occ < tmem_limit ? occ : tmem_limit;
        }
  for (int l = kFusedMinLog; l <= kFusedMaxLog && e == cudaSuccess; ++l)
    for (int sg = 0; sg < 2 && e == cudaSuccess; ++sg) {
      FusedKernel& fk = g_fused[l][sg];
      if (!fk.fn) continue;
      e = cudaFuncSetAttribute(fk.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, fk.smem);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fk.fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
      cudaFuncAttributes fa;
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fk.fn);
      if (e != cudaSuccess) break;
      const int regs_per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
      int occ = 65536 / (regs_per_warp * (kPassThreads / 32));
      const int by_smem = (228 * 1024) / (fk.smem + static_cast<int>(fa.sharedSizeBytes) + 1024);
      if (by_smem < occ) occ = by_smem;
      const int cols1 = (16384 / 16 / 128) * 32;  // Mt = 1024 tiles: 256 TMEM columns
      if (512 / cols1 < occ) occ = 512 / cols1;
      g_fused_occ[l][sg] = occ < 1 ? 1 : occ;
    }
  g_init_err = e;
}

tcfftStatus ensure_init() {
  std::call_once(g_once, init_registry);
  if (g_init_err != cudaSuccess) return TCFFT_NO_DEVICE;
  return TCFFT_OK;
}

int ilog2ll(long long v) {
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

bool is_pow2(long long v) { return v > 0 && (v & (v - 1)) == 0; }

}  // namespace

namespace tcfft {

tcfftStatus registry_ready() { return ensure_init(); }

const FusedKernel* fused_kernel(int logn, int sign_idx, int* grid_ctas) {
  if (logn < kFusedMinLog || logn > kFusedMaxLog || sign_idx < 0 || sign_idx > 1) return nullptr;
  const FusedKernel& fk = g_fused[logn][sign_idx];
  if (!fk.fn) return nullptr;
  if (grid_ctas) *grid_ctas = g_num_sms * g_fused_occ[logn][sign_idx];
  return &fk;
}

static constexpr unsigned int kDefaultWaitPolls = 1u << 24;
static std::atomic<unsigned int> g_wait_polls{kDefaultWaitPolls};

unsigned int dep_wait_polls() { return g_wait_polls.load(std::memory_order_relaxed); }

tcfftStatus record_status(tcfftStatus s, int launches) {
  g_last_launches = launches;
  return ret(s);
}

}  // namespace tcfft

struct tcfftPlanImpl {
  int dims = 1;
  long long n = 0, batch = 0;
  int nx = 0, ny = 0;
  int precision = TCFFT_FP16;
  int log_n1 = 0, log_n2 = 0;  // 1D four-step split (log_n1 == 0: single pass)
  float2* tw[2][kMaxLogL + 1] = {};
  uint16_t* bmat[2] = {};
  float2* otw_hi[2] = {};
  float2* otw_lo[2] = {};
  int otw_shift = 0, otw_logn = 0;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  void* perm_ws = nullptr;  // un-permute buffer for in-place digit-reversed input
  // fused four-step (FP16, 2^15 <= n <= 2^24): one launch, workspace ring
  bool fused = false;
  int chunk_seqs = 0, nchunks = 0, ring = 0;
  void* ring_ws = nullptr;
  int* counters = nullptr;  // [0] item counter, then done1[nchunks], done2[nchunks]
  int* err = nullptr;
};

namespace {

tcfftStatus ensure_twiddle(tcfftPlanImpl* p, int logL) {
  for (int s = 0; s < 2; ++s) {
    if (p->tw[s][logL]) continue;
    const long long L = 1ll << logL;
    if (cudaMalloc(&p->tw[s][logL], sizeof(float2) * L) != cudaSuccess) return TCFFT_ALLOC_FAILED;
    if (gen_twiddles(p->tw[s][logL], L, logL, 0, s == 0 ? -1 : 1, 0) != cudaSuccess)
      return TCFFT_LAUNCH_FAILED;
  }
  return TCFFT_OK;
}

tcfftStatus common_tables(tcfftPlanImpl* p) {
  for (int s = 0; s < 2; ++s) {
    if (cudaMalloc(&p->bmat[s], 2048 * 2) != cudaSuccess) return TCFFT_ALLOC_FAILED;
    if (gen_dft16_bmat(p->bmat[s], s == 0 ? -1 : 1, 0, 0) != cudaSuccess) return TCFFT_LAUNCH_FAILED;
    if (gen_dft16_bmat(p->bmat[s] + 1024, s == 0 ? -1 : 1, 1, 0) != cudaSuccess)
      return TCFFT_LAUNCH_FAILED;
  }
  if (cudaMalloc(&p->err, sizeof(int)) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  if (cudaMemset(p->err, 0, sizeof(int)) != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  return TCFFT_OK;
}

void free_plan(tcfftPlanImpl* p) {
  if (!p) return;
  for (int s = 0; s < 2; ++s) {
    for (int l = 0; l <= kMaxLogL; ++l) cudaFree(p->tw[s][l]);
    cudaFree(p->bmat[s]);
    cudaFree(p->otw_hi[s]);
    cudaFree(p->otw_lo[s]);
  }
  cudaFree(p->ws);
  cudaFree(p->perm_ws);
  cudaFree(p->ring_ws);
  cudaFree(p->counters);
  cudaFree(p->err);
  delete p;
}

// Launch one pass; grid = persistent CTAs (at most the co-resident count).
// 3D tensor map over column-layout lines: x = line within its sequence
// (lines adjacent in memory), y = element (stride elem_stride), z = sequence
// (stride seq_stride); 4-byte elements, boxes of G lines x min(L, 256)
// elements. False when the layout breaks a TMA rule (the caller keeps the
// cp.async path then).
// esize: bytes per element (4: FP16 complex, 8: FP32 complex).
bool encode_column_map(CUtensorMap* map, const void* base, long long lines_per_seq, long long nseq, int L,
                       long long elem_stride, long long seq_stride, int G, int esize) {
  if ((reinterpret_cast<uintptr_t>(base) & 15u) || (elem_stride * esize) % 16 || (seq_stride * esize) % 16 ||
      (G * esize) % 16)
    return false;
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(lines_per_seq), static_cast<cuuint64_t>(L),
                              static_cast<cuuint64_t>(nseq)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(elem_stride * esize),
                                 static_cast<cuuint64_t>(seq_stride * esize)};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>(G), static_cast<cuuint32_t>(L < 256 ? L : 256), 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  // the driver's encoder, found through the runtime (the library does not
  // link the driver library itself)
  static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return false;
  // element type only sets the size: tile copies move bytes unchanged
  const CUtensorMapDataType dtype = esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  return encode(map, dtype, 3, const_cast<void*>(base), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Column-layout tiles move by TMA when every tile lies inside one sequence:
// FP16 prefetching (mid-tile) kernels load and store them that way; the
// split-precision kernels store narrow tiles (G <= 8 lines, whose direct
// 8-byte stores touch only G * 8 contiguous bytes per element) that way,
// since staging waits for every MMA group and wider tiles store well directly.
template <class IO>
void attach_tensor_maps(IO& io, int kind, int tile, int logL, int G) {
  if constexpr (TensorMapIo<IO>) {
    constexpr int esize = static_cast<int>(sizeof(*io.out));
    constexpr bool split = esize == 8;
    io.in_tma = io.out_tma = false;
    if (kind == kPassRow || (!split && tile != kTileMid && tile != kTileNarrow)) return;
    const long long lps = 1ll << io.lps_log2;
    if (lps % G != 0 || io.total_lines % lps != 0 || G % 4 != 0) return;
    const long long nseq = io.total_lines / lps;
    const int L = 1 << logL;
    if (!IO::IN_VEC_L && io.in_line == 1)  // split: used for L2 prefetches of the next tile
      io.in_tma = encode_column_map(&io.in_map, io.in, lps, nseq, L, io.in_elem, io.in_seq, G, esize);
    if (!IO::OUT_VEC_L && io.out_line == 1 && (!split || G <= 8))
      io.out_tma = encode_column_map(&io.out_map, io.out, lps, nseq, L, io.out_elem, io.out_seq, G, esize);
  }
}

template <class IO>
tcfftStatus launch_pass(int prec, int kind, int logL, int tile, int sign_idx, const IO& io_in, const PassCore& core,
                        cudaStream_t stream) {
  const PassKernel& pk = g_tab[prec][kind][logL][tile][sign_idx];
  if (!pk.fn) return TCFFT_UNSUPPORTED;
  IO io = io_in;
  attach_tensor_maps(io, kind, tile, logL, pk.G);
  const long long ntiles = (io.total_lines + pk.G - 1) / pk.G;
  long long grid = static_cast<long long>(g_num_sms) * g_occ[prec][kind][logL][tile][sign_idx];
  if (grid < 1) grid = 1;
  if (grid > ntiles) grid = ntiles;
  void* kargs[] = {const_cast<IO*>(&io), const_cast<PassCore*>(&core)};
  cudaError_t e = cudaLaunchKernel(pk.fn, dim3(static_cast<unsigned>(grid)), dim3(pk.threads), kargs,
                                   static_cast<size_t>(pk.smem), stream);
  if (e != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  ++g_last_launches;
  return TCFFT_OK;
}

// Tile variant for a pass: the tuned choice if one is set and built;
// otherwise narrow or mid tiles when they fill the GPU, else big tiles, or
// small ones when big ones would leave SMs idle.
int choose_tile(int prec, int kind, int logL, long long lines) {
  std::call_once(g_tune_once, tune_reset);
  const PassKernel& small = g_tab[prec][kind][logL][kTileSmall][0];
  const PassKernel& big = g_tab[prec][kind][logL][kTileBig][0];
  const PassKernel& mid = g_tab[prec][kind][logL][kTileMid][0];
  const PassKernel& narrow = g_tab[prec][kind][logL][kTileNarrow][0];
  const int t = g_tune[prec][kind][logL];
  if (t >= 0 && t < kNumTileSel && g_tab[prec][kind][logL][t][0].fn) {
    // A preferred (tuning-file) variant was measured on batches that fill
    // the GPU. A batch that its FP16 tiles would spread over fewer than two
    // tiles per SM runs faster on narrow tiles when they are smaller (more
    // CTAs of 128 threads): N = 256 x 4096 forward + inverse 15.1 -> 14.0 us
    // from a CUDA graph against the tuned 512-row tiles.
    const int tg = g_tab[prec][kind][logL][t][0].G;
    const bool underfilled = (lines + tg - 1) / tg < 2ll * g_num_sms;
    if (g_tune_pref[prec][kind][logL] && prec == kPrecF16 && underfilled && narrow.fn && narrow.G < tg &&
        (kind == kPassRow || narrow.G >= 8))
      return kTileNarrow;
    return t;
  }
  // FP16 narrow tiles (256 rows on 128 threads, 6 CTAs/SM) when they fill
  // the GPU and column-layout rows of the tile stay >= 32 bytes (G >= 8):
  // the tuner's choice at every such length on GB300
  if (prec == kPrecF16 && narrow.fn && (kind == kPassRow || narrow.G >= 8) &&
      (lines + narrow.G - 1) / narrow.G >= 6ll * g_num_sms)
    return kTileNarrow;
  // prefetching mid tiles (3 CTAs/SM) when they fill the GPU, measured fastest
  if (mid.fn && (lines + mid.G - 1) / mid.G >= 3ll * g_num_sms) return kTileMid;
  if (!small.fn || !big.fn) return big.fn ? kTileBig : (mid.fn ? kTileMid : kTileSmall);
  const long long big_tiles = (lines + big.G - 1) / big.G;
  return big_tiles >= 2ll * g_num_sms ? kTileBig : kTileSmall;
}

PassCore make_core(tcfftPlanImpl* p, int sign_idx, int logL) {
  PassCore c;
  c.tw = p->tw[sign_idx][logL];
  c.bmat = reinterpret_cast<const uint32_t*>(p->bmat[sign_idx]);
  c.err = p->err;
  return c;
}

template <class IO, class E>
IO make_io(const void* in, void* out, long long total_lines, int lps_log2, float scale) {
  IO io;
  std::memset(&io, 0, sizeof(io));
  io.in = static_cast<const E*>(in);
  io.out = static_cast<E*>(out);
  io.total_lines = total_lines;
  io.lps_log2 = lps_log2;
  io.scale = scale;
  return io;
}

// The three pass shapes of a transform, for either storage precision.
template <template <bool, bool> class IOT, class E>
tcfftStatus exec_passes(tcfftPlanImpl* p, int prec, const void* in, void* out, int sg, float scale,
                        cudaStream_t st) {
  tcfftStatus s = TCFFT_OK;
  if (p->dims == 1 && p->log_n1 == 0) {
    const int logL = ilog2ll(p->n);
    auto io = make_io<IOT<true, true>, E>(in, out, p->batch, 0, scale);
    io.in_seq = io.out_seq = p->n;
    io.in_elem = io.out_elem = 1;
    io.in_contig = io.out_contig = true;
    io.contig_len = p->n;
    s = launch_pass(prec, kPassRow, logL, choose_tile(prec, kPassRow, logL, p->batch), sg, io, make_core(p, sg, logL), st);
  } else if (p->dims == 1) {
    const long long n1 = 1ll << p->log_n1, n2 = 1ll << p->log_n2;
    // pass 1: length-n1 FFTs down the columns of [n1][n2], times W_N^{n2*k1}
    auto a = make_io<IOT<false, false>, E>(in, p->ws, p->batch * n2, p->log_n2, 1.0f);
    a.in_seq = a.out_seq = p->n;
    a.in_line = a.out_line = 1;
    a.in_elem = a.out_elem = n2;
    a.otw.hi = p->otw_hi[sg];
    a.otw.lo = p->otw_lo[sg];
    a.otw.shift = p->otw_shift;
    a.otw.logn = p->otw_logn;
    s = launch_pass(prec, kPassCol, p->log_n1, choose_tile(prec, kPassCol, p->log_n1, a.total_lines), sg, a,
                    make_core(p, sg, p->log_n1), st);
    if (s == TCFFT_OK) {
      // pass 2: length-n2 FFTs along the rows, row k1 -> X[k1 + n1*k2]
      auto b = make_io<IOT<true, false>, E>(p->ws, out, p->batch * n1, p->log_n1, scale);
      b.in_seq = b.out_seq = p->n;
      b.in_line = n2;
      b.in_elem = 1;
      b.out_line = 1;
      b.out_elem = n1;
      b.in_contig = true;  // rows k1 of consecutive sequences follow each other
      b.contig_len = n2;
      s = launch_pass(prec, kPassRowT, p->log_n2, choose_tile(prec, kPassRowT, p->log_n2, b.total_lines), sg, b,
                      make_core(p, sg, p->log_n2), st);
    }
  } else {
    const int lx = ilog2ll(p->nx), ly = ilog2ll(p->ny);
    // rows: length ny, contiguous
    auto a = make_io<IOT<true, true>, E>(in, out, p->batch * p->nx, 0, 1.0f);
    a.in_seq = a.out_seq = p->ny;
    a.in_elem = a.out_elem = 1;
    a.in_contig = a.out_contig = true;
    a.contig_len = p->ny;
    s = launch_pass(prec, kPassRow, ly, choose_tile(prec, kPassRow, ly, a.total_lines), sg, a, make_core(p, sg, ly), st);
    if (s == TCFFT_OK) {
      // columns: length nx, stride ny, in place
      auto b = make_io<IOT<false, false>, E>(out, out, p->batch * p->ny, ly, scale);
      b.in_seq = b.out_seq = p->n;
      b.in_line = b.out_line = 1;
      b.in_elem = b.out_elem = p->ny;
      s = launch_pass(prec, kPassCol, lx, choose_tile(prec, kPassCol, lx, b.total_lines), sg, b, make_core(p, sg, lx), st);
    }
  }
  return s;
}

// Both four-step passes in one persistent launch (see fft_fused.cuh).
tcfftStatus exec_fused(tcfftPlanImpl* p, const void* in, void* out, int sg, float scale, cudaStream_t st) {
  const int logn = p->log_n1 + p->log_n2;
  const FusedKernel& fk = g_fused[logn][sg];
  const long long n1 = 1ll << p->log_n1, n2 = 1ll << p->log_n2;
  IoHalf<false, false> a;
  std::memset(&a, 0, sizeof(a));
  a.in = static_cast<const half2*>(in);
  a.out = static_cast<half2*>(p->ring_ws);
  a.lps_log2 = p->log_n2;
  a.in_seq = a.out_seq = p->n;
  a.in_line = a.out_line = 1;
  a.in_elem = a.out_elem = n2;
  a.otw.hi = p->otw_hi[sg];
  a.otw.lo = p->otw_lo[sg];
  a.otw.shift = p->otw_shift;
  a.otw.logn = p->otw_logn;
  a.scale = 1.0f;
  IoHalf<true, false, true> b;
  std::memset(&b, 0, sizeof(b));
  b.in = static_cast<const half2*>(p->ring_ws);
  b.out = static_cast<half2*>(out);
  b.lps_log2 = p->log_n1;
  b.in_seq = b.out_seq = p->n;
  b.in_line = n2;
  b.in_elem = 1;
  b.out_line = 1;
  b.out_elem = n1;
  b.scale = scale;
  PassCore c1 = make_core(p, sg, p->log_n1), c2 = make_core(p, sg, p->log_n2);
  FusedSched sc;
  sc.counter = reinterpret_cast<unsigned int*>(p->counters);
  sc.done1 = p->counters + 1;
  sc.done2 = p->counters + 1 + p->nchunks;
  sc.nchunks = p->nchunks;
  sc.tiles1 = static_cast<int>((static_cast<long long>(p->chunk_seqs) * n2 + fk.G1 - 1) / fk.G1);
  sc.tiles2 = static_cast<int>((static_cast<long long>(p->chunk_seqs) * n1 + fk.G2 - 1) / fk.G2);
  sc.ring = p->ring;
  sc.chunk_seqs = p->chunk_seqs;
  sc.batch = p->batch;
  sc.n = p->n;
  sc.wait_polls = dep_wait_polls();
  if (cudaMemsetAsync(p->counters, 0, sizeof(int) * (1 + 2 * static_cast<size_t>(p->nchunks)), st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  long long items = static_cast<long long>(sc.nchunks) * (sc.tiles1 + sc.tiles2);
  long long grid = static_cast<long long>(g_num_sms) * g_fused_occ[logn][sg];
  if (grid > items) grid = items;
  void* args[] = {&a, &b, &c1, &c2, &sc};
  if (cudaLaunchKernel(fk.fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), args,
                       static_cast<size_t>(fk.smem), st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  ++g_last_launches;
  return TCFFT_OK;
}

__global__ void digitrev_gather_kernel(const half2* __restrict__ in, half2* __restrict__ out,
                                       long long n, long long total, int nrad, int4 r03, int4 r47,
                                       int r8) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= total) return;
  const long long b = i / n, l = i % n;
  const int rad[9] = {r03.x, r03.y, r03.z, r03.w, r47.x, r47.y, r47.z, r47.w, r8};
  long long rest = l, span = n, pos = 0;
  for (int k = nrad - 1; k >= 0; --k) {
    const int r = rad[k];
    const long long d = rest % r;
    rest /= r;
    span /= r;
    pos += d * span;
  }
  out[i] = in[b * n + pos];
}

// Storage position of natural index l under a digit-reversal radix list
// (inverse of the reference's gen_rev permutation).
__device__ __forceinline__ long long digitrev_pos(long long l, long long n, const int* rad, int nrad) {
  long long rest = l, span = n, pos = 0;
  for (int k = nrad - 1; k >= 0; --k) {
    const int r = rad[k];
    const long long d = rest % r;
    rest /= r;
    span /= r;
    pos += d * span;
  }
  return pos;
}

struct Radix9 {
  int r[9];
};

__global__ void digitrev_gather_2d_kernel(const half2* __restrict__ in, half2* __restrict__ out, int nx, int ny,
                                          long long total, Radix9 rx, int nrx, Radix9 ry, int nry) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= total) return;
  const long long plane = static_cast<long long>(nx) * ny;
  const long long b = i / plane;
  const int row = static_cast<int>((i % plane) / ny), col = static_cast<int>(i % ny);
  const long long pr = nrx > 0 ? digitrev_pos(row, nx, rx.r, nrx) : row;
  const long long pc = nry > 0 ? digitrev_pos(col, ny, ry.r, nry) : col;
  out[i] = in[b * plane + pr * ny + pc];
}

}  // namespace

extern "C" {

tcfftStatus tcfft_plan_1d(tcfftPlan* plan, long long n, long long batch, int precision) {
  if (!plan) return ret(TCFFT_INVALID_VALUE);
  *plan = nullptr;
  if (!is_pow2(n) || n < 16 || n > (1ll << 24) || batch < 1) return ret(TCFFT_INVALID_SIZE);
  if (precision != TCFFT_FP16 && precision != TCFFT_SPLIT_FP32) return ret(TCFFT_INVALID_VALUE);
  // split precision: single pass up to 2^13, two passes up to 2^11 x 2^11
  if (precision == TCFFT_SPLIT_FP32 && n > (1ll << 22)) return ret(TCFFT_INVALID_SIZE);
  tcfftStatus s = ensure_init();
  if (s != TCFFT_OK) return ret(s);
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return ret(TCFFT_ALLOC_FAILED);
  p->dims = 1;
  p->n = n;
  p->batch = batch;
  p->precision = precision;
  const int logn = ilog2ll(n);
  s = common_tables(p);
  if (s == TCFFT_OK) {
    const int single_max = precision == TCFFT_FP16 ? kMaxLogL : 13;
    const int pass_max = precision == TCFFT_FP16 ? 12 : 11;
    if (logn <= single_max) {
      s = ensure_twiddle(p, logn);
    } else {
      // column pass length 2^a, row pass length 2^(logn - a), both <= 2^pass_max
      int a = logn / 2 < 10 ? logn / 2 : 10;
      if (logn - a > pass_max) a = logn - pass_max;
      std::call_once(g_tune_once, tune_reset);
      const int pr = precision == TCFFT_FP16 ? kPrecF16 : kPrecSplit;
      const int tuned = g_split[pr][logn];
      if (tuned >= 0 && pass_built(pr, kPassCol, tuned) && pass_built(pr, kPassRowT, logn - tuned)) a = tuned;
      p->log_n1 = a;
      p->log_n2 = logn - a;
      s = ensure_twiddle(p, p->log_n1);
      if (s == TCFFT_OK) s = ensure_twiddle(p, p->log_n2);
      p->otw_logn = logn;
      p->otw_shift = (logn + 1) / 2;
      for (int d = 0; d < 2 && s == TCFFT_OK; ++d) {
        const long long nlo = 1ll << p->otw_shift, nhi = 1ll << (logn - p->otw_shift);
        if (cudaMalloc(&p->otw_lo[d], sizeof(float2) * nlo) != cudaSuccess ||
            cudaMalloc(&p->otw_hi[d], sizeof(float2) * nhi) != cudaSuccess) {
          s = TCFFT_ALLOC_FAILED;
          break;
        }
        const int sg = d == 0 ? -1 : 1;
        if (gen_twiddles(p->otw_lo[d], nlo, logn, 0, sg, 0) != cudaSuccess ||
            gen_twiddles(p->otw_hi[d], nhi, logn, p->otw_shift, sg, 0) != cudaSuccess)
          s = TCFFT_LAUNCH_FAILED;
      }
      const bool can_fuse = precision == TCFFT_FP16 && logn >= kFusedMinLog && logn <= kFusedMaxLog &&
                            g_fused[logn][0].fn && g_fused[logn][0].log_n1 == p->log_n1;
      if (s == TCFFT_OK && can_fuse) {
        // fused form available (tcfft_plan_set_fused): chunks of ~16 MiB in a
        // ring of two workspace slots, allocated when it is switched on
        const long long per_seq = n * 4;
        long long cs = (16ll << 20) / per_seq;
        if (cs < 1) cs = 1;
        if (cs > batch) cs = batch;
        p->chunk_seqs = static_cast<int>(cs);
        p->nchunks = static_cast<int>((batch + cs - 1) / cs);
        p->ring = p->nchunks >= 2 ? 2 : 1;
      }
      // default: two pass launches through a full-size workspace (faster than
      // the fused launch on every size measured so far)
      if (s == TCFFT_OK) {
        p->ws_bytes = static_cast<size_t>(n) * static_cast<size_t>(batch) * (precision == TCFFT_FP16 ? 4u : 8u);
        if (cudaMalloc(&p->ws, p->ws_bytes) != cudaSuccess) s = TCFFT_ALLOC_FAILED;
      }
    }
  }
  if (s == TCFFT_OK && cudaDeviceSynchronize() != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
  if (s != TCFFT_OK) {
    free_plan(p);
    return ret(s);
  }
  *plan = p;
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_plan_2d(tcfftPlan* plan, int nx, int ny, long long batch, int precision) {
  if (!plan) return ret(TCFFT_INVALID_VALUE);
  *plan = nullptr;
  if (!is_pow2(nx) || !is_pow2(ny) || nx < 16 || ny < 16 || nx > 4096 || ny > 4096 || batch < 1)
    return ret(TCFFT_INVALID_SIZE);
  if (precision != TCFFT_FP16 && precision != TCFFT_SPLIT_FP32) return ret(TCFFT_INVALID_VALUE);
  if (precision == TCFFT_SPLIT_FP32 && (nx > 2048 || ny > 8192)) return ret(TCFFT_INVALID_SIZE);
  tcfftStatus s = ensure_init();
  if (s != TCFFT_OK) return ret(s);
  tcfftPlanImpl* p = new (std::nothrow) tcfftPlanImpl();
  if (!p) return ret(TCFFT_ALLOC_FAILED);
  p->dims = 2;
  p->nx = nx;
  p->ny = ny;
  p->n = static_cast<long long>(nx) * ny;
  p->batch = batch;
  p->precision = precision;
  s = common_tables(p);
  if (s == TCFFT_OK) s = ensure_twiddle(p, ilog2ll(nx));
  if (s == TCFFT_OK) s = ensure_twiddle(p, ilog2ll(ny));
  if (s == TCFFT_OK && cudaDeviceSynchronize() != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
  if (s != TCFFT_OK) {
    free_plan(p);
    return ret(s);
  }
  *plan = p;
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_plan_set_fused(tcfftPlan p, int enable) {
  if (!p) return ret(TCFFT_INVALID_VALUE);
  if (enable) {
    if (p->chunk_seqs == 0) return ret(TCFFT_UNSUPPORTED);
    if (!p->ring_ws) {
      const size_t ring_bytes =
          static_cast<size_t>(p->ring) * static_cast<size_t>(p->chunk_seqs) * static_cast<size_t>(p->n) * 4u;
      if (cudaMalloc(&p->ring_ws, ring_bytes) != cudaSuccess) return ret(TCFFT_ALLOC_FAILED);
      if (cudaMalloc(&p->counters, sizeof(int) * (1 + 2 * static_cast<size_t>(p->nchunks))) != cudaSuccess) {
        cudaFree(p->ring_ws);
        p->ring_ws = nullptr;
        return ret(TCFFT_ALLOC_FAILED);
      }
    }
    p->fused = true;
    return ret(TCFFT_OK);
  }
  if (!p->fused) return ret(TCFFT_OK);
  if (!p->ws) {
    const size_t bytes = static_cast<size_t>(p->n) * static_cast<size_t>(p->batch) * 4u;
    if (cudaMalloc(&p->ws, bytes) != cudaSuccess) return ret(TCFFT_ALLOC_FAILED);
  }
  p->fused = false;
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_workspace_bytes(tcfftPlan plan, size_t* bytes) {
  if (!plan || !bytes) return ret(TCFFT_INVALID_VALUE);
  *bytes = plan->ws_bytes;
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_exec(tcfftPlan p, const void* in, void* out, int direction, float scale, void* stream) {
  g_last_launches = 0;
  if (!p || !in || !out) return ret(TCFFT_INVALID_VALUE);
  if (direction != TCFFT_FORWARD && direction != TCFFT_INVERSE) return ret(TCFFT_INVALID_VALUE);
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u)
    return ret(TCFFT_INVALID_VALUE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int sg = direction == TCFFT_FORWARD ? 0 : 1;
  tcfftStatus s;
  if (p->fused)
    s = exec_fused(p, in, out, sg, scale, st);
  else if (p->precision == TCFFT_FP16)
    s = exec_passes<IoHalf, half2>(p, kPrecF16, in, out, sg, scale, st);
  else
    s = exec_passes<IoFloat, float2>(p, kPrecSplit, in, out, sg, scale, st);
  return ret(s);
}

tcfftStatus tcfft_exec_digitrev(tcfftPlan p, const void* in, void* out, const int* radices, int n_radices,
                                void* stream) {
  g_last_launches = 0;
  if (!p || !in || !out || (n_radices > 0 && !radices) || n_radices < 0 || n_radices > 9)
    return ret(TCFFT_INVALID_VALUE);
  if (p->dims != 1 || p->precision != TCFFT_FP16) return ret(TCFFT_UNSUPPORTED);
  long long prod = 1;
  int rad[9] = {1, 1, 1, 1, 1, 1, 1, 1, 1};
  for (int i = 0; i < n_radices; ++i) {
    if (radices[i] < 2) return ret(TCFFT_INVALID_VALUE);
    rad[i] = radices[i];
    prod *= radices[i];
  }
  if (n_radices > 0 && prod != p->n) return ret(TCFFT_INVALID_SIZE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const void* src = in;
  if (n_radices > 0) {
    // un-permute into the output buffer (or the workspace when in place)
    void* dst = out;
    if (in == out) {
      // first in-place call allocates the un-permute buffer (kept by the plan)
      if (!p->perm_ws &&
          cudaMalloc(&p->perm_ws, static_cast<size_t>(p->n) * static_cast<size_t>(p->batch) * 4u) !=
              cudaSuccess)
        return ret(TCFFT_ALLOC_FAILED);
      dst = p->perm_ws;
    }
    const long long total = p->n * p->batch;
    const int threads = 256;
    digitrev_gather_kernel<<<static_cast<unsigned>((total + threads - 1) / threads), threads, 0, st>>>(
        static_cast<const half2*>(in), static_cast<half2*>(dst), p->n, total, n_radices,
        make_int4(rad[0], rad[1], rad[2], rad[3]), make_int4(rad[4], rad[5], rad[6], rad[7]), rad[8]);
    if (cudaGetLastError() != cudaSuccess) return ret(TCFFT_LAUNCH_FAILED);
    src = dst;
  }
  const int launches_before = n_radices > 0 ? 1 : 0;
  tcfftStatus s = tcfft_exec(p, src, out, TCFFT_FORWARD, 1.0f, stream);
  g_last_launches += launches_before;
  return ret(s);
}

tcfftStatus tcfft_exec_digitrev_2d(tcfftPlan p, const void* in, void* out, const int* radices_x, int n_radices_x,
                                   const int* radices_y, int n_radices_y, int direction, void* stream) {
  g_last_launches = 0;
  if (!p || !in || !out || n_radices_x < 0 || n_radices_x > 9 || n_radices_y < 0 || n_radices_y > 9 ||
      (n_radices_x > 0 && !radices_x) || (n_radices_y > 0 && !radices_y))
    return ret(TCFFT_INVALID_VALUE);
  if (p->dims != 2 || p->precision != TCFFT_FP16) return ret(TCFFT_UNSUPPORTED);
  Radix9 rx{}, ry{};
  long long px = 1, py = 1;
  for (int i = 0; i < n_radices_x; ++i) {
    if (radices_x[i] < 2) return ret(TCFFT_INVALID_VALUE);
    rx.r[i] = radices_x[i];
    px *= radices_x[i];
  }
  for (int i = 0; i < n_radices_y; ++i) {
    if (radices_y[i] < 2) return ret(TCFFT_INVALID_VALUE);
    ry.r[i] = radices_y[i];
    py *= radices_y[i];
  }
  if ((n_radices_x > 0 && px != p->nx) || (n_radices_y > 0 && py != p->ny)) return ret(TCFFT_INVALID_SIZE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const void* src = in;
  if (n_radices_x > 0 || n_radices_y > 0) {
    void* dst = out;
    if (in == out) {
      if (!p->perm_ws &&
          cudaMalloc(&p->perm_ws, static_cast<size_t>(p->n) * static_cast<size_t>(p->batch) * 4u) != cudaSuccess)
        return ret(TCFFT_ALLOC_FAILED);
      dst = p->perm_ws;
    }
    const long long total = p->n * p->batch;
    const int threads = 256;
    digitrev_gather_2d_kernel<<<static_cast<unsigned>((total + threads - 1) / threads), threads, 0, st>>>(
        static_cast<const half2*>(in), static_cast<half2*>(dst), p->nx, p->ny, total, rx, n_radices_x, ry,
        n_radices_y);
    if (cudaGetLastError() != cudaSuccess) return ret(TCFFT_LAUNCH_FAILED);
    src = dst;
  }
  const int before = src != in ? 1 : 0;
  tcfftStatus s = tcfft_exec(p, src, out, direction, 1.0f, stream);
  g_last_launches += before;
  return ret(s);
}

tcfftStatus tcfft_check(tcfftPlan p, void* stream) {
  if (!p) return ret(TCFFT_INVALID_VALUE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return ret(TCFFT_LAUNCH_FAILED);
  int h = 0;
  if (cudaMemcpy(&h, p->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return ret(TCFFT_LAUNCH_FAILED);
  if (h != 0) {
    cudaMemset(p->err, 0, sizeof(int));
    // a bounded wait gave up: on the tensor cores / a copy, or (fused form)
    // on a work item the item depended on
    return ret((h & (kErrMmaTimeout | kErrQueueTimeout)) ? TCFFT_TIMEOUT : TCFFT_LAUNCH_FAILED);
  }
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_destroy(tcfftPlan p) {
  if (!p) return ret(TCFFT_INVALID_VALUE);
  free_plan(p);
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_get_last_error(void) { return g_last; }

const char* tcfft_status_string(tcfftStatus s) {
  switch (s) {
    case TCFFT_OK: return "TCFFT_OK";
    case TCFFT_INVALID_SIZE: return "TCFFT_INVALID_SIZE";
    case TCFFT_UNSUPPORTED: return "TCFFT_UNSUPPORTED";
    case TCFFT_ALLOC_FAILED: return "TCFFT_ALLOC_FAILED";
    case TCFFT_LAUNCH_FAILED: return "TCFFT_LAUNCH_FAILED";
    case TCFFT_TIMEOUT: return "TCFFT_TIMEOUT";
    case TCFFT_CAPACITY: return "TCFFT_CAPACITY";
    case TCFFT_INVALID_VALUE: return "TCFFT_INVALID_VALUE";
    case TCFFT_NO_DEVICE: return "TCFFT_NO_DEVICE";
  }
  return "TCFFT_UNKNOWN";
}

tcfftStatus tcfft_set_wait_limit(long long polls) {
  if (polls > static_cast<long long>(kDefaultWaitPolls)) return ret(TCFFT_INVALID_VALUE);
  g_wait_polls.store(polls < 0 ? kDefaultWaitPolls : static_cast<unsigned int>(polls), std::memory_order_relaxed);
  return ret(TCFFT_OK);
}

int tcfft_last_launch_count(void) { return g_last_launches; }

namespace {
tcfftStatus tune_store(int precision, int pass_kind, int log2_len, int tile, bool preferred) {
  if (precision < 0 || precision >= kNumPrec || pass_kind < 0 || pass_kind >= kNumPassKinds || log2_len < 0 ||
      log2_len > kMaxLogL || tile < -1 || tile >= kNumTileSel)
    return ret(TCFFT_INVALID_VALUE);
  std::call_once(g_tune_once, tune_reset);
  tcfftStatus s = ensure_init();
  if (s != TCFFT_OK) return ret(s);
  if (tile >= 0 && !g_tab[precision][pass_kind][log2_len][tile][0].fn) return ret(TCFFT_UNSUPPORTED);
  g_tune[precision][pass_kind][log2_len] = tile;
  g_tune_pref[precision][pass_kind][log2_len] = preferred;
  return ret(TCFFT_OK);
}
}  // namespace

tcfftStatus tcfft_tune_set(int precision, int pass_kind, int log2_len, int tile) {
  return tune_store(precision, pass_kind, log2_len, tile, false);
}

tcfftStatus tcfft_tune_prefer(int precision, int pass_kind, int log2_len, int tile) {
  return tune_store(precision, pass_kind, log2_len, tile, true);
}

tcfftStatus tcfft_tune_split(int precision, int log2_n, int log2_n1) {
  if (precision < 0 || precision >= kNumPrec || log2_n < 0 || log2_n > kMaxLogN || log2_n1 < -1)
    return ret(TCFFT_INVALID_VALUE);
  std::call_once(g_tune_once, tune_reset);
  tcfftStatus s = ensure_init();
  if (s != TCFFT_OK) return ret(s);
  if (log2_n1 >= 0 && (!pass_built(precision, kPassCol, log2_n1) || !pass_built(precision, kPassRowT, log2_n - log2_n1)))
    return ret(TCFFT_UNSUPPORTED);
  g_split[precision][log2_n] = log2_n1;
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_tune_get(int precision, int pass_kind, int log2_len, int* tile) {
  if (!tile || precision < 0 || precision >= kNumPrec || pass_kind < 0 || pass_kind >= kNumPassKinds ||
      log2_len < 0 || log2_len > kMaxLogL)
    return ret(TCFFT_INVALID_VALUE);
  std::call_once(g_tune_once, tune_reset);
  *tile = g_tune[precision][pass_kind][log2_len];
  return ret(TCFFT_OK);
}

tcfftStatus tcfft_pass_info(int precision, int pass_kind, int log2_len, int tile, int* lines_per_tile,
                            int* ctas_per_sm, int* num_sms) {
  if (precision < 0 || precision >= kNumPrec || pass_kind < 0 || pass_kind >= kNumPassKinds || log2_len < 0 ||
      log2_len > kMaxLogL || tile < 0 || tile >= kNumTileSel)
    return ret(TCFFT_INVALID_VALUE);
  tcfftStatus s = ensure_init();
  if (s != TCFFT_OK) return ret(s);
  const PassKernel& pk = g_tab[precision][pass_kind][log2_len][tile][0];
  if (!pk.fn) return ret(TCFFT_UNSUPPORTED);
  if (lines_per_tile) *lines_per_tile = pk.G;
  if (ctas_per_sm) *ctas_per_sm = g_occ[precision][pass_kind][log2_len][tile][0];
  if (num_sms) *num_sms = g_num_sms;
  return ret(TCFFT_OK);
}

}  // extern "C"
