// Persistent batch kernel: 1D transforms and 2D convolutions of uneven sizes
// in one launch, fed from a device-side work queue.
//
// The caller's transforms sit anywhere in one input and one output buffer
// (element offsets per transform); convolutions read real images from a
// second pair of buffers. The host plan writes a list of work items (tiles):
//   kItemLines : up to G = 8192 / L whole transforms of one size L <= 2^13,
//                single pass; transform offsets come from the line tables
//   kItemP1    : a column-pass tile of one larger transform (four-step pass
//                1: lines of length n1, outer twiddle W_n, into the plan's
//                workspace)
//   kItemP2    : a transposing row-pass tile of the same transform (pass 2:
//                lines of length n2, workspace -> output)
//   kItemConv* : the four stages of a convolution (see BatchConv)
// CTAs take items with one atomic counter, in list order. An item may wait
// (bounded) until a dependency counter reaches a target -- a P2 tile for all
// P1 tiles of its transform, a conv stage for all tiles of the stage before
// -- and may bump a counter when done, after a device-scope fence. The host
// puts every item after all items it waits for, so a wait only ever targets
// items that running CTAs already hold, and the chain of waits ends at an
// item that waits for nothing: the queue cannot deadlock, whether or not
// every CTA of the grid is resident at once.
//
// All tiles hold 512 rows of the 16-column MMA layout (Mt = 512), FP16 or
// split precision, so one TMEM allocation (128 columns FP16, 256 split) and
// one shared-memory carve-out serve every item kind and size.
#pragma once
#include "fft_fused.cuh"
#include "fft_io.cuh"
#include "fft_split.cuh"
#include "conv_io.cuh"
#include "fft_tile.cuh"

namespace tcfft {

enum : int {
  kItemLines = 0,    // single-pass 1D tile
  kItemP1 = 1,       // four-step pass 1 tile
  kItemP2 = 2,       // four-step pass 2 tile
  kItemConvRow = 3,  // conv: forward FFT of real rows (zero-padded to P)
  kItemConvCol = 4,  // conv: forward FFT of columns, times the filter spectrum
  kItemConvInv = 5,  // conv: second column FFT, rows of the output window kept
  kItemConvOut = 6,  // conv: row FFT, real part of the output window's columns
  kItemFiltRow = 7,  // filter spectrum: forward FFT of the (flipped) filter's rows
  kItemFiltCol = 8,  // filter spectrum: forward FFT of columns -> K
  kItemConvMid = 9,  // conv (FP16): kItemConvCol and kItemConvInv on one tile, the product on chip
};

constexpr int kBatchMt = 512;
constexpr int kBatchMinLineLog = 6, kBatchMaxLineLog = 13;  // single-pass sizes
constexpr int kBatchMinPassLog = 7, kBatchMaxPassLog = 10;  // four-step pass lengths
constexpr int kBatchMaxLog = 2 * kBatchMaxPassLog;          // largest transform
constexpr int kBatchMinConvLog = 6, kBatchMaxConvLog = 11;  // padded conv sizes P

struct BatchItem {
  int kind;
  int logl;         // pass length of this tile
  int line0;        // kItemLines: first entry of the line tables; others: first line in the pass
  int nlines;       // kItemLines: transforms in this tile
  int obj;          // transform (P1 / P2) or convolution (conv items) index
  float scale;      // applied on the tile's store
  int wait_ctr;     // counter to wait for before starting (-1: none) ...
  int wait_target;  // ... until it reaches this value
  int signal_ctr;   // counter bumped when the tile is done (-1: none)
  int pad;
};

struct BatchXform {
  long long in_off, out_off, ws_off;  // element offsets
  int logn, log_n1, log_n2, tiles1;   // tiles1: P1 tiles of this transform
};

// One 2D convolution of a real sy x sx image with a resident filter spectrum
// K (P x P, unnormalised DFT of the zero-padded, possibly flipped filter).
// Stages: rows -> X (sy x P, scale 1/P); columns of X -> Y = conj(Xf * K)
// (P x P, scale 1/P); columns of Y -> Z (the oy output rows, P wide);
// rows of Z -> out (real part of columns [c0, c0 + ox)). Since
// IDFT(y) = conj(DFT(conj(y))), storing conj(Xf * K) lets both inverse
// stages run as forward transforms, and Re(conj z) = Re(z) makes the final
// conjugation vanish. Z reuses X's space (X is dead once all column tiles of
// stage 2 are done, which stage 3 waits for).
// K itself comes from kItemFiltRow / kItemFiltCol tiles (the same passes on
// the fy x fx float filter, scale 1, rows into X's space, columns into K).
struct BatchConv {
  long long img_off, out_off;  // real elements in the conv input / output buffers
  long long x_off, y_off;      // elements in the workspace
  void* kspec;                 // P x P filter spectrum (E)
  const float* filt;           // fy x fx float filter (spectrum items)
  int sy, sx, oy, ox, r0, c0, logP, flip, fy, fx;
  int ld;          // elements between image rows in conv_in (0: sx)
  int pad0;
  void* out_base;  // real output buffer (nullptr: the launch's conv_out)
};

struct BatchArgs {
  const void* in;
  void* out;
  void* ws;
  const long long* line_in;  // per single-pass transform, sorted by size: element offsets
  const long long* line_out;
  const BatchItem* items;
  int nitems;
  const BatchXform* xforms;
  const BatchConv* convs;
  const void* conv_in;   // real images (half for FP16, float for split)
  void* conv_out;        // real outputs
  unsigned int* counter;  // queue head
  int* ctrs;              // dependency counters
  const float2* tw[kBatchMaxLineLog + 1];  // W_L, this direction
  OuterTwiddle otw[kBatchMaxLog + 1];      // W_n factor tables per log2 n
  const uint32_t* bmat;                    // DFT16 B image (hi, lo), this direction
  int* err;
  unsigned int wait_polls;  // bound of each dependency wait (tcfft_set_wait_limit)
};

// Whole lines found through per-line offset tables (each line contiguous).
template <class E>
struct IoLines {
  static constexpr bool IN_VEC_L = true;
  static constexpr bool OUT_VEC_L = true;
  struct Raw2 {
    uint4 a, b;
  };
  using Raw = typename std::conditional<sizeof(E) == 4, uint4, Raw2>::type;

  const E* in;
  E* out;
  const long long* loff_in;
  const long long* loff_out;
  long long total_lines;
  float scale;
  bool in_contig = false, out_contig = false;  // lines are scattered: no bulk tile copies
  long long contig_len = 0;

  __device__ __forceinline__ Raw fetch_l(long long line, int l0, bool ok) const {
    Raw r;
    if constexpr (sizeof(E) == 4) {
      r = make_uint4(0, 0, 0, 0);
      if (ok && line < total_lines) r = ldg_nc_v4(in + __ldg(loff_in + line) + l0);
    } else {
      r.a = r.b = make_uint4(0, 0, 0, 0);
      if (ok && line < total_lines) {
        const E* p = in + __ldg(loff_in + line) + l0;
        r.a = ldg_nc_v4(p);
        r.b = ldg_nc_v4(p + 2);
      }
    }
    return r;
  }
  __device__ __forceinline__ Raw fetch_g(long long, int, bool) const { return Raw{}; }
  __device__ __forceinline__ void decode_l(const Raw& r, long long, int, float2 (&v)[4]) const {
    if constexpr (sizeof(E) == 4) {
      unpack_h2x4(r, v);
    } else {
      v[0] = make_float2(__uint_as_float(r.a.x), __uint_as_float(r.a.y));
      v[1] = make_float2(__uint_as_float(r.a.z), __uint_as_float(r.a.w));
      v[2] = make_float2(__uint_as_float(r.b.x), __uint_as_float(r.b.y));
      v[3] = make_float2(__uint_as_float(r.b.z), __uint_as_float(r.b.w));
    }
  }
  __device__ __forceinline__ void decode_g(const Raw&, long long, int, float2 (&)[4]) const {}
  __device__ __forceinline__ void store_row16(long long line, int j, int J, float2 (&v)[16]) const {
    E* p = out + __ldg(loff_out + line) + j;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      if constexpr (sizeof(E) == 4)
        p[c * J] = __floats2half2_rn(v[c].x * scale, v[c].y * scale);
      else
        p[c * J] = make_float2(v[c].x * scale, v[c].y * scale);
    }
  }
  __device__ __forceinline__ const E* tile_src(long long) const { return in; }
  __device__ __forceinline__ E* tile_dst(long long) const { return out; }
};

// The batch kernel moves its tiles itself (no tensor maps): clear the flags
// of IO policies that have them.
template <class IO>
__device__ __forceinline__ void clear_tensor_flags(IO& io) {
  if constexpr (TensorMapIo<IO>) {
    io.in_tma = false;
    io.out_tma = false;
  }
}

template <bool SPLIT>
struct BatchPrec;

template <>
struct BatchPrec<false> {
  using E = half2;
  using State = PassState;
  static constexpr uint32_t kTmemCols = kBatchMt / 4;
  template <bool IN_L, bool OUT_L, bool COH>
  using Io = IoHalf<IN_L, OUT_L, COH>;
  template <int L, bool LM, int SIGN, class IO>
  __device__ static bool tile(State& st, const IO& io, const PassCore& core, long long line0) {
    return pass_tile<L, kBatchMt * 16 / L, LM, SIGN, IO>(st, io, core, line0);
  }
  __device__ static void setup(State& st, const uint32_t* bmat) { pass_setup<kTmemCols>(st, bmat); }
  __device__ static void teardown(State& st) { pass_teardown<kTmemCols>(st); }
};

template <>
struct BatchPrec<true> {
  using E = float2;
  using State = SplitState;
  static constexpr uint32_t kTmemCols = kBatchMt / 2;
  template <bool IN_L, bool OUT_L, bool COH>
  using Io = IoFloat<IN_L, OUT_L, COH>;
  template <int L, bool LM, int SIGN, class IO>
  __device__ static bool tile(State& st, const IO& io, const PassCore& core, long long line0) {
    return split_tile<L, kBatchMt * 16 / L, LM, SIGN, IO>(st, io, core, line0);
  }
  __device__ static void setup(State& st, const uint32_t* bmat) { split_setup<kTmemCols>(st, bmat); }
  __device__ static void teardown(State& st) { split_teardown<kTmemCols>(st); }
};

template <bool SPLIT, int SIGN, int L>
__device__ __noinline__ bool batch_lines_item(typename BatchPrec<SPLIT>::State& st, const BatchArgs& a,
                                              const BatchItem& it, const PassCore& core) {
  using P = BatchPrec<SPLIT>;
  using E = typename P::E;
  IoLines<E> io;
  io.in = static_cast<const E*>(a.in);
  io.out = static_cast<E*>(a.out);
  io.loff_in = a.line_in + it.line0;
  io.loff_out = a.line_out + it.line0;
  io.total_lines = it.nlines;
  io.scale = it.scale;
  return P::template tile<L, false, SIGN>(st, io, core, 0);
}

template <bool SPLIT, int SIGN, int L>
__device__ __noinline__ bool batch_p1_item(typename BatchPrec<SPLIT>::State& st, const BatchArgs& a,
                                           const BatchItem& it, const PassCore& core) {
  using P = BatchPrec<SPLIT>;
  using E = typename P::E;
  const BatchXform xf = a.xforms[it.obj];
  const long long n = 1ll << xf.logn, n2 = 1ll << xf.log_n2;
  typename P::template Io<false, false, false> io;
  clear_tensor_flags(io);
  io.in = static_cast<const E*>(a.in) + xf.in_off;
  io.out = static_cast<E*>(a.ws) + xf.ws_off;
  io.total_lines = n2;
  io.lps_log2 = xf.log_n2;
  io.in_seq = io.out_seq = n;
  io.in_line = io.out_line = 1;
  io.in_elem = io.out_elem = n2;
  io.otw = a.otw[xf.logn];
  io.scale = 1.0f;
  io.in_contig = io.out_contig = false;
  io.contig_len = L;
  return P::template tile<L, true, SIGN>(st, io, core, static_cast<long long>(it.line0));
}

template <bool SPLIT, int SIGN, int L>
__device__ __noinline__ bool batch_p2_item(typename BatchPrec<SPLIT>::State& st, const BatchArgs& a,
                                           const BatchItem& it, const PassCore& core) {
  using P = BatchPrec<SPLIT>;
  using E = typename P::E;
  const BatchXform xf = a.xforms[it.obj];
  const long long n = 1ll << xf.logn, n1 = 1ll << xf.log_n1, n2 = 1ll << xf.log_n2;
  typename P::template Io<true, false, true> io;
  clear_tensor_flags(io);
  io.in = static_cast<const E*>(a.ws) + xf.ws_off;
  io.out = static_cast<E*>(a.out) + xf.out_off;
  io.total_lines = n1;
  io.lps_log2 = xf.log_n1;
  io.in_seq = io.out_seq = n;
  io.in_line = n2;
  io.in_elem = 1;
  io.out_line = 1;
  io.out_elem = n1;
  io.otw = OuterTwiddle();
  io.scale = it.scale;
  io.in_contig = io.out_contig = false;
  io.contig_len = L;
  return P::template tile<L, true, SIGN>(st, io, core, static_cast<long long>(it.line0));
}

// Stage 2 of a convolution: the column pass of IoColMaskCrop (rows >= sy
// read as zero) whose store writes conj(scale * v * K) for the full P rows.
template <class E>
struct IoColMulConj : IoColMaskCrop<E> {
  const E* K;  // P x P filter spectrum (row stride P)
  __device__ __forceinline__ void store_row16(long long line, int j, int J, float2 (&v)[16]) const {
    const long long col = line & ((1ll << this->lps_log2) - 1);
    E* p = this->out + col;
    const E* k = K + col;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const long long off = static_cast<long long>(j + c * J) * this->P;
      const float2 w = from_elem(k[off]);
      const float re = (v[c].x * w.x - v[c].y * w.y) * this->scale;
      const float im = (v[c].x * w.y + v[c].y * w.x) * this->scale;
      p[off] = to_elem<E>(make_float2(re, -im));
    }
  }
};

// kItemConvMid's forward half: the column FFT's last stage multiplies by
// the spectrum and 1/P, conjugates (the second column FFT is a forward one:
// IDFT(y) = conj(DFT(conj y))) and hands the result to the planes, running
// the second transform's radix-T stage there when P is not a power of 16.
template <class E>
struct IoColMulConjMid : IoColMaskCrop<E> {
  static constexpr bool TO_PLANES = true;
  static constexpr int NEXT_SIGN = -1;
  const E* K;             // P x P filter spectrum (row stride P)
  const float2* tw_next;  // W_P^e, forward (the second transform's twiddles)
  __device__ __forceinline__ void product16(long long line, int j, int J, float2 (&v)[16]) const {
    const long long col = line & ((1ll << this->lps_log2) - 1);
    const E* k = K + col + static_cast<long long>(j) * this->P;
    const float2 s2 = f2bcast(this->scale);
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
      const float2 k0 = from_elem(k[static_cast<long long>(c) * J * this->P]);
      const float2 k1 = from_elem(k[static_cast<long long>(c + 1) * J * this->P]);
      float2 yr, yi;
      cmul_pair(make_float2(v[c].x, v[c + 1].x), make_float2(v[c].y, v[c + 1].y), twpair(k0, k1), yr, yi);
      yr = f2mul(yr, s2);
      yi = f2mul(yi, s2);
      v[c] = make_float2(yr.x, -yi.x);
      v[c + 1] = make_float2(yr.y, -yi.y);
    }
  }
};

template <class T>
__device__ __forceinline__ T zeroed() {
  T t;
  memset(&t, 0, sizeof(T));
  return t;
}

template <bool SPLIT, int L>
__device__ __noinline__ bool batch_conv_item(typename BatchPrec<SPLIT>::State& st, const BatchArgs& a,
                                             const BatchItem& it, const PassCore& core) {
  using P = BatchPrec<SPLIT>;
  using E = typename P::E;
  using R = typename std::conditional<SPLIT, float, __half>::type;
  const BatchConv cv = a.convs[it.obj];
  E* ws = static_cast<E*>(a.ws);
  const long long line0 = it.line0;
  if (it.kind == kItemConvRow) {
    auto io = zeroed<IoRealRowIn<R, E>>();
    io.in = static_cast<const R*>(a.conv_in) + cv.img_off;
    io.out = ws + cv.x_off;
    io.total_lines = cv.sy;
    io.sy = cv.sy;
    io.sx = cv.sx;
    io.P = L;
    io.in_image_stride = static_cast<long long>(cv.sy) * cv.sx;
    io.ld = cv.ld;
    io.flip = 0;  // images are never flipped; correlation flips the filter
    io.scale = it.scale;
    return P::template tile<L, false, -1>(st, io, core, line0);
  }
  if (it.kind == kItemConvCol) {
    auto io = zeroed<IoColMulConj<E>>();
    io.in = ws + cv.x_off;
    io.out = ws + cv.y_off;
    io.total_lines = L;
    io.P = L;
    io.lps_log2 = cv.logP;
    io.valid_rows = cv.sy;
    io.r0 = 0;
    io.nr = L;
    io.scale = it.scale;
    io.K = static_cast<const E*>(cv.kspec);
    return P::template tile<L, true, -1>(st, io, core, line0);
  }
  if (it.kind == kItemFiltRow) {
    auto io = zeroed<IoRealRowIn<float, E>>();
    io.in = cv.filt;
    io.out = ws + cv.x_off;
    io.total_lines = cv.fy;
    io.sy = cv.fy;
    io.sx = cv.fx;
    io.P = L;
    io.in_image_stride = static_cast<long long>(cv.fy) * cv.fx;
    io.flip = cv.flip;
    io.scale = 1.0f;
    return P::template tile<L, false, -1>(st, io, core, line0);
  }
  if (it.kind == kItemFiltCol) {
    auto io = zeroed<IoColMaskCrop<E>>();
    io.in = ws + cv.x_off;
    io.out = static_cast<E*>(cv.kspec);
    io.total_lines = L;
    io.P = L;
    io.lps_log2 = cv.logP;
    io.valid_rows = cv.fy;
    io.r0 = 0;
    io.nr = L;
    io.scale = 1.0f;
    return P::template tile<L, true, -1>(st, io, core, line0);
  }
  if constexpr (!SPLIT) {
    if (it.kind == kItemConvMid) {
      // both column FFTs of the convolution on one tile: X's columns (rows
      // past the image zero) -> times K, 1/P, conjugated, on chip -> second
      // forward column FFT -> the output window's rows, back into X (each
      // tile reads and writes only its own columns)
      constexpr int G = kBatchMt * 16 / L;
      using Tl = Tile<L, G, true>;
      auto fio = zeroed<IoColMulConjMid<E>>();
      fio.in = ws + cv.x_off;
      fio.total_lines = L;
      fio.P = L;
      fio.lps_log2 = cv.logP;
      fio.valid_rows = cv.sy;
      fio.r0 = 0;
      fio.nr = L;
      fio.scale = it.scale;
      fio.K = static_cast<const E*>(cv.kspec);
      fio.tw_next = core.tw;
      auto iio = zeroed<IoColMaskCrop<E>>();
      iio.out = ws + cv.x_off;
      iio.total_lines = L;
      iio.P = L;
      iio.lps_log2 = cv.logP;
      iio.valid_rows = L;
      iio.r0 = cv.r0;
      iio.nr = cv.oy;
      iio.scale = 1.0f;
      uint8_t* re = st.smem + kPlaneOffset;
      uint8_t* im = re + Tl::PLANE;
      if (!tile_load<L, G, true, -1, IoColMulConjMid<E>>(st, fio, core, line0, re, im)) return false;
      if (!run_stages<L, G, true, -1, IoColMulConjMid<E>>(st, fio, core, line0, re, im, false)) return false;
      return run_stages<L, G, true, -1, IoColMaskCrop<E>>(st, iio, core, line0, re, im, false);
    }
  }
  if (it.kind == kItemConvInv) {
    auto io = zeroed<IoColMaskCrop<E>>();
    io.in = ws + cv.y_off;
    io.out = ws + cv.x_off;
    io.total_lines = L;
    io.P = L;
    io.lps_log2 = cv.logP;
    io.valid_rows = L;
    io.r0 = cv.r0;
    io.nr = cv.oy;
    io.scale = it.scale;
    return P::template tile<L, true, -1>(st, io, core, line0);
  }
  auto io = zeroed<IoRowCropReal<E, R>>();
  io.in = ws + cv.x_off;
  io.out = static_cast<R*>(cv.out_base ? cv.out_base : a.conv_out) + cv.out_off;
  io.total_lines = cv.oy;
  io.P = L;
  io.c0 = cv.c0;
  io.nc = cv.ox;
  io.scale = it.scale;
  return P::template tile<L, false, -1>(st, io, core, line0);
}

template <bool SPLIT, int SIGN>
__device__ __forceinline__ bool batch_run_item(typename BatchPrec<SPLIT>::State& st, const BatchArgs& a,
                                               const BatchItem& it) {
  PassCore core;
  core.tw = a.tw[it.logl];
  core.bmat = a.bmat;
  core.err = a.err;
  if (it.kind == kItemLines) {
    switch (it.logl) {
      case 6: return batch_lines_item<SPLIT, SIGN, 64>(st, a, it, core);
      case 7: return batch_lines_item<SPLIT, SIGN, 128>(st, a, it, core);
      case 8: return batch_lines_item<SPLIT, SIGN, 256>(st, a, it, core);
      case 9: return batch_lines_item<SPLIT, SIGN, 512>(st, a, it, core);
      case 10: return batch_lines_item<SPLIT, SIGN, 1024>(st, a, it, core);
      case 11: return batch_lines_item<SPLIT, SIGN, 2048>(st, a, it, core);
      case 12: return batch_lines_item<SPLIT, SIGN, 4096>(st, a, it, core);
      case 13: return batch_lines_item<SPLIT, SIGN, 8192>(st, a, it, core);
      default: break;
    }
  } else if (it.kind == kItemP1) {
    switch (it.logl) {
      case 7: return batch_p1_item<SPLIT, SIGN, 128>(st, a, it, core);
      case 8: return batch_p1_item<SPLIT, SIGN, 256>(st, a, it, core);
      case 9: return batch_p1_item<SPLIT, SIGN, 512>(st, a, it, core);
      case 10: return batch_p1_item<SPLIT, SIGN, 1024>(st, a, it, core);
      default: break;
    }
  } else if (it.kind == kItemP2) {
    switch (it.logl) {
      case 7: return batch_p2_item<SPLIT, SIGN, 128>(st, a, it, core);
      case 8: return batch_p2_item<SPLIT, SIGN, 256>(st, a, it, core);
      case 9: return batch_p2_item<SPLIT, SIGN, 512>(st, a, it, core);
      case 10: return batch_p2_item<SPLIT, SIGN, 1024>(st, a, it, core);
      default: break;
    }
  } else if constexpr (SIGN == -1) {
    // convolution stages: all forward transforms (see BatchConv)
    switch (it.logl) {
      case 6: return batch_conv_item<SPLIT, 64>(st, a, it, core);
      case 7: return batch_conv_item<SPLIT, 128>(st, a, it, core);
      case 8: return batch_conv_item<SPLIT, 256>(st, a, it, core);
      case 9: return batch_conv_item<SPLIT, 512>(st, a, it, core);
      case 10: return batch_conv_item<SPLIT, 1024>(st, a, it, core);
      case 11: return batch_conv_item<SPLIT, 2048>(st, a, it, core);
      default: break;
    }
  }
  if (threadIdx.x == 0) atomicOr(a.err, kErrBadArgs);
  return true;
}

template <bool SPLIT, int SIGN>
__global__ void __launch_bounds__(kPassThreads, SPLIT ? 2 : 3) fft_batch_kernel(const __grid_constant__ BatchArgs a) {
  using P = BatchPrec<SPLIT>;
  __shared__ unsigned int s_item;
  __shared__ int s_ok;
  typename P::State st;
  P::setup(st, a.bmat);
  bool alive = true;
  while (alive) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1u);
    __syncthreads();
    const unsigned int i = s_item;
    if (i >= static_cast<unsigned int>(a.nitems)) break;
    const BatchItem it = a.items[i];
    if (threadIdx.x == 0) {
      bool ok = true;
      if (it.wait_ctr >= 0) ok = wait_counter(a.ctrs + it.wait_ctr, it.wait_target, a.wait_polls);
      if (!ok) atomicOr(a.err, kErrQueueTimeout);
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) alive = batch_run_item<SPLIT, SIGN>(st, a, it);
    if (it.signal_ctr >= 0) {
      // publish: every thread's stores are visible device-wide before the count
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(a.ctrs + it.signal_ctr, 1);
    }
    __syncthreads();  // s_item / s_ok are rewritten next round
  }
  P::teardown(st);
}

template <bool SPLIT>
constexpr int batch_smem_bytes() {
  if constexpr (SPLIT)
    return split_smem_bytes<64, kBatchMt * 16 / 64>();
  else
    return pass_smem_bytes<64, kBatchMt * 16 / 64>();
}

}  // namespace tcfft

namespace tcfft {

// Registry entries for the batch kernel, per precision and direction
// (index 0 forward, 1 inverse).
struct BatchKernel {
  const void* fn = nullptr;
  int smem = 0;
};
void register_batch_kernels_f16(BatchKernel (&tab)[2]);
void register_batch_kernels_split(BatchKernel (&tab)[2]);

template <bool SPLIT>
void fill_batch(BatchKernel (&tab)[2]) {
  tab[0].fn = reinterpret_cast<const void*>(&fft_batch_kernel<SPLIT, -1>);
  tab[1].fn = reinterpret_cast<const void*>(&fft_batch_kernel<SPLIT, +1>);
  tab[0].smem = tab[1].smem = batch_smem_bytes<SPLIT>();
}

}  // namespace tcfft
