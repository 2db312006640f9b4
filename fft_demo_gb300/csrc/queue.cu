// Serving queue: continuous batching of 1D FFT and 2D convolution requests
// into the persistent batch kernel (fft_batch.cuh), with everything a
// request needs kept resident on the device: twiddle and DFT tables for
// every supported size, a pool of filters and their spectra per padded size
// (made on first use), a workspace arena and four staging slots for the work
// lists, so that a submit allocates nothing except a new filter spectrum.
//
// A submit builds the work list on the host, copies it from pinned staging
// memory with one cudaMemcpyAsync, and makes one launch (two when a filter
// spectrum is new). A slot's staging is rewritten only after the launch that
// used it four submits ago has finished, so the host builds later submits
// while up to three earlier ones are on the GPU (a caller that pipelines
// copies around the launches keeps that many in flight). All submits of a
// queue share its workspace and counters: use one stream per queue.
//
// Convolutions whose own padded transform would be 2048 or more (P >= 2^11:
// images of side 1024 and up; the persistent kernel's largest is 2048) run as
// overlap-add: the image is cut into square blocks of side B = P_b - (f - 1),
// P_b = 512 (or the next power of two that keeps B >= 3/4 P_b for a large
// filter side f), so each block's full linear convolution (the filter rotated
// for a correlation) fits a P_b transform. Blocks are ordinary convolutions of
// the same launch, written to a scratch region of the workspace, and one more
// launch sums the block outputs into the requested output window
// (assemble_kernel). The padded area falls from (2 s)^2 to about
// (s P_b / B)^2: a 2048-side image with a 63-point filter runs 25 blocks of
// 512^2 instead of one 4096^2 transform, and a 1024-side one 9 blocks instead
// of one 2048^2 transform.
//
// No counterpart in the reference, whose entry points run one plan's size
// per call (tcfftExec, tcfft_half.cu:1177; fft_conv2d_half::conv2d_forward,
// tensorcore_fft_conv2d.cpp:283).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <utility>
#include <vector>

#include "../../include/tcfft_gb300.h"
#include "batch_host.cuh"
#include "capi_internal.cuh"

using namespace tcfft;
using namespace tcfft::bh;

namespace {

constexpr int kOverlapMinLogP = 11;  // own transform of this size or more: overlap-add
constexpr int kBlockLogP = 9;        // block transforms of 512 (or more for large filters)

// One overlap-add output: the window [r0, r0 + oy) x [c0, c0 + ox) of the
// full convolution, assembled from blocks [blk0, blk0 + nblk).
struct AsmJob {
  long long out_off;  // real elements in conv_out
  long long row0;     // first row of this job in the flattened row space
  int oy, ox, r0, c0, blk0, nblk;
};
// One block's full convolution in the scratch region: h x w real values at
// `off`, whose element (0, 0) is element (y0, x0) of the full convolution.
struct AsmBlock {
  long long off;
  int y0, x0, h, w;
};

template <class R>
__device__ __forceinline__ float asm_load(const R* p);
template <>
__device__ __forceinline__ float asm_load<__half>(const __half* p) {
  return __half2float(*p);
}
template <>
__device__ __forceinline__ float asm_load<float>(const float* p) {
  return *p;
}

// Sum of the block outputs covering each output element (FP32), one output
// row per CTA iteration over the rows of all jobs.
template <class R>
__global__ void assemble_kernel(const AsmJob* __restrict__ jobs, int njobs, const AsmBlock* __restrict__ blocks,
                                const R* __restrict__ scratch, R* __restrict__ out, long long total_rows) {
  for (long long row = blockIdx.x; row < total_rows; row += gridDim.x) {
    int lo = 0, hi = njobs - 1;  // last job with row0 <= row
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (jobs[mid].row0 <= row) lo = mid;
      else hi = mid - 1;
    }
    const AsmJob jb = jobs[lo];
    const int y = static_cast<int>(row - jb.row0);
    const int Y = y + jb.r0;
    R* dst = out + jb.out_off + static_cast<long long>(y) * jb.ox;
    for (int x = threadIdx.x; x < jb.ox; x += blockDim.x) {
      const int X = x + jb.c0;
      float acc = 0.f;
      for (int k = 0; k < jb.nblk; ++k) {
        const AsmBlock b = blocks[jb.blk0 + k];
        const int ly = Y - b.y0, lx = X - b.x0;
        if (ly >= 0 && ly < b.h && lx >= 0 && lx < b.w)
          acc += asm_load<R>(scratch + b.off + static_cast<long long>(ly) * b.w + lx);
      }
      if constexpr (sizeof(R) == 2) {
        dst[x] = __float2half_rn(acc);
      } else {
        dst[x] = acc;
      }
    }
  }
}

}  // namespace

struct tcfftQueueImpl {
  int precision = TCFFT_FP16;
  int pr = 0;
  size_t eb = 4;  // bytes per complex element
  void* tables = nullptr;
  BatchArgs base{};
  void* ws = nullptr;
  size_t ws_elems = 0;
  int* ctr = nullptr;
  size_t ctr_cap = 0;
  int* err = nullptr;
  struct Slot {
    unsigned char* dev = nullptr;
    unsigned char* host = nullptr;
    cudaEvent_t ev = nullptr;
    bool pending = false;
  };
  static constexpr int kSlots = 4;
  Slot slot[kSlots];
  int cur = 0;
  size_t slot_bytes = 0;
  struct Filter {
    float* dev = nullptr;
    int fy = 0, fx = 0;
    std::map<std::pair<int, int>, void*> spec;  // (log2 P, flip) -> spectrum
  };
  std::map<int, Filter> filters;
};

namespace {

void free_queue(tcfftQueueImpl* q) {
  if (!q) return;
  for (auto& s : q->slot) {
    if (s.ev) cudaEventSynchronize(s.ev);
    if (s.ev) cudaEventDestroy(s.ev);
    cudaFree(s.dev);
    cudaFreeHost(s.host);
  }
  for (auto& kv : q->filters) {
    cudaFree(kv.second.dev);
    for (auto& sp : kv.second.spec) cudaFree(sp.second);
  }
  cudaFree(q->tables);
  cudaFree(q->ws);
  cudaFree(q->ctr);
  cudaFree(q->err);
  delete q;
}

// Forward tables for every size the batch kernel runs.
tcfftStatus make_tables(tcfftQueueImpl* q) {
  size_t off_tw[kBatchMaxLineLog + 1] = {}, off_lo[kBatchMaxLog + 1] = {}, off_hi[kBatchMaxLog + 1] = {};
  size_t at = 4096;  // DFT16 B image (hi, lo) first
  for (int l = kBatchMinLineLog; l <= kBatchMaxLineLog; ++l) {
    off_tw[l] = at;
    at = align_up(at + (sizeof(float2) << l), 256);
  }
  for (int l = kBatchMaxLineLog + 1; l <= kBatchMaxLog; ++l) {
    const int sh = (l + 1) / 2;
    off_lo[l] = at;
    at = align_up(at + (sizeof(float2) << sh), 256);
    off_hi[l] = at;
    at = align_up(at + (sizeof(float2) << (l - sh)), 256);
  }
  if (cudaMalloc(&q->tables, at) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  unsigned char* A = static_cast<unsigned char*>(q->tables);
  cudaError_t e = gen_dft16_bmat(reinterpret_cast<uint16_t*>(A), -1, 0, 0);
  if (e == cudaSuccess) e = gen_dft16_bmat(reinterpret_cast<uint16_t*>(A) + 1024, -1, 1, 0);
  BatchArgs& a = q->base;
  for (int l = kBatchMinLineLog; l <= kBatchMaxLineLog && e == cudaSuccess; ++l) {
    e = gen_twiddles(reinterpret_cast<float2*>(A + off_tw[l]), 1ll << l, l, 0, -1, 0);
    a.tw[l] = reinterpret_cast<const float2*>(A + off_tw[l]);
  }
  for (int l = kBatchMaxLineLog + 1; l <= kBatchMaxLog && e == cudaSuccess; ++l) {
    const int sh = (l + 1) / 2;
    e = gen_twiddles(reinterpret_cast<float2*>(A + off_lo[l]), 1ll << sh, l, 0, -1, 0);
    if (e == cudaSuccess) e = gen_twiddles(reinterpret_cast<float2*>(A + off_hi[l]), 1ll << (l - sh), l, sh, -1, 0);
    a.otw[l].lo = reinterpret_cast<const float2*>(A + off_lo[l]);
    a.otw[l].hi = reinterpret_cast<const float2*>(A + off_hi[l]);
    a.otw[l].shift = sh;
    a.otw[l].logn = l;
  }
  a.bmat = reinterpret_cast<const uint32_t*>(A);
  return e == cudaSuccess ? TCFFT_OK : TCFFT_LAUNCH_FAILED;
}

}  // namespace

extern "C" {

tcfftStatus tcfft_queue_create(tcfftQueue* queue, int precision, size_t workspace_bytes, size_t staging_bytes) {
  if (!queue) return record_status(TCFFT_INVALID_VALUE, 0);
  *queue = nullptr;
  if (precision != TCFFT_FP16 && precision != TCFFT_SPLIT_FP32) return record_status(TCFFT_INVALID_VALUE, 0);
  if (workspace_bytes < (1u << 20) || staging_bytes < (1u << 16)) return record_status(TCFFT_INVALID_SIZE, 0);
  tcfftStatus s = batch_registry_ready();
  if (s != TCFFT_OK) return record_status(s, 0);
  tcfftQueueImpl* q = new (std::nothrow) tcfftQueueImpl();
  if (!q) return record_status(TCFFT_ALLOC_FAILED, 0);
  q->precision = precision;
  q->pr = precision == TCFFT_FP16 ? 0 : 1;
  q->eb = precision == TCFFT_FP16 ? 4 : 8;
  q->ws_elems = workspace_bytes / q->eb;
  q->slot_bytes = align_up(staging_bytes, 256);
  q->ctr_cap = q->slot_bytes / sizeof(BatchItem) + 1;  // every counter belongs to at least one item
  s = make_tables(q);
  if (s == TCFFT_OK && (cudaMalloc(&q->ws, q->ws_elems * q->eb) != cudaSuccess ||
                        cudaMalloc(&q->ctr, sizeof(int) * q->ctr_cap) != cudaSuccess ||
                        cudaMalloc(&q->err, sizeof(int)) != cudaSuccess))
    s = TCFFT_ALLOC_FAILED;
  if (s == TCFFT_OK && cudaMemset(q->err, 0, sizeof(int)) != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
  for (auto& sl : q->slot) {
    if (s != TCFFT_OK) break;
    if (cudaMalloc(&sl.dev, q->slot_bytes) != cudaSuccess ||
        cudaHostAlloc(reinterpret_cast<void**>(&sl.host), q->slot_bytes, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess)
      s = TCFFT_ALLOC_FAILED;
  }
  if (s == TCFFT_OK && cudaDeviceSynchronize() != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
  if (s != TCFFT_OK) {
    free_queue(q);
    return record_status(s, 0);
  }
  q->base.ws = q->ws;
  q->base.err = q->err;
  q->base.ctrs = q->ctr;
  q->base.counter = reinterpret_cast<unsigned int*>(q->ctr);
  *queue = q;
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_queue_set_filter(tcfftQueue q, int id, const float* filter, int fy, int fx) {
  if (!q || !filter || fy < 1 || fx < 1) return record_status(TCFFT_INVALID_VALUE, 0);
  if (q->filters.count(id)) return record_status(TCFFT_INVALID_VALUE, 0);  // ids are set once
  tcfftQueueImpl::Filter f;
  f.fy = fy;
  f.fx = fx;
  const size_t bytes = sizeof(float) * static_cast<size_t>(fy) * fx;
  if (cudaMalloc(&f.dev, bytes) != cudaSuccess) return record_status(TCFFT_ALLOC_FAILED, 0);
  if (cudaMemcpy(f.dev, filter, bytes, cudaMemcpyDefault) != cudaSuccess) {
    cudaFree(f.dev);
    return record_status(TCFFT_LAUNCH_FAILED, 0);
  }
  q->filters.emplace(id, f);
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_queue_submit(tcfftQueue q, int count, const long long* n, const long long* in_off,
                               const long long* out_off, const float* scale, int nconv, const tcfftQueueConv* convs,
                               const void* in, void* out, const void* conv_in, void* conv_out, void* stream) {
  if (!q || count < 0 || nconv < 0) return record_status(TCFFT_INVALID_VALUE, 0);
  if (count > 0 && (!n || !in_off || !out_off || !in || !out)) return record_status(TCFFT_INVALID_VALUE, 0);
  if (nconv > 0 && (!convs || !conv_in || !conv_out)) return record_status(TCFFT_INVALID_VALUE, 0);
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u)
    return record_status(TCFFT_INVALID_VALUE, 0);
  if (count + nconv == 0) return record_status(TCFFT_OK, 0);
  const long long align_elems = q->precision == TCFFT_FP16 ? 4 : 2;
  for (int i = 0; i < count; ++i) {
    const int l = ilog2_exact(n[i]);
    if (l < kBatchMinLineLog || l > kBatchMaxLog) return record_status(TCFFT_INVALID_SIZE, 0);
    if (in_off[i] < 0 || out_off[i] < 0 || in_off[i] % align_elems || out_off[i] % align_elems)
      return record_status(TCFFT_INVALID_VALUE, 0);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BatchSpec spec;
  spec.fuse_conv_columns = q->precision == TCFFT_FP16;
  std::vector<float> ones;
  if (count > 0 && !scale) {
    ones.assign(static_cast<size_t>(count), 1.0f);
    scale = ones.data();
  }
  spec.count = count;
  spec.n = n;
  spec.in_off = in_off;
  spec.out_off = out_off;
  spec.scale = scale;
  // convolutions: geometry and spectra (a new (filter, P) spectrum is made
  // by this submit's first launch)
  // the spectrum of a filter for a padded size and orientation, made by this
  // submit's first launch when it is new
  auto add_conv = [&](BatchConv cv, tcfftQueueImpl::Filter& flt) -> tcfftStatus {
    cv.filt = flt.dev;
    const auto key = std::make_pair(cv.logP, cv.flip);
    char prep = 0;
    auto sit = flt.spec.find(key);
    if (sit == flt.spec.end()) {
      void* k = nullptr;
      if (cudaMalloc(&k, q->eb << (2 * cv.logP)) != cudaSuccess) return TCFFT_ALLOC_FAILED;
      sit = flt.spec.emplace(key, k).first;
      prep = 1;
    }
    cv.kspec = sit->second;
    spec.convs.push_back(cv);
    spec.conv_prep.push_back(prep);
    return TCFFT_OK;
  };
  std::vector<AsmJob> jobs;
  std::vector<AsmBlock> blocks;
  std::vector<size_t> block_conv;  // index in spec.convs of each block
  long long scratch_elems = 0, asm_rows = 0;
  for (int c = 0; c < nconv; ++c) {
    const tcfftQueueConv& r = convs[c];
    auto fit = q->filters.find(r.filter_id);
    if (fit == q->filters.end()) return record_status(TCFFT_INVALID_VALUE, 0);
    if (r.img_off < 0 || r.out_off < 0 || r.sy < 1 || r.sx < 1) return record_status(TCFFT_INVALID_VALUE, 0);
    const int fy = fit->second.fy, fx = fit->second.fx;
    tcfftBatchConv d{r.sy, r.sx, fy, fx, r.mode, r.img_off, r.out_off, 0};
    BatchConv cv{};
    if (conv_geometry(d, cv) && cv.logP < kOverlapMinLogP) {
      cv.img_off = r.img_off;
      cv.out_off = r.out_off;
      const tcfftStatus s = add_conv(cv, fit->second);
      if (s != TCFFT_OK) return record_status(s, 0);
      continue;
    }
    // too large for one transform (or an invalid request, rejected below):
    // overlap-add of blocks, the window of the requested mode inside the
    // full convolution
    int oy, ox, r0, c0;
    if (r.mode == TCFFT_CONV_VALID_CORR) {
      if (fy > r.sy || fx > r.sx) return record_status(TCFFT_INVALID_SIZE, 0);
      oy = r.sy - fy + 1, ox = r.sx - fx + 1, r0 = fy - 1, c0 = fx - 1;
    } else if (r.mode == TCFFT_CONV_SAME) {
      if (fy % 2 == 0 || fx % 2 == 0) return record_status(TCFFT_INVALID_SIZE, 0);
      oy = r.sy, ox = r.sx, r0 = (fy - 1) / 2, c0 = (fx - 1) / 2;
    } else if (r.mode == TCFFT_CONV_FULL) {
      oy = r.sy + fy - 1, ox = r.sx + fx - 1, r0 = 0, c0 = 0;
    } else {
      return record_status(TCFFT_INVALID_VALUE, 0);
    }
    // block side: the block's full convolution (side B + f - 1) fills a
    // 2^blog transform, with B >= 3/4 of it
    const int fm1 = std::max(fy, fx) - 1;
    int blog = kBlockLogP;
    while (blog < kBatchMaxConvLog && 4 * ((1 << blog) - fm1) < 3 * (1 << blog)) ++blog;
    const int bs = (1 << blog) - fm1;
    if (bs < 1) return record_status(TCFFT_INVALID_SIZE, 0);
    AsmJob jb{r.out_off, asm_rows, oy, ox, r0, c0, static_cast<int>(blocks.size()), 0};
    for (int by0 = 0; by0 < r.sy; by0 += bs)
      for (int bx0 = 0; bx0 < r.sx; bx0 += bs) {
        const int bh = std::min(bs, r.sy - by0), bw = std::min(bs, r.sx - bx0);
        BatchConv b{};
        if (!conv_geometry(tcfftBatchConv{bh, bw, fy, fx, TCFFT_CONV_FULL, 0, 0, 0}, b))
          return record_status(TCFFT_INVALID_SIZE, 0);
        b.flip = r.mode == TCFFT_CONV_VALID_CORR ? 1 : 0;  // correlation: the rotated filter
        b.img_off = r.img_off + static_cast<long long>(by0) * r.sx + bx0;
        b.ld = r.sx;
        b.out_off = scratch_elems;  // relative to the scratch region, set below
        blocks.push_back(AsmBlock{scratch_elems, by0, bx0, b.oy, b.ox});
        block_conv.push_back(spec.convs.size());
        scratch_elems += static_cast<long long>(b.oy) * b.ox;
        const tcfftStatus s = add_conv(b, fit->second);
        if (s != TCFFT_OK) return record_status(s, 0);
        ++jb.nblk;
      }
    jobs.push_back(jb);
    asm_rows += oy;
  }
  // one prep pass per new spectrum, even if several requests share it
  for (size_t j = 0; j < spec.convs.size(); ++j)
    for (size_t i = 0; i < j; ++i)
      if (spec.conv_prep[i] && spec.convs[i].kspec == spec.convs[j].kspec) spec.conv_prep[j] = 0;
  const int ctas = batch_ctas(q->pr, 0);
  Built bl = build_items(spec, 2 * ctas);
  // scratch for the overlap-add blocks after the items' workspace (real
  // elements, half the size of a complex one)
  const size_t scratch_at = align_up(bl.ws_elems * q->eb, 256);
  const size_t scratch_bytes = static_cast<size_t>(scratch_elems) * (q->eb / 2);
  if (scratch_at + scratch_bytes > q->ws_elems * q->eb || static_cast<size_t>(bl.nctrs) > q->ctr_cap)
    return record_status(TCFFT_CAPACITY, 0);
  unsigned char* scratch = static_cast<unsigned char*>(q->ws) + scratch_at;
  for (size_t k = 0; k < block_conv.size(); ++k) bl.convs[block_conv[k]].out_base = scratch;
  // work lists -> staging slot
  size_t at = 0;
  auto place = [&](size_t bytes) {
    const size_t o = at;
    at = align_up(at + bytes, 256);
    return o;
  };
  const size_t o_lin = place(sizeof(long long) * bl.line_in.size());
  const size_t o_lout = place(sizeof(long long) * bl.line_out.size());
  const size_t o_items = place(sizeof(BatchItem) * bl.items.size());
  const size_t o_prep = place(sizeof(BatchItem) * bl.prep_items.size());
  const size_t o_xf = place(sizeof(BatchXform) * bl.xforms.size());
  const size_t o_cv = place(sizeof(BatchConv) * bl.convs.size());
  const size_t o_jobs = place(sizeof(AsmJob) * jobs.size());
  const size_t o_blocks = place(sizeof(AsmBlock) * blocks.size());
  if (at > q->slot_bytes) return record_status(TCFFT_CAPACITY, 0);
  tcfftQueueImpl::Slot& sl = q->slot[q->cur];
  if (sl.pending && cudaEventSynchronize(sl.ev) != cudaSuccess) return record_status(TCFFT_LAUNCH_FAILED, 0);
  sl.pending = false;
  auto put = [&](size_t o, const void* src, size_t bytes) {
    if (bytes) std::memcpy(sl.host + o, src, bytes);
  };
  put(o_lin, bl.line_in.data(), sizeof(long long) * bl.line_in.size());
  put(o_lout, bl.line_out.data(), sizeof(long long) * bl.line_out.size());
  put(o_items, bl.items.data(), sizeof(BatchItem) * bl.items.size());
  put(o_prep, bl.prep_items.data(), sizeof(BatchItem) * bl.prep_items.size());
  put(o_xf, bl.xforms.data(), sizeof(BatchXform) * bl.xforms.size());
  put(o_cv, bl.convs.data(), sizeof(BatchConv) * bl.convs.size());
  put(o_jobs, jobs.data(), sizeof(AsmJob) * jobs.size());
  put(o_blocks, blocks.data(), sizeof(AsmBlock) * blocks.size());
  if (cudaMemcpyAsync(sl.dev, sl.host, at, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return record_status(TCFFT_LAUNCH_FAILED, 0);
  BatchArgs a = q->base;
  a.wait_polls = dep_wait_polls();
  a.in = in;
  a.out = out;
  a.conv_in = conv_in;
  a.conv_out = conv_out;
  a.line_in = reinterpret_cast<const long long*>(sl.dev + o_lin);
  a.line_out = reinterpret_cast<const long long*>(sl.dev + o_lout);
  a.xforms = reinterpret_cast<const BatchXform*>(sl.dev + o_xf);
  a.convs = reinterpret_cast<const BatchConv*>(sl.dev + o_cv);
  const BatchKernel& k = batch_kernel(q->pr, 0);
  int launches = 0;
  auto launch = [&](size_t o, size_t nitems) -> bool {
    BatchArgs la = a;
    la.items = reinterpret_cast<const BatchItem*>(sl.dev + o);
    la.nitems = static_cast<int>(nitems);
    if (cudaMemsetAsync(q->ctr, 0, sizeof(int) * static_cast<size_t>(bl.nctrs), st) != cudaSuccess) return false;
    const int grid = static_cast<int>(std::min<size_t>(static_cast<size_t>(ctas), nitems));
    void* params[] = {&la};
    if (cudaLaunchKernel(k.fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), params,
                         static_cast<size_t>(k.smem), st) != cudaSuccess)
      return false;
    ++launches;
    return true;
  };
  if (!bl.prep_items.empty() && !launch(o_prep, bl.prep_items.size())) return record_status(TCFFT_LAUNCH_FAILED, 0);
  if (!bl.items.empty() && !launch(o_items, bl.items.size())) return record_status(TCFFT_LAUNCH_FAILED, launches);
  if (!jobs.empty()) {
    const unsigned grid = static_cast<unsigned>(std::min<long long>(asm_rows, 8192));
    const AsmJob* dj = reinterpret_cast<const AsmJob*>(sl.dev + o_jobs);
    const AsmBlock* db = reinterpret_cast<const AsmBlock*>(sl.dev + o_blocks);
    if (q->precision == TCFFT_FP16)
      assemble_kernel<__half><<<grid, 256, 0, st>>>(dj, static_cast<int>(jobs.size()), db,
                                                    reinterpret_cast<const __half*>(scratch),
                                                    static_cast<__half*>(conv_out), asm_rows);
    else
      assemble_kernel<float><<<grid, 256, 0, st>>>(dj, static_cast<int>(jobs.size()), db,
                                                   reinterpret_cast<const float*>(scratch),
                                                   static_cast<float*>(conv_out), asm_rows);
    if (cudaGetLastError() != cudaSuccess) return record_status(TCFFT_LAUNCH_FAILED, launches);
    ++launches;
  }
  if (cudaEventRecord(sl.ev, st) != cudaSuccess) return record_status(TCFFT_LAUNCH_FAILED, launches);
  sl.pending = true;
  q->cur = (q->cur + 1) % tcfftQueueImpl::kSlots;
  return record_status(TCFFT_OK, launches);
}

tcfftStatus tcfft_queue_check(tcfftQueue q, void* stream) {
  if (!q) return record_status(TCFFT_INVALID_VALUE, 0);
  if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess)
    return record_status(TCFFT_LAUNCH_FAILED, 0);
  int flag = 0;
  if (cudaMemcpy(&flag, q->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemset(q->err, 0, sizeof(int)) != cudaSuccess)
    return record_status(TCFFT_LAUNCH_FAILED, 0);
  if (flag & (kErrMmaTimeout | kErrQueueTimeout)) return record_status(TCFFT_TIMEOUT, 0);
  return record_status(flag ? TCFFT_INVALID_VALUE : TCFFT_OK, 0);
}

tcfftStatus tcfft_queue_destroy(tcfftQueue q) {
  if (!q) return record_status(TCFFT_INVALID_VALUE, 0);
  free_queue(q);
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_copy_inputs(int count, const void* const* src, const size_t* bytes, void* dst_base,
                              const size_t* dst_off, void* stream) {
  if (count < 0 || (count > 0 && (!src || !bytes || !dst_base || !dst_off)))
    return record_status(TCFFT_INVALID_VALUE, 0);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* dst = static_cast<unsigned char*>(dst_base);
  for (int i = 0; i < count; ++i)
    if (bytes[i] && cudaMemcpyAsync(dst + dst_off[i], src[i], bytes[i], cudaMemcpyHostToDevice, st) != cudaSuccess)
      return record_status(TCFFT_LAUNCH_FAILED, 0);
  return record_status(TCFFT_OK, 0);
}

}  // extern "C"
