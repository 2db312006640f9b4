// Uneven batches of 1D transforms: host plan and C ABI for the persistent
// batch kernel (fft_batch.cuh), plus the plain per-size path it is measured
// against.
//
// The reference has no counterpart: its plans hold one size and one
// contiguous batch (tcfftCreate, tcfft_half.cu:1235), so a list of transforms
// of different sizes costs one plan and one launch chain per size or per
// transform.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <utility>
#include <vector>

#include "../../include/tcfft_gb300.h"
#include "capi_internal.cuh"
#include "batch_host.cuh"
#include "fft_batch.cuh"
#include "tables.cuh"

using namespace tcfft;
using namespace tcfft::bh;

namespace {

BatchKernel g_bk[2][2];  // [precision][direction]
int g_bk_ctas[2][2];
std::once_flag g_bk_once;
cudaError_t g_bk_err = cudaSuccess;

void init_batch_registry() {
  register_batch_kernels_f16(g_bk[0]);
  register_batch_kernels_split(g_bk[1]);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (int pr = 0; pr < 2 && e == cudaSuccess; ++pr)
    for (int sg = 0; sg < 2 && e == cudaSuccess; ++sg) {
      const BatchKernel& k = g_bk[pr][sg];
      e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, k.smem);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k.fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
      cudaFuncAttributes fa;
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k.fn);
      if (e != cudaSuccess) break;
      // CTAs per SM from registers, shared memory, threads and TMEM (512
      // columns per SM). The queue does not need every CTA resident: only
      // running CTAs take items, and a wait only targets an item taken
      // earlier, so a CTA that starts late just starts on later items.
      const int regs_per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
      int occ = 65536 / (regs_per_warp * (kPassThreads / 32));
      const int by_smem = (228 * 1024) / (k.smem + static_cast<int>(fa.sharedSizeBytes) + 1024);
      const int tmem_cols = pr == 0 ? kBatchMt / 4 : kBatchMt / 2;
      occ = std::min({occ, by_smem, 2048 / kPassThreads, 512 / tmem_cols});
      g_bk_ctas[pr][sg] = sms * (occ < 1 ? 1 : occ);
    }
  g_bk_err = e;
}

struct Buffers {
  const void* in;
  void* out;
  const void* conv_in;
  void* conv_out;
  bool operator==(const Buffers& o) const {
    return in == o.in && out == o.out && conv_in == o.conv_in && conv_out == o.conv_out;
  }
};

constexpr int kMinLog = kBatchMinLineLog;  // 64 points
constexpr int kMaxLog = kBatchMaxLog;      // 2^20 points

}  // namespace

namespace tcfft {

tcfftStatus batch_registry_ready() {
  const tcfftStatus s = registry_ready();
  if (s != TCFFT_OK) return s;
  std::call_once(g_bk_once, init_batch_registry);
  return g_bk_err == cudaSuccess ? TCFFT_OK : TCFFT_NO_DEVICE;
}
const BatchKernel& batch_kernel(int precision_idx, int sign_idx) { return g_bk[precision_idx][sign_idx]; }
int batch_ctas(int precision_idx, int sign_idx) { return g_bk_ctas[precision_idx][sign_idx]; }

}  // namespace tcfft

struct tcfftBatchImpl {
  int precision = TCFFT_FP16;
  int sign_idx = 0;
  int mode = TCFFT_BATCH_PERSISTENT;
  bool use_graph = false;
  int count = 0;
  size_t elem_bytes = 4;
  // caller's description (host copies)
  std::vector<long long> n, in_off, out_off;
  std::vector<float> scale;
  // persistent launch
  int nitems = 0, nxforms = 0, nctrs = 1, ctas = 0;
  size_t ws_bytes = 0;
  void* ws = nullptr;
  void* arena = nullptr;  // tables, line tables, items, transforms
  int* ctr = nullptr;     // [0] queue head, [1 ..] per-transform done counters
  int* err = nullptr;
  BatchArgs args{};
  // convolutions: descriptors, a plan-owned copy of the filters, spectra
  std::vector<tcfftBatchConv> conv_desc;
  float* filters = nullptr;
  void* kspec = nullptr;
  std::map<int, tcfftConv> conv_plans;  // plain path: one plan per convolution
  // graph replay
  cudaGraphExec_t graph = nullptr;
  Buffers graph_io{};
  int graph_mode = -1;
  int graph_launches = 0;
  // plain per-size path: plans per (log2 n, run length)
  std::map<std::pair<int, long long>, tcfftPlan> plans;
  struct Run {
    int logn;
    long long first, len;  // transforms [first, first + len) are adjacent in memory
  };
  std::vector<Run> runs;
};

namespace {

void free_batch(tcfftBatchImpl* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (auto& kv : b->plans) tcfft_destroy(kv.second);
  for (auto& kv : b->conv_plans) tcfft_conv2d_destroy(kv.second);
  cudaFree(b->ws);
  cudaFree(b->kspec);
  cudaFree(b->filters);
  cudaFree(b->arena);
  cudaFree(b->ctr);
  cudaFree(b->err);
  delete b;
}


// Device tables, line tables, items and transforms of the persistent launch.
tcfftStatus build_persistent(tcfftBatchImpl* b) {
  const int pr = b->precision == TCFFT_FP16 ? 0 : 1;
  const int lag = 2 * g_bk_ctas[pr][b->sign_idx];
  BatchSpec spec;
  spec.fuse_conv_columns = b->precision == TCFFT_FP16;
  spec.count = b->count;
  spec.n = b->n.data();
  spec.in_off = b->in_off.data();
  spec.out_off = b->out_off.data();
  spec.scale = b->scale.data();
  size_t kspec_elems = 0;
  for (const tcfftBatchConv& d : b->conv_desc) {
    BatchConv cv{};
    conv_geometry(d, cv);  // validated at plan entry
    cv.img_off = d.img_off;
    cv.out_off = d.out_off;
    cv.kspec = reinterpret_cast<void*>(kspec_elems);       // offset until the buffer exists
    cv.filt = reinterpret_cast<const float*>(d.filt_off);  // offset until the buffer exists
    kspec_elems += static_cast<size_t>(1) << (2 * cv.logP);
    spec.convs.push_back(cv);
    spec.conv_prep.push_back(1);
  }
  Built bl = build_items(spec, lag);
  b->nitems = static_cast<int>(bl.items.size());
  b->nxforms = static_cast<int>(bl.xforms.size());
  b->nctrs = bl.nctrs;
  b->ctas = g_bk_ctas[pr][b->sign_idx];
  const int sign = b->sign_idx == 0 ? -1 : 1;
  // which tables are needed
  bool need_tw[kBatchMaxLineLog + 1] = {}, need_otw[kBatchMaxLog + 1] = {};
  for (const BatchItem& it : bl.items) need_tw[it.logl] = true;
  for (const BatchItem& it : bl.prep_items) need_tw[it.logl] = true;
  for (const BatchXform& xf : bl.xforms) need_otw[xf.logn] = true;
  // arena layout (256-byte aligned pieces)
  size_t at = 0;
  const size_t off_bmat = at;
  at = align_up(at + 4096, 256);
  size_t off_tw[kBatchMaxLineLog + 1] = {};
  for (int l = 0; l <= kBatchMaxLineLog; ++l)
    if (need_tw[l]) {
      off_tw[l] = at;
      at = align_up(at + (sizeof(float2) << l), 256);
    }
  size_t off_lo[kBatchMaxLog + 1] = {}, off_hi[kBatchMaxLog + 1] = {};
  for (int l = 0; l <= kBatchMaxLog; ++l)
    if (need_otw[l]) {
      const int sh = (l + 1) / 2;
      off_lo[l] = at;
      at = align_up(at + (sizeof(float2) << sh), 256);
      off_hi[l] = at;
      at = align_up(at + (sizeof(float2) << (l - sh)), 256);
    }
  const size_t host_begin = at;
  const size_t off_lin = at;
  at = align_up(at + sizeof(long long) * bl.line_in.size(), 256);
  const size_t off_lout = at;
  at = align_up(at + sizeof(long long) * bl.line_out.size(), 256);
  const size_t off_items = at;
  at = align_up(at + sizeof(BatchItem) * bl.items.size(), 256);
  const size_t off_xf = at;
  at = align_up(at + sizeof(BatchXform) * bl.xforms.size(), 256);
  const size_t off_conv = at;
  at = align_up(at + sizeof(BatchConv) * bl.convs.size(), 256);
  const size_t off_prep = at;
  at = align_up(at + sizeof(BatchItem) * bl.prep_items.size(), 256);
  if (cudaMalloc(&b->arena, at) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  if (cudaMalloc(&b->ctr, sizeof(int) * static_cast<size_t>(b->nctrs)) != cudaSuccess ||
      cudaMalloc(&b->err, sizeof(int)) != cudaSuccess)
    return TCFFT_ALLOC_FAILED;
  if (cudaMemset(b->err, 0, sizeof(int)) != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  b->ws_bytes = bl.ws_elems * b->elem_bytes;
  if (b->ws_bytes && cudaMalloc(&b->ws, b->ws_bytes) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  const size_t kspec_bytes = kspec_elems * b->elem_bytes;
  if (kspec_bytes && cudaMalloc(&b->kspec, kspec_bytes) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  unsigned char* A = static_cast<unsigned char*>(b->arena);
  // FP64-generated tables, rounded once
  cudaError_t e = gen_dft16_bmat(reinterpret_cast<uint16_t*>(A + off_bmat), sign, 0, 0);
  if (e == cudaSuccess) e = gen_dft16_bmat(reinterpret_cast<uint16_t*>(A + off_bmat) + 1024, sign, 1, 0);
  for (int l = 0; l <= kBatchMaxLineLog && e == cudaSuccess; ++l)
    if (need_tw[l]) e = gen_twiddles(reinterpret_cast<float2*>(A + off_tw[l]), 1ll << l, l, 0, sign, 0);
  for (int l = 0; l <= kBatchMaxLog && e == cudaSuccess; ++l)
    if (need_otw[l]) {
      const int sh = (l + 1) / 2;
      e = gen_twiddles(reinterpret_cast<float2*>(A + off_lo[l]), 1ll << sh, l, 0, sign, 0);
      if (e == cudaSuccess)
        e = gen_twiddles(reinterpret_cast<float2*>(A + off_hi[l]), 1ll << (l - sh), l, sh, sign, 0);
    }
  if (e != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  // host-built lists, one copy
  std::vector<unsigned char> host(at - host_begin, 0);
  auto put = [&](size_t off, const void* src, size_t bytes) {
    if (bytes) std::memcpy(host.data() + (off - host_begin), src, bytes);
  };
  put(off_lin, bl.line_in.data(), sizeof(long long) * bl.line_in.size());
  put(off_lout, bl.line_out.data(), sizeof(long long) * bl.line_out.size());
  put(off_items, bl.items.data(), sizeof(BatchItem) * bl.items.size());
  put(off_xf, bl.xforms.data(), sizeof(BatchXform) * bl.xforms.size());
  // offsets -> device addresses of the spectra and filters
  for (BatchConv& cv : bl.convs) {
    cv.kspec = static_cast<unsigned char*>(b->kspec) + reinterpret_cast<size_t>(cv.kspec) * b->elem_bytes;
    cv.filt = b->filters + reinterpret_cast<size_t>(cv.filt);
  }
  put(off_conv, bl.convs.data(), sizeof(BatchConv) * bl.convs.size());
  put(off_prep, bl.prep_items.data(), sizeof(BatchItem) * bl.prep_items.size());
  if (cudaMemcpy(A + host_begin, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  BatchArgs& a = b->args;
  std::memset(&a, 0, sizeof(a));
  a.ws = b->ws;
  a.line_in = reinterpret_cast<const long long*>(A + off_lin);
  a.line_out = reinterpret_cast<const long long*>(A + off_lout);
  a.items = reinterpret_cast<const BatchItem*>(A + off_items);
  a.nitems = b->nitems;
  a.xforms = reinterpret_cast<const BatchXform*>(A + off_xf);
  a.convs = reinterpret_cast<const BatchConv*>(A + off_conv);
  a.counter = reinterpret_cast<unsigned int*>(b->ctr);
  a.ctrs = b->ctr;
  for (int l = 0; l <= kBatchMaxLineLog; ++l)
    if (need_tw[l]) a.tw[l] = reinterpret_cast<const float2*>(A + off_tw[l]);
  for (int l = 0; l <= kBatchMaxLog; ++l)
    if (need_otw[l]) {
      a.otw[l].lo = reinterpret_cast<const float2*>(A + off_lo[l]);
      a.otw[l].hi = reinterpret_cast<const float2*>(A + off_hi[l]);
      a.otw[l].shift = (l + 1) / 2;
      a.otw[l].logn = l;
    }
  a.bmat = reinterpret_cast<const uint32_t*>(A + off_bmat);
  a.err = b->err;
  a.wait_polls = dep_wait_polls();  // each launch refreshes it (launch_persistent)
  if (!bl.prep_items.empty()) {
    // filter spectra: the same kernel over the filter items, once
    BatchArgs pa = a;
    pa.items = reinterpret_cast<const BatchItem*>(A + off_prep);
    pa.nitems = static_cast<int>(bl.prep_items.size());
    if (cudaMemset(b->ctr, 0, sizeof(int) * static_cast<size_t>(b->nctrs)) != cudaSuccess)
      return TCFFT_LAUNCH_FAILED;
    const int grid = std::min(b->ctas, pa.nitems);
    void* params[] = {&pa};
    if (cudaLaunchKernel(g_bk[pr][0].fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), params,
                         static_cast<size_t>(g_bk[pr][0].smem), nullptr) != cudaSuccess)
      return TCFFT_LAUNCH_FAILED;
  }
  if (cudaDeviceSynchronize() != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  int flag = 0;
  if (cudaMemcpy(&flag, b->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  return flag ? TCFFT_TIMEOUT : TCFFT_OK;
}

// Runs of adjacent same-size, same-scale transforms for the plain path, and
// one plan per (size, run length).
tcfftStatus build_per_size(tcfftBatchImpl* b) {
  b->runs.clear();
  for (int i = 0; i < b->count;) {
    int j = i + 1;
    while (j < b->count && b->n[j] == b->n[i] && b->scale[j] == b->scale[i] &&
           b->in_off[j] == b->in_off[j - 1] + b->n[i] && b->out_off[j] == b->out_off[j - 1] + b->n[i])
      ++j;
    tcfftBatchImpl::Run r{ilog2_exact(b->n[i]), i, j - i};
    b->runs.push_back(r);
    const auto key = std::make_pair(r.logn, r.len);
    if (!b->plans.count(key)) {
      tcfftPlan p = nullptr;
      const tcfftStatus s = tcfft_plan_1d(&p, b->n[i], r.len, b->precision);
      if (s != TCFFT_OK) return s;
      b->plans[key] = p;
    }
    i = j;
  }
  return TCFFT_OK;
}

tcfftStatus launch_persistent(tcfftBatchImpl* b, const Buffers& io, cudaStream_t st, int* launches) {
  const int pr = b->precision == TCFFT_FP16 ? 0 : 1;
  if (cudaMemsetAsync(b->ctr, 0, sizeof(int) * static_cast<size_t>(b->nctrs), st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  if (b->nitems == 0) return TCFFT_OK;
  BatchArgs a = b->args;
  a.wait_polls = dep_wait_polls();
  a.in = io.in;
  a.out = io.out;
  a.conv_in = io.conv_in;
  a.conv_out = io.conv_out;
  const int grid = std::min(b->ctas, b->nitems);
  void* params[] = {&a};
  if (cudaLaunchKernel(g_bk[pr][b->sign_idx].fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), params,
                       static_cast<size_t>(g_bk[pr][b->sign_idx].smem), st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  ++*launches;
  return TCFFT_OK;
}

// Plain path: one tcfft_exec per run of adjacent same-size transforms and one
// convolution plan (filters resident) per convolution, as a caller of the
// per-size API would write it.
tcfftStatus launch_per_size(tcfftBatchImpl* b, const Buffers& io, cudaStream_t st, int* launches) {
  const int direction = b->sign_idx == 0 ? TCFFT_FORWARD : TCFFT_INVERSE;
  for (const tcfftBatchImpl::Run& r : b->runs) {
    tcfftPlan p = b->plans[std::make_pair(r.logn, r.len)];
    const unsigned char* src = static_cast<const unsigned char*>(io.in) + b->in_off[r.first] * b->elem_bytes;
    unsigned char* dst = static_cast<unsigned char*>(io.out) + b->out_off[r.first] * b->elem_bytes;
    const tcfftStatus s = tcfft_exec(p, src, dst, direction, b->scale[r.first], st);
    if (s != TCFFT_OK) return s;
    *launches += tcfft_last_launch_count();
  }
  const size_t rb = b->precision == TCFFT_FP16 ? 2 : 4;  // bytes per real element
  for (size_t c = 0; c < b->conv_desc.size(); ++c) {
    const tcfftBatchConv& d = b->conv_desc[c];
    const auto itp = b->conv_plans.find(static_cast<int>(c));
    if (itp == b->conv_plans.end()) return TCFFT_INVALID_VALUE;  // made by tcfft_batch_set_mode
    const unsigned char* src = static_cast<const unsigned char*>(io.conv_in) + d.img_off * rb;
    unsigned char* dst = static_cast<unsigned char*>(io.conv_out) + d.out_off * rb;
    const tcfftStatus s = tcfft_conv2d_exec(itp->second, src, dst, 1, st);
    if (s != TCFFT_OK) return s;
    *launches += 5;  // row, column, pointwise, column, row
  }
  return TCFFT_OK;
}

tcfftStatus launch_all(tcfftBatchImpl* b, const Buffers& io, cudaStream_t st, int* launches) {
  return b->mode == TCFFT_BATCH_PERSISTENT ? launch_persistent(b, io, st, launches)
                                           : launch_per_size(b, io, st, launches);
}

// Plain-path convolution plans, one per convolution with its filter resident
// (made before any capture: plan creation allocates).
tcfftStatus make_conv_plans(tcfftBatchImpl* b) {
  for (size_t c = 0; c < b->conv_desc.size(); ++c) {
    if (b->conv_plans.count(static_cast<int>(c))) continue;
    const tcfftBatchConv& d = b->conv_desc[c];
    tcfftConv cp = nullptr;
    tcfftStatus s = tcfft_conv2d_plan(&cp, 1, 1, d.sy, d.sx, d.fy, d.fx, d.mode, b->precision, 1);
    if (s == TCFFT_OK) s = tcfft_conv2d_set_filters(cp, b->filters + d.filt_off, nullptr);
    if (s == TCFFT_OK) s = tcfft_conv2d_check(cp, nullptr);
    if (s != TCFFT_OK) {
      if (cp) tcfft_conv2d_destroy(cp);
      return s;
    }
    b->conv_plans.emplace(static_cast<int>(c), cp);
  }
  return TCFFT_OK;
}

tcfftStatus exec_buffers(tcfftBatchImpl* b, const Buffers& io, cudaStream_t st) {
  int launches = 0;
  if (!b->use_graph) {
    const tcfftStatus s = launch_all(b, io, st, &launches);
    return record_status(s, launches);
  }
  if (!b->graph || !(b->graph_io == io) || b->graph_mode != b->mode) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    cudaStream_t cap = nullptr;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess)
      return record_status(TCFFT_LAUNCH_FAILED, 0);
    tcfftStatus s = TCFFT_OK;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
    int captured = 0;
    if (s == TCFFT_OK) s = launch_all(b, io, cap, &captured);
    cudaGraph_t g = nullptr;
    const cudaError_t end = cudaStreamEndCapture(cap, &g);
    if (s == TCFFT_OK && (end != cudaSuccess || !g)) s = TCFFT_LAUNCH_FAILED;
    if (s == TCFFT_OK && cudaGraphInstantiate(&b->graph, g, 0) != cudaSuccess) {
      b->graph = nullptr;
      s = TCFFT_LAUNCH_FAILED;
    }
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cap);
    if (s != TCFFT_OK) return record_status(s, 0);
    b->graph_io = io;
    b->graph_mode = b->mode;
    b->graph_launches = captured;
  }
  if (cudaGraphLaunch(b->graph, st) != cudaSuccess) return record_status(TCFFT_LAUNCH_FAILED, 0);
  return record_status(TCFFT_OK, b->graph_launches);
}

}  // namespace

extern "C" {

tcfftStatus tcfft_batch_plan_mixed(tcfftBatch* batch, int count, const long long* n, const long long* in_off,
                                   const long long* out_off, const float* scale, int nconv,
                                   const tcfftBatchConv* convs, const float* filters, long long filter_floats,
                                   int precision, int direction) {
  if (!batch) return record_status(TCFFT_INVALID_VALUE, 0);
  *batch = nullptr;
  if (count < 0 || nconv < 0 || count + nconv < 1) return record_status(TCFFT_INVALID_VALUE, 0);
  if (count > 0 && (!n || !in_off || !out_off)) return record_status(TCFFT_INVALID_VALUE, 0);
  if (nconv > 0 && (!convs || !filters || filter_floats < 1)) return record_status(TCFFT_INVALID_VALUE, 0);
  if (precision != TCFFT_FP16 && precision != TCFFT_SPLIT_FP32) return record_status(TCFFT_INVALID_VALUE, 0);
  if (direction != TCFFT_FORWARD && direction != TCFFT_INVERSE) return record_status(TCFFT_INVALID_VALUE, 0);
  // convolutions run as forward transforms only; their plan is forward
  if (nconv > 0 && direction != TCFFT_FORWARD) return record_status(TCFFT_INVALID_VALUE, 0);
  const long long align_elems = precision == TCFFT_FP16 ? 4 : 2;  // 16 bytes
  for (int i = 0; i < count; ++i) {
    const int l = ilog2_exact(n[i]);
    if (l < kMinLog || l > kMaxLog) return record_status(TCFFT_INVALID_SIZE, 0);
    if (in_off[i] < 0 || out_off[i] < 0 || in_off[i] % align_elems || out_off[i] % align_elems)
      return record_status(TCFFT_INVALID_VALUE, 0);
  }
  for (int c = 0; c < nconv; ++c) {
    const tcfftBatchConv& d = convs[c];
    BatchConv cv{};
    if (d.sy < 1 || d.sx < 1 || d.fy < 1 || d.fx < 1 || !conv_geometry(d, cv)) return record_status(TCFFT_INVALID_SIZE, 0);
    if (d.img_off < 0 || d.out_off < 0 || d.filt_off < 0 ||
        d.filt_off + static_cast<long long>(d.fy) * d.fx > filter_floats)
      return record_status(TCFFT_INVALID_VALUE, 0);
  }
  tcfftStatus s = registry_ready();
  if (s != TCFFT_OK) return record_status(s, 0);
  std::call_once(g_bk_once, init_batch_registry);
  if (g_bk_err != cudaSuccess) return record_status(TCFFT_NO_DEVICE, 0);
  tcfftBatchImpl* b = new (std::nothrow) tcfftBatchImpl();
  if (!b) return record_status(TCFFT_ALLOC_FAILED, 0);
  b->precision = precision;
  b->sign_idx = direction == TCFFT_FORWARD ? 0 : 1;
  b->count = count;
  b->elem_bytes = precision == TCFFT_FP16 ? 4 : 8;
  if (count > 0) {
    b->n.assign(n, n + count);
    b->in_off.assign(in_off, in_off + count);
    b->out_off.assign(out_off, out_off + count);
    b->scale.assign(static_cast<size_t>(count), 1.0f);
    if (scale) b->scale.assign(scale, scale + count);
  }
  if (nconv > 0) {
    b->conv_desc.assign(convs, convs + nconv);
    // plan-owned copy of the filters: the spectra are made now, the plain
    // path's per-convolution plans later
    if (cudaMalloc(&b->filters, sizeof(float) * static_cast<size_t>(filter_floats)) != cudaSuccess ||
        cudaMemcpy(b->filters, filters, sizeof(float) * static_cast<size_t>(filter_floats),
                   cudaMemcpyDefault) != cudaSuccess)
      s = TCFFT_ALLOC_FAILED;
  }
  if (s == TCFFT_OK) s = build_persistent(b);
  if (s == TCFFT_OK) s = build_per_size(b);
  if (s != TCFFT_OK) {
    free_batch(b);
    return record_status(s, 0);
  }
  *batch = b;
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_plan(tcfftBatch* batch, int count, const long long* n, const long long* in_off,
                             const long long* out_off, const float* scale, int precision, int direction) {
  if (count < 1) {
    if (batch) *batch = nullptr;
    return record_status(TCFFT_INVALID_VALUE, 0);
  }
  return tcfft_batch_plan_mixed(batch, count, n, in_off, out_off, scale, 0, nullptr, nullptr, 0, precision,
                                direction);
}

tcfftStatus tcfft_batch_set_mode(tcfftBatch b, int mode) {
  if (!b || (mode != TCFFT_BATCH_PERSISTENT && mode != TCFFT_BATCH_PER_SIZE))
    return record_status(TCFFT_INVALID_VALUE, 0);
  if (mode == TCFFT_BATCH_PER_SIZE) {
    const tcfftStatus s = make_conv_plans(b);
    if (s != TCFFT_OK) return record_status(s, 0);
  }
  b->mode = mode;
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_set_graph(tcfftBatch b, int enable) {
  if (!b) return record_status(TCFFT_INVALID_VALUE, 0);
  b->use_graph = enable != 0;
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_exec_mixed(tcfftBatch b, const void* in, void* out, const void* conv_in, void* conv_out,
                                   void* stream) {
  if (!b) return record_status(TCFFT_INVALID_VALUE, 0);
  if (b->count > 0 && (!in || !out)) return record_status(TCFFT_INVALID_VALUE, 0);
  if (!b->conv_desc.empty() && (!conv_in || !conv_out)) return record_status(TCFFT_INVALID_VALUE, 0);
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u)
    return record_status(TCFFT_INVALID_VALUE, 0);
  return exec_buffers(b, Buffers{in, out, conv_in, conv_out}, static_cast<cudaStream_t>(stream));
}

tcfftStatus tcfft_batch_exec(tcfftBatch b, const void* in, void* out, void* stream) {
  if (!b || !in || !out) return record_status(TCFFT_INVALID_VALUE, 0);
  if (!b->conv_desc.empty()) return record_status(TCFFT_INVALID_VALUE, 0);
  return tcfft_batch_exec_mixed(b, in, out, nullptr, nullptr, stream);
}

tcfftStatus tcfft_batch_info(tcfftBatch b, int* items, size_t* workspace_bytes, int* ctas) {
  if (!b) return record_status(TCFFT_INVALID_VALUE, 0);
  if (items) *items = b->nitems;
  if (workspace_bytes) *workspace_bytes = b->ws_bytes;
  if (ctas) *ctas = std::min(b->ctas, b->nitems);
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_check(tcfftBatch b, void* stream) {
  if (!b) return record_status(TCFFT_INVALID_VALUE, 0);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return record_status(TCFFT_LAUNCH_FAILED, 0);
  int flag = 0;
  if (cudaMemcpy(&flag, b->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemset(b->err, 0, sizeof(int)) != cudaSuccess)
    return record_status(TCFFT_LAUNCH_FAILED, 0);
  for (auto& kv : b->plans) {
    const tcfftStatus s = tcfft_check(kv.second, stream);
    if (s != TCFFT_OK) return record_status(s, 0);
  }
  for (auto& kv : b->conv_plans) {
    const tcfftStatus s = tcfft_conv2d_check(kv.second, stream);
    if (s != TCFFT_OK) return record_status(s, 0);
  }
  if (flag & (kErrMmaTimeout | kErrQueueTimeout)) return record_status(TCFFT_TIMEOUT, 0);
  if (flag) return record_status(TCFFT_INVALID_VALUE, 0);
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_destroy(tcfftBatch b) {
  if (!b) return record_status(TCFFT_INVALID_VALUE, 0);
  free_batch(b);
  return record_status(TCFFT_OK, 0);
}

}  // extern "C"
