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
#include "fft_batch.cuh"
#include "tables.cuh"

using namespace tcfft;

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

int ilog2_exact(long long v) {
  if (v <= 0 || (v & (v - 1)) != 0) return -1;
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

// Four-step split used by the batch kernel: both pass lengths in [2^7, 2^10].
int batch_log_n1(int logn) {
  int a = logn / 2;
  if (a < kBatchMinPassLog) a = kBatchMinPassLog;
  if (logn - a > kBatchMaxPassLog) a = logn - kBatchMaxPassLog;
  return a;
}

constexpr int kMinLog = kBatchMinLineLog;  // 64 points
constexpr int kMaxLog = kBatchMaxLog;      // 2^20 points

}  // namespace

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
  int nitems = 0, nxforms = 0, ctas = 0;
  size_t ws_bytes = 0;
  void* ws = nullptr;
  void* arena = nullptr;  // tables, line tables, items, transforms
  int* ctr = nullptr;     // [0] queue head, [1 ..] per-transform done counters
  int* err = nullptr;
  BatchArgs args{};
  // graph replay
  cudaGraphExec_t graph = nullptr;
  const void* graph_in = nullptr;
  void* graph_out = nullptr;
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

struct Built {
  std::vector<long long> line_in, line_out;
  std::vector<BatchItem> items;
  std::vector<BatchXform> xforms;
  size_t ws_elems = 0;
};

// Work list: single-pass transforms grouped by size into tiles of
// G = 8192 / L lines; four-step transforms as P1 tiles and, `lag` items
// later, their P2 tiles; single-pass tiles are spread evenly in between.
Built build_items(const tcfftBatchImpl& b, int lag) {
  Built out;
  std::vector<BatchItem> line_items;
  for (int logl = kBatchMinLineLog; logl <= kBatchMaxLineLog; ++logl) {
    const int G = kBatchMt * 16 >> logl;
    std::vector<int> ids;
    for (int i = 0; i < b.count; ++i)
      if (ilog2_exact(b.n[i]) == logl) ids.push_back(i);
    size_t k = 0;
    while (k < ids.size()) {
      // one scale per tile: split the tile where the scale changes
      size_t end = std::min(ids.size(), k + static_cast<size_t>(G));
      for (size_t j = k + 1; j < end; ++j)
        if (b.scale[ids[j]] != b.scale[ids[k]]) {
          end = j;
          break;
        }
      BatchItem it{};
      it.kind = kItemLines;
      it.logl = logl;
      it.line0 = static_cast<int>(out.line_in.size());
      it.nlines = static_cast<int>(end - k);
      it.scale = b.scale[ids[k]];
      for (size_t j = k; j < end; ++j) {
        out.line_in.push_back(b.in_off[ids[j]]);
        out.line_out.push_back(b.out_off[ids[j]]);
      }
      line_items.push_back(it);
      k = end;
    }
  }
  // four-step transforms
  struct Four {
    std::vector<BatchItem> p1, p2;
  };
  std::vector<Four> fours;
  for (int i = 0; i < b.count; ++i) {
    const int logn = ilog2_exact(b.n[i]);
    if (logn <= kBatchMaxLineLog) continue;
    BatchXform xf{};
    xf.in_off = b.in_off[i];
    xf.out_off = b.out_off[i];
    xf.ws_off = static_cast<long long>(out.ws_elems);
    xf.logn = logn;
    xf.log_n1 = batch_log_n1(logn);
    xf.log_n2 = logn - xf.log_n1;
    out.ws_elems += static_cast<size_t>(b.n[i]);
    const int g1 = kBatchMt * 16 >> xf.log_n1, g2 = kBatchMt * 16 >> xf.log_n2;
    const int lines1 = 1 << xf.log_n2, lines2 = 1 << xf.log_n1;
    xf.tiles1 = (lines1 + g1 - 1) / g1;
    Four f;
    for (int t = 0; t < xf.tiles1; ++t) {
      BatchItem it{};
      it.kind = kItemP1;
      it.logl = xf.log_n1;
      it.line0 = t * g1;
      it.xform = static_cast<int>(out.xforms.size());
      it.scale = 1.0f;
      f.p1.push_back(it);
    }
    for (int t = 0; t < (lines2 + g2 - 1) / g2; ++t) {
      BatchItem it{};
      it.kind = kItemP2;
      it.logl = xf.log_n2;
      it.line0 = t * g2;
      it.xform = static_cast<int>(out.xforms.size());
      it.scale = b.scale[i];
      f.p2.push_back(it);
    }
    out.xforms.push_back(xf);
    fours.push_back(std::move(f));
  }
  // merge: P1 of each four-step transform, its P2 `lag` items later, single
  // pass tiles spread evenly in between
  size_t total = line_items.size();
  for (const Four& f : fours) total += f.p1.size() + f.p2.size();
  out.items.reserve(total);
  std::deque<std::pair<size_t, const std::vector<BatchItem>*>> pending;
  size_t li = 0;
  const double per_four = fours.empty() ? 0.0 : static_cast<double>(line_items.size()) / fours.size();
  double line_credit = 0.0;
  auto release = [&](bool all) {
    while (!pending.empty() && (all || pending.front().first <= out.items.size())) {
      for (const BatchItem& it : *pending.front().second) out.items.push_back(it);
      pending.pop_front();
    }
  };
  for (const Four& f : fours) {
    release(false);
    for (const BatchItem& it : f.p1) out.items.push_back(it);
    pending.emplace_back(out.items.size() + static_cast<size_t>(lag), &f.p2);
    line_credit += per_four;
    while (line_credit >= 1.0 && li < line_items.size()) {
      out.items.push_back(line_items[li++]);
      line_credit -= 1.0;
      release(false);
    }
  }
  while (li < line_items.size()) {
    out.items.push_back(line_items[li++]);
    release(false);
  }
  release(true);
  return out;
}

}  // namespace

namespace {

void free_batch(tcfftBatchImpl* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (auto& kv : b->plans) tcfft_destroy(kv.second);
  cudaFree(b->ws);
  cudaFree(b->arena);
  cudaFree(b->ctr);
  cudaFree(b->err);
  delete b;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Device tables, line tables, items and transforms of the persistent launch.
tcfftStatus build_persistent(tcfftBatchImpl* b) {
  const int pr = b->precision == TCFFT_FP16 ? 0 : 1;
  const int lag = 2 * g_bk_ctas[pr][b->sign_idx];
  Built bl = build_items(*b, lag);
  b->nitems = static_cast<int>(bl.items.size());
  b->nxforms = static_cast<int>(bl.xforms.size());
  b->ctas = g_bk_ctas[pr][b->sign_idx];
  const int sign = b->sign_idx == 0 ? -1 : 1;
  // which tables are needed
  bool need_tw[kBatchMaxLineLog + 1] = {}, need_otw[kBatchMaxLog + 1] = {};
  for (const BatchItem& it : bl.items) need_tw[it.logl] = true;
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
  if (cudaMalloc(&b->arena, at) != cudaSuccess) return TCFFT_ALLOC_FAILED;
  if (cudaMalloc(&b->ctr, sizeof(int) * (1 + static_cast<size_t>(b->nxforms))) != cudaSuccess ||
      cudaMalloc(&b->err, sizeof(int)) != cudaSuccess)
    return TCFFT_ALLOC_FAILED;
  if (cudaMemset(b->err, 0, sizeof(int)) != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  b->ws_bytes = bl.ws_elems * b->elem_bytes;
  if (b->ws_bytes && cudaMalloc(&b->ws, b->ws_bytes) != cudaSuccess) return TCFFT_ALLOC_FAILED;
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
  a.counter = reinterpret_cast<unsigned int*>(b->ctr);
  a.done = b->ctr + 1;
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
  return cudaDeviceSynchronize() == cudaSuccess ? TCFFT_OK : TCFFT_LAUNCH_FAILED;
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

tcfftStatus launch_persistent(tcfftBatchImpl* b, const void* in, void* out, cudaStream_t st, int* launches) {
  const int pr = b->precision == TCFFT_FP16 ? 0 : 1;
  if (cudaMemsetAsync(b->ctr, 0, sizeof(int) * (1 + static_cast<size_t>(b->nxforms)), st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  if (b->nitems == 0) return TCFFT_OK;
  BatchArgs a = b->args;
  a.in = in;
  a.out = out;
  const int grid = std::min(b->ctas, b->nitems);
  void* params[] = {&a};
  if (cudaLaunchKernel(g_bk[pr][b->sign_idx].fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), params,
                       static_cast<size_t>(g_bk[pr][b->sign_idx].smem), st) != cudaSuccess)
    return TCFFT_LAUNCH_FAILED;
  ++*launches;
  return TCFFT_OK;
}

tcfftStatus launch_per_size(tcfftBatchImpl* b, const void* in, void* out, cudaStream_t st, int* launches) {
  const int direction = b->sign_idx == 0 ? TCFFT_FORWARD : TCFFT_INVERSE;
  for (const tcfftBatchImpl::Run& r : b->runs) {
    tcfftPlan p = b->plans[std::make_pair(r.logn, r.len)];
    const unsigned char* src = static_cast<const unsigned char*>(in) + b->in_off[r.first] * b->elem_bytes;
    unsigned char* dst = static_cast<unsigned char*>(out) + b->out_off[r.first] * b->elem_bytes;
    const tcfftStatus s = tcfft_exec(p, src, dst, direction, b->scale[r.first], st);
    if (s != TCFFT_OK) return s;
    *launches += tcfft_last_launch_count();
  }
  return TCFFT_OK;
}

tcfftStatus launch_all(tcfftBatchImpl* b, const void* in, void* out, cudaStream_t st, int* launches) {
  return b->mode == TCFFT_BATCH_PERSISTENT ? launch_persistent(b, in, out, st, launches)
                                           : launch_per_size(b, in, out, st, launches);
}

}  // namespace

extern "C" {

tcfftStatus tcfft_batch_plan(tcfftBatch* batch, int count, const long long* n, const long long* in_off,
                             const long long* out_off, const float* scale, int precision, int direction) {
  if (!batch) return record_status(TCFFT_INVALID_VALUE, 0);
  *batch = nullptr;
  if (count < 1 || !n || !in_off || !out_off) return record_status(TCFFT_INVALID_VALUE, 0);
  if (precision != TCFFT_FP16 && precision != TCFFT_SPLIT_FP32) return record_status(TCFFT_INVALID_VALUE, 0);
  if (direction != TCFFT_FORWARD && direction != TCFFT_INVERSE) return record_status(TCFFT_INVALID_VALUE, 0);
  const long long align_elems = precision == TCFFT_FP16 ? 4 : 2;  // 16 bytes
  for (int i = 0; i < count; ++i) {
    const int l = ilog2_exact(n[i]);
    if (l < kMinLog || l > kMaxLog) return record_status(TCFFT_INVALID_SIZE, 0);
    if (in_off[i] < 0 || out_off[i] < 0 || in_off[i] % align_elems || out_off[i] % align_elems)
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
  b->n.assign(n, n + count);
  b->in_off.assign(in_off, in_off + count);
  b->out_off.assign(out_off, out_off + count);
  b->scale.assign(static_cast<size_t>(count), 1.0f);
  if (scale) b->scale.assign(scale, scale + count);
  s = build_persistent(b);
  if (s == TCFFT_OK) s = build_per_size(b);
  if (s != TCFFT_OK) {
    free_batch(b);
    return record_status(s, 0);
  }
  *batch = b;
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_set_mode(tcfftBatch b, int mode) {
  if (!b || (mode != TCFFT_BATCH_PERSISTENT && mode != TCFFT_BATCH_PER_SIZE))
    return record_status(TCFFT_INVALID_VALUE, 0);
  b->mode = mode;
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_set_graph(tcfftBatch b, int enable) {
  if (!b) return record_status(TCFFT_INVALID_VALUE, 0);
  b->use_graph = enable != 0;
  return record_status(TCFFT_OK, 0);
}

tcfftStatus tcfft_batch_exec(tcfftBatch b, const void* in, void* out, void* stream) {
  if (!b || !in || !out) return record_status(TCFFT_INVALID_VALUE, 0);
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u)
    return record_status(TCFFT_INVALID_VALUE, 0);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int launches = 0;
  if (!b->use_graph) {
    const tcfftStatus s = launch_all(b, in, out, st, &launches);
    return record_status(s, launches);
  }
  if (!b->graph || b->graph_in != in || b->graph_out != out || b->graph_mode != b->mode) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    cudaStream_t cap = nullptr;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess)
      return record_status(TCFFT_LAUNCH_FAILED, 0);
    tcfftStatus s = TCFFT_OK;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) s = TCFFT_LAUNCH_FAILED;
    int captured = 0;
    if (s == TCFFT_OK) s = launch_all(b, in, out, cap, &captured);
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
    b->graph_in = in;
    b->graph_out = out;
    b->graph_mode = b->mode;
    b->graph_launches = captured;
  }
  if (cudaGraphLaunch(b->graph, st) != cudaSuccess) return record_status(TCFFT_LAUNCH_FAILED, 0);
  return record_status(TCFFT_OK, b->graph_launches);
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
