// tcfft_exec_static: the fused four-step FP16 1D FFT (fft_fused.cuh) with all
// of its scratch in one file-scope device array, so a call allocates nothing.
//
// Scratch layout (kStaticScratchBytes = 17 MiB):
//   [0, 16 MiB)            workspace ring: two slots of 8 MiB; a chunk is
//                          2^23 / (4 n) sequences (one sequence at n = 2^21)
//   [16 MiB, +64 KiB)      word 0: error bits (sticky: cleared at set-up and
//                          by a call with wait != 0 after it reads them);
//                          from byte 256: queue counter, done1[nchunks],
//                          done2[nchunks] -- these must be zero when the
//                          kernel starts, so every call clears them on its
//                          stream before the launch
//   [16 MiB + 64 KiB, ...) tables, written once per device at set-up: the DFT16
//                          B images, W_L for L = 2^7 .. 2^11 and the outer
//                          twiddle factors W_n for n = 2^15 .. 2^21, both signs
// Every call on a device shares this array: calls whose executions overlap
// on the GPU (different streams, or host threads without ordering between
// them) race on the ring and the counters. Calls on one stream are ordered.
//
// Set-up (first call on each device, with that device current): the CUDA
// runtime loads this library's device code onto the device when it is first
// needed (lazy module loading, the default), which is when the array gets its
// device memory; cudaGetSymbolAddress triggers that, then the table kernels
// run on the caller's stream and that stream is synchronised. So the first
// call is not allocation-free at the driver level and waits for the caller's
// stream once; it must not be made while the stream is being captured into a
// CUDA graph (it returns TCFFT_UNSUPPORTED then, and set-up runs on a later
// call). A failed set-up is retried by the next call.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/tcfft_gb300.h"
#include "capi_internal.cuh"
#include "fft_fused.cuh"
#include "tables.cuh"

using namespace tcfft;

namespace {

constexpr int kStaticMinLog = 15, kStaticMaxLog = 21;
constexpr int kStaticMinPass = 7, kStaticMaxPass = 11;  // log2 of the pass lengths used
constexpr size_t kRingSlotBytes = size_t{8} << 20;
constexpr size_t kRingBytes = 2 * kRingSlotBytes;
constexpr size_t kCtrBytes = size_t{64} << 10;
constexpr size_t kCtrStart = 256;  // counters after the error word, own 256 B line
constexpr int kMaxChunks = static_cast<int>(((kCtrBytes - kCtrStart) / 4 - 1) / 2);
constexpr size_t kTableBytes = (size_t{1} << 20) - kCtrBytes;
constexpr size_t kStaticScratchBytes = kRingBytes + kCtrBytes + kTableBytes;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Byte offsets of the tables inside the table region.
struct TableLayout {
  size_t bmat[2];
  size_t tw[2][kStaticMaxPass + 1];
  size_t otw_lo[2][kStaticMaxLog + 1], otw_hi[2][kStaticMaxLog + 1];
  size_t end;
};

constexpr int outer_shift(int logn) { return (logn + 1) / 2; }

constexpr TableLayout table_layout() {
  TableLayout t{};
  size_t at = 0;
  for (int sg = 0; sg < 2; ++sg) {
    t.bmat[sg] = at;
    at += 4096;  // hi and lo images, 2 KiB each
  }
  for (int sg = 0; sg < 2; ++sg)
    for (int l = kStaticMinPass; l <= kStaticMaxPass; ++l) {
      t.tw[sg][l] = at;
      at += sizeof(float2) << l;
    }
  for (int sg = 0; sg < 2; ++sg)
    for (int l = kStaticMinLog; l <= kStaticMaxLog; ++l) {
      t.otw_lo[sg][l] = at;
      at += sizeof(float2) << outer_shift(l);
      t.otw_hi[sg][l] = at;
      at += sizeof(float2) << (l - outer_shift(l));
    }
  t.end = at;
  return t;
}

// The column/row split the plan API makes for 2^logn (tcfft_plan_1d), which
// the fused kernel of that size was instantiated for.
constexpr int split_log_n1(int logn) {
  int a = logn / 2 < 10 ? logn / 2 : 10;
  if (logn - a > 12) a = logn - 12;
  return a;
}

constexpr int kMaxDevices = 64;
struct DeviceScratch {
  std::mutex mu;
  bool done = false;  // set only after a successful set-up
  unsigned char* base = nullptr;
};
DeviceScratch g_dev[kMaxDevices];

// With the device current and d.mu held: find the array's device address
// (which loads the module onto the device if it is not yet loaded), write the
// tables and clear the error word on the caller's stream, and wait for that
// stream. Returns the status; d.done stays false on failure so that the next
// call tries again.
tcfftStatus set_up(DeviceScratch& d, cudaStream_t st) {
  tcfftStatus s = registry_ready();
  if (s != TCFFT_OK) return s;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  if (cs != cudaStreamCaptureStatusNone) return TCFFT_UNSUPPORTED;  // cannot wait inside a capture
  unsigned char* ptr = nullptr;
  if (cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_static_scratch) != cudaSuccess || !ptr)
    return TCFFT_LAUNCH_FAILED;
  const TableLayout t = table_layout();
  unsigned char* tab = ptr + kRingBytes + kCtrBytes;
  cudaError_t e = cudaMemsetAsync(ptr + kRingBytes, 0, sizeof(int), st);
  for (int sg = 0; sg < 2 && e == cudaSuccess; ++sg) {
    const int sign = sg == 0 ? -1 : 1;
    uint16_t* bm = reinterpret_cast<uint16_t*>(tab + t.bmat[sg]);
    e = gen_dft16_bmat(bm, sign, 0, st);
    if (e == cudaSuccess) e = gen_dft16_bmat(bm + 1024, sign, 1, st);
    for (int l = kStaticMinPass; l <= kStaticMaxPass && e == cudaSuccess; ++l)
      e = gen_twiddles(reinterpret_cast<float2*>(tab + t.tw[sg][l]), 1ll << l, l, 0, sign, st);
    for (int l = kStaticMinLog; l <= kStaticMaxLog && e == cudaSuccess; ++l) {
      const int sh = outer_shift(l);
      e = gen_twiddles(reinterpret_cast<float2*>(tab + t.otw_lo[sg][l]), 1ll << sh, l, 0, sign, st);
      if (e == cudaSuccess)
        e = gen_twiddles(reinterpret_cast<float2*>(tab + t.otw_hi[sg][l]), 1ll << (l - sh), l, sh, sign, st);
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  d.base = ptr;
  d.done = true;
  return TCFFT_OK;
}

static_assert(kStaticMaxLog - split_log_n1(kStaticMaxLog) <= kStaticMaxPass, "pass table range");
static_assert(split_log_n1(kStaticMinLog) >= kStaticMinPass, "pass table range");
static_assert(table_layout().end <= kTableBytes, "tables exceed their region");

}  // namespace

extern "C" tcfftStatus tcfft_exec_static(const void* in, void* out, long long n, long long batch, int direction,
                                         float scale, void* stream, int wait) {
  if (!in || !out || batch < 1) return record_status(TCFFT_INVALID_VALUE, 0);
  if (direction != TCFFT_FORWARD && direction != TCFFT_INVERSE) return record_status(TCFFT_INVALID_VALUE, 0);
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u)
    return record_status(TCFFT_INVALID_VALUE, 0);
  if (n < 1 || (n & (n - 1)) != 0) return record_status(TCFFT_INVALID_SIZE, 0);
  int logn = 0;
  while ((1ll << logn) < n) ++logn;
  if (logn < kStaticMinLog) return record_status(TCFFT_INVALID_SIZE, 0);
  if (logn > kStaticMaxLog) return record_status(TCFFT_CAPACITY, 0);  // one sequence would not fit a slot
  const long long per_seq = n * 4;
  const long long chunk_seqs_max = static_cast<long long>(kRingSlotBytes) / per_seq;
  const long long chunk_seqs = chunk_seqs_max < batch ? chunk_seqs_max : batch;
  const long long nchunks = (batch + chunk_seqs - 1) / chunk_seqs;
  if (nchunks > kMaxChunks) return record_status(TCFFT_CAPACITY, 0);  // counters would not fit

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return record_status(TCFFT_NO_DEVICE, 0);
  DeviceScratch& d = g_dev[dev];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  {
    std::lock_guard<std::mutex> lock(d.mu);
    if (!d.done) {
      const tcfftStatus s = set_up(d, st);
      if (s != TCFFT_OK) return record_status(s, 0);
    }
  }

  const int sg = direction == TCFFT_FORWARD ? 0 : 1;
  int grid_ctas = 0;
  const FusedKernel* fk = fused_kernel(logn, sg, &grid_ctas);
  const int log_n1 = split_log_n1(logn), log_n2 = logn - log_n1;
  if (!fk || fk->log_n1 != log_n1 || fk->log_n2 != log_n2) return record_status(TCFFT_UNSUPPORTED, 0);

  unsigned char* ring = d.base;
  int* err = reinterpret_cast<int*>(d.base + kRingBytes);
  int* ctr = reinterpret_cast<int*>(d.base + kRingBytes + kCtrStart);
  const unsigned char* tab = d.base + kRingBytes + kCtrBytes;
  const TableLayout t = table_layout();
  const long long n1 = 1ll << log_n1, n2 = 1ll << log_n2;

  IoHalf<false, false> a;
  std::memset(&a, 0, sizeof(a));
  a.in = static_cast<const half2*>(in);
  a.out = reinterpret_cast<half2*>(ring);
  a.lps_log2 = log_n2;
  a.in_seq = a.out_seq = n;
  a.in_line = a.out_line = 1;
  a.in_elem = a.out_elem = n2;
  a.otw.hi = reinterpret_cast<const float2*>(tab + t.otw_hi[sg][logn]);
  a.otw.lo = reinterpret_cast<const float2*>(tab + t.otw_lo[sg][logn]);
  a.otw.shift = outer_shift(logn);
  a.otw.logn = logn;
  a.scale = 1.0f;
  IoHalf<true, false, true> b;
  std::memset(&b, 0, sizeof(b));
  b.in = reinterpret_cast<const half2*>(ring);
  b.out = static_cast<half2*>(out);
  b.lps_log2 = log_n1;
  b.in_seq = b.out_seq = n;
  b.in_line = n2;
  b.in_elem = 1;
  b.out_line = 1;
  b.out_elem = n1;
  b.scale = scale;
  PassCore c1, c2;
  c1.bmat = c2.bmat = reinterpret_cast<const uint32_t*>(tab + t.bmat[sg]);
  c1.tw = reinterpret_cast<const float2*>(tab + t.tw[sg][log_n1]);
  c2.tw = reinterpret_cast<const float2*>(tab + t.tw[sg][log_n2]);
  c1.err = c2.err = err;
  FusedSched sc;
  sc.counter = reinterpret_cast<unsigned int*>(ctr);
  sc.done1 = ctr + 1;
  sc.done2 = ctr + 1 + nchunks;
  sc.nchunks = static_cast<int>(nchunks);
  sc.tiles1 = static_cast<int>((chunk_seqs * n2 + fk->G1 - 1) / fk->G1);
  sc.tiles2 = static_cast<int>((chunk_seqs * n1 + fk->G2 - 1) / fk->G2);
  sc.ring = nchunks >= 2 ? 2 : 1;
  sc.chunk_seqs = static_cast<int>(chunk_seqs);
  sc.batch = batch;
  sc.n = n;
  sc.wait_polls = dep_wait_polls();

  // queue counter and done counters start at zero; the error word keeps any
  // bit an earlier call with wait == 0 left, for the next call that waits
  if (cudaMemsetAsync(ctr, 0, sizeof(int) * (1 + 2 * static_cast<size_t>(nchunks)), st) != cudaSuccess)
    return record_status(TCFFT_LAUNCH_FAILED, 0);
  const long long items = nchunks * (sc.tiles1 + sc.tiles2);
  long long grid = grid_ctas > 0 ? grid_ctas : 1;
  if (grid > items) grid = items;
  void* args[] = {&a, &b, &c1, &c2, &sc};
  if (cudaLaunchKernel(fk->fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), args,
                       static_cast<size_t>(fk->smem), st) != cudaSuccess)
    return record_status(TCFFT_LAUNCH_FAILED, 0);
  if (!wait) return record_status(TCFFT_OK, 1);
  // this call's error bits and any left by earlier calls with wait == 0
  int flag = 0;
  if (cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return record_status(TCFFT_LAUNCH_FAILED, 1);
  if (flag && cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return record_status(TCFFT_LAUNCH_FAILED, 1);
  if (flag & (kErrMmaTimeout | kErrQueueTimeout)) return record_status(TCFFT_TIMEOUT, 1);
  if (flag) return record_status(TCFFT_INVALID_VALUE, 1);
  return record_status(TCFFT_OK, 1);
}
