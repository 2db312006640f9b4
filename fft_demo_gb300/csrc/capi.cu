// C ABI: plan creation, execution and destruction for the tensor-core FFT.
//
// Plan logic restates, for arbitrary powers of two, what the reference's
// tcfftCreate / tcfftExec do for a fixed list of sizes
// (tcfft_half.cu:1177-1345): choose a chain of passes over the data, build the
// DFT-matrix table, launch. Here a pass is one kernel that runs a complete
// FFT of length L <= 2^14 on tiles held in shared memory; sizes above 2^14
// use the four-step split N = N1 * N2 (column pass with outer twiddle, then a
// transposing row pass), so every transform is at most two HBM round trips.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/tcfft_gb300.h"
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

PassKernel g_tab[kNumPassKinds][kMaxLogL + 1][kNumTileSel][2];
int g_occ[kNumPassKinds][kMaxLogL + 1][kNumTileSel][2];
std::once_flag g_once;
cudaError_t g_init_err = cudaSuccess;
int g_num_sms = 0;

void init_registry() {
  register_row_kernels(g_tab[kPassRow]);
  register_col_kernels(g_tab[kPassCol]);
  register_rowt_kernels(g_tab[kPassRowT]);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  for (int k = 0; k < kNumPassKinds && e == cudaSuccess; ++k)
    for (int l = 0; l <= kMaxLogL && e == cudaSuccess; ++l)
      for (int t = 0; t < kNumTileSel && e == cudaSuccess; ++t)
        for (int s = 0; s < 2 && e == cudaSuccess; ++s) {
          PassKernel& pk = g_tab[k][l][t][s];
          if (!pk.fn) continue;
          e = cudaFuncSetAttribute(pk.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pk.smem);
          if (e != cudaSuccess) break;
          int occ = 0;
          e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk.fn, kPassThreads, pk.smem);
          // TMEM: 512 columns per SM, a CTA holds Mt/4 columns.
          const int tmem_limit = 512 / (pk.Mt / 4);
          g_occ[k][l][t][s] = occ < tmem_limit ? occ : tmem_limit;
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
  cudaFree(p->err);
  delete p;
}

// Launch one pass; grid = persistent CTAs (at most the co-resident count).
tcfftStatus launch_pass(int kind, int logL, int tile, int sign_idx, const PassArgs& args,
                        cudaStream_t stream) {
  const PassKernel& pk = g_tab[kind][logL][tile][sign_idx];
  if (!pk.fn) return TCFFT_UNSUPPORTED;
  const long long ntiles = (args.total_lines + pk.G - 1) / pk.G;
  long long grid = static_cast<long long>(g_num_sms) * g_occ[kind][logL][tile][sign_idx];
  if (grid < 1) grid = 1;
  if (grid > ntiles) grid = ntiles;
  void* kargs[] = {const_cast<PassArgs*>(&args)};
  cudaError_t e = cudaLaunchKernel(pk.fn, dim3(static_cast<unsigned>(grid)), dim3(kPassThreads), kargs,
                                   static_cast<size_t>(pk.smem), stream);
  if (e != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  ++g_last_launches;
  return TCFFT_OK;
}

// Tile size for a contiguous-line pass: small tiles when big ones would
// leave SMs idle.
int pick_row_tile(int logL, long long lines) {
  const PassKernel& small = g_tab[kPassRow][logL][kTileSmall][0];
  const PassKernel& big = g_tab[kPassRow][logL][kTileBig][0];
  if (!small.fn) return kTileBig;
  const long long big_tiles = (lines + big.G - 1) / big.G;
  return big_tiles >= 2ll * g_num_sms ? kTileBig : kTileSmall;
}

PassArgs base_args(tcfftPlanImpl* p, int sign_idx, int logL, float scale) {
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.tw = p->tw[sign_idx][logL];
  a.bmat = reinterpret_cast<const uint32_t*>(p->bmat[sign_idx]);
  a.scale = scale;
  a.err = p->err;
  return a;
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

}  // namespace

extern "C" {

tcfftStatus tcfft_plan_1d(tcfftPlan* plan, long long n, long long batch, int precision) {
  if (!plan) return ret(TCFFT_INVALID_VALUE);
  *plan = nullptr;
  if (!is_pow2(n) || n < 16 || n > (1ll << 24) || batch < 1) return ret(TCFFT_INVALID_SIZE);
  if (precision != TCFFT_FP16 && precision != TCFFT_SPLIT_FP32) return ret(TCFFT_INVALID_VALUE);
  if (precision == TCFFT_SPLIT_FP32) return ret(TCFFT_UNSUPPORTED);
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
    if (logn <= kMaxLogL) {
      s = ensure_twiddle(p, logn);
    } else {
      // column pass length 2^a (<= 2^12), row pass length 2^(logn - a) (<= 2^12)
      int a = logn / 2 < 10 ? logn / 2 : 10;
      if (logn - a > 12) a = logn - 12;
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
      if (s == TCFFT_OK) {
        p->ws_bytes = static_cast<size_t>(n) * static_cast<size_t>(batch) * 4u;
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
  if (precision == TCFFT_SPLIT_FP32) return ret(TCFFT_UNSUPPORTED);
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
  tcfftStatus s = TCFFT_OK;
  if (p->dims == 1 && p->log_n1 == 0) {
    const int logL = ilog2ll(p->n);
    PassArgs a = base_args(p, sg, logL, scale);
    a.in = in;
    a.out = out;
    a.total_lines = p->batch;
    a.lines_per_seq = 1;
    a.in_seq_stride = a.out_seq_stride = p->n;
    a.in_elem_stride = a.out_elem_stride = 1;
    s = launch_pass(kPassRow, logL, pick_row_tile(logL, p->batch), sg, a, st);
  } else if (p->dims == 1) {
    const long long n1 = 1ll << p->log_n1, n2 = 1ll << p->log_n2;
    // pass 1: length-n1 FFTs down the columns of [n1][n2], times W_N^{n2*k1}
    PassArgs a = base_args(p, sg, p->log_n1, 1.0f);
    a.in = in;
    a.out = p->ws;
    a.total_lines = p->batch * n2;
    a.lines_per_seq = n2;
    a.in_seq_stride = a.out_seq_stride = p->n;
    a.in_line_stride = a.out_line_stride = 1;
    a.in_elem_stride = a.out_elem_stride = n2;
    a.otw_hi = p->otw_hi[sg];
    a.otw_lo = p->otw_lo[sg];
    a.otw_shift = p->otw_shift;
    a.otw_logn = p->otw_logn;
    s = launch_pass(kPassCol, p->log_n1, kTileBig, sg, a, st);
    if (s == TCFFT_OK) {
      // pass 2: length-n2 FFTs along the rows, row k1 -> X[k1 + n1*k2]
      PassArgs b = base_args(p, sg, p->log_n2, scale);
      b.in = p->ws;
      b.out = out;
      b.total_lines = p->batch * n1;
      b.lines_per_seq = n1;
      b.in_seq_stride = b.out_seq_stride = p->n;
      b.in_line_stride = n2;
      b.in_elem_stride = 1;
      b.out_line_stride = 1;
      b.out_elem_stride = n1;
      s = launch_pass(kPassRowT, p->log_n2, kTileBig, sg, b, st);
    }
  } else {
    const int lx = ilog2ll(p->nx), ly = ilog2ll(p->ny);
    // rows: length ny, contiguous
    PassArgs a = base_args(p, sg, ly, 1.0f);
    a.in = in;
    a.out = out;
    a.total_lines = p->batch * p->nx;
    a.lines_per_seq = 1;
    a.in_seq_stride = a.out_seq_stride = p->ny;
    a.in_elem_stride = a.out_elem_stride = 1;
    s = launch_pass(kPassRow, ly, pick_row_tile(ly, a.total_lines), sg, a, st);
    if (s == TCFFT_OK) {
      // columns: length nx, stride ny, in place
      PassArgs b = base_args(p, sg, lx, scale);
      b.in = out;
      b.out = out;
      b.total_lines = p->batch * p->ny;
      b.lines_per_seq = p->ny;
      b.in_seq_stride = b.out_seq_stride = p->n;
      b.in_line_stride = b.out_line_stride = 1;
      b.in_elem_stride = b.out_elem_stride = p->ny;
      s = launch_pass(kPassCol, lx, kTileBig, sg, b, st);
    }
  }
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

tcfftStatus tcfft_check(tcfftPlan p, void* stream) {
  if (!p) return ret(TCFFT_INVALID_VALUE);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return ret(TCFFT_LAUNCH_FAILED);
  int h = 0;
  if (cudaMemcpy(&h, p->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return ret(TCFFT_LAUNCH_FAILED);
  if (h != 0) {
    cudaMemset(p->err, 0, sizeof(int));
    return ret((h & kErrMmaTimeout) ? TCFFT_TIMEOUT : TCFFT_LAUNCH_FAILED);
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

int tcfft_last_launch_count(void) { return g_last_launches; }

}  // extern "C"
