// 2D DFT of n x n planes whose non-zeros sit in a small top-left box, by
// line projections (the reference's "qdFFT", fftconvolve2d.cu:884-1260,
// kernels fft_utils.cu:161-700).
//
// Method (restated from the reference; n = 2^k):
//   directions d = 0 .. 3n/2 - 1:  (p, s) = (1, d) for d < n,
//                                  (p, s) = (2(d - n), 1) for d >= n
//   projection   v_d[t] = sum of K[x][y] over the box with p x + s y = t (mod n)
//   1D DFT       W_d[k] = sum_t v_d[t] w^(t k) = K^(k p, k s)   (w = e^(-+2 pi i / n))
//   scatter      the 2D spectrum at (k p mod n, k s mod n) is W_d[k].
// The 3n/2 lines through the origin cover every frequency. The reference
// scatters every (d, k) (several land on one frequency); here each frequency
// is gathered from one canonical (d, k), found in closed form from the 2-adic
// valuations of (u, v): a = v2(u) <= b = v2(v) -> d = (v/2^a) (u/2^a)^-1 mod
// n/2^a, k = u; else d = n + q with 2q = (u/2^b) (v/2^b)^-1 mod n/2^b, k = v.
// So the output is deterministic and each element is written once.
//
// Work per plane: box_rows * box_cols * 3n/2 projection adds (shared-memory
// atomics, one CTA per (plane, direction)), 3n/2 transforms of n points (the
// split-precision 1D plan of this library), n^2 gathered elements.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <new>

#include "../../include/tcfft_gb300.h"
#include "capi_internal.cuh"
#include "qd_internal.cuh"

using namespace tcfft;

namespace {

// Inverse of an odd x modulo 2^32 (Newton: each step doubles the correct bits).
__device__ __forceinline__ uint32_t inv_odd(uint32_t x) {
  uint32_t y = x;  // correct to 3 bits: x * x = 1 (mod 8) for odd x
#pragma unroll
  for (int i = 0; i < 4; ++i) y *= 2u - x * y;
  return y;
}

// Canonical (direction, k) holding frequency (u, v) of an n = 2^logn plane.
__device__ __forceinline__ void qd_owner(uint32_t u, uint32_t v, int logn, uint32_t& dir, uint32_t& k) {
  const uint32_t n = 1u << logn;
  if (u == 0 && v == 0) {
    dir = 0;
    k = 0;
    return;
  }
  const int a = u ? __ffs(static_cast<int>(u)) - 1 : logn;
  const int b = v ? __ffs(static_cast<int>(v)) - 1 : logn;
  if (a <= b) {
    const uint32_t mask = (n >> a) - 1u;
    dir = ((v >> a) * inv_odd(u >> a)) & mask;
    k = u;
  } else {
    const uint32_t mask = (n >> b) - 1u;
    const uint32_t two_q = ((u >> b) * inv_odd(v >> b)) & mask;
    dir = n + (two_q >> 1);
    k = v;
  }
}

// Source of the projected values: complex planes [plane][n][n] (float2),
// or real filters packed two per plane (filter 2g real part, 2g + 1
// imaginary part), each [box_rows][box_cols], optionally rotated by 180
// degrees (correlation filters).
struct QdSrcPlanes {
  const float2* planes;
  __device__ __forceinline__ float2 at(long long g, int x, int y, int n, int, int) const {
    return planes[(g * n + x) * static_cast<long long>(n) + y];
  }
};
struct QdSrcPairs {
  const float* filt;
  long long count;
  int flip;
  __device__ __forceinline__ float2 at(long long g, int x, int y, int, int br, int bc) const {
    const int xx = flip ? br - 1 - x : x, yy = flip ? bc - 1 - y : y;
    const long long i0 = 2 * g, i1 = 2 * g + 1;
    const long long per = static_cast<long long>(br) * bc;
    const float re = filt[i0 * per + static_cast<long long>(xx) * bc + yy];
    const float im = i1 < count ? filt[i1 * per + static_cast<long long>(xx) * bc + yy] : 0.f;
    return make_float2(re, im);
  }
};

// One CTA per (plane g, direction d): v_d[t] accumulated in shared memory,
// then written to proj[g][d][0..n).
template <class Src>
__global__ void qd_project_kernel(Src src, float2* __restrict__ proj, int logn, int br, int bc) {
  extern __shared__ float2 v[];
  const int n = 1 << logn;
  const int ndir = n + n / 2;
  const long long g = blockIdx.x / ndir;
  const int d = static_cast<int>(blockIdx.x % ndir);
  const uint32_t p = d < n ? 1u : 2u * static_cast<uint32_t>(d - n);
  const uint32_t s = d < n ? static_cast<uint32_t>(d) : 1u;
  for (int t = threadIdx.x; t < n; t += blockDim.x) v[t] = make_float2(0.f, 0.f);
  __syncthreads();
  const int cnt = br * bc;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int x = e / bc, y = e % bc;
    const float2 val = src.at(g, x, y, n, br, bc);
    const uint32_t t = (p * static_cast<uint32_t>(x) + s * static_cast<uint32_t>(y)) & static_cast<uint32_t>(n - 1);
    atomicAdd(&v[t].x, val.x);
    atomicAdd(&v[t].y, val.y);
  }
  __syncthreads();
  float2* dst = proj + (g * ndir + d) * static_cast<long long>(n);
  for (int t = threadIdx.x; t < n; t += blockDim.x) dst[t] = v[t];
}

// out[g][u][v] = W_g[dir(u, v)][k(u, v)] (complex float planes)
__global__ void qd_gather_kernel(const float2* __restrict__ w, float2* __restrict__ out, long long planes,
                                 int logn) {
  const long long n = 1ll << logn;
  const long long plane = n * n, ndir = n + n / 2;
  const long long total = planes * plane;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long g = i / plane;
    const uint32_t u = static_cast<uint32_t>((i % plane) >> logn), vv = static_cast<uint32_t>(i & (n - 1));
    uint32_t dir, k;
    qd_owner(u, vv, logn, dir, k);
    out[i] = w[(g * ndir + dir) * n + k];
  }
}

template <class E>
__device__ __forceinline__ E qd_elem(float2 v);
template <>
__device__ __forceinline__ float2 qd_elem<float2>(float2 v) {
  return v;
}
template <>
__device__ __forceinline__ half2 qd_elem<half2>(float2 v) {
  return __floats2half2_rn(v.x, v.y);
}

// Spectra of real filters from their paired planes Z = X_2g + i X_2g+1:
// X_2g(k) = (Z(k) + conj Z(-k)) / 2, X_2g+1(k) = (Z(k) - conj Z(-k)) / (2i);
// out[c][u][v] for c < count.
template <class E>
__global__ void qd_gather_pairs_kernel(const float2* __restrict__ w, E* __restrict__ out, long long count,
                                       int logn) {
  const long long n = 1ll << logn;
  const long long plane = n * n, ndir = n + n / 2;
  const long long total = count * plane;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long c = i / plane;
    const long long g = c >> 1;
    const uint32_t u = static_cast<uint32_t>((i % plane) >> logn), vv = static_cast<uint32_t>(i & (n - 1));
    const uint32_t um = static_cast<uint32_t>((n - u) & (n - 1)), vm = static_cast<uint32_t>((n - vv) & (n - 1));
    uint32_t d0, k0, d1, k1;
    qd_owner(u, vv, logn, d0, k0);
    qd_owner(um, vm, logn, d1, k1);
    const float2 z = w[(g * ndir + d0) * n + k0];
    const float2 zm = w[(g * ndir + d1) * n + k1];
    const float2 x = (c & 1) ? make_float2(0.5f * (z.y + zm.y), 0.5f * (zm.x - z.x))
                             : make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
    out[i] = qd_elem<E>(x);
  }
}

unsigned qd_grid(long long total) {
  long long g = (total + 255) / 256;
  if (g > 65536) g = 65536;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

int ilog2q(long long v) {
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

}  // namespace

struct tcfftQdImpl {
  int n = 0, logn = 0, br = 0, bc = 0;
  long long planes = 0;
  float2* proj = nullptr;  // [planes][3n/2][n], transformed in place
  tcfftPlan fft = nullptr;
};

namespace tcfft {

tcfftStatus qd_create(tcfftQdImpl** out, int n, long long planes, int box_rows, int box_cols) {
  *out = nullptr;
  if (n < 16 || n > 4096 || (n & (n - 1)) != 0 || planes < 1) return TCFFT_INVALID_SIZE;
  if (box_rows < 1 || box_cols < 1 || box_rows > n || box_cols > n) return TCFFT_INVALID_SIZE;
  tcfftQdImpl* q = new (std::nothrow) tcfftQdImpl();
  if (!q) return TCFFT_ALLOC_FAILED;
  q->n = n;
  q->logn = ilog2q(n);
  q->br = box_rows;
  q->bc = box_cols;
  q->planes = planes;
  const long long lines = planes * (n + n / 2);
  tcfftStatus s = TCFFT_OK;
  if (cudaMalloc(&q->proj, sizeof(float2) * static_cast<size_t>(lines) * n) != cudaSuccess) s = TCFFT_ALLOC_FAILED;
  if (s == TCFFT_OK) s = tcfft_plan_1d(&q->fft, n, lines, TCFFT_SPLIT_FP32);
  if (s != TCFFT_OK) {
    qd_free(q);
    return s;
  }
  *out = q;
  return TCFFT_OK;
}

void qd_free(tcfftQdImpl* q) {
  if (!q) return;
  cudaFree(q->proj);
  if (q->fft) tcfft_destroy(q->fft);
  delete q;
}

tcfftStatus qd_check(tcfftQdImpl* q, cudaStream_t st) { return tcfft_check(q->fft, st); }

template <class Src>
static tcfftStatus qd_project_and_transform(tcfftQdImpl* q, const Src& src, int direction, cudaStream_t st) {
  const long long ndir = q->n + q->n / 2;
  const long long blocks = q->planes * ndir;
  if (blocks > 0x7fffffffll) return TCFFT_CAPACITY;
  qd_project_kernel<Src><<<static_cast<unsigned>(blocks), 256, sizeof(float2) * q->n, st>>>(src, q->proj, q->logn,
                                                                                             q->br, q->bc);
  if (cudaGetLastError() != cudaSuccess) return TCFFT_LAUNCH_FAILED;
  return tcfft_exec(q->fft, q->proj, q->proj, direction, 1.0f, st);
}

tcfftStatus qd_exec_planes(tcfftQdImpl* q, const float2* planes, float2* out, int direction, cudaStream_t st) {
  QdSrcPlanes src{planes};
  tcfftStatus s = qd_project_and_transform(q, src, direction, st);
  if (s != TCFFT_OK) return s;
  const long long total = q->planes * q->n * static_cast<long long>(q->n);
  qd_gather_kernel<<<qd_grid(total), 256, 0, st>>>(q->proj, out, q->planes, q->logn);
  return cudaGetLastError() == cudaSuccess ? TCFFT_OK : TCFFT_LAUNCH_FAILED;
}

template <class E>
tcfftStatus qd_exec_filter_pairs(tcfftQdImpl* q, const float* filters, long long count, int flip, E* out,
                                 int direction, cudaStream_t st) {
  if ((count + 1) / 2 > q->planes) return TCFFT_CAPACITY;
  QdSrcPairs src{filters, count, flip};
  tcfftStatus s = qd_project_and_transform(q, src, direction, st);
  if (s != TCFFT_OK) return s;
  const long long total = count * q->n * static_cast<long long>(q->n);
  qd_gather_pairs_kernel<E><<<qd_grid(total), 256, 0, st>>>(q->proj, out, count, q->logn);
  return cudaGetLastError() == cudaSuccess ? TCFFT_OK : TCFFT_LAUNCH_FAILED;
}

tcfftStatus qd_exec_pairs_packed(tcfftQdImpl* q, const float* filters, long long count, float2* out, int direction,
                                 cudaStream_t st) {
  if ((count + 1) / 2 > q->planes) return TCFFT_CAPACITY;
  QdSrcPairs src{filters, count, 0};
  tcfftStatus s = qd_project_and_transform(q, src, direction, st);
  if (s != TCFFT_OK) return s;
  const long long planes = (count + 1) / 2;
  const long long total = planes * q->n * static_cast<long long>(q->n);
  qd_gather_kernel<<<qd_grid(total), 256, 0, st>>>(q->proj, out, planes, q->logn);
  return cudaGetLastError() == cudaSuccess ? TCFFT_OK : TCFFT_LAUNCH_FAILED;
}

template tcfftStatus qd_exec_filter_pairs<half2>(tcfftQdImpl*, const float*, long long, int, half2*, int,
                                                 cudaStream_t);
template tcfftStatus qd_exec_filter_pairs<float2>(tcfftQdImpl*, const float*, long long, int, float2*, int,
                                                  cudaStream_t);

}  // namespace tcfft

extern "C" {

tcfftStatus tcfft_qd_plan(tcfftQd* qd, int n, long long planes, int box_rows, int box_cols) {
  if (!qd) return record_status(TCFFT_INVALID_VALUE, 0);
  tcfftStatus s = registry_ready();
  if (s != TCFFT_OK) return record_status(s, 0);
  tcfftQdImpl* q = nullptr;
  s = qd_create(&q, n, planes, box_rows, box_cols);
  *qd = q;
  return record_status(s, 0);
}

tcfftStatus tcfft_qd_exec(tcfftQd qd, const void* planes, void* out, int direction, void* stream) {
  if (!qd || !planes || !out) return record_status(TCFFT_INVALID_VALUE, 0);
  if (direction != TCFFT_FORWARD && direction != TCFFT_INVERSE) return record_status(TCFFT_INVALID_VALUE, 0);
  if (planes == out) return record_status(TCFFT_INVALID_VALUE, 0);
  const tcfftStatus s = qd_exec_planes(qd, static_cast<const float2*>(planes), static_cast<float2*>(out), direction,
                                       static_cast<cudaStream_t>(stream));
  // projection + gather, and the 1D transform's own launches
  return record_status(s, s == TCFFT_OK ? 2 + tcfft_last_launch_count() : 0);
}

tcfftStatus tcfft_qd_check(tcfftQd qd, void* stream) {
  if (!qd) return record_status(TCFFT_INVALID_VALUE, 0);
  return record_status(qd_check(qd, static_cast<cudaStream_t>(stream)), 0);
}

tcfftStatus tcfft_qd_destroy(tcfftQd qd) {
  if (!qd) return record_status(TCFFT_INVALID_VALUE, 0);
  qd_free(qd);
  return record_status(TCFFT_OK, 0);
}

}  // extern "C"
