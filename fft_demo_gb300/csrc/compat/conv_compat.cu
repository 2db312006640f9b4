// Reference-signature shims for tensorcore_fft_conv2d.h (class
// fft_conv2d_half) and include/fftconvolve2d.cuh, implemented on the C ABI.
// See include/compat/tensorcore_fft_conv2d.h and fftconvolve2d.cuh for the
// contract each entry point keeps.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../../include/compat/fftconvolve2d.cuh"
#include "../../../include/compat/tensorcore_fft_conv2d.h"
#include "../../../include/tcfft_gb300.h"
#include "../capi_internal.cuh"
#include "../qd_internal.cuh"

namespace {

std::vector<int> digit_rev(int n, const int* radices, int nr) {
  std::vector<int> rev(static_cast<size_t>(n));
  for (int idx = 0; idx < n; ++idx) {
    int rest = idx, pos = 0, span = n;
    for (int i = nr - 1; i >= 0; --i) {
      const int r = radices[i];
      const int d = rest % r;
      rest /= r;
      span /= r;
      pos += d * span;
    }
    rev[static_cast<size_t>(pos)] = idx;
  }
  return rev;
}

// Radix list of one axis, as TensorCoreFFTCreate's switch sets it
// (tensorcore_fft_conv2d_kernel.cu:1584-1625).
void conv_axis(int n, int* n_radices, int* radices, int* merging) {
  switch (n) {
    case 256: *n_radices = 2; break;
    case 512:
      *n_radices = 3;
      *merging = 1;
      break;
    case 1024:
      *n_radices = 3;
      radices[2] = 4;
      *merging = 2;
      break;
    default: *n_radices = 0; break;
  }
}

template <class T>
T* dev_alloc(size_t count) {
  T* p = nullptr;
  if (cudaMalloc(&p, sizeof(T) * count) != cudaSuccess) return nullptr;
  return p;
}

__global__ void double_to_half_kernel(const double* __restrict__ src, __half* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    dst[i] = __double2half(src[i]);
}
__global__ void half_to_double_kernel(const __half* __restrict__ src, double* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    dst[i] = __half2float(src[i]);
}
__global__ void double_to_float_kernel(const double* __restrict__ src, float* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    dst[i] = static_cast<float>(src[i]);
}
__global__ void float_to_double_kernel(const float* __restrict__ src, double* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    dst[i] = src[i];
}
// dst[b][line][ele] = src[b][rev_y[line]][rev_x[ele]] (complex FP64 -> half2)
__global__ void rev_complex_kernel(const double* __restrict__ src, __half* __restrict__ dst, const int* rev_x,
                                   const int* rev_y, int x, int y, long long total) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long tile = static_cast<long long>(x) * y;
    const long long b = i / tile;
    const int line = static_cast<int>((i % tile) / x), ele = static_cast<int>(i % x);
    const long long s = b * tile + static_cast<long long>(rev_y[line]) * x + rev_x[ele];
    dst[2 * i] = __double2half(src[2 * s]);
    dst[2 * i + 1] = __double2half(src[2 * s + 1]);
  }
}
// Crop at (fx-1, fx-1), real part, scale (read_out_scale_* of the reference).
template <class S>
__global__ void read_out_kernel(const S* __restrict__ src, double* __restrict__ dst, int src_x, int src_y,
                                int dst_x, int dst_y, int off, double scale, long long total) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long tile = static_cast<long long>(dst_x) * dst_y;
    const long long b = i / tile;
    const int yy = static_cast<int>((i % tile) / dst_x), xx = static_cast<int>(i % dst_x);
    const long long s = b * static_cast<long long>(src_x) * src_y + static_cast<long long>(yy + off) * src_x + xx + off;
    dst[i] = static_cast<double>(static_cast<float>(src[2 * s])) * scale;
  }
}

unsigned grid_for(long long n) {
  long long g = (n + 255) / 256;
  return static_cast<unsigned>(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

tcfftConv conv_of(void* p) { return static_cast<tcfftConv>(p); }

// valid-correlation plan (FP16) for the object's shapes, filters uploaded
int make_forward_plan(fft_conv2d_half* o) {
  if (o->native_conv) {
    tcfft_conv2d_destroy(conv_of(o->native_conv));
    o->native_conv = nullptr;
  }
  tcfftConv c = nullptr;
  int st = tcfft_conv2d_plan(&c, o->S, o->F, o->sy, o->sx, o->fy, o->fx, TCFFT_CONV_VALID_CORR, TCFFT_FP16, 1);
  if (st != TCFFT_OK) return st;
  o->native_conv = c;
  int oy = 0, ox = 0, P = 0;
  tcfft_conv2d_shape(c, &oy, &ox, &P);
  o->padded_x = o->padded_y = P;
  const long long nf = static_cast<long long>(o->F) * o->S * o->fy * o->fx;
  double* dd = dev_alloc<double>(static_cast<size_t>(nf));
  float* df = dev_alloc<float>(static_cast<size_t>(nf));
  if (!dd || !df) {
    cudaFree(dd);
    cudaFree(df);
    return TCFFT_ALLOC_FAILED;
  }
  cudaMemcpy(dd, o->filter, sizeof(double) * nf, cudaMemcpyHostToDevice);
  double_to_float_kernel<<<grid_for(nf), 256>>>(dd, df, nf);
  st = tcfft_conv2d_set_filters(c, df, nullptr);
  cudaDeviceSynchronize();
  cudaFree(dd);
  cudaFree(df);
  return st;
}

// real FP64 host images -> conv -> FP64 host output, through FP16 / FP32 device buffers
int run_conv_host(tcfftConv c, int precision, const double* images, long long n_in, double* out, long long n_out) {
  double* dd = dev_alloc<double>(static_cast<size_t>(n_in > n_out ? n_in : n_out));
  void* din = nullptr;
  void* dout = nullptr;
  const size_t es = precision == TCFFT_FP16 ? 2 : 4;
  cudaMalloc(&din, es * n_in);
  cudaMalloc(&dout, es * n_out);
  int st = (!dd || !din || !dout) ? TCFFT_ALLOC_FAILED : TCFFT_OK;
  if (st == TCFFT_OK) {
    cudaMemcpy(dd, images, sizeof(double) * n_in, cudaMemcpyHostToDevice);
    if (precision == TCFFT_FP16)
      double_to_half_kernel<<<grid_for(n_in), 256>>>(dd, static_cast<__half*>(din), n_in);
    else
      double_to_float_kernel<<<grid_for(n_in), 256>>>(dd, static_cast<float*>(din), n_in);
    st = tcfft_conv2d_exec(c, din, dout, 1, nullptr);
    if (st == TCFFT_OK) st = tcfft_conv2d_check(c, nullptr);
    if (st == TCFFT_OK) {
      if (precision == TCFFT_FP16)
        half_to_double_kernel<<<grid_for(n_out), 256>>>(static_cast<__half*>(dout), dd, n_out);
      else
        float_to_double_kernel<<<grid_for(n_out), 256>>>(static_cast<float*>(dout), dd, n_out);
      cudaMemcpy(out, dd, sizeof(double) * n_out, cudaMemcpyDeviceToHost);
    }
  }
  cudaFree(dd);
  cudaFree(din);
  cudaFree(dout);
  return st;
}

}  // namespace

// ----------------------------------------------------------------------------
// fft_conv2d_half
// ----------------------------------------------------------------------------
fft_conv2d_half::fft_conv2d_half()
    : GPU(__AMPERE__), sx(0), sy(0), fx(0), fy(0), S(0), F(0), padded_x(0), padded_y(0), output_x(0), output_y(0),
      signal(nullptr), filter(nullptr), cu_signal(nullptr), cu_filter(nullptr), cu_signal_padded(nullptr),
      cu_filter_padded(nullptr), rev_x_cu(nullptr), rev_y_cu(nullptr), output(nullptr), cu_pointwise_float(nullptr),
      cu_pointwise_half(nullptr), max_per_line(nullptr), max_per_tile(nullptr),
      cu_conv2d_forward_result_padded(nullptr), cu_delta_in(nullptr), cu_delta_in_padded(nullptr),
      cu_pointwise_for_delta_filter(nullptr), cu_pointwise_for_delta_signal(nullptr), delta_weight_double(nullptr),
      delta_for_filter(nullptr), delta_for_signal(nullptr) {
  std::memset(rev_256, 0, sizeof(rev_256));
  std::memset(rev_512, 0, sizeof(rev_512));
}

fft_conv2d_half::fft_conv2d_half(int in_channel, int out_channel, int kernel_size, __GPU_ARCH__ gpu)
    : fft_conv2d_half() {
  S = in_channel;
  F = out_channel;
  fx = fy = kernel_size;
  GPU = gpu;
}

fft_conv2d_half::fft_conv2d_half(double* sig, double* filt, int S_, int F_, int sy_, int sx_, int fy_, int fx_,
                                 __GPU_ARCH__ gpu)
    : fft_conv2d_half() {
  signal = sig;
  filter = filt;
  S = S_;
  F = F_;
  sy = sy_;
  sx = sx_;
  fy = fy_;
  fx = fx_;
  GPU = gpu;
  output_x = sx - fx + 1;
  output_y = sy - fy + 1;
  last_status = make_forward_plan(this);
  gen_rev(padded_x, padded_y);
}

fft_conv2d_half::~fft_conv2d_half() {
  if (native_conv) tcfft_conv2d_destroy(conv_of(native_conv));
  native_conv = nullptr;
  cudaFree(rev_x_cu);
  cudaFree(rev_y_cu);
}

void fft_conv2d_half::conv2d_forward(double* out) {
  output = out;
  if (!native_conv) {
    last_status = TCFFT_INVALID_VALUE;
    return;
  }
  last_status = run_conv_host(conv_of(native_conv), TCFFT_FP16, signal, static_cast<long long>(S) * sy * sx, out,
                              static_cast<long long>(F) * output_y * output_x);
}

void fft_conv2d_half::conv2d_forward(double* input, double* weight, double* out, int S_, int F_, int sy_, int sx_,
                                     int fy_, int fx_, __GPU_ARCH__ gpu) {
  signal = input;
  filter = weight;
  S = S_;
  F = F_;
  sy = sy_;
  sx = sx_;
  fy = fy_;
  fx = fx_;
  GPU = gpu;
  output_x = sx - fx + 1;
  output_y = sy - fy + 1;
  last_status = make_forward_plan(this);
  if (last_status == TCFFT_OK) conv2d_forward(out);
}

void fft_conv2d_half::TENSORCORE_FFT_CONV_2D() {
  if (!output) {
    last_status = TCFFT_INVALID_VALUE;
    return;
  }
  conv2d_forward(output);
}

// The reference's constructor pads, flips and transforms the filters here
// (kernel.cu:1255); the equivalent is rebuilding the plan and its resident
// filter spectra from `filter`.
void fft_conv2d_half::fft_conv2d_inv_rev_pad() {
  if (!filter || S < 1 || F < 1) {
    last_status = TCFFT_INVALID_VALUE;
    return;
  }
  last_status = make_forward_plan(this);
}

// readout_fwd copies the cropped, scaled result to `output` (.cpp:275).
// TENSORCORE_FFT_CONV_2D already wrote `output`, so after a successful one
// there is nothing left to do; on its own it has no result to read.
void fft_conv2d_half::readout_fwd(bool) {
  if (!output || last_status != TCFFT_OK) last_status = TCFFT_UNSUPPORTED;
}

// The reference's intermediate forward steps (kernel.cu:1101,1141) leave
// FP32 / FP16 pointwise planes in cu_pointwise_float / cu_pointwise_half.
// Here the pointwise product and the inverse transform are stages of one
// pipeline that keeps those planes inside the plan, so the steps cannot run
// on their own: they report TCFFT_UNSUPPORTED instead of silently doing
// nothing.
void fft_conv2d_half::fft_pointwise(float, bool) { last_status = TCFFT_UNSUPPORTED; }
void fft_conv2d_half::fft_conv_final_stage() { last_status = TCFFT_UNSUPPORTED; }

// Gradients of out[f] = sum_s corr(x_s, w_fs) (valid):
//   dW[f][s] = corr(x_s, delta_f) (valid, size fy x fx)
//   dX[s]    = sum_f full_conv(delta_f, w_fs)   (size sy x sx)
// computed with split-precision plans; results malloc'ed like the reference.
void fft_conv2d_half::conv2d_backward(double* delta_in) {
  const int oy = output_y, ox = output_x;
  // dW: images = the S input channels (batch), filters = the F deltas
  {
    tcfftConv c = nullptr;
    last_status = tcfft_conv2d_plan(&c, 1, F, sy, sx, oy, ox, TCFFT_CONV_VALID_CORR, TCFFT_SPLIT_FP32, S);
    if (last_status != TCFFT_OK) return;
    const long long nd = static_cast<long long>(F) * oy * ox;
    double* dd = dev_alloc<double>(static_cast<size_t>(nd));
    float* df = dev_alloc<float>(static_cast<size_t>(nd));
    cudaMemcpy(dd, delta_in, sizeof(double) * nd, cudaMemcpyHostToDevice);
    double_to_float_kernel<<<grid_for(nd), 256>>>(dd, df, nd);
    tcfft_conv2d_set_filters(c, df, nullptr);
    cudaDeviceSynchronize();
    cudaFree(dd);
    cudaFree(df);
    // exec over the S channels as a batch: out [S][F][fy][fx]
    const long long nin = static_cast<long long>(S) * sy * sx, nout = static_cast<long long>(S) * F * fy * fx;
    std::vector<double> tmp(static_cast<size_t>(nout));
    double* din = dev_alloc<double>(static_cast<size_t>(nin > nout ? nin : nout));
    float* fin = dev_alloc<float>(static_cast<size_t>(nin));
    float* fout = dev_alloc<float>(static_cast<size_t>(nout));
    cudaMemcpy(din, signal, sizeof(double) * nin, cudaMemcpyHostToDevice);
    double_to_float_kernel<<<grid_for(nin), 256>>>(din, fin, nin);
    last_status = tcfft_conv2d_exec(c, fin, fout, S, nullptr);
    if (last_status == TCFFT_OK) last_status = tcfft_conv2d_check(c, nullptr);
    float_to_double_kernel<<<grid_for(nout), 256>>>(fout, din, nout);
    cudaMemcpy(tmp.data(), din, sizeof(double) * nout, cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(fin);
    cudaFree(fout);
    tcfft_conv2d_destroy(c);
    delta_for_filter = static_cast<double*>(malloc(sizeof(double) * nout));
    for (int f = 0; f < F; ++f)
      for (int s = 0; s < S; ++s)
        std::memcpy(delta_for_filter + (static_cast<size_t>(f) * S + s) * fy * fx,
                    tmp.data() + (static_cast<size_t>(s) * F + f) * fy * fx, sizeof(double) * fy * fx);
  }
  // dX: images = the F deltas as channels, filters [S][F][fy][fx] = w transposed
  {
    tcfftConv c = nullptr;
    last_status = tcfft_conv2d_plan(&c, F, S, oy, ox, fy, fx, TCFFT_CONV_FULL, TCFFT_SPLIT_FP32, 1);
    if (last_status != TCFFT_OK) return;
    const long long nw = static_cast<long long>(F) * S * fy * fx;
    std::vector<double> wt(static_cast<size_t>(nw));
    for (int f = 0; f < F; ++f)
      for (int s = 0; s < S; ++s)
        std::memcpy(wt.data() + (static_cast<size_t>(s) * F + f) * fy * fx,
                    filter + (static_cast<size_t>(f) * S + s) * fy * fx, sizeof(double) * fy * fx);
    double* dd = dev_alloc<double>(static_cast<size_t>(nw));
    float* df = dev_alloc<float>(static_cast<size_t>(nw));
    cudaMemcpy(dd, wt.data(), sizeof(double) * nw, cudaMemcpyHostToDevice);
    double_to_float_kernel<<<grid_for(nw), 256>>>(dd, df, nw);
    tcfft_conv2d_set_filters(c, df, nullptr);
    cudaDeviceSynchronize();
    cudaFree(dd);
    cudaFree(df);
    delta_for_signal = static_cast<double*>(malloc(sizeof(double) * S * sy * sx));
    last_status = run_conv_host(c, TCFFT_SPLIT_FP32, delta_in, static_cast<long long>(F) * oy * ox,
                                delta_for_signal, static_cast<long long>(S) * sy * sx);
    tcfft_conv2d_destroy(c);
  }
}

// The reference's intermediate backward steps (kernel.cu:1153,1177,1189,1211,
// 1314) fill padded FP16 planes that conv2d_backward consumes; here both
// gradients come out of conv2d_backward's own plans, so the steps cannot run
// on their own and report TCFFT_UNSUPPORTED.
void fft_conv2d_half::fft_conv2d_rev_pad(double*, double*, half*, half*, int, int, int, int, int) {
  last_status = TCFFT_UNSUPPORTED;
}
void fft_conv2d_half::inv_pad_deltain_signal(int) { last_status = TCFFT_UNSUPPORTED; }
void fft_conv2d_half::pad_fx_1_circles_of_0(double*, int, int, int) { last_status = TCFFT_UNSUPPORTED; }
void fft_conv2d_half::pointwise_for_delta_weight(int) { last_status = TCFFT_UNSUPPORTED; }
void fft_conv2d_half::pointwise_for_delta_input(int, half*) { last_status = TCFFT_UNSUPPORTED; }

void fft_conv2d_half::gen_rev(int Nx, int Ny) {
  const int r256[2] = {16, 16};
  const int r512[3] = {16, 16, 2};
  const std::vector<int> a = digit_rev(256, r256, 2), b = digit_rev(512, r512, 3);
  for (int i = 0; i < 256; ++i) rev_256[i] = a[i];
  for (int i = 0; i < 512; ++i) rev_512[i] = b[i];
  if (!rev_x_cu) cudaMalloc(&rev_x_cu, sizeof(int) * 1024);
  if (!rev_y_cu) cudaMalloc(&rev_y_cu, sizeof(int) * 1024);
  const int* tx = Nx == 512 ? rev_512 : rev_256;
  const int* ty = Ny == 512 ? rev_512 : rev_256;
  if (rev_x_cu) cudaMemcpy(rev_x_cu, tx, sizeof(int) * 1024, cudaMemcpyHostToDevice);
  if (rev_y_cu) cudaMemcpy(rev_y_cu, ty, sizeof(int) * 1024, cudaMemcpyHostToDevice);
}

void fft_conv2d_half::rev(double* src, half* dst, int x, int y, int batch, int, cudaStream_t stream) {
  int nx = 0, ny = 0, rx[3] = {16, 16, 2}, ry[3] = {16, 16, 2}, m = 0;
  conv_axis(x, &nx, rx, &m);
  conv_axis(y, &ny, ry, &m);
  const std::vector<int> vx = nx ? digit_rev(x, rx, nx) : std::vector<int>();
  const std::vector<int> vy = ny ? digit_rev(y, ry, ny) : std::vector<int>();
  std::vector<int> hx(static_cast<size_t>(x)), hy(static_cast<size_t>(y));
  for (int i = 0; i < x; ++i) hx[i] = nx ? vx[i] : i;
  for (int i = 0; i < y; ++i) hy[i] = ny ? vy[i] : i;
  int* dx = dev_alloc<int>(static_cast<size_t>(x));
  int* dy = dev_alloc<int>(static_cast<size_t>(y));
  cudaMemcpyAsync(dx, hx.data(), sizeof(int) * x, cudaMemcpyHostToDevice, stream);
  cudaMemcpyAsync(dy, hy.data(), sizeof(int) * y, cudaMemcpyHostToDevice, stream);
  const long long total = static_cast<long long>(x) * y * batch;
  rev_complex_kernel<<<grid_for(total), 256, 0, stream>>>(src, reinterpret_cast<__half*>(dst), dx, dy, x, y, total);
  cudaStreamSynchronize(stream);
  cudaFree(dx);
  cudaFree(dy);
}

void fft_conv2d_half::TensorCoreFFTCreate(fftPlan* plan, int nx, int ny, int n_batch, int fft, __GPU_ARCH__ gpu) {
  plan->GPU = gpu;
  plan->Nx = nx;
  plan->Ny = ny;
  plan->N_batch = n_batch;
  plan->fft = fft;
  for (int i = 0; i < 3; ++i) {
    plan->layer_0[i] = nullptr;
    plan->layer_1[i] = nullptr;
  }
  plan->F_real = plan->F_imag = nullptr;
  plan->F_imag_tmp = nullptr;
  conv_axis(nx, &plan->n_radices_x, plan->radices_x, &plan->mergings[1]);
  conv_axis(ny, &plan->n_radices_y, plan->radices_y, &plan->mergings[0]);
  tcfftPlan native = nullptr;
  last_status = tcfft_plan_2d(&native, nx, ny, n_batch, TCFFT_FP16);
  plan->F_real_tmp = reinterpret_cast<half*>(native);
}

void fft_conv2d_half::TensorCoreFFTExec(fftPlan plan, half* data, cudaStream_t stream) {
  tcfftPlan native = reinterpret_cast<tcfftPlan>(plan.F_real_tmp);
  if (!native) {
    last_status = TCFFT_INVALID_VALUE;
    return;
  }
  last_status = tcfft_exec_digitrev_2d(native, data, data, plan.radices_x, plan.n_radices_x, plan.radices_y,
                                       plan.n_radices_y, plan.fft == 1 ? TCFFT_FORWARD : TCFFT_INVERSE, stream);
}

void fft_conv2d_half::TensorCoreFFTExec(fftPlan plan, half* data) { TensorCoreFFTExec(plan, data, nullptr); }

void fft_conv2d_half::TensorCoreFFTDestroy(fftPlan* plan) {
  if (plan && plan->F_real_tmp) {
    tcfft_destroy(reinterpret_cast<tcfftPlan>(plan->F_real_tmp));
    plan->F_real_tmp = nullptr;
  }
}

void fft_conv2d_half::read_out_scale_half2double(half* src, double* dst, double* dst_in_host, int src_x, int src_y,
                                                 int dst_x, int dst_y, int batch, double scale) {
  const long long total = static_cast<long long>(dst_x) * dst_y * batch;
  read_out_kernel<__half><<<grid_for(total), 256>>>(reinterpret_cast<const __half*>(src), dst, src_x, src_y, dst_x,
                                                     dst_y, fx - 1, scale, total);
  cudaMemcpy(dst_in_host, dst, sizeof(double) * total, cudaMemcpyDeviceToHost);
}

void fft_conv2d_half::read_out_scale_double2double(double* src, double* dst, double* dst_in_host, int src_x,
                                                   int src_y, int dst_x, int dst_y, int batch, double scale) {
  const long long total = static_cast<long long>(dst_x) * dst_y * batch;
  read_out_kernel<double><<<grid_for(total), 256>>>(src, dst, src_x, src_y, dst_x, dst_y, fx - 1, scale, total);
  cudaMemcpy(dst_in_host, dst, sizeof(double) * total, cudaMemcpyDeviceToHost);
}

void fft_conv2d_half::half2double(half* src, double* dst, int x, int y, int item_per_group, int batch,
                                  cudaStream_t stream) {
  const long long n = static_cast<long long>(x) * y * item_per_group * batch;
  half_to_double_kernel<<<grid_for(n), 256, 0, stream>>>(reinterpret_cast<const __half*>(src), dst, n);
}

void fft_conv2d_half::double2half(double* src, half* dst, int x, int y, int item_per_group, int batch) {
  const long long n = static_cast<long long>(x) * y * item_per_group * batch;
  double_to_half_kernel<<<grid_for(n), 256>>>(src, reinterpret_cast<__half*>(dst), n);
}

namespace {
// Host FP64 in and out (the reference's fft_2d_c2c / ifft_2d_c2c contract,
// .cpp:79,147): the batch goes in up to 8 sub-batches (the reference's 8
// streams) over up to 4 streams, each with its own device buffers and plans,
// so one sub-batch's copies overlap another's conversion and transform. The
// caller's host buffers are page-locked for the call (cudaHostRegister)
// unless they already are, so the asynchronous copies run concurrently; if
// that fails the copies still run, without the overlap.
void fft_2d_host(fft_conv2d_half* o, double* input, double* output, int x, int y, int batch, int direction) {
  o->last_status = TCFFT_OK;
  if (batch <= 0) return;
  const int nchunks_max = batch < 8 ? batch : 8;
  const int per = (batch + nchunks_max - 1) / nchunks_max;
  const int nchunks = (batch + per - 1) / per;
  const int nst = nchunks < 4 ? nchunks : 4;
  const long long elems = 2ll * x * y;  // doubles per transform
  const size_t bytes = sizeof(double) * static_cast<size_t>(elems) * batch;
  auto pin = [](void* p, size_t n) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost) return false;
    cudaGetLastError();  // an unregistered pointer is not an error here
    if (cudaHostRegister(p, n, cudaHostRegisterDefault) == cudaSuccess) return true;
    cudaGetLastError();
    return false;
  };
  const bool pinned_in = pin(input, bytes);
  const bool pinned_out = output != input && pin(output, bytes);
  cudaStream_t st[4] = {};
  double* dd[4] = {};
  __half* dh[4] = {};
  tcfftPlan plan_full[4] = {}, plan_tail[4] = {};
  const int tail = batch - (nchunks - 1) * per;  // sub-batch size of the last chunk
  tcfftStatus status = TCFFT_OK;
  for (int k = 0; k < nst && status == TCFFT_OK; ++k) {
    if (cudaStreamCreateWithFlags(&st[k], cudaStreamNonBlocking) != cudaSuccess) status = TCFFT_LAUNCH_FAILED;
    dd[k] = dev_alloc<double>(static_cast<size_t>(elems) * per);
    dh[k] = dev_alloc<__half>(static_cast<size_t>(elems) * per);
    if (!dd[k] || !dh[k]) status = TCFFT_ALLOC_FAILED;
    if (status == TCFFT_OK) status = tcfft_plan_2d(&plan_full[k], y, x, per, TCFFT_FP16);
  }
  for (int c = 0; c < nchunks && status == TCFFT_OK; ++c) {
    const int k = c % nst;
    const int nb = c == nchunks - 1 ? tail : per;
    tcfftPlan p = plan_full[k];
    if (nb != per) {
      if (!plan_tail[k]) status = tcfft_plan_2d(&plan_tail[k], y, x, nb, TCFFT_FP16);
      p = plan_tail[k];
    }
    if (status != TCFFT_OK) break;
    const long long n = elems * nb;
    const long long off = elems * static_cast<long long>(c) * per;
    cudaMemcpyAsync(dd[k], input + off, sizeof(double) * n, cudaMemcpyHostToDevice, st[k]);
    double_to_half_kernel<<<grid_for(n), 256, 0, st[k]>>>(dd[k], dh[k], n);
    status = tcfft_exec(p, dh[k], dh[k], direction, 1.0f, st[k]);
    half_to_double_kernel<<<grid_for(n), 256, 0, st[k]>>>(dh[k], dd[k], n);
    cudaMemcpyAsync(output + off, dd[k], sizeof(double) * n, cudaMemcpyDeviceToHost, st[k]);
  }
  for (int k = 0; k < nst; ++k) {
    if (st[k] && cudaStreamSynchronize(st[k]) != cudaSuccess && status == TCFFT_OK) status = TCFFT_LAUNCH_FAILED;
    if (plan_full[k] && status == TCFFT_OK) status = tcfft_check(plan_full[k], st[k]);
    if (plan_tail[k] && status == TCFFT_OK) status = tcfft_check(plan_tail[k], st[k]);
  }
  for (int k = 0; k < nst; ++k) {
    if (plan_full[k]) tcfft_destroy(plan_full[k]);
    if (plan_tail[k]) tcfft_destroy(plan_tail[k]);
    cudaFree(dd[k]);
    cudaFree(dh[k]);
    if (st[k]) cudaStreamDestroy(st[k]);
  }
  if (pinned_in) cudaHostUnregister(input);
  if (pinned_out) cudaHostUnregister(output);
  o->last_status = status;
}
}  // namespace

void fft_conv2d_half::fft_2d_c2c(double* input, double* out, int x, int y, int batch, __GPU_ARCH__, int, bool) {
  fft_2d_host(this, input, out, x, y, batch, TCFFT_FORWARD);
}

void fft_conv2d_half::ifft_2d_c2c(double* input, double* out, int x, int y, int batch, __GPU_ARCH__, int, bool) {
  fft_2d_host(this, input, out, x, y, batch, TCFFT_INVERSE);
}

void fft_conv2d_half::print_cu(half* src, int x, int y, int item_per_group, int batch) {
  const size_t n = static_cast<size_t>(x) * y * item_per_group * batch;
  std::vector<half> h(n);
  cudaMemcpy(h.data(), src, sizeof(half) * n, cudaMemcpyDeviceToHost);
  for (size_t i = 0; i < n; ++i) printf("%f%c", __half2float(h[i]), (i + 1) % (static_cast<size_t>(x) * item_per_group) ? ' ' : '\n');
}
void fft_conv2d_half::print_cu(float* src, int x, int y, int item_per_group, int batch) {
  const size_t n = static_cast<size_t>(x) * y * item_per_group * batch;
  std::vector<float> h(n);
  cudaMemcpy(h.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost);
  for (size_t i = 0; i < n; ++i) printf("%f%c", h[i], (i + 1) % (static_cast<size_t>(x) * item_per_group) ? ' ' : '\n');
}
void fft_conv2d_half::print_cu(double* src, int x, int y, int item_per_group, int batch) {
  const size_t n = static_cast<size_t>(x) * y * item_per_group * batch;
  std::vector<double> h(n);
  cudaMemcpy(h.data(), src, sizeof(double) * n, cudaMemcpyDeviceToHost);
  for (size_t i = 0; i < n; ++i) printf("%f%c", h[i], (i + 1) % (static_cast<size_t>(x) * item_per_group) ? ' ' : '\n');
}
void fft_conv2d_half::printplan(fftPlan plan) {
  printf("fft:%d Nx,Ny,N_batch:%d %d %d n_radices_x,n_radices_y:%d %d mergings:%d %d\n", plan.fft, plan.Nx, plan.Ny,
         plan.N_batch, plan.n_radices_x, plan.n_radices_y, plan.mergings[0], plan.mergings[1]);
}
void fft_conv2d_half::tmp_test() {}
std::string fft_conv2d_half::toString() { return "fft_conv2d_half(tcfft_gb300)"; }

// ----------------------------------------------------------------------------
// fftconvolve2d.cuh family
// ----------------------------------------------------------------------------
namespace {
int full_conv_host(float* Signal, float* Kernels, int kernelCount, int nRows, int nCols, int kRows, int kCols,
                   float* results, bool qd_spectra) {
  tcfftConv c = nullptr;
  int st = tcfft_conv2d_plan(&c, 1, kernelCount, nRows, nCols, kRows, kCols, TCFFT_CONV_FULL, TCFFT_SPLIT_FP32, 1);
  if (st != TCFFT_OK) return st;
  const long long nk = static_cast<long long>(kernelCount) * kRows * kCols, ns = static_cast<long long>(nRows) * nCols;
  const long long no = static_cast<long long>(kernelCount) * (nRows + kRows - 1) * (nCols + kCols - 1);
  float* dk = dev_alloc<float>(static_cast<size_t>(nk));
  float* ds = dev_alloc<float>(static_cast<size_t>(ns));
  float* dout = dev_alloc<float>(static_cast<size_t>(no));
  if (!dk || !ds || !dout) st = TCFFT_ALLOC_FAILED;
  if (st == TCFFT_OK) {
    cudaMemcpy(dk, Kernels, sizeof(float) * nk, cudaMemcpyHostToDevice);
    cudaMemcpy(ds, Signal, sizeof(float) * ns, cudaMemcpyHostToDevice);
    st = qd_spectra ? tcfft_conv2d_set_filters_qd(c, dk, nullptr) : tcfft_conv2d_set_filters(c, dk, nullptr);
    if (st == TCFFT_OK) st = tcfft_conv2d_exec(c, ds, dout, 1, nullptr);
    if (st == TCFFT_OK) st = tcfft_conv2d_check(c, nullptr);
    if (st == TCFFT_OK) cudaMemcpy(results, dout, sizeof(float) * no, cudaMemcpyDeviceToHost);
  }
  cudaFree(dk);
  cudaFree(ds);
  cudaFree(dout);
  tcfft_conv2d_destroy(c);
  return st;
}

// 2D DFT (direction) of pairs of real kernels packed as (re = kernel 2g,
// im = kernel 2g+1), zero-padded to fftRows x fftCols, FP32 (split plan).
int packed_kernel_spectra(float* Kernels, int kernelCount, int fftRows, int fftCols, int kRows, int kCols,
                          cufftComplex* results, int direction, bool device_out) {
  const int groups = kernelCount / 2;
  if (groups < 1) return TCFFT_INVALID_SIZE;
  tcfftPlan p = nullptr;
  int st = tcfft_plan_2d(&p, fftRows, fftCols, groups, TCFFT_SPLIT_FP32);
  if (st != TCFFT_OK) return st;
  const size_t plane = static_cast<size_t>(fftRows) * fftCols;
  std::vector<float> packed(2 * plane * groups, 0.f);
  for (int g = 0; g < groups; ++g)
    for (int y = 0; y < kRows; ++y)
      for (int x = 0; x < kCols; ++x) {
        const size_t d = 2 * (g * plane + static_cast<size_t>(y) * fftCols + x);
        packed[d] = Kernels[(2 * static_cast<size_t>(g)) * kRows * kCols + y * kCols + x];
        packed[d + 1] = Kernels[(2 * static_cast<size_t>(g) + 1) * kRows * kCols + y * kCols + x];
      }
  float* dbuf = dev_alloc<float>(packed.size());
  if (!dbuf) st = TCFFT_ALLOC_FAILED;
  if (st == TCFFT_OK) {
    cudaMemcpy(dbuf, packed.data(), sizeof(float) * packed.size(), cudaMemcpyHostToDevice);
    st = tcfft_exec(p, dbuf, dbuf, direction, 1.0f, nullptr);
    if (st == TCFFT_OK) st = tcfft_check(p, nullptr);
    if (st == TCFFT_OK)
      cudaMemcpy(results, dbuf, sizeof(float) * packed.size(),
                 device_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost);
  }
  cudaFree(dbuf);
  tcfft_destroy(p);
  return st;
}
}  // namespace

// The reference's functions return void; each records its status, which
// tcfft_get_last_error() (include/tcfft_gb300.h) reports.
void convolve_direct_fft(float* Signal, float* Kernels, int kernelCount, int nRows, int nCols, int kRows, int kCols,
                         float* results) {
  tcfft::record_status(
      static_cast<tcfftStatus>(full_conv_host(Signal, Kernels, kernelCount, nRows, nCols, kRows, kCols, results, false)),
      0);
}

void convolve_turbo_fft_v2(float* Signal, float* Kernels, int kernelCount, int nRows, int nCols, int kRows, int kCols,
                           float* results) {
  tcfft::record_status(
      static_cast<tcfftStatus>(full_conv_host(Signal, Kernels, kernelCount, nRows, nCols, kRows, kCols, results, false)),
      0);
}

// turbo v3 = v2 with the filter spectra made by line projections
// (fftconvolve2d.cu:1263-1500, qdVector_construct / fast_fft).
void convolve_turbo_fft_v3(float* Signal, float* Kernels, int kernelCount, int nRows, int nCols, int kRows, int kCols,
                           float* results) {
  tcfft::record_status(
      static_cast<tcfftStatus>(full_conv_host(Signal, Kernels, kernelCount, nRows, nCols, kRows, kCols, results, true)),
      0);
}

void direct_fft(float* Kernels, int kernelCount, int nRows, int nCols, int kRows, int kCols, cufftComplex* results) {
  tcfft::record_status(static_cast<tcfftStatus>(packed_kernel_spectra(Kernels, kernelCount, nRows + kRows - 1,
                                                                      nCols + kCols - 1, kRows, kCols, results,
                                                                      TCFFT_INVERSE, false)),
                       0);
}

// qd_fft (fftconvolve2d.cu:1603): the same spectra as direct_fft, made by line
// projections of the packed kernel pairs (fast_fft with forward = false). The
// projections need a square padded plane (fftRows == fftCols).
void qd_fft(float* Kernels, int kernelCount, int nRows, int nCols, int kRows, int kCols, cufftComplex* results) {
  const int fr = nRows + kRows - 1, fc = nCols + kCols - 1, groups = kernelCount / 2;
  tcfftStatus st = TCFFT_OK;
  if (groups < 1 || fr != fc) st = TCFFT_INVALID_SIZE;
  tcfftQdImpl* q = nullptr;
  if (st == TCFFT_OK) st = tcfft::qd_create(&q, fc, groups, kRows, kCols);
  const long long nk = 2ll * groups * kRows * kCols;
  const size_t nout = static_cast<size_t>(groups) * fr * fc;
  float* dk = st == TCFFT_OK ? dev_alloc<float>(static_cast<size_t>(nk)) : nullptr;
  float2* dout = st == TCFFT_OK ? dev_alloc<float2>(nout) : nullptr;
  if (st == TCFFT_OK && (!dk || !dout)) st = TCFFT_ALLOC_FAILED;
  if (st == TCFFT_OK && cudaMemcpy(dk, Kernels, sizeof(float) * nk, cudaMemcpyHostToDevice) != cudaSuccess)
    st = TCFFT_LAUNCH_FAILED;
  if (st == TCFFT_OK) st = tcfft::qd_exec_pairs_packed(q, dk, 2ll * groups, dout, TCFFT_INVERSE, nullptr);
  if (st == TCFFT_OK) st = tcfft::qd_check(q, nullptr);
  if (st == TCFFT_OK && cudaMemcpy(results, dout, sizeof(float2) * nout, cudaMemcpyDeviceToHost) != cudaSuccess)
    st = TCFFT_LAUNCH_FAILED;
  cudaFree(dk);
  cudaFree(dout);
  tcfft::qd_free(q);
  tcfft::record_status(st, 0);
}

// fast_fft (fftconvolve2d.cu:1011): device planes [group_num][fftRows][fftCols]
// whose non-zeros lie in the top-left kCols x kCols box (the reference's
// sparse projection reads exactly that box), 2D DFT by line projections into
// d_results, forward (true) or inverse sign, unnormalised.
void fast_fft(cufftComplex* d_kernels, int group_num, int fftCols, int fftRows, int kCols, int, cufftComplex* d_results,
              bool forward) {
  tcfftStatus st = TCFFT_OK;
  if (group_num < 1 || fftRows != fftCols || !d_kernels || !d_results) st = TCFFT_INVALID_VALUE;
  tcfftQdImpl* q = nullptr;
  if (st == TCFFT_OK) st = tcfft::qd_create(&q, fftCols, group_num, kCols, kCols);
  if (st == TCFFT_OK)
    st = tcfft::qd_exec_planes(q, reinterpret_cast<const float2*>(d_kernels), reinterpret_cast<float2*>(d_results),
                               forward ? TCFFT_FORWARD : TCFFT_INVERSE, nullptr);
  if (st == TCFFT_OK) st = tcfft::qd_check(q, nullptr);
  tcfft::qd_free(q);
  tcfft::record_status(st, 0);
}
