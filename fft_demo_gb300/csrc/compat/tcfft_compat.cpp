// Reference-signature shims for tcfft_half.h and tcfft_half_2d.h, implemented
// on the C ABI (include/tcfft_gb300.h). See include/compat/*.h for the
// contract each function keeps.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <cstring>
#include <vector>

#include "../../../include/compat/tcfft_half.h"
#include "../../../include/compat/tcfft_half_2d.h"
#include "../../../include/tcfft_gb300.h"

namespace {

thread_local int g_compat_status = TCFFT_OK;

// Radix lists the reference's tcfftCreate assigns (tcfft_half.cu:1250-1330):
// entries of radices[] it overwrites (default 16), n_radices, n_mergings,
// mergings[]. Sizes not listed are left unconfigured (n_radices = 0).
struct Shape1d {
  int n, n_radices, n_mergings;
  int set2, set5, set8;  // value written to radices[2], [5], [8] (0 = untouched)
  int mergings[3];
};
const Shape1d kShapes1d[] = {
    {256, 2, 1, 0, 0, 0, {0, 0, 0}},
    {512, 3, 1, 2, 0, 0, {1, 0, 0}},
    {1024, 3, 1, 4, 0, 0, {2, 0, 0}},
    {131072, 5, 2, 2, 0, 0, {1, 0, 0}},
    {262144, 6, 2, 2, 2, 0, {1, 1, 0}},
    {524288, 6, 2, 4, 2, 0, {2, 1, 0}},
    {16777216, 6, 3, 0, 0, 0, {0, 0, 0}},
    {33554432, 7, 3, 2, 0, 0, {1, 0, 0}},
    {67108864, 8, 3, 2, 2, 0, {1, 1, 0}},
    {134217728, 9, 3, 2, 2, 2, {1, 1, 1}},
};

// Storage position -> natural index for a digit-reversal radix list: the
// permutation the reference's gen_rev builds (tcfft_half.cu:1351), computed
// in closed form (peel the index's digits from the last radix to the first;
// the k-th digit peeled becomes the k-th most significant digit of the
// position; what is left unpeeled keeps its place, so an empty list gives the
// identity, as gen_rev does for sizes tcfftCreate leaves unconfigured).
std::vector<int> digit_reversal(int n, const int* radices, int n_radices) {
  std::vector<int> rev(static_cast<size_t>(n));
  for (int idx = 0; idx < n; ++idx) {
    int rest = idx, pos = 0, span = n;
    for (int i = n_radices - 1; i >= 0; --i) {
      const int r = radices[i];
      const int d = rest % r;
      rest /= r;
      span /= r;
      pos += d * span;
    }
    pos += rest;
    rev[static_cast<size_t>(pos)] = idx;
  }
  return rev;
}

tcfftPlan native_of(const half* slot) { return reinterpret_cast<tcfftPlan>(const_cast<half*>(slot)); }

// setup()/doit()/finalize() state: file-scope, as in tcfft_half.cu:1347-1349.
tcfftHandle g_plan1;
int g_n1 = 0, g_b1 = 0;
half* g_dev1 = nullptr;
std::vector<half> g_host1;

tcfftHandle_2d g_plan2;
int g_nx2 = 0, g_ny2 = 0, g_b2 = 0;
half* g_dev2 = nullptr;
std::vector<half> g_host2;

}  // namespace

void tcfftCreate(tcfftHandle* plan, int n, int n_batch) {
  plan->N = n;
  plan->N_batch = n_batch;
  for (int i = 0; i < 3; ++i) {
    plan->layer_0[i] = nullptr;
    plan->layer_1[i] = nullptr;
  }
  plan->F_real = plan->F_imag = nullptr;
  plan->F_real_tmp = plan->F_imag_tmp = nullptr;
  plan->n_radices = 0;
  plan->n_mergings = 0;
  for (const Shape1d& s : kShapes1d) {
    if (s.n != n) continue;
    plan->n_radices = s.n_radices;
    plan->n_mergings = s.n_mergings;
    if (s.set2) plan->radices[2] = s.set2;
    if (s.set5) plan->radices[5] = s.set5;
    if (s.set8) plan->radices[8] = s.set8;
    for (int i = 0; i < 3; ++i) plan->mergings[i] = s.mergings[i];
  }
  tcfftPlan native = nullptr;
  g_compat_status = tcfft_plan_1d(&native, n, n_batch, TCFFT_FP16);
  plan->F_real_tmp = reinterpret_cast<half*>(native);
}

void tcfftExec(tcfftHandle plan, half* data) {
  tcfftPlan native = native_of(plan.F_real_tmp);
  if (!native) {
    g_compat_status = TCFFT_INVALID_VALUE;
    return;
  }
  g_compat_status = tcfft_exec_digitrev(native, data, data, plan.radices, plan.n_radices, nullptr);
}

void tcfftDestroy(tcfftHandle* plan) {
  if (plan && plan->F_real_tmp) {
    g_compat_status = tcfft_destroy(native_of(plan->F_real_tmp));
    plan->F_real_tmp = nullptr;
  }
}

int tcfftGetLastError() { return g_compat_status; }

void setup(double* data, int n, int n_batch) {
  if (g_plan1.F_real_tmp) tcfftDestroy(&g_plan1);
  if (g_dev1) cudaFree(g_dev1);
  g_dev1 = nullptr;
  g_plan1 = tcfftHandle();
  g_n1 = n;
  g_b1 = n_batch;
  tcfftCreate(&g_plan1, n, n_batch);
  const std::vector<int> rev = digit_reversal(n, g_plan1.radices, g_plan1.n_radices);
  const size_t count = static_cast<size_t>(n) * static_cast<size_t>(n_batch);
  g_host1.assign(2 * count, __float2half(0.f));
  for (size_t b = 0; b < static_cast<size_t>(n_batch); ++b)
    for (int i = 0; i < n; ++i) {
      const size_t dst = 2 * (b * n + i), src = 2 * (b * n + static_cast<size_t>(rev[i]));
      g_host1[dst] = __double2half(data[src]);
      g_host1[dst + 1] = __double2half(data[src + 1]);
    }
  if (cudaMalloc(&g_dev1, sizeof(half) * 2 * count) != cudaSuccess) {
    g_compat_status = TCFFT_ALLOC_FAILED;
    return;
  }
  cudaMemcpy(g_dev1, g_host1.data(), sizeof(half) * 2 * count, cudaMemcpyHostToDevice);
}

void doit(int iter) {
  for (int t = 0; t < iter; ++t) tcfftExec(g_plan1, g_dev1);
  cudaDeviceSynchronize();
}

void finalize(double* result, int N_batch) {
  const size_t count = static_cast<size_t>(g_n1) * static_cast<size_t>(N_batch);
  cudaMemcpy(g_host1.data(), g_dev1, sizeof(half) * 2 * count, cudaMemcpyDeviceToHost);
  for (size_t i = 0; i < 2 * count; ++i) result[i] = __half2float(g_host1[i]);
}

// ----------------------------------------------------------------------------
// 2D (tcfft_half_2d.cu:1151-1291)
// ----------------------------------------------------------------------------
namespace {
// Per-axis settings of tcfftCreate_2d's switches: n_radices, value written to
// radices[2] (0 = keep the default 2), merging index.
void axis_shape(int n, int* n_radices, int* radices, int* merging) {
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
}  // namespace

void tcfftCreate_2d(tcfftHandle_2d* plan, int nx, int ny, int n_batch) {
  plan->Nx = nx;
  plan->Ny = ny;
  plan->N_batch = n_batch;
  for (int i = 0; i < 3; ++i) {
    plan->layer_0[i] = nullptr;
    plan->layer_1[i] = nullptr;
  }
  plan->F_real = plan->F_imag = nullptr;
  plan->F_real_tmp = plan->F_imag_tmp = nullptr;
  axis_shape(nx, &plan->n_radices_x, plan->radices_x, &plan->mergings[1]);
  axis_shape(ny, &plan->n_radices_y, plan->radices_y, &plan->mergings[0]);
  tcfftPlan native = nullptr;
  g_compat_status = tcfft_plan_2d(&native, nx, ny, n_batch, TCFFT_FP16);
  plan->F_real_tmp = reinterpret_cast<half*>(native);
}

void tcfftExec_2d(tcfftHandle_2d plan, half* data) {
  tcfftPlan native = native_of(plan.F_real_tmp);
  if (!native) {
    g_compat_status = TCFFT_INVALID_VALUE;
    return;
  }
  g_compat_status = tcfft_exec_digitrev_2d(native, data, data, plan.radices_x, plan.n_radices_x, plan.radices_y,
                                           plan.n_radices_y, TCFFT_FORWARD, nullptr);
}

void tcfftDestroy_2d(tcfftHandle_2d* plan) {
  if (plan && plan->F_real_tmp) {
    g_compat_status = tcfft_destroy(native_of(plan->F_real_tmp));
    plan->F_real_tmp = nullptr;
  }
}

void setup_2d(double* data, int nx, int ny, int n_batch) {
  if (g_plan2.F_real_tmp) tcfftDestroy_2d(&g_plan2);
  if (g_dev2) cudaFree(g_dev2);
  g_dev2 = nullptr;
  g_plan2 = tcfftHandle_2d();
  g_nx2 = nx;
  g_ny2 = ny;
  g_b2 = n_batch;
  tcfftCreate_2d(&g_plan2, nx, ny, n_batch);
  const std::vector<int> rx = digit_reversal(nx, g_plan2.radices_x, g_plan2.n_radices_x);
  const std::vector<int> ry = digit_reversal(ny, g_plan2.radices_y, g_plan2.n_radices_y);
  const size_t plane = static_cast<size_t>(nx) * static_cast<size_t>(ny);
  const size_t count = plane * static_cast<size_t>(n_batch);
  g_host2.assign(2 * count, __float2half(0.f));
  for (size_t b = 0; b < static_cast<size_t>(n_batch); ++b)
    for (int j = 0; j < nx; ++j)
      for (int k = 0; k < ny; ++k) {
        const size_t dst = 2 * (b * plane + static_cast<size_t>(j) * ny + k);
        const size_t src = 2 * (b * plane + static_cast<size_t>(rx[j]) * ny + static_cast<size_t>(ry[k]));
        g_host2[dst] = __double2half(data[src]);
        g_host2[dst + 1] = __double2half(data[src + 1]);
      }
  if (cudaMalloc(&g_dev2, sizeof(half) * 2 * count) != cudaSuccess) {
    g_compat_status = TCFFT_ALLOC_FAILED;
    return;
  }
  cudaMemcpy(g_dev2, g_host2.data(), sizeof(half) * 2 * count, cudaMemcpyHostToDevice);
}

void doit_2d(int iter) {
  for (int t = 0; t < iter; ++t) tcfftExec_2d(g_plan2, g_dev2);
  cudaDeviceSynchronize();
}

void finalize_2d(double* result, int N_batch) {
  const size_t count = static_cast<size_t>(g_nx2) * static_cast<size_t>(g_ny2) * static_cast<size_t>(N_batch);
  cudaMemcpy(g_host2.data(), g_dev2, sizeof(half) * 2 * count, cudaMemcpyDeviceToHost);
  for (size_t i = 0; i < 2 * count; ++i) result[i] = __half2float(g_host2[i]);
}
