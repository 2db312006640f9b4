// Drop-in check: drives the library only through the reference's own headers
// and call sequences (main.cpp:164-200, 267-316; main_2d.cpp:76, 186-200),
// compiled against include/compat/*.h and linked with libtcfft_gb300.so.
// Writes raw FP64 / FP32 results for tests/test_compat_gpu.py to check against
// the FP64 oracle.
//   usage: compat_driver OUT_DIR
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "fftconvolve2d.cuh"
#include "tcfft_half.h"
#include "tcfft_half_2d.h"
#include "tensorcore_fft_conv2d.h"
#include "tcfft_gb300.h"

static unsigned long long g_state = 42;
static double next_val() {  // seeded values in {0, 0.1, ..., 0.9}, like generate_data (main.cpp:32)
  g_state = g_state * 6364136223846793005ull + 1442695040888963407ull;
  return 0.1 * static_cast<double>((g_state >> 33) % 10);
}

static void dump(const std::string& path, const void* data, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    perror(path.c_str());
    exit(2);
  }
  fwrite(data, 1, bytes, f);
  fclose(f);
}

int main(int argc, char** argv) {
  const std::string out = argc > 1 ? argv[1] : ".";
  // ---- 1D: setup / doit / finalize (main.cpp:164-180) ----
  {
    const int n = 256, batch = 64;
    std::vector<double> data(2 * n * batch), result(2 * n * batch);
    for (auto& v : data) v = next_val();
    setup(data.data(), n, batch);
    doit(1);
    finalize(result.data(), batch);
    dump(out + "/in_1d.bin", data.data(), data.size() * 8);
    dump(out + "/out_1d.bin", result.data(), result.size() * 8);
    printf("1d status %d\n", tcfftGetLastError());
  }
  // ---- 1D through tcfftCreate / tcfftExec on an unconfigured size (4096) ----
  {
    const int n = 4096, batch = 8;
    std::vector<double> data(2 * n * batch), result(2 * n * batch);
    for (auto& v : data) v = next_val();
    setup(data.data(), n, batch);
    doit(2);  // two forward transforms in a row
    finalize(result.data(), batch);
    dump(out + "/in_1d_4096.bin", data.data(), data.size() * 8);
    dump(out + "/out_1d_4096.bin", result.data(), result.size() * 8);
  }
  // ---- 2D: setup_2d / doit_2d / finalize_2d (main.cpp:182-198) ----
  {
    const int nx = 256, ny = 512, batch = 2;
    std::vector<double> data(2 * nx * ny * batch), result(2 * nx * ny * batch);
    for (auto& v : data) v = next_val();
    setup_2d(data.data(), nx, ny, batch);
    doit_2d(1);
    finalize_2d(result.data(), batch);
    dump(out + "/in_2d.bin", data.data(), data.size() * 8);
    dump(out + "/out_2d.bin", result.data(), result.size() * 8);
  }
  // ---- conv forward (main.cpp:267-305), backward, fft_2d_c2c ----
  {
    const int s = 256, f = 13, C = 1, F = 16, o = s - f + 1;
    std::vector<double> signal(s * s * C), filter(f * f * F * C), output(o * o * F);
    for (auto& v : signal) v = next_val();
    for (auto& v : filter) v = next_val();
    fft_conv2d_half conv(signal.data(), filter.data(), C, F, s, s, f, f, __AMPERE__);
    conv.conv2d_forward(output.data());
    dump(out + "/conv_signal.bin", signal.data(), signal.size() * 8);
    dump(out + "/conv_filter.bin", filter.data(), filter.size() * 8);
    dump(out + "/conv_out.bin", output.data(), output.size() * 8);
    printf("conv status %d padded %d\n", conv.last_status, conv.padded_x);
    std::vector<double> delta(o * o * F);
    for (auto& v : delta) v = next_val() - 0.45;
    conv.conv2d_backward(delta.data());
    dump(out + "/conv_delta.bin", delta.data(), delta.size() * 8);
    dump(out + "/conv_dw.bin", conv.delta_for_filter, sizeof(double) * f * f * F * C);
    dump(out + "/conv_dx.bin", conv.delta_for_signal, sizeof(double) * s * s * C);
    free(conv.delta_for_filter);
    free(conv.delta_for_signal);
    // batch 5: five sub-batches over four streams (one stream reused)
    std::vector<double> cin(5 * 256 * 256 * 2), cout_(5 * 256 * 256 * 2), cback(5 * 256 * 256 * 2);
    for (auto& v : cin) v = next_val();
    conv.fft_2d_c2c(cin.data(), cout_.data(), 256, 256, 5, __AMPERE__);
    std::vector<double> cmid(cout_);  // scaled so the unnormalised inverse stays in FP16 range
    for (auto& v : cmid) v /= 256.0 * 256.0;
    conv.ifft_2d_c2c(cmid.data(), cback.data(), 256, 256, 5, __AMPERE__);
    dump(out + "/c2c_in.bin", cin.data(), cin.size() * 8);
    dump(out + "/c2c_out.bin", cout_.data(), cout_.size() * 8);
    dump(out + "/c2c_back.bin", cback.data(), cback.size() * 8);
  }
  // ---- cuFFT-family full convolution (main.cpp:307-314) ----
  {
    const int kernelCount = 16, f = 13, o = 244;
    std::vector<float> sig(o * o), ker(f * f * kernelCount), res((o + f - 1) * (o + f - 1) * kernelCount);
    for (auto& v : sig) v = static_cast<float>(next_val());
    for (auto& v : ker) v = static_cast<float>(next_val());
    convolve_direct_fft(sig.data(), ker.data(), kernelCount, o, o, f, f, res.data());
    dump(out + "/full_sig.bin", sig.data(), sig.size() * 4);
    dump(out + "/full_ker.bin", ker.data(), ker.size() * 4);
    dump(out + "/full_out.bin", res.data(), res.size() * 4);
    std::vector<float> res2(res.size());
    convolve_turbo_fft_v2(sig.data(), ker.data(), kernelCount, o, o, f, f, res2.data());
    dump(out + "/full_out_v2.bin", res2.data(), res2.size() * 4);
    std::vector<cufftComplex> spec((kernelCount / 2) * 256 * 256);
    direct_fft(ker.data(), kernelCount, o, o, f, f, spec.data());
    dump(out + "/direct_fft.bin", spec.data(), spec.size() * sizeof(cufftComplex));
  }
  // ---- TensorCoreFFTCreate / TensorCoreFFTExec (kernel.cu:1557,1495,1526) ----
  // [batch][nx][ny] complex, both axes digit-reversed by the class's rev()
  // (its gen_rev tables), forward (fft = 1, default stream) and inverse
  // (fft = -1, stream overload); nx = 256 rows of ny = 512 elements.
  {
    const int nx = 256, ny = 512, batch = 3;
    const size_t cnt = 2ull * nx * ny * batch;
    std::vector<double> x(cnt), fwd(cnt), inv(cnt);
    for (auto& v : x) v = next_val() - 0.45;
    double* d = nullptr;
    half *h1 = nullptr, *h2 = nullptr;
    cudaMalloc(&d, sizeof(double) * cnt);
    cudaMalloc(&h1, sizeof(half) * cnt);
    cudaMalloc(&h2, sizeof(half) * cnt);
    cudaMemcpy(d, x.data(), sizeof(double) * cnt, cudaMemcpyHostToDevice);
    fft_conv2d_half obj;
    obj.rev(d, h1, ny, nx, batch, 0, nullptr);  // x = elements per row, y = rows
    obj.rev(d, h2, ny, nx, batch, 0, nullptr);
    fftPlan pf, pi;
    obj.TensorCoreFFTCreate(&pf, nx, ny, batch, 1, __AMPERE__);
    obj.TensorCoreFFTCreate(&pi, nx, ny, batch, -1, __AMPERE__);
    obj.TensorCoreFFTExec(pf, h1);
    cudaStream_t st;
    cudaStreamCreate(&st);
    obj.TensorCoreFFTExec(pi, h2, st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    printf("TensorCoreFFTExec status %d\n", obj.last_status);
    obj.half2double(h1, d, nx, ny, 2, batch, nullptr);
    cudaMemcpy(fwd.data(), d, sizeof(double) * cnt, cudaMemcpyDeviceToHost);
    obj.half2double(h2, d, nx, ny, 2, batch, nullptr);
    cudaMemcpy(inv.data(), d, sizeof(double) * cnt, cudaMemcpyDeviceToHost);
    obj.TensorCoreFFTDestroy(&pf);
    obj.TensorCoreFFTDestroy(&pi);
    cudaFree(d);
    cudaFree(h1);
    cudaFree(h2);
    dump(out + "/tc_in.bin", x.data(), cnt * 8);
    dump(out + "/tc_fwd.bin", fwd.data(), cnt * 8);
    dump(out + "/tc_inv.bin", inv.data(), cnt * 8);
    // internal pipeline steps that cannot run on their own report it
    obj.fft_pointwise();
    printf("fft_pointwise status %d\n", obj.last_status);
  }
  // ---- qdFFT route: qd_fft, fast_fft, convolve_turbo_fft_v3 ----
  {
    const int kernelCount = 16, f = 13, o = 244, P = 256;
    std::vector<float> sig(o * o), ker(f * f * kernelCount), res((o + f - 1) * (o + f - 1) * kernelCount);
    for (auto& v : sig) v = static_cast<float>(next_val());
    for (auto& v : ker) v = static_cast<float>(next_val() - 0.45);
    dump(out + "/qd_sig.bin", sig.data(), sig.size() * 4);
    dump(out + "/qd_ker.bin", ker.data(), ker.size() * 4);
    convolve_turbo_fft_v3(sig.data(), ker.data(), kernelCount, o, o, f, f, res.data());
    printf("turbo_v3 status %d\n", tcfft_get_last_error());
    dump(out + "/qd_v3.bin", res.data(), res.size() * 4);
    std::vector<cufftComplex> spec((kernelCount / 2) * P * P);
    qd_fft(ker.data(), kernelCount, o, o, f, f, spec.data());
    printf("qd_fft status %d\n", tcfft_get_last_error());
    dump(out + "/qd_fft.bin", spec.data(), spec.size() * sizeof(cufftComplex));
    // fast_fft on device planes: pairs packed as (re, im), zero-padded to P x P
    const int groups = kernelCount / 2;
    std::vector<cufftComplex> planes(static_cast<size_t>(groups) * P * P), fres(planes.size());
    for (auto& c : planes) c.x = c.y = 0.f;
    for (int g = 0; g < groups; ++g)
      for (int y = 0; y < f; ++y)
        for (int x = 0; x < f; ++x) {
          cufftComplex& c = planes[(static_cast<size_t>(g) * P + y) * P + x];
          c.x = ker[(2 * g) * f * f + y * f + x];
          c.y = ker[(2 * g + 1) * f * f + y * f + x];
        }
    cufftComplex *dp = nullptr, *dr = nullptr;
    cudaMalloc(&dp, sizeof(cufftComplex) * planes.size());
    cudaMalloc(&dr, sizeof(cufftComplex) * planes.size());
    cudaMemcpy(dp, planes.data(), sizeof(cufftComplex) * planes.size(), cudaMemcpyHostToDevice);
    fast_fft(dp, groups, P, P, f, f, dr, true);
    printf("fast_fft status %d\n", tcfft_get_last_error());
    cudaMemcpy(fres.data(), dr, sizeof(cufftComplex) * fres.size(), cudaMemcpyDeviceToHost);
    cudaFree(dp);
    cudaFree(dr);
    dump(out + "/fast_fft.bin", fres.data(), fres.size() * sizeof(cufftComplex));
  }
  // ---- full convolution at a padded size that is not a power of two ----
  // fftRows = fftCols = 84 + 13 - 1 = 96 (a multiple of 32, as the
  // reference's kernels assume): the convolution runs at the next power of
  // two and is cropped; the spectra of a 96-point grid are not produced.
  {
    const int kernelCount = 16, f = 13, o = 84, fr = o + f - 1;
    std::vector<float> sig(o * o), ker(f * f * kernelCount), res(fr * fr * kernelCount), res3(res.size());
    for (auto& v : sig) v = static_cast<float>(next_val());
    for (auto& v : ker) v = static_cast<float>(next_val() - 0.45);
    dump(out + "/np2_sig.bin", sig.data(), sig.size() * 4);
    dump(out + "/np2_ker.bin", ker.data(), ker.size() * 4);
    convolve_direct_fft(sig.data(), ker.data(), kernelCount, o, o, f, f, res.data());
    printf("np2 direct status %d\n", tcfft_get_last_error());
    dump(out + "/np2_direct.bin", res.data(), res.size() * 4);
    convolve_turbo_fft_v3(sig.data(), ker.data(), kernelCount, o, o, f, f, res3.data());
    printf("np2 turbo_v3 status %d\n", tcfft_get_last_error());
    dump(out + "/np2_v3.bin", res3.data(), res3.size() * 4);
    std::vector<cufftComplex> spec((kernelCount / 2) * fr * fr);
    direct_fft(ker.data(), kernelCount, o, o, f, f, spec.data());
    printf("np2 direct_fft status %d\n", tcfft_get_last_error());
  }
  printf("compat driver done\n");
  return 0;
}
