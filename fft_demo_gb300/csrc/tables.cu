// FP64 generation of the DFT matrix and twiddle tables on the GPU.
//
// Every table entry is computed in double precision (sincospi of an exactly
// reduced rational angle) and rounded once: to FP32 for twiddles, to an FP16
// (hi, lo) pair for the 16-point DFT matrix (lo = the residual B - hi; at most
// 2^-12, it keeps at least 8 significant bits even where it is subnormal,
// about 6e-8 absolute).
//
// The reference computes its 16x16 DFT matrix on the host in FP32 and rounds
// it to FP16 (tcfft_half.cu:1332-1339) and its twiddles per thread with
// cosf/sinf (tcfft_half.cu:40-50).
#include <cuda_fp16.h>
#include <cstdint>

#include "tc_ptx.cuh"
#include "tables.cuh"

namespace tcfft {

// W_N^e = exp(sign * 2 pi i e / N) for e in [0, count), stored as float2.
// Angle reduced exactly: e/N as a dyadic rational; sincospi evaluates
// sin/cos(pi * 2e/N) in double.
__global__ void gen_twiddle_kernel(float2* __restrict__ tw, long long count, int log2n, int stride_log2,
                                   int sign) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  const unsigned long long n = 1ull << log2n;
  const unsigned long long e = (static_cast<unsigned long long>(i) << stride_log2) & (n - 1);
  const double x = 2.0 * static_cast<double>(e) / static_cast<double>(n);
  double s, c;
  sincospi(x, &s, &c);
  tw[i] = make_float2(static_cast<float>(c), static_cast<float>(sign * s));
}

// Image of B (32 x 32, K-major, no swizzle, 8x8 core matrices: K-adjacent
// cores 128 B apart, N-adjacent cores 512 B apart) for the real form of the
// 16-point DFT F[c][r] = exp(sign * 2 pi i c r / 16):
//   B[r][c]       =  Re F[c][r]     B[r][16+c]    = Im F[c][r]
//   B[16+r][c]    = -Im F[c][r]     B[16+r][16+c] = Re F[c][r]
// part 0 = FP16 hi, part 1 = FP16 lo residual (B - hi, at its own scale).
__global__ void gen_dft16_bmat_kernel(uint16_t* __restrict__ img, int sign, int part) {
  const int idx = threadIdx.x;  // 0..1023 = n * 32 + k
  if (idx >= 1024) return;
  const int n = idx / 32, k = idx % 32;
  const int c = n % 16, r = k % 16;
  const double x = 2.0 * static_cast<double>((c * r) % 16) / 16.0;
  double s, co;
  sincospi(x, &s, &co);
  const double fr = co, fi = sign * s;
  double v;
  if (k < 16)
    v = (n < 16) ? fr : fi;
  else
    v = (n < 16) ? -fi : fr;
  const __half hi = __double2half(v);
  __half outv = hi;
  if (part == 1) outv = __double2half(v - static_cast<double>(__half2float(hi)));
  const uint32_t off = kmajor_none_offset(static_cast<uint32_t>(n), static_cast<uint32_t>(k), 128u, 512u);
  img[off / 2] = __half_as_ushort(outv);
}

cudaError_t gen_twiddles(float2* tw, long long count, int log2n, int stride_log2, int sign,
                         cudaStream_t stream) {
  const int threads = 256;
  const long long blocks = (count + threads - 1) / threads;
  gen_twiddle_kernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(tw, count, log2n,
                                                                            stride_log2, sign);
  return cudaGetLastError();
}

cudaError_t gen_dft16_bmat(uint16_t* img, int sign, int part, cudaStream_t stream) {
  gen_dft16_bmat_kernel<<<1, 1024, 0, stream>>>(img, sign, part);
  return cudaGetLastError();
}

}  // namespace tcfft
