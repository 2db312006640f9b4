// Drop-in replacement for yuelingfan/fft_demo include/fftconvolve2d.cuh: the
// FP32 FFT-convolution family, served by the split-precision (FP32 data,
// hi+lo FP16 tensor-core operands) path of include/tcfft_gb300.h instead of
// cuFFT. Same signatures (fftconvolve2d.cuh:5-14); host pointers unless noted.
//
//   convolve_direct_fft / convolve_turbo_fft_v2 / convolve_turbo_fft_v3
//       (fftconvolve2d.cu:184, :626, :1263): results[k][nRows+kRows-1]
//       [nCols+kCols-1] = full linear convolution of Signal [nRows][nCols]
//       with kernel k of Kernels [kernelCount][kRows][kCols] (the reference's
//       1/fftSize cancels its unnormalised C2R inverse). v3 makes its filter
//       spectra by line projections (qdFFT), like the reference; the others
//       by the masked row/column passes.
//   direct_fft (fftconvolve2d.cu:1510): spectra of kernel pairs packed as
//       (re = kernel 2g, im = kernel 2g+1), zero-padded to
//       (nRows+kRows-1) x (nCols+kCols-1), unnormalised inverse-sign 2D DFT;
//       results [kernelCount/2][fftRows][fftCols] (host).
//   qd_fft (fftconvolve2d.cu:1603): the same spectra by line projections:
//       3n/2 projections of the kRows x kCols box, a 1D DFT of each, gathered
//       into the 2D spectrum (fftRows == fftCols == n required).
//   fast_fft (fftconvolve2d.cu:1011): device arrays; 2D DFT by line
//       projections of each of group_num n x n complex planes whose non-zeros
//       lie in the top-left kCols x kCols box (the box the reference's sparse
//       projection reads), forward or inverse sign, unnormalised.
// The reference's functions return void and check nothing; here each records
// its status for tcfft_get_last_error() (include/tcfft_gb300.h).
// Limits: padded extents must be powers of two (<= 2048 x 8192; <= 4096 for
// the projection route); the reference's own call sites (main.cpp:312,
// main_2d.cpp:199) use 256 x 256. Unlike the reference there is no
// requirement that kernelCount be a multiple of 16.
#ifndef FFTCONVOLVE2D_CUH
#define FFTCONVOLVE2D_CUH
#include <cufft.h>

void convolve_direct_fft(float *, float *, int, int, int, int, int, float *);
void convolve_turbo_fft_v2(float *, float *, int, int, int, int, int, float *);
void convolve_turbo_fft_v3(float *, float *, int, int, int, int, int, float *);
void direct_fft(float *, int, int, int, int, int, cufftComplex *);
void qd_fft(float *, int, int, int, int, int, cufftComplex *);
void fast_fft(cufftComplex *, int, int, int, int, int, cufftComplex *, bool);
#endif
