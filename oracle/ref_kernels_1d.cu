// Harness translation unit: the reference's 1D tcFFT stage kernels, compiled
// from its own source (tcfft_half.cu, included from the reference tree by
// oracle/ref_build.sh) into a device-only cubin. Both wirings are
// instantiated: the V100 kernels tcfftCreate assigns (tcfft_half.cu:1244-1248)
// and the _A100 ones (same file) that fft_conv2d_half selects on Ampere.
// TEST INFRASTRUCTURE ONLY (parity fixtures); never linked into the product.
#include "tcfft_half.cu"

template __global__ void layer_256_0<32, 8>(half2 *, half *, half *);
template __global__ void layer_512_0<16, 8>(half2 *, half *, half *);
template __global__ void layer_1024_0<8, 8>(half2 *, half *, half *);
template __global__ void layer_256_1<32, 8>(int, half2 *, half *, half *);
template __global__ void layer_512_1<16, 8>(int, half2 *, half *, half *);
template __global__ void layer_256_0_A100<32, 8>(half2 *, half *, half *);
template __global__ void layer_512_0_A100<16, 8>(half2 *, half *, half *);
template __global__ void layer_1024_0_A100<8, 8>(half2 *, half *, half *);
template __global__ void layer_256_1_A100<32, 8>(int, half2 *, half *, half *);
template __global__ void layer_512_1_A100<16, 8>(int, half2 *, half *, half *);
