// Harness translation unit: the reference's 2D tcFFT stage kernels
// (tcfft_half_2d.cu) as a device-only cubin; separate from the 1D harness
// because both files define layer_* templates with different bodies.
// TEST INFRASTRUCTURE ONLY.
#include "tcfft_half_2d.cu"

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
