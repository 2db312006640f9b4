// Drop-in replacement for yuelingfan/fft_demo tcfft_half_2d.h (2D tensor-core
// FFT). Same struct fields and signatures (tcfft_half_2d.h:7-24).
//
// Semantics kept: tcfftExec_2d transforms [N_batch][Nx][Ny] half2 data in
// place, forward, unnormalised, with rows in the digit-reversed order of
// radices_x and each row's elements in that of radices_y, as setup_2d()
// prepares. Differences: any Nx, Ny = 2^k in [16, 4096] (the reference
// supports Nx in {256, 512} and Ny in {256, 512, 1024}); tcfftDestroy_2d added.
// F_real_tmp carries the native plan handle; layer_* / F_real / F_imag unused.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdio>
#include <cstdlib>

struct tcfftHandle_2d
{
    int Nx, Ny, N_batch;
    int radices_x[3] = {16, 16, 2};
    int radices_y[3] = {16, 16, 2};
    int n_radices_x, n_radices_y;
    int mergings[2] = {0, 0};
    void (*layer_0[3])(half2 *, half *, half *);
    void (*layer_1[3])(int, half2 *, half *, half *);
    half *F_real, *F_imag;
    half *F_real_tmp, *F_imag_tmp;
};

void tcfftExec_2d(tcfftHandle_2d plan, half *data);
void tcfftCreate_2d(tcfftHandle_2d *plan, int nx, int ny, int n_batch);
void setup_2d(double *data, int nx, int ny, int n_batch);
void doit_2d(int iter);
void finalize_2d(double *result, int N_batch);

void tcfftDestroy_2d(tcfftHandle_2d *plan);
