// Drop-in replacement for yuelingfan/fft_demo tcfft_half.h (1D tensor-core
// FFT). Same struct fields and C++ signatures (tcfft_half.h:7-24); the plan
// is served by the sm_103a library behind include/tcfft_gb300.h.
//
// Semantics kept: tcfftExec transforms `data` in place on the default
// stream, forward, unnormalised, with its input in the digit-reversed order
// that setup() produces from plan.radices (gen_rev). Differences: every power
// of two 16..2^24 works (the reference configures only 256, 512, 1024,
// 2^17..2^19 and 2^24..2^27; for other sizes it leaves n_radices = 0, so its
// permutation is the identity and the input is taken in natural order here),
// FP32 accumulation, and tcfftDestroy frees the plan.
//
// Field use: radices / n_radices / mergings / n_mergings are filled exactly as
// the reference's tcfftCreate fills them; layer_0 / layer_1 / F_real / F_imag
// are unused (null); F_real_tmp carries the native plan handle.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdio>
#include <cstdlib>

struct tcfftHandle
{
    int N, N_batch;
    int radices[9] = {16, 16, 16, 16, 16, 16, 16, 16, 16};
    int n_radices;
    int mergings[3] = {0, 0, 0};
    int n_mergings;
    void (*layer_0[3])(half2 *, half *, half *);
    void (*layer_1[3])(int, half2 *, half *, half *);
    half *F_real, *F_imag;
    half *F_real_tmp, *F_imag_tmp;
};

void tcfftExec(tcfftHandle plan, half *data);
void tcfftCreate(tcfftHandle *plan, int n, int n_batch);
void setup(double *data, int n, int n_batch);
void doit(int iter);
void finalize(double *result, int N_batch);

// Added (the reference has no destroy): releases the plan tcfftCreate made.
void tcfftDestroy(tcfftHandle *plan);
// Added: status of the last compat call (tcfftStatus from tcfft_gb300.h).
int tcfftGetLastError();
