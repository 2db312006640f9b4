// Line-projection 2D DFT (qd.cu) for other translation units of the library.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/tcfft_gb300.h"

namespace tcfft {

// Plan for `planes` n x n planes (16 <= n <= 4096) whose non-zeros lie in the
// top-left box_rows x box_cols box. Holds the projections and a
// split-precision 1D plan of n points.
tcfftStatus qd_create(tcfftQdImpl** out, int n, long long planes, int box_rows, int box_cols);
void qd_free(tcfftQdImpl* q);
// Synchronise `st`; TCFFT_TIMEOUT if a transform of the plan flagged a wait.
tcfftStatus qd_check(tcfftQdImpl* q, cudaStream_t st);
// out[g] = 2D DFT (direction) of complex planes[g] (float2 [planes][n][n]).
tcfftStatus qd_exec_planes(tcfftQdImpl* q, const float2* planes, float2* out, int direction, cudaStream_t st);
// Spectra of `count` real box_rows x box_cols filters (rotated by 180 degrees
// when flip != 0), two per projected plane; out[c] = E [n][n], c < count.
template <class E>
tcfftStatus qd_exec_filter_pairs(tcfftQdImpl* q, const float* filters, long long count, int flip, E* out,
                                 int direction, cudaStream_t st);

// Complex spectra of real filters packed two per plane (filter 2g real
// part, 2g + 1 imaginary part): out[g] = float2 [n][n], g < ceil(count / 2).
tcfftStatus qd_exec_pairs_packed(tcfftQdImpl* q, const float* filters, long long count, float2* out, int direction,
                                 cudaStream_t st);

}  // namespace tcfft
