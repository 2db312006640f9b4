#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace tcfft {

// tw[i] = exp(sign * 2 pi i * ((i << stride_log2) mod 2^log2n) / 2^log2n), i < count.
cudaError_t gen_twiddles(float2* tw, long long count, int log2n, int stride_log2, int sign,
                         cudaStream_t stream);
// 2 KB image of the 32x32 real 16-point DFT matrix (part 0 FP16 hi, part 1
// the FP16 residual B - hi).
cudaError_t gen_dft16_bmat(uint16_t* img, int sign, int part, cudaStream_t stream);

}  // namespace tcfft
