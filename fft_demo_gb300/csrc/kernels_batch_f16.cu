// Instantiations: persistent uneven-batch kernel, FP16 (fft_batch.cuh).
#include "fft_batch.cuh"

namespace tcfft {

void register_batch_kernels_f16(BatchKernel (&tab)[2]) { fill_batch<false>(tab); }

}  // namespace tcfft
