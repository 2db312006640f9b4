// Instantiations: persistent uneven-batch kernel, split precision (fft_batch.cuh).
#include "fft_batch.cuh"

namespace tcfft {

void register_batch_kernels_split(BatchKernel (&tab)[2]) { fill_batch<true>(tab); }

}  // namespace tcfft
