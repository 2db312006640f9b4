// Instantiations: fused four-step kernels (FP16), N = 2^15 .. 2^24. The split
// N1 x N2 matches the two-pass plan (N1 = 2^min(10, log2(N)/2), N2 <= 2^12).
#include "passes.cuh"

namespace tcfft {

void register_fused_kernels(FusedTable& tab) {
  fill_fused<128, 256>(tab);
  fill_fused<256, 256>(tab);
  fill_fused<256, 512>(tab);
  fill_fused<512, 512>(tab);
  fill_fused<512, 1024>(tab);
  fill_fused<1024, 1024>(tab);
  fill_fused<1024, 2048>(tab);
  fill_fused<1024, 4096>(tab);
  fill_fused<2048, 4096>(tab);
  fill_fused<4096, 4096>(tab);
}

}  // namespace tcfft
