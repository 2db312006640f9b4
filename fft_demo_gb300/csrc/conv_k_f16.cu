// Instantiations: FP16 convolution passes, P = 64 .. 4096.
#include "conv_kernels.cuh"

namespace tcfft {

void register_conv_f16(ConvTable& t) {
  conv_fill_f16<64>(t);
  conv_fill_f16<128>(t);
  conv_fill_f16<256>(t);
  conv_fill_f16<512>(t);
  conv_fill_f16<1024>(t);
  conv_fill_f16<2048>(t);
  conv_fill_f16<4096>(t);
}

}  // namespace tcfft
