// Instantiations: split-precision convolution passes, P = 64 .. 2048.
#include "conv_kernels.cuh"

namespace tcfft {

void register_conv_split(ConvTable& t) {
  conv_fill_split<64>(t);
  conv_fill_split<128>(t);
  conv_fill_split<256>(t);
  conv_fill_split<512>(t);
  conv_fill_split<1024>(t);
  conv_fill_split<2048>(t);
}

}  // namespace tcfft
