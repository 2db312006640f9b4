// Instantiations: split-precision (FP32 data, hi+lo FP16 tensor-core
// operands) passes: contiguous lines, column passes, transposing passes.
#include "passes.cuh"

namespace tcfft {

void register_split_row_kernels(PassTable& tab) {
  fill_split_entry<16, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<32, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<64, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<128, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<256, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<512, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<1024, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<2048, 128, false, true, true>(tab, kTileSmall);
  fill_split_entry<16, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<32, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<64, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<128, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<256, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<512, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<1024, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<2048, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<4096, 512, false, true, true>(tab, kTileBig);
  fill_split_entry<8192, 512, false, true, true>(tab, kTileBig);
}

}  // namespace tcfft
