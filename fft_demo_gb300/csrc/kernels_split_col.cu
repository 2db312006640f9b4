// Instantiations: split-precision column passes and transposing passes.
#include "passes.cuh"

namespace tcfft {

void register_split_col_kernels(PassTable& tab) {
  fill_split_entry<16, 512, true, false, false>(tab, kTileBig);
  fill_split_entry<32, 512, true, false, false>(tab, kTileBig);
  fill_split_entry<64, 512, true, false, false>(tab, kTileBig);
  fill_split_entry<128, 512, true, false, false>(tab, kTileBig);
  fill_split_entry<256, 512, true, false, false>(tab, kTileBig);
  fill_split_entry<512, 512, true, false, false>(tab, kTileBig);
  fill_split_entry<1024, 512, true, false, false>(tab, kTileBig);
  fill_split_entry<2048, 512, true, false, false>(tab, kTileBig);
}

void register_split_rowt_kernels(PassTable& tab) {
  fill_split_entry<16, 512, true, true, false>(tab, kTileBig);
  fill_split_entry<32, 512, true, true, false>(tab, kTileBig);
  fill_split_entry<64, 512, true, true, false>(tab, kTileBig);
  fill_split_entry<128, 512, true, true, false>(tab, kTileBig);
  fill_split_entry<256, 512, true, true, false>(tab, kTileBig);
  fill_split_entry<512, 512, true, true, false>(tab, kTileBig);
  fill_split_entry<1024, 512, true, true, false>(tab, kTileBig);
  fill_split_entry<2048, 512, true, true, false>(tab, kTileBig);
}

}  // namespace tcfft
