// Instantiations: contiguous-line passes (1D transforms up to 2^14 points,
// 2D row passes).
#include "passes.cuh"

namespace tcfft {

void register_row_kernels(PassTable& tab) {
  fill_entry<16, 128, false, true, true>(tab, kTileSmall);
  fill_entry<32, 128, false, true, true>(tab, kTileSmall);
  fill_entry<64, 128, false, true, true>(tab, kTileSmall);
  fill_entry<128, 128, false, true, true>(tab, kTileSmall);
  fill_entry<256, 128, false, true, true>(tab, kTileSmall);
  fill_entry<512, 128, false, true, true>(tab, kTileSmall);
  fill_entry<1024, 128, false, true, true>(tab, kTileSmall);
  fill_entry<2048, 128, false, true, true>(tab, kTileSmall);
  fill_entry<16, 1024, false, true, true>(tab, kTileBig);
  fill_entry<32, 1024, false, true, true>(tab, kTileBig);
  fill_entry<64, 1024, false, true, true>(tab, kTileBig);
  fill_entry<128, 1024, false, true, true>(tab, kTileBig);
  fill_entry<256, 1024, false, true, true>(tab, kTileBig);
  fill_entry<512, 1024, false, true, true>(tab, kTileBig);
  fill_entry<1024, 1024, false, true, true>(tab, kTileBig);
  fill_entry<2048, 1024, false, true, true>(tab, kTileBig);
  fill_entry<4096, 1024, false, true, true>(tab, kTileBig);
  fill_entry<8192, 1024, false, true, true>(tab, kTileBig);
  fill_entry<16384, 1024, false, true, true>(tab, kTileBig);
  fill_pf_entry<64, 512, false, true, true, 3>(tab, kTileMid);
  fill_pf_entry<128, 512, false, true, true, 3>(tab, kTileMid);
  fill_pf_entry<256, 512, false, true, true, 3>(tab, kTileMid);
  fill_pf_entry<512, 512, false, true, true, 3>(tab, kTileMid);
  fill_pf_entry<1024, 512, false, true, true, 3>(tab, kTileMid);
  fill_pf_entry<2048, 512, false, true, true, 3>(tab, kTileMid);
  fill_pf_entry<4096, 512, false, true, true, 3>(tab, kTileMid);
  fill_pf_entry<8192, 512, false, true, true, 3>(tab, kTileMid);
}

}  // namespace tcfft
