// Instantiations: column passes (lines = adjacent columns of a row-major
// array): 2D column passes and the first pass of the four-step 1D transform.
#include "passes.cuh"

namespace tcfft {

void register_col_kernels(PassTable& tab) {
  fill_entry<16, 1024, true, false, false>(tab, kTileBig);
  fill_entry<32, 1024, true, false, false>(tab, kTileBig);
  fill_entry<64, 1024, true, false, false>(tab, kTileBig);
  fill_entry<128, 1024, true, false, false>(tab, kTileBig);
  fill_entry<256, 1024, true, false, false>(tab, kTileBig);
  fill_entry<512, 1024, true, false, false>(tab, kTileBig);
  fill_entry<1024, 1024, true, false, false>(tab, kTileBig);
  fill_entry<2048, 1024, true, false, false>(tab, kTileBig);
  fill_entry<4096, 1024, true, false, false>(tab, kTileBig);
  fill_pf_entry<64, 512, true, false, false, 3>(tab, kTileMid);
  fill_pf_entry<128, 512, true, false, false, 3>(tab, kTileMid);
  fill_pf_entry<256, 512, true, false, false, 3>(tab, kTileMid);
  fill_pf_entry<512, 512, true, false, false, 3>(tab, kTileMid);
  fill_pf_entry<1024, 512, true, false, false, 3>(tab, kTileMid);
  fill_pf_entry<2048, 512, true, false, false, 3>(tab, kTileMid);
}

}  // namespace tcfft
