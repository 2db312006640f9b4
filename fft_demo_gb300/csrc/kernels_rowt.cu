// Instantiations: contiguous-line passes with a transposing store (second
// pass of the four-step 1D transform: row k1 -> X[k1 + N1 * k2]). Line-minor
// butterfly order, so a warp's stores cover adjacent lines = adjacent addresses.
#include "passes.cuh"

namespace tcfft {

void register_rowt_kernels(PassTable& tab) {
  fill_entry<16, 1024, true, true, false>(tab, kTileBig);
  fill_entry<32, 1024, true, true, false>(tab, kTileBig);
  fill_entry<64, 1024, true, true, false>(tab, kTileBig);
  fill_entry<128, 1024, true, true, false>(tab, kTileBig);
  fill_entry<256, 1024, true, true, false>(tab, kTileBig);
  fill_entry<512, 1024, true, true, false>(tab, kTileBig);
  fill_entry<1024, 1024, true, true, false>(tab, kTileBig);
  fill_entry<2048, 1024, true, true, false>(tab, kTileBig);
  fill_entry<4096, 1024, true, true, false>(tab, kTileBig);
  fill_pf_entry<64, 512, true, true, false, 3>(tab, kTileMid);
  fill_pf_entry<128, 512, true, true, false, 3>(tab, kTileMid);
  fill_pf_entry<256, 512, true, true, false, 3>(tab, kTileMid);
  fill_pf_entry<512, 512, true, true, false, 3>(tab, kTileMid);
  fill_pf_entry<1024, 512, true, true, false, 3>(tab, kTileMid);
  fill_pf_entry<2048, 512, true, true, false, 3>(tab, kTileMid);
}

}  // namespace tcfft
