// Instantiations: split-precision 256-row tiles on 128 threads (4 CTAs per
// SM: 128 TMEM columns, ~39 KB shared memory and 128 registers a thread
// each), for contiguous lines, column passes and transposing passes.
#include "passes.cuh"

namespace tcfft {

void register_split_mid_kernels(PassTable& row, PassTable& col, PassTable& rowt) {
  fill_split_entry<64, 256, false, true, true, 128>(row, kTileMid);
  fill_split_entry<128, 256, false, true, true, 128>(row, kTileMid);
  fill_split_entry<256, 256, false, true, true, 128>(row, kTileMid);
  fill_split_entry<512, 256, false, true, true, 128>(row, kTileMid);
  fill_split_entry<1024, 256, false, true, true, 128>(row, kTileMid);
  fill_split_entry<2048, 256, false, true, true, 128>(row, kTileMid);
  fill_split_entry<4096, 256, false, true, true, 128>(row, kTileMid);
  fill_split_entry<64, 256, true, false, false, 128>(col, kTileMid);
  fill_split_entry<128, 256, true, false, false, 128>(col, kTileMid);
  fill_split_entry<256, 256, true, false, false, 128>(col, kTileMid);
  fill_split_entry<512, 256, true, false, false, 128>(col, kTileMid);
  fill_split_entry<1024, 256, true, false, false, 128>(col, kTileMid);
  fill_split_entry<256, 256, true, true, false, 128>(rowt, kTileMid);
  fill_split_entry<512, 256, true, true, false, 128>(rowt, kTileMid);
  fill_split_entry<1024, 256, true, true, false, 128>(rowt, kTileMid);
  fill_split_entry<2048, 256, true, true, false, 128>(rowt, kTileMid);
}

}  // namespace tcfft
