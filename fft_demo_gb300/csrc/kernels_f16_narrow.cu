// Instantiations: FP16 prefetching passes with 256-row tiles on 128 threads
// (6 CTAs per SM: 64 TMEM columns, ~37 KB of shared memory and up to 80
// registers a thread each), for contiguous lines, column passes and
// transposing passes.
#include "passes.cuh"

namespace tcfft {

void register_f16_narrow_kernels(PassTable& row, PassTable& col, PassTable& rowt) {
  fill_pf_entry<64, 256, false, true, true, 6, 128>(row, kTileNarrow);
  fill_pf_entry<128, 256, false, true, true, 6, 128>(row, kTileNarrow);
  fill_pf_entry<256, 256, false, true, true, 6, 128>(row, kTileNarrow);
  fill_pf_entry<512, 256, false, true, true, 6, 128>(row, kTileNarrow);
  fill_pf_entry<1024, 256, false, true, true, 6, 128>(row, kTileNarrow);
  fill_pf_entry<2048, 256, false, true, true, 6, 128>(row, kTileNarrow);
  fill_pf_entry<4096, 256, false, true, true, 6, 128>(row, kTileNarrow);
  fill_pf_entry<64, 256, true, false, false, 6, 128>(col, kTileNarrow);
  fill_pf_entry<128, 256, true, false, false, 6, 128>(col, kTileNarrow);
  fill_pf_entry<256, 256, true, false, false, 6, 128>(col, kTileNarrow);
  fill_pf_entry<512, 256, true, false, false, 6, 128>(col, kTileNarrow);
  fill_pf_entry<1024, 256, true, false, false, 6, 128>(col, kTileNarrow);
  fill_pf_entry<64, 256, true, true, false, 6, 128>(rowt, kTileNarrow);
  fill_pf_entry<128, 256, true, true, false, 6, 128>(rowt, kTileNarrow);
  fill_pf_entry<256, 256, true, true, false, 6, 128>(rowt, kTileNarrow);
  fill_pf_entry<512, 256, true, true, false, 6, 128>(rowt, kTileNarrow);
  fill_pf_entry<1024, 256, true, true, false, 6, 128>(rowt, kTileNarrow);
  fill_pf_entry<2048, 256, true, true, false, 6, 128>(rowt, kTileNarrow);
}

}  // namespace tcfft
