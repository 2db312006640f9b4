// Instantiations: split-precision 256-row tiles on 128 threads with the next
// tile's input prefetched into a raw buffer (3 CTAs per SM: ~70 KB shared
// memory each), for contiguous lines, column passes and transposing passes.
#include "passes.cuh"

namespace tcfft {

void register_split_pf_kernels(PassTable& row, PassTable& col, PassTable& rowt) {
  fill_split_pf_entry<64, 256, false, true, true, 128, 3>(row, kTileNarrow);
  fill_split_pf_entry<128, 256, false, true, true, 128, 3>(row, kTileNarrow);
  fill_split_pf_entry<256, 256, false, true, true, 128, 3>(row, kTileNarrow);
  fill_split_pf_entry<512, 256, false, true, true, 128, 3>(row, kTileNarrow);
  fill_split_pf_entry<1024, 256, false, true, true, 128, 3>(row, kTileNarrow);
  fill_split_pf_entry<2048, 256, false, true, true, 128, 3>(row, kTileNarrow);
  fill_split_pf_entry<4096, 256, false, true, true, 128, 3>(row, kTileNarrow);
  fill_split_pf_entry<64, 256, true, false, false, 128, 3>(col, kTileNarrow);
  fill_split_pf_entry<128, 256, true, false, false, 128, 3>(col, kTileNarrow);
  fill_split_pf_entry<256, 256, true, false, false, 128, 3>(col, kTileNarrow);
  fill_split_pf_entry<512, 256, true, false, false, 128, 3>(col, kTileNarrow);
  fill_split_pf_entry<1024, 256, true, false, false, 128, 3>(col, kTileNarrow);
  fill_split_pf_entry<256, 256, true, true, false, 128, 3>(rowt, kTileNarrow);
  fill_split_pf_entry<512, 256, true, true, false, 128, 3>(rowt, kTileNarrow);
  fill_split_pf_entry<1024, 256, true, true, false, 128, 3>(rowt, kTileNarrow);
  fill_split_pf_entry<2048, 256, true, true, false, 128, 3>(rowt, kTileNarrow);
}

}  // namespace tcfft
