// Registry access for entry points defined outside capi.cu.
#pragma once
#include "../../include/tcfft_gb300.h"
#include "passes.cuh"

namespace tcfft {

// Loads the kernel registry on first use (current device); TCFFT_OK when ready.
tcfftStatus registry_ready();
// Fused four-step kernel for 2^logn points (sign_idx 0 forward, 1 inverse) and
// the persistent grid size for it; nullptr when not built.
const FusedKernel* fused_kernel(int logn, int sign_idx, int* grid_ctas);
// Poll bound of the persistent kernels' dependency waits for launches made
// now (tcfft_set_wait_limit; 2^24 by default).
unsigned int dep_wait_polls();
// Records the status tcfft_get_last_error reports and the launch count
// tcfft_last_launch_count reports; returns s.
tcfftStatus record_status(tcfftStatus s, int launches);

}  // namespace tcfft
