// step_mixed_2d_det.cu -- the single-run step of 2D contexts with mixed-precision transfers and
// deterministic node sums (one instantiation per translation unit, so the library
// builds in parallel).
#include "step.cuh"

template void nmg::enqueue_dim<2, true, true>(MpmGpuCtx *c, double t, int slot);
