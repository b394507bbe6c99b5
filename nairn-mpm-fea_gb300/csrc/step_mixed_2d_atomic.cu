// step_mixed_2d_atomic.cu -- the single-run step of 2D contexts with mixed-precision transfers and
// atomic node sums (one instantiation per translation unit, so the library
// builds in parallel).
#include "step.cuh"

template void nmg::enqueue_dim<2, true, false>(MpmGpuCtx *c, double t, int slot);
