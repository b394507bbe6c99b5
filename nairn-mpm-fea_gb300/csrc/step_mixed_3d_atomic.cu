// step_mixed_3d_atomic.cu -- the single-run step of 3D contexts with mixed-precision transfers and
// atomic node sums (one instantiation per translation unit, so the library
// builds in parallel).
#include "step.cuh"

template void nmg::enqueue_dim<3, true, false>(MpmGpuCtx *c, double t, int slot);
