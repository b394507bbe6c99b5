// step_mixed_3d_det.cu -- the single-run step of 3D contexts with mixed-precision transfers and
// deterministic node sums (one instantiation per translation unit, so the library
// builds in parallel).
#include "step.cuh"

template void nmg::enqueue_dim<3, true, true>(MpmGpuCtx *c, double t, int slot);
