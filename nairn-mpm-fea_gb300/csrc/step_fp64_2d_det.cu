// step_fp64_2d_det.cu -- the single-run step of 2D contexts with FP64 transfers and
// deterministic node sums (one instantiation per translation unit, so the library
// builds in parallel).
#include "step.cuh"

template void nmg::enqueue_dim<2, false, true>(MpmGpuCtx *c, double t, int slot);
