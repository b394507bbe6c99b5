// step_fp64.cu -- step kernels of the FP64 transfer mode of a single-run context.
#include "step.cuh"

void nmg::enqueue_fp64(MpmGpuCtx *c, double t, int slot, bool det) {
    if (det) enqueue_prec<false, true>(c, t, slot);
    else enqueue_prec<false, false>(c, t, slot);
}
