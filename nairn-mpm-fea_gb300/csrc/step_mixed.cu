// step_mixed.cu -- step kernels of the mixed-precision transfer mode of a single-run context.
#include "step.cuh"

void nmg::enqueue_mixed(MpmGpuCtx *c, double t, int slot, bool det) {
    if (det) enqueue_prec<true, true>(c, t, slot);
    else enqueue_prec<true, false>(c, t, slot);
}
