// step.cuh -- the kernel sequence of one explicit step of a single-run
// context, included by the step_<precision>_<dim>_<sums>.cu translation units.
#pragma once

#include "context.cuh"

namespace nmg {
namespace {

// One step on the context stream.  DET: deterministic node sums -- each
// scatter is preceded by a pass that bounds its contributions (k_det_bounds,
// k_strain_forces and k_g2p in their DET forms) and followed by k_det_resolve,
// which writes the sums into the node columns.
template <int DIM, int SHAPE, bool MIX, bool DET>
void enqueue_step(MpmGpuCtx *c, double t, int slot) {
    const int n = c->p.n, NN = c->g.nnodes;
    const int TB = 256;
    const int pb = (n + TB - 1) / TB, nb = (NN + TB - 1) / TB;
    const double dt = c->opts.timestep;
    const int method = c->opts.method;
    const double stFirst = method == MPMGPU_USAVG ? c->opts.fraction_usf * dt : dt;
    const double stLast = method == MPMGPU_USAVG ? dt - stFirst : dt;
    cudaStream_t s = c->stream;
    auto mark = [&](int k, bool begin) {
        if (c->profile) cudaEventRecord(event_at(c, slot, k, begin), s);
        if (!begin) c->launches++;
    };
    cudaMemsetAsync(c->nblock, 0, c->nblock_zero_bytes, s);
    cudaMemsetAsync(c->nd.active, 0, (size_t)NN * c->ct.nf, s);
    if (MIX) cudaMemsetAsync(c->fblock, 0, c->fblock_zero_bytes, s);
    StepParams sp;
    sp.ct = c->ct;
    sp.g = c->g;
    sp.dt = dt;
    sp.st_first = stFirst;
    sp.st_last = stLast;
    sp.t = t;
    sp.err = c->err;
    sp.runs = nullptr;
    sp.nrun = nullptr;
    sp.det = c->det;
    // PeriodicXPIC: this step's order (steps counted from 1 at time 0)
    const int xm = xpic_step_order(c->opts, (long long)llround(t / dt) + 1);
    sp.xpic = xm;
    const int xk = xm < 0 ? -xm : xm;
    const DevXpic xp = c->xpic;
    // XPIC(k)/FMPM(k) expansion of the node velocities (k > 1)
    // (every field-node; with contact, each pass's Delta v also takes the
    // incremental contact of the contact nodes)
    const bool xcontact = c->ct.nf > 1;
    sp.ct.xcache = xk > 1 && xcontact ? 1 : 0;
    if (sp.ct.xcache)  // this step's contact state: none yet
        cudaMemsetAsync(c->ct.xc_pair, 0x80, (size_t)NN * c->ct.nf * sizeof(int), s);
    auto xpic_expand = [&](int phase) {
        const int XN = NN * c->ct.nf, xb = (XN + TB - 1) / TB;  // every field-node
        k_xpic_init<DIM, MIX, false><<<xb, TB, 0, s>>>(sp, c->nd, xp, NN, phase);
        c->launches++;
        for (int k = 2; k <= xk; k++) {
            k_xpic_pass<DIM, SHAPE, MIX, false><<<pb, TB, 0, s>>>(sp, c->p, xp, c->mats, phase, k);
            k_xpic_delta<DIM, MIX, false><<<xb, TB, 0, s>>>(sp, c->nd, xp, NN, c->bcs, c->bc_group, phase, k,
                                                            xcontact ? 1 : 0);
            c->launches += 2;
            if (xcontact) {
                k_xpic_contact<DIM, MIX, false><<<nb, TB, 0, s>>>(sp, c->nd, xp, NN, phase, k);
                k_xpic_apply<DIM, MIX, false><<<xb, TB, 0, s>>>(sp, c->nd, xp, NN, phase, k);
                c->launches += 2;
            }
        }
    };
    const int NT = NN * c->ct.nf, ntb = (NT + TB - 1) / TB;
    mark(0, true);
    if (DET) {
        cudaMemsetAsync(c->det.bnd, 0, kDetBounds * sizeof(unsigned long long), s);
        cudaMemsetAsync(c->det.nbnd, 0, (size_t)NT * sizeof(unsigned long long), s);
        k_det_bounds<DIM, SHAPE, MIX><<<pb, TB, 0, s>>>(sp, c->p, c->mats);
    }
    // mixed mode, one material field, window shape functions: the scatters
    // accumulate in shared-memory node tiles (unless MPMGPU_P2G_UNTILED)
    constexpr bool kTileable = MIX && !DET && !kCpdi<SHAPE>;
    const bool tile = kTileable && c->ct.nf == 1 && c->opts.p2g != MPMGPU_P2G_UNTILED;
    if constexpr (kTileable) {
        if (tile) k_p2g_tile<DIM, SHAPE, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd);
        else k_p2g<DIM, SHAPE, MIX, false, DET><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
    } else {
        k_p2g<DIM, SHAPE, MIX, false, DET><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
    }
    if (DET) {
        k_det_resolve<DIM, MIX><<<ntb, TB, 0, s>>>(sp, c->nd, NT, 0);
        c->launches += 2;
    }
    const bool lr = c->ct.nf > 1 && c->ct.normals >= 5;
    auto lr_normals = [&](int supports_only) {
        k_lr_normals<DIM, false><<<lr_loop_blocks((long long)NN * c->ct.nf, TB), TB, 0, s>>>(
            sp, c->p, c->nd, c->mats, c->lr_start, c->lr_list, c->lr_cnt, c->lr_out, NN, c->lr_cap,
            c->ct.normals == 6 ? 1 : 0, supports_only);
        c->launches++;
    };
    if (lr) {
        // link the particles to the contact nodes, in the particles' host order
        const int m = NN + 1, nsb = (m + kScanChunk - 1) / kScanChunk;
        cudaMemsetAsync(c->lr_cnt, 0, (size_t)m * sizeof(int), s);
        k_lr_link<DIM, SHAPE, MIX, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->lr_cnt, c->lr_start, c->lr_list,
                                                            c->lr_cap, 0);
        cudaMemcpyAsync(c->lr_start, c->lr_cnt, (size_t)m * sizeof(int), cudaMemcpyDeviceToDevice, s);
        k_scan_reduce<<<nsb, kScanBlock, 0, s>>>(c->lr_start, m, c->lr_sums);
        k_scan_sums<<<1, kScanBlock, 0, s>>>(c->lr_sums, nsb);
        k_scan_apply<<<nsb, kScanBlock, 0, s>>>(c->lr_start, m, c->lr_sums);
        cudaMemsetAsync(c->lr_cnt, 0, (size_t)m * sizeof(int), s);
        k_lr_link<DIM, SHAPE, MIX, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->lr_cnt, c->lr_start, c->lr_list,
                                                            c->lr_cap, 1);
        // the nodes with links, listed in c->lr_cnt (no longer needed as the cursor)
        cudaMemsetAsync(c->lr_cnt + NN, 0, sizeof(int), s);
        k_lr_compact<<<(NN + TB - 1) / TB, TB, 0, s>>>(c->lr_start, c->lr_cnt, NN);
        k_lr_order<<<lr_loop_blocks(NN, TB), TB, 0, s>>>(c->lr_start, c->lr_list, c->orig, c->lr_cnt, NN, c->lr_cap);
        c->launches += 7;
        lr_normals(0);
    }
    mark(0, false);
    mark(1, true);
    k_node_post<DIM, MIX, false><<<nb, TB, 0, s>>>(sp, c->nd, NN, c->bcs, c->bc_group, method != MPMGPU_USL);
    mark(1, false);
    mark(2, true);
    if (xm > 1 && method != MPMGPU_USL) xpic_expand(XPIC_STRAIN);  // FMPM(k) velocities of the first strain update
    bool forces_done = false;
    if constexpr (kTileable) {
        if (tile) {
            if (method == MPMGPU_USL)
                k_strain_forces_tile<DIM, SHAPE, false, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
            else
                k_strain_forces_tile<DIM, SHAPE, true, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
            forces_done = true;
        }
    }
    if (!forces_done) {
        if (method == MPMGPU_USL)
            k_strain_forces<DIM, SHAPE, false, MIX, false, DET><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
        else
            k_strain_forces<DIM, SHAPE, true, MIX, false, DET><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
    }
    if (DET) {
        k_det_forces<DIM, SHAPE, MIX><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
        k_det_resolve<DIM, MIX><<<ntb, TB, 0, s>>>(sp, c->nd, NT, 1);
        c->launches += 2;
    }
    mark(2, false);
    mark(3, true);
    if (lr) lr_normals(1);  // same positions, deformed radii changed with the strain update
    k_node_update<DIM, MIX, false><<<nb, TB, 0, s>>>(sp, c->nd, NN, c->bcs, c->bc_group,
                                                     c->ct.nf > 1 && method != MPMGPU_USF, xk > 1 ? 0 : 1);
    mark(3, false);
    mark(4, true);
    if (xk > 1) xpic_expand(XPIC_PARTICLE);  // v(k) of the particle update
    if (method == MPMGPU_USF) {
        k_g2p<DIM, SHAPE, false, MIX, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
        mark(4, false);
        return;
    }
    bool g2p_done = false;
    if constexpr (kTileable) {
        if (tile) {
            k_g2p_tile<DIM, SHAPE, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd);
            g2p_done = true;
        }
    }
    if (!g2p_done) k_g2p<DIM, SHAPE, true, MIX, false, DET><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
    if (DET) {
        k_det_usl<DIM, SHAPE, MIX><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
        k_det_resolve<DIM, MIX><<<ntb, TB, 0, s>>>(sp, c->nd, NT, 2);
        c->launches += 2;
    }
    mark(4, false);
    mark(5, true);
    if (lr) lr_normals(0);  // the particles moved
    k_node_usl<DIM, MIX, false><<<nb, TB, 0, s>>>(sp, c->nd, NN, c->bcs, c->bc_group);
    mark(5, false);
    mark(6, true);
    if (xm > 1) xpic_expand(XPIC_STRAIN);  // FMPM(k) velocities of the second strain update
    k_strain_last<DIM, SHAPE, MIX, false><<<pb, TB, 0, s>>>(sp, c->p, c->nd, c->mats);
    mark(6, false);
}

}  // namespace

// one step of a context of dimension DIM, transfer precision MIX and node-sum
// mode DET, for its shape-function option; each combination is instantiated
// in its own translation unit (step_<precision>_<dim>_<sums>.cu)
template <int DIM, bool MIX, bool DET>
void enqueue_dim(MpmGpuCtx *c, double t, int slot) {
    const int shape = c->opts.shape;
    if (shape == MPMGPU_SHAPE_LINEAR) enqueue_step<DIM, SHAPE_LINEAR, MIX, DET>(c, t, slot);
    else if (shape == MPMGPU_SHAPE_LCPDI) enqueue_step<DIM, SHAPE_LCPDI, MIX, DET>(c, t, slot);
    else if (shape == MPMGPU_SHAPE_QCPDI) {
        if constexpr (DIM == 2) enqueue_step<DIM, SHAPE_QCPDI, MIX, DET>(c, t, slot);  // refused in 3D at create
    }
    else if (shape == MPMGPU_SHAPE_BSPLINE) enqueue_step<DIM, SHAPE_BSPLINE, MIX, DET>(c, t, slot);
    else if (shape == MPMGPU_SHAPE_BGIMP) enqueue_step<DIM, SHAPE_BGIMP, MIX, DET>(c, t, slot);
    else enqueue_step<DIM, SHAPE_UGIMP, MIX, DET>(c, t, slot);
}

}  // namespace nmg
