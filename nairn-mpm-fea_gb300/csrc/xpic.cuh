// xpic.cuh -- PeriodicXPIC grid velocities (XPIC(k) and FMPM(k)): single-run
// contexts (any number of material velocity fields, with multimaterial
// contact) and batches (one field).
//
// XPICExtrapolationTask::Execute (NairnMPM/src/NairnMPM_Class/
// XPICExtrapolationTask.cpp:50-160) expands the grid velocity in k terms:
// from v*(prev) = the lumped velocity (FMPM: p/m; XPIC: (p - f dt)/m, with
// f dt/m added to v*), each pass forms v*(next) = S+S v*(prev), the particle
// double loop Sum_p (m_p S_ip / m_i) S_jp v*(prev)_j, takes Delta v = v*(prev)
// - v*(next), zeroes the velocity conditions' directions of Delta v and adds
// it to v* (MatVelocityField::XPICSupport, MatVelocityField.cpp:318-399).
// The result replaces the node velocity that the strain update (FMPM) or the
// particle update (both) reads.
//
// The double loop factors on the device: the particle first gathers
// Sum_j S_jp v*(prev)_j, then scatters m_p S_ip (1 / m_i) times it to each
// node i (1 / m_i kept per node).  It is the reference's sum in another
// order.  The FP64 mode sums in FP64; the mixed mode gathers and scatters
// FP32 copies (FP32 atomics) and keeps v*(prev), Delta v and v* in FP64.
//
// Every column is per field-node (field f of node n at f fstride + n); a
// particle's passes use its material's field.  With multimaterial contact the
// pass's Delta v is completed in three kernels: GET_DELTAV and the velocity
// conditions (k_xpic_delta with defer), the incremental contact of every
// contact node (k_xpic_contact), then UPDATE_VSTAR (k_xpic_apply).
#pragma once

namespace nmg {

// v*(prev) / Delta v, v*(next) and 1 / mass of each field-node, and the FP32
// copies of v*(prev) and v*(next) for the mixed mode's particle passes
struct DevXpic {
    double *px, *py, *pz;
    double *nx, *ny, *nz;
    double *rm;
    float *fpx, *fpy, *fpz;
    float *fnx, *fny, *fnz;
};

// Expansion phases: before a strain update (FMPM only) or before the
// particle update.  A run takes part in phase `phase` at pass k (init: k = 1)
// when its mode of this step has order >= k and >= 2 (FMPM for phase 0).  A
// single-run context reads the mode from StepParams, a batch run from its
// DevRun.
enum { XPIC_STRAIN = 0, XPIC_PARTICLE = 1 };

__device__ __forceinline__ bool xpic_takes_part(int mode, int phase, int k) {
    const int order = mode < 0 ? -mode : mode;
    if (order < 2 || order < k) return false;
    return phase == XPIC_PARTICLE || mode > 0;
}

// The field-node of this thread in a node pass over every field: field
// t / nnodes, node t % nnodes (nnodes: nodes per field in use), at array index
// n = field fstride + node.  False past the last one.
__device__ __forceinline__ bool xpic_field_node(const StepParams &sp, int nnodes, int &n, int &node) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * sp.ct.nf) return false;
    node = t % nnodes;
    n = (t / nnodes) * sp.ct.fstride + node;
    return true;
}

// v* into the velocity columns the particle kernels read (FP32 pairs too in
// the mixed mode)
template <bool MIX>
__device__ __forceinline__ void xpic_store_velocity(const DevNodes &nd, int n, const double v[3]) {
    nd.vx[n] = v[0];
    nd.vy[n] = v[1];
    nd.vz[n] = v[2];
    if (MIX) {
        split2(v[0], nd.vhx[n], nd.vlx[n]);
        split2(v[1], nd.vhy[n], nd.vly[n]);
        split2(v[2], nd.vhz[n], nd.vlz[n]);
    }
}

// INITIALIZE_XPIC from the node momentum (and, for XPIC, force)
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_xpic_init(StepParams sp, DevNodes nd, DevXpic x, int nnodes, int phase) {
    int n, node;
    if (!xpic_field_node(sp, nnodes, n, node) || !nd.active[n]) return;
    double t, dt;
    if (!node_run<BATCH>(sp, node, t, dt)) return;
    const int mode = BATCH ? sp.runs[sp.nrun[node]].xpic : sp.xpic;
    if (!xpic_takes_part(mode, phase, 1)) return;
    const bool fmpm = phase == XPIC_STRAIN || mode > 0;
    const double m = nd.mass[n];
    const double p[3] = {nd.px[n], nd.py[n], DIM == 3 ? nd.pz[n] : 0.};
    double vp[3], vs[3];
    if (fmpm) {
        const double r = 1. / m;
#pragma unroll
        for (int a = 0; a < 3; a++) vs[a] = vp[a] = p[a] * r;
    } else {
        const double f[3] = {nd.fx[n], nd.fy[n], DIM == 3 ? nd.fz[n] : 0.};
        const double r = 1. / m, s = dt / m;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            vp[a] = p[a];
            vp[a] += f[a] * (-dt);
            vp[a] *= r;
            vs[a] = vp[a];
            vs[a] += f[a] * s;
        }
    }
    x.px[n] = vp[0];
    x.py[n] = vp[1];
    x.pz[n] = vp[2];
    x.nx[n] = 0.;
    x.ny[n] = 0.;
    x.nz[n] = 0.;
    x.rm[n] = 1. / m;
    if (MIX) {
        x.fpx[n] = (float)vp[0];
        x.fpy[n] = (float)vp[1];
        x.fpz[n] = (float)vp[2];
        x.fnx[n] = 0.f;
        x.fny[n] = 0.f;
        x.fnz[n] = 0.f;
    }
    xpic_store_velocity<MIX>(nd, n, vs);
}

// XPICDoubleLoop (XPICExtrapolationTask.cpp:182-211) of one particle:
// v*(next)_i += m_p S_ip / m_i Sum_j S_jp v*(prev)_j
template <int DIM, int SHAPE, bool MIX, bool BATCH>
static __global__ void __launch_bounds__(256, kCpdi<SHAPE> ? 2 : 1)
    k_xpic_pass(StepParams sp, DevParticles p, DevXpic x, const DevMat *mats, int phase, int k) {
    using T = typename Wt<MIX>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    RunView rv;
    if (!particle_run<BATCH>(sp, p, i, rv)) return;
    if (!xpic_takes_part(BATCH ? sp.runs[p.run[i]].xpic : sp.xpic, phase, k)) return;
    const DevGrid &g = rv.g;
    const int nb = rv.nb + field_offset(sp, mats, p, i);
    T s[3] = {0, 0, 0};
    visit_nodes<DIM, SHAPE, false, T>(g, nb, p, i, [&](int n, T N, T, T, T) {
        if (zero_weight(N)) return;
        if (MIX) {
            s[0] += x.fpx[n] * N;
            s[1] += x.fpy[n] * N;
            if (DIM == 3) s[2] += x.fpz[n] * N;
        } else {
            s[0] += x.px[n] * N;
            s[1] += x.py[n] * N;
            if (DIM == 3) s[2] += x.pz[n] * N;
        }
    });
    const T mp = (T)p.mass[i];
    visit_nodes<DIM, SHAPE, false, T>(g, nb, p, i, [&](int n, T N, T, T, T) {
        if (zero_weight(N)) return;
        if (MIX) {
            // m_p S_ip s in FP32; the division by m_i is FP64, in k_xpic_delta (an
            // FP32 1/m_i overflows at nodes that only a support's edge reaches)
            const float w = mp * N;
            atomicAdd(&x.fnx[n], w * s[0]);
            atomicAdd(&x.fny[n], w * s[1]);
            if (DIM == 3) atomicAdd(&x.fnz[n], w * s[2]);
        } else {
            const double w = mp * N * x.rm[n];
            atomicAdd(&x.nx[n], w * s[0]);
            atomicAdd(&x.ny[n], w * s[1]);
            if (DIM == 3) atomicAdd(&x.nz[n], w * s[2]);
        }
    });
}

// GET_DELTAV, the velocity conditions' zero directions (NodalVelBC::
// GridVelocityConditions for the XPIC passes, NodalVelBC.cpp:327-334, and
// MatVelocityField::ZeroVelocityBC, MatVelocityField.cpp:530-541), UPDATE_VSTAR.
// defer: stop after the velocity conditions with Delta v in v*(prev), for the
// incremental contact and k_xpic_apply.
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_xpic_delta(StepParams sp, DevNodes nd, DevXpic x, int nnodes, DevBCs b,
                                    const int *bc_group, int phase, int k, int defer) {
    int n, node;
    if (!xpic_field_node(sp, nnodes, n, node) || !nd.active[n]) return;
    double t, dt;
    if (!node_run<BATCH>(sp, node, t, dt)) return;
    if (!xpic_takes_part(BATCH ? sp.runs[sp.nrun[node]].xpic : sp.xpic, phase, k)) return;
    double d[3];
    if (MIX) {
        const double rm = x.rm[n];
        d[0] = x.px[n] - (double)x.fnx[n] * rm;
        d[1] = x.py[n] - (double)x.fny[n] * rm;
        d[2] = DIM == 3 ? x.pz[n] - (double)x.fnz[n] * rm : 0.;
    } else {
        d[0] = x.px[n] - x.nx[n];
        d[1] = x.py[n] - x.ny[n];
        d[2] = DIM == 3 ? x.pz[n] - x.nz[n] : 0.;
    }
    const int grp = bc_group[node];
    if (grp >= 0) {
        for (int e = b.start[grp]; e < b.start[grp + 1]; e++) {
            if (t < b.ftime[e]) continue;
            const int dir = b.dir[e];
            const double nrm[3] = {dir == 1 ? 1. : 0., dir == 2 ? 1. : 0., dir == 4 ? 1. : 0.};
            const double dotn = d[0] * nrm[0] + d[1] * nrm[1] + d[2] * nrm[2];
#pragma unroll
            for (int a = 0; a < 3; a++) d[a] += nrm[a] * (-dotn);
        }
    }
    x.px[n] = d[0];
    x.py[n] = d[1];
    x.pz[n] = d[2];
    if (defer) {
        if (MIX) {
            x.fnx[n] = 0.f;
            x.fny[n] = 0.f;
            x.fnz[n] = 0.f;
        } else {
            x.nx[n] = 0.;
            x.ny[n] = 0.;
            x.nz[n] = 0.;
        }
        return;
    }
    const double v[3] = {nd.vx[n] + d[0], nd.vy[n] + d[1], DIM == 3 ? nd.vz[n] + d[2] : 0.};
    if (MIX) {
        x.fpx[n] = (float)d[0];
        x.fpy[n] = (float)d[1];
        x.fpz[n] = (float)d[2];
        x.fnx[n] = 0.f;
        x.fny[n] = 0.f;
        x.fnz[n] = 0.f;
    } else {
        x.nx[n] = 0.;
        x.ny[n] = 0.;
        x.nz[n] = 0.;
    }
    xpic_store_velocity<MIX>(nd, n, v);
}

// XPICExtrapolationTask::ImposeIncrementalContact (XPICExtrapolationTask.cpp:
// 246-258) for material contact: MaterialContactNode::NodalXPICIncrement ->
// CrackVelocityFieldMulti::MaterialXPICIncrementOnCVF (CrackVelocityFieldMulti.
// cpp:1333-1514), Coulomb friction, no rigid fields.  One thread per node with
// two or more fields: each field's Delta v (in v*(prev)) moves by the increment
// of the contact law applied to the node's cached contact state -- the
// momentum change toward the centre of mass of the Delta v's, accumulated over
// the passes in priorDelPiZero, less what earlier passes applied (netDelPi);
// with two fields the other moves by the opposite change.  The reference also
// moves the node force (XPIC's particle update only), which nothing after
// the expansion reads, so it is left out.
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_xpic_contact(StepParams sp, DevNodes nd, DevXpic x, int nnodes, int phase, int k) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes) return;
    double t, dt;
    if (!node_run<BATCH>(sp, n, t, dt)) return;
    if (!xpic_takes_part(BATCH ? sp.runs[sp.nrun[n]].xpic : sp.xpic, phase, k)) return;
    const DevContact ct = node_contact_params<BATCH>(sp, n);
    if (ct.nf < 2) return;
    const int S = ct.fstride;
    int nm = 0;
    for (int f = 0; f < ct.nf; f++) nm += nd.active[f * S + n] ? 1 : 0;
    if (nm <= 1) return;
    bool hasCOM = false;
    double Pc[3] = {0., 0., 0.}, Mc = 0.;
    for (int i = 0; i < ct.nf; i++) {
        const int ki = i * S + n;
        if (!nd.active[ki]) continue;
        const int pair = ct.xc_pair[ki];
        if (pair < -1) continue;  // no contact state from this step's last contact call
        const bool isPaired = pair >= 0;
        if (!hasCOM) {
            for (int f = 0; f < ct.nf; f++) {
                const int kk = f * S + n;
                if (!nd.active[kk]) continue;
                Pc[0] += x.px[kk] * nd.mass[kk];
                Pc[1] += x.py[kk] * nd.mass[kk];
                Pc[2] += x.pz[kk] * nd.mass[kk];
                Mc += nd.mass[kk];
            }
            hasCOM = true;
        }
        const double mi = nd.mass[ki];
        const double mred = mi * (1. - mi / Mc), r = mi / Mc;
        double delPi[3] = {Pc[0] * r, Pc[1] * r, Pc[2] * r};
        delPi[0] += x.px[ki] * -mi;
        delPi[1] += x.py[ki] * -mi;
        delPi[2] += x.pz[ki] * -mi;
        double *xc = ct.xc + kXcDoubles * (size_t)ki;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            delPi[a] += xc[4 + a];
            xc[4 + a] = delPi[a];
        }
        const double norm[3] = {xc[1], xc[2], xc[3]};
        const double dotn = dot3(delPi, norm);
        const double dfi[3] = {xc[10], xc[11], xc[12]};
        if (!coulomb_delta(ct, delPi, norm, dotn, xc[0], mred, dfi, dt)) {
            // out of contact now: undo what earlier passes applied, if anything
            const bool zero = xc[7] == 0. && xc[8] == 0. && (DIM == 2 || xc[9] == 0.);
            if (zero) {
                if (isPaired) break;
                continue;
            }
            delPi[0] = delPi[1] = delPi[2] = 0.;
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double net = delPi[a];
            delPi[a] -= xc[7 + a];
            xc[7 + a] = net;
        }
        const double rm = 1. / mi;
        x.px[ki] += delPi[0] * rm;
        x.py[ki] += delPi[1] * rm;
        x.pz[ki] += delPi[2] * rm;
        if (isPaired) {
            const int kj = pair * S + n;
            const double rmj = -1. / nd.mass[kj];
            x.px[kj] += delPi[0] * rmj;
            x.py[kj] += delPi[1] * rmj;
            x.pz[kj] += delPi[2] * rmj;
            break;
        }
    }
}

// UPDATE_VSTAR after the incremental contact: v* += Delta v, and the FP32
// copy of Delta v for the next pass (mixed mode)
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_xpic_apply(StepParams sp, DevNodes nd, DevXpic x, int nnodes, int phase, int k) {
    int n, node;
    if (!xpic_field_node(sp, nnodes, n, node) || !nd.active[n]) return;
    double t, dt;
    if (!node_run<BATCH>(sp, node, t, dt)) return;
    if (!xpic_takes_part(BATCH ? sp.runs[sp.nrun[node]].xpic : sp.xpic, phase, k)) return;
    const double d[3] = {x.px[n], x.py[n], DIM == 3 ? x.pz[n] : 0.};
    if (MIX) {
        x.fpx[n] = (float)d[0];
        x.fpy[n] = (float)d[1];
        x.fpz[n] = (float)d[2];
    }
    const double v[3] = {nd.vx[n] + d[0], nd.vy[n] + d[1], DIM == 3 ? nd.vz[n] + d[2] : 0.};
    xpic_store_velocity<MIX>(nd, n, v);
}

}  // namespace nmg
