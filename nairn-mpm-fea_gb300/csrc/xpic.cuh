// xpic.cuh -- PeriodicXPIC grid velocities (XPIC(k) and FMPM(k)) of a
// single-run context with one material velocity field.
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
#pragma once

namespace nmg {

// v*(prev) / Delta v, v*(next) and 1 / mass of each node (single material
// field), and their FP32 copies of the mixed mode's particle passes
struct DevXpic {
    double *px, *py, *pz;
    double *nx, *ny, *nz;
    double *rm;
    float *fpx, *fpy, *fpz;
    float *fnx, *fny, *fnz;
    float *frm;
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
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes || !nd.active[n]) return;
    double t, dt;
    if (!node_run<BATCH>(sp, n, t, dt)) return;
    const int mode = BATCH ? sp.runs[sp.nrun[n]].xpic : sp.xpic;
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
        x.frm[n] = (float)(1. / m);
    }
    xpic_store_velocity<MIX>(nd, n, vs);
}

// XPICDoubleLoop (XPICExtrapolationTask.cpp:182-211) of one particle:
// v*(next)_i += m_p S_ip / m_i Sum_j S_jp v*(prev)_j
template <int DIM, int SHAPE, bool MIX, bool BATCH>
static __global__ void __launch_bounds__(256, SHAPE == SHAPE_LCPDI ? 2 : 1)
    k_xpic_pass(StepParams sp, DevParticles p, DevXpic x, int phase, int k) {
    using T = typename Wt<MIX>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    RunView rv;
    if (!particle_run<BATCH>(sp, p, i, rv)) return;
    if (!xpic_takes_part(BATCH ? sp.runs[p.run[i]].xpic : sp.xpic, phase, k)) return;
    const DevGrid &g = rv.g;
    T s[3] = {0, 0, 0};
    visit_nodes<DIM, SHAPE, false, T>(g, rv.nb, p, i, [&](int n, T N, T, T, T) {
        if (N == T(0)) return;
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
    visit_nodes<DIM, SHAPE, false, T>(g, rv.nb, p, i, [&](int n, T N, T, T, T) {
        if (N == T(0)) return;
        if (MIX) {
            const float w = mp * N * x.frm[n];
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
// MatVelocityField::ZeroVelocityBC, MatVelocityField.cpp:530-541), UPDATE_VSTAR
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_xpic_delta(StepParams sp, DevNodes nd, DevXpic x, int nnodes, DevBCs b,
                                    const int *bc_group, int phase, int k) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes || !nd.active[n]) return;
    double t, dt;
    if (!node_run<BATCH>(sp, n, t, dt)) return;
    if (!xpic_takes_part(BATCH ? sp.runs[sp.nrun[n]].xpic : sp.xpic, phase, k)) return;
    double d[3];
    if (MIX) {
        d[0] = x.px[n] - (double)x.fnx[n];
        d[1] = x.py[n] - (double)x.fny[n];
        d[2] = DIM == 3 ? x.pz[n] - (double)x.fnz[n] : 0.;
    } else {
        d[0] = x.px[n] - x.nx[n];
        d[1] = x.py[n] - x.ny[n];
        d[2] = DIM == 3 ? x.pz[n] - x.nz[n] : 0.;
    }
    const int grp = bc_group[n];
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
    const double v[3] = {nd.vx[n] + d[0], nd.vy[n] + d[1], DIM == 3 ? nd.vz[n] + d[2] : 0.};
    x.px[n] = d[0];
    x.py[n] = d[1];
    x.pz[n] = d[2];
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

}  // namespace nmg
