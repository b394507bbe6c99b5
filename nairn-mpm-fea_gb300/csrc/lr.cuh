// lr.cuh -- regression contact normals (MeshInfo LINEAR_REGRESSION 5 and
// LOGISTIC_REGRESSION 6, the reference's default normal method).
//
// MaterialContactNode::GetMaterialContactData (NairnMPM/src/Nodes/
// MaterialContactNode.cpp:238-353) links each particle to the contact nodes
// (nodes with particles of two or more materials) among its shape-function
// nodes, once per step at the first extrapolation.  At every contact pass
// CrackVelocityFieldMulti::LinearRegressionNormal / LogisticRegressionNormal
// (MachineLearning.cpp:58-620) then fit, per contact node and material, a
// plane separating that material's linked particles from the others' (other
// materials lumped), and take the separation of the two point clouds along
// its normal from their supports through the particles' deformed radii.
//
// Device layout: link counts and offsets by grid node, the links as particle
// slots sorted by the particles' host order (the reference's particle order),
// and the result (nx, ny, nz, deln) per material field of each node.  One warp
// per node does the regressions; its sums over the linked particles are warp
// reductions.  In a batch (BATCH = true) the nodes and particles of runs with
// other normal methods have no links, and a node's particles all belong to the
// node's run, so host order is the run's upload order.
#pragma once

namespace nmg {

// the node has particles of two or more material fields
__device__ __forceinline__ bool lr_contact_node(const StepParams &sp, const DevNodes &nd, int n) {
    int nm = 0;
    for (int f = 0; f < sp.ct.nf; f++) nm += nd.active[f * sp.ct.fstride + n] ? 1 : 0;
    return nm > 1;
}

// the distinct contact nodes among the shape-function nodes of particle i
// with nonzero weight (the contact test first: most nodes are not contact
// nodes, so few reach the duplicate search)
template <int DIM, int SHAPE, bool MIX>
__device__ __forceinline__ int lr_particle_nodes(const StepParams &sp, const DevNodes &nd, const DevGrid &g, int nb,
                                                 const DevParticles &p, int i, int out[64]) {
    using T = typename Wt<MIX>::T;
    int cnt = 0;
    visit_nodes<DIM, SHAPE, false, T>(g, nb, p, i, [&](int n, T N, T, T, T) {
        if (zero_weight(N)) return;
        if (!lr_contact_node(sp, nd, n)) return;
        for (int k = 0; k < cnt; k++)
            if (out[k] == n) return;
        if (cnt < 64) out[cnt++] = n;
    });
    return cnt;
}

// pass 0 counts the links of each contact node; pass 1 writes them at the
// node's offset (cnt cleared in between serves as the cursor).  Links past
// `cap` are dropped and fail the particle's run with ERR_RANGE.
template <int DIM, int SHAPE, bool MIX, bool BATCH>
static __global__ void __launch_bounds__(256) k_lr_link(StepParams sp, DevParticles p, DevNodes nd, int *cnt,
                                                        const int *start, int *list, long long cap, int pass) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    RunView rv;
    if (!particle_run<BATCH>(sp, p, i, rv)) return;
    if (BATCH && sp.runs[p.run[i]].normals < 5) return;
    int nodes[64];
    const int m = lr_particle_nodes<DIM, SHAPE, MIX>(sp, nd, rv.g, rv.nb, p, i, nodes);
    for (int k = 0; k < m; k++) {
        const int n = nodes[k];
        const int slot = atomicAdd(cnt + n, 1);
        if (pass == 1) {
            const long long at = (long long)start[n] + slot;
            if (at < cap) list[at] = i;
            else atomicOr(rv.err, ERR_RANGE);
        }
    }
}

// The nodes with links, in no particular order, at nodes[0 .. nodes[nnodes]):
// the regression kernels below run warps over these contact nodes only (a
// few per cent of the grid) instead of over every node.  nodes[nnodes] must
// be zero on entry.
static __global__ void k_lr_compact(const int *start, int *nodes, int nnodes) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes || start[n + 1] == start[n]) return;
    nodes[atomicAdd(nodes + nnodes, 1)] = n;
}

// grid of the warp loops over contact nodes: enough warps to fill the GPU,
// never more than the work
constexpr int kLrMaxBlocks = 4096;
inline int lr_loop_blocks(long long warps, int threads) {
    const long long b = (warps * 32 + threads - 1) / threads;
    return (int)std::max<long long>(1, std::min<long long>(b, kLrMaxBlocks));
}

// each node's links in the particles' host order: one warp per contact node
// ranks its links by host index in shared memory (host indices are distinct
// within a node, whose particles all belong to one run); lists longer than
// the shared-memory slice are sorted by insertion by one lane
constexpr int kLrSortCap = 256;
static __global__ void __launch_bounds__(256) k_lr_order(const int *start, int *list, const int *orig,
                                                         const int *nodes, int nnodes, long long cap) {
    __shared__ int skey[8][kLrSortCap], sval[8][kLrSortCap];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nc = nodes[nnodes];
    const int nw = (int)(((long long)gridDim.x * blockDim.x) >> 5);
    for (int c = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < nc; c += nw) {
        const int n = nodes[c];
        const int s0 = start[n], s1 = start[n + 1], L = s1 - s0;
        if (L < 2 || s1 > cap) continue;  // nothing to order, or dropped links (the run has failed)
        if (L > kLrSortCap) {
            if (lane == 0)
                for (int k = s0 + 1; k < s1; k++) {
                    const int v = list[k], key = orig[v];
                    int j = k - 1;
                    while (j >= s0 && orig[list[j]] > key) {
                        list[j + 1] = list[j];
                        --j;
                    }
                    list[j + 1] = v;
                }
            __syncwarp();
            continue;
        }
        for (int k = lane; k < L; k += 32) {
            const int v = list[s0 + k];
            sval[w][k] = v;
            skey[w][k] = orig[v];
        }
        __syncwarp();
        for (int k = lane; k < L; k += 32) {
            const int key = skey[w][k];
            int rank = 0;
            for (int j = 0; j < L; j++) rank += skey[w][j] < key ? 1 : 0;
            list[s0 + rank] = sval[w][k];
        }
        __syncwarp();  // the slice is rewritten by the warp's next node
    }
}

__device__ __forceinline__ double lr_wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double lr_wmin(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Inverses of the symmetric regression matrices by cofactors, each entry's
// cofactor and quotient taken by its own lane of the warp (lane l and l + 16
// or l + 9k hold entry l), then the whole inverse handed to every lane.  The
// FP64 pipe is the bound: one quotient per lane instead of 16 (9) per lane.
constexpr unsigned kFullWarp = 0xffffffffu;

// the symmetric 3x3 (a b c; b d e; c e f)
__device__ __forceinline__ void lr_inv3_warp(const double m[6], double r[9], int lane) {
    const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5];
    const double c00 = d * f - e * e, c01 = -(b * f - c * e), c02 = b * e - c * d;
    const double det = a * c00 + b * c01 + c * c02;
    const double c11 = a * f - c * c, c12 = -(a * e - b * c), c22 = a * d - b * b;
    const double cof[9] = {c00, c01, c02, c01, c11, c12, c02, c12, c22};
    const double q = cof[lane % 9] / det;
#pragma unroll
    for (int k = 0; k < 9; k++) r[k] = __shfl_sync(kFullWarp, q, k);
}

// the symmetric 4x4 whose upper triangle is mt (00 01 02 03 11 12 13 22 23 33)
__device__ __forceinline__ void lr_inv4_warp(const double mt[10], double r[16], int lane) {
    const double m[16] = {mt[0], mt[1], mt[2], mt[3], mt[1], mt[4], mt[5], mt[6],
                          mt[2], mt[5], mt[7], mt[8], mt[3], mt[6], mt[8], mt[9]};
    // cofactor (i, j): the minor without row i and column j
    const int i = (lane >> 2) & 3, j = lane & 3;
    const int a0 = i == 0 ? 1 : 0, a1 = i <= 1 ? 2 : 1, a2 = i <= 2 ? 3 : 2;
    const int b0 = j == 0 ? 1 : 0, b1 = j <= 1 ? 2 : 1, b2 = j <= 2 ? 3 : 2;
    const double s3[3][3] = {{m[4 * a0 + b0], m[4 * a0 + b1], m[4 * a0 + b2]},
                             {m[4 * a1 + b0], m[4 * a1 + b1], m[4 * a1 + b2]},
                             {m[4 * a2 + b0], m[4 * a2 + b1], m[4 * a2 + b2]}};
    const double d3 = s3[0][0] * (s3[1][1] * s3[2][2] - s3[1][2] * s3[2][1]) -
                      s3[0][1] * (s3[1][0] * s3[2][2] - s3[1][2] * s3[2][0]) +
                      s3[0][2] * (s3[1][0] * s3[2][1] - s3[1][1] * s3[2][0]);
    const double cof = ((i + j) & 1) ? -d3 : d3;
    double c0[4];
#pragma unroll
    for (int k = 0; k < 4; k++) c0[k] = __shfl_sync(kFullWarp, cof, k);
    const double det = m[0] * c0[0] + m[1] * c0[1] + m[2] * c0[2] + m[3] * c0[3];
    // inverse entry (i, j) = cofactor (j, i) / det
    const double q = __shfl_sync(kFullWarp, cof, 4 * j + i) / det;
#pragma unroll
    for (int k = 0; k < 16; k++) r[k] = __shfl_sync(kFullWarp, q, k);
}

// MatPoint2D/3D::GetDeformedRadius, ellipse method (MatPoint2D.cpp:482-495,
// MatPoint3D.cpp:497-510): distance from the particle centre to its deformed
// inscribed ellipse(oid) along the unit vector n (semi sizes 0.5 lp cell)
template <int DIM>
__device__ __forceinline__ double lr_radius(const DevGrid &g, const DevParticles &p, int q, const double *n) {
    const double px = 0.5 * p.lpx[q] * g.gx, py = 0.5 * p.lpy[q] * g.gy;
    const double F00 = 1. + p.exx[q], F11 = 1. + p.eyy[q];
    const double F01 = 0.5 * (p.exy[q] - p.wxy[q]), F10 = 0.5 * (p.exy[q] + p.wxy[q]);
    if (DIM == 2) {
        const double rdet = 1. / (F00 * F11 - F01 * F10);
        const double n0x = (F11 * n[0] - F10 * n[1]) * rdet;
        const double n0y = (-F01 * n[0] + F00 * n[1]) * rdet;
        return 1. / sqrt(n0x * n0x / (px * px) + n0y * n0y / (py * py));
    }
    const double pz = 0.5 * p.lpz[q] * g.gz;
    const double F22 = 1. + p.ezz[q];
    const double F02 = 0.5 * (p.exz[q] - p.wxz[q]), F20 = 0.5 * (p.exz[q] + p.wxz[q]);
    const double F12 = 0.5 * (p.eyz[q] - p.wyz[q]), F21 = 0.5 * (p.eyz[q] + p.wyz[q]);
    const double c00 = F11 * F22 - F12 * F21, c01 = F12 * F20 - F10 * F22, c02 = F10 * F21 - F11 * F20;
    const double det = F00 * c00 + F01 * c01 + F02 * c02;
    const double n0x = (c00 * n[0] + (F02 * F21 - F01 * F22) * n[1] + (F01 * F12 - F02 * F11) * n[2]) / det;
    const double n0y = (c01 * n[0] + (F00 * F22 - F02 * F20) * n[1] + (F02 * F10 - F00 * F12) * n[2]) / det;
    const double n0z = (c02 * n[0] + (F01 * F20 - F00 * F21) * n[1] + (F00 * F11 - F01 * F10) * n[2]) / det;
    return 1. / sqrt(n0x * n0x / (px * px) + n0y * n0y / (py * py) + n0z * n0z / (pz * pz));
}

// Separation of the two point clouds of a node along the unit normal nrm: the
// supports of material field a's linked particles and of the others', each
// through the particles' deformed radii (every lane of the warp calls this and
// gets the warp's result).
template <int DIM>
__device__ __forceinline__ double lr_supports(const DevGrid &g, const DevParticles &p, const DevMat *mats,
                                              const int *list, int s0, int s1, int a, const double nrm[3]) {
    double supA = 1.e30, supB = 1.e30;
    for (int k = s0 + (int)(threadIdx.x & 31); k < s1; k += 32) {
        const int q = list[k];
        const double xp[3] = {p.x[q], p.y[q], DIM == 3 ? p.z[q] : 0.};
        const double r = lr_radius<DIM>(g, p, q, nrm);
        const double d = nrm[0] * xp[0] + nrm[1] * xp[1] + nrm[2] * xp[2];
        if (mats[p.mat[q]].field == a) supA = fmin(supA, -d - r);
        else supB = fmin(supB, d - r);
    }
    return lr_wmin(supA) + lr_wmin(supB);
}

// One warp per grid node with links and material field present: the
// regression normal against the other materials lumped and the separation
// deln, written as (nx, ny, nz, deln) at out[4 (f fstride + n)].  Constants
// of MachineLearning.cpp with PENALIZE_NORMALS: linear offset penalty 0.1;
// logistic normal penalty 1e-7 cell^2, no offset penalty, the linear beta
// doubled as the start, convergence 1 - cos < 1e-5 within 15 iterations.
//
// supports_only: the particles have not moved since the last full pass (the
// momentum-update pass follows the mass-and-momentum pass with only the
// strain update in between), so the regression -- a function of the linked
// particles' positions and materials alone -- would give the same normal bit
// for bit; only the supports, whose deformed radii follow the strain update,
// are taken again, along the stored normal.
template <int DIM, bool BATCH>
__device__ __forceinline__ void lr_node_field(const StepParams &sp, const DevParticles &p, const DevNodes &nd,
                                              const DevMat *mats, const int *start, const int *list, double *out,
                                              int n, int a0, long long cap, int logistic, int supports_only) {
    const int lane = threadIdx.x & 31;
    const int s0 = start[n], s1 = start[n + 1];
    if (s1 == s0 || s1 > cap) return;
    {
        // a node with two materials applies the law once, from its first
        // active field (the pair, MaterialContactOnCVF's doingPairs), so only
        // that field's normal is ever read
        int nm = 0, first = -1;
        for (int f = 0; f < sp.ct.nf; f++)
            if (nd.active[f * sp.ct.fstride + n]) {
                if (first < 0) first = f;
                nm++;
            }
        if (nm == 2 && a0 != first) return;
    }
    DevGrid g = sp.g;
    int nl = n;  // the node's index in its grid
    if (BATCH) {
        const int r = sp.nrun[n];
        if (r < 0) return;
        const DevRun &R = sp.runs[r];
        if (!R.active || R.normals < 5) return;
        g = R.g;
        nl = n - R.node_base;
        logistic = R.normals == 6 ? 1 : 0;
    }
    if (supports_only) {
        const int ka = a0 * sp.ct.fstride + n;
        if (!nd.active[ka]) return;
        const double *o = out + 4 * (size_t)ka;
        const double nrm[3] = {o[0], o[1], o[2]};
        const double dn = lr_supports<DIM>(g, p, mats, list, s0, s1, a0, nrm);
        if (lane == 0) out[4 * (size_t)ka + 3] = dn;
        return;
    }
    const int nx1 = g.nx + 1, ny1 = g.ny + 1;
    const double ndx = g.xn[nl % nx1], ndy = g.yn[(nl / nx1) % ny1], ndz = DIM == 3 ? g.zn[nl / (nx1 * ny1)] : 0.;
    double cell = fmin(g.gx, g.gy);
    if (DIM == 3) cell = fmin(cell, g.gz);
    const double cell2 = cell * cell;
    const double offsetLin = 0.1, normLog = 1.e-7, offsetLog = 0., tol = 1.e-5;
    const int maxIter = 15;
    constexpr int NB = DIM == 3 ? 4 : 3, NM = DIM == 3 ? 10 : 6;
    // the lane's first kLrCached linked particles (positions relative to the
    // node and material field) stay in registers through all the regression
    // steps; longer lists read the rest from memory at each step
    constexpr int kLrCached = 4;
    double cx[kLrCached], cy[kLrCached], cz[kLrCached];
    int cf[kLrCached];
#pragma unroll
    for (int r = 0; r < kLrCached; r++) {
        const int k = s0 + lane + 32 * r;
        cx[r] = cy[r] = cz[r] = 0.;
        cf[r] = -1;
        if (k < s1) {
            const int q = list[k];
            cf[r] = mats[p.mat[q]].field;
            cx[r] = p.x[q] - ndx;
            cy[r] = p.y[q] - ndy;
            cz[r] = DIM == 3 ? p.z[q] - ndz : 0.;
        }
    }
    for (int a = a0; a <= a0; a++) {  // this warp's field
        const int ka = a * sp.ct.fstride + n;
        if (!nd.active[ka]) continue;
        double nrm[3] = {0., 0., 0.};
        double mt[NM], rhs[NB], lam[NB], beta[NB] = {};  // beta is set by the linear step first
        const double pen = logistic ? normLog * cell2 : 0.;
#pragma unroll
        for (int k = 0; k < NB; k++) lam[k] = k < NB - 1 ? pen : (logistic ? offsetLog : offsetLin);
        // sums over the linked particles of one regression step; phi2 and
        // mifi weight them (1 and mi for the linear step)
        auto accumulate = [&](bool lin) {
#pragma unroll
            for (int k = 0; k < NM; k++) mt[k] = 0.;
#pragma unroll
            for (int k = 0; k < NB; k++) rhs[k] = 0.;
            auto add = [&](double x, double y, double z, double mi) {
                double w2 = 1., wr = mi;
                if (!lin) {
                    const double dotp = DIM == 3 ? x * beta[0] + y * beta[1] + z * beta[2] + beta[3]
                                                 : x * beta[0] + y * beta[1] + beta[2];
                    const double arg = 1. + exp(-dotp);
                    const double phi = 2. * (arg - 1.) / (arg * arg);
                    w2 = phi * phi;
                    wr = (mi - 2. / arg + 1.) * phi;
                }
                if (DIM == 3) {
                    mt[0] += w2 * x * x;
                    mt[1] += w2 * x * y;
                    mt[2] += w2 * x * z;
                    mt[3] += w2 * x;
                    mt[4] += w2 * y * y;
                    mt[5] += w2 * y * z;
                    mt[6] += w2 * y;
                    mt[7] += w2 * z * z;
                    mt[8] += w2 * z;
                    mt[9] += w2;
                    rhs[0] += wr * x;
                    rhs[1] += wr * y;
                    rhs[2] += wr * z;
                    rhs[3] += wr;
                } else {
                    mt[0] += w2 * x * x;
                    mt[1] += w2 * x * y;
                    mt[2] += w2 * x;
                    mt[3] += w2 * y * y;
                    mt[4] += w2 * y;
                    mt[5] += w2;
                    rhs[0] += wr * x;
                    rhs[1] += wr * y;
                    rhs[2] += wr;
                }
            };
#pragma unroll
            for (int r = 0; r < kLrCached; r++)
                if (s0 + lane + 32 * r < s1) add(cx[r], cy[r], cz[r], cf[r] == a ? -1. : 1.);
            for (int k = s0 + lane + 32 * kLrCached; k < s1; k += 32) {
                const int q = list[k];
                const double mi = mats[p.mat[q]].field == a ? -1. : 1.;
                add(p.x[q] - ndx, p.y[q] - ndy, DIM == 3 ? p.z[q] - ndz : 0., mi);
            }
#pragma unroll
            for (int k = 0; k < NM; k++) mt[k] = lr_wsum(mt[k]);
#pragma unroll
            for (int k = 0; k < NB; k++) rhs[k] = lr_wsum(rhs[k]);
        };
        // (J^T W J + Lambda)^-1 rhs
        auto solve = [&](double *sol) {
            if (DIM == 3) {
                const double m4[10] = {mt[0] + lam[0], mt[1], mt[2], mt[3], mt[4] + lam[1],
                                       mt[5], mt[6], mt[7] + lam[2], mt[8], mt[9] + lam[3]};
                double inv[16];
                lr_inv4_warp(m4, inv, lane);
#pragma unroll
                for (int r = 0; r < 4; r++)
                    sol[r] = inv[4 * r] * rhs[0] + inv[4 * r + 1] * rhs[1] + inv[4 * r + 2] * rhs[2] +
                             inv[4 * r + 3] * rhs[3];
            } else {
                const double m3[6] = {mt[0] + lam[0], mt[1], mt[2], mt[3] + lam[1], mt[4], mt[5] + lam[2]};
                double inv[9];
                lr_inv3_warp(m3, inv, lane);
#pragma unroll
                for (int r = 0; r < 3; r++) sol[r] = inv[3 * r] * rhs[0] + inv[3 * r + 1] * rhs[1] + inv[3 * r + 2] * rhs[2];
            }
        };
        accumulate(true);
        solve(beta);
        if (!logistic) {
            nrm[0] = beta[0];
            nrm[1] = beta[1];
            nrm[2] = DIM == 3 ? beta[2] : 0.;
            const double s = 1. / sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
#pragma unroll
            for (int k = 0; k < 3; k++) nrm[k] *= s;
        } else {
#pragma unroll
            for (int k = 0; k < NB; k++) beta[k] *= 2.;
            double prev[3] = {0., 0., 0.}, lin[3];
            if (DIM == 3) {
                const double s = 1. / sqrt(beta[0] * beta[0] + beta[1] * beta[1] + beta[2] * beta[2]);
#pragma unroll
                for (int k = 0; k < 3; k++) prev[k] = beta[k] * s;
            } else {
                const double nm = sqrt(beta[0] * beta[0] + beta[1] * beta[1]);
                prev[0] = beta[0] / nm;
                prev[1] = beta[1] / nm;
            }
#pragma unroll
            for (int k = 0; k < 3; k++) lin[k] = nrm[k] = prev[k];
            double dcos = 1.;
            int iter = 0;
            while (dcos > tol && iter < maxIter) {
                accumulate(false);
                // penalty: rhs starts from -lambda beta
#pragma unroll
                for (int k = 0; k < NB; k++) rhs[k] += -lam[k] * beta[k];
                double db[NB];
                solve(db);
#pragma unroll
                for (int k = 0; k < NB; k++) beta[k] += db[k];
                if (DIM == 3) {
                    const double s = 1. / sqrt(beta[0] * beta[0] + beta[1] * beta[1] + beta[2] * beta[2]);
#pragma unroll
                    for (int k = 0; k < 3; k++) nrm[k] = beta[k] * s;
                    dcos = 1. - (nrm[0] * prev[0] + nrm[1] * prev[1] + nrm[2] * prev[2]);
                } else {
                    const double nm = sqrt(beta[0] * beta[0] + beta[1] * beta[1]);
                    nrm[0] = beta[0] / nm;
                    nrm[1] = beta[1] / nm;
                    dcos = 1. - nrm[0] * prev[0] - nrm[1] * prev[1];
                }
                iter++;
#pragma unroll
                for (int k = 0; k < 3; k++) prev[k] = nrm[k];
            }
            if (nrm[0] != nrm[0])
#pragma unroll
                for (int k = 0; k < 3; k++) nrm[k] = lin[k];
        }
        const double dn = lr_supports<DIM>(g, p, mats, list, s0, s1, a, nrm);
        if (lane == 0) {
            double *o = out + 4 * (size_t)ka;
            o[0] = nrm[0];
            o[1] = nrm[1];
            o[2] = nrm[2];
            o[3] = dn;
        }
    }
}

// one warp per (contact node, material field): the fields' regressions are
// independent
template <int DIM, bool BATCH>
static __global__ void __launch_bounds__(256, 3) k_lr_normals(StepParams sp, DevParticles p, DevNodes nd,
                                                           const DevMat *mats, const int *start, const int *list,
                                                           const int *nodes, double *out, int nnodes, long long cap,
                                                           int logistic, int supports_only) {
    const long long total = (long long)nodes[nnodes] * sp.ct.nf;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < total; w += nw)
        lr_node_field<DIM, BATCH>(sp, p, nd, mats, start, list, out, nodes[w / sp.ct.nf], (int)(w % sp.ct.nf), cap,
                                  logistic, supports_only);
}

}  // namespace nmg
