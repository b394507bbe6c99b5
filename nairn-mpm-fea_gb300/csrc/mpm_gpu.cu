// mpm_gpu.cu -- C ABI (include/nairn_mpm_gpu.h) of the GB300 explicit MPM step.
//
// One context = one run resident on the current device: particle state as
// structure-of-arrays FP64 columns, the background grid node fields, the
// material table and the velocity conditions grouped by node.  mpmgpu_step()
// enqueues the step kernels (mpm_kernels.cuh) on the context stream and checks
// the device error word once per call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "context.cuh"
#include "host_common.cuh"
#include "archive.cuh"

using namespace nmg;

// slot order = host order after an upload; flags out-of-range indices
__global__ void k_upload_check(const int *mat, const int *elem, int *orig, int n, int nmat, int nelems,
                               unsigned *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    orig[i] = i;
    const int m = mat[i], e = elem[i];
    if (m < 0 || m >= nmat || e < 0 || e >= nelems) atomicOr(err, 8u);
}

namespace {

std::string g_static_err;

int set_err(MpmGpuCtx *c, int code, const std::string &m) {
    if (c) c->msg = m;
    else g_static_err = m;
    return code;
}

int cuda_fail(MpmGpuCtx *c, cudaError_t e, const char *where) {
    return set_err(c, MPMGPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

}  // namespace

// message of a failed call that has no context (mpmgpu_last_error(NULL)),
// for the other translation units
int nmg::fail_static(int code, const std::string &m) { return set_err(nullptr, code, m); }

namespace {

#define CK(call)                                            \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
    } while (0)

// Elastic::SetAnalysisProps + FillUnrotatedElasticProperties for an isotropic
// material (Common/Materials/Elastic.cpp:43-160, 194-330), IsotropicMat
// (Common/Materials/IsotropicMat.cpp:93-170), IsoPlasticity (IsoPlasticity.cpp:58-65),
// HardeningLawBase/LinearHardening::VerifyAndLoadProperties (LinearHardening.cpp:45-58).
// Neohookean::VerifyAndLoadProperties, G and K input (Neohookean.cpp:88-141).
// kterms: MaterialBase::incrementalDefGradTerms (<= 0: 2 in 2D, 1 in 3D, as
// StartOutput.cpp:116-119 resolves the default).
}  // namespace

int nmg::derive_material(const MpmGpuMaterial &in, int np, DevMat &m, std::string &why, int kterms) {
    std::memset(&m, 0, sizeof(m));
    m.type = in.type;
    m.field = in.field;
    m.rho = in.rho * 0.001;
    m.kterms = kterms > 0 ? kterms : (np == MPMGPU_THREED ? 1 : 2);
    if (in.type == MPMGPU_MAT_NEOHOOKEAN) {
        const double rho = in.rho * 0.001;
        const double G = in.G * 1.e6, K = in.K * 1.e6;
        if (!(rho > 0.) || !(G > 0.) || !(K > 0.)) {
            why = "Neohookean needs rho > 0, G > 0 and K > 0";
            return MPMGPU_ERR_INVALID;
        }
        if (in.UJOption < 0 || in.UJOption > 2) {
            why = "Neohookean dilational energy (UJOption) must be 0, 1, or 2";
            return MPMGPU_ERR_INVALID;
        }
        if (np == MPMGPU_THREED && m.kterms > 2) {
            why = "3D incremental deformation gradient with more than 2 terms is not implemented on the device";
            return MPMGPU_ERR_UNSUPPORTED;
        }
        const double Lame = K - 2. * G / 3.;
        m.Gsp = G / rho;
        m.Lamesp = Lame / rho;
        m.uj = in.UJOption;
        return MPMGPU_OK;
    }
    if (in.type == MPMGPU_MAT_RIGID_CONTACT) {
        // RigidMaterial::VerifyAndLoadProperties (RigidMaterial.cpp:44-66): rho = 1,
        // so a particle's mass is its volume (mm^3); no mechanical properties
        m.rho = 1.;
        return MPMGPU_OK;
    }
    if (in.type != MPMGPU_MAT_ISOTROPIC && in.type != MPMGPU_MAT_ISOPLASTICITY) {
        why = "material type " + std::to_string(in.type) + " is not implemented on the device";
        return MPMGPU_ERR_UNSUPPORTED;
    }
    const double rho = in.rho * 0.001;
    const double E = in.E * 1.e6, nu = in.nu;
    if (!(rho > 0.) || !(E > 0.)) {
        why = "material needs rho > 0 and E > 0";
        return MPMGPU_ERR_INVALID;
    }
    const double G = E / (2. * (1. + nu));
    const double e1 = E, e2 = E, e3 = E, v12 = nu, v13 = nu, v23 = nu;
    const double v32 = v23 * e3 / e2, v31 = v13 * e3 / e1, v21 = v12 * e2 / e1;
    const double rrho = 1. / rho;
    double C33;
    if (np == MPMGPU_THREED) {
        const double xx = 1. - v13 * v31 - v23 * v32 - v12 * v21 - 2. * v13 * v32 * v21;
        const double C11 = e1 * (1. - v23 * v32) / xx, C12 = e2 * (v12 + v13 * v32) / xx;
        const double C13 = e3 * (v13 + v12 * v23) / xx, C22 = e2 * (1. - v13 * v31) / xx;
        const double C23 = e3 * (v23 + v21 * v13) / xx;
        C33 = e3 * (1. - v21 * v12) / xx;
        m.C00 = C11 * rrho;
        m.C01 = C12 * rrho;
        m.C02 = C13 * rrho;
        m.C11 = C22 * rrho;
        m.C12 = C23 * rrho;
        m.C22 = C33 * rrho;
        m.C33 = G * rrho;
        m.C44 = G * rrho;
        m.C55 = G * rrho;
    } else {
        const double xx = 1. - v13 * v31 - v23 * v32 - v12 * v21 - 2. * v12 * v23 * v31;
        const double C11 = e1 * (1. - v23 * v32) / xx, C12 = e2 * (v12 + v13 * v32) / xx;
        const double C22 = e2 * (1. - v13 * v31) / xx;
        const double C13 = e3 * (v13 + v12 * v23) / xx, C23 = e3 * (v23 + v21 * v13) / xx;
        C33 = e3 * (1. - v21 * v12) / xx;
        m.c11 = C11 * rrho;
        m.c12 = C12 * rrho;
        m.c22 = C22 * rrho;
        m.c33 = G * rrho;
        m.c41 = C13 * rrho;
        m.c42 = C23 * rrho;
        m.c44 = C33 * rrho;
    }
    m.Gred = G / rho;
    m.Kred = C33 / rho - 4. * m.Gred / 3.;
    if (in.type == MPMGPU_MAT_ISOPLASTICITY) {
        const double yield = in.yield * 1.e6, Ep = in.Ep * 1.e6;
        if (!(yield > 0.)) {
            why = "isoplasticity needs yield > 0";
            return MPMGPU_ERR_INVALID;
        }
        m.yldred = yield / rho;
        m.yldredMin = 0. / rho;
        const double beta = Ep >= 0. ? Ep / yield : 0.;
        m.Epred = m.yldred * beta;
        m.alphaMax = 1.e50;
        if (beta < 0.) m.alphaMax = ((m.yldredMin / m.yldred) - 1.) / beta;
    }
    return MPMGPU_OK;
}

namespace {

// Point the particle columns at a block of kParticleDoubles+1 double columns
// (the last three are the step's natural coordinates) and 3 int columns.
// The double columns of p in the device block's order (hcols gives the host
// columns in the same order; the last three are the natural coordinates).
void particle_columns(DevParticles &p, double **cols[kParticleDoubles + 1]) {
    double **tmp[kParticleDoubles + 1] = {&p.x, &p.y, &p.z, &p.vx, &p.vy, &p.vz, &p.mass, &p.lpx, &p.lpy, &p.lpz,
                                          &p.exx, &p.eyy, &p.ezz, &p.exy, &p.exz, &p.eyz, &p.wxy, &p.wxz, &p.wyz,
                                          &p.sxx, &p.syy, &p.szz, &p.sxy, &p.sxz, &p.syz, &p.pressure,
                                          &p.pxx, &p.pyy, &p.pzz, &p.pxy, &p.pxz, &p.pyz,
                                          &p.hist0, &p.hist1, &p.work, &p.plast, &p.x0, &p.y0, &p.z0,
                                          &p.xi, &p.eta, &p.zeta};
    std::memcpy(cols, tmp, sizeof(tmp));
}

void link_columns(DevParticles &p, double *pb, int *ib, int **orig) {
    const size_t n = (size_t)p.n;
    double **cols[kParticleDoubles + 1];
    particle_columns(p, cols);
    for (int k = 0; k <= kParticleDoubles; k++) *cols[k] = pb + (size_t)k * n;
    p.mat = ib;
    p.elem = ib + n;
    *orig = ib + 2 * n;
}

// Page-locked blocks from mpmgpu_host_alloc (base -> bytes).  The columns a
// step on host-resident state reads and writes must each lie inside one of
// them, so that every access of its kernels stays inside memory the device
// has mapped.
std::mutex g_host_mu;
std::map<uintptr_t, size_t> g_host_blocks;

bool in_host_block(const void *ptr, size_t bytes) {
    const uintptr_t a = (uintptr_t)ptr;
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_blocks.upper_bound(a);
    if (it == g_host_blocks.begin()) return false;
    --it;
    const size_t off = a - it->first;
    return off <= it->second && bytes <= it->second - off;
}

// The device address of n values of a host column inside one block of
// mpmgpu_host_alloc; nullptr when the column lies outside every block.
template <class T>
T *mapped_column(T *h, size_t n) {
    if (!h || !in_host_block(h, n * sizeof(T))) return nullptr;
    void *d = nullptr;
    if (cudaHostGetDevicePointer(&d, (void *)h, 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (T *)d;
}

}  // namespace

// the matching host columns of MpmGpuParticles (nullptr for the natural coordinates)
void nmg::hcols(const MpmGpuParticles *h, double *out[kParticleDoubles]) {
    double *tmp[kParticleDoubles] = {h->x, h->y, h->z, h->vx, h->vy, h->vz, h->mass, h->lpx, h->lpy, h->lpz,
                                     h->exx, h->eyy, h->ezz, h->exy, h->exz, h->eyz, h->wxy, h->wxz, h->wyz,
                                     h->sxx, h->syy, h->szz, h->sxy, h->sxz, h->syz, h->pressure,
                                     h->pxx, h->pyy, h->pzz, h->pxy, h->pxz, h->pyz,
                                     h->hist0, h->hist1, h->work, h->plast, h->x0, h->y0, h->z0, nullptr, nullptr};
    std::memcpy(out, tmp, sizeof(tmp));
}

namespace {

// Runs of host columns that sit back to back in the device's column order
// (hcols), each moved with one copy: a host that keeps its particle columns in
// one block in that order transfers them at the link's full rate instead of
// paying a copy per column.  f(k, e) moves columns k .. e-1.
template <class F>
void column_runs(double *const hc[kParticleDoubles], size_t n, F &&f) {
    int k = 0;
    while (k < kParticleDoubles) {
        if (!hc[k]) {
            k++;
            continue;
        }
        int e = k + 1;
        while (e < kParticleDoubles && hc[e] && hc[e] == hc[e - 1] + n) e++;
        f(k, e);
        k = e;
    }
}

// Columns of the per-particle window cache (DevParticles::win): FP64
// transfers with a shape function whose nodes form a box around the element
// (2, 3 or 4 nodes per axis); 0 for lCPDI and the mixed mode.
int win_cache_cols(const MpmGpuCtx *c) {
    if (c->opts.precision == MPMGPU_PREC_MIXED) return 0;
    const int s = c->opts.shape;
    const int k = s == MPMGPU_SHAPE_LINEAR ? 2 : s == MPMGPU_SHAPE_BGIMP ? 4
                : (s == MPMGPU_SHAPE_UGIMP || s == MPMGPU_SHAPE_BSPLINE) ? 3 : 0;
    return 2 * c->dim * k;
}

// Domain points per particle of the CPDI shape functions (0 for the others)
int cpdi_points(const MpmGpuCtx *c) {
    if (c->opts.shape == MPMGPU_SHAPE_QCPDI) return 9;
    return c->opts.shape == MPMGPU_SHAPE_LCPDI ? (c->dim == 3 ? 8 : 4) : 0;
}

void free_particles(MpmGpuCtx *c) {
    if (c->pblock) cudaFree(c->pblock);
    if (c->iblock) cudaFree(c->iblock);
    if (c->cpdi) cudaFree(c->cpdi);
    if (c->winblock) cudaFree(c->winblock);
    if (c->iota) cudaFree(c->iota);
    c->pblock = nullptr;
    c->iblock = nullptr;
    c->cpdi = nullptr;
    c->winblock = nullptr;
    c->iota = nullptr;
    sort_free(c->sort);
    c->p.n = 0;
}

}  // namespace

void nmg::relink_particles(DevParticles &p, double *pblock, int *iblock, int **orig) {
    link_columns(p, pblock, iblock, orig);
}

extern "C" {

int mpmgpu_abi_version(void) { return MPMGPU_ABI_VERSION; }

const char *mpmgpu_last_error(const MpmGpuCtx *c) { return c ? c->msg.c_str() : g_static_err.c_str(); }

int mpmgpu_create(const MpmGpuGrid *grid, const MpmGpuOptions *opts, MpmGpuCtx **out) {
    MpmGpuCtx *c = nullptr;
    if (!grid || !opts || !out) return set_err(nullptr, MPMGPU_ERR_INVALID, "mpmgpu_create: null argument");
    *out = nullptr;
    if (grid->dim != 2 && grid->dim != 3) return set_err(nullptr, MPMGPU_ERR_INVALID, "grid dim must be 2 or 3");
    if ((grid->dim == 3) != (opts->np == MPMGPU_THREED) ||
        (grid->dim == 2 && opts->np != MPMGPU_PLANE_STRAIN))
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED, "analysis type must be 2D plane strain or 3D");
    if (opts->shape != MPMGPU_SHAPE_LINEAR && opts->shape != MPMGPU_SHAPE_UGIMP && opts->shape != MPMGPU_SHAPE_LCPDI &&
        opts->shape != MPMGPU_SHAPE_BSPLINE && opts->shape != MPMGPU_SHAPE_BGIMP && opts->shape != MPMGPU_SHAPE_QCPDI)
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED, "shape function option not implemented on the device");
    // ElementBase::InitializeCPDI refuses qCPDI in 3D (MoreMPMElementBase.cpp:1008-1013)
    if (opts->shape == MPMGPU_SHAPE_QCPDI && grid->dim == 3)
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED, "qCPDI is defined in 2D only; use lCPDI in 3D");
    if (opts->method != MPMGPU_USF && opts->method != MPMGPU_USAVG && opts->method != MPMGPU_USL)
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED, "MPM method must be USF, USAVG or USL");
    if (opts->precision != MPMGPU_PREC_FP64 && opts->precision != MPMGPU_PREC_MIXED)
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED, "precision must be MPMGPU_PREC_FP64 or MPMGPU_PREC_MIXED");
    if (opts->p2g != MPMGPU_P2G_ATOMIC && opts->p2g != MPMGPU_P2G_DETERMINISTIC && opts->p2g != MPMGPU_P2G_UNTILED)
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED,
                       "p2g must be MPMGPU_P2G_ATOMIC, MPMGPU_P2G_DETERMINISTIC or MPMGPU_P2G_UNTILED");
    if (!(opts->timestep > 0.)) return set_err(nullptr, MPMGPU_ERR_INVALID, "timestep must be > 0");
    if (opts->xpic_order < 0 || opts->xpic_order > 64 || (opts->xpic_fmpm != 0 && opts->xpic_fmpm != 1) ||
        (opts->xpic_order > 0 && opts->xpic_period < 1))
        return set_err(nullptr, MPMGPU_ERR_INVALID, "xpic_order must be 0 to 64, xpic_fmpm 0 or 1, xpic_period >= 1");
    if (opts->xpic_order > 1 && opts->p2g == MPMGPU_P2G_DETERMINISTIC)
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED,
                       "XPIC/FMPM of order > 1 with deterministic node sums is not implemented");
    if (grid->nx < 3 || grid->ny < 3 || (grid->dim == 3 && grid->nz < 3) || !grid->xnodes || !grid->ynodes ||
        (grid->dim == 3 && !grid->znodes))
        return set_err(nullptr, MPMGPU_ERR_INVALID, "grid needs >= 3 elements per axis and node coordinates");
    long long nn = (long long)(grid->nx + 1) * (grid->ny + 1) * (grid->dim == 3 ? grid->nz + 1 : 1);
    if (nn > (1LL << 30)) return set_err(nullptr, MPMGPU_ERR_INVALID, "grid too large");
    c = new MpmGpuCtx();
    c->opts = *opts;
    if (c->opts.sort_interval < 0) c->opts.sort_interval = 0;
    c->dim = grid->dim;
    DevGrid &g = c->g;
    g.dim = grid->dim;
    g.nx = grid->nx;
    g.ny = grid->ny;
    g.nz = grid->dim == 3 ? grid->nz : 0;
    g.xplane = 1;
    g.yplane = grid->nx + 1;
    g.zplane = (grid->nx + 1) * (grid->ny + 1);
    g.nnodes = (int)nn;
    g.xmin = grid->xmin;
    g.ymin = grid->ymin;
    g.zmin = grid->zmin;
    g.gx = grid->dx;
    g.gy = grid->dy;
    g.gz = grid->dz;
    g.igx = 1. / grid->dx;
    g.igy = 1. / grid->dy;
    g.igz = grid->dim == 3 ? 1. / grid->dz : 0.;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        int st = cuda_fail(nullptr, e, "cudaStreamCreate");
        delete c;
        return st;
    }
    size_t ncoord = (size_t)(g.nx + 1) + (g.ny + 1) + (g.dim == 3 ? g.nz + 1 : 0);
    std::vector<double> coords;
    coords.insert(coords.end(), grid->xnodes, grid->xnodes + g.nx + 1);
    coords.insert(coords.end(), grid->ynodes, grid->ynodes + g.ny + 1);
    if (g.dim == 3) coords.insert(coords.end(), grid->znodes, grid->znodes + g.nz + 1);
    // node columns, one entry per material field of each node (field f of
    // node n at f*nnodes+n): mass, p(3), f(3), u(3) and, with several fields,
    // the contact terms vol, ds(3), gv(3) are cleared each step; c(3), v(3),
    // a(3) are not
    const int nf = opts->nfields > 1 ? opts->nfields : 1;
    if (nf > kMaxFields) {
        mpmgpu_destroy(c);
        return set_err(nullptr, MPMGPU_ERR_UNSUPPORTED, "more material velocity fields than the device supports (8)");
    }
    c->ct.nf = nf;
    c->ct.fstride = g.nnodes;
    const size_t NN = (size_t)g.nnodes * nf;
    const int ncleared = nf > 1 ? 17 : 10, nkept = 9;
    // FP32 columns of the mixed mode: force accumulators (cleared), velocity
    // hi/lo pairs and acceleration
    const int fcleared = 3, fkept = 9;
    if ((e = cudaMalloc(&c->grid_coords, ncoord * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&c->nblock, NN * (ncleared + nkept) * sizeof(double) + NN)) != cudaSuccess ||
        (e = cudaMalloc(&c->fblock, NN * (fcleared + fkept) * sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc(&c->bc_group, NN * sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc(&c->err, sizeof(unsigned))) != cudaSuccess) {
        std::string m = std::string("device allocation: ") + cudaGetErrorString(e);
        mpmgpu_destroy(c);
        return set_err(nullptr, MPMGPU_ERR_OOM, m);
    }
    cudaMemcpy(c->grid_coords, coords.data(), ncoord * sizeof(double), cudaMemcpyHostToDevice);
    g.xn = c->grid_coords;
    g.yn = c->grid_coords + g.nx + 1;
    g.zn = g.dim == 3 ? c->grid_coords + (g.nx + 1) + (g.ny + 1) : nullptr;
    double *b = c->nblock;
    DevNodes &nd = c->nd;
    nd.mass = b;
    nd.px = b + NN;
    nd.py = b + 2 * NN;
    nd.pz = b + 3 * NN;
    nd.fx = b + 4 * NN;
    nd.fy = b + 5 * NN;
    nd.fz = b + 6 * NN;
    nd.ux = b + 7 * NN;
    nd.uy = b + 8 * NN;
    nd.uz = b + 9 * NN;
    if (nf > 1) {
        nd.vol = b + 10 * NN;
        nd.dsx = b + 11 * NN;
        nd.dsy = b + 12 * NN;
        nd.dsz = b + 13 * NN;
        nd.gvx = b + 14 * NN;
        nd.gvy = b + 15 * NN;
        nd.gvz = b + 16 * NN;
    }
    double *kb = b + ncleared * NN;
    nd.cx = kb;
    nd.cy = kb + NN;
    nd.cz = kb + 2 * NN;
    nd.vx = kb + 3 * NN;
    nd.vy = kb + 4 * NN;
    nd.vz = kb + 5 * NN;
    nd.ax = kb + 6 * NN;
    nd.ay = kb + 7 * NN;
    nd.az = kb + 8 * NN;
    nd.active = (unsigned char *)(b + (ncleared + nkept) * NN);
    c->nblock_zero_bytes = NN * ncleared * sizeof(double);
    cudaMemset(c->nblock, 0, NN * (ncleared + nkept) * sizeof(double) + NN);
    float *fb = c->fblock;
    nd.gx = fb;
    nd.gy = fb + NN;
    nd.gz = fb + 2 * NN;
    nd.vhx = fb + 3 * NN;
    nd.vhy = fb + 4 * NN;
    nd.vhz = fb + 5 * NN;
    nd.vlx = fb + 6 * NN;
    nd.vly = fb + 7 * NN;
    nd.vlz = fb + 8 * NN;
    nd.bx = fb + 9 * NN;
    nd.by = fb + 10 * NN;
    nd.bz = fb + 11 * NN;
    c->fblock_zero_bytes = NN * fcleared * sizeof(float);
    cudaMemset(c->fblock, 0, NN * (fcleared + fkept) * sizeof(float));
    cudaMemset(c->bc_group, 0xFF, NN * sizeof(int));
    cudaMemset(c->err, 0, sizeof(unsigned));
    if (opts->p2g == MPMGPU_P2G_DETERMINISTIC) {
        // three limbs per accumulated quantity (the contact terms only with
        // several fields), zero between uses; the step's bounds
        const size_t nq = nf > 1 ? kDetQuantities : DQ_VOL;
        if ((e = cudaMalloc(&c->det.lim, nq * 3 * NN * sizeof(long long))) != cudaSuccess ||
            (e = cudaMalloc(&c->det.bnd, kDetBounds * sizeof(unsigned long long))) != cudaSuccess ||
            (e = cudaMalloc(&c->det.nbnd, NN * sizeof(unsigned long long))) != cudaSuccess) {
            std::string m = std::string("device allocation: ") + cudaGetErrorString(e);
            mpmgpu_destroy(c);
            return set_err(nullptr, MPMGPU_ERR_OOM, m);
        }
        c->det.stride = NN;
        cudaMemset(c->det.lim, 0, nq * 3 * NN * sizeof(long long));
    }
    const char *names[] = {"p2g", "node_post", "strain_forces", "node_update", "g2p", "node_usl", "strain_last",
                           "sort"};
    for (const char *n : names) c->prof.push_back(Profile{n, 0.});
    if ((e = cudaGetLastError()) != cudaSuccess) {
        int st = cuda_fail(nullptr, e, "mpmgpu_create");
        mpmgpu_destroy(c);
        return st;
    }
    *out = c;
    return MPMGPU_OK;
}

int mpmgpu_set_materials(MpmGpuCtx *c, const MpmGpuMaterial *mats, int32_t nmat) {
    if (!c || !mats || nmat <= 0) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_set_materials: bad argument");
    std::vector<DevMat> h((size_t)nmat);
    for (int i = 0; i < nmat; i++) {
        std::string why;
        int st = derive_material(mats[i], c->opts.np, h[i], why, c->opts.inc_defgrad_terms);
        if (st != MPMGPU_OK) return set_err(c, st, "material " + std::to_string(i) + ": " + why);
        if (mats[i].field < 0 || mats[i].field >= c->ct.nf)
            return set_err(c, MPMGPU_ERR_INVALID, "material " + std::to_string(i) + ": field outside 0 .. nfields-1");
    }
    if (c->mats) cudaFree(c->mats);
    c->mats = nullptr;
    CK(cudaMalloc(&c->mats, sizeof(DevMat) * nmat));
    CK(cudaMemcpy(c->mats, h.data(), sizeof(DevMat) * nmat, cudaMemcpyHostToDevice));
    c->hmats = h;
    c->nmat = nmat;
    return MPMGPU_OK;
}

// MeshInfo::MaterialOutput / CoulombFriction::VerifyAndLoadProperties
// (MeshInfo.cpp:1128-1190, CoulombFriction.cpp:80-104): normal method and the
// friction style (coefficient < 0 stick, 0 frictionless, > 0 Coulomb).
int mpmgpu_set_contact(MpmGpuCtx *c, const MpmGpuContact *contact) {
    if (!c) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_set_contact: null context");
    if (!contact || !contact->enabled) {
        c->contact_on = false;
        return MPMGPU_OK;
    }
    if (contact->normals < 0 || (contact->normals > 2 && contact->normals != 5 && contact->normals != 6))
        return set_err(c, MPMGPU_ERR_UNSUPPORTED,
                       "contact normals: methods 0 (max gradient), 1 (max volume), 2 (average gradient), 5 (linear "
                       "regression) and 6 (logistic regression) are implemented on the device");
    if (contact->contact_cutoff > 0.)
        return set_err(c, MPMGPU_ERR_UNSUPPORTED, "position-based contact is not implemented on the device");
    c->ct.normals = contact->normals;
    c->ct.friction = contact->friction;
    c->ct.style = contact->friction < 0. ? 0 : (contact->friction == 0. ? 1 : 2);
    // MeshInfo::rigidGradientBias (default 1), squared (MeshInfo.cpp:44, 1191)
    const double bias = contact->rigid_gradient_bias > 0. ? contact->rigid_gradient_bias : 1.;
    c->ct.rigid_bias = bias * bias;
    c->contact_on = true;
    return MPMGPU_OK;
}

int mpmgpu_set_velocity_bcs(MpmGpuCtx *c, const MpmGpuVelBC *bcs, int32_t nbc) {
    if (!c || (nbc > 0 && !bcs) || nbc < 0) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_set_velocity_bcs: bad argument");
    // group by node, keeping list order inside each node
    std::map<int, std::vector<int>> by_node;
    std::vector<int> order;
    for (int k = 0; k < nbc; k++) {
        const int nd = bcs[k].node - 1;
        if (nd < 0 || nd >= c->g.nnodes) return set_err(c, MPMGPU_ERR_INVALID, "velocity BC node out of range");
        const int dir = bcs[k].dir;
        if (dir != 1 && dir != 2 && dir != 4) return set_err(c, MPMGPU_ERR_UNSUPPORTED, "velocity BC dir must be 1, 2 or 4");
        if (dir == 4 && c->dim == 2) return set_err(c, MPMGPU_ERR_INVALID, "z velocity BC in 2D");
        if (!by_node.count(nd)) order.push_back(nd);
        by_node[nd].push_back(k);
    }
    const int ng = (int)order.size();
    std::vector<int> gnode(ng), start(ng + 1), dir(nbc);
    std::vector<double> val(nbc), ft(nbc);
    std::vector<int> group(c->g.nnodes, -1);
    int pos = 0;
    for (int gi = 0; gi < ng; gi++) {
        gnode[gi] = order[gi];
        start[gi] = pos;
        group[order[gi]] = gi;
        for (int k : by_node[order[gi]]) {
            dir[pos] = bcs[k].dir;
            val[pos] = bcs[k].value;
            ft[pos] = bcs[k].ftime;
            pos++;
        }
    }
    start[ng] = pos;
    if (c->bc_block) cudaFree(c->bc_block);
    c->bc_block = nullptr;
    size_t bytes = sizeof(int) * (ng + ng + 1 + nbc) + sizeof(double) * (2 * nbc) + 64;
    CK(cudaMalloc(&c->bc_block, bytes));
    char *bb = (char *)c->bc_block;
    double *dval = (double *)bb;
    double *dft = dval + nbc;
    int *dnode = (int *)(dft + nbc);
    int *dstart = dnode + ng;
    int *ddir = dstart + ng + 1;
    CK(cudaMemcpy(dval, val.data(), sizeof(double) * nbc, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dft, ft.data(), sizeof(double) * nbc, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dnode, gnode.data(), sizeof(int) * ng, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dstart, start.data(), sizeof(int) * (ng + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ddir, dir.data(), sizeof(int) * nbc, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->bc_group, group.data(), sizeof(int) * c->g.nnodes, cudaMemcpyHostToDevice));
    c->bcs.nnodes_bc = ng;
    c->bcs.node = dnode;
    c->bcs.start = dstart;
    c->bcs.dir = ddir;
    c->bcs.value = dval;
    c->bcs.ftime = dft;
    return MPMGPU_OK;
}

int mpmgpu_upload_particles(MpmGpuCtx *c, const MpmGpuParticles *h) {
    if (!c || !h || h->n <= 0) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_upload_particles: bad argument");
    if (h->n > (1LL << 31) - 1) return set_err(c, MPMGPU_ERR_INVALID, "too many particles for one context");
    if (!c->mats) return set_err(c, MPMGPU_ERR_INVALID, "set materials before uploading particles");
    if (!h->x || !h->y || !h->vx || !h->vy || !h->mass || !h->mat || !h->elem || !h->lpx || !h->lpy ||
        (c->dim == 3 && (!h->z || !h->vz || !h->lpz)))
        return set_err(c, MPMGPU_ERR_INVALID,
                       "mpmgpu_upload_particles: position, velocity, mass, size, material and element columns are required");
    const int n = (int)h->n;
    const int nelems = c->g.nx * c->g.ny * (c->dim == 3 ? c->g.nz : 1);
    const size_t dbytes = (size_t)n * (kParticleDoubles + 1) * sizeof(double);
    if (c->p.n != n || !c->pblock) {
        free_particles(c);
        cudaError_t e = cudaMalloc(&c->pblock, dbytes);
        if (e == cudaSuccess) e = cudaMalloc(&c->iblock, (size_t)n * 3 * sizeof(int));
        if (e != cudaSuccess) {
            free_particles(c);
            return set_err(c, MPMGPU_ERR_OOM, std::string("particle allocation: ") + cudaGetErrorString(e));
        }
        if (sort_alloc(c->sort, n, nelems, kParticleDoubles + 1) != 0) {
            free_particles(c);
            return set_err(c, MPMGPU_ERR_OOM, "sort workspace allocation failed");
        }
        if (cpdi_points(c) > 0) {
            // per domain point: element (int), natural coordinates and gradient weights (3 doubles each)
            const size_t nc = (size_t)cpdi_points(c);
            const size_t bytes = (size_t)n * nc * (sizeof(int) + 6 * sizeof(double)) + 256;
            e = cudaMalloc(&c->cpdi, bytes);
            if (e != cudaSuccess) {
                free_particles(c);
                return set_err(c, MPMGPU_ERR_OOM, "CPDI corner allocation failed");
            }
        }
        if (win_cache_cols(c) > 0) {
            e = cudaMalloc(&c->winblock, (size_t)n * (win_cache_cols(c) * sizeof(double) + sizeof(int)));
            if (e != cudaSuccess) {
                free_particles(c);
                return set_err(c, MPMGPU_ERR_OOM, "window cache allocation failed");
            }
        }
        CK(cudaMemsetAsync(c->pblock, 0, dbytes, c->stream));
        c->p.n = n;
    }
    link_columns(c->p, c->pblock, c->iblock, &c->orig);
    c->p.win = (double *)c->winblock;
    c->p.win_n0 = c->winblock ? (int *)(c->p.win + (size_t)win_cache_cols(c) * n) : nullptr;
    if (c->cpdi) {
        // doubles first (8-byte aligned), then the domain points' elements
        const size_t nc = (size_t)cpdi_points(c);
        c->p.cxi = (double *)c->cpdi;
        c->p.cwg = c->p.cxi + 3 * nc * (size_t)n;
        c->p.ce = (int *)(c->p.cwg + 3 * nc * (size_t)n);
    } else {
        c->p.cxi = c->p.cwg = nullptr;
        c->p.ce = nullptr;
    }
    double *hc[kParticleDoubles];
    hcols(h, hc);
    for (int k = 0; k < kParticleDoubles; k++)
        if (!hc[k]) CK(cudaMemsetAsync(c->pblock + (size_t)k * n, 0, (size_t)n * sizeof(double), c->stream));
    cudaError_t ce = cudaSuccess;
    column_runs(hc, (size_t)n, [&](int k, int e) {
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(c->pblock + (size_t)k * n, hc[k], (size_t)(e - k) * n * sizeof(double),
                                 cudaMemcpyHostToDevice, c->stream);
    });
    CK(ce);
    CK(cudaMemcpyAsync(c->p.mat, h->mat, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->p.elem, h->elem, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    // identity slot order and a range check of the indices the kernels use
    CK(cudaMemsetAsync(c->err, 0, sizeof(unsigned), c->stream));
    const int TB = 256;
    k_upload_check<<<(n + TB - 1) / TB, TB, 0, c->stream>>>(c->p.mat, c->p.elem, c->orig, n, c->nmat, nelems, c->err);
    c->launches++;
    unsigned flags = 0;
    CK(cudaMemcpyAsync(&flags, c->err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (flags) {
        cudaMemsetAsync(c->err, 0, sizeof(unsigned), c->stream);
        cudaStreamSynchronize(c->stream);
        return set_err(c, MPMGPU_ERR_INVALID, "particle material or element index out of range");
    }
    c->steps_done = 0;
    return MPMGPU_OK;
}

}  // extern "C"

namespace {

void enqueue(MpmGpuCtx *c, double t, int slot) {
    const bool det = c->det.lim != nullptr;
    const bool mix = c->opts.precision == MPMGPU_PREC_MIXED;
    if (c->dim == 3) {
        if (mix) det ? enqueue_dim<3, true, true>(c, t, slot) : enqueue_dim<3, true, false>(c, t, slot);
        else det ? enqueue_dim<3, false, true>(c, t, slot) : enqueue_dim<3, false, false>(c, t, slot);
    } else {
        if (mix) det ? enqueue_dim<2, true, true>(c, t, slot) : enqueue_dim<2, true, false>(c, t, slot);
        else det ? enqueue_dim<2, false, true>(c, t, slot) : enqueue_dim<2, false, false>(c, t, slot);
    }
}

int ensure_events(MpmGpuCtx *c, int nsteps) {
    const size_t need = (size_t)nsteps * kFamilies * 2;
    while (c->ev.size() < need) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return 1;
        c->ev.push_back(e);
    }
    return 0;
}

int error_status(MpmGpuCtx *c, unsigned bits) {
    if (bits & ERR_NAN) return set_err(c, MPMGPU_ERR_NAN, "a particle position became NaN");
    if (bits & ERR_LEFT_GRID) return set_err(c, MPMGPU_ERR_LEFT_GRID, "a particle left the grid");
    if (bits & ERR_EDGE) return set_err(c, MPMGPU_ERR_LEFT_GRID, "a particle moved into a grid edge element");
    if (bits & ERR_CPDI_NODES)
        return set_err(c, MPMGPU_ERR_CPDI_NODES, "a CPDI particle domain touches more nodes than the reference allows");
    if (bits & ERR_RANGE)
        return set_err(c, MPMGPU_ERR_RANGE, "a deterministic node sum met a NaN, infinite or out-of-bound value");
    return MPMGPU_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// Enqueue nsteps steps; when ms is given, CUDA events on the context stream
// bracket the enqueued work and *ms receives its device time.
int step_impl(MpmGpuCtx *c, int32_t nsteps, double t0, double *ms) {
    if (!c || nsteps < 0) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_step: bad argument");
    if (c->p.n <= 0 || !c->mats) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_step: no particles or materials");
    if (c->ct.nf > 1 && !c->contact_on)
        return set_err(c, MPMGPU_ERR_INVALID, "several material fields need multimaterial contact (mpmgpu_set_contact)");
    // rigid contact materials: the fields they occupy, and the options they work with
    c->ct.rigid = 0u;
    for (const DevMat &m : c->hmats)
        if (m.type == kMatRigid) c->ct.rigid |= 1u << m.field;
    if (c->ct.rigid) {
        if (c->ct.nf < 2 || !c->contact_on)
            return set_err(c, MPMGPU_ERR_UNSUPPORTED,
                           "rigid contact materials need multimaterial contact (RigidMaterial::SetField)");
        if (c->ct.normals >= 5)
            return set_err(c, MPMGPU_ERR_UNSUPPORTED, "regression normals with rigid materials are not implemented");
        if (c->opts.xpic_order > 1)
            return set_err(c, MPMGPU_ERR_UNSUPPORTED, "XPIC/FMPM of order > 1 with rigid materials is not implemented");
    }
    for (auto &pr : c->prof) pr.ms = 0.;
    if (c->profile && ensure_events(c, nsteps) != 0) return set_err(c, MPMGPU_ERR_CUDA, "event creation failed");
    if (c->ct.nf > 1 && c->ct.normals >= 5) {
        // regression normals: links of at most 64 nodes per particle (the
        // largest lCPDI domain), a result per material field of each node
        const long long need = (long long)c->p.n * (c->dim == 3 ? 64 : 16);
        if (c->lr_cap < need) {
            for (void *q : {(void *)c->lr_cnt, (void *)c->lr_start, (void *)c->lr_list, (void *)c->lr_sums,
                            (void *)c->lr_out})
                if (q) cudaFree(q);
            const size_t m = (size_t)c->g.nnodes + 1, nsums = (m + kScanChunk - 1) / kScanChunk + 1;
            cudaError_t e = cudaMalloc(&c->lr_cnt, m * sizeof(int));
            if (e == cudaSuccess) e = cudaMalloc(&c->lr_start, m * sizeof(int));
            if (e == cudaSuccess) e = cudaMalloc(&c->lr_list, (size_t)need * sizeof(int));
            if (e == cudaSuccess) e = cudaMalloc(&c->lr_sums, nsums * sizeof(int));
            if (e == cudaSuccess) e = cudaMalloc(&c->lr_out, (size_t)c->g.nnodes * c->ct.nf * 4 * sizeof(double));
            if (e != cudaSuccess) {
                c->lr_cnt = c->lr_start = c->lr_list = c->lr_sums = nullptr;
                c->lr_out = nullptr;
                c->lr_cap = 0;
                return set_err(c, MPMGPU_ERR_OOM, "regression normal buffers");
            }
            c->lr_cap = need;
        }
        c->ct.lr = c->lr_out;
    }
    if (c->opts.xpic_order > 1 && !c->xpic_block) {
        // PeriodicXPIC expansion: v*(prev), v*(next) and 1 / mass of every
        // field-node, in FP64 and FP32; with contact, each field-node's
        // contact state for the incremental contact of the passes
        const size_t nn = (size_t)c->g.nnodes * c->ct.nf;
        const size_t xc = c->ct.nf > 1 ? nn * (kXcDoubles * sizeof(double) + sizeof(int)) : 0;
        cudaError_t e = cudaMalloc(&c->xpic_block, 7 * nn * sizeof(double) + 6 * nn * sizeof(float) + xc);
        if (e != cudaSuccess) {
            c->xpic_block = nullptr;
            return set_err(c, MPMGPU_ERR_OOM, "XPIC node columns");
        }
        double *b = c->xpic_block;
        float *f = (float *)(b + 7 * nn);
        c->xpic = DevXpic{b, b + nn, b + 2 * nn, b + 3 * nn, b + 4 * nn, b + 5 * nn, b + 6 * nn,
                          f, f + nn, f + 2 * nn, f + 3 * nn, f + 4 * nn, f + 5 * nn};
        if (c->ct.nf > 1) {
            c->ct.xc = (double *)(f + 6 * nn);  // 8-byte aligned: 6 nn floats
            c->ct.xc_pair = (int *)(c->ct.xc + kXcDoubles * nn);
        }
    }
    std::vector<char> sorted((size_t)nsteps, 0);
    cudaEvent_t w0 = nullptr, w1 = nullptr;
    if (ms) {
        CK(cudaEventCreate(&w0));
        CK(cudaEventCreate(&w1));
        CK(cudaEventRecord(w0, c->stream));
    }
    double t = t0;
    for (int s = 0; s < nsteps; s++) {
        if (c->opts.sort_interval > 0 && c->steps_done % c->opts.sort_interval == 0) {
            if (c->profile) cudaEventRecord(event_at(c, s, 7, true), c->stream);
            int st = sort_particles(c->sort, c->p, c->pblock, c->iblock, c->orig, kParticleDoubles + 1, c->stream);
            if (st != 0) return set_err(c, MPMGPU_ERR_CUDA, "particle sort failed");
            c->launches += sort_launches(c->sort);
            if (c->profile) cudaEventRecord(event_at(c, s, 7, false), c->stream);
            sorted[s] = 1;
        }
        enqueue(c, t, s);
        c->steps_done++;
        t += c->opts.timestep;
    }
    if (ms) CK(cudaEventRecord(w1, c->stream));
    unsigned bits = 0;
    CK(cudaMemcpyAsync(&bits, c->err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    if (ms) {
        float f = 0.f;
        cudaEventElapsedTime(&f, w0, w1);
        *ms = f;
        cudaEventDestroy(w0);
        cudaEventDestroy(w1);
    }
    if (c->profile) {
        const bool usl = c->opts.method != MPMGPU_USF;
        for (int s = 0; s < nsteps; s++)
            for (int k = 0; k < kFamilies; k++) {
                if (k == 7 && !sorted[s]) continue;
                if (!usl && (k == 5 || k == 6)) continue;
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, event_at(c, s, k, true), event_at(c, s, k, false)) == cudaSuccess)
                    c->prof[k].ms += ms;
            }
    }
    if (bits) {
        cudaMemsetAsync(c->err, 0, sizeof(unsigned), c->stream);
        return error_status(c, bits);
    }
    return MPMGPU_OK;
}

}  // namespace

extern "C" {

int mpmgpu_step(MpmGpuCtx *c, int32_t nsteps, double t0) { return step_impl(c, nsteps, t0, nullptr); }

// Extension: the sort interval with the shortest step, by timing trial steps
// at each candidate (the steps are real; the caller's clock advances).  The
// candidates take turns in chunks of 8 steps, each chunk starting with a sort,
// in alternating order, so that a step cost that drifts as the run evolves
// (plastic zones growing) favours none of them.
int mpmgpu_autotune_sort(MpmGpuCtx *c, int32_t trial_steps, double t0, int32_t *best_interval,
                         double *ms_per_step, int32_t *steps_taken) {
    if (!c || trial_steps < 1 || !best_interval || !ms_per_step || !steps_taken)
        return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_autotune_sort: bad argument");
    const int cand[4] = {1, 2, 4, 8};
    const int chunk = 8, rounds = trial_steps > chunk ? trial_steps / chunk : 1;
    const int keep = c->opts.sort_interval;
    double total[4] = {0., 0., 0., 0.};
    double t = t0;
    *steps_taken = 0;
    for (int r = 0; r < rounds; r++)
        for (int j = 0; j < 4; j++) {
            const int k = (r & 1) ? 3 - j : j;
            c->opts.sort_interval = cand[k];
            c->steps_done = 0;  // the chunk starts with a sort
            double ms = 0.;
            const int st = step_impl(c, chunk, t, &ms);
            *steps_taken += chunk;
            t += chunk * c->opts.timestep;
            if (st != MPMGPU_OK) {
                c->opts.sort_interval = keep;
                return st;
            }
            total[k] += ms;
        }
    int best = 0;
    for (int k = 1; k < 4; k++)
        if (total[k] < total[best]) best = k;
    c->opts.sort_interval = cand[best];
    *best_interval = cand[best];
    *ms_per_step = total[best] / (rounds * chunk);
    return MPMGPU_OK;
}

// Extension: mpmgpu_step that also returns the device time of the enqueued
// steps in *ms (CUDA events recorded on the context stream).
int mpmgpu_step_timed(MpmGpuCtx *c, int32_t nsteps, double t0, double *ms) {
    if (!ms) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_step_timed: null ms");
    return step_impl(c, nsteps, t0, ms);
}

int mpmgpu_step_host(MpmGpuCtx *c, MpmGpuParticles *h, int32_t nsteps, double t0) {
    if (!c || !h || nsteps < 0) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_step_host: bad argument");
    if (c->p.n <= 0 || !c->mats || h->n != c->p.n)
        return set_err(c, MPMGPU_ERR_INVALID,
                       "mpmgpu_step_host: upload a state of the same particle count first (it sizes the work arrays)");
    const size_t n = (size_t)c->p.n;
    // the kernels' view: the caller's columns where it gives them, the
    // uploaded device columns where it gives none; the natural coordinates
    // of the step stay on the device
    DevParticles view = c->p;
    view.host_resident = 1;
    double **cols[kParticleDoubles + 1];
    particle_columns(view, cols);
    double *hc[kParticleDoubles];
    hcols(h, hc);
    for (int k = 0; k < kParticleDoubles; k++) {
        if (!hc[k]) continue;
        double *d = mapped_column(hc[k], n);
        if (!d)
            return set_err(c, MPMGPU_ERR_INVALID,
                           "mpmgpu_step_host: a particle column lies outside the blocks of mpmgpu_host_alloc");
        *cols[k] = d;
    }
    view.mat = mapped_column(h->mat, n);
    view.elem = mapped_column(h->elem, n);
    if (!view.mat || !view.elem)
        return set_err(c, MPMGPU_ERR_INVALID,
                       "mpmgpu_step_host: material and element columns inside the blocks of mpmgpu_host_alloc are required");
    if (!c->iota) {
        cudaError_t e = cudaMalloc(&c->iota, n * sizeof(int));
        if (e != cudaSuccess) {
            c->iota = nullptr;
            return set_err(c, MPMGPU_ERR_OOM, std::string("identity order: ") + cudaGetErrorString(e));
        }
    }
    // the caller's material and element indices, range-checked as an upload
    // checks them (the kernels index tables with them)
    const int nelems = c->g.nx * c->g.ny * (c->dim == 3 ? c->g.nz : 1);
    CK(cudaMemsetAsync(c->err, 0, sizeof(unsigned), c->stream));
    const int TB = 256;
    k_upload_check<<<(int)((n + TB - 1) / TB), TB, 0, c->stream>>>(view.mat, view.elem, c->iota, (int)n, c->nmat,
                                                                  nelems, c->err);
    c->launches++;
    unsigned flags = 0;
    CK(cudaMemcpyAsync(&flags, c->err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (flags) {
        cudaMemsetAsync(c->err, 0, sizeof(unsigned), c->stream);
        cudaStreamSynchronize(c->stream);
        return set_err(c, MPMGPU_ERR_INVALID, "particle material or element index out of range");
    }
    // the host order is kept: no cell sort, identity slot order
    const DevParticles saved = c->p;
    int *const saved_orig = c->orig;
    const int saved_sort = c->opts.sort_interval;
    c->p = view;
    c->orig = c->iota;
    c->opts.sort_interval = 0;
    const int st = step_impl(c, nsteps, t0, nullptr);
    c->p = saved;
    c->orig = saved_orig;
    c->opts.sort_interval = saved_sort;
    return st;
}

int mpmgpu_download_particles(MpmGpuCtx *c, MpmGpuParticles *h) {
    if (!c || !h) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_download_particles: null argument");
    if (h->n != c->p.n) return set_err(c, MPMGPU_ERR_INVALID, "mpmgpu_download_particles: particle count mismatch");
    const int n = c->p.n;
    // bring columns back in the host's original particle order
    int st = unsort_to_scratch(c->sort, c->p, c->orig, c->pblock, kParticleDoubles + 1, c->stream);
    if (st != 0) return set_err(c, MPMGPU_ERR_CUDA, "unsort failed");
    double *hc[kParticleDoubles];
    hcols(h, hc);
    cudaError_t ce = cudaSuccess;
    column_runs(hc, (size_t)n, [&](int k, int e) {
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(hc[k], c->sort.scratch + (size_t)k * n, (size_t)(e - k) * n * sizeof(double),
                                 cudaMemcpyDeviceToHost, c->stream);
    });
    CK(ce);
    CK(cudaMemcpyAsync(h->mat, c->sort.iscratch, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(h->elem, c->sort.iscratch + n, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return MPMGPU_OK;
}

int64_t mpmgpu_archive_record_size(int32_t dim, const char *mpm_order) {
    ArchiveLayout L{};
    std::string why;
    const int st = archive_layout(dim, mpm_order, L, why);
    if (st != MPMGPU_OK) {
        set_err(nullptr, st, "mpmgpu_archive_record_size: " + why);
        return -st;
    }
    return L.rec;
}

namespace {

// pack the records of the current state into the staging buffer on the
// context stream; *bytes receives their size
int archive_pack(MpmGpuCtx *c, const char *what, const char *mpm_order, double thickness, const void *host_records,
                 int64_t capacity, size_t *bytes) {
    const std::string w(what);
    if (!c || !host_records) return set_err(c, MPMGPU_ERR_INVALID, w + ": null argument");
    if (c->p.n <= 0 || !c->mats) return set_err(c, MPMGPU_ERR_INVALID, w + ": no particles");
    ArchiveLayout L{};
    std::string why;
    const int st = archive_layout(c->dim, mpm_order, L, why);
    if (st != MPMGPU_OK) return set_err(c, st, w + ": " + why);
    L.thickness = thickness;
    *bytes = (size_t)c->p.n * L.rec;
    if (capacity < (int64_t)*bytes) return set_err(c, MPMGPU_ERR_INVALID, w + ": buffer too small");
    if (c->archive_pending) {
        // the previous asynchronous copy still reads the staging buffer
        const int ws = mpmgpu_archive_wait(c);
        if (ws != MPMGPU_OK) return ws;
    }
    if (c->archive_cap < *bytes) {
        if (c->archive_buf) cudaFree(c->archive_buf);
        c->archive_buf = nullptr;
        c->archive_cap = 0;
        cudaError_t e = cudaMalloc(&c->archive_buf, *bytes);
        if (e != cudaSuccess) return set_err(c, MPMGPU_ERR_OOM, "archive staging buffer");
        c->archive_cap = *bytes;
    }
    const int TB = 256, nb = (c->p.n + TB - 1) / TB;
    if (c->dim == 3)
        k_archive_pack<3><<<nb, TB, 0, c->stream>>>(L, c->p, c->orig, c->mats, (char *)c->archive_buf);
    else
        k_archive_pack<2><<<nb, TB, 0, c->stream>>>(L, c->p, c->orig, c->mats, (char *)c->archive_buf);
    c->launches++;
    CK(cudaGetLastError());
    return MPMGPU_OK;
}

}  // namespace

int mpmgpu_archive_records(MpmGpuCtx *c, const char *mpm_order, double thickness, void *host_records,
                           int64_t capacity) {
    size_t bytes = 0;
    const int st = archive_pack(c, "mpmgpu_archive_records", mpm_order, thickness, host_records, capacity, &bytes);
    if (st != MPMGPU_OK) return st;
    CK(cudaMemcpyAsync(host_records, c->archive_buf, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return MPMGPU_OK;
}

int mpmgpu_archive_records_async(MpmGpuCtx *c, const char *mpm_order, double thickness, void *host_records,
                                 int64_t capacity) {
    size_t bytes = 0;
    const int st =
        archive_pack(c, "mpmgpu_archive_records_async", mpm_order, thickness, host_records, capacity, &bytes);
    if (st != MPMGPU_OK) return st;
    if (!c->archive_stream) {
        CK(cudaStreamCreateWithFlags(&c->archive_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->archive_packed, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->archive_copied, cudaEventDisableTiming));
    }
    // the copy waits for the pack; later steps on the context stream do not
    // wait for the copy (the next pack does)
    CK(cudaEventRecord(c->archive_packed, c->stream));
    CK(cudaStreamWaitEvent(c->archive_stream, c->archive_packed, 0));
    CK(cudaMemcpyAsync(host_records, c->archive_buf, bytes, cudaMemcpyDeviceToHost, c->archive_stream));
    CK(cudaEventRecord(c->archive_copied, c->archive_stream));
    c->archive_pending = true;
    return MPMGPU_OK;
}

int mpmgpu_archive_wait(MpmGpuCtx *c) {
    if (!c) return set_err(nullptr, MPMGPU_ERR_INVALID, "mpmgpu_archive_wait: null context");
    if (!c->archive_pending) return MPMGPU_OK;
    c->archive_pending = false;
    CK(cudaEventSynchronize(c->archive_copied));
    return MPMGPU_OK;
}

void mpmgpu_destroy(MpmGpuCtx *c) {
    if (!c) return;
    free_particles(c);
    if (c->mats) cudaFree(c->mats);
    if (c->grid_coords) cudaFree(c->grid_coords);
    if (c->nblock) cudaFree(c->nblock);
    if (c->fblock) cudaFree(c->fblock);
    if (c->bc_group) cudaFree(c->bc_group);
    if (c->bc_block) cudaFree(c->bc_block);
    if (c->err) cudaFree(c->err);
    if (c->archive_pending) cudaEventSynchronize(c->archive_copied);
    if (c->archive_buf) cudaFree(c->archive_buf);
    if (c->xpic_block) cudaFree(c->xpic_block);
    if (c->archive_packed) cudaEventDestroy(c->archive_packed);
    if (c->archive_copied) cudaEventDestroy(c->archive_copied);
    if (c->archive_stream) cudaStreamDestroy(c->archive_stream);
    for (void *q : {(void *)c->lr_cnt, (void *)c->lr_start, (void *)c->lr_list, (void *)c->lr_sums, (void *)c->lr_out})
        if (q) cudaFree(q);
    if (c->det.lim) cudaFree(c->det.lim);
    if (c->det.bnd) cudaFree(c->det.bnd);
    if (c->det.nbnd) cudaFree(c->det.nbnd);
    for (auto &e : c->ev) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int mpmgpu_profile(const MpmGpuCtx *c, const char **names, double *ms, int32_t cap) {
    if (!c) return 0;
    int k = 0;
    for (const auto &pr : c->prof) {
        if (k >= cap) break;
        if (names) names[k] = pr.name;
        if (ms) ms[k] = pr.ms;
        k++;
    }
    return k;
}

// Extension: enable per-kernel CUDA-event timing on the context stream (adds a
// synchronisation per step; for profiling runs only).
int mpmgpu_set_profiling(MpmGpuCtx *c, int32_t on) {
    if (!c) return MPMGPU_ERR_INVALID;
    c->profile = on != 0;
    return MPMGPU_OK;
}

// Extension: the context's CUDA stream, for callers that time with their own events.
void *mpmgpu_stream(MpmGpuCtx *c) { return c ? (void *)c->stream : nullptr; }

// Stable sort of particles by element: see include/nairn_mpm_gpu.h.
int mpmgpu_sort_by_cell(const int32_t *d_elem, int32_t n, int32_t nelems, int32_t *d_perm, void *stream) {
    MpmGpuCtx *c = nullptr;  // for CK: errors go to the static message
    if (!d_elem || !d_perm || n <= 0 || nelems <= 0)
        return set_err(nullptr, MPMGPU_ERR_INVALID, "mpmgpu_sort_by_cell: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    int bits = 1;
    while ((1LL << bits) < (long long)nelems) bits++;
    const int ntiles = (n + kTile - 1) / kTile;
    const size_t nsums = (size_t)(256 * ntiles + kScanChunk - 1) / kScanChunk + 1;
    int *buf = nullptr;
    const size_t ints = 4 * (size_t)n + 256 * (size_t)ntiles + nsums;
    cudaError_t e = cudaMalloc(&buf, ints * sizeof(int));
    if (e != cudaSuccess) return set_err(nullptr, MPMGPU_ERR_OOM, std::string("sort scratch: ") + cudaGetErrorString(e));
    int *keys[2] = {buf, buf + n}, *vals[2] = {buf + 2 * (size_t)n, buf + 3 * (size_t)n};
    int *hist = buf + 4 * (size_t)n, *sums = hist + 256 * (size_t)ntiles;
    const int cur = radix_sort_keys(d_elem, n, bits, keys, vals, hist, sums, s);
    e = cudaMemcpyAsync(d_perm, vals[cur], sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(c, e, "mpmgpu_sort_by_cell");
    return MPMGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free cell sort.  Its scratch (two key and two value buffers, the
// per-tile digit histogram and the scan block sums) lives in one file-scope
// device array sized for MPMGPU_NOALLOC_MAX_PARTICLES particles (2.25 MiB),
// which every GPU that loads this library holds until the process exits.
// ---------------------------------------------------------------------------
namespace {
constexpr int kNoAllocTiles = (MPMGPU_NOALLOC_MAX_PARTICLES + kTile - 1) / kTile;
constexpr size_t kNoAllocSums = (256 * (size_t)kNoAllocTiles + kScanChunk - 1) / kScanChunk + 1;
constexpr size_t kNoAllocInts = 4 * (size_t)MPMGPU_NOALLOC_MAX_PARTICLES + 256 * (size_t)kNoAllocTiles + kNoAllocSums;
}  // namespace

static __device__ __align__(256) int g_noalloc_sort_scratch[kNoAllocInts];

namespace {
// Device address of g_noalloc_sort_scratch in the context current on the
// calling thread.  In host code the array's name only stands in for the
// symbol; its address comes from cudaGetSymbolAddress with the device
// current.  The lookup is repeated on every call (it is a host-side query that
// allocates nothing), so an address never outlives the context it came from:
// after cudaDeviceReset, or with another context current on the same device,
// the next call finds the array's address there.
int noalloc_scratch(int **base) {
    int *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_sort_scratch);
    if (e != cudaSuccess || !p)
        return cuda_fail(nullptr, e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                         "mpmgpu_sort_by_cell_noalloc: cudaGetSymbolAddress");
    *base = p;
    return MPMGPU_OK;
}
}  // namespace

extern "C" {

int mpmgpu_sort_by_cell_noalloc(const int32_t *d_elem, int32_t n, int32_t nelems, int32_t *d_perm, void *stream) {
    if (!d_elem || !d_perm || n <= 0 || nelems <= 0)
        return set_err(nullptr, MPMGPU_ERR_INVALID, "mpmgpu_sort_by_cell_noalloc: bad argument");
    if (n > MPMGPU_NOALLOC_MAX_PARTICLES)
        return set_err(nullptr, MPMGPU_ERR_INVALID,
                       "mpmgpu_sort_by_cell_noalloc: n = " + std::to_string(n) + " exceeds the maximum of " +
                           std::to_string(MPMGPU_NOALLOC_MAX_PARTICLES) +
                           " particles this allocation-free variant supports; use mpmgpu_sort_by_cell");
    // an error left pending by earlier, unrelated work is reported as such
    // (and left pending for its owner) rather than blamed on this sort
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
        return set_err(nullptr, MPMGPU_ERR_CUDA,
                       std::string("mpmgpu_sort_by_cell_noalloc: a CUDA error was pending before the call: ") +
                           cudaGetErrorString(pending));
    int *base = nullptr;
    int st = noalloc_scratch(&base);
    if (st != MPMGPU_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    int bits = 1;
    while ((1LL << bits) < (long long)nelems) bits++;
    const int ntiles = (n + kTile - 1) / kTile;
    int *keys[2] = {base, base + n}, *vals[2] = {base + 2 * (size_t)n, base + 3 * (size_t)n};
    int *hist = base + 4 * (size_t)n, *sums = hist + 256 * (size_t)ntiles;
    // every scratch word the sort reads is written earlier in the same call
    // (keys/vals by k_sort_init and each scatter, the histogram for all tiles
    // and digits, the scan sums), so nothing needs clearing between calls
    const int cur = radix_sort_keys(d_elem, n, bits, keys, vals, hist, sums, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_perm, vals[cur], sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "mpmgpu_sort_by_cell_noalloc");
    return MPMGPU_OK;
}

// Extension: number of kernels this context has launched so far.
long long mpmgpu_launch_count(const MpmGpuCtx *c) { return c ? c->launches : 0; }

// Extension: page-lock caller memory so uploads and downloads run as async DMA.
int mpmgpu_host_register(void *ptr, uint64_t bytes) {
    if (!ptr || !bytes) return MPMGPU_ERR_INVALID;
    cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
    return e == cudaSuccess ? MPMGPU_OK : cuda_fail(nullptr, e, "cudaHostRegister");
}

int mpmgpu_host_unregister(void *ptr) {
    if (!ptr) return MPMGPU_ERR_INVALID;
    cudaError_t e = cudaHostUnregister(ptr);
    return e == cudaSuccess ? MPMGPU_OK : cuda_fail(nullptr, e, "cudaHostUnregister");
}

int mpmgpu_host_alloc(uint64_t bytes, void **ptr) {
    if (!ptr || !bytes) return MPMGPU_ERR_INVALID;
    *ptr = nullptr;
    cudaError_t e = cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocPortable | cudaHostAllocMapped);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return cuda_fail(nullptr, e, "cudaHostAlloc");
    }
    std::lock_guard<std::mutex> lk(g_host_mu);
    g_host_blocks[(uintptr_t)*ptr] = (size_t)bytes;
    return MPMGPU_OK;
}

void mpmgpu_host_free(void *ptr) {
    if (!ptr) return;
    {
        std::lock_guard<std::mutex> lk(g_host_mu);
        g_host_blocks.erase((uintptr_t)ptr);
    }
    cudaFreeHost(ptr);
}

}  // extern "C"
