// mpm_kernels.cuh -- kernels of one explicit MPM step (FP64 path).
//
// Step structure (the reference task chain, NairnMPM.cpp:870-1110, regrouped):
//   k_p2g            InitializationTask + MassAndMomentumTask      (particles)
//   k_node_post      PostExtrapolationTask + velocity BCs + v=p/m  (nodes)
//   k_strain_forces  UpdateStrainsFirstTask fused with GridForcesTask (particles)
//   k_node_update    PostForcesTask + UpdateMomentaTask + BCs + v  (nodes)
//   k_g2p            UpdateParticlesTask fused with the momentum
//                    re-extrapolation of UpdateStrainsLastContactTask (particles)
//   k_node_usl       velocity BCs of the second extrapolation + v  (nodes)
//   k_strain_last    second strain update fused with ResetElementsTask (particles)
// Fusing is exact: each fused pair only uses the particle's own data between
// the two halves, and the grid data both halves read is complete beforehand.
#pragma once

#include <climits>
#include <type_traits>

#include "mpm_device.cuh"

namespace nmg {

enum { SHAPE_LINEAR = 0, SHAPE_UGIMP = 1, SHAPE_LCPDI = 2, SHAPE_BSPLINE = 3, SHAPE_BGIMP = 4, SHAPE_QCPDI = 5 };

// CPDI shape functions: the particle domain's points carry the grid's linear
// shape functions (ElementBase::GetCPDIFunctions, MoreMPMElementBase.cpp:581-656)
template <int SHAPE>
constexpr bool kCpdi = SHAPE == SHAPE_LCPDI || SHAPE == SHAPE_QCPDI;
// domain points per particle (ElementBase::InitializeCPDI, MoreMPMElementBase.cpp:1005-1020):
// the lCPDI corners, or qCPDI's corners, edge midpoints and material point (2D)
template <int DIM, int SHAPE>
constexpr int kCpdiPts = SHAPE == SHAPE_QCPDI ? 9 : (DIM == 3 ? 8 : 4);

// shape weight of domain point c (MPMBase.cpp:163-173)
template <int DIM, int SHAPE, typename T>
__device__ __forceinline__ T cpdi_ws(int c) {
    if constexpr (SHAPE == SHAPE_QCPDI) return c < 4 ? T(1. / 36.) : (c < 8 ? T(1. / 9.) : T(4. / 9.));
    else return DIM == 3 ? T(0.125) : T(0.25);
}

// position of domain point c as pos + s1 r1 + s2 r2 + s3 r3 (MatPoint2D.cpp:519-640,
// MatPoint3D.cpp:538-601): lCPDI corners counter-clockwise (then the upper
// layer in 3D); qCPDI adds the edge midpoints -r2, +r1, +r2, -r1 and the
// material point itself
template <int SHAPE, typename T>
__device__ __forceinline__ void cpdi_signs(int c, T &s1, T &s2, T &s3) {
    if constexpr (SHAPE == SHAPE_QCPDI) {
        s1 = (c == 1 || c == 2 || c == 5) ? T(1) : ((c == 0 || c == 3 || c == 7) ? T(-1) : T(0));
        s2 = (c == 2 || c == 3 || c == 6) ? T(1) : ((c == 0 || c == 1 || c == 4) ? T(-1) : T(0));
        s3 = T(0);
    } else {
        s1 = (c == 1 || c == 2 || c == 5 || c == 6) ? T(1) : T(-1);
        s2 = (c == 2 || c == 3 || c == 6 || c == 7) ? T(1) : T(-1);
        s3 = c >= 4 ? T(1) : T(-1);
    }
}

// Resident 256-thread blocks per SM the strain kernels are compiled for (this
// caps their registers at 80): their FP64 constitutive updates are latency
// bound at the two blocks the uncapped register count allows.  lCPDI kernels
// keep their registers (the 27-node window); capping them spills.  So do qCPDI's.
template <int SHAPE>
constexpr int kStrainBlocks = kCpdi<SHAPE> ? 2 : 3;

// ---------------------------------------------------------------------------
// deterministic node sums (MPMGPU_P2G_DETERMINISTIC)
// ---------------------------------------------------------------------------
// Every contribution v to a node quantity is rounded once to an integer
// multiple of 2^-k, where a bound B on |v| fixes k so that |v| 2^k < 2^103,
// and that integer is added as three limbs of 42 bits (v 2^k = l0 + l1 2^42 +
// l2 2^84, each limb a signed 64-bit sum).  Integer addition is associative,
// so a node sum -- and all that is computed from it -- is the same bit for bit
// whatever order threads add in, whatever the particle order and launch shape.
// A limb holds 2^20 contributions before it could overflow.
//
// Mass-like quantities are scaled per node: B is the node's largest mass
// contribution N mp (found by k_det_bounds), times a step-wide bound on the
// ratio to mass for momentum (|v|), contact volume (V/m) and mass-weighted
// displacement (|x - x0|).  So a node touched only by the far edge of a
// particle's support (N ~ 1e-30 in uGIMP) keeps 2^-102 relative resolution:
// its velocity p/m and acceleration f/m are then as accurate as the FP64
// sums', which matters because such a node's velocity enters the particle's
// velocity gradient through grad N ~ sqrt(N).  Forces and volume gradients,
// which scale with grad N, use a step-wide B.
enum { DQ_MASS = 0, DQ_PX, DQ_PY, DQ_PZ, DQ_FX, DQ_FY, DQ_FZ, DQ_UX, DQ_UY, DQ_UZ,
       DQ_VOL, DQ_DSX, DQ_DSY, DQ_DSZ, DQ_GVX, DQ_GVY, DQ_GVZ, kDetQuantities };
// step-wide bound slots: largest |v|, internal force, |v| after the particle
// update, and for contact V/m, |x - x0| and the volume-gradient terms of the
// first (P2G) and second (USL) extrapolations
enum { DB_MOM = 0, DB_FORCE, DB_UMOM, DB_VOL, DB_DS, DB_GV, DB_UVOL, DB_UDS, DB_UGV, kDetBounds };

// exponent e of a bound (the bits of a non-negative double) with B < 2^(e+1)
__device__ __forceinline__ int det_exp(unsigned long long bits) {
    const int ex = (int)(bits >> 52);
    return ex ? ex - 1023 : -1023;
}

__device__ __forceinline__ int det_clamp(int k) { return k > 1000 ? 1000 : (k < -1000 ? -1000 : k); }

// k for contributions bounded by B: 2^(e+1) 2^k = 2^103
__device__ __forceinline__ int det_shift(unsigned long long bits) {
    return bits == 0ull ? 0 : det_clamp(102 - det_exp(bits));
}

// k for contributions bounded by the product of two bounds
__device__ __forceinline__ int det_shift2(unsigned long long a, unsigned long long b) {
    return (a == 0ull || b == 0ull) ? 0 : det_clamp(101 - det_exp(a) - det_exp(b));
}

// 2^k as a double, -1022 <= k <= 1023
__device__ __forceinline__ double pow2(int k) { return __longlong_as_double((long long)(k + 1023) << 52); }

// add v 2^k, rounded to the nearest integer (ties away from zero), to the
// limbs of quantity q at node n
__device__ __forceinline__ void det_add(const DevDet &d, int q, int n, double v, double scale, unsigned *err) {
    const double t = v * scale;
    const unsigned long long b = (unsigned long long)__double_as_longlong(t);
    const int ex = (int)((b >> 52) & 0x7ffull);
    if (ex == 0x7ff || ex > 1075 + 51) {  // NaN, infinite or beyond 2^104: the bound did not hold
        atomicOr(err, ERR_RANGE);
        return;
    }
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (ex ? (1ull << 52) : 0ull);
    const int sh = (ex ? ex : 1) - 1075;  // |t| = m 2^sh
    constexpr unsigned long long M42 = (1ull << 42) - 1;
    unsigned long long l0, l1, l2;
    if (sh >= 0) {
        const unsigned __int128 X = (unsigned __int128)m << sh;
        l0 = (unsigned long long)X & M42;
        l1 = (unsigned long long)(X >> 42) & M42;
        l2 = (unsigned long long)(X >> 84);
    } else if (sh > -54) {
        const unsigned long long X = (m + (1ull << (-sh - 1))) >> (-sh);
        l0 = X & M42;
        l1 = X >> 42;
        l2 = 0ull;
    } else {
        return;  // |t| < 1/2 rounds to zero
    }
    if (b >> 63) {
        l0 = 0ull - l0;
        l1 = 0ull - l1;
        l2 = 0ull - l2;
    }
    unsigned long long *L = (unsigned long long *)d.lim + (size_t)(3 * q) * d.stride + n;
    if (l0) atomicAdd(L, l0);
    if (l1) atomicAdd(L + d.stride, l1);
    if (l2) atomicAdd(L + 2 * d.stride, l2);
}

// the node sum of quantity q as a double (times 2^-k via inv_scale); the
// limbs are cleared for the next accumulation
__device__ __forceinline__ double det_take(const DevDet &d, int q, int n, double inv_scale) {
    long long *L = d.lim + (size_t)(3 * q) * d.stride + n;
    long long a0 = L[0], a1 = L[d.stride], a2 = L[2 * d.stride];
    if ((a0 | a1 | a2) == 0) return 0.;
    L[0] = 0;
    L[d.stride] = 0;
    L[2 * d.stride] = 0;
    // carry into normalised limbs r0, r1 in [0, 2^42)
    const long long c0 = a0 >> 42;
    const long long r0 = a0 - c0 * (1ll << 42);
    a1 += c0;
    const long long c1 = a1 >> 42;
    const long long r1 = a1 - c1 * (1ll << 42);
    a2 += c1;
    const double lowpart = (double)r1 * 4398046511104.0 + (double)r0;  // r1 2^42 + r0, one rounding
    return ((double)a2 * 19342813113834066795298816.0 + lowpart) * inv_scale;  // a2 2^84 + ...
}

// raise bound slot `slot` to at least v (v >= 0) -- one atomic per warp
__device__ __forceinline__ void det_bound(const DevDet &d, int slot, double v) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const unsigned mask = __activemask();
    const unsigned hi = __reduce_max_sync(mask, (unsigned)(bits >> 32));
    const unsigned lo = __reduce_max_sync(mask, (unsigned)(bits >> 32) == hi ? (unsigned)bits : 0u);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(mask) - 1)) {
        const unsigned long long w = ((unsigned long long)hi << 32) | lo;
        if (w > d.bnd[slot]) atomicMax(d.bnd + slot, w);
    }
}

// Visit the nodes of one particle, calling f(node0based, N, dNdx, dNdy, dNdz).
// ElementBase::GetShapeFunctions / GetShapeGradients
// (NairnMPM/src/Elements/MoreMPMElementBase.cpp:120-284).  T is the arithmetic
// of the weights: double in the FP64 path, float in the mixed-precision mode
// (natural coordinates are formed in FP64 and rounded once).
template <int DIM, int SHAPE, bool GRAD, typename T, class F>
__device__ __forceinline__ void for_each_node(const DevGrid &g, int nb, int e, double xi_d, double eta_d,
                                              double zeta_d, double lpx_d, double lpy_d, double lpz_d, F &&f) {
    int col, row, zr;
    elem_coords(g, e, col, row, zr);
    const int n0 = nb + zr * g.zplane + row * g.yplane + col;  // first node (global index)
    // reciprocal element sizes, formed once (a gradient times 1/dx differs from
    // the reference's quotient by rounding only)
    const T iDX = GRAD ? recip((T)(g.xn[col + 1] - g.xn[col])) : T(0);
    const T iDY = GRAD ? recip((T)(g.yn[row + 1] - g.yn[row])) : T(0);
    const T iDZ = GRAD && DIM == 3 ? recip((T)(g.zn[zr + 1] - g.zn[zr])) : T(0);
    const T xi = (T)xi_d, eta = (T)eta_d, zeta = (T)zeta_d;
    if (SHAPE == SHAPE_LINEAR) {
        if (DIM == 2) {
            // FourNodeIsoparam::ShapeFunction (6-argument form), FourNodeIsoparam.cpp:189-212
            const int off[4] = {0, 1, 1 + g.yplane, g.yplane};
            const T xs[4] = {-1, 1, 1, -1}, es[4] = {-1, -1, 1, 1};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const T t1 = T(1) + xs[i] * xi, t2 = T(1) + es[i] * eta;
                T dx = 0, dy = 0;
                if (GRAD) {
                    dx = T(0.5) * xs[i] * t2 * iDX;
                    dy = T(0.5) * es[i] * t1 * iDY;
                }
                f(n0 + off[i], T(0.25) * t1 * t2, dx, dy, T(0));
            }
        } else {
            // EightNodeIsoparamBrick::ShapeFunction (6-argument form), EightNodeIsoparamBrick.cpp:90-104
            const T xs[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
            const T es[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
            const T zs[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int off = (i == 1 || i == 5 ? 1 : 0) + (i == 2 || i == 6 ? 1 + g.yplane : 0) +
                                (i == 3 || i == 7 ? g.yplane : 0) + (i >= 4 ? g.zplane : 0);
                const T t1 = T(1) + xs[i] * xi, t2 = T(1) + es[i] * eta, t3 = T(1) + zs[i] * zeta;
                T dx = 0, dy = 0, dz = 0;
                if (GRAD) {
                    dx = T(0.25) * xs[i] * t2 * t3 * iDX;
                    dy = T(0.25) * es[i] * t1 * t3 * iDY;
                    dz = T(0.25) * zs[i] * t1 * t2 * iDZ;
                }
                f(n0 + off, T(0.125) * t1 * t2 * t3, dx, dy, dz);
            }
        }
        return;
    }
    const T lpx = (T)lpx_d, lpy = (T)lpy_d, lpz = (T)lpz_d;
    if constexpr (SHAPE == SHAPE_BGIMP) {
        // B2GIMP over its four-node window per axis (see bgimp_window)
        Win4<T> wx, wy;
        bgimp_window<T, DIM == 3, GRAD>(xi, lpx, GRAD ? T(2) * iDX : T(0), xi, wx);
        bgimp_window<T, DIM == 3, GRAD>(eta, lpy, GRAD ? T(2) * iDY : T(0), eta, wy);
        const int base = n0 - 1 - g.yplane;
        if (DIM == 2) {
#pragma unroll
            for (int jy = 0; jy < 4; jy++)
#pragma unroll
                for (int jx = 0; jx < 4; jx++)
                    f(base + jx + jy * g.yplane, wx.S[jx] * wy.S[jy], GRAD ? wx.dS[jx] * wy.S[jy] : T(0),
                      GRAD ? wx.S[jx] * wy.dS[jy] : T(0), T(0));
        } else {
            Win4<T> wz;
            bgimp_window<T, true, GRAD>(zeta, lpz, GRAD ? T(2) * iDZ : T(0), eta, wz);
            const int base3 = base - g.zplane;
#pragma unroll
            for (int jz = 0; jz < 4; jz++)
#pragma unroll
                for (int jy = 0; jy < 4; jy++) {
                    const T Syz = wy.S[jy] * wz.S[jz];
#pragma unroll
                    for (int jx = 0; jx < 4; jx++)
                        f(base3 + jx + jy * g.yplane + jz * g.zplane, wx.S[jx] * Syz,
                          GRAD ? wx.dS[jx] * Syz : T(0), GRAD ? wx.S[jx] * wy.dS[jy] * wz.S[jz] : T(0),
                          GRAD ? wx.S[jx] * wy.S[jy] * wz.dS[jz] : T(0));
                }
        }
        return;
    }
    // uGIMP or B2SPLINE over the particle's window (see gimp_window and
    // bspline_window); f is called for every window node, with N == 0
    // marking a node outside the support.
    Win<T> wx, wy;
    if constexpr (SHAPE == SHAPE_BSPLINE) {
        bspline_window<T, GRAD>(xi, GRAD ? iDX : T(0), wx);
        bspline_window<T, GRAD>(eta, GRAD ? iDY : T(0), wy);
    } else {
        const T ix = recip(T(4) * lpx), iy = recip(T(4) * lpy);
        gimp_window<T, DIM == 3, GRAD>(xi, lpx, ix, T(2) * ix, GRAD ? T(2) * iDX : T(0), wx);
        gimp_window<T, DIM == 3, GRAD>(eta, lpy, iy, T(2) * iy, GRAD ? T(2) * iDY : T(0), wy);
    }
    const int base = n0 + (wx.s - 1) + (wy.s - 1) * g.yplane;
    if (DIM == 2) {
#pragma unroll
        for (int jy = 0; jy < 3; jy++) {
#pragma unroll
            for (int jx = 0; jx < 3; jx++) {
                const T Sx = wx.S[jx], Sy = wy.S[jy];
                T dx = 0, dy = 0;
                if (GRAD) {
                    dx = wx.dS[jx] * Sy;
                    dy = Sx * wy.dS[jy];
                }
                f(base + jx + jy * g.yplane, Sx * Sy, dx, dy, T(0));
            }
        }
    } else {
        Win<T> wz;
        if constexpr (SHAPE == SHAPE_BSPLINE) {
            bspline_window<T, GRAD>(zeta, GRAD ? iDZ : T(0), wz);
        } else {
            // the z factor is sized by lp.y (EightNodeIsoparamBrick.cpp:289-403); its
            // gradient by lp.z
            const T iy = recip(T(4) * lpy);
            const T hz = !GRAD ? T(0) : (lpz == lpy ? T(2) * iy : recip(T(2) * lpz));
            gimp_window<T, true, GRAD>(zeta, lpz, iy, hz, GRAD ? T(2) * iDZ : T(0), wz);
        }
        const int base3 = base + (wz.s - 1) * g.zplane;
#pragma unroll
        for (int jz = 0; jz < 3; jz++) {
#pragma unroll
            for (int jy = 0; jy < 3; jy++) {
                const T Syz = wy.S[jy] * wz.S[jz];
                const T dySz = GRAD ? wy.dS[jy] * wz.S[jz] : T(0);
                const T SydZ = GRAD ? wy.S[jy] * wz.dS[jz] : T(0);
#pragma unroll
                for (int jx = 0; jx < 3; jx++) {
                    const T Sx = wx.S[jx];
                    T dx = 0, dy = 0, dz = 0;
                    if (GRAD) {
                        dx = wx.dS[jx] * Syz;
                        dy = Sx * dySz;
                        dz = Sx * SydZ;
                    }
                    f(base3 + jx + jy * g.yplane + jz * g.zplane, Sx * Syz, dx, dy, dz);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// linear CPDI
// ---------------------------------------------------------------------------

// MeshInfo::FindElementFromPoint for equal element sizes (MeshInfo.cpp:593-633):
// truncated cell index, the grid's far edge clamped; -1 when off the grid.
__device__ __forceinline__ int find_cell(double x, double xmin, double gx, double igx, int n) {
    // (x - xmin) * (1/gx) can differ from the quotient by an ulp, which moves a
    // point lying on a cell boundary to the neighbouring cell; the linear
    // shape functions of both cells agree on their shared face, so the CPDI
    // weights do not change
    int c = (int)((x - xmin) * igx);
    if (c < 0 || c >= n) {
        if (x == xmin + n * gx) c = n - 1;
        else c = -1;
    }
    return c;
}

// Corner data of the step: the FP64 path keeps natural coordinates and
// gradient weights as doubles; the mixed mode keeps them as floats in the same
// scratch (index k = (3 c + a) n + i either way).
template <typename T>
__device__ __forceinline__ T cpdi_xi(const DevParticles &p, size_t k) {
    if constexpr (std::is_same<T, float>::value) return reinterpret_cast<const float *>(p.cxi)[k];
    else return p.cxi[k];
}
template <typename T>
__device__ __forceinline__ T cpdi_wg(const DevParticles &p, size_t k) {
    if constexpr (std::is_same<T, float>::value) return reinterpret_cast<const float *>(p.cwg)[k];
    else return p.cwg[k];
}

// MatPoint2D/3D::GetCPDINodesAndWeights (MatPoint2D.cpp:519-571,
// MatPoint3D.cpp:538-601): semi-side vectors r = F * (cell * lp / 2) of the
// particle (GetSemiSideVectors, GetParticleSize), corners x +- r1 +- r2 (+- r3)
// in the reference's order, their elements and natural coordinates, and the
// gradient weights.  The reference throws when a corner is off the grid or the
// particle touches more than 16 (2D) / 49 (3D) nodes (GetCPDIFunctions); here
// those set ERR_LEFT_GRID / ERR_CPDI_NODES.  Returns false on an error.
template <int DIM, int SHAPE>
static __device__ bool cpdi_setup(const DevGrid &g, const DevParticles &p, int i, unsigned *err) {
    constexpr int NC = kCpdiPts<DIM, SHAPE>;
    const size_t n = (size_t)p.n;
    int col, row, zr;
    elem_coords(g, p.elem[i], col, row, zr);
    double pszx = g.xn[col + 1] - g.xn[col], pszy = g.yn[row + 1] - g.yn[row];
    pszx *= 0.5 * p.lpx[i];
    pszy *= 0.5 * p.lpy[i];
    const double F00 = 1. + p.exx[i], F01 = 0.5 * (p.exy[i] - p.wxy[i]), F10 = 0.5 * (p.exy[i] + p.wxy[i]);
    const double F11 = 1. + p.eyy[i];
    double r1[3], r2[3], r3[3] = {0., 0., 0.};
    r1[0] = F00 * pszx;
    r1[1] = F10 * pszx;
    r2[0] = F01 * pszy;
    r2[1] = F11 * pszy;
    if (DIM == 3) {
        double pszz = g.zn[zr + 1] - g.zn[zr];
        pszz *= 0.5 * p.lpz[i];
        const double F02 = 0.5 * (p.exz[i] - p.wxz[i]), F20 = 0.5 * (p.exz[i] + p.wxz[i]);
        const double F12 = 0.5 * (p.eyz[i] - p.wyz[i]), F21 = 0.5 * (p.eyz[i] + p.wyz[i]);
        r1[2] = F20 * pszx;
        r2[2] = F21 * pszy;
        r3[0] = F02 * pszz;
        r3[1] = F12 * pszz;
        r3[2] = (1. + p.ezz[i]) * pszz;
    } else {
        r1[2] = r2[2] = 0.;
    }
    const double pos[3] = {p.x[i], p.y[i], DIM == 3 ? p.z[i] : 0.};
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-1, -1, -1};
#pragma unroll
    for (int c = 0; c < NC; c++) {
        double s1, s2, s3;
        cpdi_signs<SHAPE>(c, s1, s2, s3);
        double cp[3];
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            cp[a] = pos[a] + s1 * r1[a] + s2 * r2[a];
            if (DIM == 3) cp[a] += s3 * r3[a];
        }
        // qCPDI's material point lies in the particle's own element
        // (MatPoint2D.cpp:627-629); the other points are looked up
        const bool own = SHAPE == SHAPE_QCPDI && c == 8;
        const int cc = own ? col : find_cell(cp[0], g.xmin, g.gx, g.igx, g.nx);
        const int cr = own ? row : find_cell(cp[1], g.ymin, g.gy, g.igy, g.ny);
        const int cz = DIM == 3 ? find_cell(cp[2], g.zmin, g.gz, g.igz, g.nz) : 0;
        if (cc < 0 || cr < 0 || cz < 0) {
            atomicOr(err, ERR_LEFT_GRID);
            return false;
        }
        p.ce[c * n + i] = DIM == 3 ? g.nx * (cz * g.ny + cr) + cc : cr * g.nx + cc;
        // GetXiPos (2x - xmin - xmax) / dx with the equal cell size of a
        // regular grid (the element extents differ from it by rounding only)
        p.cxi[(3 * c + 0) * n + i] = (2. * cp[0] - g.xn[cc] - g.xn[cc + 1]) * g.igx;
        p.cxi[(3 * c + 1) * n + i] = (2. * cp[1] - g.yn[cr] - g.yn[cr + 1]) * g.igy;
        if (DIM == 3) p.cxi[(3 * c + 2) * n + i] = (2. * cp[2] - g.zn[cz] - g.zn[cz + 1]) * g.igz;
        const int cell[3] = {cc, cr, cz};
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            lo[a] = min(lo[a], cell[a]);
            hi[a] = max(hi[a], cell[a]);
        }
    }
    // gradient weights
    if (DIM == 2) {
        // qCPDI takes the linear weights over 3 Ap, and its edge points 4 r / (3 Ap)
        // (MatPoint2D.cpp:620-640)
        const double Ap = SHAPE == SHAPE_QCPDI ? 1. / (3. * (4. * (r1[0] * r2[1] - r1[1] * r2[0])))
                                               : 1. / (4. * (r1[0] * r2[1] - r1[1] * r2[0]));
        const double wx[4] = {r1[1] - r2[1], r1[1] + r2[1], -r1[1] + r2[1], -r1[1] - r2[1]};
        const double wy[4] = {-r1[0] + r2[0], -r1[0] - r2[0], r1[0] - r2[0], r1[0] + r2[0]};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            p.cwg[(3 * c + 0) * n + i] = wx[c] * Ap;
            p.cwg[(3 * c + 1) * n + i] = wy[c] * Ap;
        }
        if constexpr (SHAPE == SHAPE_QCPDI) {
            const double ex[5] = {4. * r1[1] * Ap, 4. * r2[1] * Ap, -4. * r1[1] * Ap, -4. * r2[1] * Ap, 0.};
            const double ey[5] = {-4. * r1[0] * Ap, -4. * r2[0] * Ap, 4. * r1[0] * Ap, 4. * r2[0] * Ap, 0.};
#pragma unroll
            for (int c = 0; c < 5; c++) {
                p.cwg[(3 * (4 + c) + 0) * n + i] = ex[c];
                p.cwg[(3 * (4 + c) + 1) * n + i] = ey[c];
            }
        }
    } else {
        // the reference's per-corner expressions are signed sums of the cross
        // products r1 x r2, r1 x r3 and r2 x r3 divided by the volume
        const double a12[3] = {r1[1] * r2[2] - r1[2] * r2[1], r1[2] * r2[0] - r1[0] * r2[2], r1[0] * r2[1] - r1[1] * r2[0]};
        const double a13[3] = {r1[1] * r3[2] - r1[2] * r3[1], r1[2] * r3[0] - r1[0] * r3[2], r1[0] * r3[1] - r1[1] * r3[0]};
        const double a23[3] = {r2[1] * r3[2] - r2[2] * r3[1], r2[2] * r3[0] - r2[0] * r3[2], r2[0] * r3[1] - r2[1] * r3[0]};
        const double Vp = 1. / (8. * (r1[0] * a23[0] + r1[1] * a23[1] + r1[2] * a23[2]));
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const double s1 = (c == 1 || c == 2 || c == 5 || c == 6) ? 1. : -1.;
            const double s2 = (c == 2 || c == 3 || c == 6 || c == 7) ? 1. : -1.;
            const double s3 = c >= 4 ? 1. : -1.;
            // wg = (s1 r2 x r3 - s2 r1 x r3 + s3 r1 x r2) / V (MatPoint3D.cpp:571-594)
#pragma unroll
            for (int a = 0; a < 3; a++) p.cwg[(3 * c + a) * n + i] = (s1 * a23[a] - s2 * a13[a] + s3 * a12[a]) * Vp;
        }
    }
    // node count check (3D only: four 2D corner elements touch at most the 16
    // nodes the 2D limit allows); spans of up to 2 cells per axis touch at
    // most 27 nodes
    bool small = true;
#pragma unroll
    for (int a = 0; a < DIM; a++) small = small && hi[a] - lo[a] <= 1;
    if (DIM == 3 && !small) {
        // distinct nodes with a weight of at least 1e-15, counted on a bit
        // mask of the corner cells' bounding box (wide domains are rare)
        const int wx = hi[0] - lo[0] + 2, wy = hi[1] - lo[1] + 2, wz = DIM == 3 ? hi[2] - lo[2] + 2 : 1;
        if ((long long)wx * wy * wz > 512) {
            atomicOr(err, ERR_CPDI_NODES);
            return false;
        }
        unsigned mask[16] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        for (int c = 0; c < NC; c++) {
            const int e = p.ce[c * n + i];
            int ec, er, ez;
            elem_coords(g, e, ec, er, ez);
            const double xi = p.cxi[(3 * c) * n + i], eta = p.cxi[(3 * c + 1) * n + i];
            const double zeta = DIM == 3 ? p.cxi[(3 * c + 2) * n + i] : 0.;
            for (int k = 0; k < (DIM == 3 ? 8 : 4); k++) {
                const int dx = (k == 1 || k == 2 || k == 5 || k == 6) ? 1 : 0;
                const int dy = (k == 2 || k == 3 || k == 6 || k == 7) ? 1 : 0;
                const int dz = k >= 4 ? 1 : 0;
                const double t1 = 1. + (dx ? 1. : -1.) * xi, t2 = 1. + (dy ? 1. : -1.) * eta;
                const double cfn = DIM == 3 ? 0.125 * t1 * t2 * (1. + (dz ? 1. : -1.) * zeta) : 0.25 * t1 * t2;
                if (cfn < 1e-15) continue;
                const int oz = DIM == 3 ? ez + dz - lo[2] : 0;
                const int bit = (oz * wy + (er + dy - lo[1])) * wx + (ec + dx - lo[0]);
                mask[bit >> 5] |= 1u << (bit & 31);
            }
        }
        int count = 0;
#pragma unroll
        for (int w = 0; w < 16; w++) count += __popc(mask[w]);
        if (count > 49) {
            atomicOr(err, ERR_CPDI_NODES);
            return false;
        }
    }
    return true;
}

// cpdi_setup in the mixed mode: the same corners, elements, natural
// coordinates and gradient weights formed in FP32 from the particle position
// relative to its own cell origin (one FP64 difference per axis), the corner's
// cell found as the particle's cell plus a floored offset; results stored as
// floats.  A corner within float rounding of a cell face may land in the
// neighbouring cell; the linear shape functions of the two cells agree on the
// face, so the weights change by rounding only.
template <int DIM, int SHAPE>
static __device__ bool cpdi_setup_f32(const DevGrid &g, const DevParticles &p, int i, unsigned *err) {
    constexpr int NC = kCpdiPts<DIM, SHAPE>;
    const size_t n = (size_t)p.n;
    float *cxf = reinterpret_cast<float *>(p.cxi), *cwf = reinterpret_cast<float *>(p.cwg);
    int col, row, zr;
    elem_coords(g, p.elem[i], col, row, zr);
    const float dx = (float)g.gx, dy = (float)g.gy, dz = DIM == 3 ? (float)g.gz : 1.f;
    const float idx = (float)g.igx, idy = (float)g.igy, idz = DIM == 3 ? (float)g.igz : 0.f;
    const float rel[3] = {(float)(p.x[i] - g.xn[col]), (float)(p.y[i] - g.yn[row]),
                          DIM == 3 ? (float)(p.z[i] - g.zn[zr]) : 0.f};
    const float pszx = 0.5f * dx * (float)p.lpx[i], pszy = 0.5f * dy * (float)p.lpy[i];
    const float F00 = 1.f + (float)p.exx[i], F11 = 1.f + (float)p.eyy[i];
    const float exy = (float)p.exy[i], wxy = (float)p.wxy[i];
    const float F01 = 0.5f * (exy - wxy), F10 = 0.5f * (exy + wxy);
    float r1[3] = {F00 * pszx, F10 * pszx, 0.f}, r2[3] = {F01 * pszy, F11 * pszy, 0.f}, r3[3] = {0.f, 0.f, 0.f};
    if (DIM == 3) {
        const float pszz = 0.5f * dz * (float)p.lpz[i];
        const float exz = (float)p.exz[i], wxz = (float)p.wxz[i], eyz = (float)p.eyz[i], wyz = (float)p.wyz[i];
        r1[2] = 0.5f * (exz + wxz) * pszx;
        r2[2] = 0.5f * (eyz + wyz) * pszy;
        r3[0] = 0.5f * (exz - wxz) * pszz;
        r3[1] = 0.5f * (eyz - wyz) * pszz;
        r3[2] = (1.f + (float)p.ezz[i]) * pszz;
    }
    const int base[3] = {col, row, zr}, ncell[3] = {g.nx, g.ny, g.nz};
    const float ics[3] = {idx, idy, idz};
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-1, -1, -1};
    float xiv[NC][3];
    int cel[NC][3];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        float s1, s2, s3;
        cpdi_signs<SHAPE>(c, s1, s2, s3);
        int ce[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            float cp = rel[a] + s1 * r1[a] + s2 * r2[a];
            if (DIM == 3) cp += s3 * r3[a];
            const float q = cp * ics[a];
            // qCPDI's material point stays in the particle's own element
            const int o = SHAPE == SHAPE_QCPDI && c == 8 ? 0 : __float2int_rd(q);
            ce[a] = base[a] + o;
            if (ce[a] < 0 || ce[a] >= ncell[a]) {
                atomicOr(err, ERR_LEFT_GRID);
                return false;
            }
            // 2 (cp - (o + 1/2) cell) / cell
            xiv[c][a] = 2.f * (q - (float)o) - 1.f;
            cel[c][a] = ce[a];
            lo[a] = min(lo[a], ce[a]);
            hi[a] = max(hi[a], ce[a]);
            cxf[(3 * c + a) * n + i] = xiv[c][a];
        }
        p.ce[c * n + i] = DIM == 3 ? g.nx * (ce[2] * g.ny + ce[1]) + ce[0] : ce[1] * g.nx + ce[0];
    }
    if (DIM == 2) {
        const float Ap = SHAPE == SHAPE_QCPDI ? 1.f / (3.f * (4.f * (r1[0] * r2[1] - r1[1] * r2[0])))
                                              : 1.f / (4.f * (r1[0] * r2[1] - r1[1] * r2[0]));
        const float wx[4] = {r1[1] - r2[1], r1[1] + r2[1], -r1[1] + r2[1], -r1[1] - r2[1]};
        const float wy[4] = {-r1[0] + r2[0], -r1[0] - r2[0], r1[0] - r2[0], r1[0] + r2[0]};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            cwf[(3 * c + 0) * n + i] = wx[c] * Ap;
            cwf[(3 * c + 1) * n + i] = wy[c] * Ap;
        }
        if constexpr (SHAPE == SHAPE_QCPDI) {
            const float ex[5] = {4.f * r1[1] * Ap, 4.f * r2[1] * Ap, -4.f * r1[1] * Ap, -4.f * r2[1] * Ap, 0.f};
            const float ey[5] = {-4.f * r1[0] * Ap, -4.f * r2[0] * Ap, 4.f * r1[0] * Ap, 4.f * r2[0] * Ap, 0.f};
#pragma unroll
            for (int c = 0; c < 5; c++) {
                cwf[(3 * (4 + c) + 0) * n + i] = ex[c];
                cwf[(3 * (4 + c) + 1) * n + i] = ey[c];
            }
        }
    } else {
        const float a12[3] = {r1[1] * r2[2] - r1[2] * r2[1], r1[2] * r2[0] - r1[0] * r2[2], r1[0] * r2[1] - r1[1] * r2[0]};
        const float a13[3] = {r1[1] * r3[2] - r1[2] * r3[1], r1[2] * r3[0] - r1[0] * r3[2], r1[0] * r3[1] - r1[1] * r3[0]};
        const float a23[3] = {r2[1] * r3[2] - r2[2] * r3[1], r2[2] * r3[0] - r2[0] * r3[2], r2[0] * r3[1] - r2[1] * r3[0]};
        const float Vp = 1.f / (8.f * (r1[0] * a23[0] + r1[1] * a23[1] + r1[2] * a23[2]));
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const float s1 = (c == 1 || c == 2 || c == 5 || c == 6) ? 1.f : -1.f;
            const float s2 = (c == 2 || c == 3 || c == 6 || c == 7) ? 1.f : -1.f;
            const float s3 = c >= 4 ? 1.f : -1.f;
#pragma unroll
            for (int a = 0; a < 3; a++) cwf[(3 * c + a) * n + i] = (s1 * a23[a] - s2 * a13[a] + s3 * a12[a]) * Vp;
        }
    }
    bool small = true;
#pragma unroll
    for (int a = 0; a < DIM; a++) small = small && hi[a] - lo[a] <= 1;
    if (DIM == 3 && !small) {
        // the node count check of cpdi_setup on the float corner data
        const int wx = hi[0] - lo[0] + 2, wy = hi[1] - lo[1] + 2, wz = hi[2] - lo[2] + 2;
        if ((long long)wx * wy * wz > 512) {
            atomicOr(err, ERR_CPDI_NODES);
            return false;
        }
        unsigned mask[16] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        for (int c = 0; c < NC; c++)
            for (int k = 0; k < 8; k++) {
                const int ddx = (k == 1 || k == 2 || k == 5 || k == 6) ? 1 : 0;
                const int ddy = (k == 2 || k == 3 || k == 6 || k == 7) ? 1 : 0;
                const int ddz = k >= 4 ? 1 : 0;
                const float t1 = 1.f + (ddx ? 1.f : -1.f) * xiv[c][0], t2 = 1.f + (ddy ? 1.f : -1.f) * xiv[c][1];
                const float cfn = 0.125f * t1 * t2 * (1.f + (ddz ? 1.f : -1.f) * xiv[c][2]);
                if (cfn < 1e-15f) continue;
                const int bit = ((cel[c][2] + ddz - lo[2]) * wy + (cel[c][1] + ddy - lo[1])) * wx + (cel[c][0] + ddx - lo[0]);
                mask[bit >> 5] |= 1u << (bit & 31);
            }
        int count = 0;
#pragma unroll
        for (int w = 0; w < 16; w++) count += __popc(mask[w]);
        if (count > 49) {
            atomicOr(err, ERR_CPDI_NODES);
            return false;
        }
    }
    return true;
}

// the corner setup of the step in the transfer arithmetic of the mode
template <int DIM, int SHAPE, bool MIX>
__device__ __forceinline__ bool cpdi_setup_for(const DevGrid &g, const DevParticles &p, int i, unsigned *err) {
    if constexpr (MIX) return cpdi_setup_f32<DIM, SHAPE>(g, p, i, err);
    else return cpdi_setup<DIM, SHAPE>(g, p, i, err);
}

// GetCPDIFunctions (MoreMPMElementBase.cpp:581-656) without the node merge:
// f is called for every (corner, element node) pair with weight ws * N and
// gradient wg * N (N the corner element's linear shape function, pairs with
// N < 1e-15 skipped); the sums over pairs equal the merged node values.
template <int DIM, int SHAPE, bool GRAD, typename T, class F>
__device__ __forceinline__ void cpdi_nodes(const DevGrid &g, int nb, const DevParticles &p, int i, F &&f) {
    constexpr int NC = kCpdiPts<DIM, SHAPE>;
    const size_t n = (size_t)p.n;
#pragma unroll 1
    for (int c = 0; c < NC; c++) {
        const T ws = cpdi_ws<DIM, SHAPE, T>(c);
        int col, row, zr;
        elem_coords(g, p.ce[c * n + i], col, row, zr);
        const int n0 = nb + zr * g.zplane + row * g.yplane + col;
        const T xi = cpdi_xi<T>(p, (3 * c) * n + i), eta = cpdi_xi<T>(p, (3 * c + 1) * n + i);
        const T zeta = DIM == 3 ? cpdi_xi<T>(p, (3 * c + 2) * n + i) : T(0);
        T gx = 0, gy = 0, gz = 0;
        if (GRAD) {
            gx = cpdi_wg<T>(p, (3 * c) * n + i);
            gy = cpdi_wg<T>(p, (3 * c + 1) * n + i);
            if (DIM == 3) gz = cpdi_wg<T>(p, (3 * c + 2) * n + i);
        }
#pragma unroll
        for (int k = 0; k < (DIM == 3 ? 8 : 4); k++) {
            const int dx = (k == 1 || k == 2 || k == 5 || k == 6) ? 1 : 0;
            const int dy = (k == 2 || k == 3 || k == 6 || k == 7) ? 1 : 0;
            const int dz = k >= 4 ? 1 : 0;
            const T t1 = T(1) + (dx ? T(1) : T(-1)) * xi, t2 = T(1) + (dy ? T(1) : T(-1)) * eta;
            const T cfn = DIM == 3 ? T(0.125) * t1 * t2 * (T(1) + (dz ? T(1) : T(-1)) * zeta) : T(0.25) * t1 * t2;
            if (cfn < T(1e-15)) continue;
            f(n0 + dx + dy * g.yplane + dz * g.zplane, ws * cfn, gx * cfn, gy * cfn, gz * cfn);
        }
    }
}

// Mixed mode: the same pairs merged per node before anything touches memory.
// When every corner lies in the 2x2(x2) cells from the lowest corner cell lo
// (the usual case: a particle domain no wider than a cell), the weights of the
// 3x3(x3) nodes from lo are sums over corners of separable products
//   N = ws * Wx[a] Wy[b] Wz[c],  grad N = wg * Wx[a] Wy[b] Wz[c]
// with W the corner element's 1D linear weights placed at the corner's cell
// offset, accumulated in registers; f is then called once per node with a
// nonzero weight (at most 27 calls instead of 64 pair calls).  Wider domains
// fall back to the pair visits.  Returns false when it fell back.
template <int DIM, int SHAPE, bool GRAD, class F>
__device__ __forceinline__ void cpdi_window(const DevGrid &g, int nb, const DevParticles &p, int i, F &&f) {
    constexpr int NC = kCpdiPts<DIM, SHAPE>;
    const size_t n = (size_t)p.n;
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-1, -1, -1};
    int cell[NC][3];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        elem_coords(g, p.ce[c * n + i], cell[c][0], cell[c][1], cell[c][2]);
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            lo[a] = min(lo[a], cell[c][a]);
            hi[a] = max(hi[a], cell[c][a]);
        }
    }
    bool fits = true;
#pragma unroll
    for (int a = 0; a < DIM; a++) fits = fits && hi[a] - lo[a] <= 1;
    if (!fits) {
        cpdi_nodes<DIM, SHAPE, GRAD, float>(g, nb, p, i, f);
        return;
    }
    // per corner: natural coordinates, the corner cell's offset in the window
    // (bit a set: one cell up along axis a) and gradient weights
    float xi[NC][3], wg[NC][3];
    unsigned off = 0u;
#pragma unroll
    for (int c = 0; c < NC; c++) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            xi[c][a] = a < DIM ? cpdi_xi<float>(p, (3 * c + a) * n + i) : 0.f;
            wg[c][a] = GRAD && a < DIM ? cpdi_wg<float>(p, (3 * c + a) * n + i) : 0.f;
            if (a < DIM && cell[c][a] != lo[a]) off |= 1u << (3 * c + a);
        }
    }
    // factor 0.5 (1 -+ xi) of window position j (0..2) along axis a for corner c
    auto wt = [&](int c, int a, int j) -> float {
        const bool up = (off >> (3 * c + a)) & 1u;
        const float w0 = 0.5f * (1.f - xi[c][a]), w1 = 0.5f * (1.f + xi[c][a]);
        return j == 0 ? (up ? 0.f : w0) : (j == 1 ? (up ? w0 : w1) : (up ? w1 : 0.f));
    };
    const int base = nb + (DIM == 3 ? lo[2] * g.zplane : 0) + lo[1] * g.yplane + lo[0];
    // one window row (cy, cz) at a time: sums over the corners in corner order,
    // as the merged node list of the reference accumulates them
#pragma unroll 1
    for (int row = 0; row < (DIM == 3 ? 9 : 3); row++) {
        const int cy = row % 3, cz = row / 3;
        float N[3] = {0.f, 0.f, 0.f}, GX[3] = {0.f, 0.f, 0.f}, GY[3] = {0.f, 0.f, 0.f}, GZ[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const float wy = wt(c, 1, cy), wz = DIM == 3 ? wt(c, 2, cz) : 1.f;
#pragma unroll
            for (int cx = 0; cx < 3; cx++) {
                float sfn = wt(c, 0, cx) * wy;
                if (DIM == 3) sfn *= wz;
                if (sfn < 1e-15f) continue;
                N[cx] += cpdi_ws<DIM, SHAPE, float>(c) * sfn;
                if (GRAD) {
                    GX[cx] += wg[c][0] * sfn;
                    GY[cx] += wg[c][1] * sfn;
                    if (DIM == 3) GZ[cx] += wg[c][2] * sfn;
                }
            }
        }
#pragma unroll
        for (int cx = 0; cx < 3; cx++) {
            if (N[cx] == 0.f) continue;
            f(base + cx + cy * g.yplane + cz * g.zplane, N[cx], GX[cx], GY[cx], GZ[cx]);
        }
    }
}

// the nodes of particle i for this step, whatever the shape-function option
template <int DIM, int SHAPE, bool GRAD, typename T, class F>
__device__ __forceinline__ void visit_nodes(const DevGrid &g, int nb, const DevParticles &p, int i, F &&f) {
    if constexpr (kCpdi<SHAPE>) {
        if constexpr (std::is_same<T, float>::value) cpdi_window<DIM, SHAPE, GRAD>(g, nb, p, i, f);
        else cpdi_nodes<DIM, SHAPE, GRAD, T>(g, nb, p, i, f);
    } else {
        for_each_node<DIM, SHAPE, GRAD, T>(g, nb, p.elem[i], p.xi[i], p.eta[i], DIM == 3 ? p.zeta[i] : 0., p.lpx[i],
                                           p.lpy[i], DIM == 3 ? p.lpz[i] : 1., f);
    }
}

// ---------------------------------------------------------------------------
// particle kernels
// ---------------------------------------------------------------------------

// The run a particle belongs to: its grid, node base and time stepping.
struct RunView {
    DevGrid g;
    int nb;
    double dt, st_first, st_last;
    unsigned *err;
    bool mm;           // multimaterial contact (contact terms are extrapolated)
};

template <bool BATCH>
__device__ __forceinline__ bool particle_run(const StepParams &sp, const DevParticles &p, int i, RunView &rv) {
    if (!BATCH) {
        rv.g = sp.g;
        rv.nb = 0;
        rv.dt = sp.dt;
        rv.st_first = sp.st_first;
        rv.st_last = sp.st_last;
        rv.err = sp.err;
        rv.mm = sp.ct.nf > 1;
        return true;
    }
    const int r = p.run[i];
    if (r < 0) return false;
    DevRun &R = sp.runs[r];
    if (!R.active) return false;
    rv.g = R.g;
    rv.nb = R.node_base;
    rv.dt = R.dt;
    rv.st_first = R.st_first;
    rv.st_last = R.st_last;
    rv.err = &R.err;
    rv.mm = R.mm != 0;
    return true;
}

// Weight arithmetic of each transfer mode.
template <bool MIX>
struct Wt {
    using T = double;
};
template <>
struct Wt<true> {
    using T = float;
};

// ---------------------------------------------------------------------------
// Per-axis node windows.  For the shape functions whose nodes form a box
// around the element -- linear (2 per axis), uGIMP and B2SPLINE (3), B2GIMP
// (4) -- the weight of node (jx, jy, jz) of the window is the product of one
// factor per axis, as in for_each_node; AxisWin holds those factors, their
// gradient factors and the window's first node column, row and layer.
// ---------------------------------------------------------------------------
template <int SHAPE>
constexpr int kWinNodes = SHAPE == SHAPE_LINEAR ? 2 : (SHAPE == SHAPE_BGIMP ? 4 : 3);
// node offsets of a window relative to the element's first node: lowest, highest
template <int SHAPE>
constexpr int kWinLo = SHAPE == SHAPE_LINEAR ? 0 : -1;
template <int SHAPE>
constexpr int kWinHi = SHAPE == SHAPE_LINEAR ? 1 : 2;

template <int SHAPE, typename T>
struct AxisWin {
    T S[3][kWinNodes<SHAPE>], dS[3][kWinNodes<SHAPE>];
    int c[3];  // node column, row and layer of the window's first node
    int n0;    // that node's index relative to the run's node base
};

// The factors of for_each_node for element (col, row, zr) and natural
// coordinates xi, eta, zeta (the reference's candidate tests and the 3D
// uGIMP z factor sized by lp.y included).
template <int DIM, int SHAPE, bool GRAD, typename T>
__device__ __forceinline__ void axis_windows(const DevGrid &g, int col, int row, int zr, double xi_d, double eta_d,
                                             double zeta_d, double lpx_d, double lpy_d, double lpz_d,
                                             AxisWin<SHAPE, T> &w) {
    static_assert(!kCpdi<SHAPE>, "CPDI nodes do not form a window");
    const T xi = (T)xi_d, eta = (T)eta_d, zeta = (T)zeta_d;
    const T iD[3] = {GRAD ? recip((T)(g.xn[col + 1] - g.xn[col])) : T(0),
                     GRAD ? recip((T)(g.yn[row + 1] - g.yn[row])) : T(0),
                     GRAD && DIM == 3 ? recip((T)(g.zn[zr + 1] - g.zn[zr])) : T(0)};
    const int cc[3] = {col, row, zr};
    const T nat[3] = {xi, eta, zeta};
    w.c[2] = 0;
    if constexpr (SHAPE == SHAPE_LINEAR) {
        // FourNodeIsoparam / EightNodeIsoparamBrick::ShapeFunction: (1 -/+ xi)/2 per axis
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            w.S[a][0] = T(0.5) * (T(1) - nat[a]);
            w.S[a][1] = T(0.5) * (T(1) + nat[a]);
            w.dS[a][0] = GRAD ? -iD[a] : T(0);
            w.dS[a][1] = GRAD ? iD[a] : T(0);
            w.c[a] = cc[a];
        }
    } else if constexpr (SHAPE == SHAPE_BGIMP) {
        const T lp[3] = {(T)lpx_d, (T)lpy_d, (T)lpz_d};
        const T sgn[3] = {xi, eta, eta};  // the reference's 3D z gradient compares y
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            Win4<T> q;
            bgimp_window<T, DIM == 3, GRAD>(nat[a], lp[a], GRAD ? T(2) * iD[a] : T(0), sgn[a], q);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                w.S[a][j] = q.S[j];
                w.dS[a][j] = q.dS[j];
            }
            w.c[a] = cc[a] - 1;
        }
    } else {
        const T lp[3] = {(T)lpx_d, (T)lpy_d, (T)lpz_d};
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            Win<T> q;
            if constexpr (SHAPE == SHAPE_BSPLINE) {
                bspline_window<T, GRAD>(nat[a], GRAD ? iD[a] : T(0), q);
            } else {
                // uGIMP: the 3D z factor is sized by lp.y (EightNodeIsoparamBrick.cpp:289-403),
                // its gradient by lp.z
                const T inv = recip(T(4) * (a == 2 ? lp[1] : lp[a]));
                const T hinv = !GRAD ? T(0) : (a < 2 || lp[2] == lp[1] ? T(2) * inv : recip(T(2) * lp[2]));
                gimp_window<T, DIM == 3, GRAD>(nat[a], lp[a], inv, hinv, GRAD ? T(2) * iD[a] : T(0), q);
            }
#pragma unroll
            for (int j = 0; j < 3; j++) {
                w.S[a][j] = q.S[j];
                w.dS[a][j] = q.dS[j];
            }
            w.c[a] = cc[a] + q.s - 1;
        }
    }
    w.n0 = w.c[0] + w.c[1] * g.yplane + (DIM == 3 ? w.c[2] * g.zplane : 0);
}

// Columns of the window cache (DevParticles::win): S and dS per axis and node
template <int DIM, int SHAPE>
constexpr int kWinCacheCols = 2 * DIM * kWinNodes<SHAPE>;

template <int DIM, int SHAPE>
__device__ __forceinline__ void win_store(const DevParticles &p, int i, const AxisWin<SHAPE, double> &w) {
    constexpr int K = kWinNodes<SHAPE>;
    const size_t n = (size_t)p.n;
    double *c = p.win + i;
#pragma unroll
    for (int a = 0; a < DIM; a++)
#pragma unroll
        for (int j = 0; j < K; j++) {
            c[(size_t)(a * K + j) * n] = w.S[a][j];
            c[(size_t)((DIM + a) * K + j) * n] = w.dS[a][j];
        }
    p.win_n0[i] = w.n0;
}

// The window of particle i for this step.  FP64 with a window cache: the
// factors k_p2g stored (dS only when GRAD; the node column, row and layer
// are not restored, only n0).  Otherwise formed from the natural coordinates.
// Reading the 144 bytes of a 3D uGIMP window costs far less than the ~100
// FP64 instructions of forming it, on a GPU whose particle kernels are bound
// by the FP64 pipe.
template <int DIM, int SHAPE, bool GRAD, typename T>
__device__ __forceinline__ void particle_window(const DevGrid &g, const DevParticles &p, int i, AxisWin<SHAPE, T> &w) {
    if constexpr (std::is_same<T, double>::value) {
        if (p.win) {
            constexpr int K = kWinNodes<SHAPE>;
            const size_t n = (size_t)p.n;
            const double *c = p.win + i;
#pragma unroll
            for (int a = 0; a < DIM; a++)
#pragma unroll
                for (int j = 0; j < K; j++) {
                    w.S[a][j] = __ldg(c + (size_t)(a * K + j) * n);
                    if (GRAD) w.dS[a][j] = __ldg(c + (size_t)((DIM + a) * K + j) * n);
                }
            w.n0 = __ldg(p.win_n0 + i);
            return;
        }
    }
    int col, row, zr;
    elem_coords(g, p.elem[i], col, row, zr);
    axis_windows<DIM, SHAPE, GRAD, T>(g, col, row, zr, p.xi[i], p.eta[i], DIM == 3 ? p.zeta[i] : 0., p.lpx[i], p.lpy[i],
                                      DIM == 3 ? p.lpz[i] : 1., w);
}

// Calls f(jx, jy, jz, N, dNx, dNy, dNz) for every node of the windows, with the
// products for_each_node forms (2D: jz = 0 and dNz = 0).
template <int DIM, int SHAPE, bool GRAD, typename T, class F>
__device__ __forceinline__ void for_each_window_node(const AxisWin<SHAPE, T> &w, F &&f) {
    constexpr int K = kWinNodes<SHAPE>;
#pragma unroll
    for (int jz = 0; jz < (DIM == 3 ? K : 1); jz++)
#pragma unroll
        for (int jy = 0; jy < K; jy++) {
            const T Syz = DIM == 3 ? w.S[1][jy] * w.S[2][jz] : w.S[1][jy];
            const T dySz = GRAD ? (DIM == 3 ? w.dS[1][jy] * w.S[2][jz] : w.dS[1][jy]) : T(0);
            const T SydZ = GRAD && DIM == 3 ? w.S[1][jy] * w.dS[2][jz] : T(0);
#pragma unroll
            for (int jx = 0; jx < K; jx++) {
                const T Sx = w.S[0][jx];
                f(jx, jy, jz, Sx * Syz, GRAD ? w.dS[0][jx] * Syz : T(0), GRAD ? Sx * dySz : T(0),
                  GRAD ? Sx * SydZ : T(0));
            }
        }
}

// for_each_node's callback f(node, N, 0, 0, 0) over a precomputed window
// (node = global index, run node base nb)
template <int DIM, int SHAPE, typename T, class F>
__device__ __forceinline__ void for_each_window_node_at(const AxisWin<SHAPE, T> &w, const DevGrid &g, int nb, F &&f) {
    const int n0 = nb + w.n0;
    for_each_window_node<DIM, SHAPE, false, T>(w, [&](int jx, int jy, int jz, T N, T, T, T) {
        f(n0 + jx + jy * g.yplane + (DIM == 3 ? jz * g.zplane : 0), N, T(0), T(0), T(0));
    });
}

// Separable gradient sums over a window.  With N = X(jx) Y(jy) Z(jz), the
// velocity gradient sum_nodes v_a dN/dx_b and the internal force
// -mp (sigma - P I) . grad N factor axis by axis: contracting x first, then y,
// then z takes about 270 multiply-adds in 3D instead of the ~380 of forming
// every node's weight and gradient (and the per-node zero tests), which is
// what bounds these kernels on the FP64 pipe.  The sums equal the node-by-node
// ones up to rounding.
//
// out[a*3+b] = sum over window nodes of val_a(node) * dN(node)/dx_b, where
// val(node, v) loads the node's vector (node = global index).
template <int DIM, int SHAPE, typename T, class V>
__device__ __forceinline__ void window_grad_gather(const AxisWin<SHAPE, T> &w, int n0, int yplane, int zplane,
                                                   V &&val, T out[9]) {
    constexpr int K = kWinNodes<SHAPE>;
#pragma unroll
    for (int k = 0; k < 9; k++) out[k] = T(0);
#pragma unroll
    for (int jz = 0; jz < (DIM == 3 ? K : 1); jz++) {
        T C[3] = {0, 0, 0}, D[3] = {0, 0, 0}, E[3] = {0, 0, 0};  // sum_y Y A, sum_y Y' A, sum_y Y B
#pragma unroll
        for (int jy = 0; jy < K; jy++) {
            T A[3] = {0, 0, 0}, B[3] = {0, 0, 0};  // sum_x X v, sum_x X' v
#pragma unroll
            for (int jx = 0; jx < K; jx++) {
                T v[3];
                val(n0 + jx + jy * yplane + jz * zplane, v);
#pragma unroll
                for (int a = 0; a < DIM; a++) {
                    A[a] += w.S[0][jx] * v[a];
                    B[a] += w.dS[0][jx] * v[a];
                }
            }
#pragma unroll
            for (int a = 0; a < DIM; a++) {
                C[a] += w.S[1][jy] * A[a];
                D[a] += w.dS[1][jy] * A[a];
                E[a] += w.S[1][jy] * B[a];
            }
        }
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            if (DIM == 3) {
                out[a * 3 + 0] += w.S[2][jz] * E[a];
                out[a * 3 + 1] += w.S[2][jz] * D[a];
                out[a * 3 + 2] += w.dS[2][jz] * C[a];
            } else {
                out[a * 3 + 0] = E[a];
                out[a * 3 + 1] = D[a];
            }
        }
    }
}

// add(jx, jy, jz, f) for every window node with a non-zero weight, f_a =
// sum_b s[a][b] dN/dx_b for the symmetric tensor s (the prescaled stress).
template <int DIM, int SHAPE, typename T, class F>
__device__ __forceinline__ void window_grad_scatter(const AxisWin<SHAPE, T> &w, const T s[3][3], F &&add) {
    constexpr int K = kWinNodes<SHAPE>;
#pragma unroll
    for (int jz = 0; jz < (DIM == 3 ? K : 1); jz++)
#pragma unroll
        for (int jy = 0; jy < K; jy++) {
            const T P = DIM == 3 ? w.S[1][jy] * w.S[2][jz] : w.S[1][jy];   // Y Z
            const T Q = DIM == 3 ? w.dS[1][jy] * w.S[2][jz] : w.dS[1][jy]; // Y' Z
            const T R = DIM == 3 ? w.S[1][jy] * w.dS[2][jz] : T(0);        // Y Z'
            if (zero_weight(P)) continue;  // the row is outside the support
            T wx[3], u[3];
#pragma unroll
            for (int a = 0; a < DIM; a++) {
                wx[a] = s[a][0] * P;
                u[a] = DIM == 3 ? s[a][1] * Q + s[a][2] * R : s[a][1] * Q;
            }
#pragma unroll
            for (int jx = 0; jx < K; jx++) {
                if (zero_weight(w.S[0][jx])) continue;
                T f[3] = {0, 0, 0};
#pragma unroll
                for (int a = 0; a < DIM; a++) f[a] = w.dS[0][jx] * wx[a] + w.S[0][jx] * u[a];
                add(jx, jy, jz, f);
            }
        }
}

// ---------------------------------------------------------------------------
// Shared-memory node tiles (mixed-precision scatters).  A block's particles
// are consecutive slots, which the cell sort keeps in cell order, so their
// windows cover a small box of grid nodes.  The block accumulates its
// contributions there in shared memory -- each quantity as an FP32 two-sum
// pair (hi, lo): every add returns the old hi, and the rounding error of that
// exact addition goes into lo, so a node's tile sum carries ~2^-48 of its
// terms' magnitude -- and then adds each touched node's sum once to the FP64
// node columns.  Momentum is accumulated relative to a reference velocity of
// the block (that of its first particle), so the bulk motion is added back in
// FP64 at the flush and the FP32 sums only carry velocity differences.
// Particles of another run (batches) or blocks whose box exceeds the tile
// scatter straight to the node columns.
// ---------------------------------------------------------------------------
constexpr int kTileCap = 1280;  // nodes of one block's tile (42 KB of shared memory)
constexpr int kTileQ = 4;       // quantities per node

struct TileBox {
    int run, first;        // the tile's run; lowest thread index of its particles
    int lo[3], hi[3];      // element column, row and layer range of those particles
    int x0, y0, z0;        // node column, row and layer of the box's first node
    int bx, by, bz;        // box extent in nodes
    int nb, yplane, zplane;  // the run's node base and strides
    int on;                // the box fits the tile
};

struct NodeTile {
    TileBox box;
    double ref[3];                 // reference velocity
    float hi[kTileQ][kTileCap];
    float lo[kTileQ][kTileCap];
    unsigned char touched[kTileCap];
};

// Every thread of the block calls this (it synchronises).  valid: the thread
// has a particle; run, col, row, zr: its run and element coordinates; ref:
// its velocity (the first tiled particle's becomes the tile's reference).
// Returns whether the thread's particle accumulates into the tile, which is
// cleared for nq quantities.
template <int DIM, int SHAPE>
__device__ __forceinline__ bool tile_open(NodeTile &t, bool valid, int run, int col, int row, int zr,
                                          const RunView &rv, const double ref[3], int nq) {
    TileBox &b = t.box;
    if (threadIdx.x == 0) {
        b.run = b.first = INT_MAX;
        b.lo[0] = b.lo[1] = b.lo[2] = INT_MAX;
        b.hi[0] = b.hi[1] = b.hi[2] = INT_MIN;
        b.on = 0;
    }
    __syncthreads();
    if (valid) atomicMin(&b.run, run);
    __syncthreads();
    const bool mine = valid && run == b.run;
    if (mine) {
        atomicMin(&b.first, (int)threadIdx.x);
        atomicMin(&b.lo[0], col);
        atomicMax(&b.hi[0], col);
        atomicMin(&b.lo[1], row);
        atomicMax(&b.hi[1], row);
        if (DIM == 3) {
            atomicMin(&b.lo[2], zr);
            atomicMax(&b.hi[2], zr);
        }
    }
    __syncthreads();
    if (mine && (int)threadIdx.x == b.first) {
        constexpr int lo = kWinLo<SHAPE>, span = kWinHi<SHAPE> - kWinLo<SHAPE> + 1;
        b.x0 = b.lo[0] + lo;
        b.bx = b.hi[0] - b.lo[0] + span;
        b.y0 = b.lo[1] + lo;
        b.by = b.hi[1] - b.lo[1] + span;
        if (DIM == 3) {
            b.z0 = b.lo[2] + lo;
            b.bz = b.hi[2] - b.lo[2] + span;
        } else {
            b.z0 = 0;
            b.bz = 1;
        }
        b.nb = rv.nb;
        b.yplane = rv.g.yplane;
        b.zplane = rv.g.zplane;
        b.on = (long long)b.bx * b.by * b.bz <= kTileCap ? 1 : 0;
        t.ref[0] = ref[0];
        t.ref[1] = ref[1];
        t.ref[2] = ref[2];
    }
    __syncthreads();
    if (b.on) {
        const int total = b.bx * b.by * b.bz;
        for (int k = threadIdx.x; k < total; k += blockDim.x) {
            for (int q = 0; q < nq; q++) t.hi[q][k] = t.lo[q][k] = 0.f;
            t.touched[k] = 0;
        }
    }
    __syncthreads();
    return mine && b.on;
}

// tile slot of window node (jx, jy, jz) of a window starting at c
__device__ __forceinline__ int tile_slot(const TileBox &b, const int c[3], int jx, int jy, int jz) {
    return (c[0] + jx - b.x0) + b.bx * ((c[1] + jy - b.y0) + b.by * (c[2] + jz - b.z0));
}

// two-sum accumulation of v into quantity q of slot k
__device__ __forceinline__ void tile_add(NodeTile &t, int q, int k, float v) {
    const float old = atomicAdd(&t.hi[q][k], v);
    const float s = old + v;
    const float bp = s - old;
    atomicAdd(&t.lo[q][k], (old - (s - bp)) + (v - bp));
}

__device__ __forceinline__ double tile_sum(const NodeTile &t, int q, int k) {
    return (double)t.hi[q][k] + (double)t.lo[q][k];
}

// Particle slot of this thread in a scattering kernel: lane l of warp w of
// the block takes slot l * (warps per block) + w of the block's range.  The
// block still covers consecutive slots, but the lanes of one warp hold
// particles of different cells (sorted particles of one cell are neighbours),
// so the lanes' atomic adds -- to a shared-memory tile or to the node columns
// -- go to different nodes instead of queueing on the same address.  Columns
// in host memory (p.host_resident) take the plain order instead: there a
// warp's loads must be whole lines, or the link moves a line per lane.
__device__ __forceinline__ int tile_particle(const DevParticles &p) {
    if (p.host_resident) return blockIdx.x * blockDim.x + threadIdx.x;
    return blockIdx.x * blockDim.x + (threadIdx.x & 31) * (blockDim.x >> 5) + (threadIdx.x >> 5);
}

// Calls f(node, slot) for every touched slot of the tile (after a
// __syncthreads that ends the accumulation); node is the global node index.
template <class F>
__device__ __forceinline__ void tile_flush(const NodeTile &t, F &&f) {
    const TileBox &b = t.box;
    if (!b.on) return;
    const int total = b.bx * b.by * b.bz;
    for (int k = threadIdx.x; k < total; k += blockDim.x) {
        if (!t.touched[k]) continue;
        const int kx = k % b.bx, r = k / b.bx, ky = r % b.by, kz = r / b.by;
        f(b.nb + (b.x0 + kx) + b.yplane * (b.y0 + ky) + b.zplane * (b.z0 + kz), k);
    }
}

// node-index offset of the particle's material velocity field
__device__ __forceinline__ int field_offset(const StepParams &sp, const DevMat *mats, const DevParticles &p, int i) {
    return sp.ct.nf > 1 ? mats[p.mat[i]].field * sp.ct.fstride : 0;
}

// particle i is of a rigid contact material (MaterialBase::IsRigid); only
// asked when some field of the step is rigid
__device__ __forceinline__ bool particle_rigid(const StepParams &sp, const DevMat *mats, const DevParticles &p,
                                               int i) {
    return sp.ct.rigid != 0u && mats[p.mat[i]].type == kMatRigid;
}

// particle volume for contact (MatPoint2D/3D::GetVolume with DEFORMED_AREA,
// MatPoint2D.cpp:407-417, MatPoint3D.cpp:395-408): det F * mp / rho, the 2D
// form without F_zz
template <int DIM>
__device__ __forceinline__ double contact_volume(const DevParticles &p, int i, double rho) {
    const double F00 = 1. + p.exx[i], F01 = 0.5 * (p.exy[i] - p.wxy[i]), F10 = 0.5 * (p.exy[i] + p.wxy[i]);
    const double F11 = 1. + p.eyy[i];
    if (DIM == 2) return (F00 * F11 - F10 * F01) * p.mass[i] / rho;
    const double F22 = 1. + p.ezz[i];
    const double F02 = 0.5 * (p.exz[i] - p.wxz[i]), F20 = 0.5 * (p.exz[i] + p.wxz[i]);
    const double F12 = 0.5 * (p.eyz[i] - p.wyz[i]), F21 = 0.5 * (p.eyz[i] + p.wyz[i]);
    const double J = F00 * (F11 * F22 - F21 * F12) - F01 * (F10 * F22 - F20 * F12) + F02 * (F10 * F21 - F20 * F11);
    return J * p.mass[i] / rho;
}

// Contact volume and volume-gradient node terms (vol, gvx, gvy, gvz): FP64
// columns in the FP64 path; in the mixed mode FP32 values, k-th float of the
// same columns -- they only set the contact normal and which material is
// larger.  The mass-weighted displacement, which decides separation, stays FP64.
template <bool MIX>
__device__ __forceinline__ double cterm(const double *col, int k) {
    if constexpr (MIX) return (double)reinterpret_cast<const float *>(col)[k];
    else return col[k];
}
template <bool MIX>
__device__ __forceinline__ void cterm_set(double *col, int k, double v) {
    if constexpr (MIX) reinterpret_cast<float *>(col)[k] = (float)v;
    else col[k] = v;
}

// multimaterial contact terms of one particle at node k: volume, mass-weighted
// displacement and volume gradient (CrackVelocityField::AddVolumeDisplacement,
// CrackVelocityFieldMulti::AddVolumeGradient); T the weight arithmetic
template <int DIM, bool MIX, typename T>
__device__ __forceinline__ void add_contact_terms(const DevNodes &nd, int k, T N, double fnmp, double Vp,
                                                  const double d[3], T gx, T gy, T gz) {
    if constexpr (MIX) {
        const float V = (float)Vp;
        atomicAdd(reinterpret_cast<float *>(nd.vol) + k, (float)N * V);
        atomicAdd(reinterpret_cast<float *>(nd.gvx) + k, (float)gx * V);
        atomicAdd(reinterpret_cast<float *>(nd.gvy) + k, (float)gy * V);
        if (DIM == 3) atomicAdd(reinterpret_cast<float *>(nd.gvz) + k, (float)gz * V);
    } else {
        atomicAdd(&nd.vol[k], (double)N * Vp);
        atomicAdd(&nd.gvx[k], (double)gx * Vp);
        atomicAdd(&nd.gvy[k], (double)gy * Vp);
        if (DIM == 3) atomicAdd(&nd.gvz[k], (double)gz * Vp);
    }
    atomicAdd(&nd.dsx[k], d[0] * fnmp);
    atomicAdd(&nd.dsy[k], d[1] * fnmp);
    if (DIM == 3) atomicAdd(&nd.dsz[k], d[2] * fnmp);
}

// the same terms as deterministic node sums (scales: volume, displacement, gradient)
template <int DIM>
__device__ __forceinline__ void det_contact_terms(const DevDet &dd, int k, double N, double fnmp, double Vp,
                                                  const double d[3], double gx, double gy, double gz,
                                                  const double sc[3], unsigned *err) {
    det_add(dd, DQ_VOL, k, N * Vp, sc[0], err);
    det_add(dd, DQ_DSX, k, d[0] * fnmp, sc[1], err);
    det_add(dd, DQ_DSY, k, d[1] * fnmp, sc[1], err);
    det_add(dd, DQ_GVX, k, gx * Vp, sc[2], err);
    det_add(dd, DQ_GVY, k, gy * Vp, sc[2], err);
    if (DIM == 3) {
        det_add(dd, DQ_DSZ, k, d[2] * fnmp, sc[1], err);
        det_add(dd, DQ_GVZ, k, gz * Vp, sc[2], err);
    }
}

// A bound on every shape-function gradient component of particle i, twice
// the analytic one: 1 / cell size for linear and uGIMP weights (a GIMP weight
// changes by at most the particle width over the cell size across the particle
// width); for lCPDI the sum over corners of the largest gradient weight, as
// each node gradient is sum_c wg_c N_c(node) with 0 <= N_c <= 1.
template <int DIM, int SHAPE, bool MIX>
__device__ __forceinline__ double grad_bound(const DevGrid &g, const DevParticles &p, int i) {
    if constexpr (kCpdi<SHAPE>) {
        using T = typename Wt<MIX>::T;
        constexpr int NC = kCpdiPts<DIM, SHAPE>;
        const size_t n = (size_t)p.n;
        double s = 0.;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            double w = fmax(fabs((double)cpdi_wg<T>(p, (3 * c) * n + i)), fabs((double)cpdi_wg<T>(p, (3 * c + 1) * n + i)));
            if (DIM == 3) w = fmax(w, fabs((double)cpdi_wg<T>(p, (3 * c + 2) * n + i)));
            s += w;
        }
        return 2. * s;
    } else {
        double m = fmax(g.igx, g.igy);
        if (DIM == 3) m = fmax(m, g.igz);
        return 2. * m;
    }
}

// largest |x - x0| component of particle i at position xp
template <int DIM>
__device__ __forceinline__ double displacement_bound(const DevParticles &p, int i, const double xp[3]) {
    double m = fmax(fabs(xp[0] - p.x0[i]), fabs(xp[1] - p.y0[i]));
    if (DIM == 3) m = fmax(m, fabs(xp[2] - p.z0[i]));
    return m;
}

// Bounds of the first extrapolation's contributions, before k_p2g in the
// deterministic mode: each node's largest N mp (the visit and arithmetic of
// k_p2g, so every node k_p2g adds to has one), and the step-wide ratio bounds.
// The lCPDI corners of the step are set here (k_p2g then uses them).
template <int DIM, int SHAPE, bool MIX>
static __global__ void __launch_bounds__(256) k_det_bounds(StepParams sp, DevParticles p, const DevMat *mats) {
    using T = typename Wt<MIX>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const DevGrid &g = sp.g;
    bool ok = true;
    if constexpr (kCpdi<SHAPE>) ok = cpdi_setup_for<DIM, SHAPE, MIX>(g, p, i, sp.err);
    const double mp = p.mass[i];
    const int off = sp.ct.nf > 1 ? sp.ct.fstride * mats[p.mat[i]].field : 0;
    const bool mm = sp.ct.nf > 1;
    unsigned long long *nb = sp.det.nbnd;
    auto node = [&](int n, T N, T, T, T) {
        if (zero_weight(N)) return;
        atomicMax(nb + n + off, (unsigned long long)__double_as_longlong((double)N * mp));
    };
    if (ok) {
        if constexpr (kCpdi<SHAPE>) {
            if (mm) visit_nodes<DIM, SHAPE, true, T>(g, 0, p, i, node);
            else visit_nodes<DIM, SHAPE, false, T>(g, 0, p, i, node);
        } else {
            const int e = p.elem[i];
            double xi, eta, zeta;
            xi_position(g, e, p.x[i], p.y[i], DIM == 3 ? p.z[i] : 0., xi, eta, zeta);
            const double lz = DIM == 3 ? p.lpz[i] : 1.;
            if (mm) for_each_node<DIM, SHAPE, true, T>(g, 0, e, xi, eta, zeta, p.lpx[i], p.lpy[i], lz, node);
            else for_each_node<DIM, SHAPE, false, T>(g, 0, e, xi, eta, zeta, p.lpx[i], p.lpy[i], lz, node);
        }
    }
    double vm = fmax(fabs(p.vx[i]), fabs(p.vy[i]));
    if (DIM == 3) vm = fmax(vm, fabs(p.vz[i]));
    det_bound(sp.det, DB_MOM, vm);
    if (mm) {
        const double Vp = fabs(contact_volume<DIM>(p, i, mats[p.mat[i]].rho));
        const double xp[3] = {p.x[i], p.y[i], DIM == 3 ? p.z[i] : 0.};
        det_bound(sp.det, DB_VOL, Vp / mp);
        det_bound(sp.det, DB_DS, displacement_bound<DIM>(p, i, xp));
        det_bound(sp.det, DB_GV, Vp * grad_bound<DIM, SHAPE, MIX>(g, p, i));
    }
}

// InitializationTask::Execute (natural coordinates, InitializationTask.cpp:59-83)
// and MassAndMomentumTask::Execute with NodalPoint::AddMassMomentum
// (MassAndMomentumTask.cpp:48-127, NodalPointMPM.cpp:419-453).  Momentum and
// mass accumulate in FP64 in both modes: grid velocities carry the bulk motion
// and their differences across a cell are the strain rate.
template <int DIM, int SHAPE, bool MIX, bool BATCH, bool DET = false>
static __global__ void __launch_bounds__(256, kCpdi<SHAPE> ? 2 : 3) k_p2g(StepParams sp, DevParticles p, DevNodes nd, const DevMat *mats) {
    using T = typename Wt<MIX>::T;
    const int i = tile_particle(p);
    if (i >= p.n) return;
    RunView rv;
    if (!particle_run<BATCH>(sp, p, i, rv)) return;
    const DevGrid &g = rv.g;
    const int e = p.elem[i];
    const double x = p.x[i], y = p.y[i], z = DIM == 3 ? p.z[i] : 0.;
    double xi, eta, zeta;
    xi_position(g, e, x, y, z, xi, eta, zeta);
    p.xi[i] = xi;
    p.eta[i] = eta;
    if (DIM == 3) p.zeta[i] = zeta;
    const double mp = p.mass[i];
    const double vx = p.vx[i], vy = p.vy[i], vz = DIM == 3 ? p.vz[i] : 0.;
    const int off = field_offset(sp, mats, p, i);
    const bool mm = rv.mm;
    double Vp = 0., d[3] = {0., 0., 0.};
    if (mm) {
        Vp = contact_volume<DIM>(p, i, mats[p.mat[i]].rho);
        d[0] = p.x[i] - p.x0[i];
        d[1] = p.y[i] - p.y0[i];
        if (DIM == 3) d[2] = p.z[i] - p.z0[i];
    }
    unsigned long long bM = 0, bV = 0, bD = 0;
    double sG = 1.;
    if constexpr (DET) {
        bM = sp.det.bnd[DB_MOM];
        bV = sp.det.bnd[DB_VOL];
        bD = sp.det.bnd[DB_DS];
        sG = pow2(det_shift(sp.det.bnd[DB_GV]));
    }
    auto scatter = [&](int n, T N, T gx, T gy, T gz) {
        if (zero_weight(N)) return;
        n += off;
        const double fnmp = (double)N * mp;
        if constexpr (DET) {
            const unsigned long long nb = sp.det.nbnd[n];
            const double sP = pow2(det_shift2(nb, bM));
            det_add(sp.det, DQ_MASS, n, fnmp, pow2(det_shift(nb)), rv.err);
            det_add(sp.det, DQ_PX, n, vx * fnmp, sP, rv.err);
            det_add(sp.det, DQ_PY, n, vy * fnmp, sP, rv.err);
            if (DIM == 3) det_add(sp.det, DQ_PZ, n, vz * fnmp, sP, rv.err);
            nd.active[n] = 1;
            if (mm) {
                const double sc[3] = {pow2(det_shift2(nb, bV)), pow2(det_shift2(nb, bD)), sG};
                det_contact_terms<DIM>(sp.det, n, (double)N, fnmp, Vp, d, (double)gx, (double)gy, (double)gz, sc,
                                       rv.err);
            }
            return;
        }
        atomicAdd(&nd.mass[n], fnmp);
        atomicAdd(&nd.px[n], vx * fnmp);
        atomicAdd(&nd.py[n], vy * fnmp);
        if (DIM == 3) atomicAdd(&nd.pz[n], vz * fnmp);
        nd.active[n] = 1;
        if (mm) add_contact_terms<DIM, MIX>(nd, n, N, fnmp, Vp, d, gx, gy, gz);
    };
    if constexpr (kCpdi<SHAPE>) {
        // ElementBase::GetShapeFunctionData: the particle's CPDI corners for
        // this step (set by k_det_bounds in the deterministic mode)
        if (!DET && !cpdi_setup_for<DIM, SHAPE, MIX>(g, p, i, rv.err)) return;
        if (mm) visit_nodes<DIM, SHAPE, true, T>(g, rv.nb, p, i, scatter);
        else visit_nodes<DIM, SHAPE, false, T>(g, rv.nb, p, i, scatter);
    } else {
        if constexpr (!MIX) {
            if (p.win) {
                // the step's window with its gradient factors, kept for the
                // later particle kernels of the step (particle_window)
                int col, row, zr;
                elem_coords(g, e, col, row, zr);
                AxisWin<SHAPE, double> w;
                axis_windows<DIM, SHAPE, true, double>(g, col, row, zr, xi, eta, zeta, p.lpx[i], p.lpy[i],
                                                       DIM == 3 ? p.lpz[i] : 1., w);
                win_store<DIM, SHAPE>(p, i, w);
                const int n0 = rv.nb + w.n0;
                auto at = [&](int jx, int jy, int jz, double N, double dx, double dy, double dz) {
                    scatter(n0 + jx + jy * g.yplane + jz * g.zplane, N, dx, dy, dz);
                };
                if (mm) for_each_window_node<DIM, SHAPE, true, double>(w, at);
                else for_each_window_node<DIM, SHAPE, false, double>(w, at);
                return;
            }
        }
        if (mm)
            for_each_node<DIM, SHAPE, true, T>(g, rv.nb, e, xi, eta, zeta, p.lpx[i], p.lpy[i],
                                               DIM == 3 ? p.lpz[i] : 1., scatter);
        else
            for_each_node<DIM, SHAPE, false, T>(g, rv.nb, e, xi, eta, zeta, p.lpx[i], p.lpy[i],
                                                DIM == 3 ? p.lpz[i] : 1., scatter);
    }
}

// k_p2g of the mixed mode through a shared-memory node tile (single material
// field; linear, uGIMP, B2SPLINE and B2GIMP windows): FP32 weights and
// products, accumulated per block as two-sum pairs of mass and of mass times
// the velocity's difference from the block's reference velocity, added once
// per touched node to the FP64 mass and momentum columns.
template <int DIM, int SHAPE, bool BATCH>
static __global__ void __launch_bounds__(256) k_p2g_tile(StepParams sp, DevParticles p, DevNodes nd) {
    __shared__ NodeTile t;
    const int i = tile_particle(p);
    RunView rv;
    const bool valid = i < p.n && particle_run<BATCH>(sp, p, i, rv);
    int col = 0, row = 0, zr = 0;
    double xi = 0., eta = 0., zeta = 0., mp = 0., v[3] = {0., 0., 0.};
    if (valid) {
        const int e = p.elem[i];
        elem_coords(rv.g, e, col, row, zr);
        // natural coordinates in FP32 from the offset to the element's first
        // node (an FP64 difference): the mixed-mode kernels take them as floats
        const DevGrid &g = rv.g;
        xi = (double)(2.f * (float)(p.x[i] - g.xn[col]) * (float)g.igx - 1.f);
        eta = (double)(2.f * (float)(p.y[i] - g.yn[row]) * (float)g.igy - 1.f);
        if (DIM == 3) zeta = (double)(2.f * (float)(p.z[i] - g.zn[zr]) * (float)g.igz - 1.f);
        p.xi[i] = xi;
        p.eta[i] = eta;
        if (DIM == 3) p.zeta[i] = zeta;
        mp = p.mass[i];
        v[0] = p.vx[i];
        v[1] = p.vy[i];
        if (DIM == 3) v[2] = p.vz[i];
    }
    const bool tiled = tile_open<DIM, SHAPE>(t, valid, BATCH && valid ? p.run[i] : 0, col, row, zr, rv, v, DIM + 1);
    if (valid) {
        AxisWin<SHAPE, float> w;
        axis_windows<DIM, SHAPE, false, float>(rv.g, col, row, zr, xi, eta, zeta, p.lpx[i], p.lpy[i],
                                               DIM == 3 ? p.lpz[i] : 1., w);
        if (tiled) {
            const float mpf = (float)mp;
            const float d[3] = {(float)(v[0] - t.ref[0]), (float)(v[1] - t.ref[1]), (float)(v[2] - t.ref[2])};
            for_each_window_node<DIM, SHAPE, false, float>(w, [&](int jx, int jy, int jz, float N, float, float, float) {
                if (N == 0.f) return;
                const int k = tile_slot(t.box, w.c, jx, jy, jz);
                const float wm = N * mpf;
                tile_add(t, 0, k, wm);
#pragma unroll
                for (int a = 0; a < DIM; a++) tile_add(t, 1 + a, k, wm * d[a]);
                t.touched[k] = 1;
            });
        } else {
            // outside the tile: straight to the node columns, as k_p2g
            const DevGrid &g = rv.g;
            for_each_window_node<DIM, SHAPE, false, float>(w, [&](int jx, int jy, int jz, float N, float, float, float) {
                if (N == 0.f) return;
                const int n = rv.nb + (w.c[0] + jx) + g.yplane * (w.c[1] + jy) + g.zplane * (w.c[2] + jz);
                const double fnmp = (double)N * mp;
                atomicAdd(&nd.mass[n], fnmp);
                atomicAdd(&nd.px[n], v[0] * fnmp);
                atomicAdd(&nd.py[n], v[1] * fnmp);
                if (DIM == 3) atomicAdd(&nd.pz[n], v[2] * fnmp);
                nd.active[n] = 1;
            });
        }
    }
    __syncthreads();
    tile_flush(t, [&](int n, int k) {
        const double m = tile_sum(t, 0, k);
        atomicAdd(&nd.mass[n], m);
        atomicAdd(&nd.px[n], t.ref[0] * m + tile_sum(t, 1, k));
        atomicAdd(&nd.py[n], t.ref[1] * m + tile_sum(t, 2, k));
        if (DIM == 3) atomicAdd(&nd.pz[n], t.ref[2] * m + tile_sum(t, 3, k));
        nd.active[n] = 1;
    });
}

template <int DIM>
__device__ __forceinline__ void constitutive(const DevMat *mats, const DevParticles &p, int i, const double du[9]) {
    const DevMat &m = mats[p.mat[i]];
    if (m.type == kMatNeohookean) {
        neo_law<DIM == 3>(m, p, i, du);
        return;
    }
    if (DIM == 2) hypo_increment_F_2d(p, i, du);
    else hypo_increment_F_3d(p, i, du);
    if (m.type == kMatIsotropic) {
        if (DIM == 2) iso_law_2d(m, p, i, du);
        else iso_law_3d(m, p, i, du);
    } else {
        plastic_law<DIM == 3>(m, p, i, du);
    }
}

// gather of ExtrapVelocityGradient (MatPoint2D.cpp:57-87, MatPoint3D.cpp:50-75),
// scaled by the strain time step.  Mixed mode: sum over nodes of
// (v_node - v_particle) * grad N in FP32 -- the same value in exact arithmetic
// because the gradients sum to zero -- where the velocity difference is formed
// exactly from FP32 hi/lo pairs of both velocities, so the bulk motion cancels
// before any rounding.
template <int DIM, int SHAPE, bool MIX>
__device__ __forceinline__ void velocity_gradient(const DevGrid &g, int nb, const DevParticles &p, const DevNodes &nd,
                                                  int i, double st, double du[9], int off) {
    using T = typename Wt<MIX>::T;
    T d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float ph[3] = {0.f, 0.f, 0.f}, pl[3] = {0.f, 0.f, 0.f};
    if (MIX) {
        split2(p.vx[i], ph[0], pl[0]);
        split2(p.vy[i], ph[1], pl[1]);
        if (DIM == 3) split2(p.vz[i], ph[2], pl[2]);
    }
    if constexpr (!kCpdi<SHAPE>) {
        // window shape functions: the separable sum (window_grad_gather)
        AxisWin<SHAPE, T> w;
        particle_window<DIM, SHAPE, true, T>(g, p, i, w);
        const int n0 = nb + off + w.n0;
        window_grad_gather<DIM, SHAPE, T>(w, n0, g.yplane, g.zplane, [&](int n, T v[3]) {
            if (MIX) {
                v[0] = (T)((nd.vhx[n] - ph[0]) + (nd.vlx[n] - pl[0]));
                v[1] = (T)((nd.vhy[n] - ph[1]) + (nd.vly[n] - pl[1]));
                v[2] = DIM == 3 ? (T)((nd.vhz[n] - ph[2]) + (nd.vlz[n] - pl[2])) : T(0);
            } else {
                v[0] = (T)nd.vx[n];
                v[1] = (T)nd.vy[n];
                v[2] = DIM == 3 ? (T)nd.vz[n] : T(0);
            }
        }, d);
#pragma unroll
        for (int k = 0; k < 9; k++) du[k] = (double)d[k] * st;
        return;
    }
    visit_nodes<DIM, SHAPE, true, T>(g, nb, p, i, [&](int n, T N, T dx, T dy, T dz) {
                                           if (zero_weight(N)) return;
                                           n += off;
                                           T vx, vy, vz = 0;
                                           if (MIX) {
                                               vx = (T)((nd.vhx[n] - ph[0]) + (nd.vlx[n] - pl[0]));
                                               vy = (T)((nd.vhy[n] - ph[1]) + (nd.vly[n] - pl[1]));
                                               if (DIM == 3) vz = (T)((nd.vhz[n] - ph[2]) + (nd.vlz[n] - pl[2]));
                                           } else {
                                               vx = (T)nd.vx[n];
                                               vy = (T)nd.vy[n];
                                               if (DIM == 3) vz = (T)nd.vz[n];
                                           }
                                           d[0] += vx * dx;
                                           d[1] += vx * dy;
                                           d[3] += vy * dx;
                                           d[4] += vy * dy;
                                           if (DIM == 3) {
                                               d[2] += vx * dz;
                                               d[5] += vy * dz;
                                               d[6] += vz * dx;
                                               d[7] += vz * dy;
                                               d[8] += vz * dz;
                                           }
                                       });
#pragma unroll
    for (int k = 0; k < 9; k++) du[k] = (double)d[k] * st;
}

// GetFintPlusFext scatter of particle i: -mp (sigma - P I) . grad N to its
// nodes (FP32 products and atomics in the mixed mode; deterministic node sums
// with DET)
template <int DIM, int SHAPE, bool MIX, bool DET>
__device__ __forceinline__ void forces_scatter(const StepParams &sp, const DevParticles &p, const DevNodes &nd,
                                                 int i, const DevGrid &g, int nb, int off) {
    using T = typename Wt<MIX>::T;
    double sF = 1.;
    if constexpr (DET) sF = pow2(det_shift(sp.det.bnd[DB_FORCE]));
    // -mp * (sigma - P I): the internal force of GetFintPlusFext, scaled once
    const double mp = p.mass[i], P = p.pressure[i];
    const T sxx = (T)(-mp * (p.sxx[i] - P)), syy = (T)(-mp * (p.syy[i] - P)), sxy = (T)(-mp * p.sxy[i]);
    const T szz = DIM == 3 ? (T)(-mp * (p.szz[i] - P)) : T(0), sxz = DIM == 3 ? (T)(-mp * p.sxz[i]) : T(0),
            syz = DIM == 3 ? (T)(-mp * p.syz[i]) : T(0);
    if constexpr (!kCpdi<SHAPE>) {
        // window shape functions: the separable products (window_grad_scatter)
        AxisWin<SHAPE, T> w;
        particle_window<DIM, SHAPE, true, T>(g, p, i, w);
        const T sg[3][3] = {{sxx, sxy, sxz}, {sxy, syy, syz}, {sxz, syz, szz}};
        const int n0 = nb + off + w.n0;
        window_grad_scatter<DIM, SHAPE, T>(w, sg, [&](int jx, int jy, int jz, const T f[3]) {
            const int n = n0 + jx + jy * g.yplane + jz * g.zplane;
            if constexpr (DET) {
                det_add(sp.det, DQ_FX, n, (double)f[0], sF, sp.err);
                det_add(sp.det, DQ_FY, n, (double)f[1], sF, sp.err);
                if (DIM == 3) det_add(sp.det, DQ_FZ, n, (double)f[2], sF, sp.err);
            } else if (MIX) {
                atomicAdd(&nd.gx[n], (float)f[0]);
                atomicAdd(&nd.gy[n], (float)f[1]);
                if (DIM == 3) atomicAdd(&nd.gz[n], (float)f[2]);
            } else {
                atomicAdd(&nd.fx[n], (double)f[0]);
                atomicAdd(&nd.fy[n], (double)f[1]);
                if (DIM == 3) atomicAdd(&nd.fz[n], (double)f[2]);
            }
        });
        return;
    }
    visit_nodes<DIM, SHAPE, true, T>(g, nb, p, i, [&](int n, T N, T dx, T dy, T dz) {
                                           if (zero_weight(N)) return;
                                           n += off;
                                           T fx, fy, fz = 0;
                                           if (DIM == 2) {
                                               fx = sxx * dx + sxy * dy;
                                               fy = sxy * dx + syy * dy;
                                           } else {
                                               fx = sxx * dx + sxy * dy + sxz * dz;
                                               fy = sxy * dx + syy * dy + syz * dz;
                                               fz = sxz * dx + syz * dy + szz * dz;
                                           }
                                           if constexpr (DET) {
                                               det_add(sp.det, DQ_FX, n, (double)fx, sF, sp.err);
                                               det_add(sp.det, DQ_FY, n, (double)fy, sF, sp.err);
                                               if (DIM == 3) det_add(sp.det, DQ_FZ, n, (double)fz, sF, sp.err);
                                           } else if (MIX) {
                                               atomicAdd(&nd.gx[n], (float)fx);
                                               atomicAdd(&nd.gy[n], (float)fy);
                                               if (DIM == 3) atomicAdd(&nd.gz[n], (float)fz);
                                           } else {
                                               atomicAdd(&nd.fx[n], (double)fx);
                                               atomicAdd(&nd.fy[n], (double)fy);
                                               if (DIM == 3) atomicAdd(&nd.fz[n], (double)fz);
                                           }
                                       });
}


// UpdateStrainsFirstTask::FullStrainUpdate (UpdateStrainsFirstTask.cpp:101-168)
// fused with GridForcesTask::Execute and MatPoint2D/3D::GetFintPlusFext
// (GridForcesTask.cpp:40-153, MatPoint2D.cpp:242-262, MatPoint3D.cpp:248-269).
// Mixed mode: internal-force products in FP32 into FP32 accumulators.
template <int DIM, int SHAPE, bool STRAIN, bool MIX, bool BATCH, bool DET = false>
static __global__ void __launch_bounds__(256, kStrainBlocks<SHAPE>) k_strain_forces(StepParams sp, DevParticles p, DevNodes nd, const DevMat *mats) {
    const int i = tile_particle(p);
    if (i >= p.n) return;
    RunView rv;
    if (!particle_run<BATCH>(sp, p, i, rv)) return;
    // rigid particles have no strain update and no internal force
    // (UpdateStrainsFirstTask.cpp:123, GridForcesTask.cpp:53)
    if (particle_rigid(sp, mats, p, i)) return;
    const DevGrid &g = rv.g;
    const int off = field_offset(sp, mats, p, i);
    if (STRAIN) {
        double du[9];
        velocity_gradient<DIM, SHAPE, MIX>(g, rv.nb, p, nd, i, rv.st_first, du, off);
        constitutive<DIM>(mats, p, i, du);
    }
    if constexpr (DET) {
        // the forces are summed by k_det_forces once the bound of all of them is known
        const double mp = p.mass[i], P = p.pressure[i];
        const double a = fabs(p.sxx[i] - P), b = fabs(p.syy[i] - P), c = fabs(p.sxy[i]);
        double r = fmax(a + c, c + b);
        if (DIM == 3) {
            const double zz = fabs(p.szz[i] - P), xz = fabs(p.sxz[i]), yz = fabs(p.syz[i]);
            r = fmax(fmax(a + c + xz, c + b + yz), xz + yz + zz);
        }
        det_bound(sp.det, DB_FORCE, mp * r * grad_bound<DIM, SHAPE, MIX>(g, p, i));
        return;
    }
    forces_scatter<DIM, SHAPE, MIX, false>(sp, p, nd, i, g, rv.nb, off);
}

// k_strain_forces of the mixed mode through a shared-memory node tile (single
// material field, window shape functions): the strain and constitutive
// update, then the FP32 internal-force products accumulated per block as
// two-sum pairs and added once per touched node to the FP64 force columns
// (particles outside the tile add to the FP32 columns, which the momentum
// update adds to the FP64 ones).
template <int DIM, int SHAPE, bool STRAIN, bool BATCH>
static __global__ void __launch_bounds__(256, kStrainBlocks<SHAPE>) k_strain_forces_tile(StepParams sp, DevParticles p, DevNodes nd, const DevMat *mats) {
    __shared__ NodeTile t;
    const int i = tile_particle(p);
    RunView rv;
    const bool valid = i < p.n && particle_run<BATCH>(sp, p, i, rv);
    int col = 0, row = 0, zr = 0;
    if (valid) {
        if (STRAIN) {
            double du[9];
            velocity_gradient<DIM, SHAPE, true>(rv.g, rv.nb, p, nd, i, rv.st_first, du, 0);
            constitutive<DIM>(mats, p, i, du);
        }
        elem_coords(rv.g, p.elem[i], col, row, zr);
    }
    const double zero[3] = {0., 0., 0.};
    const bool tiled = tile_open<DIM, SHAPE>(t, valid, BATCH && valid ? p.run[i] : 0, col, row, zr, rv, zero, DIM);
    if (valid) {
        // -mp * (sigma - P I): the internal force of GetFintPlusFext, scaled once
        const double mp = p.mass[i], P = p.pressure[i];
        const float sxx = (float)(-mp * (p.sxx[i] - P)), syy = (float)(-mp * (p.syy[i] - P)),
                    sxy = (float)(-mp * p.sxy[i]);
        const float szz = DIM == 3 ? (float)(-mp * (p.szz[i] - P)) : 0.f, sxz = DIM == 3 ? (float)(-mp * p.sxz[i]) : 0.f,
                    syz = DIM == 3 ? (float)(-mp * p.syz[i]) : 0.f;
        AxisWin<SHAPE, float> w;
        axis_windows<DIM, SHAPE, true, float>(rv.g, col, row, zr, p.xi[i], p.eta[i], DIM == 3 ? p.zeta[i] : 0.,
                                              p.lpx[i], p.lpy[i], DIM == 3 ? p.lpz[i] : 1., w);
        const DevGrid &g = rv.g;
        const float sg[3][3] = {{sxx, sxy, sxz}, {sxy, syy, syz}, {sxz, syz, szz}};
        window_grad_scatter<DIM, SHAPE, float>(w, sg, [&](int jx, int jy, int jz, const float f[3]) {
            if (tiled) {
                const int k = tile_slot(t.box, w.c, jx, jy, jz);
#pragma unroll
                for (int a = 0; a < DIM; a++) tile_add(t, a, k, f[a]);
                t.touched[k] = 1;
            } else {
                const int n = rv.nb + (w.c[0] + jx) + g.yplane * (w.c[1] + jy) + g.zplane * (w.c[2] + jz);
                atomicAdd(&nd.gx[n], f[0]);
                atomicAdd(&nd.gy[n], f[1]);
                if (DIM == 3) atomicAdd(&nd.gz[n], f[2]);
            }
        });
    }
    __syncthreads();
    tile_flush(t, [&](int n, int k) {
        atomicAdd(&nd.fx[n], tile_sum(t, 0, k));
        atomicAdd(&nd.fy[n], tile_sum(t, 1, k));
        if (DIM == 3) atomicAdd(&nd.fz[n], tile_sum(t, 2, k));
    });
}

// Deterministic mode: the internal-force scatter of k_strain_forces as its own
// pass, once k_strain_forces has bounded every particle's forces.
template <int DIM, int SHAPE, bool MIX>
static __global__ void __launch_bounds__(256) k_det_forces(StepParams sp, DevParticles p, DevNodes nd, const DevMat *mats) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n || particle_rigid(sp, mats, p, i)) return;
    forces_scatter<DIM, SHAPE, MIX, true>(sp, p, nd, i, sp.g, 0, field_offset(sp, mats, p, i));
}

// ResetElementsTask::ResetElement with MeshInfo::FindElementFromPoint and
// MeshInfo::EdgeElement2D/3D (ResetElementsTask.cpp:196-228,
// MeshInfo.cpp:171-199, 593-633).
template <int DIM>
__device__ __forceinline__ void reset_element(const DevGrid &g, const DevParticles &p, int i, unsigned *err) {
    const double x = p.x[i], y = p.y[i], z = DIM == 3 ? p.z[i] : 0.;
    // the NaN and in-cell tests on integer order keys (the same outcomes as
    // the double compares, in the integer pipe)
    if (is_nan_bits(x) || is_nan_bits(y) || is_nan_bits(z)) {
        atomicOr(err, ERR_NAN);
        return;
    }
    const int e = p.elem[i];
    int col, row, zr;
    elem_coords(g, e, col, row, zr);
    const long long kx = order_key(x), ky = order_key(y);
    bool in = kx >= order_key(g.xn[col]) && kx < order_key(g.xn[col + 1]) && ky >= order_key(g.yn[row]) &&
              ky < order_key(g.yn[row + 1]);
    if (DIM == 3) {
        const long long kz = order_key(z);
        in = in && kz >= order_key(g.zn[zr]) && kz < order_key(g.zn[zr + 1]);
    }
    if (in) return;
    int c = (int)((x - g.xmin) / g.gx);
    bool bad = false;
    if (c < 0 || c >= g.nx) {
        if (x == g.xmin + g.nx * g.gx) c = g.nx - 1;
        else bad = true;
    }
    int r = (int)((y - g.ymin) / g.gy);
    if (r < 0 || r >= g.ny) {
        if (y == g.ymin + g.ny * g.gy) r = g.ny - 1;
        else bad = true;
    }
    int zz = 0;
    if (DIM == 3) {
        zz = (int)((z - g.zmin) / g.gz);
        if (zz < 0 || zz >= g.nz) {
            if (z == g.zmin + g.nz * g.gz) zz = g.nz - 1;
            else bad = true;
        }
    }
    if (bad) {
        atomicOr(err, ERR_LEFT_GRID);
        return;
    }
    const int num = DIM == 3 ? g.nx * (zz * g.ny + r) + c + 1 : r * g.nx + c + 1;
    bool edge;
    if (DIM == 2) {
        const int total = g.nx * g.ny;
        edge = num <= g.nx || num > total - g.nx || (num % g.nx) <= 1;
    } else {
        const int hv = g.nx * g.ny, total = hv * g.nz;
        const int xz = num % hv;
        edge = num <= hv || num > total - hv || (num % g.nx) <= 1 || xz <= g.nx || xz > g.nx * (g.ny - 1);
    }
    if (edge) {
        atomicOr(err, ERR_EDGE);
        return;
    }
    p.elem[i] = num - 1;
}

// The particle update of particle i: UpdateParticlesTask::Execute,
// MatVelocityField::IncrementNodalVelAcc and MatPoint2D/3D::MoveParticle
// without damping (UpdateParticlesTask.cpp:75-178, MatVelocityField.cpp:410-426,
// MatPoint2D.cpp:99-196) -- FLIP, or the XPIC/FMPM form of the step.  Gathers
// S v and S a from the nodes, moves the particle and writes its velocity and
// position; returns them in v and xp.  Mixed mode: S v is formed as
// v_particle + sum N (v_node - v_particle) (the weights sum to one) with the
// differences from FP32 pairs, S a in FP32; the update itself is FP64.
// win: the particle's window factors when the caller has them (window shapes),
// so they are not formed again here.
template <int DIM, int SHAPE, bool MIX, bool BATCH>
__device__ __forceinline__ void g2p_move(const StepParams &sp, const DevParticles &p, const DevNodes &nd, int i,
                                         const RunView &rv, int off, double v[3], double xp[3],
                                         const AxisWin<SHAPE, typename Wt<MIX>::T> *win = nullptr) {
    using T = typename Wt<MIX>::T;
    const DevGrid &g = rv.g;
    const double dt = rv.dt;
    T Sv[3] = {0, 0, 0}, Sa[3] = {0, 0, 0};
    const int e = p.elem[i];
    const double xi = p.xi[i], eta = p.eta[i], zeta = DIM == 3 ? p.zeta[i] : 0.;
    const double lx = p.lpx[i], ly = p.lpy[i], lz = DIM == 3 ? p.lpz[i] : 1.;
    v[0] = p.vx[i];
    v[1] = p.vy[i];
    v[2] = DIM == 3 ? p.vz[i] : 0.;
    float ph[3] = {0.f, 0.f, 0.f}, pl[3] = {0.f, 0.f, 0.f};
    if (MIX) {
#pragma unroll
        for (int a = 0; a < DIM; a++) split2(v[a], ph[a], pl[a]);
    }
    // the particle's nodes for this step (CPDI corners or the element window)
    auto visit = [&](auto &&fn) {
        if constexpr (kCpdi<SHAPE>) {
            visit_nodes<DIM, SHAPE, false, T>(g, rv.nb, p, i, fn);
        } else {
            if (win) for_each_window_node_at<DIM, SHAPE, T>(*win, g, rv.nb, fn);
            else for_each_node<DIM, SHAPE, false, T>(g, rv.nb, e, xi, eta, zeta, lx, ly, lz, fn);
        }
    };
    visit([&](int n, T N, T, T, T) {
        if (zero_weight(N)) return;
        n += off;
        if (MIX) {
            Sv[0] += ((nd.vhx[n] - ph[0]) + (nd.vlx[n] - pl[0])) * N;
            Sv[1] += ((nd.vhy[n] - ph[1]) + (nd.vly[n] - pl[1])) * N;
            if (DIM == 3) Sv[2] += ((nd.vhz[n] - ph[2]) + (nd.vlz[n] - pl[2])) * N;
            Sa[0] += nd.bx[n] * N;
            Sa[1] += nd.by[n] * N;
            if (DIM == 3) Sa[2] += nd.bz[n] * N;
        } else {
            Sv[0] += nd.vx[n] * N;
            Sv[1] += nd.vy[n] * N;
            if (DIM == 3) Sv[2] += nd.vz[n] * N;
            Sa[0] += nd.ax[n] * N;  // f/m of the node (the reference forms f*(N/m))
            Sa[1] += nd.ay[n] * N;
            if (DIM == 3) Sa[2] += nd.az[n] * N;
        }
    });
    xp[0] = p.x[i];
    xp[1] = p.y[i];
    xp[2] = DIM == 3 ? p.z[i] : 0.;
    const int xmode = BATCH ? sp.runs[p.run[i]].xpic : sp.xpic;
    if (xmode == 0) {
        // FLIP (MatPoint2D/3D::MoveParticle, m == 0)
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            const double sv = MIX ? v[a] + (double)Sv[a] : (double)Sv[a];
            const double sa = (double)Sa[a];
            const double vm = sv - sa * dt;
            const double dv = sa * dt;
            v[a] += dv;
            xp[a] += (vm + 0.5 * dv) * dt;
        }
    } else {
        // FMPM (m > 0) and XPIC (m < 0) take the particle velocity S v(k)
        // (MatPoint2D.cpp:120-182, MatPoint3D.cpp:124-181); no damping
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            const double sv = MIX ? v[a] + (double)Sv[a] : (double)Sv[a];
            const double vold = v[a];
            v[a] = sv;
            if (xmode > 0) xp[a] += DIM == 3 ? (vold + sv) * (0.5 * dt) : 0.5 * (vold + sv) * dt;
            else xp[a] += (sv + 0.5 * (sv - vold)) * dt;
        }
    }
    p.vx[i] = v[0];
    p.vy[i] = v[1];
    p.x[i] = xp[0];
    p.y[i] = xp[1];
    if (DIM == 3) {
        p.vz[i] = v[2];
        p.z[i] = xp[2];
    }
}

// g2p_move fused with the momentum re-extrapolation of
// UpdateStrainsLastContactTask (UpdateStrainsLastContactTask.cpp:71-146,
// NodalPoint::AddMassMomentumLast NodalPointMPM.cpp:470-486), which uses the
// same natural coordinates of the step (USL), or with the element reset.
template <int DIM, int SHAPE, bool USL, bool MIX, bool BATCH, bool DET = false>
static __global__ void __launch_bounds__(256, 2) k_g2p(StepParams sp, DevParticles p, DevNodes nd, const DevMat *mats) {
    using T = typename Wt<MIX>::T;
    const int i = tile_particle(p);
    if (i >= p.n) return;
    RunView rv;
    if (!particle_run<BATCH>(sp, p, i, rv)) return;
    const DevGrid &g = rv.g;
    const int e = p.elem[i];
    const double xi = p.xi[i], eta = p.eta[i], zeta = DIM == 3 ? p.zeta[i] : 0.;
    const double lx = p.lpx[i], ly = p.lpy[i], lz = DIM == 3 ? p.lpz[i] : 1.;
    const int off = field_offset(sp, mats, p, i);
    // the particle's nodes for this step (CPDI corners or the element window)
    auto visit = [&](auto &&fn) {
        if constexpr (kCpdi<SHAPE>) visit_nodes<DIM, SHAPE, false, T>(g, rv.nb, p, i, fn);
        else for_each_node<DIM, SHAPE, false, T>(g, rv.nb, e, xi, eta, zeta, lx, ly, lz, fn);
    };
    if (particle_rigid(sp, mats, p, i)) {
        // rigid materials move at their current velocity and do not take part
        // in the second extrapolation (UpdateParticlesTask.cpp:291-295,
        // MatPoint2D/3D::MovePosition, UpdateStrainsLastContactTask.cpp:90)
        p.x[i] += rv.dt * p.vx[i];
        p.y[i] += rv.dt * p.vy[i];
        if (DIM == 3) p.z[i] += rv.dt * p.vz[i];
        if (!USL) reset_element<DIM>(g, p, i, rv.err);
        return;
    }
    double v[3], xp[3];
    // window shapes, FP64: the factors once for the particle update and the
    // second extrapolation (both at the step's natural coordinates).  The
    // mixed mode forms its FP32 factors twice: keeping them live costs more
    // (registers) than forming them.
    AxisWin<SHAPE, T> w;
    if constexpr (!kCpdi<SHAPE> && !MIX) {
        particle_window<DIM, SHAPE, false, T>(g, p, i, w);
        g2p_move<DIM, SHAPE, MIX, BATCH>(sp, p, nd, i, rv, off, v, xp, &w);
    } else {
        g2p_move<DIM, SHAPE, MIX, BATCH>(sp, p, nd, i, rv, off, v, xp);
    }
    if (USL && DET) {
        // bounds of the second extrapolation, which k_det_usl then sums
        const double mp = p.mass[i];
        double vm = fmax(fabs(v[0]), fabs(v[1]));
        if (DIM == 3) vm = fmax(vm, fabs(v[2]));
        det_bound(sp.det, DB_UMOM, vm);
        if (rv.mm) {
            const double Vp = fabs(contact_volume<DIM>(p, i, mats[p.mat[i]].rho));
            det_bound(sp.det, DB_UVOL, Vp / mp);
            det_bound(sp.det, DB_UDS, displacement_bound<DIM>(p, i, xp));
            det_bound(sp.det, DB_UGV, Vp * grad_bound<DIM, SHAPE, MIX>(g, p, i));
        }
    } else if (USL) {
        // second extrapolation (NodalPoint::AddMassMomentumLast), with the
        // contact terms at the moved positions in multimaterial mode
        const double mp = p.mass[i];
        double Vp = 0., d[3] = {0., 0., 0.};
        if (rv.mm) {
            Vp = contact_volume<DIM>(p, i, mats[p.mat[i]].rho);
            d[0] = xp[0] - p.x0[i];
            d[1] = xp[1] - p.y0[i];
            if (DIM == 3) d[2] = xp[2] - p.z0[i];
        }
        auto scatter = [&](int n, T N, T gx, T gy, T gz) {
            if (zero_weight(N)) return;
            n += off;
            const double fnmp = (double)N * mp;
            atomicAdd(&nd.ux[n], v[0] * fnmp);
            atomicAdd(&nd.uy[n], v[1] * fnmp);
            if (DIM == 3) atomicAdd(&nd.uz[n], v[2] * fnmp);
            if (rv.mm) add_contact_terms<DIM, MIX>(nd, n, N, fnmp, Vp, d, gx, gy, gz);
        };
        if (rv.mm) {
            if constexpr (kCpdi<SHAPE>) visit_nodes<DIM, SHAPE, true, T>(g, rv.nb, p, i, scatter);
            else for_each_node<DIM, SHAPE, true, T>(g, rv.nb, e, xi, eta, zeta, lx, ly, lz, scatter);
        } else if constexpr (!kCpdi<SHAPE> && !MIX) {
            for_each_window_node_at<DIM, SHAPE, T>(w, g, rv.nb, scatter);
        } else {
            visit(scatter);
        }
    } else {
        reset_element<DIM>(g, p, i, rv.err);
    }
}

// k_g2p with USL in the mixed mode through a shared-memory node tile (single
// material field, window shape functions): the particle update, then the
// second extrapolation accumulated per block as two-sum pairs of mass and of
// mass times the new velocity's difference from the block's reference, added
// once per touched node to the FP64 columns of the second momentum.
template <int DIM, int SHAPE, bool BATCH>
static __global__ void __launch_bounds__(256) k_g2p_tile(StepParams sp, DevParticles p, DevNodes nd) {
    __shared__ NodeTile t;
    const int i = tile_particle(p);
    RunView rv;
    const bool valid = i < p.n && particle_run<BATCH>(sp, p, i, rv);
    int col = 0, row = 0, zr = 0;
    double v[3] = {0., 0., 0.}, xp[3];
    AxisWin<SHAPE, float> w;
    if (valid) {
        elem_coords(rv.g, p.elem[i], col, row, zr);
        axis_windows<DIM, SHAPE, false, float>(rv.g, col, row, zr, p.xi[i], p.eta[i], DIM == 3 ? p.zeta[i] : 0.,
                                               p.lpx[i], p.lpy[i], DIM == 3 ? p.lpz[i] : 1., w);
        g2p_move<DIM, SHAPE, true, BATCH>(sp, p, nd, i, rv, 0, v, xp, &w);
    }
    const bool tiled = tile_open<DIM, SHAPE>(t, valid, BATCH && valid ? p.run[i] : 0, col, row, zr, rv, v, DIM + 1);
    if (valid) {
        const double mp = p.mass[i];
        if (tiled) {
            const float mpf = (float)mp;
            const float d[3] = {(float)(v[0] - t.ref[0]), (float)(v[1] - t.ref[1]), (float)(v[2] - t.ref[2])};
            for_each_window_node<DIM, SHAPE, false, float>(w, [&](int jx, int jy, int jz, float N, float, float, float) {
                if (N == 0.f) return;
                const int k = tile_slot(t.box, w.c, jx, jy, jz);
                const float wm = N * mpf;
                tile_add(t, 0, k, wm);
#pragma unroll
                for (int a = 0; a < DIM; a++) tile_add(t, 1 + a, k, wm * d[a]);
                t.touched[k] = 1;
            });
        } else {
            const DevGrid &g = rv.g;
            for_each_window_node<DIM, SHAPE, false, float>(w, [&](int jx, int jy, int jz, float N, float, float, float) {
                if (N == 0.f) return;
                const int n = rv.nb + (w.c[0] + jx) + g.yplane * (w.c[1] + jy) + g.zplane * (w.c[2] + jz);
                const double fnmp = (double)N * mp;
                atomicAdd(&nd.ux[n], v[0] * fnmp);
                atomicAdd(&nd.uy[n], v[1] * fnmp);
                if (DIM == 3) atomicAdd(&nd.uz[n], v[2] * fnmp);
            });
        }
    }
    __syncthreads();
    tile_flush(t, [&](int n, int k) {
        const double m = tile_sum(t, 0, k);
        atomicAdd(&nd.ux[n], t.ref[0] * m + tile_sum(t, 1, k));
        atomicAdd(&nd.uy[n], t.ref[1] * m + tile_sum(t, 2, k));
        if (DIM == 3) atomicAdd(&nd.uz[n], t.ref[2] * m + tile_sum(t, 3, k));
    });
}

// Deterministic mode: the second extrapolation of k_g2p (momentum at the
// updated velocities, contact terms at the moved positions, the step's
// natural coordinates) as its own pass, once k_g2p has bounded it.
template <int DIM, int SHAPE, bool MIX>
static __global__ void __launch_bounds__(256) k_det_usl(StepParams sp, DevParticles p, DevNodes nd, const DevMat *mats) {
    using T = typename Wt<MIX>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n || particle_rigid(sp, mats, p, i)) return;  // non-rigid particles only
    const DevGrid &g = sp.g;
    const int off = field_offset(sp, mats, p, i);
    const bool mm = sp.ct.nf > 1;
    const double mp = p.mass[i];
    const double v[3] = {p.vx[i], p.vy[i], DIM == 3 ? p.vz[i] : 0.};
    const unsigned long long bU = sp.det.bnd[DB_UMOM], bV = sp.det.bnd[DB_UVOL], bD = sp.det.bnd[DB_UDS];
    const double sG = pow2(det_shift(sp.det.bnd[DB_UGV]));
    double Vp = 0., d[3] = {0., 0., 0.};
    if (mm) {
        Vp = contact_volume<DIM>(p, i, mats[p.mat[i]].rho);
        d[0] = p.x[i] - p.x0[i];
        d[1] = p.y[i] - p.y0[i];
        if (DIM == 3) d[2] = p.z[i] - p.z0[i];
    }
    auto scatter = [&](int n, T N, T gx, T gy, T gz) {
        if (zero_weight(N)) return;
        n += off;
        const double fnmp = (double)N * mp;
        const unsigned long long nb = sp.det.nbnd[n];
        const double sU = pow2(det_shift2(nb, bU));
        det_add(sp.det, DQ_UX, n, v[0] * fnmp, sU, sp.err);
        det_add(sp.det, DQ_UY, n, v[1] * fnmp, sU, sp.err);
        if (DIM == 3) det_add(sp.det, DQ_UZ, n, v[2] * fnmp, sU, sp.err);
        if (mm) {
            const double sc[3] = {pow2(det_shift2(nb, bV)), pow2(det_shift2(nb, bD)), sG};
            det_contact_terms<DIM>(sp.det, n, (double)N, fnmp, Vp, d, (double)gx, (double)gy, (double)gz, sc,
                                   sp.err);
        }
    };
    if constexpr (kCpdi<SHAPE>) {
        if (mm) visit_nodes<DIM, SHAPE, true, T>(g, 0, p, i, scatter);
        else visit_nodes<DIM, SHAPE, false, T>(g, 0, p, i, scatter);
    } else {
        const int e = p.elem[i];
        const double xi = p.xi[i], eta = p.eta[i], zeta = DIM == 3 ? p.zeta[i] : 0.;
        const double lx = p.lpx[i], ly = p.lpy[i], lz = DIM == 3 ? p.lpz[i] : 1.;
        if (mm) for_each_node<DIM, SHAPE, true, T>(g, 0, e, xi, eta, zeta, lx, ly, lz, scatter);
        else for_each_node<DIM, SHAPE, false, T>(g, 0, e, xi, eta, zeta, lx, ly, lz, scatter);
    }
}

// UpdateStrainsFirstTask::FullStrainUpdate called from
// UpdateStrainsLastContactTask (:149), fused with ResetElementsTask.
template <int DIM, int SHAPE, bool MIX, bool BATCH>
static __global__ void __launch_bounds__(256, kStrainBlocks<SHAPE>) k_strain_last(StepParams sp, DevParticles p, DevNodes nd, const DevMat *mats) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    RunView rv;
    if (!particle_run<BATCH>(sp, p, i, rv)) return;
    if (!particle_rigid(sp, mats, p, i)) {
        double du[9];
        velocity_gradient<DIM, SHAPE, MIX>(rv.g, rv.nb, p, nd, i, rv.st_last, du, field_offset(sp, mats, p, i));
        constitutive<DIM>(mats, p, i, du);
    }
    reset_element<DIM>(rv.g, p, i, rv.err);
}

// ---------------------------------------------------------------------------
// node kernels
// ---------------------------------------------------------------------------
enum { BC_MASS_MOMENTUM = 0, BC_UPDATE_MOMENTUM, BC_UPDATE_STRAINS_LAST, BC_GRID_FORCES };

// NodalVelBC::VelocityBCLoop for one node: zero passes then add passes, in
// list order (NodalVelBC.cpp:386-400; MatVelocityField::ZeroVelocityBC and
// AddVelocityBC, MatVelocityField.cpp:490-575).
__device__ __forceinline__ void node_bcs(const DevBCs &b, int grp, int pass, double mass, double t, double dt,
                                         double p[3], double f[3]) {
    const int s = b.start[grp], e = b.start[grp + 1];
    for (int k = s; k < e; k++) {
        if (t < b.ftime[k]) continue;
        const int dir = b.dir[k];
        const double n[3] = {dir == 1 ? 1. : 0., dir == 2 ? 1. : 0., dir == 4 ? 1. : 0.};
        if (pass == BC_GRID_FORCES) {
            const double dotf = f[0] * n[0] + f[1] * n[1] + f[2] * n[2];
            const double dotp = p[0] * n[0] + p[1] * n[1] + p[2] * n[2];
            const double sc = -dotf - dotp / dt;
#pragma unroll
            for (int a = 0; a < 3; a++) f[a] += n[a] * sc;
        } else {
            const double dotn = p[0] * n[0] + p[1] * n[1] + p[2] * n[2];
#pragma unroll
            for (int a = 0; a < 3; a++) p[a] += n[a] * (-dotn);
            if (pass == BC_UPDATE_MOMENTUM) {
#pragma unroll
                for (int a = 0; a < 3; a++) f[a] += n[a] * (-dotn / dt);
            }
        }
    }
    for (int k = s; k < e; k++) {
        if (t < b.ftime[k]) continue;
        const int dir = b.dir[k];
        const double n[3] = {dir == 1 ? 1. : 0., dir == 2 ? 1. : 0., dir == 4 ? 1. : 0.};
        const double vel = b.value[k];
        if (pass == BC_GRID_FORCES) {
            const double sc = mass * vel / dt;
#pragma unroll
            for (int a = 0; a < 3; a++) f[a] += n[a] * sc;
        } else {
            const double pv = mass * vel;
#pragma unroll
            for (int a = 0; a < 3; a++) p[a] += n[a] * pv;
            if (pass == BC_UPDATE_MOMENTUM) {
                const double sc = pv / dt;
#pragma unroll
                for (int a = 0; a < 3; a++) f[a] += n[a] * sc;
            }
        }
    }
}

// MatVelocityField::GridValueCalculation (MatVelocityField.cpp:239-251); the
// mixed mode also keeps the velocity as FP32 hi/lo pairs.
template <bool MIX>
__device__ __forceinline__ void node_velocity(const DevNodes &nd, int n, double mass, const double p[3]) {
    if (mass == 0.) return;
    const double r = 1. / mass;
    const double vx = p[0] * r, vy = p[1] * r, vz = p[2] * r;
    nd.vx[n] = vx;
    nd.vy[n] = vy;
    nd.vz[n] = vz;
    if (MIX) {
        split2(vx, nd.vhx[n], nd.vlx[n]);
        split2(vy, nd.vhy[n], nd.vly[n]);
        split2(vz, nd.vhz[n], nd.vlz[n]);
    }
}

// PostExtrapolationTask::Execute (PostExtrapolationTask.cpp:46-165):
// vk[pkCopy] = pk, velocity conditions of MASS_MOMENTUM_CALL, then grid velocity.
// time and time step of the run a node belongs to
template <bool BATCH>
__device__ __forceinline__ bool node_run(const StepParams &sp, int n, double &t, double &dt) {
    if (!BATCH) {
        t = sp.t;
        dt = sp.dt;
        return true;
    }
    const int r = sp.nrun[n];
    if (r < 0) return false;
    const DevRun &R = sp.runs[r];
    if (!R.active) return false;
    t = R.t;
    dt = R.dt;
    return true;
}

// the contact settings that apply at node n (a batch run carries its own law);
// nf == 1 means no contact at this node
template <bool BATCH>
__device__ __forceinline__ DevContact node_contact_params(const StepParams &sp, int n) {
    DevContact ct = sp.ct;
    if (BATCH && ct.nf > 1) {
        const DevRun &R = sp.runs[sp.nrun[n]];
        if (!R.mm) ct.nf = 1;
        ct.normals = R.normals;
        ct.style = R.style;
        ct.friction = R.friction;
        ct.rigid = R.rigid;
        ct.rigid_bias = R.rigid_bias;
        // the run's step keeps the contact state for XPIC/FMPM of order > 1
        ct.xcache = ct.xc != nullptr && (R.xpic > 1 || R.xpic < -1) ? 1 : 0;
    }
    return ct;
}

// field f of the node's contact holds a rigid contact material
__device__ __forceinline__ bool rigid_field(const DevContact &ct, int f) { return ((ct.rigid >> f) & 1u) != 0u; }

// ---------------------------------------------------------------------------
// multimaterial contact
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// MatVelocityField::ChangeMatMomentum (MatVelocityField.cpp:197-228)
__device__ __forceinline__ void change_momentum(const DevNodes &nd, int k, const double d[3], int pass, double dt) {
    nd.px[k] += d[0];
    nd.py[k] += d[1];
    nd.pz[k] += d[2];
    if (pass == BC_UPDATE_MOMENTUM) {
        const double s = 1. / dt;
        nd.fx[k] += d[0] * s;
        nd.fy[k] += d[1] * s;
        nd.fz[k] += d[2] * s;
    } else if (pass == BC_MASS_MOMENTUM) {
        nd.cx[k] = nd.px[k];
        nd.cy[k] = nd.py[k];
        nd.cz[k] = nd.pz[k];
    }
}

// CoulombFriction::GetFrictionalDeltaMomentum (CoulombFriction.cpp:146-262)
// without a static coefficient; false: the law leaves the momenta alone
__device__ __forceinline__ bool coulomb_delta(const DevContact &ct, double delPi[3], const double norm[3],
                                              double dotn, double deln, double mred, const double *delFi,
                                              double dt) {
    if (ct.style == 0) return true;
    // the separation adjustment after the momentum update is skipped for
    // regression normals (CoulombFriction.cpp:161-170)
    if (delFi && ct.normals < 5) deln += dt * (dotn - 0.5 * dot3(delFi, norm) * dt) / mred;
    const bool inContact = deln < 0. && dotn < 0.;
    if (ct.style == 1) {
        if (!inContact) return false;
#pragma unroll
        for (int a = 0; a < 3; a++) delPi[a] = norm[a] * dotn;
        return true;
    }
    if (!inContact) return false;
    double dott = 0., tang[3];
#pragma unroll
    for (int a = 0; a < 3; a++) tang[a] = delPi[a] + norm[a] * (-dotn);
    const double tangMag = sqrt(dot3(tang, tang));
    if (tangMag > 0.) {
        const double s = 1. / tangMag;
#pragma unroll
        for (int a = 0; a < 3; a++) tang[a] *= s;
        dott = dot3(delPi, tang);
        if (dott < 0.) {
#pragma unroll
            for (int a = 0; a < 3; a++) tang[a] = -tang[a];
            dott = -dott;
        }
    }
    const double slide = ct.friction * (-dotn);
    if (slide <= 0.) {
#pragma unroll
        for (int a = 0; a < 3; a++) delPi[a] = norm[a] * dotn;
    } else if (dott > slide) {
#pragma unroll
        for (int a = 0; a < 3; a++) delPi[a] = norm[a] * dotn + tang[a] * slide;
    }
    return true;
}

// CrackVelocityFieldMulti::MaterialContactOnCVF / MaterialContactOnCVFLumped
// (CrackVelocityFieldMulti.cpp:302-671) at node n for nonrigid materials:
// each material against the others lumped (two materials: one pair with
// equal and opposite momentum changes), normal from volume gradients
// (GetNormalVector :960-1069, methods 0-2), separation from the extrapolated
// displacements (CrackSurfaceContact::MaterialSeparation), Coulomb friction.
constexpr int kMaxFields = 8;
// CrackVelocityFieldMulti::RigidMaterialContactOnCVF (CrackVelocityFieldMulti.cpp:676-958)
// for the Coulomb law: every non-rigid field of the node moves toward the
// velocity of the rigid field rf (whose own momentum never changes), with
// mred = the field's mass and, after the momentum update, dF = -F; the normal
// is GetNormalVector's with a rigid partner (:960-1030), the rigid volume
// gradient preferred by the squared bias; the separation comes from the
// displacements (CrackSurfaceContact::MaterialSeparation).
template <bool MIX>
__device__ void rigid_contact(const DevContact &ct, const DevNodes &nd, int n, const int *act, int nm, int rf,
                              double rvol, int pass, double dt) {
    const int S = ct.fstride, kr = rf * S + n;
    const double rr = 1. / nd.mass[kr];  // the rigid field's mass is its volume
    const double rvel[3] = {nd.px[kr] * rr, nd.py[kr] * rr, nd.pz[kr] * rr};
    const double gradj[3] = {-cterm<MIX>(nd.gvx, kr), -cterm<MIX>(nd.gvy, kr), -cterm<MIX>(nd.gvz, kr)};
    const double dispR[3] = {nd.dsx[kr] * rr, nd.dsy[kr] * rr, nd.dsz[kr] * rr};
    for (int q = 0; q < nm; q++) {
        const int f = act[q];
        if (rigid_field(ct, f)) continue;
        const int ki = f * S + n;
        const double massi = nd.mass[ki], voli = cterm<MIX>(nd.vol, ki);
        double delPi[3] = {rvel[0] * massi - nd.px[ki], rvel[1] * massi - nd.py[ki], rvel[2] * massi - nd.pz[ki]};
        const double normi[3] = {cterm<MIX>(nd.gvx, ki), cterm<MIX>(nd.gvy, ki), cterm<MIX>(nd.gvz, ki)};
        double norm[3];
        if (ct.normals == 0) {
            const double magi = sqrt(dot3(normi, normi)), magj = sqrt(dot3(gradj, gradj));
            const bool useI = magi >= ct.rigid_bias * magj;
            const double s = 1. / (useI ? magi : magj);
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] = (useI ? normi[a] : gradj[a]) * s;
        } else if (ct.normals == 1) {
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] = voli >= rvol ? normi[a] : gradj[a];
            const double s = 1. / sqrt(dot3(norm, norm));
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] *= s;
        } else {
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] = normi[a] + gradj[a];
            const double magi = dot3(norm, norm), magj = dot3(gradj, gradj);
            const double vRatio = (voli + rvol) / rvol;
            if (magi >= ct.rigid_bias * magj * vRatio * vRatio) {
                const double s = 1. / sqrt(magi);
#pragma unroll
                for (int a = 0; a < 3; a++) norm[a] *= s;
            } else {
                const double s = 1. / sqrt(magj);
#pragma unroll
                for (int a = 0; a < 3; a++) norm[a] = gradj[a] * s;
            }
        }
        if (norm[0] != norm[0] || norm[1] != norm[1] || norm[2] != norm[2]) continue;
        const double dotn = dot3(delPi, norm);
        const double rmi = 1. / massi;
        const double dispi[3] = {nd.dsx[ki] * rmi, nd.dsy[ki] * rmi, nd.dsz[ki] * rmi};
        const double deln = dot3(dispR, norm) - dot3(dispi, norm);
        double delFi[3];
        const double *dfp = nullptr;
        if (pass == BC_UPDATE_MOMENTUM) {
            delFi[0] = -nd.fx[ki];
            delFi[1] = -nd.fy[ki];
            delFi[2] = -nd.fz[ki];
            dfp = delFi;
        }
        if (!coulomb_delta(ct, delPi, norm, dotn, deln, massi, dfp, dt)) continue;
        change_momentum(nd, ki, delPi, pass, dt);
    }
}

template <bool MIX>
__device__ void node_contact(const DevContact &ct, const DevNodes &nd, int n, int pass, double dt) {
    const int S = ct.fstride;
    int act[kMaxFields], nm = 0;
    double Pc[3] = {0., 0., 0.}, Mc = 0., dispc[3] = {0., 0., 0.}, voltot = 0.;
    for (int f = 0; f < ct.nf; f++) {
        const int k = f * S + n;
        if (!nd.active[k]) continue;
        Pc[0] += nd.px[k];
        Pc[1] += nd.py[k];
        Pc[2] += nd.pz[k];
        Mc += nd.mass[k];
        dispc[0] += nd.dsx[k];
        dispc[1] += nd.dsy[k];
        dispc[2] += nd.dsz[k];
        voltot += cterm<MIX>(nd.vol, k);
        act[nm++] = f;
    }
    if (nm <= 1) return;
    if (ct.rigid) {
        // a rigid field at the node: contact against it alone (the one with
        // the largest contact volume when several), CrackVelocityFieldMulti::
        // MaterialContactOnCVF (CrackVelocityFieldMulti.cpp:302-347, 688-706)
        int rf = -1;
        double rvol = 0.;
        for (int q = 0; q < nm; q++) {
            if (!rigid_field(ct, act[q])) continue;
            const double v = cterm<MIX>(nd.vol, act[q] * S + n);
            if (rf < 0 || v > rvol) {
                rf = act[q];
                rvol = v;
            }
        }
        if (rf >= 0) {
            rigid_contact<MIX>(ct, nd, n, act, nm, rf, rvol, pass, dt);
            return;
        }
    }
    const bool pairs = nm == 2;
    const int miMax = pairs ? 1 : nm;
    const double rMc = 1. / Mc;
#pragma unroll
    for (int a = 0; a < 3; a++) dispc[a] *= rMc;
    for (int mi = 0; mi < miMax; mi++) {
        const int ki = act[mi] * S + n;
        const double massi = nd.mass[ki], voli = cterm<MIX>(nd.vol, ki);
        const double volj = voltot - voli;
        int j = -1;
        double gradj[3] = {0., 0., 0.}, maxOther = 0.;
        for (int kj = 0; kj < nm; kj++) {
            if (kj == mi) continue;
            const int kk = act[kj] * S + n;
            const double vk = cterm<MIX>(nd.vol, kk);
            if (vk > maxOther) {
                maxOther = vk;
                j = act[kj];
            }
            gradj[0] -= cterm<MIX>(nd.gvx, kk);
            gradj[1] -= cterm<MIX>(nd.gvy, kk);
            gradj[2] -= cterm<MIX>(nd.gvz, kk);
        }
        if (j < 0) continue;
        const double massRatio = massi / Mc;
        double mred = 1. - massRatio;
        double delPi[3] = {Pc[0] * massRatio - nd.px[ki], Pc[1] * massRatio - nd.py[ki],
                           Pc[2] * massRatio - nd.pz[ki]};
        const double normi[3] = {cterm<MIX>(nd.gvx, ki), cterm<MIX>(nd.gvy, ki), cterm<MIX>(nd.gvz, ki)};
        double norm[3];
        bool hasDeln = false;
        double lrDeln = 0.;
        if (ct.normals >= 5) {
            // regression normal and separation of this material against the
            // others lumped (GetNormalVector, CrackVelocityFieldMulti.cpp:1033-1062)
            const double *o = ct.lr + 4 * (size_t)ki;
            norm[0] = o[0];
            norm[1] = o[1];
            norm[2] = o[2];
            lrDeln = o[3];
            hasDeln = true;
        } else if (ct.normals == 0) {
            const double magi = sqrt(dot3(normi, normi)), magj = sqrt(dot3(gradj, gradj));
            const bool useI = magi >= magj;
            const double s = 1. / (useI ? magi : magj);
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] = (useI ? normi[a] : gradj[a]) * s;
        } else if (ct.normals == 1) {
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] = voli >= volj ? normi[a] : gradj[a];
            const double s = 1. / sqrt(dot3(norm, norm));
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] *= s;
        } else {
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] = normi[a] + gradj[a];
            const double s = 1. / sqrt(dot3(norm, norm));
#pragma unroll
            for (int a = 0; a < 3; a++) norm[a] *= s;
        }
        if (norm[0] != norm[0] || norm[1] != norm[1] || norm[2] != norm[2]) continue;
        const double dotn = dot3(delPi, norm);
        const double rmi = 1. / massi, rmred = 1. / mred;
        const double dispa[3] = {nd.dsx[ki] * rmi, nd.dsy[ki] * rmi, nd.dsz[ki] * rmi};
        double dispb[3];
#pragma unroll
        for (int a = 0; a < 3; a++) dispb[a] = (dispc[a] - dispa[a]) * rmred + dispa[a];
        const double deln = hasDeln ? lrDeln : dot3(dispb, norm) - dot3(dispa, norm);
        mred *= massi;
        // MaterialContactNode::SetContactInfo (MaterialContactNode.cpp:133-151)
        double *xc = ct.xcache ? ct.xc + kXcDoubles * (size_t)ki : nullptr;
        if (xc) {
            ct.xc_pair[ki] = pairs ? j : -1;
            xc[0] = deln;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                xc[1 + a] = norm[a];
                xc[4 + a] = delPi[a];
                xc[7 + a] = 0.;
                xc[10 + a] = 0.;
            }
        }
        double delFi[3];
        const double *dfp = nullptr;
        if (pass == BC_UPDATE_MOMENTUM) {
            double Fc[3] = {0., 0., 0.};
            for (int q = 0; q < nm; q++) {
                const int k = act[q] * S + n;
                Fc[0] += nd.fx[k];
                Fc[1] += nd.fy[k];
                Fc[2] += nd.fz[k];
            }
            delFi[0] = Fc[0] * massRatio - nd.fx[ki];
            delFi[1] = Fc[1] * massRatio - nd.fy[ki];
            delFi[2] = Fc[2] * massRatio - nd.fz[ki];
            dfp = delFi;
            if (xc)
#pragma unroll
                for (int a = 0; a < 3; a++) xc[10 + a] = delFi[a];
        }
        if (!coulomb_delta(ct, delPi, norm, dotn, deln, mred, dfp, dt)) continue;
        change_momentum(nd, ki, delPi, pass, dt);
        // MaterialContactNode::ContactSetDelPi
        if (xc)
#pragma unroll
            for (int a = 0; a < 3; a++) xc[7 + a] = delPi[a];
        if (pairs) {
            const double neg[3] = {-delPi[0], -delPi[1], -delPi[2]};
            change_momentum(nd, j * S + n, neg, pass, dt);
        }
    }
}

// store the updated momentum and force, grid velocity, and the acceleration
// f/m for the particle update (every active node has mass > 0)
template <int DIM, bool MIX>
__device__ __forceinline__ void node_finish_update(const DevNodes &nd, int k, double m, const double p[3],
                                                   const double fr[3]) {
    nd.px[k] = p[0];
    nd.py[k] = p[1];
    nd.fx[k] = fr[0];
    nd.fy[k] = fr[1];
    if (DIM == 3) {
        nd.pz[k] = p[2];
        nd.fz[k] = fr[2];
    }
    node_velocity<MIX>(nd, k, m, p);
    const double r = 1. / m;
    nd.ax[k] = fr[0] * r;
    nd.ay[k] = fr[1] * r;
    if (DIM == 3) nd.az[k] = fr[2] * r;
    if (MIX) {
        nd.bx[k] = (float)(fr[0] * r);
        nd.by[k] = (float)(fr[1] * r);
        if (DIM == 3) nd.bz[k] = (float)(fr[2] * r);
    }
}

// true when any material field of node n has particles
__device__ __forceinline__ bool node_active(const StepParams &sp, const DevNodes &nd, int n) {
    for (int f = 0; f < sp.ct.nf; f++)
        if (nd.active[f * sp.ct.fstride + n]) return true;
    return false;
}

// PostExtrapolationTask::Execute (PostExtrapolationTask.cpp:46-165):
// vk[pkCopy] = pk, contact (MASS_MOMENTUM_CALL), velocity conditions, grid
// velocity, on every material field of the node.
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_node_post(StepParams sp, DevNodes nd, int nnodes, DevBCs b, const int *bc_group, int do_bcs) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes || !node_active(sp, nd, n)) return;
    double t, dt;
    if (!node_run<BATCH>(sp, n, t, dt)) return;
    const int grp = bc_group[n];
    for (int f = 0; f < sp.ct.nf; f++) {
        const int k = f * sp.ct.fstride + n;
        if (!nd.active[k]) continue;
        nd.cx[k] = nd.px[k];
        nd.cy[k] = nd.py[k];
        if (DIM == 3) nd.cz[k] = nd.pz[k];
    }
    const DevContact ct = node_contact_params<BATCH>(sp, n);
    if (ct.nf > 1) node_contact<MIX>(ct, nd, n, BC_MASS_MOMENTUM, dt);
    for (int f = 0; f < sp.ct.nf; f++) {
        const int k = f * sp.ct.fstride + n;
        if (!nd.active[k]) continue;
        double p[3] = {nd.px[k], nd.py[k], DIM == 3 ? nd.pz[k] : 0.};
        const double m = nd.mass[k];
        // velocity conditions apply to the non-rigid fields only (CrackVelocityFieldMulti.cpp:1243-1259)
        if (do_bcs && grp >= 0 && !rigid_field(ct, f)) {
            double fz[3] = {0., 0., 0.};
            node_bcs(b, grp, BC_MASS_MOMENTUM, m, t, dt, p, fz);
            nd.px[k] = p[0];
            nd.py[k] = p[1];
            if (DIM == 3) nd.pz[k] = p[2];
        }
        node_velocity<MIX>(nd, k, m, p);
    }
}

// PostForcesTask::Execute (restore momenta, GRID_FORCES_CALL velocity
// conditions; PostForcesTask.cpp:43-111) and UpdateMomentaTask::Execute
// (p += f dt, contact and UPDATE_MOMENTUM_CALL conditions;
// UpdateMomentaTask.cpp:44-94), then grid velocity and acceleration for the
// particle update.  zero_contact: clear the contact terms for the second
// extrapolation.
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_node_update(StepParams sp, DevNodes nd, int nnodes, DevBCs b, const int *bc_group,
                              int zero_contact, int update_bcs = 1) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes || !node_active(sp, nd, n)) return;
    double t, dt;
    if (!node_run<BATCH>(sp, n, t, dt)) return;
    const int grp = bc_group[n];
    const DevContact ct = node_contact_params<BATCH>(sp, n);
    const bool mm = ct.nf > 1;
    if (BATCH) {
        const int xm = sp.runs[sp.nrun[n]].xpic;
        update_bcs = xm >= -1 && xm <= 1;
    }
    for (int f = 0; f < sp.ct.nf; f++) {
        const int k = f * sp.ct.fstride + n;
        if (!nd.active[k]) continue;
        double p[3] = {nd.cx[k], nd.cy[k], DIM == 3 ? nd.cz[k] : 0.};
        double fr[3];
        if (MIX) {
            // FP64 sums of tiled blocks plus FP32 sums of the other particles
            fr[0] = nd.fx[k] + (double)nd.gx[k];
            fr[1] = nd.fy[k] + (double)nd.gy[k];
            fr[2] = DIM == 3 ? nd.fz[k] + (double)nd.gz[k] : 0.;
        } else {
            fr[0] = nd.fx[k];
            fr[1] = nd.fy[k];
            fr[2] = DIM == 3 ? nd.fz[k] : 0.;
        }
        const double m = nd.mass[k];
        const bool rigid = rigid_field(ct, f);  // no forces, no conditions: its momentum stays as extrapolated
        if (grp >= 0 && !rigid) node_bcs(b, grp, BC_GRID_FORCES, m, t, dt, p, fr);
#pragma unroll
        for (int a = 0; a < 3; a++) p[a] += fr[a] * dt;
        if (mm) {
            // staged for the contact of all the node's fields
            nd.px[k] = p[0];
            nd.py[k] = p[1];
            nd.pz[k] = p[2];
            nd.fx[k] = fr[0];
            nd.fy[k] = fr[1];
            nd.fz[k] = fr[2];
            continue;
        }
        // NodalVelBC::GridVelocityConditions skips this pass for XPIC/FMPM(k > 1)
        // (NodalVelBC.cpp:367-374)
        if (grp >= 0 && update_bcs) node_bcs(b, grp, BC_UPDATE_MOMENTUM, m, t, dt, p, fr);
        node_finish_update<DIM, MIX>(nd, k, m, p, fr);
    }
    if (!mm) return;
    node_contact<MIX>(ct, nd, n, BC_UPDATE_MOMENTUM, dt);
    for (int f = 0; f < sp.ct.nf; f++) {
        const int k = f * sp.ct.fstride + n;
        if (!nd.active[k]) continue;
        double p[3] = {nd.px[k], nd.py[k], nd.pz[k]}, fr[3] = {nd.fx[k], nd.fy[k], nd.fz[k]};
        const double m = nd.mass[k];
        const bool rigid = rigid_field(ct, f);
        if (grp >= 0 && !rigid) node_bcs(b, grp, BC_UPDATE_MOMENTUM, m, t, dt, p, fr);
        node_finish_update<DIM, MIX>(nd, k, m, p, fr);
        if (zero_contact && rigid) {
            // a rigid field keeps its momentum, volume and volume gradient for the
            // second extrapolation; its displacement moves by p dt
            // (CrackVelocityFieldMulti::RezeroNodeTask6, :157-176)
            nd.dsx[k] += p[0] * dt;
            nd.dsy[k] += p[1] * dt;
            nd.dsz[k] += p[2] * dt;
        } else if (zero_contact) {
            cterm_set<MIX>(nd.vol, k, 0.);
            nd.dsx[k] = nd.dsy[k] = nd.dsz[k] = 0.;
            cterm_set<MIX>(nd.gvx, k, 0.);
            cterm_set<MIX>(nd.gvy, k, 0.);
            cterm_set<MIX>(nd.gvz, k, 0.);
        }
    }
}

// UpdateStrainsLastContactTask: p = second extrapolation, contact and
// UPDATE_STRAINS_LAST_CALL conditions, grid velocity
// (UpdateStrainsLastContactTask.cpp:60-152).
template <int DIM, bool MIX, bool BATCH>
static __global__ void k_node_usl(StepParams sp, DevNodes nd, int nnodes, DevBCs b, const int *bc_group) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes || !node_active(sp, nd, n)) return;
    double t, dt;
    if (!node_run<BATCH>(sp, n, t, dt)) return;
    const int grp = bc_group[n];
    const DevContact ct = node_contact_params<BATCH>(sp, n);
    const bool mm = ct.nf > 1;
    if (mm) {
        for (int f = 0; f < sp.ct.nf; f++) {
            const int k = f * sp.ct.fstride + n;
            if (!nd.active[k] || rigid_field(ct, f)) continue;  // rigid: the first extrapolation's momentum
            nd.px[k] = nd.ux[k];
            nd.py[k] = nd.uy[k];
            nd.pz[k] = nd.uz[k];
        }
        node_contact<MIX>(ct, nd, n, BC_UPDATE_STRAINS_LAST, dt);
    }
    for (int f = 0; f < sp.ct.nf; f++) {
        const int k = f * sp.ct.fstride + n;
        if (!nd.active[k]) continue;
        double p[3];
        if (mm) {
            p[0] = nd.px[k];
            p[1] = nd.py[k];
            p[2] = nd.pz[k];
        } else {
            p[0] = nd.ux[k];
            p[1] = nd.uy[k];
            p[2] = DIM == 3 ? nd.uz[k] : 0.;
        }
        const double m = nd.mass[k];
        if (grp >= 0 && !rigid_field(ct, f)) {
            double fz[3] = {0., 0., 0.};
            node_bcs(b, grp, BC_UPDATE_STRAINS_LAST, m, t, dt, p, fz);
        }
        nd.px[k] = p[0];
        nd.py[k] = p[1];
        if (DIM == 3) nd.pz[k] = p[2];
        node_velocity<MIX>(nd, k, m, p);
    }
}

// Deterministic mode: the node sums of one extrapolation written over the
// node columns the node kernels read, the limbs cleared for the next one.
// Phase 0: mass and momentum (and contact terms) after k_p2g; 1: internal
// forces after k_det_forces; 2: momentum (and contact terms) after k_det_usl.
// nn counts every field of every node.
template <int DIM, bool MIX>
static __global__ void k_det_resolve(StepParams sp, DevNodes nd, int nn, int phase) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const DevDet &d = sp.det;
    auto take = [&](int q, int slot) { return det_take(d, q, n, pow2(-det_shift(d.bnd[slot]))); };
    const unsigned long long nb = d.nbnd[n];  // the node's largest mass contribution
    auto take2 = [&](int q, int slot) { return det_take(d, q, n, pow2(-det_shift2(nb, d.bnd[slot]))); };
    if (phase == 1) {
        const double fx = take(DQ_FX, DB_FORCE), fy = take(DQ_FY, DB_FORCE);
        const double fz = DIM == 3 ? take(DQ_FZ, DB_FORCE) : 0.;
        if (MIX) {
            nd.gx[n] = (float)fx;
            nd.gy[n] = (float)fy;
            if (DIM == 3) nd.gz[n] = (float)fz;
        } else {
            nd.fx[n] = fx;
            nd.fy[n] = fy;
            if (DIM == 3) nd.fz[n] = fz;
        }
        return;
    }
    const bool usl = phase == 2;
    // a rigid field has no second extrapolation: it keeps the first one's
    // momentum and contact terms (its limbs of this phase stay zero)
    if (usl && sp.ct.rigid && ((sp.ct.rigid >> (n / sp.ct.fstride)) & 1u)) return;
    if (usl) {
        nd.ux[n] = take2(DQ_UX, DB_UMOM);
        nd.uy[n] = take2(DQ_UY, DB_UMOM);
        if (DIM == 3) nd.uz[n] = take2(DQ_UZ, DB_UMOM);
    } else {
        nd.mass[n] = det_take(d, DQ_MASS, n, pow2(-det_shift(nb)));
        nd.px[n] = take2(DQ_PX, DB_MOM);
        nd.py[n] = take2(DQ_PY, DB_MOM);
        if (DIM == 3) nd.pz[n] = take2(DQ_PZ, DB_MOM);
    }
    if (sp.ct.nf > 1) {
        const int bv = usl ? DB_UVOL : DB_VOL, bd = usl ? DB_UDS : DB_DS, bg = usl ? DB_UGV : DB_GV;
        cterm_set<MIX>(nd.vol, n, take2(DQ_VOL, bv));
        nd.dsx[n] = take2(DQ_DSX, bd);
        nd.dsy[n] = take2(DQ_DSY, bd);
        cterm_set<MIX>(nd.gvx, n, take(DQ_GVX, bg));
        cterm_set<MIX>(nd.gvy, n, take(DQ_GVY, bg));
        if (DIM == 3) {
            nd.dsz[n] = take2(DQ_DSZ, bd);
            cterm_set<MIX>(nd.gvz, n, take(DQ_GVZ, bg));
        }
    }
}

// End of a batched step: advance the time of every active run and retire
// runs that have taken all their steps.  A run that raised an error stops
// here, so the error stays confined to its own particles and nodes.
static __global__ void k_advance_runs(DevRun *runs, int nruns, int xpic_order, int xpic_fmpm, int xpic_period) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nruns) return;
    DevRun &R = runs[r];
    if (!R.active) return;
    if (R.err) {
        R.active = 0;
        return;
    }
    R.t += R.dt;
    if (--R.steps_left <= 0) R.active = 0;
    // the PeriodicXPIC mode of the run's next step
    R.xpic = xpic_mode(xpic_order, xpic_fmpm, xpic_period, (long long)floor(R.t / R.dt + 0.5) + 1);
}

}  // namespace nmg

#include "lr.cuh"
#include "xpic.cuh"
