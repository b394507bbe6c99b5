// mpm_device.cuh -- device data structures and per-particle math of the
// explicit MPM step: GIMP/linear shape functions, the hypoelastic isotropic law
// and J2 plasticity with linear hardening.  Every function restates one
// reference function, cited beside it (paths relative to nairn-mpm-fea).
#pragma once

#include <cstdint>

namespace nmg {

constexpr double kSqrtTwoThirds = 0.8164965809277260;  // sqrt(2/3)

// error bits raised by kernels (reported through the C ABI status)
enum : unsigned { ERR_NAN = 1u, ERR_LEFT_GRID = 2u, ERR_EDGE = 4u, ERR_CPDI_NODES = 16u, ERR_RANGE = 32u };

// material type ids (MaterialController.cpp:105-231)
constexpr int kMatIsotropic = 1, kMatIsoPlasticity = 9, kMatNeohookean = 28;
// rigid contact material (RigidMaterial in multimaterial mode, RigidMaterial.hpp:14)
constexpr int kMatRigid = 35;

struct DevGrid {
    int dim, nx, ny, nz;
    int xplane, yplane, zplane, nnodes;  // node-number strides, node count
    double xmin, ymin, zmin, gx, gy, gz;  // origin and cell size (MeshInfo)
    double igx, igy, igz;                 // 1 / cell size
    const double *xn, *yn, *zn;           // node coordinates per axis
};

// Specific material constants, derived on the host exactly as the reference's
// VerifyAndLoadProperties does.
struct DevMat {
    int type;
    int field;                                   // material velocity field (multimaterial mode)
    double rho;                                  // density, g/mm^3 (contact volumes)
    double c11, c12, c22, c33, c41, c42, c44;    // 2D: Elastic::FillUnrotatedElasticProperties
    double C00, C01, C02, C11, C12, C22, C33, C44, C55;  // 3D specific stiffness
    double Gred, Kred;                           // IsoPlasticity specific moduli
    double yldred, Epred, alphaMax, yldredMin;   // LinearHardening
    double Gsp, Lamesp;                          // Neohookean specific moduli (pr.Gsp, pr.Lamesp)
    int uj;                                      // Neohookean U(J) option
    int kterms;                                  // terms of the incremental F exponential
};

struct DevParticles {
    int n;
    double *x, *y, *z, *vx, *vy, *vz;
    double *x0, *y0, *z0;      // original position (multimaterial contact displacement)
    double *mass;
    int *mat, *elem;
    double *lpx, *lpy, *lpz;
    double *exx, *eyy, *ezz, *exy, *exz, *eyz, *wxy, *wxz, *wyz;
    double *sxx, *syy, *szz, *sxy, *sxz, *syz, *pressure;
    double *pxx, *pyy, *pzz, *pxy, *pxz, *pyz;
    double *hist0, *hist1, *work, *plast;
    double *xi, *eta, *zeta;   // natural coordinates of the step (ncpos)
    int *run;                  // run of each slot in a batch (-1: empty); unused for one run
    // lCPDI only, rebuilt at every step start (CPDIDomain): per corner c the
    // element ce[c*n+i], natural coordinates cxi[(3c+a)*n+i] and gradient
    // weights cwg[(3c+a)*n+i]
    int *ce;
    double *cxi, *cwg;
    // FP64 single runs with window shape functions: the step's per-axis
    // window factors, formed once by k_p2g and reread by the later particle
    // kernels of the step (S then dS per axis and node: win[k*n+i]), and the
    // window's first node relative to the run's node base (win_n0[i]).
    // nullptr: every kernel forms the window from the natural coordinates.
    double *win;
    int *win_n0;
    // 1: the columns are host memory the kernels reach over the host link
    // (mpmgpu_step_host); the lanes of a warp then take consecutive slots
    // (tile_particle), so that each warp access is whole lines of the link
    int host_resident;
};

struct DevNodes {
    double *mass;
    double *px, *py, *pz;      // momentum
    double *fx, *fy, *fz;      // total force
    double *cx, *cy, *cz;      // copy of extrapolated momentum (vk[pkCopy])
    double *vx, *vy, *vz;      // velocity p/m
    double *ux, *uy, *uz;      // second (update-strains-last) momentum extrapolation
    double *ax, *ay, *az;      // acceleration f/m after the momentum update
    unsigned char *active;     // numberPoints > 0
    // mixed-precision transfer mode only
    float *vhx, *vhy, *vhz;    // velocity split v = hi + lo in FP32 pairs
    float *vlx, *vly, *vlz;
    float *gx, *gy, *gz;       // FP32 force accumulators
    float *bx, *by, *bz;       // FP32 acceleration for the particle update
    // multimaterial contact terms (ContactTerms): volume, displacement and
    // volume gradient extrapolations of each material field
    double *vol, *dsx, *dsy, *dsz, *gvx, *gvy, *gvz;
};

// Multimaterial contact settings (MeshInfo and the Coulomb friction law).
struct DevContact {
    int nf;          // material velocity fields (1: single material mode)
    int fstride;     // node-index offset between fields
    int normals;     // MeshInfo::materialNormalMethod 0, 1, 2, 5 or 6
    int style;       // CoulombFriction: 0 stick, 1 frictionless, 2 frictional
    double friction; // Coulomb coefficient
    const double *lr;  // regression normals (5, 6): 4 per field-node (n, deln)
    unsigned rigid;    // bit f set: field f holds a rigid contact material (MatVelocityField::IsRigidField)
    double rigid_bias; // MeshInfo::rigidGradientBias, squared (MeshInfo.cpp:1191)
    // XPIC/FMPM(k > 1) with contact: the FMPMContact cache of every field-node
    // (Common/System/DataTypes.hpp:90-104), set by each contact call of a step
    // whose order is > 1 (xcache != 0) -- 13 doubles at xc[13 k]: deltaDotn,
    // norm (3), priorDelPiZero (3), netDelPi (3), startDelFi (3) -- and the
    // paired field at xc_pair[k] (-1: lumped, below -1: not set this step)
    double *xc;
    int *xc_pair;
    int xcache;
};

constexpr int kXcDoubles = 13;

// Deterministic node sums (MPMGPU_P2G_DETERMINISTIC): three 64-bit integer
// limbs per accumulated node quantity -- limb l of quantity q at node n is
// lim[(3 q + l) stride + n] -- and the step's magnitude bounds, step-wide per
// bound slot and per node, as the bit patterns of non-negative doubles
// (atomicMax on the bits orders them as numbers).  lim == nullptr: hardware
// float atomics.
struct DevDet {
    long long *lim;
    size_t stride;
    unsigned long long *bnd;
    unsigned long long *nbnd;  // each node's largest mass contribution (bits)
};

// One run of a batch: its grid, where its nodes and cells start in the
// batch's node and cell arenas, and its own time stepping.
struct DevRun {
    DevGrid g;
    int node_base;     // first global node of the run
    int cell_base;     // first global cell (offset of the run's sort keys)
    int active;        // the run advances while active
    int steps_left;    // steps still to take (the run deactivates at zero)
    double dt, st_first, st_last, t;
    unsigned err;      // error bits of this run
    int mm;            // multimaterial contact on for this run
    int normals, style;
    double friction;   // the run's contact law (DevContact fields)
    int xpic;          // this step's PeriodicXPIC mode (0 FLIP, k FMPM(k), -k XPIC(k))
    unsigned rigid;    // the run's rigid contact fields (DevContact::rigid)
    double rigid_bias;
};

// PeriodicXPIC::PrepareForStep / StepCalculation (NairnMPM/src/Custom_Tasks/
// PeriodicXPIC.cpp:351-370, 427-445), the custom tasks running once before
// the first step and after each step (NairnMPM.cpp:171-200): step s (from 1)
// uses the task's order when s is a multiple of periodicSteps, FLIP (0)
// otherwise; FMPM(k) as +k, XPIC(k) as -k
__host__ __device__ __forceinline__ int xpic_mode(int order, int fmpm, int period, long long s) {
    if (order <= 0 || period <= 0 || s % period != 0) return 0;
    return fmpm ? order : -order;
}

// Per-launch step parameters.  A single-run context uses g, dt, st_first,
// st_last, t and err directly; a batch (BATCH = true in the kernels) reads the
// run of each particle (DevParticles::run) or node (nrun) from `runs`.
struct StepParams {
    DevGrid g;
    double dt, st_first, st_last, t;
    unsigned *err;
    DevRun *runs;
    const int *nrun;   // run of each node (-1: unused)
    DevContact ct;     // one field unless multimaterial mode
    DevDet det;        // deterministic node sums (single-run contexts only)
    int xpic;          // particle update of this step: 0 FLIP, k > 0 FMPM(k), -k XPIC(k)
};

// Velocity conditions grouped by node, list order kept inside a node.
struct DevBCs {
    int nnodes_bc;
    const int *node;           // 0-based node index per group
    const int *start;          // group g uses entries [start[g], start[g+1])
    const int *dir;            // 1, 2, 4
    const double *value;
    const double *ftime;
};

// ---------------------------------------------------------------------------
// element geometry
// ---------------------------------------------------------------------------
__device__ __forceinline__ void elem_coords(const DevGrid &g, int e, int &col, int &row, int &zr) {
    col = e % g.nx;
    int r = e / g.nx;
    row = r % g.ny;
    zr = g.dim == 3 ? r / g.ny : 0;
}

// FourNodeIsoparam::GetXiPos / EightNodeIsoparamBrick::GetXiPos for
// rectangular elements (Common/Elements/FourNodeIsoparam.cpp:351-366,
// NairnMPM/src/Elements/EightNodeIsoparamBrick.cpp:276-281).
// a / b, as a product when b is a power of two (the exact reciprocal from the
// exponent bits: the same bits as the quotient, without an FP64 division)
__device__ __forceinline__ double quotient(double a, double b) {
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b);
    const unsigned long long e = (bb >> 52) & 0x7ffull;
    if ((bb & 0x000fffffffffffffull) == 0ull && e >= 1ull && e <= 2045ull)
        return a * __longlong_as_double((long long)((bb & 0x8000000000000000ull) | ((2046ull - e) << 52)));
    return a / b;
}

__device__ __forceinline__ void xi_position(const DevGrid &g, int e, double x, double y, double z,
                                            double &xi, double &eta, double &zeta) {
    int col, row, zr;
    elem_coords(g, e, col, row, zr);
    double x0 = g.xn[col], x1 = g.xn[col + 1];
    double y0 = g.yn[row], y1 = g.yn[row + 1];
    xi = quotient(2. * x - x0 - x1, x1 - x0);
    eta = quotient(2. * y - y0 - y1, y1 - y0);
    if (g.dim == 3) {
        double z0 = g.zn[zr], z1 = g.zn[zr + 1];
        zeta = quotient(2. * z - z0 - z1, z1 - z0);
    } else {
        zeta = 0.;
    }
}

// ---------------------------------------------------------------------------
// uGIMP factors.  FourNodeIsoparam::GimpShapeFunction (FourNodeIsoparam.cpp:431-519)
// and EightNodeIsoparamBrick::GimpShapeFunction (EightNodeIsoparamBrick.cpp:289-403)
// evaluate, for each candidate node at natural coordinate 2k-3 (k = 0..3, node
// offset k-1 from the element's first node), a 1D factor per axis and take
// their product.  The window below computes the same 1D factors.
// ---------------------------------------------------------------------------
// Window form of the same factors.  For lp <= 1 the support of a particle
// spans three candidates per axis: k = s..s+2 with s = 1 exactly when the
// candidate at +3 passes the reference's test |xi-3| < 2+lp (then the one at -3
// cannot), else s = 0 (the -3 candidate may still be outside the support and
// gets a zero factor).  All lanes of a warp then run the same 27 (3D) or 9
// (2D) node bodies.  dS already carries the sign and the 2/dx scale.
template <typename T>
struct Win {
    T S[3], dS[3];
    int s;
};

// a < b and a <= b for non-negative a and finite b (no NaN): for doubles the
// order of the bit patterns as signed integers, which is the order of the
// values there (a negative b has a negative pattern, below every non-negative
// a), in the integer pipe instead of the FP64 pipe.  x > 0 likewise from the
// pattern (a positive double's pattern is a positive integer).
__device__ __forceinline__ bool nn_less(double a, double b) { return __double_as_longlong(a) < __double_as_longlong(b); }
__device__ __forceinline__ bool nn_less_eq(double a, double b) {
    return __double_as_longlong(a) <= __double_as_longlong(b);
}
__device__ __forceinline__ bool positive(double x) { return __double_as_longlong(x) > 0; }
// An integer key with the order of the (non-NaN) double x: its magnitude
// bits, negated for negative x (-0 and +0 both give 0, as they compare equal)
__device__ __forceinline__ long long order_key(double x) {
    const long long b = __double_as_longlong(x);
    const long long m = b & 0x7fffffffffffffffll;
    return b < 0 ? -m : m;
}
// x is NaN: all exponent bits set and a non-zero fraction
__device__ __forceinline__ bool is_nan_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) << 1) > 0xffe0000000000000ull;
}
__device__ __forceinline__ bool nn_less(float a, float b) { return a < b; }
__device__ __forceinline__ bool nn_less_eq(float a, float b) { return a <= b; }
__device__ __forceinline__ bool positive(float x) { return x > 0.f; }

// T = double in the FP64 path, float in the mixed-precision transfer mode.
// inv_size: 1/(4 lp) of the axis (the 3D z axis takes lp.y's, as the
// reference does); hinv: 1/(2 lp) of the axis, for the 3D gradient, which the
// reference forms as -xp/(2 lp) -- multiplying by the reciprocal differs from
// that quotient by rounding only and keeps divisions out of the candidate loop.
template <typename T, bool kThreeD, bool kGrad>
__device__ __forceinline__ void gimp_window(T xi, T lp, T inv_size, T hinv, T idx, Win<T> &w) {
    const T q1 = T(2) - lp, q2 = T(2) + lp;
    w.s = nn_less(fabs(xi - T(3)), q2) ? 1 : 0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const T gk = w.s ? T(2 * j - 1) : T(2 * j - 3);  // candidate at 2 (s + j) - 3
        const T dx = xi - gk;
        const T xp = fabs(dx);
        T S = T(0), dS = T(0);
        if (nn_less(xp, q2)) {
            T arg = T(0);
            if (nn_less(xp, lp)) {
                S = ((T(4) - lp) * lp - xp * xp) * inv_size;
            } else if (nn_less_eq(xp, q1)) {
                S = kThreeD ? T(0.5) * (T(2) - xp) : (T(2) - xp) / T(2);
            } else {
                arg = (q2 - xp) * inv_size;
                S = T(2) * lp * arg * arg;
            }
            if (kGrad) {
                T d;
                if (nn_less(xp, lp)) d = kThreeD ? -xp * hinv : -xp * inv_size * T(2);
                else if (nn_less_eq(xp, q1)) d = T(-0.5);
                else d = -arg;
                dS = (positive(dx) ? d : -d) * idx;
            }
        }
        w.S[j] = S;
        w.dS[j] = dS;
    }
}

// Quadratic B-spline (B2SPLINE) window: FourNodeIsoparam /
// EightNodeIsoparamBrick::SplineShapeFunction (Common/Elements/
// FourNodeIsoparam.cpp:217-293, NairnMPM/src/Elements/
// EightNodeIsoparamBrick.cpp:110-205) take the candidates within 3 half cells:
// the one at +3 exactly when xi > 0, else the one at -3 (zero at xi = 0).  The
// factor is (3 - d^2)/4 for |d| <= 1 and (3 - |d|)^2/8 beyond; idx = 1 / dx.
template <typename T, bool kGrad>
__device__ __forceinline__ void bspline_window(T xi, T idx, Win<T> &w) {
    w.s = xi > T(0) ? 1 : 0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const T d = xi - (T)(2 * (w.s + j) - 3);
        const T ad = fabs(d);
        T S = T(0), dS = T(0);
        if (ad < T(3)) {
            if (ad <= T(1)) {
                S = T(0.25) * (T(3) - d * d);
                if (kGrad) dS = -d * idx;
            } else {
                const T arg = T(3) - ad;
                S = T(0.125) * arg * arg;
                if (kGrad) dS = (d >= T(0) ? T(0.5) * (d - T(3)) : T(0.5) * (d + T(3))) * idx;
            }
        }
        w.S[j] = S;
        w.dS[j] = dS;
    }
}

// B2GIMP window: FourNodeIsoparam / EightNodeIsoparamBrick::
// BGimpShapeFunction (Common/Elements/FourNodeIsoparam.cpp:770-883) support
// 3 + lp half cells, so all four candidates per axis (at -3, -1, 1, 3, node
// offsets -1..2) may carry weight; those beyond the support get zero.  The
// gradient takes its sign from `sgn`: the particle's coordinate on the same
// axis, except that the reference's 3D z gradient compares the y coordinate.
// idx = 2 / dx.
template <typename T>
struct Win4 {
    T S[4], dS[4];
};

template <typename T, bool kThreeD, bool kGrad>
__device__ __forceinline__ void bgimp_window(T xi, T lp, T idx, T sgn, Win4<T> &w) {
    const T b1 = T(1) - lp, b2 = T(1) + lp, b3 = T(3) - lp, b4 = T(3) + lp;
    const T inv_size = T(1) / (T(48) * lp), oneTwelth = T(1) / T(12);
    const T lp2 = lp * lp;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const T gk = (T)(2 * j - 3);
        const T xp = fabs(xi - gk);
        T S = T(0), dS = T(0);
        if (xp < b4) {
            T arg = T(0);
            if (xp < b1) {
                S = (T(9) - lp2 - T(3) * xp * xp) * oneTwelth;
            } else if (xp < b2) {
                arg = xp - T(1);
                S = kThreeD ? (T(9) * lp2 * arg + T(3) * arg * arg * arg + T(3) * lp * (T(15) - xp * (T(6) + xp)) -
                               lp2 * lp) * inv_size
                            : (lp2 * (T(9) * arg - lp) + T(3) * arg * arg * arg + T(3) * lp * (T(15) - xp * (T(6) + xp))) *
                                  inv_size;
            } else if (xp <= b3) {
                arg = xp - T(3);
                S = (lp2 + T(3) * arg * arg) * T(0.5) * oneTwelth;
            } else {
                arg = T(3) + lp - xp;
                S = arg * arg * arg * inv_size;
            }
            if (kGrad) {
                T d;
                if (xp < b1) {
                    d = T(-0.5) * xp;
                } else if (xp < b2) {
                    arg = xp - T(1);
                    d = ((kThreeD ? T(3) * lp * lp : T(3) * lp2) + T(3) * arg * arg - T(2) * lp * (T(3) + xp)) * T(3) *
                        inv_size;
                } else if (xp <= b3) {
                    d = T(0.25) * (xp - T(3));
                } else {
                    arg = T(3) + lp - xp;
                    d = -arg * arg * T(3) * inv_size;
                }
                dS = (sgn > gk ? d : -d) * idx;
            }
        }
        w.S[j] = S;
        w.dS[j] = dS;
    }
}

// 1 / x.  When x is a power of two -- the usual cell sizes and particle
// semi-sizes -- the reciprocal is exact and is built from the exponent bits
// in the integer pipe, the same bits a division gives; otherwise the IEEE
// quotient.  A double division is a dozen instructions of the FP64 pipe.
__device__ __forceinline__ double recip(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long e = (b >> 52) & 0x7ffull;
    if ((b & 0x000fffffffffffffull) == 0ull && e >= 1ull && e <= 2045ull)
        return __longlong_as_double((long long)((b & 0x8000000000000000ull) | ((2046ull - e) << 52)));
    return 1. / x;
}
__device__ __forceinline__ float recip(float x) { return 1.f / x; }

// A shape-function weight of exactly zero (+0 or -0): a node outside the
// particle's support.  For doubles the test is on the bits, in the integer
// pipe: a double compare would take a slot of the FP64 pipe, which bounds the
// FP64 kernels on this GPU.
__device__ __forceinline__ bool zero_weight(double v) {
    return ((unsigned long long)__double_as_longlong(v) << 1) == 0ull;
}
__device__ __forceinline__ bool zero_weight(float v) { return v == 0.f; }

// FP64 value as an FP32 pair hi + lo (hi = nearest float, lo = nearest float of the rest)
__device__ __forceinline__ void split2(double v, float &hi, float &lo) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
}

// ---------------------------------------------------------------------------
// Constitutive updates (FP64).  du is the velocity gradient times the strain
// time step, row-major 3x3.
// ---------------------------------------------------------------------------

// Elastic::HypoIncrementDeformation (NairnMPM/src/Materials/ElasticMPM.cpp:392-403):
// F <- (I + du) F with F kept as strain ep and rotation wrot
// (MatPoint2D.cpp:309-366, MatPoint3D.cpp:320-376; Matrix3.cpp:312-351, 920-966).
__device__ __forceinline__ void hypo_increment_F_2d(const DevParticles &p, int i, const double du[9]) {
    const double a00 = 1. + du[0], a01 = du[1], a10 = du[3], a11 = 1. + du[4], a22 = 1. + du[8];
    const double exy = p.exy[i], wxy = p.wxy[i];
    const double b00 = 1. + p.exx[i], b01 = 0.5 * (exy - wxy), b10 = 0.5 * (exy + wxy), b11 = 1. + p.eyy[i],
                 b22 = 1. + p.ezz[i];
    const double f00 = a00 * b00 + a01 * b10;
    const double f01 = a00 * b01 + a01 * b11;
    const double f10 = a10 * b00 + a11 * b10;
    const double f11 = a10 * b01 + a11 * b11;
    const double f22 = a22 * b22;
    p.exx[i] = f00 - 1.;
    p.eyy[i] = f11 - 1.;
    p.ezz[i] = f22 - 1.;
    p.exy[i] = f10 + f01;
    p.wxy[i] = f10 - f01;
}

__device__ __forceinline__ void hypo_increment_F_3d(const DevParticles &p, int i, const double du[9]) {
    double b[9];
    const double exy = p.exy[i], exz = p.exz[i], eyz = p.eyz[i];
    const double wxy = p.wxy[i], wxz = p.wxz[i], wyz = p.wyz[i];
    b[0] = 1. + p.exx[i];
    b[4] = 1. + p.eyy[i];
    b[8] = 1. + p.ezz[i];
    b[1] = 0.5 * (exy - wxy);
    b[3] = 0.5 * (exy + wxy);
    b[2] = 0.5 * (exz - wxz);
    b[6] = 0.5 * (exz + wxz);
    b[5] = 0.5 * (eyz - wyz);
    b[7] = 0.5 * (eyz + wyz);
    double f[9];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const double a0 = du[3 * r] + (r == 0 ? 1. : 0.);
        const double a1 = du[3 * r + 1] + (r == 1 ? 1. : 0.);
        const double a2 = du[3 * r + 2] + (r == 2 ? 1. : 0.);
#pragma unroll
        for (int c = 0; c < 3; c++) f[3 * r + c] = a0 * b[c] + a1 * b[3 + c] + a2 * b[6 + c];
    }
    p.exx[i] = f[0] - 1.;
    p.eyy[i] = f[4] - 1.;
    p.ezz[i] = f[8] - 1.;
    p.exy[i] = f[3] + f[1];
    p.exz[i] = f[6] + f[2];
    p.eyz[i] = f[7] + f[5];
    p.wxy[i] = f[3] - f[1];
    p.wxz[i] = f[6] - f[2];
    p.wyz[i] = f[7] - f[5];
}

// IsotropicMat::SRConstitutiveLaw2D, plane strain without residual strains
// (NairnMPM/src/Materials/MoreIsotropicMat.cpp:185-279) and
// MaterialBase::Hypo2DCalculations (MaterialBaseMPM.cpp:1012-1020).
__device__ __forceinline__ void iso_law_2d(const DevMat &m, const DevParticles &p, int i, const double du[9]) {
    const double dvxx = du[0], dvyy = du[4];
    const double dgam = du[1] + du[3];
    const double dwrotxy = du[3] - du[1];
    const double s0xx = p.sxx[i], s0yy = p.syy[i], s0xy = p.sxy[i], s0zz = p.szz[i];
    const double c1 = m.c11 * dvxx + m.c12 * dvyy;
    const double c2 = m.c12 * dvxx + m.c22 * dvyy;
    const double c3 = m.c33 * dgam;
    const double dnorm = dwrotxy * s0xy;
    const double dshear = 0.5 * dwrotxy * (s0xx - s0yy);
    const double sxx = s0xx + (c1 - dnorm);
    const double syy = s0yy + (c2 + dnorm);
    const double sxy = s0xy + (c3 + dshear);
    const double szz = s0zz + (m.c41 * dvxx + m.c42 * dvyy);
    p.sxx[i] = sxx;
    p.syy[i] = syy;
    p.sxy[i] = sxy;
    p.szz[i] = szz;
    p.work[i] += 0.5 * ((s0xx + sxx) * dvxx + (s0yy + syy) * dvyy + (s0xy + sxy) * dgam);
}

// IsotropicMat::SRConstitutiveLaw3D (MoreIsotropicMat.cpp:286-348) with
// MaterialBase::Hypo3DCalculations (MaterialBaseMPM.cpp:1026-1047).
__device__ __forceinline__ void iso_law_3d(const DevMat &m, const DevParticles &p, int i, const double du[9]) {
    const double dvxx = du[0], dvyy = du[4], dvzz = du[8];
    const double dgamxy = du[1] + du[3], dgamxz = du[2] + du[6], dgamyz = du[5] + du[7];
    const double dwxy = du[3] - du[1], dwxz = du[6] - du[2], dwyz = du[7] - du[5];
    const double s0xx = p.sxx[i], s0yy = p.syy[i], s0zz = p.szz[i];
    const double s0yz = p.syz[i], s0xz = p.sxz[i], s0xy = p.sxy[i];
    const double d0 = m.C00 * dvxx + m.C01 * dvyy + m.C02 * dvzz;
    const double d1 = m.C01 * dvxx + m.C11 * dvyy + m.C12 * dvzz;
    const double d2 = m.C02 * dvxx + m.C12 * dvyy + m.C22 * dvzz;
    const double d3 = m.C33 * dgamyz, d4 = m.C44 * dgamxz, d5 = m.C55 * dgamxy;
    const double stxx = -dwxy * s0xy - dwxz * s0xz;
    const double styy = dwxy * s0xy - dwyz * s0yz;
    const double stzz = dwxz * s0xz + dwyz * s0yz;
    const double styz = 0.5 * (dwxy * s0xz + dwxz * s0xy + dwyz * (s0yy - s0zz));
    const double stxz = 0.5 * (-dwxy * s0yz + dwxz * (s0xx - s0zz) + dwyz * s0xy);
    const double stxy = 0.5 * (dwxy * (s0xx - s0yy) - dwxz * s0yz - dwyz * s0xz);
    const double sxx = s0xx + (d0 + stxx), syy = s0yy + (d1 + styy), szz = s0zz + (d2 + stzz);
    const double syz = s0yz + (d3 + styz), sxz = s0xz + (d4 + stxz), sxy = s0xy + (d5 + stxy);
    p.sxx[i] = sxx;
    p.syy[i] = syy;
    p.szz[i] = szz;
    p.syz[i] = syz;
    p.sxz[i] = sxz;
    p.sxy[i] = sxy;
    p.work[i] += 0.5 * ((s0xx + sxx) * dvxx + (s0yy + syy) * dvyy + (s0zz + szz) * dvzz + (s0yz + syz) * dgamyz +
                        (s0xz + sxz) * dgamxz + (s0xy + sxy) * dgamxy);
}

// IsoPlasticity::MPMConstitutiveLaw + PlasticityConstLaw, small rotation, no
// residual strains (NairnMPM/src/Materials/IsoPlasticity.cpp:128-451), with
// UpdatePressure (:462-492), IsotropicMat::GetMagnitudeSFromDev
// (MoreIsotropicMat.cpp:356-370) and LinearHardening's closed-form return
// (LinearHardening.cpp:124-145).  Stress on the particle is deviatoric; the
// pressure is carried separately.
template <bool kThreeD>
__device__ __forceinline__ void plastic_law(const DevMat &m, const DevParticles &p, int i, const double de[9]) {
    const double dexx = de[0], deyy = de[4], dezz = de[8];
    const double delV = dexx + deyy + dezz;
    const double dgxy = de[1] + de[3];
    const double dgxz = kThreeD ? de[2] + de[6] : 0.;
    const double dgyz = kThreeD ? de[5] + de[7] : 0.;
    // UpdatePressure
    const double Pfinal = p.pressure[i] + (-m.Kred * delV);
    p.pressure[i] = Pfinal;
    double work = p.work[i] + (-Pfinal * delV);   // work energy accumulates in the reference's order
    // rotate plastic strain and stress
    const double dwxy = de[3] - de[1];
    const double epxx = p.pxx[i], epyy = p.pyy[i], epzz = p.pzz[i], epxy = p.pxy[i];
    const double spxx = p.sxx[i], spyy = p.syy[i], spzz = p.szz[i], spxy = p.sxy[i];
    double epxz = 0., epyz = 0., spxz = 0., spyz = 0.;
    double s0xx, s0yy, s0zz, s0xy, s0xz = 0., s0yz = 0.;
    double qxx, qyy, qzz, qxy, qxz = 0., qyz = 0.;   // rotated plastic strain
    if (!kThreeD) {
        const double dnorm = 0.5 * dwxy * epxy;
        qxx = epxx - dnorm;
        qyy = epyy + dnorm;
        qzz = epzz;
        qxy = epxy + dwxy * (epxx - epyy);
        const double dn = dwxy * spxy;
        s0xx = spxx - dn;
        s0yy = spyy + dn;
        s0zz = spzz;
        s0xy = spxy + 0.5 * dwxy * (epxx - epyy);
    } else {
        epxz = p.pxz[i];
        epyz = p.pyz[i];
        spxz = p.sxz[i];
        spyz = p.syz[i];
        const double dwxz = de[6] - de[2], dwyz = de[7] - de[5];
        const double dxy = 0.5 * dwxy * epxy, dxz = 0.5 * dwxz * epxz, dyz = 0.5 * dwyz * epyz;
        qxx = epxx + (-dxy - dxz);
        qyy = epyy + (dxy - dyz);
        qzz = epzz + (dxz + dyz);
        qyz = epyz + (dwyz * (epyy - epzz) + 0.5 * (dwxz * epxy + dwxy * epxz));
        qxz = epxz + (dwxz * (epxx - epzz) + 0.5 * (dwyz * epxy - dwxy * epyz));
        qxy = epxy + (dwxy * (epxx - epyy) - 0.5 * (dwyz * epxz + dwxz * epyz));
        const double sxy = dwxy * spxy, sxz = dwxz * spxz, syz = dwyz * spyz;
        s0xx = spxx + (-sxy - sxz);
        s0yy = spyy + (sxy - syz);
        s0zz = spzz + (sxz + syz);
        s0yz = spyz + 0.5 * (dwyz * (spyy - spzz) + dwxz * spxy + dwxy * spxz);
        s0xz = spxz + 0.5 * (dwxz * (spxx - spzz) + dwyz * spxy - dwxy * spyz);
        s0xy = spxy + 0.5 * (dwxy * (spxx - spyy) - dwyz * spxz - dwxz * spyz);
    }
    // trial deviatoric stress
    const double third = delV * (1. / 3.);
    const double G = m.Gred;
    const double trxx = s0xx + 2. * G * (dexx - third);
    const double tryy = s0yy + 2. * G * (deyy - third);
    const double trzz = s0zz + 2. * G * (dezz - third);
    const double trxy = s0xy + G * dgxy;
    const double tryz = kThreeD ? s0yz + G * dgyz : 0.;
    const double trxz = kThreeD ? s0xz + G * dgxz : 0.;
    const double alpint = p.hist0[i];
    const double s2 = trxx * trxx + tryy * tryy + trzz * trzz;
    const double t2 = kThreeD ? trxy * trxy + trxz * trxz + tryz * tryz : trxy * trxy;
    const double smag = sqrt(s2 + t2 + t2);
    const double yld = alpint < m.alphaMax ? m.yldred + m.Epred * alpint : m.yldredMin;
    if (smag - kSqrtTwoThirds * yld < 0.) {
        p.sxx[i] = trxx;
        p.syy[i] = tryy;
        p.szz[i] = trzz;
        p.sxy[i] = trxy;
        p.pxx[i] = qxx;
        p.pyy[i] = qyy;
        p.pzz[i] = qzz;
        p.pxy[i] = qxy;
        if (kThreeD) {
            p.syz[i] = tryz;
            p.sxz[i] = trxz;
            p.pxz[i] = qxz;
            p.pyz[i] = qyz;
            work += trxx * dexx + tryy * deyy + trzz * dezz + tryz * dgyz + trxz * dgxz + trxy * dgxy;
        } else {
            work += trxx * dexx + tryy * deyy + trxy * dgxy;
        }
        p.work[i] = work;
        return;
    }
    // radial return
    double lam = (smag - kSqrtTwoThirds * (m.yldred + m.Epred * alpint)) / (2. * (G + m.Epred / 3.));
    if (alpint + kSqrtTwoThirds * lam > m.alphaMax) lam = (smag - kSqrtTwoThirds * m.yldredMin) / (2. * G);
    const double alpnew = alpint + kSqrtTwoThirds * lam;
    // lam * (tr / smag) with one FP64 division (the reference divides each
    // component; the products differ from it by rounding only)
    const double ls = lam / smag;
    const double dpxx = ls * trxx, dpyy = ls * tryy, dpzz = ls * trzz;
    const double dpxy = 2. * ls * trxy;
    const double dpxz = kThreeD ? 2. * ls * trxz : 0.;
    const double dpyz = kThreeD ? 2. * ls * tryz : 0.;
    const double sxx = trxx - 2. * G * dpxx, syy = tryy - 2. * G * dpyy, szz = trzz - 2. * G * dpzz;
    const double sxy = trxy - G * dpxy;
    p.sxx[i] = sxx;
    p.syy[i] = syy;
    p.szz[i] = szz;
    p.sxy[i] = sxy;
    p.pxx[i] = qxx + dpxx;
    p.pyy[i] = qyy + dpyy;
    p.pzz[i] = qzz + dpzz;
    p.pxy[i] = qxy + dpxy;
    double w = sxx * dexx + syy * deyy + sxy * dgxy;
    double pe = sxx * dpxx + syy * dpyy + szz * dpzz + sxy * dpxy;
    if (kThreeD) {
        const double syz = tryz - G * dpyz, sxz = trxz - G * dpxz;
        p.syz[i] = syz;
        p.sxz[i] = sxz;
        p.pxz[i] = qxz + dpxz;
        p.pyz[i] = qyz + dpyz;
        w += szz * dezz + syz * dgyz + sxz * dgxz;
        w += szz * dezz;   // the reference adds the zz term again when np != plane strain
        pe += sxz * dpxz + syz * dpyz;
    }
    p.work[i] = work + w;
    const double qdalpha = lam * kSqrtTwoThirds * fmax(m.Epred * alpnew, m.yldredMin - m.yldred);
    p.plast[i] += pe - qdalpha;
    p.hist0[i] = alpnew;
}


// ---------------------------------------------------------------------------
// Neohookean (type 28)
// ---------------------------------------------------------------------------

// Matrix3::Exponential (Common/System/Matrix3.cpp:312-364): dF = exp(du) with
// kmax terms; 2D uses the 2x2 Cayley-Hamilton recursion with zz separate, 3D
// takes 1 or 2 terms.  Row-major 3x3.
template <bool kThreeD>
__device__ __forceinline__ void exp_increment(const double du[9], int kmax, double dF[9]) {
    if (!kThreeD) {
        dF[2] = dF[5] = dF[6] = dF[7] = 0.;
        if (kmax == 1) {
            dF[0] = 1. + du[0];
            dF[1] = du[1];
            dF[3] = du[3];
            dF[4] = 1. + du[4];
            dF[8] = 1. + du[8];
            return;
        }
        const double c0 = du[1] * du[3] - du[0] * du[4];
        const double c1 = du[0] + du[4];
        double beta0 = 0., beta1 = 1., alpha0 = 1., alpha1 = 1.;
        double betaz = du[8], ezz = 1. + betaz;
        for (int k = 2; k <= kmax; k++) {
            const double factor = 1 / (double)k;
            const double temp = beta1;
            beta1 = factor * (c1 * temp + beta0);
            beta0 = factor * c0 * temp;
            betaz *= factor * du[8];
            alpha0 += beta0;
            alpha1 += beta1;
            ezz += betaz;
        }
        dF[0] = alpha0 + alpha1 * du[0];
        dF[1] = alpha1 * du[1];
        dF[3] = alpha1 * du[3];
        dF[4] = alpha0 + alpha1 * du[4];
        dF[8] = ezz;
        return;
    }
    if (kmax == 1) {
#pragma unroll
        for (int k = 0; k < 9; k++) dF[k] = du[k] + (k % 4 == 0 ? 1. : 0.);
        return;
    }
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double m2 = 0.;
#pragma unroll
            for (int k = 0; k < 3; k++) m2 += du[3 * r + k] * du[3 * k + c];
            dF[3 * r + c] = r == c ? 1. + du[3 * r + c] + 0.5 * m2 : du[3 * r + c] + 0.5 * m2;
        }
}

// a * b as Matrix3::operator*= forms it (Matrix3.cpp:920-966)
template <bool kThreeD>
__device__ __forceinline__ void mat_mul(const double a[9], const double b[9], double o[9]) {
    if constexpr (!kThreeD) {
        o[0] = a[0] * b[0] + a[1] * b[3];
        o[1] = a[0] * b[1] + a[1] * b[4];
        o[3] = a[3] * b[0] + a[4] * b[3];
        o[4] = a[3] * b[1] + a[4] * b[4];
        o[2] = o[5] = o[6] = o[7] = 0.;
        o[8] = a[8] * b[8];
    } else {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double v = 0.;
#pragma unroll
                for (int k = 0; k < 3; k++) v += a[3 * i + k] * b[3 * k + j];
                o[3 * i + j] = v;
            }
    }
}

// HyperElastic::GetVolumetricTerms (NairnMPM/src/Materials/HyperElastic.cpp:171-204)
__device__ __forceinline__ double volumetric_terms(int uj, double J, double Kred) {
    if (uj == 1) return Kred * (J - 1.);
    if (uj == 2) return Kred * log(J) / J;
    return 0.5 * Kred * (J - 1. / J);
}

// Neohookean::MPMConstitutiveLaw without residual strains, thermal terms or
// artificial viscosity (NairnMPM/src/Materials/Neohookean.cpp:177-331) and
// HyperElastic::IncrementDeformation (HyperElastic.cpp:104-139).  F (ep/wrot)
// and the left Cauchy-Green tensor B (plastic-strain columns) are pushed
// forward by dF = exp(du); J and Jres are history doubles 0 and 1; the stress
// is the deviatoric Kirchhoff stress per initial density, pressure separate.
template <bool kThreeD>
__device__ __forceinline__ void neo_law(const DevMat &m, const DevParticles &p, int i, const double du[9]) {
    double dF[9], pF[9], F[9], B[9], dFB[9];
    exp_increment<kThreeD>(du, m.kterms, dF);
    pF[0] = 1. + p.exx[i];
    pF[1] = 0.5 * (p.exy[i] - p.wxy[i]);
    pF[3] = 0.5 * (p.exy[i] + p.wxy[i]);
    pF[4] = 1. + p.eyy[i];
    pF[8] = 1. + p.ezz[i];
    B[0] = p.pxx[i];
    B[1] = B[3] = p.pxy[i];
    B[4] = p.pyy[i];
    B[8] = p.pzz[i];
    if (kThreeD) {
        pF[2] = 0.5 * (p.exz[i] - p.wxz[i]);
        pF[6] = 0.5 * (p.exz[i] + p.wxz[i]);
        pF[5] = 0.5 * (p.eyz[i] - p.wyz[i]);
        pF[7] = 0.5 * (p.eyz[i] + p.wyz[i]);
        B[2] = B[6] = p.pxz[i];
        B[5] = B[7] = p.pyz[i];
    } else {
        pF[2] = pF[5] = pF[6] = pF[7] = 0.;
        B[2] = B[5] = B[6] = B[7] = 0.;
    }
    mat_mul<kThreeD>(dF, pF, F);
    p.exx[i] = F[0] - 1.;
    p.eyy[i] = F[4] - 1.;
    p.ezz[i] = F[8] - 1.;
    p.exy[i] = F[3] + F[1];
    p.wxy[i] = F[3] - F[1];
    if (kThreeD) {
        p.exz[i] = F[6] + F[2];
        p.eyz[i] = F[7] + F[5];
        p.wxz[i] = F[6] - F[2];
        p.wyz[i] = F[7] - F[5];
    }
    mat_mul<kThreeD>(dF, B, dFB);
    // B = dF.Bold.dF^T, component sums in the reference's order
    const double Bxx = dFB[0] * dF[0] + dFB[1] * dF[1] + dFB[2] * dF[2];
    const double Bxy = dFB[0] * dF[3] + dFB[1] * dF[4] + dFB[2] * dF[5];
    const double Byy = dFB[3] * dF[3] + dFB[4] * dF[4] + dFB[5] * dF[5];
    const double Bzz = dFB[6] * dF[6] + dFB[7] * dF[7] + dFB[8] * dF[8];
    double Bxz = 0., Byz = 0.;
    p.pxx[i] = Bxx;
    p.pxy[i] = Bxy;
    p.pyy[i] = Byy;
    p.pzz[i] = Bzz;
    if (kThreeD) {
        Bxz = dFB[0] * dF[6] + dFB[1] * dF[7] + dFB[2] * dF[8];
        Byz = dFB[3] * dF[6] + dFB[4] * dF[7] + dFB[5] * dF[8];
        p.pxz[i] = Bxz;
        p.pyz[i] = Byz;
    }
    // Matrix3::determinant (Matrix3.cpp:1195-1202)
    const double detDf = kThreeD ? dF[0] * (dF[4] * dF[8] - dF[7] * dF[5]) - dF[3] * (dF[1] * dF[8] - dF[7] * dF[2]) +
                                       dF[6] * (dF[1] * dF[5] - dF[4] * dF[2])
                                 : dF[8] * (dF[0] * dF[4] - dF[3] * dF[1]);
    // no residual strains: Jres stays 1, so its cube root and square are 1
    const double Jres = p.hist1[i];
    const double resStretch = Jres == 1. ? 1. : cbrt(Jres);
    const double Jres23 = resStretch * resStretch;
    const double J = detDf * p.hist0[i];
    p.hist0[i] = J;
    const double st0xx = p.sxx[i], st0yy = p.syy[i], st0zz = p.szz[i], st0xy = p.sxy[i];
    const double st0xz = kThreeD ? p.sxz[i] : 0., st0yz = kThreeD ? p.syz[i] : 0.;
    const double Jeff = J / Jres;
    const double p0 = p.pressure[i];
    const double trB = Bxx + Byy + Bzz;
    const double Pterm = J * volumetric_terms(m.uj, Jeff, m.Lamesp) + Jres * m.Gsp * (trB / (3. * Jres23) - 1.);
    const double delV = 1. - 1. / detDf;
    const double Pfinal = -Pterm + 0.;
    p.pressure[i] = Pfinal;
    const double dilEnergy = -(0.5 * (p0 + Pfinal)) * delV;
    const double GJeff = resStretch * m.Gsp;
    const double I1third = trB / 3.;
    const double sxx = GJeff * (Bxx - I1third), syy = GJeff * (Byy - I1third), szz = GJeff * (Bzz - I1third);
    const double sxy = GJeff * Bxy;
    p.sxx[i] = sxx;
    p.syy[i] = syy;
    p.szz[i] = szz;
    p.sxy[i] = sxy;
    double shear = 0.5 * ((sxx + st0xx) * du[0] + (syy + st0yy) * du[4] + (szz + st0zz) * du[8] +
                          (sxy + st0xy) * (du[1] + du[3]));
    if (kThreeD) {
        const double sxz = GJeff * Bxz, syz = GJeff * Byz;
        p.sxz[i] = sxz;
        p.syz[i] = syz;
        shear += 0.5 * ((sxz + st0xz) * (du[2] + du[6]) + (syz + st0yz) * (du[5] + du[7]));
    }
    p.work[i] += dilEnergy + shear;
}

}  // namespace nmg
