/*
 * mpm_oracle.c -- CPU restatement of NairnMPM's explicit time step (FP64).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path.  Not part of the
 * product; nothing outside tests/, the smoke check and the bench CPU baseline
 * uses it.
 *
 * Each function cites the reference function it restates.  Paths are relative
 * to the nairn-mpm-fea source tree.  With nthreads == 1 the particle loops run
 * in the reference's single-patch order: P2G and grid-force loops walk the
 * patch's particle list, which GridPatch::AddParticle builds by prepending
 * (NairnMPM/src/Patches/GridPatch.cpp:256-278), i.e. in decreasing particle
 * index; the strain and particle updates walk mpm[] forward.
 */
#include "mpm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQRT_TWOTHIRDS 0.8164965809277260   /* sqrt(2/3) */

static char g_err[512];
const char *mpm_oracle_last_error(void) { return g_err; }
static int fail(int code, const char *msg) {
    snprintf(g_err, sizeof(g_err), "%s", msg);
    return code;
}

/* ------------------------------------------------------------------------ */
/* Materials: derived constants (VerifyAndLoadProperties of each class)       */
/* ------------------------------------------------------------------------ */
typedef struct {
    int type, field;
    double rho;                 /* g/mm^3                                      */
    double E, nu, G;            /* Pa                                          */
    double C2[6][6];            /* 2D specific stiffness, Elastic::FillUnrotatedElasticProperties */
    double C3[6][6];            /* 3D specific stiffness                       */
    double Gred, Kred;          /* IsoPlasticity specific moduli               */
    double yldred, Epred, alphaMax, yldredMin;  /* LinearHardening             */
    double Gpa, Kpa;            /* Neohookean moduli (Pa)                      */
    double Gsp, Lamesp, Ksp;    /* Neohookean specific moduli (pr.Gsp, ...)    */
    int uj;                     /* Neohookean UofJOption                       */
} OMat;

/* Elastic::SetAnalysisProps (Common/Materials/Elastic.cpp:194-330) for an
 * isotropic material (e1=e2=e3=E, v12=v13=v23=nu, g=G), then
 * FillUnrotatedElasticProperties (Elastic.cpp:43-160) with makeSpecific. */
static void iso_constants(OMat *m, int np) {
    double e1 = m->E, e2 = m->E, e3 = m->E;
    double v12 = m->nu, v13 = m->nu, v23 = m->nu;
    double g12 = m->G, g13 = m->G, g23 = m->G;
    double v32 = v23 * e3 / e2, v31 = v13 * e3 / e1, v21 = v12 * e2 / e1;
    double xx, C11, C12, C13, C22, C23, C33, C44, C55, C66;
    memset(m->C2, 0, sizeof(m->C2));
    memset(m->C3, 0, sizeof(m->C3));
    if (np == MPMGPU_THREED) {
        xx = 1. - v13 * v31 - v23 * v32 - v12 * v21 - 2. * v13 * v32 * v21;
        C11 = e1 * (1. - v23 * v32) / xx;
        C12 = e2 * (v12 + v13 * v32) / xx;
        C13 = e3 * (v13 + v12 * v23) / xx;
        C22 = e2 * (1. - v13 * v31) / xx;
        C23 = e3 * (v23 + v21 * v13) / xx;
        C33 = e3 * (1. - v21 * v12) / xx;
        C66 = g12; C44 = g23; C55 = g13;
        double rrho = 1. / m->rho;
        m->C3[0][0] = C11 * rrho; m->C3[0][1] = C12 * rrho; m->C3[0][2] = C13 * rrho;
        m->C3[1][0] = m->C3[0][1]; m->C3[1][1] = C22 * rrho; m->C3[1][2] = C23 * rrho;
        m->C3[2][0] = m->C3[0][2]; m->C3[2][1] = m->C3[1][2]; m->C3[2][2] = C33 * rrho;
        m->C3[3][3] = C44 * rrho; m->C3[4][4] = C55 * rrho; m->C3[5][5] = C66 * rrho;
    } else {
        /* plane strain */
        xx = 1. - v13 * v31 - v23 * v32 - v12 * v21 - 2. * v12 * v23 * v31;
        C11 = e1 * (1. - v23 * v32) / xx;
        C12 = e2 * (v12 + v13 * v32) / xx;
        C22 = e2 * (1. - v13 * v31) / xx;
        C66 = g12;
        C13 = e3 * (v13 + v12 * v23) / xx;
        C23 = e3 * (v23 + v21 * v13) / xx;
        C33 = e3 * (1. - v21 * v12) / xx;
        double rrho = 1. / m->rho;
        m->C2[1][1] = C11 * rrho; m->C2[1][2] = C12 * rrho; m->C2[2][2] = C22 * rrho;
        m->C2[3][3] = C66 * rrho;
        m->C2[4][1] = C13 * rrho; m->C2[4][2] = C23 * rrho; m->C2[4][4] = C33 * rrho;
        m->C2[2][1] = m->C2[1][2];
    }
    /* IsoPlasticity::VerifyAndLoadProperties (IsoPlasticity.cpp:58-65) uses the
     * 3D/plane-strain C66 and C33, identical expressions in both branches */
    m->Gred = C66 / m->rho;
    m->Kred = C33 / m->rho - 4. * m->Gred / 3.;
}

static int load_materials(const MpmGpuMaterial *in, int nmat, int np, OMat *out) {
    for (int i = 0; i < nmat; i++) {
        OMat *m = &out[i];
        memset(m, 0, sizeof(*m));
        m->type = in[i].type;
        m->field = in[i].field;
        m->rho = in[i].rho * 0.001;              /* MaterialBaseMPM.cpp:58 */
        if (m->type == MPMGPU_MAT_ISOTROPIC || m->type == MPMGPU_MAT_ISOPLASTICITY) {
            m->E = in[i].E * 1.e6;               /* IsotropicMat.cpp:40 */
            m->nu = in[i].nu;
            m->G = m->E / (2. * (1. + m->nu));   /* IsotropicMat.cpp:96 */
            iso_constants(m, np);
            if (m->type == MPMGPU_MAT_ISOPLASTICITY) {
                /* HardeningLawBase::VerifyAndLoadProperties, LinearHardening.cpp:45-58 */
                double yield = in[i].yield * 1.e6, Ep = in[i].Ep * 1.e6, beta;
                m->yldred = yield / m->rho;
                m->yldredMin = 0. / m->rho;
                if (Ep >= 0.) beta = Ep / yield;
                else beta = 0.;
                m->Epred = m->yldred * beta;
                m->alphaMax = 1.e50;
                if (beta < 0.) m->alphaMax = ((m->yldredMin / m->yldred) - 1.) / beta;
            }
        } else if (m->type == MPMGPU_MAT_NEOHOOKEAN) {
            /* Neohookean::VerifyAndLoadProperties, G and K branch (Neohookean.cpp:88-141);
             * G and K inputs are MPa (Neohookean.cpp:67, HyperElastic.cpp:33) */
            if (in[i].UJOption < 0 || in[i].UJOption > 2)
                return fail(MPMGPU_ERR_INVALID, "oracle: Neohookean UJOption must be 0, 1 or 2");
            m->Gpa = in[i].G * 1.e6;
            m->Kpa = in[i].K * 1.e6;
            double Lame = m->Kpa - 2. * m->Gpa / 3.;
            m->Gsp = m->Gpa / m->rho;
            m->Lamesp = Lame / m->rho;
            m->Ksp = m->Lamesp + 2. * m->Gsp / 3.;
            m->uj = in[i].UJOption;
        } else if (m->type == MPMGPU_MAT_RIGID_CONTACT) {
            /* RigidMaterial (RigidMaterial.cpp:26-60): rho = 1, so a particle's
             * mass is its volume; no mechanical properties */
            m->rho = 1.;
        } else {
            return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: material type not implemented");
        }
    }
    return MPMGPU_OK;
}

/* IsotropicMat::WaveSpeed (MoreIsotropicMat.cpp:388-395);
 * Neohookean::WaveSpeed (Neohookean.cpp:359) */
static double wave_speed(const OMat *m) {
    if (m->type == MPMGPU_MAT_NEOHOOKEAN) return sqrt((m->Kpa + 4. * m->Gpa / 3.) / m->rho);
    return sqrt(2. * m->G * (1. - m->nu) / (m->rho * (1. - 2. * m->nu)));
}

double mpm_oracle_cfl_timestep(const MpmGpuGrid *grid, const MpmGpuMaterial *mats, int nmat,
                               const int32_t *mat_used, double cfl) {
    OMat *om = (OMat *)calloc((size_t)nmat, sizeof(OMat));
    int np = grid->dim == 3 ? MPMGPU_THREED : MPMGPU_PLANE_STRAIN;
    if (load_materials(mats, nmat, np, om) != MPMGPU_OK) {
        free(om);
        return -1.;
    }
    double dcell = grid->dx;
    if (grid->dy < dcell) dcell = grid->dy;
    if (grid->dim == 3 && grid->dz < dcell) dcell = grid->dz;
    double tmin = 1.e30;
    for (int i = 0; i < nmat; i++) {
        if (mat_used && !mat_used[i]) continue;
        if (om[i].type == MPMGPU_MAT_RIGID_CONTACT) continue;  /* rigid materials set no time step */
        double tst = dcell / wave_speed(&om[i]);
        if (tst < tmin) tmin = tst;
    }
    free(om);
    return cfl * tmin;
}

/* ------------------------------------------------------------------------ */
/* Grid                                                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
    int dim, nx, ny, nz;
    long xplane, yplane, zplane, nnodes, nelems;
    const double *xn, *yn, *zn;
    double xmin, ymin, zmin, gx, gy, gz;
} OGrid;

typedef struct {            /* material velocity fields: field f of node n at f*(nnodes+1)+n */
    double *mass, *px, *py, *pz, *fx, *fy, *fz, *vx, *vy, *vz, *cx, *cy, *cz;
    int *npts;
    /* multimaterial contact terms (ContactTerms): volume, displacement and
     * volume gradient extrapolations */
    double *vol, *ux, *uy, *uz, *gvx, *gvy, *gvz;
} OField;

static void elem_extent(const OGrid *g, int e, double *x0, double *x1, double *y0, double *y1,
                        double *z0, double *z1) {
    int col = e % g->nx, row = (e / g->nx) % g->ny, zr = g->dim == 3 ? e / (g->nx * g->ny) : 0;
    *x0 = g->xn[col]; *x1 = g->xn[col + 1];
    *y0 = g->yn[row]; *y1 = g->yn[row + 1];
    if (g->dim == 3) { *z0 = g->zn[zr]; *z1 = g->zn[zr + 1]; }
    else { *z0 = 0.; *z1 = 0.; }
}

static long elem_node0(const OGrid *g, int e) {
    int col = e % g->nx, row = (e / g->nx) % g->ny, zr = g->dim == 3 ? e / (g->nx * g->ny) : 0;
    return (long)zr * g->zplane + (long)row * g->yplane + col + 1;
}

/* MeshInfo::EdgeElement2D/3D (MeshInfo.cpp:171-199), num is 1-based */
static int edge_element(const OGrid *g, int num) {
    int horiz = g->nx, vert = g->ny;
    if (g->dim == 2) {
        long total = (long)horiz * vert;
        if (num <= horiz || num > total - horiz) return 1;
        int col = num % horiz;
        return col <= 1;
    }
    long total = (long)horiz * vert * g->nz;
    if (num <= horiz * vert || num > total - (long)horiz * vert) return 1;
    if (num % horiz <= 1) return 1;
    int xz = num % (horiz * vert);
    return xz <= horiz || xz > horiz * (vert - 1);
}

/* ------------------------------------------------------------------------ */
/* Shape functions                                                           */
/* ------------------------------------------------------------------------ */
/* candidate tables, FourNodeIsoparam.cpp:27-30 and EightNodeIsoparamBrick.cpp */
static const double gxii[16] = {-1., 1., 1., -1., -3., -1., 1., 3., 3., 3., 3., 1., -1., -3., -3., -3.};
static const double geti[16] = {-1., -1., 1., 1., -3., -3., -3., -3., -1., 1., 3., 3., 3., 3., 1., -1.};
static const int xoff2[16] = {0, 1, 1, 0, -1, 0, 1, 2, 2, 2, 2, 1, 0, -1, -1, -1};
static const int yoff2[16] = {0, 0, 1, 1, -1, -1, -1, -1, 0, 1, 2, 2, 2, 2, 1, 0};
static const double xii2[4] = {-1., 1., 1., -1.};
static const double eti2[4] = {-1., -1., 1., 1.};
static const double xii3[8] = {-1., 1., 1., -1., -1., 1., 1., -1.};
static const double eti3[8] = {-1., -1., 1., 1., -1., -1., 1., 1.};
static const double zti3[8] = {-1., -1., -1., -1., 1., 1., 1., 1.};
static const int x3off[64] = {0, 1, 1, 0, 0, 1, 1, 0, -1, 0, 1, 2, 2, 2, 2, 1, 0, -1, -1, -1, -1, 0,
                              1, 2, 2, 2, 2, 1, 0, -1, -1, -1, 0, 1, 1, 0, -1, 0, 1, 2, 2, 2, 2, 1,
                              0, -1, -1, -1, 0, 1, 1, 0, -1, 0, 1, 2, 2, 2, 2, 1, 0, -1, -1, -1};
static const int y3off[64] = {0, 0, 1, 1, 0, 0, 1, 1, -1, -1, -1, -1, 0, 1, 2, 2, 2, 2, 1, 0, -1, -1,
                              -1, -1, 0, 1, 2, 2, 2, 2, 1, 0, 0, 0, 1, 1, -1, -1, -1, -1, 0, 1, 2, 2,
                              2, 2, 1, 0, 0, 0, 1, 1, -1, -1, -1, -1, 0, 1, 2, 2, 2, 2, 1, 0};
static const int z3off[64] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1,
                              1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1,
                              -1, -1, -1, -1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2};

typedef struct {
    int n;
    long nds[64];
    double fn[64], dx[64], dy[64], dz[64];
} OShape;

/* FourNodeIsoparam::GetXiPos / EightNodeIsoparamBrick::GetXiPos for rectangular
 * elements (FourNodeIsoparam.cpp:351-366, EightNodeIsoparamBrick.cpp:276-281) */
static void xi_pos(const OGrid *g, int e, double x, double y, double z, double *xi) {
    double x0, x1, y0, y1, z0, z1;
    elem_extent(g, e, &x0, &x1, &y0, &y1, &z0, &z1);
    xi[0] = (2. * x - x0 - x1) / (x1 - x0);
    xi[1] = (2. * y - y0 - y1) / (y1 - y0);
    xi[2] = g->dim == 3 ? (2. * z - z0 - z1) / (z1 - z0) : 0.;
}

/* ElementBase::GetShapeFunctions / GetShapeGradients dispatch
 * (NairnMPM/src/Elements/MoreMPMElementBase.cpp:120-284) for POINT_GIMP and
 * UNIFORM_GIMP. */
static void shape_eval(const OGrid *g, int shape, int e, const double *xi, const double *lp,
                       int grad, OShape *s) {
    double x0, x1, y0, y1, z0, z1;
    elem_extent(g, e, &x0, &x1, &y0, &y1, &z0, &z1);
    long n0 = elem_node0(g, e);
    double DX = x1 - x0, DY = y1 - y0, DZ = z1 - z0;
    if (shape == MPMGPU_SHAPE_LINEAR) {
        if (g->dim == 2) {
            /* FourNodeIsoparam::ShapeFunction (6 args), FourNodeIsoparam.cpp:189-212 */
            long nodes[4] = {n0, n0 + 1, n0 + g->yplane + 1, n0 + g->yplane};
            for (int i = 0; i < 4; i++) {
                double t1 = (1. + xii2[i] * xi[0]);
                double t2 = (1. + eti2[i] * xi[1]);
                s->nds[i] = nodes[i];
                s->fn[i] = 0.25 * t1 * t2;
                if (grad) {
                    s->dx[i] = 0.5 * xii2[i] * t2 / DX;
                    s->dy[i] = 0.5 * eti2[i] * t1 / DY;
                    s->dz[i] = 0.;
                }
            }
            s->n = 4;
        } else {
            /* EightNodeIsoparamBrick::ShapeFunction (6 args), EightNodeIsoparamBrick.cpp:90-104 */
            long nodes[8] = {n0, n0 + 1, n0 + 1 + g->yplane, n0 + g->yplane,
                             n0 + g->zplane, n0 + 1 + g->zplane, n0 + 1 + g->yplane + g->zplane,
                             n0 + g->yplane + g->zplane};
            for (int i = 0; i < 8; i++) {
                double t1 = (1. + xii3[i] * xi[0]);
                double t2 = (1. + eti3[i] * xi[1]);
                double t3 = (1. + zti3[i] * xi[2]);
                s->nds[i] = nodes[i];
                s->fn[i] = 0.125 * t1 * t2 * t3;
                if (grad) {
                    s->dx[i] = 0.25 * xii3[i] * t2 * t3 / DX;
                    s->dy[i] = 0.25 * eti3[i] * t1 * t3 / DY;
                    s->dz[i] = 0.25 * zti3[i] * t1 * t2 / DZ;
                }
            }
            s->n = 8;
        }
        return;
    }
    if (shape == MPMGPU_SHAPE_BGIMP) {
        /* B2GIMP: FourNodeIsoparam::BGimpShapeFunction (Common/Elements/
         * FourNodeIsoparam.cpp:770-883) and EightNodeIsoparamBrick::
         * BGimpShapeFunction: the quadratic B-spline convolved with the
         * particle domain, every candidate within 3 + lp half cells.  The 3D
         * gradient takes its z sign from the y coordinate, as the reference does. */
        int three = g->dim == 3, i = 0;
        double inv_d[3] = {0., 0., 0.};
        if (grad) {
            inv_d[0] = 2.0 / DX;
            inv_d[1] = 2.0 / DY;
            inv_d[2] = 2.0 / DZ;
        }
        for (int id = 0; id < (three ? 64 : 16); id++) {
            double gc[3] = {three ? (double)(2 * x3off[id] - 1) : gxii[id],
                            three ? (double)(2 * y3off[id] - 1) : geti[id],
                            three ? (double)(2 * z3off[id] - 1) : 0.};
            double S[3] = {1., 1., 1.}, dS[3] = {0., 0., 0.};
            int out = 0;
            for (int a = 0; a < (three ? 3 : 2) && !out; a++) {
                double l = lp[a], b1 = 1. - l, b2 = 1. + l, b3 = 3. - l, b4 = 3. + l;
                double inv_size = 1. / (48. * l), oneTwelth = 1. / 12.;
                double xp = fabs(xi[a] - gc[a]), arg;
                if (xp >= b4) { out = 1; break; }
                if (xp < b1) S[a] = (9. - l * l - 3. * xp * xp) * oneTwelth;
                else if (xp < b2) {
                    arg = xp - 1.;
                    if (three) {
                        double lp2 = l * l, lp3 = lp2 * l;
                        S[a] = (9. * lp2 * arg + 3. * arg * arg * arg + 3. * l * (15. - xp * (6. + xp)) - lp3) * inv_size;
                    } else {
                        double lp2 = l * l;
                        S[a] = (lp2 * (9. * arg - l) + 3. * arg * arg * arg + 3. * l * (15. - xp * (6. + xp))) * inv_size;
                    }
                } else if (xp <= b3) {
                    arg = xp - 3.;
                    S[a] = (l * l + 3. * arg * arg) * 0.5 * oneTwelth;
                } else {
                    arg = 3. + l - xp;
                    S[a] = arg * arg * arg * inv_size;
                }
                if (grad) {
                    if (xp < b1) dS[a] = -0.5 * xp;
                    else if (xp < b2) {
                        arg = xp - 1.;
                        double l3 = three ? 3 * l * l : 3 * (l * l);  /* 3D: (3 lp) lp; 2D: 3 (lp lp) */
                        dS[a] = (l3 + 3. * arg * arg - 2. * l * (3. + xp)) * 3. * inv_size;
                    }
                    else if (xp <= b3) dS[a] = 0.25 * (xp - 3.);
                    else { arg = 3. + l - xp; dS[a] = -arg * arg * 3. * inv_size; }
                }
            }
            if (out) continue;
            if (three) {
                s->fn[i] = S[0] * S[1] * S[2];
                if (grad) {
                    double xsign = xi[0] > gc[0] ? 1. : -1., ysign = xi[1] > gc[1] ? 1. : -1.;
                    double zsign = xi[1] > gc[2] ? 1. : -1.;
                    s->dx[i] = xsign * dS[0] * S[1] * S[2] * inv_d[0];
                    s->dy[i] = ysign * S[0] * dS[1] * S[2] * inv_d[1];
                    s->dz[i] = zsign * S[0] * S[1] * dS[2] * inv_d[2];
                }
                s->nds[i] = n0 + x3off[id] * g->xplane + y3off[id] * g->yplane + z3off[id] * g->zplane;
            } else {
                s->fn[i] = S[0] * S[1];
                if (grad) {
                    double xsign = xi[0] > gc[0] ? 1. : -1., ysign = xi[1] > gc[1] ? 1. : -1.;
                    s->dx[i] = xsign * dS[0] * S[1] * inv_d[0];
                    s->dy[i] = ysign * S[0] * dS[1] * inv_d[1];
                    s->dz[i] = 0.;
                }
                s->nds[i] = n0 + xoff2[id] * g->xplane + yoff2[id] * g->yplane;
            }
            i++;
        }
        s->n = i;
        return;
    }
    if (shape == MPMGPU_SHAPE_BSPLINE) {
        /* B2SPLINE: FourNodeIsoparam::SplineShapeFunction (Common/Elements/
         * FourNodeIsoparam.cpp:217-293) and EightNodeIsoparamBrick::
         * SplineShapeFunction (EightNodeIsoparamBrick.cpp:110-205): the
         * candidates of the 4x4(x4) block around the element within 3 half
         * cells, quadratic B-spline factors per axis */
        double inv_dx = 0., inv_dy = 0., inv_dz = 0.;
        if (grad) {
            inv_dx = 1. / DX;
            inv_dy = 1. / DY;
            inv_dz = 1. / DZ;
        }
        int three = g->dim == 3, i = 0;
        for (int id = 0; id < (three ? 64 : 16); id++) {
            double gx = three ? (double)(2 * x3off[id] - 1) : gxii[id];
            double gy = three ? (double)(2 * y3off[id] - 1) : geti[id];
            double etai = xi[0] - gx, t1 = fabs(etai);
            if (t1 >= 3.) continue;
            double netai = xi[1] - gy, t2 = fabs(netai);
            if (t2 >= 3.) continue;
            double zetai = 0., t3 = 0.;
            if (three) {
                zetai = xi[2] - (double)(2 * z3off[id] - 1);
                t3 = fabs(zetai);
                if (t3 >= 3.) continue;
            }
            double sx, sy, sz = 1., arg;
            if (t1 <= 1.0) sx = 0.25 * (3. - etai * etai);
            else { arg = 3. - t1; sx = 0.125 * arg * arg; }
            if (t2 <= 1.0) sy = 0.25 * (3. - netai * netai);
            else { arg = 3. - t2; sy = 0.125 * arg * arg; }
            if (three) {
                if (t3 <= 1.0) sz = 0.25 * (3. - zetai * zetai);
                else { arg = 3. - t3; sz = 0.125 * arg * arg; }
            }
            s->fn[i] = three ? sx * sy * sz : sx * sy;
            if (grad) {
                double fx = t1 <= 1.0 ? -etai : (etai >= 0. ? 0.5 * (etai - 3) : 0.5 * (etai + 3));
                double fy = t2 <= 1.0 ? -netai : (netai >= 0. ? 0.5 * (netai - 3) : 0.5 * (netai + 3));
                if (three) {
                    double fz = t3 <= 1.0 ? -zetai : (zetai >= 0. ? 0.5 * (zetai - 3) : 0.5 * (zetai + 3));
                    s->dx[i] = fx * sy * sz * inv_dx;
                    s->dy[i] = fy * sx * sz * inv_dy;
                    s->dz[i] = fz * sx * sy * inv_dz;
                } else {
                    s->dx[i] = fx * sy * inv_dx;
                    s->dy[i] = fy * sx * inv_dy;
                    s->dz[i] = 0.;
                }
            }
            s->nds[i] = three ? n0 + x3off[id] * g->xplane + y3off[id] * g->yplane + z3off[id] * g->zplane
                              : n0 + xoff2[id] * g->xplane + yoff2[id] * g->yplane;
            i++;
        }
        s->n = i;
        return;
    }
    /* UNIFORM_GIMP */
    if (g->dim == 2) {
        /* FourNodeIsoparam::GimpShapeFunction, FourNodeIsoparam.cpp:431-519 */
        double q1x = 2. - lp[0], q2x = 2. + lp[0];
        double q1y = 2. - lp[1], q2y = 2. + lp[1];
        double inv_size_x = 1. / (4. * lp[0]);
        double inv_size_y = 1. / (4. * lp[1]);
        double inv_dx = 0., inv_dy = 0.;
        if (grad) {
            inv_dx = 2.0 / DX;
            inv_dy = 2.0 / DY;
        }
        int i = 0;
        for (int id = 0; id < 16; id++) {
            double xp = fabs(xi[0] - gxii[id]);
            if (xp >= q2x) continue;
            double yp = fabs(xi[1] - geti[id]);
            if (yp >= q2y) continue;
            double Svpx, Svpy, argx = 0., argy = 0.;
            if (xp < lp[0]) Svpx = ((4. - lp[0]) * lp[0] - xp * xp) * inv_size_x;
            else if (xp <= q1x) Svpx = (2. - xp) / 2.;
            else { argx = (q2x - xp) * inv_size_x; Svpx = 2. * lp[0] * argx * argx; }
            if (yp < lp[1]) Svpy = ((4. - lp[1]) * lp[1] - yp * yp) * inv_size_y;
            else if (yp <= q1y) Svpy = (2. - yp) / 2.;
            else { argy = (q2y - yp) * inv_size_y; Svpy = 2. * lp[1] * argy * argy; }
            s->fn[i] = Svpx * Svpy;
            if (grad) {
                double xsign = xi[0] > gxii[id] ? 1. : -1.;
                double ysign = xi[1] > geti[id] ? 1. : -1.;
                double dSvpx, dSvpy;
                if (xp < lp[0]) dSvpx = -xp * inv_size_x * 2.0;
                else if (xp <= q1x) dSvpx = -0.5;
                else dSvpx = -argx;
                if (yp < lp[1]) dSvpy = -yp * inv_size_y * 2.0;
                else if (yp <= q1y) dSvpy = -0.5;
                else dSvpy = -argy;
                s->dx[i] = xsign * dSvpx * Svpy * inv_dx;
                s->dy[i] = ysign * Svpx * dSvpy * inv_dy;
                s->dz[i] = 0.;
            }
            s->nds[i] = n0 + xoff2[id] * g->xplane + yoff2[id] * g->yplane;
            i++;
        }
        s->n = i;
        return;
    }
    /* EightNodeIsoparamBrick::GimpShapeFunction, EightNodeIsoparamBrick.cpp:289-403
     * (including its z size factor taken from lp.y) */
    double q1x = 2. - lp[0], q2x = 2. + lp[0];
    double q1y = 2. - lp[1], q2y = 2. + lp[1];
    double q1z = 2. - lp[2], q2z = 2. + lp[2];
    double inv_size_x = 1. / (4. * lp[0]);
    double inv_size_y = 1. / (4. * lp[1]);
    double inv_size_z = 1. / (4. * lp[1]);
    double inv_dx = 0., inv_dy = 0., inv_dz = 0.;
    if (grad) {
        inv_dx = 2.0 / DX;
        inv_dy = 2.0 / DY;
        inv_dz = 2.0 / DZ;
    }
    int i = 0;
    for (int id = 0; id < 64; id++) {
        double gx = (double)(2 * x3off[id] - 1), gy = (double)(2 * y3off[id] - 1),
               gz = (double)(2 * z3off[id] - 1);
        double xp = fabs(xi[0] - gx);
        if (xp >= q2x) continue;
        double yp = fabs(xi[1] - gy);
        if (yp >= q2y) continue;
        double zp = fabs(xi[2] - gz);
        if (zp >= q2z) continue;
        double Svpx, Svpy, Svpz, argx = 0., argy = 0., argz = 0.;
        if (xp < lp[0]) Svpx = ((4. - lp[0]) * lp[0] - xp * xp) * inv_size_x;
        else if (xp <= q1x) Svpx = 0.5 * (2. - xp);
        else { argx = (q2x - xp) * inv_size_x; Svpx = 2. * lp[0] * argx * argx; }
        if (yp < lp[1]) Svpy = ((4. - lp[1]) * lp[1] - yp * yp) * inv_size_y;
        else if (yp <= q1y) Svpy = 0.5 * (2. - yp);
        else { argy = (q2y - yp) * inv_size_y; Svpy = 2. * lp[1] * argy * argy; }
        if (zp < lp[2]) Svpz = ((4. - lp[2]) * lp[2] - zp * zp) * inv_size_z;
        else if (zp <= q1z) Svpz = 0.5 * (2. - zp);
        else { argz = (q2z - zp) * inv_size_z; Svpz = 2. * lp[2] * argz * argz; }
        s->fn[i] = Svpx * Svpy * Svpz;
        if (grad) {
            double xsign = xi[0] > gx ? 1. : -1.;
            double ysign = xi[1] > gy ? 1. : -1.;
            double zsign = xi[2] > gz ? 1. : -1.;
            double dSvpx, dSvpy, dSvpz;
            if (xp < lp[0]) dSvpx = -xp / (2. * lp[0]);
            else if (xp <= q1x) dSvpx = -0.5;
            else dSvpx = -argx;
            if (yp < lp[1]) dSvpy = -yp / (2. * lp[1]);
            else if (yp <= q1y) dSvpy = -0.5;
            else dSvpy = -argy;
            if (zp < lp[2]) dSvpz = -zp / (2. * lp[2]);
            else if (zp <= q1z) dSvpz = -0.5;
            else dSvpz = -argz;
            s->dx[i] = xsign * dSvpx * Svpy * Svpz * inv_dx;
            s->dy[i] = ysign * Svpx * dSvpy * Svpz * inv_dy;
            s->dz[i] = zsign * Svpx * Svpy * dSvpz * inv_dz;
        }
        s->nds[i] = n0 + x3off[id] * g->xplane + y3off[id] * g->yplane + z3off[id] * g->zplane;
        i++;
    }
    s->n = i;
}

/* ------------------------------------------------------------------------ */
/* Linear CPDI (lCPDI)                                                       */
/* ------------------------------------------------------------------------ */
typedef struct {            /* CPDIDomain of each domain point, found once per step */
    int elem[9];
    double xi[9][3];
    double wg[9][3];
} OCpdi;

static const double r1s[8] = {-1., 1., 1., -1., -1., 1., 1., -1.};
static const double r2s[8] = {-1., -1., 1., 1., -1., -1., 1., 1.};
static const double r3s[8] = {-1., -1., -1., -1., 1., 1., 1., 1.};

/* MeshInfo::FindElementFromPoint, equal element sizes (MeshInfo.cpp:593-633);
 * returns the 0-based element or -1 when the point is off the grid */
static int find_element(const OGrid *g, double x, double y, double z) {
    int col = (int)((x - g->xmin) / g->gx);
    if (col < 0 || col >= g->nx) {
        if (x == g->xmin + g->nx * g->gx) col = g->nx - 1;
        else return -1;
    }
    int row = (int)((y - g->ymin) / g->gy);
    if (row < 0 || row >= g->ny) {
        if (y == g->ymin + g->ny * g->gy) row = g->ny - 1;
        else return -1;
    }
    if (g->dim == 3) {
        int zr = (int)((z - g->zmin) / g->gz);
        if (zr < 0 || zr >= g->nz) {
            if (z == g->zmin + g->nz * g->gz) zr = g->nz - 1;
            else return -1;
        }
        return g->nx * (zr * g->ny + row) + col;
    }
    return row * g->nx + col;
}

/* MatPoint2D::GetCPDINodesAndWeights (MatPoint2D.cpp:519-571) and
 * MatPoint3D::GetCPDINodesAndWeights (MatPoint3D.cpp:538-601) with
 * GetSemiSideVectors (MatPoint2D.cpp:423-439, MatPoint3D.cpp:413-433) and
 * GetParticleSize (MPMBase.cpp:519-524, MatPoint3D.cpp:227-233); no rcrit
 * rescaling (ElementBase::rcrit < 0 by default).  Returns 0, or -1 when a
 * corner is off the grid. */
static int cpdi_setup(const OGrid *g, const MpmGpuParticles *p, long q, int quad, OCpdi *cp) {
    int is3d = g->dim == 3;
    double ex0, ex1, ey0, ey1, ez0, ez1;
    elem_extent(g, p->elem[q], &ex0, &ex1, &ey0, &ey1, &ez0, &ez1);
    double pszx = ex1 - ex0, pszy = ey1 - ey0, pszz = ez1 - ez0;
    pszx *= 0.5 * p->lpx[q];
    pszy *= 0.5 * p->lpy[q];
    double F00 = 1. + p->exx[q], F01 = 0.5 * (p->exy[q] - p->wxy[q]), F10 = 0.5 * (p->exy[q] + p->wxy[q]),
           F11 = 1. + p->eyy[q], F22 = 1. + p->ezz[q];
    if (!is3d) {
        double r1x = F00 * pszx, r1y = F10 * pszx;
        double r2x = F01 * pszy, r2y = F11 * pszy;
        double Ap = 4. * (r1x * r2y - r1y * r2x);
        double px = p->x[q], py = p->y[q];
        double cx[4] = {px - r1x - r2x, px + r1x - r2x, px + r1x + r2x, px - r1x + r2x};
        double cy[4] = {py - r1y - r2y, py + r1y - r2y, py + r1y + r2y, py - r1y + r2y};
        for (int i = 0; i < 4; i++) {
            int e = find_element(g, cx[i], cy[i], 0.);
            if (e < 0) return -1;
            cp->elem[i] = e;
            xi_pos(g, e, cx[i], cy[i], 0., cp->xi[i]);
        }
        if (quad) {
            /* qCPDI (MatPoint2D.cpp:574-640): the four edge midpoints, counter
             * clockwise from the bottom edge, then the material point itself
             * in its own element; gradient weights from the linear domain
             * weights divided by 3 Ap */
            double ex[4] = {px - r2x, px + r1x, px + r2x, px - r1x};
            double ey[4] = {py - r2y, py + r1y, py + r2y, py - r1y};
            for (int i = 0; i < 4; i++) {
                int e = find_element(g, ex[i], ey[i], 0.);
                if (e < 0) return -1;
                cp->elem[4 + i] = e;
                xi_pos(g, e, ex[i], ey[i], 0., cp->xi[4 + i]);
            }
            cp->elem[8] = p->elem[q];
            xi_pos(g, p->elem[q], px, py, 0., cp->xi[8]);
            Ap = 1. / (3. * Ap);
            cp->wg[0][0] = (r1y - r2y) * Ap;
            cp->wg[0][1] = (-r1x + r2x) * Ap;
            cp->wg[1][0] = (r1y + r2y) * Ap;
            cp->wg[1][1] = (-r1x - r2x) * Ap;
            cp->wg[2][0] = (-r1y + r2y) * Ap;
            cp->wg[2][1] = (r1x - r2x) * Ap;
            cp->wg[3][0] = (-r1y - r2y) * Ap;
            cp->wg[3][1] = (r1x + r2x) * Ap;
            cp->wg[4][0] = 4. * r1y * Ap;
            cp->wg[4][1] = -4. * r1x * Ap;
            cp->wg[5][0] = 4. * r2y * Ap;
            cp->wg[5][1] = -4. * r2x * Ap;
            cp->wg[6][0] = -4. * r1y * Ap;
            cp->wg[6][1] = 4. * r1x * Ap;
            cp->wg[7][0] = -4. * r2y * Ap;
            cp->wg[7][1] = 4. * r2x * Ap;
            cp->wg[8][0] = 0.;
            cp->wg[8][1] = 0.;
            for (int i = 0; i < 9; i++) cp->wg[i][2] = 0.;
            return 0;
        }
        Ap = 1. / Ap;
        cp->wg[0][0] = (r1y - r2y) * Ap;
        cp->wg[1][0] = (r1y + r2y) * Ap;
        cp->wg[2][0] = (-r1y + r2y) * Ap;
        cp->wg[3][0] = (-r1y - r2y) * Ap;
        cp->wg[0][1] = (-r1x + r2x) * Ap;
        cp->wg[1][1] = (-r1x - r2x) * Ap;
        cp->wg[2][1] = (r1x - r2x) * Ap;
        cp->wg[3][1] = (r1x + r2x) * Ap;
        for (int i = 0; i < 4; i++) cp->wg[i][2] = 0.;
        return 0;
    }
    pszz *= 0.5 * p->lpz[q];
    double F02 = 0.5 * (p->exz[q] - p->wxz[q]), F20 = 0.5 * (p->exz[q] + p->wxz[q]);
    double F12 = 0.5 * (p->eyz[q] - p->wyz[q]), F21 = 0.5 * (p->eyz[q] + p->wyz[q]);
    double r1[3] = {F00 * pszx, F10 * pszx, F20 * pszx};
    double r2[3] = {F01 * pszy, F11 * pszy, F21 * pszy};
    double r3[3] = {F02 * pszz, F12 * pszz, F22 * pszz};
    double Vp = 8. * (r1[0] * (r2[1] * r3[2] - r2[2] * r3[1]) + r1[1] * (r2[2] * r3[0] - r2[0] * r3[2]) +
                      r1[2] * (r2[0] * r3[1] - r2[1] * r3[0]));
    for (int i = 0; i < 8; i++) {
        double cx = p->x[q] + r1s[i] * r1[0] + r2s[i] * r2[0] + r3s[i] * r3[0];
        double cy = p->y[q] + r1s[i] * r1[1] + r2s[i] * r2[1] + r3s[i] * r3[1];
        double cz = p->z[q] + r1s[i] * r1[2] + r2s[i] * r2[2] + r3s[i] * r3[2];
        int e = find_element(g, cx, cy, cz);
        if (e < 0) return -1;
        cp->elem[i] = e;
        xi_pos(g, e, cx, cy, cz, cp->xi[i]);
    }
    Vp = 1. / Vp;
    double r1x = r1[0], r1y = r1[1], r1z = r1[2], r2x = r2[0], r2y = r2[1], r2z = r2[2];
    double r3x = r3[0], r3y = r3[1], r3z = r3[2];
    /* gradient weights, term for term as MatPoint3D.cpp:571-594 writes them */
    cp->wg[0][0] = (r1z*r2y - r1y*r2z - r1z*r3y + r2z*r3y + r1y*r3z - r2y*r3z)*Vp;
    cp->wg[0][1] = (-(r1z*r2x) + r1x*r2z + r1z*r3x - r2z*r3x - r1x*r3z + r2x*r3z)*Vp;
    cp->wg[0][2] = (r1y*r2x - r1x*r2y - r1y*r3x + r2y*r3x + r1x*r3y - r2x*r3y)*Vp;
    cp->wg[1][0] = (r1z*r2y - r1y*r2z - r1z*r3y - r2z*r3y + r1y*r3z + r2y*r3z)*Vp;
    cp->wg[1][1] = (-(r1z*r2x) + r1x*r2z + r1z*r3x + r2z*r3x - r1x*r3z - r2x*r3z)*Vp;
    cp->wg[1][2] = (r1y*r2x - r1x*r2y - r1y*r3x - r2y*r3x + r1x*r3y + r2x*r3y)*Vp;
    cp->wg[2][0] = (r1z*r2y - r1y*r2z + r1z*r3y - r2z*r3y - r1y*r3z + r2y*r3z)*Vp;
    cp->wg[2][1] = (-(r1z*r2x) + r1x*r2z - r1z*r3x + r2z*r3x + r1x*r3z - r2x*r3z)*Vp;
    cp->wg[2][2] = (r1y*r2x - r1x*r2y + r1y*r3x - r2y*r3x - r1x*r3y + r2x*r3y)*Vp;
    cp->wg[3][0] = (r1z*r2y - r1y*r2z + r1z*r3y + r2z*r3y - r1y*r3z - r2y*r3z)*Vp;
    cp->wg[3][1] = (-(r1z*r2x) + r1x*r2z - r1z*r3x - r2z*r3x + r1x*r3z + r2x*r3z)*Vp;
    cp->wg[3][2] = (r1y*r2x - r1x*r2y + r1y*r3x + r2y*r3x - r1x*r3y - r2x*r3y)*Vp;
    cp->wg[4][0] = (-(r1z*r2y) + r1y*r2z - r1z*r3y + r2z*r3y + r1y*r3z - r2y*r3z)*Vp;
    cp->wg[4][1] = (r1z*r2x - r1x*r2z + r1z*r3x - r2z*r3x - r1x*r3z + r2x*r3z)*Vp;
    cp->wg[4][2] = (-(r1y*r2x) + r1x*r2y - r1y*r3x + r2y*r3x + r1x*r3y - r2x*r3y)*Vp;
    cp->wg[5][0] = (-(r1z*r2y) + r1y*r2z - r1z*r3y - r2z*r3y + r1y*r3z + r2y*r3z)*Vp;
    cp->wg[5][1] = (r1z*r2x - r1x*r2z + r1z*r3x + r2z*r3x - r1x*r3z - r2x*r3z)*Vp;
    cp->wg[5][2] = (-(r1y*r2x) + r1x*r2y - r1y*r3x - r2y*r3x + r1x*r3y + r2x*r3y)*Vp;
    cp->wg[6][0] = (-(r1z*r2y) + r1y*r2z + r1z*r3y - r2z*r3y - r1y*r3z + r2y*r3z)*Vp;
    cp->wg[6][1] = (r1z*r2x - r1x*r2z - r1z*r3x + r2z*r3x + r1x*r3z - r2x*r3z)*Vp;
    cp->wg[6][2] = (-(r1y*r2x) + r1x*r2y + r1y*r3x - r2y*r3x - r1x*r3y + r2x*r3y)*Vp;
    cp->wg[7][0] = (-(r1z*r2y) + r1y*r2z + r1z*r3y + r2z*r3y - r1y*r3z - r2y*r3z)*Vp;
    cp->wg[7][1] = (r1z*r2x - r1x*r2z - r1z*r3x - r2z*r3x + r1x*r3z + r2x*r3z)*Vp;
    cp->wg[7][2] = (-(r1y*r2x) + r1x*r2y + r1y*r3x + r2y*r3x - r1x*r3y - r2x*r3y)*Vp;
    return 0;
}

/* ElementBase::GetCPDIFunctions, FAST_CPDI branch (MoreMPMElementBase.cpp:581-656):
 * corners in order, the corner element's linear shape functions
 * (GetShapeFunctionsForTractions), contributions below 1e-15 skipped, nodes
 * merged in order of first appearance.  Returns 0, or -1 when the particle
 * needs more than maxShapeNodes-1 nodes (17 in 2D, 50 in 3D,
 * MPMReadHandler.cpp:558-562). */
static int shape_cpdi(const OGrid *g, const OCpdi *cp, int quad, int grad, OShape *s) {
    int is3d = g->dim == 3;
    int ncorner = quad ? 9 : (is3d ? 8 : 4);
    int maxnodes = quad ? 37 : (is3d ? 50 : 17);
    double lp1[3] = {1., 1., 1.};
    int ind = 0;
    for (int i = 0; i < ncorner; i++) {
        /* shape weights of the domain points (MPMBase.cpp:163-173): lCPDI 1/4
         * (2D) or 1/8 (3D); qCPDI 1/36 at the corners, 1/9 at the edges, 4/9
         * at the material point */
        double ws = quad ? (i < 4 ? 1. / 36. : (i < 8 ? 1. / 9. : 4. / 9.)) : (is3d ? 0.125 : 0.25);
        OShape cs;
        shape_eval(g, MPMGPU_SHAPE_LINEAR, cp->elem[i], cp->xi[i], lp1, 0, &cs);
        for (int j = 0; j < cs.n; j++) {
            double cfn = cs.fn[j];
            if (cfn < 1e-15) continue;
            long node = cs.nds[j];
            int found = -1;
            for (int look = ind - 1; look >= 0; look--)
                if (s->nds[look] == node) { found = look; break; }
            if (found >= 0) {
                s->fn[found] += ws * cfn;
                if (grad) {
                    s->dx[found] += cp->wg[i][0] * cfn;
                    s->dy[found] += cp->wg[i][1] * cfn;
                    s->dz[found] += cp->wg[i][2] * cfn;
                }
                continue;
            }
            if (ind + 1 >= maxnodes) return -1;
            s->nds[ind] = node;
            s->fn[ind] = ws * cfn;
            if (grad) {
                s->dx[ind] = cp->wg[i][0] * cfn;
                s->dy[ind] = cp->wg[i][1] * cfn;
                s->dz[ind] = cp->wg[i][2] * cfn;
            }
            ind++;
        }
    }
    s->n = ind;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Constitutive laws                                                         */
/* ------------------------------------------------------------------------ */
typedef struct {
    double m[3][3];
} M3;

/* Elastic::HypoIncrementDeformation (ElasticMPM.cpp:392-403): F <- (I+du)F,
 * with F stored as ep/wrot (MatPoint2D.cpp:309-366, MatPoint3D.cpp:320-376);
 * Matrix3::Exponential(1) and operator*= (Common/System/Matrix3.cpp:312-351,920-966). */
static void hypo_increment_F(MpmGpuParticles *p, long i, const M3 *du, int is3d) {
    if (!is3d) {
        double a00 = 1. + du->m[0][0], a01 = du->m[0][1], a10 = du->m[1][0], a11 = 1. + du->m[1][1],
               a22 = 1. + du->m[2][2];
        double b00 = 1. + p->exx[i], b01 = 0.5 * (p->exy[i] - p->wxy[i]),
               b10 = 0.5 * (p->exy[i] + p->wxy[i]), b11 = 1. + p->eyy[i], b22 = 1. + p->ezz[i];
        double f00 = a00 * b00 + a01 * b10;
        double f01 = a00 * b01 + a01 * b11;
        double f10 = a10 * b00 + a11 * b10;
        double f11 = a10 * b01 + a11 * b11;
        double f22 = a22 * b22;
        p->exx[i] = f00 - 1.;
        p->eyy[i] = f11 - 1.;
        p->ezz[i] = f22 - 1.;
        p->exy[i] = f10 + f01;
        p->wxy[i] = f10 - f01;
        return;
    }
    double a[3][3], b[3][3], f[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) a[r][c] = du->m[r][c] + (r == c ? 1. : 0.);
    b[0][0] = 1. + p->exx[i];
    b[1][1] = 1. + p->eyy[i];
    b[2][2] = 1. + p->ezz[i];
    b[0][1] = 0.5 * (p->exy[i] - p->wxy[i]);
    b[1][0] = 0.5 * (p->exy[i] + p->wxy[i]);
    b[0][2] = 0.5 * (p->exz[i] - p->wxz[i]);
    b[2][0] = 0.5 * (p->exz[i] + p->wxz[i]);
    b[1][2] = 0.5 * (p->eyz[i] - p->wyz[i]);
    b[2][1] = 0.5 * (p->eyz[i] + p->wyz[i]);
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) f[r][c] = a[r][0] * b[0][c] + a[r][1] * b[1][c] + a[r][2] * b[2][c];
    p->exx[i] = f[0][0] - 1.;
    p->eyy[i] = f[1][1] - 1.;
    p->ezz[i] = f[2][2] - 1.;
    p->exy[i] = f[1][0] + f[0][1];
    p->exz[i] = f[2][0] + f[0][2];
    p->eyz[i] = f[2][1] + f[1][2];
    p->wxy[i] = f[1][0] - f[0][1];
    p->wxz[i] = f[2][0] - f[0][2];
    p->wyz[i] = f[2][1] - f[1][2];
}

/* IsotropicMat::SRConstitutiveLaw2D (plane strain, no residual strains),
 * MoreIsotropicMat.cpp:185-279, with MaterialBase::Hypo2DCalculations
 * (MaterialBaseMPM.cpp:1012-1020). */
static void iso_2d(const OMat *m, MpmGpuParticles *p, long i, const M3 *du) {
    double dvxx = du->m[0][0], dvyy = du->m[1][1];
    double dgam = du->m[0][1] + du->m[1][0];
    double dwrotxy = du->m[1][0] - du->m[0][1];
    double st0xx = p->sxx[i], st0yy = p->syy[i], st0xy = p->sxy[i], st0zz = p->szz[i];
    double c1 = m->C2[1][1] * dvxx + m->C2[1][2] * dvyy;
    double c2 = m->C2[1][2] * dvxx + m->C2[2][2] * dvyy;
    double c3 = m->C2[3][3] * dgam;
    double dnorm = dwrotxy * p->sxy[i];
    double dshear = 0.5 * dwrotxy * (p->sxx[i] - p->syy[i]);
    p->sxx[i] += c1 - dnorm;
    p->syy[i] += c2 + dnorm;
    p->sxy[i] += c3 + dshear;
    double work = 0.5 * ((st0xx + p->sxx[i]) * dvxx + (st0yy + p->syy[i]) * dvyy + (st0xy + p->sxy[i]) * dgam);
    p->szz[i] += m->C2[4][1] * dvxx + m->C2[4][2] * dvyy + m->C2[4][4] * 0.;
    work += 0.5 * (st0zz + p->szz[i]) * 0.;
    if (p->work) p->work[i] += work;
}

/* IsotropicMat::SRConstitutiveLaw3D, MoreIsotropicMat.cpp:286-348, with
 * MaterialBase::Hypo3DCalculations (MaterialBaseMPM.cpp:1026-1047). */
static void iso_3d(const OMat *m, MpmGpuParticles *p, long i, const M3 *du) {
    double dvxx = du->m[0][0], dvyy = du->m[1][1], dvzz = du->m[2][2];
    double dgamxy = du->m[0][1] + du->m[1][0];
    double dgamxz = du->m[0][2] + du->m[2][0];
    double dgamyz = du->m[1][2] + du->m[2][1];
    double dwxy = du->m[1][0] - du->m[0][1];
    double dwxz = du->m[2][0] - du->m[0][2];
    double dwyz = du->m[2][1] - du->m[1][2];
    double s0xx = p->sxx[i], s0yy = p->syy[i], s0zz = p->szz[i];
    double s0yz = p->syz[i], s0xz = p->sxz[i], s0xy = p->sxy[i];
    double d[6];
    d[0] = m->C3[0][0] * dvxx + m->C3[0][1] * dvyy + m->C3[0][2] * dvzz;
    d[1] = m->C3[1][0] * dvxx + m->C3[1][1] * dvyy + m->C3[1][2] * dvzz;
    d[2] = m->C3[2][0] * dvxx + m->C3[2][1] * dvyy + m->C3[2][2] * dvzz;
    d[3] = m->C3[3][3] * dgamyz;
    d[4] = m->C3[4][4] * dgamxz;
    d[5] = m->C3[5][5] * dgamxy;
    double stxx = -dwxy * s0xy - dwxz * s0xz;
    double styy = dwxy * s0xy - dwyz * s0yz;
    double stzz = dwxz * s0xz + dwyz * s0yz;
    double styz = 0.5 * (dwxy * s0xz + dwxz * s0xy + dwyz * (s0yy - s0zz));
    double stxz = 0.5 * (-dwxy * s0yz + dwxz * (s0xx - s0zz) + dwyz * s0xy);
    double stxy = 0.5 * (dwxy * (s0xx - s0yy) - dwxz * s0yz - dwyz * s0xz);
    p->sxx[i] += d[0] + stxx;
    p->syy[i] += d[1] + styy;
    p->szz[i] += d[2] + stzz;
    p->syz[i] += d[3] + styz;
    p->sxz[i] += d[4] + stxz;
    p->sxy[i] += d[5] + stxy;
    if (p->work)
        p->work[i] += 0.5 * ((s0xx + p->sxx[i]) * dvxx + (s0yy + p->syy[i]) * dvyy + (s0zz + p->szz[i]) * dvzz +
                             (s0yz + p->syz[i]) * dgamyz + (s0xz + p->sxz[i]) * dgamxz +
                             (s0xy + p->sxy[i]) * dgamxy);
}

/* IsoPlasticity::MPMConstitutiveLaw + PlasticityConstLaw (small rotation, no
 * residual strains, linear hardening), IsoPlasticity.cpp:128-451, with
 * UpdatePressure (:462-492), GetPlasticPotential (:513-517),
 * IsotropicMat::GetMagnitudeSFromDev (MoreIsotropicMat.cpp:356-370) and
 * LinearHardening::SolveForLambdaBracketed (LinearHardening.cpp:124-145). */
static void isoplastic(const OMat *m, MpmGpuParticles *p, long i, const M3 *de, int is3d) {
    double delV = de->m[0][0] + de->m[1][1] + de->m[2][2];   /* du.trace() - 3*eres */
    double dgxy = de->m[0][1] + de->m[1][0], dgxz = 0., dgyz = 0.;
    if (is3d) {
        dgxz = de->m[0][2] + de->m[2][0];
        dgyz = de->m[1][2] + de->m[2][1];
    }
    double dexxr = de->m[0][0], deyyr = de->m[1][1], dezzr = de->m[2][2];
    /* UpdatePressure */
    double dP = -m->Kred * delV;
    double dVoverV = delV;
    p->pressure[i] += dP;
    double Pfinal = p->pressure[i];
    if (p->work) p->work[i] += -Pfinal * dVoverV;
    /* rotate plastic strain and stress (small rotation) */
    double dwrotxy = de->m[1][0] - de->m[0][1], dwrotxz = 0., dwrotyz = 0.;
    double epxx = p->pxx[i], epyy = p->pyy[i], epzz = p->pzz[i], epxy = p->pxy[i];
    double epxz = is3d ? p->pxz[i] : 0., epyz = is3d ? p->pyz[i] : 0.;
    double s0xx, s0yy, s0zz, s0xy, s0xz = 0., s0yz = 0.;
    double spxx = p->sxx[i], spyy = p->syy[i], spzz = p->szz[i], spxy = p->sxy[i];
    double spxz = is3d ? p->sxz[i] : 0., spyz = is3d ? p->syz[i] : 0.;
    if (!is3d) {
        double dnorm = 0.5 * dwrotxy * epxy;
        p->pxx[i] -= dnorm;
        p->pyy[i] += dnorm;
        p->pxy[i] += dwrotxy * (epxx - epyy);
        s0xx = spxx; s0yy = spyy; s0zz = spzz; s0xy = spxy;
        double dn = dwrotxy * spxy;
        s0xx -= dn;
        s0yy += dn;
        s0xy += 0.5 * dwrotxy * (epxx - epyy);
    } else {
        dwrotxz = de->m[2][0] - de->m[0][2];
        dwrotyz = de->m[2][1] - de->m[1][2];
        double dxy = 0.5 * dwrotxy * epxy, dxz = 0.5 * dwrotxz * epxz, dyz = 0.5 * dwrotyz * epyz;
        p->pxx[i] += -dxy - dxz;
        p->pyy[i] += dxy - dyz;
        p->pzz[i] += dxz + dyz;
        p->pyz[i] += dwrotyz * (epyy - epzz) + 0.5 * (dwrotxz * epxy + dwrotxy * epxz);
        p->pxz[i] += dwrotxz * (epxx - epzz) + 0.5 * (dwrotyz * epxy - dwrotxy * epyz);
        p->pxy[i] += dwrotxy * (epxx - epyy) - 0.5 * (dwrotyz * epxz + dwrotxz * epyz);
        s0xx = spxx; s0yy = spyy; s0zz = spzz; s0xy = spxy; s0xz = spxz; s0yz = spyz;
        double sxy = dwrotxy * spxy, sxz = dwrotxz * spxz, syz = dwrotyz * spyz;
        s0xx += -sxy - sxz;
        s0yy += sxy - syz;
        s0zz += sxz + syz;
        s0yz += 0.5 * (dwrotyz * (spyy - spzz) + dwrotxz * spxy + dwrotxy * spxz);
        s0xz += 0.5 * (dwrotxz * (spxx - spzz) + dwrotyz * spxy - dwrotxy * spyz);
        s0xy += 0.5 * (dwrotxy * (spxx - spyy) - dwrotyz * spxz - dwrotxz * spyz);
    }
    /* trial stress */
    double thirdDelV = delV / 3.;
    double dsxx = 2. * m->Gred * (dexxr - thirdDelV);
    double dsyy = 2. * m->Gred * (deyyr - thirdDelV);
    double dsxy = m->Gred * dgxy;
    double dszz = 2. * m->Gred * (dezzr - thirdDelV);
    double dsyz = 0., dsxz = 0.;
    if (is3d) {
        dsyz = m->Gred * dgyz;
        dsxz = m->Gred * dgxz;
    }
    double trxx = s0xx + dsxx, tryy = s0yy + dsyy, trzz = s0zz + dszz, trxy = s0xy + dsxy;
    double tryz = s0yz + dsyz, trxz = s0xz + dsxz;
    double alpint = p->hist0[i];
    double s2 = trxx * trxx + tryy * tryy + trzz * trzz;
    double t2 = is3d ? trxy * trxy + trxz * trxz + tryz * tryz : trxy * trxy;
    double strialmag = sqrt(s2 + t2 + t2);
    double yld = alpint < m->alphaMax ? m->yldred + m->Epred * alpint : m->yldredMin;
    double ftrial = strialmag - SQRT_TWOTHIRDS * yld;
    if (ftrial < 0.) {
        p->sxx[i] = trxx; p->syy[i] = tryy; p->szz[i] = trzz; p->sxy[i] = trxy;
        if (is3d) { p->syz[i] = tryz; p->sxz[i] = trxz; }
        if (p->work) {
            if (is3d)
                p->work[i] += trxx * de->m[0][0] + tryy * de->m[1][1] + trzz * de->m[2][2] + tryz * dgyz +
                              trxz * dgxz + trxy * dgxy;
            else
                p->work[i] += trxx * de->m[0][0] + tryy * de->m[1][1] + trxy * dgxy;
        }
        return;
    }
    /* radial return, LinearHardening::SolveForLambdaBracketed */
    double lambdak = (strialmag - SQRT_TWOTHIRDS * (m->yldred + m->Epred * alpint)) / (2. * (m->Gred + m->Epred / 3.));
    if (alpint + SQRT_TWOTHIRDS * lambdak > m->alphaMax)
        lambdak = (strialmag - SQRT_TWOTHIRDS * m->yldredMin) / (2. * m->Gred);
    double dalpha = SQRT_TWOTHIRDS * lambdak;
    double alpnew = alpint + dalpha;
    /* GetDfDsigma */
    double nxx = trxx / strialmag, nyy = tryy / strialmag, nzz = trzz / strialmag, nxy = trxy / strialmag;
    double nxz = 0., nyz = 0.;
    if (is3d) { nxz = trxz / strialmag; nyz = tryz / strialmag; }
    double depxx = lambdak * nxx, depyy = lambdak * nyy, depzz = lambdak * nzz, depxy = 2. * lambdak * nxy;
    double depxz = 0., depyz = 0.;
    if (is3d) { depxz = 2. * lambdak * nxz; depyz = 2. * lambdak * nyz; }
    p->pxx[i] += depxx; p->pyy[i] += depyy; p->pzz[i] += depzz; p->pxy[i] += depxy;
    if (is3d) { p->pxz[i] += depxz; p->pyz[i] += depyz; }
    double sxx = trxx - 2. * m->Gred * depxx;
    double syy = tryy - 2. * m->Gred * depyy;
    double szz = trzz - 2. * m->Gred * depzz;
    double sxy = trxy - m->Gred * depxy;
    double syz = 0., sxz = 0.;
    if (is3d) {
        syz = tryz - m->Gred * depyz;
        sxz = trxz - m->Gred * depxz;
    }
    p->sxx[i] = sxx; p->syy[i] = syy; p->szz[i] = szz; p->sxy[i] = sxy;
    if (is3d) { p->syz[i] = syz; p->sxz[i] = sxz; }
    double workEnergy = sxx * de->m[0][0] + syy * de->m[1][1] + sxy * dgxy;
    if (is3d) workEnergy += szz * de->m[2][2] + syz * dgyz + sxz * dgxz;
    if (is3d) workEnergy += szz * de->m[2][2];   /* np != PLANE_STRAIN_MPM adds zz again */
    if (p->work) p->work[i] += workEnergy;
    double plastEnergy = sxx * depxx + syy * depyy + szz * depzz + sxy * depxy;
    if (is3d) plastEnergy += sxz * depxz + syz * depyz;
    double qdalpha = lambdak * SQRT_TWOTHIRDS * fmax(m->Epred * alpnew, m->yldredMin - m->yldred);
    if (p->plast) p->plast[i] += plastEnergy - qdalpha;
    p->hist0[i] = alpnew;
}

/* Matrix3::Exponential (Common/System/Matrix3.cpp:312-364): dF = exp(du)
 * truncated after kmax terms.  2D: the 2x2 Cayley-Hamilton recursion with
 * the zz term separate; 3D: kmax 1 or 2. */
static void mat_exp(const M3 *a, int kmax, int is3d, M3 *out) {
    memset(out, 0, sizeof(*out));
    const double (*m)[3] = a->m;
    if (!is3d) {
        if (kmax == 1) {
            out->m[0][0] = 1. + m[0][0]; out->m[0][1] = m[0][1];
            out->m[1][0] = m[1][0]; out->m[1][1] = 1. + m[1][1];
            out->m[2][2] = 1. + m[2][2];
            return;
        }
        double c0 = m[0][1] * m[1][0] - m[0][0] * m[1][1];
        double c1 = m[0][0] + m[1][1];
        double beta0 = 0., beta1 = 1., alpha0 = 1., alpha1 = 1.;
        double betaz = m[2][2], ezz = 1. + betaz;
        for (int k = 2; k <= kmax; k++) {
            double factor = 1 / (double)k;
            double temp = beta1;
            beta1 = factor * (c1 * temp + beta0);
            beta0 = factor * c0 * temp;
            betaz *= factor * m[2][2];
            alpha0 += beta0;
            alpha1 += beta1;
            ezz += betaz;
        }
        out->m[0][0] = alpha0 + alpha1 * m[0][0]; out->m[0][1] = alpha1 * m[0][1];
        out->m[1][0] = alpha1 * m[1][0]; out->m[1][1] = alpha0 + alpha1 * m[1][1];
        out->m[2][2] = ezz;
        return;
    }
    if (kmax == 1) {
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) out->m[r][c] = m[r][c] + (r == c ? 1. : 0.);
        return;
    }
    double m2[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            m2[r][c] = 0.;
            for (int k = 0; k < 3; k++) m2[r][c] += m[r][k] * m[k][c];
        }
    /* 1. + m + 0.5*m2 on the diagonal, m + 0.5*m2 off it */
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            out->m[r][c] = r == c ? 1. + m[r][c] + 0.5 * m2[r][c] : m[r][c] + 0.5 * m2[r][c];
}

/* product of two matrices the way Matrix3::operator*= forms it
 * (Matrix3.cpp:920-966): the 2D formula when both are 2D, else the triple loop */
static void mat_mul(const M3 *a, const M3 *b, int is3d, M3 *out) {
    memset(out, 0, sizeof(*out));
    if (!is3d) {
        out->m[0][0] = a->m[0][0] * b->m[0][0] + a->m[0][1] * b->m[1][0];
        out->m[0][1] = a->m[0][0] * b->m[0][1] + a->m[0][1] * b->m[1][1];
        out->m[1][0] = a->m[1][0] * b->m[0][0] + a->m[1][1] * b->m[1][0];
        out->m[1][1] = a->m[1][0] * b->m[0][1] + a->m[1][1] * b->m[1][1];
        out->m[2][2] = a->m[2][2] * b->m[2][2];
        return;
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double v = 0.;
            for (int k = 0; k < 3; k++) v += a->m[i][k] * b->m[k][j];
            out->m[i][j] = v;
        }
}

/* HyperElastic::GetVolumetricTerms (HyperElastic.cpp:171-204) */
static double volumetric_terms(int uj, double J, double Kred) {
    if (uj == 1) return Kred * (J - 1.);
    if (uj == 2) {
        double Kterm = Kred * log(J);
        return Kterm / J;
    }
    return 0.5 * Kred * (J - 1. / J);
}

/* Neohookean::MPMConstitutiveLaw without residual strains, thermal terms or
 * artificial viscosity (Neohookean.cpp:177-331) with
 * HyperElastic::IncrementDeformation (HyperElastic.cpp:104-139): F and the
 * elastic left Cauchy-Green tensor B (held in the plastic-strain slot) are
 * pushed forward by dF = exp(du); J and Jres are history doubles 0 and 1;
 * the particle stress is the deviatoric Kirchhoff stress per unit initial
 * density and the pressure is carried separately. */
static void neohookean(const OMat *m, MpmGpuParticles *p, long i, const M3 *du, int is3d, int kterms) {
    M3 dF, pF, F, Bold, dFB;
    mat_exp(du, kterms, is3d, &dF);
    memset(&pF, 0, sizeof(pF));
    memset(&Bold, 0, sizeof(Bold));
    pF.m[0][0] = 1. + p->exx[i];
    pF.m[0][1] = 0.5 * (p->exy[i] - p->wxy[i]);
    pF.m[1][0] = 0.5 * (p->exy[i] + p->wxy[i]);
    pF.m[1][1] = 1. + p->eyy[i];
    pF.m[2][2] = 1. + p->ezz[i];
    Bold.m[0][0] = p->pxx[i]; Bold.m[0][1] = p->pxy[i];
    Bold.m[1][0] = p->pxy[i]; Bold.m[1][1] = p->pyy[i];
    Bold.m[2][2] = p->pzz[i];
    if (is3d) {
        pF.m[0][2] = 0.5 * (p->exz[i] - p->wxz[i]);
        pF.m[2][0] = 0.5 * (p->exz[i] + p->wxz[i]);
        pF.m[1][2] = 0.5 * (p->eyz[i] - p->wyz[i]);
        pF.m[2][1] = 0.5 * (p->eyz[i] + p->wyz[i]);
        Bold.m[0][2] = Bold.m[2][0] = p->pxz[i];
        Bold.m[1][2] = Bold.m[2][1] = p->pyz[i];
    }
    mat_mul(&dF, &pF, is3d, &F);
    /* SetDeformationGradientMatrix (MatPoint2D.cpp:310-322, MatPoint3D) */
    p->exx[i] = F.m[0][0] - 1.;
    p->eyy[i] = F.m[1][1] - 1.;
    p->ezz[i] = F.m[2][2] - 1.;
    p->exy[i] = F.m[1][0] + F.m[0][1];
    p->wxy[i] = F.m[1][0] - F.m[0][1];
    if (is3d) {
        p->exz[i] = F.m[2][0] + F.m[0][2];
        p->eyz[i] = F.m[2][1] + F.m[1][2];
        p->wxz[i] = F.m[2][0] - F.m[0][2];
        p->wyz[i] = F.m[2][1] - F.m[1][2];
    }
    mat_mul(&dF, &Bold, is3d, &dFB);
    const double (*a)[3] = dFB.m, (*d)[3] = dF.m;
    double Bxx = a[0][0] * d[0][0] + a[0][1] * d[0][1] + a[0][2] * d[0][2];
    double Bxy = a[0][0] * d[1][0] + a[0][1] * d[1][1] + a[0][2] * d[1][2];
    double Byy = a[1][0] * d[1][0] + a[1][1] * d[1][1] + a[1][2] * d[1][2];
    double Bzz = a[2][0] * d[2][0] + a[2][1] * d[2][1] + a[2][2] * d[2][2];
    double Bxz = 0., Byz = 0.;
    p->pxx[i] = Bxx; p->pxy[i] = Bxy; p->pyy[i] = Byy; p->pzz[i] = Bzz;
    if (is3d) {
        Bxz = a[0][0] * d[2][0] + a[0][1] * d[2][1] + a[0][2] * d[2][2];
        Byz = a[1][0] * d[2][0] + a[1][1] * d[2][1] + a[1][2] * d[2][2];
        p->pxz[i] = Bxz; p->pyz[i] = Byz;
    }
    /* Matrix3::determinant (Matrix3.cpp:1195-1202) */
    double detDf;
    if (!is3d) detDf = d[2][2] * (d[0][0] * d[1][1] - d[1][0] * d[0][1]);
    else
        detDf = d[0][0] * (d[1][1] * d[2][2] - d[2][1] * d[1][2]) - d[1][0] * (d[0][1] * d[2][2] - d[2][1] * d[0][2]) +
                d[2][0] * (d[0][1] * d[1][2] - d[1][1] * d[0][2]);
    /* residual terms with Jres = 1: resStretch = Jres23 = 1 */
    double Jres = p->hist1[i];
    double resStretch = pow(Jres, 1. / 3.);
    double Jres23 = resStretch * resStretch;
    double J = detDf * p->hist0[i];
    p->hist0[i] = J;
    double st0xx = p->sxx[i], st0yy = p->syy[i], st0zz = p->szz[i], st0xy = p->sxy[i];
    double st0xz = is3d ? p->sxz[i] : 0., st0yz = is3d ? p->syz[i] : 0.;
    double Jeff = J / Jres;
    double p0 = p->pressure[i];
    double Pterm = J * volumetric_terms(m->uj, Jeff, m->Lamesp) + Jres * m->Gsp * ((Bxx + Byy + Bzz) / (3. * Jres23) - 1.);
    double delV = 1. - 1. / detDf;
    double Pfinal = -Pterm + 0.;
    p->pressure[i] = Pfinal;
    double avgP = 0.5 * (p0 + Pfinal);
    double dilEnergy = -avgP * delV;
    double GJeff = resStretch * m->Gsp;
    double I1third = (Bxx + Byy + Bzz) / 3.;
    double sxx = GJeff * (Bxx - I1third), syy = GJeff * (Byy - I1third), szz = GJeff * (Bzz - I1third);
    double sxy = GJeff * Bxy;
    p->sxx[i] = sxx; p->syy[i] = syy; p->szz[i] = szz; p->sxy[i] = sxy;
    double sxz = 0., syz = 0.;
    if (is3d) {
        sxz = GJeff * Bxz;
        syz = GJeff * Byz;
        p->sxz[i] = sxz; p->syz[i] = syz;
    }
    double shearEnergy = 0.5 * ((sxx + st0xx) * du->m[0][0] + (syy + st0yy) * du->m[1][1] + (szz + st0zz) * du->m[2][2] +
                                (sxy + st0xy) * (du->m[0][1] + du->m[1][0]));
    if (is3d)
        shearEnergy += 0.5 * ((sxz + st0xz) * (du->m[0][2] + du->m[2][0]) + (syz + st0yz) * (du->m[1][2] + du->m[2][1]));
    if (p->work) p->work[i] += dilEnergy + shearEnergy;
}

/* ------------------------------------------------------------------------ */
/* Step                                                                      */
/* ------------------------------------------------------------------------ */
enum { MASS_MOMENTUM_CALL = 0, UPDATE_MOMENTUM_CALL, UPDATE_STRAINS_LAST_CALL, GRID_FORCES_CALL };

typedef struct {
    OGrid g;
    OField f;               /* single material field */
    const MpmGpuOptions *o;
    OMat *mats;
    const MpmGpuVelBC *bcs;
    int nbc;
    MpmGpuParticles *p;
    double *xi;             /* 3 per particle: natural coordinates (ncpos) */
    double dt, mtime;
    int nthreads;
    int kterms;             /* MaterialBase::incrementalDefGradTerms */
    OCpdi *cpdi;            /* lCPDI corners of each particle (this step) */
    int cpdi_err;           /* a particle needed more CPDI nodes than allowed */
    int nf;                 /* material velocity fields */
    long nn;                /* nodes + 1: stride between fields */
    long nfn;               /* nf * nn */
    int mm;                 /* multimaterial mode: contact terms and contact */
    int normals;            /* MeshInfo::materialNormalMethod (0, 1, 2, 5 or 6) */
    long *lr_start;         /* regression normals: particle lists of the contact */
    long *lr_list;          /*   nodes, node n's at lr_list[lr_start[n] .. lr_start[n+1]) */
    int friction_style;     /* CoulombFriction: 0 stick, 1 frictionless, 2 frictional */
    double friction;        /* Coulomb coefficient */
    int xpic;               /* this step: 0 FLIP, k > 0 FMPM(k), -k XPIC(k) (GridToParticleExtrap::m) */
    double *vpx, *vpy, *vpz;  /* XPIC v*(prev) (MatVelocityField vk[VSTARPREV_VEC]) */
    double *vnx, *vny, *vnz;  /* XPIC v*(next) (vk[VSTARNEXT_VEC]) */
    /* XPIC/FMPM(k > 1) with contact: each contact node's FMPMContact cache
     * (Common/System/DataTypes.hpp:90-104) per field, set at every contact call */
    char *xc_valid;         /* the cache was set this step (MaterialContactNode is per step) */
    int *xc_paired;         /* the other field when doing pairs, else -1 */
    double *xc_deln;        /* deltaDotn */
    double *xc_n;           /* norm (3 per field-node) */
    double *xc_prior;       /* priorDelPiZero (3) */
    double *xc_net;         /* netDelPi (3) */
    double *xc_dfi;         /* startDelFi (3) */
    int rigid_field[64];    /* field f holds a rigid contact material (MatVelocityField::IsRigidField) */
    int has_rigid;          /* some material is rigid */
    double rigid_bias;      /* MeshInfo::rigidGradientBias, squared (MeshInfo.cpp:1191) */
} OCtx;

/* field of particle q (MaterialBase::GetField) */
static int particle_field(const OCtx *c, long q) {
    return c->nf > 1 ? c->mats[c->p->mat[q]].field : 0;
}

/* particle q is of a rigid contact material (MaterialBase::IsRigid) */
static int particle_rigid(const OCtx *c, long q) {
    return c->mats[c->p->mat[q]].type == MPMGPU_MAT_RIGID_CONTACT;
}

/* shape functions of particle q for this step (GetShapeFunctions/GetShapeGradients) */
static void particle_shape(OCtx *c, long q, int grad, OShape *s) {
    if (c->o->shape == MPMGPU_SHAPE_LCPDI || c->o->shape == MPMGPU_SHAPE_QCPDI) {
        if (shape_cpdi(&c->g, &c->cpdi[q], c->o->shape == MPMGPU_SHAPE_QCPDI, grad, s) != 0) {
#pragma omp atomic write
            c->cpdi_err = 1;
            s->n = 0;
        }
        return;
    }
    MpmGpuParticles *p = c->p;
    int is3d = c->g.dim == 3;
    double lp[3] = {p->lpx[q], p->lpy[q], is3d ? p->lpz[q] : 1.};
    shape_eval(&c->g, c->o->shape, p->elem[q], &c->xi[3 * q], lp, grad, s);
}

static void bc_norm(int dir, double *n) {
    n[0] = dir == 1 ? 1. : 0.;
    n[1] = dir == 2 ? 1. : 0.;
    n[2] = dir == 4 ? 1. : 0.;
}

/* NodalVelBC::VelocityBCLoop (NodalVelBC.cpp:386-400) with
 * MatVelocityField::ZeroVelocityBC / AddVelocityBC (MatVelocityField.cpp:490-575),
 * on one material field (every nonrigid field gets the same conditions,
 * CrackVelocityFieldMulti::ZeroVelocityBC / AddVelocityBC). */
static void velocity_bc_field(OCtx *c, int pass, int fld) {
    OField *f = &c->f;
    double dt = c->dt;
    for (int b = 0; b < c->nbc; b++) {
        const MpmGpuVelBC *bc = &c->bcs[b];
        if (c->mtime < bc->ftime) continue;
        long i = (long)fld * c->nn + bc->node;
        if (f->npts[i] <= 0) continue;
        double n[3];
        bc_norm(bc->dir, n);
        double dotn, dotf, dotp;
        switch (pass) {
        case UPDATE_MOMENTUM_CALL:
            dotn = f->px[i] * n[0] + f->py[i] * n[1] + f->pz[i] * n[2];
            f->px[i] += n[0] * (-dotn); f->py[i] += n[1] * (-dotn); f->pz[i] += n[2] * (-dotn);
            f->fx[i] += n[0] * (-dotn / dt); f->fy[i] += n[1] * (-dotn / dt); f->fz[i] += n[2] * (-dotn / dt);
            break;
        case MASS_MOMENTUM_CALL:
        case UPDATE_STRAINS_LAST_CALL:
            dotn = f->px[i] * n[0] + f->py[i] * n[1] + f->pz[i] * n[2];
            f->px[i] += n[0] * (-dotn); f->py[i] += n[1] * (-dotn); f->pz[i] += n[2] * (-dotn);
            break;
        case GRID_FORCES_CALL: {
            dotf = f->fx[i] * n[0] + f->fy[i] * n[1] + f->fz[i] * n[2];
            dotp = f->px[i] * n[0] + f->py[i] * n[1] + f->pz[i] * n[2];
            double s = -dotf - dotp / dt;
            f->fx[i] += n[0] * s; f->fy[i] += n[1] * s; f->fz[i] += n[2] * s;
            break;
        }
        }
    }
    for (int b = 0; b < c->nbc; b++) {
        const MpmGpuVelBC *bc = &c->bcs[b];
        if (c->mtime < bc->ftime) continue;
        long i = (long)fld * c->nn + bc->node;
        if (f->npts[i] <= 0) continue;
        double n[3], vel = bc->value;
        bc_norm(bc->dir, n);
        double mass = f->mass[i];
        switch (pass) {
        case MASS_MOMENTUM_CALL:
        case UPDATE_STRAINS_LAST_CALL: {
            double s = mass * vel;
            f->px[i] += n[0] * s; f->py[i] += n[1] * s; f->pz[i] += n[2] * s;
            break;
        }
        case UPDATE_MOMENTUM_CALL: {
            double pvel = mass * vel;
            f->px[i] += n[0] * pvel; f->py[i] += n[1] * pvel; f->pz[i] += n[2] * pvel;
            double s = pvel / dt;
            f->fx[i] += n[0] * s; f->fy[i] += n[1] * s; f->fz[i] += n[2] * s;
            break;
        }
        case GRID_FORCES_CALL: {
            double s = mass * vel / dt;
            f->fx[i] += n[0] * s; f->fy[i] += n[1] * s; f->fz[i] += n[2] * s;
            break;
        }
        }
    }
}

/* CrackVelocityFieldMulti::ZeroVelocityBC / AddVelocityBC apply to the
 * non-rigid fields only (CrackVelocityFieldMulti.cpp:1243-1259) */
static void velocity_bc_loop(OCtx *c, int pass) {
    for (int fld = 0; fld < c->nf; fld++)
        if (!c->rigid_field[fld]) velocity_bc_field(c, pass, fld);
}

static long particle_order(const OCtx *c, long k) {
    /* reverse order of the patch list when single-threaded */
    return c->p->n - 1 - k;
}

/* MassAndMomentumTask::Execute (MassAndMomentumTask.cpp:48-127) and
 * NodalPoint::AddMassMomentum (NodalPointMPM.cpp:419-453); when last is set,
 * UpdateStrainsLastContactTask's AddMassMomentumLast (NodalPointMPM.cpp:470-486). */
/* particle volume for contact (MatPoint2D/3D::GetVolume with DEFORMED_AREA or
 * DEFORMED_AREA_FOR_GRADIENT, MatPoint2D.cpp:407-417, MatPoint3D.cpp:395-408) */
static double contact_volume(const OCtx *c, long q) {
    const MpmGpuParticles *p = c->p;
    double rho = c->mats[p->mat[q]].rho;
    double F00 = 1. + p->exx[q], F01 = 0.5 * (p->exy[q] - p->wxy[q]), F10 = 0.5 * (p->exy[q] + p->wxy[q]);
    double F11 = 1. + p->eyy[q];
    if (c->g.dim != 3) return (F00 * F11 - F10 * F01) * p->mass[q] / rho;
    double F22 = 1. + p->ezz[q];
    double F02 = 0.5 * (p->exz[q] - p->wxz[q]), F20 = 0.5 * (p->exz[q] + p->wxz[q]);
    double F12 = 0.5 * (p->eyz[q] - p->wyz[q]), F21 = 0.5 * (p->eyz[q] + p->wyz[q]);
    double J = F00 * (F11 * F22 - F21 * F12) - F01 * (F10 * F22 - F20 * F12) + F02 * (F10 * F21 - F20 * F11);
    return J * p->mass[q] / rho;
}

/* MassAndMomentumTask / UpdateStrainsLastContactTask extrapolations with
 * NodalPoint::AddMassMomentum / AddMassMomentumLast (NodalPointMPM.cpp:419-486):
 * momentum (and mass and point counts on the first pass) of the particle's
 * material field; in multimaterial mode also the contact volume, displacement
 * and volume gradient (CrackVelocityField::AddVolumeDisplacement :395-401,
 * CrackVelocityFieldMulti::AddVolumeGradient :108-112). */
static void p2g_mass_momentum(OCtx *c, int last) {
    MpmGpuParticles *p = c->p;
    OField *f = &c->f;
    int is3d = c->g.dim == 3;
#pragma omp parallel for num_threads(c->nthreads) schedule(static) if (c->nthreads > 1)
    for (long k = 0; k < p->n; k++) {
        long q = particle_order(c, k);
        /* the second extrapolation takes the non-rigid particles only
         * (UpdateStrainsLastContactTask.cpp:90); rigid particles add to their
         * field like any other on the first (NodalPointMPM.cpp:419-453, with
         * the unscaled volume, equal to the deformed one for F = I) */
        if (last && particle_rigid(c, q)) continue;
        OShape s;
        particle_shape(c, q, c->mm, &s);
        long off = (long)particle_field(c, q) * c->nn;
        double mp = p->mass[q];
        double vx = p->vx[q], vy = p->vy[q], vz = is3d ? p->vz[q] : 0.;
        double Vp = 0., dx = 0., dy = 0., dz = 0.;
        if (c->mm) {
            Vp = contact_volume(c, q);
            dx = p->x[q] - p->x0[q];
            dy = p->y[q] - p->y0[q];
            dz = is3d ? p->z[q] - p->z0[q] : 0.;
        }
        for (int j = 0; j < s.n; j++) {
            long nd = off + s.nds[j];
            double fnmp = s.fn[j] * mp;
            double ax = vx * fnmp, ay = vy * fnmp, az = vz * fnmp;
            if (c->nthreads > 1) {
#pragma omp atomic
                f->px[nd] += ax;
#pragma omp atomic
                f->py[nd] += ay;
#pragma omp atomic
                f->pz[nd] += az;
                if (!last) {
#pragma omp atomic
                    f->npts[nd] += 1;
#pragma omp atomic
                    f->mass[nd] += fnmp;
                }
                if (c->mm) {
                    double wv = s.fn[j] * Vp, gx = s.dx[j] * Vp, gy = s.dy[j] * Vp, gz = s.dz[j] * Vp;
                    double ux = dx * fnmp, uy = dy * fnmp, uz = dz * fnmp;
#pragma omp atomic
                    f->vol[nd] += wv;
#pragma omp atomic
                    f->ux[nd] += ux;
#pragma omp atomic
                    f->uy[nd] += uy;
#pragma omp atomic
                    f->uz[nd] += uz;
#pragma omp atomic
                    f->gvx[nd] += gx;
#pragma omp atomic
                    f->gvy[nd] += gy;
#pragma omp atomic
                    f->gvz[nd] += gz;
                }
            } else {
                f->px[nd] += ax;
                f->py[nd] += ay;
                f->pz[nd] += az;
                if (c->mm) {
                    f->vol[nd] += s.fn[j] * Vp;
                    f->ux[nd] += dx * fnmp;
                    f->uy[nd] += dy * fnmp;
                    f->uz[nd] += dz * fnmp;
                    f->gvx[nd] += s.dx[j] * Vp;
                    f->gvy[nd] += s.dy[j] * Vp;
                    f->gvz[nd] += s.dz[j] * Vp;
                }
                if (!last) {
                    f->npts[nd] += 1;
                    f->mass[nd] += fnmp;
                }
            }
        }
    }
}

/* MatVelocityField::GridValueCalculation (MatVelocityField.cpp:239-251) */
static void grid_velocity(OCtx *c) {
    OField *f = &c->f;
    for (long i = 1; i < c->nfn; i++) {
        if (f->npts[i] <= 0 || f->mass[i] == 0.) continue;
        double r = 1. / f->mass[i];
        f->vx[i] = f->px[i] * r;
        f->vy[i] = f->py[i] * r;
        f->vz[i] = f->pz[i] * r;
    }
}

/* UpdateStrainsFirstTask::FullStrainUpdate (UpdateStrainsFirstTask.cpp:101-168),
 * MatPoint2D/3D::UpdateStrain and ExtrapVelocityGradient
 * (MatPoint2D.cpp:37-87, MatPoint3D.cpp:40-75). */
static void xpic_extrapolate(OCtx *c, int order, int particle_update);
static void xpic_move(MpmGpuParticles *p, long q, int is3d, int m, double dt, double Svx, double Svy, double Svz);

static void strain_update(OCtx *c, double strainTime) {
    MpmGpuParticles *p = c->p;
    OField *f = &c->f;
    int is3d = c->g.dim == 3;
    /* FMPM(k > 1) takes v(k) of the XPIC expansion (UpdateStrainsFirstTask.cpp:106-125) */
    if (c->xpic > 1) xpic_extrapolate(c, c->xpic, 0);
    else grid_velocity(c);
#pragma omp parallel for num_threads(c->nthreads) schedule(static) if (c->nthreads > 1)
    for (long q = 0; q < p->n; q++) {
        if (particle_rigid(c, q)) continue;  /* non-rigid particles only (UpdateStrainsFirstTask.cpp:123) */
        OShape s;
        particle_shape(c, q, 1, &s);
        long off = (long)particle_field(c, q) * c->nn;
        M3 dv;
        memset(&dv, 0, sizeof(dv));
        for (int j = 0; j < s.n; j++) {
            long nd = off + s.nds[j];
            double vx = f->vx[nd], vy = f->vy[nd], vz = f->vz[nd];
            if (!is3d) {
                dv.m[0][0] += vx * s.dx[j];
                dv.m[0][1] += vx * s.dy[j];
                dv.m[1][0] += vy * s.dx[j];
                dv.m[1][1] += vy * s.dy[j];
            } else {
                double v[3] = {vx, vy, vz}, gr[3] = {s.dx[j], s.dy[j], s.dz[j]};
                for (int r = 0; r < 3; r++)
                    for (int cc = 0; cc < 3; cc++) dv.m[r][cc] += v[r] * gr[cc];
            }
        }
        for (int r = 0; r < 3; r++)
            for (int cc = 0; cc < 3; cc++) dv.m[r][cc] *= strainTime;
        const OMat *m = &c->mats[p->mat[q]];
        if (m->type == MPMGPU_MAT_NEOHOOKEAN) {
            neohookean(m, p, q, &dv, is3d, c->kterms);
            continue;
        }
        hypo_increment_F(p, q, &dv, is3d);
        if (m->type == MPMGPU_MAT_ISOTROPIC) {
            if (is3d) iso_3d(m, p, q, &dv);
            else iso_2d(m, p, q, &dv);
        } else {
            isoplastic(m, p, q, &dv, is3d);
        }
    }
}

/* GridForcesTask::Execute (GridForcesTask.cpp:40-153) with
 * MatPoint2D/3D::GetFintPlusFext (MatPoint2D.cpp:242-262, MatPoint3D.cpp:248-269). */
static void p2g_forces(OCtx *c) {
    MpmGpuParticles *p = c->p;
    OField *f = &c->f;
    int is3d = c->g.dim == 3;
#pragma omp parallel for num_threads(c->nthreads) schedule(static) if (c->nthreads > 1)
    for (long k = 0; k < p->n; k++) {
        long q = particle_order(c, k);
        if (particle_rigid(c, q)) continue;  /* non-rigid particles only (GridForcesTask.cpp:53) */
        OShape s;
        particle_shape(c, q, 1, &s);
        long off = (long)particle_field(c, q) * c->nn;
        double mp = p->mass[q], P = p->pressure ? p->pressure[q] : 0.;
        double sxx = p->sxx[q], syy = p->syy[q], sxy = p->sxy[q];
        double szz = is3d ? p->szz[q] : 0., sxz = is3d ? p->sxz[q] : 0., syz = is3d ? p->syz[q] : 0.;
        for (int j = 0; j < s.n; j++) {
            long nd = off + s.nds[j];
            double fx, fy, fz;
            if (!is3d) {
                fx = -mp * ((sxx - P) * s.dx[j] + sxy * s.dy[j]) + s.fn[j] * 0.;
                fy = -mp * (sxy * s.dx[j] + (syy - P) * s.dy[j]) + s.fn[j] * 0.;
                fz = 0.0;
            } else {
                fx = -mp * ((sxx - P) * s.dx[j] + sxy * s.dy[j] + sxz * s.dz[j]) + s.fn[j] * 0.;
                fy = -mp * (sxy * s.dx[j] + (syy - P) * s.dy[j] + syz * s.dz[j]) + s.fn[j] * 0.;
                fz = -mp * (sxz * s.dx[j] + syz * s.dy[j] + (szz - P) * s.dz[j]) + s.fn[j] * 0.;
            }
            if (c->nthreads > 1) {
#pragma omp atomic
                f->fx[nd] += fx;
#pragma omp atomic
                f->fy[nd] += fy;
#pragma omp atomic
                f->fz[nd] += fz;
            } else {
                f->fx[nd] += fx;
                f->fy[nd] += fy;
                f->fz[nd] += fz;
            }
        }
    }
}

/* UpdateParticlesTask::Execute (UpdateParticlesTask.cpp:44-178),
 * MatVelocityField::IncrementNodalVelAcc (MatVelocityField.cpp:410-426) and the
 * FLIP branch of MatPoint2D/3D::MoveParticle (MatPoint2D.cpp:99-196) with no damping. */
static void g2p_move(OCtx *c) {
    MpmGpuParticles *p = c->p;
    OField *f = &c->f;
    int is3d = c->g.dim == 3;
    double dt = c->dt;
    /* UpdateParticlesTask::Execute (UpdateParticlesTask.cpp:66-82): FMPM(k > 1)
     * and XPIC(k > 1) take v(k) of the XPIC expansion, FLIP and PIC the lumped
     * velocity; m > 0 FMPM, m < 0 XPIC, 0 FLIP */
    const int m = c->xpic;
    if (m > 1 || m < -1) xpic_extrapolate(c, m > 0 ? m : -m, 1);
    else grid_velocity(c);
#pragma omp parallel for num_threads(c->nthreads) schedule(static) if (c->nthreads > 1)
    for (long q = 0; q < p->n; q++) {
        if (particle_rigid(c, q)) {
            /* rigid materials move at their current velocity (UpdateParticlesTask.cpp:291-295,
             * MatPoint2D/3D::MovePosition) */
            p->x[q] += dt * p->vx[q];
            p->y[q] += dt * p->vy[q];
            if (is3d) p->z[q] += dt * p->vz[q];
            continue;
        }
        OShape s;
        particle_shape(c, q, 0, &s);
        long off = (long)particle_field(c, q) * c->nn;
        double Svx = 0., Svy = 0., Svz = 0., Sax = 0., Say = 0., Saz = 0.;
        for (int j = 0; j < s.n; j++) {
            long nd = off + s.nds[j];
            double fi = s.fn[j];
            Svx += f->vx[nd] * fi;
            Svy += f->vy[nd] * fi;
            Svz += f->vz[nd] * fi;
            double mnode = fi / f->mass[nd];
            Sax += f->fx[nd] * mnode;
            Say += f->fy[nd] * mnode;
            Saz += f->fz[nd] * mnode;
        }
        if (m != 0) {
            xpic_move(p, q, is3d, m, dt, Svx, Svy, Svz);
            continue;
        }
        double vmx = Svx - Sax * dt, vmy = Svy - Say * dt, vmz = Svz - Saz * dt;
        /* Adamp0 = 0 (no grid or particle damping) */
        double a0x = 0. * vmx + 0. * p->vx[q], a0y = 0. * vmy + 0. * p->vy[q];
        double dvx = (Sax - a0x) * dt, dvy = (Say - a0y) * dt;
        p->vx[q] += dvx;
        p->vy[q] += dvy;
        p->x[q] += (vmx + 0.5 * dvx) * dt;
        p->y[q] += (vmy + 0.5 * dvy) * dt;
        if (is3d) {
            double a0z = 0. * vmz + 0. * p->vz[q];
            double dvz = (Saz - a0z) * dt;
            p->vz[q] += dvz;
            p->z[q] += (vmz + 0.5 * dvz) * dt;
        }
    }
}

/* PeriodicXPIC::PrepareForStep / StepCalculation (PeriodicXPIC.cpp:351-370,
 * 427-445) with the custom tasks run once before the first step and after
 * every step (NairnMPM.cpp:171-200): step s (from 1) uses the task's order
 * when s is a multiple of periodicSteps, FLIP otherwise */
static int xpic_step_order(const MpmGpuOptions *o, long s) {
    if (o->xpic_order <= 0 || o->xpic_period <= 0) return 0;
    if (s % o->xpic_period != 0) return 0;
    return o->xpic_fmpm ? o->xpic_order : -o->xpic_order;
}

static int coulomb_delta(const OCtx *c, double *delPi, const double *norm, double dotn, double deln, double mred,
                         const double *delFi);
static double dot3(const double *a, const double *b);

/* XPICExtrapolationTask::ImposeIncrementalContact (XPICExtrapolationTask.cpp:
 * 246-258) for material contact: MaterialContactNode::NodalXPICIncrement and
 * CrackVelocityFieldMulti::MaterialXPICIncrementOnCVF (CrackVelocityFieldMulti.
 * cpp:1333-1514) on every node with two or more material fields, Coulomb
 * friction, no rigid fields.  Each field's Delta v(k) (v*(prev) here) is moved
 * by the increment of the contact law applied to the cached contact state of
 * the last contact call; XPIC's particle update also moves the node force. */
static void xpic_contact(OCtx *c, int particle_update) {
    OField *f = &c->f;
    const int nf = c->nf, is3d = c->g.dim == 3;
    const int xpic_force = particle_update && c->xpic < 0;
    const double dt = c->dt;
    for (long n = 1; n <= c->g.nnodes; n++) {
        int nm = 0;
        for (int fl = 0; fl < nf; fl++) nm += f->npts[fl * c->nn + n] > 0 ? 1 : 0;
        if (nm <= 1) continue;
        int hasCOM = 0;
        double Pc[3] = {0., 0., 0.}, Mc = 0.;
        for (int i = 0; i < nf; i++) {
            long ki = i * c->nn + n;
            if (f->npts[ki] <= 0) continue;
            if (!c->xc_valid[ki]) continue;
            int isPaired = c->xc_paired[ki] >= 0;
            if (!hasCOM) {
                for (int ii = 0; ii < nf; ii++) {
                    long kk = ii * c->nn + n;
                    if (f->npts[kk] <= 0) continue;
                    Pc[0] += c->vpx[kk] * f->mass[kk];
                    Pc[1] += c->vpy[kk] * f->mass[kk];
                    Pc[2] += c->vpz[kk] * f->mass[kk];
                    Mc += f->mass[kk];
                }
                hasCOM = 1;
            }
            double mi = f->mass[ki];
            double mred = mi * (1. - mi / Mc);
            double r = mi / Mc;
            double delPi[3] = {Pc[0] * r, Pc[1] * r, Pc[2] * r};
            delPi[0] += c->vpx[ki] * -mi;
            delPi[1] += c->vpy[ki] * -mi;
            delPi[2] += c->vpz[ki] * -mi;
            double *prior = &c->xc_prior[3 * ki], *net = &c->xc_net[3 * ki];
            for (int a = 0; a < 3; a++) delPi[a] += prior[a];
            for (int a = 0; a < 3; a++) prior[a] = delPi[a];
            const double *norm = &c->xc_n[3 * ki];
            double dotn = dot3(delPi, norm);
            if (!coulomb_delta(c, delPi, norm, dotn, c->xc_deln[ki], mred, &c->xc_dfi[3 * ki])) {
                int zero = net[0] == 0. && net[1] == 0. && (!is3d || net[2] == 0.);
                if (!zero) {
                    delPi[0] = delPi[1] = delPi[2] = 0.;
                } else {
                    if (isPaired) break;
                    continue;
                }
            }
            double newDelPi[3] = {delPi[0], delPi[1], delPi[2]};
            for (int a = 0; a < 3; a++) delPi[a] -= net[a];
            for (int a = 0; a < 3; a++) net[a] = newDelPi[a];
            double rm = 1. / mi, rdt = 1. / dt;
            c->vpx[ki] += delPi[0] * rm;
            c->vpy[ki] += delPi[1] * rm;
            c->vpz[ki] += delPi[2] * rm;
            if (xpic_force) {
                f->fx[ki] += delPi[0] * rdt;
                f->fy[ki] += delPi[1] * rdt;
                f->fz[ki] += delPi[2] * rdt;
            }
            if (isPaired) {
                long kj = (long)c->xc_paired[ki] * c->nn + n;
                double rmj = -1. / f->mass[kj], rdtj = -1. / dt;
                c->vpx[kj] += delPi[0] * rmj;
                c->vpy[kj] += delPi[1] * rmj;
                c->vpz[kj] += delPi[2] * rmj;
                if (xpic_force) {
                    f->fx[kj] += delPi[0] * rdtj;
                    f->fy[kj] += delPi[1] * rdtj;
                    f->fz[kj] += delPi[2] * rdtj;
                }
                break;
            }
        }
    }
}

/* XPICExtrapolationTask::Execute (XPICExtrapolationTask.cpp:50-160) with
 * MatVelocityField::XPICSupport (MatVelocityField.cpp:318-399), single
 * material field: v(k) of the order-k expansion in f->v (VSTAR_VEC is vk[0]).
 * FMPM starts from the lumped velocity p/m, XPIC from (p - f dt)/m and adds
 * f dt/m to v*.  Each pass adds (I - S+S) v*(prev) after zeroing the velocity
 * conditions' directions (NodalVelBC::GridVelocityConditions, XPIC passes,
 * NodalVelBC.cpp:327-334; MatVelocityField::ZeroVelocityBC :530-541). */
static void xpic_extrapolate(OCtx *c, int order, int particle_update) {
    MpmGpuParticles *p = c->p;
    OField *f = &c->f;
    const long nn = c->nfn;
    const double dt = c->dt;
    const int fmpm = c->xpic > 0;
    /* INITIALIZE_XPIC */
    for (long i = 1; i < nn; i++) {
        c->vnx[i] = 0.; c->vny[i] = 0.; c->vnz[i] = 0.;
        if (f->npts[i] == 0) continue;
        if (fmpm) {
            double r = 1. / f->mass[i];
            c->vpx[i] = f->px[i] * r; c->vpy[i] = f->py[i] * r; c->vpz[i] = f->pz[i] * r;
            f->vx[i] = c->vpx[i]; f->vy[i] = c->vpy[i]; f->vz[i] = c->vpz[i];
        } else {
            double r = 1. / f->mass[i];
            c->vpx[i] = f->px[i]; c->vpy[i] = f->py[i]; c->vpz[i] = f->pz[i];
            c->vpx[i] += f->fx[i] * (-dt); c->vpy[i] += f->fy[i] * (-dt); c->vpz[i] += f->fz[i] * (-dt);
            c->vpx[i] *= r; c->vpy[i] *= r; c->vpz[i] *= r;
            double s = dt / f->mass[i];
            f->vx[i] = c->vpx[i]; f->vy[i] = c->vpy[i]; f->vz[i] = c->vpz[i];
            f->vx[i] += f->fx[i] * s; f->vy[i] += f->fy[i] * s; f->vz[i] += f->fz[i] * s;
        }
    }
    for (int k = 2; k <= order; k++) {
        /* XPICDoubleLoop (XPICExtrapolationTask.cpp:182-211): v*(next) = S+S v*(prev) */
        for (long q = 0; q < p->n; q++) {
            OShape s;
            particle_shape(c, q, 0, &s);
            long off = (long)particle_field(c, q) * c->nn;
            for (int a = 0; a < s.n; a++) {
                long ni = off + s.nds[a];
                double mass = f->mass[ni];
                for (int b = 0; b < s.n; b++) {
                    long nj = off + s.nds[b];
                    double weight = s.fn[a] * s.fn[b];
                    double w = p->mass[q] * weight / mass;
                    c->vnx[ni] += w * c->vpx[nj];
                    c->vny[ni] += w * c->vpy[nj];
                    c->vnz[ni] += w * c->vpz[nj];
                }
            }
        }
        /* GET_DELTAV: Delta v(k) = v*(prev) - v*(next) */
        for (long i = 1; i < nn; i++) {
            if (f->npts[i] == 0) continue;
            c->vpx[i] -= c->vnx[i]; c->vpy[i] -= c->vny[i]; c->vpz[i] -= c->vnz[i];
        }
        /* velocity conditions zero their directions of Delta v(k) */
        for (int fld = 0; fld < c->nf; fld++)
            for (int b = 0; b < c->nbc; b++) {
                const MpmGpuVelBC *bc = &c->bcs[b];
                if (c->mtime < bc->ftime) continue;
                long i = (long)fld * c->nn + bc->node;
                if (f->npts[i] <= 0) continue;
                double n[3];
                bc_norm(bc->dir, n);
                double dotn = c->vpx[i] * n[0] + c->vpy[i] * n[1] + c->vpz[i] * n[2];
                c->vpx[i] += n[0] * (-dotn); c->vpy[i] += n[1] * (-dotn); c->vpz[i] += n[2] * (-dotn);
            }
        /* incremental material contact */
        if (c->mm) xpic_contact(c, particle_update);
        /* UPDATE_VSTAR: v* += Delta v(k), v*(next) = 0 */
        for (long i = 1; i < nn; i++) {
            if (f->npts[i] == 0) continue;
            f->vx[i] += c->vpx[i]; f->vy[i] += c->vpy[i]; f->vz[i] += c->vpz[i];
            c->vnx[i] = 0.; c->vny[i] = 0.; c->vnz[i] = 0.;
        }
    }
}

/* MatPoint2D/3D::MoveParticle (MatPoint2D.cpp:99-196, MatPoint3D.cpp:103-200)
 * for FMPM (m > 0) and XPIC (m < 0) with Svk = S v(k) (S v(k) + a dt for XPIC,
 * the lumped S v+ for order 1); no damping */
static void xpic_move(MpmGpuParticles *p, long q, int is3d, int m, double dt, double Svx, double Svy, double Svz) {
    double vmx = Svx, vmy = Svy, vmz = Svz;
    double a0x = 0. * vmx + 0. * p->vx[q], a0y = 0. * vmy + 0. * p->vy[q];
    double a0z = is3d ? 0. * vmz + 0. * p->vz[q] : 0.;
    if (m > 0) {
        double ox = p->vx[q], oy = p->vy[q], oz = is3d ? p->vz[q] : 0.;
        p->vx[q] = vmx - a0x * dt;
        p->vy[q] = vmy - a0y * dt;
        if (!is3d) {
            ox += p->vx[q];
            oy += p->vy[q];
            p->x[q] += 0.5 * ox * dt;
            p->y[q] += 0.5 * oy * dt;
        } else {
            p->vz[q] = vmz - a0z * dt;
            ox += p->vx[q];
            oy += p->vy[q];
            oz += p->vz[q];
            double h = 0.5 * dt;
            p->x[q] += ox * h;
            p->y[q] += oy * h;
            p->z[q] += oz * h;
        }
    } else {
        double ox = p->vx[q], oy = p->vy[q], oz = is3d ? p->vz[q] : 0.;
        p->vx[q] = Svx - a0x * dt;
        p->vy[q] = Svy - a0y * dt;
        double dvx = p->vx[q] - ox, dvy = p->vy[q] - oy;
        p->x[q] += (vmx + 0.5 * dvx) * dt;
        p->y[q] += (vmy + 0.5 * dvy) * dt;
        if (is3d) {
            p->vz[q] = Svz - a0z * dt;
            double dvz = p->vz[q] - oz;
            p->z[q] += (vmz + 0.5 * dvz) * dt;
        }
    }
}

/* ResetElementsTask::ResetElement (ResetElementsTask.cpp:196-228) with
 * MeshInfo::FindElementFromPoint (MeshInfo.cpp:593-633) for equal elements. */
static int reset_elements(OCtx *c) {
    MpmGpuParticles *p = c->p;
    const OGrid *g = &c->g;
    int is3d = g->dim == 3;
    int status = MPMGPU_OK;
    for (long q = 0; q < p->n; q++) {
        double x = p->x[q], y = p->y[q], z = is3d ? p->z[q] : 0.;
        if (x != x || y != y || z != z) return fail(MPMGPU_ERR_NAN, "oracle: particle position is NaN");
        double x0, x1, y0, y1, z0, z1;
        elem_extent(g, p->elem[q], &x0, &x1, &y0, &y1, &z0, &z1);
        int in = !(x < x0 || x >= x1) && !(y < y0 || y >= y1) && (!is3d || !(z < z0 || z >= z1));
        if (in) continue;
        int col = (int)((x - g->xmin) / g->gx);
        if (col < 0 || col >= g->nx) {
            if (x == g->xmin + g->nx * g->gx) col = g->nx - 1;
            else status = MPMGPU_ERR_LEFT_GRID;
        }
        int row = (int)((y - g->ymin) / g->gy);
        if (row < 0 || row >= g->ny) {
            if (y == g->ymin + g->ny * g->gy) row = g->ny - 1;
            else status = MPMGPU_ERR_LEFT_GRID;
        }
        int zr = 0;
        if (is3d) {
            zr = (int)((z - g->zmin) / g->gz);
            if (zr < 0 || zr >= g->nz) {
                if (z == g->zmin + g->nz * g->gz) zr = g->nz - 1;
                else status = MPMGPU_ERR_LEFT_GRID;
            }
        }
        if (status != MPMGPU_OK) return fail(status, "oracle: particle left the grid");
        int num = is3d ? g->nx * (zr * g->ny + row) + col + 1 : row * g->nx + col + 1;
        if (edge_element(g, num)) return fail(MPMGPU_ERR_LEFT_GRID, "oracle: particle entered an edge element");
        p->elem[q] = num - 1;
    }
    return status;
}

static void zero_field(OField *f, long nn) {
    double *cols[] = {f->mass, f->px, f->py, f->pz, f->fx, f->fy, f->fz, f->vx, f->vy, f->vz, f->cx, f->cy, f->cz,
                      f->vol, f->ux, f->uy, f->uz, f->gvx, f->gvy, f->gvz};
    for (unsigned k = 0; k < sizeof(cols) / sizeof(cols[0]); k++)
        if (cols[k]) memset(cols[k], 0, nn * sizeof(double));
    memset(f->npts, 0, nn * sizeof(int));
}

/* ------------------------------------------------------------------------ */
/* Multimaterial contact                                                     */
/* ------------------------------------------------------------------------ */
static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* MatVelocityField::ChangeMatMomentum (MatVelocityField.cpp:197-228) */
static void change_momentum(OCtx *c, long k, const double *d, int callType) {
    OField *f = &c->f;
    f->px[k] += d[0];
    f->py[k] += d[1];
    f->pz[k] += d[2];
    if (callType == UPDATE_MOMENTUM_CALL) {
        double s = 1. / c->dt;
        f->fx[k] += d[0] * s;
        f->fy[k] += d[1] * s;
        f->fz[k] += d[2] * s;
    } else if (callType == MASS_MOMENTUM_CALL) {
        f->cx[k] = f->px[k];
        f->cy[k] = f->py[k];
        f->cz[k] = f->pz[k];
    }
}

/* CoulombFriction::GetFrictionalDeltaMomentum (CoulombFriction.cpp:146-262)
 * with GetSslideAcDt (:266-285), no static coefficient.  Returns 0 when the
 * law leaves the momenta alone (not in contact). */
static int coulomb_delta(const OCtx *c, double *delPi, const double *norm, double dotn, double deln, double mred,
                         const double *delFi) {
    if (c->friction_style == 0) return 1;
    /* the separation adjustment after the momentum update is skipped for
     * regression normals (CoulombFriction.cpp:161-170) */
    if (delFi && c->normals < 5) {
        double fn = dot3(delFi, norm);
        deln += c->dt * (dotn - 0.5 * fn * c->dt) / mred;
    }
    int inContact = deln < 0. && dotn < 0.;
    if (c->friction_style == 1) {
        if (inContact) {
            for (int a = 0; a < 3; a++) delPi[a] = norm[a] * dotn;
            return 1;
        }
        return 0;
    }
    if (!inContact) return 0;
    double dott = 0., tang[3];
    for (int a = 0; a < 3; a++) tang[a] = delPi[a];
    for (int a = 0; a < 3; a++) tang[a] += norm[a] * (-dotn);
    double tangMag = sqrt(dot3(tang, tang));
    if (tangMag > 0.) {
        double s = 1. / tangMag;
        for (int a = 0; a < 3; a++) tang[a] *= s;
        dott = dot3(delPi, tang);
        if (dott < 0.) {
            for (int a = 0; a < 3; a++) tang[a] *= -1.;
            dott = -dott;
        }
    }
    double SslideAcDt = c->friction * (-dotn);
    if (SslideAcDt <= 0.) {
        for (int a = 0; a < 3; a++) delPi[a] = norm[a] * dotn;
    } else if (dott > SslideAcDt) {
        for (int a = 0; a < 3; a++) delPi[a] = norm[a] * dotn;
        for (int a = 0; a < 3; a++) delPi[a] += tang[a] * SslideAcDt;
    }
    return 1;
}

/* MaterialContactNode::ContactOnKnownNodes -> NodalPoint::MaterialContactOnNode ->
 * CrackVelocityFieldMulti::MaterialContactOnCVF / MaterialContactOnCVFLumped
 * (CrackVelocityFieldMulti.cpp:302-671) for nonrigid materials: each material
 * against the others lumped (two materials: one pair, equal and opposite
 * momentum changes), normals from volume gradients (GetNormalVector, :960-1069,
 * methods 0-2), separation from extrapolated displacements
 * (CrackSurfaceContact::MaterialSeparation), Coulomb friction. */
/* ---- regression normals (LINEAR_REGRESSION 5, LOGISTIC_REGRESSION 6) ---- */

/* a node with particles of two or more materials (NodalPoint::CalcTotalMassAndCount
 * in PostExtrapolationTask.cpp:72-78) */
static int contact_node(const OCtx *c, long n) {
    int nm = 0;
    for (int fl = 0; fl < c->nf; fl++)
        if (c->f.npts[fl * c->nn + n] > 0) nm++;
    return nm > 1;
}

/* MaterialContactNode::GetMaterialContactData (MaterialContactNode.cpp:238-353):
 * each contact node lists every particle whose shape-function nodes include
 * it, in particle order */
static void lr_build_lists(OCtx *c) {
    long nnodes = c->g.nnodes;
    long *cnt = c->lr_start;
    for (long n = 0; n <= nnodes + 1; n++) cnt[n] = 0;
    char *isc = (char *)malloc((size_t)nnodes + 1);
    for (long n = 1; n <= nnodes; n++) isc[n] = (char)contact_node(c, n);
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            long acc = 0;
            for (long n = 0; n <= nnodes; n++) {
                long k = cnt[n + 1];
                cnt[n + 1] = acc;
                acc += k;
            }
        }
        for (long q = 0; q < c->p->n; q++) {
            OShape sh;
            particle_shape(c, q, 0, &sh);
            for (int j = 0; j < sh.n; j++) {
                long n = sh.nds[j];
                if (!isc[n]) continue;
                if (pass == 0) cnt[n + 1]++;
                else c->lr_list[cnt[n + 1]++] = q;
            }
        }
    }
    /* after the fill, cnt[n+1] is the end of node n's list = start of node n+1's */
    cnt[0] = 0;
    free(isc);
}

/* node position of 1-based node n */
static void node_xyz(const OGrid *g, long n, double *x) {
    long i = n - 1;
    long nx1 = g->nx + 1, ny1 = g->ny + 1;
    x[0] = g->xn[i % nx1];
    x[1] = g->yn[(i / nx1) % ny1];
    x[2] = g->dim == 3 ? g->zn[i / (nx1 * ny1)] : 0.;
}

/* inverse of a symmetric 3x3 [a b c; b d e; c e f] (Matrix3::Inverse) */
static void inv3_sym(const double m[6], double r[9]) {
    double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5];
    double c00 = d * f - e * e, c01 = -(b * f - c * e), c02 = b * e - c * d;
    double det = a * c00 + b * c01 + c * c02;
    double c11 = a * f - c * c, c12 = -(a * e - b * c), c22 = a * d - b * b;
    r[0] = c00 / det; r[1] = c01 / det; r[2] = c02 / det;
    r[3] = c01 / det; r[4] = c11 / det; r[5] = c12 / det;
    r[6] = c02 / det; r[7] = c12 / det; r[8] = c22 / det;
}

/* inverse of a symmetric 4x4 stored as its upper triangle
 * mt[0..9] = (00 01 02 03 11 12 13 22 23 33) (Matrix4::Inverse, cofactors) */
static void inv4_sym(const double mt[10], double r[16]) {
    double m[4][4] = {{mt[0], mt[1], mt[2], mt[3]}, {mt[1], mt[4], mt[5], mt[6]},
                      {mt[2], mt[5], mt[7], mt[8]}, {mt[3], mt[6], mt[8], mt[9]}};
    double cof[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s3[3][3];
            int ri = 0;
            for (int a = 0; a < 4; a++) {
                if (a == i) continue;
                int cj = 0;
                for (int b = 0; b < 4; b++) {
                    if (b == j) continue;
                    s3[ri][cj++] = m[a][b];
                }
                ri++;
            }
            double d3 = s3[0][0] * (s3[1][1] * s3[2][2] - s3[1][2] * s3[2][1]) -
                        s3[0][1] * (s3[1][0] * s3[2][2] - s3[1][2] * s3[2][0]) +
                        s3[0][2] * (s3[1][0] * s3[2][1] - s3[1][1] * s3[2][0]);
            cof[i][j] = ((i + j) & 1) ? -d3 : d3;
        }
    double det = m[0][0] * cof[0][0] + m[0][1] * cof[0][1] + m[0][2] * cof[0][2] + m[0][3] * cof[0][3];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r[4 * i + j] = cof[j][i] / det;
}

/* MatPoint2D/3D::GetDeformedRadius, ellipse method (MatPoint2D.cpp:482-495,
 * MatPoint3D.cpp:497-510): distance from the particle centre to its deformed
 * inscribed ellipse(oid) along the unit vector n */
static double deformed_radius(const OCtx *c, long q, const double *n) {
    const MpmGpuParticles *p = c->p;
    double x0, x1, y0, y1, z0, z1;
    elem_extent(&c->g, p->elem[q], &x0, &x1, &y0, &y1, &z0, &z1);
    double px = 0.5 * p->lpx[q] * (x1 - x0), py = 0.5 * p->lpy[q] * (y1 - y0);
    double F00 = 1. + p->exx[q], F11 = 1. + p->eyy[q];
    double F01 = 0.5 * (p->exy[q] - p->wxy[q]), F10 = 0.5 * (p->exy[q] + p->wxy[q]);
    if (c->g.dim == 2) {
        double rdet = 1. / (F00 * F11 - F01 * F10);
        double n0x = (F11 * n[0] - F10 * n[1]) * rdet;
        double n0y = (-F01 * n[0] + F00 * n[1]) * rdet;
        double rd = sqrt(n0x * n0x / (px * px) + n0y * n0y / (py * py));
        return 1. / rd;
    }
    double pz = 0.5 * p->lpz[q] * (z1 - z0);
    double F22 = 1. + p->ezz[q];
    double F02 = 0.5 * (p->exz[q] - p->wxz[q]), F20 = 0.5 * (p->exz[q] + p->wxz[q]);
    double F12 = 0.5 * (p->eyz[q] - p->wyz[q]), F21 = 0.5 * (p->eyz[q] + p->wyz[q]);
    double c00 = F11 * F22 - F12 * F21, c01 = F12 * F20 - F10 * F22, c02 = F10 * F21 - F11 * F20;
    double det = F00 * c00 + F01 * c01 + F02 * c02;
    double i00 = c00 / det, i01 = (F02 * F21 - F01 * F22) / det, i02 = (F01 * F12 - F02 * F11) / det;
    double i10 = c01 / det, i11 = (F00 * F22 - F02 * F20) / det, i12 = (F02 * F10 - F00 * F12) / det;
    double i20 = c02 / det, i21 = (F01 * F20 - F00 * F21) / det, i22 = (F00 * F11 - F01 * F10) / det;
    double n0x = i00 * n[0] + i01 * n[1] + i02 * n[2];
    double n0y = i10 * n[0] + i11 * n[1] + i12 * n[2];
    double n0z = i20 * n[0] + i21 * n[1] + i22 * n[2];
    double rd = sqrt(n0x * n0x / (px * px) + n0y * n0y / (py * py) + n0z * n0z / (pz * pz));
    return 1. / rd;
}

/* CrackVelocityFieldMulti::LinearRegressionNormal and LogisticRegressionNormal
 * (MachineLearning.cpp:58-620) for material field a against all others
 * lumped (b < 0), with PENALIZE_NORMALS: the unit normal and the separation
 * deln from the two point clouds' supports along it (delMats.x) */
static void lr_normal(const OCtx *c, long n, int a, int logistic, double *norm, double *deln) {
    const MpmGpuParticles *p = c->p;
    int is3d = c->g.dim == 3;
    long s0 = c->lr_start[n], s1 = c->lr_start[n + 1];
    double nd[3];
    node_xyz(&c->g, n, nd);
    double cell = is3d ? fmin(c->g.gx, fmin(c->g.gy, c->g.gz)) : fmin(c->g.gx, c->g.gy);
    double cell2 = cell * cell;
    const double offsetLin = 0.1, normLog = 1.e-7, offsetLog = 0., tol = 1.e-5;
    const int maxIter = 15;
    double nrm[3] = {0., 0., 0.};
    if (is3d) {
        double mt[10] = {0.}, rhs[4] = {0.}, lam[4];
        double pen = logistic ? normLog * cell2 : 0.;
        lam[0] = lam[1] = lam[2] = pen;
        lam[3] = logistic ? offsetLog : offsetLin;
        for (long k = s0; k < s1; k++) {
            long q = c->lr_list[k];
            double mi = particle_field(c, q) == a ? -1. : 1.;
            double x = p->x[q] - nd[0], y = p->y[q] - nd[1], z = p->z[q] - nd[2];
            mt[0] += x * x; mt[1] += x * y; mt[2] += x * z; mt[3] += x;
            mt[4] += y * y; mt[5] += y * z; mt[6] += y;
            mt[7] += z * z; mt[8] += z; mt[9] += 1.;
            rhs[0] += mi * x; rhs[1] += mi * y; rhs[2] += mi * z; rhs[3] += mi;
        }
        double m[10] = {mt[0] + lam[0], mt[1], mt[2], mt[3], mt[4] + lam[1], mt[5], mt[6], mt[7] + lam[2], mt[8],
                        mt[9] + lam[3]};
        double inv[16], beta[4];
        inv4_sym(m, inv);
        for (int i = 0; i < 4; i++) beta[i] = inv[4 * i] * rhs[0] + inv[4 * i + 1] * rhs[1] + inv[4 * i + 2] * rhs[2] +
                                                inv[4 * i + 3] * rhs[3];
        if (!logistic) {
            for (int i = 0; i < 3; i++) nrm[i] = beta[i];
        } else {
            for (int i = 0; i < 4; i++) { beta[i] *= 2.; lam[i] *= 1.; }
            double prev[3] = {beta[0], beta[1], beta[2]};
            double nmag = sqrt(dot3(prev, prev));
            for (int i = 0; i < 3; i++) prev[i] *= 1. / nmag;
            double lin[3] = {prev[0], prev[1], prev[2]};
            double dcos = 1.;
            int iter = 0;
            while (dcos > tol && iter < maxIter) {
                for (int i = 0; i < 10; i++) mt[i] = 0.;
                for (int i = 0; i < 4; i++) rhs[i] = -lam[i] * beta[i];
                for (long k = s0; k < s1; k++) {
                    long q = c->lr_list[k];
                    double mi = particle_field(c, q) == a ? -1. : 1.;
                    double x = p->x[q] - nd[0], y = p->y[q] - nd[1], z = p->z[q] - nd[2];
                    double dotp = x * beta[0] + y * beta[1] + z * beta[2] + beta[3];
                    double arg = 1. + exp(-dotp);
                    double phi = 2. * (arg - 1.) / (arg * arg);
                    double phi2 = phi * phi;
                    mt[0] += phi2 * x * x; mt[1] += phi2 * x * y; mt[2] += phi2 * x * z; mt[3] += phi2 * x;
                    mt[4] += phi2 * y * y; mt[5] += phi2 * y * z; mt[6] += phi2 * y;
                    mt[7] += phi2 * z * z; mt[8] += phi2 * z; mt[9] += phi2;
                    double mifi = (mi - 2. / arg + 1.) * phi;
                    rhs[0] += mifi * x; rhs[1] += mifi * y; rhs[2] += mifi * z; rhs[3] += mifi;
                }
                double mm[10] = {mt[0] + lam[0], mt[1], mt[2], mt[3], mt[4] + lam[1], mt[5], mt[6],
                                 mt[7] + lam[2], mt[8], mt[9] + lam[3]};
                inv4_sym(mm, inv);
                for (int i = 0; i < 4; i++)
                    beta[i] += inv[4 * i] * rhs[0] + inv[4 * i + 1] * rhs[1] + inv[4 * i + 2] * rhs[2] +
                               inv[4 * i + 3] * rhs[3];
                double cur[3] = {beta[0], beta[1], beta[2]};
                nmag = sqrt(dot3(cur, cur));
                for (int i = 0; i < 3; i++) cur[i] *= 1. / nmag;
                dcos = 1. - dot3(cur, prev);
                iter++;
                for (int i = 0; i < 3; i++) prev[i] = nrm[i] = cur[i];
            }
            if (iter == 0) for (int i = 0; i < 3; i++) nrm[i] = prev[i];
            if (nrm[0] != nrm[0]) for (int i = 0; i < 3; i++) nrm[i] = lin[i];
        }
    } else {
        double mt[6] = {0.}, rhs[3] = {0.}, lam[3];
        double pen = logistic ? normLog * cell2 : 0.;
        lam[0] = lam[1] = pen;
        lam[2] = logistic ? offsetLog : offsetLin;
        for (long k = s0; k < s1; k++) {
            long q = c->lr_list[k];
            double mi = particle_field(c, q) == a ? -1. : 1.;
            double x = p->x[q] - nd[0], y = p->y[q] - nd[1];
            mt[0] += x * x; mt[1] += x * y; mt[2] += x;
            mt[3] += y * y; mt[4] += y; mt[5] += 1.;
            rhs[0] += mi * x; rhs[1] += mi * y; rhs[2] += mi;
        }
        double m[6] = {mt[0] + lam[0], mt[1], mt[2], mt[3] + lam[1], mt[4], mt[5] + lam[2]};
        double inv[9], beta[3];
        inv3_sym(m, inv);
        for (int i = 0; i < 3; i++) beta[i] = inv[3 * i] * rhs[0] + inv[3 * i + 1] * rhs[1] + inv[3 * i + 2] * rhs[2];
        if (!logistic) {
            nrm[0] = beta[0];
            nrm[1] = beta[1];
        } else {
            for (int i = 0; i < 3; i++) { beta[i] *= 2.; lam[i] *= 1.; }
            double prev[2], nmag = sqrt(beta[0] * beta[0] + beta[1] * beta[1]);
            prev[0] = beta[0] / nmag;
            prev[1] = beta[1] / nmag;
            double lin[2] = {prev[0], prev[1]};
            double dcos = 1.;
            int iter = 0;
            nrm[0] = prev[0];
            nrm[1] = prev[1];
            while (dcos > tol && iter < maxIter) {
                for (int i = 0; i < 6; i++) mt[i] = 0.;
                for (int i = 0; i < 3; i++) rhs[i] = -lam[i] * beta[i];
                for (long k = s0; k < s1; k++) {
                    long q = c->lr_list[k];
                    double mi = particle_field(c, q) == a ? -1. : 1.;
                    double x = p->x[q] - nd[0], y = p->y[q] - nd[1];
                    double arg = 1. + exp(-(x * beta[0] + y * beta[1] + beta[2]));
                    double phi = 2. * (arg - 1.) / (arg * arg);
                    double phi2 = phi * phi;
                    mt[0] += phi2 * x * x; mt[1] += phi2 * x * y; mt[2] += phi2 * x;
                    mt[3] += phi2 * y * y; mt[4] += phi2 * y; mt[5] += phi2;
                    double mifi = (mi - 2. / arg + 1.) * phi;
                    rhs[0] += mifi * x; rhs[1] += mifi * y; rhs[2] += mifi;
                }
                double mm[6] = {mt[0] + lam[0], mt[1], mt[2], mt[3] + lam[1], mt[4], mt[5] + lam[2]};
                inv3_sym(mm, inv);
                for (int i = 0; i < 3; i++)
                    beta[i] += inv[3 * i] * rhs[0] + inv[3 * i + 1] * rhs[1] + inv[3 * i + 2] * rhs[2];
                nmag = sqrt(beta[0] * beta[0] + beta[1] * beta[1]);
                nrm[0] = beta[0] / nmag;
                nrm[1] = beta[1] / nmag;
                dcos = 1. - nrm[0] * prev[0] - nrm[1] * prev[1];
                iter++;
                prev[0] = nrm[0];
                prev[1] = nrm[1];
            }
            if (nrm[0] != nrm[0]) { nrm[0] = lin[0]; nrm[1] = lin[1]; }
        }
        nrm[2] = 0.;
    }
    if (!logistic) {
        double mag = sqrt(dot3(nrm, nrm));
        for (int i = 0; i < 3; i++) nrm[i] *= 1. / mag;
    }
    /* separation: the supports of the two clouds along the normal */
    double supA = 1.e30, supB = 1.e30;
    for (long k = s0; k < s1; k++) {
        long q = c->lr_list[k];
        double xp[3] = {p->x[q], p->y[q], is3d ? p->z[q] : 0.};
        double r = deformed_radius(c, q, nrm);
        if (particle_field(c, q) == a) {
            double t = -dot3(nrm, xp) - r;
            if (t < supA) supA = t;
        } else {
            double t = dot3(nrm, xp) - r;
            if (t < supB) supB = t;
        }
    }
    for (int i = 0; i < 3; i++) norm[i] = nrm[i];
    *deln = supA + supB;
}

/* CrackVelocityFieldMulti::RigidMaterialContactOnCVF (CrackVelocityFieldMulti.cpp:676-958)
 * at node n for the Coulomb law: the rigid field with the largest contact
 * volume, and each non-rigid field moved toward the rigid field's velocity
 * (mred = its own mass; only the non-rigid field's momentum changes), with
 * the normal of GetNormalVector for a rigid partner (:960-1030). */
static void rigid_contact_node(OCtx *c, long n, int callType) {
    OField *f = &c->f;
    int postUpdate = callType == UPDATE_MOMENTUM_CALL;
    int rigidFld = -1;
    double rigidVolume = 0.;
    for (int fl = 0; fl < c->nf; fl++) {
        long k = fl * c->nn + n;
        if (f->npts[k] <= 0 || !c->rigid_field[fl]) continue;
        if (rigidFld < 0 || f->vol[k] > rigidVolume) {
            rigidFld = fl;
            rigidVolume = f->vol[k];
        }
    }
    long kr = (long)rigidFld * c->nn + n;
    double actualRigidVolume = f->mass[kr];
    double rr = 1. / actualRigidVolume;
    double rvel[3] = {f->px[kr] * rr, f->py[kr] * rr, f->pz[kr] * rr};
    double gradj[3] = {f->gvx[kr] * -1., f->gvy[kr] * -1., f->gvz[kr] * -1.};
    for (int fl = 0; fl < c->nf; fl++) {
        long ki = fl * c->nn + n;
        if (f->npts[ki] <= 0 || c->rigid_field[fl]) continue;
        double massi = f->mass[ki], voli = f->vol[ki];
        double delPi[3] = {f->px[ki] * -1., f->py[ki] * -1., f->pz[ki] * -1.};
        for (int a = 0; a < 3; a++) delPi[a] += rvel[a] * massi;
        double normi[3] = {f->gvx[ki] * 1., f->gvy[ki] * 1., f->gvz[ki] * 1.}, norm[3];
        if (c->normals == 0) {
            double magi = sqrt(dot3(normi, normi)), magj = sqrt(dot3(gradj, gradj));
            if (magi >= c->rigid_bias * magj) for (int a = 0; a < 3; a++) norm[a] = normi[a] * (1. / magi);
            else for (int a = 0; a < 3; a++) norm[a] = gradj[a] * (1. / magj);
        } else if (c->normals == 1) {
            if (voli >= rigidVolume) for (int a = 0; a < 3; a++) norm[a] = normi[a];
            else for (int a = 0; a < 3; a++) norm[a] = gradj[a];
            double sc = 1. / sqrt(dot3(norm, norm));
            for (int a = 0; a < 3; a++) norm[a] = norm[a] * sc;
        } else {
            for (int a = 0; a < 3; a++) norm[a] = normi[a] + gradj[a];
            double magi = dot3(norm, norm);
            double vRatio = (voli + rigidVolume) / rigidVolume;
            double magj = dot3(gradj, gradj);
            if (magi >= c->rigid_bias * magj * vRatio * vRatio) {
                double sc = 1. / sqrt(magi);
                for (int a = 0; a < 3; a++) norm[a] *= sc;
            } else {
                double sc = 1. / sqrt(magj);
                for (int a = 0; a < 3; a++) norm[a] = gradj[a] * sc;
            }
        }
        if (norm[0] != norm[0] || norm[1] != norm[1] || norm[2] != norm[2]) continue;
        double dotn = dot3(delPi, norm);
        double dispRigid[3] = {f->ux[kr] * rr, f->uy[kr] * rr, f->uz[kr] * rr};
        double rmi = 1. / massi;
        double dispi[3] = {f->ux[ki] * rmi, f->uy[ki] * rmi, f->uz[ki] * rmi};
        /* CrackSurfaceContact::MaterialSeparation with displacements (CrackSurfaceContact.cpp:278-303) */
        double deln = dot3(dispRigid, norm) - dot3(dispi, norm);
        double delFi[3], *dfp = NULL;
        if (postUpdate) {
            /* dF = -F_i for an infinitely massive partner */
            delFi[0] = f->fx[ki] * -1.;
            delFi[1] = f->fy[ki] * -1.;
            delFi[2] = f->fz[ki] * -1.;
            dfp = delFi;
        }
        if (!coulomb_delta(c, delPi, norm, dotn, deln, massi, dfp)) continue;
        change_momentum(c, ki, delPi, callType);
    }
}

static void material_contact(OCtx *c, int callType) {
    OField *f = &c->f;
    int nf = c->nf;
    int act[64];
    int postUpdate = callType == UPDATE_MOMENTUM_CALL;
    for (long n = 1; n <= c->g.nnodes; n++) {
        int nm = 0;
        double Pc[3] = {0., 0., 0.}, Mc = 0.;
        for (int fl = 0; fl < nf; fl++) {
            long k = fl * c->nn + n;
            if (f->npts[k] <= 0) continue;
            Pc[0] += f->px[k];
            Pc[1] += f->py[k];
            Pc[2] += f->pz[k];
            Mc += f->mass[k];
            act[nm++] = fl;
        }
        if (nm <= 1) continue;
        if (c->has_rigid) {
            /* a rigid field at the node: contact against it alone (MaterialContactOnCVF, :302-347) */
            int rigid_here = 0;
            for (int q = 0; q < nm; q++) rigid_here |= c->rigid_field[act[q]];
            if (rigid_here) {
                rigid_contact_node(c, n, callType);
                continue;
            }
        }
        int doingPairs = nm == 2;
        int miMax = doingPairs ? nm - 1 : nm;
        double dispc[3] = {0., 0., 0.};
        for (int fl = 0; fl < nf; fl++) {
            long k = fl * c->nn + n;
            if (f->npts[k] <= 0) continue;
            dispc[0] += f->ux[k];
            dispc[1] += f->uy[k];
            dispc[2] += f->uz[k];
        }
        double rMc = 1. / Mc;
        for (int a = 0; a < 3; a++) dispc[a] *= rMc;
        for (int mi = 0; mi < miMax; mi++) {
            long ki = act[mi] * c->nn + n;
            double massi = f->mass[ki];
            double voli = f->vol[ki];
            double voltot = 0.;
            for (int fl = 0; fl < nf; fl++) {
                long k = fl * c->nn + n;
                if (f->npts[k] > 0) voltot += f->vol[k];
            }
            double volj = voltot - voli;
            int j = -1;
            double gradj[3] = {0., 0., 0.}, maxOther = 0.;
            for (int kj = 0; kj < nm; kj++) {
                if (kj == mi) continue;
                long kk = act[kj] * c->nn + n;
                if (f->vol[kk] > maxOther) {
                    maxOther = f->vol[kk];
                    j = act[kj];
                }
                gradj[0] += f->gvx[kk] * -1.;
                gradj[1] += f->gvy[kk] * -1.;
                gradj[2] += f->gvz[kk] * -1.;
            }
            if (j < 0) continue;
            double massRatio = massi / Mc;
            double mred = 1. - massRatio;
            double delPi[3] = {f->px[ki] * -1., f->py[ki] * -1., f->pz[ki] * -1.};
            delPi[0] += Pc[0] * massRatio;
            delPi[1] += Pc[1] * massRatio;
            delPi[2] += Pc[2] * massRatio;
            double normi[3] = {f->gvx[ki] * 1., f->gvy[ki] * 1., f->gvz[ki] * 1.}, norm[3];
            int hasDeln = 0;
            double lrDeln = 0.;
            if (c->normals >= 5) {
                /* GetNormalVector's regression cases (CrackVelocityFieldMulti.cpp:1033-1062) */
                lr_normal(c, n, act[mi], c->normals == 6, norm, &lrDeln);
                hasDeln = 1;
            } else if (c->normals == 0) {
                double magi = sqrt(dot3(normi, normi)), magj = sqrt(dot3(gradj, gradj));
                if (magi >= 1. * magj) for (int a = 0; a < 3; a++) norm[a] = normi[a] * (1. / magi);
                else for (int a = 0; a < 3; a++) norm[a] = gradj[a] * (1. / magj);
            } else if (c->normals == 1) {
                if (voli >= volj) for (int a = 0; a < 3; a++) norm[a] = normi[a];
                else for (int a = 0; a < 3; a++) norm[a] = gradj[a];
                double s = 1. / sqrt(dot3(norm, norm));
                for (int a = 0; a < 3; a++) norm[a] = norm[a] * s;
            } else {
                for (int a = 0; a < 3; a++) norm[a] = normi[a] + gradj[a];
                double magi = dot3(norm, norm);
                double s = 1. / sqrt(magi);
                for (int a = 0; a < 3; a++) norm[a] *= s;
            }
            if (norm[0] != norm[0] || norm[1] != norm[1] || norm[2] != norm[2]) continue;
            double dotn = dot3(delPi, norm);
            double rmi = 1. / massi;
            double dispa[3] = {f->ux[ki] * rmi, f->uy[ki] * rmi, f->uz[ki] * rmi};
            double delta[3] = {dispc[0] - dispa[0], dispc[1] - dispa[1], dispc[2] - dispa[2]};
            double rmred = 1. / mred;
            for (int a = 0; a < 3; a++) delta[a] *= rmred;
            double dispb[3] = {delta[0] + dispa[0], delta[1] + dispa[1], delta[2] + dispa[2]};
            double deln = hasDeln ? lrDeln : dot3(dispb, norm) - dot3(dispa, norm);
            mred *= massi;
            /* MaterialContactNode::SetContactInfo (MaterialContactNode.cpp:133-151) */
            const int xcache = c->xc_valid && (c->xpic > 1 || c->xpic < -1);
            if (xcache) {
                c->xc_valid[ki] = 1;
                c->xc_paired[ki] = doingPairs ? j : -1;
                c->xc_deln[ki] = deln;
                for (int a = 0; a < 3; a++) {
                    c->xc_n[3 * ki + a] = norm[a];
                    c->xc_prior[3 * ki + a] = delPi[a];
                    c->xc_net[3 * ki + a] = 0.;
                    c->xc_dfi[3 * ki + a] = 0.;
                }
            }
            double delFi[3], *dfp = NULL;
            if (postUpdate) {
                double Fc[3] = {0., 0., 0.};
                for (int fl = 0; fl < nf; fl++) {
                    long k = fl * c->nn + n;
                    if (f->npts[k] <= 0) continue;
                    Fc[0] += f->fx[k];
                    Fc[1] += f->fy[k];
                    Fc[2] += f->fz[k];
                }
                double r = massi / Mc;
                delFi[0] = Fc[0] * r + f->fx[ki] * -1.;
                delFi[1] = Fc[1] * r + f->fy[ki] * -1.;
                delFi[2] = Fc[2] * r + f->fz[ki] * -1.;
                dfp = delFi;
                if (xcache)
                    for (int a = 0; a < 3; a++) c->xc_dfi[3 * ki + a] = delFi[a];
            }
            if (!coulomb_delta(c, delPi, norm, dotn, deln, mred, dfp)) continue;
            change_momentum(c, ki, delPi, callType);
            /* MaterialContactNode::ContactSetDelPi */
            if (xcache)
                for (int a = 0; a < 3; a++) c->xc_net[3 * ki + a] = delPi[a];
            if (doingPairs) {
                for (int a = 0; a < 3; a++) delPi[a] *= -1.;
                change_momentum(c, (long)j * c->nn + n, delPi, callType);
            }
        }
    }
}

/* One NairnMPM::MPMStep with the task chain of NairnMPM::CreateTasks
 * (NairnMPM.cpp:870-1110) for FLIP, no cracks, no transport, no custom tasks. */
static int one_step(OCtx *c) {
    MpmGpuParticles *p = c->p;
    OField *f = &c->f;
    long nn = c->nfn;   /* every field of every node */
    int method = c->o->method;
    double dt = c->dt;
    double fusf = c->o->fraction_usf;
    double stFirst = method == MPMGPU_USAVG ? fusf * dt : dt;
    double stLast = method == MPMGPU_USAVG ? dt - stFirst : dt;
    int is3d = c->g.dim == 3;

    c->xpic = xpic_step_order(c->o, (long)llround(c->mtime / dt) + 1);

    /* InitializationTask: zero nodes; ElementBase::GetShapeFunctionData: CPDI
     * corners (lCPDI) and natural coordinates (MoreMPMElementBase.cpp:50-57) */
    zero_field(f, nn);
    for (long q = 0; q < p->n; q++) {
        if ((c->o->shape == MPMGPU_SHAPE_LCPDI || c->o->shape == MPMGPU_SHAPE_QCPDI) &&
            cpdi_setup(&c->g, p, q, c->o->shape == MPMGPU_SHAPE_QCPDI, &c->cpdi[q]) != 0)
            return fail(MPMGPU_ERR_LEFT_GRID, "oracle: a CPDI particle domain node has left the grid");
        xi_pos(&c->g, p->elem[q], p->x[q], p->y[q], is3d ? p->z[q] : 0., &c->xi[3 * q]);
    }

    /* MassAndMomentumTask */
    p2g_mass_momentum(c, 0);
    if (c->cpdi_err) return fail(MPMGPU_ERR_CPDI_NODES, "oracle: too many CPDI nodes found");

    /* PostExtrapolationTask: copy momenta, BCs (MASS_MOMENTUM_CALL) */
    for (long i = 1; i < nn; i++) {
        if (f->npts[i] > 0) { f->cx[i] = f->px[i]; f->cy[i] = f->py[i]; f->cz[i] = f->pz[i]; }
    }
    if (c->mm && c->normals >= 5) lr_build_lists(c);
    /* the step's MaterialContactNodes are new (PostExtrapolationTask.cpp:74-79) */
    if (c->xc_valid) memset(c->xc_valid, 0, (size_t)c->nfn);
    if (c->mm) material_contact(c, MASS_MOMENTUM_CALL);
    if (method == MPMGPU_USF || method == MPMGPU_USAVG) velocity_bc_loop(c, MASS_MOMENTUM_CALL);

    /* UpdateStrainsFirstTask */
    if (method == MPMGPU_USF || method == MPMGPU_USAVG) strain_update(c, stFirst);

    /* GridForcesTask */
    p2g_forces(c);

    /* PostForcesTask: restore momenta, BCs (GRID_FORCES_CALL) */
    for (long i = 1; i < nn; i++) {
        if (f->npts[i] > 0) { f->px[i] = f->cx[i]; f->py[i] = f->cy[i]; f->pz[i] = f->cz[i]; }
    }
    velocity_bc_loop(c, GRID_FORCES_CALL);

    /* UpdateMomentaTask */
    for (long i = 1; i < nn; i++) {
        if (f->npts[i] > 0) {
            f->px[i] += f->fx[i] * dt;
            f->py[i] += f->fy[i] * dt;
            f->pz[i] += f->fz[i] * dt;
        }
    }
    if (c->mm) material_contact(c, UPDATE_MOMENTUM_CALL);
    /* NodalVelBC::GridVelocityConditions (NodalVelBC.cpp:367-374): not for XPIC/FMPM(k > 1) */
    if (c->xpic >= -1 && c->xpic <= 1) velocity_bc_loop(c, UPDATE_MOMENTUM_CALL);

    /* UpdateParticlesTask */
    g2p_move(c);

    /* UpdateStrainsLastContactTask */
    if (method == MPMGPU_USL || method == MPMGPU_USAVG) {
        /* RezeroNodeTask6: momenta and contact terms */
        for (long i = 1; i < nn; i++) {
            if (f->npts[i] > 0) {
                if (c->rigid_field[i / c->nn]) {
                    /* a rigid field keeps its momentum, volume and volume gradient; its
                     * displacement moves by p dt (CrackVelocityFieldMulti::RezeroNodeTask6, :157-176) */
                    f->ux[i] += f->px[i] * dt;
                    f->uy[i] += f->py[i] * dt;
                    f->uz[i] += f->pz[i] * dt;
                    continue;
                }
                f->px[i] = 0.; f->py[i] = 0.; f->pz[i] = 0.;
                if (c->mm) {
                    f->vol[i] = 0.;
                    f->ux[i] = 0.; f->uy[i] = 0.; f->uz[i] = 0.;
                    f->gvx[i] = 0.; f->gvy[i] = 0.; f->gvz[i] = 0.;
                }
            }
        }
        p2g_mass_momentum(c, 1);
        if (c->mm) material_contact(c, UPDATE_STRAINS_LAST_CALL);
        velocity_bc_loop(c, UPDATE_STRAINS_LAST_CALL);
        strain_update(c, stLast);
    }

    /* ResetElementsTask */
    return reset_elements(c);
}

int mpm_oracle_run(const MpmGpuGrid *grid, const MpmGpuOptions *opts, const MpmGpuMaterial *mats, int nmat,
                   const MpmGpuVelBC *bcs, int nbc, const MpmGpuContact *contact, MpmGpuParticles *p,
                   int nsteps, double t0, int nthreads) {
    g_err[0] = 0;
    if (!grid || !opts || !mats || !p) return fail(MPMGPU_ERR_INVALID, "oracle: null argument");
    if (opts->shape != MPMGPU_SHAPE_LINEAR && opts->shape != MPMGPU_SHAPE_UGIMP && opts->shape != MPMGPU_SHAPE_LCPDI &&
        opts->shape != MPMGPU_SHAPE_BSPLINE && opts->shape != MPMGPU_SHAPE_BGIMP && opts->shape != MPMGPU_SHAPE_QCPDI)
        return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: shape function not implemented");
    /* ElementBase::InitializeCPDI: qCPDI is 2D only (MoreMPMElementBase.cpp:1008-1013) */
    if (opts->shape == MPMGPU_SHAPE_QCPDI && grid->dim == 3)
        return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: qCPDI is not defined in 3D; use lCPDI");
    if (contact && contact->enabled) {
        if (contact->normals < 0 || (contact->normals > 2 && contact->normals != 5 && contact->normals != 6))
            return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: contact normals must be method 0, 1, 2, 5 or 6");
        if (contact->contact_cutoff > 0.)
            return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: position-based contact not implemented");
    }
    OCtx c;
    memset(&c, 0, sizeof(c));
    c.g.dim = grid->dim;
    c.g.nx = grid->nx; c.g.ny = grid->ny; c.g.nz = grid->dim == 3 ? grid->nz : 0;
    c.g.xplane = 1;
    c.g.yplane = grid->nx + 1;
    c.g.zplane = (long)(grid->nx + 1) * (grid->ny + 1);
    c.g.nnodes = grid->dim == 3 ? c.g.zplane * (grid->nz + 1) : c.g.zplane;
    c.g.nelems = (long)grid->nx * grid->ny * (grid->dim == 3 ? grid->nz : 1);
    c.g.xn = grid->xnodes; c.g.yn = grid->ynodes; c.g.zn = grid->znodes;
    c.g.xmin = grid->xmin; c.g.ymin = grid->ymin; c.g.zmin = grid->zmin;
    c.g.gx = grid->dx; c.g.gy = grid->dy; c.g.gz = grid->dz;
    c.o = opts;
    c.bcs = bcs;
    c.nbc = nbc;
    c.p = p;
    c.dt = opts->timestep;
    c.nthreads = nthreads < 1 ? 1 : nthreads;
    /* StartOutput.cpp:116-119: the default (negative) becomes 2, or 1 in 3D */
    c.kterms = opts->inc_defgrad_terms > 0 ? opts->inc_defgrad_terms : (grid->dim == 3 ? 1 : 2);
    if (grid->dim == 3 && c.kterms > 2)
        return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: 3D incremental F with more than 2 terms not implemented");
    c.mats = (OMat *)calloc((size_t)nmat, sizeof(OMat));
    int np = grid->dim == 3 ? MPMGPU_THREED : MPMGPU_PLANE_STRAIN;
    int st = load_materials(mats, nmat, np, c.mats);
    if (st != MPMGPU_OK) { free(c.mats); return st; }
    /* material velocity fields: one, or one per field in multimaterial mode */
    c.nf = 1;
    for (int i = 0; i < nmat; i++)
        if (mats[i].field + 1 > c.nf) c.nf = mats[i].field + 1;
    if (c.nf > 64) { free(c.mats); return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: more than 64 material fields"); }
    c.mm = c.nf > 1 && contact && contact->enabled;
    if (c.nf > 1 && !c.mm) { free(c.mats); return fail(MPMGPU_ERR_INVALID, "oracle: several material fields need contact"); }
    for (int i = 0; i < nmat; i++)
        if (c.mats[i].type == MPMGPU_MAT_RIGID_CONTACT) {
            c.rigid_field[c.mats[i].field] = 1;
            c.has_rigid = 1;
        }
    if (c.has_rigid && (!c.mm || c.nf < 2)) {
        free(c.mats);
        return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: rigid contact materials need multimaterial contact");
    }
    if (c.has_rigid && contact->normals >= 5) {
        free(c.mats);
        return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: regression normals with rigid materials not implemented");
    }
    if (c.mm) {
        c.rigid_bias = contact->rigid_gradient_bias > 0. ? contact->rigid_gradient_bias : 1.;
        c.rigid_bias *= c.rigid_bias;
        c.normals = contact->normals;
        c.friction = contact->friction;
        /* CoulombFriction::VerifyAndLoadProperties: <0 stick, 0 frictionless */
        c.friction_style = contact->friction < 0. ? 0 : (contact->friction == 0. ? 1 : 2);
    }
    c.nn = c.g.nnodes + 1;
    c.nfn = c.nn * c.nf;
    long nn = c.nfn;
    double **fl[] = {&c.f.mass, &c.f.px, &c.f.py, &c.f.pz, &c.f.fx, &c.f.fy, &c.f.fz,
                     &c.f.vx, &c.f.vy, &c.f.vz, &c.f.cx, &c.f.cy, &c.f.cz,
                     &c.f.vol, &c.f.ux, &c.f.uy, &c.f.uz, &c.f.gvx, &c.f.gvy, &c.f.gvz};
    for (unsigned k = 0; k < sizeof(fl) / sizeof(fl[0]); k++) *fl[k] = (double *)calloc((size_t)nn, sizeof(double));
    c.f.npts = (int *)calloc((size_t)nn, sizeof(int));
    c.xi = (double *)calloc((size_t)(3 * (p->n > 0 ? p->n : 1)), sizeof(double));
    if (opts->shape == MPMGPU_SHAPE_LCPDI || opts->shape == MPMGPU_SHAPE_QCPDI) c.cpdi = (OCpdi *)calloc((size_t)(p->n > 0 ? p->n : 1), sizeof(OCpdi));
    if (c.mm && c.normals >= 5) {
        c.lr_start = (long *)calloc((size_t)c.g.nnodes + 2, sizeof(long));
        c.lr_list = (long *)calloc((size_t)(p->n > 0 ? p->n : 1) * 64, sizeof(long));
    }
    if (opts->xpic_order > 0) {
        if (c.mm && c.has_rigid) {
            free(c.mats);
            return fail(MPMGPU_ERR_UNSUPPORTED, "oracle: XPIC/FMPM with rigid contact materials not implemented");
        }
        if (opts->xpic_period < 1) { free(c.mats); return fail(MPMGPU_ERR_INVALID, "oracle: xpic_period < 1"); }
        double **xv[] = {&c.vpx, &c.vpy, &c.vpz, &c.vnx, &c.vny, &c.vnz};
        for (unsigned k = 0; k < 6; k++) *xv[k] = (double *)calloc((size_t)nn, sizeof(double));
        if (c.mm) {
            c.xc_valid = (char *)calloc((size_t)nn, 1);
            c.xc_paired = (int *)calloc((size_t)nn, sizeof(int));
            c.xc_deln = (double *)calloc((size_t)nn, sizeof(double));
            double **xc[] = {&c.xc_n, &c.xc_prior, &c.xc_net, &c.xc_dfi};
            for (unsigned k = 0; k < 4; k++) *xc[k] = (double *)calloc((size_t)nn * 3, sizeof(double));
        }
    }
    c.mtime = t0;
    for (int s = 0; s < nsteps && st == MPMGPU_OK; s++) {
        st = one_step(&c);
        c.mtime += c.dt;
    }
    for (unsigned k = 0; k < sizeof(fl) / sizeof(fl[0]); k++) free(*fl[k]);
    free(c.f.npts);
    free(c.xi);
    free(c.cpdi);
    free(c.lr_start);
    free(c.lr_list);
    free(c.vpx); free(c.vpy); free(c.vpz); free(c.vnx); free(c.vny); free(c.vnz);
    free(c.xc_valid); free(c.xc_paired); free(c.xc_deln);
    free(c.xc_n); free(c.xc_prior); free(c.xc_net); free(c.xc_dfi);
    free(c.mats);
    return st;
}
