/*
 * mpmgpu_cpu_double.c -- TEST INFRASTRUCTURE ONLY, never part of the product.
 *
 * A stand-in for the GPU library with the single-run entry points of
 * include/nairn_mpm_gpu.h that the NairnMPM binding (nairn-mpm-fea_gb300/
 * nairnmpm/GPUStepTask.cpp) calls, implemented over the oracle
 * (mpm_oracle_run, one thread: the reference's summation order).  It lets the
 * binding -- the packing of NairnMPM's grid, materials, contact law,
 * velocity conditions and particles into the C ABI, the stepping and the
 * write-back before archives -- run end to end on a machine without a GPU:
 * NairnMPM-gpu linked with it must reproduce NairnMPM's own archives.  The
 * product library (libnairn_mpm_gb300.so) has no CPU path.
 */
#include <stdlib.h>
#include <string.h>

#include "mpm_oracle.h"
#include "nairn_mpm_gpu.h"

struct MpmGpuCtx {
    MpmGpuGrid grid;
    double *xn, *yn, *zn;
    MpmGpuOptions opts;
    MpmGpuMaterial *mats;
    int nmat;
    MpmGpuVelBC *bcs;
    int nbc;
    MpmGpuContact contact;
    int contact_on;
    MpmGpuParticles p;          /* owned columns */
    double *block;
    int32_t *ints;
    char msg[256];
};

static char g_msg[256];

#define NDOUBLE 39
/* the double columns of MpmGpuParticles, in declaration order */
static double **dcol(MpmGpuParticles *p, int k) {
    double **c[NDOUBLE] = {&p->x, &p->y, &p->z, &p->vx, &p->vy, &p->vz, &p->x0, &p->y0, &p->z0, &p->mass,
                           &p->lpx, &p->lpy, &p->lpz, &p->exx, &p->eyy, &p->ezz, &p->exy, &p->exz, &p->eyz,
                           &p->wxy, &p->wxz, &p->wyz, &p->sxx, &p->syy, &p->szz, &p->sxy, &p->sxz, &p->syz,
                           &p->pressure, &p->pxx, &p->pyy, &p->pzz, &p->pxy, &p->pxz, &p->pyz, &p->hist0,
                           &p->hist1, &p->work, &p->plast};
    return c[k];
}

static int err(MpmGpuCtx *c, int code, const char *m) {
    strncpy(c ? c->msg : g_msg, m, 255);
    return code;
}

const char *mpmgpu_last_error(const MpmGpuCtx *c) { return c ? c->msg : g_msg; }

int mpmgpu_create(const MpmGpuGrid *grid, const MpmGpuOptions *opts, MpmGpuCtx **out) {
    if (!grid || !opts || !out) return err(NULL, MPMGPU_ERR_INVALID, "null argument");
    MpmGpuCtx *c = (MpmGpuCtx *)calloc(1, sizeof(MpmGpuCtx));
    c->grid = *grid;
    c->xn = (double *)malloc(sizeof(double) * (grid->nx + 1));
    c->yn = (double *)malloc(sizeof(double) * (grid->ny + 1));
    memcpy(c->xn, grid->xnodes, sizeof(double) * (grid->nx + 1));
    memcpy(c->yn, grid->ynodes, sizeof(double) * (grid->ny + 1));
    c->grid.xnodes = c->xn;
    c->grid.ynodes = c->yn;
    if (grid->dim == 3) {
        c->zn = (double *)malloc(sizeof(double) * (grid->nz + 1));
        memcpy(c->zn, grid->znodes, sizeof(double) * (grid->nz + 1));
        c->grid.znodes = c->zn;
    }
    c->opts = *opts;
    *out = c;
    return MPMGPU_OK;
}

int mpmgpu_set_materials(MpmGpuCtx *c, const MpmGpuMaterial *mats, int32_t nmat) {
    free(c->mats);
    c->mats = (MpmGpuMaterial *)malloc(sizeof(MpmGpuMaterial) * nmat);
    memcpy(c->mats, mats, sizeof(MpmGpuMaterial) * nmat);
    c->nmat = nmat;
    return MPMGPU_OK;
}

int mpmgpu_set_contact(MpmGpuCtx *c, const MpmGpuContact *ct) {
    c->contact_on = ct && ct->enabled;
    if (ct) c->contact = *ct;
    return MPMGPU_OK;
}

int mpmgpu_set_velocity_bcs(MpmGpuCtx *c, const MpmGpuVelBC *bcs, int32_t nbc) {
    free(c->bcs);
    c->bcs = NULL;
    c->nbc = nbc;
    if (nbc > 0) {
        c->bcs = (MpmGpuVelBC *)malloc(sizeof(MpmGpuVelBC) * nbc);
        memcpy(c->bcs, bcs, sizeof(MpmGpuVelBC) * nbc);
    }
    return MPMGPU_OK;
}

int mpmgpu_upload_particles(MpmGpuCtx *c, const MpmGpuParticles *h) {
    const size_t n = (size_t)h->n;
    free(c->block);
    free(c->ints);
    c->block = (double *)calloc(n * NDOUBLE, sizeof(double));
    c->ints = (int32_t *)calloc(n * 2, sizeof(int32_t));
    memset(&c->p, 0, sizeof(c->p));
    c->p.n = h->n;
    for (int k = 0; k < NDOUBLE; k++) {
        *dcol(&c->p, k) = c->block + k * n;
        const double *src = *dcol((MpmGpuParticles *)h, k);
        if (src) memcpy(*dcol(&c->p, k), src, n * sizeof(double));
    }
    c->p.mat = c->ints;
    c->p.elem = c->ints + n;
    memcpy(c->p.mat, h->mat, n * sizeof(int32_t));
    memcpy(c->p.elem, h->elem, n * sizeof(int32_t));
    return MPMGPU_OK;
}

int mpmgpu_step(MpmGpuCtx *c, int32_t nsteps, double t0) {
    int st = mpm_oracle_run(&c->grid, &c->opts, c->mats, c->nmat, c->bcs, c->nbc,
                            c->contact_on ? &c->contact : NULL, &c->p, nsteps, t0, 1);
    if (st != MPMGPU_OK) return err(c, st, mpm_oracle_last_error());
    return MPMGPU_OK;
}

int mpmgpu_download_particles(MpmGpuCtx *c, MpmGpuParticles *h) {
    const size_t n = (size_t)c->p.n;
    for (int k = 0; k < NDOUBLE; k++) {
        double *dst = *dcol(h, k);
        if (dst) memcpy(dst, *dcol(&c->p, k), n * sizeof(double));
    }
    memcpy(h->mat, c->p.mat, n * sizeof(int32_t));
    memcpy(h->elem, c->p.elem, n * sizeof(int32_t));
    return MPMGPU_OK;
}

void mpmgpu_destroy(MpmGpuCtx *c) {
    if (!c) return;
    free(c->xn); free(c->yn); free(c->zn);
    free(c->mats); free(c->bcs); free(c->block); free(c->ints);
    free(c);
}
