/*
 * mpm_oracle.h -- CPU restatement of NairnMPM's explicit time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU path is compared
 * against (tests, smoke check, bench CPU baseline).  The product never links,
 * loads or calls it.  It reuses the plain data structs of the GPU C ABI
 * (include/nairn_mpm_gpu.h) so both sides read the same inputs.
 *
 * Parity status: pinned.  The restatement is checked against the reference
 * NairnMPM built from source (oracle/ref) on seeded inputs, see
 * tests/golden/.
 */
#ifndef NAIRN_MPM_ORACLE_H
#define NAIRN_MPM_ORACLE_H

#include "nairn_mpm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Advance nsteps FP64 steps in place on p, from time t0.  nthreads > 1 runs
 * the particle loops with OpenMP (summation order then differs from the
 * reference's single-thread order); nthreads == 1 follows the reference's
 * single-patch order exactly.  Returns an MPMGPU_* status. */
int mpm_oracle_run(const MpmGpuGrid *grid, const MpmGpuOptions *opts,
                   const MpmGpuMaterial *mats, int nmat,
                   const MpmGpuVelBC *bcs, int nbc,
                   const MpmGpuContact *contact,
                   MpmGpuParticles *p, int nsteps, double t0, int nthreads);

/* Critical time step (s) for the CFL factor, as NairnMPM::PreliminaryParticleCalcs
 * and CFLTimeStep compute it (NairnMPM.cpp:695-699, 1207-1240). */
double mpm_oracle_cfl_timestep(const MpmGpuGrid *grid, const MpmGpuMaterial *mats, int nmat,
                               const int32_t *mat_used, double cfl);

const char *mpm_oracle_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
