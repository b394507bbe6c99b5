/*
 * nairn_mpm_gpu.h -- C ABI of the GB300 explicit MPM time step.
 *
 * This is the drop-in boundary for NairnMPM's explicit step.  In the
 * reference the step is a linked list of MPMTask objects built by
 * NairnMPM::CreateTasks (NairnMPM/src/NairnMPM_Class/NairnMPM.cpp:870-1110) and
 * walked by NairnMPM::MPMStep (NairnMPM.cpp:284-335).  A host integration
 * replaces the tasks from InitializationTask through ResetElementsTask with one
 * task that calls mpmgpu_step(); everything else (XML input, archiving,
 * warnings) stays host code.  The plugin APIs the device re-implements are
 *   - MaterialBase::MPMConstitutiveLaw / GetCopyOfMechanicalProps
 *     (Common/Materials/MaterialBase.hpp:144,164; NairnMPM/src/Materials/MaterialBaseMPM.cpp:865),
 *   - ElementBase::GetShapeFunctions / GetShapeGradients
 *     (NairnMPM/src/Elements/MoreMPMElementBase.cpp:120,202),
 *   - ContactLaw::GetFrictionalDeltaMomentum (NairnMPM/src/Materials/CoulombFriction.cpp:146).
 *
 * Conventions
 *   - Plain C types, FP64 on the wire, NairnMPM "Legacy" units: mm, g, s;
 *     stresses held per unit density (Pa*mm^3/g) exactly as MPMBase::sp.
 *   - Every function returns an int status (MPMGPU_OK == 0) and never throws;
 *     the reference's error convention is CommonException
 *     (Common/Exceptions/CommonException.hpp:14-35), which the host side raises
 *     from a non-zero status.  mpmgpu_last_error() gives the message.
 *   - A context is driven from one host thread; it is not re-entrant.
 *   - Unsupported options are refused with MPMGPU_ERR_UNSUPPORTED: there is no
 *     CPU fallback.
 */
#ifndef NAIRN_MPM_GPU_H
#define NAIRN_MPM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPMGPU_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
    MPMGPU_OK = 0,
    MPMGPU_ERR_INVALID = 1,      /* bad argument or inconsistent sizes          */
    MPMGPU_ERR_UNSUPPORTED = 2,  /* option the device path does not implement   */
    MPMGPU_ERR_CUDA = 3,         /* CUDA runtime error                          */
    MPMGPU_ERR_OOM = 4,          /* device allocation failed / over HBM budget  */
    MPMGPU_ERR_NAN = 5,          /* a particle position became NaN (LEFT_GRID_NAN) */
    MPMGPU_ERR_LEFT_GRID = 6,    /* a particle left the grid (LEFT_GRID)        */
    MPMGPU_ERR_CPDI_NODES = 7,   /* CPDI domain needs more nodes than allowed   */
    MPMGPU_ERR_TIMEOUT = 8,      /* a bounded device wait gave up               */
    MPMGPU_ERR_BUSY = 9,         /* request still running (serving API)        */
    MPMGPU_ERR_RANGE = 10        /* a deterministic node sum met a contribution
                                    beyond its bound (NaN or infinite values)  */
};

/* ---- analysis options (values follow the reference's constants) -------- */
/* MPMMethod: NairnMPM/src/System/MPMPrefix.hpp:110 */
enum { MPMGPU_USF = 0, MPMGPU_USAVG = 2, MPMGPU_USL = 3 };
/* GIMP type: NairnMPM/src/System/MPMPrefix.hpp:127-140 */
enum {
    MPMGPU_SHAPE_LINEAR = 0,  /* Classic (POINT_GIMP)        */
    MPMGPU_SHAPE_UGIMP = 1,   /* uGIMP (UNIFORM_GIMP)        */
    MPMGPU_SHAPE_BGIMP = 5,   /* B2GIMP (BSPLINE_GIMP)       */
    MPMGPU_SHAPE_BSPLINE = 6, /* B2SPLINE (BSPLINE)          */
    MPMGPU_SHAPE_LCPDI = 10,  /* lCPDI (LINEAR_CPDI)         */
    MPMGPU_SHAPE_QCPDI = 11   /* qCPDI (QUADRATIC_CPDI), 2D only: nine domain points
                                 (MatPoint2D::GetCPDINodesAndWeights, MatPoint2D.cpp:574-640) */
};
/* Analysis type (np): NairnMPM/src/System/MPMPrefix.hpp:115 */
enum { MPMGPU_PLANE_STRAIN = 10, MPMGPU_THREED = 12 };
/* Arithmetic of the transfers (P2G/G2P and grid); the constitutive update,
 * deformation gradient and particle displacement are FP64 in both modes. */
enum { MPMGPU_PREC_FP64 = 0, MPMGPU_PREC_MIXED = 1 };
/* Node sums (P2G mass and momentum, internal forces, the second extrapolation,
 * contact terms): hardware FP64/FP32 atomics, whose summation order -- and so
 * the last bits of a result -- varies from run to run; or exact integer sums
 * (each contribution rounded once to a multiple of 2^-102 of the step's bound
 * on it, then added as 64-bit integer limbs), which give the same bits in every
 * run whatever the thread scheduling, launch shape or particle order
 * (single-run contexts only).  With MPMGPU_P2G_ATOMIC the mixed mode
 * accumulates each block's scatters (one material field; linear, uGIMP,
 * B2SPLINE or B2GIMP shape functions) in a shared-memory node tile of FP32
 * two-sum pairs and adds every touched node once to the FP64 node columns;
 * MPMGPU_P2G_UNTILED scatters every (particle, node) pair straight to the
 * node columns instead. */
enum { MPMGPU_P2G_ATOMIC = 0, MPMGPU_P2G_DETERMINISTIC = 1, MPMGPU_P2G_UNTILED = 2 };
/* Material types: Common/Read_XML/MaterialController.cpp:105-231.  Type 35 is
 * RigidMaterial in multimaterial mode (RIGIDCONTACTMATERIAL,
 * NairnMPM/src/Materials/RigidMaterial.hpp:14): particles that move at their
 * own constant velocity and take part in contact only; their mass is their
 * volume in mm^3 (the reference's rho = 1 for rigid materials), the rho of
 * their MpmGpuMaterial is ignored, and they need multimaterial contact. */
enum { MPMGPU_MAT_ISOTROPIC = 1, MPMGPU_MAT_ISOPLASTICITY = 9, MPMGPU_MAT_NEOHOOKEAN = 28,
       MPMGPU_MAT_RIGID_CONTACT = 35 };

/* Structured background grid, as MPMReadHandler::grid() builds it
 * (NairnMPM/src/Read_MPM/Generators.cpp:1675-1990): nx*ny(*nz) elements
 * including the one-cell border layer, nodes numbered x fastest.  The node
 * coordinates are passed so element extents match the host's bit for bit
 * (ElementBase::FindExtent, Common/Elements/ElementBase.cpp:62). */
typedef struct {
    int32_t dim;              /* 2 or 3                                      */
    int32_t nx, ny, nz;       /* element counts (nz = 0 in 2D)               */
    double xmin, ymin, zmin;  /* MeshInfo xmin,ymin,zmin (grid origin)       */
    double dx, dy, dz;        /* MeshInfo grid.x,.y,.z (dz = 0 in 2D)        */
    double thickness;         /* 2D thickness (mm); ignored in 3D            */
    const double *xnodes;     /* nx+1 node x coordinates                     */
    const double *ynodes;     /* ny+1 node y coordinates                     */
    const double *znodes;     /* nz+1 node z coordinates (NULL in 2D)        */
} MpmGpuGrid;

/* Material input properties in XML units (MPa, g/cm^3).  The library derives
 * the specific constants exactly as the reference's VerifyAndLoadProperties. */
typedef struct {
    int32_t type;             /* MPMGPU_MAT_*                                */
    int32_t field;            /* material velocity field (0 .. nfields-1)    */
    double rho;               /* g/cm^3                                      */
    double E, nu;             /* isotropic (types 1, 9)                      */
    double yield, Ep;         /* type 9, linear hardening (MPa)              */
    double G, K;              /* type 28 (MPa)                               */
    int32_t UJOption;         /* type 28 volumetric energy option (0..2)     */
    int32_t pad;
} MpmGpuMaterial;

/* Multimaterial contact (config with more than one material field).  Coulomb
 * friction law CoulombFriction (NairnMPM/src/Materials/CoulombFriction.cpp). */
typedef struct {
    int32_t enabled;
    int32_t normals;          /* MeshInfo materialNormalMethod (MeshInfo.hpp:31):
                                 0 MAXIMUM_VOLUME_GRADIENT, 1 MAXIMUM_VOLUME,
                                 2 AVERAGE_MAT_VOLUME_GRADIENTS, 5 LINEAR_REGRESSION,
                                 6 LOGISTIC_REGRESSION (the reference's default;
                                 in a batch 5 and 6 need lr_links); others refused */
    double friction;          /* Coulomb coefficient; <0 stick; 0 frictionless */
    double contact_cutoff;    /* position-based contact cutoff (cells); <0 displacement based */
    double rigid_gradient_bias;
} MpmGpuContact;

/* One nodal velocity condition (NodalVelBC, NairnMPM/src/Boundary_Conditions/NodalVelBC.cpp).
 * Applied in list order, as VelocityBCLoop does. */
typedef struct {
    int32_t node;             /* 1-based node number                         */
    int32_t dir;              /* 1 = x, 2 = y, 4 = z                         */
    double value;             /* velocity (mm/s) in that direction           */
    double ftime;             /* active for t >= ftime                       */
} MpmGpuVelBC;

typedef struct {
    int32_t np;               /* MPMGPU_PLANE_STRAIN or MPMGPU_THREED        */
    int32_t method;           /* MPMGPU_USF / _USAVG / _USL                  */
    int32_t shape;            /* MPMGPU_SHAPE_*                              */
    int32_t precision;        /* MPMGPU_PREC_*                               */
    int32_t p2g;              /* MPMGPU_P2G_*                                */
    int32_t inc_defgrad_terms;/* Exponential() terms for hyperelastic (2D: 2, 3D: 1) */
    int32_t nfields;          /* material velocity fields (1 unless contact) */
    int32_t sort_interval;    /* re-sort particles by cell every k steps (>=1) */
    double timestep;          /* s                                           */
    double fraction_usf;      /* USAVG split (0.5)                           */
    /* PeriodicXPIC custom task (NairnMPM/src/Custom_Tasks/PeriodicXPIC.cpp):
     * XPIC(k) or FMPM(k) grid-to-particle updates on every xpic_period-th step
     * (steps counted from 1 at time 0, step s at time (s-1) dt), FLIP on the
     * others.  xpic_order 0: FLIP on every step. */
    int32_t xpic_order;       /* XPICOrder or FMPMOrder (k >= 1; 1 is PIC)   */
    int32_t xpic_fmpm;        /* 1: FMPM(k) (FMPMOrder), 0: XPIC(k)          */
    int32_t xpic_period;      /* periodicSteps (>= 1 when xpic_order > 0)    */
    int32_t xpic_reserved;    /* 0                                           */
} MpmGpuOptions;

/* Particle state, structure of arrays, length n each.  Fields mirror MPMBase
 * (NairnMPM/src/MPM_Classes/MPMBase.hpp:225-263).  In 2D the z arrays and the
 * xz/yz components may be NULL.  The deformation gradient is carried the way
 * MatPoint2D/3D store it: strain ep (normal + engineering shear) and rotation
 * wrot, F = I + ep/2 +- wrot/2 off the diagonal. */
typedef struct {
    int64_t n;
    double *x, *y, *z;               /* position (mm)                        */
    double *vx, *vy, *vz;            /* velocity (mm/s)                      */
    double *x0, *y0, *z0;            /* original position (mm)               */
    double *mass;                    /* g                                    */
    int32_t *mat;                    /* 0-based material index               */
    int32_t *elem;                   /* 0-based element (ElemID())           */
    double *lpx, *lpy, *lpz;         /* dimensionless semi-size (mpm_lp)     */
    double *exx, *eyy, *ezz, *exy, *exz, *eyz;   /* ep                       */
    double *wxy, *wxz, *wyz;         /* wrot                                 */
    double *sxx, *syy, *szz, *sxy, *sxz, *syz;   /* sp (specific stress)     */
    double *pressure;                /* specific pressure (type 9 deviatoric split) */
    double *pxx, *pyy, *pzz, *pxy, *pxz, *pyz;   /* eplast (plastic strain or B) */
    double *hist0, *hist1;           /* history doubles (alpha; J, Jres)     */
    double *work, *plast;            /* work and plastic energy per unit mass */
} MpmGpuParticles;

/* ---- single-run context --------------------------------------------------- */
typedef struct MpmGpuCtx MpmGpuCtx;

/* Library ABI version (MPMGPU_ABI_VERSION). */
int mpmgpu_abi_version(void);

/* Create a context on the current CUDA device for one run.
 * Replaces the set-up the reference does in NairnMPM::CMPreparations
 * (NairnMPM.cpp:135-168) for the step's own data. */
int mpmgpu_create(const MpmGpuGrid *grid, const MpmGpuOptions *opts, MpmGpuCtx **out);

/* Materials (index = MpmGpuParticles.mat).  Replaces the property copies of
 * MaterialBase::GetCopyOfMechanicalProps (MaterialBase.hpp:144). */
int mpmgpu_set_materials(MpmGpuCtx *ctx, const MpmGpuMaterial *mats, int32_t nmat);

/* Contact settings (MeshInfo::MaterialContactPairs, MeshInfo.cpp:1231). */
int mpmgpu_set_contact(MpmGpuCtx *ctx, const MpmGpuContact *contact);

/* Nodal velocity conditions in the reference's list order (firstVelocityBC). */
int mpmgpu_set_velocity_bcs(MpmGpuCtx *ctx, const MpmGpuVelBC *bcs, int32_t nbc);

/* Copy particle state host -> device (the mpm[] sync before the first step). */
int mpmgpu_upload_particles(MpmGpuCtx *ctx, const MpmGpuParticles *p);

/* Advance nsteps explicit steps from time t0 (s).  One call replaces
 * nsteps passes of NairnMPM::MPMStep (NairnMPM.cpp:284-335). */
int mpmgpu_step(MpmGpuCtx *ctx, int32_t nsteps, double t0);

/* Copy particle state device -> host (the mpm[] sync before ArchiveResults,
 * NairnMPM.cpp:199).  Arrays of p must be allocated by the caller. */
int mpmgpu_download_particles(MpmGpuCtx *ctx, MpmGpuParticles *p);

/* Message of the last failing call on ctx (static storage when ctx is NULL). */
const char *mpmgpu_last_error(const MpmGpuCtx *ctx);

/* Free all device memory of ctx. */
void mpmgpu_destroy(MpmGpuCtx *ctx);

/* Milliseconds of device time spent in each kernel family during the last
 * mpmgpu_step call (CUDA events on the context stream); names[i] is static.
 * Returns the number of entries written (<= cap).  Mirrors the per-task
 * profile NairnMPM prints (NairnMPM.cpp:246-275, MPMTask.cpp:57-72). */
int mpmgpu_profile(const MpmGpuCtx *ctx, const char **names, double *ms, int32_t cap);

/* Stable radix sort of n particles by element (cell) index, the ordering step
 * of the GPU path.  The reference assigns the element in
 * ResetElementsTask::ResetElement / MeshInfo::FindElementFromPoint
 * (ResetElementsTask.cpp:196-228, MeshInfo.cpp:593-633) and keeps mpm[] order;
 * the device re-orders particles by that element each step.  d_elem and
 * d_perm are device pointers of n ints; each d_elem[i] must lie in
 * [0, nelems).  On return d_perm[j] is the slot of the j-th particle in
 * (element, slot) order -- equal elements keep their slot order, so the result
 * is bit-for-bit a stable argsort.  stream is a cudaStream_t (NULL: legacy
 * default stream); the call synchronizes it.  Allocates its scratch with
 * cudaMalloc. */
int mpmgpu_sort_by_cell(const int32_t *d_elem, int32_t n, int32_t nelems, int32_t *d_perm, void *stream);

/* Largest particle count mpmgpu_sort_by_cell_noalloc accepts. */
#define MPMGPU_NOALLOC_MAX_PARTICLES 131072

/* Allocation-free variant of mpmgpu_sort_by_cell, for callers that cannot
 * call cudaMalloc: a host integration whose device memory is reserved up front
 * (for example a serving loop that budgets HBM per run and must not allocate
 * while runs are in flight), or code where cudaMalloc's implicit device-wide
 * synchronisation is not acceptable.  It has no counterpart in the reference.
 * Same arguments and result as mpmgpu_sort_by_cell, for at most
 * MPMGPU_NOALLOC_MAX_PARTICLES particles; larger n is rejected with
 * MPMGPU_ERR_INVALID before any device work.  Its scratch is a fixed device
 * array inside this library (2.25 MiB per GPU, held until the process
 * exits), so it calls no cudaMalloc, cudaFree or allocating library routine.
 * Every call looks up that array's device address in the context current on
 * the calling thread (cudaGetSymbolAddress, which allocates nothing); the
 * first call on a device also loads the library's module there, so make that
 * first call before any stream capture.  Nothing is cached between calls, so
 * a cudaDeviceReset or another context made current on the device leaves
 * nothing stale for the caller to redo.  A CUDA error already pending when
 * the call starts is returned as MPMGPU_ERR_CUDA (and left pending) before
 * any work.  All calls share the one array, which keeps the last call's
 * contents: calls whose work overlaps on a GPU (different streams or host
 * threads without ordering) race and must be serialised by the caller.  The
 * call synchronizes `stream`. */
int mpmgpu_sort_by_cell_noalloc(const int32_t *d_elem, int32_t n, int32_t nelems, int32_t *d_perm, void *stream);

/* ---- archive output ----------------------------------------------------------
 * The particle records of a NairnMPM archive file (ArchiveData::ArchiveResults,
 * NairnMPM/src/System/ArchiveData.cpp:807-1100), packed on the device from the
 * current particle state and copied to the host in the host's particle order,
 * so the host writes its 64-byte header (ArchiveData::SetArchiveHeader) and
 * then the buffer -- without downloading the particle state into mpm[].
 * mpm_order is the MPMArchiveOrder string; it is padded and its forced items
 * set as ArchiveData::CalcArchiveSize does.  Items the device does not hold
 * (temperature, heat energy, element crossings, damage normals, spin, history
 * values beyond the first, particle size) and big-endian ('m') archives are
 * refused with MPMGPU_ERR_UNSUPPORTED.  Initial material angles are zero. */

/* Bytes of one particle record for a dimension (2 or 3) and order string, or
 * the negated status when the order cannot be packed. */
int64_t mpmgpu_archive_record_size(int32_t dim, const char *mpm_order);

/* Pack the records of all particles into host_records (capacity bytes, at
 * least n * record size); thickness is the 2D particles' thickness (mm). */
int mpmgpu_archive_records(MpmGpuCtx *ctx, const char *mpm_order, double thickness, void *host_records,
                           int64_t capacity);

/* The same records without waiting for them: packed in stream order after the
 * steps enqueued so far, then copied to host_records on a copy stream while
 * later mpmgpu_step calls run.  host_records should be pinned
 * (mpmgpu_host_register); it must stay valid and is complete only after
 * mpmgpu_archive_wait.  A later archive call waits for this copy first. */
int mpmgpu_archive_records_async(MpmGpuCtx *ctx, const char *mpm_order, double thickness, void *host_records,
                                 int64_t capacity);
/* Wait for the copy of the last mpmgpu_archive_records_async (no-op if none). */
int mpmgpu_archive_wait(MpmGpuCtx *ctx);

/* ---- extensions without a counterpart in the reference ----------------------
 * Host-integration and measurement helpers of this library; a NairnMPM
 * integration does not need them. */

/* mpmgpu_step plus the device time of the enqueued steps (CUDA events on the
 * context stream), in milliseconds. */
int mpmgpu_step_timed(MpmGpuCtx *ctx, int32_t nsteps, double t0, double *ms);

/* Per-kernel event timing for later mpmgpu_step calls (read with mpmgpu_profile). */
int mpmgpu_set_profiling(MpmGpuCtx *ctx, int32_t on);

/* Pick the cell-sort interval of this context by timing: about trial_steps
 * real steps (from time t0, as mpmgpu_step; whole chunks of 8, the candidates
 * taking turns) at each interval 1, 2, 4 and 8; the fastest is kept.  Results
 * do not depend on the interval beyond the order of atomic sums.
 * *steps_taken (a multiple of 32) is how far the simulation advanced;
 * *best_interval and *ms_per_step describe the choice. */
int mpmgpu_autotune_sort(MpmGpuCtx *ctx, int32_t trial_steps, double t0, int32_t *best_interval,
                         double *ms_per_step, int32_t *steps_taken);

/* The context's cudaStream_t, as an opaque pointer. */
void *mpmgpu_stream(MpmGpuCtx *ctx);

/* Number of kernels the context has launched so far. */
long long mpmgpu_launch_count(const MpmGpuCtx *ctx);

/* Page-lock caller memory (cudaHostRegister) so uploads and downloads of
 * particle columns run as asynchronous DMA; unregister before freeing. */
int mpmgpu_host_register(void *ptr, uint64_t bytes);
int mpmgpu_host_unregister(void *ptr);

/* Page-locked host memory allocated by the driver (cudaHostAlloc), for a host
 * that keeps its particle columns in memory of the library's choosing;
 * mpmgpu_host_free releases it.  Copies to memory the driver allocated run at
 * the host link's rate in both directions, where registered caller memory was
 * measured at a third of it for device-to-host copies in some runs. */
int mpmgpu_host_alloc(uint64_t bytes, void **ptr);
void mpmgpu_host_free(void *ptr);

/* Extension: advance nsteps on particle state that stays in host memory.  The
 * step kernels read and write the caller's columns in place over the host link
 * (NVLink-C2C on Grace systems), so the link traffic overlaps the kernels'
 * arithmetic instead of preceding and following it as the copies of
 * mpmgpu_upload_particles / mpmgpu_download_particles do.  Every non-null
 * column of *particles, and mat and elem (required), must lie inside one block
 * from mpmgpu_host_alloc; a null column is taken from the context's uploaded
 * state (on the device).  particles->n must equal the particle count of the
 * last mpmgpu_upload_particles, which sizes the work arrays; the device copy of
 * that state is not advanced.  The host order is kept (no cell sort).  The call
 * returns when the steps have completed; the caller must not touch the columns
 * meanwhile.  Errors as mpmgpu_step, plus MPMGPU_ERR_INVALID for a column
 * outside the blocks or material/element indices out of range (checked before
 * the steps).  No counterpart in the reference (its particle state is host
 * memory throughout). */
int mpmgpu_step_host(MpmGpuCtx *ctx, MpmGpuParticles *particles, int32_t nsteps, double t0);

/* Extension (measurement): FMA throughput of the current device in TFLOP/s
 * (2 flops per FMA), measured by one kernel of independent FMA chains timed
 * with CUDA events; *ms receives the kernel time.  The FP64 path of the step
 * is bound by the FP64 pipe, so its roofline is taken against this rate.  No
 * counterpart in the reference. */
int mpmgpu_fp64_fma_rate(int32_t iters, double *tflops, double *ms);
int mpmgpu_fp32_fma_rate(int32_t iters, double *tflops, double *ms);

/* ---- batch: many independent runs in one graph-captured step ----------------
 * A batch holds the state of many runs on the device and advances all of them
 * with one launch of each step kernel.  The runs share the batch's analysis
 * options (dimension, method, shape functions, precision) and
 * differ in grid, materials, velocity conditions, particles, time step and
 * step count.  Each run is the same computation as a single-run context given
 * the same input (mpmgpu_create ... mpmgpu_step): only the order of the atomic
 * node sums differs.  It has no counterpart in the reference, which runs one
 * analysis per process (NairnMPM::StartAnalysis, NairnMPM.cpp:91-218).  One
 * host thread drives a batch. */
typedef struct MpmGpuBatch MpmGpuBatch;

typedef struct {
    int32_t np;               /* MPMGPU_PLANE_STRAIN or MPMGPU_THREED        */
    int32_t method;           /* MPMGPU_USF / _USAVG / _USL                  */
    int32_t shape;            /* MPMGPU_SHAPE_LINEAR, _UGIMP, _BGIMP, _BSPLINE or _LCPDI */
    int32_t precision;        /* MPMGPU_PREC_*                               */
    int32_t sort_interval;    /* cell sort every k steps (0: never)          */
    int32_t block;            /* threads per block of particle kernels (0: 256) */
    int32_t max_runs;         /* run slots                                   */
    int32_t max_materials;    /* material slots (sum over resident runs)     */
    int64_t max_particles;    /* particle slots (sum over resident runs)     */
    int64_t max_nodes;        /* grid nodes (sum over resident runs)         */
    double fraction_usf;      /* USAVG split (0 -> 0.5)                      */
    int32_t inc_defgrad_terms;/* Exponential() terms of hyperelastic F (0: 2 in 2D, 1 in 3D) */
    int32_t max_fields;       /* material velocity fields per run (0, 1: single
                                 material mode; up to 8 for multimaterial contact) */
    int32_t lr_links;         /* particle-to-contact-node links reserved per
                                 particle slot for regression normals (methods
                                 5, 6; needs max_fields >= 2): 0 refuses those
                                 methods; 64 in 3D, 16 in 2D always suffice; a
                                 run whose links do not fit fails with
                                 MPMGPU_ERR_RANGE */
    int32_t xpic_order;       /* PeriodicXPIC of every run (MpmGpuOptions;  */
    int32_t xpic_fmpm;        /* each run counts its own steps from 1);    */
    int32_t xpic_period;      /* one material field only; 0: FLIP          */
} MpmGpuBatchOptions;

/* run states returned by mpmgpu_batch_run_state; a failed run reports the
 * negated status (-MPMGPU_ERR_LEFT_GRID, -MPMGPU_ERR_NAN) and stops stepping */
enum { MPMGPU_RUN_EMPTY = 0, MPMGPU_RUN_RUNNING = 1, MPMGPU_RUN_FINISHED = 2 };

typedef struct {
    int32_t runs, running;    /* resident runs, runs still stepping          */
    int32_t block, sort_interval;
    int64_t particles_used;   /* particle slots in use (including dead ones) */
    int64_t particles_dead;   /* slots of removed runs, dropped at the next sort */
    int64_t nodes_used;       /* extent of the node arena in use             */
    int64_t steps;            /* batched steps taken                         */
    int64_t launches;         /* kernels launched (graph nodes included)     */
} MpmGpuBatchInfo;

/* Device bytes mpmgpu_batch_create allocates for these capacities. */
int64_t mpmgpu_batch_bytes(const MpmGpuBatchOptions *opts);
int mpmgpu_batch_create(const MpmGpuBatchOptions *opts, MpmGpuBatch **out);
/* Admit one run; *run_id receives its slot.  contact (may be NULL) enables
 * multimaterial contact for the run; its materials' field numbers must be
 * below the batch's max_fields.  MPMGPU_ERR_BUSY: not enough free
 * run slots, particles, nodes or material slots now (retry after removals);
 * MPMGPU_ERR_OOM: the run is larger than the batch's capacities. */
int mpmgpu_batch_add_run(MpmGpuBatch *b, const MpmGpuGrid *grid, const MpmGpuMaterial *mats, int32_t nmat,
                         const MpmGpuVelBC *bcs, int32_t nbc, const MpmGpuContact *contact,
                         const MpmGpuParticles *p, double timestep, int32_t nsteps, int32_t *run_id);
/* Advance every running run by nsteps steps (a run stops at its own count). */
int mpmgpu_batch_step(MpmGpuBatch *b, int32_t nsteps);
int mpmgpu_batch_step_timed(MpmGpuBatch *b, int32_t nsteps, double *ms);
int mpmgpu_batch_run_state(const MpmGpuBatch *b, int32_t run_id, int32_t *state, int32_t *steps_done);
/* Particle state of a run in its upload order (x0 columns are not kept). */
int mpmgpu_batch_download_run(MpmGpuBatch *b, int32_t run_id, MpmGpuParticles *out);
/* Remove a run (downloading it first when out is not NULL) and free its slots. */
int mpmgpu_batch_remove_run(MpmGpuBatch *b, int32_t run_id, MpmGpuParticles *out);
/* Particle-kernel block size (64, 128, 256) and sort interval. */
int mpmgpu_batch_set_tuning(MpmGpuBatch *b, int32_t block, int32_t sort_interval);
/* Time candidate block sizes and sort intervals on real steps of the resident
 * runs (the trial steps count as steps of those runs) and keep the fastest. */
int mpmgpu_batch_autotune(MpmGpuBatch *b, int32_t trial_steps, int32_t *block, int32_t *sort_interval,
                          double *ms_per_step);
int mpmgpu_batch_info(const MpmGpuBatch *b, MpmGpuBatchInfo *info);
const char *mpmgpu_batch_last_error(const MpmGpuBatch *b);
void *mpmgpu_batch_stream(MpmGpuBatch *b);
void mpmgpu_batch_destroy(MpmGpuBatch *b);

/* ---- server: continuous batching of independent requests ------------------
 * A server keeps one batch per dimension (2D plane strain, 3D) sized within
 * an HBM budget and runs a host thread that admits queued requests as run
 * slots and memory free up, advances all admitted runs together in rounds of
 * steps_per_round batched steps (2D and 3D batches overlap on the device) and
 * retires finished runs.  Each result equals the run computed alone (within
 * the mode's tolerance; only the order of atomic node sums differs).  No
 * counterpart in the reference.  submit/poll/wait/drain/release/stats may be
 * called from any host thread. */
typedef struct MpmGpuServer MpmGpuServer;

typedef struct {
    int32_t method;             /* MPMGPU_USF / _USAVG / _USL                  */
    int32_t shape;              /* MPMGPU_SHAPE_LINEAR, _UGIMP, _BGIMP, _BSPLINE or _LCPDI */
    int32_t precision;          /* MPMGPU_PREC_*                               */
    int32_t max_runs;           /* run slots per dimension                     */
    int32_t steps_per_round;    /* steps between admissions/retirements (0: 10) */
    int32_t backfill;           /* 1: a later request that fits may pass one that does not */
    int32_t sort_interval;      /* cell sort every k steps (0: 1)              */
    int32_t block;              /* particle-kernel block size (0: 256)         */
    int64_t hbm_budget_bytes;   /* device memory the server holds (both batches) */
    double frac_3d;             /* share of the budget for 3D runs (0..1)      */
    double nodes_per_particle;  /* node slots per particle slot (0: 0.5)       */
    double fraction_usf;        /* USAVG split (0 -> 0.5)                      */
    int64_t max_resident_particles; /* admit while the running runs hold fewer
                                   particles than this (0: no cap); a request
                                   is always admitted when nothing runs      */
    int32_t order;              /* admission order: 0 arrival (FIFO), 1 least
                                   work first (particles x steps), 2 deadline:
                                   least work first, a request admitted only
                                   while every running request's predicted
                                   latency stays within slowdown_target times
                                   its predicted time alone, and while the
                                   resident particles of its dimension stay
                                   within the load at which the fitted step
                                   time reaches 90 % of the batch's asymptotic
                                   throughput (see below)                    */
    int32_t max_fields;         /* material velocity fields per run (0: 1)     */
    int32_t lr_links;           /* links per particle slot for regression normals
                                   (MpmGpuBatchOptions; capped at 16 in 2D)   */
    int32_t xpic_order, xpic_fmpm, xpic_period;  /* PeriodicXPIC of every request
                                   (MpmGpuBatchOptions)                       */
    double slowdown_target;     /* order 2: the bound k (0: 4).  The server fits
                                   step time = a + b x resident particles per
                                   dimension from CUDA-event timings of its
                                   rounds; a request of n particles and s steps
                                   takes s (a + b n) alone.  A queued request
                                   is admitted when nothing runs, or when with
                                   it resident every running request r (and
                                   itself) still has elapsed_r + steps_left_r x
                                   (a + b R) <= k x its time alone; requests
                                   already past that bound do not block, and a
                                   queued request past it goes first.        */
} MpmGpuServerOptions;

enum { MPMGPU_REQ_QUEUED = 1, MPMGPU_REQ_RUNNING = 2, MPMGPU_REQ_DONE = 3, MPMGPU_REQ_FAILED = 4 };

typedef struct {
    int32_t state;              /* MPMGPU_REQ_*                                */
    int32_t status;             /* MPMGPU_OK, or why a request failed          */
    int32_t steps_done, pad;
    double queue_ms;            /* submit -> admission (or now)                */
    double run_ms;              /* admission -> completion (or now)            */
    double total_ms;            /* submit -> completion (or now)               */
} MpmGpuRequestInfo;

typedef struct {
    int64_t submitted, completed, failed, queued, running;
    int64_t particle_steps;     /* sum of particles x steps of completed requests */
    int64_t rounds;             /* stepping rounds                             */
    int64_t reserved_bytes;     /* device bytes held by the server's batches   */
    double busy_ms;             /* wall time of the rounds that stepped        */
} MpmGpuServerStats;

int mpmgpu_server_create(const MpmGpuServerOptions *opts, MpmGpuServer **out);

/* Extension: the deadline order's admission rule (order 2 above) as a pure
 * function, for hosts that schedule runs themselves.  a_ms, b_ms: step time
 * a + b R of R resident particles; running: n, steps_left, elapsed_ms and
 * steps_total of each running request; (cand_n, cand_steps, cand_waited_ms):
 * the queued request.  Returns 1 to admit, 0 to wait, or -MPMGPU_ERR_INVALID. */
typedef struct {
    int64_t n;
    int32_t steps_left, steps_total;
    double elapsed_ms;
} MpmGpuRunLoad;
int mpmgpu_server_admits(double a_ms, double b_ms, double slowdown_target, const MpmGpuRunLoad *running,
                         int32_t nrunning, int64_t cand_n, int32_t cand_steps, double cand_waited_ms);
/* Queue one run.  The particle arrays of p are borrowed: they must stay valid
 * and unchanged until the request is done or failed; they are read at
 * admission and receive the final state (upload order) at completion.  Grid
 * coordinates, materials and velocity conditions are copied. */
int mpmgpu_server_submit(MpmGpuServer *s, const MpmGpuGrid *grid, const MpmGpuMaterial *mats, int32_t nmat,
                         const MpmGpuVelBC *bcs, int32_t nbc, const MpmGpuContact *contact, MpmGpuParticles *p,
                         double timestep, int32_t nsteps, int64_t *request_id);
int mpmgpu_server_poll(MpmGpuServer *s, int64_t request_id, MpmGpuRequestInfo *info);
/* Block until the request is done or failed; MPMGPU_ERR_TIMEOUT after timeout_s. */
int mpmgpu_server_wait(MpmGpuServer *s, int64_t request_id, double timeout_s);
/* Block until no request is queued or running; MPMGPU_ERR_TIMEOUT after timeout_s. */
int mpmgpu_server_drain(MpmGpuServer *s, double timeout_s);
/* Forget a finished request (its record and timings). */
int mpmgpu_server_release(MpmGpuServer *s, int64_t request_id);
int mpmgpu_server_stats(MpmGpuServer *s, MpmGpuServerStats *stats);
const char *mpmgpu_server_last_error(const MpmGpuServer *s);
/* Stop the loop and free the device memory.  Requests still queued or
 * running end as failed (MPMGPU_ERR_BUSY, "server stopped ...") and waiters
 * are woken, but every mpmgpu_server_wait / _drain must have returned before
 * this call: the server, its mutex and its condition variable are freed. */
void mpmgpu_server_destroy(MpmGpuServer *s);

#ifdef __cplusplus
}
#endif

#endif /* NAIRN_MPM_GPU_H */
