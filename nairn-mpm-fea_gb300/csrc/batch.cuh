// batch.cuh -- many independent MPM runs advanced together on one GPU.
// Included by batch.cu; implements the
// mpmgpu_batch_* entry points of include/nairn_mpm_gpu.h.
//
// Runs share arenas: particle slots (structure of arrays, one run id per
// slot), grid nodes (each run owns a contiguous node range), cells (the sort
// key space) and material slots.  A batched step launches every step kernel
// once over all slots and all used nodes; each thread finds its run in the
// device run table (DevRun), so runs of different sizes, grids, materials and
// time steps advance together and each stops after its own step count.  The
// step (optionally preceded by the cell sort) is captured once in a CUDA graph
// and replayed until the set of runs changes.  The particle arena has two
// buffers that the sort ping-pongs between; one graph is kept per buffer.
// Removed runs leave dead slots; the next sort puts them last and the slot
// count shrinks, so the sort is also the compaction.
#pragma once

#include <map>

namespace {

// first-fit allocator of integer ranges in [0, cap)
struct RangeAlloc {
    long long cap = 0;
    std::map<long long, long long> free;  // start -> length
    void init(long long c) {
        cap = c;
        free.clear();
        if (c > 0) free[0] = c;
    }
    long long alloc(long long n) {
        if (n <= 0) return -1;
        for (auto it = free.begin(); it != free.end(); ++it) {
            if (it->second >= n) {
                const long long s = it->first, len = it->second;
                free.erase(it);
                if (len > n) free[s + n] = len - n;
                return s;
            }
        }
        return -1;
    }
    void release(long long s, long long n) {
        if (n <= 0) return;
        auto it = free.emplace(s, n).first;
        auto nx = std::next(it);
        if (nx != free.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free.erase(nx);
        }
        if (it != free.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free.erase(it);
            }
        }
    }
    // one past the highest used index
    long long high_water() const {
        if (free.empty()) return cap;
        auto last = std::prev(free.end());
        return last->first + last->second == cap ? last->first : cap;
    }
};

struct BatchRun {
    bool used = false;
    int state = 0;  // MPMGPU_RUN_* (or the negated status of a failed run)
    int np = 0;
    long long node_base = 0, nnodes = 0, cell_base = 0, nelems = 0, mat_base = 0, nmat = 0;
    int steps_total = 0, steps_done = 0;
    bool lr = false;               // regression contact normals (methods 5, 6)
    bool rigid = false;            // rigid contact materials
    std::vector<MpmGpuVelBC> bcs;  // batch-global 1-based node numbers
};

// admission of np particles at slots [start, start+np): slot order = host
// order, run id, material index moved into the run's material slots
__global__ void k_batch_admit(int *mat, const int *elem, int *orig, int *run, int start, int np, int r, int mat_base,
                              int nmat, int nelems, unsigned *flag) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= np) return;
    const int i = start + j;
    orig[i] = j;
    run[i] = r;
    const int m = mat[i], e = elem[i];
    if (m < 0 || m >= nmat || e < 0 || e >= nelems) atomicOr(flag, 8u);
    mat[i] = m + mat_base;
}

__global__ void k_fill_int(int *a, long long start, long long n, int v) {
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j < n) a[start + j] = v;
}

// slots of run r -> packed columns of np values in the run's original order
__global__ void k_batch_extract(const double *pblock, int cap, const int *mat, const int *elem, const int *orig,
                                const int *run, int n, int r, int mat_base, double *out, int *iout, int np,
                                int ncols) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || run[i] != r) return;
    const int o = orig[i];
    for (int k = 0; k < ncols; k++) out[(size_t)k * np + o] = pblock[(size_t)k * cap + i];
    iout[o] = mat[i] - mat_base;
    iout[np + o] = elem[i];
}

// mark the slots of run r empty
__global__ void k_batch_kill(int *run, int n, int r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && run[i] == r) run[i] = -1;
}

// sort keys of a batch: the run's cell base + element; empty slots last
__global__ void k_batch_keys(const int *elem, const int *run, const DevRun *runs, int *keys, int *vals, int n,
                             int dead_key) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = run[i];
    keys[i] = r < 0 ? dead_key : runs[r].cell_base + elem[i];
    vals[i] = i;
}

// dst[k*cap + j] = src[k*cap + perm[j]] for the first n slots of every column
template <typename T>
__global__ void k_gather_cap(const T *__restrict__ src, T *__restrict__ dst, const int *__restrict__ perm, int n,
                             int ncols, int cap) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int s = perm[j];
    for (int k = 0; k < ncols; k++) dst[(size_t)k * cap + j] = src[(size_t)k * cap + s];
}

// A new run's node range: clear the velocity and acceleration columns its
// nodes may keep from an earlier run (a failed one may have left non-finite
// values); the separable gradient sums read every node of a particle's window,
// weighting those outside its support by zero.
__global__ void k_clear_run_nodes(DevNodes nd, long long nbase, long long nn, int nf, int fstride) {
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= nn) return;
    for (int f = 0; f < nf; f++) {
        const long long k = f * (long long)fstride + nbase + j;
        nd.vx[k] = nd.vy[k] = nd.vz[k] = 0.;
        nd.ax[k] = nd.ay[k] = nd.az[k] = 0.;
        nd.vhx[k] = nd.vhy[k] = nd.vhz[k] = 0.f;
        nd.vlx[k] = nd.vly[k] = nd.vlz[k] = 0.f;
        nd.bx[k] = nd.by[k] = nd.bz[k] = 0.f;
    }
}

// step-start clear of the accumulated node columns of the used node range
// (every material field, and the contact terms when there are several)
template <bool MIX>
__global__ void k_clear_nodes(DevNodes nd, int nn, int nf, int fstride) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    for (int f = 0; f < nf; f++) {
        const int k = f * fstride + n;
        nd.mass[k] = 0.;
        nd.px[k] = nd.py[k] = nd.pz[k] = 0.;
        nd.fx[k] = nd.fy[k] = nd.fz[k] = 0.;
        nd.ux[k] = nd.uy[k] = nd.uz[k] = 0.;
        nd.active[k] = 0;
        if (MIX) nd.gx[k] = nd.gy[k] = nd.gz[k] = 0.f;
        if (nf > 1) {
            // the volume and volume-gradient terms are floats in the mixed mode
            cterm_set<MIX>(nd.vol, k, 0.);
            nd.dsx[k] = nd.dsy[k] = nd.dsz[k] = 0.;
            cterm_set<MIX>(nd.gvx, k, 0.);
            cterm_set<MIX>(nd.gvy, k, 0.);
            cterm_set<MIX>(nd.gvz, k, 0.);
        }
    }
}

constexpr int kBatchIntCols = 4;  // mat, elem, orig, run

struct BatchGraph {
    cudaGraphExec_t exec = nullptr;
    long long key = -1;
};

}  // namespace

struct MpmGpuBatch {
    MpmGpuBatchOptions o{};
    int dim = 2;
    int pcap = 0, ncap = 0;
    int nf = 1;    // material velocity fields per node (node columns are nf * ncap long)
    int tb = 256;  // threads per block of the particle kernels
    void *cpdi = nullptr;  // lCPDI corner scratch for pcap slots
    // particle arena, two buffers: kParticleDoubles+1 double columns and
    // kBatchIntCols int columns of capacity pcap each; buffer `par` is current
    double *pbuf[2] = {nullptr, nullptr};
    int *ibuf[2] = {nullptr, nullptr};
    int par = 0;
    DevParticles p{};
    int *orig = nullptr;
    int n_used = 0, n_dead = 0;
    // node arena
    DevNodes nd{};
    double *nblock = nullptr;
    float *fblock = nullptr;
    double *coords = nullptr;  // node coordinates; a run's sit at its node base
    int *nrun = nullptr, *bc_group = nullptr;
    RangeAlloc nodes, cells, matslots;
    int node_used = 0;
    // sort scratch
    int *keys[2] = {nullptr, nullptr}, *vals[2] = {nullptr, nullptr}, *hist = nullptr, *sums = nullptr;
    int sort_bits = 1;
    long long since_sort = 1LL << 40;
    // regression-normal links (lr_links per particle slot) and results
    int *lr_cnt = nullptr, *lr_start = nullptr, *lr_list = nullptr, *lr_sums = nullptr;
    double *lr_out = nullptr;
    long long lr_cap = 0;
    int lr_runs = 0;  // resident runs with regression normals
    int rigid_runs = 0;  // resident runs with rigid contact materials
    // PeriodicXPIC expansion columns (xpic_order > 1)
    DevXpic xpic{};
    double *xpic_block = nullptr;
    double *xc = nullptr;     // XPIC contact state (in xpic_block), with several fields
    int *xc_pair = nullptr;
    // materials, runs, velocity conditions
    DevMat *mats = nullptr;
    DevRun *runs_dev = nullptr;
    std::vector<DevRun> runs_host;
    std::vector<BatchRun> runs;
    void *bc_block = nullptr;
    DevBCs bcs{};
    bool bcs_dirty = true;
    long long layout = 0;  // bumped whenever the captured launches would change
    unsigned *flag = nullptr;
    cudaStream_t stream = nullptr;
    BatchGraph graphs[2][2];  // [arena buffer][with sort]
    long long launches = 0;
    long long steps = 0;
    std::string msg;
};

namespace {

int berr(MpmGpuBatch *b, int code, const std::string &m) {
    if (b) b->msg = m;
    else g_static_err = m;
    return code;
}

#define BCK(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return berr(b, MPMGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void batch_link(MpmGpuBatch *b) {
    DevParticles &p = b->p;
    const size_t cap = (size_t)b->pcap;
    double *pb = b->pbuf[b->par];
    int *ib = b->ibuf[b->par];
    double **cols[kParticleDoubles + 1] = {&p.x, &p.y, &p.z, &p.vx, &p.vy, &p.vz, &p.mass, &p.lpx, &p.lpy, &p.lpz,
                                           &p.exx, &p.eyy, &p.ezz, &p.exy, &p.exz, &p.eyz, &p.wxy, &p.wxz, &p.wyz,
                                           &p.sxx, &p.syy, &p.szz, &p.sxy, &p.sxz, &p.syz, &p.pressure,
                                           &p.pxx, &p.pyy, &p.pzz, &p.pxy, &p.pxz, &p.pyz,
                                           &p.hist0, &p.hist1, &p.work, &p.plast, &p.x0, &p.y0, &p.z0, &p.xi, &p.eta, &p.zeta};
    for (int k = 0; k <= kParticleDoubles; k++) *cols[k] = pb + (size_t)k * cap;
    p.mat = ib;
    p.elem = ib + cap;
    b->orig = ib + 2 * cap;
    p.run = ib + 3 * cap;
    p.n = b->n_used;
    if (b->cpdi) {
        // domain-point scratch, rebuilt at every step start with stride n_used
        const size_t nc = b->o.shape == MPMGPU_SHAPE_QCPDI ? 9 : (b->dim == 3 ? 8 : 4);
        p.cxi = (double *)b->cpdi;
        p.cwg = p.cxi + 3 * nc * cap;
        p.ce = (int *)(p.cwg + 3 * nc * cap);
    }
}

void batch_drop_graphs(MpmGpuBatch *b) {
    for (auto &row : b->graphs)
        for (auto &g : row) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g = BatchGraph{};
        }
}

void batch_free(MpmGpuBatch *b) {
    batch_drop_graphs(b);
    void *ptrs[] = {b->pbuf[0], b->pbuf[1], b->ibuf[0], b->ibuf[1], b->nblock, b->fblock, b->coords, b->nrun,
                    b->bc_group, b->keys[0], b->keys[1], b->vals[0], b->vals[1], b->hist, b->sums, b->mats,
                    b->runs_dev, b->bc_block, b->flag, b->cpdi, b->lr_cnt, b->lr_start, b->lr_list, b->lr_sums,
                    b->lr_out, b->xpic_block};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (b->stream) cudaStreamDestroy(b->stream);
}

// rebuild the grouped velocity conditions of all runs (after runs come or go)
int batch_rebuild_bcs(MpmGpuBatch *b) {
    std::map<int, std::vector<const MpmGpuVelBC *>> by_node;
    std::vector<int> order;
    for (const auto &r : b->runs) {
        if (!r.used) continue;
        for (const auto &bc : r.bcs) {
            const int nd = bc.node - 1;
            if (!by_node.count(nd)) order.push_back(nd);
            by_node[nd].push_back(&bc);
        }
    }
    const int ng = (int)order.size();
    int nbc = 0;
    for (auto &kv : by_node) nbc += (int)kv.second.size();
    std::vector<int> gnode(ng), start(ng + 1), dir(nbc);
    std::vector<double> val(nbc), ft(nbc);
    std::vector<int> group((size_t)std::max(b->node_used, 1), -1);
    int pos = 0;
    for (int gi = 0; gi < ng; gi++) {
        gnode[gi] = order[gi];
        start[gi] = pos;
        group[order[gi]] = gi;
        for (const MpmGpuVelBC *bc : by_node[order[gi]]) {
            dir[pos] = bc->dir;
            val[pos] = bc->value;
            ft[pos] = bc->ftime;
            pos++;
        }
    }
    start[ng] = pos;
    BCK(cudaStreamSynchronize(b->stream));
    if (b->bc_block) cudaFree(b->bc_block);
    b->bc_block = nullptr;
    const size_t bytes = sizeof(int) * (ng + ng + 1 + nbc) + sizeof(double) * (2 * nbc) + 64;
    BCK(cudaMalloc(&b->bc_block, bytes));
    double *dval = (double *)b->bc_block;
    double *dft = dval + nbc;
    int *dnode = (int *)(dft + nbc);
    int *dstart = dnode + ng;
    int *ddir = dstart + ng + 1;
    cudaStream_t s = b->stream;
    if (nbc) {
        BCK(cudaMemcpyAsync(dval, val.data(), sizeof(double) * nbc, cudaMemcpyHostToDevice, s));
        BCK(cudaMemcpyAsync(dft, ft.data(), sizeof(double) * nbc, cudaMemcpyHostToDevice, s));
        BCK(cudaMemcpyAsync(ddir, dir.data(), sizeof(int) * nbc, cudaMemcpyHostToDevice, s));
    }
    if (ng) BCK(cudaMemcpyAsync(dnode, gnode.data(), sizeof(int) * ng, cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(dstart, start.data(), sizeof(int) * (ng + 1), cudaMemcpyHostToDevice, s));
    if (b->node_used > 0)
        BCK(cudaMemcpyAsync(b->bc_group, group.data(), sizeof(int) * b->node_used, cudaMemcpyHostToDevice, s));
    BCK(cudaStreamSynchronize(s));
    b->bcs.nnodes_bc = ng;
    b->bcs.node = dnode;
    b->bcs.start = dstart;
    b->bcs.dir = ddir;
    b->bcs.value = dval;
    b->bcs.ftime = dft;
    b->bcs_dirty = false;
    b->layout++;
    return MPMGPU_OK;
}

int batch_sort_launches(const MpmGpuBatch *b) { return 1 + 5 * ((b->sort_bits + 7) / 8) + 2; }

// Enqueue the cell sort of the used slots into the other arena buffer and make
// that buffer current.  Keys are (run cell base + element), so each run's
// particles are contiguous and in cell order; empty slots sort last.
void batch_enqueue_sort(MpmGpuBatch *b) {
    const int n = b->n_used;
    const int TB = 256, pb = (n + TB - 1) / TB;
    cudaStream_t s = b->stream;
    const int dead_key = (int)b->cells.cap;
    k_batch_keys<<<pb, TB, 0, s>>>(b->p.elem, b->p.run, b->runs_dev, b->keys[0], b->vals[0], n, dead_key);
    const int cur = radix_sort_passes(n, b->sort_bits, b->keys, b->vals, b->hist, b->sums, s);
    const int *perm = b->vals[cur];
    const int other = 1 - b->par;
    k_gather_cap<double><<<pb, TB, 0, s>>>(b->pbuf[b->par], b->pbuf[other], perm, n, kParticleDoubles + 1, b->pcap);
    k_gather_cap<int><<<pb, TB, 0, s>>>(b->ibuf[b->par], b->ibuf[other], perm, n, kBatchIntCols, b->pcap);
    b->par = other;
    batch_link(b);
}

// sort now (outside any graph) and drop the empty slots it moved to the end
int batch_compact(MpmGpuBatch *b) {
    if (b->n_used > 0) {
        batch_enqueue_sort(b);
        b->launches += batch_sort_launches(b);
        BCK(cudaGetLastError());
    }
    b->n_used -= b->n_dead;
    b->n_dead = 0;
    b->p.n = b->n_used;
    b->since_sort = 0;
    b->layout++;
    return MPMGPU_OK;
}

template <int DIM, int SHAPE, bool MIX>
void batch_enqueue_step(MpmGpuBatch *b) {
    const int n = b->n_used, NN = b->node_used;
    const int TB = b->tb, NTB = 256;
    const int pb = (n + TB - 1) / TB, nb = (NN + NTB - 1) / NTB;
    cudaStream_t s = b->stream;
    const int method = b->o.method;
    StepParams sp{};
    sp.runs = b->runs_dev;
    sp.nrun = b->nrun;
    sp.ct.nf = b->nf;
    sp.ct.fstride = b->ncap;
    sp.ct.lr = b->lr_out;
    sp.ct.rigid = b->rigid_runs > 0 ? 1u : 0u;  // some particle may be rigid (the runs' masks are per run)
    sp.ct.xc = b->xc;
    sp.ct.xc_pair = b->xc_pair;
    if (b->xc_pair)  // this step's contact state: none yet
        cudaMemsetAsync(b->xc_pair, 0x80, (size_t)b->nf * b->ncap * sizeof(int), s);
    k_clear_nodes<MIX><<<nb, NTB, 0, s>>>(b->nd, NN, b->nf, b->ncap);
    // mixed mode, one material field, window shape functions: the scatters
    // accumulate in shared-memory node tiles (each block's runs beyond its
    // first scatter straight to the node columns)
    constexpr bool kTileable = MIX && !kCpdi<SHAPE>;
    const bool tile = kTileable && b->nf == 1;
    if constexpr (kTileable) {
        if (tile) k_p2g_tile<DIM, SHAPE, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd);
        else k_p2g<DIM, SHAPE, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
    } else {
        k_p2g<DIM, SHAPE, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
    }
    const bool lr = b->lr_runs > 0;
    auto lr_normals = [&](int supports_only) {
        k_lr_normals<DIM, true><<<lr_loop_blocks((long long)NN * b->nf, NTB), NTB, 0, s>>>(
            sp, b->p, b->nd, b->mats, b->lr_start, b->lr_list, b->lr_cnt, b->lr_out, NN, b->lr_cap, 1, supports_only);
    };
    if (lr) {
        // link the particles of regression-normal runs to their contact nodes
        const int m = NN + 1, nsb = (m + kScanChunk - 1) / kScanChunk;
        cudaMemsetAsync(b->lr_cnt, 0, (size_t)m * sizeof(int), s);
        k_lr_link<DIM, SHAPE, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->lr_cnt, b->lr_start, b->lr_list,
                                                           b->lr_cap, 0);
        cudaMemcpyAsync(b->lr_start, b->lr_cnt, (size_t)m * sizeof(int), cudaMemcpyDeviceToDevice, s);
        k_scan_reduce<<<nsb, kScanBlock, 0, s>>>(b->lr_start, m, b->lr_sums);
        k_scan_sums<<<1, kScanBlock, 0, s>>>(b->lr_sums, nsb);
        k_scan_apply<<<nsb, kScanBlock, 0, s>>>(b->lr_start, m, b->lr_sums);
        cudaMemsetAsync(b->lr_cnt, 0, (size_t)m * sizeof(int), s);
        k_lr_link<DIM, SHAPE, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->lr_cnt, b->lr_start, b->lr_list,
                                                           b->lr_cap, 1);
        // the nodes with links, listed in b->lr_cnt (no longer needed as the cursor)
        cudaMemsetAsync(b->lr_cnt + NN, 0, sizeof(int), s);
        k_lr_compact<<<(NN + TB - 1) / TB, TB, 0, s>>>(b->lr_start, b->lr_cnt, NN);
        k_lr_order<<<lr_loop_blocks(NN, NTB), NTB, 0, s>>>(b->lr_start, b->lr_list, b->orig, b->lr_cnt, NN, b->lr_cap);
        lr_normals(0);
    }
    k_node_post<DIM, MIX, true><<<nb, NTB, 0, s>>>(sp, b->nd, NN, b->bcs, b->bc_group, method != MPMGPU_USL);
    // PeriodicXPIC expansions: every run whose mode of this step takes part
    const int xo = b->o.xpic_order, xf = b->o.xpic_fmpm;
    // (every field-node; with several fields, each pass's Delta v also takes
    // the incremental contact of the contact nodes of contact runs)
    const bool xcontact = b->nf > 1;
    auto xpic_expand = [&](int phase) {
        const int xb = (NN * b->nf + NTB - 1) / NTB;
        k_xpic_init<DIM, MIX, true><<<xb, NTB, 0, s>>>(sp, b->nd, b->xpic, NN, phase);
        for (int k = 2; k <= xo; k++) {
            k_xpic_pass<DIM, SHAPE, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->xpic, b->mats, phase, k);
            k_xpic_delta<DIM, MIX, true><<<xb, NTB, 0, s>>>(sp, b->nd, b->xpic, NN, b->bcs, b->bc_group, phase, k,
                                                            xcontact ? 1 : 0);
            if (xcontact) {
                k_xpic_contact<DIM, MIX, true><<<nb, NTB, 0, s>>>(sp, b->nd, b->xpic, NN, phase, k);
                k_xpic_apply<DIM, MIX, true><<<xb, NTB, 0, s>>>(sp, b->nd, b->xpic, NN, phase, k);
            }
        }
    };
    if (xo > 1 && xf && method != MPMGPU_USL) xpic_expand(XPIC_STRAIN);  // FMPM: first strain update
    bool forces_done = false;
    if constexpr (kTileable) {
        if (tile) {
            if (method == MPMGPU_USL)
                k_strain_forces_tile<DIM, SHAPE, false, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
            else
                k_strain_forces_tile<DIM, SHAPE, true, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
            forces_done = true;
        }
    }
    if (!forces_done) {
        if (method == MPMGPU_USL)
            k_strain_forces<DIM, SHAPE, false, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
        else
            k_strain_forces<DIM, SHAPE, true, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
    }
    if (lr) lr_normals(1);  // same positions, deformed radii changed with the strain update
    k_node_update<DIM, MIX, true><<<nb, NTB, 0, s>>>(sp, b->nd, NN, b->bcs, b->bc_group,
                                                    b->nf > 1 && method != MPMGPU_USF);
    if (xo > 1) xpic_expand(XPIC_PARTICLE);  // v(k) of the particle update
    if (method == MPMGPU_USF) {
        k_g2p<DIM, SHAPE, false, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
    } else {
        bool g2p_done = false;
        if constexpr (kTileable) {
            if (tile) {
                k_g2p_tile<DIM, SHAPE, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd);
                g2p_done = true;
            }
        }
        if (!g2p_done) k_g2p<DIM, SHAPE, true, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
        if (lr) lr_normals(0);  // the particles moved
        k_node_usl<DIM, MIX, true><<<nb, NTB, 0, s>>>(sp, b->nd, NN, b->bcs, b->bc_group);
        if (xo > 1 && xf) xpic_expand(XPIC_STRAIN);  // FMPM: second strain update
        k_strain_last<DIM, SHAPE, MIX, true><<<pb, TB, 0, s>>>(sp, b->p, b->nd, b->mats);
    }
    k_advance_runs<<<(b->o.max_runs + 127) / 128, 128, 0, s>>>(b->runs_dev, b->o.max_runs, xo, xf,
                                                                b->o.xpic_period);
}

template <int DIM, bool MIX>
void batch_enqueue_shape(MpmGpuBatch *b) {
    if (b->o.shape == MPMGPU_SHAPE_LINEAR) batch_enqueue_step<DIM, SHAPE_LINEAR, MIX>(b);
    else if (b->o.shape == MPMGPU_SHAPE_LCPDI) batch_enqueue_step<DIM, SHAPE_LCPDI, MIX>(b);
    else if (b->o.shape == MPMGPU_SHAPE_QCPDI) {
        if constexpr (DIM == 2) batch_enqueue_step<DIM, SHAPE_QCPDI, MIX>(b);  // refused in 3D at create
    }
    else if (b->o.shape == MPMGPU_SHAPE_BSPLINE) batch_enqueue_step<DIM, SHAPE_BSPLINE, MIX>(b);
    else if (b->o.shape == MPMGPU_SHAPE_BGIMP) batch_enqueue_step<DIM, SHAPE_BGIMP, MIX>(b);
    else batch_enqueue_step<DIM, SHAPE_UGIMP, MIX>(b);
}

void batch_enqueue_any(MpmGpuBatch *b) {
    const bool mix = b->o.precision == MPMGPU_PREC_MIXED;
    if (b->dim == 3) mix ? batch_enqueue_shape<3, true>(b) : batch_enqueue_shape<3, false>(b);
    else mix ? batch_enqueue_shape<2, true>(b) : batch_enqueue_shape<2, false>(b);
}

int batch_step_launches(const MpmGpuBatch *b) {
    const bool usf = b->o.method == MPMGPU_USF;
    // an expansion: init, then a particle and a node pass per order above 1;
    // one before the particle update, FMPM one before each strain update
    const int xo = b->o.xpic_order, expand = xo > 1 ? 1 + 2 * (xo - 1) : 0;
    const int strain_updates = (b->o.method != MPMGPU_USL ? 1 : 0) + (usf ? 0 : 1);
    const int expansions = xo > 1 ? 1 + (b->o.xpic_fmpm ? strain_updates : 0) : 0;
    return (usf ? 7 : 9) + (b->lr_runs > 0 ? 7 + (usf ? 2 : 3) : 0) + expansions * expand;
}

long long batch_graph_key(const MpmGpuBatch *b) {
    return ((b->layout * 1000003LL + b->n_used) * 1000003LL + b->node_used) * 1031LL + b->tb;
}

// the graph of one step (with the sort before it when with_sort) for the
// current arena buffer; captured when missing or stale
int batch_graph(MpmGpuBatch *b, int with_sort, cudaGraphExec_t *out) {
    BatchGraph &G = b->graphs[b->par][with_sort];
    const long long key = batch_graph_key(b);
    if (G.exec && G.key == key) {
        *out = G.exec;
        return MPMGPU_OK;
    }
    if (G.exec) cudaGraphExecDestroy(G.exec);
    G = BatchGraph{};
    const int par0 = b->par;
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    if (with_sort) batch_enqueue_sort(b);
    batch_enqueue_any(b);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (b->par != par0) {
        b->par = par0;
        batch_link(b);
    }
    if (e != cudaSuccess) return berr(b, MPMGPU_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&G.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        G = BatchGraph{};
        return berr(b, MPMGPU_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    G.key = key;
    *out = G.exec;
    return MPMGPU_OK;
}

// the graphs of both arena buffers: with the sort when the batch sorts, and
// without it unless it sorts every step
int batch_prepare(MpmGpuBatch *b) {
    const int si = b->o.sort_interval;
    const int par0 = b->par;
    int st = MPMGPU_OK;
    cudaGraphExec_t gx = nullptr;
    for (int q = 0; q < 2 && st == MPMGPU_OK; q++) {
        b->par = q;
        batch_link(b);
        if (si > 0) st = batch_graph(b, 1, &gx);
        if (st == MPMGPU_OK && si != 1) st = batch_graph(b, 0, &gx);
    }
    b->par = par0;
    batch_link(b);
    return st;
}

int batch_status(unsigned bits) {
    if (bits & ERR_RANGE) return MPMGPU_ERR_RANGE;  // a cause: what follows it may be NaN
    if (bits & ERR_NAN) return MPMGPU_ERR_NAN;
    if (bits & (ERR_LEFT_GRID | ERR_EDGE)) return MPMGPU_ERR_LEFT_GRID;
    if (bits & ERR_CPDI_NODES) return MPMGPU_ERR_CPDI_NODES;
    return MPMGPU_ERR_INVALID;
}

int batch_active_runs(const MpmGpuBatch *b) {
    int k = 0;
    for (const auto &r : b->runs) k += r.used && r.state == MPMGPU_RUN_RUNNING;
    return k;
}

// Enqueue nsteps batched steps (one graph launch each) without waiting for
// them; `mark`, when given, is recorded just before the first launch.  Sets
// *launched to whether any step was enqueued.
int batch_launch(MpmGpuBatch *b, int nsteps, cudaEvent_t mark, bool *launched) {
    *launched = false;
    if (b->bcs_dirty) {
        int st = batch_rebuild_bcs(b);
        if (st != MPMGPU_OK) return st;
    }
    if (b->n_dead > 0) {
        int st = batch_compact(b);
        if (st != MPMGPU_OK) return st;
    }
    if (!batch_active_runs(b) || b->n_used == 0 || nsteps == 0) return MPMGPU_OK;
    // capture every graph the steps can use before the first launch, so no
    // capture sits between launches (or inside a timed region)
    int st = batch_prepare(b);
    if (st != MPMGPU_OK) return st;
    if (mark) BCK(cudaEventRecord(mark, b->stream));
    cudaGraphExec_t gx = nullptr;
    for (int s = 0; s < nsteps; s++) {
        const int with_sort = b->o.sort_interval > 0 && b->since_sort >= b->o.sort_interval;
        st = batch_graph(b, with_sort, &gx);
        if (st != MPMGPU_OK) return st;
        BCK(cudaGraphLaunch(gx, b->stream));
        b->launches += batch_step_launches(b) + (with_sort ? batch_sort_launches(b) : 0);
        if (with_sort) {
            b->par = 1 - b->par;
            batch_link(b);
            b->since_sort = 0;
        }
        b->since_sort++;
        b->steps++;
    }
    *launched = true;
    return MPMGPU_OK;
}

// Wait for the enqueued steps and read the run table back: steps taken,
// finished runs, failed runs (with their error status).
int batch_collect(MpmGpuBatch *b) {
    BCK(cudaMemcpyAsync(b->runs_host.data(), b->runs_dev, sizeof(DevRun) * b->runs_host.size(),
                        cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    for (size_t r = 0; r < b->runs.size(); r++) {
        BatchRun &br = b->runs[r];
        if (!br.used || br.state != MPMGPU_RUN_RUNNING) continue;
        const DevRun &R = b->runs_host[r];
        br.steps_done = br.steps_total - R.steps_left;
        if (R.err) br.state = -batch_status(R.err);
        else if (!R.active) br.state = MPMGPU_RUN_FINISHED;
    }
    return MPMGPU_OK;
}

// nsteps steps, then the run states; *ms (when given) receives their device time
int batch_steps(MpmGpuBatch *b, int nsteps, double *ms) {
    if (ms) *ms = 0.;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ms) {
        BCK(cudaEventCreate(&e0));
        BCK(cudaEventCreate(&e1));
    }
    bool launched = false;
    int st = batch_launch(b, nsteps, e0, &launched);
    if (st == MPMGPU_OK && launched) {
        if (ms) BCK(cudaEventRecord(e1, b->stream));
        st = batch_collect(b);
        if (st == MPMGPU_OK && ms) {
            float f = 0.f;
            cudaEventElapsedTime(&f, e0, e1);
            *ms = f;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return st;
}

}  // namespace

extern "C" {

int64_t mpmgpu_batch_bytes(const MpmGpuBatchOptions *o) {
    if (!o || o->max_particles <= 0 || o->max_nodes <= 0) return -1;
    const int64_t P = o->max_particles, N = o->max_nodes;
    const int64_t ntiles = (P + kTile - 1) / kTile;
    const int64_t nf = o->max_fields > 1 ? o->max_fields : 1;
    const int64_t nc = o->shape == MPMGPU_SHAPE_QCPDI ? 9 : (o->np == MPMGPU_THREED ? 8 : 4);
    int64_t bytes = 2 * P * (int64_t)((kParticleDoubles + 1) * sizeof(double) + kBatchIntCols * sizeof(int));
    bytes += 4 * P * (int64_t)sizeof(int) + 2 * 256 * ntiles * (int64_t)sizeof(int);  // sort keys, histograms
    if (o->shape == MPMGPU_SHAPE_LCPDI || o->shape == MPMGPU_SHAPE_QCPDI)
        bytes += P * nc * (int64_t)(sizeof(int) + 6 * sizeof(double));
    bytes += N * nf * (int64_t)((nf > 1 ? 26 : 19) * sizeof(double) + 12 * sizeof(float) + 1);
    bytes += N * (int64_t)(2 * sizeof(int) + sizeof(double));
    bytes += (int64_t)o->max_materials * (int64_t)sizeof(DevMat) + (int64_t)o->max_runs * (int64_t)sizeof(DevRun);
    if (o->xpic_order > 1)  // XPIC columns of every field-node, contact state with several fields
        bytes += N * nf * (int64_t)(7 * sizeof(double) + 6 * sizeof(float) +
                                    (nf > 1 ? kXcDoubles * sizeof(double) + sizeof(int) : 0));
    if (nf > 1 && o->lr_links > 0) {
        // regression-normal links, counts, offsets, scan sums, results
        bytes += P * o->lr_links * (int64_t)sizeof(int) + 2 * (N + 1) * (int64_t)sizeof(int);
        bytes += ((N + 1 + kScanChunk - 1) / kScanChunk + 1) * (int64_t)sizeof(int) + 4 * N * nf * (int64_t)sizeof(double);
    }
    return bytes;
}

int mpmgpu_batch_create(const MpmGpuBatchOptions *o, MpmGpuBatch **out) {
    if (!o || !out) return berr(nullptr, MPMGPU_ERR_INVALID, "mpmgpu_batch_create: null argument");
    *out = nullptr;
    if (o->np != MPMGPU_PLANE_STRAIN && o->np != MPMGPU_THREED)
        return berr(nullptr, MPMGPU_ERR_UNSUPPORTED, "batch analysis type must be 2D plane strain or 3D");
    if (o->shape != MPMGPU_SHAPE_LINEAR && o->shape != MPMGPU_SHAPE_UGIMP && o->shape != MPMGPU_SHAPE_LCPDI &&
        o->shape != MPMGPU_SHAPE_BSPLINE && o->shape != MPMGPU_SHAPE_BGIMP && o->shape != MPMGPU_SHAPE_QCPDI)
        return berr(nullptr, MPMGPU_ERR_UNSUPPORTED, "shape function option not implemented on the device");
    if (o->shape == MPMGPU_SHAPE_QCPDI && o->np == MPMGPU_THREED)
        return berr(nullptr, MPMGPU_ERR_UNSUPPORTED, "qCPDI is defined in 2D only (the reference refuses it in 3D)");
    if (o->method != MPMGPU_USF && o->method != MPMGPU_USAVG && o->method != MPMGPU_USL)
        return berr(nullptr, MPMGPU_ERR_UNSUPPORTED, "MPM method must be USF, USAVG or USL");
    if (o->precision != MPMGPU_PREC_FP64 && o->precision != MPMGPU_PREC_MIXED)
        return berr(nullptr, MPMGPU_ERR_UNSUPPORTED, "precision must be MPMGPU_PREC_FP64 or MPMGPU_PREC_MIXED");
    if (o->max_fields < 0 || o->max_fields > kMaxFields)
        return berr(nullptr, MPMGPU_ERR_UNSUPPORTED, "max_fields must be 0 to 8");
    if (o->lr_links < 0 || o->lr_links > 64) return berr(nullptr, MPMGPU_ERR_INVALID, "lr_links must be 0 to 64");
    if (o->xpic_order < 0 || o->xpic_order > 64 || (o->xpic_fmpm != 0 && o->xpic_fmpm != 1) ||
        (o->xpic_order > 0 && o->xpic_period < 1))
        return berr(nullptr, MPMGPU_ERR_INVALID, "xpic_order must be 0 to 64, xpic_fmpm 0 or 1, xpic_period >= 1");
    if (o->max_particles <= 0 || o->max_particles > (1LL << 31) - 1 || o->max_nodes <= 0 ||
        o->max_nodes > (1LL << 30) || o->max_runs <= 0 || o->max_runs > (1 << 20) || o->max_materials <= 0 ||
        o->max_materials > (1 << 24))
        return berr(nullptr, MPMGPU_ERR_INVALID, "batch capacities out of range");
    if (o->block != 0 && o->block != 64 && o->block != 128 && o->block != 256)
        return berr(nullptr, MPMGPU_ERR_INVALID, "block must be 0, 64, 128 or 256");
    MpmGpuBatch *b = new MpmGpuBatch();
    b->o = *o;
    if (!(b->o.fraction_usf > 0.)) b->o.fraction_usf = 0.5;
    if (b->o.sort_interval < 0) b->o.sort_interval = 0;
    b->tb = o->block ? o->block : 256;
    b->dim = o->np == MPMGPU_THREED ? 3 : 2;
    b->pcap = (int)o->max_particles;
    b->ncap = (int)o->max_nodes;
    b->nf = o->max_fields > 1 ? o->max_fields : 1;
    const size_t P = (size_t)b->pcap, N = (size_t)b->ncap, NT = N * b->nf;
    const int ncleared = b->nf > 1 ? 17 : 10, ncols = ncleared + 9;
    const size_t ntiles = (P + kTile - 1) / kTile;
    const size_t nsums = (256 * ntiles + kScanChunk - 1) / kScanChunk + 1;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    auto A = [&](void **q, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(q, bytes);
    };
    for (int k = 0; k < 2; k++) {
        A((void **)&b->pbuf[k], P * (kParticleDoubles + 1) * sizeof(double));
        A((void **)&b->ibuf[k], P * kBatchIntCols * sizeof(int));
        A((void **)&b->keys[k], P * sizeof(int));
        A((void **)&b->vals[k], P * sizeof(int));
    }
    A((void **)&b->nblock, NT * ncols * sizeof(double) + NT);
    A((void **)&b->fblock, NT * 12 * sizeof(float));
    if (o->shape == MPMGPU_SHAPE_LCPDI || o->shape == MPMGPU_SHAPE_QCPDI)
        A(&b->cpdi, P * (o->shape == MPMGPU_SHAPE_QCPDI ? 9 : (b->dim == 3 ? 8 : 4)) * (sizeof(int) + 6 * sizeof(double)));
    A((void **)&b->coords, N * sizeof(double));
    A((void **)&b->nrun, N * sizeof(int));
    A((void **)&b->bc_group, N * sizeof(int));
    A((void **)&b->hist, 256 * ntiles * sizeof(int));
    A((void **)&b->sums, nsums * sizeof(int));
    A((void **)&b->mats, (size_t)o->max_materials * sizeof(DevMat));
    A((void **)&b->runs_dev, (size_t)o->max_runs * sizeof(DevRun));
    A((void **)&b->flag, sizeof(unsigned));
    if (o->xpic_order > 1) {
        // every field-node's expansion columns, and with several fields each
        // field-node's contact state for the passes' incremental contact
        const size_t XN = N * (size_t)b->nf;
        const size_t xc = b->nf > 1 ? XN * (kXcDoubles * sizeof(double) + sizeof(int)) : 0;
        A((void **)&b->xpic_block, 7 * XN * sizeof(double) + 6 * XN * sizeof(float) + xc);
        if (e == cudaSuccess) {
            double *d = b->xpic_block;
            float *f = (float *)(d + 7 * XN);
            b->xpic = DevXpic{d, d + XN, d + 2 * XN, d + 3 * XN, d + 4 * XN, d + 5 * XN, d + 6 * XN,
                              f, f + XN, f + 2 * XN, f + 3 * XN, f + 4 * XN, f + 5 * XN};
            if (b->nf > 1) {
                b->xc = (double *)(f + 6 * XN);  // 8-byte aligned: 6 XN floats
                b->xc_pair = (int *)(b->xc + kXcDoubles * XN);
            }
        }
    }
    if (b->nf > 1 && o->lr_links > 0) {
        b->lr_cap = (long long)P * o->lr_links;
        A((void **)&b->lr_cnt, (N + 1) * sizeof(int));
        A((void **)&b->lr_start, (N + 1) * sizeof(int));
        A((void **)&b->lr_sums, ((N + 1 + kScanChunk - 1) / kScanChunk + 1) * sizeof(int));
        A((void **)&b->lr_list, (size_t)b->lr_cap * sizeof(int));
        A((void **)&b->lr_out, 4 * NT * sizeof(double));
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(b->nblock, 0, NT * ncols * sizeof(double) + NT, b->stream);
    if (e == cudaSuccess && b->lr_out) e = cudaMemsetAsync(b->lr_out, 0, 4 * NT * sizeof(double), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->fblock, 0, NT * 12 * sizeof(float), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->nrun, 0xFF, N * sizeof(int), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->bc_group, 0xFF, N * sizeof(int), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->runs_dev, 0, (size_t)o->max_runs * sizeof(DevRun), b->stream);
    for (int k = 0; k < 2 && e == cudaSuccess; k++)
        e = cudaMemsetAsync(b->pbuf[k], 0, P * (kParticleDoubles + 1) * sizeof(double), b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        std::string m = std::string("batch allocation: ") + cudaGetErrorString(e);
        batch_free(b);
        delete b;
        return berr(nullptr, MPMGPU_ERR_OOM, m);
    }
    double *nb = b->nblock;
    DevNodes &nd = b->nd;
    // field f of node n at f * ncap + n in every column
    double **dc[26] = {&nd.mass, &nd.px, &nd.py, &nd.pz, &nd.fx, &nd.fy, &nd.fz, &nd.ux, &nd.uy, &nd.uz,
                       &nd.cx, &nd.cy, &nd.cz, &nd.vx, &nd.vy, &nd.vz, &nd.ax, &nd.ay, &nd.az,
                       &nd.vol, &nd.dsx, &nd.dsy, &nd.dsz, &nd.gvx, &nd.gvy, &nd.gvz};
    for (int k = 0; k < 19; k++) *dc[k] = nb + (size_t)k * NT;
    if (b->nf > 1)
        for (int k = 19; k < 26; k++) *dc[k] = nb + (size_t)k * NT;
    nd.active = (unsigned char *)(nb + (size_t)ncols * NT);
    float *fb = b->fblock;
    float **fc[12] = {&nd.gx, &nd.gy, &nd.gz, &nd.vhx, &nd.vhy, &nd.vhz,
                      &nd.vlx, &nd.vly, &nd.vlz, &nd.bx, &nd.by, &nd.bz};
    for (int k = 0; k < 12; k++) *fc[k] = fb + (size_t)k * NT;
    batch_link(b);
    b->nodes.init(b->ncap);
    b->cells.init(b->ncap);  // every run has fewer cells than nodes
    b->matslots.init(o->max_materials);
    while ((1LL << b->sort_bits) <= (long long)b->ncap) b->sort_bits++;
    b->runs.resize((size_t)o->max_runs);
    b->runs_host.assign((size_t)o->max_runs, DevRun{});
    *out = b;
    return MPMGPU_OK;
}

int mpmgpu_batch_add_run(MpmGpuBatch *b, const MpmGpuGrid *grid, const MpmGpuMaterial *mats, int32_t nmat,
                         const MpmGpuVelBC *bcs, int32_t nbc, const MpmGpuContact *contact,
                         const MpmGpuParticles *h, double timestep, int32_t nsteps, int32_t *run_id) {
    if (!b || !grid || !mats || nmat <= 0 || !h || h->n <= 0 || (nbc > 0 && !bcs) || nbc < 0 || !run_id ||
        nsteps <= 0 || !(timestep > 0.))
        return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_add_run: bad argument");
    if (grid->dim != b->dim) return berr(b, MPMGPU_ERR_INVALID, "run dimension differs from the batch");
    if (grid->nx < 3 || grid->ny < 3 || (grid->dim == 3 && grid->nz < 3) || !grid->xnodes || !grid->ynodes ||
        (grid->dim == 3 && !grid->znodes))
        return berr(b, MPMGPU_ERR_INVALID, "grid needs >= 3 elements per axis and node coordinates");
    if (!h->x || !h->y || !h->vx || !h->vy || !h->mass || !h->mat || !h->elem || !h->lpx || !h->lpy ||
        (b->dim == 3 && (!h->z || !h->vz || !h->lpz)))
        return berr(b, MPMGPU_ERR_INVALID,
                    "position, velocity, mass, size, material and element columns are required");
    const long long nnodes = (long long)(grid->nx + 1) * (grid->ny + 1) * (b->dim == 3 ? grid->nz + 1 : 1);
    const long long nelems = (long long)grid->nx * grid->ny * (b->dim == 3 ? grid->nz : 1);
    if (h->n > b->pcap) return berr(b, MPMGPU_ERR_OOM, "run has more particles than the batch capacity");
    if (nnodes > b->ncap) return berr(b, MPMGPU_ERR_OOM, "run has more nodes than the batch capacity");
    const int np = (int)h->n;
    for (int k = 0; k < nbc; k++) {
        if (bcs[k].node < 1 || bcs[k].node > nnodes)
            return berr(b, MPMGPU_ERR_INVALID, "velocity BC node out of range");
        if (bcs[k].dir != 1 && bcs[k].dir != 2 && bcs[k].dir != 4)
            return berr(b, MPMGPU_ERR_UNSUPPORTED, "velocity BC dir must be 1, 2 or 4");
        if (bcs[k].dir == 4 && b->dim == 2) return berr(b, MPMGPU_ERR_INVALID, "z velocity BC in 2D");
    }
    std::vector<DevMat> dm((size_t)nmat);
    int maxfield = 0;
    for (int i = 0; i < nmat; i++) {
        std::string why;
        const int st = derive_material(mats[i], b->o.np, dm[i], why, b->o.inc_defgrad_terms);
        if (st != MPMGPU_OK) return berr(b, st, "material " + std::to_string(i) + ": " + why);
        if (mats[i].field < 0 || mats[i].field >= b->nf)
            return berr(b, MPMGPU_ERR_INVALID, "material " + std::to_string(i) + ": field outside 0 .. max_fields-1");
        maxfield = std::max(maxfield, mats[i].field);
    }
    const bool mm = contact && contact->enabled;
    if (maxfield > 0 && !mm)
        return berr(b, MPMGPU_ERR_INVALID, "a run with several material fields needs multimaterial contact");
    unsigned rigid = 0u;  // the run's rigid contact fields
    for (int i = 0; i < nmat; i++)
        if (dm[i].type == kMatRigid) rigid |= 1u << dm[i].field;
    if (rigid && (!mm || maxfield < 1))
        return berr(b, MPMGPU_ERR_UNSUPPORTED, "rigid contact materials need multimaterial contact");
    if (rigid && contact->normals >= 5)
        return berr(b, MPMGPU_ERR_UNSUPPORTED, "regression normals with rigid materials are not implemented");
    if (rigid && b->o.xpic_order > 1)
        return berr(b, MPMGPU_ERR_UNSUPPORTED, "XPIC/FMPM of order > 1 with rigid materials is not implemented");
    if (mm) {
        if (b->nf < 2) return berr(b, MPMGPU_ERR_INVALID, "contact needs a batch with max_fields >= 2");
        if (contact->normals < 0 || (contact->normals > 2 && contact->normals < 5) || contact->normals > 6)
            return berr(b, MPMGPU_ERR_UNSUPPORTED, "contact normals: methods 0, 1, 2, 5 and 6 are implemented");
        if (contact->normals >= 5 && b->lr_cap == 0)
            return berr(b, MPMGPU_ERR_INVALID, "regression contact normals need a batch with lr_links > 0");
        if (contact->contact_cutoff > 0.)
            return berr(b, MPMGPU_ERR_UNSUPPORTED, "position-based contact is not implemented on the device");
    }
    int r = -1;
    for (int k = 0; k < (int)b->runs.size() && r < 0; k++)
        if (!b->runs[k].used) r = k;
    if (r < 0) return berr(b, MPMGPU_ERR_BUSY, "no free run slot");
    if ((long long)b->n_used + np > b->pcap && b->n_dead > 0) {
        const int st = batch_compact(b);
        if (st != MPMGPU_OK) return st;
    }
    if ((long long)b->n_used + np > b->pcap) return berr(b, MPMGPU_ERR_BUSY, "particle capacity is in use");
    const long long nbase = b->nodes.alloc(nnodes);
    if (nbase < 0) return berr(b, MPMGPU_ERR_BUSY, "node capacity is in use");
    const long long cbase = b->cells.alloc(nelems);
    const long long mbase = cbase >= 0 ? b->matslots.alloc(nmat) : -1;
    if (cbase < 0 || mbase < 0) {
        b->nodes.release(nbase, nnodes);
        if (cbase >= 0) b->cells.release(cbase, nelems);
        return berr(b, MPMGPU_ERR_BUSY, "cell or material capacity is in use");
    }
    cudaStream_t s = b->stream;
    // node coordinates at the run's node base (a run has more nodes than coordinates)
    double *xn = b->coords + nbase, *yn = xn + grid->nx + 1, *zn = yn + grid->ny + 1;
    BCK(cudaMemcpyAsync(xn, grid->xnodes, sizeof(double) * (grid->nx + 1), cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(yn, grid->ynodes, sizeof(double) * (grid->ny + 1), cudaMemcpyHostToDevice, s));
    if (b->dim == 3)
        BCK(cudaMemcpyAsync(zn, grid->znodes, sizeof(double) * (grid->nz + 1), cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(b->mats + mbase, dm.data(), sizeof(DevMat) * nmat, cudaMemcpyHostToDevice, s));
    // particles after the used slots
    const int start = b->n_used;
    double *hc[kParticleDoubles];
    hcols(h, hc);
    double *pb = b->pbuf[b->par];
    for (int k = 0; k < kParticleDoubles; k++) {
        double *dst = pb + (size_t)k * b->pcap + start;
        if (hc[k]) BCK(cudaMemcpyAsync(dst, hc[k], sizeof(double) * np, cudaMemcpyHostToDevice, s));
        else BCK(cudaMemsetAsync(dst, 0, sizeof(double) * np, s));
    }
    BCK(cudaMemcpyAsync(b->p.mat + start, h->mat, sizeof(int) * np, cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(b->p.elem + start, h->elem, sizeof(int) * np, cudaMemcpyHostToDevice, s));
    BCK(cudaMemsetAsync(b->flag, 0, sizeof(unsigned), s));
    const int TB = 256;
    k_batch_admit<<<(np + TB - 1) / TB, TB, 0, s>>>(b->p.mat, b->p.elem, b->orig, b->p.run, start, np, r,
                                                    (int)mbase, nmat, (int)nelems, b->flag);
    k_fill_int<<<(int)((nnodes + TB - 1) / TB), TB, 0, s>>>(b->nrun, nbase, nnodes, r);
    k_clear_run_nodes<<<(int)((nnodes + TB - 1) / TB), TB, 0, s>>>(b->nd, nbase, nnodes, b->nf, b->ncap);
    b->launches += 3;
    BCK(cudaGetLastError());
    DevRun R{};
    R.g.dim = b->dim;
    R.g.nx = grid->nx;
    R.g.ny = grid->ny;
    R.g.nz = b->dim == 3 ? grid->nz : 0;
    R.g.xplane = 1;
    R.g.yplane = grid->nx + 1;
    R.g.zplane = (grid->nx + 1) * (grid->ny + 1);
    R.g.nnodes = (int)nnodes;
    R.g.xmin = grid->xmin;
    R.g.ymin = grid->ymin;
    R.g.zmin = grid->zmin;
    R.g.gx = grid->dx;
    R.g.gy = grid->dy;
    R.g.gz = grid->dz;
    R.g.igx = 1. / grid->dx;
    R.g.igy = 1. / grid->dy;
    R.g.igz = b->dim == 3 ? 1. / grid->dz : 0.;
    R.g.xn = xn;
    R.g.yn = yn;
    R.g.zn = b->dim == 3 ? zn : nullptr;
    R.node_base = (int)nbase;
    R.cell_base = (int)cbase;
    R.active = 1;
    R.steps_left = nsteps;
    R.dt = timestep;
    R.st_first = b->o.method == MPMGPU_USAVG ? b->o.fraction_usf * timestep : timestep;
    R.st_last = b->o.method == MPMGPU_USAVG ? timestep - R.st_first : timestep;
    R.t = 0.;
    R.err = 0;
    R.mm = mm ? 1 : 0;
    R.normals = mm ? contact->normals : 2;
    R.friction = mm ? contact->friction : 0.;
    R.style = !mm ? 2 : (contact->friction < 0. ? 0 : (contact->friction == 0. ? 1 : 2));
    R.rigid = rigid;
    {
        const double bias = mm && contact->rigid_gradient_bias > 0. ? contact->rigid_gradient_bias : 1.;
        R.rigid_bias = bias * bias;  // MeshInfo::rigidGradientBias, squared
    }
    R.xpic = xpic_mode(b->o.xpic_order, b->o.xpic_fmpm, b->o.xpic_period, 1);  // its first step
    BCK(cudaMemcpyAsync(b->runs_dev + r, &R, sizeof(DevRun), cudaMemcpyHostToDevice, s));
    unsigned bad = 0;
    BCK(cudaMemcpyAsync(&bad, b->flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
    BatchRun &br = b->runs[r];
    br = BatchRun{};
    br.used = true;
    br.np = np;
    br.node_base = nbase;
    br.nnodes = nnodes;
    br.cell_base = cbase;
    br.nelems = nelems;
    br.mat_base = mbase;
    br.nmat = nmat;
    br.steps_total = nsteps;
    br.state = MPMGPU_RUN_RUNNING;
    br.lr = mm && contact->normals >= 5;
    b->lr_runs += br.lr ? 1 : 0;
    br.rigid = rigid != 0u;
    b->rigid_runs += br.rigid ? 1 : 0;
    br.bcs.reserve((size_t)nbc);
    for (int k = 0; k < nbc; k++) {
        MpmGpuVelBC bc = bcs[k];
        bc.node += (int)nbase;
        br.bcs.push_back(bc);
    }
    b->runs_host[r] = R;
    b->n_used += np;
    b->p.n = b->n_used;
    b->node_used = (int)b->nodes.high_water();
    b->bcs_dirty = true;
    b->layout++;
    b->since_sort = 1LL << 40;  // new slots are unsorted
    if (bad) {
        mpmgpu_batch_remove_run(b, r, nullptr);
        return berr(b, MPMGPU_ERR_INVALID, "particle material or element index out of range");
    }
    *run_id = r;
    return MPMGPU_OK;
}

int mpmgpu_batch_step(MpmGpuBatch *b, int32_t nsteps) {
    if (!b || nsteps < 0) return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_step: bad argument");
    return batch_steps(b, nsteps, nullptr);
}

int mpmgpu_batch_step_timed(MpmGpuBatch *b, int32_t nsteps, double *ms) {
    if (!b || nsteps < 0 || !ms) return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_step_timed: bad argument");
    return batch_steps(b, nsteps, ms);
}

int mpmgpu_batch_run_state(const MpmGpuBatch *b, int32_t run_id, int32_t *state, int32_t *steps_done) {
    if (!b || run_id < 0 || run_id >= (int)b->runs.size()) return MPMGPU_ERR_INVALID;
    const BatchRun &br = b->runs[run_id];
    if (state) *state = br.used ? br.state : MPMGPU_RUN_EMPTY;
    if (steps_done) *steps_done = br.used ? br.steps_done : 0;
    return MPMGPU_OK;
}

int mpmgpu_batch_download_run(MpmGpuBatch *b, int32_t run_id, MpmGpuParticles *out) {
    if (!b || !out || run_id < 0 || run_id >= (int)b->runs.size() || !b->runs[run_id].used)
        return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_download_run: bad run");
    const BatchRun &br = b->runs[run_id];
    if (out->n != br.np) return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_download_run: particle count mismatch");
    cudaStream_t s = b->stream;
    const int TB = 256, n = b->n_used;
    // the other arena buffer is free between steps: pack the run there
    double *packed = b->pbuf[1 - b->par];
    int *ipacked = b->ibuf[1 - b->par];
    if (n > 0) {
        k_batch_extract<<<(n + TB - 1) / TB, TB, 0, s>>>(b->pbuf[b->par], b->pcap, b->p.mat, b->p.elem, b->orig,
                                                         b->p.run, n, run_id, (int)br.mat_base, packed, ipacked,
                                                         br.np, kParticleDoubles);
        b->launches++;
        BCK(cudaGetLastError());
    }
    double *hc[kParticleDoubles];
    hcols(out, hc);
    for (int k = 0; k < kParticleDoubles; k++)
        if (hc[k])
            BCK(cudaMemcpyAsync(hc[k], packed + (size_t)k * br.np, sizeof(double) * br.np, cudaMemcpyDeviceToHost,
                                s));
    if (out->mat) BCK(cudaMemcpyAsync(out->mat, ipacked, sizeof(int) * br.np, cudaMemcpyDeviceToHost, s));
    if (out->elem) BCK(cudaMemcpyAsync(out->elem, ipacked + br.np, sizeof(int) * br.np, cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
    return MPMGPU_OK;
}

int mpmgpu_batch_remove_run(MpmGpuBatch *b, int32_t run_id, MpmGpuParticles *out) {
    if (!b || run_id < 0 || run_id >= (int)b->runs.size() || !b->runs[run_id].used)
        return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_remove_run: bad run");
    BatchRun &br = b->runs[run_id];
    if (out) {
        const int st = mpmgpu_batch_download_run(b, run_id, out);
        if (st != MPMGPU_OK) return st;
    }
    cudaStream_t s = b->stream;
    const int TB = 256, n = b->n_used;
    if (n > 0) k_batch_kill<<<(n + TB - 1) / TB, TB, 0, s>>>(b->p.run, n, run_id);
    k_fill_int<<<(int)((br.nnodes + TB - 1) / TB), TB, 0, s>>>(b->nrun, br.node_base, br.nnodes, -1);
    b->launches += 2;
    BCK(cudaGetLastError());
    DevRun R{};
    b->runs_host[run_id] = R;
    BCK(cudaMemcpyAsync(b->runs_dev + run_id, &R, sizeof(DevRun), cudaMemcpyHostToDevice, s));
    BCK(cudaStreamSynchronize(s));
    b->n_dead += br.np;
    b->nodes.release(br.node_base, br.nnodes);
    b->cells.release(br.cell_base, br.nelems);
    b->matslots.release(br.mat_base, br.nmat);
    b->node_used = (int)b->nodes.high_water();
    b->lr_runs -= br.lr ? 1 : 0;
    b->rigid_runs -= br.rigid ? 1 : 0;
    br = BatchRun{};
    b->bcs_dirty = true;
    b->layout++;
    return MPMGPU_OK;
}

int mpmgpu_batch_set_tuning(MpmGpuBatch *b, int32_t block, int32_t sort_interval) {
    if (!b || (block != 64 && block != 128 && block != 256) || sort_interval < 0)
        return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_set_tuning: block must be 64, 128 or 256");
    b->tb = block;
    b->o.sort_interval = sort_interval;
    return MPMGPU_OK;
}

// Pick the particle-kernel block size and the sort interval by timing real
// steps of the current runs: each candidate runs `trial_steps` steps (rounded
// up to a multiple of 8, starting from a fresh sort) after one untimed step
// that captures its graphs.  The trial steps advance the runs like any other
// steps.  Results: the chosen block and interval (also set on the batch).
int mpmgpu_batch_autotune(MpmGpuBatch *b, int32_t trial_steps, int32_t *block, int32_t *sort_interval,
                          double *ms_per_step) {
    if (!b || trial_steps <= 0) return berr(b, MPMGPU_ERR_INVALID, "mpmgpu_batch_autotune: bad argument");
    const int steps = (trial_steps + 7) / 8 * 8;
    const int blocks[] = {128, 256};
    const int intervals[] = {1, 2, 4, 8};
    double best = 1e300;
    int best_tb = b->tb, best_si = b->o.sort_interval;
    for (int tb : blocks)
        for (int si : intervals) {
            if (!batch_active_runs(b)) break;
            b->tb = tb;
            b->o.sort_interval = si;
            b->since_sort = 1LL << 40;
            int st = batch_steps(b, 1, nullptr);  // captures the graphs of this candidate
            if (st != MPMGPU_OK) return st;
            b->since_sort = 1LL << 40;
            double ms = 0.;
            st = batch_steps(b, steps, &ms);
            if (st != MPMGPU_OK) return st;
            if (ms > 0. && ms / steps < best) {
                best = ms / steps;
                best_tb = tb;
                best_si = si;
            }
        }
    b->tb = best_tb;
    b->o.sort_interval = best_si;
    if (block) *block = best_tb;
    if (sort_interval) *sort_interval = best_si;
    if (ms_per_step) *ms_per_step = best < 1e300 ? best : 0.;
    return MPMGPU_OK;
}

int mpmgpu_batch_info(const MpmGpuBatch *b, MpmGpuBatchInfo *info) {
    if (!b || !info) return MPMGPU_ERR_INVALID;
    info->runs = 0;
    info->running = 0;
    for (const auto &r : b->runs) {
        info->runs += r.used;
        info->running += r.used && r.state == MPMGPU_RUN_RUNNING;
    }
    info->particles_used = b->n_used;
    info->particles_dead = b->n_dead;
    info->nodes_used = b->node_used;
    info->block = b->tb;
    info->sort_interval = b->o.sort_interval;
    info->steps = b->steps;
    info->launches = b->launches;
    return MPMGPU_OK;
}

const char *mpmgpu_batch_last_error(const MpmGpuBatch *b) { return b ? b->msg.c_str() : g_static_err.c_str(); }

void *mpmgpu_batch_stream(MpmGpuBatch *b) { return b ? (void *)b->stream : nullptr; }

void mpmgpu_batch_destroy(MpmGpuBatch *b) {
    if (!b) return;
    cudaStreamSynchronize(b->stream);
    batch_free(b);
    delete b;
}

}  // extern "C"
