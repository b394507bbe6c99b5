// context.cuh -- the single-run context (MpmGpuCtx of include/nairn_mpm_gpu.h),
// shared by the C ABI (mpm_gpu.cu) and the step translation units
// (step_<precision>_<dim>_<sums>.cu), which instantiate the step kernels of
// one combination each so the library builds in parallel.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "mpm_kernels.cuh"
#include "nairn_mpm_gpu.h"
#include "sort.cuh"

namespace nmg {

struct Profile {
    const char *name;
    double ms;
};

constexpr int kFamilies = 8;  // p2g, node_post, strain_forces, node_update, g2p, node_usl, strain_last, sort

}  // namespace nmg

struct MpmGpuCtx {
    MpmGpuOptions opts{};
    int dim = 2;
    nmg::DevGrid g{};
    nmg::DevParticles p{};
    nmg::DevNodes nd{};
    nmg::DevBCs bcs{};
    int *bc_group = nullptr;
    nmg::DevMat *mats = nullptr;
    int nmat = 0;
    std::vector<nmg::DevMat> hmats;
    double *grid_coords = nullptr;
    double *pblock = nullptr;            // particle double columns
    int *iblock = nullptr;               // mat, elem, original index
    int *orig = nullptr;                 // original (host) index of each slot
    int *iota = nullptr;                 // identity order of steps on host-resident state (n ints)
    double *nblock = nullptr;            // node double columns
    float *fblock = nullptr;             // node float columns (mixed mode)
    size_t fblock_zero_bytes = 0;
    size_t nblock_zero_bytes = 0;        // bytes cleared at each step start
    unsigned char *active = nullptr;
    unsigned *err = nullptr;
    void *bc_block = nullptr;
    cudaStream_t stream = nullptr;
    nmg::SortWorkspace sort{};
    long long steps_done = 0;
    std::string msg;
    std::vector<nmg::Profile> prof;
    bool profile = false;
    std::vector<cudaEvent_t> ev;         // per-step kernel events when profiling
    long long launches = 0;              // kernels launched by this context
    void *cpdi = nullptr;                // lCPDI corner scratch (ints then doubles)
    void *winblock = nullptr;            // window cache of FP64 window shapes (doubles then ints)
    nmg::DevContact ct{1, 0, 2, 2, 0.};       // material fields and multimaterial contact
    bool contact_on = false;
    nmg::DevDet det{nullptr, 0, nullptr, nullptr};     // deterministic node sums (p2g option 1)
    void *archive_buf = nullptr;         // device staging of archive records
    size_t archive_cap = 0;
    cudaStream_t archive_stream = nullptr;  // copies of packed records to the host
    cudaEvent_t archive_packed = nullptr, archive_copied = nullptr;
    bool archive_pending = false;           // an asynchronous copy not yet waited for
    // regression contact normals: link counts, offsets, links, results, scan scratch
    int *lr_cnt = nullptr, *lr_start = nullptr, *lr_list = nullptr, *lr_sums = nullptr;
    double *lr_out = nullptr;
    long long lr_cap = 0;                // links the list holds
    // PeriodicXPIC expansion columns (7 FP64 and 7 FP32 per node, allocated at the first step)
    nmg::DevXpic xpic{};
    double *xpic_block = nullptr;
};

namespace nmg {

// the PeriodicXPIC mode of step s (from 1) of a single-run context
inline int xpic_step_order(const MpmGpuOptions &o, long long s) {
    return xpic_mode(o.xpic_order, o.xpic_fmpm, o.xpic_period, s);
}

// event of kernel family k in step slot `slot` of the current call
inline cudaEvent_t &event_at(MpmGpuCtx *c, int slot, int k, bool begin) {
    return c->ev[((size_t)slot * kFamilies + k) * 2 + (begin ? 0 : 1)];
}

// enqueue one step of a context (FP64 / mixed transfers; deterministic node sums)
// one step of a context (defined in step.cuh, each combination instantiated
// in its own translation unit)
template <int DIM, bool MIX, bool DET>
void enqueue_dim(MpmGpuCtx *c, double t, int slot);

}  // namespace nmg
