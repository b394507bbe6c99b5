// sort.cuh -- stable LSD radix sort of particles by element (cell) and the
// permutation of every particle column.
//
// The reference keeps particles in mpm[] order and walks them per patch
// (GridPatch, NairnMPM/src/Patches/GridPatch.cpp:256-278); on the GPU the
// particles are re-ordered by cell so that the particles of a warp touch the
// same grid nodes, which keeps the P2G atomics and G2P gathers in L2.  The sort
// is stable and deterministic: equal keys keep their previous relative order,
// so the permutation is a pure function of the element array.
//
// Each warp owns a tile of kTile keys.  Pass = histogram per tile, one
// exclusive scan over (digit, tile), then a scatter in which each warp ranks
// its keys round by round with __match_any_sync.
#pragma once

#include <cuda_runtime.h>

#include "mpm_device.cuh"

namespace nmg {

constexpr int kSortWarpsPerBlock = 4;
constexpr int kTile = 32 * 16;  // keys per warp tile

struct SortWorkspace {
    int n = 0, nelems = 0, ntiles = 0, bits = 0;
    int *keys[2] = {nullptr, nullptr};
    int *vals[2] = {nullptr, nullptr};
    int *hist = nullptr;       // 256 * ntiles
    int *sums = nullptr;       // scan block sums
    double *scratch = nullptr; // ncols * n doubles (the other particle buffer)
    int *iscratch = nullptr;   // 3 * n ints
    size_t scratch_cols = 0;
};

static __global__ void k_sort_init(const int *elem, int *k, int *v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        k[i] = elem[i];
        v[i] = i;
    }
}

static __global__ void k_sort_hist(const int *keys, int n, int shift, int *hist, int ntiles) {
    __shared__ int h[kSortWarpsPerBlock][256];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x * kSortWarpsPerBlock + w;
    for (int d = lane; d < 256; d += 32) h[w][d] = 0;
    __syncwarp();
    if (tile < ntiles) {
        const int base = tile * kTile;
        for (int j = lane; j < kTile; j += 32) {
            const int i = base + j;
            if (i < n) atomicAdd(&h[w][(keys[i] >> shift) & 255], 1);
        }
    }
    __syncwarp();
    if (tile < ntiles)
        for (int d = lane; d < 256; d += 32) hist[d * ntiles + tile] = h[w][d];
}

// Exclusive scan of m ints in three launches: per-block sums, a scan of the
// block sums in one block, then a block-local scan plus the block offset.
constexpr int kScanBlock = 1024;   // threads per scan block
constexpr int kScanItems = 4;      // ints per thread
constexpr int kScanChunk = kScanBlock * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int *sh, int &total) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < (blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    const int before = w > 0 ? sh[w - 1] : 0;
    total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

static __global__ void k_scan_reduce(const int *a, int m, int *sums) {
    __shared__ int sh[32];
    const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < m) s += a[base + k];
    int total;
    block_exclusive_scan(s, sh, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

static __global__ void k_scan_sums(int *sums, int nb) {
    __shared__ int sh[32];
    int run = 0;
    for (int base = 0; base < nb; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, sh, total);
        if (i < nb) sums[i] = run + ex;
        run += total;
    }
}

static __global__ void k_scan_apply(int *a, int m, const int *sums) {
    __shared__ int sh[32];
    const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < m ? a[base + k] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive_scan(s, sh, total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < m) a[base + k] = run;
        run += v[k];
    }
}

static __global__ void k_sort_scatter(const int *kin, const int *vin, int *kout, int *vout, int n, int shift,
                               const int *offs, int ntiles) {
    __shared__ int run[kSortWarpsPerBlock][256];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x * kSortWarpsPerBlock + w;
    if (tile >= ntiles) return;
    for (int d = lane; d < 256; d += 32) run[w][d] = offs[d * ntiles + tile];
    __syncwarp();
    const int base = tile * kTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kTile; r += 32) {
        const int i = base + r + lane;
        const bool ok = i < n;
        const int key = ok ? kin[i] : 0;
        const int d = ok ? (key >> shift) & 255 : 256 + lane;  // out-of-range lanes never match
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt);
        int dst = 0;
        if (ok) dst = run[w][d] + rank;
        __syncwarp();
        if (ok && rank == 0) run[w][d] += __popc(peers);
        __syncwarp();
        if (ok) {
            kout[dst] = key;
            vout[dst] = vin[i];
        }
    }
}

// dst[k*n + j] = src[k*n + perm[j]] for every column k
static __global__ void k_gather_cols(const double *__restrict__ src, double *__restrict__ dst, const int *__restrict__ perm,
                              int n, int ncols) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int s = perm[j];
    for (int k = 0; k < ncols; k++) dst[(size_t)k * n + j] = src[(size_t)k * n + s];
}

static __global__ void k_gather_ints(const int *__restrict__ src, int *__restrict__ dst, const int *__restrict__ perm, int n,
                              int ncols) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int s = perm[j];
    for (int k = 0; k < ncols; k++) dst[(size_t)k * n + j] = src[(size_t)k * n + s];
}

// slot[orig[j]] = j: the slot that holds host particle i (orig is a
// permutation of 0..n-1), so the host order can be gathered -- scattered
// reads, sequential writes -- instead of scattered (partial-sector writes of
// every column)
static __global__ void k_invert_perm(const int *__restrict__ orig, int *__restrict__ slot, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    slot[orig[j]] = j;
}

inline void sort_free(SortWorkspace &w) {
    for (int b = 0; b < 2; b++) {
        if (w.keys[b]) cudaFree(w.keys[b]);
        if (w.vals[b]) cudaFree(w.vals[b]);
        w.keys[b] = w.vals[b] = nullptr;
    }
    if (w.hist) cudaFree(w.hist);
    if (w.sums) cudaFree(w.sums);
    w.sums = nullptr;
    if (w.scratch) cudaFree(w.scratch);
    if (w.iscratch) cudaFree(w.iscratch);
    w.hist = nullptr;
    w.scratch = nullptr;
    w.iscratch = nullptr;
    w.n = 0;
}

inline int sort_alloc(SortWorkspace &w, int n, int nelems, int ncols) {
    sort_free(w);
    w.n = n;
    w.nelems = nelems;
    w.ntiles = (n + kTile - 1) / kTile;
    w.bits = 1;
    while ((1LL << w.bits) < (long long)nelems) w.bits++;
    w.scratch_cols = (size_t)ncols;
    bool ok = true;
    for (int b = 0; b < 2; b++) {
        ok &= cudaMalloc(&w.keys[b], sizeof(int) * n) == cudaSuccess;
        ok &= cudaMalloc(&w.vals[b], sizeof(int) * n) == cudaSuccess;
    }
    ok &= cudaMalloc(&w.hist, sizeof(int) * 256 * w.ntiles) == cudaSuccess;
    ok &= cudaMalloc(&w.sums, sizeof(int) * ((256 * w.ntiles + kScanChunk - 1) / kScanChunk + 1)) == cudaSuccess;
    ok &= cudaMalloc(&w.scratch, sizeof(double) * (size_t)ncols * n) == cudaSuccess;
    ok &= cudaMalloc(&w.iscratch, sizeof(int) * 3 * (size_t)n) == cudaSuccess;
    if (!ok) {
        sort_free(w);
        return 1;
    }
    return 0;
}

// Sort by element, permute every column into the scratch buffers and swap the
// buffers with the live ones.  Column k of the double block holds
// pblock + k*n; the int block holds mat, elem, orig.
void relink_particles(DevParticles &p, double *pblock, int *iblock, int **orig);

// Stable LSD radix sort of n keys (0 <= key < 2^bits) carrying their slot index.
// keys/vals/hist/sums are caller-provided scratch: keys[2], vals[2] of n ints,
// hist of 256*ntiles ints, sums of ceil(256*ntiles/kScanChunk) ints.  Returns
// the buffer index (0 or 1) that holds the sorted keys and the permutation.
// LSD passes over keys[0]/vals[0] already filled; returns the buffer index
// (0 or 1) that holds the sorted keys and the permutation.
inline int radix_sort_passes(int n, int bits, int *keys[2], int *vals[2], int *hist, int *sums, cudaStream_t s) {
    const int ntiles = (n + kTile - 1) / kTile;
    int cur = 0;
    const int tb = (ntiles + kSortWarpsPerBlock - 1) / kSortWarpsPerBlock;
    const int m = 256 * ntiles;
    const int nb = (m + kScanChunk - 1) / kScanChunk;
    for (int shift = 0; shift < bits; shift += 8) {
        k_sort_hist<<<tb, 32 * kSortWarpsPerBlock, 0, s>>>(keys[cur], n, shift, hist, ntiles);
        k_scan_reduce<<<nb, kScanBlock, 0, s>>>(hist, m, sums);
        k_scan_sums<<<1, kScanBlock, 0, s>>>(sums, nb);
        k_scan_apply<<<nb, kScanBlock, 0, s>>>(hist, m, sums);
        k_sort_scatter<<<tb, 32 * kSortWarpsPerBlock, 0, s>>>(keys[cur], vals[cur], keys[1 - cur], vals[1 - cur], n,
                                                              shift, hist, ntiles);
        cur = 1 - cur;
    }
    return cur;
}

// Stable LSD radix sort of n keys (0 <= key < 2^bits) carrying their slot index.
// keys/vals/hist/sums are caller-provided scratch: keys[2], vals[2] of n ints,
// hist of 256*ntiles ints, sums of ceil(256*ntiles/kScanChunk) ints.  Returns
// the buffer index (0 or 1) that holds the sorted keys and the permutation.
inline int radix_sort_keys(const int *elem, int n, int bits, int *keys[2], int *vals[2], int *hist, int *sums,
                           cudaStream_t s) {
    const int TB = 256;
    k_sort_init<<<(n + TB - 1) / TB, TB, 0, s>>>(elem, keys[0], vals[0], n);
    return radix_sort_passes(n, bits, keys, vals, hist, sums, s);
}

inline int sort_particles(SortWorkspace &w, DevParticles &p, double *&pblock, int *&iblock, int *&orig, int ncols,
                          cudaStream_t s) {
    const int n = p.n;
    if (n <= 0) return 0;
    const int TB = 256;
    const int pb = (n + TB - 1) / TB;
    const int cur = radix_sort_keys(p.elem, n, w.bits, w.keys, w.vals, w.hist, w.sums, s);
    const int *perm = w.vals[cur];
    k_gather_cols<<<pb, TB, 0, s>>>(pblock, w.scratch, perm, n, ncols);
    k_gather_ints<<<pb, TB, 0, s>>>(iblock, w.iscratch, perm, n, 3);  // mat, elem, orig
    if (cudaGetLastError() != cudaSuccess) return 1;
    double *old = pblock;
    pblock = w.scratch;
    w.scratch = old;
    int *oldi = iblock;
    iblock = w.iscratch;
    w.iscratch = oldi;
    relink_particles(p, pblock, iblock, &orig);
    return 0;
}

// kernels one sort_particles call launches
inline int sort_launches(const SortWorkspace &w) { return 1 + 5 * ((w.bits + 7) / 8) + 2; }

inline int unsort_to_scratch(SortWorkspace &w, const DevParticles &p, const int *orig, const double *pblock, int ncols,
                             cudaStream_t s) {
    const int n = p.n;
    const int TB = 256, pb = (n + TB - 1) / TB;
    int *slot = w.iscratch + 2 * (size_t)n;  // the third of the int scratch's columns
    k_invert_perm<<<pb, TB, 0, s>>>(orig, slot, n);
    k_gather_cols<<<pb, TB, 0, s>>>(pblock, w.scratch, slot, n, ncols);
    k_gather_ints<<<pb, TB, 0, s>>>(p.mat, w.iscratch, slot, n, 2);  // mat, elem
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace nmg
