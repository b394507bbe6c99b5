// probe.cu -- measured arithmetic peaks of the GPU the library runs on.
//
// The FP64 path of the step is bound by the FP64 pipe, not by HBM: GB300
// executes FP64 FMAs at a small fraction of its FP32 rate.  Its roofline
// fraction is therefore taken against the FP64 FMA throughput measured here
// on the same GPU, in the same process, rather than against a datasheet figure.
#include <cuda_runtime.h>

#include <string>

#include "host_common.cuh"
#include "nairn_mpm_gpu.h"

namespace {

constexpr int kChains = 8;  // independent FMA chains per thread, enough to fill the pipe

// Each thread runs kChains independent FMA chains for `iters` iterations; the
// values stay bounded (x <- x a + b with |a| < 1), and the sum is written when it
// equals an impossible value, so the compiler cannot drop the loop.
template <typename T>
__global__ void k_fma_chains(T *out, int iters, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (T)(threadIdx.x + c) * (T)1e-6;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == (T)-1.2345e300f) out[0] = s;
}

template <typename T>
int fma_rate(int iters, double *tflops, double *ms_out) {
    if (iters < 1 || !tflops) return MPMGPU_ERR_INVALID;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    T *out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(T));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    if (e == cudaSuccess) {
        k_fma_chains<T><<<blocks, threads, 0, s>>>(out, iters / 8 + 1, (T)0.999999, (T)1e-7);  // warm-up
        cudaEventRecord(e0, s);
        k_fma_chains<T><<<blocks, threads, 0, s>>>(out, iters, (T)0.999999, (T)1e-7);
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e1) cudaEventDestroy(e1);
    if (e0) cudaEventDestroy(e0);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    if (e != cudaSuccess) return nmg::fail_static(MPMGPU_ERR_CUDA, std::string("FMA rate probe: ") + cudaGetErrorString(e));
    const double flops = 2.0 * kChains * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
    return MPMGPU_OK;
}

}  // namespace

extern "C" {

// Extension: FP64 FMA throughput of the current device in TFLOP/s (2 flops per
// FMA), from one kernel of independent FMA chains timed with CUDA events.
int mpmgpu_fp64_fma_rate(int32_t iters, double *tflops, double *ms) { return fma_rate<double>(iters, tflops, ms); }

// Extension: the same for FP32 FMAs.
int mpmgpu_fp32_fma_rate(int32_t iters, double *tflops, double *ms) { return fma_rate<float>(iters, tflops, ms); }

}  // extern "C"
