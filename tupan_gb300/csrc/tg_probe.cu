// tg_probe.cu -- issue-rate probes that measure this GPU's FP32 and FP64
// FMA peaks, the denominators of the pairwise kernels' roofline.
//
// Each thread runs NCHAIN independent FMA chains for `iters` rounds; the
// grid is SMs x 8 CTAs of 256 threads.  The FP32 probe uses packed FFMA2 (two
// FMAs per instruction, so the FMA pipe rather than instruction issue is the
// limit).  Seconds come from CUDA events on the caller's stream.
#include <cuda_runtime.h>

#include "../../include/tupan_gb300.h"
#include "tg_device.cuh"

namespace {

constexpr int NCHAIN = 8;

__global__ void probe_fp32(float *sink, int iters, float a, float b) {
    float2 acc[NCHAIN];
    for (int k = 0; k < NCHAIN; ++k) acc[k] = make_float2(threadIdx.x * 1e-7f + k, k * 1e-3f);
    const float2 va = make_float2(a, a), vb = make_float2(b, b);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < NCHAIN; ++k) acc[k] = __ffma2_rn(acc[k], va, vb);
    }
    float s = 0.f;
    for (int k = 0; k < NCHAIN; ++k) s += acc[k].x + acc[k].y;
    if (s == 12345.678f) sink[blockIdx.x] = s;   // keeps the chains alive
}

// Packed FFMA2 chains interleaved with as many scalar FFMA chains: shows
// whether scalar FP32 work can overlap packed work on the FMA pipes.
__global__ void probe_fp32_mixed(float *sink, int iters, float a, float b) {
    float2 acc[NCHAIN];
    float sc[NCHAIN];
    for (int k = 0; k < NCHAIN; ++k) {
        acc[k] = make_float2(threadIdx.x * 1e-7f + k, k * 1e-3f);
        sc[k] = k * 2e-3f;
    }
    const float2 va = make_float2(a, a), vb = make_float2(b, b);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < NCHAIN; ++k) {
            acc[k] = __ffma2_rn(acc[k], va, vb);
            sc[k] = fmaf(sc[k], a, b);
        }
    }
    float s = 0.f;
    for (int k = 0; k < NCHAIN; ++k) s += acc[k].x + acc[k].y + sc[k];
    if (s == 12345.678f) sink[blockIdx.x] = s;
}

__global__ void probe_fp64(double *sink, int iters, double a, double b) {
    double acc[NCHAIN];
    for (int k = 0; k < NCHAIN; ++k) acc[k] = threadIdx.x * 1e-7 + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < NCHAIN; ++k) acc[k] = fma(acc[k], a, b);
    }
    double s = 0.0;
    for (int k = 0; k < NCHAIN; ++k) s += acc[k];
    if (s == 12345.678) sink[blockIdx.x] = s;
}

// One CTA waits, with the pairwise kernels' bounded poll, on an mbarrier
// that expects one arrival; thread 0 arrives only if `arrive` is set.  A wait
// that gives up raises TG_ST_MBAR_TIMEOUT in *status, as the split-FP32
// kernels do when a j-tile copy never completes.
__global__ void bounded_wait(unsigned polls, int arrive, unsigned *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tg::mbar_init(&bar, 1);
        tg::fence_mbar_init();
    }
    __syncthreads();
    if (arrive && threadIdx.x == 0) tg::mbar_expect_tx(&bar, 0);   // an arrival with no bytes
    const bool ok = tg::mbar_wait(&bar, 0, polls);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(status, TG_ST_MBAR_TIMEOUT);
}

}  // namespace

extern "C" {

// Runs bounded_wait once on the current device and returns the status bits
// it raised (0 or TG_ST_MBAR_TIMEOUT), or a negative TG_E* code; *ms gets
// the kernel's duration.
int tg_check_bounded_wait(unsigned polls, int arrive, double *ms) {
    unsigned *d = nullptr, h = 0;
    if (cudaMalloc(&d, sizeof(unsigned)) != cudaSuccess) return TG_ENOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemset(d, 0, sizeof(unsigned));
    cudaEventRecord(e0, 0);
    bounded_wait<<<1, 32>>>(polls, arrive, d);
    cudaEventRecord(e1, 0);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) return TG_ECUDA;
    if (ms) *ms = t;
    return (int)h;
}

// Measured dense FMA throughput in TFLOP/s (2 flops per FMA) for FP32
// (which = 0) or FP64 (which = 1) on the current device; negative on error.
double tg_probe_fma_tflops(int which, int iters, void *stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    const int blocks = sms * 8, threads = 256;
    void *sink = nullptr;
    if (cudaMalloc(&sink, blocks * sizeof(double)) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, s);
        if (which == 0)
            probe_fp32<<<blocks, threads, 0, s>>>(static_cast<float *>(sink), iters, 0.999999f, 1e-6f);
        else if (which == 2)
            probe_fp32_mixed<<<blocks, threads, 0, s>>>(static_cast<float *>(sink), iters, 0.999999f, 1e-6f);
        else
            probe_fp64<<<blocks, threads, 0, s>>>(static_cast<double *>(sink), iters, 0.999999, 1e-6);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) { best = -1.0; break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double fmas = (double)blocks * threads * iters * NCHAIN * (which == 0 ? 2.0 : which == 2 ? 3.0 : 1.0);
        const double tf = 2.0 * fmas / (ms * 1e-3) / 1e12;
        if (rep > 0 && tf > best) best = tf;   // first launch is warm-up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (cudaGetLastError() != cudaSuccess) return -1.0;
    return best;
}

}  // extern "C"
