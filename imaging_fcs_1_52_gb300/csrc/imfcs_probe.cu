// imfcs_probe.cu -- FP32 issue-rate probe: the denominator of the fit
// stage's roofline (the LM and the correlator are FP32 CUDA-core work, and
// no FP32 figure comes with the device's measured peaks).
//
// Every thread runs kChains independent FMA chains a <- a * b + c for
// `iters` steps, so the FP32 pipe is fed without dependency stalls; the grid
// fills every SM with kBlocksPerSm blocks of 256 threads.  The chains' sum is
// stored only when it equals a value no chain reaches (b, c are run-time
// arguments), which keeps the compiler from removing the loop.
#include "imfcs_gb300.h"
#include "imfcs_host.h"

using namespace imfcs;

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kBlocksPerSm = 8;

__global__ void __launch_bounds__(kThreads) fma_probe_kernel(float b, float c, int iters, float *sink)
{
    float a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = (float)(threadIdx.x + i) * 1e-3f;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int i = 0; i < kChains; i++) a[i] = fmaf(a[i], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kChains; i++) s += a[i];
    if (s == -1.2345e30f) sink[0] = s;
}

}  // namespace

extern "C" int imfcs_measure_fp32_fma_rate(double *fma_per_s, void *stream)
{
    if (!fma_per_s) { set_error("null argument"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *sink = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int iters = 16384;
    const dim3 grid(sms * kBlocksPerSm);
    float best = 0.f;
    for (int rep = 0; rep < 6 && e == cudaSuccess; rep++) {   // the first launch warms up
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) {
            fma_probe_kernel<<<grid, kThreads, 0, s>>>(0.999f, 1e-4f, iters, sink);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "FP32 FMA probe")); return 1; }
    const double fmas = (double)grid.x * kThreads * kChains * iters;
    *fma_per_s = fmas / (best * 1e-3);
    return 0;
}
