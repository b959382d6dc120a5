/*
 * probe.cu -- FP64 throughput probe (c2a_probe.h).  Each thread keeps eight
 * independent chains so that the pipe, not the chain latency, limits the
 * rate; the chains' values stay bounded (x -> x * a + b with a < 1) and feed
 * one guarded store so nothing is optimised away.
 */
#include <cuda_runtime.h>

#include "../../include/c2a_probe.h"

namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeChains = 8;
constexpr int kProbeIters = 4096;

template <bool FMA>
__global__ void __launch_bounds__(kProbeThreads) c2a_fp64_probe_kernel(double *sink, double a, double b)
{
    double x[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; k++) x[k] = 1.0 + 1e-9 * (threadIdx.x + 7 * k);
#pragma unroll 4
    for (int i = 0; i < kProbeIters; i++) {
#pragma unroll
        for (int k = 0; k < kProbeChains; k++) {
            if (FMA)
                x[k] = fma(x[k], a, b);
            else
                x[k] = __dadd_rn(x[k], b);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kProbeChains; k++) s += x[k];
    if (s == -1.0) sink[threadIdx.x] = s; /* never true: keeps the chains live */
}

} // namespace

extern "C" c2a_status c2a_probe_fp64_peak(int device, int repeats, double *fma_flops, double *add_flops)
{
    if (!fma_flops || !add_flops || repeats < 1) return C2A_ERR_INVALID_ARGUMENT;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return C2A_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return C2A_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return C2A_ERR_CUDA;
    double *sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    c2a_status st = C2A_OK;
    if (cudaMalloc(&sink, sizeof(double) * kProbeThreads) != cudaSuccess) return C2A_ERR_OUT_OF_MEMORY;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        st = C2A_ERR_CUDA;
    const int blocks = sms * (2048 / kProbeThreads);
    const double per_launch = (double)blocks * kProbeThreads * kProbeChains * kProbeIters;
    for (int variant = 0; variant < 2 && st == C2A_OK; variant++) {
        double best = 0.0;
        for (int r = -1; r < repeats && st == C2A_OK; r++) { /* r = -1: untimed warm-up */
            cudaEventRecord(e0, s);
            if (variant == 0)
                c2a_fp64_probe_kernel<true><<<blocks, kProbeThreads, 0, s>>>(sink, 0.999999, 1e-7);
            else
                c2a_fp64_probe_kernel<false><<<blocks, kProbeThreads, 0, s>>>(sink, 0.999999, 1e-7);
            cudaEventRecord(e1, s);
            float ms = 0.f;
            if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                st = C2A_ERR_CUDA;
                break;
            }
            const double rate = per_launch * (variant == 0 ? 2.0 : 1.0) / (ms * 1e-3);
            if (r >= 0 && rate > best) best = rate;
        }
        (variant == 0 ? *fma_flops : *add_flops) = best;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(sink);
    return st;
}
