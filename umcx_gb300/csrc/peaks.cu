// peaks.cu - micro-benchmarks for the rooflines of the propagation kernel: FP32 FMA issue rate, SFU (MUFU) rate
// and the L2 float-atomic rate at scattered addresses.  The photon kernel is bound by FP32/SFU issue and by L2
// atomics, not by HBM or tensor cores, so these are its denominators.
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/umcx_gpu.h"

namespace {

__global__ void k_fma_rate(float* sink, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-3f, x2 = x0 + 2e-3f, x3 = x0 + 3e-3f;
    float x4 = x0 + 4e-3f, x5 = x0 + 5e-3f, x6 = x0 + 6e-3f, x7 = x0 + 7e-3f;
#pragma unroll 4
    for (int i = 0; i < iters; i++) {
        x0 = fmaf(x0, a, b);
        x1 = fmaf(x1, a, b);
        x2 = fmaf(x2, a, b);
        x3 = fmaf(x3, a, b);
        x4 = fmaf(x4, a, b);
        x5 = fmaf(x5, a, b);
        x6 = fmaf(x6, a, b);
        x7 = fmaf(x7, a, b);
    }
    const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_sfu_rate(float* sink, int iters) {
    float x0 = -0.1f - threadIdx.x * 1e-7f, x1 = x0 - 0.01f, x2 = x0 - 0.02f, x3 = x0 - 0.03f;
#pragma unroll 4
    for (int i = 0; i < iters; i++) {
        x0 = __expf(x0) - 1.0f;
        x1 = __expf(x1) - 1.0f;
        x2 = __expf(x2) - 1.0f;
        x3 = __expf(x3) - 1.0f;
    }
    const float s = x0 + x1 + x2 + x3;
    if (s == 12345.678f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_atomic_rate(float* buf, unsigned n, int iters) {
    unsigned h = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u + 12345u;
    for (int i = 0; i < iters; i++) {
        h ^= h << 13;
        h ^= h >> 17;
        h ^= h << 5;
        atomicAdd(buf + (h % n), 1.0f);
    }
}

}  // namespace

extern "C" int umcx_measure_peaks(int device, umcx_peaks* out) {
    if (!out) return UMCX_ERR_INPUT;
    std::memset(out, 0, sizeof(*out));
    if (cudaSetDevice(device) != cudaSuccess) return UMCX_ERR_NODEV;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 256, grid = sms * 8;
    const unsigned n = 11u << 20;  // 44 MB of floats: L2-resident scattered targets
    float* buf = nullptr;
    if (cudaMalloc(&buf, n * sizeof(float)) != cudaSuccess) return UMCX_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms = 0.f;
    const int fma_iters = 1 << 13, sfu_iters = 1 << 11, at_iters = 64;
    // warm-up, then timed runs
    k_fma_rate<<<grid, block>>>(buf, 64, 0.999f, 1e-3f);
    cudaEventRecord(e0);
    k_fma_rate<<<grid, block>>>(buf, fma_iters, 0.999f, 1e-3f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    out->fp32_fma_per_s = 8.0 * grid * block * static_cast<double>(fma_iters) / (ms * 1e-3);
    k_sfu_rate<<<grid, block>>>(buf, 64);
    cudaEventRecord(e0);
    k_sfu_rate<<<grid, block>>>(buf, sfu_iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    out->sfu_per_s = 4.0 * grid * block * static_cast<double>(sfu_iters) / (ms * 1e-3);
    cudaMemset(buf, 0, n * sizeof(float));
    k_atomic_rate<<<grid, block>>>(buf, n, 4);
    cudaEventRecord(e0);
    k_atomic_rate<<<grid, block>>>(buf, n, at_iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    out->l2_atomic_per_s = static_cast<double>(grid) * block * at_iters / (ms * 1e-3);
    int clk = 0;
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, device);
    out->sm_count = sms;
    out->sm_clock_khz = clk;
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    return err == cudaSuccess ? UMCX_OK : UMCX_ERR_CUDA;
}
