// bem_peaks.cu - issue-rate micro-kernels: the FP32 FMA, special-function
// (sin / cos / rsqrt approximations) and FP64 FMA peaks of the device, the
// denominators of the compute-bound stages' rooflines (assembly, projection,
// block inverses).  Each kernel runs independent dependency chains in every
// lane of a full grid, so the pipe, not latency, bounds it; the result is the
// instruction rate over the CUDA-event time of the launch.
#include <cuda_runtime.h>

#include "../../include/bem_gb300.h"
#include "bem_internal.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) k_peak_ffma(float *out, float b, float c) {
    float a[kChains];
#pragma unroll
    for (int q = 0; q < kChains; ++q) a[q] = (float)(threadIdx.x + q);
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int q = 0; q < kChains; ++q) a[q] = fmaf(a[q], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < kChains; ++q) s += a[q];
    if (s == 1234.5f) out[blockIdx.x] = s;   // keeps the chains alive
}

__global__ void __launch_bounds__(256) k_peak_mufu(float *out) {
    float a[kChains];
#pragma unroll
    for (int q = 0; q < kChains; ++q) a[q] = 0.1f * (float)(threadIdx.x + q);
    for (int it = 0; it < kIters / 4; ++it) {
#pragma unroll
        for (int q = 0; q < kChains; ++q) {
            float s, c, r;
            asm volatile("sin.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(a[q]));
            asm volatile("cos.approx.ftz.f32 %0, %1;" : "=f"(c) : "f"(s));
            asm volatile("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(c));
            asm volatile("sin.approx.ftz.f32 %0, %1;" : "=f"(a[q]) : "f"(r));
        }
    }
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < kChains; ++q) s += a[q];
    if (s == 1234.5f) out[blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_peak_dfma(double *out, double b, double c) {
    double a[kChains];
#pragma unroll
    for (int q = 0; q < kChains; ++q) a[q] = (double)(threadIdx.x + q);
    for (int it = 0; it < kIters / 8; ++it) {
#pragma unroll
        for (int q = 0; q < kChains; ++q) a[q] = fma(a[q], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kChains; ++q) s += a[q];
    if (s == 1234.5) out[blockIdx.x] = s;
}

}  // namespace

extern "C" bem_status bem_measure_issue_peaks(int32_t device, double *rates) {
    if (!rates) {
        bem::set_error("bem_measure_issue_peaks: null output");
        return BEM_ERR_INVALID;
    }
    cudaError_t e = cudaSetDevice(device);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        bem::set_error(cudaGetErrorString(e));
        return BEM_ERR_CUDA;
    }
    const int blocks = sms * 8, threads = 256;   // 2048 resident threads per SM
    const double lanes = (double)blocks * threads;
    double *buf = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    e = cudaMalloc(&buf, (size_t)blocks * sizeof(double));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    for (auto &v : ev)
        if (e == cudaSuccess) e = cudaEventCreate(&v);
    // per kernel: operations per lane, best of three timed launches after one warm-up
    const double ops[3] = {(double)kIters * kChains, (double)(kIters / 4) * kChains * 4,
                           (double)(kIters / 8) * kChains};
    for (int kind = 0; kind < 3 && e == cudaSuccess; ++kind) {
        float best = 1e30f;
        for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
            e = cudaEventRecord(ev[0], st);
            if (kind == 0) k_peak_ffma<<<blocks, threads, 0, st>>>((float *)buf, 0.999f, 1e-3f);
            else if (kind == 1) k_peak_mufu<<<blocks, threads, 0, st>>>((float *)buf);
            else k_peak_dfma<<<blocks, threads, 0, st>>>(buf, 0.999, 1e-3);
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (e == cudaSuccess && rep > 0 && ms < best) best = ms;
        }
        bem::count_launches(4);
        rates[kind] = e == cudaSuccess ? lanes * ops[kind] / (best * 1e-3) : 0.0;
    }
    for (auto &v : ev)
        if (v) cudaEventDestroy(v);
    if (st) cudaStreamDestroy(st);
    cudaFree(buf);
    if (e != cudaSuccess) {
        bem::set_error(cudaGetErrorString(e));
        return BEM_ERR_CUDA;
    }
    return BEM_OK;
}
