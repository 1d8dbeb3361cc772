/* mwsep_peaks.cu -- the project's own pipe microbenchmark.
 *
 * The separation kernels are bound by arithmetic pipes, not by HBM or the
 * tensor cores: the plain form by the FP64 pipe, the compensated form by the
 * FP32 pipe and the SFU (ex2 / rsqrt / rcp approximations).  These kernels
 * measure each pipe's throughput on this GPU with long chains of independent
 * operations, so the roofline fractions are taken against measured peaks.
 */
#include <cuda_runtime.h>
#include "milkyway_separation_gb300.h"
#include "mwsep_status.h"

namespace {

constexpr int kChains = 8;
/* iterations per pipe, sized so each launch runs for roughly 0.1-0.3 s */
constexpr int kItersF64 = 128;
constexpr int kItersF32 = 2048;
constexpr int kItersMufu = 512;

__global__ void dfma_kernel(double* out, double a, double b)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-9 + c;
    for (int i = 0; i < kItersF64; ++i)
    {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678) out[0] = s;
}

__global__ void ffma_kernel(float* out, float a, float b)
{
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 1e-6f + c;
    for (int i = 0; i < kItersF32; ++i)
    {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678f) out[0] = s;
}

template <int OP>
__global__ void mufu_kernel(float* out)
{
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 0.5f + threadIdx.x * 1e-7f + c * 1e-3f;
    for (int i = 0; i < kItersMufu; ++i)
    {
#pragma unroll
        for (int c = 0; c < kChains; ++c)
        {
            /* y = f(x) + k keeps every chain bounded and stops the
             * compiler from folding f(f(x)) (rcp of rcp is the identity) */
            float y;
            if (OP == 0) asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            else if (OP == 1) asm volatile("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            else asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            x[c] = y + (OP == 0 ? -1.0f : 0.5f);
        }
    }
    float s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678f) out[0] = s;
}

template <typename F>
int time_kernel(F launch, cudaStream_t st, float& ms)
{
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return MWSEP_ERR_CUDA;
    launch(); /* warm-up */
    cudaEventRecord(a, st);
    for (int r = 0; r < 3; ++r) launch();
    cudaEventRecord(b, st);
    if (cudaEventSynchronize(b) != cudaSuccess) return MWSEP_ERR_CUDA;
    cudaEventElapsedTime(&ms, a, b);
    ms /= 3.0f;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return cudaGetLastError() == cudaSuccess ? MWSEP_OK : MWSEP_ERR_CUDA;
}

} // namespace

extern "C" int mwsep_measure_pipe_peaks(int device, mwsep_pipe_peaks* out)
{
    if (!out) return mwsep_fail(MWSEP_ERR_ARG);
    if (cudaSetDevice(device) != cudaSuccess) return mwsep_fail(MWSEP_ERR_CUDA);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return mwsep_fail(MWSEP_ERR_CUDA);
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return mwsep_fail(MWSEP_ERR_CUDA);
    void* buf = nullptr;
    if (cudaMalloc(&buf, 64) != cudaSuccess)
    {
        cudaStreamDestroy(st);
        return mwsep_fail(MWSEP_ERR_NOMEM);
    }
    const int sms = prop.multiProcessorCount;
    const int block = 256, grid = sms * 8;
    const double lanes = (double)grid * block * kChains;
    float ms = 0.f;
    int rc = MWSEP_OK;
    rc |= time_kernel([&] { dfma_kernel<<<grid, block, 0, st>>>((double*)buf, 0.999999, 1e-7); }, st, ms);
    out->fp64_fma_tflops = 2.0 * lanes * kItersF64 / (ms * 1e-3) / 1e12;
    rc |= time_kernel([&] { ffma_kernel<<<grid, block, 0, st>>>((float*)buf, 0.999999f, 1e-7f); }, st, ms);
    out->fp32_fma_tflops = 2.0 * lanes * kItersF32 / (ms * 1e-3) / 1e12;
    rc |= time_kernel([&] { mufu_kernel<0><<<grid, block, 0, st>>>((float*)buf); }, st, ms);
    out->ex2_gops = lanes * kItersMufu / (ms * 1e-3) / 1e9;
    rc |= time_kernel([&] { mufu_kernel<1><<<grid, block, 0, st>>>((float*)buf); }, st, ms);
    out->rsqrt_gops = lanes * kItersMufu / (ms * 1e-3) / 1e9;
    rc |= time_kernel([&] { mufu_kernel<2><<<grid, block, 0, st>>>((float*)buf); }, st, ms);
    out->rcp_gops = lanes * kItersMufu / (ms * 1e-3) / 1e9;
    out->sm_count = sms;
    cudaFree(buf);
    cudaStreamDestroy(st);
    return rc ? mwsep_fail(MWSEP_ERR_CUDA) : MWSEP_OK;
}
