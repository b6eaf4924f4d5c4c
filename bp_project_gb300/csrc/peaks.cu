// FP32 issue-rate microbenchmark: the measured denominator of the back-projection kernels'
// FP32 roofline.  Every thread runs eight independent FMA chains (scalar FFMA or packed f32x2
// FFMA2), enough to cover the pipe's latency at full occupancy, on values that stay finite
// (x <- x * a + b with a slightly below one).  The result is flops (FMA = 2, a packed FMA = 4)
// per second over the kernel's CUDA-event duration.
#include "common.cuh"

namespace sarbp {
namespace {

__device__ float g_peak_sink;

template <bool PACKED>
__global__ void __launch_bounds__(256) fp32_peak_kernel(int iters, float seed) {
    const float a = 0.9999999f, b = 1e-7f * (float)(threadIdx.x & 7);
    if (PACKED) {
        float2 x[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = make_float2(seed + (float)i, seed - (float)i);
        const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
#pragma unroll 4
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int i = 0; i < 8; ++i) x[i] = __ffma2_rn(x[i], a2, b2);
        }
        float s = 0.0f;
#pragma unroll
        for (int i = 0; i < 8; ++i) s += x[i].x + x[i].y;
        if (s == 1.2345678e30f) g_peak_sink = s;  // never true: keeps the chains live
    } else {
        float x[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = seed + (float)i;
#pragma unroll 4
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int i = 0; i < 8; ++i) x[i] = fmaf(x[i], a, b);
        }
        float s = 0.0f;
#pragma unroll
        for (int i = 0; i < 8; ++i) s += x[i];
        if (s == 1.2345678e30f) g_peak_sink = s;
    }
}

}  // namespace
}  // namespace sarbp

using namespace sarbp;

extern "C" int sarbp_fp32_peak(int packed, int iters, double* tflops) {
    if (!tflops) return fail(SARBP_ERR_TYPE, "tflops must not be NULL");
    if (packed != 0 && packed != 1) return fail(SARBP_ERR_VALUE, "packed must be 0 or 1");
    if (iters < 1 || iters > (1 << 24)) return fail(SARBP_ERR_VALUE, "iters must be in [1, 2^24]");
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, packed ? (const void*)fp32_peak_kernel<true> : (const void*)fp32_peak_kernel<false>, 256, 0);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "fp32_peak: %s", cudaGetErrorString(e));
    const int blocks = sms * (per_sm > 0 ? per_sm : 1);
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    float ms = 0.0f;
    if (e == cudaSuccess) {
        // One untimed launch, then the timed one, both on the legacy default stream.
        for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
            if (rep == 1) e = cudaEventRecord(t0, 0);
            if (packed)
                fp32_peak_kernel<true><<<blocks, 256>>>(iters, 1.0f);
            else
                fp32_peak_kernel<false><<<blocks, 256>>>(iters, 1.0f);
            if (e == cudaSuccess) e = cudaGetLastError();
        }
        note_launches(2);
        if (e == cudaSuccess) e = cudaEventRecord(t1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(t1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (e != cudaSuccess) return fail(SARBP_ERR_CUDA, "fp32_peak: %s", cudaGetErrorString(e));
    const double flops = (double)blocks * 256.0 * iters * 8.0 * (packed ? 4.0 : 2.0);
    *tflops = flops / (ms * 1e-3) / 1e12;
    return SARBP_OK;
}
