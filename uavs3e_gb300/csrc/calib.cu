// Throughput calibration for roofline reporting: the issue rates of the 4-sample SAD
// instruction (vabsdiff4 with accumulate) that bounds the integer motion search and of the
// 2-way halfword dot product (dp2a) that carries the intra lattice's transforms, measured with
// independent accumulation chains and no memory traffic.
#include "common.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

namespace uc {

constexpr int CAL_ITERS = 4096;
constexpr int CAL_CHAINS = 8;

__global__ void __launch_bounds__(256) k_sad4_rate(u32 *sink, u32 seed)
{
    u32 a[CAL_CHAINS], acc[CAL_CHAINS];
#pragma unroll
    for (int i = 0; i < CAL_CHAINS; i++) { a[i] = seed * (i + 1) + threadIdx.x; acc[i] = 0; }
    u32 b = seed ^ threadIdx.x;
    for (int it = 0; it < CAL_ITERS; it++) {
#pragma unroll
        for (int i = 0; i < CAL_CHAINS; i++) acc[i] = sad4(a[i], b, acc[i]);
        b += 0x01010101u;
    }
    u32 t = 0;
#pragma unroll
    for (int i = 0; i < CAL_CHAINS; i++) t += acc[i];
    if (t == 0x9E3779B9u) sink[0] = t;   // keeps the chains live; practically never taken
}

__global__ void __launch_bounds__(256) k_dp2a_rate(u32 *sink, u32 seed)
{
    int acc[CAL_CHAINS];
    u32 a[CAL_CHAINS];
#pragma unroll
    for (int i = 0; i < CAL_CHAINS; i++) { a[i] = seed * (i + 1) + threadIdx.x; acc[i] = 0; }
    u32 b = seed ^ threadIdx.x;
    for (int it = 0; it < CAL_ITERS; it++) {
#pragma unroll
        for (int i = 0; i < CAL_CHAINS; i++) asm("dp2a.lo.s32.s32 %0, %1, %2, %0;" : "+r"(acc[i]) : "r"(a[i]), "r"(b));
        b += 0x01010101u;
    }
    int t = 0;
#pragma unroll
    for (int i = 0; i < CAL_CHAINS; i++) t += acc[i];
    if (t == 0x1E3779B9) sink[0] = (u32)t;   // keeps the chains live; practically never taken
}

// instructions per second and per clock per SM of one of the calibration kernels
static int measure_rate(void (*k)(u32 *, u32), double *ops_per_s, double *ops_per_clk_sm)
{
    int r = ensure_init();
    if (r) return r;
    int dev = 0, sms = 0, clk_khz = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "measure: device index");
    UC_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    UC_CHECK(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev));
    static u32 *sink[64];
    if (!sink[dev]) UC_CHECK(cudaMalloc(&sink[dev], 64));
    const int blocks = sms * 8, threads = 256, reps = 5;
    cudaEvent_t e0, e1;
    UC_CHECK(cudaEventCreate(&e0));
    UC_CHECK(cudaEventCreate(&e1));
    k<<<blocks, threads>>>(sink[dev], 1);
    UC_CHECK(cudaDeviceSynchronize());
    UC_CHECK(cudaEventRecord(e0));
    for (int i = 0; i < reps; i++) k<<<blocks, threads>>>(sink[dev], i + 2);
    UC_CHECK(cudaEventRecord(e1));
    UC_CHECK(cudaEventSynchronize(e1));
    float ms = 0;
    UC_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    count_launch(reps + 1);
    const double ops = (double)reps * blocks * threads * CAL_ITERS * CAL_CHAINS;
    const double rate = ops / (ms / 1e3);
    if (ops_per_s) *ops_per_s = rate;
    if (ops_per_clk_sm) *ops_per_clk_sm = rate / ((double)clk_khz * 1e3) / sms;
    return UC_OK;
}

}  // namespace uc

using namespace uc;

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_measure_sad4_rate(double *ops_per_s, double *ops_per_clk_sm)
{
    return measure_rate(k_sad4_rate, ops_per_s, ops_per_clk_sm);
}

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_measure_dp2a_rate(double *ops_per_s, double *ops_per_clk_sm)
{
    return measure_rate(k_dp2a_rate, ops_per_s, ops_per_clk_sm);
}
