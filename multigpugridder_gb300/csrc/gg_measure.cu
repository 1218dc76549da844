// Bandwidth probe for the roofline the projection kernels are reported against.
//
// gg_measure_l2_read_gbs measures the L2 read bandwidth of the current
// device: a buffer a little under half the L2 (so that it stays resident)
// is read over and over with L2-only loads (ld.global.cg, no L1), by a grid
// of a few CTAs per SM; the time comes from CUDA events around each run and
// the best of the runs is reported.  The reference has no counterpart (it
// measures nothing beyond MATLAB tic/toc).
#include <algorithm>

#include "gg_internal.h"
#include "../../include/gg_gridder.h"

namespace gg {

constexpr int kProbeThreads = 512;

__global__ void __launch_bounds__(kProbeThreads) l2_read_kernel(const float4 *__restrict__ p, size_t n4, int passes,
                                                                float *__restrict__ sink)
{
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int r = 0; r < passes; r++) {
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
            const float4 v = __ldcg(p + i);
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
        }
    }
    // keeps the loads; the buffer is zero, so the sum is zero and nothing is stored
    if (acc.x + acc.y + acc.z + acc.w != 0.0f) sink[blockIdx.x] = acc.x + acc.y + acc.z + acc.w;
}

} // namespace gg

using namespace gg;

extern "C" int gg_measure_l2_read_gbs(int runs, double *gbs_out)
{
    if (!gbs_out || runs <= 0) {
        set_global_error("gg_measure_l2_read_gbs: gbs_out is required and runs must be positive");
        return GG_ERR_INVALID_ARG;
    }
    int dev = 0, l2 = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || l2 <= 0 || sms <= 0) {
        set_global_error(e != cudaSuccess ? cudaGetErrorString(e) : "no L2 size or SM count for this device");
        return GG_ERR_CUDA;
    }
    // under half the L2, a multiple of 1 MiB
    const size_t bytes = std::max<size_t>((size_t)l2 * 4 / 10 / (1 << 20), 1) << 20;
    const size_t n4 = bytes / sizeof(float4);
    float4 *buf = nullptr;
    float *sink = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    const int grid = sms * 4;
    const int passes = 40;
    double best = 0.0;
    e = cudaMalloc(&buf, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&sink, grid * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(buf, 0, bytes);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    if (e == cudaSuccess) {
        l2_read_kernel<<<grid, kProbeThreads>>>(buf, n4, 2, sink); // warm: the buffer into L2
        count_launches(1);
        e = cudaGetLastError();
    }
    for (int r = 0; r < runs && e == cudaSuccess; r++) {
        cudaEventRecord(a);
        l2_read_kernel<<<grid, kProbeThreads>>>(buf, n4, passes, sink);
        count_launches(1);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess && ms > 0.0f) best = std::max(best, (double)bytes * passes / (ms * 1e-3) / 1e9);
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (sink) cudaFree(sink);
    if (buf) cudaFree(buf);
    if (e != cudaSuccess) {
        set_global_error(cudaGetErrorString(e));
        return GG_ERR_CUDA;
    }
    *gbs_out = best;
    return GG_OK;
}
