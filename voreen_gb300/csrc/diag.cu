// Diagnostics: the L2 read bandwidth the march's gathers are measured
// against (an L2-resident buffer read repeatedly by every SM).
#include <cuda_runtime.h>

#include <string>

#include "vrc_internal.h"

namespace {

__global__ void l2_read_kernel(const uint4* __restrict__ buf, long long n, int reps, uint4* __restrict__ sink) {
    uint4 acc = make_uint4(0, 0, 0, 0);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; ++r)
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
            const uint4 v = __ldcg(buf + i);
            acc.x ^= v.x;
            acc.y ^= v.y;
            acc.z ^= v.z;
            acc.w ^= v.w;
        }
    sink[blockIdx.x * (long long)blockDim.x + threadIdx.x] = acc;
}

}  // namespace

extern "C" vrc_status vrc_occupancy_distance(vrc_context* ctx, const uint32_t* d_bits, int nx, int ny, int nz,
                                             uint8_t* d_out) {
    if (!ctx || !d_bits || !d_out || nx < 1 || ny < 1 || nz < 1) return VRC_ERR_INVALID_ARG;
    const long long n = (long long)nx * ny * nz;
    if (n >= (1LL << 32)) return VRC_ERR_INVALID_ARG;
    const int nc[3] = {nx, ny, nz};
    uint8_t* tmp = nullptr;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaMalloc(&tmp, (size_t)n);
    if (e == cudaSuccess) e = vrc::launch_occ_distance(d_bits, nc, d_out, tmp, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) {
        ctx->last_error = std::string("vrc_occupancy_distance: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? VRC_ERR_OUT_OF_MEMORY : VRC_ERR_CUDA;
    }
    return VRC_OK;
}

extern "C" vrc_status vrc_measure_l2_read(vrc_context* ctx, size_t bytes, int reps, float* gbs) {
    if (!ctx || !gbs || bytes < (1u << 20) || reps < 1) return VRC_ERR_INVALID_ARG;
    *gbs = 0.f;
    cudaError_t e = cudaSetDevice(ctx->device);
    const long long n = (long long)(bytes / 16);
    const int blocks = ctx->num_sms * 8, threads = 256;
    uint4 *buf = nullptr, *sink = nullptr;
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaMalloc(&buf, (size_t)n * 16);
    if (e == cudaSuccess) e = cudaMalloc(&sink, (size_t)blocks * threads * 16);
    if (e == cudaSuccess) e = cudaMemsetAsync(buf, 1, (size_t)n * 16, ctx->stream);
    if (e == cudaSuccess) {
        l2_read_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, n, 2, sink);  // bring the buffer into L2
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[0], ctx->stream);
    if (e == cudaSuccess) {
        l2_read_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, n, reps, sink);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[1], ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) {
        ctx->last_error = std::string("vrc_measure_l2_read: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? VRC_ERR_OUT_OF_MEMORY : VRC_ERR_CUDA;
    }
    *gbs = ms > 0.f ? (float)((double)n * 16.0 * reps / (ms * 1e-3) / 1e9) : 0.f;
    return VRC_OK;
}
