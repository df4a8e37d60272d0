// Rescale of a rendered RGBA image to the output size: the copy that
// VolumeRaycaster::rescaleRendering (src/core/processors/volumeraycaster.cpp:348-375)
// draws after an interaction-coarseness render (singlevolumeraycaster.cpp:253-256,
// 413-419): the source bound with GL_LINEAR, clamped to the edge, sampled at
// the destination pixel centres.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vrc_internal.h"

namespace {

template <typename T> __device__ __forceinline__ float4 load_px(const T* img, int i);
template <> __device__ __forceinline__ float4 load_px<uchar4>(const uchar4* img, int i) {
    const uchar4 v = img[i];
    return make_float4(v.x / 255.f, v.y / 255.f, v.z / 255.f, v.w / 255.f);
}
template <> __device__ __forceinline__ float4 load_px<float4>(const float4* img, int i) { return img[i]; }

__device__ __forceinline__ void store_px(uchar4* img, size_t i, float4 v) {
    auto q = [](float x) { return (unsigned char)floorf(fminf(fmaxf(x, 0.f), 1.f) * 255.f + 0.5f); };
    img[i] = make_uchar4(q(v.x), q(v.y), q(v.z), q(v.w));
}
__device__ __forceinline__ void store_px(float4* img, size_t i, float4 v) { img[i] = v; }

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
    return make_float4(__fmaf_rn(t, b.x - a.x, a.x), __fmaf_rn(t, b.y - a.y, a.y), __fmaf_rn(t, b.z - a.z, a.z),
                       __fmaf_rn(t, b.w - a.w, a.w));
}

template <typename T>
__global__ void rescale_kernel(const T* __restrict__ src, int w, int h, T* __restrict__ dst, int W, int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    // texel coordinate of the destination pixel centre: u = (x + 0.5) / W * w - 0.5
    const float u = __fmul_rn(__fdiv_rn(x + 0.5f, (float)W), (float)w) - 0.5f;
    const float v = __fmul_rn(__fdiv_rn(y + 0.5f, (float)H), (float)h) - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float au = u - fu, av = v - fv;
    const int x0 = min(max((int)fu, 0), w - 1), x1 = min(max((int)fu + 1, 0), w - 1);
    const int y0 = min(max((int)fv, 0), h - 1), y1 = min(max((int)fv + 1, 0), h - 1);
    const float4 top = lerp4(load_px(src, y0 * w + x0), load_px(src, y0 * w + x1), au);
    const float4 bot = lerp4(load_px(src, y1 * w + x0), load_px(src, y1 * w + x1), au);
    store_px(dst, (size_t)y * W + x, lerp4(top, bot, av));
}

}  // namespace

extern "C" vrc_status vrc_image_rescale(vrc_context* ctx, const void* d_src, int w, int h, void* d_dst, int W, int H,
                                        int format) {
    if (!ctx) return VRC_ERR_INVALID_ARG;
    if (!d_src || !d_dst || w < 1 || h < 1 || W < 1 || H < 1 || H > 65535 ||
        (format != VRC_OUT_RGBA8 && format != VRC_OUT_RGBA32F)) {
        ctx->last_error = "vrc_image_rescale: null image, bad size or format (RGBA8 or RGBA32F)";
        return VRC_ERR_INVALID_ARG;
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) {
        dim3 grid((W + 127) / 128, H);
        if (format == VRC_OUT_RGBA8)
            rescale_kernel<<<grid, 128, 0, ctx->stream>>>(static_cast<const uchar4*>(d_src), w, h,
                                                          static_cast<uchar4*>(d_dst), W, H);
        else
            rescale_kernel<<<grid, 128, 0, ctx->stream>>>(static_cast<const float4*>(d_src), w, h,
                                                          static_cast<float4*>(d_dst), W, H);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        ctx->last_error = std::string("vrc_image_rescale: ") + cudaGetErrorString(e);
        return VRC_ERR_CUDA;
    }
    return VRC_OK;
}
