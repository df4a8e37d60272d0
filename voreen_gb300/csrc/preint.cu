// Pre-integrated classification tables (PreIntegrationTable,
// src/core/datastructures/transfunc/1d/preintegrationtable.cpp:67-204).
//
// Entry [back * res + front] holds the colour of a ray segment whose
// previous sample has TF coordinate front and whose current sample has
// coordinate back. The exact table composites the TF entries between the two
// one by one with a per-entry opacity correction for the segment length
// (O(res^3) work): one CUDA thread per entry, the corrections
// 1 - (1 - a)^(step * 200 / (k + 1)) precomputed on the host with the same
// powf the CPU build calls (there are only res x 256 distinct ones), every
// other operation explicitly rounded in the reference's order, so the table
// equals the CPU build bit for bit. The integral-function approximation is
// O(res^2) with one expf per entry and is built on the host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "vrc_internal.h"

namespace vrc {
namespace {

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.f), 1.f); }

__global__ void preint_exact_kernel(const float4* __restrict__ tb, const uint8_t* __restrict__ a8,
                                    const float* __restrict__ corr, int res, float4* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)res * res) return;
    const int sb = (int)(idx / res), sf = (int)(idx % res);
    float4 r;
    if (sb == sf) {
        const float4 c = tb[sf];
        r = make_float4(clamp01(c.x), clamp01(c.y), clamp01(c.z), corr[a8[sf]]);
    } else {
        const int k = sb > sf ? sb - sf : sf - sb;
        const int incr = sb < sf ? -1 : 1;
        const float* ck = corr + (size_t)k * 256;
        r = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int s = sf; (incr == 1 ? s <= sb : s >= sb) && r.w < 0.95f; s += incr) {
            const float4 c = tb[s];
            if (c.w > 0.f) {
                const float a = __ldg(ck + a8[s]);
                const float w = __fmul_rn(__fsub_rn(1.f, r.w), a);
                r.x = __fadd_rn(r.x, __fmul_rn(w, c.x));
                r.y = __fadd_rn(r.y, __fmul_rn(w, c.y));
                r.z = __fadd_rn(r.z, __fmul_rn(w, c.z));
                r.w = __fadd_rn(r.w, __fmul_rn(__fsub_rn(1.f, r.w), a));
            }
        }
        const float m = fmaxf(r.w, 0.001f);
        r = make_float4(clamp01(__fdiv_rn(r.x, m)), clamp01(__fdiv_rn(r.y, m)), clamp01(__fdiv_rn(r.z, m)),
                        clamp01(r.w));
    }
    out[idx] = r;
}

}  // namespace

cudaError_t launch_preint_exact(const float4* tb, const uint8_t* a8, const float* corr, int res, float4* out,
                                cudaStream_t s) {
    const long long n = (long long)res * res;
    preint_exact_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(tb, a8, corr, res, out);
    return cudaGetLastError();
}

}  // namespace vrc

namespace {

vrc_status pfail(vrc_context* ctx, vrc_status st, const char* msg) {
    if (ctx) ctx->last_error = msg;
    return st;
}

vrc_status pcuda(vrc_context* ctx, cudaError_t e, const char* what) {
    if (ctx) ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? VRC_ERR_OUT_OF_MEMORY : VRC_ERR_CUDA;
}

struct HostF4 {
    float r, g, b, a;
};

}  // namespace

extern "C" {

int vrc_preint_resolution(int tf_width, int requested) {
    if (requested > 0) return requested;
    return std::min(tf_width, 1024);
}

vrc_status vrc_preint_bake_source(const vrc_tf_key* keys, int nkeys, int res, float gamma, float threshold_lo,
                                  float threshold_hi, uint8_t* out) {
    if (!out || res < 2 || res > 4096 || nkeys < 0 || (nkeys > 0 && !keys)) return VRC_ERR_INVALID_ARG;
    // the texture's key mapping at res entries (no thresholds there), then the
    // table build's own threshold rule: zero below front_end and from back_start on
    vrc_status st = vrc_tf_bake_keys(keys, nkeys, res, gamma, 0.f, 1.f, out);
    if (st != VRC_OK) return st;
    const int front_end = (int)std::floor(threshold_lo * float(res) + 0.5f);
    const int back_start = (int)std::floor(threshold_hi * float(res) + 0.5f);
    for (int i = 0; i < res; ++i)
        if (i < front_end || i >= back_start) std::memset(out + 4 * i, 0, 4);
    return VRC_OK;
}

vrc_status vrc_preint_create(vrc_context* ctx, const uint8_t* src, int res, float step, int use_integral,
                             vrc_preint** out) {
    if (!ctx) return VRC_ERR_INVALID_ARG;
    if (!src || !out || res < 2 || res > 4096 || !(step > 0.f) || !std::isfinite(step))
        return pfail(ctx, VRC_ERR_INVALID_ARG, "vrc_preint_create: need a source table, 2 <= res <= 4096 and step > 0");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return pcuda(ctx, e, "cudaSetDevice");
    const float k200 = step * 200.0f;
    std::vector<HostF4> tb(res);
    std::vector<int> prefix(res + 1, 0);
    for (int i = 0; i < res; ++i) {
        const uint8_t* c = src + 4 * i;
        tb[i] = HostF4{float(c[0]) / 255.f, float(c[1]) / 255.f, float(c[2]) / 255.f, float(c[3]) / 255.f};
        prefix[i + 1] = prefix[i] + (c[3] > 0 ? 1 : 0);
    }
    const size_t n = (size_t)res * res;
    vrc_preint* t = new vrc_preint();
    t->ctx = ctx;
    t->res = res;
    t->step = step;
    t->use_integral = use_integral ? 1 : 0;
    cudaStream_t s = ctx->stream;
    float4* d_tb = nullptr;
    uint8_t* d_a8 = nullptr;
    float* d_corr = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_tb);
        cudaFree(d_a8);
        cudaFree(d_corr);
    };
    auto bail = [&](cudaError_t err, const char* what) {
        vrc_status st = pcuda(ctx, err, what);
        cudaStreamSynchronize(s);
        cleanup();
        cudaFree(t->d_table);
        cudaFree(t->d_prefix);
        delete t;
        return st;
    };
    if ((e = cudaMalloc(&t->d_table, n * sizeof(float4))) != cudaSuccess) return bail(e, "pre-integration table");
    if ((e = cudaMalloc(&t->d_prefix, (res + 1) * sizeof(int))) != cudaSuccess) return bail(e, "pre-integration prefix");
    if ((e = cudaMemcpyAsync(t->d_prefix, prefix.data(), (res + 1) * sizeof(int), cudaMemcpyHostToDevice, s)) !=
        cudaSuccess)
        return bail(e, "pre-integration prefix upload");
    if (!use_integral) {
        // corr[k][a] = 1 - (1 - a/255)^((step * 200) * (1 / (k + 1))), the
        // per-entry correction of a segment spanning k + 1 entries
        std::vector<float> corr((size_t)res * 256);
        for (int k = 0; k < res; ++k) {
            const float scale = 1.0f / (std::fabs(static_cast<float>(k)) + 1);
            const float ex = k200 * scale;
            corr[(size_t)k * 256] = 0.f;
            for (int a = 1; a < 256; ++a) corr[(size_t)k * 256 + a] = 1.f - powf(1.f - float(a) / 255.f, ex);
        }
        std::vector<uint8_t> a8(res);
        std::vector<float4> tb4(res);
        for (int i = 0; i < res; ++i) {
            a8[i] = src[4 * i + 3];
            tb4[i] = make_float4(tb[i].r, tb[i].g, tb[i].b, tb[i].a);
        }
        if ((e = cudaMalloc(&d_tb, res * sizeof(float4))) != cudaSuccess ||
            (e = cudaMalloc(&d_a8, res)) != cudaSuccess ||
            (e = cudaMalloc(&d_corr, corr.size() * sizeof(float))) != cudaSuccess)
            return bail(e, "pre-integration scratch");
        if ((e = cudaMemcpyAsync(d_tb, tb4.data(), res * sizeof(float4), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_a8, a8.data(), res, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_corr, corr.data(), corr.size() * sizeof(float), cudaMemcpyHostToDevice, s)) !=
                cudaSuccess)
            return bail(e, "pre-integration scratch upload");
        if ((e = vrc::launch_preint_exact(d_tb, d_a8, d_corr, res, t->d_table, s)) != cudaSuccess)
            return bail(e, "pre-integration kernel");
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return bail(e, "pre-integration kernel");
        cleanup();
    } else {
        // integral functions (Real-Time Volume Graphics p. 96)
        std::vector<HostF4> I(res);
        HostF4 acc{0.f, 0.f, 0.f, 0.f};
        for (int i = 0; i < res; ++i) {
            const HostF4 c = tb[i];
            if (c.a > 0.0f) {
                acc.r += c.r * c.a;
                acc.g += c.g * c.a;
                acc.b += c.b * c.a;
                acc.a += c.a;
            }
            I[i] = acc;
        }
        auto c01 = [](float x) { return std::min(std::max(x, 0.f), 1.f); };
        std::vector<float4> h(n);
        for (int sb = 0; sb < res; ++sb) {
            for (int sf = 0; sf < res; ++sf) {
                const int smin = std::min(sb, sf), smax = std::max(sb, sf);
                HostF4 col;
                if (smax != smin) {
                    const float factor = k200 / static_cast<float>(smax - smin);
                    col.r = (I[smax].r - I[smin].r) * factor;
                    col.g = (I[smax].g - I[smin].g) * factor;
                    col.b = (I[smax].b - I[smin].b) * factor;
                    col.a = 1.f - expf(-(I[smax].a - I[smin].a) * factor);
                    const float m = std::max(col.a, 0.001f);
                    col.r /= m;
                    col.g /= m;
                    col.b /= m;
                } else {
                    col = tb[smin];
                    col.a = 1.f - powf(1.f - col.a, k200);
                }
                h[(size_t)sb * res + sf] = make_float4(c01(col.r), c01(col.g), c01(col.b), c01(col.a));
            }
        }
        if ((e = cudaMemcpy(t->d_table, h.data(), n * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(e, "pre-integration table upload");
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return bail(e, "pre-integration prefix upload");
    }
    *out = t;
    return VRC_OK;
}

vrc_status vrc_preint_download(const vrc_preint* t, float* out) {
    if (!t || !out) return VRC_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(t->ctx->device);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpy(out, t->d_table, (size_t)t->res * t->res * sizeof(float4), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? VRC_OK : pcuda(t->ctx, e, "vrc_preint_download");
}

vrc_status vrc_preint_destroy(vrc_preint* t) {
    if (!t) return VRC_OK;
    cudaSetDevice(t->ctx->device);
    cudaStreamSynchronize(t->ctx->stream);
    cudaFree(t->d_table);
    cudaFree(t->d_prefix);
    delete t;
    return VRC_OK;
}

vrc_status vrc_tf_set_preintegration(vrc_tf* tf, const vrc_preint* t) {
    if (!tf) return VRC_ERR_INVALID_ARG;
    if (t && t->ctx != tf->ctx) return pfail(tf->ctx, VRC_ERR_INVALID_ARG, "vrc_tf_set_preintegration: table from another context");
    tf->preint = t;
    return VRC_OK;
}

}  // extern "C"
