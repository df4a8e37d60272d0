// Host side of the C ABI (include/vrc.h): context, volume ingest, transfer
// function bake and tables, camera matrices, and the frame driver that
// replaces CPURaycaster::process (modules/base/processors/render/cpuraycaster.cpp:90-206).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "vrc_internal.h"

using vrc::BrickLayout;
using vrc::MarchParams;

namespace {

vrc_status fail(vrc_context* ctx, vrc_status s, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

vrc_status cuda_fail(vrc_context* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return fail(ctx, VRC_ERR_OUT_OF_MEMORY, m);
    return fail(ctx, VRC_ERR_CUDA, m);
}

#define VRC_CUDA(ctx, call)                                    \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

// Grow-only device scratch owned by the context.
cudaError_t ensure(void** p, size_t* cap, size_t need) {
    if (*cap >= need && *p) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, need);
    if (e == cudaSuccess) *cap = need;
    return e;
}

// ---- 4x4 row-major double matrices (tgt::Matrix4 semantics) ----
struct M4 {
    double m[16];
};
M4 mul(const M4& a, const M4& b) {
    M4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += a.m[4 * i + k] * b.m[4 * k + j];
            r.m[4 * i + j] = s;
        }
    return r;
}
bool invert(const M4& in, M4& out) {
    double a[4][8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 8; ++j) a[i][j] = j < 4 ? in.m[4 * i + j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (std::fabs(a[piv][c]) < 1e-300) return false;
        if (piv != c)
            for (int j = 0; j < 8; ++j) std::swap(a[c][j], a[piv][j]);
        const double d = a[c][c];
        for (int j = 0; j < 8; ++j) a[c][j] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double f = a[r][c];
                for (int j = 0; j < 8; ++j) a[r][j] -= f * a[c][j];
            }
    }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) out.m[4 * i + j] = a[i][j + 4];
    return true;
}

void norm3(double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l > 0) {
        v[0] /= l;
        v[1] /= l;
        v[2] /= l;
    }
}
void cross3(const double a[3], const double b[3], double r[3]) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

// Matrix4::createLookAt (ext/tgt/matrix.h:1196-1209)
M4 look_at(const float e[3], const float f[3], const float u[3]) {
    double look[3] = {double(f[0]) - e[0], double(f[1]) - e[1], double(f[2]) - e[2]};
    norm3(look);
    double up[3] = {u[0], u[1], u[2]};
    norm3(up);
    double strafe[3];
    cross3(look, up, strafe);
    norm3(strafe);
    double up2[3];
    cross3(strafe, look, up2);
    M4 r{};
    for (int j = 0; j < 3; ++j) {
        r.m[j] = strafe[j];
        r.m[4 + j] = up2[j];
        r.m[8 + j] = -look[j];
    }
    r.m[15] = 1;
    M4 t{};
    for (int i = 0; i < 4; ++i) t.m[5 * i] = 1;
    t.m[3] = -e[0];
    t.m[7] = -e[1];
    t.m[11] = -e[2];
    return mul(r, t);
}

// Matrix4::createPerspective (ext/tgt/matrix.h:1229-1247) as used by
// Camera::getProjectionMatrix for PERSPECTIVE (ext/tgt/camera.cpp:196-205).
M4 perspective(const vrc_camera& c, double window_ratio) {
    double fovy = c.fovy_deg;
    if (fovy < 6.0) fovy = 6.0;
    if (fovy > 175.0) fovy = 175.0;
    const double ratio = c.frustum_ratio > 0 ? c.frustum_ratio : 1.0;
    const double deg = M_PI / 180.0;
    double fov = fovy * deg;
    if (window_ratio < 1.0) fov = std::atan(std::tan(fovy * deg / 2.0) / (window_ratio * ratio)) * 2.0;
    const double aspect = ratio * window_ratio;
    const double f = 1.0 / std::tan(fov / 2.0);
    const double n = c.near_dist, fa = c.far_dist;
    M4 r{};
    r.m[0] = f / aspect;
    r.m[5] = f;
    r.m[10] = (n + fa) / (n - fa);
    r.m[11] = (2.0 * fa * n) / (n - fa);
    r.m[14] = -1.0;
    return r;
}

// textureToWorld = physicalToWorld (identity) * voxelToPhysical * textureToVoxel
// (src/core/datastructures/volume/volumebase.cpp:194-229).
M4 texture_to_world(const vrc_volume_desc& d) {
    M4 r{};
    for (int i = 0; i < 3; ++i) {
        r.m[5 * i] = double(d.spacing[i]) * d.dims[i];
        r.m[4 * i + 3] = double(d.offset[i]) - 0.5 * d.spacing[i];
    }
    r.m[15] = 1;
    return r;
}

bool valid_desc(const vrc_volume_desc* d) {
    if (!d) return false;
    if (d->dtype < VRC_U8 || d->dtype > VRC_F32) return false;
    for (int i = 0; i < 3; ++i) {
        if (d->dims[i] < 1 || d->dims[i] > 65536) return false;
        if (!(d->spacing[i] > 0.f) || !std::isfinite(d->spacing[i])) return false;
    }
    return true;
}

int ilog2(int v) {
    int s = 0;
    while ((1 << s) < v) ++s;
    return s;
}

}  // namespace

extern "C" {

int vrc_abi_version(void) { return VRC_ABI_VERSION; }

const char* vrc_status_string(vrc_status s) {
    switch (s) {
        case VRC_OK: return "ok";
        case VRC_ERR_INVALID_ARG: return "invalid argument";
        case VRC_ERR_CUDA: return "CUDA error";
        case VRC_ERR_OUT_OF_MEMORY: return "out of memory";
        case VRC_ERR_UNSUPPORTED: return "unsupported";
        case VRC_ERR_TIMEOUT: return "timeout";
        case VRC_ERR_NOT_READY: return "not ready";
        case VRC_ERR_DEVICE: return "device error";
        case VRC_ERR_SCRATCH_LIMIT: return "request exceeds the fixed scratch of vrc_render_noalloc";
    }
    return "unknown status";
}

const char* vrc_last_error(const vrc_context* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

vrc_status vrc_context_create(int device, vrc_context** out) {
    if (!out) return VRC_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return VRC_ERR_CUDA;
    if (device < 0 || device >= n) return VRC_ERR_INVALID_ARG;
    vrc_context* c = new (std::nothrow) vrc_context();
    if (!c) return VRC_ERR_OUT_OF_MEMORY;
    c->device = device;
    if ((e = cudaSetDevice(device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) {
        delete c;
        return VRC_ERR_CUDA;
    }
    for (auto& ev : c->ev) {
        if (cudaEventCreate(&ev) != cudaSuccess) {
            vrc_context_destroy(c);
            return VRC_ERR_CUDA;
        }
    }
    if (cudaMalloc(&c->d_counters, 16 * sizeof(unsigned long long)) != cudaSuccess) {
        vrc_context_destroy(c);
        return VRC_ERR_OUT_OF_MEMORY;
    }
    *out = c;
    return VRC_OK;
}

vrc_status vrc_context_destroy(vrc_context* c) {
    if (!c) return VRC_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& ev : c->ev)
        if (ev) cudaEventDestroy(ev);
    cudaFree(c->d_ee);
    cudaFree(c->d_out);
    cudaFree(c->d_occ);
    cudaFree(c->d_occ_coarse);
    cudaFree(c->d_dist);
    cudaFree(c->d_dist_tmp);
    cudaFree(c->d_prefix);
    cudaFree(c->d_counters);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return VRC_OK;
}

vrc_status vrc_context_synchronize(vrc_context* c) {
    if (!c) return VRC_ERR_INVALID_ARG;
    VRC_CUDA(c, cudaStreamSynchronize(c->stream));
    return VRC_OK;
}

void* vrc_context_stream(vrc_context* c) { return c ? (void*)c->stream : nullptr; }

vrc_status vrc_volume_upload(vrc_context* ctx, const vrc_volume_desc* desc, const void* voxels, int on_device,
                             int brick_size, vrc_volume** out) {
    return vrc_volume_upload_placed(ctx, desc, voxels, on_device, brick_size, VRC_PLACE_DEVICE, out);
}

vrc_status vrc_volume_upload_placed(vrc_context* ctx, const vrc_volume_desc* desc, const void* voxels, int on_device,
                                    int brick_size, int placement, vrc_volume** out) {
    if (!ctx || !out || !voxels) return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_volume_upload: null argument");
    if (placement != VRC_PLACE_DEVICE && placement != VRC_PLACE_HOST)
        return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_volume_upload: unknown placement");
    *out = nullptr;
    if (!valid_desc(desc)) return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_volume_upload: invalid volume descriptor");
    if (brick_size == 0) brick_size = 32;
    if (brick_size != 8 && brick_size != 16 && brick_size != 32 && brick_size != 64)
        return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_volume_upload: brick_size must be 8, 16, 32 or 64");
    VRC_CUDA(ctx, cudaSetDevice(ctx->device));
    vrc_volume* v = new (std::nothrow) vrc_volume();
    if (!v) return fail(ctx, VRC_ERR_OUT_OF_MEMORY, "vrc_volume_upload: host allocation");
    v->ctx = ctx;
    v->desc = *desc;
    BrickLayout& L = v->L;
    for (int i = 0; i < 3; ++i) {
        L.dims[i] = desc->dims[i];
        L.nb[i] = (desc->dims[i] + brick_size - 1) / brick_size;
    }
    L.B = brick_size;
    L.shift = ilog2(brick_size);
    L.S = brick_size + vrc::APRON_LO + vrc::APRON_HI;
    L.brick_stride = (((long long)L.S * L.S * L.S) + 63) / 64 * 64;
    const int bpv = vrc::dtype_bytes(desc->dtype);
    const size_t nvox = (size_t)desc->dims[0] * desc->dims[1] * desc->dims[2];
    const size_t brick_bytes = (size_t)L.nbricks() * L.brick_stride * bpv;
    // the march indexes bricks and skip cells with 32-bit integers (2^31
    // bricks of 8^3 voxels are 1.1e12 voxels, more than any memory holds)
    if (L.nbricks() >= (1LL << 31)) {
        delete v;
        return fail(ctx, VRC_ERR_UNSUPPORTED, "vrc_volume_upload: more than 2^31 bricks");
    }
    void* staging = nullptr;
    const void* registered = nullptr;  // caller's host voxels registered for direct device reads
    cudaError_t e = cudaSuccess;
    auto cleanup = [&](vrc_status s, const std::string& m) {
        cudaStreamSynchronize(ctx->stream);
        if (staging) cudaFree(staging);
        if (registered) cudaHostUnregister(const_cast<void*>(registered));
        vrc_volume_destroy(v);
        return fail(ctx, s, m);
    };
    if (placement == VRC_PLACE_HOST) {
        // brick pool in pinned host memory, read by the kernels through its
        // mapped device address (NVLink-C2C on Grace hosts)
        if ((e = cudaHostAlloc(&v->h_bricks, brick_bytes, cudaHostAllocMapped)) != cudaSuccess ||
            (e = cudaHostGetDevicePointer(&v->d_bricks, v->h_bricks, 0)) != cudaSuccess)
            return cleanup(VRC_ERR_OUT_OF_MEMORY, "vrc_volume_upload: host brick pool allocation failed");
        v->host_bytes = brick_bytes;
    } else if ((e = cudaMalloc(&v->d_bricks, brick_bytes)) != cudaSuccess) {
        return cleanup(VRC_ERR_OUT_OF_MEMORY, "vrc_volume_upload: brick pool allocation failed");
    }
    if ((e = cudaMalloc((void**)&v->d_bmin, L.nbricks() * sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc((void**)&v->d_bmax, L.nbricks() * sizeof(float))) != cudaSuccess)
        return cleanup(VRC_ERR_OUT_OF_MEMORY, "vrc_volume_upload: min/max table allocation failed");
    v->bytes = (placement == VRC_PLACE_HOST ? 0 : brick_bytes) + 2 * L.nbricks() * sizeof(float);
    const void* lin = voxels;
    if (!on_device && placement == VRC_PLACE_HOST) {
        // no device copy of the linear volume either: the bricking kernels read
        // the caller's voxels through a mapped registration
        void* dp = nullptr;
        if ((e = cudaHostRegister(const_cast<void*>(voxels), nvox * bpv, cudaHostRegisterMapped)) != cudaSuccess)
            return cleanup(VRC_ERR_CUDA, std::string("vrc_volume_upload: host registration: ") + cudaGetErrorString(e));
        registered = voxels;
        if ((e = cudaHostGetDevicePointer(&dp, const_cast<void*>(voxels), 0)) != cudaSuccess)
            return cleanup(VRC_ERR_CUDA, std::string("vrc_volume_upload: mapped address: ") + cudaGetErrorString(e));
        lin = dp;
    } else if (!on_device) {
        if ((e = cudaMalloc(&staging, nvox * bpv)) != cudaSuccess)
            return cleanup(VRC_ERR_OUT_OF_MEMORY, "vrc_volume_upload: staging allocation failed");
        if ((e = cudaMemcpyAsync(staging, voxels, nvox * bpv, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
            return cleanup(VRC_ERR_CUDA, std::string("vrc_volume_upload: copy: ") + cudaGetErrorString(e));
        lin = staging;
    }
    if ((e = vrc::launch_brick_build(lin, desc->dtype, L, v->d_bricks, ctx->stream)) != cudaSuccess ||
        (e = vrc::launch_brick_minmax(v->d_bricks, desc->dtype, L, v->d_bmin, v->d_bmax, ctx->stream)) != cudaSuccess)
        return cleanup(VRC_ERR_CUDA, std::string("vrc_volume_upload: kernel: ") + cudaGetErrorString(e));
    // finer empty-space cells (2^3, 4^3, 8^3, 16^3) below the brick size;
    // 2^3 cells (8 bytes of tables per 8 voxels) only up to
    // 2^VRC_CELL2_LOG2_MAX of them
    for (int li = 0; li < 4; ++li) {
        const int C = 2 << li;
        if (C >= brick_size) continue;
        vrc_cell_level& lv = v->levels[li];
        lv.C = C;
        for (int i = 0; i < 3; ++i) lv.nc[i] = (desc->dims[i] + C - 1) / C;
        if (lv.count() >= (1LL << 32) || (C == 2 && lv.count() > (1LL << VRC_CELL2_LOG2_MAX))) {
            lv.C = 0;  // beyond the march's 32-bit cell index, or the 2^3 table budget
            continue;
        }
        if ((e = cudaMalloc((void**)&lv.d_min, lv.count() * sizeof(float))) != cudaSuccess ||
            (e = cudaMalloc((void**)&lv.d_max, lv.count() * sizeof(float))) != cudaSuccess)
            return cleanup(VRC_ERR_OUT_OF_MEMORY, "vrc_volume_upload: cell table allocation failed");
        v->bytes += 2 * lv.count() * sizeof(float);
        if ((e = vrc::launch_cell_minmax(lin, desc->dtype, desc->dims, C, lv.d_min, lv.d_max, ctx->stream)) != cudaSuccess)
            return cleanup(VRC_ERR_CUDA, std::string("vrc_volume_upload: cell kernel: ") + cudaGetErrorString(e));
    }
    std::vector<float> mn(L.nbricks()), mx(L.nbricks());
    if ((e = cudaMemcpyAsync(mn.data(), v->d_bmin, mn.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(mx.data(), v->d_bmax, mx.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
        return cleanup(VRC_ERR_CUDA, std::string("vrc_volume_upload: ") + cudaGetErrorString(e));
    if (staging) cudaFree(staging);
    staging = nullptr;
    if (registered) cudaHostUnregister(const_cast<void*>(registered));
    registered = nullptr;
    v->vmin = *std::min_element(mn.begin(), mn.end());
    v->vmax = *std::max_element(mx.begin(), mx.end());
    *out = v;
    return VRC_OK;
}

vrc_status vrc_volume_destroy(vrc_volume* v) {
    if (!v) return VRC_ERR_INVALID_ARG;
    if (v->ctx) cudaSetDevice(v->ctx->device);
    if (v->h_bricks)
        cudaFreeHost(v->h_bricks);
    else
        cudaFree(v->d_bricks);
    cudaFree(v->d_cache);
    cudaFree(v->d_slot);
    cudaFree(v->d_occ_brick);
    cudaFree(v->d_cache_ids);
    cudaFree(v->d_cache_dst);
    cudaFree(v->d_used);
    cudaFree(v->d_lod);
    cudaFree(v->d_bmin);
    cudaFree(v->d_bmax);
    for (auto& lv : v->levels) {
        cudaFree(lv.d_min);
        cudaFree(lv.d_max);
    }
    delete v;
    return VRC_OK;
}

vrc_status vrc_volume_minmax(vrc_volume* v, float* mn, float* mx) {
    if (!v || !mn || !mx) return VRC_ERR_INVALID_ARG;
    *mn = v->vmin;
    *mx = v->vmax;
    return VRC_OK;
}

vrc_status vrc_volume_brick_minmax(vrc_volume* v, int nb[3], float* out_min, float* out_max) {
    if (!v || !nb) return VRC_ERR_INVALID_ARG;
    for (int i = 0; i < 3; ++i) nb[i] = v->L.nb[i];
    if (!out_min && !out_max) return VRC_OK;
    vrc_context* ctx = v->ctx;
    VRC_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t n = v->L.nbricks() * sizeof(float);
    if (out_min) VRC_CUDA(ctx, cudaMemcpy(out_min, v->d_bmin, n, cudaMemcpyDeviceToHost));
    if (out_max) VRC_CUDA(ctx, cudaMemcpy(out_max, v->d_bmax, n, cudaMemcpyDeviceToHost));
    return VRC_OK;
}

size_t vrc_volume_device_bytes(const vrc_volume* v) { return v ? v->bytes : 0; }
size_t vrc_volume_host_bytes(const vrc_volume* v) { return v ? v->host_bytes : 0; }

vrc_status vrc_volume_set_cache_limit(vrc_volume* v, size_t bytes) {
    if (!v) return VRC_ERR_INVALID_ARG;
    v->cache_limit = bytes;
    const size_t brick_bytes = (size_t)v->L.brick_stride * vrc::dtype_bytes(v->desc.dtype);
    if (v->cache_slots > 0 && (size_t)v->cache_slots > bytes / brick_bytes) {
        // shrink: release the cache, the next render fills a smaller one
        if (v->ctx) cudaSetDevice(v->ctx->device);
        cudaFree(v->d_cache);
        cudaFree(v->d_cache_ids);
        cudaFree(v->d_cache_dst);
        v->d_cache = nullptr;
        v->d_cache_ids = v->d_cache_dst = nullptr;
        v->cache_slots = 0;
        v->h_slot_brick.clear();
        v->free_slots.clear();
        std::fill(v->h_slot.begin(), v->h_slot.end(), -1);
    }
    v->cache_valid = false;
    return VRC_OK;
}

vrc_status vrc_volume_set_cache_upload_budget(vrc_volume* v, size_t bytes_per_render) {
    if (!v) return VRC_ERR_INVALID_ARG;
    v->upload_budget = bytes_per_render;
    return VRC_OK;
}

vrc_status vrc_volume_cache_info(const vrc_volume* v, long long* cached, long long* reachable, long long* missed) {
    if (!v || !cached || !reachable || !missed) return VRC_ERR_INVALID_ARG;
    long long n = 0;
    for (long long b : v->h_slot_brick) n += b >= 0 ? 1 : 0;
    *cached = n;
    *reachable = v->cache_reachable;
    *missed = v->last_misses;
    if (v->used_pending && v->ctx) {
        // the last render's bits (refinement consumes them at the next render)
        const long long nb = v->L.nbricks();
        const size_t words = (size_t)vrc::occupancy_bytes(nb) / 4;
        std::vector<uint32_t> used(words);
        cudaError_t e = cudaSetDevice(v->ctx->device);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(used.data(), v->d_used, words * 4, cudaMemcpyDeviceToHost, v->ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(v->ctx->stream);
        if (e != cudaSuccess) return cuda_fail(v->ctx, e, "vrc_volume_cache_info");
        long long m = 0;
        for (size_t w = 0; w < words; ++w)
            for (uint32_t bits = used[w]; bits; bits &= bits - 1) {
                const long long b = (long long)w * 32 + __builtin_ctz(bits);
                if (b < nb && v->h_slot[b] < 0) ++m;
            }
        *missed = m;
    }
    return VRC_OK;
}

vrc_status vrc_volume_set_lod(vrc_volume* v, int level) {
    if (!v || !v->ctx) return VRC_ERR_INVALID_ARG;
    vrc_context* ctx = v->ctx;
    if (level < 0 || level > VRC_MAX_LOD_LEVEL)
        return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_volume_set_lod: level out of range");
    if (!v->h_bricks) return fail(ctx, VRC_ERR_UNSUPPORTED, "vrc_volume_set_lod: the volume's brick pool is in device memory");
    if (level > 0 && (!v->d_lod || v->lod_level != level)) {
        // level k: the 2x2x2 mean of level k - 1 (level 0 = the host pool),
        // each intermediate level freed once the next is built
        VRC_CUDA(ctx, cudaSetDevice(ctx->device));
        const int bpv = vrc::dtype_bytes(v->desc.dtype);
        if (v->d_lod) {
            v->bytes -= (size_t)v->lod_L.nbricks() * v->lod_L.brick_stride * bpv;
            cudaFree(v->d_lod);
            v->d_lod = nullptr;
            v->lod_level = 0;
        }
        const void* src = v->d_bricks;
        BrickLayout srcL = v->L;
        void* prev = nullptr;  // the device level being halved (never the pool)
        cudaError_t e = cudaSuccess;
        for (int k = 1; k <= level && e == cudaSuccess; ++k) {
            BrickLayout H = srcL;
            for (int i = 0; i < 3; ++i) {
                H.dims[i] = (srcL.dims[i] + 1) / 2;
                H.nb[i] = (H.dims[i] + H.B - 1) / H.B;
            }
            const size_t n1 = (size_t)H.dims[0] * H.dims[1] * H.dims[2];
            void* lin = nullptr;
            void* bricks = nullptr;
            e = cudaMalloc(&lin, n1 * bpv);
            if (e == cudaSuccess) e = cudaMalloc(&bricks, (size_t)H.nbricks() * H.brick_stride * bpv);
            if (e == cudaSuccess) e = vrc::launch_half_sample(src, v->desc.dtype, srcL, H.dims, lin, ctx->stream);
            if (e == cudaSuccess) e = vrc::launch_brick_build(lin, v->desc.dtype, H, bricks, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            cudaFree(lin);
            cudaFree(prev);
            prev = bricks;
            src = bricks;
            srcL = H;
        }
        if (e != cudaSuccess) {
            cudaFree(prev);
            return cuda_fail(ctx, e, "vrc_volume_set_lod");
        }
        v->d_lod = prev;
        v->lod_L = srcL;
        v->lod_level = level;
        v->bytes += (size_t)srcL.nbricks() * srcL.brick_stride * bpv;
    }
    v->lod_on = level > 0;
    return VRC_OK;
}

vrc_status vrc_tf_bake_keys(const vrc_tf_key* keys, int nkeys, int width, float gamma, float threshold_lo,
                            float threshold_hi, uint8_t* out) {
    if (!out || width < 2 || width > 65536 || nkeys < 0 || (nkeys > 0 && !keys)) return VRC_ERR_INVALID_ARG;
    for (int k = 1; k < nkeys; ++k)
        if (keys[k].intensity < keys[k - 1].intensity) return VRC_ERR_INVALID_ARG;
    // TransFunc1D::createTextureData (transfunc1d.cpp:85-116)
    const int front_end = (int)std::floor(threshold_lo * float(width) + 0.5f);
    const int back_start = (int)std::floor(threshold_hi * float(width) + 0.5f);
    for (int x = 0; x < width; ++x) {
        uint8_t* o = out + 4 * x;
        if (x < front_end || x > back_start || nkeys == 0) {
            std::memset(o, 0, 4);
            continue;
        }
        float value = float(x) / float(width - 1);
        if (gamma != 1.f) value = powf(value, gamma);
        // TransFunc1DKeys::getMappingForValueUByte (transfunc1dkeys.cpp:119-154)
        value = value < 0.f ? 0.f : (value > 1.f ? 1.f : value);
        int k = 0;
        while (k < nkeys && value > keys[k].intensity) ++k;
        if (k == 0) {
            std::memcpy(o, keys[0].color_l, 4);
        } else if (k == nkeys) {
            std::memcpy(o, keys[nkeys - 1].color_r, 4);
        } else {
            const vrc_tf_key& a = keys[k - 1];
            const vrc_tf_key& b = keys[k];
            const float fraction = (value - a.intensity) / (b.intensity - a.intensity);
            for (int ch = 0; ch < 4; ++ch) {
                const float diff = float(int(b.color_l[ch]) - int(a.color_r[ch]));
                const float prod = diff * fraction;  // separate statements: no fused multiply-add
                const float sum = float(a.color_r[ch]) + prod;
                o[ch] = static_cast<uint8_t>(sum);
            }
        }
    }
    return VRC_OK;
}

int vrc_tf_table_width(int dtype) {
    // bits per voxel, float treated as 16 bit, capped at 4096 entries
    int bits = dtype == VRC_U8 ? 8 : 16;
    int w = 1 << bits;
    return w > 4096 ? 4096 : w;
}

vrc_status vrc_tf_create(vrc_context* ctx, const uint8_t* rgba, int width, float lo, float hi, vrc_tf** out) {
    if (!ctx || !rgba || !out || width < 2 || width > 4096)
        return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_tf_create: width must be in [2, 4096]");
    if (!(lo <= hi) || !std::isfinite(lo) || !std::isfinite(hi))
        return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_tf_create: invalid domain");
    *out = nullptr;
    VRC_CUDA(ctx, cudaSetDevice(ctx->device));
    vrc_tf* t = new (std::nothrow) vrc_tf();
    if (!t) return fail(ctx, VRC_ERR_OUT_OF_MEMORY, "vrc_tf_create: host allocation");
    t->ctx = ctx;
    t->width = width;
    t->lo = lo;
    t->hi = hi;
    t->h_rgba = new (std::nothrow) uint8_t[4 * width];
    if (!t->h_rgba) {
        delete t;
        return fail(ctx, VRC_ERR_OUT_OF_MEMORY, "vrc_tf_create: host allocation");
    }
    std::memcpy(t->h_rgba, rgba, 4 * width);
    std::vector<int> prefix(width + 1, 0);
    for (int i = 0; i < width; ++i) prefix[i + 1] = prefix[i] + (rgba[4 * i + 3] > 0 ? 1 : 0);
    cudaError_t e = cudaMalloc(&t->d_prefix, (width + 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(t->d_prefix, prefix.data(), (width + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->d_rgba8, (size_t)width * 4);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_rgba8, rgba, (size_t)width * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        vrc_tf_destroy(t);
        return cuda_fail(ctx, e, "vrc_tf_create");
    }
    *out = t;
    return VRC_OK;
}

vrc_status vrc_tf_destroy(vrc_tf* t) {
    if (!t) return VRC_ERR_INVALID_ARG;
    if (t->ctx) cudaSetDevice(t->ctx->device);
    for (auto& kv : t->alpha_tables) cudaFree(kv.second);
    cudaFree(t->d_rgba8);
    cudaFree(t->d_prefix);
    delete[] t->h_rgba;
    delete t;
    return VRC_OK;
}

vrc_status vrc_camera_matrices(const vrc_camera* cam, const vrc_volume_desc* vol, int W, int H, double* view,
                               double* proj, double* inv_mvp) {
    if (!cam || W < 1 || H < 1) return VRC_ERR_INVALID_ARG;
    if (inv_mvp && !valid_desc(vol)) return VRC_ERR_INVALID_ARG;
    const M4 V = look_at(cam->position, cam->focus, cam->up);
    const M4 P = perspective(*cam, double(W) / double(H));
    if (view) std::memcpy(view, V.m, sizeof(V.m));
    if (proj) std::memcpy(proj, P.m, sizeof(P.m));
    if (inv_mvp) {
        const M4 mvp = mul(mul(P, V), texture_to_world(*vol));
        M4 inv;
        if (!invert(mvp, inv)) return VRC_ERR_INVALID_ARG;
        std::memcpy(inv_mvp, inv.m, sizeof(inv.m));
    }
    return VRC_OK;
}

void vrc_render_params_default(vrc_render_params* p, int W, int H) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->width = W;
    p->height = H;
    p->sampling_rate = 2.f;              // volumeraycaster.cpp:56
    p->compositing = VRC_DVR;
    p->shading = VRC_SHADE_NONE;
    p->iso_value = 0.5f;                 // volumeraycaster.cpp:57
    p->ert_threshold = 0.95f;            // mod_raysetup.frag:36
    const float lp[4] = {2.3f, 1.5f, 1.5f, 1.f};  // volumerenderer.cpp:43-53
    std::memcpy(p->light_position, lp, sizeof(lp));
    for (int i = 0; i < 3; ++i) {
        p->light_ambient[i] = 0.4f;
        p->light_diffuse[i] = 0.8f;
        p->light_specular[i] = 0.6f;
    }
    p->material_shininess = 60.f;
    p->apply_attenuation = 0;
    p->light_attenuation[0] = 1.f;
    p->camera.up[1] = 1.f;
    p->camera.position[2] = 3.f;
    p->camera.fovy_deg = 45.f;
    p->camera.near_dist = 0.1f;
    p->camera.far_dist = 50.f;
    p->camera.frustum_ratio = 1.f;
    p->entry_exit_mode = VRC_EE_BUFFERS;
    p->quantize_entry_exit = 0;
    p->empty_space_skipping = 1;
    p->classification = VRC_CLASSIFY_TF;
    p->mida_gamma = 0.f;                 // volumeraycaster.cpp:66 ("gammaValue")
}

float vrc_sampling_step(const vrc_volume* vol, float sampling_rate) {
    if (!vol || !(sampling_rate > 0.f)) return 0.f;
    const int* d = vol->desc.dims;
    const int maxdim = std::max(d[0], std::max(d[1], d[2]));
    return 1.f / (float(maxdim) * sampling_rate);
}

}  // extern "C"

namespace {

}  // namespace

namespace vrc {

// Alpha per alpha byte for a render: the opacity-corrected alpha
// 1 - (1 - a/255)^(step * 200) for DVR (cpuraycaster.cpp:291) and the plain
// a/255 for MIP / ISO -- the values CPURaycaster computes per sample, here
// once per byte with the same float arithmetic and powf.
void tf_alpha_values(bool corrected, float kcorr, float out[256]) {
    for (int a = 0; a < 256; ++a) {
        float x = float(a) / 255.f;
        if (corrected) x = 1.f - powf(1.f - x, kcorr);
        out[a] = x;
    }
}

vrc_status tf_alpha(vrc_context* ctx, vrc_tf* tf, bool corrected, float kcorr, float** out) {
    uint32_t bits = 0;
    std::memcpy(&bits, &kcorr, 4);
    const auto key = std::make_pair(corrected ? 1 : 0, corrected ? bits : 0u);
    auto it = tf->alpha_tables.find(key);
    if (it != tf->alpha_tables.end()) {
        *out = it->second;
        return VRC_OK;
    }
    float h[256];
    tf_alpha_values(corrected, kcorr, h);
    float* d = nullptr;
    cudaError_t e0 = cudaMalloc(&d, sizeof(h));
    if (e0 != cudaSuccess) return cuda_fail(ctx, e0, "tf alpha table allocation");
    cudaError_t e = cudaMemcpy(d, h, sizeof(h), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(ctx, e, "tf alpha table upload");
    }
    tf->alpha_tables[key] = d;
    *out = d;
    return VRC_OK;
}

vrc_status fill_params(vrc_context* ctx, const vrc_volume* vol, const vrc_render_params* p, MarchParams& P) {
    std::memset(&P, 0, sizeof(P));
    const vrc_volume_desc& d = vol->desc;
    P.bricks = vol->d_bricks;
    P.L = vol->L;
    const int maxdim = std::max(d.dims[0], std::max(d.dims[1], d.dims[2]));
    // samplingStepSize = 1 / (max(dim) * samplingRate) (cpuraycaster.cpp:104)
    P.step = 1.f / (float(maxdim) * p->sampling_rate);
    for (int i = 0; i < 3; ++i) {
        P.dimf[i] = float(d.dims[i]);
        P.dim_m1[i] = float(d.dims[i]) - 1.f;
        P.offs[i] = 1.f / float(d.dims[i]);
        P.spacing[i] = d.spacing[i];
        P.spacing_rcp_half[i] = (1.f / d.spacing[i]) * 0.5f;
        const float range = d.dtype == VRC_U8 ? 255.f : (d.dtype == VRC_U16 ? 65535.f : 1.f);
        P.gscale[i] = P.spacing_rcp_half[i] * d.rwm_scale / range;
        P.vol_offset[i] = d.offset[i];
        // physicalToWorld is the identity: physical == world
        P.light_phys[i] = p->light_position[i];
        P.cam_phys[i] = p->camera.position[i];
        P.amb[i] = p->light_ambient[i];
        P.dif[i] = p->light_diffuse[i];
        P.spec[i] = p->light_specular[i];
        P.att[i] = p->light_attenuation[i];
    }
    P.rwm_scale = d.rwm_scale;
    P.rwm_offset = d.rwm_offset;
    P.ert = p->ert_threshold;
    P.iso = p->iso_value;
    P.shininess = p->material_shininess;
    P.atten_on = p->apply_attenuation;
    P.mida_gamma = p->mida_gamma;
    P.W = p->width;
    P.H = p->height;
    P.ee_mode = p->entry_exit_mode;
    P.quantize = p->quantize_entry_exit;
    const int tw = p->tile_width == 0 ? 8 : p->tile_width;
    P.tile_wshift = ilog2(tw);
    if (p->region[2] > 0 && p->region[3] > 0) {
        P.rx0 = std::max(0, p->region[0]);
        P.ry0 = std::max(0, p->region[1]);
        P.rx1 = std::min(p->width, p->region[0] + p->region[2]);
        P.ry1 = std::min(p->height, p->region[1] + p->region[3]);
        if (P.rx1 <= P.rx0 || P.ry1 <= P.ry0) return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: empty region");
    } else {
        P.rx0 = P.ry0 = 0;
        P.rx1 = p->width;
        P.ry1 = p->height;
    }
    P.tiles_x = (P.rx1 - P.rx0 + tw - 1) / tw;
    P.tiles_y = (P.ry1 - P.ry0 + (32 / tw) - 1) / (32 / tw);
    for (int i = 0; i < 3; ++i) {
        P.box_lo[i] = 0.f;
        P.box_hi[i] = 1.f;
    }
    if (p->enable_clipping) {
        // OptimizedProxyGeometry::processCube: voxel box [llf - 0.5, urb + 0.5]
        // intersected with the volume, then voxelToTexture = (v + 0.5) / dim
        for (int i = 0; i < 3; ++i) {
            if (p->clip_llf[i] > p->clip_urb[i])
                return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: clip region with llf > urb");
            const double dim = double(d.dims[i]);
            P.box_lo[i] = float(std::max(0.0, double(p->clip_llf[i]) / dim));
            P.box_hi[i] = float(std::min(1.0, (double(p->clip_urb[i]) + 1.0) / dim));
        }
    }
    if (p->entry_exit_mode == VRC_EE_ANALYTIC) {
        double inv[16];
        if (vrc_camera_matrices(&p->camera, &d, p->width, p->height, nullptr, nullptr, inv) != VRC_OK)
            return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: camera matrix is singular");
        for (int i = 0; i < 16; ++i) P.inv_mvp[i] = float(inv[i]);
    }
    return VRC_OK;
}

vrc_status check_params(vrc_context* ctx, const vrc_render_params* p) {
    if (!p) return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: null params");
    if (p->width < 1 || p->height < 1 || (long long)p->width * p->height > (1LL << 28))
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: image size out of range");
    if (!(p->sampling_rate > 0.f) || !std::isfinite(p->sampling_rate))
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: sampling_rate must be > 0");
    if (p->compositing < VRC_DVR || p->compositing > VRC_FHN)
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: unknown compositing mode");
    if (p->classification != VRC_CLASSIFY_TF && p->classification != VRC_CLASSIFY_PREINTEGRATED)
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: unknown classification mode");
    if (p->classification == VRC_CLASSIFY_PREINTEGRATED && p->compositing != VRC_DVR)
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: pre-integrated classification needs DVR compositing");
    if (!std::isfinite(p->mida_gamma))
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: mida_gamma must be finite");
    if (p->shading < VRC_SHADE_NONE || p->shading > VRC_SHADE_PHONG)
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: unknown shading mode");
    if (p->entry_exit_mode != VRC_EE_BUFFERS && p->entry_exit_mode != VRC_EE_ANALYTIC)
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: unknown entry/exit mode");
    if (p->tile_width != 0 && p->tile_width != 1 && p->tile_width != 2 && p->tile_width != 4 && p->tile_width != 8 &&
        p->tile_width != 16 && p->tile_width != 32)
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: tile_width must be 0, 1, 2, 4, 8, 16 or 32");
    if (p->skip_cell_size != 0 && p->skip_cell_size != 2 && p->skip_cell_size != 4 && p->skip_cell_size != 8 &&
        p->skip_cell_size != 16 && p->skip_cell_size != 32 && p->skip_cell_size != 64)
        return ::fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: skip_cell_size must be 0, 2, 4, 8, 16, 32 or 64");
    return VRC_OK;
}

}  // namespace vrc

using vrc::check_params;
using vrc::fill_params;
using vrc::tf_alpha;


extern "C" {

}  // extern "C"

namespace {

// Copies bricks ids[i] of the host pool to cache slots dst[i] and uploads
// the slot table; waits for both, since they read the host vectors.
vrc_status commit_slots(vrc_context* ctx, vrc_volume* vol, const std::vector<long long>& ids,
                        const std::vector<long long>& dst, size_t brick_bytes, cudaStream_t s, int* launches) {
    if (!ids.empty()) {
        ++*launches;
        VRC_CUDA(ctx, cudaMemcpyAsync(vol->d_cache_ids, ids.data(), ids.size() * sizeof(long long),
                                      cudaMemcpyHostToDevice, s));
        VRC_CUDA(ctx, cudaMemcpyAsync(vol->d_cache_dst, dst.data(), dst.size() * sizeof(long long),
                                      cudaMemcpyHostToDevice, s));
        VRC_CUDA(ctx, vrc::launch_brick_gather(vol->d_bricks, vol->d_cache_ids, vol->d_cache_dst, (long long)ids.size(),
                                               brick_bytes, vol->d_cache, s));
    }
    VRC_CUDA(ctx, cudaMemcpyAsync(vol->d_slot, vol->h_slot.data(), vol->h_slot.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, s));
    VRC_CUDA(ctx, cudaStreamSynchronize(s));
    return VRC_OK;
}

// Device cache of a host-resident brick pool, refreshed before each march.
//
// Prefetch by TF: when the TF (its per-brick occupancy) changes, the cache
// is filled with the bricks the TF can reach -- bricks whose value range
// meets a visible TF entry first, then their 26 neighbours (a sample near a
// face, a gradient tap or the previous sample of a pre-integrated segment
// reads there) -- as many as the cache limit holds. Bricks already cached
// keep their slot; only new ones are gathered over the host link.
//
// Refinement by view: while the cache holds fewer bricks than the TF
// reaches (or a level of detail is attached), the march records every brick
// it reads. Before the next frame, bricks it read without a slot displace
// cached bricks it did not read, least recently read first -- the
// used/missing brick flags and LRU brick pool of Voreen's octree raycaster
// (singleoctreeraycaster.cl, octreebrickpoolmanager.h:99-165).
//
// A brick without a slot is read from the host pool (exact) or, with a level
// of detail attached, from the device-resident half-resolution level.
vrc_status prepare_brick_cache(vrc_context* ctx, vrc_volume* vol, const int* occ_prefix, int occ_width,
                               uint64_t occ_source, const vrc_tf* tf, MarchParams& P, cudaStream_t s,
                               int* launches) {
    const vrc::BrickLayout& L = vol->L;
    const long long nb = L.nbricks();
    const size_t words = (size_t)vrc::occupancy_bytes(nb) / 4;
    // The plan depends on the TF (or pre-integration table) only through the
    // per-brick occupancy. With the same source, nothing queued and no read
    // bits to fold in, it cannot have changed: no occupancy launch, no copy
    // back, no host synchronisation (frames stay asynchronous).
    uint32_t lo_bits, hi_bits;
    std::memcpy(&lo_bits, &tf->lo, 4);
    std::memcpy(&hi_bits, &tf->hi, 4);
    const uint64_t src_key[4] = {occ_source, (uint64_t)occ_width, lo_bits, hi_bits};
    const bool same_plan = vol->cache_valid && !vol->used_pending && vol->pending_pos >= vol->pending.size() &&
                           std::memcmp(src_key, vol->cache_src_key, sizeof(src_key)) == 0;
    if (!same_plan) {
        if (!vol->d_occ_brick) VRC_CUDA(ctx, cudaMalloc((void**)&vol->d_occ_brick, words * 4));
        VRC_CUDA(ctx, vrc::launch_occupancy(vol->d_bmin, vol->d_bmax, nb, occ_prefix, occ_width, vol->desc.rwm_scale,
                                            vol->desc.rwm_offset, tf->lo, tf->hi, vol->d_occ_brick, s));
        ++*launches;
        std::vector<uint32_t> occ(words), used;
        VRC_CUDA(ctx, cudaMemcpyAsync(occ.data(), vol->d_occ_brick, words * 4, cudaMemcpyDeviceToHost, s));
        if (vol->used_pending) {
            used.resize(words);
            VRC_CUDA(ctx, cudaMemcpyAsync(used.data(), vol->d_used, words * 4, cudaMemcpyDeviceToHost, s));
            vol->used_pending = false;
        }
        VRC_CUDA(ctx, cudaStreamSynchronize(s));
        const size_t brick_bytes = (size_t)L.brick_stride * vrc::dtype_bytes(vol->desc.dtype);
        if (vol->h_slot.size() != (size_t)nb) vol->h_slot.assign((size_t)nb, -1);
        if (vol->h_last_used.size() != (size_t)nb) vol->h_last_used.assign((size_t)nb, 0);
        if (!vol->d_slot) VRC_CUDA(ctx, cudaMalloc((void**)&vol->d_slot, (size_t)nb * sizeof(int)));
        bool table_changed = false;
        if (!(vol->cache_valid && occ == vol->h_occ)) {
            // the slot table is uploaded whenever the cache is (re)planned: a new
            // table, a reallocation or evictions all change it
            table_changed = true;
            // wanted bricks in priority order: occupied, then the dilation ring
            std::vector<uint8_t> mark(nb, 0);
            std::vector<long long> want;
            for (long long b = 0; b < nb; ++b)
                if ((occ[b >> 5] >> (b & 31)) & 1u) {
                    mark[b] = 2;
                    want.push_back(b);
                }
            const size_t n_occ = want.size();
            for (size_t k = 0; k < n_occ; ++k) {
                const long long b = want[k];
                const int bx = int(b % L.nb[0]), by = int((b / L.nb[0]) % L.nb[1]), bz = int(b / ((long long)L.nb[0] * L.nb[1]));
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const int x = bx + dx, y = by + dy, z = bz + dz;
                            if (x < 0 || y < 0 || z < 0 || x >= L.nb[0] || y >= L.nb[1] || z >= L.nb[2]) continue;
                            const long long n = ((long long)z * L.nb[1] + y) * L.nb[0] + x;
                            if (!mark[n]) {
                                mark[n] = 1;
                                want.push_back(n);
                            }
                        }
            }
            vol->cache_reachable = (long long)want.size();
            long long slots = std::min<long long>((long long)want.size(), (long long)(vol->cache_limit / brick_bytes));
            if (slots > vol->cache_slots) {
                // grow: fresh allocation, every wanted brick gathered again
                size_t free_b = 0, total_b = 0;
                VRC_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
                const size_t reserve = (size_t)1 << 30;  // left for the frame buffers and other work
                const long long fit = free_b > reserve ? (long long)((free_b - reserve) / brick_bytes) : 0;
                slots = std::min(slots, fit + vol->cache_slots);
            }
            if (slots > vol->cache_slots) {
                cudaFree(vol->d_cache);
                cudaFree(vol->d_cache_ids);
                cudaFree(vol->d_cache_dst);
                vol->d_cache = nullptr;
                vol->d_cache_ids = vol->d_cache_dst = nullptr;
                vol->cache_slots = 0;
                vol->h_slot_brick.clear();
                vol->free_slots.clear();
                std::fill(vol->h_slot.begin(), vol->h_slot.end(), -1);
                cudaError_t e = cudaMalloc(&vol->d_cache, (size_t)slots * brick_bytes);
                if (e == cudaSuccess) e = cudaMalloc((void**)&vol->d_cache_ids, (size_t)slots * sizeof(long long));
                if (e == cudaSuccess) e = cudaMalloc((void**)&vol->d_cache_dst, (size_t)slots * sizeof(long long));
                if (e != cudaSuccess) {
                    cudaGetLastError();
                    cudaFree(vol->d_cache);
                    cudaFree(vol->d_cache_ids);
                    vol->d_cache = nullptr;
                    vol->d_cache_ids = nullptr;
                    vol->d_cache_dst = nullptr;
                    slots = 0;  // no cache: every brick is read from the host pool (or the level of detail)
                } else {
                    vol->cache_slots = slots;
                    vol->h_slot_brick.assign((size_t)slots, -1);
                    for (long long sl = slots - 1; sl >= 0; --sl) vol->free_slots.push_back(sl);
                }
            }
            // keep cached bricks that are still wanted within the slot budget;
            // the wanted ones not cached yet queue for gathering
            std::vector<uint8_t> keep(nb, 0);
            for (long long k = 0; k < slots; ++k) keep[want[k]] = 1;
            for (long long sl = 0; sl < vol->cache_slots; ++sl) {
                const long long b = vol->h_slot_brick[sl];
                if (b < 0 || keep[b]) continue;
                vol->h_slot[b] = -1;
                vol->h_slot_brick[sl] = -1;
                vol->free_slots.push_back(sl);
            }
            vol->pending.clear();
            vol->pending_pos = 0;
            for (long long k = 0; k < slots; ++k)
                if (vol->h_slot[want[k]] < 0) vol->pending.push_back(want[k]);
            vol->h_occ = occ;
            vol->cache_valid = true;
        }
        // this render's gathers: bricks the last frame read without a slot first
        // (into free slots, else slots of bricks it did not read, oldest first),
        // then queued TF-wanted bricks into free slots, up to the upload budget
        const size_t budget = vol->upload_budget ? std::max<size_t>(1, vol->upload_budget / brick_bytes) : SIZE_MAX;
        std::vector<long long> ids, dst;
        auto place = [&](long long b, long long sl) {
            const long long old = vol->h_slot_brick[sl];
            if (old >= 0) vol->h_slot[old] = -1;
            vol->h_slot[b] = (int)sl;
            vol->h_slot_brick[sl] = b;
            ids.push_back(b);
            dst.push_back(sl);
        };
        if (!used.empty()) {
            const uint32_t stamp = ++vol->frame;
            std::vector<long long> missed;
            for (size_t w = 0; w < words; ++w)
                for (uint32_t bits = used[w]; bits; bits &= bits - 1) {
                    const long long b = (long long)w * 32 + __builtin_ctz(bits);
                    if (b >= nb) break;
                    vol->h_last_used[b] = stamp;
                    if (vol->h_slot[b] < 0) missed.push_back(b);
                }
            vol->last_misses = (long long)missed.size();
            if (!missed.empty() && vol->cache_slots > 0) {
                std::vector<std::pair<uint32_t, long long>> stale;
                for (long long sl = 0; sl < vol->cache_slots; ++sl) {
                    const long long b = vol->h_slot_brick[sl];
                    if (b >= 0 && vol->h_last_used[b] != stamp) stale.emplace_back(vol->h_last_used[b], sl);
                }
                std::stable_sort(stale.begin(), stale.end(),
                                 [](const std::pair<uint32_t, long long>& x, const std::pair<uint32_t, long long>& y) {
                                     return x.first < y.first;
                                 });
                size_t next_stale = 0;
                for (long long b : missed) {
                    if (ids.size() >= budget) break;
                    if (!vol->free_slots.empty()) {
                        place(b, vol->free_slots.back());
                        vol->free_slots.pop_back();
                    } else if (next_stale < stale.size()) {
                        place(b, stale[next_stale++].second);
                    } else {
                        break;
                    }
                }
            }
        }
        while (vol->pending_pos < vol->pending.size() && ids.size() < budget && !vol->free_slots.empty()) {
            const long long b = vol->pending[vol->pending_pos++];
            if (vol->h_slot[b] >= 0) continue;
            place(b, vol->free_slots.back());
            vol->free_slots.pop_back();
        }
        if (!ids.empty() || table_changed) {
            vrc_status st = commit_slots(ctx, vol, ids, dst, brick_bytes, s, launches);
            if (st != VRC_OK) return st;
        }
        std::memcpy(vol->cache_src_key, src_key, sizeof(src_key));
    }
    const long long resident = vol->cache_slots - (long long)vol->free_slots.size();
    const bool lod = vol->lod_on && vol->d_lod;
    if (vol->cache_slots > 0 || lod) {
        P.bricks = vol->d_cache ? vol->d_cache : vol->d_bricks;
        P.brick_slot = vol->d_slot;
        P.host_pool = vol->d_bricks;
    }
    if (lod) {
        P.lod_bricks = vol->d_lod;
        for (int i = 0; i < 3; ++i) {
            P.lod_nb[i] = vol->lod_L.nb[i];
            P.lod_dimf[i] = float(vol->lod_L.dims[i]);
            P.lod_dim_m1[i] = float(vol->lod_L.dims[i] - 1);
        }
    }
    if (vol->cache_slots > 0 && (lod || resident < vol->cache_reachable)) {
        if (!vol->d_used) VRC_CUDA(ctx, cudaMalloc((void**)&vol->d_used, words * 4));
        VRC_CUDA(ctx, cudaMemsetAsync(vol->d_used, 0, words * 4, s));
        P.brick_used = vol->d_used;
        vol->used_pending = true;
    } else {
        vol->last_misses = 0;
    }
    return VRC_OK;
}

vrc_status render_impl(vrc_context* ctx, const vrc_volume* vol, const vrc_tf* tf_c, const vrc_render_params* p,
                       const float* entry, const float* exitp, int ee_on_device, void* out, int out_format,
                       int out_on_device, float* aux, vrc_render_stats* stats) {
    if (!ctx) return VRC_ERR_INVALID_ARG;
    if (!vol || !tf_c) return fail(ctx, VRC_ERR_NOT_READY, "vrc_render: volume and transfer function are required");
    if (vol->ctx != ctx || tf_c->ctx != ctx) return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: handle from another context");
    vrc_status st = check_params(ctx, p);
    if (st != VRC_OK) return st;
    if (!out) return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: null output");
    if (out_format < VRC_OUT_RGBA8 || out_format > VRC_OUT_RGBA16)
        return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: unknown output format");
    if (p->entry_exit_mode == VRC_EE_BUFFERS && (!entry || !exitp))
        return fail(ctx, VRC_ERR_NOT_READY, "vrc_render: entry/exit points are required in buffer mode");
    vrc_tf* tf = const_cast<vrc_tf*>(tf_c);
    VRC_CUDA(ctx, cudaSetDevice(ctx->device));
    MarchParams P;
    if ((st = fill_params(ctx, vol, p, P)) != VRC_OK) return st;
    const float kcorr = P.step * 200.f;  // SAMPLING_BASE_INTERVAL_RCP
    const int* occ_prefix = tf->d_prefix;
    int occ_width = tf->width;
    uint64_t occ_source = tf->uid;
    if (p->classification == VRC_CLASSIFY_PREINTEGRATED) {
        const vrc_preint* pi = tf->preint;
        if (!pi) return fail(ctx, VRC_ERR_NOT_READY, "vrc_render: no pre-integration table attached to the TF");
        if (pi->step != P.step)
            return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render: the pre-integration table was built for another step size");
        P.pi_table = pi->d_table;
        P.pi_res = pi->res;
        {
            const int* d = vol->desc.dims;
            P.pi_chain = P.step * float(std::max(d[0], std::max(d[1], d[2]))) <= 0.99f ? 1 : 0;
        }
        P.tf_rgba8 = nullptr;
        P.tf_alpha = nullptr;
        P.tf_width = 0;  // the TF table is not read
        occ_prefix = pi->d_prefix;
        occ_width = pi->res;
        occ_source = pi->uid;
    } else {
        float* alpha = nullptr;
        if ((st = tf_alpha(ctx, tf, vrc::alpha_corrected(p->compositing, p->classification), kcorr, &alpha)) !=
            VRC_OK)
            return st;
        P.tf_rgba8 = tf->d_rgba8;
        P.tf_alpha = alpha;
        P.tf_width = tf->width;
    }
    P.tf_lo = tf->lo;
    P.tf_hi = tf->hi;
    const size_t npix = (size_t)p->width * p->height;
    cudaStream_t s = ctx->stream;
    VRC_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
    // Pinned host buffers (cudaHostAlloc / cudaHostRegister) are read and
    // written by the kernel in place through their mapped addresses (over
    // NVLink-C2C on Grace hosts): each pixel's entry/exit points are read once
    // and its colour written once, so staging them through device memory
    // would only add a copy before and after the march. Pageable buffers are
    // staged.
    auto mapped = [](const void* h) -> void* {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
    };
    if (p->entry_exit_mode == VRC_EE_BUFFERS) {
        void* me = ee_on_device ? nullptr : mapped(entry);
        void* mx = ee_on_device || !me ? nullptr : mapped(exitp);
        if (ee_on_device) {
            P.entry = reinterpret_cast<const float4*>(entry);
            P.exitp = reinterpret_cast<const float4*>(exitp);
        } else if (me && mx) {
            P.entry = reinterpret_cast<const float4*>(me);
            P.exitp = reinterpret_cast<const float4*>(mx);
        } else {
            VRC_CUDA(ctx, ensure(&ctx->d_ee, &ctx->ee_bytes, 2 * npix * sizeof(float4)));
            float4* d = reinterpret_cast<float4*>(ctx->d_ee);
            VRC_CUDA(ctx, cudaMemcpyAsync(d, entry, npix * sizeof(float4), cudaMemcpyHostToDevice, s));
            VRC_CUDA(ctx, cudaMemcpyAsync(d + npix, exitp, npix * sizeof(float4), cudaMemcpyHostToDevice, s));
            P.entry = d;
            P.exitp = d + npix;
        }
    }
    const size_t px_bytes = out_format == VRC_OUT_RGBA32F ? 16 : (out_format == VRC_OUT_RGBA16 ? 8 : 4);
    void* mout = out_on_device ? nullptr : mapped(out);
    if (out_on_device) {
        P.out = out;
    } else if (mout) {
        P.out = mout;
    } else {
        VRC_CUDA(ctx, ensure(&ctx->d_out, &ctx->out_bytes, npix * px_bytes));
        P.out = ctx->d_out;
    }
    P.out_format = out_format;
    if (aux) {
        P.aux = reinterpret_cast<float2*>(aux);
        const float dom = std::max(tf->hi - tf->lo, 1e-12f);
        const float msp = std::min(vol->desc.spacing[0], std::min(vol->desc.spacing[1], vol->desc.spacing[2]));
        P.aux_gscale = msp / dom;
    }
    int occ_launches = 0;
    if (p->empty_space_skipping) {
        // skip cells: the requested edge if the volume holds that level, else
        // the brick; by default the finest level held of 2^3 and 4^3, whose
        // runs the distance field keeps long
        const int want = p->skip_cell_size == 0 ? vrc::default_skip_cell(vol) : p->skip_cell_size;
        const float* cmin = vol->d_bmin;
        const float* cmax = vol->d_bmax;
        int C = vol->L.B;
        int nc[3] = {vol->L.nb[0], vol->L.nb[1], vol->L.nb[2]};
        for (const auto& lv : vol->levels)
            if (lv.C == want && lv.d_min) {
                cmin = lv.d_min;
                cmax = lv.d_max;
                C = lv.C;
                for (int i = 0; i < 3; ++i) nc[i] = lv.nc[i];
            }
        const long long n = (long long)nc[0] * nc[1] * nc[2];
        // the occupancy bits are a function of the volume's min/max tables,
        // the TF (or table) and the cell edge: reuse them while those stay
        uint32_t lo_bits, hi_bits;
        std::memcpy(&lo_bits, &tf->lo, 4);
        std::memcpy(&hi_bits, &tf->hi, 4);
        // The distance field serves TF-empty cells, and replaces the coarse
        // (brick) level unless MIP's max-based skipping needs the bricks' max.
        // Pre-integration takes it only when a step moves less than a voxel
        // per axis: consecutive samples in an all-empty box then lie in the
        // same or adjacent empty cells, whose value ranges overlap, so every
        // table entry between them has alpha 0 (with longer steps two empty
        // cells apart can hold values between them that an entry reaches).
        const bool mip_skip = p->compositing == VRC_MIP && vol->desc.rwm_scale >= 0.f;
        const bool use_dist = p->classification == VRC_CLASSIFY_TF || P.pi_chain;
        const bool use_coarse = C < vol->L.B && (!use_dist || mip_skip);
        const uint64_t key[6] = {vol->uid, occ_source, (uint64_t)occ_width, lo_bits, hi_bits,
                                 (uint64_t)C | (use_dist ? 1ull << 32 : 0ull) | (use_coarse ? 1ull << 33 : 0ull)};
        const uint32_t* occ_before = ctx->d_occ;
        const uint32_t* coarse_before = ctx->d_occ_coarse;
        const uint8_t* dist_before = ctx->d_dist;
        VRC_CUDA(ctx, ensure((void**)&ctx->d_occ, &ctx->occ_bytes, vrc::occupancy_bytes(n)));
        if (use_dist) {
            VRC_CUDA(ctx, ensure((void**)&ctx->d_dist, &ctx->dist_bytes, (size_t)n));
            VRC_CUDA(ctx, ensure((void**)&ctx->d_dist_tmp, &ctx->dist_tmp_bytes, (size_t)n));
        }
        if (use_coarse)
            VRC_CUDA(ctx, ensure((void**)&ctx->d_occ_coarse, &ctx->occ_coarse_bytes,
                                 vrc::occupancy_bytes(vol->L.nbricks())));
        const bool cached = std::memcmp(key, ctx->occ_key, sizeof(key)) == 0 && ctx->d_occ == occ_before &&
                            (!use_coarse || ctx->d_occ_coarse == coarse_before) &&
                            (!use_dist || ctx->d_dist == dist_before);
        if (!cached) {
            std::memset(ctx->occ_key, 0, sizeof(ctx->occ_key));
            VRC_CUDA(ctx, vrc::launch_occupancy(cmin, cmax, n, occ_prefix, occ_width, vol->desc.rwm_scale,
                                                vol->desc.rwm_offset, tf->lo, tf->hi, ctx->d_occ, s));
            ++occ_launches;
        }
        P.occupancy = ctx->d_occ;
        // MIP: cells that cannot raise a ray's maximum are skipped too; that
        // needs a monotone real-world mapping
        if (mip_skip) {
            P.mip_skip = 1;
            P.cell_max = cmax;
            P.brick_max = vol->d_bmax;
        }
        P.cshift = ilog2(C);
        for (int i = 0; i < 3; ++i) P.nc[i] = nc[i];
        const int maxdim = std::max(vol->desc.dims[0], std::max(vol->desc.dims[1], vol->desc.dims[2]));
        P.skip_margin = 0.01f + 2e-5f * float(maxdim);
        if (use_dist) {
            if (!cached) {
                VRC_CUDA(ctx, vrc::launch_occ_distance(ctx->d_occ, nc, ctx->d_dist, ctx->d_dist_tmp, s));
                occ_launches += 3;
            }
            P.occ_dist = ctx->d_dist;
        }
        if (use_coarse) {
            // coarse level: whole bricks, tested where the fine cell is empty
            const long long nb = vol->L.nbricks();
            if (!cached) {
                VRC_CUDA(ctx, vrc::launch_occupancy(vol->d_bmin, vol->d_bmax, nb, occ_prefix, occ_width,
                                                    vol->desc.rwm_scale, vol->desc.rwm_offset, tf->lo, tf->hi,
                                                    ctx->d_occ_coarse, s));
                ++occ_launches;
            }
            P.occ_coarse = ctx->d_occ_coarse;
            P.cshift_coarse = vol->L.shift;
            for (int i = 0; i < 3; ++i) P.ncc[i] = vol->L.nb[i];
        }
        std::memcpy(ctx->occ_key, key, sizeof(key));
    }
    if (vol->h_bricks && (vol->cache_limit > 0 || vol->lod_on)) {
        if ((st = prepare_brick_cache(ctx, const_cast<vrc_volume*>(vol), occ_prefix, occ_width, occ_source, tf, P,
                                      s, &occ_launches)) != VRC_OK)
            return st;
    }
    VRC_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 16 * sizeof(unsigned long long), s));
    P.counters = ctx->d_counters;
    P.status = reinterpret_cast<int*>(ctx->d_counters + 4);
    P.tile_counter = reinterpret_cast<unsigned int*>(ctx->d_counters + 5);
    VRC_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
    VRC_CUDA(ctx, vrc::launch_march(P, vol->desc.dtype, p->compositing, p->shading, ctx->num_sms, s));
    VRC_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
    if (!out_on_device && !mout) VRC_CUDA(ctx, cudaMemcpyAsync(out, P.out, npix * px_bytes, cudaMemcpyDeviceToHost, s));
    VRC_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
    if (stats || !out_on_device) VRC_CUDA(ctx, cudaStreamSynchronize(s));
    if (stats) {
        unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
        VRC_CUDA(ctx, cudaMemcpy(h, ctx->d_counters, sizeof(h), cudaMemcpyDeviceToHost));
        stats->samples = double(h[0]);
        stats->samples_fetched = double(h[1]);
        stats->samples_shaded = double(h[2]);
        stats->skip_runs = double(h[3]);
        stats->device_status = int(h[4] & 0xffffffffu);
        stats->kernel_launches = 1 + occ_launches;
        VRC_CUDA(ctx, cudaEventElapsedTime(&stats->kernel_ms, ctx->ev[1], ctx->ev[2]));
        VRC_CUDA(ctx, cudaEventElapsedTime(&stats->total_ms, ctx->ev[0], ctx->ev[3]));
        if (stats->device_status != 0) return fail(ctx, VRC_ERR_DEVICE, "vrc_render: kernel reported an error status");
    }
    return VRC_OK;
}

}  // namespace

extern "C" {

vrc_status vrc_render(vrc_context* ctx, const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p,
                      const float* entry, const float* exitp, int ee_on_device, void* out, int out_format,
                      int out_on_device, vrc_render_stats* stats) {
    return render_impl(ctx, vol, tf, p, entry, exitp, ee_on_device, out, out_format, out_on_device, nullptr, stats);
}

vrc_status vrc_render_aux(vrc_context* ctx, const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p,
                          const float* d_entry, const float* d_exit, void* d_out, int out_format, float* d_aux,
                          vrc_render_stats* stats) {
    if (!d_aux) return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_render_aux: null aux image");
    return render_impl(ctx, vol, tf, p, d_entry, d_exit, 1, d_out, out_format, 1, d_aux, stats);
}

vrc_status vrc_entry_exit(vrc_context* ctx, const vrc_volume* vol, const vrc_render_params* p, float* entry,
                          float* exitp, int out_on_device) {
    if (!ctx) return VRC_ERR_INVALID_ARG;
    if (!vol || !entry || !exitp) return fail(ctx, VRC_ERR_INVALID_ARG, "vrc_entry_exit: null argument");
    vrc_status st = check_params(ctx, p);
    if (st != VRC_OK) return st;
    VRC_CUDA(ctx, cudaSetDevice(ctx->device));
    vrc_render_params q = *p;
    q.entry_exit_mode = VRC_EE_ANALYTIC;
    MarchParams P;
    if ((st = fill_params(ctx, vol, &q, P)) != VRC_OK) return st;
    const size_t npix = (size_t)p->width * p->height;
    float4 *de = reinterpret_cast<float4*>(entry), *dx = reinterpret_cast<float4*>(exitp);
    if (!out_on_device) {
        VRC_CUDA(ctx, ensure(&ctx->d_ee, &ctx->ee_bytes, 2 * npix * sizeof(float4)));
        de = reinterpret_cast<float4*>(ctx->d_ee);
        dx = de + npix;
    }
    VRC_CUDA(ctx, vrc::launch_entry_exit(P, de, dx, ctx->stream));
    if (!out_on_device) {
        VRC_CUDA(ctx, cudaMemcpyAsync(entry, de, npix * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
        VRC_CUDA(ctx, cudaMemcpyAsync(exitp, dx, npix * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
        VRC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return VRC_OK;
}

}  // extern "C"
