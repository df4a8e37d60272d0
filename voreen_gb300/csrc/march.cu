// Frame-level launch dispatch of the ray march (one translation unit per
// compositing family: march_dvr.cu, march_mip_iso.cu, march_mop_mida.cu,
// march_first_hit.cu), the analytic entry/exit kernel and the batched
// persistent render.
#include "march_core.cuh"

namespace vrc {
namespace {

__global__ void entry_exit_kernel(MarchParams P, float4* entry, float4* exitp) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
    if (px >= P.W) return;
    float4 e, l;
    analytic_entry_exit(P, px, py, e, l);
    entry[(size_t)py * P.W + px] = e;
    exitp[(size_t)py * P.W + px] = l;
}

}  // namespace

cudaError_t launch_march(const MarchParams& p, int dtype, int compositing, int shading, int num_sms,
                         cudaStream_t s) {
    switch (compositing) {
        case VRC_MIP:
        case VRC_ISO: return launch_march_mip_iso(p, dtype, compositing, shading, num_sms, s);
        case VRC_MOP:
        case VRC_MIDA: return launch_march_mop_mida(p, dtype, compositing, shading, num_sms, s);
        case VRC_FHP:
        case VRC_FHN: return launch_march_first_hit(p, dtype, compositing, num_sms, s);
        default: return launch_march_dvr(p, dtype, shading, num_sms, s);
    }
}

cudaError_t launch_entry_exit(const MarchParams& p, float4* entry, float4* exitp, cudaStream_t s) {
    dim3 grid((p.W + 127) / 128, p.H);
    entry_exit_kernel<<<grid, 128, 0, s>>>(p, entry, exitp);
    return cudaGetLastError();
}

}  // namespace vrc

// ---- batched persistent render ------------------------------------------
// Many requests (uneven volumes, dtypes, image sizes) in one persistent
// launch: warps claim ray tiles from a global counter over the concatenated
// tile lists (requests ordered longest first), copy the request's parameters
// into shared memory when they move to another request, and march with the
// request's dtype. Per-request completion times are stamped with the global
// timer (state layout: [0] tile counter, [1] start ns, [2] samples,
// [3 + r] request r's last tile completion ns).
namespace vrc {
namespace {

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void batch_begin_kernel(unsigned long long* state, int nreq) {
    for (int i = threadIdx.x; i < 3 + nreq; i += blockDim.x) state[i] = 0ull;
    __syncthreads();
    if (threadIdx.x == 0) state[1] = global_ns();
}

template <int COMP, int SHADE>
__global__ void __launch_bounds__(256, VRC_MARCH_MIN_BLOCKS)
    march_batch_kernel(const BatchReq* __restrict__ reqs, int nreq, const unsigned* __restrict__ tile_prefix,
                       unsigned total_tiles, unsigned long long* state) {
    __shared__ MarchParams s_par[8];
    __shared__ int s_dtype[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    MarchParams& P = s_par[wib];
    int cur = -1;
    Counters cnt;
    for (;;) {
        unsigned tile = 0;
        if (lane == 0) tile = atomicAdd(reinterpret_cast<unsigned*>(state), 1u);
        tile = __shfl_sync(FULL, tile, 0);
        if (tile >= total_tiles) break;
        int lo = 0, hi = nreq;  // largest r with tile_prefix[r] <= tile
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (tile_prefix[mid] <= tile) lo = mid;
            else hi = mid;
        }
        const int r = lo;
        if (r != cur) {
            __syncwarp();
            const int* src = reinterpret_cast<const int*>(&reqs[r].P);
            int* dst = reinterpret_cast<int*>(&P);
            for (int i = lane; i < (int)(sizeof(MarchParams) / sizeof(int)); i += 32) dst[i] = src[i];
            if (lane == 0) s_dtype[wib] = reqs[r].dtype;
            __syncwarp();
            cur = r;
        }
        const unsigned lt = tile - tile_prefix[r];
        const int tx = (int)(lt % (unsigned)P.tiles_x), ty = (int)(lt / (unsigned)P.tiles_x);
        const int tw = 1 << P.tile_wshift;
        const int px = P.rx0 + tx * tw + (lane & (tw - 1));
        const int py = P.ry0 + ty * (32 >> P.tile_wshift) + (lane >> P.tile_wshift);
        if (px < P.rx1 && py < P.ry1) {
            float4 f, l;
            analytic_entry_exit(P, px, py, f, l);
            const bool bg = f.x == 0.f && f.y == 0.f && f.z == 0.f && f.w == 0.f && l.x == 0.f && l.y == 0.f &&
                            l.z == 0.f && l.w == 0.f;
            float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
            float2 ax = make_float2(1.f, 0.f);
            if (!bg) {
                const int dt = s_dtype[wib];
                if (dt == VRC_U8)
                    res = march_ray<VRC_U8, COMP, SHADE, VRC_EE_ANALYTIC>(P, P.tf_rgba8, P.tf_alpha, f, l, px, py, cnt, ax);
                else if (dt == VRC_U16)
                    res = march_ray<VRC_U16, COMP, SHADE, VRC_EE_ANALYTIC>(P, P.tf_rgba8, P.tf_alpha, f, l, px, py, cnt, ax);
                else res = march_ray<VRC_F32, COMP, SHADE, VRC_EE_ANALYTIC>(P, P.tf_rgba8, P.tf_alpha, f, l, px, py, cnt, ax);
            }
            write_out(P, (size_t)py * P.W + px, res);
            if (P.aux) P.aux[(size_t)py * P.W + px] = ax;
        }
        __syncwarp();
        if (lane == 0) {
            __threadfence();
            atomicMax(state + 3 + r, global_ns());
        }
    }
    unsigned long long a = cnt.samples;
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(FULL, a, o);
    if (lane == 0) atomicAdd(state + 2, a);
}

template <int COMP, int SHADE>
cudaError_t launch_batch_t(const BatchReq* reqs, int nreq, const unsigned* prefix, unsigned total,
                           unsigned long long* state, int num_sms, cudaStream_t s) {
    auto k = march_batch_kernel<COMP, SHADE>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    long long grid = (long long)num_sms * per_sm;
    const long long need = ((long long)total + 7) / 8;
    if (grid > need) grid = need < 1 ? 1 : need;
    k<<<(unsigned)grid, 256, 0, s>>>(reqs, nreq, prefix, total, state);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_batch_begin(unsigned long long* state, int nreq, cudaStream_t s) {
    batch_begin_kernel<<<1, 256, 0, s>>>(state, nreq);
    return cudaGetLastError();
}

cudaError_t launch_march_batch(const BatchReq* reqs, int nreq, const unsigned* prefix, unsigned total,
                               unsigned long long* state, int compositing, int shading, int num_sms,
                               cudaStream_t s) {
    const bool ph = shading == VRC_SHADE_PHONG;
    switch (compositing) {
        case VRC_MIP:
            return ph ? launch_batch_t<VRC_MIP, VRC_SHADE_PHONG>(reqs, nreq, prefix, total, state, num_sms, s)
                      : launch_batch_t<VRC_MIP, VRC_SHADE_NONE>(reqs, nreq, prefix, total, state, num_sms, s);
        case VRC_ISO:
            return ph ? launch_batch_t<VRC_ISO, VRC_SHADE_PHONG>(reqs, nreq, prefix, total, state, num_sms, s)
                      : launch_batch_t<VRC_ISO, VRC_SHADE_NONE>(reqs, nreq, prefix, total, state, num_sms, s);
        default:
            return ph ? launch_batch_t<VRC_DVR, VRC_SHADE_PHONG>(reqs, nreq, prefix, total, state, num_sms, s)
                      : launch_batch_t<VRC_DVR, VRC_SHADE_NONE>(reqs, nreq, prefix, total, state, num_sms, s);
    }
}

}  // namespace vrc
