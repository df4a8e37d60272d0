// Segmented ray march for the learned upsampler's input (vrc_render_aux_segments).
//
// Not the reference's loop: an approximation whose frames are judged by PSNR
// against the plain render. At half resolution and half rate the plain march
// is bound by the serial sample chain of the longest rays (a 64x64 window at
// the centre of the CT-like frame costs as much as half the frame), so here
// each ray is cut into G segments of whole sample steps, G adjacent lanes
// march one segment each with march_ray (a segment is a shorter ray from the
// segment's first sample point), and the segments are composited front to
// back: colour += (1 - alpha) * segment colour, alpha likewise, with the
// early termination rule (alpha >= threshold -> 1) applied after every
// segment. Differences from the exact march: the segments' sample points are
// re-started from their first point (the step grid shifts by rounding), each
// segment terminates early on its own alpha, and a segment's first sample has
// no predecessor for the clip-border gradient rule.
#include "march_core.cuh"

namespace vrc {
namespace {

template <int DT, int SHADE, int G>
__global__ void __launch_bounds__(256, VRC_MARCH_MIN_BLOCKS) march_segments_kernel(MarchParams P) {
    extern __shared__ float4 s_raw[];
    float* s_alpha = reinterpret_cast<float*>(s_raw);
    uchar4* s_tf = reinterpret_cast<uchar4*>(s_alpha + 256);
    for (int i = threadIdx.x; i < P.tf_width; i += blockDim.x) s_tf[i] = P.tf_rgba8[i];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_alpha[i] = P.tf_alpha[i];
    __syncthreads();
    constexpr int RW = 32 / G;  // rays per warp: a row of RW pixels
    const int lane = threadIdx.x & 31, g = lane % G, ray = lane / G, base = lane - g;
    const int tiles_x = (P.rx1 - P.rx0 + RW - 1) / RW, tiles_y = P.ry1 - P.ry0;
    const int ntiles = tiles_x * tiles_y;
    Counters cnt;
    for (;;) {
        int tile = 0;
        if (lane == 0) tile = (int)atomicAdd(P.tile_counter, 1u);
        tile = __shfl_sync(FULL, tile, 0);
        if (tile >= ntiles) break;
        const int px = P.rx0 + (tile % tiles_x) * RW + ray, py = P.ry0 + tile / tiles_x;
        const bool inside = px < P.rx1;
        float4 f = make_float4(0.f, 0.f, 0.f, 0.f), l = f;
        bool hit = false;
        if (inside) hit = analytic_entry_exit(P, px, py, f, l);
        // this lane's segment: samples [k0, k1) of the ray's n samples
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 ax = make_float2(1.f, 0.f);
        float t0 = 0.f, seg_len = 0.f, tend = 0.f;
        if (hit) {
            const float dx = l.x - f.x, dy = l.y - f.y, dz = l.z - f.z;
            tend = sqrtf(dx * dx + dy * dy + dz * dz);
            const int n = (int)floorf(tend / P.step) + 1;
            const int k0 = (n * g) / G, k1 = (n * (g + 1)) / G;
            if (k1 > k0 && tend > 0.f) {
                const float inv = 1.f / tend;
                t0 = (float)k0 * P.step;
                const float t1 = g == G - 1 ? tend : ((float)k1 - 0.5f) * P.step;
                seg_len = t1 - t0;
                const float4 fs = make_float4(f.x + t0 * dx * inv, f.y + t0 * dy * inv, f.z + t0 * dz * inv, 1.f);
                const float4 ls = make_float4(f.x + t1 * dx * inv, f.y + t1 * dy * inv, f.z + t1 * dz * inv, 1.f);
                r = march_ray<DT, VRC_DVR, SHADE, VRC_EE_ANALYTIC>(P, s_tf, s_alpha, fs, ls, px, py, cnt, ax);
            }
        }
        // front-to-back over the G segments, in every lane of the group
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 aux = make_float2(1.f, 0.f);
        bool done = false;
#pragma unroll
        for (int k = 0; k < G; ++k) {
            const float sr = __shfl_sync(FULL, r.x, base + k), sg = __shfl_sync(FULL, r.y, base + k);
            const float sb = __shfl_sync(FULL, r.z, base + k), sa = __shfl_sync(FULL, r.w, base + k);
            const float hx = __shfl_sync(FULL, ax.x, base + k), hg = __shfl_sync(FULL, ax.y, base + k);
            const float st0 = __shfl_sync(FULL, t0, base + k), slen = __shfl_sync(FULL, seg_len, base + k);
            if (done) continue;
            if (aux.x >= 1.f && hx < 1.f && tend > 0.f) aux = make_float2((st0 + hx * slen) / tend, hg);
            const float w = 1.f - acc.w;
            acc.x += w * sr;
            acc.y += w * sg;
            acc.z += w * sb;
            acc.w += w * sa;
            if (acc.w >= P.ert) {
                acc.w = 1.f;
                done = true;
            }
        }
        if (inside && g == 0) {
            const size_t pix = (size_t)py * P.W + px;
            write_out(P, pix, acc);
            if (P.aux) P.aux[pix] = aux;
        }
    }
    if (P.counters) {
        unsigned long long a = cnt.samples, b = cnt.fetched, c = cnt.shaded, d = cnt.runs;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(FULL, a, o);
            b += __shfl_xor_sync(FULL, b, o);
            c += __shfl_xor_sync(FULL, c, o);
            d += __shfl_xor_sync(FULL, d, o);
        }
        if (lane == 0) {
            atomicAdd(P.counters + 0, a);
            atomicAdd(P.counters + 1, b);
            atomicAdd(P.counters + 2, c);
            atomicAdd(P.counters + 3, d);
        }
    }
}

template <int DT, int SHADE>
cudaError_t launch_seg(const MarchParams& p, int num_sms, cudaStream_t s) {
    auto k = march_segments_kernel<DT, SHADE, 4>;
    const size_t smem = 256 * sizeof(float) + (size_t)p.tf_width * sizeof(uchar4);
    int per_sm = 0;
    cudaError_t e = resident_ctas(k, smem, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long tiles = (long long)((p.rx1 - p.rx0 + 7) / 8) * (p.ry1 - p.ry0);
    long long grid = (long long)num_sms * per_sm;
    const long long need = (tiles + 7) / 8;  // 8 warps per CTA
    if (grid > need) grid = need < 1 ? 1 : need;
    k<<<(unsigned)grid, 256, smem, s>>>(p);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_march_segments(const MarchParams& p, int dtype, int shading, int num_sms, cudaStream_t s) {
    const bool ph = shading == VRC_SHADE_PHONG;
    switch (dtype) {
        case VRC_U8: return ph ? launch_seg<VRC_U8, VRC_SHADE_PHONG>(p, num_sms, s) : launch_seg<VRC_U8, VRC_SHADE_NONE>(p, num_sms, s);
        case VRC_U16: return ph ? launch_seg<VRC_U16, VRC_SHADE_PHONG>(p, num_sms, s) : launch_seg<VRC_U16, VRC_SHADE_NONE>(p, num_sms, s);
        default: return ph ? launch_seg<VRC_F32, VRC_SHADE_PHONG>(p, num_sms, s) : launch_seg<VRC_F32, VRC_SHADE_NONE>(p, num_sms, s);
    }
}

}  // namespace vrc
