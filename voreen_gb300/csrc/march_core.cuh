// The ray-march kernel (shared by the march_*.cu translation units): a GB300 restatement of CPURaycaster::directRendering
// (modules/base/processors/render/cpuraycaster.cpp:210-326) with the GLSL-only
// compositing and shading rules of rc_singlevolume.frag:116-312.
//
// Design:
//  * persistent grid (a few CTAs per SM); each warp pulls 8x4 ray tiles from
//    a global counter, so a warp's 32 rays are adjacent on screen and walk
//    the same bricks;
//  * the transfer function sits in shared memory as its RGBA8 entries plus
//    a table of 256 alphas (one per alpha byte) that already carry the
//    opacity correction 1-(1-a)^(step*200), computed on the host with the
//    same powf the CPU path calls; r/255, g/255, b/255 are the exact 8-bit
//    normalisation. 17 KB per CTA at 4096 entries, so most of the SM's
//    unified L1 / shared array stays L1 for the voxel gathers;
//  * voxels come from the bricked layout (32^3 core + apron), so a stencil
//    never crosses a brick; empty bricks (per-brick min/max against the TF)
//    are skipped without reading voxels while t still advances sample by
//    sample, which keeps results identical to the unskipped march;
//  * every operation on the sample path is an explicitly rounded FP32
//    intrinsic in the reference's order (no FMA contraction), so positions,
//    trilinear values, TF indices, compositing and the t > tend stop match
//    the FP32 CPU path bit for bit. Voxel normalisation v/255 and v/65535 is
//    computed as q0 = v*r, q = fma(fma(-q0, d, v), r, q0), which equals the
//    correctly rounded quotient for every 8- and 16-bit value;
//  * gradients (central differences, mod_gradients.frag:202-214) are six
//    lookups at +-1/dim in texture space, clamped like the intensity sample
//    and read from the centre's brick apron (another brick only when rounding
//    puts a tap two voxels away); they interpolate raw voxel values with FMA
//    lerps. Phong (mod_shading.frag:134-151) runs in registers with fast
//    reciprocal square roots and __powf. Shading only colours samples whose
//    alpha is already decided, so it changes no discrete decision; its
//    colours differ from the CPU path by ~1e-6.
#pragma once
#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "vrc_internal.h"

namespace vrc {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int LOOP_CAP = 255 * 255;  // cpuraycaster.cpp:239

__device__ __forceinline__ float m_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float a_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float s_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float d_(float a, float b) { return __fdiv_rn(a, b); }

// Exact voxel normalisation v / 255 and v / 65535 (VolumeRAM's
// getVoxelNormalized: float division, correctly rounded), without a
// division or an integer-to-float conversion instruction.
// For D = 2^k - 1, 1/D = 2^-k (1 + 2^-k + 2^-2k + ...), so
//   v / D = v (2^-k + 2^-2k) + v (2^-3k [+ 2^-4k + 2^-5k for k = 8]) + tail,
// tail >= 0 and smaller than the spacing of the fused sum's grid (2^-48 for
// k = 16, 2^-40 for k = 8). The fused sum lies on that grid, as do all
// rounding midpoints of the result, and it is never a midpoint itself: for a
// result in [2^e, 2^(e+1)), v would need a factor 2^(e + 24) (k = 16) or
// 2^(e + 16) (k = 8), more than v < 2^(e + k + 1) holds. So the tail cannot
// change the rounding: fma(v, A, v * B) = RN(v / D) for every v in [0, D]. (Checked exhaustively by the test suite.) v as a float: the bits
// 0x4B000000 | v are the float 2^23 + v.
__device__ __forceinline__ float small_uint_to_float(unsigned v) {
    return __fsub_rn(__int_as_float(0x4B000000u | v), 8388608.f);
}
template <int DT> struct Vox;
template <> struct Vox<VRC_U8> {
    using T = uint8_t;
    static __device__ __forceinline__ float norm(T v) {
        const float x = small_uint_to_float(v);
        return __fmaf_rn(x, 0x1.01p-8f, __fmul_rn(x, 0x1.0101p-24f));
    }
};
template <> struct Vox<VRC_U16> {
    using T = uint16_t;
    static __device__ __forceinline__ float norm(T v) {
        const float x = small_uint_to_float(v);
        return __fmaf_rn(x, 0x1.0001p-16f, __fmul_rn(x, 0x1p-48f));
    }
};
template <> struct Vox<VRC_F32> {
    using T = float;
    static __device__ __forceinline__ float norm(T v) { return v; }
};

struct F3 {
    float x, y, z;
};

// VolumeRAM::getVoxelNormalizedLinear summation order (volumeram.cpp:89-96).
__device__ __forceinline__ float tri8(float v000, float v100, float v110, float v010, float v001, float v101,
                                      float v111, float v011, float fx, float fy, float fz) {
    const float ox = s_(1.f, fx), oy = s_(1.f, fy), oz = s_(1.f, fz);
    float s = m_(m_(m_(v000, ox), oy), oz);
    s = a_(s, m_(m_(m_(v100, fx), oy), oz));
    s = a_(s, m_(m_(m_(v110, fx), fy), oz));
    s = a_(s, m_(m_(m_(v010, ox), fy), oz));
    s = a_(s, m_(m_(m_(v001, ox), oy), fz));
    s = a_(s, m_(m_(m_(v101, fx), oy), fz));
    s = a_(s, m_(m_(m_(v111, fx), fy), fz));
    s = a_(s, m_(m_(m_(v011, ox), fy), fz));
    return s;
}

template <int DT>
__device__ __forceinline__ float tri_at(const typename Vox<DT>::T* __restrict__ b, int o, int S, int S2, float fx,
                                        float fy, float fz) {
    using V = Vox<DT>;
    return tri8(V::norm(__ldg(b + o)), V::norm(__ldg(b + o + 1)), V::norm(__ldg(b + o + S + 1)),
                V::norm(__ldg(b + o + S)), V::norm(__ldg(b + o + S2)), V::norm(__ldg(b + o + S2 + 1)),
                V::norm(__ldg(b + o + S2 + S + 1)), V::norm(__ldg(b + o + S2 + S)), fx, fy, fz);
}

__device__ __forceinline__ float clampf_(float x, float lo, float hi) {
    x = x > lo ? x : lo;
    return x < hi ? x : hi;
}

__device__ __forceinline__ float rw_to_tf(float rw, float lo, float hi) {
    if (rw < lo) return 0.f;
    if (rw > hi) return 1.f;
    if (lo == hi) return 0.f;
    return d_(s_(rw, lo), s_(hi, lo));
}

__device__ __forceinline__ int tf_index(float x, int w) {
    const float f = m_(x, (float)(w - 1));
    const int i = (int)floorf(a_(f, 0.5f));
    return i < 0 ? 0 : (i > w - 1 ? w - 1 : i);
}

__device__ __forceinline__ float len3(float x, float y, float z) {
    float s = m_(x, x);
    s = a_(s, m_(y, y));
    s = a_(s, m_(z, z));
    return __fsqrt_rn(s);
}

__device__ __forceinline__ F3 normalize3(F3 v) {
    const float l = len3(v.x, v.y, v.z);
    if (l == 0.f) return F3{0.f, 0.f, 0.f};
    const float r = d_(1.f, l);
    return F3{m_(v.x, r), m_(v.y, r), m_(v.z, r)};
}

__device__ __forceinline__ float dot3(F3 a, F3 b) {
    float s = m_(a.x, b.x);
    s = a_(s, m_(a.y, b.y));
    s = a_(s, m_(a.z, b.z));
    return s;
}

// ---- shading path ----------------------------------------------------
// Shading feeds only the colour of samples with alpha > 0; it has no
// discrete decision and its pow is not correctly rounded on any platform, so
// it uses fused multiply-adds, fast reciprocal square roots and __powf. The
// resulting colour differs from the CPU path by ~1e-6 relative.
__device__ __forceinline__ F3 fnormalize(F3 v) {
    const float l2 = __fmaf_rn(v.x, v.x, __fmaf_rn(v.y, v.y, __fmul_rn(v.z, v.z)));
    if (l2 == 0.f) return F3{0.f, 0.f, 0.f};
    const float r = rsqrtf(l2);
    return F3{v.x * r, v.y * r, v.z * r};
}
__device__ __forceinline__ float fdot(F3 a, F3 b) { return __fmaf_rn(a.x, b.x, __fmaf_rn(a.y, b.y, __fmul_rn(a.z, b.z))); }

// Trilinear interpolation of raw voxel values with FMA lerps (gradient taps).
template <int DT>
__device__ __forceinline__ float tri_raw(const typename Vox<DT>::T* __restrict__ b, int o, int S, int S2, float fx,
                                         float fy, float fz) {
    const float v000 = (float)__ldg(b + o), v100 = (float)__ldg(b + o + 1);
    const float v010 = (float)__ldg(b + o + S), v110 = (float)__ldg(b + o + S + 1);
    const float v001 = (float)__ldg(b + o + S2), v101 = (float)__ldg(b + o + S2 + 1);
    const float v011 = (float)__ldg(b + o + S2 + S), v111 = (float)__ldg(b + o + S2 + S + 1);
    const float x00 = __fmaf_rn(fx, v100 - v000, v000), x10 = __fmaf_rn(fx, v110 - v010, v010);
    const float x01 = __fmaf_rn(fx, v101 - v001, v001), x11 = __fmaf_rn(fx, v111 - v011, v011);
    const float y0 = __fmaf_rn(fy, x10 - x00, x00), y1 = __fmaf_rn(fy, x11 - x01, x01);
    return __fmaf_rn(fz, y1 - y0, y0);
}

// tri_raw on voxel values already in registers (v<x><y><z>), the same
// arithmetic in the same order.
__device__ __forceinline__ float tri_regs(float v000, float v100, float v010, float v110, float v001, float v101,
                                          float v011, float v111, float fx, float fy, float fz) {
    const float x00 = __fmaf_rn(fx, v100 - v000, v000), x10 = __fmaf_rn(fx, v110 - v010, v010);
    const float x01 = __fmaf_rn(fx, v101 - v001, v001), x11 = __fmaf_rn(fx, v111 - v011, v011);
    const float y0 = __fmaf_rn(fy, x10 - x00, x00), y1 = __fmaf_rn(fy, x11 - x01, x01);
    return __fmaf_rn(fz, y1 - y0, y0);
}

// Start of brick `brick`: in the pool directly, or, for a host-resident pool
// with a device cache (brick_slot != nullptr), in the cache slot the table
// names. A brick the cache does not hold (slot -1) is read in the mapped
// host pool, so every brick stays readable whatever the cache holds -- or,
// with a level of detail attached, not at all: nullptr, and the caller
// samples the half-resolution level instead.
template <bool POOL, typename T>
__device__ __forceinline__ const T* brick_base(const MarchParams& P, const T* __restrict__ bricks, long long brick) {
    if (!POOL) return bricks + brick * P.L.brick_stride;
    const int slot = __ldg(P.brick_slot + brick);
    if (slot >= 0) return bricks + (long long)slot * P.L.brick_stride;
    return P.lod_bricks ? nullptr : reinterpret_cast<const T*>(P.host_pool) + brick * P.L.brick_stride;
}

// Records that a brick was read this frame (cache refinement). Lanes of the
// warp reading the same brick share one atomic.
__device__ __forceinline__ void mark_used(const MarchParams& P, long long brick) {
    const unsigned peers = __match_any_sync(__activemask(), (unsigned long long)brick);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicOr(P.brick_used + (brick >> 5), 1u << (brick & 31));
}

// The half-resolution level at texture-space point (sx, sy, sz), sampled
// like the full level (clamped voxel position, trilinear from the brick
// holding the floor voxel): normalised (RAW false) or raw values. This is
// the coarser octree level Voreen's octree raycaster reads where a brick is
// not on the GPU (singleoctreeraycaster.cl), here the 2x2x2 mean of
// VolumeOctree's half-sampled parent bricks (volumeoctree.cpp:188-202).
template <int DT, bool RAW>
__device__ __noinline__ float lod_tap(const MarchParams& P, float sx, float sy, float sz) {
    using T = typename Vox<DT>::T;
    const BrickLayout& L = P.L;
    const float vx = clampf_(s_(m_(P.lod_dimf[0], sx), 0.5f), 0.f, P.lod_dim_m1[0]);
    const float vy = clampf_(s_(m_(P.lod_dimf[1], sy), 0.5f), 0.f, P.lod_dim_m1[1]);
    const float vz = clampf_(s_(m_(P.lod_dimf[2], sz), 0.5f), 0.f, P.lod_dim_m1[2]);
    const float flx = floorf(vx), fly = floorf(vy), flz = floorf(vz);
    const int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    const int bx = ix >> L.shift, by = iy >> L.shift, bz = iz >> L.shift;
    const long long brick = ((long long)bz * P.lod_nb[1] + by) * P.lod_nb[0] + bx;
    const T* b = reinterpret_cast<const T*>(P.lod_bricks) + brick * L.brick_stride;
    const int o = ((iz - (bz << L.shift) + APRON_LO) * L.S + (iy - (by << L.shift) + APRON_LO)) * L.S +
                  (ix - (bx << L.shift) + APRON_LO);
    const float fx = s_(vx, flx), fy = s_(vy, fly), fz = s_(vz, flz);
    return RAW ? tri_raw<DT>(b, o, L.S, L.S * L.S, fx, fy, fz) : tri_at<DT>(b, o, L.S, L.S * L.S, fx, fy, fz);
}

// The same from a full-resolution voxel position (gradient and previous-sample
// taps of a brick without a cache slot). These taps read the coarser level
// and so approximate the full-resolution values whatever the rounding of
// their texture-space position; a fast division serves.
template <int DT, bool RAW>
__device__ __forceinline__ float lod_tap_voxel(const MarchParams& P, float vx, float vy, float vz) {
    return lod_tap<DT, RAW>(P, __fdividef(vx + 0.5f, P.dimf[0]), __fdividef(vy + 0.5f, P.dimf[1]),
                            __fdividef(vz + 0.5f, P.dimf[2]));
}

template <int DT, bool POOL>
__device__ __noinline__ float tap_raw_any_brick(const MarchParams& P, const typename Vox<DT>::T* __restrict__ bricks,
                                                float vx, float vy, float vz) {
    const BrickLayout& L = P.L;
    const float flx = floorf(vx), fly = floorf(vy), flz = floorf(vz);
    const int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    const int bx = ix >> L.shift, by = iy >> L.shift, bz = iz >> L.shift;
    const long long brick = ((long long)bz * L.nb[1] + by) * L.nb[0] + bx;
    const int o = ((iz - (bz << L.shift) + APRON_LO) * L.S + (iy - (by << L.shift) + APRON_LO)) * L.S +
                  (ix - (bx << L.shift) + APRON_LO);
    if (POOL && P.brick_used) atomicOr(P.brick_used + (brick >> 5), 1u << (brick & 31));
    const typename Vox<DT>::T* b = brick_base<POOL>(P, bricks, brick);
    if (POOL && !b) return lod_tap_voxel<DT, true>(P, vx, vy, vz);
    return tri_raw<DT>(b, o, L.S, L.S * L.S, vx - flx, vy - fly, vz - flz);
}

// One central-difference lookup displaced along one axis: tap position `vt`
// (clamped voxel coordinate on that axis, as calcGradientA's texture lookup
// gives it) with the centre's coordinates on the other axes. Reads from the
// centre's brick when the stencil fits in its apron.
template <int DT, int AXIS, bool POOL>
__device__ __forceinline__ float grad_tap(const MarchParams& P, const typename Vox<DT>::T* __restrict__ bricks,
                                          const typename Vox<DT>::T* __restrict__ b, int o, int lc, int ic, float vt,
                                          float vx, float vy, float vz, float fx, float fy, float fz) {
    const float fl = floorf(vt);
    const int it = (int)fl;
    const int lt = lc + (it - ic);
    const int S = P.L.S, S2 = P.L.S * P.L.S;
    if ((!POOL || b) && lt >= 0 && lt <= P.L.B + 1) {
        const int stride = AXIS == 0 ? 1 : (AXIS == 1 ? S : S2);
        const float ft = vt - fl;
        return tri_raw<DT>(b, o + (it - ic) * stride, S, S2, AXIS == 0 ? ft : fx, AXIS == 1 ? ft : fy,
                           AXIS == 2 ? ft : fz);
    }
    return tap_raw_any_brick<DT, POOL>(P, bricks, AXIS == 0 ? vt : vx, AXIS == 1 ? vt : vy, AXIS == 2 ? vt : vz);
}

// phongShading (mod_shading.frag:134-151), ka = kd = TF colour, ks = 1.
__device__ __forceinline__ F3 phong_fast(const MarchParams& P, F3 n, F3 pos, F3 col) {
    const F3 N = fnormalize(n);
    F3 L{P.light_phys[0] - pos.x, P.light_phys[1] - pos.y, P.light_phys[2] - pos.z};
    const F3 V = fnormalize(F3{P.cam_phys[0] - pos.x, P.cam_phys[1] - pos.y, P.cam_phys[2] - pos.z});
    const float d2 = fdot(L, L);
    const float rd = d2 > 0.f ? rsqrtf(d2) : 0.f;
    const float d = d2 * rd;
    L = F3{L.x * rd, L.y * rd, L.z * rd};
    const float ndl = fmaxf(fdot(N, L), 0.f);
    const F3 Hh = fnormalize(F3{V.x + L.x, V.y + L.y, V.z + L.z});
    const float ndh = fmaxf(fdot(N, Hh), 0.f);
    const float spec = __powf(ndh, P.shininess);
    F3 out{__fmaf_rn(col.x * P.dif[0], ndl, __fmaf_rn(P.spec[0], spec, col.x * P.amb[0])),
           __fmaf_rn(col.y * P.dif[1], ndl, __fmaf_rn(P.spec[1], spec, col.y * P.amb[1])),
           __fmaf_rn(col.z * P.dif[2], ndl, __fmaf_rn(P.spec[2], spec, col.z * P.amb[2]))};
    if (P.atten_on) {
        const float att = fminf(__fdividef(1.f, __fmaf_rn(P.att[2] * d, d, __fmaf_rn(P.att[1], d, P.att[0]))), 1.f);
        out = F3{out.x * att, out.y * att, out.z * att};
    }
    return out;
}

// Analytic entry/exit for pixel (px, py): the pixel-centre ray through the
// unit texture cube, clipped to the near/far planes. Returns false for
// background.
__device__ bool analytic_entry_exit(const MarchParams& P, int px, int py, float4& e, float4& l) {
    const float nx = s_(d_(m_(2.f, a_((float)px, 0.5f)), (float)P.W), 1.f);
    const float ny = s_(d_(m_(2.f, a_((float)py, 0.5f)), (float)P.H), 1.f);
    float pn[4], pf[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const float* M = P.inv_mvp + 4 * r;
        const float base = a_(m_(M[0], nx), m_(M[1], ny));
        pn[r] = a_(s_(base, M[2]), M[3]);
        pf[r] = a_(a_(base, M[2]), M[3]);
    }
    float o[3], d[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o[i] = d_(pn[i], pn[3]);
        d[i] = s_(d_(pf[i], pf[3]), o[i]);
    }
    float s0 = 0.f, s1 = 1.f;
    bool hit = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (d[i] == 0.f) {
            if (o[i] < P.box_lo[i] || o[i] > P.box_hi[i]) hit = false;
        } else {
            float a = d_(s_(P.box_lo[i], o[i]), d[i]), b = d_(s_(P.box_hi[i], o[i]), d[i]);
            if (a > b) {
                const float t = a;
                a = b;
                b = t;
            }
            s0 = fmaxf(s0, a);
            s1 = fminf(s1, b);
        }
    }
    if (!hit || !(s0 < s1)) {
        e = make_float4(0.f, 0.f, 0.f, 0.f);
        l = e;
        return false;
    }
    float en[3], ex[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float a = clampf_(a_(o[i], m_(s0, d[i])), P.box_lo[i], P.box_hi[i]);
        float b = clampf_(a_(o[i], m_(s1, d[i])), P.box_lo[i], P.box_hi[i]);
        if (P.quantize) {
            a = d_(floorf(a_(m_(a, 65535.f), 0.5f)), 65535.f);
            b = d_(floorf(a_(m_(b, 65535.f), 0.5f)), 65535.f);
        }
        en[i] = a;
        ex[i] = b;
    }
    e = make_float4(en[0], en[1], en[2], 1.f);
    l = make_float4(ex[0], ex[1], ex[2], 1.f);
    return true;
}

template <int EE> __device__ __forceinline__ F3 entry_point_at(const MarchParams& P, int x, int y) {
    x = min(max(x, 0), P.W - 1);
    y = min(max(y, 0), P.H - 1);
    float4 e, l;
    if (EE == VRC_EE_BUFFERS) {
        e = P.entry[(size_t)y * P.W + x];
    } else {
        analytic_entry_exit(P, x, y, e, l);
    }
    return F3{e.x, e.y, e.z};
}

// fixClipBorderGradient (mod_gradients.frag:39-46)
template <int EE> __device__ F3 clip_border_gradient(const MarchParams& P, F3 s, F3 dir, int px, int py) {
    const F3 a = entry_point_at<EE>(P, px + 2, py), b = entry_point_at<EE>(P, px, py + 2);
    const F3 v0 = normalize3(F3{s_(a.x, s.x), s_(a.y, s.y), s_(a.z, s.z)});
    const F3 v1 = normalize3(F3{s_(b.x, s.x), s_(b.y, s.y), s_(b.z, s.z)});
    F3 g{s_(m_(v0.y, v1.z), m_(v0.z, v1.y)), s_(m_(v0.z, v1.x), m_(v0.x, v1.z)), s_(m_(v0.x, v1.y), m_(v0.y, v1.x))};
    if (!(dot3(g, dir) < 0.f)) g = F3{-g.x, -g.y, -g.z};
    return g;
}

__device__ __forceinline__ void write_out(const MarchParams& P, size_t pix, float4 r) {
    if (P.out_format == VRC_OUT_RGBA32F) {
        reinterpret_cast<float4*>(P.out)[pix] = r;
    } else if (P.out_format == VRC_OUT_RGBA8) {
        auto q = [](float v) -> unsigned {
            v = fminf(fmaxf(v, 0.f), 1.f);
            return (unsigned)floorf(v * 255.f + 0.5f);
        };
        reinterpret_cast<uchar4*>(P.out)[pix] = make_uchar4(q(r.x), q(r.y), q(r.z), q(r.w));
    } else {
        auto q = [](float v) -> unsigned {
            v = fminf(fmaxf(v, 0.f), 1.f);
            return (unsigned)floorf(v * 65535.f + 0.5f);
        };
        reinterpret_cast<ushort4*>(P.out)[pix] = make_ushort4(q(r.x), q(r.y), q(r.z), q(r.w));
    }
}

struct Counters {
    unsigned long long samples = 0, fetched = 0, shaded = 0, runs = 0;
};

// MIP: true when no sample of a cell whose largest normalised value is `m`
// can exceed the ray's maximum real-world intensity `max_int`, so the cell
// changes nothing (compositeMIP replaces the result only for a larger value).
// A trilinear sample exceeds its largest voxel by at most ~13 ulp of rounding
// (three products, seven sums, weights summing to at most (1 + u)^3); m is
// raised by 2e-6 relative, well above that, and the real-world mapping is
// monotone (scale >= 0, checked on the host), so the test is exact.
__device__ __forceinline__ bool mip_cell_below(const MarchParams& P, float m, float max_int) {
    const float mb = m + fabsf(m) * 2e-6f;
    return a_(m_(mb, P.rwm_scale), P.rwm_offset) <= max_int;
}

// Largest ray parameter up to which every sample's floor voxel stays in skip
// cell (cx, cy, cz): per axis, where the unclamped voxel coordinate
// dim * (first + t * dir) - 0.5 reaches the cell face it moves toward, pulled
// in by skip_margin voxels to absorb rounding (the margin exceeds the error of
// the sample-position arithmetic and of the fast division here by orders of
// magnitude). Cells on the volume border have no face on their outer side:
// clamping keeps samples there.
__device__ __forceinline__ float cell_exit_t(const MarchParams& P, float4 f, float dx, float dy, float dz, int cx,
                                             int cy, int cz, int shift, const int* nc) {
    const int C = 1 << shift;
    const float fo[3] = {f.x, f.y, f.z}, di[3] = {dx, dy, dz};
    const int ci[3] = {cx, cy, cz};
    float tmax = INFINITY;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float a = P.dimf[i] * fo[i] - 0.5f, b = P.dimf[i] * di[i];
        if (b > 0.f && ci[i] < nc[i] - 1) {
            tmax = fminf(tmax, __fdividef((float)((ci[i] + 1) * C) - P.skip_margin - a, b));
        } else if (b < 0.f && ci[i] > 0) {
            tmax = fminf(tmax, __fdividef((float)(ci[i] * C) + P.skip_margin - a, b));
        }
    }
    return tmax;
}

// The same for a box of cells [c - r, c + r] on each axis (clipped to the
// grid: a face on the grid's border is never left, samples beyond it clamp
// to the border cells).
__device__ __forceinline__ float box_exit_t(const MarchParams& P, float4 f, float dx, float dy, float dz, int cx,
                                            int cy, int cz, int r, int shift, const int* nc) {
    const int C = 1 << shift;
    const float fo[3] = {f.x, f.y, f.z}, di[3] = {dx, dy, dz};
    const int ci[3] = {cx, cy, cz};
    float tmax = INFINITY;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float a = P.dimf[i] * fo[i] - 0.5f, b = P.dimf[i] * di[i];
        if (b > 0.f && ci[i] + r < nc[i] - 1) {
            tmax = fminf(tmax, __fdividef((float)((ci[i] + r + 1) * C) - P.skip_margin - a, b));
        } else if (b < 0.f && ci[i] - r > 0) {
            tmax = fminf(tmax, __fdividef((float)((ci[i] - r) * C) + P.skip_margin - a, b));
        }
    }
    return tmax;
}

// Advances (t, loop) over the samples of an empty run in closed form: every
// sample with t <= lim is processed (and changes nothing). The FP32 sum
// t + step, for t on the grid of its binade [2^(e-1), 2^e) with spacing u,
// is exactly t + q with q = round(step / u) * u unless step / u ends in .5
// (a rounding tie, left to the caller's exact loop). So n steps inside the
// binade give exactly t + n * q, the value the reference's one-at-a-time
// accumulation t += samplingStepSize produces. Stops short of the binade end
// and of LOOP_CAP; the caller finishes with exact single steps.
template <bool TRACK = false>
__device__ __forceinline__ void jump_empty_run(float& t, int& loop, float step, float lim, float* tprev = nullptr) {
    const int bits = __float_as_int(t);
    const int ex = (bits >> 23) & 0xff;  // biased exponent, t normal and > 0
    if (ex < 24 || ex > 250) return;
    const float u = __int_as_float((ex - 23) << 23);     // ulp of t: 2^(ex - 127 - 23)
    const float top = __int_as_float((ex + 1) << 23);    // 2^(ex - 127 + 1): end of t's binade
    const float k = __fmul_rn(step, __int_as_float((127 + 150 - ex) << 23));  // step / u, exact
    const float kf = floorf(k);
    if (__fsub_rn(k, kf) == 0.5f) return;
    const float q = __fmul_rn(rintf(k), u);
    if (q <= 0.f) return;
    float nf = floorf(__fdividef(__fsub_rn(lim, t), q)) + 1.f;
    nf = fminf(nf, floorf(__fdividef(__fsub_rn(top, t), q)));
    nf = fminf(nf, (float)(LOOP_CAP - loop));
    int n = nf > 0.f ? (int)nf : 0;
    while (n > 0 && (__fadd_rn(t, __fmul_rn((float)(n - 1), q)) > lim || __fadd_rn(t, __fmul_rn((float)n, q)) >= top))
        --n;
    if (TRACK && n > 0) *tprev = __fadd_rn(t, __fmul_rn((float)(n - 1), q));  // the last sample jumped over
    t = __fadd_rn(t, __fmul_rn((float)n, q));
    loop += n;
}

// Normalised trilinear value at a clamped voxel position, read from the
// brick holding its floor voxel, in the exact order of the intensity sample.
template <int DT, bool POOL>
__device__ __forceinline__ float tap_norm(const MarchParams& P, const typename Vox<DT>::T* __restrict__ bricks,
                                          float vx, float vy, float vz) {
    const BrickLayout& L = P.L;
    const float flx = floorf(vx), fly = floorf(vy), flz = floorf(vz);
    const int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    const int bx = ix >> L.shift, by = iy >> L.shift, bz = iz >> L.shift;
    const long long brick = ((long long)bz * L.nb[1] + by) * L.nb[0] + bx;
    const int lx = ix - (bx << L.shift) + APRON_LO, ly = iy - (by << L.shift) + APRON_LO,
              lz = iz - (bz << L.shift) + APRON_LO;
    if (POOL && P.brick_used) atomicOr(P.brick_used + (brick >> 5), 1u << (brick & 31));
    const typename Vox<DT>::T* b = brick_base<POOL>(P, bricks, brick);
    if (POOL && !b) return lod_tap_voxel<DT, false>(P, vx, vy, vz);
    return tri_at<DT>(b, (lz * L.S + ly) * L.S + lx, L.S, L.S * L.S, s_(vx, flx),
                      s_(vy, fly), s_(vz, flz));
}

// Texture-space point -> clamped voxel position (cpuraycaster.cpp:243).
__device__ __forceinline__ float to_voxel(const MarchParams& P, int axis, float s) {
    return clampf_(s_(m_(P.dimf[axis], s), 0.5f), 0.f, P.dim_m1[axis]);
}

// calcGradientA (mod_gradients.frag:202-214) with exactly rounded taps, in
// the order the CPU restatement evaluates it: six normalised trilinear
// lookups at +-1/dim in texture space, (v(-) - v(+)) * 0.5/spacing * rwmScale.
template <int DT, bool POOL>
__device__ F3 gradient_exact(const MarchParams& P, const typename Vox<DT>::T* __restrict__ bricks, float sx, float sy,
                             float sz, float vx, float vy, float vz) {
    const float v0 = tap_norm<DT, POOL>(P, bricks, to_voxel(P, 0, a_(sx, P.offs[0])), vy, vz);
    const float v1 = tap_norm<DT, POOL>(P, bricks, vx, to_voxel(P, 1, a_(sy, P.offs[1])), vz);
    const float v2 = tap_norm<DT, POOL>(P, bricks, vx, vy, to_voxel(P, 2, a_(sz, P.offs[2])));
    const float v3 = tap_norm<DT, POOL>(P, bricks, to_voxel(P, 0, s_(sx, P.offs[0])), vy, vz);
    const float v4 = tap_norm<DT, POOL>(P, bricks, vx, to_voxel(P, 1, s_(sy, P.offs[1])), vz);
    const float v5 = tap_norm<DT, POOL>(P, bricks, vx, vy, to_voxel(P, 2, s_(sz, P.offs[2])));
    return F3{m_(m_(s_(v3, v0), P.spacing_rcp_half[0]), P.rwm_scale),
              m_(m_(s_(v4, v1), P.spacing_rcp_half[1]), P.rwm_scale),
              m_(m_(s_(v5, v2), P.spacing_rcp_half[2]), P.rwm_scale)};
}

// compositeMIDAhelper (mod_compositing.frag:109-125): delta = max intensity
// increase, beta = 1 - delta * (1 + gamma), then a DVR step weighted by beta.
__device__ __forceinline__ float4 mida_step(float4 r, float v, float4 c, float maxi, float gamma) {
    const float delta = v > maxi ? s_(v, maxi) : 0.f;
    const float beta = s_(1.f, m_(delta, a_(1.f, gamma)));
    const float wa = m_(s_(1.f, m_(beta, r.w)), c.w);
    return make_float4(a_(m_(beta, r.x), m_(wa, c.x)), a_(m_(beta, r.y), m_(wa, c.y)), a_(m_(beta, r.z), m_(wa, c.z)),
                       a_(m_(beta, r.w), wa));
}

// calcGradientA (mod_gradients.frag:202-214) of the sample at texture point
// (sx, sy, sz): six lookups at +-1/dim in texture space, each clamped like
// the intensity sample, interpolated on raw values. (vx, vy, vz): the
// sample's clamped voxel position, (ix, iy, iz) its floor, (fx, fy, fz) the
// fractions, b / o / (lx, ly, lz) its brick start, offset and brick-local
// voxel. The same function runs wherever a sample is shaded, so its bits do
// not depend on where.
template <int DT, bool POOL>
__device__ __forceinline__ F3 central_gradient(const MarchParams& P, const typename Vox<DT>::T* __restrict__ bricks,
                                               const typename Vox<DT>::T* __restrict__ b, int o, int lx, int ly,
                                               int lz, int ix, int iy, int iz, float vx, float vy, float vz, float fx,
                                               float fy, float fz, float sx, float sy, float sz) {
    const BrickLayout& L = P.L;
    const int S = L.S, S2 = L.S * L.S;
    // calcGradientA: six lookups at +-1/dim in texture space, each
    // clamped like the intensity sample; interpolated on raw values
    const float vxp = clampf_(s_(m_(P.dimf[0], a_(sx, P.offs[0])), 0.5f), 0.f, P.dim_m1[0]);
    const float vyp = clampf_(s_(m_(P.dimf[1], a_(sy, P.offs[1])), 0.5f), 0.f, P.dim_m1[1]);
    const float vzp = clampf_(s_(m_(P.dimf[2], a_(sz, P.offs[2])), 0.5f), 0.f, P.dim_m1[2]);
    const float vxm = clampf_(s_(m_(P.dimf[0], s_(sx, P.offs[0])), 0.5f), 0.f, P.dim_m1[0]);
    const float vym = clampf_(s_(m_(P.dimf[1], s_(sy, P.offs[1])), 0.5f), 0.f, P.dim_m1[1]);
    const float vzm = clampf_(s_(m_(P.dimf[2], s_(sz, P.offs[2])), 0.5f), 0.f, P.dim_m1[2]);
    // The taps lie at or beyond the sample on their axis, so
    // the "+" taps can only leave the apron upward and the
    // "-" taps downward. When all six stay inside (away from
    // the volume's faces, always), they are read in one
    // straight block whose 48 loads are in flight together.
    const float fxp = floorf(vxp), fyp = floorf(vyp), fzp = floorf(vzp);
    const float fxm = floorf(vxm), fym = floorf(vym), fzm = floorf(vzm);
    const int dxp = (int)fxp - ix, dyp = (int)fyp - iy, dzp = (int)fzp - iz;
    const int dxm = (int)fxm - ix, dym = (int)fym - iy, dzm = (int)fzm - iz;
    const int top = L.B + 1;
    float v0, v1, v2, v3, v4, v5;
    if ((!POOL || b) && dxp == 1 && dyp == 1 && dzp == 1 && dxm == -1 && dym == -1 && dzm == -1 &&
        lx + 1 <= top && ly + 1 <= top && lz + 1 <= top && lx >= 1 && ly >= 1 && lz >= 1) {
        // The usual case, each tap one voxel from the sample's floor
        // voxel: the six stencils cover 32 voxels (the centre 2^3 and
        // 4 more on each side), read once and interpolated from
        // registers in tri_raw's order. r<axis><side><a><b>: the
        // extension voxels on that side, (a, b) along the other two axes.
#define VRC_R(X, Y, Z) ((float)__ldg(b + o + (X) + (Y) * S + (Z) * S2))
        const float c000 = VRC_R(0, 0, 0), c100 = VRC_R(1, 0, 0), c010 = VRC_R(0, 1, 0),
                    c110 = VRC_R(1, 1, 0), c001 = VRC_R(0, 0, 1), c101 = VRC_R(1, 0, 1),
                    c011 = VRC_R(0, 1, 1), c111 = VRC_R(1, 1, 1);
        const float rxm00 = VRC_R(-1, 0, 0), rxm10 = VRC_R(-1, 1, 0), rxm01 = VRC_R(-1, 0, 1),
                    rxm11 = VRC_R(-1, 1, 1);
        const float rxp00 = VRC_R(2, 0, 0), rxp10 = VRC_R(2, 1, 0), rxp01 = VRC_R(2, 0, 1),
                    rxp11 = VRC_R(2, 1, 1);
        const float rym00 = VRC_R(0, -1, 0), rym10 = VRC_R(1, -1, 0), rym01 = VRC_R(0, -1, 1),
                    rym11 = VRC_R(1, -1, 1);
        const float ryp00 = VRC_R(0, 2, 0), ryp10 = VRC_R(1, 2, 0), ryp01 = VRC_R(0, 2, 1),
                    ryp11 = VRC_R(1, 2, 1);
        const float rzm00 = VRC_R(0, 0, -1), rzm10 = VRC_R(1, 0, -1), rzm01 = VRC_R(0, 1, -1),
                    rzm11 = VRC_R(1, 1, -1);
        const float rzp00 = VRC_R(0, 0, 2), rzp10 = VRC_R(1, 0, 2), rzp01 = VRC_R(0, 1, 2),
                    rzp11 = VRC_R(1, 1, 2);
#undef VRC_R
        v0 = tri_regs(c100, rxp00, c110, rxp10, c101, rxp01, c111, rxp11, vxp - fxp, fy, fz);
        v1 = tri_regs(c010, c110, ryp00, ryp10, c011, c111, ryp01, ryp11, fx, vyp - fyp, fz);
        v2 = tri_regs(c001, c101, c011, c111, rzp00, rzp10, rzp01, rzp11, fx, fy, vzp - fzp);
        v3 = tri_regs(rxm00, c000, rxm10, c010, rxm01, c001, rxm11, c011, vxm - fxm, fy, fz);
        v4 = tri_regs(rym00, rym10, c000, c100, rym01, rym11, c001, c101, fx, vym - fym, fz);
        v5 = tri_regs(rzm00, rzm10, rzm01, rzm11, c000, c100, c010, c110, fx, fy, vzm - fzm);
    } else if ((!POOL || b) && lx + dxp <= top && ly + dyp <= top && lz + dzp <= top &&
               lx + dxm >= 0 && ly + dym >= 0 && lz + dzm >= 0) {
        v0 = tri_raw<DT>(b, o + dxp, S, S2, vxp - fxp, fy, fz);
        v1 = tri_raw<DT>(b, o + dyp * S, S, S2, fx, vyp - fyp, fz);
        v2 = tri_raw<DT>(b, o + dzp * S2, S, S2, fx, fy, vzp - fzp);
        v3 = tri_raw<DT>(b, o + dxm, S, S2, vxm - fxm, fy, fz);
        v4 = tri_raw<DT>(b, o + dym * S, S, S2, fx, vym - fym, fz);
        v5 = tri_raw<DT>(b, o + dzm * S2, S, S2, fx, fy, vzm - fzm);
    } else {
        v0 = grad_tap<DT, 0, POOL>(P, bricks, b, o, lx, ix, vxp, vx, vy, vz, fx, fy, fz);
        v1 = grad_tap<DT, 1, POOL>(P, bricks, b, o, ly, iy, vyp, vx, vy, vz, fx, fy, fz);
        v2 = grad_tap<DT, 2, POOL>(P, bricks, b, o, lz, iz, vzp, vx, vy, vz, fx, fy, fz);
        v3 = grad_tap<DT, 0, POOL>(P, bricks, b, o, lx, ix, vxm, vx, vy, vz, fx, fy, fz);
        v4 = grad_tap<DT, 1, POOL>(P, bricks, b, o, ly, iy, vym, vx, vy, vz, fx, fy, fz);
        v5 = grad_tap<DT, 2, POOL>(P, bricks, b, o, lz, iz, vzm, vx, vy, vz, fx, fy, fz);
    }
    return F3{(v3 - v0) * P.gscale[0], (v4 - v1) * P.gscale[1], (v5 - v2) * P.gscale[2]};
}

// One ray: the loop of cpuraycaster.cpp:239-317 with the GLSL compositing.
template <int DT, int COMP, int SHADE, int EE, bool POOL = false>
__device__ float4 march_ray(const MarchParams& P, const uchar4* __restrict__ s_tf, const float* __restrict__ s_alpha,
                            float4 f, float4 l, int px,
                            int py, Counters& cnt, float2& aux) {
    using T = typename Vox<DT>::T;
    const T* __restrict__ bricks = reinterpret_cast<const T*>(P.bricks);
    const BrickLayout& L = P.L;
    const int S = L.S, S2 = L.S * L.S;
    const float step = P.step;
    float dx = s_(l.x, f.x), dy = s_(l.y, f.y), dz = s_(l.z, f.z);
    const bool dir0 = dx == 0.f && dy == 0.f && dz == 0.f;
    const bool last0 = l.x == 0.f && l.y == 0.f && l.z == 0.f;
    const bool first0 = f.x == 0.f && f.y == 0.f && f.z == 0.f;
    float tend;
    if (dir0 && !last0 && !first0) {
        tend = d_(step, 2.f);
    } else {
        tend = len3(dx, dy, dz);
        const float rl = d_(1.f, tend);
        dx = m_(dx, rl);
        dy = m_(dy, rl);
        dz = m_(dz, rl);
    }
    // pre-integrated classification (cpuraycaster.cpp:255-261); no early ray
    // termination for mip / mop / mida (volumeraycaster.cpp:226-228)
    constexpr bool PI = COMP == COMP_DVR_PREINT;
    constexpr bool ERT = !(COMP == VRC_MIP || COMP == VRC_MOP || COMP == VRC_MIDA);
    float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
    float max_int = 0.f;
    float last = 0.f;  // lastIntensity (cpuraycaster.cpp:235), TF-normalised
    // pre-integration: whether the previous sample lay in an empty cell, and
    // whether `last` still has to be read at t_last (the last skipped sample)
    bool prev_empty = false, last_stale = false;
    float t_last = 0.f;
    float t = 0.f;
    float hit_t = -1.f, hit_g = 0.f;  // first sample with alpha > 0 (auxiliary output)
    long long marked = -1;             // last brick recorded as read (cache refinement)
    // the brick of the last fetched sample and its start: consecutive samples
    // mostly stay in one brick
    int cached_brick = -1;
    const T* cached_base = nullptr;
    bool finished = false;
    int loop = 0;
    while (!finished && loop < LOOP_CAP) {
        const float sx = a_(f.x, m_(t, dx)), sy = a_(f.y, m_(t, dy)), sz = a_(f.z, m_(t, dz));
        const float vx = clampf_(s_(m_(P.dimf[0], sx), 0.5f), 0.f, P.dim_m1[0]);
        const float vy = clampf_(s_(m_(P.dimf[1], sy), 0.5f), 0.f, P.dim_m1[1]);
        const float vz = clampf_(s_(m_(P.dimf[2], sz), 0.5f), 0.f, P.dim_m1[2]);
        const float flx = floorf(vx), fly = floorf(vy), flz = floorf(vz);
        const int ix = (int)flx, iy = (int)fly, iz = (int)flz;
        bool skip_after = false;  // pre-integration: skip the samples after this one in its empty cell
        float skip_lim = 0.f;
        if (P.occupancy) {
            // The fine cell (2^3 or 4^3 by default) decides whether the sample
            // is skipped at all. A TF-empty cell with the cells' distance field
            // given jumps the whole empty box around it; otherwise (MIP's
            // max-based skipping, pre-integration with steps of a voxel or
            // more) a coarse (brick-sized) cell, which holds its fine cells'
            // value ranges and so can be empty only where the fine cell is,
            // is read to jump the whole brick at once.
            float tsafe = 0.f;
            bool empty = false;
            // cell and brick indices fit 32 bits (checked when the volume is uploaded)
            const int fcx = ix >> P.cshift, fcy = iy >> P.cshift, fcz = iz >> P.cshift;
            const unsigned fc = ((unsigned)fcz * (unsigned)P.nc[1] + (unsigned)fcy) * (unsigned)P.nc[0] + (unsigned)fcx;
            const uint32_t fine_word = __ldg(P.occupancy + (fc >> 5));
            constexpr bool MIPS = COMP == VRC_MIP;
            const bool mip_skip = MIPS && P.mip_skip;
            const float fine_max = mip_skip ? __ldg(P.cell_max + fc) : 0.f;
            const bool fine_bit_empty = ((fine_word >> (fc & 31)) & 1u) == 0u;
            if (fine_bit_empty || (mip_skip && mip_cell_below(P, fine_max, max_int))) {
                empty = true;
                bool coarse_empty = false;
                if (P.occ_dist && fine_bit_empty) {
                    // jump the empty box around the cell that the distance to
                    // the nearest occupied cell guarantees
                    const int r = (int)__ldg(P.occ_dist + fc) - 1;
                    tsafe = box_exit_t(P, f, dx, dy, dz, fcx, fcy, fcz, r, P.cshift, P.nc);
                    coarse_empty = true;
                } else if (P.occ_coarse) {
                    const int cx = ix >> P.cshift_coarse, cy = iy >> P.cshift_coarse, cz = iz >> P.cshift_coarse;
                    const unsigned c =
                        ((unsigned)cz * (unsigned)P.ncc[1] + (unsigned)cy) * (unsigned)P.ncc[0] + (unsigned)cx;
                    const uint32_t coarse_word = __ldg(P.occ_coarse + (c >> 5));
                    const float coarse_max = mip_skip ? __ldg(P.brick_max + c) : 0.f;
                    if (((coarse_word >> (c & 31)) & 1u) == 0u ||
                        (mip_skip && mip_cell_below(P, coarse_max, max_int))) {
                        tsafe = cell_exit_t(P, f, dx, dy, dz, cx, cy, cz, P.cshift_coarse, P.ncc);
                        coarse_empty = true;
                    }
                }
                if (!coarse_empty) tsafe = cell_exit_t(P, f, dx, dy, dz, fcx, fcy, fcz, P.cshift, P.nc);
            }
            if (PI && empty && P.pi_chain && prev_empty) {
                // This sample and the previous one lie in empty cells that
                // share a voxel (a step moves less than a voxel per axis), so
                // their value ranges overlap and every table entry between
                // the two samples has alpha 0: skip it and the rest of its
                // cell; `last` is read when a sample is next classified.
                ++cnt.runs;
                float tp = t;
                t = a_(t, step);
                ++loop;
                const float lim = fminf(tsafe, tend);
                while (t <= lim && loop < LOOP_CAP) {
                    jump_empty_run<true>(t, loop, step, lim, &tp);
                    if (t <= lim && loop < LOOP_CAP) {
                        tp = t;
                        t = a_(t, step);
                        ++loop;
                    }
                }
                finished = t > tend;
                last_stale = true;
                t_last = tp;
                continue;
            } else if (PI && empty) {
                // A pre-integrated colour also depends on the previous sample,
                // which may lie outside the cell: classify this sample as
                // usual, skip the ones after it that stay in the cell (both
                // ends of their segments are in the cell, so every table
                // entry they reach has alpha 0).
                skip_after = true;
                skip_lim = fminf(tsafe, tend);
            } else if (empty) {
                // This sample lies in a cell where every reachable TF entry has
                // alpha 0: it changes nothing. So do all following samples that
                // provably stay in the cell; only t and the count advance.
                ++cnt.runs;
                t = a_(t, step);
                ++loop;
                // samples are processed while t <= tend and t <= tsafe: jump to
                // the end of t's binade in closed form, step across the binade
                // edge (or a rounding tie) singly, repeat
                const float lim = fminf(tsafe, tend);
                while (t <= lim && loop < LOOP_CAP) {
                    jump_empty_run(t, loop, step, lim);
                    if (t <= lim && loop < LOOP_CAP) {
                        t = a_(t, step);
                        ++loop;
                    }
                }
                finished = t > tend;
                continue;
            }
        }
        {
            const int bx = ix >> L.shift, by = iy >> L.shift, bz = iz >> L.shift;
            const int brick = (bz * L.nb[1] + by) * L.nb[0] + bx;
            if (brick != cached_brick) {
                cached_brick = brick;
                cached_base = brick_base<POOL>(P, bricks, (long long)brick);
            }
            ++cnt.fetched;
            const float fx = s_(vx, flx), fy = s_(vy, fly), fz = s_(vz, flz);
            const T* __restrict__ b = cached_base;
            if (POOL && P.brick_used && brick != marked) {
                marked = brick;
                mark_used(P, brick);
            }
            const int lx = ix - (bx << L.shift) + APRON_LO, ly = iy - (by << L.shift) + APRON_LO,
                      lz = iz - (bz << L.shift) + APRON_LO;
            const int o = (lz * S + ly) * S + lx;
            const float intensity =
                (!POOL || b) ? tri_at<DT>(b, o, S, S2, fx, fy, fz) : lod_tap<DT, false>(P, sx, sy, sz);
            const float rw = a_(m_(intensity, P.rwm_scale), P.rwm_offset);
            float4 c;
            if (PI) {
                if (last_stale) {  // the previous sample was skipped: read its TF coordinate
                    ++cnt.fetched;
                    const float px_ = a_(f.x, m_(t_last, dx)), py_ = a_(f.y, m_(t_last, dy)),
                                pz_ = a_(f.z, m_(t_last, dz));
                    const float rwp = a_(m_(tap_norm<DT, POOL>(P, bricks, to_voxel(P, 0, px_), to_voxel(P, 1, py_),
                                                        to_voxel(P, 2, pz_)),
                                            P.rwm_scale),
                                         P.rwm_offset);
                    last = rw_to_tf(rwp, P.tf_lo, P.tf_hi);
                    last_stale = false;
                }
                prev_empty = skip_after;  // this sample is classified; its cell was empty iff skip_after
                // PreIntegrationTable::classify(last, cur) (preintegrationtable.cpp:256-279)
                const float cur = rw_to_tf(rw, P.tf_lo, P.tf_hi);
                c = __ldg(P.pi_table + (size_t)tf_index(cur, P.pi_res) * P.pi_res + tf_index(last, P.pi_res));
                last = cur;
            } else {
                // apply1DTF: the entry's bytes / 255 (exact), alpha from the per-byte table
                const uchar4 e8 = s_tf[tf_index(rw_to_tf(rw, P.tf_lo, P.tf_hi), P.tf_width)];
                c = make_float4(Vox<VRC_U8>::norm(e8.x), Vox<VRC_U8>::norm(e8.y), Vox<VRC_U8>::norm(e8.z),
                                s_alpha[e8.w]);
            }
            if (c.w > 0.f) {
                if (SHADE == VRC_SHADE_PHONG) {
                    ++cnt.shaded;
                    F3 g;
                    if (t == 0.f) {
                        g = clip_border_gradient<EE>(P, F3{sx, sy, sz}, F3{dx, dy, dz}, px, py);
                    } else {
                        g = central_gradient<DT, POOL>(P, bricks, b, o, lx, ly, lz, ix, iy, iz, vx, vy, vz, fx, fy,
                                                       fz, sx, sy, sz);
                    }
                    const F3 pos{a_(m_(s_(m_(sx, P.dimf[0]), 0.5f), P.spacing[0]), P.vol_offset[0]),
                                 a_(m_(s_(m_(sy, P.dimf[1]), 0.5f), P.spacing[1]), P.vol_offset[1]),
                                 a_(m_(s_(m_(sz, P.dimf[2]), 0.5f), P.spacing[2]), P.vol_offset[2])};
                    if (hit_t < 0.f) hit_g = sqrtf(g.x * g.x + g.y * g.y + g.z * g.z);
                    const F3 sh = phong_fast(P, g, pos, F3{c.x, c.y, c.z});
                    c.x = sh.x;
                    c.y = sh.y;
                    c.z = sh.z;
                }
                if (hit_t < 0.f) hit_t = t;
                if (COMP == VRC_DVR || PI) {
                    const float w = m_(s_(1.f, res.w), c.w);
                    res.x = a_(res.x, m_(w, c.x));
                    res.y = a_(res.y, m_(w, c.y));
                    res.z = a_(res.z, m_(w, c.z));
                    res.w = a_(res.w, m_(s_(1.f, res.w), c.w));
                } else if (COMP == VRC_MIP) {
                    if (rw > max_int) {
                        res = c;
                        max_int = rw;
                    }
                } else if (COMP == VRC_ISO) {
                    if (c.w >= s_(P.iso, 0.02f) && c.w <= a_(P.iso, 0.02f)) res = make_float4(c.x, c.y, c.z, 1.f);
                } else if (COMP == VRC_MOP) {
                    // compositeMOP (mod_compositing.frag:97-107)
                    if (c.w > res.w) res = c;
                } else if (COMP == VRC_MIDA) {
                    // compositeMIDA (mod_compositing.frag:127-146); as there, only
                    // the MIP half (gamma > 0) ever raises the maximum intensity
                    const float gm = P.mida_gamma;
                    if (gm <= 0.f) {
                        res = mida_step(res, rw, c, max_int, gm);
                    } else {
                        float4 mip = res;
                        if (rw > max_int) {
                            mip = c;
                            max_int = rw;
                        }
                        const float4 md = mida_step(res, rw, c, max_int, 0.f);
                        const float og = s_(1.f, gm);
                        res = make_float4(a_(m_(gm, mip.x), m_(og, md.x)), a_(m_(gm, mip.y), m_(og, md.y)),
                                          a_(m_(gm, mip.z), m_(og, md.z)), a_(m_(gm, mip.w), m_(og, md.w)));
                    }
                } else if (COMP == VRC_FHP) {
                    // compositeFHP (mod_compositing.frag:168-181): texture-space position
                    if (res.x == 0.f && res.y == 0.f && res.z == 0.f) res = make_float4(sx, sy, sz, 1.f);
                } else if (COMP == VRC_FHN) {
                    // compositeFHN (mod_compositing.frag:183-196): normalize(gradient) / 2 + 0.5,
                    // the gradient exactly rounded; a zero gradient gives 0.5
                    if (res.x == 0.f && res.y == 0.f && res.z == 0.f) {
                        const F3 g = t == 0.f ? clip_border_gradient<EE>(P, F3{sx, sy, sz}, F3{dx, dy, dz}, px, py)
                                              : gradient_exact<DT, POOL>(P, bricks, sx, sy, sz, vx, vy, vz);
                        const F3 n = normalize3(g);
                        res = make_float4(a_(d_(n.x, 2.f), 0.5f), a_(d_(n.y, 2.f), 0.5f), a_(d_(n.z, 2.f), 0.5f), 1.f);
                    }
                }
            }
        }
        if (ERT && res.w >= P.ert) {
            res.w = 1.f;
            finished = true;
        }
        t = a_(t, step);
        ++loop;
        finished = finished || (t > tend);
        if (PI && skip_after && !finished) {
            // skip the rest of the empty cell's samples; the next classified
            // sample needs the TF coordinate of the last one skipped
            ++cnt.runs;
            float tp = 0.f;
            bool skipped = false;
            while (t <= skip_lim && loop < LOOP_CAP) {
                const int l0 = loop;
                jump_empty_run<true>(t, loop, step, skip_lim, &tp);
                skipped = skipped || loop > l0;
                if (t <= skip_lim && loop < LOOP_CAP) {
                    tp = t;
                    skipped = true;
                    t = a_(t, step);
                    ++loop;
                }
            }
            finished = t > tend;
            if (skipped) {  // `last` is read when a sample is next classified
                last_stale = true;
                t_last = tp;
            }
        }
    }
    cnt.samples += (unsigned long long)loop;
    aux = hit_t < 0.f ? make_float2(1.f, 0.f) : make_float2(__fdividef(hit_t, fmaxf(tend, 1e-20f)), hit_g * P.aux_gscale);
    return res;
}

#ifndef VRC_MARCH_MIN_BLOCKS
#define VRC_MARCH_MIN_BLOCKS 3
#endif

template <int DT, int COMP, int SHADE, int EE, bool POOL>
__global__ void __launch_bounds__(256, VRC_MARCH_MIN_BLOCKS) march_kernel(MarchParams P) {
    // the TF in shared memory: 256 alphas, then the RGBA8 entries (17 KB at
    // 4096 entries, leaving most of the SM's 256 KB to the L1 that serves the
    // voxel gathers)
    extern __shared__ float4 s_raw[];
    float* s_alpha = reinterpret_cast<float*>(s_raw);
    uchar4* s_tf = reinterpret_cast<uchar4*>(s_alpha + 256);
    if (P.tf_width > 0) {
        for (int i = threadIdx.x; i < P.tf_width; i += blockDim.x) s_tf[i] = P.tf_rgba8[i];
        for (int i = threadIdx.x; i < 256; i += blockDim.x) s_alpha[i] = P.tf_alpha[i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int ntiles = P.tiles_x * P.tiles_y;
    Counters cnt;
    for (;;) {
        int tile = 0;
        if (lane == 0) tile = (int)atomicAdd(P.tile_counter, 1u);
        tile = __shfl_sync(FULL, tile, 0);
        if (tile >= ntiles) break;
        const int tx = tile % P.tiles_x, ty = tile / P.tiles_x;
        const int tw = 1 << P.tile_wshift;
        const int px = P.rx0 + tx * tw + (lane & (tw - 1));
        const int py = P.ry0 + ty * (32 >> P.tile_wshift) + (lane >> P.tile_wshift);
        if (px < P.rx1 && py < P.ry1) {
            const size_t pix = (size_t)py * P.W + px;
            float4 f, l;
            if (EE == VRC_EE_BUFFERS) {
                f = P.entry[pix];
                l = P.exitp[pix];
            } else {
                analytic_entry_exit(P, px, py, f, l);
            }
            const bool bg = f.x == 0.f && f.y == 0.f && f.z == 0.f && f.w == 0.f && l.x == 0.f && l.y == 0.f &&
                            l.z == 0.f && l.w == 0.f;
            float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
            float2 ax = make_float2(1.f, 0.f);
            if (!bg) r = march_ray<DT, COMP, SHADE, EE, POOL>(P, s_tf, s_alpha, f, l, px, py, cnt, ax);
            write_out(P, pix, r);
            if (P.aux) P.aux[pix] = ax;
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

// Resident CTAs per SM of one kernel for a dynamic shared memory size,
// queried once per (kernel, device, size): the attribute call and the
// occupancy query cost more host time than a frame's launch. Every march
// instantiation has the same function type, so entries are keyed by the
// kernel's address.
template <typename K>
cudaError_t resident_ctas(K k, size_t smem, int* per_sm) {
    struct Entry {
        const void* fn;
        int dev;
        size_t smem;
        int per_sm;
    };
    static std::mutex m;
    static std::vector<Entry> seen;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const void* fn = reinterpret_cast<const void*>(k);
    std::lock_guard<std::mutex> lock(m);
    for (const Entry& x : seen)
        if (x.fn == fn && x.dev == dev && x.smem == smem) {
            *per_sm = x.per_sm;
            return cudaSuccess;
        }
    // the largest table (4096 entries) once per device; smaller ones fit under it
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)std::max(smem, 256 * sizeof(float) + (size_t)4096 * sizeof(uchar4)));
    if (e != cudaSuccess) return e;
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 256, smem);
    if (e != cudaSuccess) return e;
    seen.push_back(Entry{fn, dev, smem, n});
    *per_sm = n;
    return cudaSuccess;
}

template <int DT, int COMP, int SHADE, int EE, bool POOL>
cudaError_t launch_t(const MarchParams& p, int num_sms, cudaStream_t s) {
    auto k = march_kernel<DT, COMP, SHADE, EE, POOL>;
    const size_t smem = 256 * sizeof(float) + (size_t)p.tf_width * sizeof(uchar4);
    int per_sm = 0;
    cudaError_t e = resident_ctas(k, smem, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long tiles = (long long)p.tiles_x * p.tiles_y;
    long long grid = (long long)num_sms * per_sm;
    const long long need = (tiles + 7) / 8;  // 8 warps per CTA
    if (grid > need) grid = need < 1 ? 1 : need;
    k<<<(unsigned)grid, 256, smem, s>>>(p);
    return cudaGetLastError();
}

template <int DT, int COMP, int SHADE>
cudaError_t launch_ee(const MarchParams& p, int num_sms, cudaStream_t s) {
    // POOL: a host-resident brick pool read through the device cache's slot
    // table (and its level of detail); device-resident pools compile without it
    if (p.brick_slot)
        return p.ee_mode == VRC_EE_ANALYTIC ? launch_t<DT, COMP, SHADE, VRC_EE_ANALYTIC, true>(p, num_sms, s)
                                            : launch_t<DT, COMP, SHADE, VRC_EE_BUFFERS, true>(p, num_sms, s);
    return p.ee_mode == VRC_EE_ANALYTIC ? launch_t<DT, COMP, SHADE, VRC_EE_ANALYTIC, false>(p, num_sms, s)
                                        : launch_t<DT, COMP, SHADE, VRC_EE_BUFFERS, false>(p, num_sms, s);
}

template <int DT, int COMP>
cudaError_t launch_sh(const MarchParams& p, int shading, int num_sms, cudaStream_t s) {
    return shading == VRC_SHADE_PHONG ? launch_ee<DT, COMP, VRC_SHADE_PHONG>(p, num_sms, s)
                                      : launch_ee<DT, COMP, VRC_SHADE_NONE>(p, num_sms, s);
}

}  // namespace
}  // namespace vrc
