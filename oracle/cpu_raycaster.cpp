/*
 * CPU oracle for the single-volume ray march -- TEST INFRASTRUCTURE ONLY.
 *
 * Only the tests, the smoke check and the benchmark's CPU-baseline leg load
 * this file's library, and only to compare results with or as the timed CPU
 * reference. The product library (voreen_gb300/csrc) never includes or
 * links it.
 *
 * Restates, in plain C++ (reference paths are relative to the Voreen tree):
 *   CPURaycaster::process / directRendering / apply1DTF
 *       modules/base/processors/render/cpuraycaster.cpp:90-331
 *   VolumeRAM::getVoxelNormalizedLinear   src/core/datastructures/volume/volumeram.cpp:78-97
 *   VolumeAtomic<T>::getVoxelNormalized / calcPos
 *       include/voreen/core/datastructures/volume/volumeatomic.h:521-536, 599-602
 *   getTypeAsFloat (u8 /255, u16 /65535)
 *       include/voreen/core/datastructures/volume/volumeelement.h:1261-1276
 *   textureToVoxel = T(-0.5) S(dim)       src/core/datastructures/volume/volumebase.cpp:221-224
 *   RealWorldMapping::normalizedToRealWorld
 *       src/core/datastructures/meta/realworldmappingmetadata.cpp:65-67
 *   TransFuncBase::realWorldToNormalized  src/core/datastructures/transfunc/transfuncbase.cpp:244-259
 *   TransFunc1D::createTextureData        src/core/datastructures/transfunc/1d/transfunc1d.cpp:85-116
 *   TransFunc1DKeys::getMappingForValueUByte
 *       src/core/datastructures/transfunc/1d/1dkeys/transfunc1dkeys.cpp:119-154
 *   tgt::round / iround (floor(x + 0.5))  ext/tgt/tgt_math.h:213-229
 *   tgt length / normalize (v * (1/len))  ext/tgt/vector.h:801-819
 * and the GLSL-only rules of SingleVolumeRaycaster:
 *   rayTraversal                          modules/base/glsl/rc_singlevolume.frag:116-312
 *   compositeDVR / MIP / ISO              modules/core/glsl/modules/mod_compositing.frag:47-59, 85-95, 156-166
 *   compositeMOP / MIDA / FHP / FHN       mod_compositing.frag:97-146, 168-196; no early ray
 *                                         termination for mip/mop/mida (volumeraycaster.cpp:226-228)
 *   pre-integrated classification         cpuraycaster.cpp:255-261 (classify(last, cur), no opacity
 *                                         correction), PreIntegrationTable::computeTable / classify
 *                                         src/core/datastructures/transfunc/1d/preintegrationtable.cpp:67-204, 256-279
 *   calcGradientA / fixClipBorderGradient modules/core/glsl/modules/mod_gradients.frag:202-214, 39-46
 *   phongShading and its terms            modules/core/glsl/modules/mod_shading.frag:52-151
 *   texToPhysical                         modules/core/glsl/modules/mod_sampler3d.frag:179-181
 *   EARLY_RAY_TERMINATION_OPACITY         modules/core/glsl/modules/mod_raysetup.frag:36
 *
 * Build with -ffp-contract=off: the FP32 path must round every operation on
 * its own, exactly as the reference's scalar code does on x86-64.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename R> struct V3 {
    R x, y, z;
};

template <typename R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }

/* getTypeAsFloat(value): static_cast<float>(value) / rangeMaxElement(). */
template <typename R> inline R norm_voxel(const OrcVolume* v, size_t idx) {
    switch (v->dtype) {
        case ORC_U8: return R(static_cast<const uint8_t*>(v->data)[idx]) / R(255);
        case ORC_U16: return R(static_cast<const uint16_t*>(v->data)[idx]) / R(65535);
        default: return R(static_cast<const float*>(v->data)[idx]);
    }
}

/* VolumeRAM::getVoxelNormalizedLinear (volumeram.cpp:78-97): corners from
 * floor/ceil clamped to dim-1, weights from the fractional part, eight taps
 * summed in the reference's order (llB, lrB, urB, ulB, llF, lrF, urF, ulF). */
template <typename R> R trilinear(const OrcVolume* v, R px, R py, R pz) {
    px = px > R(0) ? px : R(0);
    py = py > R(0) ? py : R(0);
    pz = pz > R(0) ? pz : R(0);
    const R fx = px - std::floor(px), fy = py - std::floor(py), fz = pz - std::floor(pz);
    const size_t dx1 = size_t(v->dims[0]) - 1, dy1 = size_t(v->dims[1]) - 1, dz1 = size_t(v->dims[2]) - 1;
    size_t lx = size_t(px), ly = size_t(py), lz = size_t(pz);
    size_t ux = size_t(std::ceil(px)), uy = size_t(std::ceil(py)), uz = size_t(std::ceil(pz));
    ux = std::min(ux, dx1); uy = std::min(uy, dy1); uz = std::min(uz, dz1);
    lx = std::min(lx, dx1); ly = std::min(ly, dy1); lz = std::min(lz, dz1);
    const size_t X = size_t(v->dims[0]), XY = size_t(v->dims[0]) * size_t(v->dims[1]);
    auto at = [&](size_t x, size_t y, size_t z) { return norm_voxel<R>(v, z * XY + y * X + x); };
    return at(lx, ly, lz) * (R(1) - fx) * (R(1) - fy) * (R(1) - fz)
         + at(ux, ly, lz) * (fx) * (R(1) - fy) * (R(1) - fz)
         + at(ux, uy, lz) * (fx) * (fy) * (R(1) - fz)
         + at(lx, uy, lz) * (R(1) - fx) * (fy) * (R(1) - fz)
         + at(lx, ly, uz) * (R(1) - fx) * (R(1) - fy) * (fz)
         + at(ux, ly, uz) * (fx) * (R(1) - fy) * (fz)
         + at(ux, uy, uz) * (fx) * (fy) * (fz)
         + at(lx, uy, uz) * (R(1) - fx) * (fy) * (fz);
}

template <typename R> inline R clampr(R x, R lo, R hi) {
    x = x > lo ? x : lo;  /* tgt::clamp = min(max(x, lo), hi) */
    return x < hi ? x : hi;
}

/* Texture-space sample -> clamped voxel position -> trilinear value
 * (cpuraycaster.cpp:243-249). */
template <typename R> inline R sample_tex(const OrcVolume* v, R sx, R sy, R sz) {
    const R vx = clampr(R(v->dims[0]) * sx - R(0.5), R(0), R(v->dims[0]) - R(1));
    const R vy = clampr(R(v->dims[1]) * sy - R(0.5), R(0), R(v->dims[1]) - R(1));
    const R vz = clampr(R(v->dims[2]) * sz - R(0.5), R(0), R(v->dims[2]) - R(1));
    return trilinear<R>(v, vx, vy, vz);
}

/* TransFuncBase::realWorldToNormalized (transfuncbase.cpp:244-259). */
template <typename R> inline R rw_to_tf(R rw, R lo, R hi) {
    if (rw < lo) return R(0);
    if (rw > hi) return R(1);
    if (lo == hi) return R(0);
    return (rw - lo) / (hi - lo);
}

/* CPURaycaster::apply1DTF index: clamp(iround(x * (w-1)), 0, w-1) with
 * tgt::round(x) = floor(x + 0.5). */
template <typename R> inline int tf_index(R x, int w) {
    const R f = x * R(w - 1);
    int i = static_cast<int>(std::floor(f + R(0.5)));
    return i < 0 ? 0 : (i > w - 1 ? w - 1 : i);
}

template <typename R> inline R len3(R x, R y, R z) {
    R s = R(0);  /* lengthSq accumulates from 0 in component order */
    s += x * x;
    s += y * y;
    s += z * z;
    return std::sqrt(s);
}

/* tgt::normalize: v * (1 / length(v)). A zero vector maps to zero (GLSL's
 * normalize(0) is undefined; both oracle and kernel pick 0). */
template <typename R> inline V3<R> normalize3(V3<R> v) {
    const R l = len3(v.x, v.y, v.z);
    if (l == R(0)) return v3<R>(0, 0, 0);
    const R r = R(1) / l;
    return v3<R>(v.x * r, v.y * r, v.z * r);
}

template <typename R> inline R dot3(V3<R> a, V3<R> b) {
    R s = R(0);
    s += a.x * b.x;
    s += a.y * b.y;
    s += a.z * b.z;
    return s;
}

template <typename R> inline R rpow(R b, R e);
template <> inline float rpow<float>(float b, float e) { return std::pow(b, e); }
template <> inline double rpow<double>(double b, double e) { return std::pow(b, e); }

template <typename R> struct Ctx {
    const OrcVolume* vol;
    const OrcTF* tf;
    const OrcParams* p;
    const float* entry;
    int W, H;
    R step;
    R dimf[3];
    R offs[3];        /* datasetDimensionsRCP_ */
    R spacing_rcp[3]; /* datasetSpacingRCP_ */
};

/* calcGradientA (mod_gradients.frag:202-214): six lookups at +-1/dim in
 * texture space, v(-) - v(+), times spacingRCP * 0.5 * rwmScale. Lookups use
 * the same clamped trilinear as the intensity sample (the GL texture with
 * clamp-to-edge wrapping computes the same function). */
template <typename R> V3<R> calc_gradient(const Ctx<R>& c, R sx, R sy, R sz) {
    const OrcVolume* v = c.vol;
    const R v0 = sample_tex<R>(v, sx + c.offs[0], sy, sz);
    const R v1 = sample_tex<R>(v, sx, sy + c.offs[1], sz);
    const R v2 = sample_tex<R>(v, sx, sy, sz + c.offs[2]);
    const R v3_ = sample_tex<R>(v, sx - c.offs[0], sy, sz);
    const R v4 = sample_tex<R>(v, sx, sy - c.offs[1], sz);
    const R v5 = sample_tex<R>(v, sx, sy, sz - c.offs[2]);
    V3<R> g = v3<R>(v3_ - v0, v4 - v1, v5 - v2);
    g.x = g.x * (c.spacing_rcp[0] * R(0.5));
    g.y = g.y * (c.spacing_rcp[1] * R(0.5));
    g.z = g.z * (c.spacing_rcp[2] * R(0.5));
    const R s = R(c.vol->rwm_scale);
    return v3<R>(g.x * s, g.y * s, g.z * s);
}

/* Entry point of pixel (x, y), clamped to the image like a clamp-to-edge
 * texture lookup. */
template <typename R> V3<R> entry_at(const Ctx<R>& c, int x, int y) {
    x = std::min(std::max(x, 0), c.W - 1);
    y = std::min(std::max(y, 0), c.H - 1);
    const float* e = c.entry + 4 * (size_t(y) * c.W + x);
    return v3<R>(R(e[0]), R(e[1]), R(e[2]));
}

/* fixClipBorderGradient (mod_gradients.frag:39-46). */
template <typename R> V3<R> clip_border_gradient(const Ctx<R>& c, V3<R> s, V3<R> dir, int px, int py) {
    const V3<R> a = entry_at(c, px + 2, py), b = entry_at(c, px, py + 2);
    const V3<R> v0 = normalize3(v3<R>(a.x - s.x, a.y - s.y, a.z - s.z));
    const V3<R> v1 = normalize3(v3<R>(b.x - s.x, b.y - s.y, b.z - s.z));
    V3<R> g = v3<R>(v0.y * v1.z - v0.z * v1.y, v0.z * v1.x - v0.x * v1.z, v0.x * v1.y - v0.y * v1.x);
    /* faceforward(N, I, Nref) = dot(Nref, I) < 0 ? N : -N */
    if (!(dot3(g, dir) < R(0))) g = v3<R>(-g.x, -g.y, -g.z);
    return g;
}

/* phongShading (mod_shading.frag:134-151) with ka = kd = TF colour and
 * ks = (1,1,1) as rc_singlevolume.frag:234 passes them. */
template <typename R> V3<R> phong(const Ctx<R>& c, V3<R> n, V3<R> pos, V3<R> col) {
    const OrcParams* p = c.p;
    const V3<R> N = normalize3(n);
    V3<R> L = v3<R>(R(p->light_pos_phys[0]) - pos.x, R(p->light_pos_phys[1]) - pos.y, R(p->light_pos_phys[2]) - pos.z);
    const V3<R> V = normalize3(v3<R>(R(p->camera_pos_phys[0]) - pos.x, R(p->camera_pos_phys[1]) - pos.y,
                                     R(p->camera_pos_phys[2]) - pos.z));
    const R d = len3(L.x, L.y, L.z);
    L = v3<R>(L.x / d, L.y / d, L.z / d);
    /* ambient */
    V3<R> out = v3<R>(col.x * R(p->light_ambient[0]), col.y * R(p->light_ambient[1]), col.z * R(p->light_ambient[2]));
    /* diffuse */
    R ndl = dot3(N, L);
    ndl = ndl > R(0) ? ndl : R(0);
    out.x += col.x * R(p->light_diffuse[0]) * ndl;
    out.y += col.y * R(p->light_diffuse[1]) * ndl;
    out.z += col.z * R(p->light_diffuse[2]) * ndl;
    /* specular, Blinn half vector */
    const V3<R> Hh = normalize3(v3<R>(V.x + L.x, V.y + L.y, V.z + L.z));
    R ndh = dot3(N, Hh);
    ndh = ndh > R(0) ? ndh : R(0);
    const R spec = rpow<R>(ndh, R(p->shininess));
    out.x += R(p->light_specular[0]) * spec;
    out.y += R(p->light_specular[1]) * spec;
    out.z += R(p->light_specular[2]) * spec;
    if (p->apply_attenuation) {
        R att = R(1) / (R(p->attenuation[0]) + R(p->attenuation[1]) * d + R(p->attenuation[2]) * d * d);
        att = att < R(1) ? att : R(1);
        out = v3<R>(out.x * att, out.y * att, out.z * att);
    }
    return out;
}

/* Decision signature of a ray: a hash of (loop index, TF entry) over the
 * samples whose TF entry has alpha > 0 (for pre-integration, the table
 * entry (front, back)). Two evaluations of a ray that pick the same entries
 * at the same samples have the same signature; test infrastructure uses it
 * to tell rounding differences from different discrete decisions. */
inline uint32_t sig_mix(uint32_t h, uint32_t loop, uint32_t entry) {
    h ^= loop * 0x9E3779B1u + entry * 0x85EBCA77u + 0x27D4EB2Fu;
    h *= 0x01000193u;
    return h ^ (h >> 15);
}

/* One ray. Returns the loop iteration count. */
template <typename R>
int march_ray(const Ctx<R>& c, V3<R> first, V3<R> last, int px, int py, R out[4], R* first_hit, uint32_t* sig_out) {
    const OrcParams* p = c.p;
    const OrcVolume* v = c.vol;
    const OrcTF* tf = c.tf;
    const R step = c.step;
    R tend;
    R t = R(0);
    V3<R> dir = v3<R>(last.x - first.x, last.y - first.y, last.z - first.z);
    const bool dir0 = dir.x == R(0) && dir.y == R(0) && dir.z == R(0);
    const bool last0 = last.x == R(0) && last.y == R(0) && last.z == R(0);
    const bool first0 = first.x == R(0) && first.y == R(0) && first.z == R(0);
    if (dir0 && !last0 && !first0) {
        tend = step / R(2);  /* cpuraycaster.cpp:226-227 */
    } else {
        tend = len3(dir.x, dir.y, dir.z);
        const R rl = R(1) / tend;
        dir = v3<R>(dir.x * rl, dir.y * rl, dir.z * rl);
    }
    const R ert = R(p->ert_threshold);
    const int comp = p->compositing;
    /* no early ray termination for mip / mop / mida (volumeraycaster.cpp:226-228) */
    const bool use_ert = comp != ORC_MIP && comp != ORC_MOP && comp != ORC_MIDA;
    const bool preint = p->preint != nullptr;
    const int pres = p->preint_res;
    R last_int = R(0);  /* lastIntensity, cpuraycaster.cpp:235 */
    const R lo = R(tf->domain_lo), hi = R(tf->domain_hi);
    const R rs = R(v->rwm_scale), ro = R(v->rwm_offset);
    const R kcorr = step * R(200);  /* SAMPLING_BASE_INTERVAL_RCP */
    R res[4] = {0, 0, 0, 0};
    R depth_t = R(-1);
    R max_int = R(0);
    uint32_t sig = 0x811C9DC5u;
    bool finished = false;
    int loop = 0;
    for (loop = 0; !finished && loop < 255 * 255; ++loop) {
        const V3<R> s = v3<R>(first.x + t * dir.x, first.y + t * dir.y, first.z + t * dir.z);
        const R intensity = sample_tex<R>(v, s.x, s.y, s.z);
        const R rw = intensity * rs + ro;
        R col[4];
        if (preint) {
            /* PreIntegrationTable::classify(last, cur) (preintegrationtable.cpp:256-279) */
            const R cur = rw_to_tf<R>(rw, lo, hi);
            const int i1 = tf_index<R>(last_int, pres), i2 = tf_index<R>(cur, pres);
            const float* e = p->preint + 4 * (size_t(i2) * size_t(pres) + size_t(i1));
            for (int k = 0; k < 4; ++k) col[k] = R(e[k]);
            last_int = cur;
            if (e[3] > 0.f) sig = sig_mix(sig, uint32_t(loop), uint32_t(i2) * uint32_t(pres) + uint32_t(i1));
        } else {
            const int idx = tf_index<R>(rw_to_tf<R>(rw, lo, hi), tf->width);
            const uint8_t* e = tf->rgba + 4 * idx;
            for (int k = 0; k < 4; ++k) col[k] = R(e[k]) / R(255);
            if (e[3] > 0) sig = sig_mix(sig, uint32_t(loop), uint32_t(idx));
        }
        if (col[3] > R(0)) {
            V3<R> g = v3<R>(0, 0, 0);
            if (p->shading == ORC_SHADE_PHONG || comp == ORC_FHN)
                g = (t == R(0)) ? clip_border_gradient<R>(c, s, dir, px, py) : calc_gradient<R>(c, s.x, s.y, s.z);
            if (p->shading == ORC_SHADE_PHONG) {
                /* texToPhysical (mod_sampler3d.frag:179-181) */
                const V3<R> pos = v3<R>((s.x * c.dimf[0] - R(0.5)) * R(v->spacing[0]) + R(v->offset[0]),
                                        (s.y * c.dimf[1] - R(0.5)) * R(v->spacing[1]) + R(v->offset[1]),
                                        (s.z * c.dimf[2] - R(0.5)) * R(v->spacing[2]) + R(v->offset[2]));
                const V3<R> sh = phong<R>(c, g, pos, v3<R>(col[0], col[1], col[2]));
                col[0] = sh.x; col[1] = sh.y; col[2] = sh.z;
            }
            if (comp == ORC_DVR) {
                /* opacity correction (none for a pre-integrated colour), then
                 * front-to-back (cpuraycaster.cpp:291-303) */
                if (!preint) col[3] = R(1) - rpow<R>(R(1) - col[3], kcorr);
                if (col[3] > R(0)) {
                    const R w = (R(1) - res[3]) * col[3];
                    res[0] = res[0] + w * col[0];
                    res[1] = res[1] + w * col[1];
                    res[2] = res[2] + w * col[2];
                    res[3] = res[3] + (R(1) - res[3]) * col[3];
                }
                if (depth_t < R(0) && res[3] > R(0)) depth_t = t;
            } else if (comp == ORC_MIP) {
                if (rw > max_int) {
                    res[0] = col[0]; res[1] = col[1]; res[2] = col[2]; res[3] = col[3];
                    max_int = rw;
                    depth_t = t;
                }
            } else if (comp == ORC_ISO) {
                const R iso = R(p->iso_value), eps = R(0.02);
                if (col[3] >= iso - eps && col[3] <= iso + eps) {
                    res[0] = col[0]; res[1] = col[1]; res[2] = col[2]; res[3] = R(1);
                    depth_t = t;
                }
            } else if (comp == ORC_MOP) {
                /* compositeMOP (mod_compositing.frag:97-107) */
                if (col[3] > res[3]) {
                    res[0] = col[0]; res[1] = col[1]; res[2] = col[2]; res[3] = col[3];
                    depth_t = t;
                }
            } else if (comp == ORC_MIDA) {
                /* compositeMIDA / compositeMIDAhelper (mod_compositing.frag:109-146).
                 * As there, the helper never raises maxIntensity: with gamma <= 0
                 * it stays at its initial 0, with gamma > 0 only the MIP half
                 * raises it (before the helper reads it). */
                col[3] = R(1) - rpow<R>(R(1) - col[3], kcorr);
                const R gamma = R(p->mida_gamma);
                auto helper = [&](const R* in, R maxi, R gm, R* o) {
                    R delta = R(0);
                    if (rw > maxi) delta = rw - maxi;
                    const R beta = R(1) - delta * (R(1) + gm);
                    for (int k = 0; k < 3; ++k) o[k] = beta * in[k] + (R(1) - beta * in[3]) * col[3] * col[k];
                    o[3] = beta * in[3] + (R(1) - beta * in[3]) * col[3];
                };
                if (gamma <= R(0)) {
                    R o[4];
                    helper(res, max_int, gamma, o);
                    for (int k = 0; k < 4; ++k) res[k] = o[k];
                } else {
                    R mip[4] = {res[0], res[1], res[2], res[3]};
                    if (rw > max_int) {
                        for (int k = 0; k < 4; ++k) mip[k] = col[k];
                        max_int = rw;
                        depth_t = t;
                    }
                    R mida[4];
                    helper(res, max_int, R(0), mida);
                    for (int k = 0; k < 4; ++k) res[k] = gamma * mip[k] + (R(1) - gamma) * mida[k];
                }
                if (depth_t < R(0)) depth_t = t;
            } else if (comp == ORC_FHP) {
                /* compositeFHP (mod_compositing.frag:168-181): texture-space position */
                if (res[0] == R(0) && res[1] == R(0) && res[2] == R(0)) {
                    res[0] = s.x; res[1] = s.y; res[2] = s.z; res[3] = R(1);
                    if (depth_t < R(0)) depth_t = t;
                }
            } else if (comp == ORC_FHN) {
                /* compositeFHN (mod_compositing.frag:183-196): normalize(gradient)/2 + 0.5;
                 * a zero gradient (undefined in GLSL) gives 0.5 */
                if (res[0] == R(0) && res[1] == R(0) && res[2] == R(0)) {
                    const V3<R> n = normalize3(g);
                    res[0] = n.x / R(2) + R(0.5); res[1] = n.y / R(2) + R(0.5); res[2] = n.z / R(2) + R(0.5);
                    res[3] = R(1);
                    if (depth_t < R(0)) depth_t = t;
                }
            }
        }
        if (use_ert && res[3] >= ert) {
            res[3] = R(1);
            finished = true;
        }
        t += step;
        finished = finished || (t > tend);
    }
    out[0] = res[0]; out[1] = res[1]; out[2] = res[2]; out[3] = res[3];
    if (first_hit) *first_hit = depth_t;
    if (sig_out) *sig_out = sig;
    return loop;
}

template <typename R>
void render(const OrcVolume* vol, const OrcTF* tf, const OrcParams* p, const float* entry, const float* exitp,
            int W, int H, int row_begin, int row_end, int nthreads, R* out, int32_t* samples, R* first_hit,
            uint32_t* sig) {
    Ctx<R> c;
    c.vol = vol; c.tf = tf; c.p = p; c.entry = entry; c.W = W; c.H = H;
    const int maxdim = std::max(vol->dims[0], std::max(vol->dims[1], vol->dims[2]));
    /* samplingStepSize = 1 / (max(dim) * samplingRate) (cpuraycaster.cpp:104) */
    c.step = R(1) / (R(maxdim) * R(p->sampling_rate));
    for (int i = 0; i < 3; ++i) {
        c.dimf[i] = R(vol->dims[i]);
        c.offs[i] = R(1) / R(vol->dims[i]);
        c.spacing_rcp[i] = R(1) / R(vol->spacing[i]);
    }
    row_begin = std::max(0, row_begin);
    row_end = std::min(H, row_end);
#ifdef _OPENMP
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
#endif
    /* Row loop with a parallel loop over x, schedule(dynamic), as
     * cpuraycaster.cpp:173-193 does. */
    for (int y = row_begin; y < row_end; ++y) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(nt)
#endif
        for (int x = 0; x < W; ++x) {
            const size_t pix = size_t(y) * W + x;
            const float* f = entry + 4 * pix;
            const float* l = exitp + 4 * pix;
            R res[4] = {0, 0, 0, 0};
            R fh = R(-1);
            uint32_t sg = 0;
            int n = 0;
            const bool bg = f[0] == 0.f && f[1] == 0.f && f[2] == 0.f && f[3] == 0.f &&
                            l[0] == 0.f && l[1] == 0.f && l[2] == 0.f && l[3] == 0.f;
            if (!bg) {
                n = march_ray<R>(c, v3<R>(R(f[0]), R(f[1]), R(f[2])), v3<R>(R(l[0]), R(l[1]), R(l[2])), x, y, res, &fh,
                                 &sg);
            }
            for (int k = 0; k < 4; ++k) out[4 * pix + k] = res[k];
            if (samples) samples[pix] = n;
            if (first_hit) first_hit[pix] = fh;
            if (sig) sig[pix] = sg;
        }
    }
}

}  // namespace

extern "C" {

void oracle_bake_tf_keys(const OrcTFKey* keys, int nkeys, int width, float gamma, float threshold_lo,
                         float threshold_hi, uint8_t* out) {
    /* TransFunc1D::createTextureData (transfunc1d.cpp:85-116) */
    const int front_end = static_cast<int>(std::floor(threshold_lo * float(width) + 0.5f));
    const int back_start = static_cast<int>(std::floor(threshold_hi * float(width) + 0.5f));
    for (int x = 0; x < width; ++x) {
        uint8_t* o = out + 4 * x;
        if (x < front_end || x > back_start || nkeys == 0) {
            o[0] = o[1] = o[2] = o[3] = 0;
            continue;
        }
        float value = static_cast<float>(x) / float(width - 1);
        if (gamma != 1.f) value = std::pow(value, gamma);
        /* TransFunc1DKeys::getMappingForValueUByte (transfunc1dkeys.cpp:119-154) */
        value = value < 0.f ? 0.f : value;
        value = value > 1.f ? 1.f : value;
        int k = 0;
        while (k < nkeys && value > keys[k].intensity) ++k;
        if (k == 0) {
            std::memcpy(o, keys[0].color_l, 4);
        } else if (k == nkeys) {
            std::memcpy(o, keys[nkeys - 1].color_r, 4);
        } else {
            const OrcTFKey& L = keys[k - 1];
            const OrcTFKey& Rk = keys[k];
            const float fraction = (value - L.intensity) / (Rk.intensity - L.intensity);
            for (int ch = 0; ch < 4; ++ch) {
                /* uint8 channel += (int diff) * fraction, truncated on store */
                const float diff = float(int(Rk.color_l[ch]) - int(L.color_r[ch]));
                const float sum = float(L.color_r[ch]) + diff * fraction;
                o[ch] = static_cast<uint8_t>(sum);
            }
        }
    }
}

void oracle_preint_source(const OrcTFKey* keys, int nkeys, int res, float gamma, float threshold_lo,
                          float threshold_hi, uint8_t* out) {
    /* PreIntegrationTable::computeTable's TF buffer (preintegrationtable.cpp:71-104):
     * the same key mapping as the texture, sampled at `res` entries, but
     * zeroed from back_start on (the texture keeps entry back_start). */
    const int front_end = static_cast<int>(std::floor(threshold_lo * float(res) + 0.5f));
    const int back_start = static_cast<int>(std::floor(threshold_hi * float(res) + 0.5f));
    oracle_bake_tf_keys(keys, nkeys, res, gamma, 0.f, 1.f, out);
    for (int i = 0; i < res; ++i)
        if (i < front_end || i >= back_start) std::memset(out + 4 * i, 0, 4);
}

void oracle_preint_table(const uint8_t* src, int res, float d, int use_integral, float* out) {
    /* PreIntegrationTable::computeTable (preintegrationtable.cpp:67-204), FP32 */
    struct F4 {
        float r, g, b, a;
    };
    std::vector<F4> tb(res);
    for (int i = 0; i < res; ++i)  /* tgt::vec4(ubyte) / 255.f */
        tb[i] = F4{float(src[4 * i]) / 255.f, float(src[4 * i + 1]) / 255.f, float(src[4 * i + 2]) / 255.f,
                   float(src[4 * i + 3]) / 255.f};
    auto clamp01 = [](float x) { return std::min(std::max(x, 0.f), 1.f); };
    auto store = [&](size_t idx, F4 c) {
        out[4 * idx] = clamp01(c.r);
        out[4 * idx + 1] = clamp01(c.g);
        out[4 * idx + 2] = clamp01(c.b);
        out[4 * idx + 3] = clamp01(c.a);
    };
    const float k200 = d * 200.0f;
    if (!use_integral) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic)
#endif
        for (int sb = 0; sb < res; ++sb) {
            for (int sf = 0; sf < res; ++sf) {
                const size_t idx = size_t(sb) * res + sf;
                if (sb != sf) {
                    const float scale = 1.0f / (std::fabs(static_cast<float>(sb - sf)) + 1);
                    const int incr = sb < sf ? -1 : 1;
                    F4 r{0.f, 0.f, 0.f, 0.f};
                    for (int s = sf; (incr == 1 ? s <= sb : s >= sb) && (r.a < 0.95f); s += incr) {
                        F4 c = tb[s];
                        if (c.a > 0.0f) {
                            c.a = 1.f - std::pow(1.f - c.a, k200 * scale);
                            const float w = (1.0f - r.a) * c.a;
                            const float nr = r.r + w * c.r, ng = r.g + w * c.g, nb = r.b + w * c.b;
                            r.a = r.a + (1.0f - r.a) * c.a;
                            r.r = nr; r.g = ng; r.b = nb;
                        }
                    }
                    const float m = std::max(r.a, 0.001f);
                    r.r /= m; r.g /= m; r.b /= m;
                    store(idx, r);
                } else {
                    F4 r{clamp01(tb[sf].r), clamp01(tb[sf].g), clamp01(tb[sf].b), clamp01(tb[sf].a)};
                    r.a = 1.f - std::pow(1.f - r.a, k200);
                    store(idx, r);
                }
            }
        }
    } else {
        /* integral functions (Real-Time Volume Graphics p. 96) */
        std::vector<F4> I(res);
        F4 acc{0.f, 0.f, 0.f, 0.f};
        for (int i = 0; i < res; ++i) {
            const F4 c = tb[i];
            if (c.a > 0.0f) {
                acc.r += c.r * c.a; acc.g += c.g * c.a; acc.b += c.b * c.a;
                acc.a += c.a;
            }
            I[i] = acc;
        }
        for (int sb = 0; sb < res; ++sb) {
            for (int sf = 0; sf < res; ++sf) {
                const int smin = std::min(sb, sf), smax = std::max(sb, sf);
                F4 col;
                if (smax != smin) {
                    const float factor = k200 / static_cast<float>(smax - smin);
                    col.r = (I[smax].r - I[smin].r) * factor;
                    col.g = (I[smax].g - I[smin].g) * factor;
                    col.b = (I[smax].b - I[smin].b) * factor;
                    col.a = 1.f - std::exp(-(I[smax].a - I[smin].a) * factor);
                    const float m = std::max(col.a, 0.001f);
                    col.r /= m; col.g /= m; col.b /= m;
                } else {
                    col = tb[smin];
                    col.a = 1.f - std::pow(1.f - col.a, k200);
                }
                store(size_t(sb) * res + sf, col);
            }
        }
    }
}

void oracle_entry_exit(const double* m, int W, int H, int quantize16, float* entry, float* exitp) {
    const double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {1.0, 1.0, 1.0};
    oracle_entry_exit_box(m, W, H, quantize16, lo, hi, entry, exitp);
}

void oracle_entry_exit_box(const double* m, int W, int H, int quantize16, const double* box_lo, const double* box_hi,
                           float* entry, float* exitp) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const size_t pix = size_t(y) * W + x;
            const double nx = 2.0 * (x + 0.5) / W - 1.0, ny = 2.0 * (y + 0.5) / H - 1.0;
            double pn[4], pf[4];
            for (int r = 0; r < 4; ++r) {
                pn[r] = m[4 * r + 0] * nx + m[4 * r + 1] * ny + m[4 * r + 2] * -1.0 + m[4 * r + 3];
                pf[r] = m[4 * r + 0] * nx + m[4 * r + 1] * ny + m[4 * r + 2] * 1.0 + m[4 * r + 3];
            }
            double o[3], d[3];
            for (int i = 0; i < 3; ++i) {
                o[i] = pn[i] / pn[3];
                d[i] = pf[i] / pf[3] - o[i];
            }
            /* Slab test against the unit texture cube, segment s in [0,1]
             * between the near and far planes: the front faces clipped by the
             * near plane give the entry, the farthest back faces the exit. */
            double s0 = 0.0, s1 = 1.0;
            bool hit = true;
            for (int i = 0; i < 3 && hit; ++i) {
                if (d[i] == 0.0) {
                    if (o[i] < box_lo[i] || o[i] > box_hi[i]) hit = false;
                } else {
                    double a = (box_lo[i] - o[i]) / d[i], b = (box_hi[i] - o[i]) / d[i];
                    if (a > b) std::swap(a, b);
                    s0 = std::max(s0, a);
                    s1 = std::min(s1, b);
                }
            }
            float* e = entry + 4 * pix;
            float* l = exitp + 4 * pix;
            if (!hit || !(s0 < s1)) {
                for (int k = 0; k < 4; ++k) e[k] = l[k] = 0.f;
                continue;
            }
            for (int i = 0; i < 3; ++i) {
                double a = o[i] + s0 * d[i], b = o[i] + s1 * d[i];
                a = std::min(box_hi[i], std::max(box_lo[i], a));
                b = std::min(box_hi[i], std::max(box_lo[i], b));
                if (quantize16) {
                    a = std::floor(a * 65535.0 + 0.5) / 65535.0;
                    b = std::floor(b * 65535.0 + 0.5) / 65535.0;
                }
                e[i] = float(a);
                l[i] = float(b);
            }
            e[3] = l[3] = 1.f;
        }
    }
}

void oracle_render_f32(const OrcVolume* vol, const OrcTF* tf, const OrcParams* p, const float* entry,
                       const float* exitp, int W, int H, int row_begin, int row_end, int nthreads, float* out,
                       int32_t* samples, float* first_hit, uint32_t* signature) {
    render<float>(vol, tf, p, entry, exitp, W, H, row_begin, row_end, nthreads, out, samples, first_hit, signature);
}

void oracle_render_f64(const OrcVolume* vol, const OrcTF* tf, const OrcParams* p, const float* entry,
                       const float* exitp, int W, int H, int row_begin, int row_end, int nthreads, double* out,
                       int32_t* samples, double* first_hit, uint32_t* signature) {
    render<double>(vol, tf, p, entry, exitp, W, H, row_begin, row_end, nthreads, out, samples, first_hit, signature);
}

void oracle_trilinear_f32(const OrcVolume* vol, const float* pos, int n, float* out) {
    for (int i = 0; i < n; ++i) out[i] = trilinear<float>(vol, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
}

void oracle_brick_minmax(const OrcVolume* vol, int brick, int apron_hi, float* out_min, float* out_max) {
    const int X = vol->dims[0], Y = vol->dims[1], Z = vol->dims[2];
    const int nbx = (X + brick - 1) / brick, nby = (Y + brick - 1) / brick, nbz = (Z + brick - 1) / brick;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (int bz = 0; bz < nbz; ++bz)
        for (int by = 0; by < nby; ++by)
            for (int bx = 0; bx < nbx; ++bx) {
                float mn = INFINITY, mx = -INFINITY;
                for (int z = bz * brick; z < std::min(Z, (bz + 1) * brick + apron_hi); ++z)
                    for (int y = by * brick; y < std::min(Y, (by + 1) * brick + apron_hi); ++y)
                        for (int x = bx * brick; x < std::min(X, (bx + 1) * brick + apron_hi); ++x) {
                            const float f = norm_voxel<float>(vol, size_t(z) * X * Y + size_t(y) * X + x);
                            mn = std::min(mn, f);
                            mx = std::max(mx, f);
                        }
                const size_t b = (size_t(bz) * nby + by) * nbx + bx;
                out_min[b] = mn;
                out_max[b] = mx;
            }
}

}  // extern "C"
