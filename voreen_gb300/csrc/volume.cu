// Volume ingest: linear VolumeRAM layout -> bricked device layout, per-brick
// min/max, and the per-(volume, TF) brick occupancy used for empty-space
// skipping.
//
// Reference behaviour this replaces / follows:
//   VolumeGL upload (linear 3D texture)       src/core/datastructures/volume/volumegl.cpp:126-168
//   per-region min/max with 1-voxel overlap   modules/base/processors/proxygeometry/optimizedproxygeometry.cpp:894-987
//   region emptiness from TF opacity          optimizedproxygeometry.cpp:878-880
// The brick test here is exact for the march: a brick is empty when every TF
// entry its trilinear samples can select has alpha 0.
#include <cstdint>

#include "vrc_internal.h"

namespace vrc {
namespace {

template <typename T>
__global__ void brick_build_kernel(const T* __restrict__ lin, BrickLayout L, T* __restrict__ bricks) {
    const long long S3 = (long long)L.S * L.S * L.S;
    const long long total = L.nbricks() * S3;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long b = i / S3;
        const int r = (int)(i - b * S3);
        const int lx = r % L.S, ly = (r / L.S) % L.S, lz = r / (L.S * L.S);
        const int bx = (int)(b % L.nb[0]);
        const int by = (int)((b / L.nb[0]) % L.nb[1]);
        const int bz = (int)(b / ((long long)L.nb[0] * L.nb[1]));
        int gx = bx * L.B + lx - APRON_LO, gy = by * L.B + ly - APRON_LO, gz = bz * L.B + lz - APRON_LO;
        gx = min(max(gx, 0), L.dims[0] - 1);
        gy = min(max(gy, 0), L.dims[1] - 1);
        gz = min(max(gz, 0), L.dims[2] - 1);
        bricks[b * L.brick_stride + r] = lin[((long long)gz * L.dims[1] + gy) * L.dims[0] + gx];
    }
}

template <typename T> __device__ __forceinline__ float raw_to_float(T v) { return (float)v; }

// Voxel (x, y, z) of a bricked volume (core voxels, no apron lookup needed).
template <typename T>
__device__ __forceinline__ T brick_voxel(const T* __restrict__ bricks, const BrickLayout& L, int x, int y, int z) {
    const int bx = x >> L.shift, by = y >> L.shift, bz = z >> L.shift;
    const long long b = ((long long)bz * L.nb[1] + by) * L.nb[0] + bx;
    return bricks[b * L.brick_stride +
                  ((z - (bz << L.shift) + APRON_LO) * L.S + (y - (by << L.shift) + APRON_LO)) * L.S +
                  (x - (bx << L.shift) + APRON_LO)];
}

// HalfSampleMean (volumeoctree.cpp:188-202) on the stored type: integers
// summed exactly, divided by 8 with truncation; floats summed in z, y, x
// order and scaled by 1/8.
template <typename T> struct HalfSum { using A = uint32_t; };
template <> struct HalfSum<float> { using A = float; };
template <typename T> __device__ __forceinline__ T half_mean(typename HalfSum<T>::A s) { return (T)(s / 8u); }
template <> __device__ __forceinline__ float half_mean<float>(float s) { return __fmul_rn(s, 0.125f); }

template <typename T>
__global__ void half_sample_kernel(const T* __restrict__ bricks, BrickLayout L, int d1x, int d1y, int d1z,
                                   T* __restrict__ out) {
    const long long total = (long long)d1x * d1y * d1z;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int x1 = (int)(i % d1x), y1 = (int)((i / d1x) % d1y), z1 = (int)(i / ((long long)d1x * d1y));
        typename HalfSum<T>::A sum = 0;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    const int x = min(2 * x1 + dx, L.dims[0] - 1), y = min(2 * y1 + dy, L.dims[1] - 1),
                              z = min(2 * z1 + dz, L.dims[2] - 1);
                    sum += (typename HalfSum<T>::A)brick_voxel(bricks, L, x, y, z);
                }
        out[i] = half_mean<T>(sum);
    }
}

// One CTA per brick: min/max of the stored values over local [APRON_LO,
// APRON_LO + B] on each axis (core + one voxel on the high side), i.e. the
// voxels any trilinear stencil whose floor lies in the brick can touch.
template <typename T>
__global__ void brick_minmax_kernel(const T* __restrict__ bricks, BrickLayout L, float norm, float* bmin,
                                    float* bmax) {
    const long long b = blockIdx.x;
    const T* base = bricks + b * L.brick_stride;
    const int E = L.B + 1;
    float mn = INFINITY, mx = -INFINITY;
    for (int i = threadIdx.x; i < E * E * E; i += blockDim.x) {
        const int x = i % E + APRON_LO, y = (i / E) % E + APRON_LO, z = i / (E * E) + APRON_LO;
        const float v = raw_to_float(base[(z * L.S + y) * L.S + x]);
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
    }
    __shared__ float smn[32], smx[32];
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { smn[w] = mn; smx[w] = mx; }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        mn = lane < nw ? smn[lane] : INFINITY;
        mx = lane < nw ? smx[lane] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (lane == 0) {
            // getTypeAsFloat: value / rangeMax, correctly rounded (monotone)
            bmin[b] = norm > 0.f ? __fdiv_rn(mn, norm) : mn;
            bmax[b] = norm > 0.f ? __fdiv_rn(mx, norm) : mx;
        }
    }
}

// One thread per cell: min/max over the cell's voxels plus one voxel on the
// high side of every axis (clamped), i.e. the trilinear support of all
// samples whose floor voxel lies in the cell.
template <typename T>
__global__ void cell_minmax_kernel(const T* __restrict__ lin, int X, int Y, int Z, int C, int ncx, int ncy,
                                   long long ncells, float norm, float* cmin, float* cmax) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncells;
         c += (long long)gridDim.x * blockDim.x) {
        const int cx = (int)(c % ncx), cy = (int)((c / ncx) % ncy), cz = (int)(c / ((long long)ncx * ncy));
        const int x0 = cx * C, y0 = cy * C, z0 = cz * C;
        const int x1 = min(x0 + C, X - 1), y1 = min(y0 + C, Y - 1), z1 = min(z0 + C, Z - 1);
        float mn = INFINITY, mx = -INFINITY;
        for (int z = z0; z <= z1; ++z)
            for (int y = y0; y <= y1; ++y) {
                const T* row = lin + ((long long)z * Y + y) * X;
                for (int x = x0; x <= x1; ++x) {
                    const float v = raw_to_float(row[x]);
                    mn = fminf(mn, v);
                    mx = fmaxf(mx, v);
                }
            }
        cmin[c] = norm > 0.f ? __fdiv_rn(mn, norm) : mn;
        cmax[c] = norm > 0.f ? __fdiv_rn(mx, norm) : mx;
    }
}

__device__ __forceinline__ float rw_to_tf(float rw, float lo, float hi) {
    if (rw < lo) return 0.f;
    if (rw > hi) return 1.f;
    if (lo == hi) return 0.f;
    return __fdiv_rn(__fsub_rn(rw, lo), __fsub_rn(hi, lo));
}

__device__ __forceinline__ int tf_index(float x, int w) {
    const float f = __fmul_rn(x, (float)(w - 1));
    int i = (int)floorf(__fadd_rn(f, 0.5f));
    return i < 0 ? 0 : (i > w - 1 ? w - 1 : i);
}

// Bit c of the map is set if any TF entry with index in
// [idx(min_c) - 1, idx(max_c) + 1] has alpha > 0 (alpha_prefix[i] = number of
// entries below i with alpha > 0). One thread per 32-cell word.
__global__ void occupancy_kernel(const float* bmin, const float* bmax, long long n, const int* prefix, int w,
                                 float rs, float ro, float lo, float hi, uint32_t* occ) {
    const long long nwords = (n + 31) / 32;
    for (long long wd = blockIdx.x * (long long)blockDim.x + threadIdx.x; wd < nwords;
         wd += (long long)gridDim.x * blockDim.x) {
        uint32_t bits = 0;
        for (int k = 0; k < 32; ++k) {
            const long long b = wd * 32 + k;
            if (b >= n) break;
            const float r0 = __fadd_rn(__fmul_rn(bmin[b], rs), ro);
            const float r1 = __fadd_rn(__fmul_rn(bmax[b], rs), ro);
            int i0 = tf_index(rw_to_tf(fminf(r0, r1), lo, hi), w);
            int i1 = tf_index(rw_to_tf(fmaxf(r0, r1), lo, hi), w);
            i0 = max(i0 - 1, 0);
            i1 = min(i1 + 1, w - 1);
            if (prefix[i1 + 1] - prefix[i0] > 0) bits |= 1u << k;
        }
        occ[wd] = bits;
    }
}

// Chebyshev distance to the nearest occupied cell, capped at OCC_DIST_CAP:
// d(c) = min over occupied o of max(|cx-ox|, |cy-oy|, |cz-oz|). The max of
// the axis offsets composes per axis, so three passes give it exactly:
// along x the distance to the nearest occupied cell of the row, then along
// y and along z the min over offsets k of max(|k|, previous pass at c + k).
// Offsets beyond the cap only give values above it, so each pass looks at
// |k| < OCC_DIST_CAP. One thread per cell; consecutive threads take
// consecutive x, so every pass reads coalesced.
__global__ void occ_dist_x_kernel(const uint32_t* __restrict__ occ, int nx, int ny, int nz, uint8_t* __restrict__ out) {
    const long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(c % nx);
        const long long row = c - x;
        int d = OCC_DIST_CAP;
        for (int k = 0; k < OCC_DIST_CAP && k < d; ++k) {
            const int xa = x - k, xb = x + k;
            if (xa >= 0) {
                const long long i = row + xa;
                if ((__ldg(occ + (i >> 5)) >> (i & 31)) & 1u) d = k;
            }
            if (xb < nx && d > k) {
                const long long i = row + xb;
                if ((__ldg(occ + (i >> 5)) >> (i & 31)) & 1u) d = k;
            }
        }
        out[c] = (uint8_t)d;
    }
}

__global__ void occ_dist_axis_kernel(const uint8_t* __restrict__ in, int nx, int ny, int nz, int axis,
                                     uint8_t* __restrict__ out) {
    const long long n = (long long)nx * ny * nz;
    const long long stride = axis == 1 ? nx : (long long)nx * ny;
    const int len = axis == 1 ? ny : nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const int pos = axis == 1 ? (int)((c / nx) % ny) : (int)(c / ((long long)nx * ny));
        int d = __ldg(in + c);
        for (int k = 1; k < d; ++k) {
            if (pos - k >= 0) d = min(d, max(k, (int)__ldg(in + c - k * stride)));
            if (pos + k < len) d = min(d, max(k, (int)__ldg(in + c + k * stride)));
        }
        out[c] = (uint8_t)d;
    }
}

int grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    if (g > 152LL * 64) g = 152LL * 64;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

// One CTA per cached brick: 16-byte copies from the (host-resident) pool.
// One CTA per cached brick; four 16-byte loads in flight per thread, since
// the source is host memory read over the C2C link.
__global__ void brick_gather_kernel(const uint4* __restrict__ pool, const long long* __restrict__ ids,
                                    const long long* __restrict__ slots, long long words, uint4* __restrict__ cache) {
    const uint4* src = pool + ids[blockIdx.x] * words;
    uint4* dst = cache + slots[blockIdx.x] * words;
    long long i = threadIdx.x;
    for (; i + 3 * blockDim.x < words; i += 4 * blockDim.x) {
        const uint4 a = src[i], b = src[i + blockDim.x], c = src[i + 2 * blockDim.x], d = src[i + 3 * blockDim.x];
        dst[i] = a;
        dst[i + blockDim.x] = b;
        dst[i + 2 * blockDim.x] = c;
        dst[i + 3 * blockDim.x] = d;
    }
    for (; i < words; i += blockDim.x) dst[i] = src[i];
}

cudaError_t launch_brick_gather(const void* pool, const long long* ids, const long long* dst, long long n,
                                size_t brick_stride_bytes, void* cache, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (n > 0x7fffffffLL || brick_stride_bytes % 16) return cudaErrorInvalidValue;
    brick_gather_kernel<<<(unsigned)n, 256, 0, s>>>(static_cast<const uint4*>(pool), ids, dst,
                                                    (long long)(brick_stride_bytes / 16), static_cast<uint4*>(cache));
    return cudaGetLastError();
}

cudaError_t launch_brick_build(const void* linear, int dtype, const BrickLayout& L, void* bricks, cudaStream_t s) {
    const long long total = L.nbricks() * (long long)L.S * L.S * L.S;
    const int g = grid_for(total, 256);
    switch (dtype) {
        case VRC_U8:
            brick_build_kernel<uint8_t><<<g, 256, 0, s>>>((const uint8_t*)linear, L, (uint8_t*)bricks);
            break;
        case VRC_U16:
            brick_build_kernel<uint16_t><<<g, 256, 0, s>>>((const uint16_t*)linear, L, (uint16_t*)bricks);
            break;
        default:
            brick_build_kernel<float><<<g, 256, 0, s>>>((const float*)linear, L, (float*)bricks);
            break;
    }
    return cudaGetLastError();
}

cudaError_t launch_half_sample(const void* bricks, int dtype, const BrickLayout& L, const int dims1[3], void* out,
                               cudaStream_t s) {
    const long long total = (long long)dims1[0] * dims1[1] * dims1[2];
    const int g = grid_for(total, 256);
    switch (dtype) {
        case VRC_U8:
            half_sample_kernel<uint8_t><<<g, 256, 0, s>>>((const uint8_t*)bricks, L, dims1[0], dims1[1], dims1[2],
                                                          (uint8_t*)out);
            break;
        case VRC_U16:
            half_sample_kernel<uint16_t><<<g, 256, 0, s>>>((const uint16_t*)bricks, L, dims1[0], dims1[1], dims1[2],
                                                           (uint16_t*)out);
            break;
        default:
            half_sample_kernel<float><<<g, 256, 0, s>>>((const float*)bricks, L, dims1[0], dims1[1], dims1[2],
                                                        (float*)out);
            break;
    }
    return cudaGetLastError();
}

cudaError_t launch_brick_minmax(const void* bricks, int dtype, const BrickLayout& L, float* bmin, float* bmax,
                                cudaStream_t s) {
    const long long n = L.nbricks();
    if (n > 0x7fffffffLL) return cudaErrorInvalidValue;
    switch (dtype) {
        case VRC_U8:
            brick_minmax_kernel<uint8_t><<<(unsigned)n, 256, 0, s>>>((const uint8_t*)bricks, L, 255.f, bmin, bmax);
            break;
        case VRC_U16:
            brick_minmax_kernel<uint16_t><<<(unsigned)n, 256, 0, s>>>((const uint16_t*)bricks, L, 65535.f, bmin,
                                                                      bmax);
            break;
        default:
            brick_minmax_kernel<float><<<(unsigned)n, 256, 0, s>>>((const float*)bricks, L, 0.f, bmin, bmax);
            break;
    }
    return cudaGetLastError();
}

cudaError_t launch_cell_minmax(const void* linear, int dtype, const int d[3], int C, float* cmin, float* cmax,
                               cudaStream_t s) {
    const int ncx = (d[0] + C - 1) / C, ncy = (d[1] + C - 1) / C, ncz = (d[2] + C - 1) / C;
    const long long n = (long long)ncx * ncy * ncz;
    const int g = grid_for(n, 128);
    switch (dtype) {
        case VRC_U8:
            cell_minmax_kernel<uint8_t><<<g, 128, 0, s>>>((const uint8_t*)linear, d[0], d[1], d[2], C, ncx, ncy, n,
                                                          255.f, cmin, cmax);
            break;
        case VRC_U16:
            cell_minmax_kernel<uint16_t><<<g, 128, 0, s>>>((const uint16_t*)linear, d[0], d[1], d[2], C, ncx, ncy, n,
                                                           65535.f, cmin, cmax);
            break;
        default:
            cell_minmax_kernel<float><<<g, 128, 0, s>>>((const float*)linear, d[0], d[1], d[2], C, ncx, ncy, n, 0.f,
                                                        cmin, cmax);
            break;
    }
    return cudaGetLastError();
}

cudaError_t launch_occupancy(const float* bmin, const float* bmax, long long ncells, const int* alpha_prefix,
                             int tf_width, float rwm_scale, float rwm_offset, float tf_lo, float tf_hi,
                             uint32_t* occ, cudaStream_t s) {
    occupancy_kernel<<<grid_for((ncells + 31) / 32, 128), 128, 0, s>>>(bmin, bmax, ncells, alpha_prefix, tf_width,
                                                                       rwm_scale, rwm_offset, tf_lo, tf_hi, occ);
    return cudaGetLastError();
}

cudaError_t launch_occ_distance(const uint32_t* occ, const int nc[3], uint8_t* dist, uint8_t* tmp, cudaStream_t s) {
    const long long n = (long long)nc[0] * nc[1] * nc[2];
    const int g = grid_for(n, 256);
    occ_dist_x_kernel<<<g, 256, 0, s>>>(occ, nc[0], nc[1], nc[2], dist);
    occ_dist_axis_kernel<<<g, 256, 0, s>>>(dist, nc[0], nc[1], nc[2], 1, tmp);
    occ_dist_axis_kernel<<<g, 256, 0, s>>>(tmp, nc[0], nc[1], nc[2], 2, dist);
    return cudaGetLastError();
}

}  // namespace vrc
