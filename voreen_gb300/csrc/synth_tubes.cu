// Seeded tube volumes generated on the device (the large sparse workload):
// `ntubes` tubes along Catmull-Rom splines through random control points,
// radius U[2, 20] voxels, intensity U[1500, 4000] (of 4095), on a zero
// background, plus N(0, sigma) noise, clamped to [0, 4095], uint16.
//
// Each tube is cut into capsules (segments with the tube radius); one CTA
// per capsule visits the voxels of the capsule's bounding box and raises the
// voxels inside it to the tube intensity with a 32-bit compare-and-swap max
// on the word holding the voxel (so the result does not depend on order).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstddef>

#include "../../include/vrc_synth.h"

namespace {

__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__host__ __device__ inline double u01(uint64_t seed, uint64_t i) {
    return double(mix64(seed * 0x9E3779B97F4A7C15ULL + i + 1) >> 11) * (1.0 / 9007199254740992.0);
}

struct Capsule {
    float ax, ay, az, bx, by, bz, r;
    unsigned value;
};

__device__ void atomic_max_u16(uint16_t* base, long long idx, unsigned v) {
    unsigned* word = reinterpret_cast<unsigned*>(reinterpret_cast<uintptr_t>(base + idx) & ~uintptr_t(3));
    const unsigned shift = ((reinterpret_cast<uintptr_t>(base + idx) & 2) != 0) ? 16u : 0u;
    unsigned old = *word, assumed;
    do {
        assumed = old;
        const unsigned cur = (assumed >> shift) & 0xffffu;
        if (cur >= v) return;
        const unsigned nw = (assumed & ~(0xffffu << shift)) | (v << shift);
        old = atomicCAS(word, assumed, nw);
    } while (old != assumed);
}

__global__ void capsule_kernel(const Capsule* caps, int X, int Y, int Z, uint16_t* vol) {
    const Capsule c = caps[blockIdx.x];
    const int x0 = max(0, (int)floorf(fminf(c.ax, c.bx) - c.r)), x1 = min(X - 1, (int)ceilf(fmaxf(c.ax, c.bx) + c.r));
    const int y0 = max(0, (int)floorf(fminf(c.ay, c.by) - c.r)), y1 = min(Y - 1, (int)ceilf(fmaxf(c.ay, c.by) + c.r));
    const int z0 = max(0, (int)floorf(fminf(c.az, c.bz) - c.r)), z1 = min(Z - 1, (int)ceilf(fmaxf(c.az, c.bz) + c.r));
    if (x1 < x0 || y1 < y0 || z1 < z0) return;
    const float dx = c.bx - c.ax, dy = c.by - c.ay, dz = c.bz - c.az;
    const float len2 = fmaxf(dx * dx + dy * dy + dz * dz, 1e-12f);
    const long long nx = x1 - x0 + 1, ny = y1 - y0 + 1, nz = z1 - z0 + 1;
    const long long n = nx * ny * nz;
    const float r2 = c.r * c.r;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const int x = x0 + (int)(i % nx), y = y0 + (int)((i / nx) % ny), z = z0 + (int)(i / (nx * ny));
        const float px = x - c.ax, py = y - c.ay, pz = z - c.az;
        const float t = fminf(fmaxf((px * dx + py * dy + pz * dz) / len2, 0.f), 1.f);
        const float qx = px - t * dx, qy = py - t * dy, qz = pz - t * dz;
        if (qx * qx + qy * qy + qz * qz <= r2) atomic_max_u16(vol, ((long long)z * Y + y) * X + x, c.value);
    }
}

__global__ void noise_kernel(uint16_t* vol, long long n, uint64_t seed, float sigma) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t h = mix64(seed * 0x9E3779B97F4A7C15ULL + (uint64_t)i + 1);
        const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);            // (0, 1)
        const float u2 = (float)((h >> 16) & 0xffffffu) * (1.0f / 16777216.0f);      // [0, 1)
        const float g = sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
        float v = (float)vol[i] + sigma * g;
        v = fminf(fmaxf(rintf(v), 0.f), 4095.f);
        vol[i] = (uint16_t)v;
    }
}

void catmull_rom(const double* p0, const double* p1, const double* p2, const double* p3, double t, double* out) {
    const double t2 = t * t, t3 = t2 * t;
    for (int k = 0; k < 3; ++k)
        out[k] = 0.5 * ((2 * p1[k]) + (-p0[k] + p2[k]) * t + (2 * p0[k] - 5 * p1[k] + 4 * p2[k] - p3[k]) * t2 +
                        (-p0[k] + 3 * p1[k] - 3 * p2[k] + p3[k]) * t3);
}

}  // namespace

extern "C" int vrc_synth_tubes_device(void* d_vol, const int dims[3], int ntubes, uint64_t seed, float noise_sigma,
                                      void* stream) {
    // X even: the 32-bit compare-and-swap on a voxel pair never reaches past the volume
    if (!d_vol || !dims || dims[0] < 2 || dims[0] % 2 || dims[1] < 1 || dims[2] < 1 || ntubes < 0) return 1;
    const int X = dims[0], Y = dims[1], Z = dims[2];
    const long long n = (long long)X * Y * Z;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint16_t* vol = static_cast<uint16_t*>(d_vol);
    if (cudaMemsetAsync(vol, 0, n * sizeof(uint16_t), s) != cudaSuccess) return 2;
    constexpr int CTRL = 6, SEG_PER_SPAN = 16;
    std::size_t ncaps = (std::size_t)ntubes * (CTRL - 3) * SEG_PER_SPAN;
    Capsule* h = new Capsule[ncaps > 0 ? ncaps : 1];
    uint64_t k = 0;
    std::size_t ci = 0;
    for (int tb = 0; tb < ntubes; ++tb) {
        double P[CTRL][3];
        // control points: a random walk across the volume
        for (int j = 0; j < CTRL; ++j) {
            P[j][0] = u01(seed, k++) * X;
            P[j][1] = u01(seed, k++) * Y;
            P[j][2] = u01(seed, k++) * Z;
        }
        const float r = (float)(2.0 + 18.0 * u01(seed, k++));
        const unsigned value = (unsigned)(1500.0 + 2500.0 * u01(seed, k++));
        for (int sp = 0; sp + 3 < CTRL; ++sp) {
            double prev[3];
            catmull_rom(P[sp], P[sp + 1], P[sp + 2], P[sp + 3], 0.0, prev);
            for (int q = 1; q <= SEG_PER_SPAN; ++q) {
                double cur[3];
                catmull_rom(P[sp], P[sp + 1], P[sp + 2], P[sp + 3], double(q) / SEG_PER_SPAN, cur);
                h[ci++] = Capsule{(float)prev[0], (float)prev[1], (float)prev[2], (float)cur[0], (float)cur[1],
                                  (float)cur[2], r, value};
                prev[0] = cur[0];
                prev[1] = cur[1];
                prev[2] = cur[2];
            }
        }
    }
    int status = 0;
    Capsule* d = nullptr;
    if (ncaps > 0) {
        if (cudaMalloc(&d, ncaps * sizeof(Capsule)) != cudaSuccess ||
            cudaMemcpyAsync(d, h, ncaps * sizeof(Capsule), cudaMemcpyHostToDevice, s) != cudaSuccess) {
            status = 2;
        } else {
            capsule_kernel<<<(unsigned)ncaps, 256, 0, s>>>(d, X, Y, Z, vol);
            if (cudaGetLastError() != cudaSuccess) status = 2;
        }
    }
    if (status == 0 && noise_sigma > 0.f) {
        const long long g = std::min<long long>((n + 255) / 256, 152LL * 64);
        noise_kernel<<<(unsigned)g, 256, 0, s>>>(vol, n, seed ^ 0x5eedULL, noise_sigma);
        if (cudaGetLastError() != cudaSuccess) status = 2;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) status = 2;
    cudaFree(d);
    delete[] h;
    return status;
}
