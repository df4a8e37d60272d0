// Seeded procedural volumes: the benchmark workloads and the training data
// of the learned upsampler are rendered from these. Deterministic for a given
// seed on any host (integer hashing; per-voxel work is independent, so the
// OpenMP schedule does not change the result).
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/vrc_synth.h"

namespace {

inline uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
inline uint64_t hash2(uint64_t a, uint64_t b) {
    uint64_t s = a * 0xD6E8FEB86659FD93ULL + b;
    return splitmix(s);
}
// uniform in [0, 1) with 53 random bits
inline double u01(uint64_t h) { return double(h >> 11) * (1.0 / 9007199254740992.0); }

struct Rng {
    uint64_t s;
    double uniform(double lo, double hi) { return lo + (hi - lo) * u01(splitmix(s)); }
};

double gauss_noise(uint64_t seed, uint64_t idx) {
    const double u1 = u01(hash2(seed, 2 * idx)) + 1e-300;
    const double u2 = u01(hash2(seed, 2 * idx + 1));
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

template <typename T> T quantize(double unit, int dtype);
template <> uint8_t quantize<uint8_t>(double unit, int) {
    double v = std::floor(unit * 255.0 + 0.5);
    return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
}
template <> uint16_t quantize<uint16_t>(double unit, int) {
    double v = std::floor(unit * 4095.0 + 0.5);
    return (uint16_t)(v < 0 ? 0 : (v > 4095 ? 4095 : v));
}
template <> float quantize<float>(double unit, int) {
    return (float)(unit < 0 ? 0.0 : (unit > 1.0 ? 1.0 : unit));
}

// Sum of 8 isotropic Gaussians + uniform noise (the 128^3 blob family).
template <typename T> void blobs(const int d[3], uint64_t seed, T* out, double full_scale) {
    Rng r{seed};
    double c[8][3], sig[8], amp[8];
    for (int k = 0; k < 8; ++k) {
        for (int i = 0; i < 3; ++i) c[k][i] = r.uniform(0.2, 0.8) * d[i];
        sig[k] = r.uniform(4.0, 16.0);
        amp[k] = r.uniform(80.0, 255.0) / 255.0;
    }
    const uint64_t nseed = splitmix(r.s);
    const long long nvox = (long long)d[0] * d[1] * d[2];
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nvox; ++i) {
        const int x = int(i % d[0]), y = int((i / d[0]) % d[1]), z = int(i / ((long long)d[0] * d[1]));
        double v = 0.0;
        for (int k = 0; k < 8; ++k) {
            const double dx = x - c[k][0], dy = y - c[k][1], dz = z - c[k][2];
            v += amp[k] * std::exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * sig[k] * sig[k]));
        }
        v += 10.0 / 255.0 * u01(hash2(nseed, (uint64_t)i));
        (void)full_scale;
        out[i] = quantize<T>(v > 1.0 ? 1.0 : v, 0);
    }
}

// Six nested, randomly oriented ellipsoid shells on a zero background plus
// Gaussian noise (the CT-like family). Intensities are given on a 0..4095
// scale and mapped to the dtype's unit range.
template <typename T> void shells(const int d[3], uint64_t seed, T* out) {
    Rng r{seed};
    static const double inten[6] = {200, 1000, 1800, 2600, 3200, 4000};
    double c[3], a0[3];
    for (int i = 0; i < 3; ++i) {
        c[i] = d[i] * (0.5 + r.uniform(-0.05, 0.05));
        a0[i] = d[i] * r.uniform(0.30, 0.45);
    }
    const double ax = r.uniform(0, 6.283185307179586), ay = r.uniform(0, 6.283185307179586),
                 az = r.uniform(0, 6.283185307179586);
    const double cx = std::cos(ax), sx = std::sin(ax), cy = std::cos(ay), sy = std::sin(ay), cz = std::cos(az),
                 sz = std::sin(az);
    // R = Rz * Ry * Rx
    const double R[9] = {cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx,
                         sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx,
                         -sy,     cy * sx,                cy * cx};
    double outer[6][3], inner[6][3];
    // a shell's thickness in voxels must stay below the gap to the next one
    const double scale_unit = std::min(std::min(d[0], d[1]), d[2]) / 512.0;
    for (int k = 0; k < 6; ++k) {
        const double th = r.uniform(3.0, 12.0) * (scale_unit < 1.0 ? std::max(scale_unit, 0.25) : 1.0);
        for (int i = 0; i < 3; ++i) {
            outer[k][i] = a0[i] * (1.0 - 0.14 * k);
            inner[k][i] = std::max(outer[k][i] - th, 0.5);
        }
    }
    const uint64_t nseed = splitmix(r.s);
    const long long nvox = (long long)d[0] * d[1] * d[2];
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nvox; ++i) {
        const int x = int(i % d[0]), y = int((i / d[0]) % d[1]), z = int(i / ((long long)d[0] * d[1]));
        const double px = x - c[0], py = y - c[1], pz = z - c[2];
        const double q[3] = {R[0] * px + R[1] * py + R[2] * pz, R[3] * px + R[4] * py + R[5] * pz,
                             R[6] * px + R[7] * py + R[8] * pz};
        double v = 0.0;
        for (int k = 5; k >= 0; --k) {
            double ro = 0, ri = 0;
            for (int j = 0; j < 3; ++j) {
                ro += (q[j] / outer[k][j]) * (q[j] / outer[k][j]);
                ri += (q[j] / inner[k][j]) * (q[j] / inner[k][j]);
            }
            if (ro <= 1.0 && ri > 1.0) {
                v = inten[k];
                break;
            }
            if (ri <= 1.0) break;  // inside shell k's cavity: nested shells are tested first
        }
        v += 20.0 * gauss_noise(nseed, (uint64_t)i);
        out[i] = quantize<T>(v / 4095.0, 0);
    }
}

}  // namespace

extern "C" {

int vrc_synth_volume(int kind, int dtype, const int dims[3], uint64_t seed, void* out) {
    if (!dims || !out || dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return 1;
    if (kind == VRC_SYNTH_BLOBS) {
        if (dtype == 0) blobs<uint8_t>(dims, seed, (uint8_t*)out, 255.0);
        else if (dtype == 1) blobs<uint16_t>(dims, seed, (uint16_t*)out, 4095.0);
        else blobs<float>(dims, seed, (float*)out, 1.0);
        return 0;
    }
    if (kind == VRC_SYNTH_SHELLS) {
        if (dtype == 0) shells<uint8_t>(dims, seed, (uint8_t*)out);
        else if (dtype == 1) shells<uint16_t>(dims, seed, (uint16_t*)out);
        else shells<float>(dims, seed, (float*)out);
        return 0;
    }
    return 1;
}

}  // extern "C"
