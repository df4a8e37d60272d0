/*
 * vrc_synth -- seeded procedural volumes (no counterpart in the reference).
 *
 * The raycaster's benchmark workloads and the learned upsampler's training
 * pairs are rendered from these volumes. Values are deterministic for a seed.
 *   VRC_SYNTH_BLOBS : sum of 8 isotropic Gaussians (centres U[0.2,0.8]^3 * dim,
 *                     sigma U[4,16] voxels, amplitude U[80,255]/255) plus
 *                     U[0,10]/255 noise, clamped.
 *   VRC_SYNTH_SHELLS: 6 nested, randomly rotated ellipsoid shells at
 *                     intensities 200..4000 of 4095 (thickness 3-12 voxels)
 *                     on a zero background plus N(0, 20/4095) noise, clamped.
 * Unit-range values map to u8 as round(v*255), to u16 as round(v*4095)
 * (12-bit data, CT-like) and to f32 unchanged.
 */
#ifndef VRC_SYNTH_H
#define VRC_SYNTH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { VRC_SYNTH_BLOBS = 0, VRC_SYNTH_SHELLS = 1 };

/* dtype: 0 = u8, 1 = u16, 2 = f32. Returns 0 on success. */
int vrc_synth_volume(int kind, int dtype, const int dims[3], uint64_t seed, void* out);

/* Large sparse uint16 volume generated on the device into d_vol (x fastest):
 * `ntubes` tubes along Catmull-Rom splines through 6 random control points,
 * radius U[2,20] voxels, intensity U[1500,4000], on a zero background, plus
 * N(0, noise_sigma) noise, clamped to [0, 4095]. dims[0] must be even. `stream` is a cudaStream_t;
 * returns after the volume is complete (0 on success). */
int vrc_synth_tubes_device(void* d_vol, const int dims[3], int ntubes, uint64_t seed, float noise_sigma,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif
