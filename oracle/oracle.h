/*
 * CPU oracle for the single-volume ray march -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++ restatement of Voreen's CPURaycaster path (and of the GLSL-only
 * shading / MIP / ISO rules of SingleVolumeRaycaster), used by the tests, the
 * smoke check and the CPU-baseline leg of the benchmark to compare results
 * with. The product library never links, loads or calls anything in this
 * directory.
 *
 * Parity status: the trilinear interpolation and voxel normalisation are
 * pinned against the reference's own compiled VolumeRAM code (oracle/ref_pin,
 * golden vectors in tests/golden); the camera matrices against the
 * reference's tgt::Matrix4 header code. The TF bake, the march loop and the
 * GLSL-only rules are restatements of the cited source (no golden outputs for
 * them exist in the reference), so for those parts parity is unpinned.
 *
 * Two precisions are exported:
 *   *_f32  -- FP32, operation-for-operation the order CPURaycaster uses
 *             (compile with -ffp-contract=off so no FMA is fused in).
 *   *_f64  -- the same algorithm evaluated in FP64.
 *
 * Image convention: row 0 is the bottom row (OpenGL window coordinates).
 */
#ifndef VRC_ORACLE_H
#define VRC_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_U8 = 0, ORC_U16 = 1, ORC_F32 = 2 };
enum { ORC_DVR = 0, ORC_MIP = 1, ORC_ISO = 2, ORC_MOP = 3, ORC_MIDA = 4, ORC_FHP = 5, ORC_FHN = 6 };
enum { ORC_SHADE_NONE = 0, ORC_SHADE_PHONG = 1 };

typedef struct {
    const void* data;      /* x-fastest linear voxels (VolumeAtomic::calcPos) */
    int dtype;             /* ORC_U8 / ORC_U16 / ORC_F32 */
    int dims[3];
    float spacing[3];
    float offset[3];
    float rwm_scale, rwm_offset;
} OrcVolume;

typedef struct {
    const uint8_t* rgba;   /* width x RGBA8, baked table */
    int width;
    float domain_lo, domain_hi;
} OrcTF;

typedef struct {
    float sampling_rate;        /* VolumeRaycaster "samplingRate" */
    int compositing;            /* ORC_DVR / ORC_MIP / ORC_ISO */
    int shading;                /* ORC_SHADE_NONE / ORC_SHADE_PHONG */
    float iso_value;            /* "isoValue" */
    float ert_threshold;        /* 0.95 (mod_raysetup.frag:36); >=1 disables */
    float light_pos_phys[3];    /* light position in volume physical coords */
    float camera_pos_phys[3];   /* camera position in volume physical coords */
    float light_ambient[3], light_diffuse[3], light_specular[3];
    float shininess;
    int apply_attenuation;
    float attenuation[3];
    float mida_gamma;           /* "gammaValue" (ORC_MIDA) */
    const float* preint;        /* pre-integration table (res*res RGBA, [back*res + front]), NULL = TF */
    int preint_res;
} OrcParams;

/* One TF key as TransFuncMappingKey holds it: intensity in [0,1], left/right
 * RGBA8 colours (equal unless the key is split). */
typedef struct {
    float intensity;
    uint8_t color_l[4];
    uint8_t color_r[4];
} OrcTFKey;

/* TransFunc1D::createTextureData + TransFunc1DKeys::getMappingForValueUByte. */
void oracle_bake_tf_keys(const OrcTFKey* keys, int nkeys, int width, float gamma,
                         float threshold_lo, float threshold_hi, uint8_t* out_rgba);

/* PreIntegrationTable::computeTable's TF buffer (preintegrationtable.cpp:71-104):
 * entry i = the keys' mapping at gamma(i/(res-1)), zero below
 * iround(threshold_lo*res) and from iround(threshold_hi*res) on. */
void oracle_preint_source(const OrcTFKey* keys, int nkeys, int res, float gamma, float threshold_lo,
                          float threshold_hi, uint8_t* out_rgba);

/* PreIntegrationTable::computeTable (preintegrationtable.cpp:67-204): the
 * exact table (use_integral 0) or the integral-function approximation (1),
 * FP32, out[4 * (back * res + front) + c]. */
void oracle_preint_table(const uint8_t* source_rgba, int res, float step, int use_integral, float* out);

/* Texture-space entry/exit points of the unit-cube proxy for a perspective
 * camera, in FP64 (MeshEntryExitPoints rendering processCube's cube).
 * inv_mvp: row-major inverse of (projection * view * textureToWorld).
 * quantize16 != 0 rounds every coordinate to k/65535 as the RGBA16 render
 * targets of the reference do. Outputs are float4 (w = 1 where hit, else
 * the whole pixel is 0). */
void oracle_entry_exit(const double* inv_mvp, int width, int height, int quantize16,
                       float* entry_rgba, float* exit_rgba);
/* The same for the proxy cube clipped to [box_lo, box_hi] in texture space
 * (OptimizedProxyGeometry::processCube with clipping,
 * modules/base/processors/proxygeometry/optimizedproxygeometry.cpp:420-448). */
void oracle_entry_exit_box(const double* inv_mvp, int width, int height, int quantize16, const double* box_lo,
                           const double* box_hi, float* entry_rgba, float* exit_rgba);

/* Full-frame march. entry/exit: W*H float4. out: W*H float4 (RGBA, not
 * clamped). samples_out (nullable): per-pixel loop iteration count.
 * first_hit_out (nullable): per-pixel first-hit ray parameter (-1 if none).
 * signature_out (nullable): per-pixel hash of (loop index, TF entry) over the
 * samples whose TF entry has alpha > 0 -- equal in two precisions exactly
 * when they take the same TF-entry decisions at the same samples.
 * row_begin/row_end restrict the rows marched (others untouched).
 * nthreads <= 0 uses all OpenMP threads. */
void oracle_render_f32(const OrcVolume* vol, const OrcTF* tf, const OrcParams* p,
                       const float* entry, const float* exit_pts, int width, int height,
                       int row_begin, int row_end, int nthreads,
                       float* out, int32_t* samples_out, float* first_hit_out, uint32_t* signature_out);
void oracle_render_f64(const OrcVolume* vol, const OrcTF* tf, const OrcParams* p,
                       const float* entry, const float* exit_pts, int width, int height,
                       int row_begin, int row_end, int nthreads,
                       double* out, int32_t* samples_out, double* first_hit_out, uint32_t* signature_out);

/* Single trilinear lookup at a (clamped) voxel position, FP32 path. Used to
 * check the restatement against the reference's compiled VolumeRAM code. */
void oracle_trilinear_f32(const OrcVolume* vol, const float* pos_xyz, int n, float* out);

/* Per-brick min/max of normalised intensity over the brick's core voxels plus
 * `apron_hi` voxels on the high side (clamped to the volume).
 * Output arrays have nbx*nby*nbz entries, brick x fastest. */
void oracle_brick_minmax(const OrcVolume* vol, int brick, int apron_hi,
                         float* out_min, float* out_max);

#ifdef __cplusplus
}
#endif
#endif
