/*
 * vrc -- GB300-native single-volume raycaster, C ABI.
 *
 * This is the drop-in boundary for Voreen's CPURaycaster / SingleVolumeRaycaster
 * path. Every entry point takes plain pointers and sizes, returns a vrc_status
 * and never throws. Handles own device memory; the caller owns host buffers.
 * A context owns one CUDA stream; all work of a context is ordered on it.
 *
 * Reference interfaces each entry point replaces (paths in the Voreen tree):
 *   vrc_volume_upload   VolumeGL upload of a VolumeRAM representation
 *                       src/core/datastructures/volume/volumegl.cpp:126-168
 *                       (+ brick min/max, optimizedproxygeometry.cpp:894-987)
 *   vrc_vvd_read_header, vrc_volume_load_vvd
 *   vrc_tf_read_tfi     TransFunc1DKeys::loadTfi (.tfi transfer-function files)
 *                       VvdVolumeReader::read, modules/core/io/vvdvolumereader.cpp,
 *                       modules/core/io/vvdformat.cpp:53-89
 *   vrc_volume_minmax   VolumeMinMax derived data used for TF domain fitting
 *                       src/core/properties/transfunc/1d/1dkeys/transfunc1dkeysproperty.cpp:104-140
 *   vrc_tf_bake_keys    TransFunc1D::createTextureData + TransFunc1DKeys::getMappingForValueUByte
 *                       src/core/datastructures/transfunc/1d/transfunc1d.cpp:85-116,
 *                       src/core/datastructures/transfunc/1d/1dkeys/transfunc1dkeys.cpp:119-154
 *   vrc_tf_table_width  TransFuncPropertyBase::setVolume width rule + 4096 cap
 *                       src/core/properties/transfunc/transfuncpropertybase.cpp:134-174,
 *                       transfunc1dkeysproperty.cpp:94-97
 *   vrc_tf_create       TransFuncBase::getTexture (RGBA8 table, NEAREST lookup)
 *                       src/core/datastructures/transfunc/transfuncbase.cpp:99-161
 *   vrc_render          CPURaycaster::process / directRendering
 *                       modules/base/processors/render/cpuraycaster.cpp:90-331, and
 *                       SingleVolumeRaycaster::process + rc_singlevolume.frag
 *                       modules/base/processors/render/singlevolumeraycaster.cpp:246-425,
 *                       modules/base/glsl/rc_singlevolume.frag:116-340
 *   vrc_entry_exit      MeshEntryExitPoints::process on OptimizedProxyGeometry::processCube
 *                       modules/base/processors/entryexitpoints/meshentryexitpoints.cpp:188-273,
 *                       modules/base/processors/proxygeometry/optimizedproxygeometry.cpp:420-448
 *   vrc_camera_matrices tgt::Camera::getViewMatrix / getProjectionMatrix
 *                       ext/tgt/camera.cpp:133-216, ext/tgt/matrix.h:1196-1248
 *   vrc_preint_*        PreIntegrationTable::computeTable / classify and the
 *                       table map's resolution rule
 *                       src/core/datastructures/transfunc/1d/preintegrationtable.cpp:67-204, 256-279,
 *                       src/core/datastructures/transfunc/1d/preintegrationtablemap.cpp:59-69
 *   vrc_tf_set_preintegration  TransFunc1D::getPreIntegrationTable as CPURaycaster
 *                       calls it, transfunc1d.cpp:121-128, cpuraycaster.cpp:112-123
 *   vrc_sampling_step   VolumeRaycaster::getSamplingStepSize / cpuraycaster.cpp:104
 *   vrc_image_rescale   VolumeRaycaster::rescaleRendering
 *                       src/core/processors/volumeraycaster.cpp:348-375 (interaction
 *                       coarseness, singlevolumeraycaster.cpp:253-256)
 *
 * Conventions: images are row-major with row 0 at the bottom (OpenGL window
 * coordinates); entry/exit points are texture-space float4 (w = 1 on hit, the
 * whole pixel 0 for background), as CPURaycaster downloads them.
 */
#ifndef VRC_H
#define VRC_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VRC_ABI_VERSION 2

typedef enum {
    VRC_OK = 0,
    VRC_ERR_INVALID_ARG = 1,   /* bad pointer, size, enum or dimension */
    VRC_ERR_CUDA = 2,          /* a CUDA runtime call failed (see vrc_last_error) */
    VRC_ERR_OUT_OF_MEMORY = 3, /* a device or host allocation was refused */
    VRC_ERR_UNSUPPORTED = 4,   /* valid request the library does not implement */
    VRC_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
    VRC_ERR_NOT_READY = 6,     /* missing input (isReady() == false in the reference) */
    VRC_ERR_DEVICE = 7,        /* a kernel reported an internal error status */
    VRC_ERR_SCRATCH_LIMIT = 8  /* request exceeds vrc_render_noalloc's fixed scratch capacity */
} vrc_status;

typedef enum { VRC_U8 = 0, VRC_U16 = 1, VRC_F32 = 2 } vrc_dtype;
/* Compositing ("compositing"): dvr, mip, iso as both CPURaycaster and the GLSL
 * raycaster do them; mop (maximum opacity), mida (maximum intensity difference
 * accumulation, "gammaValue"), fhp (first-hit position) and fhn (first-hit
 * normal) as mod_compositing.frag:97-214 does them. mip, mop and mida run
 * without early ray termination (volumeraycaster.cpp:226-228). */
typedef enum {
    VRC_DVR = 0,
    VRC_MIP = 1,
    VRC_ISO = 2,
    VRC_MOP = 3,
    VRC_MIDA = 4,
    VRC_FHP = 5,
    VRC_FHN = 6
} vrc_compositing;
/* Classification ("classification"): the 1D TF table, or the pre-integration
 * table attached to the TF (vrc_tf_set_preintegration) -- CPURaycaster's
 * "pre-integrated-cpu" / "pre-integrated-approximation" (cpuraycaster.cpp:112-123,
 * 255-261); DVR compositing only. */
typedef enum { VRC_CLASSIFY_TF = 0, VRC_CLASSIFY_PREINTEGRATED = 1 } vrc_classification;
typedef enum { VRC_SHADE_NONE = 0, VRC_SHADE_PHONG = 1 } vrc_shading;
typedef enum { VRC_OUT_RGBA8 = 0, VRC_OUT_RGBA32F = 1, VRC_OUT_RGBA16 = 2 } vrc_out_format;
typedef enum { VRC_EE_BUFFERS = 0, VRC_EE_ANALYTIC = 1 } vrc_entry_exit_mode;

typedef struct vrc_context vrc_context;
typedef struct vrc_volume vrc_volume;
typedef struct vrc_tf vrc_tf;

/* ---- context ---------------------------------------------------------- */
vrc_status vrc_context_create(int device, vrc_context** out);
/* Destroy the context's volumes, TFs, pre-integration tables and batches
 * first: they keep a pointer to it. */
vrc_status vrc_context_destroy(vrc_context* ctx);
vrc_status vrc_context_synchronize(vrc_context* ctx);
/* The context's cudaStream_t, for callers that order their own work with it. */
void* vrc_context_stream(vrc_context* ctx);
const char* vrc_status_string(vrc_status s);
/* Human-readable detail of the last failing call on this context. */
const char* vrc_last_error(const vrc_context* ctx);
int vrc_abi_version(void);

/* ---- volume ----------------------------------------------------------- */
typedef struct {
    int dtype;            /* vrc_dtype */
    int dims[3];          /* voxels, x fastest (VolumeAtomic::calcPos) */
    float spacing[3];     /* voxel size in physical units */
    float offset[3];      /* physical position of voxel (0,0,0)'s lower corner + 0.5 spacing */
    float rwm_scale;      /* RealWorldMapping: rw = normalized * scale + offset */
    float rwm_offset;
} vrc_volume_desc;

/* Upload a linear x-fastest volume into the bricked device layout and build
 * the per-brick min/max table and the empty-space cell tables (2^3 cells up
 * to 2^30 of them -- 1 byte of tables per voxel --, 4^3, 8^3, 16^3 below the
 * brick size). `voxels_on_device` != 0 means `voxels` is a device pointer.
 * brick_size: 0 = default (32); otherwise 8, 16, 32 or 64. */
vrc_status vrc_volume_upload(vrc_context* ctx, const vrc_volume_desc* desc, const void* voxels,
                             int voxels_on_device, int brick_size, vrc_volume** out);
/* Brick-pool placement: device memory (HBM), or pinned host memory that
 * the kernels read through its mapped device address -- over NVLink-C2C on
 * Grace hosts -- so a volume larger than the GPU's memory can be rendered
 * (the min/max tables stay in device memory). With VRC_PLACE_HOST and host
 * voxels, the bricking kernels also read the caller's voxels in place
 * (cudaHostRegister for the duration of the call), so no device copy of
 * the volume is made at any point. */
typedef enum { VRC_PLACE_DEVICE = 0, VRC_PLACE_HOST = 1 } vrc_placement;
vrc_status vrc_volume_upload_placed(vrc_context* ctx, const vrc_volume_desc* desc, const void* voxels,
                                    int voxels_on_device, int brick_size, int placement, vrc_volume** out);
vrc_status vrc_volume_destroy(vrc_volume* vol);
/* Min/max of the normalised intensity (getVoxelNormalized) over the volume. */
vrc_status vrc_volume_minmax(vrc_volume* vol, float* min_norm, float* max_norm);
/* Brick grid and per-brick min/max of normalised intensity (core voxels plus
 * one voxel on the high side, the trilinear support). out_* may be NULL to
 * query nbricks only. */
vrc_status vrc_volume_brick_minmax(vrc_volume* vol, int nbricks_out[3], float* out_min, float* out_max);
/* Device bytes held by the bricked layout (and its tables). */
size_t vrc_volume_device_bytes(const vrc_volume* vol);
/* Pinned host bytes of a VRC_PLACE_HOST brick pool (0 otherwise). */
size_t vrc_volume_host_bytes(const vrc_volume* vol);
/* Device brick cache of a VRC_PLACE_HOST pool. vrc_render copies the bricks
 * the current transfer function can reach (value range meets a visible
 * entry, plus their 26 neighbours) into device memory before the march, up
 * to `bytes` (default: unlimited, bounded by free device memory less 1 GiB;
 * 0 = no cache). Bricks already cached are kept across TF changes; bricks
 * left out are read from the host pool, so the image never depends on the
 * cache. The device-side counterpart of the reference's brick pool
 * managers, which keep a bounded set of bricks resident in RAM in front of
 * a larger store (OctreeBrickPoolManagerBase::getBrick,
 * include/voreen/core/datastructures/octree/octreebrickpoolmanager.h:99-165). */
vrc_status vrc_volume_set_cache_limit(vrc_volume* vol, size_t bytes);
/* Bytes of bricks gathered into the cache per render (0, the default =
 * unlimited); at least one brick. With a budget, a TF change or a new view
 * streams its bricks in over several renders, the bricks the last render
 * read without a slot first -- Voreen's octree raycaster's per-frame brick
 * upload budget (brickUploadBudgetMB, modules/opencl/processors/
 * singleoctreeraycastercl.cpp:304). Images stay exact (or, with the level
 * of detail on, converge) whatever the budget. */
vrc_status vrc_volume_set_cache_upload_budget(vrc_volume* vol, size_t bytes_per_render);
/* While the cache holds fewer bricks than the TF reaches (or a level of
 * detail is attached), each render records the bricks it reads; before the
 * next render, bricks read without a cache slot displace cached bricks that
 * were not read, least recently read first (the used/missing brick flags and
 * LRU brick pool of Voreen's octree raycaster, singleoctreeraycaster.cl).
 * A still view converges to a cache holding its working set.
 * vrc_volume_cache_info: bricks held by the cache, bricks the last TF could
 * reach, and bricks the last tracked render read without a slot. */
vrc_status vrc_volume_cache_info(const vrc_volume* vol, long long* cached, long long* reachable, long long* missed);
/* Level of detail for a VRC_PLACE_HOST pool: a device-resident coarser
 * level of the pyramid VolumeOctree builds (each voxel the mean of 2x2x2
 * voxels of the level above, clamped at that level's edges: HalfSampleMean
 * parent bricks, volumeoctree.cpp:188-202). `level` k = 1 is half
 * resolution, k = 2 quarter, ..., up to VRC_MAX_LOD_LEVEL; 0 turns the level
 * of detail off. Built on enable (again when k changes; only level k stays
 * on the device, 8^-k of the volume). While enabled, a brick without a cache
 * slot is sampled from level k at the same texture-space point instead of
 * from the host pool -- the coarser node Voreen's octree raycaster reads
 * where a brick is not on the GPU -- so frames stay fast, degrade by level
 * when the cache budget is below the view's working set, and approach the
 * full-resolution image as refinement fills the cache. VRC_ERR_UNSUPPORTED
 * for device-resident pools. */
#define VRC_MAX_LOD_LEVEL 6
vrc_status vrc_volume_set_lod(vrc_volume* vol, int level);

/* ---- volume ingest (.vvd) ------------------------------------------------
 * Voreen's .vvd volume files (VvdVolumeReader, modules/core/io/vvdvolumereader.cpp,
 * vvdformat.cpp:53-89): the header's RawData format ("uint8", "uint16",
 * "float"), dimensions and raw file (a `filename` attribute relative to the
 * .vvd, or the path list of VoreenFilePathHelper, first existing entry), the
 * Offset / Spacing / RealWorldMapping meta items (Voreen's defaults when
 * absent) and the VolumeMinMax derived item. */
typedef struct {
    int dtype;              /* vrc_dtype of the raw voxels */
    int dims[3];
    float spacing[3], offset[3];
    float rwm_scale, rwm_offset;
    int has_minmax;         /* the file holds a VolumeMinMax item: */
    float min_norm, max_norm;  /* its minNorm / maxNorm */
    char raw_path[4096];    /* the resolved raw file */
} vrc_vvd_info;

/* Host-only header parse. VRC_ERR_UNSUPPORTED for other formats or voxels
 * stored inside the XML; VRC_ERR_NOT_READY when the file or its raw file is
 * missing. */
vrc_status vrc_vvd_read_header(const char* vvd_path, vrc_vvd_info* info);
/* Header parse, then the raw file streamed through two 64 MiB pinned host
 * chunks (read of one chunk overlaps the device copy of the other) into a
 * bricked device volume with its min/max tables (vrc_volume_upload).
 * info_out may be NULL. */
vrc_status vrc_volume_load_vvd(vrc_context* ctx, const char* vvd_path, int brick_size, vrc_volume** out,
                               vrc_vvd_info* info_out);

/* ---- transfer function --------------------------------------------------- */
typedef struct {
    float intensity;      /* key position in [0,1] */
    uint8_t color_l[4];   /* RGBA8 left of the key */
    uint8_t color_r[4];   /* RGBA8 right of the key (== color_l unless split) */
} vrc_tf_key;

/* Host-only bake of a keyed 1D TF into a width x RGBA8 table. Keys must be
 * sorted by intensity. gamma 1 and thresholds (0,1) are the defaults. */
vrc_status vrc_tf_bake_keys(const vrc_tf_key* keys, int nkeys, int width, float gamma, float threshold_lo,
                            float threshold_hi, uint8_t* out_rgba);
/* TF table width for a volume dtype: 2^bits (float as 16 bit), capped at 4096. */
int vrc_tf_table_width(int dtype);
/* Device copy of a baked table with its real-world domain. width <= 4096. */
vrc_status vrc_tf_create(vrc_context* ctx, const uint8_t* rgba, int width, float domain_lo, float domain_hi,
                         vrc_tf** out);
vrc_status vrc_tf_destroy(vrc_tf* tf);

/* Voreen's .tfi transfer-function files (TransFunc1DKeys::loadTfi,
 * src/core/datastructures/transfunc/1d/1dkeys/transfunc1dkeys.cpp:685-712):
 * the TransFuncIntensity element's alphaMode, texDimensions, gammaValue,
 * domain and threshold (TransFuncBase::deserialize, transfuncbase.cpp:222-232;
 * TransFunc1D::deserialize, transfunc1d.cpp:206-212; the reference's
 * defaults when absent) and its keys in file order (intensity, split, colorL,
 * colorR when split: TransFuncMappingKey::deserialize,
 * transfuncmappingkey.cpp:150-161). Writes at most max_keys keys; info->nkeys
 * is the number in the file. VRC_ERR_NOT_READY when the file cannot be read,
 * VRC_ERR_UNSUPPORTED when it holds no TransFuncIntensity. */
typedef struct {
    int width;           /* texDimensions x, 0 when absent */
    int alpha_mode;      /* alphaMode, 1 (use alpha) when absent */
    float gamma;         /* gammaValue, 1 when absent */
    float domain[2];     /* domain (real-world), (0, 1) when absent */
    float threshold[2];  /* threshold (normalised), (0, 1) when absent */
    int nkeys;
} vrc_tfi_info;
vrc_status vrc_tf_read_tfi(const char* path, vrc_tfi_info* info, vrc_tf_key* keys, int max_keys);

/* ---- pre-integrated classification --------------------------------------
 * PreIntegrationTable (src/core/datastructures/transfunc/1d/preintegrationtable.cpp):
 * an res x res RGBA table, entry [back * res + front] = the TF integrated
 * between the previous sample's TF coordinate (front) and the current one
 * (back) over one sampling step. */
typedef struct vrc_preint vrc_preint;

/* Table resolution: `requested` if > 0, else min(TF width, 1024)
 * (PreIntegrationTableMap::getPreIntegrationTable, preintegrationtablemap.cpp:64-69). */
int vrc_preint_resolution(int tf_width, int requested);
/* Host-only: the TF sampled at `res` entries as PreIntegrationTable::computeTable
 * does (preintegrationtable.cpp:71-104): entry i = the keys' RGBA8 mapping at
 * gamma(i / (res - 1)), zero for i < iround(threshold_lo * res) and for
 * i >= iround(threshold_hi * res). */
vrc_status vrc_preint_bake_source(const vrc_tf_key* keys, int nkeys, int res, float gamma, float threshold_lo,
                                  float threshold_hi, uint8_t* out_rgba);
/* Builds the table for sampling step `step` (vrc_sampling_step) on the
 * device from the res x RGBA8 source. use_integral = 0: the exact table
 * (composited entry by entry, O(res^3), built by a CUDA kernel); 1: the
 * integral-function approximation (O(res^2), built on the host). 2 <= res <= 4096. */
vrc_status vrc_preint_create(vrc_context* ctx, const uint8_t* source_rgba, int res, float step, int use_integral,
                             vrc_preint** out);
/* Copies the table to the host: res * res * 4 floats, entry [back * res + front]. */
vrc_status vrc_preint_download(const vrc_preint* t, float* out_rgba);
vrc_status vrc_preint_destroy(vrc_preint* t);
/* Attaches `t` to `tf` for renders with classification VRC_CLASSIFY_PREINTEGRATED
 * (NULL detaches). The table must outlive its use by the TF. */
vrc_status vrc_tf_set_preintegration(vrc_tf* tf, const vrc_preint* t);
/* samplingStepSize = 1 / (max(dim) * samplingRate) (cpuraycaster.cpp:104), as the march uses it. */
float vrc_sampling_step(const vrc_volume* vol, float sampling_rate);

/* ---- camera ------------------------------------------------------------ */
typedef struct {
    float position[3], focus[3], up[3];  /* world coordinates */
    float fovy_deg;                      /* vertical field of view */
    float near_dist, far_dist;
    float frustum_ratio;                 /* tgt::Frustum ratio, 1 by default */
} vrc_camera;

/* Row-major view, projection and inverse(projection * view * textureToWorld)
 * for a W x H viewport, computed in double. Any output may be NULL. */
vrc_status vrc_camera_matrices(const vrc_camera* cam, const vrc_volume_desc* vol, int width, int height,
                               double* view, double* proj, double* inv_mvp_tex);

/* ---- render ------------------------------------------------------------ */
typedef struct {
    int width, height;
    float sampling_rate;        /* "samplingRate", default 2 */
    int compositing;            /* vrc_compositing ("compositing": dvr / mip / iso) */
    int shading;                /* vrc_shading ("shading": none / phong) */
    float iso_value;            /* "isoValue", default 0.5 */
    float ert_threshold;        /* 0.95; >= 1 disables early ray termination */
    float light_position[4];    /* "lightPosition" (world), default (2.3, 1.5, 1.5, 1) */
    float light_ambient[3];     /* "lightAmbient", default 0.4 */
    float light_diffuse[3];     /* "lightDiffuse", default 0.8 */
    float light_specular[3];    /* "lightSpecular", default 0.6 */
    float material_shininess;   /* "materialShininess", default 60 */
    int apply_attenuation;      /* "applyLightAttenuation", default 0 */
    float light_attenuation[3]; /* "lightAttenuation", default (1, 0, 0) */
    vrc_camera camera;          /* "camera": used for shading and analytic entry/exit */
    int entry_exit_mode;        /* vrc_entry_exit_mode */
    int quantize_entry_exit;    /* analytic mode: round coordinates to k/65535 like RGBA16 targets */
    int empty_space_skipping;   /* skip cells whose TF opacity is zero (exact: results unchanged) */
    int skip_cell_size;         /* empty-space cell edge in voxels: 0 = default (vrc_render: 2 where the volume
                                   holds the 2^3 level -- up to 2^30 cells -- else 4, also for batches;
                                   vrc_render_noalloc: the finest of 2, 4, 8 that fits its scratch), else 2,
                                   4, 8, 16 or the brick size */
    int tile_width;             /* ray tile per warp: tile_width x (32 / tile_width) pixels; 0 = default (8) */
    int region[4];              /* x, y, w, h of the pixel window to render; w or h 0 = the whole image */
    int classification;         /* vrc_classification, default VRC_CLASSIFY_TF */
    float mida_gamma;           /* "gammaValue" for VRC_MIDA, in [-1, 1], default 0 */
    /* Proxy-geometry clipping of analytic entry/exit (and vrc_entry_exit):
     * OptimizedProxyGeometry "enableClipping" / "clipRegion", an inclusive
     * voxel box; the cube becomes [llf - 0.5, urb + 0.5] in voxel coordinates
     * (optimizedproxygeometry.cpp:420-448). Ignored in buffer mode. */
    int enable_clipping;
    int clip_llf[3], clip_urb[3];
} vrc_render_params;

/* Fills `p` with the reference's property defaults for a W x H image. */
void vrc_render_params_default(vrc_render_params* p, int width, int height);

typedef struct {
    double samples;          /* loop iterations of all rays (the reference's sample count) */
    double samples_fetched;  /* samples whose voxels were read (not skipped) */
    double samples_shaded;   /* samples with TF alpha > 0 under shading */
    double skip_runs;        /* runs of samples skipped through empty cells */
    float kernel_ms;         /* device time of the march kernel on the context stream */
    float total_ms;          /* device time from first copy-in to last copy-out */
    int device_status;       /* 0, or an internal error code from the kernel */
    int kernel_launches;     /* kernels this frame launched (occupancy levels + march) */
} vrc_render_stats;

/* Render one frame.
 *   entry/exit: W*H float4 texture-space points (VRC_EE_BUFFERS), else ignored.
 *   ee_on_device / out_on_device: 0 = host pointers (copied on the context
 *   stream, call returns after the frame is on the host), 1 = device pointers
 *   (call returns after the launch; synchronize before reading).
 *   out: W*H pixels in `out_format`.
 *   stats: may be NULL; sample counters need a synchronize, done when non-NULL. */
vrc_status vrc_render(vrc_context* ctx, const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p,
                      const float* entry, const float* exit_pts, int ee_on_device, void* out, int out_format,
                      int out_on_device, vrc_render_stats* stats);

/* Diagnostics: read bandwidth of an L2-resident buffer of `bytes` (every SM
 * reading it `reps` times with 16-byte loads), in GB/s: the on-chip peak the
 * march's gathers are compared with beside the HBM copy peak. */
vrc_status vrc_measure_l2_read(vrc_context* ctx, size_t bytes, int reps, float* gbs);

/* Diagnostics: the empty-space distance field the march skips by, computed
 * from a device bitmap of nx x ny x nz cells (bit i of word i / 32 set =
 * occupied, cells x-fastest): d_out[i] = the Chebyshev distance in cells
 * from cell i to the nearest occupied cell, capped at 16 in the default
 * build (0 for occupied cells). Device pointers; runs on the context stream and returns when done. */
vrc_status vrc_occupancy_distance(vrc_context* ctx, const uint32_t* d_bits, int nx, int ny, int nz, uint8_t* d_out);

/* Bilinear rescale of a device RGBA image (w x h) to W x H on the context
 * stream: VolumeRaycaster::rescaleRendering (GL_LINEAR, clamp to edge) as
 * SingleVolumeRaycaster applies it after an interaction-coarseness render.
 * format: VRC_OUT_RGBA8 or VRC_OUT_RGBA32F (same for both images). */
vrc_status vrc_image_rescale(vrc_context* ctx, const void* d_src, int w, int h, void* d_dst, int W, int H,
                             int format);

/* ---- batched persistent render ----------------------------------------------
 * No counterpart in the reference (it renders one request per processor
 * call). Many requests -- uneven volumes, dtypes and image sizes -- march in
 * ONE persistent kernel launch; every request's empty-space maps are built
 * once, when the batch is created (volumes and TFs do not change after
 * creation), and the per-launch sequence (state reset, the march) is
 * captured as a CUDA graph on the context's stream and replayed by
 * vrc_batch_launch. All items
 * share compositing and shading and use analytic entry/exit (the camera in
 * their params); each writes its own device image. */
typedef struct {
    const vrc_volume* volume;
    const vrc_tf* tf;
    vrc_render_params params;
    void* out;          /* device image, params.width x params.height pixels */
    int out_format;     /* vrc_out_format */
} vrc_batch_item;

typedef struct vrc_batch vrc_batch;

typedef struct {
    double samples;          /* loop iterations of all rays of all requests */
    float total_ms;          /* device time of the last launch (first kernel start to last tile) */
    float latency_p50_ms;    /* per-request completion time after the launch start: median */
    float latency_p99_ms;    /* ... 99th percentile */
    float latency_max_ms;
    int kernels_per_launch;  /* kernel nodes in the captured graph */
} vrc_batch_stats;

/* Builds device descriptors and TF tables (allocating), orders requests
 * longest first and captures the launch sequence. Items are copied. */
vrc_status vrc_batch_create(vrc_context* ctx, const vrc_batch_item* items, int n, vrc_batch** out);
/* As vrc_batch_create, with each request isolated from the others: a request
 * that fails its checks (null or foreign handles, invalid parameters, a
 * singular camera, an unsupported mode, or compositing / shading other than
 * the first valid request's) is left out of the launch instead of failing
 * the batch, and status[i] (n entries, required) receives each request's
 * vrc_status -- VRC_OK for the requests that run. Returns an error only when
 * no request is valid or on a batch-wide failure (allocation, capture).
 * Stats report latency -1 for requests left out. The per-job isolation of
 * SIMDRaycaster's job queue (modules/staging/processors/simdraycaster/
 * simdraycaster.cpp:401-414) at request granularity. */
vrc_status vrc_batch_create_isolated(vrc_context* ctx, const vrc_batch_item* items, int n, int* status,
                                     vrc_batch** out);
/* Enqueues one replay of the captured graph on the context's stream. */
vrc_status vrc_batch_launch(vrc_batch* b);
/* Synchronizes the context stream, then reports the last launch:
 * latency_ms (nullable, n floats in item order) and totals. */
vrc_status vrc_batch_stats_get(vrc_batch* b, float* latency_ms, vrc_batch_stats* st);
vrc_status vrc_batch_destroy(vrc_batch* b);

/* ---- render without allocating ---------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc while they render -- a real-time frame loop (cudaMalloc can
 * synchronise the device and stall the frame), or hosts whose device memory
 * belongs to their own fixed-budget pool or to another runtime. It renders
 * like vrc_render but keeps its scratch (sample and tile counters, the
 * per-render alpha table, the empty-space cell map and its distance field)
 * in one fixed-size array (4.5 MB) in device global memory that every GPU
 * loading the library holds until exit, and it allocates nothing.
 * Limits: at most VRC_NOALLOC_MAX_CELLS empty-space cells when skipping is on
 * (skip_cell_size 0 takes 2^3 cells up to 256^3 voxels, 4^3 up to 512^3
 * and 8^3, up to a 1024^3 volume, above) and TF width <= 4096; larger
 * requests return
 * VRC_ERR_SCRATCH_LIMIT and render nothing. TF classification only
 * (VRC_ERR_UNSUPPORTED otherwise). Frames equal vrc_render's, but MIP's
 * max-based cell skipping is not taken, and a host-placed brick pool
 * is read in place (no device brick cache, no level of detail), so some
 * frames take longer than vrc_render's.
 * The caller passes the inputs (an uploaded volume, a TF of the same
 * context, device entry/exit images unless analytic), the device output
 * image and the cudaStream_t to run on; the call returns after enqueueing
 * (no host buffer is read afterwards) and leaves the calling thread's
 * current device as it found it. Its first call on a device sets up the
 * scratch address for that device. All calls share the array: calls that
 * overlap on the GPU race. The kernel's device status word is not reported
 * (vrc_render's stats report it); the returned status covers the arguments
 * and the launches. */
#define VRC_NOALLOC_MAX_CELLS 2097152
vrc_status vrc_render_noalloc(const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p,
                              const float* d_entry, const float* d_exit, void* d_out, int out_format, void* stream);

/* vrc_render into device buffers plus an auxiliary per-pixel float2 image:
 * (first-hit ray parameter / ray length, or 1 without a hit; gradient
 * magnitude at the first hit scaled by min(spacing) / TF domain width, 0
 * without shading). No counterpart in the reference: it feeds the learned
 * upsampler (include/vrc_nn.h). entry/exit may be NULL in analytic mode. */
vrc_status vrc_render_aux(vrc_context* ctx, const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p,
                          const float* d_entry, const float* d_exit, void* d_out, int out_format, float* d_aux,
                          vrc_render_stats* stats);

/* Analytic entry/exit points (texture space) for `p->camera`, written as
 * float4 images, host or device destination. */
vrc_status vrc_entry_exit(vrc_context* ctx, const vrc_volume* vol, const vrc_render_params* p, float* entry,
                          float* exit_pts, int out_on_device);

#ifdef __cplusplus
}
#endif
#endif
