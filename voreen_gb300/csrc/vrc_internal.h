// Internal declarations shared by the host API (api.cpp) and the CUDA
// translation units. Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/vrc.h"

namespace vrc {

// Bricked volume layout: bricks of B^3 core voxels stored with an apron of
// APRON_LO voxel below and APRON_HI voxels above on every axis, filled with
// the clamp-to-edge value. A sample whose floor voxel lies in a brick then
// reads its trilinear stencil (+1) and the central-difference stencil
// (-1 .. +2) from that brick alone.
constexpr int APRON_LO = 1;
constexpr int APRON_HI = 2;

inline int dtype_bytes(int dt) { return dt == VRC_U8 ? 1 : (dt == VRC_U16 ? 2 : 4); }

struct BrickLayout {
    int dims[3];
    int B;        // core edge
    int shift;    // log2(B)
    int S;        // stored edge = B + APRON_LO + APRON_HI
    int nb[3];    // brick grid
    long long brick_stride;  // voxels per stored brick (S^3 rounded up to 64)
#ifdef __CUDACC__
    __host__ __device__
#endif
    long long nbricks() const { return (long long)nb[0] * nb[1] * nb[2]; }
};

// Parameters of one march launch (passed by value).
struct MarchParams {
    const void* bricks;
    const uint32_t* occupancy;  // one bit per skip cell (cell index order); nullptr = no skipping
    int cshift;                 // log2(skip cell edge)
    int nc[3];                  // skip cell grid
    float skip_margin;          // voxels kept clear of a cell face when skipping by t range
    const uint32_t* occ_coarse; // optional coarser skip level (one bit per brick); nullptr = single level
    int cshift_coarse;
    int ncc[3];
    // optional, per skip cell: Chebyshev distance in cells to the nearest
    // occupied cell, capped at OCC_DIST_CAP (an empty cell at distance d is
    // the centre of an empty box of (2d - 1)^3 cells); used instead of the
    // coarse level when set, nullptr = off
    const uint8_t* occ_dist;
    // TF classification: the RGBA8 entries (the CPU path's texel bytes) and,
    // per alpha byte, the alpha the march composites -- 1-(1-a/255)^(step*200)
    // for DVR / MIDA, a/255 otherwise (computed on the host with the same powf
    // the CPU path calls). r/255, g/255, b/255 are formed in the kernel with
    // the exact 8-bit normalisation.
    const uchar4* tf_rgba8;
    const float* tf_alpha;      // 256 entries
    int tf_width;
    BrickLayout L;
    float dimf[3], dim_m1[3], offs[3];
    float spacing[3], spacing_rcp_half[3], vol_offset[3];
    float gscale[3];            // raw-value central difference -> gradient: 0.5/spacing * rwmScale / rangeMax
    float rwm_scale, rwm_offset, tf_lo, tf_hi;
    float step, ert;
    int use_ert;
    float iso;
    float light_phys[3], cam_phys[3];
    float amb[3], dif[3], spec[3];
    float shininess;
    int atten_on;
    float att[3];
    int W, H;
    int ee_mode;                 // VRC_EE_BUFFERS / VRC_EE_ANALYTIC
    int quantize;
    const float4* entry;
    const float4* exitp;
    float inv_mvp[16];
    float box_lo[3], box_hi[3];  // proxy cube in texture space ([0, 1] unless clipped)
    void* out;
    int out_format;
    unsigned long long* counters;  // [samples, fetched, shaded]
    int* status;
    unsigned int* tile_counter;
    int tiles_x, tiles_y;
    int tile_wshift;             // ray tile = (1 << tile_wshift) x (32 >> tile_wshift) pixels per warp
    int rx0, ry0, rx1, ry1;      // rendered pixel window [rx0, rx1) x [ry0, ry1) (the whole image by default)
    float2* aux;                 // optional per pixel (first-hit depth / ray length, |gradient| there), nullptr = off
    float aux_gscale;            // gradient magnitude scale for aux.y
    const float4* pi_table;      // pre-integration table [back * pi_res + front]; nullptr = classify by the TF
    int pi_res;
    int pi_chain;                // a step moves less than 0.99 voxel per axis: empty-to-empty segments skip
    // MIP: skip cells whose largest value cannot raise the ray's maximum
    // (max tables of the skip level and of the bricks; mip_skip = 0: off)
    const float* cell_max;
    const float* brick_max;
    int mip_skip;
    const int* brick_slot;       // brick -> slot in `bricks` (a device brick cache) or -1, nullptr = direct
    const void* host_pool;       // mapped host pool read for slot -1 (when lod_bricks is null)
    const void* lod_bricks;      // half-resolution level read for slot -1, nullptr = read the host pool
    int lod_nb[3];               // its brick grid (same brick size and stride as the full level)
    float lod_dimf[3], lod_dim_m1[3];
    uint32_t* brick_used;        // one bit per brick touched by a sample or tap, nullptr = not tracked
    float mida_gamma;            // "gammaValue" of MIDA compositing
};

#ifndef VRC_OCC_DIST_CAP
#define VRC_OCC_DIST_CAP 16
#endif
constexpr int OCC_DIST_CAP = VRC_OCC_DIST_CAP;

// Internal compositing code of the march kernels: DVR with pre-integrated
// classification (no opacity correction, classify(previous, current)).
constexpr int COMP_DVR_PREINT = 16;

// Whether the TF table carries the opacity correction 1-(1-a)^(step*200):
// DVR with TF classification (cpuraycaster.cpp:291) and MIDA
// (mod_compositing.frag:134); MIP / ISO / MOP / FHP / FHN use the TF alpha.
inline bool alpha_corrected(int compositing, int classification) {
    return (compositing == VRC_DVR && classification == VRC_CLASSIFY_TF) || compositing == VRC_MIDA;
}

// One request of a batched launch.
struct BatchReq {
    MarchParams P;
    int dtype;
    int pad[3];
};

// Host helpers shared by the render entry points (api.cpp).
vrc_status check_params(vrc_context* ctx, const vrc_render_params* p);
vrc_status fill_params(vrc_context* ctx, const vrc_volume* vol, const vrc_render_params* p, MarchParams& P);
// Device alpha table of a TF (256 floats, alpha' per alpha byte), cached on
// the TF per (opacity-corrected, correction exponent).
vrc_status tf_alpha(vrc_context* ctx, vrc_tf* tf, bool corrected, float kcorr, float** out);
// The 256 alphas themselves (host): a/255, opacity-corrected when `corrected`.
void tf_alpha_values(bool corrected, float kcorr, float out[256]);

// Kernel launchers (march.cu / volume.cu). Return cudaError_t.
cudaError_t launch_march(const MarchParams& p, int dtype, int compositing, int shading, int num_sms,
                         cudaStream_t s);
// Per compositing family (one translation unit each, compiled in parallel).
cudaError_t launch_march_dvr(const MarchParams& p, int dtype, int shading, int num_sms, cudaStream_t s);
cudaError_t launch_march_mip_iso(const MarchParams& p, int dtype, int compositing, int shading, int num_sms,
                                 cudaStream_t s);
cudaError_t launch_march_mop_mida(const MarchParams& p, int dtype, int compositing, int shading, int num_sms,
                                  cudaStream_t s);
cudaError_t launch_march_first_hit(const MarchParams& p, int dtype, int compositing, int num_sms, cudaStream_t s);
// Exact pre-integration table: one thread per (back, front) entry.
// tb: res float4 TF entries; a8: their alpha bytes; corr[k * 256 + a] =
// 1 - (1 - a/255)^(step * 200 / (k + 1)).
cudaError_t launch_preint_exact(const float4* tb, const uint8_t* a8, const float* corr, int res, float4* out,
                                cudaStream_t s);
cudaError_t launch_entry_exit(const MarchParams& p, float4* entry, float4* exitp, cudaStream_t s);
// Batch: zero the per-launch state and stamp the start time, then one
// persistent launch over every request's ray tiles (tile_prefix[r] = first
// tile of request r in launch order; n + 1 entries).
cudaError_t launch_batch_begin(unsigned long long* state, int nreq, cudaStream_t s);
cudaError_t launch_march_batch(const BatchReq* reqs, int nreq, const unsigned* tile_prefix, unsigned total_tiles,
                               unsigned long long* state, int compositing, int shading, int num_sms, cudaStream_t s);
// Copies brick ids[i] of `pool` to slot dst[i] of `cache` (brick_stride_bytes
// each), i in [0, n).
cudaError_t launch_brick_gather(const void* pool, const long long* ids, const long long* dst, long long n,
                                size_t brick_stride_bytes, void* cache, cudaStream_t s);
cudaError_t launch_brick_build(const void* linear, int dtype, const BrickLayout& L, void* bricks, cudaStream_t s);
// Half-resolution linear volume from a bricked one: voxel (x, y, z) = mean of
// the full-resolution voxels 2x..2x+1 (clamped to the volume) on each axis;
// integers summed exactly and divided by 8 with truncation.
cudaError_t launch_half_sample(const void* bricks, int dtype, const BrickLayout& L, const int dims1[3], void* out,
                               cudaStream_t s);
cudaError_t launch_brick_minmax(const void* bricks, int dtype, const BrickLayout& L, float* bmin, float* bmax,
                                cudaStream_t s);
// Min/max of normalised intensity per cell of edge C over the cell's voxels
// plus one voxel on the high side (clamped), from the linear volume.
cudaError_t launch_cell_minmax(const void* linear, int dtype, const int dims[3], int C, float* cmin, float* cmax,
                               cudaStream_t s);
// Writes ceil(ncells / 32) words: bit (c & 31) of word (c >> 5) is set when
// cell c may hold a sample with TF alpha > 0.
cudaError_t launch_occupancy(const float* bmin, const float* bmax, long long ncells, const int* alpha_prefix,
                             int tf_width, float rwm_scale, float rwm_offset, float tf_lo, float tf_hi,
                             uint32_t* occ, cudaStream_t s);
// occ_dist from the occupancy bits of an nc[0] x nc[1] x nc[2] cell grid
// (three separable passes; tmp holds as many bytes as dist).
cudaError_t launch_occ_distance(const uint32_t* occ, const int nc[3], uint8_t* dist, uint8_t* tmp, cudaStream_t s);
inline size_t occupancy_bytes(long long ncells) { return (size_t)((ncells + 31) / 32) * 4; }

// Process-unique id of a volume, TF or pre-integration table: identifies
// the derived data cached for it even when an address is reused later.
inline uint64_t next_uid() {
    static std::atomic<uint64_t> n{1};
    return n.fetch_add(1);
}

}  // namespace vrc

// Opaque handle definitions.
struct vrc_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::string last_error;
    // scratch (grown on demand, owned by the context)
    void* d_ee = nullptr;
    size_t ee_bytes = 0;
    void* d_out = nullptr;
    size_t out_bytes = 0;
    uint32_t* d_occ = nullptr;
    size_t occ_bytes = 0;
    uint32_t* d_occ_coarse = nullptr;
    size_t occ_coarse_bytes = 0;
    uint8_t* d_dist = nullptr;       // occ_dist of the skip cells, and the passes' scratch
    uint8_t* d_dist_tmp = nullptr;
    size_t dist_bytes = 0, dist_tmp_bytes = 0;
    int* d_prefix = nullptr;
    size_t prefix_bytes = 0;
    unsigned long long* d_counters = nullptr;  // 4 counters + status + tile counter
    // what d_occ / d_occ_coarse hold: (volume uid, TF or table uid, table
    // width, domain lo/hi bits, skip cell edge); both are pure functions of it
    uint64_t occ_key[6] = {0, 0, 0, 0, 0, 0};
};

struct vrc_cell_level {
    int C = 0;
    int nc[3] = {0, 0, 0};
    float* d_min = nullptr;
    float* d_max = nullptr;
    long long count() const { return (long long)nc[0] * nc[1] * nc[2]; }
};

struct vrc_volume {
    vrc_context* ctx = nullptr;
    uint64_t uid = vrc::next_uid();
    vrc_volume_desc desc{};

    vrc::BrickLayout L{};
    void* d_bricks = nullptr;     // device address of the brick pool
    void* h_bricks = nullptr;     // the pool's pinned host allocation (VRC_PLACE_HOST), else null
    size_t host_bytes = 0;
    // device cache of a host-resident pool: the bricks the current TF can
    // reach (non-empty, dilated by one brick), as many as cache_limit bytes
    // hold; the rest stay in the host pool and are read there
    size_t cache_limit = SIZE_MAX;     // bytes; 0 = no cache
    void* d_cache = nullptr;
    long long cache_slots = 0;         // slots allocated in d_cache
    int* d_slot = nullptr;             // nbricks entries: cache slot or -1
    uint32_t* d_occ_brick = nullptr;   // per-brick occupancy bits under the current TF
    long long* d_cache_ids = nullptr;  // bricks to gather (cache_slots entries)
    long long* d_cache_dst = nullptr;  // their slots
    std::vector<int> h_slot;           // host copy of d_slot
    std::vector<long long> h_slot_brick;  // slot -> brick, -1 = free
    std::vector<uint32_t> h_occ;       // occupancy the cache was filled for
    std::vector<long long> free_slots; // slots holding no brick
    std::vector<long long> pending;    // TF-wanted bricks not gathered yet, priority order
    size_t pending_pos = 0;
    size_t upload_budget = 0;          // bytes gathered per render, 0 = unlimited
    bool cache_valid = false;
    uint64_t cache_src_key[4] = {0, 0, 0, 0};  // (TF or table uid, width, domain bits) the plan was made for
    long long cache_reachable = 0;     // bricks the current TF can reach
    // refinement: bricks the last frame touched (d_used) displace bricks it
    // did not touch; h_last_used = frame that last touched a brick
    uint32_t* d_used = nullptr;
    std::vector<uint32_t> h_last_used;
    uint32_t frame = 0;
    bool used_pending = false;         // d_used holds the last frame's bits
    long long last_misses = 0;         // bricks touched without a slot in the last frame
    // a coarser level (2x2x2 means applied lod_level times), device
    // resident, sampled for bricks without a slot when lod_on
    void* d_lod = nullptr;
    vrc::BrickLayout lod_L{};
    int lod_level = 0;                 // level d_lod holds: 1 = half resolution, k = 2^-k
    bool lod_on = false;
    float* d_bmin = nullptr;
    float* d_bmax = nullptr;
    vrc_cell_level levels[4];  // skip cells of edge 2, 4, 8 and 16 (when smaller than the brick; 2 up to 2^30 cells)
    size_t bytes = 0;
    float vmin = 0.f, vmax = 0.f;
};

// The 2^3 cell level is built up to 2^VRC_CELL2_LOG2_MAX cells (2^30: an
// 8-Gvoxel volume, 8.6 GB of min/max tables).
#ifndef VRC_CELL2_LOG2_MAX
#define VRC_CELL2_LOG2_MAX 30
#endif

namespace vrc {
// The default skip-cell edge of a volume: 2 where it holds the 2^3 level,
// else 4.
inline int default_skip_cell(const vrc_volume* v) {
    for (const auto& lv : v->levels)
        if (lv.C == 2 && lv.d_min) return 2;
    return 4;
}
}  // namespace vrc

struct vrc_tf {
    vrc_context* ctx = nullptr;
    uint64_t uid = vrc::next_uid();
    int width = 0;
    float lo = 0.f, hi = 1.f;
    uint8_t* h_rgba = nullptr;
    uchar4* d_rgba8 = nullptr;  // the entries on the device
    // device alpha tables (256 floats) keyed by (opacity-corrected?, correction exponent bits)
    std::map<std::pair<int, uint32_t>, float*> alpha_tables;
    int* d_prefix = nullptr;  // prefix count of entries with alpha > 0 (width + 1 ints)
    const vrc_preint* preint = nullptr;  // attached pre-integration table (not owned)
};

struct vrc_preint {
    vrc_context* ctx = nullptr;
    uint64_t uid = vrc::next_uid();
    int res = 0;
    float step = 0.f;
    int use_integral = 0;
    float4* d_table = nullptr;  // res * res entries, [back * res + front]
    int* d_prefix = nullptr;    // prefix count of source entries with alpha > 0 (res + 1 ints)
};
