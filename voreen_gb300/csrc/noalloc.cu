// vrc_render_noalloc: a render that allocates nothing.
//
// Some callers cannot call cudaMalloc while they render: a real-time frame
// loop (cudaMalloc can synchronise the device and stall the frame), or a
// host application whose device memory is handed out by its own
// fixed-budget pool or by another runtime. vrc_render grows scratch buffers
// on demand; this variant keeps the same scratch -- the sample counters and
// tile counter, the per-render alpha table, the empty-space cell map and its
// distance field (with the passes' scratch) -- in one fixed-size array in
// device global memory.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds NOALLOC_SCRATCH_BYTES of it until the process exits. Host
// code never uses the symbol as an address: at set-up (the first call on a
// device, with that device current) cudaGetSymbolAddress resolves its device
// address once, and that address is what the kernels receive. Every call
// shares the array and it keeps the last call's contents: the counters are
// cleared on each call, and calls that overlap on the GPU (other streams, or
// threads without ordering) race.
//
// The march reads the TF's RGBA8 entries where the TF object keeps them on
// the device, and a table of the (opacity-corrected) alpha of each of the 256
// alpha bytes, computed on the host with the same powf vrc_render uses and
// written into the scratch array by a small kernel whose by-value parameters
// carry it; so no host buffer is read after the call returns and the frame
// equals vrc_render's bit for bit.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "vrc_internal.h"

namespace {

constexpr size_t COUNTER_BYTES = 256;                        // 16 x u64 counters, padded
constexpr int MAX_TF = 4096;
constexpr size_t ALPHA_BYTES = 256 * sizeof(float);           // alpha per alpha byte of the TF
constexpr size_t OCC_OFFSET = COUNTER_BYTES + ALPHA_BYTES;
constexpr size_t DIST_OFFSET = OCC_OFFSET + (size_t)VRC_NOALLOC_MAX_CELLS / 8;     // one bit per cell
constexpr size_t SCRATCH_BYTES = DIST_OFFSET + 2 * (size_t)VRC_NOALLOC_MAX_CELLS;   // distance byte + pass scratch

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

// Kernel parameters of the alpha table build: the 256 alphas by value, so no
// host buffer is read after the launch.
struct AlphaArgs {
    float alpha[256];  // alpha' for each alpha byte
};

__global__ void alpha_table_kernel(const AlphaArgs a, float* out) { out[threadIdx.x] = a.alpha[threadIdx.x]; }

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[MAX_DEVICES] = {};
int g_num_sms[MAX_DEVICES] = {};

// Once per device, with that device current: resolve the scratch address.
cudaError_t setup_device(int dev) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_addr[dev]) return cudaSuccess;
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_num_sms[dev] = sms;
    g_scratch_addr[dev] = ptr;
    return cudaSuccess;
}

vrc_status cuda_status(cudaError_t e) { return e == cudaSuccess ? VRC_OK : VRC_ERR_CUDA; }

// Makes `dev` current for the call and puts the caller's device back on
// every return path.
struct DeviceScope {
    int prev = -1;
    cudaError_t enter(int dev) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) {
            prev = -1;
            return e;
        }
        return prev == dev ? cudaSuccess : cudaSetDevice(dev);
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

vrc_status render_noalloc(const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p, const float* d_entry,
                          const float* d_exit, void* d_out, int out_format, cudaStream_t s, int dev) {
    unsigned char* scratch = static_cast<unsigned char*>(g_scratch_addr[dev]);
    vrc::MarchParams P;
    vrc_status st = vrc::fill_params(nullptr, vol, p, P);
    if (st != VRC_OK) return st;

    // empty-space cells: the requested level, else the brick grid (as
    // vrc_render); by default the finest of 2^3, 4^3 and 8^3 whose cells fit
    // the scratch (2^3 up to 256^3 voxels, 4^3 up to 512^3)
    int want = p->skip_cell_size;
    if (want == 0) {
        want = 8;
        for (const auto& lv : vol->levels)
            if (lv.C < want && lv.C >= 2 && lv.d_min && lv.count() <= (long long)VRC_NOALLOC_MAX_CELLS) want = lv.C;
    }
    const float* cmin = vol->d_bmin;
    const float* cmax = vol->d_bmax;
    int C = vol->L.B;
    int nc[3] = {vol->L.nb[0], vol->L.nb[1], vol->L.nb[2]};
    for (const auto& lv : vol->levels)
        if (lv.C == want && lv.d_min) {
            cmin = lv.d_min;
            cmax = lv.d_max;
            C = lv.C;
            for (int i = 0; i < 3; ++i) nc[i] = lv.nc[i];
        }
    const long long ncells = (long long)nc[0] * nc[1] * nc[2];
    if (p->empty_space_skipping && ncells > (long long)VRC_NOALLOC_MAX_CELLS) return VRC_ERR_SCRATCH_LIMIT;

    // The TF's RGBA8 entries are read where the TF object keeps them on the
    // device; its alpha per alpha byte (vrc_render's host arithmetic) goes into
    // the scratch array.
    AlphaArgs args;
    vrc::tf_alpha_values(vrc::alpha_corrected(p->compositing, p->classification), P.step * 200.f, args.alpha);
    float* d_alpha = reinterpret_cast<float*>(scratch + COUNTER_BYTES);
    alpha_table_kernel<<<1, 256, 0, s>>>(args, d_alpha);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    P.tf_rgba8 = tf->d_rgba8;
    P.tf_alpha = d_alpha;
    P.tf_width = tf->width;
    P.tf_lo = tf->lo;
    P.tf_hi = tf->hi;
    if (p->entry_exit_mode == VRC_EE_BUFFERS) {
        P.entry = reinterpret_cast<const float4*>(d_entry);
        P.exitp = reinterpret_cast<const float4*>(d_exit);
    }
    P.out = d_out;
    P.out_format = out_format;
    if (p->empty_space_skipping) {
        uint32_t* occ = reinterpret_cast<uint32_t*>(scratch + OCC_OFFSET);
        if ((e = vrc::launch_occupancy(cmin, cmax, ncells, tf->d_prefix, tf->width, vol->desc.rwm_scale,
                                       vol->desc.rwm_offset, tf->lo, tf->hi, occ, s)) != cudaSuccess)
            return cuda_status(e);
        P.occupancy = occ;
        // the cells' distance field: an empty run jumps the whole empty box
        // around its cell (MIP's max-based skipping is not taken here)
        uint8_t* dist = scratch + DIST_OFFSET;
        if ((e = vrc::launch_occ_distance(occ, nc, dist, dist + VRC_NOALLOC_MAX_CELLS, s)) != cudaSuccess)
            return cuda_status(e);
        P.occ_dist = dist;
        int shift = 0;
        while ((1 << shift) < C) ++shift;
        P.cshift = shift;
        for (int i = 0; i < 3; ++i) P.nc[i] = nc[i];
        const int maxdim = std::max(vol->desc.dims[0], std::max(vol->desc.dims[1], vol->desc.dims[2]));
        P.skip_margin = 0.01f + 2e-5f * float(maxdim);
    }
    // counters, status and tile counter start at zero on every call
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(scratch);
    if ((e = cudaMemsetAsync(counters, 0, COUNTER_BYTES, s)) != cudaSuccess) return cuda_status(e);
    P.counters = counters;
    P.status = reinterpret_cast<int*>(counters + 4);
    P.tile_counter = reinterpret_cast<unsigned int*>(counters + 5);
    return cuda_status(vrc::launch_march(P, vol->desc.dtype, p->compositing, p->shading, g_num_sms[dev], s));
}

}  // namespace

extern "C" vrc_status vrc_render_noalloc(const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p,
                                         const float* d_entry, const float* d_exit, void* d_out, int out_format,
                                         void* stream) {
    if (!vol || !tf || !p || !d_out) return VRC_ERR_INVALID_ARG;
    if (vol->ctx != tf->ctx) return VRC_ERR_INVALID_ARG;  // handles of two contexts (possibly two GPUs)
    vrc_status st = vrc::check_params(nullptr, p);
    if (st != VRC_OK) return st;
    if (out_format < VRC_OUT_RGBA8 || out_format > VRC_OUT_RGBA16) return VRC_ERR_INVALID_ARG;
    if (p->entry_exit_mode == VRC_EE_BUFFERS && (!d_entry || !d_exit)) return VRC_ERR_NOT_READY;
    if (tf->width > MAX_TF) return VRC_ERR_SCRATCH_LIMIT;
    if (p->classification != VRC_CLASSIFY_TF) return VRC_ERR_UNSUPPORTED;  // TF classification only

    const int dev = vol->ctx ? vol->ctx->device : 0;
    if (dev < 0 || dev >= MAX_DEVICES) return VRC_ERR_INVALID_ARG;
    DeviceScope scope;
    cudaError_t e = scope.enter(dev);
    if (e != cudaSuccess) return cuda_status(e);
    if ((e = setup_device(dev)) != cudaSuccess) return cuda_status(e);
    return render_noalloc(vol, tf, p, d_entry, d_exit, d_out, out_format, static_cast<cudaStream_t>(stream), dev);
}
