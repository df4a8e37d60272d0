// vrc_render_noalloc: a render that allocates nothing.
//
// Some callers cannot call cudaMalloc while they render: code running inside
// a CUDA graph capture or a real-time frame loop (cudaMalloc can synchronise
// the device), or a host application whose device memory is handed out by
// its own fixed-budget pool or by another runtime. vrc_render grows scratch
// buffers on demand; this variant keeps the same scratch -- the sample
// counters and tile counter, the per-render float4 TF table and the
// empty-space cell map -- in one fixed-size array in device global memory.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds NOALLOC_SCRATCH_BYTES of it until the process exits. Host
// code never uses the symbol as an address: at set-up (the first call on a
// device, with that device current) cudaGetSymbolAddress resolves its device
// address once, and that address is what the kernels receive. Make that first
// call before any stream capture. Every call shares the array and it keeps
// the last call's contents: the counters are cleared on each call, and calls
// that overlap on the GPU (other streams, or threads without ordering) race.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "vrc_internal.h"

namespace {

constexpr size_t COUNTER_BYTES = 256;                        // 16 x u64 counters, padded
constexpr size_t TF_BYTES = (size_t)4096 * sizeof(float4);    // widest TF table
constexpr size_t OCC_OFFSET = COUNTER_BYTES + TF_BYTES;
constexpr size_t SCRATCH_BYTES = OCC_OFFSET + (size_t)VRC_NOALLOC_MAX_CELLS / 8;  // one bit per cell

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

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

// Host staging for the TF table: thread-local static storage, no allocation
// per call.
thread_local float4 t_tf_host[4096];

vrc_status cuda_status(cudaError_t e) { return e == cudaSuccess ? VRC_OK : VRC_ERR_CUDA; }

}  // namespace

extern "C" vrc_status vrc_render_noalloc(const vrc_volume* vol, const vrc_tf* tf, const vrc_render_params* p,
                                         const float* d_entry, const float* d_exit, void* d_out, int out_format,
                                         void* stream) {
    if (!vol || !tf || !p || !d_out) return VRC_ERR_INVALID_ARG;
    vrc_status st = vrc::check_params(nullptr, p);
    if (st != VRC_OK) return st;
    if (out_format < VRC_OUT_RGBA8 || out_format > VRC_OUT_RGBA16) return VRC_ERR_INVALID_ARG;
    if (p->entry_exit_mode == VRC_EE_BUFFERS && (!d_entry || !d_exit)) return VRC_ERR_NOT_READY;
    if (tf->width > 4096) return VRC_ERR_SCRATCH_LIMIT;
    if (p->classification != VRC_CLASSIFY_TF) return VRC_ERR_UNSUPPORTED;  // TF classification only

    // empty-space cells: the requested level, else the brick grid (as vrc_render)
    const int want = p->skip_cell_size == 0 ? 8 : p->skip_cell_size;
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

    const int dev = vol->ctx ? vol->ctx->device : 0;
    if (dev < 0 || dev >= MAX_DEVICES) return VRC_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return cuda_status(e);
    if ((e = setup_device(dev)) != cudaSuccess) return cuda_status(e);
    unsigned char* scratch = static_cast<unsigned char*>(g_scratch_addr[dev]);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    vrc::MarchParams P;
    if ((st = vrc::fill_params(nullptr, vol, p, P)) != VRC_OK) return st;

    // TF table (r/255, g/255, b/255, alpha') into the scratch array; the same
    // host arithmetic as vrc_render's table, so results match it exactly
    const bool corrected = vrc::alpha_corrected(p->compositing, p->classification);
    const float kcorr = P.step * 200.f;
    for (int i = 0; i < tf->width; ++i) {
        const uint8_t* c = tf->h_rgba + 4 * i;
        float a = float(c[3]) / 255.f;
        if (corrected) a = 1.f - powf(1.f - a, kcorr);
        t_tf_host[i] = make_float4(float(c[0]) / 255.f, float(c[1]) / 255.f, float(c[2]) / 255.f, a);
    }
    float4* d_tf = reinterpret_cast<float4*>(scratch + COUNTER_BYTES);
    if ((e = cudaMemcpyAsync(d_tf, t_tf_host, tf->width * sizeof(float4), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_status(e);
    P.tf_table = d_tf;
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
    if ((e = vrc::launch_march(P, vol->desc.dtype, p->compositing, p->shading, g_num_sms[dev], s)) != cudaSuccess)
        return cuda_status(e);
    return VRC_OK;
}
