// Batched persistent render (host side): descriptors, launch order, graph
// capture and per-request latency statistics for vrc_batch_* (include/vrc.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "vrc_internal.h"

struct vrc_batch {
    vrc_context* ctx = nullptr;
    int n = 0;                              // requests in the launch
    int n_items = 0;                        // items given (requests left out included)
    int compositing = 0, shading = 0;
    std::vector<int> order;                 // launch position -> item index
    vrc::BatchReq* d_reqs = nullptr;
    unsigned* d_prefix = nullptr;
    unsigned long long* d_state = nullptr;  // [tile counter, start ns, samples, end ns per launch position]
    std::vector<uint32_t*> occ;             // per request: the cell bitmap
    std::vector<uint8_t*> dist;             // per request: the cells' distance field; one shared scratch last
    unsigned total_tiles = 0;
    int kernels = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

vrc_status bfail(vrc_context* ctx, vrc_status s, const std::string& m) {
    if (ctx) ctx->last_error = m;
    return s;
}

void release(vrc_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->d_reqs);
    cudaFree(b->d_prefix);
    cudaFree(b->d_state);
    for (auto* p : b->occ) cudaFree(p);
    for (auto* p : b->dist) cudaFree(p);
    delete b;
}

// Select the empty-space level for a request (as vrc_render does).
void pick_level(const vrc_volume* vol, int want, const float** mn, const float** mx, int* C, int nc[3]) {
    *mn = vol->d_bmin;
    *mx = vol->d_bmax;
    *C = vol->L.B;
    for (int i = 0; i < 3; ++i) nc[i] = vol->L.nb[i];
    for (const auto& lv : vol->levels)
        if (lv.C == want && lv.d_min) {
            *mn = lv.d_min;
            *mx = lv.d_max;
            *C = lv.C;
            for (int i = 0; i < 3; ++i) nc[i] = lv.nc[i];
        }
}

}  // namespace

namespace {

// Checks one request against the batch's rules; `first` is the first valid
// request (its compositing and shading are the batch's), or null.
vrc_status check_item(vrc_context* ctx, const vrc_batch_item& it, int i, const vrc_batch_item* first) {
    if (!it.volume || !it.tf || !it.out || it.volume->ctx != ctx || it.tf->ctx != ctx)
        return bfail(ctx, VRC_ERR_INVALID_ARG, "vrc_batch_create: item " + std::to_string(i) + " is incomplete");
    vrc_status st = vrc::check_params(ctx, &it.params);
    if (st != VRC_OK) return st;
    if (it.params.entry_exit_mode != VRC_EE_ANALYTIC)
        return bfail(ctx, VRC_ERR_UNSUPPORTED, "vrc_batch_create: batched requests use analytic entry/exit");
    if (it.params.compositing > VRC_ISO || it.params.classification != VRC_CLASSIFY_TF)
        return bfail(ctx, VRC_ERR_UNSUPPORTED,
                     "vrc_batch_create: batches take dvr / mip / iso compositing with TF classification");
    if (first && (it.params.compositing != first->params.compositing || it.params.shading != first->params.shading))
        return bfail(ctx, VRC_ERR_UNSUPPORTED, "vrc_batch_create: all requests must share compositing and shading");
    if (it.out_format < VRC_OUT_RGBA8 || it.out_format > VRC_OUT_RGBA16)
        return bfail(ctx, VRC_ERR_INVALID_ARG, "vrc_batch_create: unknown output format");
    vrc::MarchParams P;  // camera and region checks
    return vrc::fill_params(ctx, it.volume, &it.params, P);
}

// status == nullptr: any invalid request fails the batch. Otherwise invalid
// requests are left out and status[i] holds each request's vrc_status.
vrc_status create_batch(vrc_context* ctx, const vrc_batch_item* all, int n_items, int* status, vrc_batch** out) {
    if (!ctx || !all || !out || n_items < 1) return bfail(ctx, VRC_ERR_INVALID_ARG, "vrc_batch_create: bad arguments");
    *out = nullptr;
    std::vector<int> valid;  // launch requests -> item index
    const vrc_batch_item* first = nullptr;
    std::string first_error;
    for (int i = 0; i < n_items; ++i) {
        const vrc_status st = check_item(ctx, all[i], i, first);
        if (status) status[i] = st;
        if (st != VRC_OK) {
            if (!status) return st;
            if (first_error.empty()) first_error = ctx->last_error;
            continue;
        }
        if (!first) first = &all[i];
        valid.push_back(i);
    }
    if (valid.empty()) return bfail(ctx, VRC_ERR_INVALID_ARG, "vrc_batch_create: no valid request (" + first_error + ")");
    const int n = (int)valid.size();
    std::vector<vrc_batch_item> items(n);
    for (int k = 0; k < n; ++k) items[k] = all[valid[k]];
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return bfail(ctx, VRC_ERR_CUDA, cudaGetErrorString(e));
    vrc_batch* b = new (std::nothrow) vrc_batch();
    if (!b) return VRC_ERR_OUT_OF_MEMORY;
    b->ctx = ctx;
    b->n = n;
    b->n_items = n_items;
    b->compositing = items[0].params.compositing;
    b->shading = items[0].params.shading;

    std::vector<vrc::BatchReq> reqs(n);
    std::vector<double> cost(n);
    struct Occ {
        const float *mn, *mx;
        long long cells;
        uint32_t* map;
        const vrc_tf* tf;
        const vrc_volume* vol;
        uint8_t* dist;
        int nc[3];
    };
    std::vector<Occ> occ_jobs;
    long long max_cells = 0;
    for (int i = 0; i < n; ++i) {
        const vrc_batch_item& it = items[i];
        vrc::BatchReq& R = reqs[i];
        std::memset(&R, 0, sizeof(R));
        vrc_status st = vrc::fill_params(ctx, it.volume, &it.params, R.P);
        if (st != VRC_OK) {
            release(b);
            return st;
        }
        R.dtype = it.volume->desc.dtype;
        float* alpha = nullptr;
        if ((st = vrc::tf_alpha(ctx, const_cast<vrc_tf*>(it.tf), it.params.compositing == VRC_DVR, R.P.step * 200.f,
                                &alpha)) != VRC_OK) {
            release(b);
            return st;
        }
        R.P.tf_rgba8 = it.tf->d_rgba8;
        R.P.tf_alpha = alpha;
        R.P.tf_width = it.tf->width;
        R.P.tf_lo = it.tf->lo;
        R.P.tf_hi = it.tf->hi;
        R.P.out = it.out;
        R.P.out_format = it.out_format;
        if (it.params.empty_space_skipping) {
            // as vrc_render: the finest of 2^3 and 4^3 cells by default, and
            // the cells' distance field, so an empty run jumps the whole empty
            // box around its cell
            const float *mn, *mx;
            int C, nc[3];
            pick_level(it.volume, it.params.skip_cell_size == 0 ? vrc::default_skip_cell(it.volume) : it.params.skip_cell_size,
                       &mn, &mx, &C, nc);
            const long long cells = (long long)nc[0] * nc[1] * nc[2];
            uint32_t* map = nullptr;
            uint8_t* dist = nullptr;
            if ((e = cudaMalloc((void**)&map, vrc::occupancy_bytes(cells))) == cudaSuccess) b->occ.push_back(map);
            if (e == cudaSuccess && (e = cudaMalloc((void**)&dist, (size_t)cells)) == cudaSuccess) b->dist.push_back(dist);
            if (e != cudaSuccess) {
                release(b);
                return bfail(ctx, VRC_ERR_OUT_OF_MEMORY, "vrc_batch_create: occupancy allocation");
            }
            occ_jobs.push_back({mn, mx, cells, map, it.tf, it.volume, dist, {nc[0], nc[1], nc[2]}});
            max_cells = std::max(max_cells, cells);
            R.P.occupancy = map;
            R.P.occ_dist = dist;
            int sh = 0;
            while ((1 << sh) < C) ++sh;
            R.P.cshift = sh;
            for (int k = 0; k < 3; ++k) R.P.nc[k] = nc[k];
            const int maxdim = std::max(it.volume->desc.dims[0], std::max(it.volume->desc.dims[1], it.volume->desc.dims[2]));
            R.P.skip_margin = 0.01f + 2e-5f * float(maxdim);
        }
        const int maxdim = std::max(it.volume->desc.dims[0], std::max(it.volume->desc.dims[1], it.volume->desc.dims[2]));
        cost[i] = double(it.params.width) * it.params.height * maxdim * it.params.sampling_rate;
    }
    // longest requests first, so the tail of the launch holds short tiles
    b->order.resize(n);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) { return cost[a] > cost[c]; });
    std::vector<vrc::BatchReq> ordered(n);
    std::vector<unsigned> prefix(n + 1, 0);
    for (int k = 0; k < n; ++k) {
        ordered[k] = reqs[b->order[k]];
        b->order[k] = valid[b->order[k]];  // launch position -> item index
        const unsigned long long t = (unsigned long long)ordered[k].P.tiles_x * ordered[k].P.tiles_y;
        if (prefix[k] + t > 0xffffffffULL) {
            release(b);
            return bfail(ctx, VRC_ERR_INVALID_ARG, "vrc_batch_create: too many ray tiles in one batch");
        }
        prefix[k + 1] = prefix[k] + (unsigned)t;
    }
    b->total_tiles = prefix[n];
    if ((e = cudaMalloc((void**)&b->d_reqs, n * sizeof(vrc::BatchReq))) != cudaSuccess ||
        (e = cudaMalloc((void**)&b->d_prefix, (n + 1) * sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMalloc((void**)&b->d_state, (3 + n) * sizeof(unsigned long long))) != cudaSuccess) {
        release(b);
        return bfail(ctx, VRC_ERR_OUT_OF_MEMORY, "vrc_batch_create: descriptor allocation");
    }
    if ((e = cudaMemcpy(b->d_reqs, ordered.data(), n * sizeof(vrc::BatchReq), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_prefix, prefix.data(), (n + 1) * sizeof(unsigned), cudaMemcpyHostToDevice)) != cudaSuccess) {
        release(b);
        return bfail(ctx, VRC_ERR_CUDA, cudaGetErrorString(e));
    }
    // Empty-space maps, built once: a request's cell map and distance field
    // depend only on its volume, TF and cell edge, none of which changes
    // after creation, so launches replay the march alone.
    cudaStream_t s = ctx->stream;
    if (!occ_jobs.empty()) {
        uint8_t* dist_tmp = nullptr;  // scratch of the distance passes, shared by the requests in turn
        if ((e = cudaMalloc((void**)&dist_tmp, (size_t)max_cells)) != cudaSuccess) {
            release(b);
            return bfail(ctx, VRC_ERR_OUT_OF_MEMORY, "vrc_batch_create: distance scratch allocation");
        }
        cudaError_t me = cudaSuccess;
        for (const Occ& j : occ_jobs) {
            if (me == cudaSuccess)
                me = vrc::launch_occupancy(j.mn, j.mx, j.cells, j.tf->d_prefix, j.tf->width, j.vol->desc.rwm_scale,
                                           j.vol->desc.rwm_offset, j.tf->lo, j.tf->hi, j.map, s);
            if (me == cudaSuccess) me = vrc::launch_occ_distance(j.map, j.nc, j.dist, dist_tmp, s);
        }
        if (me == cudaSuccess) me = cudaStreamSynchronize(s);
        cudaFree(dist_tmp);
        if (me != cudaSuccess) {
            release(b);
            return bfail(ctx, VRC_ERR_CUDA, std::string("vrc_batch_create: empty-space maps: ") + cudaGetErrorString(me));
        }
    }
    // capture: state reset + start stamp, one persistent march
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        release(b);
        return bfail(ctx, VRC_ERR_CUDA, std::string("vrc_batch_create: capture: ") + cudaGetErrorString(e));
    }
    cudaError_t ce = vrc::launch_batch_begin(b->d_state, n, s);
    if (ce == cudaSuccess)
        ce = vrc::launch_march_batch(b->d_reqs, n, b->d_prefix, b->total_tiles, b->d_state, b->compositing,
                                     b->shading, ctx->num_sms, s);
    e = cudaStreamEndCapture(s, &b->graph);
    if (ce != cudaSuccess || e != cudaSuccess) {
        release(b);
        return bfail(ctx, VRC_ERR_CUDA, std::string("vrc_batch_create: capture failed: ") +
                                            cudaGetErrorString(ce != cudaSuccess ? ce : e));
    }
    b->kernels = 2;
    if ((e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess) {
        release(b);
        return bfail(ctx, VRC_ERR_CUDA, std::string("vrc_batch_create: instantiate: ") + cudaGetErrorString(e));
    }
    *out = b;
    return VRC_OK;
}

}  // namespace

extern "C" {

vrc_status vrc_batch_create(vrc_context* ctx, const vrc_batch_item* items, int n, vrc_batch** out) {
    return create_batch(ctx, items, n, nullptr, out);
}

vrc_status vrc_batch_create_isolated(vrc_context* ctx, const vrc_batch_item* items, int n, int* status,
                                     vrc_batch** out) {
    if (!status) return bfail(ctx, VRC_ERR_INVALID_ARG, "vrc_batch_create_isolated: null status array");
    return create_batch(ctx, items, n, status, out);
}

vrc_status vrc_batch_launch(vrc_batch* b) {
    if (!b) return VRC_ERR_INVALID_ARG;
    cudaError_t e = cudaGraphLaunch(b->exec, b->ctx->stream);
    if (e != cudaSuccess) return bfail(b->ctx, VRC_ERR_CUDA, std::string("vrc_batch_launch: ") + cudaGetErrorString(e));
    return VRC_OK;
}

vrc_status vrc_batch_stats_get(vrc_batch* b, float* latency_ms, vrc_batch_stats* st) {
    if (!b) return VRC_ERR_INVALID_ARG;
    cudaError_t e = cudaStreamSynchronize(b->ctx->stream);
    std::vector<unsigned long long> h(3 + b->n);
    if (e == cudaSuccess)
        e = cudaMemcpy(h.data(), b->d_state, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return bfail(b->ctx, VRC_ERR_CUDA, cudaGetErrorString(e));
    std::vector<float> lat(b->n);
    float mx = 0.f;
    if (latency_ms)
        for (int i = 0; i < b->n_items; ++i) latency_ms[i] = -1.f;  // requests left out of the launch
    for (int k = 0; k < b->n; ++k) {
        const unsigned long long end = h[3 + k];
        lat[k] = end > h[1] ? float(double(end - h[1]) * 1e-6) : 0.f;
        mx = std::max(mx, lat[k]);
        if (latency_ms) latency_ms[b->order[k]] = lat[k];
    }
    if (st) {
        std::vector<float> sorted = lat;
        std::sort(sorted.begin(), sorted.end());
        auto pct = [&](double q) {
            const double pos = q * (sorted.size() - 1);
            const size_t i = (size_t)pos;
            const double fr = pos - i;
            return float(i + 1 < sorted.size() ? sorted[i] * (1 - fr) + sorted[i + 1] * fr : sorted[i]);
        };
        st->samples = double(h[2]);
        st->total_ms = mx;
        st->latency_p50_ms = pct(0.5);
        st->latency_p99_ms = pct(0.99);
        st->latency_max_ms = mx;
        st->kernels_per_launch = b->kernels;
    }
    return VRC_OK;
}

vrc_status vrc_batch_destroy(vrc_batch* b) {
    if (!b) return VRC_ERR_INVALID_ARG;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    release(b);
    return VRC_OK;
}

}  // extern "C"
