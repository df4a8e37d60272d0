// CudaRaycaster: Voreen's raycaster processor surface (ports, properties,
// isReady, process, error behaviour) in C++ over the C ABI, and the C shim of
// include/vrc_processor.h. Reference: CPURaycaster
// (modules/base/processors/render/cpuraycaster.cpp:51-206), VolumeRaycaster
// (src/core/processors/volumeraycaster.cpp:42-157, 312-322, 348-375),
// SingleVolumeRaycaster::process interaction mode
// (modules/base/processors/render/singlevolumeraycaster.cpp:253-256) and the
// brick streaming properties of SingleOctreeRaycasterCL
// (modules/opencl/processors/singleoctreeraycastercl.cpp:294-305, 780-894).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/vrc_processor.h"

namespace {

const char* const COMPOSITING[] = {"dvr", "mip", "iso", "mop", "mida", "fhp", "fhn"};
const char* const CLASSIFICATION[] = {"transfer-function", "pre-integrated-gpu", "pre-integrated-cpu",
                                      "pre-integrated-approximation"};
const int PREINT_TABLE_SIZES[] = {0, 256, 512, 1024};

int index_of(const char* const* names, int n, const std::string& s) {
    for (int i = 0; i < n; ++i)
        if (s == names[i]) return i;
    return -1;
}

// What the volume inport carries: a borrowed host volume and its metadata.
struct VolumePortData {
    vrc_volume_desc desc{};
    const void* voxels = nullptr;
    unsigned generation = 0;  // bumped by every setData, as a new VolumeBase would be
};

// TransFunc1DKeysProperty: keys + gamma + thresholds, and the width and
// domain fitted to the volume.
struct TransFunc1DKeys {
    std::vector<vrc_tf_key> keys;
    float gamma = 1.f, threshold_lo = 0.f, threshold_hi = 1.f;
    float domain_lo = 0.f, domain_hi = 1.f;
    bool domain_fitted = false;
    int width = 256;
    TransFunc1DKeys() {
        vrc_tf_key a{}, b{};
        a.intensity = 0.f;
        b.intensity = 1.f;
        for (int c = 0; c < 4; ++c) b.color_l[c] = b.color_r[c] = 255;
        keys = {a, b};
    }
};

}  // namespace

class CudaRaycaster {
   public:
    explicit CudaRaycaster(int device) : device_(device) { vrc_render_params_default(&defaults_, 1, 1); }
    ~CudaRaycaster() { deinitialize(); }

    // ---- ports ("volumehandle.volumehandle", "image.entrypoints", "image.exitpoints", "image.output")
    VolumePortData volume;
    const float* entry = nullptr;
    const float* exitp = nullptr;
    int ee_w = 0, ee_h = 0;
    int out_w = 0, out_h = 0;  // render target size for analytic entry/exit
    std::vector<float> output;
    bool has_output = false;

    // ---- properties (ids and defaults of the reference)
    float samplingRate = 2.f;         // 0.01 .. 20
    float isoValue = 0.5f;
    std::string compositing = "dvr";  // dvr / mip / iso / mop / mida / fhp / fhn
    std::string shading = "none";     // none / phong
    std::string gradient = "central-differences";
    std::string classification = "transfer-function";
    int preIntegrationTableSize = 0;  // deriveFromBitDepth / 256 / 512 / 1024
    float gammaValue = 0.f;           // MIDA, -1 .. 1
    int interactionCoarseness = 3;    // 1 .. 8
    float interactionQuality = 1.f;   // 0.01 .. 1
    bool enableClipping = false;
    int clipRegion[6] = {0, 0, 0, 0, 0, 0};
    bool clipRegionSet = false;
    TransFunc1DKeys transferFunction;
    float lightPosition[4] = {2.3f, 1.5f, 1.5f, 1.f};
    float lightAmbient[4] = {0.4f, 0.4f, 0.4f, 1.f};
    float lightDiffuse[4] = {0.8f, 0.8f, 0.8f, 1.f};
    float lightSpecular[4] = {0.6f, 0.6f, 0.6f, 1.f};
    float materialShininess = 60.f;
    bool applyLightAttenuation = false;
    float lightAttenuation[3] = {1.f, 0.f, 0.f};
    vrc_camera camera{};
    std::string brickPoolPlacement = "device";  // device / host
    int brickBufferSizeMB = 0;                  // 0 = bounded by free device memory
    int brickUploadBudgetMB = 32;               // 1 .. 1024
    bool useLevelOfDetail = false;
    bool useIterativeRefinement = true;

    std::string lastError;
    vrc_render_stats lastStats{};
    bool invalidated = false;

    void initialize() {
        if (!ctx_) vrc_context_create(device_, &ctx_);
    }

    void deinitialize() {
        drop_preint();
        if (vol_) vrc_volume_destroy(vol_);
        vol_ = nullptr;
        if (ctx_) vrc_context_destroy(ctx_);
        ctx_ = nullptr;
    }

    // CPURaycaster::isReady (cpuraycaster.cpp:82-84): volume and both entry/exit ports.
    bool isReady() const { return volume.voxels && entry && exitp; }

    void process(bool analytic, bool interacting);

   private:
    int device_;
    vrc_render_params defaults_{};
    vrc_context* ctx_ = nullptr;
    vrc_volume* vol_ = nullptr;
    unsigned vol_generation_ = 0;
    int vol_placement_ = -1;
    // PreIntegrationTableMap with its default size 1: one table, keyed by
    // everything it is built from (preintegrationtablemap.cpp:59-95)
    vrc_preint* preint_ = nullptr;
    std::string preint_key_;
    long long last_missed_ = -1;

    void error(const std::string& m) {
        lastError = m;
        std::fprintf(stderr, "[voreen.CudaRaycaster] %s\n", m.c_str());
    }
    bool check(vrc_status s, const char* what) {
        if (s == VRC_OK) return true;
        const char* d = ctx_ ? vrc_last_error(ctx_) : "";
        error(std::string(what) + ": " + vrc_status_string(s) + (d && *d ? std::string(": ") + d : ""));
        return false;
    }
    void drop_preint() {
        if (preint_) vrc_preint_destroy(preint_);
        preint_ = nullptr;
        preint_key_.clear();
    }
    bool ensure_volume(int placement);
    void fit_tf();
    vrc_preint* preint_table(float step, bool* ok);
};

bool CudaRaycaster::ensure_volume(int placement) {
    if (vol_ && vol_generation_ == volume.generation && vol_placement_ == placement) return true;
    if (vol_) vrc_volume_destroy(vol_);
    vol_ = nullptr;
    if (!check(vrc_volume_upload_placed(ctx_, &volume.desc, volume.voxels, 0, 0, placement, &vol_), "volume upload"))
        return false;
    vol_generation_ = volume.generation;
    vol_placement_ = placement;
    return true;
}

// TF width from the volume's bit depth, and on first use the domain from its
// real-world min/max (transfuncpropertybase.cpp:134-174, transfunc1dkeysproperty.cpp:94-140).
void CudaRaycaster::fit_tf() {
    TransFunc1DKeys& t = transferFunction;
    t.width = vrc_tf_table_width(volume.desc.dtype);
    if (!t.domain_fitted && t.domain_lo == 0.f && t.domain_hi == 1.f) {
        float lo = 0.f, hi = 1.f;
        vrc_volume_minmax(vol_, &lo, &hi);
        const float s = volume.desc.rwm_scale, o = volume.desc.rwm_offset;
        t.domain_lo = lo * s + o;
        t.domain_hi = hi * s + o;
        t.domain_fitted = true;
    }
}

vrc_preint* CudaRaycaster::preint_table(float step, bool* ok) {
    *ok = false;
    const TransFunc1DKeys& t = transferFunction;
    const int res = vrc_preint_resolution(t.width, preIntegrationTableSize);
    const int integral = classification == "pre-integrated-approximation" ? 1 : 0;
    std::string key(reinterpret_cast<const char*>(t.keys.data()), t.keys.size() * sizeof(vrc_tf_key));
    char buf[128];
    std::snprintf(buf, sizeof(buf), "|%a|%d|%d|%a|%a|%a", step, res, integral, t.gamma, t.threshold_lo, t.threshold_hi);
    key += buf;
    if (!preint_ || key != preint_key_) {
        drop_preint();
        std::vector<uint8_t> src((size_t)res * 4);
        if (!check(vrc_preint_bake_source(t.keys.data(), (int)t.keys.size(), res, t.gamma, t.threshold_lo,
                                          t.threshold_hi, src.data()),
                   "pre-integration source"))
            return nullptr;
        if (!check(vrc_preint_create(ctx_, src.data(), res, step, integral, &preint_), "pre-integration table"))
            return nullptr;
        preint_key_ = key;
    }
    *ok = true;
    return preint_;
}

void CudaRaycaster::process(bool analytic, bool interacting) {
    has_output = false;
    invalidated = false;
    if (!(volume.voxels && (analytic || isReady()))) {
        error("not ready: volume and entry/exit points are required");
        return;
    }
    const int comp = index_of(COMPOSITING, 7, compositing);
    if (comp < 0 || (shading != "none" && shading != "phong")) {
        error("unsupported compositing/shading: " + compositing + "/" + shading);
        return;
    }
    const int cls = index_of(CLASSIFICATION, 4, classification);
    if (cls < 0 || std::find(std::begin(PREINT_TABLE_SIZES), std::end(PREINT_TABLE_SIZES), preIntegrationTableSize) ==
                       std::end(PREINT_TABLE_SIZES)) {
        error("unsupported classification: " + classification + "/" + std::to_string(preIntegrationTableSize));
        return;
    }
    if (classification == "pre-integrated-gpu") {
        // cpuraycaster.cpp:123-129
        error("CPU raycaster does not support computing the pre-integration table on the GPU. Falling back to CPU.");
        classification = "pre-integrated-cpu";
        return;
    }
    if (interactionCoarseness < 1 || interactionCoarseness > 8 || !(interactionQuality >= 0.01f) ||
        !(interactionQuality <= 1.f)) {
        error("interaction settings out of range: " + std::to_string(interactionCoarseness) + "/" +
              std::to_string(interactionQuality));
        return;
    }
    if (!(samplingRate >= 0.01f && samplingRate <= 20.f)) {
        error("samplingRate " + std::to_string(samplingRate) + " outside [0.01, 20]");
        return;
    }
    const int placement = brickPoolPlacement == "device" ? VRC_PLACE_DEVICE
                          : brickPoolPlacement == "host" ? VRC_PLACE_HOST
                                                         : -1;
    if (placement < 0 || brickBufferSizeMB < 0 || brickUploadBudgetMB < 1 || brickUploadBudgetMB > 1024) {
        error("brick settings out of range: " + brickPoolPlacement + "/" + std::to_string(brickBufferSizeMB) + "/" +
              std::to_string(brickUploadBudgetMB));
        return;
    }
    int W = 0, H = 0;
    if (analytic) {
        W = out_w > 0 ? out_w : 512;
        H = out_h > 0 ? out_h : 512;
    } else {
        W = ee_w;
        H = ee_h;
    }
    if (W < 1 || H < 1) {
        error("empty output size");
        return;
    }
    initialize();
    if (!ctx_) {
        error("no CUDA device");
        return;
    }
    if (!ensure_volume(placement)) return;
    if (placement == VRC_PLACE_HOST) {
        const size_t mb = (size_t)1 << 20;
        if (!check(vrc_volume_set_cache_limit(vol_, brickBufferSizeMB ? (size_t)brickBufferSizeMB * mb
                                                                      : ((size_t)1 << 62)),
                   "brick cache") ||
            !check(vrc_volume_set_cache_upload_budget(vol_, (size_t)brickUploadBudgetMB * mb), "brick cache") ||
            !check(vrc_volume_set_lod(vol_, useLevelOfDetail ? 1 : 0), "level of detail"))
            return;
    }
    fit_tf();
    TransFunc1DKeys& t = transferFunction;
    std::vector<uint8_t> rgba((size_t)t.width * 4);
    if (!check(vrc_tf_bake_keys(t.keys.data(), (int)t.keys.size(), t.width, t.gamma, t.threshold_lo, t.threshold_hi,
                                rgba.data()),
               "transfer function"))
        return;
    vrc_tf* tf = nullptr;
    if (!check(vrc_tf_create(ctx_, rgba.data(), t.width, t.domain_lo, t.domain_hi, &tf), "transfer function")) return;
    struct TfGuard {
        vrc_tf* t;
        ~TfGuard() { vrc_tf_destroy(t); }
    } guard{tf};

    vrc_render_params p = defaults_;
    p.width = W;
    p.height = H;
    p.sampling_rate = samplingRate;
    p.compositing = comp;
    p.shading = shading == "phong" ? VRC_SHADE_PHONG : VRC_SHADE_NONE;
    p.iso_value = isoValue;
    p.mida_gamma = gammaValue;
    if (interacting) p.sampling_rate = samplingRate * interactionQuality;  // getSamplingStepSize (:312-322)
    if (classification.rfind("pre-integrated", 0) == 0) {
        // the table is built for the step this frame marches with
        p.classification = VRC_CLASSIFY_PREINTEGRATED;
        bool ok = false;
        vrc_preint* table = preint_table(vrc_sampling_step(vol_, p.sampling_rate), &ok);
        if (!ok || !check(vrc_tf_set_preintegration(tf, table), "pre-integration table")) return;
    }
    std::memcpy(p.light_position, lightPosition, sizeof(p.light_position));
    std::memcpy(p.light_ambient, lightAmbient, sizeof(p.light_ambient));
    std::memcpy(p.light_diffuse, lightDiffuse, sizeof(p.light_diffuse));
    std::memcpy(p.light_specular, lightSpecular, sizeof(p.light_specular));
    p.material_shininess = materialShininess;
    p.apply_attenuation = applyLightAttenuation ? 1 : 0;
    std::memcpy(p.light_attenuation, lightAttenuation, sizeof(p.light_attenuation));
    p.camera = camera;
    p.entry_exit_mode = analytic ? VRC_EE_ANALYTIC : VRC_EE_BUFFERS;
    if (enableClipping && clipRegionSet) {
        p.enable_clipping = 1;
        for (int i = 0; i < 3; ++i) {
            p.clip_llf[i] = clipRegion[i];
            p.clip_urb[i] = clipRegion[3 + i];
        }
    }
    const bool coarse = interacting && interactionCoarseness > 1;
    output.assign((size_t)W * H * 4, 0.f);
    if (coarse) {
        // a coarse frame through the coarse pixel centres, rescaled with
        // GL_LINEAR to the output size (rescaleRendering, :348-375)
        p.width = std::max(1, W / interactionCoarseness);
        p.height = std::max(1, H / interactionCoarseness);
        p.entry_exit_mode = VRC_EE_ANALYTIC;
        void* small = nullptr;
        void* full = nullptr;
        cudaError_t e = cudaMalloc(&small, (size_t)p.width * p.height * 16);
        if (e == cudaSuccess) e = cudaMalloc(&full, (size_t)W * H * 16);
        bool ok = e == cudaSuccess;
        if (!ok) error(std::string("interaction buffers: ") + cudaGetErrorString(e));
        ok = ok && check(vrc_render(ctx_, vol_, tf, &p, nullptr, nullptr, 0, small, VRC_OUT_RGBA32F, 1, &lastStats),
                         "render");
        ok = ok && check(vrc_image_rescale(ctx_, small, p.width, p.height, full, W, H, VRC_OUT_RGBA32F), "rescale");
        ok = ok && check(vrc_context_synchronize(ctx_), "rescale");
        if (ok) {
            e = cudaMemcpy(output.data(), full, (size_t)W * H * 16, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) {
                error(std::string("rescale copy: ") + cudaGetErrorString(e));
                ok = false;
            }
        }
        cudaFree(small);
        cudaFree(full);
        if (!ok) return;
    } else if (!check(vrc_render(ctx_, vol_, tf, &p, analytic ? nullptr : entry, analytic ? nullptr : exitp, 0,
                                 output.data(), VRC_OUT_RGBA32F, 0, &lastStats),
                      "render")) {
        return;
    }
    out_w = W;
    out_h = H;
    has_output = true;
    lastError.clear();
    if (placement == VRC_PLACE_HOST && useIterativeRefinement) {
        // another frame helps while the cache is still filling, or while the
        // bricks read without a slot keep changing; a frame that can bring in
        // nothing new ends the refinement (singleoctreeraycastercl.cpp:780-838)
        long long cached = 0, reachable = 0, missed = 0;
        if (vrc_volume_cache_info(vol_, &cached, &reachable, &missed) == VRC_OK) {
            int nb[3] = {0, 0, 0};
            vrc_volume_brick_minmax(vol_, nb, nullptr, nullptr);
            const long long nbricks = (long long)nb[0] * nb[1] * nb[2];
            const long long brick_bytes = nbricks ? (long long)(vrc_volume_host_bytes(vol_) / nbricks) : 1;
            const long long capacity =
                brickBufferSizeMB ? ((long long)brickBufferSizeMB << 20) / std::max(1LL, brick_bytes) : reachable;
            invalidated = cached < std::min(reachable, capacity) || (missed > 0 && missed != last_missed_);
            last_missed_ = missed;
        }
    }
}

// ---- C shim ------------------------------------------------------------------

struct vrcp_processor {
    CudaRaycaster r;
    explicit vrcp_processor(int device) : r(device) {}
};

namespace {

float* floatv(CudaRaycaster& r, const std::string& id, int* n) {
    float* v = nullptr;
    *n = 4;
    if (id == "lightPosition") v = r.lightPosition;
    else if (id == "lightAmbient") v = r.lightAmbient;
    else if (id == "lightDiffuse") v = r.lightDiffuse;
    else if (id == "lightSpecular") v = r.lightSpecular;
    else if (id == "lightAttenuation") {
        v = r.lightAttenuation;
        *n = 3;
    }
    return v;
}
float* floatp(CudaRaycaster& r, const std::string& id) {
    if (id == "samplingRate") return &r.samplingRate;
    if (id == "isoValue") return &r.isoValue;
    if (id == "gammaValue") return &r.gammaValue;
    if (id == "interactionQuality") return &r.interactionQuality;
    if (id == "materialShininess") return &r.materialShininess;
    return nullptr;
}
int* intp(CudaRaycaster& r, const std::string& id) {
    if (id == "preIntegrationTableSize") return &r.preIntegrationTableSize;
    if (id == "interactionCoarseness") return &r.interactionCoarseness;
    if (id == "brickBufferSizeMB") return &r.brickBufferSizeMB;
    if (id == "brickUploadBudgetMB") return &r.brickUploadBudgetMB;
    return nullptr;
}
bool* boolp(CudaRaycaster& r, const std::string& id) {
    if (id == "enableClipping") return &r.enableClipping;
    if (id == "applyLightAttenuation") return &r.applyLightAttenuation;
    if (id == "useLevelOfDetail") return &r.useLevelOfDetail;
    if (id == "useIterativeRefinement") return &r.useIterativeRefinement;
    return nullptr;
}
std::string* stringp(CudaRaycaster& r, const std::string& id) {
    if (id == "compositing") return &r.compositing;
    if (id == "shading") return &r.shading;
    if (id == "gradient") return &r.gradient;
    if (id == "classification") return &r.classification;
    if (id == "brickPoolPlacement") return &r.brickPoolPlacement;
    return nullptr;
}
CudaRaycaster& R(const vrcp_processor* p) { return const_cast<vrcp_processor*>(p)->r; }

}  // namespace

extern "C" {

vrc_status vrcp_create(int device, vrcp_processor** out) {
    if (!out) return VRC_ERR_INVALID_ARG;
    *out = new (std::nothrow) vrcp_processor(device);
    return *out ? VRC_OK : VRC_ERR_OUT_OF_MEMORY;
}

vrc_status vrcp_destroy(vrcp_processor* p) {
    if (!p) return VRC_ERR_INVALID_ARG;
    delete p;
    return VRC_OK;
}

const char* vrcp_class_name(void) { return "CudaRaycaster"; }
const char* vrcp_category(void) { return "Raycasting"; }

vrc_status vrcp_set_float(vrcp_processor* p, const char* id, float v) {
    float* f = p && id ? floatp(p->r, id) : nullptr;
    if (!f) return VRC_ERR_INVALID_ARG;
    *f = v;
    return VRC_OK;
}

vrc_status vrcp_get_float(const vrcp_processor* p, const char* id, float* v) {
    float* f = p && id && v ? floatp(R(p), id) : nullptr;
    if (!f) return VRC_ERR_INVALID_ARG;
    *v = *f;
    return VRC_OK;
}

vrc_status vrcp_set_int(vrcp_processor* p, const char* id, int v) {
    if (!p || !id) return VRC_ERR_INVALID_ARG;
    if (int* i = intp(p->r, id)) {
        *i = v;
        return VRC_OK;
    }
    if (bool* b = boolp(p->r, id)) {
        *b = v != 0;
        return VRC_OK;
    }
    return VRC_ERR_INVALID_ARG;
}

vrc_status vrcp_get_int(const vrcp_processor* p, const char* id, int* v) {
    if (!p || !id || !v) return VRC_ERR_INVALID_ARG;
    if (int* i = intp(R(p), id)) {
        *v = *i;
        return VRC_OK;
    }
    if (bool* b = boolp(R(p), id)) {
        *v = *b ? 1 : 0;
        return VRC_OK;
    }
    return VRC_ERR_INVALID_ARG;
}

vrc_status vrcp_set_string(vrcp_processor* p, const char* id, const char* v) {
    std::string* s = p && id && v ? stringp(p->r, id) : nullptr;
    if (!s) return VRC_ERR_INVALID_ARG;
    *s = v;
    return VRC_OK;
}

vrc_status vrcp_get_string(const vrcp_processor* p, const char* id, char* buf, int cap) {
    std::string* s = p && id && buf && cap > 0 ? stringp(R(p), id) : nullptr;
    if (!s) return VRC_ERR_INVALID_ARG;
    std::snprintf(buf, (size_t)cap, "%s", s->c_str());
    return VRC_OK;
}

vrc_status vrcp_set_floatv(vrcp_processor* p, const char* id, const float* v, int n) {
    int m = 0;
    float* f = p && id && v ? floatv(p->r, id, &m) : nullptr;
    if (!f || n != m) return VRC_ERR_INVALID_ARG;
    std::memcpy(f, v, sizeof(float) * n);
    return VRC_OK;
}

vrc_status vrcp_get_floatv(const vrcp_processor* p, const char* id, float* v, int n) {
    int m = 0;
    float* f = p && id && v ? floatv(R(p), id, &m) : nullptr;
    if (!f || n != m) return VRC_ERR_INVALID_ARG;
    std::memcpy(v, f, sizeof(float) * n);
    return VRC_OK;
}

vrc_status vrcp_set_intv(vrcp_processor* p, const char* id, const int* v, int n) {
    if (!p || !id || std::string(id) != "clipRegion") return VRC_ERR_INVALID_ARG;
    if (!v) {
        p->r.clipRegionSet = false;
        return VRC_OK;
    }
    if (n != 6) return VRC_ERR_INVALID_ARG;
    std::memcpy(p->r.clipRegion, v, sizeof(p->r.clipRegion));
    p->r.clipRegionSet = true;
    return VRC_OK;
}

vrc_status vrcp_get_intv(const vrcp_processor* p, const char* id, int* v, int n) {
    if (!p || !id || !v || n != 6 || std::string(id) != "clipRegion") return VRC_ERR_INVALID_ARG;
    if (!p->r.clipRegionSet) return VRC_ERR_NOT_READY;
    std::memcpy(v, p->r.clipRegion, sizeof(p->r.clipRegion));
    return VRC_OK;
}

vrc_status vrcp_set_camera(vrcp_processor* p, const vrc_camera* c) {
    if (!p || !c) return VRC_ERR_INVALID_ARG;
    p->r.camera = *c;
    return VRC_OK;
}

vrc_status vrcp_get_camera(const vrcp_processor* p, vrc_camera* c) {
    if (!p || !c) return VRC_ERR_INVALID_ARG;
    *c = p->r.camera;
    return VRC_OK;
}

vrc_status vrcp_set_tf_keys(vrcp_processor* p, const vrc_tf_key* keys, int nkeys, float gamma, float threshold_lo,
                            float threshold_hi) {
    if (!p || nkeys < 0 || (nkeys > 0 && !keys)) return VRC_ERR_INVALID_ARG;
    auto& t = p->r.transferFunction;
    t.keys.assign(keys, keys + nkeys);
    t.gamma = gamma;
    t.threshold_lo = threshold_lo;
    t.threshold_hi = threshold_hi;
    return VRC_OK;
}

vrc_status vrcp_set_tf_domain(vrcp_processor* p, float lo, float hi, int fitted, int width) {
    if (!p || width < 2 || width > 4096) return VRC_ERR_INVALID_ARG;
    auto& t = p->r.transferFunction;
    t.domain_lo = lo;
    t.domain_hi = hi;
    t.domain_fitted = fitted != 0;
    t.width = width;
    return VRC_OK;
}

vrc_status vrcp_get_tf(const vrcp_processor* p, int* width, float* lo, float* hi, int* fitted) {
    if (!p || !width || !lo || !hi || !fitted) return VRC_ERR_INVALID_ARG;
    const auto& t = p->r.transferFunction;
    *width = t.width;
    *lo = t.domain_lo;
    *hi = t.domain_hi;
    *fitted = t.domain_fitted ? 1 : 0;
    return VRC_OK;
}

vrc_status vrcp_load_tf(vrcp_processor* p, const char* path) {
    if (!p || !path) return VRC_ERR_INVALID_ARG;
    vrc_tfi_info info;
    vrc_status st = vrc_tf_read_tfi(path, &info, nullptr, 0);
    if (st != VRC_OK) return st;
    std::vector<vrc_tf_key> keys((size_t)info.nkeys);
    if ((st = vrc_tf_read_tfi(path, &info, keys.data(), info.nkeys)) != VRC_OK) return st;
    auto& t = p->r.transferFunction;
    t.keys = keys;
    t.gamma = info.gamma;
    t.threshold_lo = info.threshold[0];
    t.threshold_hi = info.threshold[1];
    t.domain_lo = info.domain[0];
    t.domain_hi = info.domain[1];
    t.domain_fitted = true;  // the file's domain is kept
    return VRC_OK;
}

vrc_status vrcp_set_volume(vrcp_processor* p, const vrc_volume_desc* desc, const void* voxels) {
    if (!p || (voxels && !desc)) return VRC_ERR_INVALID_ARG;
    auto& v = p->r.volume;
    v.voxels = voxels;
    if (desc) v.desc = *desc;
    ++v.generation;
    return VRC_OK;
}

vrc_status vrcp_set_entry_exit(vrcp_processor* p, const float* entry, const float* exit_pts, int width, int height) {
    if (!p || ((entry || exit_pts) && (width < 1 || height < 1))) return VRC_ERR_INVALID_ARG;
    p->r.entry = entry;
    p->r.exitp = exit_pts;
    p->r.ee_w = width;
    p->r.ee_h = height;
    return VRC_OK;
}

vrc_status vrcp_set_output_size(vrcp_processor* p, int width, int height) {
    if (!p || width < 0 || height < 0) return VRC_ERR_INVALID_ARG;
    p->r.out_w = width;
    p->r.out_h = height;
    return VRC_OK;
}

int vrcp_is_ready(const vrcp_processor* p) { return p && p->r.isReady() ? 1 : 0; }

void vrcp_initialize(vrcp_processor* p) {
    if (p) p->r.initialize();
}

void vrcp_deinitialize(vrcp_processor* p) {
    if (p) p->r.deinitialize();
}

void vrcp_process(vrcp_processor* p, int analytic_entry_exit, int interacting) {
    if (p) p->r.process(analytic_entry_exit != 0, interacting != 0);
}

int vrcp_output(const vrcp_processor* p, const float** rgba, int* width, int* height) {
    if (!p || !p->r.has_output) return 0;
    if (rgba) *rgba = p->r.output.data();
    if (width) *width = p->r.out_w;
    if (height) *height = p->r.out_h;
    return 1;
}

const char* vrcp_last_error(const vrcp_processor* p) { return p ? p->r.lastError.c_str() : "no processor"; }

vrc_status vrcp_last_stats(const vrcp_processor* p, vrc_render_stats* stats) {
    if (!p || !stats) return VRC_ERR_INVALID_ARG;
    *stats = p->r.lastStats;
    return VRC_OK;
}

int vrcp_invalidated(const vrcp_processor* p) { return p && p->r.invalidated ? 1 : 0; }

}  // extern "C"
