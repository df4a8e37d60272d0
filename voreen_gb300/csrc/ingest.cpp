// Volume ingest from Voreen's .vvd format (modules/core/io/vvdvolumereader.cpp,
// vvdformat.cpp): the XML header's RawData (format, dimensions, raw file
// name either as a `filename` attribute or as the VoreenFilePathHelper path
// list, src/core/utils/voreenfilepathhelper.cpp:73-110), the Offset, Spacing
// and RealWorldMapping meta items and the VolumeMinMax derived item.
//
// The loader streams the raw file through two pinned host chunks: chunk i is
// read from the file while chunk i - 1 is copied to the device on the context
// stream, into a linear device buffer that is then bricked (with its min/max
// tables) on the device by vrc_volume_upload.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "vrc_internal.h"

namespace {

vrc_status ifail(vrc_context* ctx, vrc_status st, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return st;
}

bool read_file(const char* path, std::string& out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
    std::fclose(f);
    return true;
}

// Value of attribute `name` inside the tag text [b, e), or empty.
bool attr(const std::string& s, size_t b, size_t e, const char* name, std::string& val) {
    const std::string key = std::string(name) + "=\"";
    size_t p = b;
    while ((p = s.find(key, p)) != std::string::npos && p < e) {
        if (p == 0 || s[p - 1] == ' ' || s[p - 1] == '\t' || s[p - 1] == '\n' || s[p - 1] == '\r') {
            const size_t v0 = p + key.size();
            const size_t v1 = s.find('"', v0);
            if (v1 == std::string::npos || v1 > e) return false;
            val = s.substr(v0, v1 - v0);
            return true;
        }
        p += key.size();
    }
    return false;
}

// [begin, end) of the first start tag `<tag` at or after `from` (the tag text).
bool find_tag(const std::string& s, const char* tag, size_t from, size_t& b, size_t& e) {
    const std::string open = std::string("<") + tag;
    size_t p = from;
    while ((p = s.find(open, p)) != std::string::npos) {
        const char c = p + open.size() < s.size() ? s[p + open.size()] : '\0';
        if (c == ' ' || c == '>' || c == '/' || c == '\n' || c == '\t' || c == '\r') {
            b = p;
            e = s.find('>', p);
            return e != std::string::npos;
        }
        p += open.size();
    }
    return false;
}

// The <value .../> of <MetaItem name="name" ...>.
bool meta_value(const std::string& s, const char* name, size_t& b, size_t& e) {
    size_t p = 0, tb, te;
    while (find_tag(s, "MetaItem", p, tb, te)) {
        std::string n;
        if (attr(s, tb, te, "name", n) && n == name) return find_tag(s, "value", te, b, e);
        p = te;
    }
    return false;
}

bool to_float(const std::string& v, float& out) {
    char* end = nullptr;
    out = std::strtof(v.c_str(), &end);
    return end && end != v.c_str();
}

bool file_exists(const std::string& p) {
    FILE* f = std::fopen(p.c_str(), "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

std::string dir_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string(".") : path.substr(0, k);
}

}  // namespace

extern "C" {

vrc_status vrc_vvd_read_header(const char* vvd_path, vrc_vvd_info* info) {
    if (!vvd_path || !info) return VRC_ERR_INVALID_ARG;
    std::memset(info, 0, sizeof(*info));
    std::string s;
    if (!read_file(vvd_path, s)) return VRC_ERR_NOT_READY;
    size_t b, e;
    if (!find_tag(s, "RawData", 0, b, e)) {
        // RawDataNoExternalFile (voxels in the XML) and multi-channel formats are not read
        return VRC_ERR_UNSUPPORTED;
    }
    std::string fmt, x, y, z;
    if (!attr(s, b, e, "format", fmt) || !attr(s, b, e, "x", x) || !attr(s, b, e, "y", y) || !attr(s, b, e, "z", z))
        return VRC_ERR_INVALID_ARG;
    if (fmt == "uint8") info->dtype = VRC_U8;
    else if (fmt == "uint16") info->dtype = VRC_U16;
    else if (fmt == "float") info->dtype = VRC_F32;
    else return VRC_ERR_UNSUPPORTED;
    info->dims[0] = std::atoi(x.c_str());
    info->dims[1] = std::atoi(y.c_str());
    info->dims[2] = std::atoi(z.c_str());
    if (info->dims[0] < 1 || info->dims[1] < 1 || info->dims[2] < 1) return VRC_ERR_INVALID_ARG;
    // raw file: the old `filename` attribute (relative to the .vvd), else the path list
    const std::string dir = dir_of(vvd_path);
    std::string raw, name;
    if (attr(s, b, e, "filename", name)) {
        raw = (!name.empty() && name[0] == '/') ? name : dir + "/" + name;
    } else {
        const size_t close = s.find("</RawData>", e);
        size_t p = e, ib, ie;
        while (find_tag(s, "item", p, ib, ie) && (close == std::string::npos || ib < close)) {
            std::string v;
            if (attr(s, ib, ie, "value", v) && !v.empty()) {
                const std::string cand = v[0] == '/' ? v : dir + "/" + v;
                if (file_exists(cand)) {
                    raw = cand;
                    break;
                }
            }
            p = ie;
        }
    }
    if (raw.empty() || raw.size() >= sizeof(info->raw_path)) return VRC_ERR_NOT_READY;
    std::memcpy(info->raw_path, raw.c_str(), raw.size() + 1);
    // meta data (Voreen's defaults when absent)
    for (int i = 0; i < 3; ++i) {
        info->spacing[i] = 1.f;
        info->offset[i] = 0.f;
    }
    // No RealWorldMapping item: VvdVolumeReader gives the volume the
    // denormalizing mapping of its format (modules/core/io/vvdvolumereader.cpp:
    // 102-120, RealWorldMapping::createDenormalizingMapping): scale = the
    // largest value of an unsigned integer type, 1 for float, offset 0. The
    // file's VolumeMinMax items are normalised values, which the mapping does
    // not change.
    info->rwm_scale = info->dtype == VRC_U8 ? 255.f : (info->dtype == VRC_U16 ? 65535.f : 1.f);
    info->rwm_offset = 0.f;
    const char* axes[3] = {"x", "y", "z"};
    if (meta_value(s, "Spacing", b, e))
        for (int i = 0; i < 3; ++i) {
            std::string v;
            if (attr(s, b, e, axes[i], v)) to_float(v, info->spacing[i]);
        }
    if (meta_value(s, "Offset", b, e))
        for (int i = 0; i < 3; ++i) {
            std::string v;
            if (attr(s, b, e, axes[i], v)) to_float(v, info->offset[i]);
        }
    if (meta_value(s, "RealWorldMapping", b, e)) {
        std::string v;
        if (attr(s, b, e, "scale", v)) to_float(v, info->rwm_scale);
        if (attr(s, b, e, "offset", v)) to_float(v, info->rwm_offset);
    }
    // VolumeMinMax: minNorm / maxNorm attributes (older files) or the first
    // channel of <minNormValues> / <maxNormValues> (newer files)
    size_t p = 0;
    while (find_tag(s, "DerivedItem", p, b, e)) {
        std::string t, mn, mx;
        if (attr(s, b, e, "type", t) && t == "VolumeMinMax") {
            if (attr(s, b, e, "minNorm", mn) && attr(s, b, e, "maxNorm", mx)) {
                info->has_minmax = to_float(mn, info->min_norm) && to_float(mx, info->max_norm) ? 1 : 0;
            } else {
                const size_t close = s.find("</DerivedItem>", e);
                size_t cb, ce, vb, ve;
                if (close != std::string::npos && find_tag(s, "minNormValues", e, cb, ce) && cb < close &&
                    find_tag(s, "channel", ce, vb, ve) && vb < close && attr(s, vb, ve, "value", mn) &&
                    find_tag(s, "maxNormValues", e, cb, ce) && cb < close && find_tag(s, "channel", ce, vb, ve) &&
                    vb < close && attr(s, vb, ve, "value", mx))
                    info->has_minmax = to_float(mn, info->min_norm) && to_float(mx, info->max_norm) ? 1 : 0;
            }
            break;
        }
        p = e;
    }
    return VRC_OK;
}

vrc_status vrc_tf_read_tfi(const char* path, vrc_tfi_info* info, vrc_tf_key* keys, int max_keys) {
    if (!path || !info || max_keys < 0 || (max_keys > 0 && !keys)) return VRC_ERR_INVALID_ARG;
    std::memset(info, 0, sizeof(*info));
    info->alpha_mode = 1;
    info->gamma = 1.f;
    info->domain[1] = 1.f;
    info->threshold[1] = 1.f;
    std::string s;
    if (!read_file(path, s)) return VRC_ERR_NOT_READY;
    size_t tb, te;
    if (!find_tag(s, "TransFuncIntensity", 0, tb, te)) return VRC_ERR_UNSUPPORTED;
    size_t kb = std::string::npos, ke = std::string::npos;
    const bool have_keys = find_tag(s, "Keys", te, kb, ke);
    const size_t keys_end = have_keys ? s.find("</Keys>", ke) : std::string::npos;
    // a scalar element of the function (before its key list): attribute `a` of <tag>
    auto field = [&](const char* tag, const char* a, float& out) {
        size_t b, e;
        std::string v;
        if (find_tag(s, tag, te, b, e) && (!have_keys || b < kb) && attr(s, b, e, a, v)) to_float(v, out);
    };
    float f = 0.f;
    f = (float)info->alpha_mode;
    field("alphaMode", "value", f);
    info->alpha_mode = (int)f;
    f = 0.f;
    field("texDimensions", "x", f);
    info->width = (int)f;
    field("gammaValue", "value", info->gamma);
    field("domain", "x", info->domain[0]);
    field("domain", "y", info->domain[1]);
    field("threshold", "x", info->threshold[0]);
    field("threshold", "y", info->threshold[1]);
    int n = 0;
    size_t p = have_keys ? ke : std::string::npos;
    size_t b, e;
    while (have_keys && find_tag(s, "key", p, b, e) && (keys_end == std::string::npos || b < keys_end)) {
        const size_t end = s.find("</key>", e);
        if (end == std::string::npos) return VRC_ERR_INVALID_ARG;
        vrc_tf_key k{};
        size_t xb, xe;
        std::string v;
        if (!find_tag(s, "intensity", e, xb, xe) || xb > end || !attr(s, xb, xe, "value", v) || !to_float(v, k.intensity))
            return VRC_ERR_INVALID_ARG;
        bool split = false;
        if (find_tag(s, "split", e, xb, xe) && xb < end && attr(s, xb, xe, "value", v)) split = v == "true" || v == "1";
        auto color = [&](const char* tag, uint8_t* c) {
            size_t cb, ce;
            if (!find_tag(s, tag, e, cb, ce) || cb > end) return false;
            const char* ch[4] = {"r", "g", "b", "a"};
            for (int i = 0; i < 4; ++i) {
                std::string cv;
                c[i] = attr(s, cb, ce, ch[i], cv) ? (uint8_t)std::atoi(cv.c_str()) : (uint8_t)(i == 3 ? 255 : 0);
            }
            return true;
        };
        if (!color("colorL", k.color_l)) return VRC_ERR_INVALID_ARG;
        if (!split || !color("colorR", k.color_r)) std::memcpy(k.color_r, k.color_l, 4);
        if (n < max_keys) keys[n] = k;
        ++n;
        p = end;
    }
    info->nkeys = n;
    return VRC_OK;
}

vrc_status vrc_volume_load_vvd(vrc_context* ctx, const char* vvd_path, int brick_size, vrc_volume** out,
                               vrc_vvd_info* info_out) {
    if (!ctx) return VRC_ERR_INVALID_ARG;
    if (!vvd_path || !out) return ifail(ctx, VRC_ERR_INVALID_ARG, "vrc_volume_load_vvd: null argument");
    *out = nullptr;
    vrc_vvd_info info;
    vrc_status st = vrc_vvd_read_header(vvd_path, &info);
    if (st != VRC_OK) return ifail(ctx, st, std::string("vrc_volume_load_vvd: cannot read header ") + vvd_path);
    if (info_out) *info_out = info;
    const size_t bytes = (size_t)info.dims[0] * info.dims[1] * info.dims[2] * vrc::dtype_bytes(info.dtype);
    FILE* f = std::fopen(info.raw_path, "rb");
    if (!f) return ifail(ctx, VRC_ERR_NOT_READY, std::string("vrc_volume_load_vvd: cannot open ") + info.raw_path);
    cudaError_t e = cudaSetDevice(ctx->device);
    void* d_lin = nullptr;
    void* h_chunk[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    constexpr size_t CHUNK = size_t(64) << 20;
    auto cleanup = [&](vrc_status s, const std::string& m) {
        std::fclose(f);
        cudaStreamSynchronize(ctx->stream);
        for (int i = 0; i < 2; ++i) {
            if (h_chunk[i]) cudaFreeHost(h_chunk[i]);
            if (done[i]) cudaEventDestroy(done[i]);
        }
        if (d_lin) cudaFree(d_lin);
        return s == VRC_OK ? VRC_OK : ifail(ctx, s, m);
    };
    if (e != cudaSuccess) return cleanup(VRC_ERR_CUDA, "vrc_volume_load_vvd: cudaSetDevice");
    if ((e = cudaMalloc(&d_lin, bytes)) != cudaSuccess)
        return cleanup(VRC_ERR_OUT_OF_MEMORY, "vrc_volume_load_vvd: device staging allocation");
    const size_t chunk = bytes < CHUNK ? bytes : CHUNK;
    for (int i = 0; i < 2; ++i) {
        if ((e = cudaHostAlloc(&h_chunk[i], chunk, cudaHostAllocDefault)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming)) != cudaSuccess)
            return cleanup(VRC_ERR_OUT_OF_MEMORY, "vrc_volume_load_vvd: pinned staging allocation");
    }
    size_t off = 0;
    for (int k = 0; off < bytes; ++k) {
        const int b = k & 1;
        const size_t n = bytes - off < chunk ? bytes - off : chunk;
        // the copy that last used this pinned chunk has finished
        if ((e = cudaEventSynchronize(done[b])) != cudaSuccess)
            return cleanup(VRC_ERR_CUDA, "vrc_volume_load_vvd: copy");
        if (std::fread(h_chunk[b], 1, n, f) != n)
            return cleanup(VRC_ERR_INVALID_ARG, std::string("vrc_volume_load_vvd: raw file shorter than the header's "
                                                            "dimensions: ") + info.raw_path);
        if ((e = cudaMemcpyAsync(static_cast<char*>(d_lin) + off, h_chunk[b], n, cudaMemcpyHostToDevice,
                                 ctx->stream)) != cudaSuccess ||
            (e = cudaEventRecord(done[b], ctx->stream)) != cudaSuccess)
            return cleanup(VRC_ERR_CUDA, "vrc_volume_load_vvd: copy");
        off += n;
    }
    vrc_volume_desc d{};
    d.dtype = info.dtype;
    for (int i = 0; i < 3; ++i) {
        d.dims[i] = info.dims[i];
        d.spacing[i] = info.spacing[i];
        d.offset[i] = info.offset[i];
    }
    d.rwm_scale = info.rwm_scale;
    d.rwm_offset = info.rwm_offset;
    st = vrc_volume_upload(ctx, &d, d_lin, 1, brick_size, out);
    if (st != VRC_OK) {
        const std::string m = ctx->last_error;
        return cleanup(st, m);
    }
    return cleanup(VRC_OK, "");
}

}  // extern "C"
