// C entry point over the reference's own transfer-function code (test
// infrastructure only): TransFunc1DKeys::getMappingForValueUByte
// (src/core/datastructures/transfunc/1d/1dkeys/transfunc1dkeys.cpp:119-154),
// TransFunc1D::applyGammaToIntensity (transfunc1d.cpp:144-149) and the
// TransFuncMappingKey accessors, compiled from the reference tree.
//
// Constructing a TransFunc1DKeys would pull in the GL texture, shader and
// serialisation stack. The pinned functions are non-virtual when called by
// qualified name and read only the key list and the gamma value, so they
// run on an object whose storage is zeroed and whose key vector and gamma are
// set directly; the keys are set through their own public setters. The
// texel loop around them is TransFunc1D::createTextureData
// (transfunc1d.cpp:85-103): zero outside iround(threshold * width), else the
// mapping at gamma(x / (width - 1)).
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "tgt/tgt_math.h"
#include "voreen/core/datastructures/transfunc/1d/1dkeys/transfunc1dkeys.h"
#include "voreen/core/datastructures/transfunc/1d/1dkeys/utils/transfuncmappingkey.h"

namespace {

using voreen::TransFunc1DKeys;
using voreen::TransFuncMappingKey;

// Names the protected key list and mapping through a derived class (never
// instantiated); the mapping is called by qualified name, without dispatch.
struct KeysAccess : TransFunc1DKeys {
    using TransFunc1DKeys::keys_;
    static tgt::Vector4<GLubyte> map(TransFunc1DKeys* tf, float value) {
        return static_cast<KeysAccess*>(tf)->TransFunc1DKeys::getMappingForValueUByte(value);
    }
};

template <typename T>
struct Zeroed {
    alignas(T) unsigned char bytes[sizeof(T)];
    Zeroed() { std::memset(bytes, 0, sizeof(bytes)); }
    T* get() { return reinterpret_cast<T*>(bytes); }
};

}  // namespace

extern "C" {

/* keys: nkeys x (intensity, colorL RGBA, colorR RGBA) as
 * float intensity[nkeys] and uint8 colors[nkeys * 8];
 * out: width x RGBA8. */
__attribute__((visibility("default"))) void ref_tf_bake(const float* intensity, const uint8_t* colors, int nkeys,
                                                        int width, float gamma, float threshold_lo,
                                                        float threshold_hi, uint8_t* out) {
    std::vector<Zeroed<TransFuncMappingKey>> keys(nkeys);
    Zeroed<TransFunc1DKeys> tf;
    auto& list = tf.get()->*(&KeysAccess::keys_);
    new (&list) std::vector<TransFuncMappingKey*>();
    for (int k = 0; k < nkeys; ++k) {
        TransFuncMappingKey* key = keys[k].get();
        key->TransFuncMappingKey::setIntensity(intensity[k]);
        key->TransFuncMappingKey::setSplit(true, true);
        const uint8_t* c = colors + 8 * k;
        key->TransFuncMappingKey::setColorL(tgt::col4(c[0], c[1], c[2], c[3]));
        key->TransFuncMappingKey::setColorR(tgt::col4(c[4], c[5], c[6], c[7]));
        list.push_back(key);
    }
    tf.get()->gammaValue_ = gamma;
    const int front_end = tgt::iround(threshold_lo * width);
    const int back_start = tgt::iround(threshold_hi * width);
    for (int x = 0; x < width; ++x) {
        uint8_t* o = out + 4 * x;
        if (x < front_end || x > back_start) {
            std::memset(o, 0, 4);
            continue;
        }
        const float value = tf.get()->voreen::TransFunc1D::applyGammaToIntensity(static_cast<float>(x) / (width - 1));
        const tgt::Vector4<GLubyte> c = KeysAccess::map(tf.get(), value);
        o[0] = c.r;
        o[1] = c.g;
        o[2] = c.b;
        o[3] = c.a;
    }
    list.~vector();
}
}
