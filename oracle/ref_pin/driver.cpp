// C entry points over the reference's own code (test infrastructure only):
// VolumeAtomic<T>::getVoxelNormalizedLinear and tgt's header-only math.
#include <cstdint>
#include <cstring>

#include "tgt/matrix.h"
#include "tgt/tgt_math.h"
#include "voreen/core/datastructures/volume/volumeatomic.h"

namespace {
template <typename T>
void tri(const void* data, const int d[3], const float* pos, int n, float* out) {
    voreen::VolumeAtomic<T> v(const_cast<T*>(static_cast<const T*>(data)), tgt::svec3(d[0], d[1], d[2]), false);
    for (int i = 0; i < n; ++i)
        out[i] = v.getVoxelNormalizedLinear(tgt::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
}
void put(const tgt::mat4& m, float* out) {
    for (int i = 0; i < 16; ++i) out[i] = m.elem[i];
}
}  // namespace

extern "C" {
/* dtype 0 = uint8, 1 = uint16, 2 = float */
void ref_trilinear(int dtype, const void* data, const int dims[3], const float* pos, int n, float* out) {
    if (dtype == 0) tri<uint8_t>(data, dims, pos, n, out);
    else if (dtype == 1) tri<uint16_t>(data, dims, pos, n, out);
    else tri<float>(data, dims, pos, n, out);
}
void ref_lookat(const float* eye, const float* focus, const float* up, float* out) {
    put(tgt::mat4::createLookAt(tgt::vec3(eye[0], eye[1], eye[2]), tgt::vec3(focus[0], focus[1], focus[2]),
                                tgt::vec3(up[0], up[1], up[2])), out);
}
void ref_perspective(float fov_rad, float aspect, float pnear, float pfar, float* out) {
    put(tgt::mat4::createPerspective(fov_rad, aspect, pnear, pfar), out);
}
int ref_iround(float f) { return tgt::iround(f); }
}
