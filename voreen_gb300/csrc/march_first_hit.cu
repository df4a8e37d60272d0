// Instantiations of the march kernel for first-hit position / normal compositing (mod_compositing.frag:168-196).
// Their output does not depend on the sample colour, so they run unshaded.
#include "march_core.cuh"

namespace vrc {
namespace {

template <int DT, int COMP>
cudaError_t launch_unshaded(const MarchParams& p, int, int num_sms, cudaStream_t s) {
    return launch_ee<DT, COMP, VRC_SHADE_NONE>(p, num_sms, s);
}

template <int COMP>
cudaError_t by_dtype(const MarchParams& p, int dtype, int shading, int num_sms, cudaStream_t s) {
    switch (dtype) {
        case VRC_U8: return launch_unshaded<VRC_U8, COMP>(p, shading, num_sms, s);
        case VRC_U16: return launch_unshaded<VRC_U16, COMP>(p, shading, num_sms, s);
        default: return launch_unshaded<VRC_F32, COMP>(p, shading, num_sms, s);
    }
}

}  // namespace

cudaError_t launch_march_first_hit(const MarchParams& p, int dtype, int compositing, int num_sms, cudaStream_t s) {
    return compositing == VRC_FHN ? by_dtype<VRC_FHN>(p, dtype, VRC_SHADE_NONE, num_sms, s)
                                  : by_dtype<VRC_FHP>(p, dtype, VRC_SHADE_NONE, num_sms, s);
}

}  // namespace vrc
