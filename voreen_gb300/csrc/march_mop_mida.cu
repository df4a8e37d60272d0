// Instantiations of the march kernel for MOP and MIDA compositing (mod_compositing.frag:97-146).
#include "march_core.cuh"

namespace vrc {
namespace {

template <int COMP>
cudaError_t by_dtype(const MarchParams& p, int dtype, int shading, int num_sms, cudaStream_t s) {
    switch (dtype) {
        case VRC_U8: return launch_sh<VRC_U8, COMP>(p, shading, num_sms, s);
        case VRC_U16: return launch_sh<VRC_U16, COMP>(p, shading, num_sms, s);
        default: return launch_sh<VRC_F32, COMP>(p, shading, num_sms, s);
    }
}

}  // namespace

cudaError_t launch_march_mop_mida(const MarchParams& p, int dtype, int compositing, int shading, int num_sms,
                                  cudaStream_t s) {
    return compositing == VRC_MIDA ? by_dtype<VRC_MIDA>(p, dtype, shading, num_sms, s)
                                   : by_dtype<VRC_MOP>(p, dtype, shading, num_sms, s);
}

}  // namespace vrc
