// Instantiations of the march kernel for DVR compositing, with TF or pre-integrated classification.
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

cudaError_t launch_march_dvr(const MarchParams& p, int dtype, int shading, int num_sms, cudaStream_t s) {
    return p.pi_table ? by_dtype<COMP_DVR_PREINT>(p, dtype, shading, num_sms, s)
                      : by_dtype<VRC_DVR>(p, dtype, shading, num_sms, s);
}

}  // namespace vrc
