// The processor shim from C++ the way a Voreen-side processor forwards its
// properties (Processor::getProperty(id)->set()), host-only: property ids,
// kinds and defaults, and the settings check of process(). Exit code 0 =
// all checks passed.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vrc_processor.h"

#define CHECK(c)                                                            \
    do {                                                                    \
        if (!(c)) {                                                         \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            return 1;                                                       \
        }                                                                   \
    } while (0)

int main() {
    vrcp_processor* p = nullptr;
    CHECK(vrcp_create(0, &p) == VRC_OK);
    struct F { const char* id; float def; };
    for (const F& f : std::vector<F>{{"samplingRate", 2.f}, {"isoValue", 0.5f}, {"gammaValue", 0.f},
                                     {"interactionQuality", 1.f}, {"materialShininess", 60.f}}) {
        float v = -1.f;
        CHECK(vrcp_get_float(p, f.id, &v) == VRC_OK && v == f.def);
    }
    int i = 0;
    CHECK(vrcp_get_int(p, "interactionCoarseness", &i) == VRC_OK && i == 3);
    CHECK(vrcp_get_int(p, "brickUploadBudgetMB", &i) == VRC_OK && i == 32);
    CHECK(vrcp_get_int(p, "useIterativeRefinement", &i) == VRC_OK && i == 1);
    char buf[64];
    CHECK(vrcp_get_string(p, "shading", buf, sizeof(buf)) == VRC_OK && std::string(buf) == "none");
    CHECK(vrcp_set_float(p, "compositing", 1.f) == VRC_ERR_INVALID_ARG);  // a string property
    CHECK(vrcp_set_string(p, "noSuchProperty", "x") == VRC_ERR_INVALID_ARG);
    float light[4];
    CHECK(vrcp_get_floatv(p, "lightPosition", light, 4) == VRC_OK && light[0] == 2.3f);

    std::vector<unsigned char> vox(4 * 4 * 4, 0);
    vrc_volume_desc d{};
    d.dtype = VRC_U8;
    d.dims[0] = d.dims[1] = d.dims[2] = 4;
    d.spacing[0] = d.spacing[1] = d.spacing[2] = 1.f;
    d.rwm_scale = 1.f;
    CHECK(vrcp_set_volume(p, &d, vox.data()) == VRC_OK);
    CHECK(vrcp_set_float(p, "samplingRate", 50.f) == VRC_OK);  // accepted, rejected by process()
    vrcp_process(p, 1, 0);
    CHECK(std::strstr(vrcp_last_error(p), "samplingRate") != nullptr && !vrcp_output(p, nullptr, nullptr, nullptr));
    CHECK(vrcp_destroy(p) == VRC_OK);
    std::puts("processor_cpp ok");
    return 0;
}
