/* The C ABI from plain C99: the headers compile as C and the host-only
 * entry points work without a GPU (TF bake, table width, status strings,
 * camera matrices, .tfi reading). Exit code 0 = all checks passed. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "vrc.h"
#include "vrc_nn.h"
#include "vrc_processor.h"

#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            return 1;                                              \
        }                                                          \
    } while (0)

int main(int argc, char** argv) {
    CHECK(vrc_abi_version() == VRC_ABI_VERSION);
    CHECK(strcmp(vrc_status_string(VRC_OK), "ok") == 0);
    CHECK(vrc_tf_table_width(VRC_U8) == 256 && vrc_tf_table_width(VRC_U16) == 4096);

    vrc_tf_key keys[2];
    memset(keys, 0, sizeof(keys));
    keys[1].intensity = 1.f;
    for (int c = 0; c < 4; ++c) keys[1].color_l[c] = keys[1].color_r[c] = 255;
    unsigned char rgba[256 * 4];
    CHECK(vrc_tf_bake_keys(keys, 2, 256, 1.f, 0.f, 1.f, rgba) == VRC_OK);
    CHECK(rgba[0] == 0 && rgba[255 * 4 + 3] == 255);
    CHECK(vrc_tf_bake_keys(keys, 2, 1, 1.f, 0.f, 1.f, rgba) == VRC_ERR_INVALID_ARG);

    vrc_camera cam;
    memset(&cam, 0, sizeof(cam));
    cam.position[2] = 3.f;
    cam.up[1] = 1.f;
    cam.fovy_deg = 45.f;
    cam.near_dist = 0.1f;
    cam.far_dist = 50.f;
    cam.frustum_ratio = 1.f;
    vrc_volume_desc d;
    memset(&d, 0, sizeof(d));
    d.dtype = VRC_U8;
    d.dims[0] = d.dims[1] = d.dims[2] = 8;
    d.spacing[0] = d.spacing[1] = d.spacing[2] = 1.f;
    d.rwm_scale = 1.f;
    double view[16], proj[16], inv[16];
    CHECK(vrc_camera_matrices(&cam, &d, 64, 64, view, proj, inv) == VRC_OK);
    CHECK(fabs(view[15] - 1.0) < 1e-12 && proj[14] == -1.0);

    vrcp_processor* p = NULL;
    CHECK(vrcp_create(0, &p) == VRC_OK && p);
    CHECK(strcmp(vrcp_class_name(), "CudaRaycaster") == 0);
    float f = 0.f;
    CHECK(vrcp_get_float(p, "samplingRate", &f) == VRC_OK && f == 2.f);
    CHECK(vrcp_set_string(p, "compositing", "mip") == VRC_OK);
    vrcp_process(p, 1, 0); /* no volume: an error, no output, no device touched */
    CHECK(strstr(vrcp_last_error(p), "not ready") != NULL && !vrcp_output(p, NULL, NULL, NULL));
    CHECK(vrcp_destroy(p) == VRC_OK);

    if (argc > 1) { /* a .tfi file given on the command line */
        vrc_tfi_info info;
        CHECK(vrc_tf_read_tfi(argv[1], &info, NULL, 0) == VRC_OK && info.nkeys > 0);
    }
    puts("abi_c99 ok");
    return 0;
}
