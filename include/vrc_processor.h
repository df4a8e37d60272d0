/* CudaRaycaster: the Voreen processor surface of vrc, in C++ over the C ABI
 * of vrc.h, with a C shim so other languages drive it the way Voreen's
 * property system does (Processor::getProperty(id)->set(value)).
 *
 * Reference interface it mirrors (Voreen tree):
 *   ports         VolumeRaycaster::VolumeRaycaster, src/core/processors/volumeraycaster.cpp:44-47
 *                 ("volumehandle.volumehandle", "image.entrypoints", "image.exitpoints", "image.output")
 *   properties    volumeraycaster.cpp:42-157, volumerenderer.cpp:41-53 (ids and defaults),
 *                 cpuraycaster.cpp:51-74 (classification, preIntegrationTableSize),
 *                 optimizedproxygeometry.cpp:434-437 (enableClipping, clipRegion),
 *                 singleoctreeraycastercl.cpp:294-305 (brick streaming)
 *   isReady       CPURaycaster::isReady, modules/base/processors/render/cpuraycaster.cpp:82-84
 *   process       CPURaycaster::process, cpuraycaster.cpp:90-206, with the interaction
 *                 mode of SingleVolumeRaycaster::process, singlevolumeraycaster.cpp:253-256
 *   errors        LERROR + return without output, cpuraycaster.cpp:125-146
 *
 * vrcp_set_* / vrcp_get_* return VRC_ERR_INVALID_ARG for an unknown id or a
 * value of the wrong kind; values outside a property's range are accepted
 * and rejected by process() with an error, as Voreen logs them there. */
#ifndef VRC_PROCESSOR_H
#define VRC_PROCESSOR_H

#include "vrc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vrcp_processor vrcp_processor;

vrc_status vrcp_create(int device, vrcp_processor** out);
vrc_status vrcp_destroy(vrcp_processor* p);
const char* vrcp_class_name(void); /* "CudaRaycaster" */
const char* vrcp_category(void);   /* "Raycasting" */

/* Properties by id. Floats: samplingRate, isoValue, gammaValue,
 * interactionQuality, materialShininess. Ints (bools as 0/1):
 * preIntegrationTableSize, interactionCoarseness, enableClipping,
 * applyLightAttenuation, brickBufferSizeMB, brickUploadBudgetMB,
 * useLevelOfDetail, useIterativeRefinement. Strings: compositing, shading,
 * gradient, classification, brickPoolPlacement. Float vectors: lightPosition
 * (4), lightAmbient, lightDiffuse, lightSpecular (4), lightAttenuation (3).
 * Int vector: clipRegion (6: llf x y z, urb x y z). */
vrc_status vrcp_set_float(vrcp_processor* p, const char* id, float v);
vrc_status vrcp_get_float(const vrcp_processor* p, const char* id, float* v);
vrc_status vrcp_set_int(vrcp_processor* p, const char* id, int v);
vrc_status vrcp_get_int(const vrcp_processor* p, const char* id, int* v);
vrc_status vrcp_set_string(vrcp_processor* p, const char* id, const char* v);
/* Copies at most `cap` bytes including the terminating zero. */
vrc_status vrcp_get_string(const vrcp_processor* p, const char* id, char* buf, int cap);
vrc_status vrcp_set_floatv(vrcp_processor* p, const char* id, const float* v, int n);
vrc_status vrcp_get_floatv(const vrcp_processor* p, const char* id, float* v, int n);
vrc_status vrcp_set_intv(vrcp_processor* p, const char* id, const int* v, int n);
vrc_status vrcp_get_intv(const vrcp_processor* p, const char* id, int* v, int n);
vrc_status vrcp_set_camera(vrcp_processor* p, const vrc_camera* c);
vrc_status vrcp_get_camera(const vrcp_processor* p, vrc_camera* c);

/* "transferFunction" (TransFunc1DKeysProperty): keys, gamma, thresholds;
 * width and domain are fitted to the volume by process() (the width always,
 * the domain on first use when it is still [0, 1] and not fitted). */
vrc_status vrcp_set_tf_keys(vrcp_processor* p, const vrc_tf_key* keys, int nkeys, float gamma, float threshold_lo,
                            float threshold_hi);
vrc_status vrcp_set_tf_domain(vrcp_processor* p, float lo, float hi, int fitted, int width);
vrc_status vrcp_get_tf(const vrcp_processor* p, int* width, float* lo, float* hi, int* fitted);
/* Loads a .tfi file into "transferFunction" (vrc_tf_read_tfi), as
 * TransFunc1DKeysProperty loads one: keys, gamma, thresholds and the file's
 * domain, which process() then keeps. */
vrc_status vrcp_load_tf(vrcp_processor* p, const char* path);

/* Ports. Data is borrowed: it must stay valid until process() returns.
 * A NULL pointer disconnects the port. A volume is uploaded again when
 * vrcp_set_volume is called again, as a new VolumeBase on the inport. */
vrc_status vrcp_set_volume(vrcp_processor* p, const vrc_volume_desc* desc, const void* voxels);
vrc_status vrcp_set_entry_exit(vrcp_processor* p, const float* entry, const float* exit_pts, int width, int height);
/* Size of image.output for analytic entry/exit (render target size). */
vrc_status vrcp_set_output_size(vrcp_processor* p, int width, int height);
int vrcp_is_ready(const vrcp_processor* p);

void vrcp_initialize(vrcp_processor* p);
void vrcp_deinitialize(vrcp_processor* p);
/* One frame into image.output (W x H RGBA float, row 0 at the bottom). On
 * failure: no output, vrcp_last_error() holds the message. */
void vrcp_process(vrcp_processor* p, int analytic_entry_exit, int interacting);
/* 1 and the outport's image if it holds one, else 0. */
int vrcp_output(const vrcp_processor* p, const float** rgba, int* width, int* height);
const char* vrcp_last_error(const vrcp_processor* p);
vrc_status vrcp_last_stats(const vrcp_processor* p, vrc_render_stats* stats);
/* 1 after a frame that read bricks a further frame could bring in (brick
 * streaming with useIterativeRefinement), as the reference invalidates itself. */
int vrcp_invalidated(const vrcp_processor* p);

#ifdef __cplusplus
}
#endif

#endif
