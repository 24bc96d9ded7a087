/*
 * milton_plugin.h -- Milton's dynamic-plugin ABI as exported by libmgpu.so, and the C view of
 * the renderer object that plugin_new() returns.
 *
 * Milton's loader resolves plugin_type/plugin_new with dlsym, checks the type and casts the
 * result of plugin_new() (mlt/src/milton/dynamic/DynamicPlugin.h:34-62,
 * mlt/src/milton/loaders/MiltonJSONSceneLoader.cpp:1770-1813).  The object behind the handle is
 * a GPU PathTracer: the mgpu_renderer_* calls below are the virtual calls Milton makes on a
 * PointSampleRenderer (Renderer::init / render, PropertyMap keys, setScene / setCamera /
 * setOutput; mlt/src/milton/renderers/Renderer.h:52-62, PointSampleRenderer.h:61-95).  A real
 * Milton binary reaches them through the small PointSampleRenderer subclass shown in
 * INTEGRATION.md, which owns one handle.
 */
#ifndef MILTON_PLUGIN_H_
#define MILTON_PLUGIN_H_

#include "mgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* DynamicPlugin.h:38-49 */
typedef enum {
  MILTON_PLUGIN_TYPE_RENDERER = 0,
  MILTON_PLUGIN_TYPE_CAMERA,
  MILTON_PLUGIN_TYPE_OUTPUT,
  MILTON_PLUGIN_TYPE_FILTER,
  MILTON_PLUGIN_TYPE_SHAPE,
  MILTON_PLUGIN_TYPE_BSDF,
  MILTON_PLUGIN_TYPE_EMITTER,
  MILTON_PLUGIN_TYPE_MEDIUM,
  MILTON_PLUGIN_TYPE_GENERATOR,
  MILTON_PLUGIN_TYPE_METAOBJECT
} MILTON_PLUGIN_TYPE;

/* DynamicPlugin.h:51-53 */
MILTON_PLUGIN_TYPE plugin_type(void); /* returns MILTON_PLUGIN_TYPE_RENDERER */
void *plugin_new(void);               /* a new mgpu_renderer (NULL on failure, reason in mgpu_last_error) */
void plugin_delete(void *plugin);

typedef struct mgpu_renderer mgpu_renderer;

/* PropertyMap::operator[] for the renderer's keys (values as text, like the scene file):
 * noDirectSamples, noSuperSamples, efficientDirect, maxDepth, rrStartDepth, seed,
 * kdMinPrimitives, kdMaxDepth, kdCostTraversal, kdEmptyBias, wavePaths.  Unknown keys are
 * stored and ignored, as a PropertyMap would.                                               */
int mgpu_renderer_set_value(mgpu_renderer *r, const char *key, const char *value);
int mgpu_renderer_get_value(mgpu_renderer *r, const char *key, char *buf, size_t buflen);
/* Renderer::setScene: the flattened scene (arrays are copied) */
int mgpu_renderer_set_scene(mgpu_renderer *r, const mgpu_scene_desc *desc);
/* Renderer::setCamera: eye[3], look[3], up[3], heightAngle, aspectRatio */
int mgpu_renderer_set_camera(mgpu_renderer *r, const float *camera11);
/* ThinLensCamera's lens (ThinLensCamera.cpp:88-124): aperture in metres (0 = pinhole, the
 * PinholeCamera), focal length = fstop x aperture, focal distance (autofocus resolved by the
 * caller).  Default: pinhole.                                                              */
int mgpu_renderer_set_lens(mgpu_renderer *r, float aperture, float focal_length, float focal_distance);
/* PointSampleRenderer::setOutput: film size */
int mgpu_renderer_set_output(mgpu_renderer *r, int32_t width, int32_t height);
/* Renderer::init: builds the kd-tree and makes the scene resident on the current device */
int mgpu_renderer_init(mgpu_renderer *r);
/* Renderer::render: all noSuperSamples passes, synchronous */
int mgpu_renderer_render(mgpu_renderer *r);
/* RenderOutput finalised value: per-pixel mean radiance, width*height*3 doubles */
int mgpu_renderer_get_output(mgpu_renderer *r, double *rgb);

#ifdef __cplusplus
}
#endif
#endif /* MILTON_PLUGIN_H_ */
