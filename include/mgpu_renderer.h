/*
 * mgpu_renderer.h -- the GPU PathTracer as a C object (libmgpu.so), for hosts that speak C.
 *
 * The calls mirror what Milton does to a PointSampleRenderer: PropertyMap keys, setScene /
 * setCamera / setOutput, Renderer::init, Renderer::render, and the finalized output
 * (mlt/src/milton/renderers/Renderer.h:52-62, PointSampleRenderer.h:61-95,
 * RenderOutput.h:69-94).  Milton itself loads the C++ plugin libmgpu_milton.so instead
 * (include/milton_plugin.h), which derives from Milton's PointSampleRenderer and calls the
 * same C ABI underneath.
 */
#ifndef MGPU_RENDERER_H_
#define MGPU_RENDERER_H_

#include "mgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mgpu_renderer mgpu_renderer;

/* A new renderer object with no scene, camera or output (the PathTracer a scene file's
 * renderer block creates); destroy releases its device scene and film. */
int mgpu_renderer_create(mgpu_renderer **out);
int mgpu_renderer_destroy(mgpu_renderer *r);

/* PropertyMap::operator[] for the renderer's keys (values as text, like the scene file):
 * noDirectSamples, noSuperSamples, efficientDirect, maxDepth, rrStartDepth, seed,
 * kdMinPrimitives, kdMaxDepth, kdCostTraversal, kdEmptyBias, wavePaths.  Unknown keys are
 * stored and ignored, as a PropertyMap would.  The kd keys default to Milton's values except
 * kdCostTraversal, which defaults to MGPU_KD_COST_TRAVERSAL (mgpu.h).                       */
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
#endif /* MGPU_RENDERER_H_ */
