/*
 * milton_plugin.h -- the entry points of libmgpu_milton.so, Milton's dynamic renderer plugin.
 *
 * Milton's scene loader selects the plugin with `"renderer": {"type": "dynamic", "path":
 * "libmgpu_milton.so", ...}`, resolves these three symbols with dlsym, checks plugin_type() and
 * casts the result of plugin_new() to milton::Renderer*
 * (mlt/src/milton/dynamic/DynamicPlugin.h:34-62,
 * mlt/src/milton/loaders/MiltonJSONSceneLoader.cpp:1770-1813).  The object is a C++
 * milton::PointSampleRenderer (milton_gb300/milton_plugin/gpu_path_tracer.cpp) whose init()
 * builds the kd-tree and makes the scene resident and whose render() runs every super-sample
 * pass on the GPU through the C ABI of mgpu.h, then hands the per-pixel means to Milton's
 * RenderOutput.  Declared here in namespace milton, extern "C", as Milton's own header declares
 * them; the symbols are the plain C names.
 */
#ifndef MILTON_PLUGIN_H_
#define MILTON_PLUGIN_H_

#ifdef __cplusplus
namespace milton {
extern "C" {
#endif

/* DynamicPlugin.h:38-49; MILTON_PLUGIN_TYPE_RENDERER = 0 */
int plugin_type(void);
/* a new GPU PathTracer as a milton::Renderer* (NULL if out of host memory) */
void *plugin_new(void);
/* deletes an object plugin_new returned (Milton never calls it) */
void plugin_delete(void *plugin);

#ifdef __cplusplus
}
}
#endif
#endif /* MILTON_PLUGIN_H_ */
