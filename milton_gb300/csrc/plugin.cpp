// plugin.cpp -- the renderer object of the C ABI (include/mgpu_renderer.h): Milton's PathTracer
// keys, scene, camera and output behind plain C calls, for hosts that speak C.  Milton itself
// loads the C++ plugin libmgpu_milton.so (milton_gb300/milton_plugin/gpu_path_tracer.cpp).
#include <stdlib.h>
#include <string.h>

#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/mgpu_renderer.h"

struct mgpu_renderer {
  std::map<std::string, std::string> props;  // PropertyMap (text values)
  // owned copies of the scene arrays
  int64_t ntri = 0;
  std::vector<float> v, n, mats, lights, light_ext, uv;
  std::vector<int32_t> mat, light;
  std::vector<uint32_t> flags;
  std::vector<std::vector<float>> tex_rgb;  // owned texel data of each texture
  std::vector<mgpu_texture> tex;
  int32_t bg_tex = 0;
  float bg_le[3] = {0, 0, 0};
  std::vector<float> sph;
  std::vector<int32_t> sph_mat, sph_light;
  bool has_scene = false, has_n = false, has_light = false, has_flags = false;
  int32_t nmat = 0, nlight = 0;
  float camera[16] = {0, 0, 0, 0, 0, -1, 0, 1, 0, 45, 1, 0, 0, 1, 0, 0};
  int32_t width = 0, height = 0;
  mgpu_accel *accel = nullptr;
  mgpu_scene *scene = nullptr;
  mgpu_film *film = nullptr;
  bool initted = false;

  ~mgpu_renderer() {
    if (film) mgpu_film_destroy(film);
    if (scene) mgpu_scene_destroy(scene);
    if (accel) mgpu_accel_destroy(accel);
  }

  // PropertyMap::getValue(key, default) (PropertyMap.h:107-112) -- here without inserting
  double num(const char *key, double def) const {
    auto it = props.find(key);
    if (it == props.end()) return def;
    char *end = nullptr;
    double x = strtod(it->second.c_str(), &end);
    if (end == it->second.c_str()) {
      if (it->second == "true") return 1;
      if (it->second == "false") return 0;
      return def;
    }
    return x;
  }
  mgpu_scene_desc desc() const {
    mgpu_scene_desc d;
    d.ntri = ntri;
    d.tri_v = v.data();
    d.tri_n = has_n ? n.data() : nullptr;
    d.tri_mat = mat.data();
    d.tri_light = has_light ? light.data() : nullptr;
    d.tri_flags = has_flags ? flags.data() : nullptr;
    d.nmat = nmat;
    d.materials = mats.data();
    d.nlight = nlight;
    d.lights = lights.data();
    d.light_ext = light_ext.empty() ? nullptr : light_ext.data();
    d.tri_uv = uv.empty() ? nullptr : uv.data();
    d.ntex = (int32_t)tex.size();
    d.textures = tex.empty() ? nullptr : tex.data();
    d.background_tex = bg_tex;
    for (int k = 0; k < 3; ++k) d.background_le[k] = bg_le[k];
    d.nsphere = (int32_t)sph_mat.size();
    d.spheres = sph.empty() ? nullptr : sph.data();
    d.sphere_mat = sph_mat.empty() ? nullptr : sph_mat.data();
    d.sphere_light = sph_light.empty() ? nullptr : sph_light.data();
    return d;
  }
};

// errors go through the library's thread-local message
namespace mgpu {
int fail(int code, const std::string &msg);
}
static int bad(const char *msg) { return mgpu::fail(MGPU_E_INVALID, msg); }

extern "C" {

int mgpu_renderer_create(mgpu_renderer **out) {
  if (!out) return bad("mgpu_renderer_create: null argument");
  *out = new (std::nothrow) mgpu_renderer();
  if (!*out) return mgpu::fail(MGPU_E_NOMEM, "mgpu_renderer_create: out of host memory");
  return MGPU_OK;
}

int mgpu_renderer_destroy(mgpu_renderer *r) {
  delete r;
  return MGPU_OK;
}

int mgpu_renderer_set_value(mgpu_renderer *r, const char *key, const char *value) {
  if (!r || !key || !value) return bad("mgpu_renderer_set_value: null argument");
  r->props[key] = value;
  return MGPU_OK;
}

int mgpu_renderer_get_value(mgpu_renderer *r, const char *key, char *buf, size_t buflen) {
  if (!r || !key || !buf || buflen == 0) return bad("mgpu_renderer_get_value: null argument");
  auto it = r->props.find(key);
  if (it == r->props.end()) return bad("mgpu_renderer_get_value: no such key");
  strncpy(buf, it->second.c_str(), buflen - 1);
  buf[buflen - 1] = 0;
  return MGPU_OK;
}

int mgpu_renderer_set_scene(mgpu_renderer *r, const mgpu_scene_desc *d) {
  if (!r || !d) return bad("mgpu_renderer_set_scene: null argument");
  if (d->ntri < 0 || (d->ntri > 0 && (!d->tri_v || !d->tri_mat)) || d->nmat <= 0 || !d->materials ||
      d->nlight < 0 || (d->nlight > 0 && !d->lights))
    return bad("mgpu_renderer_set_scene: incomplete scene description");
  size_t T = (size_t)d->ntri;
  r->ntri = d->ntri;
  r->v.assign(d->tri_v, d->tri_v + 9 * T);
  r->has_n = d->tri_n != nullptr;
  if (r->has_n) r->n.assign(d->tri_n, d->tri_n + 9 * T);
  r->mat.assign(d->tri_mat, d->tri_mat + T);
  r->has_light = d->tri_light != nullptr;
  if (r->has_light) r->light.assign(d->tri_light, d->tri_light + T);
  r->has_flags = d->tri_flags != nullptr;
  if (r->has_flags) r->flags.assign(d->tri_flags, d->tri_flags + T);
  r->nmat = d->nmat;
  r->mats.assign(d->materials, d->materials + 16 * (size_t)d->nmat);
  r->nlight = d->nlight;
  if (d->nlight > 0) r->lights.assign(d->lights, d->lights + 16 * (size_t)d->nlight);
  else r->lights.assign(16, 0.0f);
  if (d->nlight > 0 && d->light_ext) r->light_ext.assign(d->light_ext, d->light_ext + 16 * (size_t)d->nlight);
  else r->light_ext.clear();
  if (d->tri_uv) r->uv.assign(d->tri_uv, d->tri_uv + 6 * T);
  else r->uv.clear();
  if (d->ntex < 0 || (d->ntex > 0 && !d->textures)) return bad("mgpu_renderer_set_scene: bad textures");
  r->tex_rgb.clear();
  r->tex.clear();
  for (int32_t i = 0; i < d->ntex; ++i) {
    mgpu_texture t = d->textures[i];
    if (t.width <= 0 || t.height <= 0 || !t.rgb) return bad("mgpu_renderer_set_scene: bad texture");
    r->tex_rgb.emplace_back(t.rgb, t.rgb + (size_t)t.width * t.height * 3);
    r->tex.push_back(t);
  }
  for (int32_t i = 0; i < d->ntex; ++i) r->tex[i].rgb = r->tex_rgb[i].data();
  r->bg_tex = d->background_tex;
  for (int k = 0; k < 3; ++k) r->bg_le[k] = d->background_le[k];
  if (d->nsphere < 0 || (d->nsphere > 0 && (!d->spheres || !d->sphere_mat)))
    return bad("mgpu_renderer_set_scene: bad spheres");
  r->sph.assign(d->spheres, d->spheres + 8 * (size_t)std::max(d->nsphere, 0));
  r->sph_mat.assign(d->sphere_mat, d->sphere_mat + std::max(d->nsphere, 0));
  if (d->sphere_light) r->sph_light.assign(d->sphere_light, d->sphere_light + std::max(d->nsphere, 0));
  else r->sph_light.clear();
  r->has_scene = true;
  r->initted = false;
  return MGPU_OK;
}

int mgpu_renderer_set_camera(mgpu_renderer *r, const float *c) {
  if (!r || !c) return bad("mgpu_renderer_set_camera: null argument");
  memcpy(r->camera, c, 11 * sizeof(float));  // the lens stays as mgpu_renderer_set_lens left it
  return MGPU_OK;
}

int mgpu_renderer_set_lens(mgpu_renderer *r, float aperture, float focal_length, float focal_distance) {
  if (!r) return bad("mgpu_renderer_set_lens: null renderer");
  if (!(aperture >= 0.0f) || (aperture > 0.0f && !(focal_distance > 0.0f && focal_length > 0.0f)))
    return bad("mgpu_renderer_set_lens: aperture must be >= 0, focal length and distance > 0");
  r->camera[11] = aperture;
  r->camera[12] = focal_length;
  r->camera[13] = focal_distance;
  return MGPU_OK;
}

int mgpu_renderer_set_output(mgpu_renderer *r, int32_t width, int32_t height) {
  if (!r || width <= 0 || height <= 0) return bad("mgpu_renderer_set_output: bad size");
  r->width = width;
  r->height = height;
  r->initted = false;
  return MGPU_OK;
}

// Renderer::init (Renderer.cpp:28-53): scene (kd-tree) and output must be set
int mgpu_renderer_init(mgpu_renderer *r) {
  if (!r) return bad("mgpu_renderer_init: null renderer");
  if (!r->has_scene) return bad("mgpu_renderer_init: no scene set");
  if (r->width <= 0) return bad("mgpu_renderer_init: no output set");
  if (r->film) { mgpu_film_destroy(r->film); r->film = nullptr; }
  if (r->scene) { mgpu_scene_destroy(r->scene); r->scene = nullptr; }
  if (r->accel) { mgpu_accel_destroy(r->accel); r->accel = nullptr; }
  mgpu_kd_params kp;
  kp.min_prims = (uint32_t)r->num("kdMinPrimitives", 3);
  kp.max_depth = (uint32_t)r->num("kdMaxDepth", 24);
  kp.cost_traversal = r->num("kdCostTraversal", MGPU_KD_COST_TRAVERSAL);
  kp.empty_bias = r->num("kdEmptyBias", 0.9);
  kp.threads = (uint32_t)r->num("kdNoThreads", 0);
  mgpu_scene_desc d = r->desc();
  int rc = mgpu_accel_build(&d, &kp, &r->accel);
  if (rc != MGPU_OK) return rc;
  rc = mgpu_scene_create(&d, r->accel, nullptr, &r->scene);
  if (rc != MGPU_OK) return rc;
  rc = mgpu_film_create(r->width, r->height, nullptr, &r->film);
  if (rc != MGPU_OK) return rc;
  r->initted = true;
  return MGPU_OK;
}

// Renderer::render: every super-sample pass (SuperSampleGenerator.cpp:60-90)
int mgpu_renderer_render(mgpu_renderer *r) {
  if (!r || !r->initted) return bad("mgpu_renderer_render: init() has not succeeded");
  mgpu_render_params p;
  memset(&p, 0, sizeof(p));
  p.width = r->width;
  p.height = r->height;
  p.spp = (int32_t)r->num("noSuperSamples", 4);
  if (p.spp <= 0) return bad("mgpu_renderer_render: noSuperSamples must be > 0 (progressive mode is driven by the caller)");
  p.sample_begin = 0;
  p.sample_count = p.spp;
  p.no_direct_samples = (int32_t)r->num("noDirectSamples", 1);
  p.max_depth = (int32_t)r->num("maxDepth", 0);
  p.rr_start_depth = (int32_t)r->num("rrStartDepth", 2);
  p.efficient_direct = (int32_t)r->num("efficientDirect", 1);
  p.wave_paths = (int32_t)r->num("wavePaths", 0);
  p.seed = (uint64_t)r->num("seed", 0);
  p.stream_id = 0;
  memcpy(p.camera, r->camera, sizeof(p.camera));
  int rc = mgpu_film_clear(r->film, nullptr);
  if (rc != MGPU_OK) return rc;
  return mgpu_render(r->scene, &p, r->film, nullptr);
}

int mgpu_renderer_get_output(mgpu_renderer *r, double *rgb) {
  if (!r || !rgb || !r->initted) return bad("mgpu_renderer_get_output: nothing rendered");
  return mgpu_film_read(r->film, rgb, nullptr);
}

}  // extern "C"

