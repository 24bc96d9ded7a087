// gpu_path_tracer.cpp -- Milton's dynamic renderer plugin: a PointSampleRenderer whose render()
// runs the whole image as sm_103a wavefront kernels through libmgpu.so.
//
// Milton loads it from a scene file's `"renderer": {"type": "dynamic", "path":
// "libmgpu_milton.so", ...}` (mlt/src/milton/loaders/MiltonJSONSceneLoader.cpp:739-741): its
// loader resolves plugin_type / plugin_new, checks the type, casts the new object to
// milton::Renderer* and copies the renderer's other keys into its PropertyMap (:1770-1813, :775);
// then it sets the output, scene and camera (:314-333), MiltonApp::addRenderer calls init()
// (mlt/src/gui/MiltonApp.cpp:218-223) and a RenderThread calls render()
// (mlt/src/gui/RenderThread.cpp:26-29).
//
//   init()    Renderer::init (mlt/src/milton/renderers/Renderer.cpp:28-53): the scene flattened in
//             ShapeSet order, the SAH kd-tree built on the host, scene and film made resident
//   render()  PointSampleRenderer::render (mlt/src/milton/renderers/PointSampleRenderer.cpp:24-81)
//             over every noSuperSamples pass on the GPU; the finalized per-pixel means go to the
//             RenderOutput as one sample per pixel at its centre (RenderOutput::addSample), so the
//             output's value of every pixel is the GPU film's FP64 mean
//   sample()  a single point sample is not rendered on the GPU: it returns black, as the base
//             PointSampleRenderer::sample does (:83-85); render() never calls it
//
// Keys (PropertyMap, as the scene file's renderer block gives them): noSuperSamples (4),
// noDirectSamples (1), efficientDirect (true), maxDepth (0 = none), rrStartDepth (2), seed (0),
// kdMinPrimitives (3), kdMaxDepth (24), kdCostTraversal (MGPU_KD_COST_TRAVERSAL, 3; Milton's is 1),
// kdEmptyBias (0.9), wavePaths (0).
// Milton has no error codes on this path; a failed init() or render() leaves the reason in
// mgpu_last_error() and on stderr, and render() then outputs nothing.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "milton_api.h"
#include "../../include/mgpu.h"

namespace mgpu_milton {

// The flattened scene: owned arrays behind an mgpu_scene_desc.
struct FlatScene {
  std::vector<float> v, n, mats, lights, light_ext;
  std::vector<int32_t> mat, light;
  std::vector<uint32_t> flags;
  float camera[16] = {0};
  mgpu_scene_desc desc() const {
    mgpu_scene_desc d;
    memset(&d, 0, sizeof(d));
    d.ntri = (int64_t)mat.size();
    d.tri_v = v.data();
    d.tri_n = n.data();
    d.tri_mat = mat.data();
    d.tri_light = light.data();
    d.tri_flags = flags.data();
    d.nmat = (int32_t)(mats.size() / 16);
    d.materials = mats.data();
    d.nlight = (int32_t)(lights.size() / 16);
    d.lights = d.nlight ? lights.data() : nullptr;
    d.light_ext = d.nlight ? light_ext.data() : nullptr;
    return d;
  }
};

static bool fail(std::string &err, const std::string &msg) {
  err = msg;
  return false;
}

#ifdef MGPU_WITH_MILTON_HEADERS
// ---- Milton's scene graph -> the flattened soup (the same rules as milton_gb300/sceneloader.py
// applies to scene files, here over the objects Milton's loader built) -------------------------
using milton::real_t;

static void spectrum3(milton::Material *m, const char *key, double def, double out[3]) {
  if (!m->contains(key)) {
    out[0] = out[1] = out[2] = def;
    return;
  }
  const milton::SpectralSampleSet &s = m->getValue<milton::SpectralSampleSet>(key);
  for (unsigned k = 0; k < 3; ++k) out[k] = s[k < s.getN() ? k : 0].value;
}

static double scalar(milton::Material *m, const char *key, double def) {
  return m->contains(key) ? (double)m->getValue<real_t>(key, (real_t)def) : def;
}

// material record (include/mgpu.h): Material::getBSDF keys with the BSDFs' defaults
// (DiffuseBSDF kd 0.5; ModifiedPhongBSDF kd / ks, ModifiedPhongBSDF.cpp:48-60; DielectricBSDF)
static bool material_record(milton::Material *m, std::vector<float> &mats, std::string &err) {
  float r[16] = {0};
  const std::string bsdf = m->contains("bsdf") ? m->getValue<std::string>("bsdf") : std::string("diffuse");
  double kd[3], ks[3];
  if (bsdf == "diffuse" || bsdf == "absorbent") {
    spectrum3(m, "kd", bsdf == "absorbent" ? 0.0 : 0.5, kd);
    if (bsdf == "absorbent") kd[0] = kd[1] = kd[2] = 0.0;
    r[0] = MGPU_MAT_DIFFUSE;
    for (int k = 0; k < 3; ++k) r[1 + k] = (float)kd[k];
  } else if (bsdf == "modifiedPhong" || bsdf == "phong") {
    const bool none = !m->contains("kd") && !m->contains("ks");
    spectrum3(m, "kd", none ? 0.5 : 0.0, kd);
    spectrum3(m, "ks", none ? 0.5 : 0.0, ks);
    r[0] = MGPU_MAT_PHONG;
    for (int k = 0; k < 3; ++k) r[1 + k] = (float)kd[k], r[4 + k] = (float)ks[k];
    r[7] = (float)scalar(m, "n", 1.0);
  } else if (bsdf == "dielectric") {
    spectrum3(m, "ks", 1.0, ks);
    r[0] = MGPU_MAT_DIELECTRIC;
    for (int k = 0; k < 3; ++k) r[4 + k] = (float)ks[k];
    r[9] = (float)scalar(m, "transparency", 1.0);
  } else {
    return fail(err, "material bsdf '" + bsdf + "' is not rendered by the GPU path");
  }
  double ior[3];
  spectrum3(m, "ior", 1.000293, ior);  // IndexOfRefraction::AIR
  r[8] = (float)ior[0];
  if (ior[1] != ior[0] || ior[2] != ior[0]) r[14] = (float)ior[1], r[15] = (float)ior[2];
  mats.insert(mats.end(), r, r + 16);
  return true;
}

static void xf_point(const milton::Matrix4x4 &M, const milton::Point3 &p, float *out) {
  const milton::Point3 q = M * p;
  out[0] = (float)q[0], out[1] = (float)q[1], out[2] = (float)q[2];
}

// inverse transpose of the upper 3x3, as Transformable::_transformVector3ObjToWorld
static void xf_normal(const milton::Matrix4x4 &inv, const milton::Vector3 &nObj, float *out) {
  const real_t *m = *inv;
  milton::Vector3 w(nObj[0] * m[0] + nObj[1] * m[4] + nObj[2] * m[8],
                    nObj[0] * m[1] + nObj[1] * m[5] + nObj[2] * m[9],
                    nObj[0] * m[2] + nObj[1] * m[6] + nObj[2] * m[10]);
  w.normalize();
  out[0] = (float)w[0], out[1] = (float)w[1], out[2] = (float)w[2];
}

static bool flatten(milton::Scene *scene, milton::Camera *camera, FlatScene &f, std::string &err) {
  if (!scene || !scene->getShapes()) return fail(err, "no scene set");
  std::vector<milton::Material *> seen;
  auto mat_index = [&](milton::Material *m, int32_t &out) -> bool {
    for (size_t i = 0; i < seen.size(); ++i)
      if (seen[i] == m) return (out = (int32_t)i), true;
    if (!material_record(m, f.mats, err)) return false;
    seen.push_back(m);
    out = (int32_t)seen.size() - 1;
    return true;
  };
  for (milton::Shape *shape : scene->getShapes()->getPrimitives()) {
    milton::Material *m = shape->getMaterial();
    if (!m) return fail(err, "a shape without a material");
    int32_t mi;
    if (!mat_index(m, mi)) return false;
    const std::string emitter = m->contains("emitter") ? m->getValue<std::string>("emitter") : std::string("null");
    auto push_tri = [&](const float *a, const float *b, const float *c, const float *na, const float *nb,
                        const float *nc, uint32_t flag, int32_t light) {
      const float *vs[3] = {a, b, c}, *ns[3] = {na, nb, nc};
      for (int k = 0; k < 3; ++k) {
        f.v.insert(f.v.end(), vs[k], vs[k] + 3);
        f.n.insert(f.n.end(), ns[k], ns[k] + 3);
      }
      f.mat.push_back(mi);
      f.light.push_back(light);
      f.flags.push_back(flag);
    };
    if (auto *mesh = dynamic_cast<milton::Mesh *>(shape)) {
      if (emitter != "null") return fail(err, "an emitting Mesh is not taken by this plugin (use planes)");
      const milton::Matrix4x4 &M = mesh->getTransToWorld(), &Mi = mesh->getTransToWorldInv();
      unsigned nt = 0;
      const milton::MeshTriangle *tris = mesh->getTriangles(nt);
      const milton::Vertex *vert = mesh->getVertices();
      const milton::Normal *nrm = mesh->getNormals();
      for (unsigned t = 0; t < nt; ++t) {
        float p[3][3], q[3][3];
        const unsigned vi[3] = {tris[t].A, tris[t].B, tris[t].C}, ni[3] = {tris[t].nA, tris[t].nB, tris[t].nC};
        for (int k = 0; k < 3; ++k) {
          xf_point(M, milton::Point3(vert[vi[k]][0], vert[vi[k]][1], vert[vi[k]][2]), p[k]);
          xf_normal(Mi, nrm[ni[k]], q[k]);
        }
        push_tri(p[0], p[1], p[2], q[0], q[1], q[2], 0u, -1);
      }
    } else if (auto *tri = dynamic_cast<milton::Triangle *>(shape)) {
      if (emitter != "null") return fail(err, "an emitting Triangle is not taken by this plugin (use planes)");
      const milton::Matrix4x4 &M = tri->getTransToWorld();
      float p[3][3], q[3];
      for (int k = 0; k < 3; ++k)
        xf_point(M, milton::Point3(tri->vertices[k][0], tri->vertices[k][1], tri->vertices[k][2]), p[k]);
      milton::Vector3 e1 = tri->vertices[1] - tri->vertices[0], e2 = tri->vertices[2] - tri->vertices[0];
      xf_normal(tri->getTransToWorldInv(), e1.cross(e2).getNormalized(), q);
      push_tri(p[0], p[1], p[2], q, q, q, MGPU_TRI_CULLED, -1);
    } else if (auto *pl = dynamic_cast<milton::Plane *>(shape)) {
      // the unit plane y = 0, |x|, |z| <= 1/2 under its transform (Plane.cpp:25-59, 91-93)
      const milton::Matrix4x4 &M = pl->getTransToWorld();
      float c[4][3], ctr[3], q[3];
      const double cx[4] = {-0.5, 0.5, 0.5, -0.5}, cz[4] = {-0.5, -0.5, 0.5, 0.5};
      for (int k = 0; k < 4; ++k) xf_point(M, milton::Point3(cx[k], 0, cz[k]), c[k]);
      xf_point(M, milton::Point3(0, 0, 0), ctr);
      xf_normal(pl->getTransToWorldInv(), milton::Vector3(0, 1, 0), q);
      int32_t li = -1;
      if (emitter == "oriented" || emitter == "omni") {
        float ex[3], ez[3], L[16] = {0}, X[16] = {0};
        for (int k = 0; k < 3; ++k) ex[k] = c[1][k] - c[0][k], ez[k] = c[3][k] - c[0][k];
        const double ax = ex[1] * ez[2] - ex[2] * ez[1], ay = ex[2] * ez[0] - ex[0] * ez[2],
                     az = ex[0] * ez[1] - ex[1] * ez[0];
        const double area = sqrt(ax * ax + ay * ay + az * az);
        double power[3];
        spectrum3(m, "power", 1.0, power);
        const double per_sr = emitter == "oriented" ? M_PI : 4.0 * M_PI;  // Emitter.cpp:34-50, OmniEmitter.cpp
        for (int k = 0; k < 3; ++k) {
          L[k] = ctr[k], L[3 + k] = ex[k], L[6 + k] = ez[k], L[9 + k] = q[k];
          L[13 + k] = (float)(power[k] / (area * per_sr));
        }
        L[12] = (float)area;
        X[15] = emitter == "omni" ? 1.0f : 0.0f;
        f.lights.insert(f.lights.end(), L, L + 16);
        f.light_ext.insert(f.light_ext.end(), X, X + 16);
        li = (int32_t)(f.lights.size() / 16) - 1;
      } else if (emitter != "null") {
        return fail(err, "'" + emitter + "' emitters are not rendered by the GPU path");
      }
      push_tri(c[0], c[3], c[2], q, q, q, 0u, li);
      push_tri(c[0], c[2], c[1], q, q, q, 0u, li);
    } else {
      return fail(err, "a shape other than Mesh, Triangle or Plane is not rendered by the GPU path");
    }
  }
  // ThinLensCamera keys (ThinLensCamera.cpp:62-124); the aperture is given in mm
  if (!camera) return fail(err, "no camera set");
  const milton::Point3 eye = camera->getValue<milton::Point3>("eye", milton::Point3(2, 2, 2));
  const milton::Point3 focus = camera->getValue<milton::Point3>("focus", milton::Point3());
  const milton::Vector3 look = camera->getValue<milton::Vector3>("look", (focus - eye).getNormalized());
  const milton::Vector3 up = camera->getValue<milton::Vector3>("up", milton::Vector3(0, 1, 0));
  for (int k = 0; k < 3; ++k) f.camera[k] = (float)eye[k], f.camera[3 + k] = (float)look[k], f.camera[6 + k] = (float)up[k];
  f.camera[9] = (float)camera->getValue<real_t>("heightAngle", 45);
  f.camera[10] = (float)camera->getValue<real_t>("aspectRatio", 1);
  const double aperture = camera->contains("aperture") ? camera->getValue<real_t>("aperture", 0) / 1000.0 : 0.0;
  f.camera[11] = (float)aperture;
  f.camera[12] = (float)(camera->getValue<real_t>("fstop", 14) * aperture);
  f.camera[13] = (float)camera->getValue<real_t>("focalDistance", 1);
  return true;
}
#else
// ---- the stand-in host's scene: already flattened -------------------------------------------
static bool flatten(milton::Scene *scene, milton::Camera *camera, FlatScene &f, std::string &err) {
  const mgpu_scene_desc *d = scene ? scene->flattened() : nullptr;
  if (!d || d->ntri <= 0) return fail(err, "no scene set");
  const size_t T = (size_t)d->ntri;
  f.v.assign(d->tri_v, d->tri_v + 9 * T);
  if (d->tri_n) f.n.assign(d->tri_n, d->tri_n + 9 * T);
  else return fail(err, "the scene has no shading normals");
  f.mat.assign(d->tri_mat, d->tri_mat + T);
  if (d->tri_light) f.light.assign(d->tri_light, d->tri_light + T);
  else f.light.assign(T, -1);
  if (d->tri_flags) f.flags.assign(d->tri_flags, d->tri_flags + T);
  else f.flags.assign(T, 0u);
  f.mats.assign(d->materials, d->materials + 16 * (size_t)d->nmat);
  if (d->nlight > 0) {
    f.lights.assign(d->lights, d->lights + 16 * (size_t)d->nlight);
    if (d->light_ext) f.light_ext.assign(d->light_ext, d->light_ext + 16 * (size_t)d->nlight);
    else f.light_ext.assign(16 * (size_t)d->nlight, 0.0f);
  }
  if (!camera) return fail(err, "no camera set");
  std::vector<milton::real_t> &cam = camera->getValue<std::vector<milton::real_t>>("mgpu.camera", {});
  if (cam.size() < 11) return fail(err, "no camera set");
  for (size_t k = 0; k < cam.size() && k < 16; ++k) f.camera[k] = (float)cam[k];
  return true;
}
#endif

class GpuPathTracer : public milton::PointSampleRenderer {
 public:
  GpuPathTracer() {}
  ~GpuPathTracer() override { release(); }

  void init() override {
    release();
    m_initted = false;
    if (!m_output) return report("init: no output set");
    const milton::Viewport &vp = m_output->getViewport();
    width_ = (int32_t)vp.getWidth();
    height_ = (int32_t)vp.getHeight();
    flat_ = FlatScene();
    if (!flatten(m_scene, m_camera, flat_, error_)) return report("init: " + error_);
    mgpu_kd_params kp;
    kp.min_prims = (uint32_t)num("kdMinPrimitives", 3);
    kp.max_depth = (uint32_t)num("kdMaxDepth", 24);
    kp.cost_traversal = num("kdCostTraversal", MGPU_KD_COST_TRAVERSAL);
    kp.empty_bias = num("kdEmptyBias", 0.9);
    kp.threads = (uint32_t)num("kdNoThreads", 0);
    const mgpu_scene_desc d = flat_.desc();
    if (mgpu_accel_build(&d, &kp, &accel_) != MGPU_OK || mgpu_scene_create(&d, accel_, nullptr, &scene_) != MGPU_OK ||
        mgpu_film_create(width_, height_, nullptr, &film_) != MGPU_OK)
      return report(std::string("init: ") + mgpu_last_error());
    m_initted = true;
  }

  void render() override {
    if (!m_initted) init();
    if (!m_initted || !m_output) return;
    m_timer.reset();
    m_output->setParent(this);
    m_output->init();
    mgpu_render_params p;
    memset(&p, 0, sizeof(p));
    p.width = width_;
    p.height = height_;
    p.spp = (int32_t)num("noSuperSamples", 4);
    if (p.spp <= 0) return report("render: noSuperSamples must be > 0 (progressive mode is the render service's)");
    p.sample_count = p.spp;
    p.no_direct_samples = (int32_t)num("noDirectSamples", 1);
    p.max_depth = (int32_t)num("maxDepth", 0);
    p.rr_start_depth = (int32_t)num("rrStartDepth", 2);
    p.efficient_direct = (int32_t)num("efficientDirect", 1);
    p.wave_paths = (int32_t)num("wavePaths", 0);
    p.seed = (uint64_t)num("seed", 0);
    memcpy(p.camera, flat_.camera, sizeof(p.camera));
    std::vector<double> rgb((size_t)width_ * height_ * 3);
    if (mgpu_film_clear(film_, nullptr) != MGPU_OK || mgpu_render(scene_, &p, film_, nullptr) != MGPU_OK ||
        mgpu_film_read(film_, rgb.data(), nullptr) != MGPU_OK)
      return report(std::string("render: ") + mgpu_last_error());
    // one sample per pixel, at its centre, carrying the pixel's mean over all passes
    for (int32_t y = 0; y < height_; ++y)
      for (int32_t x = 0; x < width_; ++x) {
        const double *c = &rgb[((size_t)y * width_ + x) * 3];
        milton::PointSample s((x + 0.5) / width_, (y + 0.5) / height_);
        s.value.setValue(milton::SpectralSampleSet(c[0], c[1], c[2]));
        m_output->addSample(s);
      }
    m_output->finalize();
    finalize();
  }

  void sample(milton::PointSample &out) override { out.value.setValue(milton::SpectralSampleSet()); }
  void finalize() override {}
  milton::RenderOutput *getOutput() override { return m_output; }
  void setOutput(milton::RenderOutput *output) override { m_output = output; }

 private:
  // PropertyMap values as numbers; scene files give integers or reals, booleans as true/false
  double num(const char *key, double def) {
    if (!contains(key)) return def;
#ifdef MGPU_WITH_MILTON_HEADERS
    if ((*this)[key].type() == typeid(bool)) return boost::any_cast<bool>((*this)[key]) ? 1.0 : 0.0;
#endif
    return (double)getValue<milton::real_t>(key, (milton::real_t)def);
  }
  void report(const std::string &msg) {
    error_ = msg;
    fprintf(stderr, "mgpu GpuPathTracer: %s\n", msg.c_str());
  }
  void release() {
    if (film_) mgpu_film_destroy(film_);
    if (scene_) mgpu_scene_destroy(scene_);
    if (accel_) mgpu_accel_destroy(accel_);
    film_ = nullptr;
    scene_ = nullptr;
    accel_ = nullptr;
  }

  FlatScene flat_;
  mgpu_accel *accel_ = nullptr;
  mgpu_scene *scene_ = nullptr;
  mgpu_film *film_ = nullptr;
  int32_t width_ = 0, height_ = 0;
  std::string error_;
};

}  // namespace mgpu_milton

namespace milton {
extern "C" {
// DynamicPlugin.h:51-53
MILTON_PLUGIN_TYPE plugin_type() { return MILTON_PLUGIN_TYPE_RENDERER; }
void *plugin_new() {
  return static_cast<milton::Renderer *>(new (std::nothrow) mgpu_milton::GpuPathTracer());
}
void plugin_delete(void *plugin) { delete static_cast<milton::Renderer *>(plugin); }
}
}  // namespace milton
