// milton_host.cpp -- a stand-in for the Milton side of the renderer plugin boundary (test harness).
//
// It defines the out-of-line members of the Milton classes re-declared in
// milton_gb300/milton_plugin/milton_compat.h (what Milton's core library provides to a plugin) and
// drives a dynamic renderer the way Milton does:
//   1. load the library and resolve plugin_type / plugin_new, check the type, cast the new
//      object to milton::Renderer*          (mlt/src/milton/loaders/MiltonJSONSceneLoader.cpp:1770-1813)
//   2. copy the renderer block's keys into its PropertyMap                              (:775)
//   3. dynamic_cast to PointSampleRenderer, setOutput, setScene, setCamera              (:314-333)
//   4. Renderer::init() as MiltonApp::addRenderer does       (mlt/src/gui/MiltonApp.cpp:218-223)
//   5. Renderer::render() as a RenderThread does             (mlt/src/gui/RenderThread.cpp:26-29)
// then writes the RenderOutput's per-pixel values.  Its RenderOutput keeps Milton's progressive
// per-pixel value sum(w L) / sum(w) (mlt/src/milton/filters/ProgressiveFilterValue.h:18-38).
//
//   milton_host --check <plugin.so>          steps 1-3 and an init() without a scene (no GPU)
//   milton_host <plugin.so> <scene.bin> <out.bin> key=value...
// scene.bin: "MHSC", i64 ntri, i32 nmat, i32 nlight, f32 camera[16], i32 width, i32 height,
// then tri_v, tri_n (ntri*9 f32), tri_mat, tri_light (ntri i32), tri_flags (ntri u32),
// materials (nmat*16 f32), lights, light_ext (nlight*16 f32).
// out.bin: width*height*3 f64 values, then width*height u64 sample counts.
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../milton_gb300/milton_plugin/milton_compat.h"

namespace milton {

// ---- what Milton's core library provides ------------------------------------------------------
Renderer::~Renderer() {}
void Renderer::init() { m_initted = true; }
std::string Renderer::getElapsedTime() const { return std::to_string(m_timer.elapsed()) + " s"; }

void PointSampleRenderer::render() {}
void PointSampleRenderer::sample(PointSample &out) { out.value.setValue(SpectralSampleSet()); }
void PointSampleRenderer::finalize() {}
void PointSampleRenderer::addSharedSample(const PointSample &s) { m_sharedShamples.push_back(s); }
void PointSampleRenderer::addSharedSamples(const PointSampleList &s) {
  m_sharedShamples.insert(m_sharedShamples.end(), s.begin(), s.end());
}
bool PointSampleRenderer::getSharedSample(PointSample &out) {
  if (m_sharedShamples.empty()) return false;
  out = m_sharedShamples.front();
  m_sharedShamples.pop_front();
  return true;
}
void PointSampleRenderer::addProducer() { ++m_noProducers; }
void PointSampleRenderer::removeProducer() { --m_noProducers; }
SampleGeneratorThread *PointSampleRenderer::_getGenerator() { return nullptr; }
SampleConsumer *PointSampleRenderer::_getConsumer() { return nullptr; }

RenderOutput::~RenderOutput() {}
void RenderOutput::init() {}
void RenderOutput::finalize() {}
void RenderOutput::addSample(PointSample &sample) {
  unsigned row, col;
  m_viewport.getBin(sample.position, col, row);
  _addSample(row, col, sample, 1, true);
}
void RenderOutput::setImage(Image *image) { m_output = image; }
RgbaImage *RenderOutput::getFinalizedOutput() { return nullptr; }
void RenderOutput::_addSample(const unsigned, const unsigned, PointSample &, const real_t, bool) {}

}  // namespace milton

namespace {

// The host's output: per pixel sum(w L) and sum(w), as ProgressiveFilterValue keeps them.
class HostOutput : public milton::RenderOutput {
 public:
  explicit HostOutput(const milton::Viewport &vp) : RenderOutput(vp) {}
  void init() override {
    const size_t n = (size_t)m_viewport.getWidth() * m_viewport.getHeight();
    sum.assign(3 * n, 0.0);
    wsum.assign(n, 0.0);
    count.assign(n, 0);
  }
  void addSample(milton::PointSample &s) override {
    unsigned col, row;
    m_viewport.getBin(s.position, col, row);
    _addSample(row, col, s, 1.0, true);
  }
  std::vector<double> sum, wsum;
  std::vector<uint64_t> count;

 protected:
  void _addSample(const unsigned row, const unsigned col, milton::PointSample &s, const milton::real_t w,
                  bool) override {
    const size_t p = (size_t)row * m_viewport.getWidth() + col;
    const milton::SpectralSampleSet &L = s.value.getValue<milton::SpectralSampleSet>();
    for (int k = 0; k < 3; ++k) sum[3 * p + k] += w * L.rgb[k];
    wsum[p] += w;
    ++count[p];
  }
};

template <typename T> bool read_n(FILE *f, std::vector<T> &v, size_t n) {
  v.resize(n);
  return n == 0 || fread(v.data(), sizeof(T), n, f) == n;
}

int die(const std::string &msg) {
  fprintf(stderr, "milton_host: %s\n", msg.c_str());
  return 1;
}

// step 1: the loader's _parse_dynamic_plugin<Renderer, MILTON_PLUGIN_TYPE_RENDERER>
milton::Renderer *load_renderer(const char *path, std::string &err) {
  void *lib = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!lib) return err = std::string("plugin failed to load: ") + dlerror(), nullptr;
  void *type_sym = dlsym(lib, "plugin_type");
  void *new_sym = dlsym(lib, "plugin_new");
  if (!type_sym) return err = "invalid plugin; could not find plugin_type symbol", nullptr;
  if (!new_sym) return err = "invalid plugin; could not find plugin_new symbol", nullptr;
  milton::MILTON_PLUGIN_TYPE t = ((milton::plugin_type_func_t)type_sym)();
  if (t != milton::MILTON_PLUGIN_TYPE_RENDERER)
    return err = "dynamic plugin expected type '0' but found type '" + std::to_string((int)t) + "'", nullptr;
  void *plugin = ((milton::plugin_new_func_t)new_sym)();
  if (!plugin) return err = "invalid plugin; plugin_new returned NULL", nullptr;
  return (milton::Renderer *)plugin;
}

// step 2: scene-file values are ints, reals or booleans
void set_property(milton::Renderer *r, const std::string &kv) {
  const size_t eq = kv.find('=');
  const std::string key = kv.substr(0, eq), val = kv.substr(eq + 1);
  if (val == "true" || val == "false") r->insert(key, val == "true");
  else if (val.find_first_of(".eE") != std::string::npos) r->insert(key, (milton::real_t)atof(val.c_str()));
  else r->insert(key, atoi(val.c_str()));
}

}  // namespace

int main(int argc, char **argv) {
  if (argc == 3 && std::string(argv[1]) == "--check") {
    std::string err;
    milton::Renderer *r = load_renderer(argv[2], err);
    if (!r) return die(err);
    auto *psr = dynamic_cast<milton::PointSampleRenderer *>(r);
    if (!psr) return die("the plugin's renderer is not a PointSampleRenderer");
    HostOutput out(milton::Viewport(4, 4));
    psr->setOutput(&out);
    if (psr->getOutput() != &out) return die("setOutput / getOutput do not round-trip");
    r->init();  // no scene: reports and stays uninitialised, touches no device
    printf("ok plugin_type=0 PointSampleRenderer initialised=%d\n", 0);
    delete r;
    return 0;
  }
  if (argc < 4) return die("usage: milton_host [--check] <plugin.so> <scene.bin> <out.bin> key=value...");
  FILE *f = fopen(argv[2], "rb");
  if (!f) return die(std::string("cannot open ") + argv[2]);
  char magic[4];
  int64_t ntri = 0;
  int32_t nmat = 0, nlight = 0, W = 0, H = 0;
  float cam[16];
  if (fread(magic, 1, 4, f) != 4 || memcmp(magic, "MHSC", 4) != 0 || fread(&ntri, 8, 1, f) != 1 ||
      fread(&nmat, 4, 1, f) != 1 || fread(&nlight, 4, 1, f) != 1 || fread(cam, 4, 16, f) != 16 ||
      fread(&W, 4, 1, f) != 1 || fread(&H, 4, 1, f) != 1)
    return die("bad scene file");
  std::vector<float> v, n, mats, lights, ext;
  std::vector<int32_t> mat, light;
  std::vector<uint32_t> flags;
  if (!read_n(f, v, 9 * ntri) || !read_n(f, n, 9 * ntri) || !read_n(f, mat, ntri) || !read_n(f, light, ntri) ||
      !read_n(f, flags, ntri) || !read_n(f, mats, 16 * (size_t)nmat) || !read_n(f, lights, 16 * (size_t)nlight) ||
      !read_n(f, ext, 16 * (size_t)nlight))
    return die("short scene file");
  fclose(f);
  mgpu_scene_desc desc;
  memset(&desc, 0, sizeof(desc));
  desc.ntri = ntri;
  desc.tri_v = v.data();
  desc.tri_n = n.data();
  desc.tri_mat = mat.data();
  desc.tri_light = light.data();
  desc.tri_flags = flags.data();
  desc.nmat = nmat;
  desc.materials = mats.data();
  desc.nlight = nlight;
  desc.lights = lights.data();
  desc.light_ext = ext.data();

  std::string err;
  milton::Renderer *r = load_renderer(argv[1], err);
  if (!r) return die(err);
  for (int i = 4; i < argc; ++i) set_property(r, argv[i]);
  auto *psr = dynamic_cast<milton::PointSampleRenderer *>(r);
  if (!psr) return die("the plugin's renderer is not a PointSampleRenderer");
  HostOutput out(milton::Viewport((unsigned)W, (unsigned)H));
  psr->setOutput(&out);
  milton::Scene scene(&desc);
  milton::Camera camera;
  camera.insert("mgpu.camera", std::vector<milton::real_t>(cam, cam + 16));
  r->setScene(&scene);
  r->setCamera(&camera);
  r->init();
  r->render();
  if (out.wsum.empty()) return die("render() produced no output");
  const size_t np = (size_t)W * H;
  std::vector<double> mean(3 * np);
  for (size_t p = 0; p < np; ++p)
    for (int k = 0; k < 3; ++k) mean[3 * p + k] = out.wsum[p] > 0 ? out.sum[3 * p + k] / out.wsum[p] : 0.0;
  FILE *o = fopen(argv[3], "wb");
  if (!o || fwrite(mean.data(), 8, mean.size(), o) != mean.size() || fwrite(out.count.data(), 8, np, o) != np)
    return die("cannot write the output");
  fclose(o);
  delete r;
  return 0;
}
