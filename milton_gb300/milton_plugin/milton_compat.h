// milton_compat.h -- Milton's renderer-plugin interface, re-declared for building the GPU
// renderer plugin outside Milton's tree.
//
// A Milton dynamic renderer is a C++ object that the host casts to milton::Renderer* and drives
// through virtual calls (mlt/src/milton/loaders/MiltonJSONSceneLoader.cpp:1770-1813, 314-333;
// mlt/src/gui/MiltonApp.cpp:218-223).  These declarations keep, class by class, the virtual
// functions of Milton's headers in their declaration order (so every vtable slot is where
// Milton's code looks for it) and the data members in their order:
//   PropertyMap           mlt/src/milton/utils/PropertyMap.h:31-196
//   Renderer              mlt/src/milton/renderers/Renderer.h:30-127
//   PointSampleRenderer   mlt/src/milton/renderers/PointSampleRenderer.h:40-139
//   RenderOutput          mlt/src/milton/renderers/RenderOutput.h:34-158
//   PointSample, Viewport mlt/src/milton/renderers/PointSample.h:20-61, core/Viewport.h:20-100
// Members whose types come from Boost or Qt 4 (boost::any values, QMutex, QWaitCondition) are
// same-size stand-ins here: a build inside Milton's tree uses Milton's own headers instead
// (milton_api.h, MGPU_WITH_MILTON_HEADERS).  Scene and Camera are opaque to the plugin in that
// build and are walked through Milton's API; in this build Scene carries the flattened scene
// description the stand-in host hands over (there is no Milton scene graph to walk).
#ifndef MGPU_MILTON_COMPAT_H_
#define MGPU_MILTON_COMPAT_H_

#include <sys/time.h>

#include <deque>
#include <map>
#include <memory>
#include <string>
#include <typeinfo>
#include <vector>

#include "../../include/mgpu.h"

namespace milton {

typedef double real_t;

// boost::any: one pointer to a type-erased holder
class AnyValue {
 public:
  AnyValue() : holder_(nullptr) {}
  AnyValue(const AnyValue &o) : holder_(o.holder_ ? o.holder_->clone() : nullptr) {}
  template <typename T> AnyValue(const T &v) : holder_(new Holder<T>(v)) {}
  ~AnyValue() { delete holder_; }
  AnyValue &operator=(AnyValue o) {
    std::swap(holder_, o.holder_);
    return *this;
  }
  bool empty() const { return holder_ == nullptr; }
  const std::type_info &type() const { return holder_ ? holder_->type() : typeid(void); }
  template <typename T> T *get() {
    return holder_ && holder_->type() == typeid(T) ? &static_cast<Holder<T> *>(holder_)->value : nullptr;
  }

 private:
  struct HolderBase {
    virtual ~HolderBase() {}
    virtual const std::type_info &type() const = 0;
    virtual HolderBase *clone() const = 0;
  };
  template <typename T> struct Holder : HolderBase {
    explicit Holder(const T &v) : value(v) {}
    const std::type_info &type() const override { return typeid(T); }
    HolderBase *clone() const override { return new Holder(value); }
    T value;
  };
  HolderBase *holder_;
};

class PropertyMap {
 public:
  PropertyMap() {}
  PropertyMap(const PropertyMap &o) : map_(o.map_) {}
  virtual ~PropertyMap() {}
  virtual void inherit(const PropertyMap &m, bool overwrite = true) {
    for (auto &kv : m.map_)
      if (overwrite || !contains(kv.first)) map_[kv.first] = kv.second;
  }
  bool contains(const std::string &key) const {
    auto it = map_.find(key);
    return it != map_.end() && !it->second.empty();
  }
  template <typename T> void insert(const std::string &key, const T &value) { map_[key] = AnyValue(value); }
  // getValue(key, default): inserts the default when absent, as Milton's does
  template <typename T> T &getValue(const std::string &key, const T &def) {
    if (!contains(key)) map_[key] = AnyValue(def);
    T *p = map_[key].get<T>();
    if (!p) {  // another numeric type under this key (scene files give ints for reals)
      T v = def;
      if (auto *i = map_[key].get<int>()) v = (T)*i;
      else if (auto *u = map_[key].get<unsigned>()) v = (T)*u;
      else if (auto *d = map_[key].get<double>()) v = (T)*d;
      else if (auto *f = map_[key].get<float>()) v = (T)*f;
      else if (auto *b = map_[key].get<bool>()) v = (T)*b;
      map_[key] = AnyValue(v);
      p = map_[key].get<T>();
    }
    return *p;
  }
  AnyValue &operator[](const std::string &key) { return map_[key]; }

 protected:
  std::map<std::string, AnyValue> map_;
};

struct Point2 {
  real_t data[2];
  Point2() : data{0, 0} {}
  Point2(real_t x, real_t y) : data{x, y} {}
  real_t operator[](int i) const { return data[i]; }
};

// The radiance of a sample: rgb here (Milton's SpectralSampleSet, utils/SpectralSampleSet.h)
struct SpectralSampleSet {
  real_t rgb[3];
  SpectralSampleSet() : rgb{0, 0, 0} {}
  SpectralSampleSet(real_t r, real_t g, real_t b) : rgb{r, g, b} {}
};

// stats/Event.h: a sampled value; the renderer output reads it as a SpectralSampleSet
struct Event {
  AnyValue value;
  template <typename T> void setValue(const T &v) { value = AnyValue(v); }
  template <typename T> T &getValue() { return *value.get<T>(); }
};

struct PointSample {
  Point2 position;
  Event value;
  bool update;
  bool save;
  PointSample() : update(false), save(false) {}
  PointSample(real_t x, real_t y, bool update_ = false, bool save_ = false)
      : position(x, y), update(update_), save(save_) {}
};
typedef std::vector<PointSample> PointSampleList;
typedef std::deque<PointSample> PointSampleQueue;

struct Viewport {
  Viewport(unsigned w, unsigned h) : m_width(w), m_height(h), m_invWidth(1.0 / w), m_invHeight(1.0 / h) {}
  Viewport() : m_width(1), m_height(1), m_invWidth(1), m_invHeight(1) {}
  unsigned getWidth() const { return m_width; }
  unsigned getHeight() const { return m_height; }
  // the pixel a film position falls in, clamped to the film
  void getBin(const Point2 &pt, unsigned &x, unsigned &y) const {
    double fx = pt[0] * m_width, fy = pt[1] * m_height;
    x = fx <= 0 ? 0u : (fx >= m_width - 1 ? m_width - 1 : (unsigned)fx);
    y = fy <= 0 ? 0u : (fy >= m_height - 1 ? m_height - 1 : (unsigned)fy);
  }

 private:
  unsigned m_width, m_height;
  real_t m_invWidth, m_invHeight;
};

struct Timer {
  Timer() { reset(); }
  void reset() { gettimeofday(&m_startTime, 0); }
  double elapsed() const {
    timeval now;
    gettimeofday(&now, 0);
    return (now.tv_sec - m_startTime.tv_sec) + 1e-6 * (now.tv_usec - m_startTime.tv_usec);
  }

 private:
  timeval m_startTime;
};

// Qt 4's QMutex / QWaitCondition hold one private pointer each
struct QtMutexSlot {
  void *d = nullptr;
};
struct QtWaitConditionSlot {
  void *d = nullptr;
};

class Camera;  // a PropertyMap of camera keys here (ThinLensCamera's, cameras/ThinLensCamera.cpp:62-124)
class Scene;   // the flattened scene the stand-in host hands over
class DirectIllumination;
class Image;
class RgbaImage;
class ToneMap;
class SampleGeneratorThread;
class SampleConsumer;
template <typename T> struct ProgressiveFilterValue;

class Camera : public PropertyMap {
 public:
  virtual ~Camera() {}
};

class Scene {
 public:
  explicit Scene(const mgpu_scene_desc *desc = nullptr) : desc_(desc) {}
  virtual ~Scene() {}
  const mgpu_scene_desc *flattened() const { return desc_; }

 private:
  const mgpu_scene_desc *desc_;
};

class Renderer : public PropertyMap {
 public:
  Renderer(Camera *camera = nullptr, Scene *scene = nullptr)
      : m_camera(camera), m_scene(scene), m_initted(false), m_directIllumination(nullptr) {}
  virtual ~Renderer();
  virtual void init();
  virtual void render() = 0;
  Camera *getCamera() { return m_camera; }
  void setCamera(Camera *camera) { m_camera = camera; }
  Scene *getScene() { return m_scene; }
  void setScene(Scene *scene) { m_scene = scene; }
  virtual bool supportsOpenGL() { return false; }
  virtual bool isMLT() const { return false; }
  DirectIllumination *getDirectIllumination() { return m_directIllumination; }
  const Timer &getTimer() const { return m_timer; }
  virtual std::string getElapsedTime() const;

 protected:
  Camera *m_camera;
  Scene *m_scene;
  bool m_initted;
  DirectIllumination *m_directIllumination;
  Timer m_timer;
};

class RenderOutput : public PropertyMap {
 public:
  explicit RenderOutput(const Viewport &d)
      : m_viewport(d), m_isMLT(false), m_filterProposed(true), m_output(nullptr), m_progressiveValues(nullptr),
        m_tonemap(nullptr), m_proposed(nullptr), m_noSamples(nullptr), m_locks(nullptr), m_parent(nullptr),
        m_seconds(0) {}
  virtual ~RenderOutput();
  virtual void init();
  virtual void finalize();
  virtual void addSample(PointSample &sample);
  const Viewport &getViewport() const { return m_viewport; }
  void setViewport(const Viewport &d) { m_viewport = d; }
  ToneMap *getToneMap() { return m_tonemap; }
  Image *getImage() { return m_output; }
  virtual void setImage(Image *image);
  void setParent(Renderer *r) { m_parent = r; }
  virtual RgbaImage *getFinalizedOutput();

 protected:
  virtual void _addSample(const unsigned row, const unsigned col, PointSample &value, const real_t weight,
                          bool lock = false);

 protected:
  Viewport m_viewport;
  bool m_isMLT, m_filterProposed;
  Image *m_output;
  ProgressiveFilterValue<SpectralSampleSet> *m_progressiveValues;
  ToneMap *m_tonemap;
  unsigned long *m_proposed;
  unsigned long *m_noSamples;
  QtMutexSlot *m_locks;
  Renderer *m_parent;
  unsigned long m_seconds;
};

class PointSampleRenderer : public Renderer {
 public:
  PointSampleRenderer(RenderOutput *output = nullptr, Camera *camera = nullptr, Scene *scene = nullptr)
      : Renderer(camera, scene), m_noProducers(0), m_output(output) {}
  virtual ~PointSampleRenderer() {}
  virtual void render();
  virtual void sample(PointSample &outSample);
  virtual void finalize();
  virtual RenderOutput *getOutput() { return m_output; }
  virtual void setOutput(RenderOutput *output) { m_output = output; }
  virtual void addSharedSample(const PointSample &s);
  virtual void addSharedSamples(const PointSampleList &s);
  virtual bool getSharedSample(PointSample &outSample);
  virtual void addProducer();
  virtual void removeProducer();

 protected:
  virtual SampleGeneratorThread *_getGenerator();
  virtual SampleConsumer *_getConsumer();

 protected:
  QtMutexSlot m_renderMutex;
  QtMutexSlot m_mutex;
  QtWaitConditionSlot m_producer;
  QtWaitConditionSlot m_consumer;
  PointSampleQueue m_sharedShamples;
  unsigned m_noProducers;
  RenderOutput *m_output;
};

// DynamicPlugin.h:38-64: the plugin entry points Milton's loader resolves by name
extern "C" {
enum MILTON_PLUGIN_TYPE {
  MILTON_PLUGIN_TYPE_RENDERER = 0,
  MILTON_PLUGIN_TYPE_CAMERA,
  MILTON_PLUGIN_TYPE_OUTPUT,
  MILTON_PLUGIN_TYPE_FILTER,
  MILTON_PLUGIN_TYPE_SHAPE,
  MILTON_PLUGIN_TYPE_BSDF,
  MILTON_PLUGIN_TYPE_EMITTER,
  MILTON_PLUGIN_TYPE_MEDIUM,
  MILTON_PLUGIN_TYPE_GENERATOR,
  MILTON_PLUGIN_TYPE_METAOBJECT,
};
MILTON_PLUGIN_TYPE plugin_type();
void *plugin_new();
void plugin_delete(void *plugin);
typedef MILTON_PLUGIN_TYPE (*plugin_type_func_t)();
typedef void *(*plugin_new_func_t)();
}

}  // namespace milton

#endif  // MGPU_MILTON_COMPAT_H_
