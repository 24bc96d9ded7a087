// milton_layout.cpp -- prints where the plugin-facing Milton classes keep each virtual function
// (vtable byte offset, from the Itanium C++ ABI's pointer-to-member-function representation:
// 1 + offset for a virtual function) and each data member the plugin touches (byte offset).
// Test harness: compiled once against milton_gb300/milton_plugin/milton_compat.h and once
// against Milton's own headers (MGPU_WITH_MILTON_HEADERS), the two outputs must be equal.
#include <stdio.h>
#include <string.h>

#include <cstddef>

#include "../../milton_gb300/milton_plugin/milton_api.h"

template <typename F> static long slot(F f) {
  static_assert(sizeof(F) == 2 * sizeof(long), "Itanium ABI member-function pointer");
  long v[2];
  memcpy(v, &f, sizeof(v));
  return v[0] & 1 ? v[0] - 1 : -1;  // -1: not virtual
}

// a derived probe reaches the protected members; a data-member pointer holds the byte offset
struct Probe : milton::PointSampleRenderer {
  template <typename M> static long off(M m) {
    long v;
    memcpy(&v, &m, sizeof(v));
    return v;
  }
  static void print() {
    printf("Renderer::m_camera %ld\n", off(&Probe::m_camera));
    printf("Renderer::m_scene %ld\n", off(&Probe::m_scene));
    printf("Renderer::m_initted %ld\n", off(&Probe::m_initted));
    printf("Renderer::m_directIllumination %ld\n", off(&Probe::m_directIllumination));
    printf("Renderer::m_timer %ld\n", off(&Probe::m_timer));
  }
};

struct OutputProbe : milton::RenderOutput {
  template <typename M> static long off(M m) {
    long v;
    memcpy(&v, &m, sizeof(v));
    return v;
  }
  static void print() { printf("RenderOutput::m_viewport %ld\n", off(&OutputProbe::m_viewport)); }
};

int main() {
  using milton::PointSampleRenderer;
  using milton::PropertyMap;
  using milton::RenderOutput;
  using milton::Renderer;
  printf("PropertyMap::inherit %ld\n", slot(&PropertyMap::inherit));
  printf("Renderer::init %ld\n", slot(&Renderer::init));
  printf("Renderer::render %ld\n", slot(&Renderer::render));
  printf("Renderer::supportsOpenGL %ld\n", slot(&Renderer::supportsOpenGL));
  printf("Renderer::isMLT %ld\n", slot(&Renderer::isMLT));
  printf("Renderer::getElapsedTime %ld\n", slot(&Renderer::getElapsedTime));
  printf("PointSampleRenderer::render %ld\n", slot(&PointSampleRenderer::render));
  printf("PointSampleRenderer::sample %ld\n", slot(&PointSampleRenderer::sample));
  printf("PointSampleRenderer::finalize %ld\n", slot(&PointSampleRenderer::finalize));
  printf("PointSampleRenderer::getOutput %ld\n", slot(&PointSampleRenderer::getOutput));
  printf("PointSampleRenderer::setOutput %ld\n", slot(&PointSampleRenderer::setOutput));
  printf("PointSampleRenderer::addSharedSample %ld\n", slot(&PointSampleRenderer::addSharedSample));
  printf("PointSampleRenderer::addSharedSamples %ld\n", slot(&PointSampleRenderer::addSharedSamples));
  printf("PointSampleRenderer::getSharedSample %ld\n", slot(&PointSampleRenderer::getSharedSample));
  printf("PointSampleRenderer::addProducer %ld\n", slot(&PointSampleRenderer::addProducer));
  printf("PointSampleRenderer::removeProducer %ld\n", slot(&PointSampleRenderer::removeProducer));
  printf("RenderOutput::init %ld\n", slot(&RenderOutput::init));
  printf("RenderOutput::finalize %ld\n", slot(&RenderOutput::finalize));
  printf("RenderOutput::addSample %ld\n", slot(&RenderOutput::addSample));
  printf("RenderOutput::setImage %ld\n", slot(&RenderOutput::setImage));
  printf("RenderOutput::getFinalizedOutput %ld\n", slot(&RenderOutput::getFinalizedOutput));
  printf("sizeof(PropertyMap) %zu\n", sizeof(PropertyMap));
  printf("sizeof(Viewport) %zu\n", sizeof(milton::Viewport));
  Probe::print();
  OutputProbe::print();
  return 0;
}
