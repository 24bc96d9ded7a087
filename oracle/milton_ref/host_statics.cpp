// host_statics.cpp -- test-oracle support: the static state of Milton's ResourceManager (its
// .cpp needs Milton's plugin loader, which the oracle does not build) and an image loader that
// loads nothing (no image maps on the paths the oracle runs).
#include <ResourceManager.h>
#include <common/image/Image.h>

namespace milton {
ImagePtrMap ResourceManager::s_imagePtrMap;
PropertyMap ResourceManager::s_propertyMap;
QMutex ResourceManager::s_mutex;
Log ResourceManager::log;
Image *Image::load(const std::string &) { return NULL; }
}  // namespace milton
