// milton_api.h -- the Milton classes the GPU renderer plugin derives from and calls.
//
// Inside Milton's source tree (MGPU_WITH_MILTON_HEADERS defined, Milton's include directories on
// the path) these are Milton's own headers.  Elsewhere they are the re-declarations of
// milton_compat.h, with the same virtual functions in the same order.
#ifndef MGPU_MILTON_API_H_
#define MGPU_MILTON_API_H_

#ifdef MGPU_WITH_MILTON_HEADERS
#include <Material.h>
#include <Mesh.h>
#include <Plane.h>
#include <ShapeSet.h>
#include <Triangle.h>
#include <cameras/Camera.h>
#include <core/Scene.h>
#include <dynamic/DynamicPlugin.h>
#include <renderers/PointSample.h>
#include <renderers/PointSampleRenderer.h>
#include <renderers/RenderOutput.h>
#else
#include "milton_compat.h"
#endif

#endif  // MGPU_MILTON_API_H_
