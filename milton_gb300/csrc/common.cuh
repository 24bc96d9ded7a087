// common.cuh -- internal declarations shared by the libmgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/mgpu.h"
#include "hd_shade.h"
#include "hd_trace.h"
#include "kdbuild.h"

namespace mgpu {

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

extern std::atomic<uint64_t> g_launches;

#define MGPU_CUDA(call)                                  \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// device-side error word bits (kernels set a bit and skip the access instead of faulting)
constexpr uint32_t kErrStack = 1u;
constexpr uint32_t kErrIndex = 2u;

int device_sm_count();

// material image maps (texture.cu): texel offsets of each texture in the scene's texel pool
struct TexPlan {
  bool uv = false;               // per-vertex uvs uploaded
  std::vector<uint64_t> offset;  // first texel of each texture
  uint64_t texels = 0;           // texels in the pool
  uint64_t max_src = 0;          // texels of the largest texture
};
int tex_plan(const mgpu_scene_desc *desc, TexPlan &plan);
int tex_upload(const mgpu_scene_desc *desc, const TexPlan &plan, float4 *d_texrec, float4 *d_texels, cudaStream_t st);

}  // namespace mgpu

struct mgpu_accel {
  mgpu::KdTree tree;
  int64_t ntri = 0;
  // device-ready host staging, built once with the tree and uploaded by every mgpu_scene_create:
  // pairs with leaf slots pointing into ltris, leaf-ordered triangle records, triangles by id
  // and shading records.  Registered as page-locked memory on the first upload.
  std::vector<mgpu::Pair> dpairs;
  std::vector<mgpu::F4> ltris, tris;
  std::vector<float4> shade;
  bool registered = false;
  ~mgpu_accel();
};

struct mgpu_scene {
  int device = 0;
  mgpu::SceneView view{};       // device pointers
  float4 *d_shade = nullptr;    // 3 per triangle: (n0, mat), (n1, light), (n2, 0)
  float *d_mats = nullptr;
  float *d_lights = nullptr;
  float2 *d_uv = nullptr;       // 3 per triangle by id (nullptr: every uv is (0, 0))
  float4 *d_texrec = nullptr;   // 2 per texture: (texel offset, width, height, kind), (repeat u, v, bump intensity, 0)
  float4 *d_texels = nullptr;   // filtered colour texels / bump gradients
  int32_t bg_tex = 0;           // background: 1 + colour map index (environment), or 0
  float bg_le[3] = {0, 0, 0};   // constant background radiance when bg_tex == 0
  std::vector<uint64_t> tex_offset;
  std::vector<int32_t> tex_w, tex_h;
  int32_t nmat = 0, nlight = 0;
  uint32_t top_pairs = 0;       // pairs staged in shared memory by the traversal kernels
  uint32_t top_pairs_max = 0;   // breadth-first pairs available for staging
  void *d_block = nullptr;      // one allocation holding everything above
  uint64_t bytes = 0;
  uint32_t *d_err = nullptr;    // device error word
};

struct mgpu_film {
  int device = 0;
  int32_t width = 0, height = 0;
  float4 *d_sum = nullptr;  // rgb sum + sample count
  float4 *d_c = nullptr;    // Kahan compensation + sum of squared luminance
  // reconstruction filter (type kFilterNone = per-pixel mean): splatted sums w L (rgb) and w per
  // pixel in 2^-24 fixed point, so that the atomic additions are order-independent
  mgpu::FilmFilter filter{mgpu::kFilterNone, 0, 0.0f, 0.0f, 0.0f};
  unsigned long long *d_fx = nullptr;
};
