// api.cu -- error reporting, host kd-tree objects, scene upload and film objects of libmgpu.
#include <string.h>

#include <cmath>
#include <mutex>
#include <new>
#include <vector>

#include "common.cuh"

namespace mgpu {

static thread_local std::string t_last_error;
std::atomic<uint64_t> g_launches{0};

void set_error(const std::string &msg) { t_last_error = msg; }
int fail(int code, const std::string &msg) {
  t_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char *what) {
  t_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? MGPU_E_NOMEM : MGPU_E_CUDA;
}

int device_sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Device-ready copies of the scene's triangles: tree layout with leaf-ordered records,
// triangles by id (3 x float4, v0.w = flags) and shading records (3 x float4: (n0, material),
// (n1, light), (n2, 0)).
static void stage_device_arrays(const mgpu_scene_desc *desc, mgpu_accel *a) {
  const int64_t T = desc->ntri;
  kd_device_layout(a->tree, desc->tri_v, desc->tri_flags, a->dpairs, a->ltris);
  a->tris.resize((size_t)T * 3);
  a->shade.resize((size_t)T * 3);
  for (int64_t t = 0; t < T; ++t) {
    const float *v = desc->tri_v + t * 9;
    uint32_t fl = desc->tri_flags ? desc->tri_flags[t] : 0u;
    for (int k = 0; k < 3; ++k) {
      F4 q; q.x = v[3 * k]; q.y = v[3 * k + 1]; q.z = v[3 * k + 2]; q.w = 0.0f;
      if (k == 0) memcpy(&q.w, &fl, 4);
      a->tris[3 * t + k] = q;
    }
    V3 e1 = v3(v[3] - v[0], v[4] - v[1], v[5] - v[2]);
    V3 e2 = v3(v[6] - v[0], v[7] - v[1], v[8] - v[2]);
    V3 fn = normalize(cross(e1, e2));
    int32_t mat = desc->tri_mat[t];
    int32_t li = desc->tri_light ? desc->tri_light[t] : -1;
    for (int k = 0; k < 3; ++k) {
      float4 q;
      if (desc->tri_n) {
        const float *n = desc->tri_n + t * 9 + 3 * k;
        q = make_float4(n[0], n[1], n[2], 0.0f);
      } else {
        q = make_float4(fn.x, fn.y, fn.z, 0.0f);
      }
      if (k == 0) memcpy(&q.w, &mat, 4);
      if (k == 1) memcpy(&q.w, &li, 4);
      a->shade[3 * t + k] = q;
    }
  }
}

static void register_staging(mgpu_accel *a) {
  // page-locked staging makes every later upload a direct DMA; failure just leaves it pageable
  if (a->registered) return;
  a->registered = true;
  auto reg = [](void *p, size_t n) {
    if (n) cudaHostRegister(p, n, cudaHostRegisterDefault);
  };
  reg(a->dpairs.data(), a->dpairs.size() * sizeof(Pair));
  reg(a->ltris.data(), a->ltris.size() * sizeof(F4));
  reg(a->tris.data(), a->tris.size() * sizeof(F4));
  reg(a->shade.data(), a->shade.size() * sizeof(float4));
  cudaGetLastError();  // clear a failed registration
}

// Offsets of the arrays in a scene's one device allocation (256-byte aligned each).
struct SceneLayout {
  size_t off_pairs, off_refs, off_tris, off_shade, off_mats, off_lights, off_uv, off_texrec, off_texels, off_sph,
      off_err, total;
};
// uv_tris: triangles with uploaded uvs (0 or all); ntex textures holding texels texels in all;
// nsph analytic spheres (2 float4 each, and 3 shading records after the triangles')
static SceneLayout scene_layout(const mgpu_accel *a, int32_t nmat, int32_t nlight, int64_t uv_tris = 0,
                                int32_t ntex = 0, uint64_t texels = 0, int32_t nsph = 0) {
  SceneLayout L;
  L.off_pairs = 0;
  L.off_refs = align_up(L.off_pairs + a->dpairs.size() * sizeof(Pair), 256);
  L.off_tris = align_up(L.off_refs + std::max<size_t>(a->ltris.size(), 1) * sizeof(F4), 256);
  L.off_shade = align_up(L.off_tris + std::max<size_t>(a->tris.size(), 1) * sizeof(F4), 256);
  L.off_mats = align_up(L.off_shade + std::max<size_t>(a->shade.size() + 3 * (size_t)std::max(nsph, 0), 1) *
                                          sizeof(float4), 256);
  L.off_lights = align_up(L.off_mats + (size_t)std::max(nmat, 0) * 16 * sizeof(float), 256);
  L.off_uv = align_up(L.off_lights + std::max<size_t>((size_t)std::max(nlight, 0), 1) * 32 * sizeof(float), 256);
  L.off_texrec = align_up(L.off_uv + (size_t)std::max<int64_t>(uv_tris, 0) * 3 * sizeof(float2), 256);
  L.off_texels = align_up(L.off_texrec + (size_t)std::max(ntex, 0) * 2 * sizeof(float4), 256);
  L.off_sph = align_up(L.off_texels + (size_t)texels * sizeof(float4), 256);
  L.off_err = align_up(L.off_sph + (size_t)std::max(nsph, 0) * 2 * sizeof(float4), 256);
  L.total = L.off_err + 256;
  return L;
}

// Film error estimate.  Per pixel with n > 1 samples: the sample variance of the per-sample
// luminance (r+g+b)/3 from the film's sum and sum of squares, divided by n, is the variance
// of the pixel's mean; the film's estimate is the square root of its average over those
// pixels (the expected RMSE of the image against the converged one).  Each film is reduced by
// kErrBlocks blocks in a fixed order, so the value is deterministic.
struct FilmRef {
  const float4 *sum;
  const float4 *c;
  int64_t npix;
};
constexpr int kErrBlocks = 64, kErrThreads = 256;

__global__ void __launch_bounds__(kErrThreads) k_film_error_partial(const FilmRef *films, double2 *partial) {
  const FilmRef f = films[blockIdx.y];
  double acc = 0.0, cnt = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kErrThreads + threadIdx.x; i < f.npix; i += (int64_t)kErrBlocks * kErrThreads) {
    const float4 S = f.sum[i], C = f.c[i];
    const double n = S.w;
    if (n > 1.0) {
      const double mean = ((((double)S.x - C.x) + ((double)S.y - C.y)) + ((double)S.z - C.z)) / (3.0 * n);
      const double var = fmax((double)C.w / n - mean * mean, 0.0) * n / (n - 1.0);
      acc += var / n;
      cnt += 1.0;
    }
  }
  __shared__ double sa[kErrThreads], sc[kErrThreads];
  sa[threadIdx.x] = acc;
  sc[threadIdx.x] = cnt;
  __syncthreads();
  for (int w = kErrThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sa[threadIdx.x] += sa[threadIdx.x + w];
      sc[threadIdx.x] += sc[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * kErrBlocks + blockIdx.x] = make_double2(sa[0], sc[0]);
}

__global__ void k_film_error_final(const double2 *partial, int32_t n, double *out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n) return;
  double a = 0.0, c = 0.0;
  for (int b = 0; b < kErrBlocks; ++b) {
    const double2 p = partial[(int64_t)f * kErrBlocks + b];
    a += p.x;
    c += p.y;
  }
  out[f] = c > 0.0 ? sqrt(a / c) : INFINITY;
}

// Reinhard tone map (ReinhardToneMap::map, M/renderers/tonemaps/ReinhardToneMap.cpp:25-94) of the
// film's per-pixel means, in FP64: key = exp(mean log(1e-7 + Y)), white = 1 / max(Y)^2 (the
// unscaled maximum, as the reference has it), Y' = L (1 + L white) / (1 + L) with L = 0.18 Y /
// key, chromaticity kept, gamma 2.22, clamp to [0, 255] and truncate (a NaN, as from an
// all-black pixel, becomes 0).  sRGB <-> XYZ matrices as ColorUtils.cpp:115-133 (the standard
// D65 pair).
__device__ const double kRgbToXyz[9] = {0.41245322014416, 0.35757958129350, 0.18042258997054,
                                        0.21267112134122, 0.71515920531078, 0.07216877677613,
                                        0.01933381646199, 0.11919354020663, 0.95022692228971};
__device__ const double kXyzToRgb[9] = {3.240479, -1.537150, -0.498535, -0.969256, 1.875992,
                                        0.041556, 0.055648, -0.204043, 1.057311};

struct ToneSrc {
  FilmRef f;
  const unsigned long long *fx;  // filtered sums, or null for the per-pixel mean
};

__device__ __forceinline__ void film_xyz(const ToneSrc &t, int64_t i, double &X, double &Y, double &Z) {
  double r = 0.0, g = 0.0, b = 0.0;
  if (t.fx) {
    const double w = (double)t.fx[4 * i + 3];
    if (w > 0.0) {
      r = (double)t.fx[4 * i] / w;
      g = (double)t.fx[4 * i + 1] / w;
      b = (double)t.fx[4 * i + 2] / w;
    }
  } else {
    const float4 S = t.f.sum[i], C = t.f.c[i];
    const double n = S.w;
    if (n > 0.0) {
      r = ((double)S.x - C.x) / n;
      g = ((double)S.y - C.y) / n;
      b = ((double)S.z - C.z) / n;
    }
  }
  X = kRgbToXyz[0] * r + kRgbToXyz[1] * g + kRgbToXyz[2] * b;
  Y = kRgbToXyz[3] * r + kRgbToXyz[4] * g + kRgbToXyz[5] * b;
  Z = kRgbToXyz[6] * r + kRgbToXyz[7] * g + kRgbToXyz[8] * b;
}

__global__ void __launch_bounds__(kErrThreads) k_tonemap_reduce(ToneSrc t, double2 *partial) {
  double lsum = 0.0, ymax = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kErrThreads + threadIdx.x; i < t.f.npix;
       i += (int64_t)kErrBlocks * kErrThreads) {
    double X, Y, Z;
    film_xyz(t, i, X, Y, Z);
    lsum += log(1e-7 + Y);
    ymax = fmax(ymax, Y);
  }
  __shared__ double sa[kErrThreads], sm[kErrThreads];
  sa[threadIdx.x] = lsum;
  sm[threadIdx.x] = ymax;
  __syncthreads();
  for (int w = kErrThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sa[threadIdx.x] += sa[threadIdx.x + w];
      sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = make_double2(sa[0], sm[0]);
}

__global__ void k_tonemap_map(ToneSrc t, const double2 *partial, uchar4 *out) {
  const FilmRef &f = t.f;
  __shared__ double s_scale, s_white;
  if (threadIdx.x == 0) {
    double a = 0.0, m = 0.0;
    for (int b = 0; b < kErrBlocks; ++b) {
      a += partial[b].x;
      m = fmax(m, partial[b].y);
    }
    const double key = exp(a / (double)f.npix);
    s_scale = key <= 0.0 ? 0.0 : 0.18 / key;
    s_white = m <= 0.0 ? 0.0 : 1.0 / (m * m);
  }
  __syncthreads();
  const double scale = s_scale, white = s_white, corr = 1.0 / 2.22;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < f.npix; i += (int64_t)gridDim.x * blockDim.x) {
    double X, Y, Z;
    film_xyz(t, i, X, Y, Z);
    const double s = X + Y + Z;
    const double cx = X / s, cy = Y / s;  // xyY chromaticity (NaN for a black pixel)
    const double lum = scale * Y;
    const double Yd = lum * (1.0 + lum * white) / (1.0 + lum);
    const double Xd = Yd * cx / cy, Zd = Yd * (1.0 - cx - cy) / cy;
    double rgb[3];
    for (int k = 0; k < 3; ++k)
      rgb[k] = 255.0 * pow(kXyzToRgb[3 * k] * Xd + kXyzToRgb[3 * k + 1] * Yd + kXyzToRgb[3 * k + 2] * Zd, corr);
    unsigned char o[3];
    for (int k = 0; k < 3; ++k) {
      const double v = rgb[k];
      o[k] = v >= 255.0 ? 255 : (v <= 0.0 ? 0 : (v == v ? (unsigned char)v : 0));
    }
    out[i] = make_uchar4(o[0], o[1], o[2], 255);
  }
}

// per-thread device scratch of the error estimate (grown as needed, per device)
struct ErrScratch {
  int device = -1;
  size_t bytes = 0;
  void *d = nullptr;
  ~ErrScratch() {
    if (d) cudaFree(d);
  }
};
static thread_local ErrScratch t_err;

}  // namespace mgpu

mgpu_accel::~mgpu_accel() {
  if (!registered) return;
  for (void *p : {(void *)dpairs.data(), (void *)ltris.data(), (void *)tris.data(), (void *)shade.data()})
    if (p) cudaHostUnregister(p);
  cudaGetLastError();
}

using namespace mgpu;

extern "C" {

const char *mgpu_last_error(void) { return t_last_error.c_str(); }
int mgpu_version(void) { return 1; }
uint64_t mgpu_launch_count(void) { return g_launches.load(); }

int mgpu_accel_build(const mgpu_scene_desc *desc, const mgpu_kd_params *params, mgpu_accel **out) {
  if (!desc || !out) return fail(MGPU_E_INVALID, "mgpu_accel_build: null argument");
  if (desc->ntri < 0 || (desc->ntri > 0 && !desc->tri_v)) return fail(MGPU_E_INVALID, "mgpu_accel_build: bad geometry");
  KdParams p;
  if (params) {
    p.min_prims = params->min_prims;
    p.max_depth = params->max_depth;
    p.cost_traversal = params->cost_traversal;
    p.empty_bias = params->empty_bias;
    p.threads = params->threads;
  }
  if (desc->ntri > 0 && !desc->tri_mat) return fail(MGPU_E_INVALID, "mgpu_accel_build: missing material indices");
  mgpu_accel *a = new (std::nothrow) mgpu_accel();
  if (!a) return fail(MGPU_E_NOMEM, "mgpu_accel_build: out of host memory");
  const char *err = nullptr;
  try {
    if (!kd_build(desc->tri_v, desc->ntri, p, a->tree, &err)) {
      delete a;
      return fail(MGPU_E_INVALID, std::string("mgpu_accel_build: ") + err);
    }
    a->ntri = desc->ntri;
    stage_device_arrays(desc, a);
  } catch (const std::bad_alloc &) {
    delete a;
    return fail(MGPU_E_NOMEM, "mgpu_accel_build: out of host memory");
  }
  *out = a;
  return MGPU_OK;
}

int mgpu_accel_stats(const mgpu_accel *a, mgpu_kd_stats *o) {
  if (!a || !o) return fail(MGPU_E_INVALID, "mgpu_accel_stats: null argument");
  const KdLog &l = a->tree.log;
  o->no_internal = l.no_internal;
  o->no_leaves = l.no_leaves;
  o->min_depth = l.min_depth;
  o->max_depth = l.max_depth;
  o->sum_depth = l.sum_depth;
  o->min_prims = l.min_prims;
  o->max_prims = l.max_prims;
  o->sum_prims = l.sum_prims;
  o->node_pairs = a->tree.pairs.size();
  o->refs = a->tree.refs.size();
  o->bytes_nodes = a->tree.pairs.size() * sizeof(Pair);
  o->bytes_refs = a->tree.refs.size() * sizeof(uint32_t);
  o->build_seconds = a->tree.build_seconds;
  return MGPU_OK;
}

int mgpu_accel_serialize(const mgpu_accel *a, int32_t *kind, float *split, int32_t *count, int32_t *prims,
                         int64_t *n_nodes, int64_t *n_prims) {
  if (!a) return fail(MGPU_E_INVALID, "mgpu_accel_serialize: null accel");
  kd_serialize(a->tree, kind, split, count, prims, n_nodes, n_prims);
  return MGPU_OK;
}

int mgpu_accel_destroy(mgpu_accel *a) {
  delete a;
  return MGPU_OK;
}

int mgpu_scene_create(const mgpu_scene_desc *desc, const mgpu_accel *accel, void *stream, mgpu_scene **out) {
  if (!desc || !accel || !out) return fail(MGPU_E_INVALID, "mgpu_scene_create: null argument");
  if (desc->ntri != accel->ntri) return fail(MGPU_E_INVALID, "mgpu_scene_create: accel built for another triangle count");
  if (desc->ntri > 0 && (!desc->tri_v || !desc->tri_mat)) return fail(MGPU_E_INVALID, "mgpu_scene_create: missing arrays");
  if (desc->nmat <= 0 || !desc->materials) return fail(MGPU_E_INVALID, "mgpu_scene_create: at least one material required");
  if (desc->nlight < 0 || (desc->nlight > 0 && !desc->lights)) return fail(MGPU_E_INVALID, "mgpu_scene_create: bad lights");
  const int64_t T = desc->ntri;
  for (int64_t t = 0; t < T; ++t) {
    if (desc->tri_mat[t] < 0 || desc->tri_mat[t] >= desc->nmat)
      return fail(MGPU_E_INVALID, "mgpu_scene_create: material index out of range at triangle " + std::to_string(t));
    if (desc->tri_light && (desc->tri_light[t] < -1 || desc->tri_light[t] >= desc->nlight))
      return fail(MGPU_E_INVALID, "mgpu_scene_create: light index out of range at triangle " + std::to_string(t));
  }
  for (int i = 0; i < desc->nmat; ++i) {
    float ty = desc->materials[16 * i];
    if (!(ty == 0.0f || ty == 1.0f || ty == 2.0f))
      return fail(MGPU_E_INVALID, "mgpu_scene_create: unknown material type at material " + std::to_string(i));
  }
  // device light records: the 16-float base record, then the 16-float extension
  std::vector<float> lrec((size_t)std::max(desc->nlight, 0) * 32, 0.0f);
  for (int i = 0; i < desc->nlight; ++i) {
    memcpy(&lrec[32 * (size_t)i], desc->lights + 16 * (size_t)i, 16 * sizeof(float));
    if (!desc->light_ext) continue;
    const float *x = desc->light_ext + 16 * (size_t)i;
    memcpy(&lrec[32 * (size_t)i + 16], x, 16 * sizeof(float));
    if (!(x[0] == 0.0f || x[0] == 1.0f || x[0] == 2.0f || x[0] == 3.0f || x[0] == 4.0f))
      return fail(MGPU_E_INVALID, "mgpu_scene_create: unknown light type at light " + std::to_string(i));
    if (x[0] == 2.0f) {
      uint32_t first, count;
      memcpy(&first, x + 8, 4);
      memcpy(&count, x + 9, 4);
      if (count == 0 || (uint64_t)first + count > (uint64_t)T)
        return fail(MGPU_E_INVALID, "mgpu_scene_create: mesh light " + std::to_string(i) + " has a bad triangle run");
    }
  }
  TexPlan tp;
  if (int rc = tex_plan(desc, tp)) return rc;
  // triangles cannot emit as a point light (it has no surface)
  if (desc->tri_light && desc->light_ext)
    for (int64_t t = 0; t < T; ++t)
      if (desc->tri_light[t] >= 0 && desc->light_ext[16 * (size_t)desc->tri_light[t]] == 3.0f)
        return fail(MGPU_E_INVALID, "mgpu_scene_create: triangle " + std::to_string(t) + " names a point light");
  // analytic spheres: records as the traversal reads them, shading records after the triangles'
  if (desc->nsphere < 0 || desc->nsphere > MGPU_MAX_SPHERES || (desc->nsphere > 0 && (!desc->spheres || !desc->sphere_mat)))
    return fail(MGPU_E_INVALID, "mgpu_scene_create: bad spheres (at most " + std::to_string(MGPU_MAX_SPHERES) + ")");
  std::vector<float4> sph((size_t)std::max(desc->nsphere, 0) * 2), sph_shade((size_t)std::max(desc->nsphere, 0) * 3);
  for (int i = 0; i < desc->nsphere; ++i) {
    const float *q = desc->spheres + 8 * (size_t)i;
    bool ok = q[3] > 0.0f;
    for (int k = 0; k < 8; ++k) ok = ok && std::isfinite(q[k]);
    if (!ok || desc->sphere_mat[i] < 0 || desc->sphere_mat[i] >= desc->nmat)
      return fail(MGPU_E_INVALID, "mgpu_scene_create: bad sphere " + std::to_string(i));
    sph[2 * i] = make_float4(q[0], q[1], q[2], q[3]);
    sph[2 * i + 1] = make_float4(q[4], q[5], q[6], q[7]);
    int32_t mat = desc->sphere_mat[i], li = desc->sphere_light ? desc->sphere_light[i] : -1;
    if (li < -1 || li >= desc->nlight)
      return fail(MGPU_E_INVALID, "mgpu_scene_create: light index out of range at sphere " + std::to_string(i));
    float4 a = make_float4(0, 0, 0, 0), b = a;
    memcpy(&a.w, &mat, 4);
    memcpy(&b.w, &li, 4);
    sph_shade[3 * i] = a;
    sph_shade[3 * i + 1] = b;
    sph_shade[3 * i + 2] = make_float4(0, 0, 0, 0);
  }
  const KdTree &tr = accel->tree;
  mgpu_accel *acc = const_cast<mgpu_accel *>(accel);
  register_staging(acc);
  const std::vector<Pair> &dpairs = accel->dpairs;
  const std::vector<F4> &ltris = accel->ltris, &tris = accel->tris;
  const std::vector<float4> &shade = accel->shade;
  const SceneLayout L = scene_layout(accel, desc->nmat, desc->nlight, tp.uv ? T : 0, desc->ntex, tp.texels,
                                     desc->nsphere);
  const size_t off_pairs = L.off_pairs, off_refs = L.off_refs, off_tris = L.off_tris, off_shade = L.off_shade,
               off_mats = L.off_mats, off_lights = L.off_lights, off_err = L.off_err, total = L.total;
  const size_t sz_pairs = dpairs.size() * sizeof(Pair), sz_mats = (size_t)desc->nmat * 16 * sizeof(float);

  mgpu_scene *s = new (std::nothrow) mgpu_scene();
  if (!s) return fail(MGPU_E_NOMEM, "mgpu_scene_create: out of host memory");
  cudaGetDevice(&s->device);
  cudaError_t e = cudaMalloc(&s->d_block, total);
  if (e != cudaSuccess) {
    delete s;
    return cuda_fail(e, "mgpu_scene_create: cudaMalloc");
  }
  char *base = (char *)s->d_block;
  cudaStream_t st = as_stream(stream);
  auto up = [&](size_t off, const void *src, size_t n) -> cudaError_t {
    if (n == 0) return cudaSuccess;
    return cudaMemcpyAsync(base + off, src, n, cudaMemcpyHostToDevice, st);
  };
  e = up(off_pairs, dpairs.data(), sz_pairs);
  if (e == cudaSuccess) e = up(off_refs, ltris.data(), ltris.size() * sizeof(F4));
  if (e == cudaSuccess) e = up(off_tris, tris.data(), tris.size() * sizeof(F4));
  if (e == cudaSuccess) e = up(off_shade, shade.data(), shade.size() * sizeof(float4));
  if (e == cudaSuccess) e = up(off_mats, desc->materials, sz_mats);
  if (e == cudaSuccess && desc->nlight > 0) e = up(off_lights, lrec.data(), lrec.size() * sizeof(float));
  if (e == cudaSuccess && tp.uv) e = up(L.off_uv, desc->tri_uv, (size_t)T * 6 * sizeof(float));
  if (e == cudaSuccess && desc->nsphere > 0) {
    e = up(L.off_sph, sph.data(), sph.size() * sizeof(float4));
    if (e == cudaSuccess)
      e = up(off_shade + shade.size() * sizeof(float4), sph_shade.data(), sph_shade.size() * sizeof(float4));
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(base + off_err, 0, 256, st);
  // materials and lights are the caller's pageable arrays: wait for the copies
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaFree(s->d_block);
    delete s;
    return cuda_fail(e, "mgpu_scene_create: upload");
  }
  if (desc->ntex > 0) {
    if (int rc = tex_upload(desc, tp, (float4 *)(base + L.off_texrec), (float4 *)(base + L.off_texels), st)) {
      cudaFree(s->d_block);
      delete s;
      return rc;
    }
    s->d_texrec = (float4 *)(base + L.off_texrec);
    s->d_texels = (float4 *)(base + L.off_texels);
    s->tex_offset = tp.offset;
    for (int i = 0; i < desc->ntex; ++i) {
      s->tex_w.push_back(desc->textures[i].width);
      s->tex_h.push_back(desc->textures[i].height);
    }
  }
  if (tp.uv) s->d_uv = (float2 *)(base + L.off_uv);
  s->bg_tex = desc->background_tex;
  for (int k = 0; k < 3; ++k) s->bg_le[k] = desc->background_le[k];
  s->view.pairs = (const Pair *)(base + off_pairs);
  s->view.ltris = (const F4 *)(base + off_refs);
  s->view.tris = (const F4 *)(base + off_tris);
  for (int k = 0; k < 3; ++k) { s->view.bmin[k] = (float)tr.bmin[k]; s->view.bmax[k] = (float)tr.bmax[k]; }
  s->view.ntri = T;
  s->view.npairs = tr.pairs.size();
  s->view.nrefs = ltris.size() / 3;
  s->view.spheres = desc->nsphere > 0 ? (const F4 *)(base + L.off_sph) : nullptr;
  s->view.nsphere = desc->nsphere;
  s->d_shade = (float4 *)(base + off_shade);
  s->d_mats = (float *)(base + off_mats);
  s->d_lights = (float *)(base + off_lights);
  s->nmat = desc->nmat;
  s->nlight = desc->nlight;
  // staging the top of the tree in shared memory costs more occupancy than it saves on GB300
  // (the L1 keeps those pairs anyway); mgpu_scene_set_top_pairs turns it on
  s->top_pairs = 0;
  s->top_pairs_max = tr.top_pairs;
  s->d_err = (uint32_t *)(base + off_err);
  s->bytes = total;
  *out = s;
  return MGPU_OK;
}

int mgpu_scene_destroy(mgpu_scene *s) {
  if (!s) return MGPU_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != s->device) cudaSetDevice(s->device);
  cudaError_t e = cudaFree(s->d_block);
  if (cur != s->device) cudaSetDevice(cur);
  delete s;
  if (e != cudaSuccess) return cuda_fail(e, "mgpu_scene_destroy: cudaFree");
  return MGPU_OK;
}

int mgpu_scene_set_top_pairs(mgpu_scene *s, uint32_t n) {
  if (!s) return fail(MGPU_E_INVALID, "mgpu_scene_set_top_pairs: null scene");
  if (n > s->top_pairs_max) n = s->top_pairs_max;
  if ((size_t)n * 16 > 96 * 1024) return fail(MGPU_E_INVALID, "mgpu_scene_set_top_pairs: more than 96 KiB of shared memory");
  s->top_pairs = n;
  return MGPU_OK;
}

int mgpu_scene_bytes(const mgpu_scene *s, uint64_t *out) {
  if (!s || !out) return fail(MGPU_E_INVALID, "mgpu_scene_bytes: null argument");
  *out = s->bytes;
  return MGPU_OK;
}

int mgpu_accel_device_bytes(const mgpu_accel *a, int32_t nmat, int32_t nlight, uint64_t *out) {
  if (!a || !out || nmat < 0 || nlight < 0) return fail(MGPU_E_INVALID, "mgpu_accel_device_bytes: bad argument");
  *out = scene_layout(a, nmat, nlight).total;
  return MGPU_OK;
}

int mgpu_scene_device_bytes(const mgpu_scene_desc *desc, const mgpu_accel *a, uint64_t *out) {
  if (!desc || !a || !out || desc->nmat < 0 || desc->nlight < 0)
    return fail(MGPU_E_INVALID, "mgpu_scene_device_bytes: bad argument");
  TexPlan tp;
  if (int rc = tex_plan(desc, tp)) return rc;
  *out = scene_layout(a, desc->nmat, desc->nlight, tp.uv ? desc->ntri : 0, desc->ntex, tp.texels,
                      std::max(desc->nsphere, 0)).total;
  return MGPU_OK;
}

int mgpu_scene_read_texels(const mgpu_scene *s, int32_t tex, float *out, void *stream) {
  if (!s || !out || tex < 0 || tex >= (int32_t)s->tex_offset.size())
    return fail(MGPU_E_INVALID, "mgpu_scene_read_texels: bad argument");
  cudaStream_t st = as_stream(stream);
  const size_t n = (size_t)s->tex_w[tex] * s->tex_h[tex];
  MGPU_CUDA(cudaMemcpyAsync(out, s->d_texels + s->tex_offset[tex], n * sizeof(float4), cudaMemcpyDeviceToHost, st));
  MGPU_CUDA(cudaStreamSynchronize(st));
  return MGPU_OK;
}

int mgpu_film_create(int32_t width, int32_t height, void *stream, mgpu_film **out) {
  if (!out || width <= 0 || height <= 0 || (int64_t)width * height > (int64_t)1 << 31)
    return fail(MGPU_E_INVALID, "mgpu_film_create: bad size");
  mgpu_film *f = new (std::nothrow) mgpu_film();
  if (!f) return fail(MGPU_E_NOMEM, "mgpu_film_create: out of host memory");
  cudaGetDevice(&f->device);
  f->width = width;
  f->height = height;
  size_t n = (size_t)width * height;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, 2 * n * sizeof(float4));
  if (e != cudaSuccess) {
    delete f;
    return cuda_fail(e, "mgpu_film_create: cudaMalloc");
  }
  f->d_sum = (float4 *)p;
  f->d_c = f->d_sum + n;
  e = cudaMemsetAsync(p, 0, 2 * n * sizeof(float4), as_stream(stream));
  if (e != cudaSuccess) {
    cudaFree(p);
    delete f;
    return cuda_fail(e, "mgpu_film_create: clear");
  }
  *out = f;
  return MGPU_OK;
}

int mgpu_film_clear(mgpu_film *f, void *stream) {
  if (!f) return fail(MGPU_E_INVALID, "mgpu_film_clear: null film");
  MGPU_CUDA(cudaMemsetAsync(f->d_sum, 0, 2 * (size_t)f->width * f->height * sizeof(float4), as_stream(stream)));
  if (f->d_fx)
    MGPU_CUDA(cudaMemsetAsync(f->d_fx, 0, 4 * (size_t)f->width * f->height * sizeof(unsigned long long),
                              as_stream(stream)));
  return MGPU_OK;
}

int mgpu_film_set_filter(mgpu_film *f, int32_t type, float support, float p1, float p2, void *stream) {
  if (!f) return fail(MGPU_E_INVALID, "mgpu_film_set_filter: null film");
  if (type < kFilterNone || type > kFilterLanczos || (type != kFilterNone && !(support > 0.0f && support <= 64.0f)) ||
      (type == kFilterGaussian && !(p1 > 0.0f)) || (type == kFilterLanczos && !(p1 > 0.0f)))
    return fail(MGPU_E_INVALID, "mgpu_film_set_filter: bad filter type or parameters");
  if (f->d_fx) {
    cudaFree(f->d_fx);
    f->d_fx = nullptr;
  }
  f->filter = FilmFilter{type, type == kFilterNone ? 0 : (int)(((unsigned)ceilf(support) | 1u) >> 1), support, p1, p2};
  if (type == kFilterNone) return MGPU_OK;
  const size_t bytes = 4 * (size_t)f->width * f->height * sizeof(unsigned long long);
  MGPU_CUDA(cudaMalloc(&f->d_fx, bytes));
  MGPU_CUDA(cudaMemsetAsync(f->d_fx, 0, bytes, as_stream(stream)));
  return MGPU_OK;
}

int mgpu_film_destroy(mgpu_film *f) {
  if (!f) return MGPU_OK;
  cudaError_t e = cudaFree(f->d_sum);
  if (f->d_fx) cudaFree(f->d_fx);
  delete f;
  if (e != cudaSuccess) return cuda_fail(e, "mgpu_film_destroy: cudaFree");
  return MGPU_OK;
}

int mgpu_film_read_raw(mgpu_film *f, float *out8, void *stream) {
  if (!f || !out8) return fail(MGPU_E_INVALID, "mgpu_film_read_raw: null argument");
  size_t n = (size_t)f->width * f->height;
  cudaStream_t st = as_stream(stream);
  MGPU_CUDA(cudaMemcpyAsync(out8, f->d_sum, 2 * n * sizeof(float4), cudaMemcpyDeviceToHost, st));
  MGPU_CUDA(cudaStreamSynchronize(st));
  return MGPU_OK;
}

// mean = (sum - compensation) / count in FP64 (ProgressiveFilterValue::getValue,
// ProgressiveFilterValue.h:26-31; a pixel with no samples reads as black)
// Device scratch and page-locked host staging of the film reads of one host thread: grown to the
// largest read and kept for the next, released when the thread exits.  A film read is
// synchronous, so the thread's next read finds them free.
struct MeanScratch {
  void *p = nullptr, *h = nullptr;  // device buffer, page-locked host staging of the same size
  size_t bytes = 0;
  int device = -1;
  void release() {
    if (p) cudaFree(p);
    if (h) cudaFreeHost(h);
    p = h = nullptr;
    bytes = 0;
  }
  cudaError_t get(int dev, size_t need, void **out, void **host) {
    if (p && (dev != device || need > bytes)) release();
    if (!p) {
      cudaError_t e = cudaMalloc(&p, need);
      if (e == cudaSuccess) e = cudaMallocHost(&h, need);
      if (e != cudaSuccess) {
        release();
        return e;
      }
      bytes = need;
      device = dev;
    }
    *out = p;
    *host = h;
    return cudaSuccess;
  }
  ~MeanScratch() { release(); }
};
static thread_local MeanScratch t_mean_scratch;

// Per pixel mean of the compensated film: (sum - compensation) / count in FP64, 0 for a pixel
// without samples.
__global__ void __launch_bounds__(256) k_film_mean(const float4 *__restrict__ sum, const float4 *__restrict__ comp,
                                                   int64_t npix, double *__restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 s = sum[i], c = comp[i];
    const double cnt = s.w;
    double r = 0.0, g = 0.0, b = 0.0;
    if (cnt > 0) {
      r = ((double)s.x - (double)c.x) / cnt;
      g = ((double)s.y - (double)c.y) / cnt;
      b = ((double)s.z - (double)c.z) / cnt;
    }
    out[3 * i + 0] = r;
    out[3 * i + 1] = g;
    out[3 * i + 2] = b;
  }
}

int mgpu_film_read(mgpu_film *f, double *out_mean, void *stream) {
  if (!f || !out_mean) return fail(MGPU_E_INVALID, "mgpu_film_read: null argument");
  size_t n = (size_t)f->width * f->height;
  if (f->d_fx) {
    // reconstruction filter: per pixel sum(w L) / sum(w) (ProgressiveFilterValue, weights > 0)
    std::vector<unsigned long long> fx(4 * n);
    cudaStream_t st = as_stream(stream);
    MGPU_CUDA(cudaMemcpyAsync(fx.data(), f->d_fx, fx.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    MGPU_CUDA(cudaStreamSynchronize(st));
    for (size_t i = 0; i < n; ++i) {
      const double w = (double)fx[4 * i + 3];
      for (int k = 0; k < 3; ++k) out_mean[3 * i + k] = w > 0 ? (double)fx[4 * i + k] / w : 0.0;
    }
    return MGPU_OK;
  }
  // the FP64 means are taken on the device; only they cross to the host, through page-locked
  // staging, and are copied from there into the caller's array
  cudaStream_t st = as_stream(stream);
  const size_t bytes = 3 * n * sizeof(double);
  double *d_mean = nullptr, *h_mean = nullptr;
  MGPU_CUDA(t_mean_scratch.get(f->device, bytes, (void **)&d_mean, (void **)&h_mean));
  k_film_mean<<<device_sm_count() * 4, 256, 0, st>>>(f->d_sum, f->d_c, (int64_t)n, d_mean);
  g_launches.fetch_add(1);
  MGPU_CUDA(cudaGetLastError());
  MGPU_CUDA(cudaMemcpyAsync(h_mean, d_mean, bytes, cudaMemcpyDeviceToHost, st));
  MGPU_CUDA(cudaStreamSynchronize(st));
  memcpy(out_mean, h_mean, bytes);
  return MGPU_OK;
}

int mgpu_film_tonemap(mgpu_film *f, uint8_t *out_rgba, void *stream) {
  if (!f || !out_rgba) return fail(MGPU_E_INVALID, "mgpu_film_tonemap: null argument");
  const int64_t npix = (int64_t)f->width * f->height;
  ToneSrc ref{FilmRef{f->d_sum, f->d_c, npix}, f->d_fx};
  void *d = nullptr;
  const size_t b_part = align_up(kErrBlocks * sizeof(double2), 256);
  MGPU_CUDA(cudaMalloc(&d, b_part + (size_t)npix * sizeof(uchar4)));
  double2 *part = (double2 *)d;
  uchar4 *img = (uchar4 *)((char *)d + b_part);
  cudaStream_t st = as_stream(stream);
  k_tonemap_reduce<<<kErrBlocks, kErrThreads, 0, st>>>(ref, part);
  k_tonemap_map<<<device_sm_count() * 4, 256, 0, st>>>(ref, part, img);
  g_launches.fetch_add(2);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_rgba, img, (size_t)npix * sizeof(uchar4), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "mgpu_film_tonemap");
  return MGPU_OK;
}

int mgpu_film_error(mgpu_film *const *films, int32_t n, double *out_rmse, void *stream) {
  if (n < 0 || n > 65535 || (n > 0 && (!films || !out_rmse)))
    return fail(MGPU_E_INVALID, "mgpu_film_error: bad argument");
  if (n == 0) return MGPU_OK;
  std::vector<FilmRef> refs((size_t)n);
  for (int32_t i = 0; i < n; ++i) {
    if (!films[i]) return fail(MGPU_E_INVALID, "mgpu_film_error: null film");
    refs[i].sum = films[i]->d_sum;
    refs[i].c = films[i]->d_c;
    refs[i].npix = (int64_t)films[i]->width * films[i]->height;
  }
  const size_t b_refs = align_up((size_t)n * sizeof(FilmRef), 256);
  const size_t b_part = align_up((size_t)n * kErrBlocks * sizeof(double2), 256);
  const size_t need = b_refs + b_part + (size_t)n * sizeof(double);
  int dev = 0;
  MGPU_CUDA(cudaGetDevice(&dev));
  if (t_err.device != dev || t_err.bytes < need) {
    if (t_err.d) {
      int cur = dev;
      if (t_err.device != dev) cudaSetDevice(t_err.device);
      cudaFree(t_err.d);
      if (t_err.device != dev) cudaSetDevice(cur);
      t_err.d = nullptr;
    }
    t_err.bytes = 0;
    MGPU_CUDA(cudaMalloc(&t_err.d, need));
    t_err.device = dev;
    t_err.bytes = need;
  }
  char *base = (char *)t_err.d;
  FilmRef *d_refs = (FilmRef *)base;
  double2 *d_part = (double2 *)(base + b_refs);
  double *d_out = (double *)(base + b_refs + b_part);
  cudaStream_t st = as_stream(stream);
  MGPU_CUDA(cudaMemcpyAsync(d_refs, refs.data(), (size_t)n * sizeof(FilmRef), cudaMemcpyHostToDevice, st));
  k_film_error_partial<<<dim3(kErrBlocks, n), kErrThreads, 0, st>>>(d_refs, d_part);
  k_film_error_final<<<(n + 127) / 128, 128, 0, st>>>(d_part, n, d_out);
  g_launches.fetch_add(2);
  MGPU_CUDA(cudaGetLastError());
  MGPU_CUDA(cudaMemcpyAsync(out_rmse, d_out, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
  MGPU_CUDA(cudaStreamSynchronize(st));
  return MGPU_OK;
}

}  // extern "C"
