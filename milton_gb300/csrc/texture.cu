// texture.cu -- material image maps in device memory: validation, layout and the one-time
// per-texel filtering done when a scene is created.
//
// Milton looks a texture up at the integer texel floor(frac(u repeatU) width) and filters the
// image around that texel with the material's kernel filter (Material::getSample,
// Material.cpp:285-301; KernelFilter::apply, KernelFilter.cpp:106-140).  Because the lookup
// position is floored first, the filtered value depends on the texel only: it is computed
// here once per texel, and a hit reads one float4.  Bump maps keep the two luminance
// differences Material::_initShadingNormal takes at the texel (Material.cpp:179-225).
#include <string.h>

#include <cmath>
#include <vector>

#include "common.cuh"

namespace mgpu {

constexpr int kMaxTexFilterWidth = 63;  // (ceil(support) | 1) <= 63: at most 3,969 weights

// KernelFilter::_computeKernel (KernelFilter.cpp:143-156): weight (i, j) of the width^2 kernel
// is filter(i - width / 2, j - width / 2) -- offsets from -width/2, so the window is sampled
// half a texel off its centre, as in the reference.
static std::vector<float> tex_kernel(const mgpu_texture &t, double &sum) {
  const int kw = (int)((unsigned)ceilf(t.support) | 1u);
  FilmFilter f{t.filter, kw >> 1, t.support, t.p1, t.p2};
  std::vector<float> w((size_t)kw * kw);
  sum = 0.0;
  const float h = (float)kw / 2.0f;
  for (int i = 0; i < kw; ++i)
    for (int j = 0; j < kw; ++j) {
      w[(size_t)i * kw + j] = filter_eval(f, (float)i - h, (float)j - h);
      sum += w[(size_t)i * kw + j];
    }
  return w;
}

int tex_plan(const mgpu_scene_desc *d, TexPlan &p) {
  p = TexPlan();
  if (d->ntex < 0 || (d->ntex > 0 && !d->textures)) return fail(MGPU_E_INVALID, "mgpu_scene_create: bad textures");
  p.uv = d->tri_uv != nullptr && d->ntri > 0;
  p.offset.resize((size_t)d->ntex);
  for (int i = 0; i < d->ntex; ++i) {
    const mgpu_texture &t = d->textures[i];
    const std::string at = " (texture " + std::to_string(i) + ")";
    if (t.width <= 0 || t.height <= 0 || !t.rgb || (int64_t)t.width * t.height > ((int64_t)1 << 31))
      return fail(MGPU_E_INVALID, "mgpu_scene_create: bad texture size or data" + at);
    if (t.kind != MGPU_TEX_COLOR && t.kind != MGPU_TEX_BUMP)
      return fail(MGPU_E_INVALID, "mgpu_scene_create: unknown texture kind" + at);
    if (!(std::isfinite(t.repeat_u) && std::isfinite(t.repeat_v) && std::isfinite(t.bump_intensity)))
      return fail(MGPU_E_INVALID, "mgpu_scene_create: non-finite texture repeat or intensity" + at);
    if (t.kind == MGPU_TEX_COLOR) {
      if (t.filter < MGPU_FILTER_BOX || t.filter > MGPU_FILTER_LANCZOS_SINC)
        return fail(MGPU_E_INVALID, "mgpu_scene_create: unknown texture filter" + at);
      if (!(t.support > 0.0f) || ceilf(t.support) > (float)kMaxTexFilterWidth)
        return fail(MGPU_E_INVALID, "mgpu_scene_create: texture filter support outside (0, 63]" + at);
      double sum = 0.0;
      tex_kernel(t, sum);
      // the reference divides by this sum; with no weight at all every texel would be 0 / 0
      if (sum == 0.0 || !std::isfinite(sum))
        return fail(MGPU_E_INVALID, "mgpu_scene_create: texture filter has zero total weight" + at);
    }
    p.offset[i] = p.texels;
    p.texels += (uint64_t)t.width * t.height;
    p.max_src = std::max<uint64_t>(p.max_src, (uint64_t)t.width * t.height);
  }
  if (p.texels >= ((uint64_t)1 << 32)) return fail(MGPU_E_INVALID, "mgpu_scene_create: more than 2^32 texels");
  // texture slots of the materials, and no bump map on an emitter (its light samples would
  // need the bumped normal at the light point)
  std::vector<char> bumped((size_t)std::max(d->nmat, 0), 0);
  for (int m = 0; m < d->nmat; ++m) {
    const float *r = d->materials + 16 * (size_t)m;
    for (int k = 10; k < 14; ++k) {
      const float s = r[k];
      if (!(s >= 0.0f && s <= (float)d->ntex && s == floorf(s)))
        return fail(MGPU_E_INVALID, "mgpu_scene_create: bad texture slot at material " + std::to_string(m));
      if (s == 0.0f) continue;
      const int kind = d->textures[(int)s - 1].kind;
      if ((k == 13) != (kind == MGPU_TEX_BUMP))
        return fail(MGPU_E_INVALID, "mgpu_scene_create: material " + std::to_string(m) +
                                        (k == 13 ? " uses a colour map as bump map" : " uses a bump map as colour map"));
    }
    bumped[m] = r[13] != 0.0f;
  }
  if (d->background_tex < 0 || d->background_tex > d->ntex)
    return fail(MGPU_E_INVALID, "mgpu_scene_create: background texture out of range");
  if (d->background_tex > 0 && d->textures[d->background_tex - 1].kind != MGPU_TEX_COLOR)
    return fail(MGPU_E_INVALID, "mgpu_scene_create: the background must be a colour map");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(d->background_le[k]) || d->background_le[k] < 0.0f)
      return fail(MGPU_E_INVALID, "mgpu_scene_create: bad background radiance");
  if (d->tri_light)
    for (int64_t t = 0; t < d->ntri; ++t)
      if (d->tri_light[t] >= 0 && bumped[d->tri_mat[t]])
        return fail(MGPU_E_INVALID, "mgpu_scene_create: bump-mapped emitter at triangle " + std::to_string(t));
  return MGPU_OK;
}

// Colour texel (x, y): sum w(i, j) rgb[clamp(y + i - h), clamp(x + j - h)] / sum w.
__global__ void k_tex_filter(const float *__restrict__ src, int W, int H, const float *__restrict__ w, int kw,
                             float wsum, float4 *__restrict__ dst) {
  const int64_t n = (int64_t)W * H;
  const int h = kw >> 1;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(k / W), x = (int)(k - (int64_t)y * W);
    float r = 0.0f, g = 0.0f, b = 0.0f;
    for (int i = 0; i < kw; ++i) {
      const int row = min(max(y + i - h, 0), H - 1);
      const float *line = src + (int64_t)row * W * 3;
      for (int j = 0; j < kw; ++j) {
        const int col = min(max(x + j - h, 0), W - 1);
        const float wt = __ldg(w + i * kw + j);
        r += __ldg(line + 3 * col) * wt;
        g += __ldg(line + 3 * col + 1) * wt;
        b += __ldg(line + 3 * col + 2) * wt;
      }
    }
    dst[k] = make_float4(r / wsum, g / wsum, b / wsum, 0.0f);
  }
}

__device__ __forceinline__ float tex_lum(const float *src, int W, int row, int col) {
  const float *p = src + ((int64_t)row * W + col) * 3;
  return 0.2126f * __ldg(p) + 0.7152f * __ldg(p + 1) + 0.0722f * __ldg(p + 2);  // Rgba32::luminance
}

// Bump texel (x, y): the luminance differences of Material::_initShadingNormal.
__global__ void k_tex_bump(const float *__restrict__ src, int W, int H, float4 *__restrict__ dst) {
  const int64_t n = (int64_t)W * H;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(k / W), x = (int)(k - (int64_t)y * W);
    const float gx = tex_lum(src, W, y, x - (x > 0)) - tex_lum(src, W, y, x + (x < W - 1));
    const float gy = tex_lum(src, W, y - (y > 0), x) - tex_lum(src, W, y + (y < H - 1), x);
    dst[k] = make_float4(gx, gy, 0.0f, 0.0f);
  }
}

int tex_upload(const mgpu_scene_desc *d, const TexPlan &p, float4 *d_texrec, float4 *d_texels, cudaStream_t st) {
  if (d->ntex == 0) return MGPU_OK;
  std::vector<float4> rec((size_t)d->ntex * 2);
  for (int i = 0; i < d->ntex; ++i) {
    const mgpu_texture &t = d->textures[i];
    rec[2 * i] = make_float4(bits_f((uint32_t)p.offset[i]), bits_f((uint32_t)t.width), bits_f((uint32_t)t.height),
                             bits_f((uint32_t)t.kind));
    rec[2 * i + 1] = make_float4(t.repeat_u, t.repeat_v, t.bump_intensity, 0.0f);
  }
  MGPU_CUDA(cudaMemcpyAsync(d_texrec, rec.data(), rec.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
  // one scratch buffer for the largest source image and the largest kernel, reused per texture
  float *scratch = nullptr;
  const size_t src_bytes = p.max_src * 3 * sizeof(float);
  const size_t w_off = (src_bytes + 255) / 256 * 256;
  const size_t w_bytes = (size_t)kMaxTexFilterWidth * kMaxTexFilterWidth * sizeof(float);
  MGPU_CUDA(cudaMalloc(&scratch, w_off + w_bytes));
  float *d_w = (float *)((char *)scratch + w_off);
  int rc = MGPU_OK;
  const int grid = device_sm_count() * 8;
  for (int i = 0; i < d->ntex && rc == MGPU_OK; ++i) {
    const mgpu_texture &t = d->textures[i];
    const size_t n = (size_t)t.width * t.height;
    cudaError_t e = cudaMemcpyAsync(scratch, t.rgb, n * 3 * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && t.kind == MGPU_TEX_COLOR) {
      double sum = 0.0;
      std::vector<float> w = tex_kernel(t, sum);
      const int kw = (int)((unsigned)ceilf(t.support) | 1u);
      e = cudaMemcpyAsync(d_w, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) {
        k_tex_filter<<<grid, 256, 0, st>>>(scratch, t.width, t.height, d_w, kw, (float)sum, d_texels + p.offset[i]);
        e = cudaGetLastError();
      }
      // the host vector w and the source go out of scope: wait before the next texture
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    } else if (e == cudaSuccess) {
      k_tex_bump<<<grid, 256, 0, st>>>(scratch, t.width, t.height, d_texels + p.offset[i]);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) rc = cuda_fail(e, "mgpu_scene_create: texture upload");
    g_launches += 1;
  }
  cudaError_t e = cudaStreamSynchronize(st);
  if (rc == MGPU_OK && e != cudaSuccess) rc = cuda_fail(e, "mgpu_scene_create: texture upload");
  cudaFree(scratch);
  return rc;
}

}  // namespace mgpu
