// render.cu -- wavefront path tracer: generate -> (extend -> shade -> shadow)* -> accumulate.
//
// One wave = a range of pixel slots (8x8 tiles, row-major tile order) x a range of sample
// passes.  Per path the state is split in two:
//   path_L[p]     float4  radiance accumulated so far (rgb) + path flags (w) -- path-indexed,
//                          updated by shade (emission) and shadow (direct light), read once by
//                          accumulate;
//   ray queue     3 x float4 per live path (origin + path index, direction, throughput + depth
//                          state), compacted every bounce by warp ballot + one atomicAdd per warp.
// Direct light (DirectIllumination::evaluate over all lights x noDirectSamples,
// DirectIllumination.cpp:46-138) is split in two: shade samples every light, evaluates the BSDF,
// writes each sample's contribution into the path's slot for that sample and queues one shadow
// ray per non-zero contribution; the shadow kernel is a plain any-hit query that zeroes the slot
// of an occluded sample.  The next kernel to see the path (shade at the next bounce, or
// accumulate) folds its slots into the radiance in slot order, so every sum runs in a fixed
// order and the image does not depend on queue order.
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace mgpu {

constexpr int kBlock = 128;
constexpr int kHardCap = 1024;          // vertex cap when max_depth = 0 (Milton has none)
constexpr int kCtrRay = 0;              // counters[kCtrRay + b]  live paths at bounce b
constexpr int kCtrNee = kHardCap + 8;   // counters[kCtrNee + b]  shadow rays at bounce b
constexpr int kCtrFetchExt = 2 * (kHardCap + 8);   // work counters of the persistent extend kernel
constexpr int kCtrFetchSh = 3 * (kHardCap + 8);    // ... and of the persistent shadow kernel
constexpr int kCtrTrunc = 4 * (kHardCap + 8);
constexpr int kNumCounters = kCtrTrunc + 8;
constexpr float kShadowMargin = 1e-4f;  // shadow rays stop this fraction short of the light

struct RenderArgs {
  SceneView view;
  uint32_t ntop;
  const float4 *shade;
  const float4 *mats;    // 4 per material
  const float4 *lights;  // 4 per light
  int32_t nlight;
  Camera cam;
  Rng rng;
  int32_t W, H, spp, side, s2;
  int32_t nds, nds_side;
  int32_t max_depth, rr_start, efficient;
  int32_t tiles_x;
  int64_t slot0, nslots;
  int32_t s0, ns;        // samples [s0, s0 + ns) of this wave
  int32_t sample_begin, sample_count;
  float4 *path_L;
  float4 *qo[2], *qd[2], *qt[2];
  float4 *qhit;
  float4 *so, *sd;       // shadow ray queue: origin + slot index, direction + tmax
  float4 *qo_u, *qd_u, *qt_u;  // unsorted next-ray queue (binning on)
  float4 *so_u, *sd_u;         // unsorted shadow queue (binning on)
  uint32_t *qkey, *skey;       // bin keys of the unsorted queues
  int32_t bin_ext, bin_sh;     // counting-sort the queues by (direction octant | light, origin cell)
  int32_t sh_cell_bits;        // Morton bits of the origin cell in the shadow key
  float4 *slots;         // nl_slots per path: direct-light contribution per light sample
  int32_t nl_slots;      // nlight * nds_side^2
  uint32_t *counters;
  unsigned long long *stats;  // [0] extension rays, [1] shadow rays, [2] truncated paths, [3] bounces
  unsigned long long *tcount; // counted mode: ext nodes, refs, tris, rays; shadow nodes, refs, tris, rays
  int32_t max_b;
  float4 *film_sum, *film_c;
  float4 *path_out;      // optional
};

__device__ __forceinline__ bool slot_pixel(const RenderArgs &a, int64_t slot, int &x, int &y) {
  int64_t tile = slot >> 6;
  int within = (int)(slot & 63);
  x = (int)(tile % a.tiles_x) * 8 + (within & 7);
  y = (int)(tile / a.tiles_x) * 8 + (within >> 3);
  return x < a.W && y < a.H;
}

// global path id (pixel * spp + sample) for wave-local path p
__device__ __forceinline__ uint64_t path_id(const RenderArgs &a, int64_t p, int &x, int &y, int &s) {
  int64_t slot = a.slot0 + p / a.ns;
  s = a.s0 + (int)(p % a.ns);
  slot_pixel(a, slot, x, y);
  return ((uint64_t)y * a.W + x) * (uint64_t)a.spp + (uint64_t)s;
}

// warp-aggregated queue append: returns the slot for this lane (valid only if want)
__device__ __forceinline__ uint32_t warp_append(uint32_t *counter, bool want) {
  unsigned active = __activemask();
  unsigned mask = __ballot_sync(active, want);
  if (mask == 0) return 0;
  int lane = threadIdx.x & 31;
  int leader = __ffs(mask) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
  base = __shfl_sync(active, base, leader);
  return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ Material load_mat(const RenderArgs &a, int i) {
  float m[16];
  float4 *mm = reinterpret_cast<float4 *>(m);
#pragma unroll
  for (int k = 0; k < 4; ++k) mm[k] = __ldg(a.mats + 4 * i + k);
  return material_from(m);
}

__device__ __forceinline__ Light load_light(const RenderArgs &a, int i) {
  float l[16];
  float4 *ll = reinterpret_cast<float4 *>(l);
#pragma unroll
  for (int k = 0; k < 4; ++k) ll[k] = __ldg(a.lights + 4 * i + k);
  return light_from(l);
}

__device__ __forceinline__ void load_top(const RenderArgs &a) {
  extern __shared__ uint4 smem_top[];
  for (uint32_t i = threadIdx.x; i < a.ntop; i += blockDim.x)
    smem_top[i] = __ldg(reinterpret_cast<const uint4 *>(a.view.pairs) + i);
  __syncthreads();
}

__device__ __forceinline__ const Pair *top_ptr(const RenderArgs &a) {
  extern __shared__ uint4 smem_top[];
  return a.ntop ? reinterpret_cast<const Pair *>(smem_top) : nullptr;
}

// Binning keys (kBins = 4096).  Ray coherence: rays of one warp should start close together
// and head the same way, so that they visit the same nodes.  Keys combine the direction
// octant (extension rays) or the light index (shadow rays) with the Morton code of the
// origin's cell in a 16x16x16 grid over the scene bounds.
constexpr int kBins = 4096;

__device__ __forceinline__ uint32_t spread4(uint32_t v) {  // 4 bits -> every third bit
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

__device__ __forceinline__ uint32_t morton12(const RenderArgs &a, V3 p) {
  const float *lo = a.view.bmin, *hi = a.view.bmax;
  uint32_t c[3];
  const float pp[3] = {p.x, p.y, p.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float ext = hi[k] - lo[k];
    float f = ext > 0.0f ? (pp[k] - lo[k]) / ext : 0.0f;
    int q = (int)(f * 16.0f);
    c[k] = (uint32_t)min(max(q, 0), 15);
  }
  return (spread4(c[0]) << 2) | (spread4(c[1]) << 1) | spread4(c[2]);
}

__device__ __forceinline__ uint32_t ext_key(const RenderArgs &a, V3 o, V3 d) {
  uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
  return (oct << 9) | (morton12(a, o) >> 3);
}

__device__ __forceinline__ uint32_t sh_key(const RenderArgs &a, int light, V3 o) {
  uint32_t cell = morton12(a, o) >> (12 - a.sh_cell_bits);
  return (((uint32_t)light << a.sh_cell_bits) | cell) & (kBins - 1);
}

// ---------------------------------------------------------------------------------------
// generate: camera rays for every path of the wave (RayTracer::sample, RayTracer.cpp:19-30;
// SuperSampleGenerator strata, SuperSampleGenerator.cpp:60-90)
__global__ void __launch_bounds__(kBlock) k_generate(RenderArgs a) {
  const int64_t n = a.nslots * a.ns;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    int64_t p = base + threadIdx.x;
    bool valid = p < n;
    bool live = false;
    float4 o4 = make_float4(0, 0, 0, 0), d4 = o4;
    if (valid) {
      int x, y, s;
      uint64_t pid = path_id(a, p, x, y, s);
      live = x < a.W && y < a.H;
      uint32_t flags = 0;
      if (live) {
        uint64_t pix = (uint64_t)y * a.W + x;
        int k = s % a.s2;
        F4u j = uniforms(a.rng, pix * (uint64_t)a.s2 + (uint64_t)k, kDepthJitter, 0);
        float px = ((float)x + ((float)(k % a.side) + j.a) / (float)a.side) / (float)a.W;
        float py = ((float)y + ((float)(k / a.side) + j.b) / (float)a.side) / (float)a.H;
        F4u ui = uniforms(a.rng, pid, kDepthPathInit, 0);
        uint32_t ior = min((uint32_t)(ui.a * 3.0f), 2u);
        flags = ior;
        V3 d = camera_dir(a.cam, px, py);
        o4 = make_float4(a.cam.eye.x, a.cam.eye.y, a.cam.eye.z, __int_as_float((int)p));
        d4 = make_float4(d.x, d.y, d.z, 0.0f);
      }
      a.path_L[p] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(flags));
    }
    uint32_t q = warp_append(&a.counters[kCtrRay + 0], live);
    if (live) {
      a.qo[0][q] = o4;
      a.qd[0][q] = d4;
      a.qt[0][q] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
    }
  }
}

// extend: closest hit for the live queue of bounce b
template <bool COUNT, bool PERSIST>
__global__ void __launch_bounds__(kBlock) k_extend(RenderArgs a, int b) {
  load_top(a);
  const Pair *top = top_ptr(a);
  const uint32_t n = a.counters[kCtrRay + b];
  const float4 *qo = a.qo[b & 1], *qd = a.qd[b & 1];
  float4 *qhit = a.qhit;
  TraceCounts c = {0, 0, 0, 0};
  uint32_t rays = 0;
  auto load = [&](uint32_t i, Ray &r) {
    float4 o = qo[i], d = qd[i];
    r.o = v3(o.x, o.y, o.z);
    r.tmin = 0.0f;
    r.d = v3(d.x, d.y, d.z);
    r.tmax = INFINITY;
  };
  auto store = [&](uint32_t i, bool hit, const TravState &st) {
    qhit[i] = make_float4(hit ? st.best : INFINITY, __int_as_float(hit ? st.best_prim : -1), hit ? st.bb1 : 0.0f,
                          hit ? st.bb2 : 0.0f);
  };
  if (PERSIST)
    persistent_trace<false, COUNT>(a.view, top, a.ntop, n, &a.counters[kCtrFetchExt + b], load, store, &c, rays);
  else
    grid_trace<false, COUNT>(a.view, top, a.ntop, n, load, store, &c, rays);
  if (COUNT && rays) {
    atomicAdd(&a.tcount[0], (unsigned long long)c.nodes);
    atomicAdd(&a.tcount[1], (unsigned long long)c.refs);
    atomicAdd(&a.tcount[2], (unsigned long long)c.tris);
    atomicAdd(&a.tcount[3], (unsigned long long)rays);
  }
}

// shade: pending direct light, emission, light sampling, BSDF sample and Russian roulette
// (PathTracer.cpp:36-115, DirectIllumination.cpp:46-138)
__device__ __forceinline__ V3 fold_slots(const RenderArgs &a, int64_t p, V3 L) {
  const float4 *sl = a.slots + p * a.nl_slots;
  for (int k = 0; k < a.nl_slots; ++k) {
    float4 c = sl[k];
    L = L + v3(c.x, c.y, c.z);
  }
  return L;
}

__global__ void __launch_bounds__(kBlock) k_shade(RenderArgs a, int b) {
  const uint32_t n = a.counters[kCtrRay + b];
  const int cur = b & 1, nxt = (b + 1) & 1;
  const uint32_t stride = gridDim.x * blockDim.x;
  const int s2n = a.nds_side * a.nds_side;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    uint32_t i = base + threadIdx.x;
    bool valid = i < n;
    bool want_next = false, do_nee = false;
    float4 no_o, no_d, no_t;
    int64_t p = 0;
    uint64_t pid = 0;
    int depth = 0, self = -1;
    V3 P = v3(0, 0, 0), ns = P, ng = P, d = P, thr = P;
    Material m;
    m.type = 0;
    if (valid) {
      float4 o4 = a.qo[cur][i], d4 = a.qd[cur][i], t4 = a.qt[cur][i], h4 = a.qhit[i];
      p = (int64_t)__float_as_int(o4.w);
      uint32_t state = __float_as_uint(t4.w);
      depth = (int)(state & 0xFFFFu);
      bool ec = (state >> 16) & 1u;
      thr = v3(t4.x, t4.y, t4.z);
      d = v3(d4.x, d4.y, d4.z);
      int prim = __float_as_int(h4.y);
      float4 L4 = a.path_L[p];
      uint32_t flags = __float_as_uint(L4.w);
      V3 L = v3(L4.x, L4.y, L4.z);
      if (flags & kFlagNeePending) {
        L = fold_slots(a, p, L);
        flags &= ~kFlagNeePending;
      }
      if (prim >= 0) {
        int x, y, s;
        pid = path_id(a, p, x, y, s);
        float t = h4.x, b1 = h4.z, b2 = h4.w, b0 = 1.0f - b1 - b2;
        float4 va = __ldg(reinterpret_cast<const float4 *>(a.view.tris) + 3 * (int64_t)prim);
        float4 vb = __ldg(reinterpret_cast<const float4 *>(a.view.tris) + 3 * (int64_t)prim + 1);
        float4 vc = __ldg(reinterpret_cast<const float4 *>(a.view.tris) + 3 * (int64_t)prim + 2);
        float4 s0 = __ldg(a.shade + 3 * (int64_t)prim), s1 = __ldg(a.shade + 3 * (int64_t)prim + 1),
               s2 = __ldg(a.shade + 3 * (int64_t)prim + 2);
        V3 v0 = v3(va.x, va.y, va.z), v1 = v3(vb.x, vb.y, vb.z), v2 = v3(vc.x, vc.y, vc.z);
        P = v0 * b0 + v1 * b1 + v2 * b2;
        ns = normalize(v3(s0.x, s0.y, s0.z) * b0 + v3(s1.x, s1.y, s1.z) * b1 + v3(s2.x, s2.y, s2.z) * b2);
        ng = normalize(cross(v1 - v0, v2 - v0));
        int mi = __float_as_int(s0.w);
        self = __float_as_int(s1.w);
        m = load_mat(a, mi);
        bool spec = is_specular(m);
        if (spec) flags |= kFlagSpecular;
        if (self >= 0) {
          Light lt = load_light(a, self);
          V3 Le = emitted(lt.Le, ns, -d);
          if (!a.efficient || depth == 0) L = L + mul(thr, Le);
          else if (ec) L = L + mul(thr, Le) * (lt.area / (t * t));
        }
        if (a.efficient && !spec && a.nlight > 0) {
          do_nee = true;
          flags |= kFlagNeePending;
        }
        F4u u = uniforms(a.rng, pid, (uint32_t)depth, 0);
        V3 wo, fs;
        int ev = bsdf_sample(m, ns, d, flags & kFlagIorMask, u.a, u.b, u.c, wo, fs);
        if (ev > 0) {
          float pc = depth < a.rr_start ? (nonzero(fs) ? 1.0f : 0.0f) : fminf(0.95f, maxc(fs));
          bool capped = (a.max_depth > 0 && depth + 1 >= a.max_depth);
          if (!capped && u.d < pc) {
            if (depth + 1 >= kHardCap) {
              flags |= kFlagTruncated;
              atomicAdd(&a.counters[kCtrTrunc], 1u);
            } else {
              want_next = true;
              if (depth == 0) flags |= kFlagContinued0;
              V3 nthr = mul(thr, fs) * (1.0f / pc);
              bool nec = spec && dot(ns, wo) > kEps;
              V3 org = offset_origin(P, dot(ng, wo) > 0.0f ? ng : -ng);
              no_o = make_float4(org.x, org.y, org.z, o4.w);
              no_d = make_float4(wo.x, wo.y, wo.z, 0.0f);
              no_t = make_float4(nthr.x, nthr.y, nthr.z, __uint_as_float((uint32_t)(depth + 1) | (nec ? 0x10000u : 0u)));
            }
          }
        }
      }
      a.path_L[p] = make_float4(L.x, L.y, L.z, __uint_as_float(flags));
    }
    uint32_t q = warp_append(&a.counters[kCtrRay + b + 1], want_next);
    if (want_next) {
      if (a.bin_ext) {
        a.qo_u[q] = no_o;
        a.qd_u[q] = no_d;
        a.qt_u[q] = no_t;
        a.qkey[q] = ext_key(a, v3(no_o.x, no_o.y, no_o.z), v3(no_d.x, no_d.y, no_d.z));
      } else {
        a.qo[nxt][q] = no_o;
        a.qd[nxt][q] = no_d;
        a.qt[nxt][q] = no_t;
      }
    }
    // light samples: every lane of the warp runs the same k loop (uniform trip count), so the
    // warp-aggregated append stays converged
    const float inv_nds = 1.0f / (float)a.nds;
    for (int k = 0; k < a.nl_slots; ++k) {
      bool want = false;
      float4 so4, sd4;
      if (do_nee) {
        int li = k / s2n, within = k - li * s2n;
        int sy = within / a.nds_side, sx = within - sy * a.nds_side;
        V3 c = v3(0.0f, 0.0f, 0.0f);
        if (li != self) {
          Light lt = load_light(a, li);
          F4u u = uniforms(a.rng, pid, (uint32_t)depth, 1u + (uint32_t)(k >> 1));
          float ux = ((float)sx + ((k & 1) ? u.c : u.a)) / (float)a.nds_side;
          float uy = ((float)sy + ((k & 1) ? u.d : u.b)) / (float)a.nds_side;
          V3 lp = lt.center + lt.ex * (ux - 0.5f) + lt.ez * (uy - 0.5f);
          V3 wo = lp - P;
          float t = length(wo);
          wo = wo * (1.0f / t);
          float cwo = fabsf(dot(ns, wo)), cwi = fabsf(dot(lt.normal, wo));
          V3 fr = bsdf_eval(m, ns, d, wo);
          if (cwo > 0.0f && cwi > 0.0f && nonzero(fr)) {
            V3 Le = emitted(lt.Le, lt.normal, -wo);
            c = mul(thr, mul(fr, Le)) * (cwo * cwi / (t * t) * lt.area * inv_nds);
            if (nonzero(c)) {
              want = true;
              V3 org = offset_origin(P, dot(ng, wo) > 0.0f ? ng : -ng);
              so4 = make_float4(org.x, org.y, org.z, __uint_as_float((uint32_t)(p * a.nl_slots + k)));
              sd4 = make_float4(wo.x, wo.y, wo.z, t * (1.0f - kShadowMargin));
            }
          }
        }
        a.slots[p * a.nl_slots + k] = make_float4(c.x, c.y, c.z, 0.0f);
      }
      uint32_t e = warp_append(&a.counters[kCtrNee + b], want);
      if (want) {
        if (a.bin_sh) {
          a.so_u[e] = so4;
          a.sd_u[e] = sd4;
          a.skey[e] = sh_key(a, k / s2n, P);
        } else {
          a.so[e] = so4;
          a.sd[e] = sd4;
        }
      }
    }
  }
}

// shadow: any-hit query per queued light sample; an occluded sample's slot is zeroed
template <bool COUNT, bool PERSIST>
__global__ void __launch_bounds__(kBlock) k_shadow(RenderArgs a, int b) {
  load_top(a);
  const Pair *top = top_ptr(a);
  const uint32_t n = a.counters[kCtrNee + b];
  const float4 *so = a.so, *sd = a.sd;
  float4 *slots = a.slots;
  TraceCounts c = {0, 0, 0, 0};
  uint32_t rays = 0;
  auto load = [&](uint32_t i, Ray &r) {
    float4 o = so[i], d = sd[i];
    r.o = v3(o.x, o.y, o.z);
    r.tmin = 0.0f;
    r.d = v3(d.x, d.y, d.z);
    r.tmax = d.w;
  };
  auto store = [&](uint32_t i, bool hit, const TravState &) {
    if (hit) slots[__float_as_uint(so[i].w)] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  };
  if (PERSIST)
    persistent_trace<true, COUNT>(a.view, top, a.ntop, n, &a.counters[kCtrFetchSh + b], load, store, &c, rays);
  else
    grid_trace<true, COUNT>(a.view, top, a.ntop, n, load, store, &c, rays);
  if (COUNT && rays) {
    atomicAdd(&a.tcount[4], (unsigned long long)c.nodes);
    atomicAdd(&a.tcount[5], (unsigned long long)c.refs);
    atomicAdd(&a.tcount[6], (unsigned long long)c.tris);
    atomicAdd(&a.tcount[7], (unsigned long long)rays);
  }
}

// ---------------------------------------------------------------------------------------
// counting sort of a queue by key: histogram -> exclusive scan -> scatter with per-block
// range reservations (one global atomic per block chunk and non-empty bin)
__global__ void __launch_bounds__(256) k_bin_hist(const uint32_t *__restrict__ keys, const uint32_t *count,
                                                 uint32_t *__restrict__ hist) {
  __shared__ uint32_t h[kBins];
  for (int i = threadIdx.x; i < kBins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const uint32_t n = *count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&h[keys[i] & (kBins - 1)], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < kBins; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

// single block of 1024 threads: hist -> cursor (exclusive prefix sum)
__global__ void __launch_bounds__(1024) k_bin_scan(const uint32_t *__restrict__ hist, uint32_t *__restrict__ cursor) {
  __shared__ uint32_t part[1024];
  const int per = kBins / 1024;
  uint32_t loc[kBins / 1024];
  uint32_t sum = 0;
  for (int k = 0; k < per; ++k) {
    loc[k] = sum;
    sum += hist[threadIdx.x * per + k];
  }
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t base = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (int k = 0; k < per; ++k) cursor[threadIdx.x * per + k] = base + loc[k];
}

template <int NF4>
__global__ void __launch_bounds__(256) k_bin_scatter(const uint32_t *__restrict__ keys, const uint32_t *count,
                                                    uint32_t *__restrict__ cursor, const float4 *__restrict__ in0,
                                                    const float4 *__restrict__ in1, const float4 *__restrict__ in2,
                                                    float4 *__restrict__ out0, float4 *__restrict__ out1,
                                                    float4 *__restrict__ out2) {
  constexpr int kPer = 16;                 // entries per thread per chunk
  constexpr int kChunk = 256 * kPer;
  __shared__ uint32_t h[kBins];
  const uint32_t n = *count;
  for (uint32_t c0 = blockIdx.x * kChunk; c0 < n; c0 += gridDim.x * kChunk) {
    for (int i = threadIdx.x; i < kBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    uint32_t key[kPer], rank[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      uint32_t i = c0 + k * 256 + threadIdx.x;
      key[k] = i < n ? (keys[i] & (kBins - 1)) : 0u;
      rank[k] = i < n ? atomicAdd(&h[key[k]], 1u) : 0u;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBins; i += blockDim.x)
      if (h[i]) h[i] = atomicAdd(&cursor[i], h[i]);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      uint32_t i = c0 + k * 256 + threadIdx.x;
      if (i < n) {
        uint32_t pos = h[key[k]] + rank[k];
        out0[pos] = in0[i];
        if (NF4 > 1) out1[pos] = in1[i];
        if (NF4 > 2) out2[pos] = in2[i];
      }
    }
    __syncthreads();
  }
}

// accumulate: per pixel, Kahan-add the wave's samples into the compensated FP32 film
// (ProgressiveFilterValue::addSample, ProgressiveFilterValue.h:33-36, box weight 1)
__global__ void __launch_bounds__(kBlock) k_accumulate(RenderArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long ext = 0, bounces = 0;
    for (int b = 0; b < a.max_b; ++b) {
      uint32_t c = a.counters[kCtrRay + b];
      ext += c;
      bounces += c ? 1ull : 0ull;
    }
    unsigned long long sh = 0;
    for (int b = 0; b < a.max_b; ++b) sh += a.counters[kCtrNee + b];
    a.stats[0] += ext;
    a.stats[1] += sh;
    a.stats[2] += a.counters[kCtrTrunc];
    a.stats[3] += bounces;
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < a.nslots; q += stride) {
    int x, y;
    if (!slot_pixel(a, a.slot0 + q, x, y)) continue;
    int64_t pix = (int64_t)y * a.W + x;
    float4 S = a.film_sum[pix], C = a.film_c[pix];
    for (int si = 0; si < a.ns; ++si) {
      const int64_t p = q * a.ns + si;
      float4 L4 = a.path_L[p];
      V3 L = v3(L4.x, L4.y, L4.z);
      if (__float_as_uint(L4.w) & kFlagNeePending) L = fold_slots(a, p, L);
      L = apply_mask(L, __float_as_uint(L4.w));
      if (a.path_out) {
        int s = a.s0 + si - a.sample_begin;
        a.path_out[pix * a.sample_count + s] = make_float4(L.x, L.y, L.z, L4.w);
      }
      float yx = L.x - C.x, tx = S.x + yx; C.x = (tx - S.x) - yx; S.x = tx;
      float yy = L.y - C.y, ty = S.y + yy; C.y = (ty - S.y) - yy; S.y = ty;
      float yz = L.z - C.z, tz = S.z + yz; C.z = (tz - S.z) - yz; S.z = tz;
    }
    S.w += (float)a.ns;
    a.film_sum[pix] = S;
    a.film_c[pix] = C;
  }
}

// ---------------------------------------------------------------------------------------
// host driver

struct Workspace {
  int device = -1;
  int64_t cap = 0;  // paths
  void *block = nullptr;
  float4 *path_L = nullptr, *qo[2] = {}, *qd[2] = {}, *qt[2] = {}, *qhit = nullptr;
  float4 *so = nullptr, *sd = nullptr, *slots = nullptr;
  float4 *qo_u = nullptr, *qd_u = nullptr, *qt_u = nullptr, *so_u = nullptr, *sd_u = nullptr;
  uint32_t *qkey = nullptr, *skey = nullptr, *hist = nullptr, *cursor = nullptr;  // hist/cursor: kBins each
  int64_t slot_cap = 0;  // light-sample slots
  uint32_t *counters = nullptr;
  unsigned long long *stats = nullptr;   // 4
  unsigned long long *tcount = nullptr;  // 8
  uint32_t *h_counters = nullptr;  // pinned (owned) or a static host word (allocation-free path)
  bool owned = true;
  ~Workspace() {
    if (!owned) return;
    if (block) cudaFree(block);
    if (h_counters) cudaFreeHost(h_counters);
  }
};

// process-wide tuning knobs (mgpu_tune_set)
struct Tuning {
  std::atomic<int> persistent{0};     // persistent warp-level traversal with ray refill
  std::atomic<int> bin_shadow{1};     // counting-sort shadow rays by (light, origin cell)
  std::atomic<int> bin_extension{1};  // counting-sort extension rays by (octant, origin cell)
};
static Tuning g_tune;

static thread_local Workspace *t_ws = nullptr;
static thread_local mgpu_render_stats t_stats{};
static thread_local cudaStream_t t_stats_stream = nullptr;
static thread_local bool t_stats_pending = false;
static thread_local unsigned long long *t_stats_dev = nullptr;  // device stats of the last render
static thread_local uint32_t *t_counters_dev = nullptr;          // queue counters of its last wave

// Per-kernel timing with CUDA events recorded on the launching stream around every launch.
enum { kProfGenerate = 0, kProfExtend, kProfShade, kProfShadow, kProfAccumulate, kProfBin, kProfClasses };
struct Profiler {
  bool enabled = false;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  std::vector<std::pair<int, size_t>> marks;  // (class, index of begin event); end = begin + 1
  cudaStream_t stream = nullptr;
  double ms[kProfClasses] = {0, 0, 0, 0, 0, 0};
  uint64_t launches[kProfClasses] = {0, 0, 0, 0, 0, 0};
  cudaEvent_t next() {
    if (used == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[used++];
  }
  int begin(int cls, cudaStream_t st) {
    if (!enabled) return -1;
    stream = st;
    size_t i = used;
    cudaEventRecord(next(), st);
    next();
    marks.push_back({cls, i});
    return (int)marks.size() - 1;
  }
  void end(int mark, cudaStream_t st) {
    if (mark < 0) return;
    cudaEventRecord(pool[marks[(size_t)mark].second + 1], st);
  }
  int flush() {
    if (marks.empty()) return MGPU_OK;
    MGPU_CUDA(cudaStreamSynchronize(stream));
    for (auto &m : marks) {
      float t = 0;
      MGPU_CUDA(cudaEventElapsedTime(&t, pool[m.second], pool[m.second + 1]));
      ms[m.first] += t;
      launches[m.first] += 1;
    }
    marks.clear();
    used = 0;
    return MGPU_OK;
  }
};
static thread_local Profiler t_prof;

// float4 arrays: path_L, 2 x (qo, qd, qt), qhit, unsorted (qo, qd, qt) = 11 per path;
// so, sd, slots, unsorted (so, sd) = 5 per light sample; uint32 keys per path and per sample
static size_t workspace_bytes(int64_t paths, int64_t slots) {
  size_t f4 = (size_t)paths * 11 + (size_t)slots * 5;
  size_t u32 = (size_t)paths + (size_t)slots + 2 * kBins + kNumCounters;
  return f4 * sizeof(float4) + 12 * sizeof(unsigned long long) + u32 * sizeof(uint32_t) + 1024;
}

static void workspace_layout(Workspace *w, void *block, int64_t paths, int64_t slots) {
  w->cap = paths;
  w->slot_cap = slots;
  w->block = block;
  float4 *f = (float4 *)block;
  w->path_L = f; f += paths;
  for (int k = 0; k < 2; ++k) { w->qo[k] = f; f += paths; w->qd[k] = f; f += paths; w->qt[k] = f; f += paths; }
  w->qhit = f; f += paths;
  w->qo_u = f; f += paths; w->qd_u = f; f += paths; w->qt_u = f; f += paths;
  w->so = f; f += slots; w->sd = f; f += slots; w->slots = f; f += slots;
  w->so_u = f; f += slots; w->sd_u = f; f += slots;
  w->stats = (unsigned long long *)f;
  w->tcount = w->stats + 4;
  uint32_t *u = (uint32_t *)(w->tcount + 8);
  w->qkey = u; u += paths;
  w->skey = u; u += slots;
  w->hist = u; u += kBins;
  w->cursor = u; u += kBins;
  w->counters = u;
}

static int ensure_workspace(int64_t paths, int64_t slots) {
  int dev = 0;
  MGPU_CUDA(cudaGetDevice(&dev));
  if (t_ws && t_ws->device == dev && t_ws->cap >= paths && t_ws->slot_cap >= slots) return MGPU_OK;
  if (t_ws) {
    cudaDeviceSynchronize();
    delete t_ws;
    t_ws = nullptr;
  }
  Workspace *w = new Workspace();
  w->device = dev;
  void *block = nullptr;
  cudaError_t e = cudaMalloc(&block, workspace_bytes(paths, slots));
  if (e != cudaSuccess) {
    delete w;
    return cuda_fail(e, "render workspace cudaMalloc");
  }
  workspace_layout(w, block, paths, slots);
  e = cudaMallocHost(&w->h_counters, 64);
  if (e != cudaSuccess) {
    delete w;
    return cuda_fail(e, "render workspace cudaMallocHost");
  }
  t_ws = w;
  return MGPU_OK;
}

// ---------------------------------------------------------------------------------------
// Fixed scratch for mgpu_render_noalloc: one static device array per process and device,
// resident from module load until exit.  Host code only holds a stand-in for the array's
// name; the device address comes from cudaGetSymbolAddress, once per device.
constexpr size_t kNoAllocBytes = (size_t)32 << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];
constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[kNoAllocMaxDevices];
static uint32_t g_noalloc_host_counter[16];  // pageable host word for live-path counts

static int noalloc_scratch(void **out) {
  int dev = 0;
  MGPU_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(MGPU_E_INVALID, "mgpu_render_noalloc: device ordinal too large");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "mgpu_render_noalloc: cudaGetSymbolAddress of the fixed scratch");
    if (!p) return fail(MGPU_E_CUDA, "mgpu_render_noalloc: fixed scratch has no device address");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return MGPU_OK;
}

// paths per wave that fit the fixed scratch for nl_slots light samples per path
static int64_t noalloc_paths(int64_t nl_slots) {
  const size_t fixed = workspace_bytes(0, 0);
  const size_t per = 11 * sizeof(float4) + sizeof(uint32_t) + (size_t)nl_slots * (5 * sizeof(float4) + sizeof(uint32_t));
  if (kNoAllocBytes <= fixed) return 0;
  int64_t p = (int64_t)((kNoAllocBytes - fixed) / per);
  return p / 64 * 64;
}

static int grid_for(const void *kern, size_t smem) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem);
  if (per_sm < 1) per_sm = 1;
  return device_sm_count() * per_sm;
}

static Camera make_camera(const float *c) {
  // ThinLensCamera::setOrientation (ThinLensCamera.cpp:241-259) and _computeMatrix (:204-210)
  double eye[3] = {c[0], c[1], c[2]}, look[3] = {c[3], c[4], c[5]}, up[3] = {c[6], c[7], c[8]};
  double n[3] = {-look[0], -look[1], -look[2]};
  double u[3] = {up[1] * n[2] - up[2] * n[1], up[2] * n[0] - up[0] * n[2], up[0] * n[1] - up[1] * n[0]};
  double ln = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]), lu = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  for (int k = 0; k < 3; ++k) { n[k] /= ln; u[k] /= lu; }
  double v[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2], n[0] * u[1] - n[1] * u[0]};
  double va = c[9] * (3.14159265358979323846 / 180.0);
  double th = tan(va / 2), tw = c[10] * th;
  Camera k;
  k.eye = v3((float)eye[0], (float)eye[1], (float)eye[2]);
  k.u = v3((float)u[0], (float)u[1], (float)u[2]);
  k.v = v3((float)v[0], (float)v[1], (float)v[2]);
  k.n = v3((float)n[0], (float)n[1], (float)n[2]);
  k.tan_w = (float)tw;
  k.tan_h = (float)th;
  return k;
}

template <bool COUNT>
static int render_impl(const mgpu_scene *sc, const mgpu_render_params *rp, mgpu_film *film, float *d_path_out,
                       void *stream, bool noalloc = false) {
  if (!sc || !rp || !film) return fail(MGPU_E_INVALID, "mgpu_render: null argument");
  if (rp->width != film->width || rp->height != film->height)
    return fail(MGPU_E_INVALID, "mgpu_render: film size differs from the render size");
  if (rp->width <= 0 || rp->height <= 0 || rp->spp <= 0 || rp->sample_count < 0 || rp->sample_begin < 0 ||
      rp->no_direct_samples <= 0 || rp->max_depth < 0 || rp->rr_start_depth < 0)
    return fail(MGPU_E_INVALID, "mgpu_render: bad parameters");
  if (rp->sample_count == 0) return MGPU_OK;
  if ((int64_t)rp->sample_begin + rp->sample_count > (int64_t)1 << 30)
    return fail(MGPU_E_INVALID, "mgpu_render: sample range too large");
  cudaStream_t st = as_stream(stream);
  RenderArgs a;
  memset(&a, 0, sizeof(a));
  a.view = sc->view;
  a.ntop = sc->top_pairs;
  a.shade = sc->d_shade;
  a.mats = (const float4 *)sc->d_mats;
  a.lights = (const float4 *)sc->d_lights;
  a.nlight = sc->nlight;
  a.cam = make_camera(rp->camera);
  a.rng.k0 = (uint32_t)rp->seed;
  a.rng.k1 = (uint32_t)(rp->seed >> 32);
  a.rng.stream = rp->stream_id;
  a.W = rp->width;
  a.H = rp->height;
  a.spp = rp->spp;
  a.side = std::max(1, (int)sqrt((double)rp->spp));
  a.s2 = a.side * a.side;
  a.nds = rp->no_direct_samples;
  a.nds_side = std::max(1, (int)sqrt((double)rp->no_direct_samples));
  a.max_depth = rp->max_depth;
  a.rr_start = rp->rr_start_depth;
  a.efficient = rp->efficient_direct;
  a.tiles_x = (a.W + 7) / 8;
  a.sample_begin = rp->sample_begin;
  a.sample_count = rp->sample_count;
  a.film_sum = film->d_sum;
  a.film_c = film->d_c;
  a.path_out = (float4 *)d_path_out;
  const int64_t tiles_y = (a.H + 7) / 8;
  const int64_t total_slots = (int64_t)a.tiles_x * tiles_y * 64;
  int64_t wave = rp->wave_paths > 0 ? rp->wave_paths : (int64_t)1 << 24;
  a.nl_slots = sc->nlight * a.nds_side * a.nds_side;
  if (a.nl_slots > 4096) return fail(MGPU_E_INVALID, "mgpu_render: too many light samples per vertex");
  if (noalloc) {
    const int64_t pmax = noalloc_paths(a.nl_slots);
    if (pmax < 64)
      return fail(MGPU_E_INVALID, "mgpu_render_noalloc: " + std::to_string(a.nl_slots) +
                                      " light samples per vertex do not fit the 32 MiB fixed scratch");
    if (rp->wave_paths > pmax)
      return fail(MGPU_E_INVALID, "mgpu_render_noalloc: wave_paths " + std::to_string(rp->wave_paths) +
                                      " exceeds the fixed scratch (32 MiB holds " + std::to_string(pmax) +
                                      " paths at " + std::to_string(a.nl_slots) + " light samples per vertex)");
    wave = rp->wave_paths > 0 ? rp->wave_paths : pmax;
  }
  // samples per wave: as many passes of the whole image as fit, else one pass over a slot range
  int ns = (int)std::max<int64_t>(1, std::min<int64_t>(rp->sample_count, wave / total_slots));
  int64_t slots_per_wave = std::min<int64_t>(total_slots, std::max<int64_t>(64, wave / ns) / 64 * 64);
  int64_t cap = slots_per_wave * ns;
  Workspace fixed_ws;
  Workspace *w = nullptr;
  if (noalloc) {
    void *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc != MGPU_OK) return rc;
    fixed_ws.owned = false;
    MGPU_CUDA(cudaGetDevice(&fixed_ws.device));
    workspace_layout(&fixed_ws, base, cap, std::max<int64_t>(1, cap * a.nl_slots));
    fixed_ws.h_counters = g_noalloc_host_counter;
    w = &fixed_ws;
  } else {
    int rc = ensure_workspace(cap, std::max<int64_t>(1, cap * a.nl_slots));
    if (rc != MGPU_OK) return rc;
    w = t_ws;
  }
  a.path_L = w->path_L;
  for (int k = 0; k < 2; ++k) { a.qo[k] = w->qo[k]; a.qd[k] = w->qd[k]; a.qt[k] = w->qt[k]; }
  a.qhit = w->qhit;
  a.so = w->so; a.sd = w->sd; a.slots = w->slots;
  a.qo_u = w->qo_u; a.qd_u = w->qd_u; a.qt_u = w->qt_u; a.so_u = w->so_u; a.sd_u = w->sd_u;
  a.qkey = w->qkey; a.skey = w->skey;
  a.bin_ext = g_tune.bin_extension.load();
  a.bin_sh = g_tune.bin_shadow.load();
  {
    int nlp = 1;
    while (nlp < std::min(sc->nlight, 16)) nlp <<= 1;
    int lb = 0;
    while ((1 << lb) < nlp) ++lb;
    a.sh_cell_bits = 12 - lb;  // light index in the top bits, origin cell below
  }
  a.counters = w->counters;
  a.stats = w->stats;
  a.tcount = w->tcount;

  const bool persist = g_tune.persistent.load() != 0;
  auto kext = persist ? k_extend<COUNT, true> : k_extend<COUNT, false>;
  auto kshw = persist ? k_shadow<COUNT, true> : k_shadow<COUNT, false>;
  size_t smem = (size_t)a.ntop * sizeof(uint4);
  if (smem > 48 * 1024) {
    MGPU_CUDA(cudaFuncSetAttribute(kext, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MGPU_CUDA(cudaFuncSetAttribute(kshw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int g_gen = grid_for((const void *)k_generate, 0);
  const int g_ext = grid_for((const void *)kext, smem);
  const int g_sha = grid_for((const void *)k_shade, 0);
  const int g_shw = grid_for((const void *)kshw, smem);
  const int g_acc = grid_for((const void *)k_accumulate, 0);
  const int g_bin = device_sm_count() * 4;

  mgpu_render_stats stats{};
  uint64_t launches = 0;
  const int max_b = rp->max_depth > 0 ? std::min(rp->max_depth, kHardCap) : kHardCap;
  a.max_b = max_b;
  MGPU_CUDA(cudaMemsetAsync(w->stats, 0, 12 * sizeof(unsigned long long), st));
  Profiler off;  // the allocation-free path records no events
  Profiler &pf = noalloc ? off : t_prof;
  for (int s0 = rp->sample_begin; s0 < rp->sample_begin + rp->sample_count; s0 += ns) {
    a.s0 = s0;
    a.ns = std::min(ns, rp->sample_begin + rp->sample_count - s0);
    for (int64_t slot0 = 0; slot0 < total_slots; slot0 += slots_per_wave) {
      a.slot0 = slot0;
      a.nslots = std::min(slots_per_wave, total_slots - slot0);
      MGPU_CUDA(cudaMemsetAsync(w->counters, 0, kNumCounters * sizeof(uint32_t), st));
      int m = pf.begin(kProfGenerate, st);
      k_generate<<<g_gen, kBlock, 0, st>>>(a);
      pf.end(m, st);
      ++launches;
      int b = 0;
      while (b < max_b) {
        // with a fixed depth cap every bounce is launched blind; without one, check the live
        // count every 4 bounces and stop when the wave has drained
        int chunk = rp->max_depth > 0 ? max_b : std::min(4, max_b - b);
        for (int k = 0; k < chunk; ++k, ++b) {
          m = pf.begin(kProfExtend, st);
          kext<<<g_ext, kBlock, smem, st>>>(a, b);
          pf.end(m, st);
          m = pf.begin(kProfShade, st);
          k_shade<<<g_sha, kBlock, 0, st>>>(a, b);
          pf.end(m, st);
          if (a.bin_sh || a.bin_ext) {
            m = pf.begin(kProfBin, st);
            if (a.bin_sh) {
              MGPU_CUDA(cudaMemsetAsync(w->hist, 0, kBins * sizeof(uint32_t), st));
              k_bin_hist<<<g_bin, 256, 0, st>>>(w->skey, a.counters + kCtrNee + b, w->hist);
              k_bin_scan<<<1, 1024, 0, st>>>(w->hist, w->cursor);
              k_bin_scatter<2><<<g_bin, 256, 0, st>>>(w->skey, a.counters + kCtrNee + b, w->cursor, w->so_u, w->sd_u,
                                                      nullptr, w->so, w->sd, nullptr);
              launches += 3;
            }
            if (a.bin_ext && b + 1 < max_b) {
              const int nx = (b + 1) & 1;
              MGPU_CUDA(cudaMemsetAsync(w->hist, 0, kBins * sizeof(uint32_t), st));
              k_bin_hist<<<g_bin, 256, 0, st>>>(w->qkey, a.counters + kCtrRay + b + 1, w->hist);
              k_bin_scan<<<1, 1024, 0, st>>>(w->hist, w->cursor);
              k_bin_scatter<3><<<g_bin, 256, 0, st>>>(w->qkey, a.counters + kCtrRay + b + 1, w->cursor, w->qo_u,
                                                      w->qd_u, w->qt_u, w->qo[nx], w->qd[nx], w->qt[nx]);
              launches += 3;
            }
            pf.end(m, st);
          }
          m = pf.begin(kProfShadow, st);
          kshw<<<g_shw, kBlock, smem, st>>>(a, b);
          pf.end(m, st);
          launches += 3;
        }
        if (rp->max_depth > 0) break;
        MGPU_CUDA(cudaMemcpyAsync(w->h_counters, w->counters + kCtrRay + b, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        MGPU_CUDA(cudaStreamSynchronize(st));
        if (w->h_counters[0] == 0) break;
      }
      m = pf.begin(kProfAccumulate, st);
      k_accumulate<<<g_acc, kBlock, 0, st>>>(a);
      pf.end(m, st);
      ++launches;
      MGPU_CUDA(cudaGetLastError());
    }
  }
  g_launches.fetch_add(launches);
  stats.paths = (uint64_t)a.W * a.H * (uint64_t)rp->sample_count;
  stats.kernel_launches = launches;
  t_stats = stats;
  t_stats_stream = st;
  t_stats_dev = w->stats;
  t_counters_dev = w->counters;
  t_stats_pending = true;
  return MGPU_OK;
}

}  // namespace mgpu

using namespace mgpu;

extern "C" {

int mgpu_render(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, void *stream) {
  return render_impl<false>(scene, params, film, nullptr, stream);
}

int mgpu_render_paths(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, float *d_path_L,
                      void *stream) {
  if (!d_path_L) return fail(MGPU_E_INVALID, "mgpu_render_paths: null path buffer");
  return render_impl<false>(scene, params, film, d_path_L, stream);
}

// Allocation-free render: the same estimator and film as mgpu_render, over the fixed 32 MiB
// scratch instead of a cudaMalloc'd workspace.  See include/mgpu.h for the contract.
int mgpu_render_noalloc(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, void *stream) {
  return render_impl<false>(scene, params, film, nullptr, stream, true);
}

int mgpu_render_counted(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film,
                        uint64_t *counts8, void *stream) {
  if (!counts8) return fail(MGPU_E_INVALID, "mgpu_render_counted: null output");
  int rc = render_impl<true>(scene, params, film, nullptr, stream);
  if (rc != MGPU_OK) return rc;
  MGPU_CUDA(cudaStreamSynchronize(as_stream(stream)));
  MGPU_CUDA(cudaMemcpy(counts8, t_ws->tcount, 8 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return MGPU_OK;
}

int mgpu_render_wave_queues(uint32_t *ext, uint32_t *shadow, int32_t max_bounces) {
  if (!ext || !shadow || max_bounces <= 0) return fail(MGPU_E_INVALID, "mgpu_render_wave_queues: bad argument");
  if (!t_stats_dev) return fail(MGPU_E_STATE, "mgpu_render_wave_queues: nothing rendered on this thread");
  MGPU_CUDA(cudaStreamSynchronize(t_stats_stream));
  const uint32_t *ctr = t_counters_dev;
  int n = std::min(max_bounces, kHardCap);
  MGPU_CUDA(cudaMemcpy(ext, ctr + kCtrRay, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  MGPU_CUDA(cudaMemcpy(shadow, ctr + kCtrNee, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  return MGPU_OK;
}

int mgpu_render_stats_get(mgpu_render_stats *out) {
  if (!out) return fail(MGPU_E_INVALID, "mgpu_render_stats_get: null argument");
  if (t_stats_pending && t_stats_dev) {
    unsigned long long h[4];
    MGPU_CUDA(cudaStreamSynchronize(t_stats_stream));
    MGPU_CUDA(cudaMemcpy(h, t_stats_dev, sizeof(h), cudaMemcpyDeviceToHost));
    t_stats.extension_rays = h[0];
    t_stats.shadow_rays = h[1];
    t_stats.truncated_paths = h[2];
    t_stats.bounces = h[3];
    t_stats_pending = false;
  }
  *out = t_stats;
  return MGPU_OK;
}

int mgpu_profile_enable(int enable) {
  Profiler &p = t_prof;
  int rc = p.flush();
  if (rc != MGPU_OK) return rc;
  p.enabled = enable != 0;
  for (int k = 0; k < kProfClasses; ++k) { p.ms[k] = 0; p.launches[k] = 0; }
  return MGPU_OK;
}

int mgpu_profile_read(double *ms6, uint64_t *launches6) {
  if (!ms6 || !launches6) return fail(MGPU_E_INVALID, "mgpu_profile_read: null argument");
  Profiler &p = t_prof;
  int rc = p.flush();
  if (rc != MGPU_OK) return rc;
  for (int k = 0; k < kProfClasses; ++k) { ms6[k] = p.ms[k]; launches6[k] = p.launches[k]; }
  return MGPU_OK;
}

int mgpu_tune_set(const char *key, int64_t value) {
  if (!key) return fail(MGPU_E_INVALID, "mgpu_tune_set: null key");
  std::string k(key);
  if (k == "persistent") g_tune.persistent.store(value != 0);
  else if (k == "bin_shadow") g_tune.bin_shadow.store(value != 0);
  else if (k == "bin_extension") g_tune.bin_extension.store(value != 0);
  else return fail(MGPU_E_INVALID, "mgpu_tune_set: unknown key " + k);
  return MGPU_OK;
}

int mgpu_tune_get(const char *key, int64_t *value) {
  if (!key || !value) return fail(MGPU_E_INVALID, "mgpu_tune_get: null argument");
  std::string k(key);
  if (k == "persistent") *value = g_tune.persistent.load();
  else if (k == "bin_shadow") *value = g_tune.bin_shadow.load();
  else if (k == "bin_extension") *value = g_tune.bin_extension.load();
  else return fail(MGPU_E_INVALID, "mgpu_tune_get: unknown key " + k);
  return MGPU_OK;
}

}  // extern "C"
