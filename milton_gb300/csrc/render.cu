// render.cu -- wavefront path tracer: generate -> (extend -> shade -> shadow)* -> accumulate.
//
// Work is organised in waves of paths.  A wave holds one or more job chunks; a chunk is a range
// of pixel slots (8x8 tiles, row-major tile order) x a range of sample passes of one render job
// (one scene, camera, film and set of PathTracer parameters).  A plain render is one job; a batch
// (mgpu_batch_*) packs the chunks of many jobs of uneven size into shared waves, so small scenes
// fill the GPU together.  Per-chunk parameters live in a device array of JobArgs; every path
// records its chunk in path_job[], and every kernel reads its chunk's scene and parameters there.
//
// Per path the state is split in two:
//   path_L[p]     float4  radiance accumulated so far (rgb) + path flags (w) -- path-indexed,
//                          updated by shade (emission, folded direct light), read by accumulate;
//   ray queue     3 x float4 per live path (origin + path index, direction + chunk, throughput +
//                          depth state), compacted every bounce by warp ballot + one atomicAdd per
//                          warp.
// Direct light (DirectIllumination::evaluate over all lights x noDirectSamples,
// DirectIllumination.cpp:46-138) is split in two: shade samples every light, evaluates the BSDF,
// writes each sample's contribution into the path's slot for that sample and queues one shadow
// ray per non-zero contribution; the shadow kernel is a plain any-hit query that zeroes the slot
// of an occluded sample.  The next kernel to see the path (shade at the next bounce, or
// accumulate) folds its slots into the radiance in slot order, so every sum runs in a fixed
// order and the image does not depend on queue order, wave size or batch composition.
#include <string.h>

#include <algorithm>
#include <climits>
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
constexpr int kBinBits = 14;           // queue binning keys: 2^14 bins
constexpr int kBins = 1 << kBinBits;
constexpr int kBinSmem = kBins * 4;    // dynamic shared memory of a sorting block
constexpr double kAutoWaveBytes = 40e9;  // workspace budget of an automatic wave
#ifndef MGPU_TRAV_MIN_BLOCKS
#define MGPU_TRAV_MIN_BLOCKS 12
#endif
// Resident 128-thread blocks per SM the traversal kernels are compiled for: 12 caps them at 40
// registers (a few bytes of spills to L1) for 48 warps per SM instead of 36-40, which hides more
// of the node-load latency (mid frame: 215 -> 226 Mpaths/s; 10 and 16 blocks measured 221).
constexpr int kTravMinBlocks = MGPU_TRAV_MIN_BLOCKS;
#ifndef MGPU_SHADE_MIN_BLOCKS
#define MGPU_SHADE_MIN_BLOCKS 8
#endif
// the shade kernel at 8 blocks per SM (64 registers, spilling ~0.8 KB to L1) against its natural
// 125 registers: 211 -> 184 ms per 5 mid frames
constexpr int kShadeMinBlocks = MGPU_SHADE_MIN_BLOCKS;

// One job chunk of a wave (device memory).
struct JobArgs {
  SceneView view;
  const float4 *shade;
  const float4 *mats;    // 4 per material
  const float4 *lights;  // 4 per light
  const float2 *uv;      // 3 per triangle (nullptr: every uv is (0, 0))
  const float4 *texrec;  // 2 per texture
  const float4 *texels;
  int32_t bg_tex;          // background environment map (1 + texture index) or 0
  float bg_le[3];          // constant background radiance (bg_tex == 0)
  int32_t nlight, nl_slots, sh_cell_bits;
  float cell_scale[3];     // queue-bin cells: 32 / the scene's extent per axis (0: a flat axis)
  Camera cam;
  Rng rng;
  int32_t W, H, spp, side, s2, nds, nds_side, max_depth, rr_start, efficient, tiles_x;
  int32_t s0, ns;                 // samples [s0, s0 + ns) of this chunk
  int32_t sample_begin, sample_count;
  int64_t slot0, nslots;          // slots [slot0, slot0 + nslots)
  int64_t path_base;              // first wave path of the chunk
  int64_t slot_base;              // first accumulate slot of the chunk in the wave
  float4 *film_sum, *film_c;
  FilmFilter filt;                 // reconstruction filter of the film (kFilterNone: mean only)
  unsigned long long *film_fx;     // its fixed-point splat sums (4 per pixel)
  float4 *path_out;               // optional per-path radiance
};

// One wave (kernel parameter).
struct RenderArgs {
  const JobArgs *jobs;
  int32_t njobs;
  int64_t npaths, nslots;         // paths and accumulate slots in the wave
  int32_t nl_stride;              // light-sample slots per path (max over the wave's chunks)
  uint32_t *path_job;
  float4 *path_L;
  float4 *qo[2], *qd[2], *qt[2];
  float4 *qhit;
  float4 *so, *sd;               // shadow ray queue: origin + slot index, direction + tmax
  float4 *slots;                 // nl_stride per path: direct-light contribution per light sample
  float4 *qo_u, *qd_u, *qt_u;    // unsorted next-ray queue (binning on)
  float4 *so_u, *sd_u;           // unsorted shadow queue (binning on)
  uint32_t *qkey, *skey;         // bin keys of the unsorted queues
  int32_t bin_ext, bin_sh;       // counting-sort the queues by (direction octant | light, origin cell)
  uint32_t *counters;
  unsigned long long *stats;     // [0] extension rays, [1] shadow rays, [2] truncated paths, [3] bounces
  unsigned long long *tcount;    // counted mode: ext nodes, refs, tris, rays; shadow nodes, refs, tris, rays
  int32_t max_b;
  SceneView view0;               // the scene of a wave of one scene (njobs == 1)
};

// A film has fewer than 2^31 pixels and a wave fewer than 2^31 paths (both checked on the host),
// so slot and path indices within a chunk are divided in 32-bit unsigned arithmetic (a 64-bit
// division is several times the instructions, and these run for every path in three kernels).
__device__ __forceinline__ bool slot_pixel(const JobArgs &J, int64_t slot, int &x, int &y) {
  const uint32_t tile = (uint32_t)(slot >> 6), tx = (uint32_t)J.tiles_x;
  const uint32_t ty = tile / tx;
  const int within = (int)(slot & 63);
  x = (int)(tile - ty * tx) * 8 + (within & 7);
  y = (int)ty * 8 + (within >> 3);
  return x < J.W && y < J.H;
}

// global path id (pixel * spp + sample) for wave path p of chunk J
__device__ __forceinline__ uint64_t path_id(const JobArgs &J, int64_t p, int &x, int &y, int &s) {
  const uint32_t lp = (uint32_t)(p - J.path_base), ns = (uint32_t)J.ns;
  const uint32_t q = lp / ns;
  const int64_t slot = J.slot0 + q;
  s = J.s0 + (int)(lp - q * ns);
  slot_pixel(J, slot, x, y);
  return ((uint64_t)y * J.W + x) * (uint64_t)J.spp + (uint64_t)s;
}

// chunk holding wave path p / accumulate slot q (binary search over the sorted bases)
__device__ __forceinline__ int job_of_path(const RenderArgs &a, int64_t p) {
  int lo = 0, hi = a.njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (a.jobs[mid].path_base <= p) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int job_of_slot(const RenderArgs &a, int64_t q) {
  int lo = 0, hi = a.njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (a.jobs[mid].slot_base <= q) lo = mid; else hi = mid - 1;
  }
  return lo;
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

__device__ __forceinline__ Material load_mat(const JobArgs &J, int i, uint32_t ior_index) {
  float m[16];
  float4 *mm = reinterpret_cast<float4 *>(m);
#pragma unroll
  for (int k = 0; k < 4; ++k) mm[k] = __ldg(J.mats + 4 * i + k);
  return material_from(m, ior_index);
}

// Image maps at a hit of triangle prim with barycentrics (b0, b1, b2): the uv (Shape::_getUV,
// interpolated from the per-vertex uvs), then each textured key of the material and the bump
// map (Material::initSurfacePoint, Material.cpp:157-225).
__device__ __noinline__ void apply_textures(const JobArgs &J, int prim, float b0, float b1, float b2, V3 P,
                                            Material &m, V3 &ns) {
  float u = 0.0f, v = 0.0f;
  if (prim >= J.view.ntri) {
    // Sphere::_getUV (Sphere.cpp:78-85) of the object-space point: the offset from the centre,
    // rotated into the sphere's frame, over its diameter
    const float4 c = __ldg(reinterpret_cast<const float4 *>(J.view.spheres) + 2 * (prim - J.view.ntri));
    const float4 q = __ldg(reinterpret_cast<const float4 *>(J.view.spheres) + 2 * (prim - J.view.ntri) + 1);
    sphere_uv(quat_rotate(q.x, q.y, q.z, q.w, (P - v3(c.x, c.y, c.z)) * (0.5f / c.w)), u, v);
  } else if (J.uv) {
    const float2 a = __ldg(J.uv + 3 * (int64_t)prim), b = __ldg(J.uv + 3 * (int64_t)prim + 1),
                 c = __ldg(J.uv + 3 * (int64_t)prim + 2);
    u = a.x * b0 + b.x * b1 + c.x * b2;
    v = a.y * b0 + b.y * b1 + c.y * b2;
  }
  const int slots[4] = {m.tex_kd, m.tex_ks, m.tex_tr, m.tex_bump};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (slots[k] == 0) continue;
    const float4 r0 = __ldg(J.texrec + 2 * (slots[k] - 1)), r1 = __ldg(J.texrec + 2 * (slots[k] - 1) + 1);
    const int w = __float_as_int(r0.y), h = __float_as_int(r0.z);
    const float4 t = __ldg(J.texels + __float_as_uint(r0.x) + tex_texel(u, v, w, h, r1.x, r1.y));
    if (k < 3) tex_apply(m, k, t.x, t.y, t.z);
    else ns = bump_normal(ns, t.x, t.y, r1.z);
  }
}

// Background radiance of a ray leaving the scene in direction d: EnvironmentMap::getLe(-d)
// (the map's filtered texel at the uv of -d) or the constant of an omni background.
__device__ __noinline__ V3 background(const JobArgs &J, V3 d) {
  if (J.bg_tex == 0) return v3(J.bg_le[0], J.bg_le[1], J.bg_le[2]);
  float u, v;
  env_uv(-d, u, v);
  const float4 r0 = __ldg(J.texrec + 2 * (J.bg_tex - 1)), r1 = __ldg(J.texrec + 2 * (J.bg_tex - 1) + 1);
  const int w = __float_as_int(r0.y), h = __float_as_int(r0.z);
  const float4 t = __ldg(J.texels + __float_as_uint(r0.x) + tex_texel(u, v, w, h, r1.x, r1.y));
  return v3(t.x, t.y, t.z);
}

// light records: 8 float4 each (base record, then the extension)
__device__ __forceinline__ Light load_light(const JobArgs &J, int i) {
  float l[32];
  float4 *ll = reinterpret_cast<float4 *>(l);
#pragma unroll
  for (int k = 0; k < 8; ++k) ll[k] = __ldg(J.lights + 8 * i + k);
  return light_from(l, l + 16);
}

// Binning keys (kBins = 16384).  Ray coherence: rays of one warp should start close together
// and head the same way, so that they visit the same nodes.  Keys combine the direction
// octant (extension rays) or the light index (shadow rays) with the Morton code of the
// origin's cell in a 32x32x32 grid over the scene bounds (the top bits of it that fit).
__device__ __forceinline__ uint32_t spread4(uint32_t v) {  // 4 bits -> every third bit
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

__device__ __forceinline__ uint32_t spread5(uint32_t v) {  // 5 bits -> every third bit
  return spread4(v & 15u) | ((v & 16u) << 8);
}

// The keys only order the queues (no result depends on them), so the cell is taken with a
// multiplication by the precomputed 32 / extent rather than a division per axis.
__device__ __forceinline__ uint32_t morton15(const JobArgs &J, V3 p) {
  uint32_t c[3];
  const float pp[3] = {p.x, p.y, p.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int q = (int)((pp[k] - J.view.bmin[k]) * J.cell_scale[k]);
    c[k] = (uint32_t)min(max(q, 0), 31);
  }
  return (spread5(c[0]) << 2) | (spread5(c[1]) << 1) | spread5(c[2]);
}

__device__ __forceinline__ uint32_t ext_key(const JobArgs &J, V3 o, V3 d) {
  uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
  return (oct << (kBinBits - 3)) | (morton15(J, o) >> (18 - kBinBits));
}

__device__ __forceinline__ uint32_t sh_key(const JobArgs &J, int light, V3 o) {
  uint32_t cell = morton15(J, o) >> (15 - J.sh_cell_bits);
  return (((uint32_t)light << J.sh_cell_bits) | cell) & (kBins - 1);
}

// ---------------------------------------------------------------------------------------
// generate: camera rays for every path of the wave (RayTracer::sample, RayTracer.cpp:19-30;
// SuperSampleGenerator strata, SuperSampleGenerator.cpp:60-90)
__global__ void __launch_bounds__(kBlock) k_generate(RenderArgs a) {
  const int64_t n = a.npaths;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    int64_t p = base + threadIdx.x;
    bool valid = p < n;
    bool live = false;
    float4 o4 = make_float4(0, 0, 0, 0), d4 = o4;
    if (valid) {
      const int j = job_of_path(a, p);
      const JobArgs &J = a.jobs[j];
      a.path_job[p] = (uint32_t)j;
      int x, y, s;
      uint64_t pid = path_id(J, p, x, y, s);
      live = x < J.W && y < J.H;
      uint32_t flags = 0;
      if (live) {
        uint64_t pix = (uint64_t)y * J.W + x;
        int k = s % J.s2;
        F4u jt = uniforms(J.rng, pix * (uint64_t)J.s2 + (uint64_t)k, kDepthJitter, 0);
        float px = ((float)x + ((float)(k % J.side) + jt.a) / (float)J.side) / (float)J.W;
        float py = ((float)y + ((float)(k / J.side) + jt.b) / (float)J.side) / (float)J.H;
        F4u ui = uniforms(J.rng, pid, kDepthPathInit, 0);
        uint32_t ior = min((uint32_t)(ui.a * 3.0f), 2u);
        flags = ior;
        V3 o, d;
        camera_ray(J.cam, px, py, ui.b, ui.c, o, d);
        o4 = make_float4(o.x, o.y, o.z, __int_as_float((int)p));
        d4 = make_float4(d.x, d.y, d.z, __int_as_float(j));
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
// traversal kernel shapes (mgpu_tune_set "persistent" / "coop_leaf")
constexpr int kShapeGrid = 0;     // grid-stride, one ray per lane to completion
constexpr int kShapePersist = 1;  // persistent warps with per-lane refill
constexpr int kShapeCoop = 2;     // grid-stride, leaf triangles shared by the warp
#ifndef MGPU_COOP_MIN_BLOCKS
#define MGPU_COOP_MIN_BLOCKS 12
#endif
#ifndef MGPU_COOP_EXT_MIN_BLOCKS
#define MGPU_COOP_EXT_MIN_BLOCKS 10
#endif
// resident 128-thread blocks per SM (their register budget) of the warp-cooperative traversal
// shape: any hit 12 (40 registers), closest hit 10 (48 registers: its shared-memory reduction and
// winner re-test hold more state; mid frame 90.7 ms at 10 against 95.7 at 12 and 97.7 at 14, the
// any-hit kernel 116.0 at 10 against 113.2 at 12)
constexpr int kCoopMinBlocks = MGPU_COOP_MIN_BLOCKS;
constexpr int kCoopExtMinBlocks = MGPU_COOP_EXT_MIN_BLOCKS;

// BLK: threads per block of a traversal kernel (mgpu_tune_set "trav_block"); the resident
// blocks per SM scale with it, so every block size gets the same register budget per thread
template <bool COUNT, int SHAPE, bool SPH = false, int BLK = kBlock>
__global__ void __launch_bounds__(BLK, (SHAPE == kShapeCoop ? kCoopExtMinBlocks : kTravMinBlocks) * kBlock / BLK)
    k_extend(RenderArgs a, int b) {
  const uint32_t n = a.counters[kCtrRay + b];
  const float4 *qo = a.qo[b & 1], *qd = a.qd[b & 1];
  float4 *qhit = a.qhit;
  TraceCounts c = {0, 0, 0, 0};
  uint32_t rays = 0;
  const bool single = a.njobs == 1;
  const SceneView *view0 = &a.jobs[0].view;
  auto view_of = [&](uint32_t i) -> const SceneView & {
    return single ? *view0 : a.jobs[__float_as_int(qd[i].w)].view;
  };
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
  if (SHAPE == kShapePersist) {
    persistent_trace<false, COUNT, SPH>(view_of, nullptr, 0, n, &a.counters[kCtrFetchExt + b], load, store, &c, rays);
  } else if (SHAPE == kShapeCoop) {
    // per warp: the closest-hit keys of the shared leaf tests and the lanes' ray constants
    __shared__ unsigned long long wkey[BLK];
    __shared__ float4 wray[2 * BLK];
    __shared__ uint32_t wk[BLK];
    if (single)
      grid_trace_coop<false, COUNT, SPH, true>([&](uint32_t) -> const SceneView & { return a.view0; }, n, load, store,
                                               &c, rays, wkey + (threadIdx.x & ~31u), wray + 2 * (threadIdx.x & ~31u),
                                               wk + (threadIdx.x & ~31u));
    else
      grid_trace_coop<false, COUNT, SPH>(view_of, n, load, store, &c, rays, wkey + (threadIdx.x & ~31u),
                                         wray + 2 * (threadIdx.x & ~31u), wk + (threadIdx.x & ~31u));
  } else {
    grid_trace<false, COUNT, SPH>(view_of, nullptr, 0, n, load, store, &c, rays);
  }
  if (COUNT && rays) {
    atomicAdd(&a.tcount[0], (unsigned long long)c.nodes);
    atomicAdd(&a.tcount[1], (unsigned long long)c.refs);
    atomicAdd(&a.tcount[2], (unsigned long long)c.tris);
    atomicAdd(&a.tcount[3], (unsigned long long)rays);
  }
}

// shade: pending direct light, emission, light sampling, BSDF sample and Russian roulette
// (PathTracer.cpp:36-115, DirectIllumination.cpp:46-138)
__device__ __forceinline__ V3 fold_slots(const RenderArgs &a, int nl, int64_t p, V3 L) {
  const float4 *sl = a.slots + p * a.nl_stride;
  for (int k = 0; k < nl; ++k) {
    float4 c = sl[k];
    L = L + v3(c.x, c.y, c.z);
  }
  return L;
}

// SURF: the wave has a scene with image maps, a background or analytic spheres.  Scenes without
// them run the variant that has none of those branches, whose register allocation (and spilling)
// is the lighter.
template <bool SURF>
__global__ void __launch_bounds__(kBlock, kShadeMinBlocks) k_shade(RenderArgs a, int b) {
  const uint32_t n = a.counters[kCtrRay + b];
  const int cur = b & 1, nxt = (b + 1) & 1;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    uint32_t i = base + threadIdx.x;
    bool valid = i < n;
    bool want_next = false, do_nee = false;
    float4 no_o, no_d, no_t;
    int64_t p = 0;
    uint64_t pid = 0;
    int depth = 0, self = -1, j = 0;
    V3 P = v3(0, 0, 0), ns = P, ng = P, d = P, thr = P;
    Material m;
    m.type = 0;
    if (valid) {
      float4 o4 = a.qo[cur][i], d4 = a.qd[cur][i], t4 = a.qt[cur][i], h4 = a.qhit[i];
      p = (int64_t)__float_as_int(o4.w);
      j = __float_as_int(d4.w);
      const JobArgs &J = a.jobs[j];
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
        L = fold_slots(a, J.nl_slots, p, L);
        flags &= ~kFlagNeePending;
      }
      if (prim >= 0) {
        int x, y, s;
        pid = path_id(J, p, x, y, s);
        float t = h4.x, b1 = h4.z, b2 = h4.w, b0 = 1.0f - b1 - b2;
        float4 s0 = __ldg(J.shade + 3 * (int64_t)prim), s1 = __ldg(J.shade + 3 * (int64_t)prim + 1);
        if (SURF && prim >= J.view.ntri) {
          // analytic sphere: the hit on the ray, the radial normal (Sphere::_getGeometricNormal)
          const float4 c = __ldg(reinterpret_cast<const float4 *>(J.view.spheres) + 2 * (prim - J.view.ntri));
          P = v3(o4.x, o4.y, o4.z) + d * t;
          ns = normalize(P - v3(c.x, c.y, c.z));
          ng = ns;
        } else {
          float4 va = __ldg(reinterpret_cast<const float4 *>(J.view.tris) + 3 * (int64_t)prim);
          float4 vb = __ldg(reinterpret_cast<const float4 *>(J.view.tris) + 3 * (int64_t)prim + 1);
          float4 vc = __ldg(reinterpret_cast<const float4 *>(J.view.tris) + 3 * (int64_t)prim + 2);
          float4 s2 = __ldg(J.shade + 3 * (int64_t)prim + 2);
          V3 v0 = v3(va.x, va.y, va.z), v1 = v3(vb.x, vb.y, vb.z), v2 = v3(vc.x, vc.y, vc.z);
          P = v0 * b0 + v1 * b1 + v2 * b2;
          ns = normalize(v3(s0.x, s0.y, s0.z) * b0 + v3(s1.x, s1.y, s1.z) * b1 + v3(s2.x, s2.y, s2.z) * b2);
          ng = normalize(cross(v1 - v0, v2 - v0));
        }
        int mi = __float_as_int(s0.w);
        self = __float_as_int(s1.w);
        m = load_mat(J, mi, flags & kFlagIorMask);
        if (SURF && (m.tex_kd | m.tex_ks | m.tex_tr | m.tex_bump) != 0) apply_textures(J, prim, b0, b1, b2, P, m, ns);
        bool spec = is_specular(m);
        if (spec) flags |= kFlagSpecular;
        if (self >= 0) {
          Light lt = load_light(J, self);
          V3 Le = light_le(lt, ns, -d);
          if (!J.efficient || depth == 0) L = L + mul(thr, Le);
          else if (ec) L = L + mul(thr, Le) * (lt.area / (t * t));
        }
        if (J.efficient && !spec && J.nlight > 0) {
          do_nee = true;
          flags |= kFlagNeePending;
        }
        F4u u = uniforms(J.rng, pid, (uint32_t)depth, 0);
        V3 wo, fs;
        int ev = bsdf_sample(m, ns, d, flags & kFlagIorMask, u.a, u.b, u.c, wo, fs);
        if (ev > 0) {
          float pc = depth < J.rr_start ? (nonzero(fs) ? 1.0f : 0.0f) : fminf(0.95f, maxc(fs));
          bool capped = (J.max_depth > 0 && depth + 1 >= J.max_depth);
          if (!capped && u.d < pc) {
            if (depth + 1 >= kHardCap) {
              flags |= kFlagTruncated;
              atomicAdd(&a.counters[kCtrTrunc], 1u);
            } else {
              want_next = true;
              if (depth == 0) flags |= kFlagContinued0;
              V3 nthr = mul(thr, fs) * rcp(pc);
              bool nec = spec && dot(ns, wo) > kEps;
              V3 org = offset_origin(P, dot(ng, wo) > 0.0f ? ng : -ng);
              no_o = make_float4(org.x, org.y, org.z, o4.w);
              no_d = make_float4(wo.x, wo.y, wo.z, d4.w);
              no_t = make_float4(nthr.x, nthr.y, nthr.z, __uint_as_float((uint32_t)(depth + 1) | (nec ? 0x10000u : 0u)));
            }
          }
        }
      } else if (SURF && (J.bg_tex != 0 || J.bg_le[0] != 0.0f || J.bg_le[1] != 0.0f || J.bg_le[2] != 0.0f)) {
        L = L + mul(thr, background(J, d));  // PathTracer.cpp:39-42: a miss adds the background
      }
      a.path_L[p] = make_float4(L.x, L.y, L.z, __uint_as_float(flags));
    }
    const JobArgs &J = a.jobs[j];
    uint32_t q = warp_append(&a.counters[kCtrRay + b + 1], want_next);
    if (want_next) {
      if (a.bin_ext) {
        a.qo_u[q] = no_o;
        a.qd_u[q] = no_d;
        a.qt_u[q] = no_t;
        a.qkey[q] = ext_key(J, v3(no_o.x, no_o.y, no_o.z), v3(no_d.x, no_d.y, no_d.z));
      } else {
        a.qo[nxt][q] = no_o;
        a.qd[nxt][q] = no_d;
        a.qt[nxt][q] = no_t;
      }
    }
    // light samples: every lane of the warp runs the same k loop (uniform trip count: the
    // wave's stride), so the warp-aggregated append stays converged
    const int s2n = J.nds_side * J.nds_side;
    const float inv_nds = rcp((float)J.nds);
    F4u u = {0.0f, 0.0f, 0.0f, 0.0f};  // light samples 2m and 2m + 1 share counter block 1 + m
    for (int k = 0; k < a.nl_stride; ++k) {
      bool want = false;
      float4 so4, sd4;
      if (do_nee && k < J.nl_slots) {
        int li = k / s2n, within = k - li * s2n;
        int sy = within / J.nds_side, sx = within - sy * J.nds_side;
        V3 c = v3(0.0f, 0.0f, 0.0f);
        Light lt = load_light(J, li);
        if ((k & 1) == 0) u = uniforms(J.rng, pid, (uint32_t)depth, 1u + (uint32_t)(k >> 1));
        // a point light takes one sample (DirectIllumination.cpp:97-99): the first stratum
        if (li != self && (lt.type != kLightPoint || within == 0)) {
          float ux = (float)sx + ((k & 1) ? u.c : u.a), uy = (float)sy + ((k & 1) ? u.d : u.b);
          if (J.nds_side != 1) {  // x / 1 = x: one light sample per light needs no division
            ux = ux / (float)J.nds_side;
            uy = uy / (float)J.nds_side;
          }
          float r1 = 0.0f, r2 = 0.0f;
          if (lt.type == kLightMesh) {
            F4u um = uniforms(J.rng, pid, (uint32_t)depth, kMeshLightBlock + (uint32_t)k);
            r1 = um.a;
            r2 = um.b;
          }
          V3 lp, ln, lg;
          light_point(
              lt, ux, uy, r1, r2,
              [&](uint32_t t, int c) {
                const float4 q = __ldg(reinterpret_cast<const float4 *>(J.view.tris) + 3 * (int64_t)t + c);
                return v3(q.x, q.y, q.z);
              },
              [&](uint32_t t, int c) {
                const float4 q = __ldg(J.shade + 3 * (int64_t)t + c);
                return v3(q.x, q.y, q.z);
              },
              lp, ln, lg);
          V3 wo = lp - P;
          float t = length(wo);
          wo = wo * rcp(t);
          const bool point = lt.type == kLightPoint;
          float cwo = fabsf(dot(ns, wo)), cwi = point ? 1.0f : fabsf(dot(ln, wo));
          V3 fr = bsdf_eval(m, ns, d, wo);
          if (cwo > 0.0f && cwi > 0.0f && nonzero(fr)) {
            V3 Le = light_le(lt, ln, -wo);
            // area / samples for an area light, 1 for a point (DirectIllumination.cpp:127-128)
            c = mul(thr, mul(fr, Le)) * (cwo * cwi / (t * t) * (point ? 1.0f : lt.area * inv_nds));
            if (nonzero(c)) {
              want = true;
              // both ends of the shadow segment are moved off their surfaces toward each other
              // (Wachter and Binder), so that neither the shading point's nor the light's own
              // surface can occlude it, however grazing the direction
              V3 org = offset_origin(P, dot(ng, wo) > 0.0f ? ng : -ng);
              V3 tgt = offset_origin(lp, dot(lg, wo) < 0.0f ? lg : -lg);
              V3 sdir = tgt - org;
              const float sl = length(sdir);
              sdir = sdir * rcp(sl);
              so4 = make_float4(org.x, org.y, org.z, __uint_as_float((uint32_t)(p * a.nl_stride + k)));
              sd4 = make_float4(sdir.x, sdir.y, sdir.z, sl);
            }
          }
        }
        a.slots[p * a.nl_stride + k] = make_float4(c.x, c.y, c.z, 0.0f);
      }
      uint32_t e = warp_append(&a.counters[kCtrNee + b], want);
      if (want) {
        if (a.bin_sh) {
          a.so_u[e] = so4;
          a.sd_u[e] = sd4;
          a.skey[e] = sh_key(J, k / s2n, P);
        } else {
          a.so[e] = so4;
          a.sd[e] = sd4;
        }
      }
    }
  }
}

// shadow: any-hit query per queued light sample; an occluded sample's slot is zeroed
template <bool COUNT, int SHAPE, bool SPH = false, int BLK = kBlock>
__global__ void __launch_bounds__(BLK, (SHAPE == kShapeCoop ? kCoopMinBlocks : kTravMinBlocks) * kBlock / BLK)
    k_shadow(RenderArgs a, int b) {
  const uint32_t n = a.counters[kCtrNee + b];
  const float4 *so = a.so, *sd = a.sd;
  float4 *slots = a.slots;
  TraceCounts c = {0, 0, 0, 0};
  uint32_t rays = 0;
  const bool single = a.njobs == 1;
  const SceneView *view0 = &a.jobs[0].view;
  auto view_of = [&](uint32_t i) -> const SceneView & {
    if (single) return *view0;
    const uint32_t slot = __float_as_uint(so[i].w);
    return a.jobs[a.path_job[slot / (uint32_t)a.nl_stride]].view;
  };
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
  if (SHAPE == kShapePersist) {
    persistent_trace<true, COUNT, SPH>(view_of, nullptr, 0, n, &a.counters[kCtrFetchSh + b], load, store, &c, rays);
  } else if (SHAPE == kShapeCoop) {
    // per warp: the lanes' ray constants for the shared leaf tests
    __shared__ float4 wray[2 * BLK];
    __shared__ uint32_t wk[BLK];
    if (single)
      grid_trace_coop<true, COUNT, SPH, true>([&](uint32_t) -> const SceneView & { return a.view0; }, n, load, store,
                                              &c, rays, nullptr, wray + 2 * (threadIdx.x & ~31u),
                                              wk + (threadIdx.x & ~31u));
    else
      grid_trace_coop<true, COUNT, SPH>(view_of, n, load, store, &c, rays, nullptr, wray + 2 * (threadIdx.x & ~31u),
                                        wk + (threadIdx.x & ~31u));
  } else {
    grid_trace<true, COUNT, SPH>(view_of, nullptr, 0, n, load, store, &c, rays);
  }
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
  extern __shared__ uint32_t h[];  // kBins
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
  constexpr int kPer = 32;                 // entries per thread per chunk
  constexpr int kChunk = 256 * kPer;
  extern __shared__ uint32_t h[];  // kBins
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
// Reconstruction splat of one sample (ReconstructionRenderOutput::addSample,
// ReconstructionRenderOutput.cpp:30-83): the sample's film position is regenerated from its
// jitter (as k_generate draws it) and its radiance is added, weighted, to every pixel within the
// filter's half width whose weight is positive.  Fixed point 2^-24 makes the sums independent of
// the order of the atomic additions; non-finite or oversized contributions are dropped.
__device__ void splat(const JobArgs &J, int x, int y, int s, V3 L) {
  const int k = s % J.s2;
  const uint64_t pix = (uint64_t)y * J.W + x;
  const F4u jt = uniforms(J.rng, pix * (uint64_t)J.s2 + (uint64_t)k, kDepthJitter, 0);
  const float px = ((float)x + ((float)(k % J.side) + jt.a) / (float)J.side) / (float)J.W;
  const float py = ((float)y + ((float)(k / J.side) + jt.b) / (float)J.side) / (float)J.H;
  const float cx = px * (float)J.W, cy = py * (float)J.H;
  const int h = J.filt.half;
  const int y0 = max(0, y - h), y1 = min(J.H - 1, y + h), x0 = max(0, x - h), x1 = min(J.W - 1, x + h);
  const float scale = 16777216.0f;  // 2^24
  for (int yy = y0; yy <= y1; ++yy)
    for (int xx = x0; xx <= x1; ++xx) {
      const float w = filter_eval(J.filt, (float)xx - cx, (float)yy - cy);
      if (!(w > 0.0f)) continue;
      const float v[4] = {w * L.x * scale, w * L.y * scale, w * L.z * scale, w * scale};
      if (!(v[0] < 1e18f && v[1] < 1e18f && v[2] < 1e18f && v[3] < 1e18f)) continue;
      unsigned long long *dst = J.film_fx + 4 * ((int64_t)yy * J.W + xx);
#pragma unroll
      for (int c = 0; c < 4; ++c) atomicAdd(dst + c, (unsigned long long)llrintf(v[c]));
    }
}

__global__ void __launch_bounds__(kBlock) k_accumulate(RenderArgs a) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long ext = 0, bounces = 0, sh = 0;
    for (int b = 0; b < a.max_b; ++b) {
      uint32_t c = a.counters[kCtrRay + b];
      ext += c;
      bounces += c ? 1ull : 0ull;
      sh += a.counters[kCtrNee + b];
    }
    a.stats[0] += ext;
    a.stats[1] += sh;
    a.stats[2] += a.counters[kCtrTrunc];
    a.stats[3] += bounces;
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < a.nslots; q += stride) {
    const JobArgs &J = a.jobs[job_of_slot(a, q)];
    const int64_t lq = q - J.slot_base;
    int x, y;
    if (!slot_pixel(J, J.slot0 + lq, x, y)) continue;
    int64_t pix = (int64_t)y * J.W + x;
    float4 S = J.film_sum[pix], C = J.film_c[pix];
    for (int si = 0; si < J.ns; ++si) {
      const int64_t p = J.path_base + lq * J.ns + si;
      float4 L4 = a.path_L[p];
      V3 L = v3(L4.x, L4.y, L4.z);
      if (__float_as_uint(L4.w) & kFlagNeePending) L = fold_slots(a, J.nl_slots, p, L);
      L = apply_mask(L, __float_as_uint(L4.w));
      if (J.path_out) {
        int s = J.s0 + si - J.sample_begin;
        J.path_out[pix * J.sample_count + s] = make_float4(L.x, L.y, L.z, L4.w);
      }
      float yx = L.x - C.x, tx = S.x + yx; C.x = (tx - S.x) - yx; S.x = tx;
      float yy = L.y - C.y, ty = S.y + yy; C.y = (ty - S.y) - yy; S.y = ty;
      float yz = L.z - C.z, tz = S.z + yz; C.z = (tz - S.z) - yz; S.z = tz;
      // second moment of the per-sample luminance (variance / error estimates), unfused
      const float lum = __fmul_rn(__fadd_rn(__fadd_rn(L.x, L.y), L.z), 1.0f / 3.0f);
      C.w = __fadd_rn(C.w, __fmul_rn(lum, lum));
      if (J.film_fx) splat(J, x, y, J.s0 + si, L);
    }
    S.w += (float)J.ns;
    J.film_sum[pix] = S;
    J.film_c[pix] = C;
  }
}

// ---------------------------------------------------------------------------------------
// host driver

struct Workspace {
  int device = -1;
  int64_t cap = 0;       // paths
  int64_t slot_cap = 0;  // light-sample slots
  int64_t job_cap = 0;   // JobArgs entries
  void *block = nullptr;
  float4 *path_L = nullptr, *qo[2] = {}, *qd[2] = {}, *qt[2] = {}, *qhit = nullptr;
  float4 *so = nullptr, *sd = nullptr, *slots = nullptr;
  float4 *qo_u = nullptr, *qd_u = nullptr, *qt_u = nullptr, *so_u = nullptr, *sd_u = nullptr;
  uint32_t *qkey = nullptr, *skey = nullptr, *hist = nullptr, *cursor = nullptr;  // hist/cursor: kBins each
  uint32_t *path_job = nullptr;
  JobArgs *jobs = nullptr;
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

constexpr int kCarveoutAuto = -2;

// process-wide tuning knobs (mgpu_tune_set)
struct Tuning {
  std::atomic<int> persistent{0};     // persistent warp-level traversal with ray refill
  // grid-stride traversal with the leaf triangles shared by the warp: bit 0 for the shadow
  // (any-hit) kernel, bit 1 for the extension (closest-hit) kernel
  std::atomic<int> coop_leaf{3};
  // threads per block of the grid-stride and warp-shared traversal kernels: 64, 128 or 256 (mid
  // frame: 256 is 0.6 % faster than 128, 64 equal to 128)
  std::atomic<int> trav_block{256};
  std::atomic<int> bin_shadow{1};     // counting-sort shadow rays by (light, origin cell)
  std::atomic<int> bin_extension{1};  // counting-sort extension rays by (octant, origin cell)
  // waves of fewer paths skip binning: sorting a few hundred thousand rays costs more (four
  // latency-bound launches per bounce) than the coherence it buys
  std::atomic<int64_t> bin_min_paths{(int64_t)1 << 22};
  // shared-memory carveout (%) of the traversal / shade kernels: -2 = per kernel, the least that
  // keeps its resident blocks (the rest of the SM's 256 KB is L1); -1 = the driver's choice
  std::atomic<int> carveout{kCarveoutAuto};
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
// so, sd, slots, unsorted (so, sd) = 5 per light sample; uint32 keys per path and per sample,
// path_job per path; JobArgs entries
static size_t workspace_bytes(int64_t paths, int64_t slots, int64_t jobs) {
  size_t f4 = (size_t)paths * 11 + (size_t)slots * 5;
  size_t u32 = (size_t)paths * 2 + (size_t)slots + 2 * kBins + kNumCounters;
  return f4 * sizeof(float4) + (size_t)jobs * sizeof(JobArgs) + 12 * sizeof(unsigned long long) +
         u32 * sizeof(uint32_t) + 1024;
}

static void workspace_layout(Workspace *w, void *block, int64_t paths, int64_t slots, int64_t jobs) {
  w->cap = paths;
  w->slot_cap = slots;
  w->job_cap = jobs;
  w->block = block;
  float4 *f = (float4 *)block;
  w->path_L = f; f += paths;
  for (int k = 0; k < 2; ++k) { w->qo[k] = f; f += paths; w->qd[k] = f; f += paths; w->qt[k] = f; f += paths; }
  w->qhit = f; f += paths;
  w->qo_u = f; f += paths; w->qd_u = f; f += paths; w->qt_u = f; f += paths;
  w->so = f; f += slots; w->sd = f; f += slots; w->slots = f; f += slots;
  w->so_u = f; f += slots; w->sd_u = f; f += slots;
  w->jobs = (JobArgs *)f;  // JobArgs is a multiple of 8 bytes; float4 alignment holds
  w->stats = (unsigned long long *)(w->jobs + jobs);
  w->tcount = w->stats + 4;
  uint32_t *u = (uint32_t *)(w->tcount + 8);
  w->qkey = u; u += paths;
  w->path_job = u; u += paths;
  w->skey = u; u += slots;
  w->hist = u; u += kBins;
  w->cursor = u; u += kBins;
  w->counters = u;
}

static int ensure_workspace(int64_t paths, int64_t slots, int64_t jobs) {
  int dev = 0;
  MGPU_CUDA(cudaGetDevice(&dev));
  if (t_ws && t_ws->device == dev && t_ws->cap >= paths && t_ws->slot_cap >= slots && t_ws->job_cap >= jobs)
    return MGPU_OK;
  if (t_ws) {
    paths = std::max(paths, t_ws->cap);
    slots = std::max(slots, t_ws->slot_cap);
    jobs = std::max(jobs, t_ws->job_cap);
    cudaDeviceSynchronize();
    delete t_ws;
    t_ws = nullptr;
  }
  Workspace *w = new Workspace();
  w->device = dev;
  void *block = nullptr;
  cudaError_t e = cudaMalloc(&block, workspace_bytes(paths, slots, jobs));
  if (e != cudaSuccess) {
    delete w;
    return cuda_fail(e, "render workspace cudaMalloc");
  }
  workspace_layout(w, block, paths, slots, jobs);
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
constexpr int64_t kNoAllocJobs = 256;              // chunk descriptors kept in the scratch
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
  const size_t fixed = workspace_bytes(0, 0, kNoAllocJobs);
  const size_t per = 11 * sizeof(float4) + 2 * sizeof(uint32_t) +
                     (size_t)nl_slots * (5 * sizeof(float4) + sizeof(uint32_t));
  if (kNoAllocBytes <= fixed) return 0;
  int64_t p = (int64_t)((kNoAllocBytes - fixed) / per);
  return p / 64 * 64;
}

// Function attributes belong to a device's context: they are set on the current device before
// its first render and again after the carveout knob changes.
//   the sorting blocks: kBins counters of dynamic shared memory, above the 48 KB default;
//   the traversal and shade kernels: the L1 / shared-memory split ("carveout").  These kernels
//   chase pointers through L1 and their block needs little shared memory (none, or the shared
//   leaf tests' per-warp records); the driver's own choice for the shared-leaf shadow kernel is a
//   132 KB shared-memory configuration where 64 KB keeps all its blocks resident, and the L1 it
//   gives up makes that kernel 4 % slower on the mid frame.  The automatic carveout asks for the
//   least shared memory that keeps the kernel's register-limited number of resident blocks.
struct CarveoutKernel {
  const void *f;
  int block;
};

static std::vector<CarveoutKernel> carveout_kernels() {
  return {{(const void *)k_extend<false, kShapeGrid>, kBlock},      {(const void *)k_extend<false, kShapePersist>, kBlock},
          {(const void *)k_extend<false, kShapeCoop>, kBlock},      {(const void *)k_extend<true, kShapeGrid>, kBlock},
          {(const void *)k_extend<true, kShapePersist>, kBlock},    {(const void *)k_extend<true, kShapeCoop>, kBlock},
          {(const void *)k_extend<false, kShapeGrid, true>, kBlock}, {(const void *)k_extend<true, kShapeGrid, true>, kBlock},
          {(const void *)k_shadow<false, kShapeGrid>, kBlock},      {(const void *)k_shadow<false, kShapePersist>, kBlock},
          {(const void *)k_shadow<false, kShapeCoop>, kBlock},      {(const void *)k_shadow<true, kShapeGrid>, kBlock},
          {(const void *)k_shadow<true, kShapePersist>, kBlock},    {(const void *)k_shadow<true, kShapeCoop>, kBlock},
          {(const void *)k_shadow<false, kShapeGrid, true>, kBlock}, {(const void *)k_shadow<true, kShapeGrid, true>, kBlock},
          {(const void *)k_extend<false, kShapeGrid, false, 64>, 64},
          {(const void *)k_extend<false, kShapeGrid, false, 256>, 256},
          {(const void *)k_extend<false, kShapeCoop, false, 64>, 64},
          {(const void *)k_extend<false, kShapeCoop, false, 256>, 256},
          {(const void *)k_shadow<false, kShapeGrid, false, 64>, 64},
          {(const void *)k_shadow<false, kShapeGrid, false, 256>, 256},
          {(const void *)k_shadow<false, kShapeCoop, false, 64>, 64},
          {(const void *)k_shadow<false, kShapeCoop, false, 256>, 256},
          {(const void *)k_shade<false>, kBlock},                    {(const void *)k_shade<true>, kBlock}};
}

// percent of the SM's shared memory that holds the kernel's resident blocks (registers and
// threads permitting) with their static shared memory and the per-block reservation
static cudaError_t auto_carveout(const CarveoutKernel &k, int smem_sm, int reserved, int &pct) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k.f);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k.f, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  int blocks = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k.f, k.block, 0);
  if (e != cudaSuccess) return e;
  const int64_t need = (int64_t)blocks * (int64_t)(fa.sharedSizeBytes + (size_t)reserved);
  pct = (int)std::min<int64_t>(100, (need * 100 + smem_sm - 1) / smem_sm);
  return cudaSuccess;
}

static cudaError_t kernel_attributes() {
  static std::mutex mu;
  static std::vector<int> applied;  // per device: the carveout knob last applied, INT_MIN = none
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const int want = g_tune.carveout.load();
  std::lock_guard<std::mutex> lock(mu);
  if ((int)applied.size() <= dev) applied.resize((size_t)dev + 1, INT_MIN);
  if (applied[(size_t)dev] == want) return cudaSuccess;
  if (applied[(size_t)dev] == INT_MIN) {
    const void *bins[] = {(const void *)k_bin_hist, (const void *)k_bin_scatter<2>, (const void *)k_bin_scatter<3>};
    for (const void *kf : bins)
      if ((e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, kBinSmem)) != cudaSuccess) return e;
  }
  int smem_sm = 0, reserved = 0;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return e;
  for (const CarveoutKernel &k : carveout_kernels()) {
    int pct = want;
    if (want == kCarveoutAuto && (e = auto_carveout(k, smem_sm, reserved, pct)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k.f, cudaFuncAttributePreferredSharedMemoryCarveout, pct)) != cudaSuccess) return e;
  }
  applied[(size_t)dev] = want;
  return cudaSuccess;
}

static int grid_for(const void *kern, size_t smem, int block = kBlock) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
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
  k.aperture = c[11];
  k.focal_len = c[12];
  k.focal_dist = c[13];
  return k;
}

// A render request: one scene, parameters, film, optional per-path output.
struct Job {
  const mgpu_scene *scene;
  mgpu_render_params p;
  mgpu_film *film;
  float *path_out;
};

static int validate(const Job &j) {
  const mgpu_render_params *rp = &j.p;
  if (!j.scene || !j.film) return fail(MGPU_E_INVALID, "mgpu_render: null argument");
  if (rp->width != j.film->width || rp->height != j.film->height)
    return fail(MGPU_E_INVALID, "mgpu_render: film size differs from the render size");
  if (rp->width <= 0 || rp->height <= 0 || rp->spp <= 0 || rp->sample_count < 0 || rp->sample_begin < 0 ||
      rp->no_direct_samples <= 0 || rp->max_depth < 0 || rp->rr_start_depth < 0)
    return fail(MGPU_E_INVALID, "mgpu_render: bad parameters");
  if ((int64_t)rp->sample_begin + rp->sample_count > (int64_t)1 << 30)
    return fail(MGPU_E_INVALID, "mgpu_render: sample range too large");
  if (!(rp->camera[11] >= 0.0f) ||
      (rp->camera[11] > 0.0f && !(rp->camera[12] > 0.0f && rp->camera[13] > 0.0f)))
    return fail(MGPU_E_INVALID, "mgpu_render: a thin lens needs focal length and focal distance > 0 "
                                "(resolve autofocus before rendering)");
  int nds_side = std::max(1, (int)sqrt((double)rp->no_direct_samples));
  if ((int64_t)j.scene->nlight * nds_side * nds_side > 4096)
    return fail(MGPU_E_INVALID, "mgpu_render: too many light samples per vertex");
  return MGPU_OK;
}

// the job-level part of JobArgs
static JobArgs job_args(const Job &j) {
  const mgpu_scene *sc = j.scene;
  const mgpu_render_params *rp = &j.p;
  JobArgs J;
  memset(&J, 0, sizeof(J));
  J.view = sc->view;
  J.shade = sc->d_shade;
  J.mats = (const float4 *)sc->d_mats;
  J.lights = (const float4 *)sc->d_lights;
  J.uv = sc->d_uv;
  J.texrec = sc->d_texrec;
  J.texels = sc->d_texels;
  J.bg_tex = sc->bg_tex;
  for (int k = 0; k < 3; ++k) J.bg_le[k] = sc->bg_le[k];
  J.nlight = sc->nlight;
  J.cam = make_camera(rp->camera);
  J.rng.k0 = (uint32_t)rp->seed;
  J.rng.k1 = (uint32_t)(rp->seed >> 32);
  J.rng.stream = rp->stream_id;
  J.W = rp->width;
  J.H = rp->height;
  J.spp = rp->spp;
  J.side = std::max(1, (int)sqrt((double)rp->spp));
  J.s2 = J.side * J.side;
  J.nds = rp->no_direct_samples;
  J.nds_side = std::max(1, (int)sqrt((double)rp->no_direct_samples));
  J.nl_slots = sc->nlight * J.nds_side * J.nds_side;
  J.max_depth = rp->max_depth;
  J.rr_start = rp->rr_start_depth;
  J.efficient = rp->efficient_direct;
  J.tiles_x = (J.W + 7) / 8;
  J.sample_begin = rp->sample_begin;
  J.sample_count = rp->sample_count;
  J.film_sum = j.film->d_sum;
  J.film_c = j.film->d_c;
  J.filt = j.film->filter;
  J.film_fx = j.film->d_fx;
  J.path_out = (float4 *)j.path_out;
  int nlp = 1;
  while (nlp < std::min(sc->nlight, 16)) nlp <<= 1;
  int lb = 0;
  while ((1 << lb) < nlp) ++lb;
  J.sh_cell_bits = std::min(15, kBinBits - lb);  // light index in the top bits, origin cell below
  for (int k = 0; k < 3; ++k) {
    const float ext = J.view.bmax[k] - J.view.bmin[k];
    J.cell_scale[k] = ext > 0.0f ? 32.0f / ext : 0.0f;
  }
  return J;
}

struct Wave {
  std::vector<JobArgs> chunks;
  int64_t npaths = 0, nslots = 0;
  int32_t nl_stride = 1;
  int32_t max_b = 1;
  bool unlimited = false;  // a chunk has no depth cap: drain by reading the live count
};

// Splits every job into chunks (sample passes outer, slot ranges inner, as many passes of the
// whole image as fit a wave) and packs them into waves of at most `cap` paths.  Two chunks of
// one job that share pixels never go into the same wave (their accumulate threads would race
// on the film); chunks of one job keep their sample order across waves.
static void pack_waves(const std::vector<Job> &jobs, int64_t cap, std::vector<Wave> &waves) {
  waves.clear();
  Wave cur;
  std::vector<int> last_job_wave(jobs.size(), -1);
  auto flush = [&]() {
    if (!cur.chunks.empty()) waves.push_back(cur);
    cur = Wave();
  };
  for (size_t ji = 0; ji < jobs.size(); ++ji) {
    const Job &job = jobs[ji];
    if (job.p.sample_count == 0) continue;
    JobArgs base = job_args(job);
    const int64_t total_slots = (int64_t)base.tiles_x * ((base.H + 7) / 8) * 64;
    const int ns = (int)std::max<int64_t>(1, std::min<int64_t>(job.p.sample_count, cap / total_slots));
    const int64_t spw = std::min<int64_t>(total_slots, std::max<int64_t>(64, cap / ns) / 64 * 64);
    bool job_in_cur = false;
    for (int s0 = job.p.sample_begin; s0 < job.p.sample_begin + job.p.sample_count; s0 += ns) {
      const int nsc = std::min(ns, job.p.sample_begin + job.p.sample_count - s0);
      for (int64_t slot0 = 0; slot0 < total_slots; slot0 += spw) {
        const int64_t nsl = std::min(spw, total_slots - slot0);
        const int64_t np = nsl * nsc;
        // a new sample range of a job already in this wave would revisit its pixels
        const bool conflict = job_in_cur && slot0 == 0;
        if (cur.npaths + np > cap || conflict) {
          flush();
          job_in_cur = false;
        }
        JobArgs J = base;
        J.s0 = s0;
        J.ns = nsc;
        J.slot0 = slot0;
        J.nslots = nsl;
        J.path_base = cur.npaths;
        J.slot_base = cur.nslots;
        cur.chunks.push_back(J);
        cur.npaths += np;
        cur.nslots += nsl;
        cur.nl_stride = std::max(cur.nl_stride, std::max(1, J.nl_slots));
        if (job.p.max_depth > 0) cur.max_b = std::max(cur.max_b, std::min(job.p.max_depth, kHardCap));
        else cur.unlimited = true;
        job_in_cur = true;
      }
    }
  }
  flush();
  for (auto &w : waves)
    if (w.unlimited) w.max_b = kHardCap;
}

// Renders a list of jobs.  noalloc: use the fixed scratch instead of the cached workspace.
template <bool COUNT>
static int render_jobs(const std::vector<Job> &jobs, void *stream, bool noalloc, int64_t wave_req,
                       uint64_t *graph_launches = nullptr, bool capture = false) {
  for (const Job &j : jobs) {
    int rc = validate(j);
    if (rc != MGPU_OK) return rc;
  }
  cudaStream_t caller = as_stream(stream);
  cudaStream_t st = caller;
  int32_t nl_max = 1;
  for (const Job &j : jobs)
    nl_max = std::max(nl_max, std::max(1, job_args(j).nl_slots));
  // automatic wave: the largest power of two up to 2^26 paths whose workspace fits 40 GB (larger
  // waves mean fewer bounce tails: mid frame 226 / 236 / 241 Mpaths/s at 2^24 / 2^25 / 2^26)
  int64_t wave = wave_req;
  if (wave <= 0) {
    const double per_path = (double)workspace_bytes((int64_t)1 << 20, ((int64_t)1 << 20) * nl_max, 1) / (1 << 20);
    wave = (int64_t)1 << 26;
    while (wave > ((int64_t)1 << 20) && (double)wave * per_path > kAutoWaveBytes) wave >>= 1;
  }
  if (noalloc) {
    const int64_t pmax = noalloc_paths(nl_max);
    if (pmax < 64)
      return fail(MGPU_E_INVALID, "mgpu_render_noalloc: " + std::to_string(nl_max) +
                                      " light samples per vertex do not fit the 32 MiB fixed scratch");
    if (wave_req > pmax)
      return fail(MGPU_E_INVALID, "mgpu_render_noalloc: wave_paths " + std::to_string(wave_req) +
                                      " exceeds the fixed scratch (32 MiB holds " + std::to_string(pmax) +
                                      " paths at " + std::to_string(nl_max) + " light samples per vertex)");
    wave = wave_req > 0 ? wave_req : pmax;
  }
  std::vector<Wave> waves;
  bool use_graph = false;
  int64_t cap = 0, ncap = 0, nmax = 0, job_slots = 0;
  Workspace fixed_ws;
  Workspace *w = nullptr;
  for (;;) {
    pack_waves(jobs, wave, waves);
    if (waves.empty()) return MGPU_OK;
    bool any_unlimited = false;
    for (auto &wv : waves) any_unlimited |= wv.unlimited;
    use_graph = capture && !any_unlimited && !noalloc;
    // chunk descriptors: all of them up front when the launches are captured in a graph (no
    // host copies inside a capture), else each wave's own before its launches
    cap = ncap = nmax = 0;
    for (auto &wv : waves) {
      cap = std::max(cap, wv.npaths);
      ncap += (int64_t)wv.chunks.size();
      nmax = std::max(nmax, (int64_t)wv.chunks.size());
    }
    job_slots = use_graph ? ncap : nmax;
    if (noalloc) {
      if (job_slots > kNoAllocJobs)
        return fail(MGPU_E_INVALID, "mgpu_render_noalloc: more than " + std::to_string(kNoAllocJobs) +
                                        " chunks in one wave");
      void *base = nullptr;
      int rc = noalloc_scratch(&base);
      if (rc != MGPU_OK) return rc;
      fixed_ws.owned = false;
      MGPU_CUDA(cudaGetDevice(&fixed_ws.device));
      workspace_layout(&fixed_ws, base, cap, std::max<int64_t>(1, cap * nl_max), kNoAllocJobs);
      fixed_ws.h_counters = g_noalloc_host_counter;
      w = &fixed_ws;
      break;
    }
    int rc = ensure_workspace(cap, std::max<int64_t>(1, cap * nl_max), job_slots);
    if (rc == MGPU_E_NOMEM && wave_req <= 0 && wave > ((int64_t)1 << 20)) {
      cudaGetLastError();  // clear the failed allocation
      wave >>= 1;          // an automatic wave that does not fit the free memory: halve it
      continue;
    }
    if (rc != MGPU_OK) return rc;
    w = t_ws;
    break;
  }
  // (a copy from pageable memory returns once the runtime has staged the source)
  if (use_graph) {
    std::vector<JobArgs> all;
    all.reserve((size_t)ncap);
    for (auto &wv : waves) all.insert(all.end(), wv.chunks.begin(), wv.chunks.end());
    MGPU_CUDA(cudaMemcpyAsync(w->jobs, all.data(), all.size() * sizeof(JobArgs), cudaMemcpyHostToDevice, st));
  }

  const bool persist = g_tune.persistent.load() != 0;
  const bool coop_sh = (g_tune.coop_leaf.load() & 1) != 0, coop_ext = (g_tune.coop_leaf.load() & 2) != 0;
  bool sph = false;  // a job's scene has analytic spheres: the traversal kernels that test them
  for (const Job &j : jobs) sph = sph || j.scene->view.nsphere > 0;
  // threads per traversal block: 128 for the persistent, sphere and counted kernels; the
  // grid-stride and warp-shared shapes of the plain render also come in 64 and 256
  const int tb = (sph || persist || COUNT) ? kBlock : g_tune.trav_block.load();
  auto kext = sph        ? k_extend<COUNT, kShapeGrid, true>
              : persist  ? k_extend<COUNT, kShapePersist>
              : coop_ext ? (tb == 64 ? k_extend<COUNT, kShapeCoop, false, 64>
                            : tb == 256 ? k_extend<COUNT, kShapeCoop, false, 256> : k_extend<COUNT, kShapeCoop>)
                         : (tb == 64 ? k_extend<COUNT, kShapeGrid, false, 64>
                            : tb == 256 ? k_extend<COUNT, kShapeGrid, false, 256> : k_extend<COUNT, kShapeGrid>);
  auto kshw = sph        ? k_shadow<COUNT, kShapeGrid, true>
              : persist  ? k_shadow<COUNT, kShapePersist>
              : coop_sh  ? (tb == 64 ? k_shadow<COUNT, kShapeCoop, false, 64>
                            : tb == 256 ? k_shadow<COUNT, kShapeCoop, false, 256> : k_shadow<COUNT, kShapeCoop>)
                         : (tb == 64 ? k_shadow<COUNT, kShapeGrid, false, 64>
                            : tb == 256 ? k_shadow<COUNT, kShapeGrid, false, 256> : k_shadow<COUNT, kShapeGrid>);
  const int tb_ext = (sph || persist || COUNT) ? kBlock : tb, tb_sh = tb_ext;
  MGPU_CUDA(kernel_attributes());
  const int g_gen = grid_for((const void *)k_generate, 0);
  const int g_ext = grid_for((const void *)kext, 0, tb_ext);
  const int g_sha = grid_for((const void *)k_shade<true>, 0);
  const int g_shw = grid_for((const void *)kshw, 0, tb_sh);
  const int g_acc = grid_for((const void *)k_accumulate, 0);
  const int g_bin = device_sm_count() * 4;
  const int bin_ext = g_tune.bin_extension.load(), bin_sh = g_tune.bin_shadow.load();
  const int64_t bin_min = g_tune.bin_min_paths.load();

  // The launches are captured on a private stream (the caller's may be the legacy default
  // stream, which cannot capture) and the graph is launched on the caller's stream.
  cudaGraph_t graph = nullptr;
  if (use_graph) {
    static thread_local cudaStream_t t_capture = nullptr;
    if (!t_capture) MGPU_CUDA(cudaStreamCreateWithFlags(&t_capture, cudaStreamNonBlocking));
    st = t_capture;
    MGPU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  }

  mgpu_render_stats stats{};
  uint64_t launches = 0;
  Profiler off;  // the allocation-free and graph paths record no events
  Profiler &pf = (noalloc || use_graph) ? off : t_prof;
  cudaError_t err = cudaMemsetAsync(w->stats, 0, 12 * sizeof(unsigned long long), st);
  size_t job_off = 0;
  for (size_t wi = 0; wi < waves.size() && err == cudaSuccess; ++wi) {
    const Wave &wv = waves[wi];
    RenderArgs a;
    memset(&a, 0, sizeof(a));
    if (use_graph) {
      a.jobs = w->jobs + job_off;
      job_off += wv.chunks.size();
    } else {
      a.jobs = w->jobs;
      err = cudaMemcpyAsync(w->jobs, wv.chunks.data(), wv.chunks.size() * sizeof(JobArgs), cudaMemcpyHostToDevice, st);
      if (err != cudaSuccess) break;
    }
    a.njobs = (int32_t)wv.chunks.size();
    a.view0 = wv.chunks[0].view;
    a.npaths = wv.npaths;
    a.nslots = wv.nslots;
    a.nl_stride = wv.nl_stride;
    a.path_job = w->path_job;
    a.path_L = w->path_L;
    for (int k = 0; k < 2; ++k) { a.qo[k] = w->qo[k]; a.qd[k] = w->qd[k]; a.qt[k] = w->qt[k]; }
    a.qhit = w->qhit;
    a.so = w->so; a.sd = w->sd; a.slots = w->slots;
    a.qo_u = w->qo_u; a.qd_u = w->qd_u; a.qt_u = w->qt_u; a.so_u = w->so_u; a.sd_u = w->sd_u;
    a.qkey = w->qkey; a.skey = w->skey;
    a.bin_ext = wv.npaths >= bin_min ? bin_ext : 0;
    a.bin_sh = wv.npaths >= bin_min ? bin_sh : 0;
    a.counters = w->counters;
    a.stats = w->stats;
    a.tcount = w->tcount;
    a.max_b = wv.max_b;
    const int max_b = wv.max_b;
    bool surf = false;  // a chunk's scene has image maps, a background or analytic spheres
    for (const JobArgs &c : wv.chunks)
      surf = surf || c.texrec != nullptr || c.bg_tex != 0 || c.bg_le[0] != 0.0f || c.bg_le[1] != 0.0f ||
             c.bg_le[2] != 0.0f || c.view.nsphere > 0;
    err = cudaMemsetAsync(w->counters, 0, kNumCounters * sizeof(uint32_t), st);
    int m = pf.begin(kProfGenerate, st);
    k_generate<<<g_gen, kBlock, 0, st>>>(a);
    pf.end(m, st);
    ++launches;
    int b = 0;
    while (b < max_b && err == cudaSuccess) {
      // with a fixed depth cap every bounce is launched blind; without one, check the live
      // count every 4 bounces and stop when the wave has drained
      int chunk = wv.unlimited ? std::min(4, max_b - b) : max_b;
      for (int k = 0; k < chunk; ++k, ++b) {
        m = pf.begin(kProfExtend, st);
        kext<<<g_ext, tb_ext, 0, st>>>(a, b);
        pf.end(m, st);
        m = pf.begin(kProfShade, st);
        if (surf) k_shade<true><<<g_sha, kBlock, 0, st>>>(a, b);
        else k_shade<false><<<g_sha, kBlock, 0, st>>>(a, b);
        pf.end(m, st);
        if (a.bin_sh || a.bin_ext) {
          m = pf.begin(kProfBin, st);
          if (a.bin_sh) {
            cudaMemsetAsync(w->hist, 0, kBins * sizeof(uint32_t), st);
            k_bin_hist<<<g_bin, 256, kBinSmem, st>>>(w->skey, a.counters + kCtrNee + b, w->hist);
            k_bin_scan<<<1, 1024, 0, st>>>(w->hist, w->cursor);
            k_bin_scatter<2><<<g_bin, 256, kBinSmem, st>>>(w->skey, a.counters + kCtrNee + b, w->cursor, w->so_u, w->sd_u,
                                                    nullptr, w->so, w->sd, nullptr);
            launches += 3;
          }
          if (a.bin_ext && b + 1 < max_b) {
            const int nx = (b + 1) & 1;
            cudaMemsetAsync(w->hist, 0, kBins * sizeof(uint32_t), st);
            k_bin_hist<<<g_bin, 256, kBinSmem, st>>>(w->qkey, a.counters + kCtrRay + b + 1, w->hist);
            k_bin_scan<<<1, 1024, 0, st>>>(w->hist, w->cursor);
            k_bin_scatter<3><<<g_bin, 256, kBinSmem, st>>>(w->qkey, a.counters + kCtrRay + b + 1, w->cursor, w->qo_u,
                                                    w->qd_u, w->qt_u, w->qo[nx], w->qd[nx], w->qt[nx]);
            launches += 3;
          }
          pf.end(m, st);
        }
        m = pf.begin(kProfShadow, st);
        kshw<<<g_shw, tb_sh, 0, st>>>(a, b);
        pf.end(m, st);
        launches += 3;
      }
      if (!wv.unlimited) break;
      err = cudaMemcpyAsync(w->h_counters, w->counters + kCtrRay + b, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
      if (err == cudaSuccess) err = cudaStreamSynchronize(st);
      if (err != cudaSuccess || w->h_counters[0] == 0) break;
    }
    m = pf.begin(kProfAccumulate, st);
    k_accumulate<<<g_acc, kBlock, 0, st>>>(a);
    pf.end(m, st);
    ++launches;
    if (err == cudaSuccess) err = cudaGetLastError();
  }
  if (use_graph) {
    cudaError_t ec = cudaStreamEndCapture(st, &graph);
    if (err == cudaSuccess) err = ec;
    if (err == cudaSuccess) {
      cudaGraphExec_t exec = nullptr;
      err = cudaGraphInstantiate(&exec, graph, 0);
      if (err == cudaSuccess) err = cudaGraphLaunch(exec, caller);
      if (exec) cudaGraphExecDestroy(exec);
    }
    if (graph) cudaGraphDestroy(graph);
    if (graph_launches) *graph_launches += 1;
  }
  if (err != cudaSuccess) return cuda_fail(err, "render");
  g_launches.fetch_add(launches);
  stats.paths = 0;
  for (const Job &j : jobs) stats.paths += (uint64_t)j.p.width * j.p.height * (uint64_t)j.p.sample_count;
  stats.kernel_launches = launches;
  t_stats = stats;
  t_stats_stream = caller;
  t_stats_dev = w->stats;
  t_counters_dev = w->counters;
  t_stats_pending = true;
  return MGPU_OK;
}

template <bool COUNT>
static int render_one(const mgpu_scene *sc, const mgpu_render_params *rp, mgpu_film *film, float *d_path_out,
                      void *stream, bool noalloc = false) {
  if (!sc || !rp || !film) return fail(MGPU_E_INVALID, "mgpu_render: null argument");
  std::vector<Job> jobs(1);
  jobs[0].scene = sc;
  jobs[0].p = *rp;
  jobs[0].film = film;
  jobs[0].path_out = d_path_out;
  if (rp->sample_count == 0) return validate(jobs[0]);
  return render_jobs<COUNT>(jobs, stream, noalloc, rp->wave_paths);
}

}  // namespace mgpu

// A batch: render requests that share waves (mgpu_batch_*).
struct mgpu_batch {
  std::vector<mgpu::Job> jobs;
  int64_t wave_paths = 0;
  int use_graph = 1;
  uint64_t graph_launches = 0;
};

using namespace mgpu;

extern "C" {

int mgpu_render(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, void *stream) {
  return render_one<false>(scene, params, film, nullptr, stream);
}

int mgpu_render_paths(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, float *d_path_L,
                      void *stream) {
  if (!d_path_L) return fail(MGPU_E_INVALID, "mgpu_render_paths: null path buffer");
  return render_one<false>(scene, params, film, d_path_L, stream);
}

// Allocation-free render: the same estimator and film as mgpu_render, over the fixed 32 MiB
// scratch instead of a cudaMalloc'd workspace.  See include/mgpu.h for the contract.
int mgpu_render_noalloc(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film, void *stream) {
  return render_one<false>(scene, params, film, nullptr, stream, true);
}

int mgpu_render_counted(const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film,
                        uint64_t *counts8, void *stream) {
  if (!counts8) return fail(MGPU_E_INVALID, "mgpu_render_counted: null output");
  int rc = render_one<true>(scene, params, film, nullptr, stream);
  if (rc != MGPU_OK) return rc;
  MGPU_CUDA(cudaStreamSynchronize(as_stream(stream)));
  MGPU_CUDA(cudaMemcpy(counts8, t_ws->tcount, 8 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return MGPU_OK;
}

int mgpu_batch_create(mgpu_batch **out) {
  if (!out) return fail(MGPU_E_INVALID, "mgpu_batch_create: null argument");
  *out = new (std::nothrow) mgpu_batch();
  if (!*out) return fail(MGPU_E_NOMEM, "mgpu_batch_create: out of host memory");
  return MGPU_OK;
}

int mgpu_batch_add(mgpu_batch *b, const mgpu_scene *scene, const mgpu_render_params *params, mgpu_film *film) {
  if (!b || !scene || !params || !film) return fail(MGPU_E_INVALID, "mgpu_batch_add: null argument");
  Job j;
  j.scene = scene;
  j.p = *params;
  j.film = film;
  j.path_out = nullptr;
  int rc = validate(j);
  if (rc != MGPU_OK) return rc;
  b->jobs.push_back(j);
  return MGPU_OK;
}

int mgpu_batch_set(mgpu_batch *b, int64_t wave_paths, int32_t use_graph) {
  if (!b || wave_paths < 0 || wave_paths > INT32_MAX) return fail(MGPU_E_INVALID, "mgpu_batch_set: bad argument");
  b->wave_paths = wave_paths;
  b->use_graph = use_graph;
  return MGPU_OK;
}

int mgpu_batch_render(mgpu_batch *b, void *stream) {
  if (!b) return fail(MGPU_E_INVALID, "mgpu_batch_render: null batch");
  if (b->jobs.empty()) return MGPU_OK;
  return render_jobs<false>(b->jobs, stream, false, b->wave_paths, &b->graph_launches, b->use_graph != 0);
}

int mgpu_batch_clear(mgpu_batch *b) {
  if (!b) return fail(MGPU_E_INVALID, "mgpu_batch_clear: null batch");
  b->jobs.clear();
  return MGPU_OK;
}

int mgpu_batch_destroy(mgpu_batch *b) {
  delete b;
  return MGPU_OK;
}

int mgpu_render_wave_queues(uint32_t *ext, uint32_t *shadow, int32_t max_bounces) {
  if (!ext || !shadow || max_bounces <= 0) return fail(MGPU_E_INVALID, "mgpu_render_wave_queues: bad argument");
  if (!t_counters_dev) return fail(MGPU_E_STATE, "mgpu_render_wave_queues: nothing rendered on this thread");
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
  else if (k == "coop_leaf" && value >= 0 && value <= 3) g_tune.coop_leaf.store((int)value);
  else if (k == "trav_block" && (value == 64 || value == 128 || value == 256)) g_tune.trav_block.store((int)value);
  else if (k == "bin_shadow") g_tune.bin_shadow.store(value != 0);
  else if (k == "bin_extension") g_tune.bin_extension.store(value != 0);
  else if (k == "bin_min_paths" && value >= 0) g_tune.bin_min_paths.store(value);
  else if (k == "carveout" && value >= kCarveoutAuto && value <= 100) {
    // applied per device before its next render (kernel_attributes)
    g_tune.carveout.store((int)value);
  } else return fail(MGPU_E_INVALID, "mgpu_tune_set: unknown key or bad value " + k);
  return MGPU_OK;
}

int mgpu_tune_get(const char *key, int64_t *value) {
  if (!key || !value) return fail(MGPU_E_INVALID, "mgpu_tune_get: null argument");
  std::string k(key);
  if (k == "persistent") *value = g_tune.persistent.load();
  else if (k == "coop_leaf") *value = g_tune.coop_leaf.load();
  else if (k == "trav_block") *value = g_tune.trav_block.load();
  else if (k == "bin_shadow") *value = g_tune.bin_shadow.load();
  else if (k == "bin_extension") *value = g_tune.bin_extension.load();
  else if (k == "bin_min_paths") *value = g_tune.bin_min_paths.load();
  else if (k == "carveout") *value = g_tune.carveout.load();
  else return fail(MGPU_E_INVALID, "mgpu_tune_get: unknown key " + k);
  return MGPU_OK;
}

}  // extern "C"
