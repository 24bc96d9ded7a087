// hd_trace.h -- kd-tree traversal and watertight FP32 ray/triangle tests (host/device).
//
// Layout in device memory (built by kdbuild.cpp):
//   pairs  uint4[npairs]   one 16-byte record = the two children of an interior node, fetched
//                          with a single 128-bit load; pair 0 holds the root (slot 0) and an
//                          unused slot.  Each 8-byte slot is {w0, w1}:
//                            interior: w0 = child_pair << 2 | axis (0..2), w1 = split (float bits)
//                            leaf:     w0 = count << 2 | 3, w1 = first ref (count > 1) or the
//                                      triangle itself (count == 1)
//   ltris  float4[3*nref]  leaf triangle records in leaf order, so a leaf's triangles are one
//                          contiguous run read without an index indirection: (v0, prim id),
//                          (v1, flags), (v2, 0).  Each leaf's run is in reverse of Milton's list
//                          order, so a forward scan visits primitives in the order kdTreeAccel's
//                          `for (i = n; i--;)` loop does (kdTreeAccel.cpp:973-996).  On the device
//                          a leaf slot's w1 is the index of its first record.
//   tris   float4[3*ntri]  v0, v1, v2 by primitive id (read by shading, not by traversal).
//
// The traversal follows kdTreeAccel::getIntersection / intersects (kdTreeAccel.cpp:893-1094):
// root slab clip, near/far ordering by the sign of (split - origin) and the direction, a stack
// of (far node, tmax), early exit once the best hit lies inside the current cell.  Two things
// differ on purpose: the best hit is kept across leaves (not reset per cell), and the cell
// interval is widened by a relative epsilon instead of Milton's absolute 1e-7, both because
// the arithmetic is FP32.
#pragma once

#include "hd_math.h"

#if !defined(__CUDACC__)
#include <math.h>
#endif

namespace mgpu {

constexpr int kMaxStack = 64;      // >= the deepest tree the builder will emit
constexpr uint32_t kLeafTag = 3u;

struct F4 {
  float x, y, z, w;
};

struct Pair {
  uint32_t a0, a1, b0, b1;
};

struct SceneView {
  const Pair *pairs;
  const F4 *ltris;         // 3 per leaf triangle record, leaf order
  const F4 *tris;          // 3 per triangle, by primitive id
  float bmin[3], bmax[3];  // root bounds
  int64_t ntri;
  uint64_t npairs, nrefs;
  const F4 *spheres;       // 2 per analytic sphere: (center, radius), world-to-object quaternion
  int32_t nsphere;         // spheres are primitives ntri .. ntri + nsphere - 1
};

struct Ray {
  V3 o;
  float tmin;
  V3 d;
  float tmax;
};

struct Hit {
  float t;
  int32_t prim;
  float b1, b2;  // barycentric weights of v1 and v2
};

struct TraceCounts {
  uint32_t nodes, refs, tris, max_stack;
};

MGPU_HD float fabs_(float x) { return fabsf(x); }

// Watertight ray/triangle intersection: Woop, Benthin, Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1), 2013.  Per-ray shear constants are precomputed in RayPre.
struct RayPre {
  int kx, ky, kz;
  float sx, sy, sz;
  V3 o;
};

MGPU_HD RayPre precompute(const Ray &r) {
  RayPre p;
  float ax = fabsf(r.d.x), ay = fabsf(r.d.y), az = fabsf(r.d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  float dz = comp(r.d, kz);
  if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }
  p.kx = kx; p.ky = ky; p.kz = kz;
  p.sx = comp(r.d, kx) / dz;
  p.sy = comp(r.d, ky) / dz;
  p.sz = 1.0f / dz;
  p.o = r.o;
  return p;
}

// Rounded product / difference that the device compiler may not fuse (host code is built with
// -ffp-contract=off).
MGPU_HD float mul_nc(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
MGPU_HD float sub_nc(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}

// Tests one triangle.  On a hit with tmin < t < tbest returns true and fills t, b1, b2.
// culled: accept only rays arriving on the side that (v1-v0) x (v2-v0) faces, like Milton's
// back-face culled `Triangle` (det = e1 . (d x e2) > 0 in Triangle.cpp:245-248).
MGPU_HD bool intersect_tri(const RayPre &p, V3 v0, V3 v1, V3 v2, bool culled, float tmin, float tbest, float &t_out,
                           float &b1_out, float &b2_out) {
  V3 A = v0 - p.o, B = v1 - p.o, C = v2 - p.o;
  float Akz = comp(A, p.kz), Bkz = comp(B, p.kz), Ckz = comp(C, p.kz);
  float Ax = comp(A, p.kx) - p.sx * Akz, Ay = comp(A, p.ky) - p.sy * Akz;
  float Bx = comp(B, p.kx) - p.sx * Bkz, By = comp(B, p.ky) - p.sy * Bkz;
  float Cx = comp(C, p.kx) - p.sx * Ckz, Cy = comp(C, p.ky) - p.sy * Ckz;
  // The edge functions must round the same way in the two triangles that share an edge (there
  // they are exact negatives): products and difference without contraction into an FMA, which
  // rounds a * b - c * d and d * c - b * a differently and lets rays through shared edges.
  float U = sub_nc(mul_nc(Cx, By), mul_nc(Cy, Bx));
  float Vv = sub_nc(mul_nc(Ax, Cy), mul_nc(Ay, Cx));
  float W = sub_nc(mul_nc(Bx, Ay), mul_nc(By, Ax));
  if (U == 0.0f || Vv == 0.0f || W == 0.0f) {
    // edge case: redo the 2D cross products in double so that shared edges stay watertight
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    Vv = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  bool anyneg = (U < 0.0f || Vv < 0.0f || W < 0.0f);
  bool anypos = (U > 0.0f || Vv > 0.0f || W > 0.0f);
  if (anyneg && anypos) return false;
  float det = U + Vv + W;
  if (det == 0.0f) return false;
  // orientation: with this permutation det > 0 <=> the ray arrives on the side that
  // (v1-v0) x (v2-v0) faces, i.e. Milton's det = e1 . (d x e2) > 0
  if (culled && det < 0.0f) return false;
  float Az = p.sz * Akz, Bz = p.sz * Bkz, Cz = p.sz * Ckz;
  float T = U * Az + Vv * Bz + W * Cz;
  // range test before dividing: t = T / det in (tmin, tbest) <=> T' in (tmin det', tbest det')
  // with det' = |det| and T' = T sign(det)
  float adet = fabsf(det);
  float sT = det < 0.0f ? -T : T;
  if (!(sT > tmin * adet && sT < tbest * adet)) return false;
#if defined(__CUDA_ARCH__)
  float rcp = __frcp_rn(det);
#else
  float rcp = 1.0f / det;
#endif
  t_out = T * rcp;
  b1_out = Vv * rcp;
  b2_out = W * rcp;
  return true;
}

// Node fetch: device code reads through the read-only path; a shared-memory copy of the top
// pairs can be supplied by the kernel (top != nullptr, ntop pairs).
MGPU_HD Pair load_pair(const SceneView &s, const Pair *top, uint32_t ntop, uint32_t idx) {
  if (top != nullptr && idx < ntop) return top[idx];
#if defined(__CUDA_ARCH__)
  uint4 q = __ldg(reinterpret_cast<const uint4 *>(s.pairs) + idx);
  Pair r; r.a0 = q.x; r.a1 = q.y; r.b0 = q.z; r.b1 = q.w;
  return r;
#else
  return s.pairs[idx];
#endif
}

MGPU_HD F4 load_f4(const F4 *p, int64_t i) {
#if defined(__CUDA_ARCH__)
  float4 q = __ldg(reinterpret_cast<const float4 *>(p) + i);
  F4 r; r.x = q.x; r.y = q.y; r.z = q.z; r.w = q.w;
  return r;
#else
  return p[i];
#endif
}

MGPU_HD uint32_t load_u32(const uint32_t *p, uint64_t i) {
#if defined(__CUDA_ARCH__)
  return __ldg(p + i);
#else
  return p[i];
#endif
}

// root slab clip, AABB.inl:25-56
MGPU_HD bool clip_root(const SceneView &s, const Ray &r, V3 inv, float &t0, float &t1) {
  float lo = -INFINITY, hi = INFINITY;
  const float o[3] = {r.o.x, r.o.y, r.o.z};
  const float iv[3] = {inv.x, inv.y, inv.z};
  for (int k = 0; k < 3; ++k) {
    float a = (s.bmin[k] - o[k]) * iv[k];
    float b = (s.bmax[k] - o[k]) * iv[k];
    float n = fminf(a, b), f = fmaxf(a, b);
    if (a != a || b != b) {  // 0 * inf: origin on a slab plane with d parallel to it
      n = -INFINITY; f = INFINITY;
      if (o[k] < s.bmin[k] || o[k] > s.bmax[k]) return false;
    }
    lo = fmaxf(lo, n);
    hi = fminf(hi, f);
  }
  t0 = lo; t1 = hi;
  return lo <= hi;
}

constexpr float kCellEps = 1.0f / 262144.0f;  // relative widening of cell intervals (2^-18)

// Resumable traversal state: one call of trav_step descends to the next leaf, tests it and
// either finishes or pops the next cell.  The scalar state stays in registers; the far-child
// stack is a separate array (local memory, kMaxStack >= the deepest tree the builder emits).
constexpr uint32_t kMaxLeafSteps = 1u << 20;  // guard: a ray that takes more leaf steps is abandoned

struct TravEntry {
  uint32_t w0, w1;
  float tmax;
};

// The far-cell stack (the thread's local memory).  sp is the entry's index: push writes entry sp,
// pop reads entry sp (the caller has decremented it).
MGPU_HD void stk_push(TravEntry *e, int sp, uint32_t w0, uint32_t w1, float tmax) {
  e[sp].w0 = w0; e[sp].w1 = w1; e[sp].tmax = tmax;
}
MGPU_HD void stk_pop(TravEntry *e, int sp, uint32_t &w0, uint32_t &w1, float &tmax) {
  w0 = e[sp].w0; w1 = e[sp].w1; tmax = e[sp].tmax;
}

struct TravState {
  RayPre pre;
  V3 inv;
  float tmin, tmax;   // current cell interval
  float ray_tmin;
  float best;         // closest accepted t so far (starts at the ray's tmax)
  int32_t best_prim;
  float bb1, bb2;
  uint32_t w0, w1;    // current node slot
  uint32_t steps;
  int sp;
};

MGPU_HD float safe_rcp(float d) {
  const float tiny = 1e-30f;
  if (d == 0.0f) d = f_bits(d) ? -tiny : tiny;  // keeps the sign of -0
  return 1.0f / d;
}

// Ray-sphere test (Sphere::getIntersection, Sphere.cpp:17-48), FP32 with the roots taken as
// c / q and q / a (q = b' + sign(b') sqrt(a disc)) and the discriminant from the closest approach
// f = oc - (oc.d / a) d, which avoid the cancellations of the textbook formula (Haines et al.,
// "Precision Improvements for Ray/Sphere Intersection", Ray Tracing Gems ch. 7): the smallest
// root in (tmin, tbest) in t; false when there is none.
MGPU_HD bool sphere_t(V3 o, V3 d, V3 c, float rad, float tmin, float tbest, float &t) {
  const V3 oc = o - c;
  const float a = dot(d, d);
  const float bp = -dot(oc, d);
  const V3 f = oc + d * (bp / a);
  const float disc = rad * rad - dot(f, f);
  if (!(disc >= 0.0f)) return false;
  const float h = sqrtf(a * disc);
  const float q = bp + (bp >= 0.0f ? h : -h);
  const float cc = dot(oc, oc) - rad * rad;
  float t0 = q != 0.0f ? cc / q : 0.0f, t1 = q / a;
  if (t0 > t1) { const float x = t0; t0 = t1; t1 = x; }
  if (t0 > tmin && t0 < tbest) { t = t0; return true; }
  if (t1 > tmin && t1 < tbest) { t = t1; return true; }
  return false;
}

// Closest (or, with any, first) sphere hit in (r.tmin, st.best): updates st.best / best_prim.
#if defined(__CUDA_ARCH__)
__device__ __noinline__
#else
inline
#endif
void spheres_hit(const SceneView &s, const Ray &r, TravState &st, bool any) {
  for (int i = 0; i < s.nsphere; ++i) {
#if defined(__CUDA_ARCH__)
    const float4 q = __ldg(reinterpret_cast<const float4 *>(s.spheres) + 2 * i);
#else
    const F4 q = s.spheres[2 * i];
#endif
    float t;
    if (sphere_t(r.o, r.d, v3(q.x, q.y, q.z), q.w, r.tmin, st.best, t)) {
      st.best = t;
      st.best_prim = (int32_t)(s.ntri + i);
      st.bb1 = st.bb2 = 0.0f;
      if (any) return;
    }
  }
}

// returns false when no traversal step is needed: the ray misses the tree, or (any) a sphere
// already occludes it; st.best_prim then holds the sphere hit, if any.  SPH: the scene may have
// analytic spheres (kernels for scenes without them carry no sphere code).
template <bool SPH = false>
MGPU_HD bool trav_init(const SceneView &s, const Ray &r, const Pair *top, uint32_t ntop, TravState &st,
                       bool any = false) {
  st.best = r.tmax;
  st.best_prim = -1;
  st.bb1 = st.bb2 = 0.0f;
  if (SPH && s.nsphere > 0) {
    spheres_hit(s, r, st, any);
    if (any && st.best_prim >= 0) return false;
  }
  if (s.ntri <= 0) return false;
  {
    V3 inv = v3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
    float t0, t1;
    if (!clip_root(s, r, inv, t0, t1)) return false;
    st.tmin = fmaxf(t0, r.tmin);
    st.tmax = fminf(t1, r.tmax);
  }
  // reciprocal direction for the split planes: a zero component becomes a huge finite value of
  // the same sign, so a ray parallel to a plane gets dt = +-huge (only the side holding its
  // origin) without a special case per node.  Milton's traversal instead evaluates 0 * inf and,
  // for a +0 component, can descend into the wrong child (kdTreeAccel.cpp:933-960).
  st.inv = v3(safe_rcp(r.d.x), safe_rcp(r.d.y), safe_rcp(r.d.z));
  float t0 = st.tmin, t1 = st.tmax;
  (void)t0;
  (void)t1;
  if (st.tmin > st.tmax) return false;
  st.ray_tmin = r.tmin;
  st.pre = precompute(r);
  st.sp = 0;
  st.steps = 0;
  Pair root = load_pair(s, top, ntop, 0);
  st.w0 = root.a0;
  st.w1 = root.a1;
  return true;
}

// Descends from the current node to the next leaf: returns the leaf slot (w0: count << 2 | 3,
// w1: first leaf record) and the exit t of its cell in tmax_out; far children go on the stack.
template <bool COUNT, class Stk>
MGPU_HD void trav_descend(const SceneView &s, TravState &st, Stk stack, const Pair *top, uint32_t ntop,
                          TraceCounts *cnt, uint32_t &leaf_w0, uint32_t &leaf_w1, float &tmax_out) {
  const float o[3] = {st.pre.o.x, st.pre.o.y, st.pre.o.z};
  const float iv[3] = {st.inv.x, st.inv.y, st.inv.z};
  uint32_t w0 = st.w0, w1 = st.w1;
  float tmin = st.tmin, tmax = st.tmax;
  while ((w0 & 3u) != kLeafTag) {
    if (COUNT) cnt->nodes++;
    int ax = (int)(w0 & 3u);
    float split = bits_f(w1);
    float diff = split - o[ax];
    float dinv = iv[ax];
    Pair pr = load_pair(s, top, ntop, w0 >> 2);
    uint32_t n0, n1;
    bool both;
    const float dt = diff * dinv;
    // near child = the side of the origin (Milton's ordering by the signs of diff and d)
    const bool rev = diff <= 0.0f ? (dinv <= 0.0f) : (dinv < 0.0f);
    const float slack = kCellEps * tmax;  // cells lie at t >= 0, so tmax bounds |t| in the cell
    if (dt > tmax + slack) {              // far child not reached inside this cell
      n0 = rev ? pr.b0 : pr.a0; n1 = rev ? pr.b1 : pr.a1; both = false;
    } else if (dt < tmin - slack) {       // near child lies behind the cell
      n0 = rev ? pr.a0 : pr.b0; n1 = rev ? pr.a1 : pr.b1; both = false;
    } else {
      n0 = rev ? pr.b0 : pr.a0; n1 = rev ? pr.b1 : pr.a1; both = true;
    }
    if (both) {
      // near child first, far child on the stack
      if (st.sp < kMaxStack) {
        uint32_t f0 = (n0 == pr.a0 && n1 == pr.a1) ? pr.b0 : pr.a0;
        uint32_t f1 = (n0 == pr.a0 && n1 == pr.a1) ? pr.b1 : pr.a1;
        stk_push(stack, st.sp, f0, f1, tmax);
        ++st.sp;
        if (COUNT && (uint32_t)st.sp > cnt->max_stack) cnt->max_stack = (uint32_t)st.sp;
      }
      tmax = fminf(tmax, dt);
    }
    w0 = n0; w1 = n1;
  }
  if (COUNT) cnt->nodes++;
  leaf_w0 = w0;
  leaf_w1 = w1;
  tmax_out = tmax;
}

// After a leaf has been tested: finish (true) or move to the next cell on the stack (false).
template <bool ANY, class Stk>
MGPU_HD bool trav_after_leaf(TravState &st, Stk stack, float tmax) {
  // early exit: the best hit lies inside this cell, later cells are farther
  if (!ANY && st.best_prim >= 0 && st.best <= tmax + kCellEps * fabsf(tmax)) return true;
  if (st.sp == 0 || ++st.steps >= kMaxLeafSteps) return true;
  --st.sp;
  st.tmin = tmax;
  stk_pop(stack, st.sp, st.w0, st.w1, st.tmax);
  if (!ANY && st.best_prim >= 0 && st.best < st.tmin) return true;
  return false;
}

// One leaf: descend, test, then finish (true) or move to the next cell (false).
template <bool ANY, bool COUNT, class Stk>
MGPU_HD bool trav_step(const SceneView &s, TravState &st, Stk stack, const Pair *top, uint32_t ntop,
                       TraceCounts *cnt) {
  uint32_t w0, w1;
  float tmax;
  trav_descend<COUNT>(s, st, stack, top, ntop, cnt, w0, w1, tmax);
  const uint32_t count = w0 >> 2;
  for (uint32_t i = 0; i < count; ++i) {
    if (COUNT) cnt->tris++;
    const int64_t r = 3 * ((int64_t)w1 + i);
    F4 a = load_f4(s.ltris, r + 0);
    F4 b = load_f4(s.ltris, r + 1);
    F4 c = load_f4(s.ltris, r + 2);
    bool culled = (f_bits(b.w) & 1u) != 0u;
    float t, b1, b2;
    if (intersect_tri(st.pre, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), culled, st.ray_tmin, st.best, t,
                      b1, b2)) {
      st.best = t; st.best_prim = (int32_t)f_bits(a.w); st.bb1 = b1; st.bb2 = b2;
      if (ANY) return true;
    }
  }
  return trav_after_leaf<ANY>(st, stack, tmax);
}

// ANY = shadow query (returns on the first hit inside (tmin, tmax)).
template <bool ANY, bool COUNT, bool SPH = false>
MGPU_HD bool traverse(const SceneView &s, const Ray &r, Hit &hit, const Pair *top, uint32_t ntop, TraceCounts *cnt) {
  TravState st;
  TravEntry stack[kMaxStack];
  hit.t = INFINITY; hit.prim = -1; hit.b1 = 0.0f; hit.b2 = 0.0f;
  if (trav_init<SPH>(s, r, top, ntop, st, ANY)) {
    while (!trav_step<ANY, COUNT>(s, st, stack, top, ntop, cnt)) {
    }
  }
  if (st.best_prim < 0) return false;
  hit.t = st.best; hit.prim = st.best_prim; hit.b1 = st.bb1; hit.b2 = st.bb2;
  return true;
}

#if defined(__CUDACC__)
// Grid-stride traversal: every thread traces rays i, i + stride, ... to completion.
//   view(i)                 the scene of the i-th ray (one scene, or a batch job's scene)
//   load(i, ray)            fills the i-th ray of the batch
//   store(i, found, state)  consumes the i-th result
template <bool ANY, bool COUNT, bool SPH, class View, class Load, class Store>
__device__ __forceinline__ void grid_trace(View view, const Pair *top, uint32_t ntop, uint32_t n, Load load,
                                           Store store, TraceCounts *cnt, uint32_t &rays_done) {
  TravState st;
  TravEntry stack[kMaxStack];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const SceneView &s = view(i);
    Ray r;
    load(i, r);
    ++rays_done;
    if (!trav_init<SPH>(s, r, top, ntop, st, ANY)) {
      store(i, st.best_prim >= 0, st);
      continue;
    }
    while (!trav_step<ANY, COUNT>(s, st, stack, top, ntop, cnt)) {
    }
    store(i, st.best_prim >= 0, st);
  }
}

// Persistent warp-level traversal (Aila and Laine, "Understanding the Efficiency of Ray
// Traversal on GPUs", HPG 2009): every lane owns one ray; after each leaf step, lanes whose
// ray finished take new rays from a global counter with one warp-aggregated atomicAdd, so a
// warp never idles behind its slowest ray.  All 32 lanes of every warp must call this.
template <bool ANY, bool COUNT, bool SPH, class View, class Load, class Store>
__device__ __forceinline__ void persistent_trace(View view, const Pair *top, uint32_t ntop, uint32_t n,
                                                 uint32_t *fetch, Load load, Store store, TraceCounts *cnt,
                                                 uint32_t &rays_done) {
  const unsigned kFull = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  TravState st;
  TravEntry stack[kMaxStack];
  const SceneView *sv = nullptr;
  uint32_t idx = 0;
  bool have = false, exhausted = false;
  for (;;) {
    bool need = !have && !exhausted;
    unsigned m = __ballot_sync(kFull, need);
    if (m) {
      int leader = __ffs(m) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(m));
      base = __shfl_sync(kFull, base, leader);
      if (need) {
        uint32_t my = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
        if (my < n) {
          idx = my;
          sv = &view(idx);
          Ray r;
          load(idx, r);
          ++rays_done;
          if (trav_init<SPH>(*sv, r, top, ntop, st, ANY)) have = true;
          else store(idx, st.best_prim >= 0, st);
        } else {
          exhausted = true;
        }
      }
    }
    if (__all_sync(kFull, exhausted && !have)) break;
    if (have && trav_step<ANY, COUNT>(*sv, st, stack, top, ntop, cnt)) {
      store(idx, st.best_prim >= 0, st);
      have = false;
    }
  }
}

// Grid-stride traversal with the leaf triangles shared by the warp.  Every lane descends its own
// ray to its next leaf; then the warp tests the triangles of all the lanes' leaves together, 32
// (ray, triangle) pairs at a time, each test with the owning lane's ray (its shear constants,
// tmin and current best), and the results go back to the owners: for a closest hit the smallest
// (t, index in the leaf) per owner through a shared-memory atomicMin on wkey[32] (a per-warp array
// in shared memory; reducing each owner's run of lanes with __reduce_min_sync instead measured 45 %
// slower), for an any hit a bit per owner.  Lanes whose ray has
// finished test other lanes' triangles instead of idling, so a leaf of many triangles no longer
// holds the warp in a loop that few lanes execute.  The result of every ray is the one trav_step
// gives: the winner is the smallest t below the ray's best, ties to the first triangle in the
// leaf's order, and its owner re-runs that one test for t and barycentrics.
// All 32 lanes of every warp must call this (rays are taken in warp-aligned rounds).
// With wray / wk (per-warp shared memory: 64 float4, 32 words) each lane's ray constants for the
// tests are written there once per ray and read by the testers, instead of living in registers
// through the descent and travelling by shuffles.
// SINGLE: every ray of the launch is in one scene, view(0), which the kernel passes from its
// parameter space; the scene's pointers and bounds are then read as launch constants instead of
// through a per-lane pointer into device memory.
template <bool ANY, bool COUNT, bool SPH, bool SINGLE = false, class View, class Load, class Store>
__device__ __forceinline__ void grid_trace_coop(View view, uint32_t n, Load load, Store store, TraceCounts *cnt,
                                                uint32_t &rays_done, unsigned long long *wkey, float4 *wray = nullptr,
                                                uint32_t *wk = nullptr) {
  const unsigned kFull = 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  TravState st{};
  TravEntry stack[kMaxStack];
  const bool smray = wray != nullptr;
  const SceneView *svp = nullptr;
  auto SV = [&]() -> const SceneView & {
    if constexpr (SINGLE) return view(0u);
    else return *svp;
  };
  for (uint32_t r0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < n; r0 += stride) {
    const uint32_t i = r0 + lane;
    bool active = false;
    if (smray) __syncwarp(kFull);  // the previous round's readers are done with wray
    if (i < n) {
      if constexpr (!SINGLE) svp = &view(i);
      Ray r;
      load(i, r);
      ++rays_done;
      active = trav_init<SPH>(SV(), r, nullptr, 0, st, ANY);
      if (!active) store(i, st.best_prim >= 0, st);
      if (active && smray) {
        wray[lane] = make_float4(st.pre.o.x, st.pre.o.y, st.pre.o.z, st.ray_tmin);
        wray[32 + lane] = make_float4(st.pre.sx, st.pre.sy, st.pre.sz, st.best);
        wk[lane] = (uint32_t)st.pre.kx | ((uint32_t)st.pre.ky << 2) | ((uint32_t)st.pre.kz << 4);
      }
    }
    while (__any_sync(kFull, active)) {
      uint32_t lw0 = kLeafTag, lw1 = 0;
      float cell_tmax = 0.0f;
      if (active) trav_descend<COUNT>(SV(), st, stack, nullptr, 0, cnt, lw0, lw1, cell_tmax);
      const uint32_t count = active ? (lw0 >> 2) : 0u;
      // inclusive prefix sum of the leaf sizes over the warp
      uint32_t incl = count;
      for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += v;
      }
      const uint32_t total = __shfl_sync(kFull, incl, 31);
      const uint32_t excl = incl - count;
      // the owner's ray, as the tests need it
      const uint32_t kpack = smray ? 0u : ((uint32_t)st.pre.kx | ((uint32_t)st.pre.ky << 2) | ((uint32_t)st.pre.kz << 4));
      const unsigned long long ltp = (!SINGLE && active) ? (unsigned long long)SV().ltris : 0ull;
      if (!ANY) wkey[lane] = ~0ull;
      if (!ANY && smray && active) wray[32 + lane].w = st.best;
      __syncwarp(kFull);
      uint32_t hit_owners = 0u;
      for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t k = base + lane;
        // owner = the first lane whose inclusive sum exceeds k
        uint32_t o = 0;
        for (uint32_t step = 16; step >= 1; step >>= 1) {
          const uint32_t v = __shfl_sync(kFull, incl, o + step - 1);
          if (v <= k) o += step;
        }
        RayPre p;
        uint32_t kp;
        float tmin_o, best_o;
        if (smray) {
          const float4 ra = wray[o], rb = wray[32 + o];
          p.o.x = ra.x; p.o.y = ra.y; p.o.z = ra.z; tmin_o = ra.w;
          p.sx = rb.x; p.sy = rb.y; p.sz = rb.z; best_o = rb.w;
          kp = wk[o];
        } else {
          p.o.x = __shfl_sync(kFull, st.pre.o.x, o);
          p.o.y = __shfl_sync(kFull, st.pre.o.y, o);
          p.o.z = __shfl_sync(kFull, st.pre.o.z, o);
          p.sx = __shfl_sync(kFull, st.pre.sx, o);
          p.sy = __shfl_sync(kFull, st.pre.sy, o);
          p.sz = __shfl_sync(kFull, st.pre.sz, o);
          kp = __shfl_sync(kFull, kpack, o);
          tmin_o = __shfl_sync(kFull, st.ray_tmin, o);
          best_o = __shfl_sync(kFull, st.best, o);
        }
        p.kx = (int)(kp & 3u); p.ky = (int)((kp >> 2) & 3u); p.kz = (int)((kp >> 4) & 3u);
        const uint32_t first_o = __shfl_sync(kFull, lw1, o);
        const uint32_t excl_o = __shfl_sync(kFull, excl, o);
        const F4 *lt = SINGLE ? view(0u).ltris : reinterpret_cast<const F4 *>(__shfl_sync(kFull, ltp, o));
        if (k < total) {
          if (COUNT) cnt->tris++;
          const uint32_t idx = k - excl_o;
          const int64_t r = 3 * ((int64_t)first_o + idx);
          F4 a = load_f4(lt, r + 0);
          F4 b = load_f4(lt, r + 1);
          F4 c = load_f4(lt, r + 2);
          const bool culled = (f_bits(b.w) & 1u) != 0u;
          float t, b1, b2;
          if (intersect_tri(p, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), culled, tmin_o, best_o, t,
                            b1, b2)) {
            if (ANY) hit_owners |= 1u << o;
            else atomicMin(&wkey[o], ((unsigned long long)f_bits(t) << 32) | idx);
          }
        }
      }
      bool found = false;
      if (ANY) {
        found = ((__reduce_or_sync(kFull, hit_owners) >> lane) & 1u) != 0u;
      } else {
        __syncwarp(kFull);
        const unsigned long long key = wkey[lane];
        __syncwarp(kFull);
        if (active && key != ~0ull) {
          // the winner: redo its test for t and the barycentrics (the same inputs, the same result)
          const uint32_t idx = (uint32_t)(key & 0xFFFFFFFFull);
          const int64_t r = 3 * ((int64_t)lw1 + idx);
          F4 a = load_f4(SV().ltris, r + 0);
          F4 b = load_f4(SV().ltris, r + 1);
          F4 c = load_f4(SV().ltris, r + 2);
          float t, b1, b2;
          RayPre q = st.pre;
          if (smray) {  // the constants as the testers read them, not held in registers
            const float4 ra = wray[lane], rb = wray[32 + lane];
            const uint32_t kq = wk[lane];
            q.o = v3(ra.x, ra.y, ra.z);
            q.sx = rb.x; q.sy = rb.y; q.sz = rb.z;
            q.kx = (int)(kq & 3u); q.ky = (int)((kq >> 2) & 3u); q.kz = (int)((kq >> 4) & 3u);
          }
          if (intersect_tri(q, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z),
                            (f_bits(b.w) & 1u) != 0u, st.ray_tmin, st.best, t, b1, b2)) {
            st.best = t; st.best_prim = (int32_t)f_bits(a.w); st.bb1 = b1; st.bb2 = b2;
          }
        }
      }
      if (active) {
        bool done;
        if (ANY && found) {
          st.best_prim = 0;  // occluded: any non-negative value
          done = true;
        } else {
          done = trav_after_leaf<ANY>(st, stack, cell_tmax);
        }
        if (done) {
          store(i, st.best_prim >= 0, st);
          active = false;
        }
      }
    }
  }
}
#endif

}  // namespace mgpu
