/*
 * oracle.c -- FP64 CPU restatement of Milton's unidirectional PathTracer hot path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference arm load this library, and only as the
 * checker or as the timed CPU baseline.  The product (milton_gb300, libmgpu.so)
 * never links, loads or calls it.
 *
 * What it restates (file:line within the reference project, mlt/src/milton/ = M/):
 *   kd-tree build          M/accel/kdTreeAccel.cpp:403-472 (init), :533-630 (_buildTree),
 *                          :632-662 (_buildTreeHelper), :722-811 (_computeSplitPlaneSAH),
 *                          :813-853 (_computeSplitPlanesSAH), :855-877 (_computeSplitCostSAH),
 *                          M/accel/kdTreeAccel.h:97-104 (build defaults),
 *                          M/accel/SpatialAccel.h:43-56 (root AABB), M/accel/AABB.inl:67-72,
 *                          :112-135 (AABB add / surface areas)
 *   kd traversal           M/accel/kdTreeAccel.cpp:893-1016 (closest), :1018-1094 (any hit),
 *                          M/accel/AABB.inl:25-56 (slab test)
 *   triangle tests         M/shapes/MeshTriangle.cpp:92-168 (two-sided MT, EQ(det,0) reject),
 *                          M/shapes/Triangle.cpp:220-272 (culled MT, det < EPSILON reject),
 *                          M/shapes/Intersectable.cpp:20-25 (any-hit window)
 *   shading point          M/core/SurfacePoint.cpp:49-65, M/shapes/Mesh.cpp:419-433,
 *                          M/shapes/MeshTriangle.cpp:344-361, M/shapes/Transformable.inl:37-48
 *   camera                 M/cameras/ThinLensCamera.cpp:131-175 (getWorldRay, thin lens), :181-259
 *   super-sampling         M/renderers/generators/SuperSampleGenerator.cpp:23-91,
 *                          M/renderers/generators/JitteredSampleGenerator.cpp:19-39, M/core/Viewport.h:29-37
 *   estimator              M/renderers/renderers/PathTracer.cpp:28-116
 *   direct lighting        M/renderers/DirectIllumination.cpp:46-138, M/shapes/Plane.cpp:91-105
 *   light sample points    M/shapes/Shape.cpp:52-64, M/shapes/Triangle.cpp:332-362,
 *                          M/shapes/Mesh.cpp:419-465, M/shapes/MeshTriangle.cpp:299-333
 *   BSDFs                  M/materials/bsdfs/DiffuseBSDF.cpp:21-48,
 *                          M/materials/bsdfs/ModifiedPhongBSDF.cpp:48-181,
 *                          M/materials/bsdfs/DielectricBSDF.cpp:48-157, M/materials/bsdfs/Fresnel.h:45-90,
 *                          M/common/math/Vector.cpp:21-29, M/common/math/Vector.inl:460-495,527-538,
 *                          M/common/math/sisd/Vector3.inl:18-21, M/common/math/Vector.h:113-117
 *   emitters               M/materials/Emitter.cpp:34-50, M/materials/emitters/OrientedEmitter.cpp:17-23
 *   film                   M/renderers/RenderOutput.cpp:72-101, M/filters/ProgressiveFilterValue.h:18-38
 *   image maps             M/materials/Material.cpp:157-225 (uv, bump map), :229-301 (textured keys,
 *                          getSample), M/filters/KernelFilter.cpp:18-40,106-156 (filter kernel and
 *                          its application at one texel), M/filters/{Box,Triangle,Gaussian,Mitchell,
 *                          LanczosSinc}Filter.cpp (evaluate), M/shapes/Triangle.cpp:23-39 (uv),
 *                          M/common/image/Rgba.inl:32-45 (byte / 255, luminance)
 *   spheres                M/shapes/Sphere.cpp:17-85 (intersection in object space, uv, normal)
 *   background             M/core/Scene.cpp:116-118, M/renderers/renderers/PathTracer.cpp:39-42,
 *                          M/materials/emitters/EnvironmentMap.cpp:40-96, OmniEmitter.cpp
 *   constants              M/common/arch.h:120-137 (EPSILON 1e-7, double), M/common/utilities.h:240 (EQ),
 *                          M/materials/IndexOfRefraction.cpp:16 (AIR = 1.0003)
 *
 * Parity unpinned against the reference itself: Milton ships no golden vectors or known-answer
 * tests for this path, and its sources need Boost, Qt 4 and OpenGL headers (external libraries)
 * to compile, so no reference build exists to compare with.  This restatement is pinned instead by
 * the Random123 Philox known answers, brute-force ray queries, an analytic direct-lighting known
 * answer and BSDF property checks (tests/test_oracle.py), and its kd builder agrees node by node
 * with the product's.
 *
 * Random numbers.  The reference draws from one global boost::mt19937 (M/stats/Random.cpp:22-56),
 * which is not reproducible across threads.  The oracle and the GPU path instead draw every
 * uniform from Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11) keyed by (seed, path, depth, block), so that a path's random numbers do
 * not depend on which thread or kernel evaluates it.  The distribution of every draw matches
 * the reference's; per-sample streams do not (boost's version is unpinned).
 *
 * Deliberate deviation (named): where the reference divides 0 by a zero pdf (Phong's mirror
 * fallback below the surface, M/materials/bsdfs/ModifiedPhongBSDF.cpp:118-122 with :139-141;
 * its ASSERTs compile out in OPT and the pixel turns NaN), the oracle ends the path as
 * absorbed and counts the event.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EPS 1e-7
#define ORC_AIR 1.0003
#define ORC_PI 3.14159265358979323846
#define ORC_INF (1.0 / 0.0)

#define ORC_MAX_STACK 64
#define ORC_HARD_DEPTH_CAP 1024

/* ------------------------------------------------------------------------- */
/* fuzzy equality exactly as the reference defines it (M/common/utilities.h:240,
 * including its operator precedence)                                          */
static inline int orc_eq(double a, double b) {
  return fabs(a - b) < ORC_EPS || (fabs(a - b / ((fabs(b) > fabs(a)) ? b : a)) <= ORC_EPS);
}

typedef struct { double x, y, z; } v3;
static inline v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, double s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
  return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double vlen(v3 a) { return sqrt(vdot(a, a)); }
static inline v3 vnorm(v3 a) { double l = vlen(a); return l > 0 ? vmul(a, 1.0 / l) : a; }
static inline double vget(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline int veq(v3 a, v3 b) { return orc_eq(a.x, b.x) && orc_eq(a.y, b.y) && orc_eq(a.z, b.z); }

/* ------------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon et al., SC'11).  Shared specification with the GPU path:
 *   counter = {path_lo, path_hi, (depth << 16) | block, stream}, key = {seed_lo, seed_hi},
 *   uniform = (word >> 8) * 2^-24 in [0, 1).                                      */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct { uint32_t key[2]; uint32_t stream; } orc_rng;

static inline void orc_u4(const orc_rng *g, uint64_t path, uint32_t depth, uint32_t block, double u[4]) {
  uint32_t ctr[4] = {(uint32_t)path, (uint32_t)(path >> 32), (depth << 16) | (block & 0xFFFFu), g->stream};
  uint32_t o[4];
  orc_philox4x32_10(ctr, g->key, o);
  for (int i = 0; i < 4; ++i) u[i] = (double)(o[i] >> 8) * (1.0 / 16777216.0);
}

/* dimension map (identical on the GPU):
 *   depth 0xFFFF, block 0, path = pixel * side^2 + stratum : {jitter x, jitter y, -, -}
 *   depth 0xFFFE, block 0, path = global path id           : {ior index, lens e1, lens e2, -}
 *   depth d,      block 0                                  : {bsdf0, bsdf1, bsdf2, russian roulette}
 *   depth d,      block 1 + m/2                            : NEE sample m, lanes 2(m%2), 2(m%2)+1  */
#define ORC_DEPTH_JITTER 0xFFFFu
#define ORC_DEPTH_PATHINIT 0xFFFEu

/* ------------------------------------------------------------------------- */
/* scene                                                                        */
enum { MAT_DIFFUSE = 0, MAT_PHONG = 1, MAT_DIELECTRIC = 2 };
#define TRI_CULLED 1u

typedef struct {
  int type;
  double kd[3], ks[3], n, ior, transparency;
  double ior3[3]; /* per-channel IOR (the "ior" spectrum); a path refracts with its channel's */
  int tex[4]; /* 1 + texture index for kd, ks, transparency, bump map; 0 = none */
} orc_mat;

/* A material's image map: rgb h x w x 3 linear values, row 0 on top.  Colour maps carry the
 * kernel KernelFilter::_computeKernel builds for the material's filter. */
typedef struct {
  int w, h, kind; /* kind 0 colour, 1 bump */
  const float *rgb;
  int kw;         /* kernel width (ceil(support) | 1) */
  double *wts;    /* kw * kw weights */
  double ru, rv, intensity;
} orc_tex;

/* Area light: Milton Plane (type 0), Triangle (1) or Mesh (2) emitter.  Triangle: center = v1,
 * ex = v2 - v1, ez = v3 - v1, uv frame (uv0, a, b, 1/|a x b|).  Mesh: triangle run [first,
 * first + count) of the soup. */
typedef struct {
  v3 center, ex, ez, normal;
  double area;
  double Le[3];
  int type;
  double u0, v0, ax, ay, bx, by, inv_ab;
  int64_t first, count;
  int omni;  /* OmniEmitter (both sides; every point light) */
} orc_light;

typedef struct {
  int64_t ntri;
  const float *v;      /* ntri * 9, world space */
  const float *n;      /* ntri * 9, per-vertex shading normals */
  const int32_t *mat;  /* ntri */
  const int32_t *light;/* ntri, light index or -1 */
  const uint32_t *flags;
  int nmat;
  orc_mat *mats;
  int nlight;
  orc_light *lights;
  const float *uv;     /* ntri * 6 per-vertex uvs, or NULL */
  int ntex;
  orc_tex *tex;
  int bg_tex;          /* background: 1 + colour map (environment map) or 0 */
  double bg_le[3];     /* constant background radiance when bg_tex == 0 */
  int nsph;            /* analytic spheres: primitive ids ntri .. ntri + nsph - 1 */
  const float *sph;    /* 8 floats each: center, radius, world-to-object quaternion */
  const int32_t *sph_mat;
  const int32_t *sph_light; /* or NULL */
} orc_scene;

static inline v3 tri_vert(const orc_scene *s, int64_t t, int k) {
  const float *p = s->v + t * 9 + k * 3;
  return V(p[0], p[1], p[2]);
}
static inline v3 tri_nrm(const orc_scene *s, int64_t t, int k) {
  const float *p = s->n + t * 9 + k * 3;
  return V(p[0], p[1], p[2]);
}

/* ------------------------------------------------------------------------- */
/* triangle tests                                                               */

/* two-sided Moller-Trumbore, M/shapes/MeshTriangle.cpp:92-168 (non-culling branch) */
static double isect_mesh_tri(v3 o, v3 d, v3 a, v3 b, v3 c) {
  v3 e1 = vsub(b, a), e2 = vsub(c, a);
  v3 pv = vcross(d, e2);
  double det = vdot(e1, pv);
  if (orc_eq(det, 0.0)) return ORC_INF;
  double inv = 1.0 / det;
  v3 tv = vsub(o, a);
  double u = vdot(tv, pv) * inv;
  if (u < 0.0 || u > 1.0) return ORC_INF;
  v3 qv = vcross(tv, e1);
  double v = vdot(d, qv) * inv;
  if (v < 0.0 || u + v > 1.0) return ORC_INF;
  return vdot(e2, qv) * inv;
}

/* back-face culled Moller-Trumbore, M/shapes/Triangle.cpp:220-272 (culling branch) */
static double isect_culled_tri(v3 o, v3 d, v3 a, v3 b, v3 c) {
  v3 e1 = vsub(b, a), e2 = vsub(c, a);
  v3 pv = vcross(d, e2);
  double det = vdot(e1, pv);
  if (det < ORC_EPS) return ORC_INF;
  v3 tv = vsub(o, a);
  double u = vdot(tv, pv);
  if (u < 0.0 || u > det) return ORC_INF;
  v3 qv = vcross(tv, e1);
  double v = vdot(d, qv);
  if (v < 0.0 || u + v > det) return ORC_INF;
  return vdot(e2, qv) * (1.0 / det);
}

static inline double isect_tri(const orc_scene *s, int64_t t, v3 o, v3 d) {
  v3 a = tri_vert(s, t, 0), b = tri_vert(s, t, 1), c = tri_vert(s, t, 2);
  if (s->flags && (s->flags[t] & TRI_CULLED)) return isect_culled_tri(o, d, a, b, c);
  return isect_mesh_tri(o, d, a, b, c);
}

/* ------------------------------------------------------------------------- */
/* kd-tree build (restated from M/accel/kdTreeAccel.cpp:403-877)                */

typedef struct { double mn[3], mx[3]; } orc_aabb;

typedef struct orc_node {
  int leaf;     /* 1 = leaf */
  int axis;     /* split axis for interior nodes */
  float split;  /* stored as float, :606 */
  struct orc_node *child; /* two adjacent children */
  int32_t *prims;
  int nprims;
} orc_node;

typedef struct {
  unsigned min_prims, max_depth;
  double cost_trav, empty_bias;
} orc_kd_params;

typedef struct {
  unsigned no_internal, no_leaves, min_depth, max_depth;
  unsigned long long sum_depth, sum_prims;
  unsigned min_prims, max_prims;
} orc_kd_log;

typedef struct {
  orc_node *root;
  orc_aabb box;
  orc_aabb *tri_box;
  int64_t ntri;
  orc_kd_params p;
  orc_kd_log log;
} orc_tree;

typedef struct { double pos; int type; } orc_plane; /* type: 0 MAX, 1 PLANE, 2 MIN (:274) */

static int plane_cmp(const void *pa, const void *pb) {
  const orc_plane *a = pa, *b = pb;
  if (a->pos < b->pos) return -1;
  if (a->pos > b->pos) return 1;
  return (a->type > b->type) - (a->type < b->type);
}

static inline int box_is_point(const orc_aabb *b) {
  return b->mn[0] == b->mx[0] && b->mn[1] == b->mx[1] && b->mn[2] == b->mx[2];
}

static inline double box_area(const orc_aabb *b) {
  double d0 = b->mx[0] - b->mn[0], d1 = b->mx[1] - b->mn[1], d2 = b->mx[2] - b->mn[2];
  return 2 * (d0 * d1 + d1 * d2 + d2 * d0);
}

static inline void box_split_areas(const orc_aabb *b, int axis, double pos, double *l, double *r) {
  double d[3] = {b->mx[0] - b->mn[0], b->mx[1] - b->mn[1], b->mx[2] - b->mn[2]};
  d[axis] = pos - b->mn[axis];
  *l = 2 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
  d[axis] = b->mx[axis] - pos;
  *r = 2 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
}

typedef struct {
  orc_tree *tr;
  orc_plane *planes;
  orc_aabb box;
} orc_build_ctx;

static void log_leaf(orc_kd_log *lg, int n, unsigned depth) {
  lg->no_leaves++;
  if ((unsigned)n < lg->min_prims) lg->min_prims = n;
  if ((unsigned)n > lg->max_prims) lg->max_prims = n;
  lg->sum_prims += n;
  if (depth < lg->min_depth) lg->min_depth = depth;
  if (depth > lg->max_depth) lg->max_depth = depth;
  lg->sum_depth += depth;
}

static void make_leaf(orc_build_ctx *c, orc_node *nd, int32_t *prims, int n, unsigned depth) {
  nd->leaf = 1;
  nd->prims = prims;
  nd->nprims = n;
  nd->child = NULL;
  log_leaf(&c->tr->log, n, depth);
}

/* candidate planes along one axis, :813-853 */
static unsigned collect_planes(orc_build_ctx *c, const int32_t *prims, int n, int axis) {
  unsigned m = 0;
  for (int i = n; i--;) {
    const orc_aabb *b = &c->tr->tri_box[prims[i]];
    if (box_is_point(b)) continue;
    double mn = b->mn[axis], mx = b->mx[axis];
    if (mn == mx) {
      c->planes[m].pos = mn; c->planes[m].type = 1; ++m;
    } else {
      c->planes[m].pos = mn; c->planes[m].type = 2; ++m;
      c->planes[m].pos = mx; c->planes[m].type = 0; ++m;
    }
  }
  if (m > 0) qsort(c->planes, m, sizeof(orc_plane), plane_cmp);
  return m;
}

static void build_rec(orc_build_ctx *c, orc_node *nd, int32_t *prims, int n, int parent_axis, unsigned depth);

static void build_helper(orc_build_ctx *c, orc_node *child, int32_t *prims, int n, int parent_axis, unsigned depth) {
  if (n > 0) build_rec(c, child, prims, n, parent_axis, depth);
  else make_leaf(c, child, prims, 0, depth);
}

static void build_rec(orc_build_ctx *c, orc_node *nd, int32_t *prims, int n, int parent_axis, unsigned depth) {
  orc_tree *tr = c->tr;
  if (depth > tr->log.max_depth) tr->log.max_depth = depth;
  if ((unsigned)n < tr->p.min_prims || depth >= tr->p.max_depth) {
    make_leaf(c, nd, prims, n, depth);
    return;
  }
  /* SAH plane selection, :722-811 */
  double best_cost = ORC_INF, best_pos = 0;
  int best_axis = 0;
  for (int axis = 0; axis < 3; ++axis) {
    if (axis == parent_axis || c->box.mn[axis] >= c->box.mx[axis]) continue;
    unsigned m = collect_planes(c, prims, n, axis);
    if (m == 0) continue;
    unsigned idx = 0, nl = 0, nr = (unsigned)n;
    while (idx < m - 1) {
      double cur = c->planes[idx].pos;
      unsigned cnt[3] = {0, 0, 0};
      do {
        ++cnt[c->planes[idx].type];
      } while (idx < m - 1 && c->planes[++idx].pos == cur);
      unsigned np = cnt[1];
      nr -= cnt[0] + np;
      if (cur > c->box.mn[axis] && cur < c->box.mx[axis]) {
        double la, ra;
        box_split_areas(&c->box, axis, cur, &la, &ra);
        unsigned l = nl + np;
        double cost = la * l + ra * nr;
        if (l + np == 0 || nr == 0) cost *= tr->p.empty_bias;
        if (cost < best_cost) { best_cost = cost; best_pos = cur; best_axis = axis; }
      }
      nl += cnt[2] + np;
    }
  }
  if (best_cost == ORC_INF) { make_leaf(c, nd, prims, n, depth); return; }
  double leaf_cost = (n - tr->p.cost_trav) * box_area(&c->box);
  if (best_cost > leaf_cost) { make_leaf(c, nd, prims, n, depth); return; }

  /* partition, :562-583 */
  int32_t *lp = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
  int32_t *rp = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
  int nlft = 0, nrgt = 0;
  for (int i = 0; i < n; ++i) {
    const orc_aabb *b = &tr->tri_box[prims[i]];
    if (box_is_point(b)) continue;
    double mn = b->mn[best_axis], mx = b->mx[best_axis];
    if (mx > best_pos) rp[nrgt++] = prims[i];
    if (mn <= best_pos) lp[nlft++] = prims[i];
  }
  /* stop when the split separates nothing (SAH form of :586-597) */
  if (nlft == n && nrgt == n) {
    free(lp); free(rp);
    make_leaf(c, nd, prims, n, depth);
    return;
  }
  free(prims);
  orc_node *kids = (orc_node *)calloc(2, sizeof(orc_node));
  nd->leaf = 0;
  nd->axis = best_axis;
  nd->split = (float)best_pos;
  nd->child = kids;
  nd->prims = NULL;
  nd->nprims = 0;
  tr->log.no_internal++;
  double prev_max = c->box.mx[best_axis];
  c->box.mx[best_axis] = best_pos;
  build_helper(c, &kids[0], lp, nlft, best_axis, depth + 1);
  c->box.mx[best_axis] = prev_max;
  double prev_min = c->box.mn[best_axis];
  c->box.mn[best_axis] = best_pos;
  build_helper(c, &kids[1], rp, nrgt, best_axis, depth + 1);
  c->box.mn[best_axis] = prev_min;
}

static void free_node(orc_node *nd) {
  if (!nd) return;
  if (nd->leaf) { free(nd->prims); return; }
  if (!nd->child) return;  /* a node of a partly read serialisation */
  free_node(&nd->child[0]);
  free_node(&nd->child[1]);
  free(nd->child);
}

orc_tree *orc_kd_build(const float *v, int64_t ntri, unsigned min_prims, unsigned max_depth,
                       double cost_trav, double empty_bias) {
  orc_tree *tr = (orc_tree *)calloc(1, sizeof(orc_tree));
  tr->ntri = ntri;
  tr->p.min_prims = min_prims;
  tr->p.max_depth = max_depth;
  tr->p.cost_trav = cost_trav;
  tr->p.empty_bias = empty_bias;
  tr->log.min_depth = 0xFFFFFFFFu;
  tr->log.min_prims = 0xFFFFFFFFu;
  tr->tri_box = (orc_aabb *)malloc(sizeof(orc_aabb) * (ntri > 0 ? ntri : 1));
  for (int k = 0; k < 3; ++k) { tr->box.mn[k] = ORC_INF; tr->box.mx[k] = -ORC_INF; }
  for (int64_t t = 0; t < ntri; ++t) {
    orc_aabb *b = &tr->tri_box[t];
    for (int k = 0; k < 3; ++k) { b->mn[k] = ORC_INF; b->mx[k] = -ORC_INF; }
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        double x = v[t * 9 + j * 3 + k];
        if (x < b->mn[k]) b->mn[k] = x;
        if (x > b->mx[k]) b->mx[k] = x;
      }
    /* SpatialAccel::init adds non-point boxes; AABB::add(AABB) skips min ~= max (fuzzy) */
    if (!box_is_point(b)) {
      int same = orc_eq(b->mn[0], b->mx[0]) && orc_eq(b->mn[1], b->mx[1]) && orc_eq(b->mn[2], b->mx[2]);
      if (!same)
        for (int k = 0; k < 3; ++k) {
          if (b->mn[k] < tr->box.mn[k]) tr->box.mn[k] = b->mn[k];
          if (b->mx[k] > tr->box.mx[k]) tr->box.mx[k] = b->mx[k];
        }
    }
  }
  orc_build_ctx c;
  c.tr = tr;
  c.planes = (orc_plane *)malloc(sizeof(orc_plane) * (2 * ntri + 2));
  c.box = tr->box;
  tr->root = (orc_node *)calloc(1, sizeof(orc_node));
  int32_t *prims = (int32_t *)malloc(sizeof(int32_t) * (ntri + 1));
  for (int64_t i = 0; i < ntri; ++i) prims[i] = (int32_t)i;
  build_helper(&c, tr->root, prims, (int)ntri, 3, 0);
  free(c.planes);
  return tr;
}

/* A tree from its depth-first serialisation (the layout of orc_kd_serialize, which the product's
 * mgpu_accel_serialize also writes): for scenes too large for the restated build above, the
 * oracle traverses the product builder's tree, which is node-for-node the one that build gives
 * wherever both are run (tests/test_kdtree.py).  The root box is computed as orc_kd_build does.
 * Returns NULL on a malformed serialisation. */
void orc_kd_free(orc_tree *tr);
static int from_ser_rec(orc_node *nd, const int32_t *kind, const float *split, const int32_t *count,
                        const int32_t *prims, int64_t n_nodes, int64_t n_prims, int64_t *ni, int64_t *np) {
  if (*ni >= n_nodes) return 0;
  int64_t i = (*ni)++;
  if (kind[i] == 3) {
    nd->leaf = 1;
    nd->nprims = count[i];
    if (count[i] < 0 || *np + count[i] > n_prims) return 0;
    nd->prims = (int32_t *)malloc(sizeof(int32_t) * (count[i] > 0 ? count[i] : 1));
    memcpy(nd->prims, prims + *np, sizeof(int32_t) * (size_t)count[i]);
    *np += count[i];
    return 1;
  }
  if (kind[i] < 0 || kind[i] > 2) return 0;
  nd->leaf = 0;
  nd->axis = kind[i];
  nd->split = split[i];
  nd->child = (orc_node *)calloc(2, sizeof(orc_node));
  return from_ser_rec(&nd->child[0], kind, split, count, prims, n_nodes, n_prims, ni, np) &&
         from_ser_rec(&nd->child[1], kind, split, count, prims, n_nodes, n_prims, ni, np);
}

orc_tree *orc_kd_from_serial(const float *v, int64_t ntri, const int32_t *kind, const float *split,
                             const int32_t *count, const int32_t *prims, int64_t n_nodes, int64_t n_prims) {
  orc_tree *tr = (orc_tree *)calloc(1, sizeof(orc_tree));
  tr->ntri = ntri;
  tr->tri_box = (orc_aabb *)malloc(sizeof(orc_aabb));
  for (int k = 0; k < 3; ++k) { tr->box.mn[k] = ORC_INF; tr->box.mx[k] = -ORC_INF; }
  for (int64_t t = 0; t < ntri; ++t) {
    orc_aabb b;
    for (int k = 0; k < 3; ++k) { b.mn[k] = ORC_INF; b.mx[k] = -ORC_INF; }
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        double x = v[t * 9 + j * 3 + k];
        if (x < b.mn[k]) b.mn[k] = x;
        if (x > b.mx[k]) b.mx[k] = x;
      }
    if (!box_is_point(&b)) {
      int same = orc_eq(b.mn[0], b.mx[0]) && orc_eq(b.mn[1], b.mx[1]) && orc_eq(b.mn[2], b.mx[2]);
      if (!same)
        for (int k = 0; k < 3; ++k) {
          if (b.mn[k] < tr->box.mn[k]) tr->box.mn[k] = b.mn[k];
          if (b.mx[k] > tr->box.mx[k]) tr->box.mx[k] = b.mx[k];
        }
    }
  }
  tr->root = (orc_node *)calloc(1, sizeof(orc_node));
  int64_t ni = 0, np = 0;
  if (!from_ser_rec(tr->root, kind, split, count, prims, n_nodes, n_prims, &ni, &np) || ni != n_nodes) {
    orc_kd_free(tr);
    return NULL;
  }
  return tr;
}

void orc_kd_free(orc_tree *tr) {
  if (!tr) return;
  if (tr->root) { free_node(tr->root); free(tr->root); }
  free(tr->tri_box);
  free(tr);
}

/* stats in the reference's log layout (:460-471):
 * out[0..7] = noInternal, noLeaves, minDepth, maxDepth, sumDepth, minPrims, maxPrims, sumPrims */
void orc_kd_stats(const orc_tree *tr, uint64_t out[8]) {
  out[0] = tr->log.no_internal;
  out[1] = tr->log.no_leaves;
  out[2] = tr->log.min_depth;
  out[3] = tr->log.max_depth;
  out[4] = tr->log.sum_depth;
  out[5] = tr->log.min_prims;
  out[6] = tr->log.max_prims;
  out[7] = tr->log.sum_prims;
}

void orc_kd_bounds(const orc_tree *tr, double out[6]) {
  for (int k = 0; k < 3; ++k) { out[k] = tr->box.mn[k]; out[3 + k] = tr->box.mx[k]; }
}

/* Depth-first (left before right) serialisation used to compare trees node by node:
 * per node: kind (0,1,2 = split axis, 3 = leaf), split bits or prim count; leaf prims are
 * appended to prim_out in stored order.  Returns the node count; with NULL outputs it only
 * counts.  *nprim_out receives the number of prim references.                              */
static void ser_rec(const orc_node *nd, int32_t *kind, float *split, int32_t *count, int32_t *prim_out,
                    int64_t *ni, int64_t *np) {
  int64_t i = (*ni)++;
  if (nd->leaf) {
    if (kind) { kind[i] = 3; split[i] = 0.0f; count[i] = nd->nprims; }
    for (int k = 0; k < nd->nprims; ++k) {
      if (prim_out) prim_out[*np] = nd->prims[k];
      ++*np;
    }
    return;
  }
  if (kind) { kind[i] = nd->axis; split[i] = nd->split; count[i] = 0; }
  ser_rec(&nd->child[0], kind, split, count, prim_out, ni, np);
  ser_rec(&nd->child[1], kind, split, count, prim_out, ni, np);
}

int64_t orc_kd_serialize(const orc_tree *tr, int32_t *kind, float *split, int32_t *count, int32_t *prims,
                         int64_t *nprim_out) {
  int64_t ni = 0, np = 0;
  ser_rec(tr->root, kind, split, count, prims, &ni, &np);
  if (nprim_out) *nprim_out = np;
  return ni;
}

/* ------------------------------------------------------------------------- */
/* traversal (restated from :893-1094)                                        */

typedef struct { uint64_t nodes, refs, tris; } orc_counters;

static int slab(const orc_aabb *b, v3 o, v3 inv, double *tmin, double *tmax) {
  const double bo[3] = {o.x, o.y, o.z}, bi[3] = {inv.x, inv.y, inv.z};
  int xs = bi[0] < 0, ys = bi[1] < 0, zs = bi[2] < 0;
  double t0 = ((xs ? b->mx[0] : b->mn[0]) - bo[0]) * bi[0];
  double t1 = ((xs ? b->mn[0] : b->mx[0]) - bo[0]) * bi[0];
  double y0 = ((ys ? b->mx[1] : b->mn[1]) - bo[1]) * bi[1];
  double y1 = ((ys ? b->mn[1] : b->mx[1]) - bo[1]) * bi[1];
  if (t0 > y1 || y0 > t1) return 0;
  if (y0 > t0) t0 = y0;
  if (y1 < t1) t1 = y1;
  double z0 = ((zs ? b->mx[2] : b->mn[2]) - bo[2]) * bi[2];
  double z1 = ((zs ? b->mn[2] : b->mx[2]) - bo[2]) * bi[2];
  if (t0 > z1 || z0 > t1) return 0;
  if (z0 > t0) t0 = z0;
  if (z1 < t1) t1 = z1;
  *tmin = t0;
  *tmax = t1;
  return t0 <= t1;
}

typedef struct { const orc_node *node; double tmax; } orc_stk;

/* closest hit: returns t (INF on miss), *prim = triangle index */
static double kd_closest(const orc_scene *s, const orc_tree *tr, v3 o, v3 d, int64_t *prim, orc_counters *cn) {
  v3 inv = V(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
  double tmin, tmax;
  *prim = -1;
  if (!slab(&tr->box, o, inv, &tmin, &tmax)) return ORC_INF;
  tmin -= ORC_EPS;
  tmax += ORC_EPS;
  orc_stk stk[ORC_MAX_STACK];
  int sp = 0;
  const orc_node *cur = tr->root;
  const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, ii[3] = {inv.x, inv.y, inv.z};
  for (;;) {
    while (!cur->leaf) {
      if (cn) cn->nodes++;
      int ax = cur->axis;
      double diff = (double)cur->split - oo[ax];
      double dt = diff * ii[ax];
      int rev = diff <= 0 ? (dd[ax] <= 0) : (dd[ax] < 0);
      const orc_node *nearn = &cur->child[rev];
      const orc_node *farn = &cur->child[1 - rev];
      cur = nearn;
      if (dt > tmax) continue;
      if (dt < tmin) {
        cur = farn;
      } else {
        if (sp < ORC_MAX_STACK) { stk[sp].node = farn; stk[sp].tmax = tmax; ++sp; }
        tmax = dt + ORC_EPS;
      }
    }
    if (cn) cn->nodes++;
    double tcell = ORC_INF;
    int64_t best = -1;
    for (int i = cur->nprims; i--;) {
      int32_t pi = cur->prims[i];
      if (cn) { cn->refs++; cn->tris++; }
      double t = isect_tri(s, pi, o, d);
      if (t > ORC_EPS && t < tcell) { tcell = t; best = pi; }
    }
    if (tcell <= tmax) { *prim = best; return tcell; }
    if (sp == 0) return ORC_INF;
    tmin = tmax - 2 * ORC_EPS;
    --sp;
    cur = stk[sp].node;
    tmax = stk[sp].tmax;
  }
}

/* any hit inside (EPSILON, clip_max - EPSILON), :1018-1094 + Intersectable.cpp:20-25 */
static int kd_any(const orc_scene *s, const orc_tree *tr, v3 o, v3 d, double clip_max, orc_counters *cn) {
  v3 inv = V(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
  double tmin, tmax;
  if (!slab(&tr->box, o, inv, &tmin, &tmax) || clip_max < tmin) return 0;
  if (clip_max < tmax) tmax = clip_max;
  tmin -= ORC_EPS;
  tmax += ORC_EPS;
  orc_stk stk[ORC_MAX_STACK];
  int sp = 0;
  const orc_node *cur = tr->root;
  const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, ii[3] = {inv.x, inv.y, inv.z};
  for (;;) {
    while (!cur->leaf) {
      if (cn) cn->nodes++;
      int ax = cur->axis;
      double diff = (double)cur->split - oo[ax];
      double dt = diff * ii[ax];
      int rev = diff <= 0 ? (dd[ax] <= 0) : (dd[ax] < 0);
      const orc_node *nearn = &cur->child[rev];
      const orc_node *farn = &cur->child[1 - rev];
      cur = nearn;
      if (dt > tmax) continue;
      if (dt < tmin) {
        cur = farn;
      } else {
        if (sp < ORC_MAX_STACK) { stk[sp].node = farn; stk[sp].tmax = tmax; ++sp; }
        tmax = dt + ORC_EPS;
      }
    }
    if (cn) cn->nodes++;
    for (int i = cur->nprims; i--;) {
      if (cn) { cn->refs++; cn->tris++; }
      double t = isect_tri(s, cur->prims[i], o, d);
      if (t < clip_max - ORC_EPS && t > ORC_EPS) return 1;
    }
    if (sp == 0) return 0;
    tmin = tmax;
    --sp;
    cur = stk[sp].node;
    tmax = stk[sp].tmax;
  }
}

/* ------------------------------------------------------------------------- */
/* scene construction from flat arrays                                         */
/* material record (16 floats): type, kd[3], ks[3], n, ior, transparency, ...
 * light record (16 floats): center[3], ex[3], ez[3], normal[3], area, Le[3]   */
/* Filter2D::evaluate of the kernel filters (M/filters/BoxFilter.cpp, TriangleFilter.cpp,
 * GaussianFilter.cpp, MitchellFilter.cpp, LanczosSincFilter.cpp), in FP64.  kind: 1 box,
 * 2 triangle, 3 gaussian (p1 sigma), 4 mitchell (p1 B, p2 C), 5 lanczosSinc (p1 tau).  The
 * triangle filter is not mirrored for negative offsets and Mitchell's outer branch has no 1/6
 * and no cut-off, as in the reference. */
static double mitchell_1d(double x, double support, double B, double C) {
  x = fabs(2.0 * x / support);
  if (x > 1.0) return (((-B / 6.0 - C) * x + (B + 5.0 * C)) * x + (-2.0 * B - 8.0 * C)) * x + (4.0 / 3.0 * B + 4.0 * C);
  return x * x * ((2.0 - 1.5 * B - C) * x + (-3.0 + 2.0 * B + C)) + (1.0 - B / 3.0);
}

static double lanczos_1d(double x, double support, double tau) {
  x = fabs(x / support);
  if (x < ORC_EPS) return 1.0;
  if (x > 1.0) return 0.0;
  x *= ORC_PI;
  return sin(x * tau) / (x * tau) * sin(x) / x;
}

static double filter_eval(int kind, double support, double p1, double p2, double x, double y) {
  switch (kind) {
    case 1: return 2.0 * sqrt(x * x + y * y) < support ? 1.0 : 0.0;
    case 2: {
      double r = support / 2.0;
      double a = 1.0 - x / r, b = 1.0 - y / r;
      return (a > 0 ? a : 0) * (b > 0 ? b : 0);
    }
    case 3: {
      double g = (1.0 / (sqrt(2.0 * ORC_PI) * p1)) * exp(-0.5 / (p1 * p1) * (x * x + y * y));
      return g > 0 ? g : 0;
    }
    case 4: return mitchell_1d(x, support, p1, p2) * mitchell_1d(y, support, p1, p2);
    case 5: return lanczos_1d(x, support, p1) * lanczos_1d(y, support, p1);
    default: return 0.0;
  }
}

/* tex_params: 12 floats per texture: width, height, kind, filter, support, p1, p2, repeat u,
 * repeat v, bump intensity, 0, 0 */
static orc_tex *textures_from(int ntex, const float *params, const float *const *rgb) {
  orc_tex *t = (orc_tex *)calloc(ntex > 0 ? ntex : 1, sizeof(orc_tex));
  for (int i = 0; i < ntex; ++i) {
    const float *q = params + 12 * i;
    t[i].w = (int)q[0]; t[i].h = (int)q[1]; t[i].kind = (int)q[2];
    t[i].rgb = rgb[i];
    t[i].ru = q[7]; t[i].rv = q[8]; t[i].intensity = q[9];
    if (t[i].kind == 0) {
      /* KernelFilter::_computeKernel: kernel[i w + j] = evaluate(i - w / 2, j - w / 2) */
      int kw = ((int)ceil((double)q[4])) | 1;
      double half = kw / 2.0;
      t[i].kw = kw;
      t[i].wts = (double *)calloc((size_t)kw * kw, sizeof(double));
      for (int a = 0; a < kw; ++a)
        for (int b = 0; b < kw; ++b) t[i].wts[a * kw + b] = filter_eval((int)q[3], q[4], q[5], q[6], a - half, b - half);
    }
  }
  return t;
}

/* material record [8] = IOR of channel 0 (all channels when [14] = [15] = 0), [14], [15] = the
 * IOR of channels 1 and 2 */
static void mat_ior3(orc_mat *m, const float *rec) {
  const int per = rec[14] != 0.0f || rec[15] != 0.0f;
  m->ior3[0] = rec[8];
  m->ior3[1] = per ? rec[14] : rec[8];
  m->ior3[2] = per ? rec[15] : rec[8];
}

static orc_scene *scene_from_arrays(int64_t ntri, const float *v, const float *n, const int32_t *mat,
                                    const int32_t *light, const uint32_t *flags, int nmat, const float *mats,
                                    int nlight, const float *lights, const float *light_ext) {
  orc_scene *s = (orc_scene *)calloc(1, sizeof(orc_scene));
  s->ntri = ntri; s->v = v; s->n = n; s->mat = mat; s->light = light; s->flags = flags;
  s->nmat = nmat;
  s->mats = (orc_mat *)calloc(nmat > 0 ? nmat : 1, sizeof(orc_mat));
  for (int i = 0; i < nmat; ++i) {
    const float *m = mats + i * 16;
    s->mats[i].type = (int)m[0];
    for (int k = 0; k < 3; ++k) { s->mats[i].kd[k] = m[1 + k]; s->mats[i].ks[k] = m[4 + k]; }
    s->mats[i].n = m[7];
    s->mats[i].ior = m[8];
    mat_ior3(&s->mats[i], m);
    s->mats[i].transparency = m[9];
    for (int k = 0; k < 4; ++k) s->mats[i].tex[k] = (int)m[10 + k];
  }
  s->nlight = nlight;
  s->lights = (orc_light *)calloc(nlight > 0 ? nlight : 1, sizeof(orc_light));
  for (int i = 0; i < nlight; ++i) {
    const float *l = lights + i * 16;
    s->lights[i].center = V(l[0], l[1], l[2]);
    s->lights[i].ex = V(l[3], l[4], l[5]);
    s->lights[i].ez = V(l[6], l[7], l[8]);
    s->lights[i].normal = vnorm(V(l[9], l[10], l[11]));
    s->lights[i].area = l[12];
    for (int k = 0; k < 3; ++k) s->lights[i].Le[k] = l[13 + k];
    if (light_ext) {
      const float *x = light_ext + i * 16;
      uint32_t first, count;
      memcpy(&first, x + 8, 4);
      memcpy(&count, x + 9, 4);
      s->lights[i].type = (int)x[0];
      s->lights[i].u0 = x[1]; s->lights[i].v0 = x[2];
      s->lights[i].ax = x[3]; s->lights[i].ay = x[4];
      s->lights[i].bx = x[5]; s->lights[i].by = x[6];
      s->lights[i].inv_ab = x[7];
      s->lights[i].first = first;
      s->lights[i].count = count;
      s->lights[i].omni = x[15] != 0.0f || s->lights[i].type == 3;
    }
  }
  return s;
}

static void scene_free(orc_scene *s) {
  if (!s) return;
  for (int i = 0; i < s->ntex; ++i) free(s->tex[i].wts);
  free(s->tex);
  free(s->mats);
  free(s->lights);
  free(s);
}

/* ------------------------------------------------------------------------- */
/* exported ray queries.  rays: n * 8 floats (o.xyz, tmin, d.xyz, tmax).
 * closest: t_out (INF on miss), prim_out (-1), t2_out (nearest t among the other prims, from
 * the brute-force pass only).  tree == NULL means brute force over all triangles.          */
void orc_trace_closest(const orc_tree *tr, int64_t ntri, const float *v, const uint32_t *flags, const float *rays,
                       int64_t n, double *t_out, int64_t *prim_out, double *t2_out, uint64_t *counters) {
  orc_scene sc;
  memset(&sc, 0, sizeof(sc));
  sc.ntri = ntri; sc.v = v; sc.flags = flags;
  orc_counters cn = {0, 0, 0};
  for (int64_t i = 0; i < n; ++i) {
    const float *r = rays + i * 8;
    v3 o = V(r[0], r[1], r[2]), d = V(r[4], r[5], r[6]);
    if (tr) {
      int64_t p;
      t_out[i] = kd_closest(&sc, tr, o, d, &p, counters ? &cn : NULL);
      prim_out[i] = p;
      if (t2_out) t2_out[i] = ORC_INF;
    } else {
      double b1 = ORC_INF, b2 = ORC_INF;
      int64_t p1 = -1;
      for (int64_t t = 0; t < ntri; ++t) {
        double th = isect_tri(&sc, t, o, d);
        if (!(th > ORC_EPS && th < ORC_INF)) continue;
        if (th < b1) { b2 = b1; b1 = th; p1 = t; }
        else if (th < b2) { b2 = th; }
      }
      t_out[i] = b1;
      prim_out[i] = p1;
      if (t2_out) t2_out[i] = b2;
    }
  }
  if (counters) { counters[0] = cn.nodes; counters[1] = cn.refs; counters[2] = cn.tris; }
}

/* any hit in (EPSILON, tmax - EPSILON) with the traversal clip at tmax (rays[i*8+7]) */
void orc_trace_any(const orc_tree *tr, int64_t ntri, const float *v, const uint32_t *flags, const float *rays,
                   int64_t n, uint8_t *occ_out, uint64_t *counters) {
  orc_scene sc;
  memset(&sc, 0, sizeof(sc));
  sc.ntri = ntri; sc.v = v; sc.flags = flags;
  orc_counters cn = {0, 0, 0};
  for (int64_t i = 0; i < n; ++i) {
    const float *r = rays + i * 8;
    v3 o = V(r[0], r[1], r[2]), d = V(r[4], r[5], r[6]);
    double tmax = r[7];
    if (tr) {
      occ_out[i] = (uint8_t)kd_any(&sc, tr, o, d, tmax, counters ? &cn : NULL);
    } else {
      int hit = 0;
      for (int64_t t = 0; t < ntri && !hit; ++t) {
        double th = isect_tri(&sc, t, o, d);
        if (th < tmax - ORC_EPS && th > ORC_EPS) hit = 1;
      }
      occ_out[i] = (uint8_t)hit;
    }
  }
  if (counters) { counters[0] = cn.nodes; counters[1] = cn.refs; counters[2] = cn.tris; }
}

/* ------------------------------------------------------------------------- */
/* camera (ThinLensCamera)                                                     */
typedef struct { v3 eye, u, v, n; double tan_w, tan_h, aperture, focal_len, focal_dist; } orc_cam;

static orc_cam cam_from(const float *c) {
  /* c: eye[3], look[3], up[3], heightAngle (deg), aspect, aperture, focal length, focal distance */
  orc_cam k;
  k.eye = V(c[0], c[1], c[2]);
  v3 look = V(c[3], c[4], c[5]);
  v3 up = V(c[6], c[7], c[8]);
  double hang = c[9], aspect = c[10];
  /* setOrientation, :241-259 */
  k.n = vneg(look);
  k.u = vcross(up, k.n);
  k.n = vnorm(k.n);
  k.u = vnorm(k.u);
  k.v = vcross(k.n, k.u);
  double va = hang * (ORC_PI / 180.0);
  k.tan_h = tan(va / 2);
  k.tan_w = aspect * k.tan_h;
  k.aperture = c[11];
  k.focal_len = c[12];
  k.focal_dist = c[13];
  return k;
}

static inline v3 cam_dir(const orc_cam *k, double x, double y) {
  double nx = 2 * x - 1, ny = 1 - 2 * y;
  v3 d = vadd(vadd(vmul(k->u, k->tan_w * nx), vmul(k->v, k->tan_h * ny)), vneg(k->n));
  return vnorm(d);
}

/* ThinLensCamera::getWorldRay, M/cameras/ThinLensCamera.cpp:131-175: with an aperture the ray
 * is refocused through its focal-plane point from a lens point at radius cofRadius sin(e1),
 * angle e2, e1 = U(0, pi/2), e2 = U(0, 2 pi) (here u1, u2: the path-init draw's lanes 1, 2). */
static inline void cam_ray(const orc_cam *k, double x, double y, double u1, double u2, v3 *o, v3 *d) {
  *d = cam_dir(k, x, y);
  *o = k->eye;
  if (k->aperture > 0) {
    double t = -k->focal_dist / vdot(*d, k->n);
    if (t == k->focal_len) return;
    v3 focus = vadd(k->eye, vmul(*d, t));
    double l_image = k->focal_len * t / (t - k->focal_len);
    double cof = k->aperture * (l_image - k->focal_dist) / l_image;
    double r = cof * sin(u1 * (ORC_PI / 2));
    double e2 = u2 * (2 * ORC_PI);
    *o = vadd(vadd(k->eye, vmul(k->u, r * cos(e2))), vmul(k->v, r * sin(e2)));
    *d = vnorm(vsub(focus, *o));
  }
}

/* ------------------------------------------------------------------------- */
/* BSDFs                                                                       */

/* getOrthonormalBasis, M/common/math/Vector.inl:527-538 */
static void onb(v3 nrm, v3 *U, v3 *Vv) {
  v3 n = vnorm(nrm);
  v3 up = V(0, 1, 0);
  if (fabs(vdot(up, n)) > 0.8) up = V(1, 0, 0);
  *U = vnorm(vcross(up, n));
  *Vv = vnorm(vcross(n, *U));
}

static inline v3 from_spherical(double theta, double phi) {
  return vnorm(V(sin(theta) * cos(phi), cos(theta), sin(theta) * sin(phi)));
}

/* cosRandom, Vector.cpp:21-29 and convertHemisphere, Vector3.inl:18-21 */
static v3 cos_random(v3 nrm, double u1, double u2) {
  double theta = acos(sqrt(u1));
  double phi = 2.0 * ORC_PI * u2;
  v3 w = from_spherical(theta, phi);
  v3 U, W;
  onb(nrm, &U, &W);
  return vadd(vadd(vmul(U, w.x), vmul(vnorm(nrm), w.y)), vmul(W, w.z));
}

static inline v3 reflect_v(v3 wi, v3 n) { return vadd(vmul(n, -2 * vdot(wi, n)), wi); }

static v3 refract_v(v3 wi, v3 normal, double in, double out, int *ok) {
  v3 w = vneg(wi), norm;
  double eta;
  if (vdot(wi, normal) < 0) { norm = normal; eta = in / out; }
  else { norm = vneg(normal); eta = out / in; }
  double d = vdot(w, norm);
  double det = 1 - eta * eta * (1 - d * d);
  if (det < 0) { *ok = 0; return V(0, 0, 0); }
  *ok = 1;
  return vadd(vmul(w, -eta), vmul(norm, eta * d - sqrt(det)));
}

static double fresnel_fr_cos(double ci, double n1, double n2) {
  double snell = (n1 / n2) * sin(acos(ci));
  if (fabs(snell) >= 1) return 1;
  double ct = cos(asin(snell));
  double n1ci = n1 * ci, n1ct = n1 * ct, n2ci = n2 * ci, n2ct = n2 * ct;
  double rs = (n1ci - n2ct) / (n1ci + n2ct);
  double rp = (n1ct - n2ci) / (n1ct + n2ci);
  return (rs * rs + rp * rp) / 2.0;
}

static double fresnel_fr(v3 wi, v3 N, double n1, double n2) {
  double c = vdot(N, wi);
  if (c < 0) return fresnel_fr_cos(-c, n1, n2);
  return fresnel_fr_cos(c, n2, n1);
}

typedef struct {
  const orc_mat *m;
  v3 ns;      /* shading normal (= geometric here) */
  v3 wi;      /* incident direction (ray direction) */
  unsigned ior_index; /* 1-based as set by PathTracer */
} orc_bsdf;

enum { EV_NONE = 0, EV_DIFFUSE, EV_SPECULAR, EV_REFLECT, EV_REFRACT };

static inline double avg3(const double *a) { return (a[0] + a[1] + a[2]) / 3.0; }

/* evaluate fs(wi -> wo) */
static void bsdf_eval(const orc_bsdf *b, v3 wo, double f[3]) {
  const orc_mat *m = b->m;
  f[0] = f[1] = f[2] = 0;
  if (m->type == MAT_DIFFUSE) {
    if (vdot(b->ns, b->wi) >= 0 || vdot(b->ns, wo) <= 0) return;
    for (int k = 0; k < 3; ++k) f[k] = m->kd[k] / ORC_PI;
  } else if (m->type == MAT_PHONG) {
    if (vdot(b->ns, wo) <= 0) return;
    v3 r = reflect_v(b->wi, b->ns);
    double a = vdot(r, wo);
    if (a < 0) a = 0;
    if (a > 1) a = 1;
    double kda = avg3(m->kd), ksa = avg3(m->ks);
    double fsd = kda > 0 ? 1.0 / (ORC_PI * kda) : 0;
    for (int k = 0; k < 3; ++k) {
      double fss = ksa > 0 ? ((m->n + 2) / (2 * ORC_PI * ksa)) * pow(a, m->n) : 0;
      f[k] = m->kd[k] * fsd + m->ks[k] * fss;
    }
  }
  /* dielectric handled through lobe flags in bsdf_sample (only ever evaluated on its own sample) */
}

/* sample: returns event type (EV_NONE = absorbed), wo, fs = f/pdf (with pdf == 0 flagged) */
static int bsdf_sample(const orc_bsdf *b, const double u[3], v3 *wo, double fs[3], int *pdf_zero) {
  const orc_mat *m = b->m;
  *pdf_zero = 0;
  if (m->type == MAT_DIFFUSE) {
    if (vdot(b->ns, b->wi) > 0) return EV_NONE;
    *wo = cos_random(b->ns, u[0], u[1]);
    double c = vdot(b->ns, *wo);
    double pdf = c > 0 ? 1.0 / ORC_PI : 0;
    double f[3];
    bsdf_eval(b, *wo, f);
    if (pdf == 0) { *pdf_zero = 1; return EV_DIFFUSE; }
    for (int k = 0; k < 3; ++k) fs[k] = f[k] / pdf;
    return EV_DIFFUSE;
  }
  if (m->type == MAT_PHONG) {
    double kda = avg3(m->kd), ksa = avg3(m->ks), na = m->n;
    double p0 = u[0] - ORC_EPS;
    int ev;
    if (p0 <= kda) {
      ev = EV_DIFFUSE;
      *wo = cos_random(b->ns, u[1], u[2]);
    } else if (p0 <= kda + ksa) {
      ev = EV_SPECULAR;
      double alpha = acos(pow(u[1], 1.0 / (na + 1)));
      double phi = 2.0 * ORC_PI * u[2];
      v3 R = reflect_v(b->wi, b->ns);
      v3 r = R, uu, vv;
      if (fabs(vdot(b->ns, r)) < .95) {
        uu = vnorm(vcross(r, b->ns));
        vv = vcross(uu, r);
      } else {
        onb(r, &vv, &uu);
        r = vnorm(r);
      }
      v3 w = from_spherical(alpha, phi);
      v3 cand = vadd(vadd(vmul(uu, w.x), vmul(r, w.y)), vmul(vv, w.z));
      *wo = vdot(b->ns, cand) > 0 ? cand : R;
    } else {
      return EV_NONE;
    }
    /* getPd, :128-158 */
    double cosA = vdot(b->ns, *wo), pdf;
    if (cosA <= 0) {
      pdf = 0;
    } else if (ev == EV_SPECULAR) {
      v3 r = reflect_v(b->wi, b->ns);
      double ca = fabs(vdot(r, *wo));
      pdf = (na + 1) / (2 * ORC_PI) * pow(ca, na);
      if (pdf > 1.0) pdf = 1.0;
      pdf /= cosA;
    } else {
      pdf = (fabs(vdot(b->ns, *wo)) / ORC_PI) / cosA;
    }
    if (pdf == 0) { *pdf_zero = 1; return ev; }
    double f[3];
    bsdf_eval(b, *wo, f);
    for (int k = 0; k < 3; ++k) fs[k] = f[k] / pdf;
    return ev;
  }
  /* dielectric, :56-157 with the caller-set ior index and pdf/eval by lobe */
  v3 N = vdot(b->ns, b->wi) > 0 ? vneg(b->ns) : b->ns;
  unsigned idx = b->ior_index > 0 ? b->ior_index - 1 : 0;
  double ior = m->ior3[idx]; /* m_ior[index] (DielectricBSDF.cpp:79-87) */
  int ok;
  v3 wt = refract_v(b->wi, b->ns, ORC_AIR, ior, &ok);
  if (ok) {
    double fr = fresnel_fr(b->wi, b->ns, ORC_AIR, ior);
    double fst = m->transparency * (1 - fr);
    if (u[0] < fst) {
      *wo = wt;
      fs[0] = fs[1] = fs[2] = 0;
      fs[idx] = m->ks[idx]; /* evaluate = ks * [i == iorIndex-1], pdf = 1 */
      return EV_REFRACT;
    }
  }
  *wo = reflect_v(b->wi, N);
  for (int k = 0; k < 3; ++k) fs[k] = m->ks[k];
  return EV_REFLECT;
}

/* ------------------------------------------------------------------------- */
/* path tracer                                                                 */

typedef struct {
  int width, height, spp, nds, max_depth, rr_start, efficient_direct;
  int sample_begin, sample_count;
  uint64_t seed;
  uint32_t stream;
} orc_rparams;

typedef struct {
  const orc_scene *s;
  const orc_tree *tr;
  orc_cam cam;
  orc_rparams p;
  orc_rng rng;
} orc_render_ctx;

typedef struct {
  unsigned ior_index; /* 0..2 */
  int specular;
  double emitted_contribution;
  uint64_t path;
  uint64_t rays_ext, rays_shadow, pdf_zero, truncated;
} orc_path;

static inline int is_specular(const orc_mat *m) { return m->type == MAT_DIELECTRIC; }

/* shading normal at a hit: interpolated vertex normals with area-ratio barycentrics */
static v3 shading_normal(const orc_scene *s, int64_t tri, v3 p) {
  v3 a = tri_vert(s, tri, 0), b = tri_vert(s, tri, 1), c = tri_vert(s, tri, 2);
  double A = 1.0 / vlen(vcross(vsub(b, a), vsub(c, a)));
  double pa = vlen(vcross(vsub(b, p), vsub(c, p))) * A;
  double pb = vlen(vcross(vsub(p, a), vsub(c, a))) * A;
  double pc = 1 - pa - pb;
  v3 n = vadd(vadd(vmul(tri_nrm(s, tri, 0), pa), vmul(tri_nrm(s, tri, 1), pb)), vmul(tri_nrm(s, tri, 2), pc));
  return vnorm(n);
}

/* Analytic spheres: Milton's Sphere (Sphere.cpp), a sphere of radius 1/2 under T(center)
 * R^T S(2 radius); rays are taken to its object space, where the quadratic is solved
 * (getIntersection / intersects, Sphere.cpp:17-75, INTERSECT_TOLERANCE = EPSILON).          */
static v3 qrot(const float *q, v3 v) { /* rotation by the unit quaternion (x, y, z, w) */
  v3 u = V(q[0], q[1], q[2]);
  v3 t = vmul(vcross(u, v), 2.0);
  return vadd(vadd(v, vmul(t, q[3])), vcross(u, t));
}

static void sphere_obj(const float *sp, v3 o, v3 d, v3 *P, v3 *D) {
  double k = 1.0 / (2.0 * sp[3]);
  *P = vmul(qrot(sp + 4, vsub(o, V(sp[0], sp[1], sp[2]))), k);
  *D = vmul(qrot(sp + 4, d), k);
}

static double sphere_closest(const float *sp, v3 o, v3 d) {
  v3 P, D;
  sphere_obj(sp, o, d, &P, &D);
  double A = 2 * vdot(D, D), B = -2 * vdot(P, D), C = vdot(P, P) - 0.25;
  double disc = B * B - 2 * A * C;
  if (disc < 0) return ORC_INF;
  disc = sqrt(disc);
  double F = 1 / A, t = (B - disc) * F;
  if (t > ORC_EPS) return t;
  t = (B + disc) * F;
  return t > ORC_EPS ? t : ORC_INF;
}

static int sphere_any(const float *sp, v3 o, v3 d, double tmax) {
  v3 P, D;
  sphere_obj(sp, o, d, &P, &D);
  double A = 2 * vdot(D, D), B = -2 * vdot(P, D), C = vdot(P, P) - 0.25;
  double disc = B * B - 2 * A * C;
  if (disc < 0) return 0;
  disc = sqrt(disc);
  double F = 1 / A, t = (B + disc) * F;
  if (t < tmax && t > ORC_EPS) return 1;
  t = (B - disc) * F;
  return t < tmax && t > ORC_EPS;
}

/* closest hit among the triangles (kd-tree) and the spheres: t, and the primitive in *prim */
static double scene_closest(const orc_scene *s, const orc_tree *tr, v3 o, v3 d, int64_t *prim);
static int scene_any(const orc_scene *s, const orc_tree *tr, v3 o, v3 d, double tmax);

/* uv at a hit (Triangle::_getUV, Triangle.cpp:23-39: area-ratio barycentrics of the hit point
 * weighting the three vertex uvs; the other shapes' _getUV are affine over each of their
 * triangles, which the per-vertex uvs encode) */
static void hit_uv(const orc_scene *s, int64_t tri, v3 p, double *u, double *v) {
  *u = *v = 0.0;
  if (tri >= s->ntri) { /* Sphere::_getUV of the object-space point (Sphere.cpp:78-85) */
    const float *sp = s->sph + 8 * (tri - s->ntri);
    v3 P, D;
    sphere_obj(sp, p, V(0, 0, 1), &P, &D);
    *u = 1 - atan2(P.z, P.x) * (1 / (2 * ORC_PI));
    double y2 = 2 * P.y;
    *v = 0.5 - asin(y2 > 1 ? 1 : (y2 < -1 ? -1 : y2)) * (1 / ORC_PI);
    return;
  }
  if (!s->uv) return;
  v3 a = tri_vert(s, tri, 0), b = tri_vert(s, tri, 1), c = tri_vert(s, tri, 2);
  double A = 1.0 / vlen(vcross(vsub(b, a), vsub(c, a)));
  double pa = vlen(vcross(vsub(b, p), vsub(c, p))) * A;
  double pb = vlen(vcross(vsub(p, a), vsub(c, a))) * A;
  double pc = 1 - pa - pb;
  const float *q = s->uv + tri * 6;
  *u = pa * q[0] + pb * q[2] + pc * q[4];
  *v = pa * q[1] + pb * q[3] + pc * q[5];
}

/* lookup texel of Material::getSample / _initShadingNormal (Material.cpp:196-201, 292-299) */
static void tex_texel(const orc_tex *t, double u, double v, int *x, int *y) {
  double s = u * t->ru, r = v * t->rv;
  double fx = (s - floor(s)) * t->w, fy = (r - floor(r)) * t->h;
  fx = fx >= t->w - 1 ? t->w - 1 : (fx <= 0 ? 0 : fx);
  fy = fy >= t->h - 1 ? t->h - 1 : (fy <= 0 ? 0 : fy);
  *x = (int)floor(fx);
  *y = (int)floor(fy);
}

static inline int clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }

/* KernelFilter::apply(image, x, y) (KernelFilter.cpp:106-140) at the lookup texel */
static void tex_color(const orc_tex *t, double u, double v, double out[3]) {
  int x, y;
  tex_texel(t, u, v, &x, &y);
  int half = t->kw >> 1;
  const double *w = t->wts;
  double sum = 0, rgb[3] = {0, 0, 0};
  for (int i = -half; i <= half; ++i) {
    int row = clampi(i + y, 0, t->h - 1);
    for (int j = -half; j <= half; ++j) {
      int col = clampi(j + x, 0, t->w - 1);
      const float *px = t->rgb + ((size_t)row * t->w + col) * 3;
      double wt = *w++;
      sum += wt;
      for (int k = 0; k < 3; ++k) rgb[k] += px[k] * wt;
    }
  }
  for (int k = 0; k < 3; ++k) out[k] = rgb[k] / sum;
}

static double tex_lum(const orc_tex *t, int row, int col) {
  const float *px = t->rgb + ((size_t)row * t->w + col) * 3;
  return 0.2126 * px[0] + 0.7152 * px[1] + 0.0722 * px[2]; /* Rgba32::luminance, on byte / 255 */
}

/* Material::_initShadingNormal with a bump map (Material.cpp:179-225) */
static v3 tex_bump(const orc_tex *t, double u, double v, v3 N) {
  int x, y;
  tex_texel(t, u, v, &x, &y);
  double gx = tex_lum(t, y, x - (x > 0)) - tex_lum(t, y, x + (x < t->w - 1));
  double gy = tex_lum(t, y - (y > 0), x) - tex_lum(t, y + (y < t->h - 1), x);
  if (orc_eq(gx, 0.0) && orc_eq(gy, 0.0)) return N;
  v3 U, V2;
  onb(N, &U, &V2);
  return vnorm(vadd(N, vmul(vadd(vmul(U, gx), vmul(V2, gy)), t->intensity)));
}

/* Material::initSurfacePoint's textured inputs at a hit: kd, ks and transparency from their
 * maps (getSpectralSampleSet with a file name, Material.cpp:260-283; DielectricBSDF averages
 * the transparency, DielectricBSDF.cpp:51-52), the shading normal from the bump map */
static void apply_textures(const orc_scene *s, int64_t tri, v3 p, orc_mat *m, v3 *ns) {
  double u, v;
  hit_uv(s, tri, p, &u, &v);
  for (int k = 0; k < 3; ++k) {
    if (!m->tex[k]) continue;
    double c[3];
    tex_color(&s->tex[m->tex[k] - 1], u, v, c);
    if (k == 0) for (int q = 0; q < 3; ++q) m->kd[q] = c[q];
    else if (k == 1) for (int q = 0; q < 3; ++q) m->ks[q] = c[q];
    else m->transparency = (c[0] + c[1] + c[2]) / 3.0;
  }
  if (m->tex[3]) *ns = tex_bump(&s->tex[m->tex[3] - 1], u, v, *ns);
}

/* Scene::getBackgroundRadiance(d) = background->getLe(-d) (Scene.cpp:116-118): an
 * EnvironmentMap's lookup (EnvironmentMap.cpp:40-96: latitude-longitude uv of the direction,
 * then the material's getSample-style filtered texel) or an omni background's constant */
static void background(const orc_scene *s, v3 d, double out[3]) {
  if (!s->bg_tex) {
    for (int k = 0; k < 3; ++k) out[k] = s->bg_le[k];
    return;
  }
  v3 w = vneg(d);
  double rho = sqrt(w.x * w.x + w.z * w.z), mag = vlen(w);
  double theta = rho < fabs(w.y) ? acos(rho / mag) * (w.y >= 0 ? 1 : -1) : asin(w.y / mag);
  double phi = (w.x == 0 && w.z == 0) ? 0 : atan2(w.x, w.z);
  tex_color(&s->tex[s->bg_tex - 1], phi / (-2 * ORC_PI) + 0.5, theta / -ORC_PI + 0.5, out);
}

/* Shape::getPoint for light sample m at (u, v) (Shape.cpp:52-64): Plane::getPosition
 * (Plane.cpp:91-93); Triangle::getPosition (Triangle.cpp:332-354), whose "barycentrics" are
 * magnitudes of 2-D cross products in the triangle's uv frame; Mesh::getPosition / getPoint
 * (Mesh.cpp:436-448) with MeshTriangle::getPosition (MeshTriangle.cpp:299-333): triangle
 * min(floor(u n), n - 1), barycentrics (r1, v, r2) / (r1 + v + r2) with two more uniforms (the
 * reference draws them from its global generator; here block 0x4000 + m of the path's stream),
 * normal = the interpolated vertex normals (Mesh::_getGeometricNormal, Mesh.cpp:419-433). */
static void light_point(const orc_render_ctx *c, const orc_path *ph, int depth, int m, const orc_light *L, double u,
                        double v, v3 *pos, v3 *nrm) {
  const orc_scene *s = c->s;
  if (L->type == 1) {
    double cx = u - L->u0, cy = v - L->v0;
    double pb = fabs(cx * L->by - cy * L->bx) * L->inv_ab;
    double pc = fabs(cx * L->ay - cy * L->ax) * L->inv_ab;
    *pos = vadd(vadd(L->center, vmul(L->ex, pb)), vmul(L->ez, pc));
    *nrm = L->normal;
  } else if (L->type == 2) {
    double u4[4];
    orc_u4(&c->rng, ph->path, (uint32_t)depth, 0x4000u + (uint32_t)m, u4);
    int64_t k = (int64_t)floor(u * (double)L->count);
    if (k > L->count - 1) k = L->count - 1;
    int64_t t = L->first + k;
    double r1 = u4[0], r2 = u4[1];
    double sum = r1 + v + r2;
    double b0 = 1.0 / 3, b1 = 1.0 / 3, b2 = 1.0 / 3;
    if (sum > 0) { b0 = r1 / sum; b1 = v / sum; b2 = r2 / sum; }
    *pos = vadd(vadd(vmul(tri_vert(s, t, 0), b0), vmul(tri_vert(s, t, 1), b1)), vmul(tri_vert(s, t, 2), b2));
    *nrm = vnorm(vadd(vadd(vmul(tri_nrm(s, t, 0), b0), vmul(tri_nrm(s, t, 1), b1)), vmul(tri_nrm(s, t, 2), b2)));
  } else if (L->type == 4) {
    /* Sphere::getPosition (Sphere.cpp:114-121) in object space under T(center) R S(2 radius),
     * normal = the object point's direction (Sphere::_getGeometricNormal); the quaternion
     * (object to world) sits in the uv-frame slots, the radius in bx */
    double x = tan((1.0 - u) / (2 * ORC_PI)), y = sin((0.5 - v) / ORC_PI) * 0.5;
    x = x < -0.5 ? -0.5 : (x > 0.5 ? 0.5 : x);
    y = y < -0.5 ? -0.5 : (y > 0.5 ? 0.5 : y);
    double zz = 1 - x * x - y * y;
    float q[4] = {(float)L->u0, (float)L->v0, (float)L->ax, (float)L->ay};
    v3 pw = qrot(q, V(x, y, sqrt(zz > 0 ? zz : 0)));
    *pos = vadd(L->center, vmul(pw, 2 * L->bx));
    *nrm = vnorm(pw);
  } else if (L->type == 3) {
    *pos = L->center; /* PointShape: no normal (SurfacePoint.h:130-151: its dot product is 1) */
    *nrm = V(0, 0, 0);
  } else {
    *pos = vadd(vadd(L->center, vmul(L->ex, u - 0.5)), vmul(L->ez, v - 0.5));
    *nrm = L->normal;
  }
}

static void direct_light(const orc_render_ctx *c, orc_path *ph, int depth, v3 p, const orc_bsdf *b, int light_self,
                         double out[3]) {
  const orc_scene *s = c->s;
  out[0] = out[1] = out[2] = 0;
  if (is_specular(b->m)) return;
  int side = (int)sqrt((double)c->p.nds);
  if (side < 1) side = 1;
  for (int i = s->nlight; i--;) {
    if (i == light_self) continue;
    const orc_light *L = &s->lights[i];
    double dir[3] = {0, 0, 0};
    /* isPoint (area <= EPSILON for a PointShape): one sample, no area factor (:90-130) */
    const int point = L->type == 3;
    for (int sy = 0; sy < (point ? 1 : side); ++sy)
      for (int sx = 0; sx < (point ? 1 : side); ++sx) {
        int m = (i * side + sy) * side + sx; /* flat NEE sample index */
        double u4[4];
        orc_u4(&c->rng, ph->path, (uint32_t)depth, 1u + (uint32_t)(m >> 1), u4);
        double ux = (sx + u4[2 * (m & 1)]) / side;
        double uy = (sy + u4[2 * (m & 1) + 1]) / side;
        v3 lp, ln;
        light_point(c, ph, depth, m, L, ux, uy, &lp, &ln);
        v3 wo = vsub(lp, p);
        double t = vlen(wo);
        wo = vmul(wo, 1.0 / t);
        double cwo = fabs(vdot(b->ns, wo));
        double cwi = point ? 1.0 : fabs(vdot(ln, vneg(wo)));
        double fr[3];
        bsdf_eval(b, wo, fr);
        if (cwo > 0 && cwi > 0 && (fr[0] != 0 || fr[1] != 0 || fr[2] != 0)) {
          ph->rays_shadow++;
          /* Scene::intersects(ray, t - EPS) -> ShapeSet/kd intersects(ray, t - 2 EPS) */
          if (!scene_any(s, c->tr, p, wo, t - 2 * ORC_EPS)) {
            /* OrientedEmitter: the light's normal side only; OmniEmitter: every direction */
            double le = (L->omni || vdot(ln, vneg(wo)) > 0) ? 1.0 : 0.0;
            for (int k = 0; k < 3; ++k) dir[k] += (fr[k] * L->Le[k] * le * cwo * cwi) / (t * t);
          }
        }
      }
    for (int k = 0; k < 3; ++k) out[k] += point ? dir[k] : dir[k] * (L->area / c->p.nds);
  }
}

static double scene_closest(const orc_scene *s, const orc_tree *tr, v3 o, v3 d, int64_t *prim) {
  double t = kd_closest(s, tr, o, d, prim, NULL);
  for (int i = 0; i < s->nsph; ++i) {
    double ts = sphere_closest(s->sph + 8 * i, o, d);
    if (ts < t) {
      t = ts;
      *prim = s->ntri + i;
    }
  }
  return t;
}

static int scene_any(const orc_scene *s, const orc_tree *tr, v3 o, v3 d, double tmax) {
  for (int i = 0; i < s->nsph; ++i)
    if (sphere_any(s->sph + 8 * i, o, d, tmax)) return 1;
  return kd_any(s, tr, o, d, tmax, NULL);
}

static void evaluate(const orc_render_ctx *c, orc_path *ph, v3 o, v3 d, int depth, double out[3]) {
  const orc_scene *s = c->s;
  out[0] = out[1] = out[2] = 0;
  if (depth >= ORC_HARD_DEPTH_CAP) { ph->truncated++; return; }
  int64_t tri;
  ph->rays_ext++;
  double t = scene_closest(s, c->tr, o, d, &tri);
  if (!(t > ORC_EPS && t < ORC_INF)) { /* PathTracer.cpp:39-42: a miss adds the background */
    background(s, d, out);
    return;
  }
  v3 p = vadd(o, vmul(d, t));
  const int on_sphere = tri >= s->ntri;
  /* a sphere's normal is radial (Sphere::_getGeometricNormal with a similarity transform) */
  v3 ns = on_sphere ? vnorm(vsub(p, V(s->sph[8 * (tri - s->ntri)], s->sph[8 * (tri - s->ntri) + 1],
                                          s->sph[8 * (tri - s->ntri) + 2])))
                    : shading_normal(s, tri, p);
  const orc_mat *m = &s->mats[on_sphere ? s->sph_mat[tri - s->ntri] : s->mat[tri]];
  orc_mat mt;
  if (m->tex[0] || m->tex[1] || m->tex[2] || m->tex[3]) {
    mt = *m;
    apply_textures(s, tri, p, &mt, &ns);
    m = &mt;
  }
  orc_bsdf b = {m, ns, d, ph->ior_index + 1};
  if (is_specular(m)) ph->specular = 1;
  int li = on_sphere ? (s->sph_light ? s->sph_light[tri - s->ntri] : -1) : (s->light ? s->light[tri] : -1);
  if (li >= 0) {
    const orc_light *L = &s->lights[li];
    double le = (L->omni || vdot(ns, vneg(d)) > 0) ? 1.0 : 0.0; /* OrientedEmitter on the hit's normal */
    if (!c->p.efficient_direct || depth == 0) {
      for (int k = 0; k < 3; ++k) out[k] += L->Le[k] * le;
    } else if (ph->emitted_contribution > ORC_EPS) {
      for (int k = 0; k < 3; ++k) out[k] += L->Le[k] * le * (L->area / (t * t));
    }
  }
  if (c->p.efficient_direct) {
    double dl[3];
    direct_light(c, ph, depth, p, &b, li, dl);
    for (int k = 0; k < 3; ++k) out[k] += dl[k];
  }
  double u4[4];
  orc_u4(&c->rng, ph->path, (uint32_t)depth, 0u, u4);
  v3 wo;
  double fs[3] = {0, 0, 0};
  int pz;
  int ev = bsdf_sample(&b, u4, &wo, fs, &pz);
  if (ev == EV_NONE) return;
  if (pz) { ph->pdf_zero++; return; }
  double pc;
  if (depth < c->p.rr_start) {
    pc = (fs[0] != 0 || fs[1] != 0 || fs[2] != 0) ? 1.0 : 0.0;
  } else {
    int mi = 0;
    double mv = fs[0];
    for (int k = 1; k < 3; ++k) if (fs[k] > mv) { mv = fs[k]; mi = k; }
    pc = mv < .95 ? mv : .95; /* MIN(.95, fs[fs.getMaxSample()]) */
    (void)mi;
  }
  if (c->p.max_depth > 0 && depth + 1 >= c->p.max_depth) return;
  if (u4[3] < pc) {
    ph->emitted_contribution = is_specular(m) ? vdot(ns, wo) : 0;
    double li3[3];
    evaluate(c, ph, p, wo, depth + 1, li3);
    for (int k = 0; k < 3; ++k) out[k] += fs[k] * li3[k] / pc;
    if (depth == 0 && ph->specular) {
      for (int k = 0; k < 3; ++k) out[k] = (k == (int)ph->ior_index) ? out[k] * 3 : 0;
    }
  }
}

/* Work is handed out in spans of ORC_SPAN pixels of one row (not whole rows), so that a sample
 * of a few rows still keeps every host thread busy. */
#define ORC_SPAN 32

typedef struct {
  const orc_render_ctx *c;
  int row_begin, row_end;
  int64_t *next_span; /* shared work counter: spans of ORC_SPAN pixels, row-major from row_begin */
  pthread_mutex_t *lock;
  double *film;       /* width*height*3 sums */
  double *path_out;   /* optional per-path radiance: (pixel - row_begin * width) * sample_count + s, 3 each */
  uint64_t stats[4];
} orc_job;

static void render_span(orc_job *j, int y, int x0, int x1) {
  const orc_render_ctx *c = j->c;
  int W = c->p.width, H = c->p.height;
  int side = (int)sqrt((double)c->p.spp);
  if (side < 1) side = 1;
  int s2 = side * side;
  for (int x = x0; x < x1; ++x) {
    uint64_t pix = (uint64_t)y * W + x;
    double acc[3] = {0, 0, 0};
    for (int si = 0; si < c->p.sample_count; ++si) {
      int s = c->p.sample_begin + si;
      int k = s % s2;
      double jit[4];
      orc_u4(&c->rng, pix * (uint64_t)s2 + (uint64_t)k, ORC_DEPTH_JITTER, 0u, jit);
      double px = (x + ((k % side) + jit[0]) / side) / W;
      double py = (y + ((k / side) + jit[1]) / side) / H;
      orc_path ph;
      memset(&ph, 0, sizeof(ph));
      ph.path = pix * (uint64_t)c->p.spp + (uint64_t)s;
      double ui[4];
      orc_u4(&c->rng, ph.path, ORC_DEPTH_PATHINIT, 0u, ui);
      ph.ior_index = (unsigned)floor(ui[0] * 3.0);
      if (ph.ior_index > 2) ph.ior_index = 2;
      v3 o, d;
      cam_ray(&c->cam, px, py, ui[1], ui[2], &o, &d);
      double L[3];
      evaluate(c, &ph, o, d, 0, L);
      for (int k3 = 0; k3 < 3; ++k3) acc[k3] += L[k3];
      if (j->path_out) {
        uint64_t band_pix = pix - (uint64_t)j->row_begin * (uint64_t)W;
        double *po = j->path_out + (band_pix * (uint64_t)c->p.sample_count + (uint64_t)si) * 3;
        po[0] = L[0]; po[1] = L[1]; po[2] = L[2];
      }
      j->stats[0] += ph.rays_ext;
      j->stats[1] += ph.rays_shadow;
      j->stats[2] += ph.pdf_zero;
      j->stats[3] += ph.truncated;
    }
    for (int k3 = 0; k3 < 3; ++k3) j->film[pix * 3 + k3] += acc[k3];
  }
}

static void *render_thread(void *arg) {
  orc_job *j = (orc_job *)arg;
  const int W = j->c->p.width;
  const int64_t per_row = (W + ORC_SPAN - 1) / ORC_SPAN;
  const int64_t total = per_row * (int64_t)(j->row_end - j->row_begin);
  for (;;) {
    pthread_mutex_lock(j->lock);
    int64_t k = (*j->next_span)++;
    pthread_mutex_unlock(j->lock);
    if (k >= total) break;
    int y = j->row_begin + (int)(k / per_row);
    int x0 = (int)(k % per_row) * ORC_SPAN;
    render_span(j, y, x0, x0 + ORC_SPAN < W ? x0 + ORC_SPAN : W);
  }
  return NULL;
}

/* Render sample passes [sample_begin, sample_begin + sample_count) of every pixel in rows
 * [row_begin, row_end).  film_sum receives per-pixel radiance sums (divide by sample_count for
 * the mean).  ip: width, height, spp, nds, max_depth (0 = none), rr_start, efficient_direct,
 * sample_begin, sample_count, row_begin, row_end, nthreads.  stats_out: extension rays, shadow
 * rays, zero-pdf terminations, truncated paths.  Every pixel is evaluated by exactly one thread
 * with its own counter-based random numbers, so the result does not depend on nthreads.     */
int orc_render(int64_t ntri, const float *v, const float *n, const int32_t *mat, const int32_t *light,
               const uint32_t *flags, int nmat, const float *mats, int nlight, const float *lights,
               const float *light_ext, const float *tri_uv, int ntex, const float *tex_params,
               const float *const *tex_rgb, const float *bg, int nsph, const float *sph, const int32_t *sph_mat,
               const int32_t *sph_light, const orc_tree *tr, const float *camera, const int32_t *ip, uint64_t seed, uint32_t stream,
               double *film_sum, double *path_out, uint64_t *stats_out) {
  orc_scene *s = scene_from_arrays(ntri, v, n, mat, light, flags, nmat, mats, nlight, lights, light_ext);
  s->uv = tri_uv;
  s->ntex = ntex;
  s->tex = textures_from(ntex, tex_params, tex_rgb);
  /* bg: 1 + background texture, then the constant background radiance (NULL = black) */
  if (bg) {
    s->bg_tex = (int)bg[0];
    for (int k = 0; k < 3; ++k) s->bg_le[k] = bg[1 + k];
  }
  s->nsph = nsph;
  s->sph = sph;
  s->sph_mat = sph_mat;
  s->sph_light = sph_light;
  orc_render_ctx c;
  c.s = s;
  c.tr = tr;
  c.cam = cam_from(camera);
  c.p.width = ip[0]; c.p.height = ip[1]; c.p.spp = ip[2]; c.p.nds = ip[3];
  c.p.max_depth = ip[4]; c.p.rr_start = ip[5]; c.p.efficient_direct = ip[6];
  c.p.sample_begin = ip[7]; c.p.sample_count = ip[8];
  int row0 = ip[9], row1 = ip[10], nth = ip[11];
  c.p.seed = seed;
  c.p.stream = stream;
  c.rng.key[0] = (uint32_t)seed;
  c.rng.key[1] = (uint32_t)(seed >> 32);
  c.rng.stream = stream;
  if (nth < 1) nth = 1;
  orc_job *jobs = (orc_job *)calloc(nth, sizeof(orc_job));
  pthread_t *th = (pthread_t *)calloc(nth, sizeof(pthread_t));
  pthread_mutex_t lock;
  pthread_mutex_init(&lock, NULL);
  int64_t next = 0;
  for (int t = 0; t < nth; ++t) {
    jobs[t].c = &c; jobs[t].film = film_sum; jobs[t].path_out = path_out;
    jobs[t].row_begin = row0; jobs[t].row_end = row1; jobs[t].next_span = &next; jobs[t].lock = &lock;
  }
  for (int t = 1; t < nth; ++t) pthread_create(&th[t], NULL, render_thread, &jobs[t]);
  render_thread(&jobs[0]);
  for (int t = 1; t < nth; ++t) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&lock);
  if (stats_out) {
    memset(stats_out, 0, sizeof(uint64_t) * 4);
    for (int t = 0; t < nth; ++t)
      for (int k = 0; k < 4; ++k) stats_out[k] += jobs[t].stats[k];
  }
  free(jobs);
  free(th);
  scene_free(s);
  return 0;
}

/* per-sample helpers exposed for unit tests of the restated pieces */
/* camera ray with the thin lens: camera = 16 floats, (u1, u2) the lens lanes */
void orc_camera_ray(const float *camera, double x, double y, double u1, double u2, double o_out[3],
                    double d_out[3]) {
  orc_cam k = cam_from(camera);
  v3 o, d;
  cam_ray(&k, x, y, u1, u2, &o, &d);
  o_out[0] = o.x; o_out[1] = o.y; o_out[2] = o.z;
  d_out[0] = d.x; d_out[1] = d.y; d_out[2] = d.z;
}

void orc_camera_dir(const float *camera, double x, double y, double out[3]) {
  orc_cam k = cam_from(camera);
  v3 d = cam_dir(&k, x, y);
  out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

/* bsdf sample for a single configuration: mat16 = material record, ns, wi, ior_index (0..2),
 * u[3]; writes wo[3], fs[3]; returns event code (0 none, 1 diffuse, 2 phong-specular,
 * 3 reflect, 4 refract, -1 zero pdf)                                                      */
int orc_bsdf_sample(const float *mat16, const double *ns, const double *wi, int ior_index, const double *u,
                    double *wo_out, double *fs_out) {
  orc_mat m;
  m.type = (int)mat16[0];
  for (int k = 0; k < 3; ++k) { m.kd[k] = mat16[1 + k]; m.ks[k] = mat16[4 + k]; }
  m.n = mat16[7]; m.ior = mat16[8]; m.transparency = mat16[9];
  mat_ior3(&m, mat16);
  orc_bsdf b = {&m, V(ns[0], ns[1], ns[2]), V(wi[0], wi[1], wi[2]), (unsigned)ior_index + 1};
  v3 wo = V(0, 0, 0);
  double fs[3] = {0, 0, 0};
  int pz;
  int ev = bsdf_sample(&b, u, &wo, fs, &pz);
  wo_out[0] = wo.x; wo_out[1] = wo.y; wo_out[2] = wo.z;
  for (int k = 0; k < 3; ++k) fs_out[k] = fs[k];
  return pz ? -1 : ev;
}

void orc_bsdf_eval(const float *mat16, const double *ns, const double *wi, const double *wo, double *f_out) {
  orc_mat m;
  m.type = (int)mat16[0];
  for (int k = 0; k < 3; ++k) { m.kd[k] = mat16[1 + k]; m.ks[k] = mat16[4 + k]; }
  m.n = mat16[7]; m.ior = mat16[8]; m.transparency = mat16[9];
  mat_ior3(&m, mat16);
  orc_bsdf b = {&m, V(ns[0], ns[1], ns[2]), V(wi[0], wi[1], wi[2]), 1};
  bsdf_eval(&b, V(wo[0], wo[1], wo[2]), f_out);
}

/* One texture lookup at (u, v): params = the 12 floats of orc_render's tex_params.  Colour
 * maps write the filtered rgb to out[0..2]; bump maps write the luminance differences (gx, gy)
 * to out[0..1] and the bumped normal of N = n_in to out[2..4] (n_in may be NULL). */
void orc_texture_lookup(const float *params, const float *rgb, double u, double v, const double *n_in, double *out) {
  orc_tex *t = textures_from(1, params, &rgb);
  if (t->kind == 0) {
    tex_color(t, u, v, out);
  } else {
    int x, y;
    tex_texel(t, u, v, &x, &y);
    out[0] = tex_lum(t, y, x - (x > 0)) - tex_lum(t, y, x + (x < t->w - 1));
    out[1] = tex_lum(t, y - (y > 0), x) - tex_lum(t, y + (y < t->h - 1), x);
    if (n_in) {
      v3 nb = tex_bump(t, u, v, vnorm(V(n_in[0], n_in[1], n_in[2])));
      out[2] = nb.x; out[3] = nb.y; out[4] = nb.z;
    }
  }
  free(t->wts);
  free(t);
}

/* Sphere::getIntersection of one sphere record (8 floats) for the ray (o, d) (tests) */
double orc_sphere_closest(const float *sp, const double *o, const double *d) {
  return sphere_closest(sp, V(o[0], o[1], o[2]), V(d[0], d[1], d[2]));
}

/* background radiance of a ray with direction d (tests): params / rgb describe the environment
 * map (NULL: constant le) */
void orc_background(const float *params, const float *rgb, const double *le, const double *d, double *out) {
  orc_scene s;
  memset(&s, 0, sizeof(s));
  if (params) {
    s.ntex = 1;
    s.tex = textures_from(1, params, &rgb);
    s.bg_tex = 1;
  } else {
    for (int k = 0; k < 3; ++k) s.bg_le[k] = le[k];
  }
  background(&s, V(d[0], d[1], d[2]), out);
  if (s.tex) {
    free(s.tex[0].wts);
    free(s.tex);
  }
}

void orc_uniforms(uint64_t seed, uint32_t stream, uint64_t path, uint32_t depth, uint32_t block, double *u4) {
  orc_rng g;
  g.key[0] = (uint32_t)seed;
  g.key[1] = (uint32_t)(seed >> 32);
  g.stream = stream;
  orc_u4(&g, path, depth, block, u4);
}
