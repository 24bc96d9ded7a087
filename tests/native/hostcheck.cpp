// hostcheck.cpp -- test harness: the product's host/device traversal and shading code
// (milton_gb300/csrc/hd_*.h) compiled for the CPU, so that the FP32 arithmetic the kernels run
// can be checked against the oracle without a GPU.  Test infrastructure only; it is not part of
// libmgpu.so and nothing in the product calls it.
#include <cmath>
#include <string.h>

#include "../../milton_gb300/csrc/hd_shade.h"
#include "../../milton_gb300/csrc/hd_trace.h"
#include "../../milton_gb300/csrc/kdbuild.h"

using namespace mgpu;

extern "C" {

// Builds the product tree over v (ntri*9) and traces n rays (n*8 floats) with the FP32 traversal.
// hits: n*4 floats (t, prim bits, b1, b2); occ: n bytes (any hit); counts: n*4 uint32.
int hc_trace_kd(const float *v, const uint32_t *flags, int64_t ntri, const float *rays, int64_t n, float *hits,
                uint8_t *occ, uint32_t *counts, uint32_t max_depth, int use_top, uint32_t min_prims, double cost_trav,
                double empty_bias);

int hc_trace(const float *v, const uint32_t *flags, int64_t ntri, const float *rays, int64_t n, float *hits,
             uint8_t *occ, uint32_t *counts, uint32_t max_depth, int use_top) {
  return hc_trace_kd(v, flags, ntri, rays, n, hits, occ, counts, max_depth, use_top, 3, 1.0, 0.9);
}

// same, with the kd build parameters exposed
int hc_trace_kd(const float *v, const uint32_t *flags, int64_t ntri, const float *rays, int64_t n, float *hits,
                uint8_t *occ, uint32_t *counts, uint32_t max_depth, int use_top, uint32_t min_prims, double cost_trav,
                double empty_bias) {
  KdParams p;
  p.max_depth = max_depth;
  p.min_prims = min_prims;
  p.cost_traversal = cost_trav;
  p.empty_bias = empty_bias;
  KdTree t;
  const char *err = nullptr;
  if (!kd_build(v, ntri, p, t, &err)) return -1;
  std::vector<F4> tris((size_t)ntri * 3);
  for (int64_t i = 0; i < ntri; ++i)
    for (int k = 0; k < 3; ++k) {
      F4 q; q.x = v[i * 9 + 3 * k]; q.y = v[i * 9 + 3 * k + 1]; q.z = v[i * 9 + 3 * k + 2]; q.w = 0.0f;
      if (k == 0 && flags) memcpy(&q.w, &flags[i], 4);
      tris[3 * i + k] = q;
    }
  std::vector<Pair> dpairs;
  std::vector<F4> ltris;
  kd_device_layout(t, v, flags, dpairs, ltris);
  SceneView s;
  s.pairs = dpairs.data();
  s.ltris = ltris.data();
  s.tris = tris.data();
  for (int k = 0; k < 3; ++k) { s.bmin[k] = (float)t.bmin[k]; s.bmax[k] = (float)t.bmax[k]; }
  s.ntri = ntri;
  s.npairs = t.pairs.size();
  s.nrefs = ltris.size() / 3;
  s.spheres = nullptr;
  s.nsphere = 0;
  const Pair *top = use_top ? dpairs.data() : nullptr;
  uint32_t ntop = use_top ? t.top_pairs : 0;
  for (int64_t i = 0; i < n; ++i) {
    const float *r = rays + 8 * i;
    Ray ray;
    ray.o = v3(r[0], r[1], r[2]);
    ray.tmin = r[3];
    ray.d = v3(r[4], r[5], r[6]);
    ray.tmax = r[7];
    Hit h;
    TraceCounts c = {0, 0, 0, 0};
    if (hits) {
      bool hit = traverse<false, true>(s, ray, h, top, ntop, &c);
      hits[4 * i + 0] = hit ? h.t : INFINITY;
      int32_t pr = hit ? h.prim : -1;
      memcpy(&hits[4 * i + 1], &pr, 4);
      hits[4 * i + 2] = h.b1;
      hits[4 * i + 3] = h.b2;
      if (counts) { counts[4 * i] = c.nodes; counts[4 * i + 1] = c.refs; counts[4 * i + 2] = c.tris; counts[4 * i + 3] = c.max_stack; }
    }
    if (occ) occ[i] = traverse<true, false>(s, ray, h, top, ntop, nullptr) ? 1 : 0;
  }
  return 0;
}

int hc_bsdf_sample(const float *mat16, const float *ns, const float *wi, int ior_index, const float *u, float *wo_out,
                   float *fs_out) {
  Material m = material_from(mat16, (uint32_t)ior_index);
  V3 wo = v3(0, 0, 0), fs;
  int ev = bsdf_sample(m, v3(ns[0], ns[1], ns[2]), v3(wi[0], wi[1], wi[2]), (uint32_t)ior_index, u[0], u[1], u[2], wo, fs);
  wo_out[0] = wo.x; wo_out[1] = wo.y; wo_out[2] = wo.z;
  fs_out[0] = fs.x; fs_out[1] = fs.y; fs_out[2] = fs.z;
  return ev;
}

void hc_bsdf_eval(const float *mat16, const float *ns, const float *wi, const float *wo, float *f) {
  Material m = material_from(mat16);
  V3 r = bsdf_eval(m, v3(ns[0], ns[1], ns[2]), v3(wi[0], wi[1], wi[2]), v3(wo[0], wo[1], wo[2]));
  f[0] = r.x; f[1] = r.y; f[2] = r.z;
}

void hc_uniforms(uint64_t seed, uint32_t stream, uint64_t path, uint32_t depth, uint32_t block, float *u4) {
  Rng g; g.k0 = (uint32_t)seed; g.k1 = (uint32_t)(seed >> 32); g.stream = stream;
  F4u u = uniforms(g, path, depth, block);
  u4[0] = u.a; u4[1] = u.b; u4[2] = u.c; u4[3] = u.d;
}

void hc_offset(const float *p, const float *n, float *out) {
  V3 o = offset_origin(v3(p[0], p[1], p[2]), v3(n[0], n[1], n[2]));
  out[0] = o.x; out[1] = o.y; out[2] = o.z;
}

// camera_ray on the host: camera16 as the render parameters carry it; out: o[3], d[3]
void hc_camera_ray(const float *c, float x, float y, float u1, float u2, float *out) {
  // setOrientation / _computeMatrix as make_camera does on the host side of the library
  double n[3] = {-c[3], -c[4], -c[5]}, up[3] = {c[6], c[7], c[8]};
  double u[3] = {up[1] * n[2] - up[2] * n[1], up[2] * n[0] - up[0] * n[2], up[0] * n[1] - up[1] * n[0]};
  double ln = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]), lu = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  for (int k = 0; k < 3; ++k) { n[k] /= ln; u[k] /= lu; }
  double v[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2], n[0] * u[1] - n[1] * u[0]};
  double th = tan(c[9] * (3.14159265358979323846 / 180.0) / 2);
  Camera k;
  k.eye = v3(c[0], c[1], c[2]);
  k.u = v3((float)u[0], (float)u[1], (float)u[2]);
  k.v = v3((float)v[0], (float)v[1], (float)v[2]);
  k.n = v3((float)n[0], (float)n[1], (float)n[2]);
  k.tan_h = (float)th;
  k.tan_w = (float)(c[10] * th);
  k.aperture = c[11];
  k.focal_len = c[12];
  k.focal_dist = c[13];
  V3 o, d;
  camera_ray(k, x, y, u1, u2, o, d);
  out[0] = o.x; out[1] = o.y; out[2] = o.z;
  out[3] = d.x; out[4] = d.y; out[5] = d.z;
}

// light_point on the host: rec16 + ext16 light record, (u, v, r1, r2); tri_v / tri_n the soup
// (9 floats per triangle) for mesh lights.  out: position[3], normal[3].
void hc_light_point(const float *rec16, const float *ext16, const float *uvr, const float *tri_v, const float *tri_n,
                    float *out) {
  Light L = light_from(rec16, ext16);
  V3 p, n, g;
  light_point(
      L, uvr[0], uvr[1], uvr[2], uvr[3],
      [&](uint32_t t, int c) { const float *q = tri_v + 9 * (size_t)t + 3 * c; return v3(q[0], q[1], q[2]); },
      [&](uint32_t t, int c) { const float *q = tri_n + 9 * (size_t)t + 3 * c; return v3(q[0], q[1], q[2]); }, p, n,
      g);
  out[0] = p.x; out[1] = p.y; out[2] = p.z;
  out[3] = n.x; out[4] = n.y; out[5] = n.z;
}

}  // extern "C"
