// hd_shade.h -- camera rays, Milton's BSDFs and emitters, area-light sampling (host/device).
//
// FP32 restatement of the shading half of PathTracer::_evaluate.  Each function names the
// Milton routine whose behaviour it reproduces; lobe choice and pdf follow the reference
// exactly (including its quirks), only the precision differs.
#pragma once

#include "hd_math.h"

namespace mgpu {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kEps = 1e-7f;      // Milton's EPSILON, used where it shapes sampling (Phong lobe pick)
constexpr float kAir = 1.0003f;    // IndexOfRefraction::AIR (IndexOfRefraction.cpp:16)

// Material record (16 floats, 4 x float4 in device memory)
struct Material {
  int type;          // 0 diffuse, 1 modified Phong, 2 dielectric
  V3 kd, ks;
  float n, ior, transparency;
  float kda, ksa;    // channel averages (ModifiedPhongBSDF::init)
  int tex_kd, tex_ks, tex_tr, tex_bump;  // 1 + texture index, 0 = none
};

// ior_index: the path's colour channel (0..2).  A dielectric refracts with that channel's IOR
// (DielectricBSDF.cpp:79-87): record [8] (all channels when [14] = [15] = 0), [14], [15].
MGPU_HD Material material_from(const float *m, uint32_t ior_index = 0) {
  Material r;
  r.type = (int)m[0];
  r.kd = v3(m[1], m[2], m[3]);
  r.ks = v3(m[4], m[5], m[6]);
  r.n = m[7];
  r.ior = (ior_index == 0 || (m[14] == 0.0f && m[15] == 0.0f)) ? m[8] : (ior_index == 1 ? m[14] : m[15]);
  r.transparency = m[9];
  r.kda = (r.kd.x + r.kd.y + r.kd.z) / 3.0f;
  r.ksa = (r.ks.x + r.ks.y + r.ks.z) / 3.0f;
  r.tex_kd = (int)m[10];
  r.tex_ks = (int)m[11];
  r.tex_tr = (int)m[12];
  r.tex_bump = (int)m[13];
  return r;
}

// Texel of a lookup at (u, v) in a width x height map repeated (ru, rv) times: Milton's
// getSample / _initShadingNormal position, x = clamp((s - floor(s)) width, 0, width - 1) with
// s = u ru, floored (Material.cpp:196-201, 292-299).
MGPU_HD int tex_texel(float u, float v, int w, int h, float ru, float rv) {
  const float s = u * ru, t = v * rv;
  const float x = fminf(fmaxf((s - floorf(s)) * (float)w, 0.0f), (float)(w - 1));
  const float y = fminf(fmaxf((t - floorf(t)) * (float)h, 0.0f), (float)(h - 1));
  return (int)y * w + (int)x;
}

// uv of Milton's latitude-longitude EnvironmentMap in direction w (EnvironmentMap.cpp:62-86):
// theta = asin(y / |w|) (acos(rho / |w|) with y's sign where rho = |(x, z)| < |y|), phi =
// atan2(x, z) (0 on the y axis), u = phi / (-2 pi) + 1/2, v = theta / -pi + 1/2.
MGPU_HD void env_uv(V3 w, float &u, float &v) {
  const float rho = sqrtf(w.x * w.x + w.z * w.z), mag = length(w);
  const float theta = rho < fabsf(w.y) ? acosf(rho / mag) * (w.y >= 0.0f ? 1.0f : -1.0f) : asinf(w.y / mag);
  const float phi = (w.x == 0.0f && w.z == 0.0f) ? 0.0f : atan2f(w.x, w.z);
  u = phi / (-2.0f * kPi) + 0.5f;
  v = theta / -kPi + 0.5f;
}

// Sphere::_getUV (Sphere.cpp:78-85) of an object-space point p of the unit-diameter sphere:
// u = 1 - atan2(z, x) / 2 pi, v = 1/2 - asin(2 y) / pi.
MGPU_HD void sphere_uv(V3 p, float &u, float &v) {
  u = 1.0f - atan2f(p.z, p.x) * (1.0f / (2.0f * kPi));
  v = 0.5f - asinf(fminf(fmaxf(2.0f * p.y, -1.0f), 1.0f)) * (1.0f / kPi);
}

// Textured keys replace the constants (Material::getSpectralSampleSet with a file name,
// Material.cpp:260-283); DielectricBSDF uses the average transparency (DielectricBSDF.cpp:51-52).
MGPU_HD void tex_apply(Material &m, int slot, float r, float g, float b) {
  if (slot == 0) {
    m.kd = v3(r, g, b);
    m.kda = (r + g + b) / 3.0f;
  } else if (slot == 1) {
    m.ks = v3(r, g, b);
    m.ksa = (r + g + b) / 3.0f;
  } else {
    m.transparency = (r + g + b) / 3.0f;
  }
}

MGPU_HD bool is_specular(const Material &m) { return m.type == 2; }

// Rotation of v by the unit quaternion q = (x, y, z, w): v + 2 w (u x v) + 2 u x (u x v), u = q.xyz.
MGPU_HD V3 quat_rotate(float qx, float qy, float qz, float qw, V3 v) {
  const V3 u = v3(qx, qy, qz);
  const V3 t = cross(u, v) * 2.0f;
  return v + t * qw + cross(u, t);
}

// Light: a Milton `Plane` under a transform (type 0), a standalone `Triangle` (type 1), a `Mesh`
// (type 2), a `PointShape` (type 3, area 0) or a `Sphere` (type 4: quaternion in the uv-frame
// slots u0, v0, ax, ay, radius in bx).  Record: 16 floats (center / v1, ex, ez, normal,
// area, Le) + 16 extension floats (type, triangle uv frame, mesh triangle run, [15] omni).
constexpr int kLightPlane = 0, kLightTriangle = 1, kLightMesh = 2, kLightPoint = 3, kLightSphere = 4;
constexpr uint32_t kMeshLightBlock = 0x4000u;  // RNG block of a mesh light sample's extra pair

struct Light {
  V3 center, ex, ez, normal;
  float area;
  V3 Le;
  int type;
  float u0, v0, ax, ay, bx, by, inv_ab;  // Triangle: uv0, a = uv1 - uv0, b = uv2 - uv0, 1/|a x b|
  uint32_t first, count;                  // Mesh: triangle run in the soup
  bool omni;                              // OmniEmitter: emits on both sides (and points)
};

MGPU_HD Light light_from(const float *l, const float *x) {
  Light r;
  r.center = v3(l[0], l[1], l[2]);
  r.ex = v3(l[3], l[4], l[5]);
  r.ez = v3(l[6], l[7], l[8]);
  r.normal = normalize(v3(l[9], l[10], l[11]));
  r.area = l[12];
  r.Le = v3(l[13], l[14], l[15]);
  r.type = (int)x[0];
  r.u0 = x[1]; r.v0 = x[2]; r.ax = x[3]; r.ay = x[4]; r.bx = x[5]; r.by = x[6]; r.inv_ab = x[7];
  r.first = f_bits(x[8]);
  r.count = f_bits(x[9]);
  r.omni = x[15] != 0.0f || r.type == kLightPoint;
  return r;
}

// Shape::getPoint for a light sample (u, v): position and normal.  Plane::getPosition
// (Plane.cpp:91-93); Triangle::getPosition with its uv frame (Triangle.cpp:332-354: both
// "barycentrics" are magnitudes of 2-D cross products, so (u, v) outside the uv triangle maps
// outside the triangle, as in the reference); Mesh::getPosition / MeshTriangle::getPosition
// (Mesh.cpp:436-448, MeshTriangle.cpp:299-333): triangle floor(u count), barycentrics
// (r1, v, r2) / (r1 + v + r2).  vert(i, k) / nrm(i, k) read vertex k of soup triangle i.
// n is the emitter's normal at p (a mesh's interpolated vertex normals), g the normal of the
// surface p lies on (unoriented), for moving the shadow ray's end off it.
template <class Vert, class Nrm>
MGPU_HD void light_point(const Light &L, float u, float v, float r1, float r2, Vert vert, Nrm nrm, V3 &p, V3 &n,
                         V3 &g) {
  if (L.type == kLightTriangle) {
    const float cx = u - L.u0, cy = v - L.v0;
    const float pb = fabsf(cx * L.by - cy * L.bx) * L.inv_ab;
    const float pc = fabsf(cx * L.ay - cy * L.ax) * L.inv_ab;
    p = L.center + L.ex * pb + L.ez * pc;
    n = L.normal;
    g = L.normal;
  } else if (L.type == kLightMesh) {
    uint32_t k = (uint32_t)floorf(u * (float)L.count);
    if (k > L.count - 1u) k = L.count - 1u;
    const uint32_t t = L.first + k;
    float s = r1 + v + r2;
    float b0 = 1.0f / 3.0f, b1 = 1.0f / 3.0f, b2 = 1.0f / 3.0f;
    if (s > 0.0f) {
      const float is = rcp(s);
      b0 = r1 * is; b1 = v * is; b2 = r2 * is;
    }
    const V3 a = vert(t, 0), b = vert(t, 1), c = vert(t, 2);
    p = a * b0 + b * b1 + c * b2;
    n = normalize(nrm(t, 0) * b0 + nrm(t, 1) * b1 + nrm(t, 2) * b2);
    g = normalize(cross(b - a, c - a));
  } else if (L.type == kLightSphere) {
    // Sphere::getPosition (Sphere.cpp:114-121) in object space, under T(center) R S(2 radius);
    // the normal is the object point's direction (Sphere::_getGeometricNormal).  The point lies
    // off the sphere, as in the reference, so there is no surface to move the shadow ray off.
    const float x = fminf(fmaxf(tanf((1.0f - u) / (2.0f * kPi)), -0.5f), 0.5f);
    const float y = fminf(fmaxf(sinf((0.5f - v) / kPi) * 0.5f, -0.5f), 0.5f);
    const V3 po = v3(x, y, sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y)));
    const V3 pw = quat_rotate(L.u0, L.v0, L.ax, L.ay, po);  // uv-frame slots hold the quaternion
    p = L.center + pw * (2.0f * L.bx);
    n = normalize(pw);
    g = v3(0.0f, 0.0f, 0.0f);
  } else if (L.type == kLightPoint) {
    // PointShape: the point itself, no normal (SurfacePoint's stand-in dot product is 1) and no
    // surface to move the shadow ray's end off
    p = L.center;
    n = v3(0.0f, 0.0f, 0.0f);
    g = n;
  } else {
    p = L.center + L.ex * (u - 0.5f) + L.ez * (v - 0.5f);
    n = L.normal;
    g = L.normal;
  }
}

// Pinhole camera (ThinLensCamera::getWorldRay with aperture 0, ThinLensCamera.cpp:131-135)
struct Camera {
  V3 eye, u, v, n;
  float tan_w, tan_h;
  float aperture, focal_len, focal_dist;  // thin lens (aperture 0 = pinhole)
};

MGPU_HD V3 camera_dir(const Camera &c, float x, float y) {
  float nx = 2.0f * x - 1.0f, ny = 1.0f - 2.0f * y;
  return normalize(c.u * (c.tan_w * nx) + c.v * (c.tan_h * ny) - c.n);
}

// ThinLensCamera::getWorldRay (ThinLensCamera.cpp:131-175): the pinhole direction through the
// film point; with an aperture, the ray is refocused through the point where it meets the
// focal plane, from an origin shifted by r = cofRadius sin(e1) at angle e2 on the lens
// (e1 = u1 pi/2, e2 = u2 2 pi: the reference's radius distribution, not a uniform disc).
MGPU_HD void camera_ray(const Camera &c, float x, float y, float u1, float u2, V3 &o, V3 &d) {
  d = camera_dir(c, x, y);
  o = c.eye;
  if (c.aperture > 0.0f) {
    const float t = c.focal_dist / -dot(d, c.n);
    if (t == c.focal_len) return;
    const V3 focus = c.eye + d * t;
    const float l_image = c.focal_len * t / (t - c.focal_len);
    const float cof = c.aperture * (l_image - c.focal_dist) / l_image;
    const float r = cof * sinf(u1 * (0.5f * kPi));
    const float e2 = u2 * (2.0f * kPi);
    o = c.eye + c.u * (r * cosf(e2)) + c.v * (r * sinf(e2));
    d = normalize(focus - o);
  }
}

// Reconstruction filters of ReconstructionRenderOutput (M/filters/BoxFilter.cpp,
// TriangleFilter.cpp, GaussianFilter.cpp, MitchellFilter.cpp, LanczosSincFilter.cpp), evaluated
// at the offset from a sample's film position to a pixel's integer coordinates, as
// ReconstructionRenderOutput::addSample does (ReconstructionRenderOutput.cpp:30-83), quirks
// included (the triangle filter is not mirrored for negative offsets; Mitchell's outer branch
// has no 1/6 and no cut-off).  half = (ceil(support) | 1) >> 1 (KernelFilter.h:28).
constexpr int kFilterNone = 0, kFilterBox = 1, kFilterTriangle = 2, kFilterGaussian = 3, kFilterMitchell = 4,
              kFilterLanczos = 5;

struct FilmFilter {
  int type, half;
  float support, p1, p2;  // gaussian: sigma; mitchell: B, C; lanczosSinc: tau
};

MGPU_HD float mitchell_1d(float x, float support, float B, float C) {
  x = fabsf(2.0f * x / support);
  if (x > 1.0f)
    return (((-B / 6.0f - C) * x + (B + 5.0f * C)) * x + (-2.0f * B - 8.0f * C)) * x + (4.0f / 3.0f * B + 4.0f * C);
  return x * x * ((2.0f - 1.5f * B - C) * x + (-3.0f + 2.0f * B + C)) + (1.0f - B / 3.0f);
}

MGPU_HD float lanczos_1d(float x, float support, float tau) {
  x = fabsf(x / support);
  if (x < kEps) return 1.0f;
  if (x > 1.0f) return 0.0f;
  x *= kPi;
  return sinf(x * tau) / (x * tau) * (sinf(x) / x);
}

MGPU_HD float filter_eval(const FilmFilter &f, float dx, float dy) {
  switch (f.type) {
    case kFilterBox:
      return 2.0f * sqrtf(dx * dx + dy * dy) < f.support ? 1.0f : 0.0f;
    case kFilterTriangle: {
      const float r = f.support / 2.0f;
      return fmaxf(0.0f, 1.0f - dx / r) * fmaxf(0.0f, 1.0f - dy / r);
    }
    case kFilterGaussian: {
      const float coeff = -0.5f / (f.p1 * f.p1);
      return fmaxf(0.0f, (1.0f / (sqrtf(2.0f * kPi) * f.p1)) * expf(coeff * (dx * dx + dy * dy)));
    }
    case kFilterMitchell:
      return mitchell_1d(dx, f.support, f.p1, f.p2) * mitchell_1d(dy, f.support, f.p1, f.p2);
    case kFilterLanczos:
      return lanczos_1d(dx, f.support, f.p1) * lanczos_1d(dy, f.support, f.p1);
    default:
      return 0.0f;
  }
}

// Vector::getOrthonormalBasis (Vector.inl:527-538)
MGPU_HD void onb(V3 n, V3 &U, V3 &W) {
  V3 up = v3(0.0f, 1.0f, 0.0f);
  if (fabsf(dot(up, n)) > 0.8f) up = v3(1.0f, 0.0f, 0.0f);
  U = normalize(cross(up, n));
  W = normalize(cross(n, U));
}

// Bump-mapped shading normal (Material::_initShadingNormal, Material.cpp:205-224): N unchanged
// where both luminance differences are 0 (EQ against 0 is |x| < EPSILON), else
// normalize(N + intensity (gx U + gy V)) with U, V = N's orthonormal basis.
MGPU_HD V3 bump_normal(V3 N, float gx, float gy, float intensity) {
  if (fabsf(gx) < kEps && fabsf(gy) < kEps) return N;
  V3 U, W;
  onb(N, U, W);
  return normalize(N + (U * gx + W * gy) * intensity);
}

// Vector3::cosRandom + convertHemisphere (Vector.cpp:21-29, Vector3.inl:18-21):
// theta = acos(sqrt(u1)), phi = 2 pi u2, local (sin t cos p, cos t, sin t sin p)
MGPU_HD V3 cos_random(V3 n, float u1, float u2) {
  float ct = sqrtf(u1), st = sqrtf(fmaxf(0.0f, 1.0f - u1));
  float phi = 2.0f * kPi * u2;
  float sp, cp;
#if defined(__CUDA_ARCH__)
  sincosf(phi, &sp, &cp);
#else
  sp = sinf(phi); cp = cosf(phi);
#endif
  V3 U, W;
  onb(n, U, W);
  return U * (st * cp) + n * ct + W * (st * sp);
}

MGPU_HD V3 reflect(V3 wi, V3 n) { return n * (-2.0f * dot(wi, n)) + wi; }

// Vector::refractVector (Vector.inl:467-495); ok = false on total internal reflection
MGPU_HD V3 refract(V3 wi, V3 normal, float in, float out, bool &ok) {
  V3 w = -wi, nrm;
  float eta;
  if (dot(wi, normal) < 0.0f) { nrm = normal; eta = in / out; }
  else { nrm = -normal; eta = out / in; }
  float d = dot(w, nrm);
  float det = 1.0f - eta * eta * (1.0f - d * d);
  if (det < 0.0f) { ok = false; return v3(0.0f, 0.0f, 0.0f); }
  ok = true;
  return w * (-eta) + nrm * (eta * d - sqrtf(det));
}

// Fresnel::getFr (Fresnel.h:45-90), unpolarised dielectric reflectance
MGPU_HD float fresnel_cos(float ci, float n1, float n2) {
  float si = sqrtf(fmaxf(0.0f, 1.0f - ci * ci));
  float snell = (n1 / n2) * si;
  if (fabsf(snell) >= 1.0f) return 1.0f;
  float ct = sqrtf(fmaxf(0.0f, 1.0f - snell * snell));
  float n1ci = n1 * ci, n1ct = n1 * ct, n2ci = n2 * ci, n2ct = n2 * ct;
  float rs = (n1ci - n2ct) / (n1ci + n2ct);
  float rp = (n1ct - n2ci) / (n1ct + n2ci);
  return (rs * rs + rp * rp) * 0.5f;
}

MGPU_HD float fresnel(V3 wi, V3 N, float n1, float n2) {
  float c = dot(N, wi);
  if (c < 0.0f) return fresnel_cos(-c, n1, n2);
  return fresnel_cos(c, n2, n1);
}

// BSDF evaluate fs(wi -> wo) for the non-specular BSDFs (the dielectric is only ever
// evaluated on its own sample, which bsdf_sample handles through lobe flags).
//   Diffuse: DiffuseBSDF::evaluate (DiffuseBSDF.cpp:41-48), one-sided
//   Phong:   ModifiedPhongBSDF::evaluate (ModifiedPhongBSDF.cpp:163-181), including the
//            reference's 1/kda and 1/ksa lobe normalisation
MGPU_HD V3 bsdf_eval(const Material &m, V3 ns, V3 wi, V3 wo) {
  if (m.type == 0) {
    if (dot(ns, wi) >= 0.0f || dot(ns, wo) <= 0.0f) return v3(0.0f, 0.0f, 0.0f);
    return m.kd * (1.0f / kPi);
  }
  if (m.type == 1) {
    if (dot(ns, wo) <= 0.0f) return v3(0.0f, 0.0f, 0.0f);
    V3 r = reflect(wi, ns);
    float a = fminf(fmaxf(dot(r, wo), 0.0f), 1.0f);
    float fsd = m.kda > 0.0f ? rcp(kPi * m.kda) : 0.0f;
    float fss = m.ksa > 0.0f ? ((m.n + 2.0f) / (2.0f * kPi * m.ksa)) * powf(a, m.n) : 0.0f;
    return m.kd * fsd + m.ks * fss;
  }
  return v3(0.0f, 0.0f, 0.0f);
}

enum Event { EV_NONE = 0, EV_DIFFUSE = 1, EV_SPECULAR = 2, EV_REFLECT = 3, EV_REFRACT = 4, EV_ZERO_PDF = -1 };

// BSDF::sample + getPd + evaluate/pdf; returns the event and fs = f / pdf.
//   Diffuse:    DiffuseBSDF.cpp:21-39
//   Phong:      ModifiedPhongBSDF.cpp:83-158 (lobe by p0 = U - EPSILON against kda, kda + ksa)
//   Dielectric: DielectricBSDF.cpp:56-157 with the path's ior index (fs = ks on reflection,
//               ks * e_index on refraction, pdf 1)
MGPU_HD int bsdf_sample(const Material &m, V3 ns, V3 wi, uint32_t ior_index, float u0, float u1, float u2, V3 &wo,
                        V3 &fs) {
  fs = v3(0.0f, 0.0f, 0.0f);
  if (m.type == 0) {
    if (dot(ns, wi) > 0.0f) return EV_NONE;
    wo = cos_random(ns, u0, u1);
    float c = dot(ns, wo);
    if (!(c > 0.0f)) return EV_ZERO_PDF;
    fs = bsdf_eval(m, ns, wi, wo) * kPi;
    return EV_DIFFUSE;
  }
  if (m.type == 1) {
    float p0 = u0 - kEps;
    int ev;
    if (p0 <= m.kda) {
      ev = EV_DIFFUSE;
      wo = cos_random(ns, u1, u2);
    } else if (p0 <= m.kda + m.ksa) {
      ev = EV_SPECULAR;
      float ca = powf(u1, rcp(m.n + 1.0f));
      float sa = sqrtf(fmaxf(0.0f, 1.0f - ca * ca));
      float phi = 2.0f * kPi * u2;
      float sp, cp;
#if defined(__CUDA_ARCH__)
      sincosf(phi, &sp, &cp);
#else
      sp = sinf(phi); cp = cosf(phi);
#endif
      V3 R = reflect(wi, ns);
      V3 r = R, uu, vv;
      if (fabsf(dot(ns, r)) < 0.95f) {
        uu = normalize(cross(r, ns));
        vv = cross(uu, r);
      } else {
        r = normalize(r);
        onb(r, vv, uu);
      }
      V3 cand = uu * (sa * cp) + r * ca + vv * (sa * sp);
      wo = dot(ns, cand) > 0.0f ? cand : R;
    } else {
      return EV_NONE;
    }
    float cosA = dot(ns, wo);
    if (!(cosA > 0.0f)) return EV_ZERO_PDF;
    float pdf;
    if (ev == EV_SPECULAR) {
      V3 r = reflect(wi, ns);
      float ca = fabsf(dot(r, wo));
      pdf = fminf(1.0f, (m.n + 1.0f) / (2.0f * kPi) * powf(ca, m.n)) / cosA;
    } else {
      pdf = (fabsf(cosA) / kPi) / cosA;
    }
    if (!(pdf > 0.0f)) return EV_ZERO_PDF;
    fs = bsdf_eval(m, ns, wi, wo) * rcp(pdf);
    return ev;
  }
  // dielectric
  V3 N = dot(ns, wi) > 0.0f ? -ns : ns;
  bool ok;
  V3 wt = refract(wi, ns, kAir, m.ior, ok);
  if (ok) {
    float fr = fresnel(wi, ns, kAir, m.ior);
    float fst = m.transparency * (1.0f - fr);
    if (u0 < fst) {
      wo = wt;
      fs = v3(ior_index == 0 ? m.ks.x : 0.0f, ior_index == 1 ? m.ks.y : 0.0f, ior_index == 2 ? m.ks.z : 0.0f);
      return EV_REFRACT;
    }
  }
  wo = reflect(wi, N);
  fs = m.ks;
  return EV_REFLECT;
}

// OrientedEmitter::getLe (OrientedEmitter.cpp:17-23) with radiance already power/(area pi)
MGPU_HD V3 emitted(V3 Le, V3 n, V3 w) { return dot(n, w) > 0.0f ? Le : v3(0.0f, 0.0f, 0.0f); }

// Emitter::getLe of a light in direction w from a point with normal n: OrientedEmitter on the
// normal's side only (OrientedEmitter.cpp:17-23), OmniEmitter in every direction (OmniEmitter.cpp)
MGPU_HD V3 light_le(const Light &L, V3 n, V3 w) { return L.omni ? L.Le : emitted(L.Le, n, w); }

// Origin offset against self-intersection: Waechter and Binder, "A Fast and Robust Method
// for Avoiding Self-Intersection", Ray Tracing Gems ch. 6 (2019).  n points to the side the
// new ray leaves from.
MGPU_HD V3 offset_origin(V3 p, V3 n) {
  const float origin = 1.0f / 32.0f, fscale = 1.0f / 65536.0f, iscale = 256.0f;
  int ix = (int)(iscale * n.x), iy = (int)(iscale * n.y), iz = (int)(iscale * n.z);
  float px = bits_f(f_bits(p.x) + (uint32_t)((p.x < 0.0f) ? -ix : ix));
  float py = bits_f(f_bits(p.y) + (uint32_t)((p.y < 0.0f) ? -iy : iy));
  float pz = bits_f(f_bits(p.z) + (uint32_t)((p.z < 0.0f) ? -iz : iz));
  return v3(fabsf(p.x) < origin ? p.x + fscale * n.x : px, fabsf(p.y) < origin ? p.y + fscale * n.y : py,
            fabsf(p.z) < origin ? p.z + fscale * n.z : pz);
}

// Path flags kept in the radiance record's w word
constexpr uint32_t kFlagIorMask = 3u;       // ior index 0..2 (PathTracer.cpp:32)
constexpr uint32_t kFlagSpecular = 4u;      // data["specular"] (PathTracer.cpp:45-46)
constexpr uint32_t kFlagContinued0 = 8u;    // the depth-0 vertex spawned a continuation
constexpr uint32_t kFlagTruncated = 16u;    // hit the hard depth cap
constexpr uint32_t kFlagNeePending = 32u;   // light-sample slots hold unfolded direct light

// Milton's single-wavelength masking at depth 0 (PathTracer.cpp:107-114)
MGPU_HD V3 apply_mask(V3 L, uint32_t flags) {
  if ((flags & kFlagSpecular) && (flags & kFlagContinued0)) {
    uint32_t k = flags & kFlagIorMask;
    return v3(k == 0 ? 3.0f * L.x : 0.0f, k == 1 ? 3.0f * L.y : 0.0f, k == 2 ? 3.0f * L.z : 0.0f);
  }
  return L;
}

}  // namespace mgpu
