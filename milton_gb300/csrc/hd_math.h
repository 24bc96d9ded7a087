// hd_math.h -- small host/device vector math and the Philox4x32-10 counter-based generator.
//
// Everything here compiles both as CUDA device code (inside the sm_103a kernels) and as plain
// C++ (so the same arithmetic can be unit-tested on the host).  Nothing in this header touches
// device memory.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define MGPU_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define MGPU_HD inline
#endif

namespace mgpu {

struct V3 {
  float x, y, z;
};

MGPU_HD V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
MGPU_HD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
MGPU_HD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
MGPU_HD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
MGPU_HD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
MGPU_HD V3 operator*(float s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
MGPU_HD V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
MGPU_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
MGPU_HD V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
MGPU_HD float length(V3 a) { return sqrtf(dot(a, a)); }
// 1 / x rounded to nearest, as the division 1.0f / x gives it (the device intrinsic skips the
// general division's path)
MGPU_HD float rcp(float x) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}
MGPU_HD V3 normalize(V3 a) {
  float l2 = dot(a, a);
  if (!(l2 > 0.0f)) return a;
  float inv = rcp(sqrtf(l2));
  return a * inv;
}
MGPU_HD float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
MGPU_HD float maxc(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
MGPU_HD bool nonzero(V3 a) { return a.x != 0.0f || a.y != 0.0f || a.z != 0.0f; }

MGPU_HD float bits_f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
MGPU_HD uint32_t f_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

MGPU_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Same specification as the oracle:
//   counter = {path_lo, path_hi, (depth << 16) | block, stream}, key = {seed_lo, seed_hi}.
struct U4 {
  uint32_t x, y, z, w;
};

MGPU_HD U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  U4 o; o.x = c0; o.y = c1; o.z = c2; o.w = c3;
  return o;
}

struct Rng {
  uint32_t k0, k1, stream;
};

MGPU_HD float u01(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

struct F4u {
  float a, b, c, d;
};

// four uniforms in [0, 1) for (path, depth, block)
MGPU_HD F4u uniforms(const Rng &g, uint64_t path, uint32_t depth, uint32_t block) {
  U4 w = philox4x32_10((uint32_t)path, (uint32_t)(path >> 32), (depth << 16) | (block & 0xFFFFu), g.stream, g.k0, g.k1);
  F4u r; r.a = u01(w.x); r.b = u01(w.y); r.c = u01(w.z); r.d = u01(w.w);
  return r;
}

// dimension map shared with the oracle
constexpr uint32_t kDepthJitter = 0xFFFFu;   // path = pixel * side^2 + stratum: {jx, jy}
constexpr uint32_t kDepthPathInit = 0xFFFEu; // path = global path id: {ior index, lens e1, lens e2}
// depth d, block 0: {bsdf0, bsdf1, bsdf2, rr};  depth d, block 1 + m/2: NEE sample m

}  // namespace mgpu
