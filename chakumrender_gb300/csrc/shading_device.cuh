// shading_device.cuh — FP32 materials, direction samplers and LTC polygon-light
// integration, usable from device code and (for host-side checks) host code.
//
// Each function restates the reference's FP64 code in FP32 (the reference file
// and lines are named per function).  PI is the reference's 3.14159265359.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SHD __host__ __device__ __forceinline__
#else
#define SHD inline
#endif

namespace ckr {

constexpr float kPi = 3.14159265359f;
constexpr double kPiD = 3.14159265359;

struct F3 {
  float x, y, z;
};
SHD F3 f3(float x, float y, float z) { return F3{x, y, z}; }
SHD F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
SHD F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
SHD F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
SHD F3 operator-(F3 a) { return f3(-a.x, -a.y, -a.z); }
SHD float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SHD F3 cross(F3 a, F3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
// Cross product with separately rounded products (no fused multiply-add): a
// component whose two products are equal comes out exactly zero, as in the
// reference's arithmetic.  Geometric normals use it because ref_frame branches
// on n.x != 0, so a rounding residue there would rotate the sampling frame.
SHD F3 cross_rn(F3 a, F3 b) {
#if defined(__CUDA_ARCH__)
  return f3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
#else
  return cross(a, b);  // host code is built without contraction
#endif
}
SHD float length(F3 a) { return sqrtf(dot(a, a)); }
// Unit vector.  On the device by the reciprocal square root instruction (within 2
// ulp) instead of a correctly rounded square root and division: signs and zero
// components are kept exactly (ref_frame branches on n.x != 0) and directions move by
// FP32 noise.  LTC shading 0.502 -> 0.378 ms per 1024^2 frame with 8 quads, box path
// tracer frame 1.133 -> 1.095 ms, 64-job batch 0.820 -> 0.787 s, every parity test
// unchanged.  The host build (the test replays) keeps the exact form.
SHD F3 normalize(F3 a) {
#if defined(__CUDA_ARCH__)
  return a * rsqrtf(dot(a, a));
#else
  return a * (1.0f / sqrtf(dot(a, a)));
#endif
}
SHD F3 mulc(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }

// BRDFType numbering of the reference (headers/materialTypes.h:7).
enum : int32_t { kBrdfNone = 0, kClassicPhong = 1, kGGX = 2, kBeckmann = 3, kPhong = 4, kGGXApprox = 5 };

struct Material {
  int32_t brdf;
  float alpha, phong_exp, spec, int_ior, ext_ior;
};

// ---- BRDF (src/materialTypes.cpp:9-50, 156-258) ---------------------------------
SHD float fresnel(const Material &m, float c) {
  float g = m.int_ior / m.ext_ior;
  g *= g;
  g += c * c - 1.0f;
  g = sqrtf(g);
  float t1 = g - c, t2 = g + c;
  float tmp = c * t2 - 1.0f;
  float F = tmp * tmp;
  tmp = c * t1 + 1.0f;
  F /= (tmp * tmp);
  F += 1.0f;
  tmp = t1 / t2;
  tmp *= tmp;
  return F * 0.5f * tmp;
}
// tan^2 of the angle between unit vectors v and n.  The reference computes
// 1/cos^2 - 1 (FP64); in FP32 that cancels near cos = 1, which for the
// near-mirror roughness of its scenes (alpha 5e-4) moves D by tens of percent.
// |v x n|^2 / cos^2 is the same quantity without the cancellation.
SHD float tan2_of(F3 v, F3 n) {
  float c = dot(v, n);
  F3 s = cross(v, n);
  return dot(s, s) / (c * c);
}

SHD float ggx_dist(float alpha, F3 h, F3 n) {
  float cs = dot(h, n);
  cs *= cs;
  float ts = tan2_of(h, n);
  float as = alpha * alpha;
  ts += as;
  ts *= ts;
  return as / (kPi * cs * cs * ts);
}
SHD float ggx_g1(float alpha, F3 v, F3 h, F3 n) {
  float ts = tan2_of(v, n);
  if (ts <= 1e-15f) return 1.0f;
  if (dot(h, v) <= 1e-15f) return 0.0f;
  ts = ts * (alpha * alpha) + 1.0f;
  return 2.0f / (1.0f + sqrtf(ts));
}
SHD float beckmann_dist(float alpha, F3 h, F3 n) {
  float cs = dot(h, n);
  cs *= cs;
  float ts = tan2_of(h, n);
  float as = alpha * alpha;
  return expf(-ts / as) / (kPi * cs * cs * as);
}
SHD float rational_g1(float a) { return (3.535f * a + 2.181f * a * a) / (1.0f + 2.276f * a + 2.577f * a * a); }
SHD float beckmann_g1(float alpha, F3 v, F3 h, F3 n) {
  float cs = dot(v, n);
  cs *= cs;
  if (cs >= 0.999999f) return 1.0f;
  if (dot(h, v) <= 1e-15f) return 0.0f;
  float a = 1.0f / (alpha * sqrtf(tan2_of(v, n)));
  return a < 1.6f ? rational_g1(a) : 1.0f;
}
SHD float phong_g1(float alpha, F3 v, F3 h, F3 n) {
  float cs = dot(v, n);
  cs *= cs;
  if (cs >= 0.999999f) return 1.0f;
  if (dot(h, v) <= 1e-15f) return 0.0f;
  float a = sqrtf((0.5f * alpha + 1.0f) / tan2_of(v, n));
  return a < 1.6f ? rational_g1(a) : 1.0f;
}
SHD float phong_dist(float alpha, F3 h, F3 n) { return (alpha + 2.0f) * powf(dot(h, n), alpha) / (2.0f * kPi); }

// MaterialType::brdf without the LTC branch (reflectance not included).
SHD float brdf_eval(const Material &m, F3 n, F3 wo_ref, F3 wo, F3 wi) {
  float s = m.spec;
  if (m.brdf == kClassicPhong) {
    float c = dot(wo_ref, wi);
    return s * (m.phong_exp + 1.0f) * powf(c > 0.f ? c : 0.f, m.phong_exp) / (2.0f * kPi) + (1.0f - s) / kPi;
  }
  if (m.brdf == kGGX || m.brdf == kBeckmann || m.brdf == kPhong) {
    F3 h = normalize(wo + wi);
    float F = fresnel(m, dot(h, wi));
    float D, G;
    if (m.brdf == kGGX) {
      D = ggx_dist(m.alpha, h, n);
      G = ggx_g1(m.alpha, wo, h, n) * ggx_g1(m.alpha, wi, h, n);
    } else if (m.brdf == kBeckmann) {
      D = beckmann_dist(m.alpha, h, n);
      G = beckmann_g1(m.alpha, wo, h, n) * beckmann_g1(m.alpha, wi, h, n);
    } else {
      D = phong_dist(m.alpha, h, n);
      G = phong_g1(m.alpha, wo, h, n) * phong_g1(m.alpha, wi, h, n);
    }
    return (s * F * D * G) / (4.0f * dot(wi, n) * dot(wo, n)) + (1.0f - s) / kPi;
  }
  return 0.0f;
}

// MaterialType::pdfEval (src/materialTypes.cpp:89-116): the one-sample mixture
// of the specular lobe (probability spec) and cosine sampling.
SHD float pdf_eval(const Material &m, F3 n, F3 wo_ref, F3 wo, F3 wi) {
  float diffuse = (1.0f - m.spec) * dot(wi, n) / kPi;
  float s = m.spec;
  if (m.brdf == kClassicPhong) {
    float c = dot(wi, wo_ref);
    s *= (m.phong_exp + 1.0f) * powf(c > 0.f ? c : 0.f, m.phong_exp) / (2.0f * kPi);
  } else if (m.brdf == kGGX || m.brdf == kBeckmann || m.brdf == kPhong) {
    F3 h = normalize(wo + wi);
    float D = m.brdf == kGGX ? ggx_dist(m.alpha, h, n)
                             : (m.brdf == kBeckmann ? beckmann_dist(m.alpha, h, n) : phong_dist(m.alpha, h, n));
    s *= D * dot(h, n) / (4.0f * dot(h, wo));
  }
  return s + diffuse;
}

// ---- samplers (src/domainSampler.cpp) ------------------------------------------
// Tangent frame of the reference (src/domainSampler.cpp:163-176):
// X = normalize((-n.y - n.z) / n.x, 1, 1) when n.x != 0, else
// normalize(1, -n.z / n.y, 1), else (1, 1, 0)/sqrt 2.  Evaluated as
// sign(n.x) normalize(-n.y - n.z, n.x, n.x) (the same vector), which cannot
// overflow in FP32 when |n.x| is tiny.
SHD void ref_frame(F3 n, F3 &X, F3 &Y) {
  if (n.x != 0.f) X = normalize(f3(-n.y - n.z, n.x, n.x)) * (n.x > 0.f ? 1.0f : -1.0f);
  else if (n.y != 0.f) X = normalize(f3(n.y, -n.z, n.y)) * (n.y > 0.f ? 1.0f : -1.0f);
  else X = normalize(f3(1.0f, 1.0f, 0.0f));
  Y = normalize(cross(n, X));
}
SHD F3 to_world(F3 X, F3 Y, F3 Z, float x, float y, float z) { return X * x + Y * y + Z * z; }

// Cosine-weighted direction (the table construction at src/domainSampler.cpp:29-40
// with theta = asin(sqrt(e1)), mapped through the frame of :154-189).
SHD F3 sample_cosine(F3 n, float e1, float e2) {
  F3 X, Y;
  ref_frame(n, X, Y);
  float st = sqrtf(e1), ct = sqrtf(1.0f - e1), ph = 2.0f * kPi * e2;
  float sp, cp;
  sincosf(ph, &sp, &cp);
  return to_world(X, Y, n, st * cp, st * sp, ct);
}

// Uniform direction on the hemisphere about n (getHemiDirectionSamples,
// src/domainSampler.cpp:89-100: a uniform sphere direction turned into n's
// hemisphere; 1/pdf = 2 pi).
SHD F3 sample_hemisphere(F3 n, float e1, float e2) {
  F3 X, Y;
  ref_frame(n, X, Y);
  float ct = e1, st = sqrtf(fmaxf(0.0f, 1.0f - e1 * e1)), sp, cp;
  sincosf(2.0f * kPi * e2, &sp, &cp);
  return to_world(X, Y, n, st * cp, st * sp, ct);
}

// Specular lobe of getBrdfDirectionSamples / getClassicPhongDirectionSamples
// (src/domainSampler.cpp:193-314).
SHD F3 sample_lobe(const Material &m, F3 n, F3 wo_ref, F3 wo, float e1, float e2) {
  float sp, cp;
  sincosf(2.0f * kPi * e2, &sp, &cp);
  F3 X, Y;
  if (m.brdf == kClassicPhong) {
    ref_frame(wo_ref, X, Y);
    float ct = powf(1.0f - e1, 1.0f / (m.phong_exp + 1.0f));
    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    return to_world(X, Y, wo_ref, st * cp, st * sp, ct);
  }
  ref_frame(n, X, Y);
  float ct, st;
  if (m.brdf == kGGX) {
    float tt = m.alpha * sqrtf(e1) / sqrtf(1.0f - e1 + 1e-10f);
    ct = 1.0f / sqrtf(1.0f + tt * tt);
    st = tt * ct;
  } else if (m.brdf == kBeckmann) {
    float tt = sqrtf(-(m.alpha * m.alpha) * logf(1.0f - e1 + 1e-20f));
    ct = 1.0f / sqrtf(1.0f + tt * tt);
    st = tt * ct;
  } else {
    ct = powf(e1, 1.0f / (m.alpha + 2.0f));
    st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  }
  F3 h = to_world(X, Y, n, st * cp, st * sp, ct);
  return normalize(h * (2.0f * dot(h, wo)) - wo);
}

// getBrdfDirectionSampleRandomized (src/materialTypes.cpp:136-153): the lobe with
// probability spec, else cosine.
SHD F3 sample_brdf(const Material &m, F3 n, F3 wo_ref, F3 wo, float e0, float e1, float e2) {
  return e0 < m.spec ? sample_lobe(m, n, wo_ref, wo, e1, e2) : sample_cosine(n, e1, e2);
}

// Cone of half-angle theta_max about w (getSolidDirectionSamples,
// src/domainSampler.cpp:320-369); 1/pdf = 2 pi (1 - cos theta_max).
SHD F3 sample_cone(F3 w, float cos_max, float e1, float e2) {
  F3 X, Y;
  ref_frame(w, X, Y);
  float ct = 1.0f - (1.0f - cos_max) * e1;
  float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  float sp, cp;
  sincosf(2.0f * kPi * e2, &sp, &cp);
  return to_world(X, Y, w, st * cp, st * sp, ct);
}

// Uniform point on a triangle (getTriLightSurfaceSamples, src/domainSampler.cpp:138-150).
SHD F3 sample_triangle(F3 a, F3 b, F3 c, float e1, float e2) {
  float s = sqrtf(e1);
  return a * (1.0f - s) + b * (s * (1.0f - e2)) + c * (e2 * s);
}

// ---- LTC ------------------------------------------------------------------------
// Device LTC table entry (FP32): the five structural non-zeros of Minv and M
// (row-major slots 0, 2, 4, 6, 8; the fit leaves 1, 3, 5, 7 zero), the
// amplitude, and det(M) of the entry itself (M_GGX never refreshes det after
// interpolating, headers/ltc.h:36-60).
struct LtcEntry {
  float mi0, mi2, mi4, mi6, mi8, amp;
  float m0, m2, m4, m6, m8, det;
};

struct LtcLookup {
  float mi[5], m[5], amp, det;
};

// M_GGX index math (headers/ltc.h:18-34): theta bins over [0, pi/2], alpha bins
// over sqrt(alpha); linear interpolation in theta only.  The alpha index has no
// interpolation, so it is computed in FP64 (as the reference does) when FP32
// lands within 1e-4 of a bin edge.
SHD void ltc_index(float theta, float alpha, int &t, int &a, int &t1, float &mult) {
  const int size = 64;
  float tf = theta / (0.5f * kPi) * (float)size;
  t = (int)floorf(tf);
  t = t < size - 1 ? t : size - 1;
  t = t > 0 ? t : 0;
  float af = sqrtf(alpha) * (float)size;
  float fr = af - floorf(af);
  if (fr < 1e-4f || fr > 1.0f - 1e-4f) af = (float)floor(sqrt((double)alpha) * size);
  a = (int)floorf(af);
  a = a < size - 1 ? a : size - 1;
  a = a > 0 ? a : 0;
  t1 = (t + 1) < (size - 1) ? (t + 1) : (size - 1);
  mult = tf - (float)t;
}

template <typename Table>
SHD LtcLookup ltc_lookup(const Table &tab, float theta, float alpha) {
  int t, a, t1;
  float mult;
  ltc_index(theta, alpha, t, a, t1, mult);
  LtcEntry e0 = tab(a + t * 64), e1 = tab(a + t1 * 64);
  LtcLookup r;
  if (t == t1) mult = 0.0f;
  r.mi[0] = e0.mi0 + (e1.mi0 - e0.mi0) * mult;
  r.mi[1] = e0.mi2 + (e1.mi2 - e0.mi2) * mult;
  r.mi[2] = e0.mi4 + (e1.mi4 - e0.mi4) * mult;
  r.mi[3] = e0.mi6 + (e1.mi6 - e0.mi6) * mult;
  r.mi[4] = e0.mi8 + (e1.mi8 - e0.mi8) * mult;
  r.m[0] = e0.m0 + (e1.m0 - e0.m0) * mult;
  r.m[1] = e0.m2 + (e1.m2 - e0.m2) * mult;
  r.m[2] = e0.m4 + (e1.m4 - e0.m4) * mult;
  r.m[3] = e0.m6 + (e1.m6 - e0.m6) * mult;
  r.m[4] = e0.m8 + (e1.m8 - e0.m8) * mult;
  r.amp = e0.amp + (e1.amp - e0.amp) * mult;
  r.det = e0.det;
  return r;
}

// 3x3 row-major matrix.
struct M3f {
  float a[9];
};
SHD F3 mul(const M3f &m, F3 v) {
  return f3(m.a[0] * v.x + m.a[1] * v.y + m.a[2] * v.z, m.a[3] * v.x + m.a[4] * v.y + m.a[5] * v.z,
            m.a[6] * v.x + m.a[7] * v.y + m.a[8] * v.z);
}

// getBrdfApproxParam (src/materialTypes.cpp:52-74): Minv . R^T with R^T's rows
// (T1, T2, n), T1 the tangent in the plane of n and wo.
// At (near) normal incidence wo - n (n.wo) vanishes; the reference then
// normalises a zero vector (NaN).  The fit is isotropic at theta = 0, so the
// sampling frame's X axis is used there instead.
SHD M3f ltc_minv_world(const LtcLookup &L, F3 n, F3 wo) {
  F3 t = wo - n * dot(n, wo);
  F3 T1, T2;
  if (dot(t, t) < 1e-12f) {
    ref_frame(n, T1, T2);
  } else {
    T1 = normalize(t);
  }
  T2 = normalize(cross(n, T1));
  // Minv = [[mi0, 0, mi2], [0, mi4, 0], [mi6, 0, mi8]]
  M3f r;
  r.a[0] = L.mi[0] * T1.x + L.mi[1] * n.x;
  r.a[1] = L.mi[0] * T1.y + L.mi[1] * n.y;
  r.a[2] = L.mi[0] * T1.z + L.mi[1] * n.z;
  r.a[3] = L.mi[2] * T2.x;
  r.a[4] = L.mi[2] * T2.y;
  r.a[5] = L.mi[2] * T2.z;
  r.a[6] = L.mi[3] * T1.x + L.mi[4] * n.x;
  r.a[7] = L.mi[3] * T1.y + L.mi[4] * n.y;
  r.a[8] = L.mi[3] * T1.z + L.mi[4] * n.z;
  return r;
}

// theta / sin(theta) for theta = acos(c), the factor of the edge integral.  With u =
// |c|, g(u) = acos(u) / sqrt(1 - u^2) is analytic on [0, 1] (at u = 1 the square-root
// behaviours of acos and of the sine cancel, g(1) = 1; the nearest singularity is at
// u = -1), so a polynomial converges fast there: the degree-9 least-squares fit to g on
// 4,000 Chebyshev nodes of [0, 1] (computed in FP64, rounded to FP32) is within 2e-8
// of g, below the FP32 rounding of its Horner evaluation (2e-7 relative).  For c < 0,
// acos(c) = pi - acos(u) gives pi / sqrt(1 - u^2) - g(u) (4e-7 relative with an exact
// reciprocal square root).  Nine FMAs and, for c < 0, one reciprocal square root
// replace acos, a square root and a division.
SHD float theta_over_sin(float c) {
  constexpr float kG[10] = {1.570796251296997f,  -0.9999964833259583f, 0.7852754592895508f,
                            -0.6649839878082275f, 0.5770568251609802f,  -0.48246079683303833f,
                            0.35151180624961853f, -0.19518974423408508f, 0.06951962411403656f,
                            -0.011529042385518551f};
  c = fminf(1.0f, fmaxf(-1.0f, c));
  const float u = fabsf(c);
  float g = kG[9];
  for (int k = 8; k >= 0; --k) g = fmaf(g, u, kG[k]);
  if (c >= 0.0f) return g;
#if defined(__CUDA_ARCH__)
  const float rs = rsqrtf((1.0f - u) * (1.0f + u));
#else
  const float rs = 1.0f / sqrtf((1.0f - u) * (1.0f + u));
#endif
  return fmaf(kPi, rs, -g);
}

// integrateEdge (src/lightSources_CV.cpp:8-25): (v1 x v2).n * theta / sin(theta),
// theta = acos(v1.v2).  (Before theta_over_sin: acos, sin(acos c) as sqrt((1 - c)(1 +
// c)) and a division; with the polynomial the LTC kernel runs a 1024^2 G-buffer with 8
// quads in 0.500 ms instead of 0.725, its output within FP32 rounding of the previous
// one.)
SHD float edge_factor(F3 v1, F3 v2) { return theta_over_sin(dot(v1, v2)); }
SHD float integrate_edge(F3 v1, F3 v2, F3 n) { return dot(cross(v1, v2), n) * edge_factor(v1, v2); }
SHD float integrate_edge_z(F3 v1, F3 v2) { return (v1.x * v2.y - v1.y * v2.x) * edge_factor(v1, v2); }

// Edge crossing test of clipTriangle.  The reference intersects edge PQ with the
// plane at i = P + (P - Q) d and accepts it when (i - P).(Q - i) > 0 (for edge CA
// it compares x coordinates only, :101-102).  Since i - P = (P - Q) d and
// Q - i = (Q - P)(1 + d), that product is -|P - Q|^2 d (1 + d) (x only for CA),
// positive exactly when -1 < d < 0 (and, for CA, A.x != C.x).  Testing d
// directly gives the same answer without the cancellation that makes the
// product round to zero in FP32 when a vertex lies within ~1e-4 of the plane.
SHD bool edge_crossed(float d) { return d > -1.0f && d < 0.0f; }

// Records a clipped edge segment: the first two points go to q0, q1, the next
// two to q2, q3 (clipTriangle's clip[idx++] sequence without a local array).
struct Clip4 {
  F3 q0, q1, q2, q3;
  int idx;
  SHD void push(F3 a, F3 b) {
    if (idx == 0) {
      q0 = a;
      q1 = b;
    } else if (idx == 2) {
      q2 = a;
      q3 = b;
    }
    idx += 2;
  }
};

// clipTriangle against the plane through P with normal n, general variant
// (src/lightSources_CV.cpp:28-130), including its test on edge CA that looks
// at x coordinates only (:101-102).
SHD bool clip_triangle(F3 A, F3 B, F3 C, F3 n, F3 P, float nA, float nB, float nC, Clip4 &clip) {
  const float eps = 1e-15f;
  int hits = 0;
  clip.idx = 0;
  F3 dAB = A - B, dBC = B - C, dCA = C - A;
  float nAB = dot(n, dAB), nBC = dot(n, dBC), nCA = dot(n, dCA);
  float pA = dot(n, P - A), pB = dot(n, P - B), pC = dot(n, P - C);
  if (nAB * nAB > eps) {
    float d = pA / nAB;
    F3 i = dAB * d + A;
    if (edge_crossed(d)) {
      ++hits;
      if (nA < 0.f) clip.push(i, B);
      else clip.push(A, i);
    }
  } else if (pA * pA < eps) {
    return false;
  }
  if (nBC * nBC > eps) {
    float d = pB / nBC;
    F3 i = dBC * d + B;
    if (edge_crossed(d)) {
      ++hits;
      if (nB < 0.f) clip.push(i, C);
      else clip.push(B, i);
    }
  } else if (pB * pB < eps) {
    return false;
  }
  if (nCA * nCA > eps) {
    float d = pC / nCA;
    F3 i = dCA * d + C;
    if (edge_crossed(d) && A.x != C.x) {
      ++hits;
      if (nC < 0.f) clip.push(i, A);
      else clip.push(C, i);
    }
  } else if (pC * pC < eps) {
    return false;
  }
  return hits > 1;
}

// Same against the plane z = 0 (src/lightSources_CV.cpp:133-219).
SHD bool clip_triangle_z(F3 A, F3 B, F3 C, float nA, float nB, float nC, Clip4 &clip) {
  const float eps = 1e-15f;
  int hits = 0;
  clip.idx = 0;
  F3 dAB = A - B, dBC = B - C, dCA = C - A;
  if (dAB.z * dAB.z > eps) {
    float d = -A.z / dAB.z;
    F3 i = dAB * d + A;
    if (edge_crossed(d)) {
      ++hits;
      if (nA < 0.f) clip.push(i, B);
      else clip.push(A, i);
    }
  } else if (A.z * A.z < eps) {
    return false;
  }
  if (dBC.z * dBC.z > eps) {
    float d = -B.z / dBC.z;
    F3 i = dBC * d + B;
    if (edge_crossed(d)) {
      ++hits;
      if (nB < 0.f) clip.push(i, C);
      else clip.push(B, i);
    }
  } else if (B.z * B.z < eps) {
    return false;
  }
  if (dCA.z * dCA.z > eps) {
    float d = -C.z / dCA.z;
    F3 i = dCA * d + C;
    if (edge_crossed(d) && A.x != C.x) {
      ++hits;
      if (nC < 0.f) clip.push(i, A);
      else clip.push(C, i);
    }
  } else if (C.z * C.z < eps) {
    return false;
  }
  return hits > 1;
}

// |polygon integral| of one emitter triangle for the cosine lobe about n at x
// (getLightAnalyticDiffuse inner loop, src/lightSources_CV.cpp:226-264), in two
// parts: ltc_diffuse_case settles a triangle wholly above (1, |integral| in d) or
// below (0, d = 0) the horizon and returns -1 for one across it, whose clipped
// integral is ltc_diffuse_clipped.
SHD int ltc_diffuse_case(F3 A, F3 B, F3 C, F3 n, F3 x, float &d) {
  F3 e1 = normalize(A - x), e2 = normalize(B - x), e3 = normalize(C - x);
  float nA = dot(e1, n), nB = dot(e2, n), nC = dot(e3, n);
  d = 0.0f;
  if (nA > 0.f && nB > 0.f && nC > 0.f) {
    d = fabsf(integrate_edge(e1, e2, n) + integrate_edge(e2, e3, n) + integrate_edge(e3, e1, n));
    return 1;
  }
  if (nA < 0.f && nB < 0.f && nC < 0.f) return 0;
  return -1;
}

SHD float ltc_diffuse_clipped(F3 A, F3 B, F3 C, F3 n, F3 x) {
  F3 e1 = normalize(A - x), e2 = normalize(B - x), e3 = normalize(C - x);
  float nA = dot(e1, n), nB = dot(e2, n), nC = dot(e3, n);
  Clip4 clip;
  clip.q0 = clip.q1 = clip.q2 = clip.q3 = f3(0, 0, 0);
  if (!clip_triangle(A, B, C, n, x, nA, nB, nC, clip)) return 0.0f;
  F3 c0 = normalize(clip.q0 - x), c1 = normalize(clip.q1 - x), c2 = normalize(clip.q2 - x),
     c3 = normalize(clip.q3 - x);
  return fabsf(integrate_edge(c0, c1, n) + integrate_edge(c1, c2, n) + integrate_edge(c2, c3, n) +
               integrate_edge(c3, c0, n));
}

SHD float ltc_diffuse_tri(F3 A, F3 B, F3 C, F3 n, F3 x) {
  float d;
  return ltc_diffuse_case(A, B, C, n, x, d) < 0 ? ltc_diffuse_clipped(A, B, C, n, x) : d;
}

// |polygon integral| of one emitter triangle in the LTC's canonical space
// (getLightAnalytic inner loop, src/lightSources_CV.cpp:278-317), split the same way.
SHD int ltc_spec_case(F3 A, F3 B, F3 C, F3 x, const M3f &minv, float &s) {
  F3 e1 = mul(minv, A - x), e2 = mul(minv, B - x), e3 = mul(minv, C - x);
  s = 0.0f;
  if (e1.z > 0.f && e2.z > 0.f && e3.z > 0.f) {
    e1 = normalize(e1);
    e2 = normalize(e2);
    e3 = normalize(e3);
    s = fabsf(integrate_edge_z(e1, e2) + integrate_edge_z(e2, e3) + integrate_edge_z(e3, e1));
    return 1;
  }
  if (e1.z < 0.f && e2.z < 0.f && e3.z < 0.f) return 0;
  return -1;
}

SHD float ltc_spec_clipped(F3 A, F3 B, F3 C, F3 x, const M3f &minv) {
  F3 e1 = mul(minv, A - x), e2 = mul(minv, B - x), e3 = mul(minv, C - x);
  Clip4 clip;
  clip.q0 = clip.q1 = clip.q2 = clip.q3 = f3(0, 0, 0);
  if (!clip_triangle_z(e1, e2, e3, e1.z / length(e1), e2.z / length(e2), e3.z / length(e3), clip)) return 0.0f;
  F3 c0 = normalize(clip.q0), c1 = normalize(clip.q1), c2 = normalize(clip.q2),
     c3 = normalize(clip.q3);
  return fabsf(integrate_edge_z(c0, c1) + integrate_edge_z(c1, c2) + integrate_edge_z(c2, c3) +
               integrate_edge_z(c3, c0));
}

SHD float ltc_spec_tri(F3 A, F3 B, F3 C, F3 x, const M3f &minv) {
  float s;
  return ltc_spec_case(A, B, C, x, minv, s) < 0 ? ltc_spec_clipped(A, B, C, x, minv) : s;
}

// getLightFromMeshSource_Analytic for one shading point (src/lightSources_CV.cpp:323-333):
// spec * amplitude * sum|I_ltc| / 2pi + (1 - spec) * sum|I_cos| / 2pi, radiance-weighted.
// `light(k, A, B, C, rgb)` fetches emitter triangle k.
template <typename Table, typename LightFetch>
SHD void ltc_shade_point(const Table &tab, F3 x, F3 n, F3 wo, float alpha, float spec, uint32_t nlight,
                         const LightFetch &light, float out[3]) {
  float theta = acosf(fminf(1.0f, fmaxf(-1.0f, dot(n, wo))));
  LtcLookup L = ltc_lookup(tab, theta, alpha);
  M3f minv = ltc_minv_world(L, n, wo);
  float s3[3] = {0.f, 0.f, 0.f}, d3[3] = {0.f, 0.f, 0.f};
  for (uint32_t k = 0; k < nlight; ++k) {
    F3 A, B, C;
    float c[3];
    light(k, A, B, C, c);
    float s = ltc_spec_tri(A, B, C, x, minv);
    float d = ltc_diffuse_tri(A, B, C, n, x);
    for (int j = 0; j < 3; ++j) {
      s3[j] += c[j] * s;
      d3[j] += c[j] * d;
    }
  }
  const float inv2pi = 1.0f / (2.0f * kPi);
  for (int j = 0; j < 3; ++j) out[j] = s3[j] * inv2pi * L.amp * spec + d3[j] * inv2pi * (1.0f - spec);
}

// approxLTC_BRDF (src/materialTypes.cpp:76-87) divided by cos, times spec, plus
// the diffuse term: the `brdfApprox.isSet` branch of MaterialType::brdf (:11-12).
SHD float brdf_ltc(const Material &m, const LtcLookup &L, const M3f &minv, F3 n, F3 wi) {
  F3 lo = normalize(mul(minv, wi));
  // M = [[m0, 0, m2], [0, m4, 0], [m6, 0, m8]]
  F3 l_ = f3(L.m[0] * lo.x + L.m[1] * lo.z, L.m[2] * lo.y, L.m[3] * lo.x + L.m[4] * lo.z);
  float l = length(l_);
  float jac = L.det / (l * l * l);
  float D = (1.0f / kPi) * fmaxf(0.0f, lo.z);
  return m.spec * (L.amp * D / jac) / dot(wi, n) + (1.0f - m.spec) / kPi;
}

}  // namespace ckr
