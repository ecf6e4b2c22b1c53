// render_device.cuh — per-hit shading logic of the renderer (device code):
// surface interaction, light sampling and the MIS pdf sums of the reference's
// MIS sampler (src/mis.cpp:18-223), offsets for secondary rays.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ckr_rng.h"
#include "scene.h"
#include "shading_device.cuh"
#include "trace_device.cuh"

namespace ckr {

// Robust ray-origin offset along the geometric normal (Wachter and Binder,
// "A Fast and Robust Method for Avoiding Self-Intersection", Ray Tracing Gems,
// 2019): integer ulp offsets away from the origin, a fixed offset near it.
// Stands in for the reference's x + n * 1e-8 (src/lightSources.cpp:43), which
// FP32 cannot represent at scene scale.
__device__ __forceinline__ F3 offset_origin(F3 p, F3 n) {
  const float origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f, int_scale = 256.0f;
  int ox = (int)(int_scale * n.x), oy = (int)(int_scale * n.y), oz = (int)(int_scale * n.z);
  float px = __int_as_float(__float_as_int(p.x) + (p.x < 0.f ? -ox : ox));
  float py = __int_as_float(__float_as_int(p.y) + (p.y < 0.f ? -oy : oy));
  float pz = __int_as_float(__float_as_int(p.z) + (p.z < 0.f ? -oz : oz));
  return f3(fabsf(p.x) < origin ? p.x + float_scale * n.x : px, fabsf(p.y) < origin ? p.y + float_scale * n.y : py,
            fabsf(p.z) < origin ? p.z + float_scale * n.z : pz);
}

// Shadow-ray upper bound for a light at distance d: the reference's shadow()
// slack t + 1e-5 < d (src/shader.cpp:84-92), made relative for FP32 at large d.
__device__ __forceinline__ float shadow_tmax(float d) { return d - 1e-5f * fmaxf(1.0f, d); }

// Shadow ray from the offset origin o to the light point p: direction and tmax.  The
// ray must aim from o itself: aimed along the direction from the unoffset surface
// point, it meets the light's plane up to |offset| (1/cos - cos) before p, which
// exceeds the slack at moderate angles, and the light would occlude itself.
__device__ __forceinline__ float4 shadow_dir(F3 o, F3 p) {
  F3 v = p - o;
  float l = length(v);
  v = v * (1.0f / l);
  return make_float4(v.x, v.y, v.z, shadow_tmax(l));
}

struct Surface {
  F3 x, n, wo, wo_ref;
  uint32_t mat;
};

// Hit point and normal facing the ray: Triangle::intersect flips n
// (src/geometryPrimitives.cpp:35-41); spheres use normalize(centre - x) turned
// towards the viewer (src/shader.cpp:43-49).  wo_ref is the mirror direction
// (src/lightSources.cpp:45-46).
__device__ __forceinline__ Surface make_surface(const ShadeView &sv, F3 o, F3 d, uint32_t id, float t) {
  Surface s;
  s.x = o + d * t;
  F3 n;
  if (id & kSphereBit) {
    uint32_t j = id & ~kSphereBit;
    float4 c = __ldg(&sv.sph[j]);
    n = normalize(f3(c.x, c.y, c.z) - s.x);
    s.mat = __ldg(&sv.sph_mat[j]);
  } else {
    // normalize(cross_rn(C - A, B - A)) of the vertices and the material, one load
    // (ShadeView::tri_nm).
    const float4 nm = __ldg(&sv.tri_nm[id]);
    n = f3(nm.x, nm.y, nm.z);
    s.mat = __float_as_uint(nm.w);
  }
  if (dot(d, n) > 0.f) n = -n;
  s.n = n;
  s.wo = -d;
  s.wo_ref = normalize(n * (2.0f * dot(n, s.wo)) + d);
  return s;
}

__device__ __forceinline__ Material material_of(const ckr_material &m) {
  Material r;
  r.brdf = m.brdf;
  r.alpha = m.alpha;
  r.phong_exp = m.phong_exp;
  r.spec = m.spec;
  r.int_ior = m.int_ior;
  r.ext_ior = m.ext_ior;
  return r;
}

__device__ __forceinline__ RayPre ray_pre(F3 o, F3 d, float tmin) {
  return make_ray(make_float4(o.x, o.y, o.z, tmin), make_float4(d.x, d.y, d.z, 0.f));
}

// Closest emitter triangle of a mesh/tri light along the ray (MeshLight::intersect,
// src/lightSources.cpp:830-847, watertight FP32).  Returns the triangle index or kMiss.
__device__ __forceinline__ uint32_t light_tri_hit(const ShadeView &sv, const DevLight &L, const RayPre &r, float &t) {
  t = 3.0e38f;
  uint32_t best = kMiss;
  for (uint32_t k = 0; k < L.count; ++k) {
    uint32_t id = L.first + k;
    const float *t9 = sv.tri9 + 9 * (size_t)id;
    float4 v0 = make_float4(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2), 0.f);
    float4 v1 = make_float4(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5), 0.f);
    float4 v2 = make_float4(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8), 0.f);
    float th;
    if (hit_triangle(r, v0, v1, v2, t, th)) {
      t = th;
      best = id;
    }
  }
  return best;
}

__device__ __forceinline__ F3 tri_normal(const ShadeView &sv, uint32_t id) {
  const float *t9 = sv.tri9 + 9 * (size_t)id;
  F3 A = f3(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2));
  F3 B = f3(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5));
  F3 C = f3(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8));
  return normalize(cross_rn(C - A, B - A));
}

__device__ __forceinline__ F3 mat_radiance(const ShadeView &sv, uint32_t m) {
  const ckr_material &mm = sv.mats[m];
  return f3(mm.radiance[0], mm.radiance[1], mm.radiance[2]);
}

// ---- environment light (EnvSource, headers/lightSources.h:33-109) ----

// World direction -> the map's frame: z along the up axis (EnvSource::getRadiance).
__device__ __forceinline__ F3 env_local(uint32_t axis, F3 w) {
  return axis == 0 ? f3(w.y, w.z, w.x) : axis == 1 ? f3(w.x, w.z, w.y) : w;
}
__device__ __forceinline__ F3 env_world(uint32_t axis, F3 l) {
  return axis == 0 ? f3(l.z, l.x, l.y) : axis == 1 ? f3(l.x, l.z, l.y) : l;
}

// EnvSource::getThetaPhi + getRadiance's pixel: theta = acos z, phi from the
// asin of the normalised (x, y) by quadrant, col = phi / 2pi * w, row = theta / pi
// * h (clamped to the image; the reference indexes past it at phi = 2pi).
__device__ __forceinline__ float4 env_lookup(const ShadeView &sv, F3 w) {
  const F3 l = env_local(sv.env_axis, w);
  const float z = fminf(1.0f, fmaxf(-1.0f, l.z));
  const float theta = acosf(z);
  const float st = sqrtf(fmaxf(0.f, 1.0f - z * z));
  float phi = 0.f;
  if (st >= 1e-12f) {
    const float x = fminf(1.0f, fmaxf(-1.0f, l.x / st)), y = fminf(1.0f, fmaxf(-1.0f, l.y / st));
    if (y >= 0.f && x >= 0.f) phi = asinf(y);
    else if (y >= 0.f && x <= 0.f) phi = kPi - asinf(y);
    else if (y <= 0.f && x <= 0.f) phi = kPi + asinf(-y);
    else phi = 2.0f * kPi - asinf(-y);
  }
  uint32_t col = (uint32_t)(phi / (2.0f * kPi) * (float)sv.env_w);
  uint32_t row = (uint32_t)(theta / kPi * (float)sv.env_h);
  col = col < sv.env_w ? col : sv.env_w - 1;
  row = row < sv.env_h ? row : sv.env_h - 1;
  return __ldg(&sv.env[(size_t)row * sv.env_w + col]);
}

// Largest i in [0, n) with cdf[i] <= u (cdf[0] = 0 <= u < 1 = cdf[n]); rows or
// columns of zero weight are never returned.
__device__ __forceinline__ uint32_t env_search(const float *cdf, uint32_t n, float u) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&cdf[mid]) <= u) lo = mid;
    else hi = mid;
  }
  return lo;
}

// A direction with density luminance(L) / A in solid angle: a row by the
// marginal CDF (e0), a column by that row's CDF (e1), phi uniform across the
// pixel (e1's remainder in its column), cos theta uniform across the row's band
// (e2).
__device__ __forceinline__ F3 env_sample(const ShadeView &sv, float e0, float e1, float e2) {
  const uint32_t r = env_search(sv.env_marg, sv.env_h, e0);
  const float *cr = sv.env_cond + (size_t)r * (sv.env_w + 1);
  const uint32_t c = env_search(cr, sv.env_w, e1);
  const float c0 = __ldg(&cr[c]), c1 = __ldg(&cr[c + 1]);
  const float u = c1 > c0 ? fminf(fmaxf((e1 - c0) / (c1 - c0), 0.f), 1.0f) : 0.5f;
  const float phi = ((float)c + u) * (2.0f * kPi / (float)sv.env_w);
  const float ca = __ldg(&sv.env_cos[r]), cb = __ldg(&sv.env_cos[r + 1]);
  const float ct = ca - e2 * (ca - cb);
  const float st = sqrtf(fmaxf(0.f, 1.0f - ct * ct));
  float sp, cp;
  sincosf(phi, &sp, &cp);
  return env_world(sv.env_axis, f3(st * cp, st * sp, ct));
}

// Result of testing one direction against every area/sphere light: the sum
// sum_k N_k p_k(w) of the light techniques' pdfs (Pdf::pdfVal, src/mis.cpp:34-94)
// and the nearest light surface the ray meets (its distance and radiance).
struct LightQuery {
  float pdf_sum;
  float d;
  F3 Le;
  bool hit;
};

// Light kinds a shading kernel is compiled for: kernels for scenes whose lights
// are all MESH / TRI lights leave out the code of the others (a smaller loop body
// for the instruction caches of the path shader).
constexpr uint32_t kLightPoint = 1, kLightSphere = 2, kLightEnv = 4;
constexpr uint32_t kLightsAll = kLightPoint | kLightSphere | kLightEnv, kLightsMeshOnly = 0;

// ENV: the environment light takes part (pdf n_env luminance / A for every
// direction; seen when no other light is met, src/lightSources.cpp:103-106).
template <bool ENV = false, uint32_t LF = kLightsAll>
__device__ __forceinline__ LightQuery query_lights(const ShadeView &sv, F3 x, F3 o_off, F3 w, uint32_t n_per_light) {
  LightQuery q;
  q.pdf_sum = 0.f;
  q.d = 3.0e38f;
  q.Le = f3(0.f, 0.f, 0.f);
  q.hit = false;
  RayPre r = ray_pre(o_off, w, 0.f);
  for (uint32_t k = 0; k < sv.nlights; ++k) {
    DevLight L = sv.lights[k];
    if (L.type == CKR_LIGHT_MESH || L.type == CKR_LIGHT_TRI) {
      float t;
      uint32_t id = light_tri_hit(sv, L, r, t);
      if (id == kMiss) continue;
      F3 ne = tri_normal(sv, id);
      float c1 = fabsf(dot(w, ne));
      q.pdf_sum += (float)n_per_light * (t * t) / (c1 * L.area);
      if (t < q.d) {
        q.d = t;
        q.Le = mat_radiance(sv, sv.tri_mat[id]);
        q.hit = true;
      }
    } else if ((LF & kLightSphere) && L.type == CKR_LIGHT_SPHERE) {
      F3 c = f3(L.px, L.py, L.pz);
      F3 wl = c - x;
      float len = length(wl);
      float s = L.radius / len;
      float cmax = sqrtf(fmaxf(0.f, 1.0f - s * s));
      if (dot(w, wl * (1.0f / len)) >= cmax) q.pdf_sum += (float)n_per_light / (2.0f * kPi * (1.0f - cmax));
      double ts = hit_sphere(r, make_float4(L.px, L.py, L.pz, L.radius));
      if (ts < 1e299 && (float)ts < q.d) {
        q.d = (float)ts;
        q.Le = mat_radiance(sv, sv.sph_mat[L.first]);
        q.hit = true;
      }
    }
  }
  if (ENV && (LF & kLightEnv) && sv.env_n) {
    const float4 e = env_lookup(sv, w);
    q.pdf_sum += (float)sv.env_n * e.w * sv.env_inv_area;
    if (!q.hit) {
      q.hit = true;
      q.d = 3.0e38f;
      q.Le = f3(e.x, e.y, e.z);
    }
  }
  return q;
}

// One light-technique sample of light L from x (MeshLight::getSamples,
// getTriLightSurfaceSamples, getSolidDirectionSamples), as a unit direction.
template <uint32_t LF = kLightsAll>
__device__ __forceinline__ F3 sample_light(const ShadeView &sv, const DevLight &L, F3 x, float e0, float e1,
                                           float e2) {
  if ((LF & kLightSphere) && L.type == CKR_LIGHT_SPHERE) {
    F3 wl = f3(L.px, L.py, L.pz) - x;
    float len = length(wl);
    float s = L.radius / len;
    float cmax = sqrtf(fmaxf(0.f, 1.0f - s * s));
    return sample_cone(wl * (1.0f / len), cmax, e0, e1);
  }
  uint32_t k = 0;
  if (L.type == CKR_LIGHT_MESH) {
    uint32_t b = (uint32_t)(e0 * (float)kInvCdfBins);
    b = b >= kInvCdfBins ? kInvCdfBins - 1 : b;
    k = __ldg(&sv.cdf[L.cdf + b]);
  }
  const float *t9 = sv.tri9 + 9 * (size_t)(L.first + k);
  F3 A = f3(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2));
  F3 B = f3(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5));
  F3 C = f3(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8));
  // The mesh sampler draws (index, sqrt(u1), u2); a tri light draws (sqrt(u0), u1).
  F3 p = L.type == CKR_LIGHT_MESH ? sample_triangle(A, B, C, e1, e2) : sample_triangle(A, B, C, e0, e1);
  return normalize(p - x);
}

// ---- one-sample NEE over many lights ---------------------------------------------
// First index j of cdf[0, n) with cdf[j] > u (n >= 1; the last entry is 1).
__device__ __forceinline__ uint32_t cdf_pick(const float *cdf, uint32_t n, float u) {
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(cdf + mid) > u) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}
__device__ __forceinline__ float cdf_mass(const float *cdf, uint32_t j) {
  return __ldg(cdf + j) - (j ? __ldg(cdf + j - 1) : 0.f);
}

// Light-selection distribution at one vertex over the emitter lights
// [first_emit, first_emit + n_emit): their power CDF, or a proposal's 16-bit
// cumulative table (64 entries; pmf(j) = (cdf[j] - cdf[j-1]) / 65535, the
// sampler below draws exactly that pmf).
struct Select {
  const uint16_t *cdf;  // nullptr: power
};

__device__ __forceinline__ float select_prob(const ShadeView &sv, const Select &s, uint32_t j) {
  if (!s.cdf) return cdf_mass(sv.sel_cdf, j);
  const uint32_t hi = __ldg(s.cdf + j), lo = j ? __ldg(s.cdf + j - 1) : 0u;
  return (float)(hi - lo) * (1.0f / 65535.0f);
}

__device__ __forceinline__ uint32_t select_pick(const ShadeView &sv, const Select &s, float u) {
  if (!s.cdf) return cdf_pick(sv.sel_cdf, sv.n_emit, u);
  const float x = u * 65535.0f;
  uint32_t lo = 0, hi = sv.n_emit - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (x < (float)__ldg(s.cdf + mid)) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// Solid-angle pdf of the light technique for a direction that meets emitter
// triangle `tri` of light k at distance t with |cos| cl at the emitter.
__device__ __forceinline__ float nee_pdf(const ShadeView &sv, float q, const DevLight &L, uint32_t tri, float t,
                                         float area, float cl) {
  float ptri = cdf_mass(sv.pcdf + L.pcdf, tri - L.first);
  return q * ptri * t * t / (area * cl);
}

}  // namespace ckr
