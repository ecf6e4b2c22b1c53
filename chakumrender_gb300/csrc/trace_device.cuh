// trace_device.cuh — device-side ray traversal shared by the trace kernels and
// the path tracer.
//
// Geometry is FP32 and the triangle test is watertight (Woop, Benthin, Wald,
// "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013): the 2-D edge
// functions are evaluated without fused multiply-adds so that the two
// triangles sharing an edge compute exactly negated values, and exact zeros
// are re-evaluated in FP64.  Boxes use the robust slab test of Ize ("Robust
// BVH Ray Traversal", JCGT 2(2), 2013).  Spheres are tested in FP64 exactly as
// the reference's Sphere::intersect (src/geometryPrimitives.cpp:12-27).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ckr {

constexpr int32_t kDone = (int32_t)0x80000000;  // also the root link of an empty tree
constexpr uint32_t kMiss = 0xFFFFFFFFu;
constexpr uint32_t kSphereBit = 0x80000000u;
// 1 + 2 * gamma(3), gamma(n) = n u / (1 - n u), u = 2^-24 (Ize 2013).
constexpr float kRobustFar = 1.0000003576278687f;

struct SceneView {
  const float4 *nodes;    // 4 words per interior node
  const float4 *tris;     // 3 words per triangle, leaf order
  const float4 *spheres;  // centre.xyz, radius
  int32_t root;
  uint32_t nsph;
  int *status;            // first device error (CKR_ERR_*), 0 when none
};

struct RayPre {
  float ox, oy, oz, tmin;
  float dx, dy, dz;
  float ix, iy, iz;        // 1 / d
  float mx0, mx1, mx2;     // shear rows: sheared x = mx . (v - o)
  float my0, my1, my2;
  float mz0, mz1, mz2;
};

#if defined(__CUDACC__)
__device__ __forceinline__ RayPre make_ray(float4 a, float4 b) {
  RayPre r;
  r.ox = a.x; r.oy = a.y; r.oz = a.z; r.tmin = a.w;
  r.dx = b.x; r.dy = b.y; r.dz = b.z;
  r.ix = 1.0f / r.dx; r.iy = 1.0f / r.dy; r.iz = 1.0f / r.dz;
  float ax = fabsf(r.dx), ay = fabsf(r.dy), az = fabsf(r.dz);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  float dkz = kz == 0 ? r.dx : (kz == 1 ? r.dy : r.dz);
  if (dkz < 0.f) { int t = kx; kx = ky; ky = t; }
  float dkx = kx == 0 ? r.dx : (kx == 1 ? r.dy : r.dz);
  float dky = ky == 0 ? r.dx : (ky == 1 ? r.dy : r.dz);
  float sx = dkx / dkz, sy = dky / dkz, sz = 1.0f / dkz;
  r.mx0 = (kx == 0) ? 1.f : (kz == 0 ? -sx : 0.f);
  r.mx1 = (kx == 1) ? 1.f : (kz == 1 ? -sx : 0.f);
  r.mx2 = (kx == 2) ? 1.f : (kz == 2 ? -sx : 0.f);
  r.my0 = (ky == 0) ? 1.f : (kz == 0 ? -sy : 0.f);
  r.my1 = (ky == 1) ? 1.f : (kz == 1 ? -sy : 0.f);
  r.my2 = (ky == 2) ? 1.f : (kz == 2 ? -sy : 0.f);
  r.mz0 = kz == 0 ? sz : 0.f;
  r.mz1 = kz == 1 ? sz : 0.f;
  r.mz2 = kz == 2 ? sz : 0.f;
  return r;
}

// Watertight test of one triangle; on a hit inside (tmin, tbest) stores t and
// returns true.  Also applies the reference's near-parallel rejection
// (d.n)^2 <= 1e-10 with n the unit normal (src/geometryPrimitives.cpp:43).
__device__ __forceinline__ bool hit_triangle(const RayPre &r, float4 v0, float4 v1, float4 v2,
                                             float tbest, float &t_out) {
  float a0 = v0.x - r.ox, a1 = v0.y - r.oy, a2 = v0.z - r.oz;
  float b0 = v1.x - r.ox, b1 = v1.y - r.oy, b2 = v1.z - r.oz;
  float c0 = v2.x - r.ox, c1 = v2.y - r.oy, c2 = v2.z - r.oz;
  float Ax = fmaf(r.mx0, a0, fmaf(r.mx1, a1, r.mx2 * a2));
  float Ay = fmaf(r.my0, a0, fmaf(r.my1, a1, r.my2 * a2));
  float Bx = fmaf(r.mx0, b0, fmaf(r.mx1, b1, r.mx2 * b2));
  float By = fmaf(r.my0, b0, fmaf(r.my1, b1, r.my2 * b2));
  float Cx = fmaf(r.mx0, c0, fmaf(r.mx1, c1, r.mx2 * c2));
  float Cy = fmaf(r.my0, c0, fmaf(r.my1, c1, r.my2 * c2));
  float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (U == 0.f || V == 0.f || W == 0.f) {
    // Products of two floats are exact in FP64, so the signs are exact.
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  float det = U + V + W;
  if (det == 0.f) return false;
  float Az = fmaf(r.mz0, a0, fmaf(r.mz1, a1, r.mz2 * a2));
  float Bz = fmaf(r.mz0, b0, fmaf(r.mz1, b1, r.mz2 * b2));
  float Cz = fmaf(r.mz0, c0, fmaf(r.mz1, c1, r.mz2 * c2));
  float T = fmaf(U, Az, fmaf(V, Bz, W * Cz));
  float t = __fdiv_rn(T, det);
  if (!(t > r.tmin) || !(t < tbest)) return false;
  // Near-parallel rejection on the unit normal n = (C - A) x (B - A) / |.|.
  float e10 = v1.x - v0.x, e11 = v1.y - v0.y, e12 = v1.z - v0.z;
  float e20 = v2.x - v0.x, e21 = v2.y - v0.y, e22 = v2.z - v0.z;
  float n0 = e21 * e12 - e22 * e11, n1 = e22 * e10 - e20 * e12, n2 = e20 * e11 - e21 * e10;
  float dn = r.dx * n0 + r.dy * n1 + r.dz * n2;
  if (dn * dn <= 1e-10f * (n0 * n0 + n1 * n1 + n2 * n2)) return false;
  t_out = t;
  return true;
}

// Sphere::intersect in FP64 (src/geometryPrimitives.cpp:12-27), with the
// root taken above max(tmin, 1e-4).
__device__ __forceinline__ double hit_sphere(const RayPre &r, float4 s) {
  double opx = (double)s.x - r.ox, opy = (double)s.y - r.oy, opz = (double)s.z - r.oz;
  double dx = r.dx, dy = r.dy, dz = r.dz;
  double b = opx * dx + opy * dy + opz * dz;
  double rr = (double)s.w;
  double det = b * b - (opx * opx + opy * opy + opz * opz) + rr * rr;
  if (det < 0.0) return 1e300;
  det = sqrt(det);
  double eps = fmax(1e-4, (double)r.tmin);
  double t = b - det;
  if (t > eps) return t;
  t = b + det;
  return t > eps ? t : 1e300;
}

// Both child boxes of an interior node; returns entry distances (or +inf on a miss).
__device__ __forceinline__ void hit_children(const RayPre &r, float4 n0, float4 n1, float4 n2,
                                             float tbest, float &t0, float &t1) {
  float lx = (n0.x - r.ox) * r.ix, hx = (n0.y - r.ox) * r.ix;
  float ly = (n0.z - r.oy) * r.iy, hy = (n0.w - r.oy) * r.iy;
  float lz = (n2.x - r.oz) * r.iz, hz = (n2.y - r.oz) * r.iz;
  float en = fmaxf(fmaxf(fminf(lx, hx), fminf(ly, hy)), fmaxf(fminf(lz, hz), r.tmin));
  float ex = fminf(fminf(fmaxf(lx, hx), fmaxf(ly, hy)), fmaxf(lz, hz)) * kRobustFar;
  ex = fminf(ex, tbest);
  t0 = en <= ex ? en : __int_as_float(0x7f800000);
  lx = (n1.x - r.ox) * r.ix; hx = (n1.y - r.ox) * r.ix;
  ly = (n1.z - r.oy) * r.iy; hy = (n1.w - r.oy) * r.iy;
  lz = (n2.z - r.oz) * r.iz; hz = (n2.w - r.oz) * r.iz;
  en = fmaxf(fmaxf(fminf(lx, hx), fminf(ly, hy)), fmaxf(fminf(lz, hz), r.tmin));
  ex = fminf(fminf(fmaxf(lx, hx), fmaxf(ly, hy)), fmaxf(lz, hz)) * kRobustFar;
  ex = fminf(ex, tbest);
  t1 = en <= ex ? en : __int_as_float(0x7f800000);
}

// One traversal step of a ray: an interior node (both child boxes; the nearer hit
// child next, the farther pushed) or a leaf (its triangles, then a pop).  `node` is
// kDone when the ray is finished.  Stack as in trace_ray.
template <bool ANY>
__device__ __forceinline__ void trace_step(const SceneView &s, const RayPre &r, float &tbest, uint32_t &best,
                                           int32_t &node, int &sp, int32_t *stack, int stride, int depth) {
  if (node >= 0) {
    const float4 *np = s.nodes + 4 * (size_t)node;
    float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3);
    float t0, t1;
    hit_children(r, n0, n1, n2, tbest, t0, t1);
    int32_t l0 = __float_as_int(n3.x), l1 = __float_as_int(n3.y);
    bool h0 = t0 != __int_as_float(0x7f800000), h1 = t1 != __int_as_float(0x7f800000);
    if (h0 && h1) {
      int32_t near = l0, far = l1;
      if (t1 < t0) { near = l1; far = l0; }
      if (sp >= depth) {
        atomicCAS(s.status, 0, -4 /* CKR_ERR_STACK_OVERFLOW */);
        best = kMiss;
        node = kDone;
        return;
      }
      stack[sp * stride] = far;
      ++sp;
      node = near;
    } else if (h0 | h1) {
      node = h0 ? l0 : l1;
    } else {
      node = sp > 0 ? stack[--sp * stride] : kDone;
    }
    return;
  }
  // Leaf: ~node = (first << 3) | (count - 1).
  uint32_t code = ~(uint32_t)node;
  uint32_t first = code >> 3, count = (code & 7u) + 1u;
  const float4 *tp = s.tris + 3 * (size_t)first;
  for (uint32_t k = 0; k < count; ++k) {
    float4 v0 = __ldg(tp + 3 * k), v1 = __ldg(tp + 3 * k + 1), v2 = __ldg(tp + 3 * k + 2);
    float t;
    if (hit_triangle(r, v0, v1, v2, tbest, t)) {
      tbest = t;
      best = __float_as_uint(v0.w);
      if (ANY) {
        node = kDone;
        return;
      }
    }
  }
  node = sp > 0 ? stack[--sp * stride] : kDone;
}

// Traces one ray.  ANY: stop at the first hit.  The stack lives in shared
// memory, one column per thread (stack[level * stride]), `depth` entries.
// Returns the hit id (kMiss, triangle index, or kSphereBit | sphere index)
// and updates tbest to the hit distance.
template <bool ANY>
__device__ __forceinline__ uint32_t trace_ray(const SceneView &s, const RayPre &r, float &tbest,
                                              int32_t *stack, int stride, int depth) {
  uint32_t best = kMiss;
  for (uint32_t k = 0; k < s.nsph; ++k) {
    double t = hit_sphere(r, __ldg(&s.spheres[k]));
    if (t < (double)tbest) {
      tbest = (float)t;
      best = kSphereBit | k;
      if (ANY) return best;
    }
  }
  int32_t node = s.root;
  int sp = 0;
  while (node != kDone) {
    if (node >= 0) {
      const float4 *np = s.nodes + 4 * (size_t)node;
      float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3);
      float t0, t1;
      hit_children(r, n0, n1, n2, tbest, t0, t1);
      int32_t l0 = __float_as_int(n3.x), l1 = __float_as_int(n3.y);
      bool h0 = t0 != __int_as_float(0x7f800000), h1 = t1 != __int_as_float(0x7f800000);
      if (h0 && h1) {
        int32_t near = l0, far = l1;
        if (t1 < t0) { near = l1; far = l0; }
        if (sp >= depth) {
          atomicCAS(s.status, 0, -4 /* CKR_ERR_STACK_OVERFLOW */);
          return kMiss;
        }
        stack[sp * stride] = far;
        ++sp;
        node = near;
      } else if (h0 | h1) {
        node = h0 ? l0 : l1;
      } else {
        node = sp > 0 ? stack[--sp * stride] : kDone;
      }
      continue;
    }
    // Leaf: ~node = (first << 3) | (count - 1).
    uint32_t code = ~(uint32_t)node;
    uint32_t first = code >> 3, count = (code & 7u) + 1u;
    const float4 *tp = s.tris + 3 * (size_t)first;
    for (uint32_t k = 0; k < count; ++k) {
      float4 v0 = __ldg(tp + 3 * k), v1 = __ldg(tp + 3 * k + 1), v2 = __ldg(tp + 3 * k + 2);
      float t;
      if (hit_triangle(r, v0, v1, v2, tbest, t)) {
        tbest = t;
        best = __float_as_uint(v0.w);
        if (ANY) return best;
      }
    }
    node = sp > 0 ? stack[--sp * stride] : kDone;
  }
  return best;
}

#endif  // __CUDACC__
}  // namespace ckr
