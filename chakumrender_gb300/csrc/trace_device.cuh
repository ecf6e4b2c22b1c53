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
  const float4 *nodes;    // 5 words per wide node (layout in bvh_build.h)
  const float4 *tris;     // 3 words per triangle, leaf order
  const float4 *spheres;  // centre.xyz, radius
  int32_t root;           // 0, or kDone when no triangle is indexed
  uint32_t nsph;
  int *status;            // first device error (CKR_ERR_*), 0 when none
  const uint4 *slot_bits; // per wide node, its eight slots' hit bits (two uint4)
};

struct RayPre {
  float ox, oy, oz, tmin;
  float dx, dy, dz;
  float ix, iy, iz;        // 1 / d
  float mx0, mx1, mx2;     // shear rows: sheared x = mx . (v - o)
  float my0, my1, my2;
  float mz0, mz1, mz2;
  uint32_t oct;            // 7 ^ octant (bit 2: dx < 0, bit 1: dy < 0, bit 0: dz < 0)
};

// Largest |1/d| the slab tests use.  A ray with d = +-0 on an axis must keep an
// exact test on that axis (its origin inside the slab or not); with 1/d = inf
// the quantised test would compute 0 * inf = NaN, drop the axis, and visit every
// node the other two axes admit.  With 1/d capped the test is that of a ray
// tilted by at most 1e-20 per unit length, which moves no hit by a
// representable amount at scene coordinates.
constexpr float kMaxInvDir = 1e20f;

#if defined(__CUDACC__)
__device__ __forceinline__ float inv_dir(float d) {
  const float i = 1.0f / d;
  return fabsf(i) > kMaxInvDir ? copysignf(kMaxInvDir, i) : i;
}

__device__ __forceinline__ RayPre make_ray(float4 a, float4 b) {
  RayPre r;
  r.ox = a.x; r.oy = a.y; r.oz = a.z; r.tmin = a.w;
  r.dx = b.x; r.dy = b.y; r.dz = b.z;
  r.ix = inv_dir(r.dx); r.iy = inv_dir(r.dy); r.iz = inv_dir(r.dz);
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
  r.oct = 7u ^ ((r.dx < 0.f ? 4u : 0u) | (r.dy < 0.f ? 2u : 0u) | (r.dz < 0.f ? 1u : 0u));
  return r;
}

// Watertight test of one triangle; on a hit inside (tmin, tbest) stores t and
// returns true.  Also applies the reference's near-parallel rejection
// (d.n)^2 <= 1e-10 with n the unit normal (src/geometryPrimitives.cpp:43).
// What the triangle test reads of a ray besides its origin and tmin: the shear rows
// and the direction (RayPre::m*, d*), for callers that keep them outside RayPre.
struct Shear {
  float mx0, mx1, mx2, my0, my1, my2, mz0, mz1, mz2, dx, dy, dz;
};

__device__ __forceinline__ bool hit_triangle_sheared(const RayPre &r, const Shear &m, float4 v0, float4 v1,
                                                     float4 v2, float tbest, float &t_out);

__device__ __forceinline__ bool hit_triangle(const RayPre &r, float4 v0, float4 v1, float4 v2,
                                             float tbest, float &t_out) {
  const Shear m{r.mx0, r.mx1, r.mx2, r.my0, r.my1, r.my2, r.mz0, r.mz1, r.mz2, r.dx, r.dy, r.dz};
  return hit_triangle_sheared(r, m, v0, v1, v2, tbest, t_out);
}

__device__ __forceinline__ bool hit_triangle_sheared(const RayPre &r, const Shear &m, float4 v0, float4 v1,
                                                     float4 v2, float tbest, float &t_out) {
  float a0 = v0.x - r.ox, a1 = v0.y - r.oy, a2 = v0.z - r.oz;
  float b0 = v1.x - r.ox, b1 = v1.y - r.oy, b2 = v1.z - r.oz;
  float c0 = v2.x - r.ox, c1 = v2.y - r.oy, c2 = v2.z - r.oz;
  float Ax = fmaf(m.mx0, a0, fmaf(m.mx1, a1, m.mx2 * a2));
  float Ay = fmaf(m.my0, a0, fmaf(m.my1, a1, m.my2 * a2));
  float Bx = fmaf(m.mx0, b0, fmaf(m.mx1, b1, m.mx2 * b2));
  float By = fmaf(m.my0, b0, fmaf(m.my1, b1, m.my2 * b2));
  float Cx = fmaf(m.mx0, c0, fmaf(m.mx1, c1, m.mx2 * c2));
  float Cy = fmaf(m.my0, c0, fmaf(m.my1, c1, m.my2 * c2));
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
  float Az = fmaf(m.mz0, a0, fmaf(m.mz1, a1, m.mz2 * a2));
  float Bz = fmaf(m.mz0, b0, fmaf(m.mz1, b1, m.mz2 * b2));
  float Cz = fmaf(m.mz0, c0, fmaf(m.mz1, c1, m.mz2 * c2));
  float T = fmaf(U, Az, fmaf(V, Bz, W * Cz));
  float t = __fdiv_rn(T, det);
  if (!(t > r.tmin) || !(t < tbest)) return false;
  // Near-parallel rejection on the unit normal n = (C - A) x (B - A) / |.|.
  float e10 = v1.x - v0.x, e11 = v1.y - v0.y, e12 = v1.z - v0.z;
  float e20 = v2.x - v0.x, e21 = v2.y - v0.y, e22 = v2.z - v0.z;
  float n0 = e21 * e12 - e22 * e11, n1 = e22 * e10 - e20 * e12, n2 = e20 * e11 - e21 * e10;
  float dn = m.dx * n0 + m.dy * n1 + m.dz * n2;
  if (dn * dn <= 1e-10f * (n0 * n0 + n1 * n1 + n2 * n2)) return false;
  t_out = t;
  return true;
}

// Sphere::intersect in FP64 (src/geometryPrimitives.cpp:12-27), with the
// root taken above max(tmin, 1e-4).
// LEAVING: also the second pre-test, for rays leaving the sphere.  The traversal
// kernels with dynamic fetching leave it out: their scenes here have no spheres, and
// the extra code in their refill path cost 0.7 % (many-light frame, A/B).
template <bool LEAVING = true>
__device__ __forceinline__ double hit_sphere(const RayPre &r, float4 s) {
  {
    // FP32 pre-tests (FP64 is slow on this part).  A ray whose line passes the sphere
    // by more than 1e-5 of the squared magnitudes involved -- orders of magnitude
    // above the FP32 rounding of these few operations -- has a negative FP64
    // discriminant too, so the miss is decided without FP64.  The rounding of b =
    // (c - o).d grows with |d|, so the bound scales the (c - o) terms by
    // max(1, |d|^2): directions need not have unit length.  NaN and overflow fall
    // through to the FP64 test.
    const float ox = s.x - r.ox, oy = s.y - r.oy, oz = s.z - r.oz;
    const float b = ox * r.dx + oy * r.dy + oz * r.dz;
    const float oo = ox * ox + oy * oy + oz * oz;
    const float dd = fmaxf(1.f, r.dx * r.dx + r.dy * r.dy + r.dz * r.dz);
    const float m = fmaxf(fmaxf(fmaxf(fabsf(s.x), fabsf(s.y)), fabsf(s.z)),
                          fmaxf(fmaxf(fabsf(r.ox), fabsf(r.oy)), fabsf(r.oz)));
    const float T = (m * m + oo) * dd + b * b + s.w * s.w;
    const float det = b * b - oo + s.w * s.w;
    if (det < -1e-5f * T) return 1e300;
    // A ray leaving the sphere (bounce and shadow rays from its surface, rays moving
    // away from it): the far root b + sqrt(det) is below 5e-5 even with b and det
    // raised by bounds on their FP32 rounding (4e-6 sqrt(T) and 4e-6 T, several times
    // the few-ulp errors of these sums), so both roots are below the 1e-4 the FP64 test
    // requires and it would report a miss.  NaN fails the comparison.
    if constexpr (LEAVING) {
      const float t2u = (b + 4e-6f * sqrtf(T)) + sqrtf(fmaxf(0.f, det + 4e-6f * T));
      if (t2u < 5e-5f) return 1e300;
    }
  }
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

// Slack of the quantised slab test, 4 u (u = 2^-24).  The entry distance of a
// quantised plane p + q 2^e is q a + o with a = 2^e / d and o = (p - o_ray) / d,
// and o is rounded twice; widening o by 4 u of its magnitude (down for the near
// plane, up for the far one) bounds that rounding so that the computed interval
// contains the exact one up to the relative factor that kRobustFar absorbs, as in
// Ize's robust test.
constexpr float kQuantSlack = 2.384185791015625e-07f;

// Tests the eight child boxes of wide node `node` (layout in bvh_build.h).  Two
// forms of the same conservative test: PERMUTE, a plane byte becomes a float
// through a byte permute folded into the plane's FMA (no integer-to-float
// conversions on the XU pipe: the traversal kernels, 2.27 -> 2.20 ms per 2^23
// rays); otherwise through an integer-to-float conversion, whose per-node set-up
// needs fewer registers (the renderer's one-ray-per-thread kernels, capped at 64
// registers, spill with the first form and ran 5-10 % slower).  A slot's hit bits
// are either assembled from its meta byte or, with Tri::kSlotBits (the traversal
// kernels), read from the scene's slot_bits array.  Out:
// ng = (child_base, hit interior children at bits 24 + (slot ^ oct) | imask),
// tg = (tri_base, hit triangles at their offsets from tri_base).
template <bool PERMUTE, class Tri>
__device__ __forceinline__ void wide_node(const SceneView &s, const RayPre &r, float tbest, uint32_t node,
                                          uint2 &ng, uint2 &tg, const Tri &tri) {
  const float4 *np = s.nodes + 5 * (size_t)node;
  // With slot bits (Tri::kSlotBits) each slot's hit bits come ready-made from the
  // scene's slot_bits array instead of being assembled from its meta byte.
  uint4 cb0 = make_uint4(0, 0, 0, 0), cb1 = cb0;
  if constexpr (Tri::kSlotBits) {
    cb0 = __ldg(s.slot_bits + 2 * (size_t)node);
    cb1 = __ldg(s.slot_bits + 2 * (size_t)node + 1);
  }
  const float4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
  const uint32_t ei = __float_as_uint(w0.w);
  const float ax = __fmul_rn(__uint_as_float((ei & 0xffu) << 23), r.ix);
  const float ay = __fmul_rn(__uint_as_float(((ei >> 8) & 0xffu) << 23), r.iy);
  const float az = __fmul_rn(__uint_as_float(((ei >> 16) & 0xffu) << 23), r.iz);
  const float ox = __fmul_rn(__fsub_rn(w0.x, r.ox), r.ix);
  const float oy = __fmul_rn(__fsub_rn(w0.y, r.oy), r.iy);
  const float oz = __fmul_rn(__fsub_rn(w0.z, r.oz), r.iz);
  float sax, say, saz, fax, fay, faz, nox, noy, noz, fox, foy, foz;
  if constexpr (PERMUTE) {
    // A plane byte q is read as the float 1 + q 2^-15 (one byte permute puts q in
    // mantissa bits 8..15 of 1.0f, no integer-to-float conversion), so its distance
    // q a + o is fma(1 + q 2^-15, 2^15 a, o - 2^15 a).  2^15 a is exact, and
    // o - 2^15 a is rounded down for near planes and up for far ones, so the FMA's
    // exact value is never inside q a + o; one rounding follows, as with fma(q, a, o).
    sax = ax * 32768.f;
    say = ay * 32768.f;
    saz = az * 32768.f;
    nox = __fsub_rd(__fmaf_rn(-kQuantSlack, fabsf(ox), ox), sax);
    noy = __fsub_rd(__fmaf_rn(-kQuantSlack, fabsf(oy), oy), say);
    noz = __fsub_rd(__fmaf_rn(-kQuantSlack, fabsf(oz), oz), saz);
    // Far planes also carry kRobustFar, in both FMA operands and rounded up, so that
    // the exit is min(far planes, tbest) with no multiply per child.
    fax = __fmul_ru(sax, kRobustFar);
    fay = __fmul_ru(say, kRobustFar);
    faz = __fmul_ru(saz, kRobustFar);
    fox = __fmul_ru(__fsub_ru(__fmaf_rn(kQuantSlack, fabsf(ox), ox), sax), kRobustFar);
    foy = __fmul_ru(__fsub_ru(__fmaf_rn(kQuantSlack, fabsf(oy), oy), say), kRobustFar);
    foz = __fmul_ru(__fsub_ru(__fmaf_rn(kQuantSlack, fabsf(oz), oz), saz), kRobustFar);
  } else {
    sax = fax = ax;
    say = fay = ay;
    saz = faz = az;
    nox = __fmaf_rn(-kQuantSlack, fabsf(ox), ox);
    fox = __fmaf_rn(kQuantSlack, fabsf(ox), ox);
    noy = __fmaf_rn(-kQuantSlack, fabsf(oy), oy);
    foy = __fmaf_rn(kQuantSlack, fabsf(oy), oy);
    noz = __fmaf_rn(-kQuantSlack, fabsf(oz), oz);
    foz = __fmaf_rn(kQuantSlack, fabsf(oz), oz);
  }
  // Near planes are the lo planes on axes the ray travels up, the hi planes otherwise.
  const bool sx = r.ix < 0.f, sy = r.iy < 0.f, sz = r.iz < 0.f;
  const uint32_t lx0 = __float_as_uint(w2.x), lx1 = __float_as_uint(w2.y);
  const uint32_t hx0 = __float_as_uint(w2.z), hx1 = __float_as_uint(w2.w);
  const uint32_t ly0 = __float_as_uint(w3.x), ly1 = __float_as_uint(w3.y);
  const uint32_t hy0 = __float_as_uint(w3.z), hy1 = __float_as_uint(w3.w);
  const uint32_t lz0 = __float_as_uint(w4.x), lz1 = __float_as_uint(w4.y);
  const uint32_t hz0 = __float_as_uint(w4.z), hz1 = __float_as_uint(w4.w);
  const uint32_t nx[2] = {sx ? hx0 : lx0, sx ? hx1 : lx1}, fx[2] = {sx ? lx0 : hx0, sx ? lx1 : hx1};
  const uint32_t ny[2] = {sy ? hy0 : ly0, sy ? hy1 : ly1}, fy[2] = {sy ? ly0 : hy0, sy ? ly1 : hy1};
  const uint32_t nz[2] = {sz ? hz0 : lz0, sz ? hz1 : lz1}, fz[2] = {sz ? lz0 : hz0, sz ? lz1 : hz1};
  // Without slot bits, interior slots' meta bytes (0x38 + slot) become 0x38 + (slot ^
  // oct): their hit bit then orders the children front to back for the ray's octant.
  const uint32_t x4 = r.oct * 0x01010101u;
  uint32_t meta[2] = {__float_as_uint(w1.z), __float_as_uint(w1.w)};
  if constexpr (!Tri::kSlotBits)
#pragma unroll
    for (int h = 0; h < 2; ++h) meta[h] ^= (((meta[h] >> 3) & (meta[h] >> 4) & 0x01010101u) * 7u) & x4;
  uint32_t hits = 0;
#pragma unroll
  for (int slot = 0; slot < 8; ++slot) {
    const int h = slot >> 2, sh = (slot & 3) * 8;
    // The plane byte of this slot as the FMA's first operand.
    const uint32_t sel = 0x7604u | ((uint32_t)(slot & 3) << 4);
    auto qf = [&](uint32_t w) {
      return PERMUTE ? __uint_as_float(__byte_perm(w, 0x3F800000u, sel)) : __uint2float_rn((w >> sh) & 0xffu);
    };
    const float tnx = __fmaf_rn(qf(nx[h]), sax, nox), tfx = __fmaf_rn(qf(fx[h]), fax, fox);
    const float tny = __fmaf_rn(qf(ny[h]), say, noy), tfy = __fmaf_rn(qf(fy[h]), fay, foy);
    const float tnz = __fmaf_rn(qf(nz[h]), saz, noz), tfz = __fmaf_rn(qf(fz[h]), faz, foz);
    const float en = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, r.tmin));
    const float ex = PERMUTE ? fminf(fminf(tfx, tfy), fminf(tfz, tbest))
                             : fminf(__fmul_rn(fminf(fminf(tfx, tfy), tfz), kRobustFar), tbest);
    // The slot's hit bits: its pattern (bits 5..7 of the meta byte) shifted to its
    // position (bits 0..4).  The funnel shift wraps its shift amount, so the bits
    // above the byte's low five need not be masked off.
    if constexpr (Tri::kSlotBits) {
      const uint32_t cw[8] = {cb0.x, cb0.y, cb0.z, cb0.w, cb1.x, cb1.y, cb1.z, cb1.w};
      if (en <= ex) hits |= cw[slot];
      continue;
    }
    const uint32_t m = meta[h] >> sh;
    if (en <= ex) hits |= __funnelshift_l(0u, (m >> 5) & 7u, m);
  }
  // Slot bits keep interior children at 24 + slot: one table lookup moves them to
  // 24 + (slot ^ oct) for the ray's octant.
  if constexpr (Tri::kSlotBits) hits = (hits & 0x00ffffffu) | ((uint32_t)tri.lut[(r.oct << 8) | (hits >> 24)] << 24);
  ng = make_uint2(__float_as_uint(w1.x), (hits & 0xff000000u) | (ei >> 24));
  tg = make_uint2(__float_as_uint(w1.y), hits & 0x00ffffffu);
}

// Traversal state of one ray: ng = the node group being expanded (child_base,
// remaining interior-child hit bits | imask), tg = the triangles still to test
// (tri_base, hit bits), sp = node groups on the stack.
struct Trav {
  uint2 ng, tg;
  int sp;
};

// A pseudo group whose only hit bit selects node 0, the root.  A ray with a NaN
// origin or direction can hit nothing (every triangle test fails) but would pass
// every box test, so it does not enter the tree.
__device__ __forceinline__ Trav trav_start(const SceneView &s, const RayPre &r) {
  const bool ok = !isnan(r.ox + r.oy + r.oz + r.dx + r.dy + r.dz);
  return Trav{make_uint2(0u, s.root == 0 && ok ? 0x80000000u : 0u), make_uint2(0u, 0u), 0};
}

// One traversal step: when no triangle is pending, visits the next node (the
// group's highest-priority hit child; the rest of the group is pushed), then
// tests one pending triangle.  The stack lives in shared memory, one column per
// thread (stack[level * stride]), `depth` entries.  Returns false when the ray is
// finished (ANY: at its first hit).
// `any` is a compile-time constant in the traversal kernels (trace_step<ANY>);
// the persistent renderer passes it at run time so that one copy of the loop
// serves its closest-hit and shadow rays.
// The traversal policy of trace_step: where the triangle test reads the ray's shear
// rows and direction (by default the ray's own registers; TriShearSmem reads them
// from shared memory) and which form of the box test wide_node uses.
struct TriInRegs {
  static constexpr bool kPermutePlanes = false;
  static constexpr bool kSlotBits = false;
  static constexpr bool kSphereLeaving = true;
  const uint8_t *lut = nullptr;
  __device__ __forceinline__ bool operator()(const RayPre &r, float4 v0, float4 v1, float4 v2, float tbest,
                                             float &t) const {
    return hit_triangle(r, v0, v1, v2, tbest, t);
  }
};

template <class Tri = TriInRegs>
__device__ __forceinline__ bool trace_step_rt(const SceneView &s, const RayPre &r, float &tbest, uint32_t &best,
                                              Trav &st, uint2 *stack, int stride, int depth, const bool ANY,
                                              Tri tri = Tri{}) {
  // One exit at the end: early returns for the any-hit case split the warp's
  // control flow and cost more issue slots than the work they skip.
  bool live = true;
  if (st.tg.y == 0) {
    if ((st.ng.y & 0xff000000u) == 0) {
      if (st.sp == 0)
        live = false;
      else
        st.ng = stack[--st.sp * stride];
    }
    if (live) {
      const uint32_t bit = 31 - __clz(st.ng.y);
      st.ng.y &= ~(1u << bit);
      const uint32_t slot = (bit - 24) ^ r.oct;
      const uint32_t child = st.ng.x + __popc(st.ng.y & ((1u << slot) - 1u) & 0xffu);
      if (st.ng.y & 0xff000000u) {
        if (st.sp < depth) {
          stack[st.sp++ * stride] = st.ng;
        } else {
          atomicCAS(s.status, 0, -4 /* CKR_ERR_STACK_OVERFLOW */);
          best = kMiss;
          live = false;
        }
      }
      if (live) wide_node<Tri::kPermutePlanes>(s, r, tbest, child, st.ng, st.tg, tri);
    }
  }
  if (live && st.tg.y != 0) {
    const uint32_t k = __ffs(st.tg.y) - 1;
    st.tg.y &= st.tg.y - 1;
    const float4 *tp = s.tris + 3 * (size_t)(st.tg.x + k);
    const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
    float t;
    if (tri(r, v0, v1, v2, tbest, t)) {
      tbest = t;
      best = __float_as_uint(v0.w);
      if (ANY) live = false;
    }
  }
  return live;
}

template <bool ANY, class Tri = TriInRegs>
__device__ __forceinline__ bool trace_step(const SceneView &s, const RayPre &r, float &tbest, uint32_t &best,
                                           Trav &st, uint2 *stack, int stride, int depth, Tri tri = Tri{}) {
  return trace_step_rt(s, r, tbest, best, st, stack, stride, depth, ANY, tri);
}

// Spheres of the scene, tested before the triangles.  Returns false when ANY is
// satisfied by a sphere.
template <bool LEAVING = true>
__device__ __forceinline__ bool trace_spheres_rt(const SceneView &s, const RayPre &r, float &tbest, uint32_t &best,
                                                 const bool ANY) {
  for (uint32_t k = 0; k < s.nsph; ++k) {
    double t = hit_sphere<LEAVING>(r, __ldg(&s.spheres[k]));
    if (t < (double)tbest) {
      tbest = (float)t;
      best = kSphereBit | k;
      if (ANY) return false;
    }
  }
  return true;
}

template <bool ANY>
__device__ __forceinline__ bool trace_spheres(const SceneView &s, const RayPre &r, float &tbest, uint32_t &best) {
  return trace_spheres_rt(s, r, tbest, best, ANY);
}

// Traces one ray.  ANY: stop at the first hit.  Returns the hit id (kMiss,
// triangle index, or kSphereBit | sphere index) and updates tbest to the hit
// distance.
template <bool ANY>
__device__ __forceinline__ uint32_t trace_ray(const SceneView &s, const RayPre &r, float &tbest, uint2 *stack,
                                              int stride, int depth) {
  uint32_t best = kMiss;
  if (!trace_spheres<ANY>(s, r, tbest, best)) return best;
  Trav st = trav_start(s, r);
  while (trace_step<ANY>(s, r, tbest, best, st, stack, stride, depth)) {
  }
  return best;
}

// trace_ray with `any` chosen at run time, not inlined: one copy of the traversal
// for callers that trace both kinds of ray from one loop (persistent.cuh).
static __device__ __noinline__ uint32_t trace_ray_rt(const SceneView &s, const RayPre &r, float &tbest, uint2 *stack,
                                              int stride, int depth, bool any) {
  uint32_t best = kMiss;
  if (!trace_spheres_rt(s, r, tbest, best, any)) return best;
  Trav st = trav_start(s, r);
  while (trace_step_rt(s, r, tbest, best, st, stack, stride, depth, any)) {
  }
  return best;
}

// Lanes of a warp take new work once this many of them are idle (swept: 4 and 16
// were 4 % and 6 % slower on the 1.3M-triangle workload).
constexpr int kRefill = 8;

// Traversal loop with dynamic ray fetching (after Aila and Laine, "Understanding
// the Efficiency of Ray Traversal on GPUs", HPG 2009): a lane whose ray is finished
// takes the next work item from the global counter `next` (one atomicAdd per warp
// refill, for as many items as the warp has idle lanes) instead of idling until its
// whole warp is done; each iteration advances every active lane by one trace_step.
// Taking 32..128 items per atomic into a warp-private range was 4-5 % slower.  The
// caller zeroes `next` before the launch and runs every lane of every warp through
// here (the loop votes over full warps).
//   fetch(i, r, tbest) -> bool: sets up work item i < n (ray, tmax); false skips it.
//   finish(i, best, tbest): stores the result of item i.
// The triangle test's ray data (shear rows and direction, Shear) kept in shared
// memory instead of registers: three float4 per thread in a column of stride TPB
// after the traversal stacks (depth x TPB uint2), written once per ray by the
// kernel's fetch and read back by the triangle test (2.5 tests per ray against 11
// node visits on the 1.3M-triangle mesh).  Frees twelve registers across the
// traversal loop.
constexpr size_t shear_smem_bytes(int tpb) { return 3 * (size_t)tpb * sizeof(float4); }

template <int TPB>
__device__ __forceinline__ float4 *shear_column(uint2 *smem_stacks, int depth) {
  return reinterpret_cast<float4 *>(smem_stacks + (size_t)depth * TPB) + threadIdx.x;
}

template <int TPB>
__device__ __forceinline__ void store_shear(float4 *col, const RayPre &r) {
  col[0] = make_float4(r.mx0, r.mx1, r.mx2, r.my0);
  col[TPB] = make_float4(r.my1, r.my2, r.mz0, r.mz1);
  col[2 * TPB] = make_float4(r.mz2, r.dx, r.dy, r.dz);
}

// The octant table of slot bits: lut[oct * 256 + x] has bit s ^ oct set for every
// bit s of x, so the interior children's hit bits, kept at 24 + slot in the scene's
// slot_bits, move to 24 + (slot ^ oct) with one shared-memory load per node.  Filled
// by the block at kernel start (the call ends with a block barrier).
constexpr size_t kSlotLutBytes = 2048;

template <int TPB>
__device__ __forceinline__ const uint8_t *fill_slot_lut(uint8_t *lut) {
  for (uint32_t i = threadIdx.x; i < kSlotLutBytes; i += TPB) {
    const uint32_t o = i >> 8, x = i & 255u;
    uint32_t y = 0;
    for (uint32_t b = 0; b < 8; ++b)
      if (x >> b & 1u) y |= 1u << (b ^ o);
    lut[i] = (uint8_t)y;
  }
  __syncthreads();
  return lut;
}

template <int TPB, bool PERMUTE, bool SLOTBITS = false>
struct TriShearSmem {
  static constexpr bool kPermutePlanes = PERMUTE;
  static constexpr bool kSlotBits = SLOTBITS;
  static constexpr bool kSphereLeaving = false;
  const float4 *col;  // this thread's first float4 (shear_column)
  const uint8_t *lut = nullptr;
  __device__ __forceinline__ bool operator()(const RayPre &r, float4 v0, float4 v1, float4 v2, float tbest,
                                             float &t) const {
    const float4 p = col[0], q = col[TPB], u = col[2 * TPB];
    const Shear m{p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w, u.x, u.y, u.z, u.w};
    return hit_triangle_sheared(r, m, v0, v1, v2, tbest, t);
  }
};

template <bool ANY, class Fetch, class Finish, class Tri = TriInRegs>
__device__ __forceinline__ void trace_dynamic(const SceneView &s, uint32_t n, uint32_t *next, uint2 *stack,
                                              int stride, int depth, Fetch fetch, Finish finish, Tri tri = Tri{}) {
  const uint32_t lane = threadIdx.x & 31u;
  RayPre r{};
  float tbest = 0.f;
  uint32_t best = kMiss, idx = 0;
  Trav st{};
  bool active = false, live = false, more = true;
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !active);
    if (more && (idle == 0xffffffffu || __popc(idle) >= kRefill)) {
      const uint32_t want = (uint32_t)__popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(next, want);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((uint64_t)base + want >= n) more = false;
      if (!active) {
        idx = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (idx < n && fetch(idx, r, tbest)) {
          best = kMiss;
          st = trav_start(s, r);
          live = trace_spheres_rt<Tri::kSphereLeaving>(s, r, tbest, best, ANY);
          active = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) {
      if (!more) break;
      continue;  // every lane idle: the next iteration refills the whole warp
    }
    if (active) {
      if (live) live = trace_step<ANY>(s, r, tbest, best, st, stack, stride, depth, tri);
      if (!live) {
        finish(idx, best, tbest);
        active = false;
      }
    }
  }
}

// The same work with one item per thread in a grid-stride loop: faster than
// trace_dynamic when every traversal is a step or two (trees of one or two
// levels), where the votes and refills cost more than the idle lanes.
template <bool ANY, int TPB, class Fetch, class Finish>
__device__ __forceinline__ void trace_static(const SceneView &s, uint32_t n, uint2 *stack, int depth, Fetch fetch,
                                             Finish finish) {
  for (uint32_t i = blockIdx.x * TPB + threadIdx.x; i < n; i += gridDim.x * TPB) {
    RayPre r;
    float t;
    if (!fetch(i, r, t)) continue;
    const uint32_t best = trace_ray<ANY>(s, r, t, stack, TPB, depth);
    finish(i, best, t);
  }
}

#endif  // __CUDACC__
}  // namespace ckr
