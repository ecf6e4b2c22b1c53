// trace_stats.cpp — host replay of the device traversal (closest-hit mode) that
// counts the wide nodes and triangles visited per ray.  The counts define the
// algorithmic bytes per ray of the traversal roofline:
//   bytes/ray = 32 (ray) + 8 (id + t) + nodes * 80 + triangles * 36.
// The arithmetic and the visiting order mirror trace_device.cuh (FP32, the same
// fused operations), so the replay reports the device's hits as well.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/ckr.h"
#include "../../include/ckr_test.h"
#include "bvh_build.h"

namespace ckr {
void scene_host_arrays(const ckr_scene *s, const uint32_t **nodes, const float **tris, const float **spheres,
                       int32_t *root, uint32_t *nsph, uint32_t *depth);
}

namespace {

constexpr int32_t kDone = (int32_t)0x80000000;
constexpr float kRobustFar = 1.0000003576278687f;

struct Pre {
  float o[3], d[3], inv[3], tmin;
  float mx[3], my[3], mz[3];
  uint32_t oct;
};

Pre make_pre(const ckr_ray &ray) {
  Pre r;
  r.o[0] = ray.ox; r.o[1] = ray.oy; r.o[2] = ray.oz;
  r.d[0] = ray.dx; r.d[1] = ray.dy; r.d[2] = ray.dz;
  r.tmin = ray.tmin;
  for (int k = 0; k < 3; ++k) {
    float i = 1.0f / r.d[k];
    r.inv[k] = std::fabs(i) > 1e20f ? std::copysign(1e20f, i) : i;  // kMaxInvDir of trace_device.cuh
  }
  float ax = std::fabs(r.d[0]), ay = std::fabs(r.d[1]), az = std::fabs(r.d[2]);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  if (r.d[kz] < 0.f) std::swap(kx, ky);
  float sx = r.d[kx] / r.d[kz], sy = r.d[ky] / r.d[kz], sz = 1.0f / r.d[kz];
  for (int k = 0; k < 3; ++k) {
    r.mx[k] = (kx == k) ? 1.f : (kz == k ? -sx : 0.f);
    r.my[k] = (ky == k) ? 1.f : (kz == k ? -sy : 0.f);
    r.mz[k] = (kz == k) ? sz : 0.f;
  }
  r.oct = 7u ^ ((r.d[0] < 0.f ? 4u : 0u) | (r.d[1] < 0.f ? 2u : 0u) | (r.d[2] < 0.f ? 1u : 0u));
  return r;
}

inline float shear(const float *m, const float *a) { return std::fma(m[0], a[0], std::fma(m[1], a[1], m[2] * a[2])); }

bool hit_tri(const Pre &r, const float *t12, float tbest, float &tout) {
  float a[3], b[3], c[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = t12[k] - r.o[k];
    b[k] = t12[4 + k] - r.o[k];
    c[k] = t12[8 + k] - r.o[k];
  }
  float Ax = shear(r.mx, a), Ay = shear(r.my, a);
  float Bx = shear(r.mx, b), By = shear(r.my, b);
  float Cx = shear(r.mx, c), Cy = shear(r.my, c);
  float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = (float)((double)Cx * By - (double)Cy * Bx);
    V = (float)((double)Ax * Cy - (double)Ay * Cx);
    W = (float)((double)Bx * Ay - (double)By * Ax);
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  float det = U + V + W;
  if (det == 0.f) return false;
  float T = std::fma(U, shear(r.mz, a), std::fma(V, shear(r.mz, b), W * shear(r.mz, c)));
  float t = T / det;
  if (!(t > r.tmin) || !(t < tbest)) return false;
  float e1[3], e2[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = t12[4 + k] - t12[k];
    e2[k] = t12[8 + k] - t12[k];
  }
  float n0 = e2[1] * e1[2] - e2[2] * e1[1], n1 = e2[2] * e1[0] - e2[0] * e1[2], n2 = e2[0] * e1[1] - e2[1] * e1[0];
  float dn = r.d[0] * n0 + r.d[1] * n1 + r.d[2] * n2;
  if (dn * dn <= 1e-10f * (n0 * n0 + n1 * n1 + n2 * n2)) return false;
  tout = t;
  return true;
}

constexpr float kQuantSlack = 2.384185791015625e-07f;

inline float f_of(uint32_t w) {
  float f;
  std::memcpy(&f, &w, 4);
  return f;
}

// a - b and a * b rounded down / up, as the device's __fsub_rd / __fsub_ru /
// __fmul_ru: the round-to-nearest result corrected by the sign of its exact error
// (TwoSum, and the FMA residual of the product).
inline float sub_dir(float a, float b, bool up) {
  const float r = a - b;
  if (!std::isfinite(r)) return r;
  const float bb = a - r, err = (a - (r + bb)) + (bb - b);  // a - b = r + err exactly (nb = -b)
  if (up && err > 0.f) return std::nextafter(r, INFINITY);
  if (!up && err < 0.f) return std::nextafter(r, -INFINITY);
  return r;
}
inline float mul_up(float a, float b) {
  const float p = a * b;
  if (!std::isfinite(p)) return p;
  return std::fma(a, b, -p) > 0.f ? std::nextafter(p, INFINITY) : p;
}

// wide_node of trace_device.cuh.
void wide_node(const uint32_t *w, const Pre &r, float tbest, uint32_t ng[2], uint32_t tg[2]) {
  float sa[3], fa[3], on[3], of[3];
  for (int a = 0; a < 3; ++a) {
    float scale = f_of(((w[3] >> (8 * a)) & 0xffu) << 23);
    sa[a] = scale * r.inv[a] * 32768.f;
    fa[a] = mul_up(sa[a], kRobustFar);
    float o = (f_of(w[a]) - r.o[a]) * r.inv[a];
    on[a] = sub_dir(std::fma(-kQuantSlack, std::fabs(o), o), sa[a], false);
    of[a] = mul_up(sub_dir(std::fma(kQuantSlack, std::fabs(o), o), sa[a], true), kRobustFar);
  }
  uint32_t meta[2] = {w[6], w[7]};
  const uint32_t x4 = r.oct * 0x01010101u;
  for (int h = 0; h < 2; ++h) meta[h] ^= (((meta[h] >> 3) & (meta[h] >> 4) & 0x01010101u) * 7u) & x4;
  uint32_t hits = 0;
  for (int slot = 0; slot < 8; ++slot) {
    const int h = slot >> 2, sh = (slot & 3) * 8;
    float tn[3], tf[3];
    for (int a = 0; a < 3; ++a) {
      const bool neg = r.inv[a] < 0.f;
      const uint32_t lo = w[8 + 4 * a + h], hi = w[10 + 4 * a + h];
      // The byte q as the float 1 + q 2^-15.
      const float qn = f_of(0x3F800000u | ((((neg ? hi : lo) >> sh) & 0xffu) << 8));
      const float qf = f_of(0x3F800000u | ((((neg ? lo : hi) >> sh) & 0xffu) << 8));
      tn[a] = std::fma(qn, sa[a], on[a]);
      tf[a] = std::fma(qf, fa[a], of[a]);
    }
    const float en = std::fmax(std::fmax(tn[0], tn[1]), std::fmax(tn[2], r.tmin));
    const float ex = std::fmin(std::fmin(tf[0], tf[1]), std::fmin(tf[2], tbest));
    const uint32_t m = (meta[h] >> sh) & 0xffu;
    if (en <= ex) hits |= (m >> 5) << (m & 31u);
  }
  ng[0] = w[4];
  ng[1] = (hits & 0xff000000u) | (w[3] >> 24);
  tg[0] = w[5];
  tg[1] = hits & 0x00ffffffu;
}

inline int highest_bit(uint32_t x) { return 31 - __builtin_clz(x); }

uint32_t replay(const uint32_t *nodes, const float *tris, int32_t root, const ckr_ray &ray, uint64_t &nnodes,
                uint64_t &ntris, float &tbest, bool any = false) {
  Pre r = make_pre(ray);
  tbest = ray.tmax;
  uint32_t best = 0xFFFFFFFFu;
  std::vector<std::pair<uint32_t, uint32_t>> stack;
  const bool ok = !std::isnan(r.o[0] + r.o[1] + r.o[2] + r.d[0] + r.d[1] + r.d[2]);
  uint32_t ng[2] = {0u, root == 0 && ok ? 0x80000000u : 0u}, tg[2] = {0u, 0u};
  for (;;) {
    if (tg[1] == 0) {
      if ((ng[1] & 0xff000000u) == 0) {
        if (stack.empty()) break;
        ng[0] = stack.back().first;
        ng[1] = stack.back().second;
        stack.pop_back();
      }
      const int bit = highest_bit(ng[1]);
      ng[1] &= ~(1u << bit);
      const uint32_t slot = (uint32_t)(bit - 24) ^ r.oct;
      const uint32_t child = ng[0] + (uint32_t)__builtin_popcount(ng[1] & ((1u << slot) - 1u) & 0xffu);
      if (ng[1] & 0xff000000u) stack.push_back({ng[0], ng[1]});
      nnodes++;
      wide_node(nodes + (size_t)child * ckr::kWideWords, r, tbest, ng, tg);
    }
    if (tg[1] != 0) {
      const uint32_t k = (uint32_t)__builtin_ctz(tg[1]);
      tg[1] &= tg[1] - 1;
      ntris++;
      float t;
      const float *tp = tris + 12 * (size_t)(tg[0] + k);
      if (hit_tri(r, tp, tbest, t)) {
        tbest = t;
        std::memcpy(&best, &tp[3], 4);
        if (any) break;
      }
    }
  }
  return best;
}

}  // namespace

extern "C" int ckr_trace_stats(const ckr_scene *scene, const ckr_ray *rays, uint32_t n, double *mean_nodes,
                               double *mean_tris) {
  if (!scene || (n && !rays) || !mean_nodes || !mean_tris) return CKR_ERR_INVALID_ARGUMENT;
  const uint32_t *nodes;
  const float *tris, *spheres;
  int32_t root;
  uint32_t nsph, depth;
  ckr::scene_host_arrays(scene, &nodes, &tris, &spheres, &root, &nsph, &depth);
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  std::vector<uint64_t> bx(nt, 0), tr(nt, 0);
  std::vector<std::thread> pool;
  for (unsigned w = 0; w < nt; ++w)
    pool.emplace_back([&, w] {
      float t;
      for (uint64_t i = w; i < n; i += nt) replay(nodes, tris, root, rays[i], bx[w], tr[w], t);
    });
  for (auto &t : pool) t.join();
  uint64_t B = 0, T = 0;
  for (unsigned w = 0; w < nt; ++w) {
    B += bx[w];
    T += tr[w];
  }
  *mean_nodes = n ? (double)B / n : 0.0;
  *mean_tris = n ? (double)T / n : 0.0;
  return CKR_OK;
}

// Host-only replay of the whole closest-hit (any = 0) or any-hit path (SAH build +
// FP32 traversal)
// without a device, for the CPU test suite: it lets the builder and the
// traversal logic be checked against the oracle before any kernel runs.  Not
// part of the public ABI and not used by any product entry point.
extern "C" int ckr_internal_replay(const float *tri9, uint32_t ntri, uint32_t max_leaf, const ckr_ray *rays,
                                   uint32_t n, int any, uint32_t *hit_id, float *hit_t, double *mean_nodes,
                                   double *mean_tris) {
  ckr::FlatBvh bvh;
  ckr_build_params p{max_leaf, 0, 0};
  int st = ckr::build_bvh(tri9, ntri, p, bvh);
  if (st != CKR_OK) return st;
  uint64_t B = 0, T = 0;
  for (uint32_t i = 0; i < n; ++i) {
    float t;
    hit_id[i] = replay(bvh.nodes.data(), bvh.tris.data(), bvh.root, rays[i], B, T, t, any != 0);
    hit_t[i] = t;
  }
  if (mean_nodes) *mean_nodes = n ? (double)B / n : 0.0;
  if (mean_tris) *mean_tris = n ? (double)T / n : 0.0;
  return CKR_OK;
}

// Host-only build with an explicit thread count, for the CPU test suite: an FNV-1a
// digest of the flattened tree (nodes, then triangle records) and its node count,
// so that builds on different numbers of threads can be compared.  Not part of the
// public ABI.
extern "C" int ckr_internal_bvh_digest(const float *tri9, uint32_t ntri, uint32_t max_leaf, uint32_t threads,
                                       uint64_t *digest, uint32_t *nnodes) {
  if (!digest || !nnodes) return CKR_ERR_INVALID_ARGUMENT;
  ckr::FlatBvh bvh;
  ckr_build_params p{max_leaf, 0, threads};
  int st = ckr::build_bvh(tri9, ntri, p, bvh);
  if (st != CKR_OK) return st;
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](const void *data, size_t bytes) {
    const unsigned char *c = static_cast<const unsigned char *>(data);
    for (size_t i = 0; i < bytes; ++i) {
      h ^= c[i];
      h *= 1099511628211ull;
    }
  };
  mix(bvh.nodes.data(), bvh.nodes.size() * sizeof(uint32_t));
  mix(bvh.tris.data(), bvh.tris.size() * sizeof(float));
  *digest = h;
  *nnodes = bvh.nnodes;
  return CKR_OK;
}
