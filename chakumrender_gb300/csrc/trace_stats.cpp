// trace_stats.cpp — host replay of the device traversal (closest-hit mode) that
// counts child boxes and triangles tested per ray.  The counts define the
// algorithmic bytes per ray of the traversal roofline:
//   bytes/ray = 32 (ray) + 8 (id + t) + boxes * 32 + triangles * 36.
// The arithmetic mirrors trace_device.cuh (FP32, the same fused operations).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/ckr.h"
#include "bvh_build.h"

namespace ckr {
void scene_host_arrays(const ckr_scene *s, const float **nodes, const float **tris, const float **spheres,
                       int32_t *root, uint32_t *nsph, uint32_t *depth);
}

namespace {

constexpr int32_t kDone = (int32_t)0x80000000;
constexpr float kRobustFar = 1.0000003576278687f;

struct Pre {
  float o[3], d[3], inv[3], tmin;
  float mx[3], my[3], mz[3];
};

Pre make_pre(const ckr_ray &ray) {
  Pre r;
  r.o[0] = ray.ox; r.o[1] = ray.oy; r.o[2] = ray.oz;
  r.d[0] = ray.dx; r.d[1] = ray.dy; r.d[2] = ray.dz;
  r.tmin = ray.tmin;
  for (int k = 0; k < 3; ++k) r.inv[k] = 1.0f / r.d[k];
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

float child_entry(const Pre &r, float lx_, float hx_, float ly_, float hy_, float lz_, float hz_, float tbest) {
  float lx = (lx_ - r.o[0]) * r.inv[0], hx = (hx_ - r.o[0]) * r.inv[0];
  float ly = (ly_ - r.o[1]) * r.inv[1], hy = (hy_ - r.o[1]) * r.inv[1];
  float lz = (lz_ - r.o[2]) * r.inv[2], hz = (hz_ - r.o[2]) * r.inv[2];
  float en = std::fmax(std::fmax(std::fmin(lx, hx), std::fmin(ly, hy)), std::fmax(std::fmin(lz, hz), r.tmin));
  float ex = std::fmin(std::fmin(std::fmax(lx, hx), std::fmax(ly, hy)), std::fmax(lz, hz)) * kRobustFar;
  ex = std::fmin(ex, tbest);
  return en <= ex ? en : INFINITY;
}

uint32_t replay(const float *nodes, const float *tris, int32_t root, const ckr_ray &ray, uint64_t &boxes,
                uint64_t &ntris, float &tbest) {
  Pre r = make_pre(ray);
  tbest = ray.tmax;
  uint32_t best = 0xFFFFFFFFu;
  std::vector<int32_t> stack;
  int32_t node = root;
  while (node != kDone) {
    if (node >= 0) {
      const float *n = nodes + 16 * (size_t)node;
      boxes += 2;
      float t0 = child_entry(r, n[0], n[1], n[2], n[3], n[8], n[9], tbest);
      float t1 = child_entry(r, n[4], n[5], n[6], n[7], n[10], n[11], tbest);
      int32_t l0, l1;
      std::memcpy(&l0, &n[12], 4);
      std::memcpy(&l1, &n[13], 4);
      bool h0 = t0 != INFINITY, h1 = t1 != INFINITY;
      if (h0 && h1) {
        int32_t near = l0, far = l1;
        if (t1 < t0) std::swap(near, far);
        stack.push_back(far);
        node = near;
      } else if (h0 || h1) {
        node = h0 ? l0 : l1;
      } else if (!stack.empty()) {
        node = stack.back();
        stack.pop_back();
      } else {
        node = kDone;
      }
      continue;
    }
    uint32_t code = ~(uint32_t)node;
    uint32_t first = code >> 3, count = (code & 7u) + 1u;
    for (uint32_t k = 0; k < count; ++k) {
      ntris++;
      float t;
      const float *tp = tris + 12 * (size_t)(first + k);
      if (hit_tri(r, tp, tbest, t)) {
        tbest = t;
        std::memcpy(&best, &tp[3], 4);
      }
    }
    if (!stack.empty()) {
      node = stack.back();
      stack.pop_back();
    } else {
      node = kDone;
    }
  }
  return best;
}

}  // namespace

extern "C" int ckr_trace_stats(const ckr_scene *scene, const ckr_ray *rays, uint32_t n, double *mean_boxes,
                               double *mean_tris) {
  if (!scene || (n && !rays) || !mean_boxes || !mean_tris) return CKR_ERR_INVALID_ARGUMENT;
  const float *nodes, *tris, *spheres;
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
  *mean_boxes = n ? (double)B / n : 0.0;
  *mean_tris = n ? (double)T / n : 0.0;
  return CKR_OK;
}

// Host-only replay of the whole closest-hit path (SAH build + FP32 traversal)
// without a device, for the CPU test suite: it lets the builder and the
// traversal logic be checked against the oracle before any kernel runs.  Not
// part of the public ABI and not used by any product entry point.
extern "C" int ckr_internal_replay_closest(const float *tri9, uint32_t ntri, uint32_t max_leaf,
                                           const ckr_ray *rays, uint32_t n, uint32_t *hit_id, float *hit_t,
                                           double *mean_boxes, double *mean_tris) {
  ckr::FlatBvh bvh;
  ckr_build_params p{max_leaf, 0, 0};
  int st = ckr::build_bvh(tri9, ntri, p, bvh);
  if (st != CKR_OK) return st;
  uint64_t B = 0, T = 0;
  for (uint32_t i = 0; i < n; ++i) {
    float t;
    hit_id[i] = replay(bvh.nodes.data(), bvh.tris.data(), bvh.root, rays[i], B, T, t);
    hit_t[i] = t;
  }
  if (mean_boxes) *mean_boxes = n ? (double)B / n : 0.0;
  if (mean_tris) *mean_tris = n ? (double)T / n : 0.0;
  return CKR_OK;
}
