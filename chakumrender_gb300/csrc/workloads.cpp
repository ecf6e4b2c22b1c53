// workloads.cpp — deterministic synthetic inputs (icosphere mesh, ray sets).
//
// No reference counterpart: the reference renders hand-written XML scenes.
// These generators stand in for the benchmark scenes.  They use only
// +, -, *, /, sqrt and floor in FP64 (compiled with -ffp-contract=off), so
// x86-64 and aarch64 produce bit-identical outputs.
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/ckr.h"
#include "ckr_rng.h"

namespace {

struct D3 {
  double x, y, z;
};

inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
inline D3 add(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline D3 sub(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline D3 mul(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline D3 normalize(D3 a) { return mul(a, 1.0 / std::sqrt(dot(a, a))); }

// Lattice value in [-1, 1) for integer point (ix, iy, iz).
inline double lattice(uint64_t seed, int64_t ix, int64_t iy, int64_t iz) {
  uint64_t h = ckr_mix64(seed ^ ((uint64_t)ix * 0x8CB92BA72F3D8DD7ull));
  h = ckr_mix64(h ^ ((uint64_t)iy * 0xD6E8FEB86659FD93ull));
  h = ckr_mix64(h ^ ((uint64_t)iz * 0xA0761D6478BD642Full));
  return (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// Quintic fade 6t^5 - 15t^4 + 10t^3.
inline double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }

double value_noise(uint64_t seed, double x, double y, double z) {
  double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
  double u = fade(x - fx), v = fade(y - fy), w = fade(z - fz);
  double c[2][2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(seed, ix + a, iy + b, iz + d);
  double x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * u;
  double x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * u;
  double x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * u;
  double x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * u;
  double y0 = x00 + (x10 - x00) * v;
  double y1 = x01 + (x11 - x01) * v;
  return y0 + (y1 - y0) * w;
}

double fbm(uint64_t seed, D3 p, uint32_t octaves) {
  double sum = 0.0, norm = 0.0, amp = 1.0, freq = 2.0;
  for (uint32_t o = 0; o < octaves; ++o) {
    uint64_t s = ckr_mix64(seed + 0x9E3779B97F4A7C15ull * (o + 1));
    sum += amp * value_noise(s, p.x * freq, p.y * freq, p.z * freq);
    norm += amp;
    amp *= 0.5;
    freq *= 2.0;
  }
  return norm > 0.0 ? sum / norm : 0.0;
}

}  // namespace

extern "C" int ckr_workload_icosphere(uint32_t subdiv, float noise_amp, uint32_t octaves,
                                      uint64_t seed, float *tri9_out, uint32_t capacity,
                                      uint32_t *ntri_out) {
  if (subdiv > 10 || !ntri_out) return CKR_ERR_INVALID_ARGUMENT;
  uint64_t ntri = 20ull << (2 * subdiv);
  *ntri_out = (uint32_t)ntri;
  if (!tri9_out) return CKR_OK;  // size query
  if (capacity < ntri) return CKR_ERR_TOO_LARGE;

  const double phi = (1.0 + std::sqrt(5.0)) * 0.5;
  std::vector<D3> v = {d3(-1, phi, 0), d3(1, phi, 0),  d3(-1, -phi, 0), d3(1, -phi, 0),
                       d3(0, -1, phi), d3(0, 1, phi),  d3(0, -1, -phi), d3(0, 1, -phi),
                       d3(phi, 0, -1), d3(phi, 0, 1),  d3(-phi, 0, -1), d3(-phi, 0, 1)};
  for (auto &p : v) p = normalize(p);
  std::vector<uint32_t> f = {0, 11, 5, 0, 5,  1, 0, 1, 7, 0, 7,  10, 0, 10, 11, 1, 5, 9, 5, 11,
                             4, 11, 10, 2, 10, 7, 6, 7, 1, 8,  3, 9,  4,  3, 4, 2, 3, 2, 6, 3,
                             6, 8, 3, 8,  9, 4, 9, 5, 2, 4,  11, 6, 2,  10, 8, 6, 7, 9, 8, 1};
  for (uint32_t level = 0; level < subdiv; ++level) {
    std::unordered_map<uint64_t, uint32_t> mid;
    mid.reserve(f.size());
    auto midpoint = [&](uint32_t a, uint32_t b) -> uint32_t {
      uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      v.push_back(normalize(mul(add(v[a], v[b]), 0.5)));
      uint32_t id = (uint32_t)v.size() - 1;
      mid.emplace(key, id);
      return id;
    };
    std::vector<uint32_t> g;
    g.reserve(f.size() * 4);
    for (size_t i = 0; i < f.size(); i += 3) {
      uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
      uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      uint32_t quad[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      g.insert(g.end(), quad, quad + 12);
    }
    f.swap(g);
  }
  std::vector<float> pos(v.size() * 3);
  for (size_t i = 0; i < v.size(); ++i) {
    double r = 1.0 + (double)noise_amp * fbm(seed, v[i], octaves);
    pos[3 * i + 0] = (float)(v[i].x * r);
    pos[3 * i + 1] = (float)(v[i].y * r);
    pos[3 * i + 2] = (float)(v[i].z * r);
  }
  for (size_t t = 0; t < ntri; ++t)
    for (int k = 0; k < 3; ++k) std::memcpy(tri9_out + 9 * t + 3 * k, &pos[3 * f[3 * t + k]], 3 * sizeof(float));
  return CKR_OK;
}

extern "C" int ckr_workload_rays_pinhole(const float eye[3], const float target[3], const float up[3],
                                         float vfov_deg, uint32_t width, uint32_t height, float tmax,
                                         ckr_ray *out) {
  if (!eye || !target || !up || !out || width == 0 || height == 0 || !(vfov_deg > 0.f && vfov_deg < 180.f))
    return CKR_ERR_INVALID_ARGUMENT;
  D3 e = d3(eye[0], eye[1], eye[2]);
  D3 fwd = normalize(sub(d3(target[0], target[1], target[2]), e));
  D3 right = cross(fwd, d3(up[0], up[1], up[2]));
  if (dot(right, right) < 1e-30) return CKR_ERR_INVALID_ARGUMENT;
  right = normalize(right);
  D3 upv = cross(right, fwd);
  double th = std::tan((double)vfov_deg * (3.14159265358979323846 / 360.0));
  double tw = th * (double)width / (double)height;
  for (uint32_t y = 0; y < height; ++y) {
    double sy = (1.0 - 2.0 * ((double)y + 0.5) / (double)height) * th;
    for (uint32_t x = 0; x < width; ++x) {
      double sx = (2.0 * ((double)x + 0.5) / (double)width - 1.0) * tw;
      D3 d = normalize(add(add(fwd, mul(right, sx)), mul(upv, sy)));
      ckr_ray &r = out[(size_t)y * width + x];
      r.ox = eye[0];
      r.oy = eye[1];
      r.oz = eye[2];
      r.tmin = 0.f;
      r.dx = (float)d.x;
      r.dy = (float)d.y;
      r.dz = (float)d.z;
      r.tmax = tmax;
    }
  }
  return CKR_OK;
}

extern "C" int ckr_workload_rays_incoherent(const float lo[3], const float hi[3], uint64_t seed,
                                            uint32_t n, float tmax_lo, float tmax_hi, ckr_ray *out) {
  if (!lo || !hi || (!out && n)) return CKR_ERR_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < n; ++i) {
    uint64_t key = ckr_key(seed, i);
    ckr_ray &r = out[i];
    r.ox = (float)((double)lo[0] + ((double)hi[0] - lo[0]) * ckr_draw_f(key, 0));
    r.oy = (float)((double)lo[1] + ((double)hi[1] - lo[1]) * ckr_draw_f(key, 1));
    r.oz = (float)((double)lo[2] + ((double)hi[2] - lo[2]) * ckr_draw_f(key, 2));
    r.tmin = 0.f;
    // Marsaglia (1972): (x1, x2) uniform in the unit disc maps to the sphere.
    double x1, x2, s;
    uint32_t c = 3;
    do {
      x1 = 2.0 * ckr_draw_f(key, c) - 1.0;
      x2 = 2.0 * ckr_draw_f(key, c + 1) - 1.0;
      s = x1 * x1 + x2 * x2;
      c += 2;
    } while (s >= 1.0 || s == 0.0);
    double q = 2.0 * std::sqrt(1.0 - s);
    D3 d = normalize(d3(x1 * q, x2 * q, 1.0 - 2.0 * s));
    r.dx = (float)d.x;
    r.dy = (float)d.y;
    r.dz = (float)d.z;
    r.tmax = (float)((double)tmax_lo + ((double)tmax_hi - tmax_lo) * ckr_draw_f(key, 1000));
  }
  return CKR_OK;
}

extern "C" float ckr_rng_uniform(uint64_t seed, uint64_t index, uint32_t counter) {
  return ckr_draw_f(ckr_key(seed, index), counter);
}

namespace {
// Orthonormal basis about a unit vector (Duff et al. 2017, "Building an
// Orthonormal Basis, Revisited").
void onb(D3 n, D3 &t, D3 &b) {
  double s = n.z >= 0.0 ? 1.0 : -1.0;
  double a = -1.0 / (s + n.z);
  double c = n.x * n.y * a;
  t = d3(1.0 + s * n.x * n.x * a, s * c, -s * n.x);
  b = d3(c, s + n.y * n.y * a, -n.y);
}

// Uniform on the unit sphere from the stream (Marsaglia 1972), from counter c.
D3 sphere_dir(uint64_t key, uint32_t &c) {
  double x1, x2, s;
  do {
    x1 = 2.0 * ckr_draw_f(key, c) - 1.0;
    x2 = 2.0 * ckr_draw_f(key, c + 1) - 1.0;
    s = x1 * x1 + x2 * x2;
    c += 2;
  } while (s >= 1.0 || s == 0.0);
  double q = 2.0 * std::sqrt(1.0 - s);
  return normalize(d3(x1 * q, x2 * q, 1.0 - 2.0 * s));
}
}  // namespace

extern "C" int ckr_workload_gbuffer(uint64_t seed, uint32_t npx, float *out12) {
  if (!out12 && npx) return CKR_ERR_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < npx; ++i) {
    uint64_t key = ckr_key(seed, i);
    float *g = out12 + 12 * (size_t)i;
    for (int k = 0; k < 3; ++k) g[k] = (float)(2.0 * ckr_draw_f(key, k) - 1.0);
    uint32_t c = 16;
    D3 n = sphere_dir(key, c);
    if (n.z < 0) n.z = -n.z;  // uniform on the +z hemisphere
    // View direction: cosine lobe about n (Malley's method on a disc sample).
    double x1, x2, s;
    uint32_t c2 = 200;
    do {
      x1 = 2.0 * ckr_draw_f(key, c2) - 1.0;
      x2 = 2.0 * ckr_draw_f(key, c2 + 1) - 1.0;
      s = x1 * x1 + x2 * x2;
      c2 += 2;
    } while (s >= 1.0);
    D3 t, b;
    onb(n, t, b);
    D3 v = normalize(add(add(mul(t, x1), mul(b, x2)), mul(n, std::sqrt(1.0 - s))));
    g[3] = (float)(0.05 + 0.95 * ckr_draw_f(key, 3));   // GGX alpha in [0.05, 1]
    g[4] = (float)n.x; g[5] = (float)n.y; g[6] = (float)n.z;
    g[7] = (float)(0.02 + 0.88 * ckr_draw_f(key, 4));   // F0 in [0.02, 0.9]
    g[8] = (float)v.x; g[9] = (float)v.y; g[10] = (float)v.z;
    g[11] = ckr_draw_f(key, 5);                          // specular coefficient in [0, 1)
  }
  return CKR_OK;
}

extern "C" int ckr_workload_quad_lights(uint64_t seed, uint32_t nquads, float side_lo, float side_hi, float radiance,
                                        float *tri9_out, float *rgb_out) {
  if ((!tri9_out || !rgb_out) && nquads) return CKR_ERR_INVALID_ARGUMENT;
  for (uint32_t q = 0; q < nquads; ++q) {
    uint64_t key = ckr_key(seed, q);
    double side = side_lo + ((double)side_hi - side_lo) * ckr_draw_f(key, 0);
    double cx = -2.0 + 4.0 * ckr_draw_f(key, 1), cy = -2.0 + 4.0 * ckr_draw_f(key, 2), cz = 1.0 + 2.0 * ckr_draw_f(key, 3);
    double h = 0.5 * side;
    double p[4][3] = {{cx - h, cy - h, cz}, {cx + h, cy - h, cz}, {cx + h, cy + h, cz}, {cx - h, cy + h, cz}};
    const int tri[2][3] = {{0, 2, 1}, {0, 3, 2}};  // facing -z
    for (int k = 0; k < 2; ++k)
      for (int v = 0; v < 3; ++v)
        for (int j = 0; j < 3; ++j) tri9_out[9 * (2 * q + k) + 3 * v + j] = (float)p[tri[k][v]][j];
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 3; ++j) rgb_out[3 * (2 * q + k) + j] = radiance;
  }
  return CKR_OK;
}

// Many-light scene: the displaced icosphere (GGX, per-triangle roughness) in a
// diffuse room whose ceiling and walls carry small emissive triangles, grouped
// by k-means on their centroids into mesh lights (one light per cluster).
extern "C" int ckr_workload_manylight(const ckr_manylight_spec *sp, float *tri9, uint32_t *tri_mat,
                                      ckr_material *mats, ckr_light *lights, ckr_camera *cam, uint32_t *counts) {
  if (!sp || !counts || sp->nemit == 0 || sp->nclusters == 0 || sp->nclusters > sp->nemit || sp->subdiv > 10)
    return CKR_ERR_INVALID_ARGUMENT;
  const uint32_t nmesh = 20u << (2 * sp->subdiv), nroom = 12, ne = sp->nemit;
  const uint64_t ntri = (uint64_t)nmesh + nroom + ne;
  if (ntri > 0xFFFFFFF0ull) return CKR_ERR_TOO_LARGE;
  // Emitters: face, centre, orientation and radiance from the stream (seed, i).
  const double lo = -5.0, hi = 5.0, y0 = sp->floor_y, y1 = sp->floor_y + 10.0, eps = 1e-3;
  std::vector<D3> cen(ne);
  std::vector<double> tri(9 * (size_t)ne), rad(ne);
  for (uint32_t i = 0; i < ne; ++i) {
    uint64_t key = ckr_key(sp->emit_seed, i);
    uint32_t face = (uint32_t)(5.0 * ckr_draw_f(key, 0));
    double u = 0.2 + 9.6 * ckr_draw_f(key, 1), v = 0.2 + 9.6 * ckr_draw_f(key, 2);
    double th = 6.283185307179586 * ckr_draw_f(key, 3);
    rad[i] = sp->radiance_lo * std::exp(std::log((double)sp->radiance_hi / sp->radiance_lo) * ckr_draw_f(key, 4));
    D3 c, t, b;  // centre on the face, two in-plane axes
    switch (face) {
      case 0: c = d3(lo + u, y1 - eps, lo + v); t = d3(1, 0, 0); b = d3(0, 0, 1); break;   // ceiling
      case 1: c = d3(lo + eps, y0 + u, lo + v); t = d3(0, 1, 0); b = d3(0, 0, 1); break;   // x = -5
      case 2: c = d3(hi - eps, y0 + u, lo + v); t = d3(0, 1, 0); b = d3(0, 0, 1); break;   // x = +5
      case 3: c = d3(lo + u, y0 + v, lo + eps); t = d3(1, 0, 0); b = d3(0, 1, 0); break;   // z = -5
      default: c = d3(lo + u, y0 + v, hi - eps); t = d3(1, 0, 0); b = d3(0, 1, 0); break;  // z = +5
    }
    cen[i] = c;
    const double r = sp->emit_side / std::sqrt(3.0);
    for (int j = 0; j < 3; ++j) {
      double a = th + 2.0943951023931957 * j;
      D3 p = add(c, add(mul(t, r * std::cos(a)), mul(b, r * std::sin(a))));
      tri[9 * i + 3 * j] = p.x;
      tri[9 * i + 3 * j + 1] = p.y;
      tri[9 * i + 3 * j + 2] = p.z;
    }
  }
  // k-means (Lloyd), deterministic: centroids start at evenly spaced emitters.
  const uint32_t K = sp->nclusters;
  std::vector<D3> ctr(K);
  for (uint32_t k = 0; k < K; ++k) ctr[k] = cen[(size_t)k * ne / K];
  std::vector<uint32_t> asg(ne, 0);
  for (int it = 0; it < 20; ++it) {
    for (uint32_t i = 0; i < ne; ++i) {
      double best = 1e300;
      for (uint32_t k = 0; k < K; ++k) {
        D3 d = sub(cen[i], ctr[k]);
        double q = dot(d, d);
        if (q < best) best = q, asg[i] = k;
      }
    }
    std::vector<D3> sum(K, d3(0, 0, 0));
    std::vector<uint32_t> cnt(K, 0);
    for (uint32_t i = 0; i < ne; ++i) sum[asg[i]] = add(sum[asg[i]], cen[i]), ++cnt[asg[i]];
    for (uint32_t k = 0; k < K; ++k)
      if (cnt[k]) ctr[k] = mul(sum[k], 1.0 / cnt[k]);
  }
  std::vector<uint32_t> order(ne), start(K + 1, 0);
  for (uint32_t i = 0; i < ne; ++i) ++start[asg[i] + 1];
  for (uint32_t k = 0; k < K; ++k) start[k + 1] += start[k];
  {
    std::vector<uint32_t> fill(start.begin(), start.end() - 1);
    for (uint32_t i = 0; i < ne; ++i) order[fill[asg[i]]++] = i;
  }
  uint32_t nl = 0;
  for (uint32_t k = 0; k < K; ++k) nl += start[k + 1] > start[k];
  counts[0] = (uint32_t)ntri;
  counts[1] = nmesh + 1 + ne;  // materials
  counts[2] = nl;
  if (!tri9) return CKR_OK;  // size query
  if (!tri_mat || !mats || !lights || !cam) return CKR_ERR_INVALID_ARGUMENT;
  uint32_t n = 0;
  int st = ckr_workload_icosphere(sp->subdiv, sp->noise_amp, sp->octaves, sp->mesh_seed, tri9, nmesh, &n);
  if (st != CKR_OK) return st;
  ckr_material m;
  std::memset(&m, 0, sizeof(m));
  for (uint32_t i = 0; i < nmesh; ++i) {
    m.brdf = 2;  // GGX
    m.alpha = (float)(sp->alpha_lo + ((double)sp->alpha_hi - sp->alpha_lo) * ckr_draw_f(ckr_key(sp->rough_seed, i), 0));
    m.spec = sp->mesh_spec;
    m.int_ior = 1e5f;  // F = 1 to within 4e-5
    m.ext_ior = 1.0f;
    m.reflectance = 1.0f;
    m.color[0] = m.color[1] = m.color[2] = sp->mesh_albedo;
    mats[i] = m;
    tri_mat[i] = i;
  }
  // Room: 6 faces x 2 triangles, Lambertian (GGX with specularCoef 0).
  std::memset(&m, 0, sizeof(m));
  m.brdf = 2;
  m.alpha = 0.5f;
  m.int_ior = 1.5f;
  m.ext_ior = 1.0f;
  m.reflectance = 1.0f;
  m.color[0] = m.color[1] = m.color[2] = sp->room_albedo;
  mats[nmesh] = m;
  const double P[8][3] = {{lo, y0, lo}, {hi, y0, lo}, {hi, y0, hi}, {lo, y0, hi},
                          {lo, y1, lo}, {hi, y1, lo}, {hi, y1, hi}, {lo, y1, hi}};
  const int Q[6][4] = {{0, 1, 2, 3}, {4, 7, 6, 5}, {0, 3, 7, 4}, {1, 5, 6, 2}, {0, 4, 5, 1}, {3, 2, 6, 7}};
  for (int f = 0; f < 6; ++f) {
    const int T[2][3] = {{Q[f][0], Q[f][1], Q[f][2]}, {Q[f][0], Q[f][2], Q[f][3]}};
    for (int h = 0; h < 2; ++h) {
      uint32_t id = nmesh + 2 * f + h;
      for (int v = 0; v < 3; ++v)
        for (int j = 0; j < 3; ++j) tri9[9 * (size_t)id + 3 * v + j] = (float)P[T[h][v]][j];
      tri_mat[id] = nmesh;
    }
  }
  // Emitters in cluster order, one material (radiance) each, one mesh light per cluster.
  const uint32_t ebase = nmesh + nroom;
  std::memset(&m, 0, sizeof(m));
  m.light_type = 4;  // MESH
  for (uint32_t s = 0; s < ne; ++s) {
    uint32_t i = order[s];
    for (int j = 0; j < 9; ++j) tri9[9 * (size_t)(ebase + s) + j] = (float)tri[9 * (size_t)i + j];
    m.radiance[0] = m.radiance[1] = m.radiance[2] = (float)rad[i];
    mats[nmesh + 1 + s] = m;
    tri_mat[ebase + s] = nmesh + 1 + s;
  }
  uint32_t l = 0;
  for (uint32_t k = 0; k < K; ++k) {
    if (start[k + 1] == start[k]) continue;
    ckr_light L;
    std::memset(&L, 0, sizeof(L));
    L.type = CKR_LIGHT_MESH;
    L.first = ebase + start[k];
    L.count = start[k + 1] - start[k];
    lights[l++] = L;
  }
  // Camera in the reference's convention (src/prepareScene.cpp:12-36).
  D3 pos = d3(sp->cam_pos[0], sp->cam_pos[1], sp->cam_pos[2]);
  D3 cd = normalize(sub(d3(sp->cam_target[0], sp->cam_target[1], sp->cam_target[2]), pos));
  D3 cx = normalize(cross(cd, d3(0, 1, 0)));
  const double tf = std::tan(sp->fov_deg * 3.141592653589793 / 360.0);
  cx = mul(cx, (double)sp->width / sp->height * tf);
  D3 cy = mul(normalize(cross(cx, cd)), tf);
  std::memset(cam, 0, sizeof(*cam));
  const D3 src[4] = {pos, cd, cx, cy};
  float *dst[4] = {cam->pos, cam->dir, cam->cx, cam->cy};
  for (int k = 0; k < 4; ++k) dst[k][0] = (float)src[k].x, dst[k][1] = (float)src[k].y, dst[k][2] = (float)src[k].z;
  cam->width = sp->width;
  cam->height = sp->height;
  return CKR_OK;
}
