/*
 * orc_workload.c — the synthetic traversal workload (displaced icosphere,
 * pinhole rays, incoherent rays) restated in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference renders hand-written XML scenes
 * and has no generator for this workload; the library generates it with
 * ckr_workload_icosphere / ckr_workload_rays_pinhole /
 * ckr_workload_rays_incoherent (chakumrender_gb300/csrc/workloads.cpp).
 * This file produces the same bytes without loading the library, so the CPU
 * timing of the reference traversal (bench.py --impl reference) runs on
 * inputs made by the oracle alone.  tests/test_workloads.py checks that the
 * two generators agree byte for byte.
 *
 * Arithmetic: FP64 +, -, *, /, sqrt, floor (and tan for the camera), in the
 * same order as the library, compiled with -ffp-contract=off.
 */
#include "ckr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double x, y, z;
} W3;

static W3 w3(double x, double y, double z) {
  W3 r = {x, y, z};
  return r;
}
static W3 w_add(W3 a, W3 b) { return w3(a.x + b.x, a.y + b.y, a.z + b.z); }
static W3 w_sub(W3 a, W3 b) { return w3(a.x - b.x, a.y - b.y, a.z - b.z); }
static W3 w_scale(W3 a, double s) { return w3(a.x * s, a.y * s, a.z * s); }
static double w_dot(W3 a, W3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static W3 w_cross(W3 a, W3 b) {
  return w3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static W3 w_unit(W3 a) { return w_scale(a, 1.0 / sqrt(w_dot(a, a))); }

/* splitmix64 finaliser and the library's stream keys (csrc/ckr_rng.h). */
static uint64_t w_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static uint64_t w_key(uint64_t seed, uint64_t index) {
  return w_mix(seed * 0x9E3779B97F4A7C15ull + w_mix(index + 0x632BE59BD9B4E019ull));
}
static double w_uniform(uint64_t key, uint32_t counter) {
  uint32_t u = (uint32_t)(w_mix(key + (uint64_t)(counter + 1u) * 0xD1B54A32D192ED03ull) >> 32);
  return (double)(float)((float)(u >> 8) * (1.0f / 16777216.0f));
}

/* Value noise: hashed lattice values in [-1, 1), quintic fade, trilinear. */
static double w_lattice(uint64_t seed, int64_t ix, int64_t iy, int64_t iz) {
  uint64_t h = w_mix(seed ^ ((uint64_t)ix * 0x8CB92BA72F3D8DD7ull));
  h = w_mix(h ^ ((uint64_t)iy * 0xD6E8FEB86659FD93ull));
  h = w_mix(h ^ ((uint64_t)iz * 0xA0761D6478BD642Full));
  return (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}
static double w_fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
static double w_lerp(double a, double b, double t) { return a + (b - a) * t; }

static double w_noise(uint64_t seed, double x, double y, double z) {
  double fx = floor(x), fy = floor(y), fz = floor(z);
  int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
  double u = w_fade(x - fx), v = w_fade(y - fy), w = w_fade(z - fz);
  /* corners c[dx][dy][dz]; interpolate along x, then y, then z */
  double c000 = w_lattice(seed, ix, iy, iz), c100 = w_lattice(seed, ix + 1, iy, iz);
  double c010 = w_lattice(seed, ix, iy + 1, iz), c110 = w_lattice(seed, ix + 1, iy + 1, iz);
  double c001 = w_lattice(seed, ix, iy, iz + 1), c101 = w_lattice(seed, ix + 1, iy, iz + 1);
  double c011 = w_lattice(seed, ix, iy + 1, iz + 1), c111 = w_lattice(seed, ix + 1, iy + 1, iz + 1);
  double y0 = w_lerp(w_lerp(c000, c100, u), w_lerp(c010, c110, u), v);
  double y1 = w_lerp(w_lerp(c001, c101, u), w_lerp(c011, c111, u), v);
  return w_lerp(y0, y1, w);
}

/* Fractal sum: octave o at frequency 2^(o+1), amplitude 2^-o, own seed. */
static double w_fbm(uint64_t seed, W3 p, uint32_t octaves) {
  double sum = 0.0, norm = 0.0, amp = 1.0, freq = 2.0;
  for (uint32_t o = 0; o < octaves; ++o) {
    uint64_t s = w_mix(seed + 0x9E3779B97F4A7C15ull * (o + 1));
    sum += amp * w_noise(s, p.x * freq, p.y * freq, p.z * freq);
    norm += amp;
    amp *= 0.5;
    freq *= 2.0;
  }
  return norm > 0.0 ? sum / norm : 0.0;
}

/* Edge -> midpoint vertex index, open addressing over (min, max) pairs. */
typedef struct {
  uint64_t *key;
  uint32_t *val;
  size_t mask;
} w_edges;

static int w_edges_init(w_edges *e, size_t nedges) {
  size_t cap = 16;
  while (cap < 2 * nedges) cap <<= 1;
  e->key = (uint64_t *)malloc(cap * sizeof(uint64_t));
  e->val = (uint32_t *)malloc(cap * sizeof(uint32_t));
  e->mask = cap - 1;
  if (!e->key || !e->val) return -1;
  memset(e->key, 0xFF, cap * sizeof(uint64_t));
  return 0;
}

static void w_edges_free(w_edges *e) {
  free(e->key);
  free(e->val);
}

/* The midpoint of edge (a, b) projected to the unit sphere; created once per
 * edge, so both faces that share the edge use one vertex. */
static uint32_t w_midpoint(w_edges *e, W3 *v, uint32_t *nv, uint32_t a, uint32_t b) {
  uint64_t k = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
  size_t h = (size_t)w_mix(k) & e->mask;
  while (e->key[h] != ~0ull) {
    if (e->key[h] == k) return e->val[h];
    h = (h + 1) & e->mask;
  }
  v[*nv] = w_unit(w_scale(w_add(v[a], v[b]), 0.5));
  e->key[h] = k;
  e->val[h] = *nv;
  return (*nv)++;
}

int orc_workload_icosphere(uint32_t subdiv, float noise_amp, uint32_t octaves, uint64_t seed,
                           float *tri9_out, uint32_t capacity, uint32_t *ntri_out) {
  if (subdiv > 10 || !ntri_out) return -1;
  uint64_t ntri = 20ull << (2 * subdiv);
  *ntri_out = (uint32_t)ntri;
  if (!tri9_out) return 0;
  if (capacity < ntri) return -2;

  /* Icosahedron: the 12 vertices (+-1, +-phi, 0) and cyclic permutations,
   * normalised, and its 20 faces (counter-clockwise seen from outside). */
  const double phi = (1.0 + sqrt(5.0)) * 0.5;
  static const signed char base[12][3] = {{-1, 2, 0}, {1, 2, 0},  {-1, -2, 0}, {1, -2, 0},
                                          {0, -1, 2}, {0, 1, 2},  {0, -1, -2}, {0, 1, -2},
                                          {2, 0, -1}, {2, 0, 1},  {-2, 0, -1}, {-2, 0, 1}};
  static const uint8_t faces[60] = {0, 11, 5, 0, 5,  1, 0, 1, 7, 0, 7,  10, 0, 10, 11, 1, 5, 9, 5, 11,
                                    4, 11, 10, 2, 10, 7, 6, 7, 1, 8,  3, 9,  4,  3, 4, 2, 3, 2, 6, 3,
                                    6, 8, 3, 8,  9, 4, 9, 5, 2, 4,  11, 6, 2,  10, 8, 6, 7, 9, 8, 1};
  size_t nv_max = 10 * ((size_t)1 << (2 * subdiv)) + 2; /* V = 10 * 4^s + 2 */
  W3 *v = (W3 *)malloc(nv_max * sizeof(W3));
  uint32_t *f = (uint32_t *)malloc(ntri * 3 * sizeof(uint32_t));
  uint32_t *g = (uint32_t *)malloc(ntri * 3 * sizeof(uint32_t));
  if (!v || !f || !g) {
    free(v), free(f), free(g);
    return -3;
  }
  for (int i = 0; i < 12; ++i) {
    double c[3];
    for (int k = 0; k < 3; ++k) c[k] = base[i][k] == 2 ? phi : base[i][k] == -2 ? -phi : (double)base[i][k];
    v[i] = w_unit(w3(c[0], c[1], c[2]));
  }
  for (int i = 0; i < 60; ++i) f[i] = faces[i];
  uint32_t nv = 12;
  size_t nf = 20;
  for (uint32_t level = 0; level < subdiv; ++level) {
    w_edges e;
    if (w_edges_init(&e, nf * 3 / 2) != 0) {
      w_edges_free(&e);
      free(v), free(f), free(g);
      return -3;
    }
    /* each face (a, b, c) becomes (a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca) */
    for (size_t i = 0; i < nf; ++i) {
      uint32_t a = f[3 * i], b = f[3 * i + 1], c = f[3 * i + 2];
      uint32_t ab = w_midpoint(&e, v, &nv, a, b);
      uint32_t bc = w_midpoint(&e, v, &nv, b, c);
      uint32_t ca = w_midpoint(&e, v, &nv, c, a);
      uint32_t q[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      memcpy(g + 12 * i, q, sizeof(q));
    }
    w_edges_free(&e);
    uint32_t *t = f;
    f = g;
    g = t;
    nf *= 4;
  }
  /* radial displacement by the fractal noise at each unit-sphere vertex */
  float *pos = (float *)malloc((size_t)nv * 3 * sizeof(float));
  if (!pos) {
    free(v), free(f), free(g);
    return -3;
  }
  for (uint32_t i = 0; i < nv; ++i) {
    double r = 1.0 + (double)noise_amp * w_fbm(seed, v[i], octaves);
    pos[3 * i + 0] = (float)(v[i].x * r);
    pos[3 * i + 1] = (float)(v[i].y * r);
    pos[3 * i + 2] = (float)(v[i].z * r);
  }
  for (size_t t = 0; t < ntri; ++t)
    for (int k = 0; k < 3; ++k) memcpy(tri9_out + 9 * t + 3 * k, pos + 3 * (size_t)f[3 * t + k], 3 * sizeof(float));
  free(pos), free(v), free(f), free(g);
  return 0;
}

int orc_workload_rays_pinhole(const float eye[3], const float target[3], const float up[3], float vfov_deg,
                              uint32_t width, uint32_t height, float tmax, float *rays8) {
  if (!eye || !target || !up || !rays8 || width == 0 || height == 0 || !(vfov_deg > 0.f && vfov_deg < 180.f))
    return -1;
  W3 e = w3(eye[0], eye[1], eye[2]);
  W3 fwd = w_unit(w_sub(w3(target[0], target[1], target[2]), e));
  W3 right = w_cross(fwd, w3(up[0], up[1], up[2]));
  if (w_dot(right, right) < 1e-30) return -1;
  right = w_unit(right);
  W3 upv = w_cross(right, fwd);
  double th = tan((double)vfov_deg * (3.14159265358979323846 / 360.0));
  double tw = th * (double)width / (double)height;
  for (uint32_t y = 0; y < height; ++y) {
    double sy = (1.0 - 2.0 * ((double)y + 0.5) / (double)height) * th;
    for (uint32_t x = 0; x < width; ++x) {
      double sx = (2.0 * ((double)x + 0.5) / (double)width - 1.0) * tw;
      W3 d = w_unit(w_add(w_add(fwd, w_scale(right, sx)), w_scale(upv, sy)));
      float *r = rays8 + 8 * ((size_t)y * width + x);
      r[0] = eye[0], r[1] = eye[1], r[2] = eye[2], r[3] = 0.f;
      r[4] = (float)d.x, r[5] = (float)d.y, r[6] = (float)d.z, r[7] = tmax;
    }
  }
  return 0;
}

int orc_workload_rays_incoherent(const float lo[3], const float hi[3], uint64_t seed, uint32_t n, float tmax_lo,
                                 float tmax_hi, float *rays8) {
  if (!lo || !hi || (!rays8 && n)) return -1;
  for (uint32_t i = 0; i < n; ++i) {
    uint64_t key = w_key(seed, i);
    float *r = rays8 + 8 * (size_t)i;
    for (int k = 0; k < 3; ++k) r[k] = (float)((double)lo[k] + ((double)hi[k] - lo[k]) * w_uniform(key, (uint32_t)k));
    r[3] = 0.f;
    /* a uniform point of the unit disc by rejection, mapped to the sphere
     * (Marsaglia 1972) */
    double x1, x2, s;
    uint32_t c = 3;
    do {
      x1 = 2.0 * w_uniform(key, c) - 1.0;
      x2 = 2.0 * w_uniform(key, c + 1) - 1.0;
      s = x1 * x1 + x2 * x2;
      c += 2;
    } while (s >= 1.0 || s == 0.0);
    double q = 2.0 * sqrt(1.0 - s);
    W3 d = w_unit(w3(x1 * q, x2 * q, 1.0 - 2.0 * s));
    r[4] = (float)d.x, r[5] = (float)d.y, r[6] = (float)d.z;
    r[7] = (float)((double)tmax_lo + ((double)tmax_hi - tmax_lo) * w_uniform(key, 1000));
  }
  return 0;
}
