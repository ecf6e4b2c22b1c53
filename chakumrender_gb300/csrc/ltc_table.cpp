// ltc_table.cpp — reads the LTC fit table and converts it to FP32 device entries.
//
// The file holds the reference's tabM / tabMinv rows as written in its
// headers/ltc.inc (m0..m8) and the float amplitudes.  The reference turns each
// row into a mat3 through the 9-argument constructor, which stores the
// transpose (headers/mathPrimitives.h:151-165), and caches its determinant;
// the entries here keep that layout's non-zero slots a0, a2, a4, a6, a8.
#include "ltc_table.h"

#include <dlfcn.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "ckr_internal.h"
#include "ckr_test.h"

namespace ckr {

namespace {

std::string default_path() {
  Dl_info info;
  if (dladdr((void *)&default_path, &info) && info.dli_fname) {
    std::string so = info.dli_fname;
    size_t slash = so.find_last_of('/');
    std::string dir = slash == std::string::npos ? "." : so.substr(0, slash);
    return dir + "/data/ltc_ggx.bin";
  }
  return "data/ltc_ggx.bin";
}

// Transposed storage of the 9-argument mat3 constructor.
void to_mat3(const double *m, double *a) {
  a[0] = m[0]; a[3] = m[1]; a[6] = m[2];
  a[1] = m[3]; a[4] = m[4]; a[7] = m[5];
  a[2] = m[6]; a[5] = m[7]; a[8] = m[8];
}

double det3(const double *a) {
  return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) + a[2] * (a[3] * a[7] - a[4] * a[6]);
}

std::mutex g_mu;
std::vector<LtcEntry> g_host;
const LtcEntry *g_dev[64] = {nullptr};

}  // namespace

int load_ltc_table(const char *path, std::vector<LtcEntry> &out) {
  std::string p = path ? std::string(path) : default_path();
  FILE *f = std::fopen(p.c_str(), "rb");
  if (!f) return CKR_ERR_IO;
  char magic[8];
  int hdr[2];
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "CKRLTC1", 7) == 0 && std::fread(hdr, 4, 2, f) == 2 &&
            hdr[0] == 64;
  if (!ok) {
    std::fclose(f);
    return CKR_ERR_PARSE;
  }
  const int n = 64 * 64;
  std::vector<double> tm(9 * n), ti(9 * n);
  std::vector<float> ta(n);
  ok = std::fread(tm.data(), 8, tm.size(), f) == tm.size() && std::fread(ti.data(), 8, ti.size(), f) == ti.size() &&
       std::fread(ta.data(), 4, ta.size(), f) == ta.size();
  std::fclose(f);
  if (!ok) return CKR_ERR_PARSE;
  out.resize(n);
  for (int i = 0; i < n; ++i) {
    double M[9], Mi[9];
    to_mat3(&tm[9 * i], M);
    to_mat3(&ti[9 * i], Mi);
    LtcEntry &e = out[i];
    e.mi0 = (float)Mi[0]; e.mi2 = (float)Mi[2]; e.mi4 = (float)Mi[4]; e.mi6 = (float)Mi[6]; e.mi8 = (float)Mi[8];
    e.amp = ta[i];
    e.m0 = (float)M[0]; e.m2 = (float)M[2]; e.m4 = (float)M[4]; e.m6 = (float)M[6]; e.m8 = (float)M[8];
    e.det = (float)det3(M);
  }
  return CKR_OK;
}

const LtcEntry *device_ltc_table(int *status) {
  std::lock_guard<std::mutex> lock(g_mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    *status = CKR_ERR_CUDA;
    return nullptr;
  }
  if (g_dev[dev]) {
    *status = CKR_OK;
    return g_dev[dev];
  }
  if (g_host.empty()) {
    int st = load_ltc_table(nullptr, g_host);
    if (st != CKR_OK) {
      g_host.clear();
      *status = st;
      return nullptr;
    }
  }
  LtcEntry *d = nullptr;
  if (cudaMalloc((void **)&d, g_host.size() * sizeof(LtcEntry)) != cudaSuccess ||
      cudaMemcpy(d, g_host.data(), g_host.size() * sizeof(LtcEntry), cudaMemcpyHostToDevice) != cudaSuccess) {
    if (d) cudaFree(d);
    *status = CKR_ERR_CUDA;
    return nullptr;
  }
  g_dev[dev] = d;
  *status = CKR_OK;
  return d;
}

}  // namespace ckr

extern "C" int ckr_ltc_init(const char *table_path) {
  std::lock_guard<std::mutex> lock(ckr::g_mu);
  std::vector<ckr::LtcEntry> t;
  int st = ckr::load_ltc_table(table_path, t);
  if (st == CKR_OK) ckr::g_host.swap(t);
  return st;
}

// Host-only replay of the renderer's FP32 BRDF and pdf (brdf_eval / pdf_eval of
// shading_device.cuh), for the CPU test suite: vectors are 3 floats per row.
// Not part of the public ABI and not used by any product entry point.
extern "C" int ckr_internal_brdf_host(const ckr_material *mats, uint32_t count, const float *n, const float *wo_ref,
                                      const float *wo, const float *wi, float *brdf, float *pdf) {
  for (uint32_t i = 0; i < count; ++i) {
    ckr::Material m;
    m.brdf = mats[i].brdf;
    m.alpha = mats[i].alpha;
    m.phong_exp = mats[i].phong_exp;
    m.spec = mats[i].spec;
    m.int_ior = mats[i].int_ior;
    m.ext_ior = mats[i].ext_ior;
    auto v = [&](const float *p) { return ckr::f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); };
    brdf[i] = ckr::brdf_eval(m, v(n), v(wo_ref), v(wo), v(wi));
    pdf[i] = ckr::pdf_eval(m, v(n), v(wo_ref), v(wo), v(wi));
  }
  return CKR_OK;
}

// Host-only replay of the renderer's FP32 LTC-approximate BRDF (the
// `brdfApprox.isSet` branch of MaterialType::brdf after getBrdfApproxParam with
// force, as the MISCV residual uses it); GGX materials only.  For tests.
extern "C" int ckr_internal_brdf_ltc_host(const ckr_material *mats, uint32_t count, const float *n, const float *wo,
                                          const float *wi, float *brdf) {
  std::vector<ckr::LtcEntry> tab;
  {
    std::lock_guard<std::mutex> lock(ckr::g_mu);
    if (ckr::g_host.empty()) {
      int st = ckr::load_ltc_table(nullptr, ckr::g_host);
      if (st != CKR_OK) return st;
    }
    tab = ckr::g_host;
  }
  auto table = [&](int i) { return tab[i]; };
  for (uint32_t i = 0; i < count; ++i) {
    ckr::Material m;
    m.brdf = mats[i].brdf;
    m.alpha = mats[i].alpha;
    m.phong_exp = mats[i].phong_exp;
    m.spec = mats[i].spec;
    m.int_ior = mats[i].int_ior;
    m.ext_ior = mats[i].ext_ior;
    auto v = [&](const float *p) { return ckr::f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); };
    ckr::F3 N = v(n), O = v(wo), I = v(wi);
    float theta = acosf(fminf(1.0f, fmaxf(-1.0f, ckr::dot(N, O))));
    ckr::LtcLookup L = ckr::ltc_lookup(table, theta, m.alpha);
    ckr::M3f minv = ckr::ltc_minv_world(L, N, O);
    brdf[i] = ckr::brdf_ltc(m, L, minv, N, I);
  }
  return CKR_OK;
}

// Host-only replay of ckr_ltc_shade's per-pixel FP32 code (the same functions
// from shading_device.cuh compiled for the host), for the CPU test suite.  Not
// part of the public ABI and not used by any product entry point.
extern "C" int ckr_internal_ltc_shade_host(const float *gbuf, uint32_t npx, const float *light_tri9,
                                           const float *light_rgb, uint32_t nlight, float *rgb) {
  std::vector<ckr::LtcEntry> tab;
  {
    std::lock_guard<std::mutex> lock(ckr::g_mu);
    if (ckr::g_host.empty()) {
      int st = ckr::load_ltc_table(nullptr, ckr::g_host);
      if (st != CKR_OK) return st;
    }
    tab = ckr::g_host;
  }
  auto table = [&](int i) { return tab[i]; };
  auto light = [&](uint32_t k, ckr::F3 &A, ckr::F3 &B, ckr::F3 &C, float *c) {
    const float *t = light_tri9 + 9 * (size_t)k;
    A = ckr::f3(t[0], t[1], t[2]);
    B = ckr::f3(t[3], t[4], t[5]);
    C = ckr::f3(t[6], t[7], t[8]);
    for (int j = 0; j < 3; ++j) c[j] = light_rgb[3 * k + j];
  };
  for (uint32_t p = 0; p < npx; ++p) {
    const float *g = gbuf + 12 * (size_t)p;
    ckr::ltc_shade_point(table, ckr::f3(g[0], g[1], g[2]), ckr::f3(g[4], g[5], g[6]), ckr::f3(g[8], g[9], g[10]),
                         g[3], g[11], nlight, light, rgb + 3 * (size_t)p);
  }
  return CKR_OK;
}

extern "C" int ckr_internal_theta_over_sin_host(const float *c, uint32_t n, float *out) {
  if (n && (!c || !out)) return CKR_ERR_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < n; ++i) out[i] = ckr::theta_over_sin(c[i]);
  return CKR_OK;
}
