// scene_ex.cpp — ckr_scene_create_ex: geometry + BVH (ckr_scene_create) plus the
// shading data the renderer needs (materials, per-primitive material ids,
// input-order triangles, light sources with their sampling tables).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "scene.h"

namespace ckr {

ShadeView shade_view_of(const ckr_scene *s) {
  ShadeView v;
  v.mats = s->mats.ptr;
  v.tri_mat = s->tri_mat.ptr;
  v.tri9 = s->tri9.ptr;
  v.tri_nm = s->tri_nm.ptr;
  v.sph_mat = s->sph_mat.ptr;
  v.sph = s->spheres.ptr;
  v.lights = s->lights.ptr;
  v.nlights = s->nlights;
  v.first_point = s->first_point;
  v.cdf = s->cdf.ptr;
  v.tri_light = s->tri_light.ptr;
  v.pcdf = s->pcdf.ptr;
  v.sel_cdf = s->sel_cdf.ptr;
  v.first_emit = s->first_emit;
  v.n_emit = s->n_emit;
  v.env = s->env.ptr;
  v.env_marg = s->env_marg.ptr;
  v.env_cond = s->env_cond.ptr;
  v.env_cos = s->env_cos.ptr;
  v.env_w = s->env_w;
  v.env_h = s->env_h;
  v.env_axis = s->env_axis;
  v.env_n = s->env_n;
  v.env_inv_area = s->env_inv_area;
  return v;
}

namespace {

// Triangle::area (headers/geometryPrimitives.h:70-76): 0.5 |(C - A) x (B - A)| in FP64.
double tri_area(const float *t) {
  double bx = (double)t[3] - t[0], by = (double)t[4] - t[1], bz = (double)t[5] - t[2];
  double cx = (double)t[6] - t[0], cy = (double)t[7] - t[1], cz = (double)t[8] - t[2];
  double nx = cy * bz - cz * by, ny = cz * bx - cx * bz, nz = cx * by - cy * bx;
  return 0.5 * std::sqrt(nx * nx + ny * ny + nz * nz);
}

// MeshLight::initMeshLight (src/lightSources.cpp:784-807).
double build_inv_cdf(const float *tri9, uint32_t first, uint32_t count, uint32_t *inv) {
  double area = 0;
  for (uint32_t i = 0; i < count; ++i) area += tri_area(tri9 + 9 * (size_t)(first + i));
  double cdf = 0;
  uint32_t last = 0;
  for (uint32_t i = 0; i < count; ++i) {
    cdf += tri_area(tri9 + 9 * (size_t)(first + i)) / area;
    uint32_t index = (uint32_t)(cdf * kInvCdfBins);
    if (index >= kInvCdfBins) index = kInvCdfBins - 1;
    for (uint32_t j = last; j <= index; ++j) inv[j] = i;
    last = index + 1;
  }
  for (uint32_t i = last; i < kInvCdfBins; ++i) inv[i] = count - 1;
  return area;
}

// Tables of the environment light: per-pixel radiance and luminance, the row
// CDF weighted by luminance x solid angle, each row's column CDF, and the band
// boundaries' cosines.  Built in FP64, stored in FP32 with the last CDF entries 1.
struct EnvTables {
  std::vector<float4> px;
  std::vector<float> marg, cond, cosr;
  double area = 0;
};

int build_env(const ckr_env_light &e, EnvTables &t) {
  const uint32_t w = e.width, h = e.height;
  if (!e.rgb || w == 0 || h == 0 || (uint64_t)w * h > (1ull << 28) || e.axis > 2 || e.n_samples > 256)
    return CKR_ERR_INVALID_ARGUMENT;
  // BaseSource: the colour divided by its largest component (Vec::maxnorm), times
  // the intensity.
  double c[3] = {e.color[0], e.color[1], e.color[2]};
  double mx = c[0];
  if (mx < c[1]) mx = c[1];
  if (mx < c[2]) mx = c[2];
  if (!(mx > 0) || !std::isfinite(mx) || !std::isfinite((double)e.intensity)) return CKR_ERR_INVALID_ARGUMENT;
  for (int k = 0; k < 3; ++k) c[k] = c[k] / mx * e.intensity;
  t.px.resize((size_t)w * h);
  t.cosr.resize(h + 1);
  for (uint32_t r = 0; r <= h; ++r) t.cosr[r] = (float)std::cos(M_PI * r / h);
  t.cosr[0] = 1.0f;
  t.cosr[h] = -1.0f;
  std::vector<double> rowsum(h, 0.0), lum((size_t)w * h);
  for (uint32_t r = 0; r < h; ++r)
    for (uint32_t col = 0; col < w; ++col) {
      const size_t i = (size_t)r * w + col;
      double L[3];
      for (int k = 0; k < 3; ++k) {
        L[k] = (double)e.rgb[3 * i + k] * c[k];
        if (!std::isfinite(L[k])) return CKR_ERR_INVALID_ARGUMENT;
      }
      double g = L[0] * 0.3 + L[1] * 0.59 + L[2] * 0.11;  // to_greyScale
      lum[i] = g > 0 ? g : 0.0;
      t.px[i] = make_float4((float)L[0], (float)L[1], (float)L[2], (float)lum[i]);
      rowsum[r] += lum[i];
    }
  const double dphi = 2.0 * M_PI / w;
  std::vector<double> band(h);
  for (uint32_t r = 0; r < h; ++r) {
    band[r] = (std::cos(M_PI * r / h) - std::cos(M_PI * (r + 1) / h)) * dphi;  // solid angle of one pixel
    t.area += rowsum[r] * band[r];
  }
  if (!(t.area > 0)) return CKR_ERR_INVALID_ARGUMENT;  // a black environment cannot be sampled
  t.marg.resize(h + 1);
  t.cond.resize((size_t)h * (w + 1));
  double run = 0;
  t.marg[0] = 0.f;
  for (uint32_t r = 0; r < h; ++r) {
    run += rowsum[r] * band[r];
    t.marg[r + 1] = (float)(run / t.area);
    float *cr = &t.cond[(size_t)r * (w + 1)];
    double cr_run = 0;
    cr[0] = 0.f;
    for (uint32_t col = 0; col < w; ++col) {
      cr_run += lum[(size_t)r * w + col];
      cr[col + 1] = rowsum[r] > 0 ? (float)(cr_run / rowsum[r]) : (float)(col + 1) / (float)w;
    }
    cr[w] = 1.0f;
  }
  t.marg[h] = 1.0f;
  return CKR_OK;
}

template <typename T>
int upload(DevBuf<T> &buf, const T *src, size_t n) {
  if (buf.reserve(n ? n : 1) != cudaSuccess) return CKR_ERR_OUT_OF_MEMORY;
  if (n && cudaMemcpy(buf.ptr, src, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return CKR_ERR_CUDA;
  return CKR_OK;
}

}  // namespace
}  // namespace ckr

using namespace ckr;

extern "C" int ckr_scene_create_ex(const ckr_scene_desc *d, ckr_scene **out) {
  if (!d || !out || (d->ntri && !d->tri9) || (d->nsph && !d->sph4) || (d->nlights && !d->lights) ||
      (d->nmaterials && !d->materials))
    return CKR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  uint32_t nm = d->nmaterials;
  for (uint32_t i = 0; i < d->ntri; ++i)
    if ((d->tri_material ? d->tri_material[i] : 0) >= std::max<uint32_t>(nm, 1) || (!nm)) return CKR_ERR_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < d->nsph; ++i)
    if ((d->sph_material ? d->sph_material[i] : 0) >= std::max<uint32_t>(nm, 1) || (!nm)) return CKR_ERR_INVALID_ARGUMENT;
  // Light tables.
  std::vector<DevLight> lights(d->nlights);
  std::vector<uint32_t> cdf;
  for (uint32_t k = 0; k < d->nlights; ++k) {
    const ckr_light &L = d->lights[k];
    DevLight &g = lights[k];
    std::memset(&g, 0, sizeof(g));
    g.type = L.type;
    g.first = L.first;
    g.count = L.count;
    g.px = L.pos[0]; g.py = L.pos[1]; g.pz = L.pos[2];
    g.pr = L.power[0]; g.pg = L.power[1]; g.pb = L.power[2];
    if (L.type == CKR_LIGHT_MESH) {
      if (L.count == 0 || (uint64_t)L.first + L.count > d->ntri) return CKR_ERR_INVALID_ARGUMENT;
      g.cdf = (uint32_t)cdf.size();
      cdf.resize(cdf.size() + kInvCdfBins);
      g.area = (float)build_inv_cdf(d->tri9, L.first, L.count, &cdf[g.cdf]);
    } else if (L.type == CKR_LIGHT_TRI) {
      if (L.first >= d->ntri) return CKR_ERR_INVALID_ARGUMENT;
      g.count = 1;
      g.area = (float)tri_area(d->tri9 + 9 * (size_t)L.first);
    } else if (L.type == CKR_LIGHT_SPHERE) {
      if (L.first >= d->nsph) return CKR_ERR_INVALID_ARGUMENT;
      const float *s = d->sph4 + 4 * (size_t)L.first;
      g.px = s[0]; g.py = s[1]; g.pz = s[2];
      g.radius = s[3];
    } else if (L.type != CKR_LIGHT_POINT) {
      return CKR_ERR_INVALID_ARGUMENT;
    }
  }
  // The reference's MIS::getSamples visits sphere, mesh and triangle sources in
  // that order (src/mis.cpp:100-146); point lights are handled separately.
  auto rank = [](int32_t t) { return t == CKR_LIGHT_SPHERE ? 0 : t == CKR_LIGHT_MESH ? 1 : t == CKR_LIGHT_TRI ? 2 : 3; };
  std::stable_sort(lights.begin(), lights.end(),
                   [&](const DevLight &a, const DevLight &b) { return rank(a.type) < rank(b.type); });
  uint32_t first_point = 0;
  while (first_point < lights.size() && lights[first_point].type != CKR_LIGHT_POINT) ++first_point;
  // One-sample NEE tables: each emitter triangle's light, per light the CDF of
  // its triangles' power (luminance x area), and the power CDF over the
  // MESH/TRI lights, which sit contiguously after the sphere lights.
  uint32_t first_emit = 0;
  while (first_emit < first_point && lights[first_emit].type == CKR_LIGHT_SPHERE) ++first_emit;
  const uint32_t n_emit = first_point - first_emit;
  std::vector<uint32_t> tri_light(d->ntri, kNoLight);
  std::vector<float> pcdf, sel_cdf(n_emit);
  double total = 0;
  for (uint32_t k = first_emit; k < first_point; ++k) {
    DevLight &g = lights[k];
    g.pcdf = (uint32_t)pcdf.size();
    std::vector<double> pw(g.count);
    double sum = 0;
    for (uint32_t i = 0; i < g.count; ++i) {
      uint32_t tri = g.first + i;
      uint32_t mi = d->tri_material ? d->tri_material[tri] : 0;
      const float *r = d->materials[mi].radiance;
      pw[i] = ((double)r[0] + r[1] + r[2]) / 3.0 * tri_area(d->tri9 + 9 * (size_t)tri);
      sum += pw[i];
      if (tri_light[tri] == kNoLight) tri_light[tri] = k;
    }
    double run = 0;
    for (uint32_t i = 0; i < g.count; ++i) {
      run += pw[i];
      pcdf.push_back(sum > 0 ? (float)(run / sum) : (float)(i + 1) / (float)g.count);
    }
    if (g.count) pcdf.back() = 1.0f;
    g.power = (float)sum;
    total += sum;
  }
  double run = 0;
  for (uint32_t k = first_emit; k < first_point; ++k) {
    lights[k].sel = total > 0 ? (float)(lights[k].power / total) : 1.0f / (float)n_emit;
    run += lights[k].power;
    sel_cdf[k - first_emit] = total > 0 ? (float)(run / total) : (float)(k - first_emit + 1) / (float)n_emit;
  }
  if (n_emit) sel_cdf.back() = 1.0f;
  EnvTables env;
  if (d->env) {
    const int es = build_env(*d->env, env);
    if (es != CKR_OK) return es;
  }
  ckr_scene *s = nullptr;
  int st = ckr_scene_create(d->tri9, d->ntri, d->sph4, d->nsph, &d->build, &s);
  if (st != CKR_OK) return st;
  std::vector<uint32_t> tm(d->ntri, 0), sm(d->nsph, 0);
  if (d->tri_material) std::memcpy(tm.data(), d->tri_material, 4 * (size_t)d->ntri);
  if (d->sph_material) std::memcpy(sm.data(), d->sph_material, 4 * (size_t)d->nsph);
  if ((st = upload(s->mats, d->materials, nm)) != CKR_OK || (st = upload(s->tri_mat, tm.data(), tm.size())) != CKR_OK ||
      (st = upload(s->sph_mat, sm.data(), sm.size())) != CKR_OK ||
      (st = upload(s->tri9, d->tri9, 9 * (size_t)d->ntri)) != CKR_OK ||
      (st = upload(s->lights, lights.data(), lights.size())) != CKR_OK ||
      (st = upload(s->cdf, cdf.data(), cdf.size())) != CKR_OK ||
      (st = upload(s->tri_light, tri_light.data(), tri_light.size())) != CKR_OK ||
      (st = upload(s->pcdf, pcdf.data(), pcdf.size())) != CKR_OK ||
      (st = upload(s->sel_cdf, sel_cdf.data(), sel_cdf.size())) != CKR_OK ||
      (st = upload(s->env, env.px.data(), env.px.size())) != CKR_OK ||
      (st = upload(s->env_marg, env.marg.data(), env.marg.size())) != CKR_OK ||
      (st = upload(s->env_cond, env.cond.data(), env.cond.size())) != CKR_OK ||
      (st = upload(s->env_cos, env.cosr.data(), env.cosr.size())) != CKR_OK) {
    ckr_scene_destroy(s);
    return st;
  }
  if ((st = build_tri_nm(s)) != CKR_OK) {
    ckr_scene_destroy(s);
    return st;
  }
  if (d->env) {
    s->env_w = d->env->width;
    s->env_h = d->env->height;
    s->env_axis = d->env->axis;
    s->env_n = d->env->n_samples ? d->env->n_samples : 10;  // MIS::nEnMpIS
    s->env_inv_area = (float)(1.0 / env.area);
  }
  s->nlights = d->nlights;
  s->first_point = first_point;
  s->first_emit = first_emit;
  s->n_emit = n_emit;
  float lo[3] = {3e38f, 3e38f, 3e38f}, hi[3] = {-3e38f, -3e38f, -3e38f};
  for (size_t i = 0; i < 3 * (size_t)d->ntri; ++i)
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::min(lo[c], d->tri9[3 * i + c]);
      hi[c] = std::max(hi[c], d->tri9[3 * i + c]);
    }
  for (uint32_t i = 0; i < d->nsph; ++i)
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::min(lo[c], d->sph4[4 * i + c] - d->sph4[4 * i + 3]);
      hi[c] = std::max(hi[c], d->sph4[4 * i + c] + d->sph4[4 * i + 3]);
    }
  for (int c = 0; c < 3; ++c) {
    s->bounds[c] = lo[c] <= hi[c] ? lo[c] : 0.f;
    s->bounds[3 + c] = lo[c] <= hi[c] ? hi[c] : 0.f;
  }
  s->host_mats.assign(d->materials, d->materials + nm);
  s->host_lights = lights;
  s->has_shading = true;
  *out = s;
  return CKR_OK;
}
