// render.cu — wavefront renderer: camera rays -> closest hit -> shade (MIS light
// sampling, BRDF-sampled continuation) -> shadow rays -> FP64 accumulation.
//
// Paths are processed in waves of up to `wave` paths.  Each bounce runs three
// persistent kernels over device-side queues: k_extend (closest hit),
// k_shade (emits shadow rays and the continuation ray into queues whose slots
// are reserved once per warp: a warp-wide prefix sum of the per-lane counts and
// one atomicAdd by lane 0), k_shadow (any hit, adds unoccluded contributions).
// Queue lengths live in device memory, so a whole render is a fixed sequence of
// launches with no host synchronisation (capturable in a CUDA graph).
//
// Shaders (ckr_render_cfg.shader):
//   DIRECT_MISCV  shadeDirectOnly + getLightFromMeshSource_Analytic_MISCV
//                 (src/shader.cpp:339-359, src/lightSources_CV.cpp:399-450):
//                 LTC analytic term + MIS residual (brdf - LTC approximation),
//                 visibility fixed to 1 as in the reference (:434-438).
//   DIRECT_MIS    shadeDirectOnly + getLightFromAllSources_MIS
//                 (src/lightSources.cpp:32-109) with MIS::getSamples counts.
//   PATH          the path loop: at every vertex the same MIS estimator with
//                 n_light_samples per light and one BRDF sample that also
//                 continues the path; Russian roulette with rr_prob.
#include <algorithm>

#include "ckr_internal.h"
#include "ltc_table.h"
#include "mlp.h"
#include "proposal.h"
#include "render_device.cuh"

namespace ckr {
namespace {

constexpr int kRTPB = 128;
constexpr uint32_t kCtrDim = 1024;  // counter dims per (sample, vertex)
constexpr uint32_t kDimBrdf = 1000, kDimRR = 1003, kDimTrain = 1010;
constexpr uint32_t kNoRec = 0xFFFFFFFFu;

// Hooks of the learned light selection (CKR_SHADER_PATH_NEE with a proposal
// network); all null for selection in proportion to power.
struct Learn {
  const uint16_t *sel;       // [queue row x 64] selection CDFs at this bounce's vertices
  const uint16_t *sel_prev;  // the same at the previous bounce (rows by Paths::prev_row)
  float4 *rec;               // training records, 3 float4 each: (x, alpha), (n, value), (wo, cluster)
  uint32_t *rec_count;
  uint32_t rec_cap;
};

__device__ __forceinline__ uint32_t ctr(uint32_t sample, uint32_t depth, uint32_t dim) {
  return ((sample * 64u + depth) * kCtrDim) + dim;
}

// Reference camera (src/main.cpp:77) with the fixed sub-pixel offsets of
// src/main.cpp:23-24 for the first eight samples.
__constant__ float c_jx[8] = {0.34f, 0.86f, 0.20f, 0.86f, 0.66f, 0.34f, 0.20f, 0.66f};
__constant__ float c_jy[8] = {0.20f, 0.66f, 0.66f, 0.34f, 0.86f, 0.86f, 0.34f, 0.20f};

struct Cam {
  F3 pos, dir, cx, cy;
  uint32_t w, h;
};

struct Paths {
  float4 *ray_o;   // ox oy oz tmin
  float4 *ray_d;   // dx dy dz tmax
  float4 *beta;    // throughput rgb, MIS weight of the BRDF sample that made the ray
  uint4 *meta;     // out-pixel index, sample, depth, flags (1 = emission only)
  uint32_t *hit_id;
  float *hit_t;
  uint32_t *q0, *q1;  // path-slot queues
  float4 *sh_o, *sh_d, *sh_c;  // shadow rays and their contributions
  uint32_t *sh_px;
  uint32_t *prev_row;  // learned selection: the path's row in the previous bounce's probabilities
  uint32_t *sh_rec;    // training: per shadow ray, its training record (kNoRec: none)
  uint32_t *counts;  // [0] q[0] length, [1] q[1] length, [2] shadow count
  unsigned long long *stats;  // cumulative closest-hit rays, shadow rays
  double *accum;     // 3 per output pixel
};

struct Params {
  uint32_t shader, spp, max_depth, n_light, n_brdf;
  float rr_prob;
  uint64_t seed;
  uint32_t npix;
  uint32_t shadow_per_path;
};

// Reserves `k` consecutive slots per lane in a queue; all 32 lanes must call.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t *counter, uint32_t k) {
  const int lane = threadIdx.x & 31;
  uint32_t incl = k;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(counter, total);
  base = __shfl_sync(0xffffffffu, base, 31);
  return base + incl - k;
}

__device__ __forceinline__ void add_px(double *accum, uint32_t px, F3 c) {
  atomicAdd(&accum[3 * (size_t)px], (double)c.x);
  atomicAdd(&accum[3 * (size_t)px + 1], (double)c.y);
  atomicAdd(&accum[3 * (size_t)px + 2], (double)c.z);
}

__global__ void __launch_bounds__(kRTPB) k_camera(Cam cam, Paths P, Params prm, uint64_t wave_base,
                                                  uint32_t wave_n) {
  for (uint32_t i = blockIdx.x * kRTPB + threadIdx.x; i < wave_n; i += gridDim.x * kRTPB) {
    uint64_t g = wave_base + i;  // path index = sample * npix + pixel
    uint32_t sample = (uint32_t)(g / prm.npix), pix = (uint32_t)(g % prm.npix);
    uint32_t x = pix % cam.w, y = pix / cam.w;
    float jx = sample < 8 ? c_jx[sample] : 0.f, jy = sample < 8 ? c_jy[sample] : 0.f;
    F3 d = cam.cx * (((float)x + jx) / (float)cam.w - 0.5f) + cam.cy * (((float)y + jy) / (float)cam.h - 0.5f) +
           cam.dir;
    d = normalize(d);
    P.ray_o[i] = make_float4(cam.pos.x, cam.pos.y, cam.pos.z, 0.f);
    P.ray_d[i] = make_float4(d.x, d.y, d.z, 3.0e38f);
    P.beta[i] = make_float4(1.f, 1.f, 1.f, 1.f);
    uint32_t out_px = (cam.h - 1 - y) * cam.w + x;
    P.meta[i] = make_uint4(out_px, sample, 0u, 0u);
    P.q0[i] = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) P.counts[0] = wave_n;
}

__global__ void __launch_bounds__(kRTPB) k_extend(SceneView s, Paths P, int cur, int depth) {
  extern __shared__ int32_t smem_stack[];
  int32_t *stack = smem_stack + threadIdx.x;
  const uint32_t n = P.counts[cur];
  const uint32_t *q = cur ? P.q1 : P.q0;
  for (uint32_t i = blockIdx.x * kRTPB + threadIdx.x; i < n; i += gridDim.x * kRTPB) {
    uint32_t slot = q[i];
    float4 a = P.ray_o[slot], b = P.ray_d[slot];
    RayPre r = make_ray(a, b);
    float t = b.w;
    uint32_t id = trace_ray<false>(s, r, t, stack, kRTPB, depth);
    P.hit_id[slot] = id;
    P.hit_t[slot] = t;
  }
}

__global__ void __launch_bounds__(kRTPB) k_shadow(SceneView s, Paths P, int depth, int cur, float4 *rec) {
  extern __shared__ int32_t smem_stack[];
  int32_t *stack = smem_stack + threadIdx.x;
  const uint32_t n = P.counts[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // Ray statistics: closest-hit rays of this bounce and its shadow rays.
    atomicAdd(&P.stats[0], (unsigned long long)P.counts[cur]);
    atomicAdd(&P.stats[1], (unsigned long long)n);
  }
  for (uint32_t i = blockIdx.x * kRTPB + threadIdx.x; i < n; i += gridDim.x * kRTPB) {
    float4 a = P.sh_o[i], b = P.sh_d[i];
    RayPre r = make_ray(a, b);
    float t = b.w;
    if (trace_ray<true>(s, r, t, stack, kRTPB, depth) == kMiss) {
      float4 c = P.sh_c[i];
      add_px(P.accum, P.sh_px[i], f3(c.x, c.y, c.z));
    } else if (rec) {
      uint32_t ri = P.sh_rec[i];
      if (ri != kNoRec) rec[3 * (size_t)ri + 1].w = 0.f;  // occluded: the sample contributed nothing
    }
  }
}

// Light-technique samples at one surface: returns the number of shadow rays
// written (one per sample whose direction meets a light), each with its
// pre-weighted contribution  f * L * cos / sum_k N_k p_k.
template <bool DETERMINISTIC_SPLIT>
__device__ uint32_t light_samples(const ShadeView &sv, const Params &prm, const Surface &S, const Material &M,
                                  F3 fcol, F3 beta, uint64_t key, uint32_t sample, uint32_t depth, F3 o_off,
                                  float4 *so, float4 *sd, float4 *sc, bool write) {
  uint32_t cnt = 0, sidx = 0;
  // Point lights: deterministic, no MIS (src/lightSources.cpp:48-63).
  for (uint32_t k = sv.first_point; k < sv.nlights; ++k) {
    DevLight L = sv.lights[k];
    F3 dl = f3(L.px, L.py, L.pz) - S.x;
    float dist = length(dl);
    F3 w = dl * (1.0f / dist);
    float c = dot(w, S.n);
    if (c < 0.f) continue;
    if (write) {
      float f = brdf_eval(M, S.n, S.wo_ref, S.wo, w);
      float sc4 = c * f / (4.0f * kPi * dist * dist);
      F3 contrib = mulc(beta, mulc(fcol, f3(L.pr, L.pg, L.pb))) * sc4;
      so[cnt] = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
      sd[cnt] = make_float4(w.x, w.y, w.z, shadow_tmax(length(f3(L.px, L.py, L.pz) - o_off)));
      sc[cnt] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
    }
    ++cnt;
  }
  // Area and sphere lights: N samples each.  Lights are stored in the reference's
  // getSamples order (sphere sources, mesh sources, triangle sources, then point
  // lights; src/mis.cpp:100-146), so sample s belongs to light s / N.
  for (uint32_t k = 0; k < sv.nlights; ++k) {
    DevLight L = sv.lights[k];
    if (L.type == CKR_LIGHT_POINT) break;
    for (uint32_t i = 0; i < prm.n_light; ++i, ++sidx) {
      float e0 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx));
      float e1 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx + 1));
      float e2 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx + 2));
      F3 w = sample_light(sv, L, S.x, e0, e1, e2);
      float c = dot(w, S.n);
      if (c < 0.f) continue;
      LightQuery lq = query_lights(sv, S.x, o_off, w, prm.n_light);
      if (!lq.hit) continue;
      if (write) {
        float denom = lq.pdf_sum + (float)prm.n_brdf * pdf_eval(M, S.n, S.wo_ref, S.wo, w);
        float f = brdf_eval(M, S.n, S.wo_ref, S.wo, w);
        F3 contrib = mulc(beta, mulc(fcol, lq.Le)) * (f * c / (denom + 1e-20f));
        so[cnt] = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
        sd[cnt] = make_float4(w.x, w.y, w.z, shadow_tmax(lq.d));
        sc[cnt] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
      }
      ++cnt;
    }
  }
  if (DETERMINISTIC_SPLIT) {
    // BRDF technique of MIS::getSamples: N*spec lobe samples, the rest cosine
    // (MaterialType::getBrdfDirectionSamples, src/materialTypes.cpp:118-134).
    uint32_t nb = prm.n_brdf, nlobe = (uint32_t)((float)nb * M.spec);
    for (uint32_t i = 0; i < nb; ++i, ++sidx) {
      float e1 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx + 1));
      float e2 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx + 2));
      F3 w = i < nlobe ? sample_lobe(M, S.n, S.wo_ref, S.wo, e1, e2) : sample_cosine(S.n, e1, e2);
      float c = dot(w, S.n);
      if (c < 0.f) continue;
      LightQuery lq = query_lights(sv, S.x, o_off, w, prm.n_light);
      if (!lq.hit) continue;
      if (write) {
        float denom = lq.pdf_sum + (float)nb * pdf_eval(M, S.n, S.wo_ref, S.wo, w);
        float f = brdf_eval(M, S.n, S.wo_ref, S.wo, w);
        F3 contrib = mulc(beta, mulc(fcol, lq.Le)) * (f * c / (denom + 1e-20f));
        so[cnt] = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
        sd[cnt] = make_float4(w.x, w.y, w.z, shadow_tmax(lq.d));
        sc[cnt] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
      }
      ++cnt;
    }
  }
  return cnt;
}

template <uint32_t SHADER>
__global__ void __launch_bounds__(kRTPB) k_shade(ShadeView sv, Paths P, Params prm, int cur, int depth,
                                                 const LtcEntry *__restrict__ ltc) {
  const uint32_t n = P.counts[cur];
  const uint32_t *q = cur ? P.q1 : P.q0;
  uint32_t *qn = cur ? P.q0 : P.q1;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (kRTPB / 32);
  const uint32_t warp_id = blockIdx.x * (kRTPB / 32) + (threadIdx.x >> 5);
  for (uint32_t base = warp_id * 32; base < n; base += warps * 32) {
    uint32_t i = base + lane;
    bool valid = i < n;
    uint32_t slot = valid ? q[i] : 0;
    uint32_t nshadow = 0;
    bool cont = false;
    float4 next_d = make_float4(0, 0, 0, 0), next_b = make_float4(0, 0, 0, 0);
    F3 next_o = f3(0, 0, 0);
    Surface S;
    Material M;
    F3 fcol = f3(0, 0, 0), beta = f3(0, 0, 0);
    uint4 meta = make_uint4(0, 0, 0, 0);
    uint64_t key = 0;
    F3 o_off = f3(0, 0, 0);
    bool surface = false;
    if (valid) {
      uint32_t id = P.hit_id[slot];
      meta = P.meta[slot];
      if (id != kMiss) {
        float4 ro = P.ray_o[slot], rd = P.ray_d[slot], b4 = P.beta[slot];
        beta = f3(b4.x, b4.y, b4.z);
        S = make_surface(sv, f3(ro.x, ro.y, ro.z), f3(rd.x, rd.y, rd.z), id, P.hit_t[slot]);
        const ckr_material &mm = sv.mats[S.mat];
        if (mm.light_type != 0) {
          // Emitter.  Camera rays see MaterialType::getRadiance, the radiance
          // divided by its largest component (headers/materialTypes.h:34-38);
          // BRDF-sampled rays carry their MIS weight.
          F3 Le = f3(mm.radiance[0], mm.radiance[1], mm.radiance[2]);
          if (meta.z == 0) {
            float mx = fmaxf(Le.x, fmaxf(Le.y, Le.z));
            // Vec::maxnorm picks the largest component in x, y, z order.
            mx = Le.x;
            if (mx < Le.y) mx = Le.y;
            if (mx < Le.z) mx = Le.z;
            add_px(P.accum, meta.x, Le * (1.0f / mx));
          } else {
            add_px(P.accum, meta.x, mulc(beta, Le) * b4.w);
          }
        } else if (!(meta.w & 1u)) {
          surface = true;
          M = material_of(mm);
          fcol = f3(mm.color[0], mm.color[1], mm.color[2]) * mm.reflectance;
          key = ckr_key(prm.seed, meta.x);
          o_off = offset_origin(S.x, S.n);
        }
      }
    }
    // ---- direct light: count the shadow rays, reserve, then write them ----
    if (surface && SHADER != CKR_SHADER_DIRECT_MISCV)
      nshadow = light_samples<SHADER == CKR_SHADER_DIRECT_MIS>(sv, prm, S, M, fcol, beta, key, meta.y, meta.z, o_off,
                                                               nullptr, nullptr, nullptr, false);
    uint32_t sbase = warp_reserve(&P.counts[2], nshadow);
    if (nshadow) {
      light_samples<SHADER == CKR_SHADER_DIRECT_MIS>(sv, prm, S, M, fcol, beta, key, meta.y, meta.z, o_off,
                                                     P.sh_o + sbase, P.sh_d + sbase, P.sh_c + sbase, true);
      for (uint32_t k = 0; k < nshadow; ++k) P.sh_px[sbase + k] = meta.x;
    }
    if (surface && SHADER == CKR_SHADER_DIRECT_MISCV) {
      // getLightFromMeshSource_Analytic_MISCV (src/lightSources_CV.cpp:399-450).
      auto tab = [&](int idx) { return ltc[idx]; };
      float theta = acosf(fminf(1.0f, fmaxf(-1.0f, dot(S.n, S.wo))));
      LtcLookup Lk = ltc_lookup(tab, theta, M.alpha);
      M3f minv = ltc_minv_world(Lk, S.n, S.wo);
      bool ltc_on = M.brdf == kGGX || M.brdf == kGGXApprox;
      F3 G = f3(0, 0, 0);
      for (uint32_t k = 0; k < sv.nlights; ++k) {
        DevLight L = sv.lights[k];
        if (L.type != CKR_LIGHT_MESH) continue;
        F3 gs = f3(0, 0, 0), gd = f3(0, 0, 0);
        for (uint32_t j = 0; j < L.count; ++j) {
          const float *t9 = sv.tri9 + 9 * (size_t)(L.first + j);
          F3 A = f3(t9[0], t9[1], t9[2]), B = f3(t9[3], t9[4], t9[5]), C = f3(t9[6], t9[7], t9[8]);
          F3 Le = mat_radiance(sv, sv.tri_mat[L.first + j]);
          float s = ltc_on ? ltc_spec_tri(A, B, C, S.x, minv) : 0.f;
          float d = ltc_diffuse_tri(A, B, C, S.n, S.x);
          gs = gs + Le * s;
          gd = gd + Le * d;
        }
        const float inv2pi = 1.0f / (2.0f * kPi);
        G = G + gs * (inv2pi * (ltc_on ? Lk.amp : 0.f) * M.spec) + gd * (inv2pi * (1.0f - M.spec));
      }
      // MIS residual over the getSamples set; visibility is 1 in the reference.
      F3 res = f3(0, 0, 0);
      const uint32_t nb = prm.n_brdf, nlobe = (uint32_t)((float)nb * M.spec);
      const uint32_t nls = sv.first_point * prm.n_light;
      for (uint32_t si = 0; si < nls + nb; ++si) {
        float e0 = ckr_draw_f(key, ctr(meta.y, 0, 3 * si));
        float e1 = ckr_draw_f(key, ctr(meta.y, 0, 3 * si + 1));
        float e2 = ckr_draw_f(key, ctr(meta.y, 0, 3 * si + 2));
        F3 w = si < nls ? sample_light(sv, sv.lights[si / prm.n_light], S.x, e0, e1, e2)
                        : (si - nls < nlobe ? sample_lobe(M, S.n, S.wo_ref, S.wo, e1, e2) : sample_cosine(S.n, e1, e2));
        float c = dot(w, S.n);
        if (c < 0.f) continue;
        LightQuery lq = query_lights(sv, S.x, o_off, w, prm.n_light);
        float denom = lq.pdf_sum + (float)nb * pdf_eval(M, S.n, S.wo_ref, S.wo, w);
        // First mesh light in list order that the direction meets.
        RayPre r = ray_pre(o_off, w, 0.f);
        for (uint32_t k = 0; k < sv.nlights; ++k) {
          DevLight L = sv.lights[k];
          if (L.type != CKR_LIGHT_MESH) continue;
          float t;
          uint32_t id = light_tri_hit(sv, L, r, t);
          if (id == kMiss) continue;
          float fa = brdf_eval(M, S.n, S.wo_ref, S.wo, w) * sv.mats[S.mat].reflectance;
          float fl = (ltc_on ? brdf_ltc(M, Lk, minv, S.n, w) : brdf_eval(M, S.n, S.wo_ref, S.wo, w)) *
                     sv.mats[S.mat].reflectance;
          res = res + mat_radiance(sv, sv.tri_mat[id]) * ((fa - fl) * c / (denom + 1e-20f));
          break;
        }
      }
      const ckr_material &mm = sv.mats[S.mat];
      F3 col = f3(mm.color[0], mm.color[1], mm.color[2]);
      add_px(P.accum, meta.x, mulc(col, res + G));
    }
    // ---- continuation (path tracer) ----
    if (surface && SHADER == CKR_SHADER_PATH) {
      float e0 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf));
      float e1 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 1));
      float e2 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 2));
      F3 w = sample_brdf(M, S.n, S.wo_ref, S.wo, e0, e1, e2);
      float c = dot(w, S.n);
      float err = ckr_draw_f(key, ctr(meta.y, meta.z, kDimRR));
      if (c > 0.f && err >= prm.rr_prob) {
        float pb = pdf_eval(M, S.n, S.wo_ref, S.wo, w);
        float f = brdf_eval(M, S.n, S.wo_ref, S.wo, w);
        if (pb > 0.f && f > 0.f) {
          LightQuery lq = query_lights(sv, S.x, o_off, w, prm.n_light);
          float wb = (float)prm.n_brdf * pb / ((float)prm.n_brdf * pb + lq.pdf_sum);
          F3 nb = mulc(beta, fcol) * (f * c / (pb * (1.0f - prm.rr_prob)));
          cont = true;
          next_o = o_off;
          next_d = make_float4(w.x, w.y, w.z, 3.0e38f);
          next_b = make_float4(nb.x, nb.y, nb.z, wb);
        }
      }
    }
    uint32_t cbase = warp_reserve(&P.counts[cur ^ 1], cont ? 1u : 0u);
    if (cont) {
      // Continue in place: the path keeps its slot.
      P.ray_o[slot] = make_float4(next_o.x, next_o.y, next_o.z, 0.f);
      P.ray_d[slot] = next_d;
      P.beta[slot] = next_b;
      uint32_t nd = meta.z + 1;
      P.meta[slot] = make_uint4(meta.x, meta.y, nd, nd + 1 >= prm.max_depth + 1 ? 1u : 0u);
      qn[cbase] = slot;
    }
  }
}

// CKR_SHADER_PATH_NEE: one light sample and one BRDF sample per vertex over many
// lights.  The light technique draws an emitter light from the selection
// distribution, one of its triangles in proportion to power and a uniform point
// on it; the BRDF sample continues the path and, if it meets an emitter, is
// weighted at the next vertex with the light technique's pdf of the previous
// vertex (its pdf is carried in beta.w).  Balance heuristic throughout.
__global__ void __launch_bounds__(kRTPB) k_shade_nee(ShadeView sv, Paths P, Params prm, int cur, Learn lr) {
  const uint32_t n = P.counts[cur];
  const uint32_t *q = cur ? P.q1 : P.q0;
  uint32_t *qn = cur ? P.q0 : P.q1;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (kRTPB / 32);
  const uint32_t warp_id = blockIdx.x * (kRTPB / 32) + (threadIdx.x >> 5);
  const float train_frac = lr.rec && n ? fminf(1.0f, (float)lr.rec_cap / (float)n) : 0.f;
  for (uint32_t base = warp_id * 32; base < n; base += warps * 32) {
    const uint32_t i = base + lane;
    const bool valid = i < n;
    const uint32_t slot = valid ? q[i] : 0;
    uint32_t nshadow = 0;
    bool cont = false, rec_ok = false;
    float4 next_d = make_float4(0, 0, 0, 0), next_b = make_float4(0, 0, 0, 0);
    float4 so = make_float4(0, 0, 0, 0), sd = so, sc = so, r0 = so, r1 = so, r2 = so;
    F3 next_o = f3(0, 0, 0);
    uint4 meta = make_uint4(0, 0, 0, 0);
    if (valid) {
      uint32_t id = P.hit_id[slot];
      meta = P.meta[slot];
      if (id != kMiss) {
        float4 ro = P.ray_o[slot], rd = P.ray_d[slot], b4 = P.beta[slot];
        F3 beta = f3(b4.x, b4.y, b4.z);
        Surface S = make_surface(sv, f3(ro.x, ro.y, ro.z), f3(rd.x, rd.y, rd.z), id, P.hit_t[slot]);
        const ckr_material &mm = sv.mats[S.mat];
        if (mm.light_type != 0) {
          F3 Le = f3(mm.radiance[0], mm.radiance[1], mm.radiance[2]);
          if (meta.z == 0) {
            float mx = Le.x;  // Vec::maxnorm, as the other shaders
            if (mx < Le.y) mx = Le.y;
            if (mx < Le.z) mx = Le.z;
            add_px(P.accum, meta.x, Le * (1.0f / mx));
          } else {
            float wb = 1.0f;
            uint32_t k = (id & kSphereBit) ? kNoLight : __ldg(&sv.tri_light[id]);
            if (k != kNoLight && b4.w > 0.f) {
              DevLight L = sv.lights[k];
              Select sel{lr.sel_prev ? lr.sel_prev + 64 * (size_t)P.prev_row[slot] : nullptr};
              const float *t9 = sv.tri9 + 9 * (size_t)id;
              F3 A = f3(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2));
              F3 B = f3(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5));
              F3 C = f3(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8));
              F3 nrm = cross_rn(C - A, B - A);
              float len = length(nrm);
              float cl = fabsf(dot(nrm, f3(rd.x, rd.y, rd.z))) / len;
              float pl = nee_pdf(sv, select_prob(sv, sel, k - sv.first_emit), L, id, P.hit_t[slot], 0.5f * len, cl);
              if (pl > 0.f && pl < 3.0e38f) wb = b4.w / (b4.w + pl);
            }
            add_px(P.accum, meta.x, mulc(beta, Le) * wb);
          }
        } else if (!(meta.w & 1u)) {
          Material M = material_of(mm);
          F3 fcol = f3(mm.color[0], mm.color[1], mm.color[2]) * mm.reflectance;
          uint64_t key = ckr_key(prm.seed, meta.x);
          F3 o_off = offset_origin(S.x, S.n);
          // ---- light technique: one sample ----
          float e0 = ckr_draw_f(key, ctr(meta.y, meta.z, 0)), e1 = ckr_draw_f(key, ctr(meta.y, meta.z, 1));
          float e2 = ckr_draw_f(key, ctr(meta.y, meta.z, 2)), e3 = ckr_draw_f(key, ctr(meta.y, meta.z, 3));
          Select sel{lr.sel ? lr.sel + 64 * (size_t)i : nullptr};
          uint32_t j = select_pick(sv, sel, e0);
          DevLight L = sv.lights[sv.first_emit + j];
          uint32_t tri = L.first + cdf_pick(sv.pcdf + L.pcdf, L.count, e1);
          const float *t9 = sv.tri9 + 9 * (size_t)tri;
          F3 A = f3(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2));
          F3 B = f3(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5));
          F3 C = f3(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8));
          F3 Pl = sample_triangle(A, B, C, e2, e3);
          F3 dv = Pl - S.x;
          float dist = length(dv);
          F3 w = dv * (1.0f / dist);
          float c = dot(w, S.n);
          F3 nrm = cross_rn(C - A, B - A);
          float len = length(nrm);
          float cl = fabsf(dot(nrm, w)) / len;
          if (c > 0.f && cl > 0.f && len > 0.f && dist > 0.f) {
            float pl = nee_pdf(sv, select_prob(sv, sel, j), L, tri, dist, 0.5f * len, cl);
            float f = brdf_eval(M, S.n, S.wo_ref, S.wo, w);
            if (pl > 0.f && f > 0.f) {
              float pb = pdf_eval(M, S.n, S.wo_ref, S.wo, w);
              F3 Le = mat_radiance(sv, sv.tri_mat[tri]);
              float g = f * c / pl;
              F3 contrib = mulc(beta, mulc(fcol, Le)) * (g * (pl / (pl + pb)));
              nshadow = 1;
              so = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
              sd = make_float4(w.x, w.y, w.z, shadow_tmax(length(Pl - o_off)));
              sc = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
              if (train_frac > 0.f && ckr_draw_f(key, ctr(meta.y, meta.z, kDimTrain)) < train_frac) {
                // Training sample: the unweighted estimate of cluster j's direct light
                // (luminance), zeroed by the shadow kernel if the ray is blocked.
                F3 fl = mulc(fcol, Le);
                rec_ok = true;
                r0 = make_float4(S.x.x, S.x.y, S.x.z, M.alpha);
                r1 = make_float4(S.n.x, S.n.y, S.n.z, (fl.x + fl.y + fl.z) * (1.0f / 3.0f) * g);
                r2 = make_float4(S.wo.x, S.wo.y, S.wo.z, __uint_as_float(j));
              }
            }
          }
          // ---- BRDF technique: continues the path ----
          if (meta.z + 1 <= prm.max_depth) {
            float b0 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf));
            float b1 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 1));
            float b2 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 2));
            F3 wn = sample_brdf(M, S.n, S.wo_ref, S.wo, b0, b1, b2);
            float cn = dot(wn, S.n);
            float err = ckr_draw_f(key, ctr(meta.y, meta.z, kDimRR));
            if (cn > 0.f && err >= prm.rr_prob) {
              float pb = pdf_eval(M, S.n, S.wo_ref, S.wo, wn);
              float f = brdf_eval(M, S.n, S.wo_ref, S.wo, wn);
              if (pb > 0.f && f > 0.f) {
                F3 nb = mulc(beta, fcol) * (f * cn / (pb * (1.0f - prm.rr_prob)));
                cont = true;
                next_o = o_off;
                next_d = make_float4(wn.x, wn.y, wn.z, 3.0e38f);
                next_b = make_float4(nb.x, nb.y, nb.z, pb);
              }
            }
          }
        }
      }
    }
    uint32_t rbase = kNoRec;
    if (lr.rec) {
      rbase = warp_reserve(lr.rec_count, rec_ok ? 1u : 0u);
      if (rec_ok && rbase < lr.rec_cap) {
        lr.rec[3 * (size_t)rbase] = r0;
        lr.rec[3 * (size_t)rbase + 1] = r1;
        lr.rec[3 * (size_t)rbase + 2] = r2;
      } else {
        rbase = kNoRec;
      }
    }
    uint32_t sbase = warp_reserve(&P.counts[2], nshadow);
    if (nshadow) {
      P.sh_o[sbase] = so;
      P.sh_d[sbase] = sd;
      P.sh_c[sbase] = sc;
      P.sh_px[sbase] = meta.x;
      if (lr.rec) P.sh_rec[sbase] = rbase;
    }
    uint32_t cbase = warp_reserve(&P.counts[cur ^ 1], cont ? 1u : 0u);
    if (cont) {
      P.ray_o[slot] = make_float4(next_o.x, next_o.y, next_o.z, 0.f);
      P.ray_d[slot] = next_d;
      P.beta[slot] = next_b;
      uint32_t nd = meta.z + 1;
      P.meta[slot] = make_uint4(meta.x, meta.y, nd, nd >= prm.max_depth ? 1u : 0u);
      if (lr.sel) P.prev_row[slot] = i;
      qn[cbase] = slot;
    }
  }
}

__global__ void k_resolve(const double *accum, float *rgb, uint32_t n3, double inv_spp) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x)
    rgb[i] = (float)(accum[i] * inv_spp);
}

struct Workspace {
  DevBuf<float4> ray_o, ray_d, beta, sh_o, sh_d, sh_c;
  DevBuf<uint4> meta;
  DevBuf<uint32_t> hit_id, q0, q1, sh_px, counts;
  DevBuf<unsigned long long> stats;
  DevBuf<float> hit_t;
  DevBuf<double> accum;
  size_t wave = 0, shadow = 0, pixels = 0;
};

int grid_for(const void *fn, size_t smem, int tpb) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, tpb, smem);
  return std::max(1, sms * std::max(1, per));
}

}  // namespace
}  // namespace ckr

using namespace ckr;

namespace {
void free_ws(void *p) { delete static_cast<Workspace *>(p); }
}  // namespace

namespace {

int render_impl(ckr_scene *s, ckr_proposal *prop, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb,
                double *accum, void *stream_) {
  if (!s || !cam || !cfg || !rgb || cam->width == 0 || cam->height == 0 || cfg->spp == 0 || cfg->shader > 3)
    return CKR_ERR_INVALID_ARGUMENT;
  if (!s->has_shading) return CKR_ERR_INVALID_ARGUMENT;
  if (cfg->max_depth > 60 || cfg->spp > 65536 || cfg->n_light_samples > 256 || cfg->n_brdf_samples > 256)
    return CKR_ERR_TOO_LARGE;
  if (prop && (cfg->shader != CKR_SHADER_PATH_NEE || prop->net.nclusters != s->n_emit))
    return CKR_ERR_INVALID_ARGUMENT;
  cudaStream_t stream = (cudaStream_t)stream_;
  std::lock_guard<std::mutex> lock(s->host_mu);
  std::unique_lock<std::mutex> plock;
  if (prop) plock = std::unique_lock<std::mutex>(prop->mu);
  int st = CKR_OK;
  const LtcEntry *ltc = device_ltc_table(&st);
  if (!ltc) return st;
  Params prm;
  prm.shader = cfg->shader;
  prm.spp = cfg->spp;
  const bool path = cfg->shader == CKR_SHADER_PATH || cfg->shader == CKR_SHADER_PATH_NEE;
  if (cfg->shader == CKR_SHADER_PATH_NEE && s->n_emit == 0) return CKR_ERR_INVALID_ARGUMENT;
  prm.max_depth = path ? std::max(1u, cfg->max_depth) : 1u;
  prm.n_light = cfg->n_light_samples;
  prm.n_brdf = path ? 1u : cfg->n_brdf_samples;
  prm.rr_prob = path ? cfg->rr_prob : 0.f;
  prm.seed = cfg->seed;
  prm.npix = cam->width * cam->height;
  uint32_t area_lights = 0, point_lights = 0;
  for (const DevLight &L : s->host_lights) (L.type == CKR_LIGHT_POINT ? point_lights : area_lights)++;
  uint32_t per_path = cfg->shader == CKR_SHADER_PATH_NEE
                          ? 1u
                          : point_lights + area_lights * prm.n_light + (cfg->shader == CKR_SHADER_DIRECT_MIS ? prm.n_brdf : 0);
  prm.shadow_per_path = std::max(1u, per_path);
  uint64_t total = (uint64_t)prm.npix * prm.spp;
  size_t wave = (size_t)std::min<uint64_t>(total, std::max<uint64_t>(32768, (1ull << 23) / prm.shadow_per_path));
  wave = std::min<size_t>(wave, 1u << 21);
  if (!s->render_ws) {
    s->render_ws = new Workspace();
    s->render_ws_free = free_ws;
  }
  Workspace &W = *static_cast<Workspace *>(s->render_ws);
  size_t shadow = wave * prm.shadow_per_path;
  CKR_CUDA_TRY(W.ray_o.reserve(wave));
  CKR_CUDA_TRY(W.ray_d.reserve(wave));
  CKR_CUDA_TRY(W.beta.reserve(wave));
  CKR_CUDA_TRY(W.meta.reserve(wave));
  CKR_CUDA_TRY(W.hit_id.reserve(wave));
  CKR_CUDA_TRY(W.hit_t.reserve(wave));
  CKR_CUDA_TRY(W.q0.reserve(wave));
  CKR_CUDA_TRY(W.q1.reserve(wave));
  CKR_CUDA_TRY(W.sh_o.reserve(shadow));
  CKR_CUDA_TRY(W.sh_d.reserve(shadow));
  CKR_CUDA_TRY(W.sh_c.reserve(shadow));
  CKR_CUDA_TRY(W.sh_px.reserve(shadow));
  CKR_CUDA_TRY(W.counts.reserve(4));
  if (!W.stats.ptr) {
    CKR_CUDA_TRY(W.stats.reserve(2));
    CKR_CUDA_TRY(cudaMemset(W.stats.ptr, 0, 2 * sizeof(unsigned long long)));
  }
  double *acc = accum;
  if (!acc) {
    CKR_CUDA_TRY(W.accum.reserve((size_t)prm.npix * 3));
    acc = W.accum.ptr;
  }
  CKR_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(double) * 3 * (size_t)prm.npix, stream));
  Paths P{};
  P.ray_o = W.ray_o.ptr; P.ray_d = W.ray_d.ptr; P.beta = W.beta.ptr; P.meta = W.meta.ptr;
  P.hit_id = W.hit_id.ptr; P.hit_t = W.hit_t.ptr; P.q0 = W.q0.ptr; P.q1 = W.q1.ptr;
  P.sh_o = W.sh_o.ptr; P.sh_d = W.sh_d.ptr; P.sh_c = W.sh_c.ptr; P.sh_px = W.sh_px.ptr;
  P.counts = W.counts.ptr;
  P.stats = W.stats.ptr;
  P.accum = acc;
  bool train = prop && prop->train && (!prop->max_steps || prop->net.step < prop->max_steps);
  if (prop) {
    CKR_CUDA_TRY(prop->sel[0].reserve(64 * wave));
    CKR_CUDA_TRY(prop->sel[1].reserve(64 * wave));
    CKR_CUDA_TRY(prop->prev_row.reserve(wave));
    CKR_CUDA_TRY(prop->sh_rec.reserve(shadow));
    CKR_CUDA_TRY(prop->rec.reserve(3 * (size_t)prop->batch));
    P.prev_row = prop->prev_row.ptr;
    P.sh_rec = prop->sh_rec.ptr;
    CKR_CUDA_TRY(cudaMemsetAsync(prop->rec_count.ptr, 0, 4, stream));
  }
  Cam c;
  c.pos = f3(cam->pos[0], cam->pos[1], cam->pos[2]);
  c.dir = f3(cam->dir[0], cam->dir[1], cam->dir[2]);
  c.cx = f3(cam->cx[0], cam->cx[1], cam->cx[2]);
  c.cy = f3(cam->cy[0], cam->cy[1], cam->cy[2]);
  c.w = cam->width;
  c.h = cam->height;
  SceneView sv = view_of(s);
  ShadeView shv = shade_view_of(s);
  int depth = (int)stack_depth_of(s);
  size_t smem = (size_t)depth * kRTPB * sizeof(int32_t);
  if (smem > 48 * 1024) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_extend, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_shadow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int g_ext = grid_for((const void *)k_extend, smem, kRTPB);
  const int g_sh = grid_for((const void *)k_shadow, smem, kRTPB);
  const void *shade_fn = cfg->shader == CKR_SHADER_PATH_NEE ? (const void *)k_shade_nee
                         : cfg->shader == CKR_SHADER_PATH      ? (const void *)k_shade<CKR_SHADER_PATH>
                         : cfg->shader == CKR_SHADER_DIRECT_MIS ? (const void *)k_shade<CKR_SHADER_DIRECT_MIS>
                                                                : (const void *)k_shade<CKR_SHADER_DIRECT_MISCV>;
  const int g_shade = grid_for(shade_fn, 0, kRTPB);
  for (uint64_t base = 0; base < total; base += wave) {
    uint32_t n = (uint32_t)std::min<uint64_t>(wave, total - base);
    k_camera<<<std::min<int>(g_ext, ceil_div(n, kRTPB)), kRTPB, 0, stream>>>(c, P, prm, base, n);
    int cur = 0;
    for (uint32_t d = 0; d <= prm.max_depth; ++d) {
      k_extend<<<g_ext, kRTPB, smem, stream>>>(sv, P, cur, depth);
      CKR_CUDA_TRY(cudaMemsetAsync(P.counts + (cur ^ 1), 0, sizeof(uint32_t), stream));
      CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 2, 0, sizeof(uint32_t), stream));
      Learn lr{};
      if (prop) {
        // Light distributions at this bounce's vertices.
        mlp::PathRows pr;
        pr.queue = cur ? P.q1 : P.q0;
        pr.hit_id = P.hit_id;
        pr.ray_o = P.ray_o;
        pr.ray_d = P.ray_d;
        pr.hit_t = P.hit_t;
        pr.meta = P.meta;
        pr.sv = shv;
        int ms = mlp::infer_paths(prop->net, pr, (uint32_t)wave, P.counts + cur, prop->sel[d & 1].ptr,
                                  prop->defensive, stream);
        if (ms != CKR_OK) return ms;
        lr.sel = prop->sel[d & 1].ptr;
        lr.sel_prev = d ? prop->sel[(d - 1) & 1].ptr : nullptr;
        if (train) {
          lr.rec = prop->rec.ptr;
          lr.rec_count = prop->rec_count.ptr;
          lr.rec_cap = prop->batch;
        }
      }
      if (cfg->shader == CKR_SHADER_PATH_NEE)
        k_shade_nee<<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, lr);
      else if (cfg->shader == CKR_SHADER_PATH)
        k_shade<CKR_SHADER_PATH><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      else if (cfg->shader == CKR_SHADER_DIRECT_MIS)
        k_shade<CKR_SHADER_DIRECT_MIS><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      else
        k_shade<CKR_SHADER_DIRECT_MISCV><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      k_shadow<<<g_sh, kRTPB, smem, stream>>>(sv, P, depth, cur, train ? prop->rec.ptr : nullptr);
      if (train) {
        // Adam steps on this bounce's light samples (visibility applied above),
        // minibatch by minibatch; steps past the records actually written are no-ops.
        for (uint32_t off = 0; off < prop->batch; off += prop->minibatch) {
          int ts = mlp::train_step(prop->net, prop->rec.ptr + 3 * (size_t)off,
                                   std::min(prop->minibatch, prop->batch - off), prop->rec_count.ptr, off, stream);
          if (ts != CKR_OK) return ts;
        }
        CKR_CUDA_TRY(cudaMemsetAsync(prop->rec_count.ptr, 0, 4, stream));
        if (prop->max_steps && prop->net.step >= prop->max_steps) train = false;  // converged: inference only
      }
      cur ^= 1;
      if (!path) break;
    }
  }
  uint32_t n3 = prm.npix * 3;
  k_resolve<<<std::min<unsigned>(1024, ceil_div(n3, 256)), 256, 0, stream>>>(acc, rgb, n3, 1.0 / prm.spp);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}

}  // namespace

extern "C" int ckr_render(ckr_scene *s, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb, double *accum,
                          void *stream) {
  return render_impl(s, nullptr, cam, cfg, rgb, accum, stream);
}

extern "C" int ckr_render_learned(ckr_scene *s, ckr_proposal *prop, const ckr_camera *cam, const ckr_render_cfg *cfg,
                                  float *rgb, double *accum, void *stream) {
  if (!prop) return CKR_ERR_INVALID_ARGUMENT;
  return render_impl(s, prop, cam, cfg, rgb, accum, stream);
}

extern "C" int ckr_render_stats(ckr_scene *s, uint64_t *closest_rays, uint64_t *shadow_rays, int reset) {
  if (!s || !closest_rays || !shadow_rays) return CKR_ERR_INVALID_ARGUMENT;
  *closest_rays = *shadow_rays = 0;
  if (!s->render_ws) return CKR_OK;
  Workspace &W = *static_cast<Workspace *>(s->render_ws);
  if (!W.stats.ptr) return CKR_OK;
  unsigned long long h[2];
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  CKR_CUDA_TRY(cudaMemcpy(h, W.stats.ptr, sizeof(h), cudaMemcpyDeviceToHost));
  *closest_rays = h[0];
  *shadow_rays = h[1];
  if (reset) CKR_CUDA_TRY(cudaMemset(W.stats.ptr, 0, sizeof(h)));
  return CKR_OK;
}

extern "C" int ckr_render_host(ckr_scene *s, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb,
                               void *stream) {
  if (!s || !cam || !rgb) return CKR_ERR_INVALID_ARGUMENT;
  size_t n = (size_t)cam->width * cam->height * 3;
  float *d = nullptr;
  CKR_CUDA_TRY(cudaMalloc((void **)&d, n * sizeof(float)));
  int st = ckr_render(s, cam, cfg, d, nullptr, stream);
  if (st == CKR_OK) {
    cudaError_t e = cudaMemcpyAsync(rgb, d, n * sizeof(float), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) st = CKR_ERR_CUDA;
  }
  cudaFree(d);
  if (st == CKR_OK) {
    int h = ckr_scene_check(s, stream);
    if (h != 0) st = h;
  }
  return st;
}

// ---- rendering from a static arena (no device allocation) -------------------
//
// For callers that may not allocate device memory while they render: code that
// runs during CUDA stream capture (cudaMalloc / cudaFree are not capturable and
// may synchronise the device), frame loops that cannot afford the implicit
// synchronisation of an allocation, and hosts whose device memory is owned by
// their own allocator.  ckr_render_noalloc runs the same kernels as ckr_render,
// but its scratch memory (path state, path and shadow-ray queues, FP64 sums,
// a copy of the LTC table) lives in file-scope device arrays that every GPU
// loading the library holds until the process exits.
namespace ckr {
namespace {

constexpr uint32_t kNoAllocWave = 32768;         // paths per wave
constexpr uint32_t kNoAllocShadow = 131072;      // shadow rays per wave
constexpr uint32_t kNoAllocMaxPixels = 262144;   // output pixels (512 x 512)
constexpr size_t kNoAllocArenaBytes = 16u << 20;  // 16 MiB

constexpr size_t a256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kPathBytes = 4 * a256(16ull * kNoAllocWave) + 4 * a256(4ull * kNoAllocWave);
constexpr size_t kShadowBytes = 3 * a256(16ull * kNoAllocShadow) + a256(4ull * kNoAllocShadow);
constexpr size_t kAccumBytes = a256(24ull * kNoAllocMaxPixels);
static_assert(kPathBytes + kShadowBytes + 2 * 256 + kAccumBytes <= kNoAllocArenaBytes, "arena too small");

static __device__ __align__(256) unsigned char g_noalloc_arena[kNoAllocArenaBytes];
static __device__ __align__(256) LtcEntry g_noalloc_ltc[4096];

std::mutex g_noalloc_mu;
unsigned char *g_noalloc_arena_dev[64] = {};
LtcEntry *g_noalloc_ltc_dev[64] = {};

// Once per device, with that device current: the arrays' device addresses
// (the host-side names are only stand-ins) and the LTC table upload.
int noalloc_setup(int dev) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_arena_dev[dev]) return CKR_OK;
  std::vector<LtcEntry> table;
  int st = load_ltc_table(nullptr, table);
  if (st != CKR_OK) return st;
  void *arena = nullptr, *ltc = nullptr;
  CKR_CUDA_TRY(cudaGetSymbolAddress(&arena, g_noalloc_arena));
  CKR_CUDA_TRY(cudaGetSymbolAddress(&ltc, g_noalloc_ltc));
  CKR_CUDA_TRY(cudaMemcpy(ltc, table.data(), table.size() * sizeof(LtcEntry), cudaMemcpyHostToDevice));
  g_noalloc_ltc_dev[dev] = static_cast<LtcEntry *>(ltc);
  g_noalloc_arena_dev[dev] = static_cast<unsigned char *>(arena);
  return CKR_OK;
}

}  // namespace
}  // namespace ckr

extern "C" int ckr_render_noalloc(ckr_scene *s, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb,
                                  void *stream_) {
  if (!s || !cam || !cfg || !rgb || cam->width == 0 || cam->height == 0 || cfg->spp == 0 || cfg->shader > 3)
    return CKR_ERR_INVALID_ARGUMENT;
  if (!s->has_shading) return CKR_ERR_INVALID_ARGUMENT;
  if (cfg->max_depth > 60 || cfg->spp > 65536 || cfg->n_light_samples > 256 || cfg->n_brdf_samples > 256)
    return CKR_ERR_TOO_LARGE;
  if ((uint64_t)cam->width * cam->height > kNoAllocMaxPixels) return CKR_ERR_TOO_LARGE;
  cudaStream_t stream = (cudaStream_t)stream_;
  int dev = 0;
  CKR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return CKR_ERR_INVALID_ARGUMENT;
  int st = noalloc_setup(dev);
  if (st != CKR_OK) return st;
  Params prm;
  prm.shader = cfg->shader;
  prm.spp = cfg->spp;
  const bool path = cfg->shader == CKR_SHADER_PATH || cfg->shader == CKR_SHADER_PATH_NEE;
  if (cfg->shader == CKR_SHADER_PATH_NEE && s->n_emit == 0) return CKR_ERR_INVALID_ARGUMENT;
  prm.max_depth = path ? std::max(1u, cfg->max_depth) : 1u;
  prm.n_light = cfg->n_light_samples;
  prm.n_brdf = path ? 1u : cfg->n_brdf_samples;
  prm.rr_prob = path ? cfg->rr_prob : 0.f;
  prm.seed = cfg->seed;
  prm.npix = cam->width * cam->height;
  uint32_t area_lights = 0, point_lights = 0;
  for (const DevLight &L : s->host_lights) (L.type == CKR_LIGHT_POINT ? point_lights : area_lights)++;
  uint64_t per_path = cfg->shader == CKR_SHADER_PATH_NEE
                          ? 1u
                          : (uint64_t)point_lights + (uint64_t)area_lights * prm.n_light +
                                (cfg->shader == CKR_SHADER_DIRECT_MIS ? prm.n_brdf : 0);
  if (per_path > kNoAllocShadow) return CKR_ERR_TOO_LARGE;
  prm.shadow_per_path = (uint32_t)std::max<uint64_t>(1, per_path);
  uint64_t total = (uint64_t)prm.npix * prm.spp;
  uint32_t wave = (uint32_t)std::min<uint64_t>(total, std::min<uint64_t>(kNoAllocWave, kNoAllocShadow / prm.shadow_per_path));
  // Carve the arena.
  unsigned char *p = g_noalloc_arena_dev[dev];
  auto take = [&](size_t bytes) {
    unsigned char *r = p;
    p += a256(bytes);
    return r;
  };
  Paths P{};
  P.ray_o = reinterpret_cast<float4 *>(take(16ull * kNoAllocWave));
  P.ray_d = reinterpret_cast<float4 *>(take(16ull * kNoAllocWave));
  P.beta = reinterpret_cast<float4 *>(take(16ull * kNoAllocWave));
  P.meta = reinterpret_cast<uint4 *>(take(16ull * kNoAllocWave));
  P.hit_id = reinterpret_cast<uint32_t *>(take(4ull * kNoAllocWave));
  P.hit_t = reinterpret_cast<float *>(take(4ull * kNoAllocWave));
  P.q0 = reinterpret_cast<uint32_t *>(take(4ull * kNoAllocWave));
  P.q1 = reinterpret_cast<uint32_t *>(take(4ull * kNoAllocWave));
  P.sh_o = reinterpret_cast<float4 *>(take(16ull * kNoAllocShadow));
  P.sh_d = reinterpret_cast<float4 *>(take(16ull * kNoAllocShadow));
  P.sh_c = reinterpret_cast<float4 *>(take(16ull * kNoAllocShadow));
  P.sh_px = reinterpret_cast<uint32_t *>(take(4ull * kNoAllocShadow));
  P.counts = reinterpret_cast<uint32_t *>(take(16));
  P.stats = reinterpret_cast<unsigned long long *>(take(16));
  P.accum = reinterpret_cast<double *>(take(24ull * kNoAllocMaxPixels));
  // The arena keeps the previous call's contents: clear what must start at zero.
  CKR_CUDA_TRY(cudaMemsetAsync(P.counts, 0, 16, stream));
  CKR_CUDA_TRY(cudaMemsetAsync(P.stats, 0, 16, stream));
  CKR_CUDA_TRY(cudaMemsetAsync(P.accum, 0, sizeof(double) * 3 * (size_t)prm.npix, stream));
  Cam c;
  c.pos = f3(cam->pos[0], cam->pos[1], cam->pos[2]);
  c.dir = f3(cam->dir[0], cam->dir[1], cam->dir[2]);
  c.cx = f3(cam->cx[0], cam->cx[1], cam->cx[2]);
  c.cy = f3(cam->cy[0], cam->cy[1], cam->cy[2]);
  c.w = cam->width;
  c.h = cam->height;
  SceneView sv = view_of(s);
  ShadeView shv = shade_view_of(s);
  const LtcEntry *ltc = g_noalloc_ltc_dev[dev];
  int depth = (int)stack_depth_of(s);
  size_t smem = (size_t)depth * kRTPB * sizeof(int32_t);
  if (smem > 48 * 1024) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_extend, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_shadow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int g_ext = grid_for((const void *)k_extend, smem, kRTPB);
  const int g_sh = grid_for((const void *)k_shadow, smem, kRTPB);
  const void *shade_fn = cfg->shader == CKR_SHADER_PATH_NEE ? (const void *)k_shade_nee
                         : cfg->shader == CKR_SHADER_PATH      ? (const void *)k_shade<CKR_SHADER_PATH>
                         : cfg->shader == CKR_SHADER_DIRECT_MIS ? (const void *)k_shade<CKR_SHADER_DIRECT_MIS>
                                                                : (const void *)k_shade<CKR_SHADER_DIRECT_MISCV>;
  const int g_shade = grid_for(shade_fn, 0, kRTPB);
  for (uint64_t base = 0; base < total; base += wave) {
    uint32_t n = (uint32_t)std::min<uint64_t>(wave, total - base);
    k_camera<<<std::min<int>(g_ext, ceil_div(n, kRTPB)), kRTPB, 0, stream>>>(c, P, prm, base, n);
    int cur = 0;
    for (uint32_t d = 0; d <= prm.max_depth; ++d) {
      k_extend<<<g_ext, kRTPB, smem, stream>>>(sv, P, cur, depth);
      CKR_CUDA_TRY(cudaMemsetAsync(P.counts + (cur ^ 1), 0, sizeof(uint32_t), stream));
      CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 2, 0, sizeof(uint32_t), stream));
      if (cfg->shader == CKR_SHADER_PATH_NEE)
        k_shade_nee<<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, Learn{});
      else if (cfg->shader == CKR_SHADER_PATH)
        k_shade<CKR_SHADER_PATH><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      else if (cfg->shader == CKR_SHADER_DIRECT_MIS)
        k_shade<CKR_SHADER_DIRECT_MIS><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      else
        k_shade<CKR_SHADER_DIRECT_MISCV><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      k_shadow<<<g_sh, kRTPB, smem, stream>>>(sv, P, depth, cur, nullptr);
      cur ^= 1;
      if (!path) break;
    }
  }
  uint32_t n3 = prm.npix * 3;
  k_resolve<<<std::min<unsigned>(1024, ceil_div(n3, 256)), 256, 0, stream>>>(P.accum, rgb, n3, 1.0 / prm.spp);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}
