// ltc.cu — LTC polygon-light shading of a G-buffer (getLightFromMeshSource_Analytic,
// src/lightSources_CV.cpp:323-333, per pixel).
//
// The kernel is FP32-ALU bound (per pixel and emitter triangle: three
// transformed vertices, horizon clipping, 3-4 edge integrals, for both the
// specular LTC lobe and the diffuse cosine lobe) and its lanes disagree on the
// path a triangle takes (above, below or across the horizon), so triangles across
// the horizon are queued per warp and clipped by all lanes together (k_ltc_shade).
// CTAs are persistent (three per SM) and stride over pixels; the 64x64 LTC table is
// read from global memory (two entries per pixel), emitter triangles through the
// read-only path (every lane of a warp reads the same triangle, a broadcast).
#include <algorithm>

#include "ckr_internal.h"
#include "ckr_rng.h"
#include "ltc_table.h"
#include "shading_device.cuh"

namespace ckr {
namespace {

constexpr int kLtcTPB = 256, kLtcWarps = kLtcTPB / 32;
// Deferred triangles per warp and batch of 32 pixels.  256 entries (7.3 KB of shared
// memory per warp) let three CTAs share an SM: 24 warps at 80 registers with a few
// spills ran 0.725 ms per 1024^2 frame against 0.846 ms at 512 entries and two CTAs
// (104 registers); 128 entries at four CTAs (64 registers, 236 bytes of spills) ran
// 0.966 ms, its queues overflowing into in-place clipping.
constexpr uint32_t kLtcQueue = 256;

// The clipped integrals for a lane whose warp's queue is full.  Out of line: inlined
// into the classifying loop they pushed it past 128 registers (60 bytes of spills,
// 1.20 ms per 1024^2 frame against 0.84 ms).
__device__ __noinline__ float clipped_diffuse_here(F3 A, F3 B, F3 C, F3 n, F3 x) {
  return ltc_diffuse_clipped(A, B, C, n, x);
}
__device__ __noinline__ float clipped_spec_here(F3 A, F3 B, F3 C, F3 x, M3f m) {
  return ltc_spec_clipped(A, B, C, x, m);
}

// LTC table entries straight from global memory: two per pixel, through L1.
struct GlobalTable {
  const LtcEntry *t;
  SHD LtcEntry operator()(int i) const { return t[i]; }
};

// Per warp: its 32 pixels' shading frames and the emitter triangles it deferred.
struct LtcWarp {
  float px[32][17];          // x (3), n (3), Minv in world space (9); padded against bank conflicts
  float res[kLtcQueue][3];   // a deferred triangle's contribution, colour-weighted
  uint2 item[kLtcQueue];     // (lane | lobe << 5 | light << 6, previous item of the same lane or ~0)
};

// getLightFromMeshSource_Analytic per pixel, one pixel per lane.  Per emitter
// triangle and lobe a lane settles the triangles wholly above or below its horizon
// at once; a triangle across the horizon (clipping, four edge integrals) is queued,
// and the warp then works through its queue with every lane busy instead of letting
// the few lanes that clip hold up the rest.  Each lane adds its queued terms in a
// fixed order (newest first), so the result does not depend on scheduling.  A full
// queue falls back to clipping in place.
__global__ void __launch_bounds__(kLtcTPB, 3) k_ltc_shade(const float4 *__restrict__ gbuf, uint32_t npx,
                                                       const float *__restrict__ light_tri9,
                                                       const float *__restrict__ light_rgb, uint32_t nlight,
                                                       float *__restrict__ rgb, const LtcEntry *__restrict__ table) {
  extern __shared__ __align__(16) unsigned char ltc_smem[];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  LtcWarp &W = reinterpret_cast<LtcWarp *>(ltc_smem)[warp];
  const GlobalTable tab{table};
  auto light = [&](uint32_t k, F3 &A, F3 &B, F3 &C, float *c) {
    const float *t = light_tri9 + 9 * (size_t)k;
    A = f3(__ldg(t), __ldg(t + 1), __ldg(t + 2));
    B = f3(__ldg(t + 3), __ldg(t + 4), __ldg(t + 5));
    C = f3(__ldg(t + 6), __ldg(t + 7), __ldg(t + 8));
    c[0] = __ldg(light_rgb + 3 * k);
    c[1] = __ldg(light_rgb + 3 * k + 1);
    c[2] = __ldg(light_rgb + 3 * k + 2);
  };
  const float inv2pi = 1.0f / (2.0f * kPi);
  for (uint32_t base = (blockIdx.x * kLtcWarps + warp) * 32u; base < npx; base += gridDim.x * (uint32_t)kLtcTPB) {
    const uint32_t p = base + lane;
    const bool active = p < npx;
    F3 x = f3(0, 0, 0), n = f3(0, 0, 1);
    M3f minv{};
    float amp = 0.f, spec = 0.f;
    if (active) {
      const float4 g0 = gbuf[3 * (size_t)p], g1 = gbuf[3 * (size_t)p + 1], g2 = gbuf[3 * (size_t)p + 2];
      x = f3(g0.x, g0.y, g0.z);
      n = f3(g1.x, g1.y, g1.z);
      const F3 wo = f3(g2.x, g2.y, g2.z);
      const float theta = acosf(fminf(1.0f, fmaxf(-1.0f, dot(n, wo))));
      const LtcLookup L = ltc_lookup(tab, theta, g0.w);
      minv = ltc_minv_world(L, n, wo);
      amp = L.amp;
      spec = g2.w;
    }
    float *mine = W.px[lane];
    mine[0] = x.x; mine[1] = x.y; mine[2] = x.z;
    mine[3] = n.x; mine[4] = n.y; mine[5] = n.z;
    for (int i = 0; i < 9; ++i) mine[6 + i] = minv.a[i];
    float s3[3] = {0.f, 0.f, 0.f}, d3[3] = {0.f, 0.f, 0.f};
    uint32_t head = ~0u, count = 0;  // count: the same in every lane
    for (uint32_t k = 0; k < nlight; ++k) {
      F3 A, B, C;
      float c[3];
      light(k, A, B, C, c);
      float s = 0.f, d = 0.f;
      int cs = 0, cd = 0;
      if (active) {
        cs = ltc_spec_case(A, B, C, x, minv, s);
        cd = ltc_diffuse_case(A, B, C, n, x, d);
      }
      for (int j = 0; j < 3; ++j) {
        s3[j] += c[j] * s;
        d3[j] += c[j] * d;
      }
      for (uint32_t lobe = 0; lobe < 2; ++lobe) {
        const bool want = (lobe ? cd : cs) < 0;
        const unsigned m = __ballot_sync(0xffffffffu, want);
        const uint32_t slot = count + (uint32_t)__popc(m & ((1u << lane) - 1u));
        if (want) {
          if (slot < kLtcQueue) {
            W.item[slot] = make_uint2(lane | lobe << 5 | k << 6, head);
            head = slot;
          } else if (lobe) {
            const float v = clipped_diffuse_here(A, B, C, n, x);
            for (int j = 0; j < 3; ++j) d3[j] += c[j] * v;
          } else {
            const float v = clipped_spec_here(A, B, C, x, minv);
            for (int j = 0; j < 3; ++j) s3[j] += c[j] * v;
          }
        }
        count += (uint32_t)__popc(m);
      }
    }
    __syncwarp();
    // The warp's queued triangles, every lane taking the next one.
    const uint32_t nq = count < kLtcQueue ? count : kLtcQueue;
    for (uint32_t i = lane; i < nq; i += 32) {
      const uint2 it = W.item[i];
      const uint32_t pl = it.x & 31u, k = it.x >> 6;
      const float *q = W.px[pl];
      F3 A, B, C;
      float c[3];
      light(k, A, B, C, c);
      const F3 qx = f3(q[0], q[1], q[2]);
      float v;
      if ((it.x >> 5) & 1u) {
        v = ltc_diffuse_clipped(A, B, C, f3(q[3], q[4], q[5]), qx);
      } else {
        M3f qm;
        for (int j = 0; j < 9; ++j) qm.a[j] = q[6 + j];
        v = ltc_spec_clipped(A, B, C, qx, qm);
      }
      for (int j = 0; j < 3; ++j) W.res[i][j] = c[j] * v;
    }
    __syncwarp();
    for (uint32_t i = head; i != ~0u; i = W.item[i].y) {
      if ((W.item[i].x >> 5) & 1u) {
        for (int j = 0; j < 3; ++j) d3[j] += W.res[i][j];
      } else {
        for (int j = 0; j < 3; ++j) s3[j] += W.res[i][j];
      }
    }
    if (active)
      for (int j = 0; j < 3; ++j) rgb[3 * (size_t)p + j] = s3[j] * inv2pi * amp * spec + d3[j] * inv2pi * (1.0f - spec);
    __syncwarp();  // the next batch reuses the warp's shared memory
  }
}

// ---- Monte Carlo reference for the LTC integral -----------------------------------
// Per pixel, the integral over the emitter triangles of brdf x cos x radiance,
// treating the emitters as the LTC integral does: two-sided and unoccluded, a
// direction that crosses several emitters collecting each one's radiance.
// Half of the samples pick an emitter point by area, half sample the BRDF
// (getBrdfDirectionSampleRandomized); both are weighted by the balance heuristic,
// f cos L / (n_a p_area(w) + n_b p_brdf(w)) with p_area(w) = sum over the
// emitters w crosses of t^2 / (A_total |cos_l|).  Sums are FP64 per pixel.

constexpr int kMcTPB = 128;
constexpr uint32_t kMcMaxLights = 256;

// Two-sided ray/triangle distance (Moller & Trumbore 1997); 0 on a miss.
__device__ __forceinline__ float emitter_t(F3 o, F3 w, F3 a, F3 e1, F3 e2) {
  F3 p = cross(w, e2);
  float det = dot(e1, p);
  if (fabsf(det) < 1e-20f) return 0.f;
  float inv = 1.0f / det;
  F3 tv = o - a;
  float u = dot(tv, p) * inv;
  if (u < 0.f || u > 1.f) return 0.f;
  F3 q = cross(tv, e1);
  float v = dot(w, q) * inv;
  if (v < 0.f || u + v > 1.f) return 0.f;
  float t = dot(e2, q) * inv;
  return t > 0.f ? t : 0.f;
}

__global__ void __launch_bounds__(kMcTPB) k_ltc_mc(const float4 *__restrict__ gbuf, uint32_t npx,
                                                   const float *__restrict__ light_tri9,
                                                   const float *__restrict__ light_rgb, uint32_t nlight, uint32_t spp,
                                                   uint64_t seed, int fresnel, double *__restrict__ rgb) {
  __shared__ float4 s_a[kMcMaxLights], s_e1[kMcMaxLights], s_e2[kMcMaxLights];  // .w: r, g, b
  __shared__ float4 s_n[kMcMaxLights];  // unit normal, 1 / A_total
  __shared__ float s_cdf[kMcMaxLights];
  for (uint32_t k = threadIdx.x; k < nlight; k += kMcTPB) {
    const float *t = light_tri9 + 9 * (size_t)k;
    F3 a = f3(t[0], t[1], t[2]), b = f3(t[3], t[4], t[5]), c = f3(t[6], t[7], t[8]);
    F3 e1 = b - a, e2 = c - a, nn = cross_rn(e1, e2);
    float len = length(nn);
    s_a[k] = make_float4(a.x, a.y, a.z, light_rgb[3 * k]);
    s_e1[k] = make_float4(e1.x, e1.y, e1.z, light_rgb[3 * k + 1]);
    s_e2[k] = make_float4(e2.x, e2.y, e2.z, light_rgb[3 * k + 2]);
    F3 un = len > 0.f ? nn * (1.0f / len) : f3(0.f, 0.f, 0.f);
    s_n[k] = make_float4(un.x, un.y, un.z, 0.f);
    s_cdf[k] = 0.5f * len;  // area, turned into the CDF below
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float total = 0.f;
    for (uint32_t k = 0; k < nlight; ++k) total += s_cdf[k];
    float run = 0.f;
    for (uint32_t k = 0; k < nlight; ++k) {
      run += s_cdf[k];
      s_cdf[k] = run / total;
      s_n[k].w = 1.0f / total;
    }
  }
  __syncthreads();
  const uint32_t p = blockIdx.x * kMcTPB + threadIdx.x;
  if (p >= npx) return;
  float4 g0 = gbuf[3 * (size_t)p], g1 = gbuf[3 * (size_t)p + 1], g2 = gbuf[3 * (size_t)p + 2];
  F3 x = f3(g0.x, g0.y, g0.z), n = f3(g1.x, g1.y, g1.z), wo = f3(g2.x, g2.y, g2.z);
  Material M;
  M.brdf = kGGX;
  M.alpha = g0.w;
  M.phong_exp = 0.f;
  M.spec = g2.w;
  float sf = sqrtf(g1.w);
  M.int_ior = fresnel ? (1.0f + sf) / (1.0f - sf) : 1e5f;
  M.ext_ior = 1.0f;
  F3 wo_ref = normalize(n * (2.0f * dot(n, wo)) - wo);
  const uint64_t key = ckr_key(seed, p);
  const float half = 0.5f * (float)spp;
  double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
  for (uint32_t s = 0; s < spp; ++s) {
    float e0 = ckr_draw_f(key, 4 * s), e1 = ckr_draw_f(key, 4 * s + 1), e2 = ckr_draw_f(key, 4 * s + 2);
    F3 w;
    if ((s & 1u) == 0) {
      uint32_t k = 0;
      while (k + 1 < nlight && s_cdf[k] <= e0) ++k;
      float4 a = s_a[k], u = s_e1[k], v = s_e2[k];
      F3 A = f3(a.x, a.y, a.z);
      F3 P = sample_triangle(A, A + f3(u.x, u.y, u.z), A + f3(v.x, v.y, v.z), e1, e2);
      w = normalize(P - x);
    } else {
      w = sample_brdf(M, n, wo_ref, wo, e0, e1, e2);
    }
    float c = dot(w, n);
    if (!(c > 0.f)) continue;
    float pa = 0.f, L0 = 0.f, L1 = 0.f, L2 = 0.f;
    for (uint32_t k = 0; k < nlight; ++k) {
      float4 a = s_a[k], u = s_e1[k], v = s_e2[k];
      float t = emitter_t(x, w, f3(a.x, a.y, a.z), f3(u.x, u.y, u.z), f3(v.x, v.y, v.z));
      if (t > 0.f) {
        float4 un = s_n[k];
        float cl = fabsf(un.x * w.x + un.y * w.y + un.z * w.z);
        pa += t * t * un.w / cl;
        L0 += a.w;
        L1 += u.w;
        L2 += v.w;
      }
    }
    if (!(pa > 0.f)) continue;
    float f = brdf_eval(M, n, wo_ref, wo, w);
    float pb = pdf_eval(M, n, wo_ref, wo, w);
    float wgt = f * c / (half * (pa + pb));
    if (!(wgt < 3.0e38f)) continue;
    acc0 += (double)(L0 * wgt);
    acc1 += (double)(L1 * wgt);
    acc2 += (double)(L2 * wgt);
  }
  rgb[3 * (size_t)p] = acc0;
  rgb[3 * (size_t)p + 1] = acc1;
  rgb[3 * (size_t)p + 2] = acc2;
}

}  // namespace
}  // namespace ckr

using namespace ckr;

extern "C" int ckr_ltc_shade(const float *gbuf, uint32_t npx, const float *light_tri9, const float *light_rgb,
                             uint32_t nlight, float *rgb, void *stream) {
  if ((npx && (!gbuf || !rgb)) || (nlight && (!light_tri9 || !light_rgb)) || ((uintptr_t)gbuf & 15u))
    return CKR_ERR_INVALID_ARGUMENT;
  if (npx == 0) return CKR_OK;
  int st = CKR_OK;
  const LtcEntry *table = device_ltc_table(&st);
  if (!table) return st;
  if (nlight >= (1u << 26)) return CKR_ERR_TOO_LARGE;  // light index in a queue item
  const size_t smem = kLtcWarps * sizeof(LtcWarp);
  static bool attr_set[64] = {false};
  int dev = 0, sms = 0, per_sm = 0;
  CKR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_ltc_shade, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set[dev] = true;
  }
  CKR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CKR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ltc_shade, kLtcTPB, smem));
  if (per_sm < 1) return CKR_ERR_CUDA;
  int grid = (int)std::min<uint64_t>(ceil_div(npx, kLtcTPB), (uint64_t)sms * per_sm);
  k_ltc_shade<<<grid, kLtcTPB, smem, (cudaStream_t)stream>>>(reinterpret_cast<const float4 *>(gbuf), npx, light_tri9,
                                                               light_rgb, nlight, rgb, table);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}

extern "C" int ckr_ltc_mc(const float *gbuf, uint32_t npx, const float *light_tri9, const float *light_rgb,
                          uint32_t nlight, uint32_t spp, uint64_t seed, int fresnel, double *rgb, void *stream) {
  if ((npx && (!gbuf || !rgb)) || !light_tri9 || !light_rgb || nlight == 0 || ((uintptr_t)gbuf & 15u) ||
      spp == 0 || (spp & 1u) || spp > (1u << 28))
    return CKR_ERR_INVALID_ARGUMENT;
  if (nlight > kMcMaxLights) return CKR_ERR_TOO_LARGE;
  if (npx == 0) return CKR_OK;
  k_ltc_mc<<<(unsigned)ceil_div(npx, kMcTPB), kMcTPB, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4 *>(gbuf), npx, light_tri9, light_rgb, nlight, spp, seed, fresnel, rgb);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}
