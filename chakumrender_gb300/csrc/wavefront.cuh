// wavefront.cuh — the renderer's wavefront kernels (device code shared by the
// single-render entry points, render.cu, and the batched renderer, batch.cu).
//
// Paths occupy path slots.  Each step runs three persistent kernels over
// device-side queues: k_extend (closest hit), k_shade (emits shadow rays and the
// continuation ray into queues whose slots are reserved once per warp: a
// warp-wide prefix sum of the per-lane counts and one atomicAdd by lane 31),
// k_shadow (any hit, adds unoccluded contributions).  Queue lengths live in device
// memory.  Paths run in waves (a fixed sequence of launches with no host
// synchronisation, capturable in a CUDA graph), or, with Params::regen_total set,
// a shading step that ends a path starts the next camera path in its slot
// (regenerate).  Kernels are templated on the block size (the traversal stack in
// shared memory is laid out [level][thread]).
//
// Batches: with Params::jobs set, a path carries its job index in meta.w >> 8 and
// the job supplies the camera, the material table offset, the random seed, the
// depth limit and the output pixel base (JobDev).
#pragma once
#include <cuda_fp16.h>

#include <algorithm>

#include "ckr_internal.h"
#include "ltc_table.h"
#include "render_device.cuh"

namespace ckr {
namespace {

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
  uint32_t *counts;  // [0] q[0] length, [1] q[1] length, [2] shadow count, [3] [4] work counters of
                     // k_extend and k_shadow (zeroed before each k_extend)
  unsigned long long *stats;  // cumulative closest-hit rays, shadow rays
  double *accum;     // 3 per output pixel
  uint32_t sh_cap;   // shadow-queue capacity (rays)
  int *status;       // the scene's device status word (first CKR_ERR_*)
};

// Shadow rays of one shading step past the queue's capacity are dropped and the
// status word records CKR_ERR_QUEUE_OVERFLOW (the host sizes the queue so that
// this cannot happen; the check keeps a wrong size from writing out of bounds).
__device__ __forceinline__ uint32_t shadow_fit(const Paths &P, uint32_t sbase, uint32_t nshadow) {
  if (nshadow && sbase + nshadow > P.sh_cap) {
    atomicCAS(P.status, 0, CKR_ERR_QUEUE_OVERFLOW);
    return 0;
  }
  return nshadow;
}

// One job of a batched render: its paths are the global path indices
// [path_begin, path_begin + npix * spp), its pixels the accumulation rows
// [accum_off, accum_off + npix), its materials sv.mats[mat_off ...].
struct JobDev {
  Cam cam;
  uint64_t path_begin;
  uint64_t seed;
  uint32_t npix, spp, max_depth, mat_off, accum_off;
  float *rgb;  // output, npix x 3
};

struct Params {
  uint32_t shader, spp, max_depth, n_light, n_brdf;
  float rr_prob;
  uint64_t seed;
  uint32_t npix;
  uint32_t shadow_per_path;
  const JobDev *jobs;  // batched render (nullptr: one render described by the fields above)
  uint32_t njobs;
  // Path regeneration (single render): a shading kernel that ends a path starts
  // camera path P.counts[5]++ in its slot while that index is below regen_total
  // (0: off); cam is the camera of those paths.
  uint32_t regen_total;
  Cam cam;
  // Caller rays (ckr_shade_rays): path g traces ray g % npix (two float4 per ray)
  // as sample g / npix, keyed and accumulated as output row g % npix; nullptr:
  // camera rays.
  const float4 *rays;
};

// Per-path values that a batch takes from the path's job.
struct PathCtx {
  uint64_t seed;
  uint32_t max_depth, px_base, mat_off;
};

__device__ __forceinline__ PathCtx path_ctx(const Params &prm, uint32_t flags) {
  PathCtx c;
  if (prm.jobs) {
    const JobDev &J = prm.jobs[flags >> 8];
    c.seed = J.seed;
    c.max_depth = J.max_depth;
    c.px_base = J.accum_off;
    c.mat_off = J.mat_off;
  } else {
    c.seed = prm.seed;
    c.max_depth = prm.max_depth;
    c.px_base = 0;
    c.mat_off = 0;
  }
  return c;
}

// Job of global path index g (jobs sorted by path_begin).
__device__ __forceinline__ uint32_t job_of(const JobDev *jobs, uint32_t njobs, uint64_t g) {
  uint32_t lo = 0, hi = njobs - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (jobs[mid].path_begin <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

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

// The state of camera path g (path index = sample * npix + pixel, within a job):
// ray origin (tmin in w), direction (tmax in w), throughput (MIS weight in w) and
// meta (output pixel, sample, depth, flags with the job index above bit 8).
__device__ __forceinline__ void camera_ray(const Cam &cam0, const Params &prm, uint64_t g, float4 &ro, float4 &rd,
                                           float4 &b4, uint4 &meta) {
  b4 = make_float4(1.f, 1.f, 1.f, 1.f);
  if (prm.rays) {
    const uint32_t sample = (uint32_t)(g / prm.npix), row = (uint32_t)(g % prm.npix);
    const float4 o = prm.rays[2 * (size_t)row], d4 = prm.rays[2 * (size_t)row + 1];
    const F3 d = normalize(f3(d4.x, d4.y, d4.z));  // shade() takes normalised directions
    ro = make_float4(o.x, o.y, o.z, fmaxf(o.w, 0.f));  // a negative tmin marks explicit rays
    rd = make_float4(d.x, d.y, d.z, d4.w);
    meta = make_uint4(row, sample, 0u, 0u);
    return;
  }
  Cam cam = cam0;
  uint32_t npix = prm.npix, job = 0, px_base = 0;
  if (prm.jobs) {
    job = job_of(prm.jobs, prm.njobs, g);
    const JobDev &J = prm.jobs[job];
    cam = J.cam;
    npix = J.npix;
    px_base = J.accum_off;
    g -= J.path_begin;
  }
  uint32_t sample = (uint32_t)(g / npix), pix = (uint32_t)(g % npix);
  uint32_t x = pix % cam.w, y = pix / cam.w;
  float jx = sample < 8 ? c_jx[sample] : 0.f, jy = sample < 8 ? c_jy[sample] : 0.f;
  F3 d = cam.cx * (((float)x + jx) / (float)cam.w - 0.5f) + cam.cy * (((float)y + jy) / (float)cam.h - 0.5f) +
         cam.dir;
  d = normalize(d);
  ro = make_float4(cam.pos.x, cam.pos.y, cam.pos.z, 0.f);
  rd = make_float4(d.x, d.y, d.z, 3.0e38f);
  uint32_t out_px = (cam.h - 1 - y) * cam.w + x;
  meta = make_uint4(px_base + out_px, sample, 0u, job << 8);
}

// Starts camera path g in path slot `slot`.
__device__ __forceinline__ void camera_path(const Cam &cam0, const Params &prm, const Paths &P, uint64_t g,
                                            uint32_t slot) {
  float4 ro, rd, b4;
  uint4 meta;
  camera_ray(cam0, prm, g, ro, rd, b4, meta);
  P.ray_o[slot] = ro;
  P.ray_d[slot] = rd;
  P.beta[slot] = b4;
  P.meta[slot] = meta;
}

// Camera paths wave_base + [0, wave_n) into slots [0, wave_n) and queue 0; the
// next path to start (regeneration) is wave_base + wave_n.
template <int TPB>
__global__ void __launch_bounds__(TPB) k_camera(Cam cam0, Paths P, Params prm, uint64_t wave_base,
                                                  uint32_t wave_n) {
  for (uint32_t i = blockIdx.x * TPB + threadIdx.x; i < wave_n; i += gridDim.x * TPB) {
    camera_path(cam0, prm, P, wave_base + i, i);
    P.q0[i] = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.counts[0] = wave_n;
    P.counts[5] = (uint32_t)(wave_base + wave_n);
  }
}

// Path regeneration at the end of a shading step: lanes whose path ended take the
// next camera paths (one warp-wide reservation).  Returns true when this lane's
// slot now holds a fresh camera path.  All 32 lanes must call.
__device__ __forceinline__ bool regenerate(const Params &prm, const Paths &P, bool ended, uint32_t slot) {
  if (!prm.regen_total) return false;
  const uint32_t g = warp_reserve(&P.counts[5], ended ? 1u : 0u);
  if (!ended || g >= prm.regen_total) return false;
  camera_path(prm.cam, prm, P, g, slot);
  return true;
}

// Trees at least this many levels deep are traversed with dynamic fetching
// (trace_dynamic); shallower ones with one ray per thread (trace_static).  Box
// scene (one level), 256^2 x 16 spp: 1.64 ms static, 1.75 ms dynamic; many-light
// scene (eight levels), 960x540 x 16 spp: 26.3 ms static, 23.0 ms dynamic.
constexpr uint32_t kDynamicDepth = 3;

// Resident blocks of k_extend / k_shadow: 1024 / TPB, i.e. 64 registers.  One ray
// per thread (shallow trees): box frame 1.233 -> 1.208 ms against the compiler's
// choice.  Dynamic fetching (deep trees), where the triangle test's ray data (shear
// rows, direction) sit in shared memory after the stacks (TriShearSmem): with the
// rows in registers the kernels took 92 / 89 registers (five CTAs per SM), with them
// in shared memory 78 / 72 (six / seven CTAs; 1080p 64-spp many-light frame 0.332 ->
// 0.309 s), and capped at 64 registers without spills, eight CTAs: 0.299 s.  Their
// box test keeps the conversion form (the permute form at eight CTAs: 0.301 s).
constexpr int trace_blocks(int tpb) { return 1024 / tpb < 1 ? 1 : 1024 / tpb; }

// Closest hit of the paths in queue `cur`.  DYN: dynamic fetching over the queue,
// work counter P.counts[3] (zeroed before the launch).
template <int TPB, bool DYN>
__global__ void __launch_bounds__(TPB, trace_blocks(TPB)) k_extend(SceneView s, Paths P, int cur, int depth) {
  extern __shared__ uint2 smem_trav[];
  const uint32_t *q = cur ? P.q1 : P.q0;
  auto fetch = [&](uint32_t i, RayPre &r, float &tmax) {
    const uint32_t slot = q[i];
    const float4 a = P.ray_o[slot], b = P.ray_d[slot];
    if (a.w < 0.f) return false;  // traced by the shading kernel (CKR_SHADER_EXPLICIT)
    r = make_ray(a, b);
    tmax = b.w;
    return true;
  };
  auto finish = [&](uint32_t i, uint32_t best, float t) {
    const uint32_t slot = q[i];
    P.hit_id[slot] = best;
    P.hit_t[slot] = t;
  };
  if (DYN) {
    float4 *col = shear_column<TPB>(smem_trav, depth);
    auto fetch_s = [&](uint32_t i, RayPre &r, float &tmax) {
      if (!fetch(i, r, tmax)) return false;
      store_shear<TPB>(col, r);
      return true;
    };
    trace_dynamic<false>(s, P.counts[cur], P.counts + 3, smem_trav + threadIdx.x, TPB, depth, fetch_s, finish,
                         TriShearSmem<TPB, false>{col});
  } else
    trace_static<false, TPB>(s, P.counts[cur], smem_trav + threadIdx.x, depth, fetch, finish);
}

// Any hit of the shadow queue: unoccluded rays add their contribution to the
// pixel; occluded ones zero their training record's weight.  DYN: dynamic
// fetching, work counter P.counts[4] (zeroed before the launch).
template <int TPB, bool DYN>
__global__ void __launch_bounds__(TPB, trace_blocks(TPB)) k_shadow(SceneView s, Paths P, int depth, int cur, float4 *rec) {
  extern __shared__ uint2 smem_trav[];
  const uint32_t n = min(P.counts[2], P.sh_cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // Ray statistics: closest-hit rays of this bounce and its shadow rays.
    atomicAdd(&P.stats[0], (unsigned long long)P.counts[cur]);
    atomicAdd(&P.stats[1], (unsigned long long)n);
  }
  auto fetch = [&](uint32_t i, RayPre &r, float &tmax) {
    const float4 a = P.sh_o[i], b = P.sh_d[i];
    r = make_ray(a, b);
    tmax = b.w;
    return true;
  };
  auto finish = [&](uint32_t i, uint32_t best, float) {
    if (best == kMiss) {
      const float4 c = P.sh_c[i];
      add_px(P.accum, P.sh_px[i], f3(c.x, c.y, c.z));
    } else if (rec) {
      const uint32_t ri = P.sh_rec[i];
      if (ri != kNoRec) rec[3 * (size_t)ri + 1].w = 0.f;  // occluded: the sample contributed nothing
    }
  };
  if (DYN) {
    float4 *col = shear_column<TPB>(smem_trav, depth);
    auto fetch_s = [&](uint32_t i, RayPre &r, float &tmax) {
      fetch(i, r, tmax);
      store_shear<TPB>(col, r);
      return true;
    };
    trace_dynamic<true>(s, n, P.counts + 4, smem_trav + threadIdx.x, TPB, depth, fetch_s, finish,
                        TriShearSmem<TPB, false>{col});
  } else
    trace_static<true, TPB>(s, n, smem_trav + threadIdx.x, depth, fetch, finish);
}

// Light-technique samples at one surface: returns the number of shadow rays
// written (one per sample whose direction meets a light), each with its
// pre-weighted contribution  f * L * cos / sum_k N_k p_k.
template <bool DETERMINISTIC_SPLIT, uint32_t LF = kLightsAll>
__device__ uint32_t light_samples(const ShadeView &sv, const Params &prm, const Surface &S, const Material &M,
                                  F3 fcol, F3 beta, uint64_t key, uint32_t sample, uint32_t depth, F3 o_off,
                                  float4 *so, float4 *sd, float4 *sc, bool write) {
  uint32_t cnt = 0, sidx = 0;
  // Point lights: deterministic, no MIS (src/lightSources.cpp:48-63).
  for (uint32_t k = sv.first_point; (LF & kLightPoint) && k < sv.nlights; ++k) {
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
      F3 w = sample_light<LF>(sv, L, S.x, e0, e1, e2);
      float c = dot(w, S.n);
      if (c < 0.f) continue;
      LightQuery lq = query_lights<true, LF>(sv, S.x, o_off, w, prm.n_light);
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
  // Environment light: its own technique after the area lights (EnMpIS of
  // MIS::getSamples, src/mis.cpp:154-166).
  for (uint32_t i = 0; (LF & kLightEnv) && i < sv.env_n; ++i, ++sidx) {
    float e0 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx));
    float e1 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx + 1));
    float e2 = ckr_draw_f(key, ctr(sample, depth, 3 * sidx + 2));
    F3 w = env_sample(sv, e0, e1, e2);
    float c = dot(w, S.n);
    if (c < 0.f) continue;
    LightQuery lq = query_lights<true, LF>(sv, S.x, o_off, w, prm.n_light);
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
      LightQuery lq = query_lights<true, LF>(sv, S.x, o_off, w, prm.n_light);
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

// getLightAnalytic / getLightAnalyticDiffuse over every mesh light
// (src/lightSources_CV.cpp:221-321): spec * amplitude * sum L |I_ltc| / 2pi +
// (1 - spec) * sum L |I_cos| / 2pi.
__device__ __forceinline__ F3 ltc_term(const ShadeView &sv, const Surface &S, const Material &M, const LtcLookup &Lk,
                                       const M3f &minv, bool ltc_on) {
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
  return G;
}

// The sampled part of getLightFromMeshSource_AnalyticCV (src/lightSources_CV.cpp:335-397):
// per mesh light, n_light points by MeshLight::getSamples (300-bin CDF, sqrt(u1)
// barycentrics), each adding Le (V f - f_ltc) cos cos_l / d^2 * area / n.  The
// unoccluded -f_ltc part is summed into `neg`; each +f part is a shadow ray whose
// contribution is returned through so/sd/sc when WRITE.  Returns the ray count.
template <bool WRITE>
__device__ uint32_t cv_samples(const ShadeView &sv, const Params &prm, const Surface &S, const Material &M, float refl,
                               const LtcLookup &Lk, const M3f &minv, bool ltc_on, F3 col, uint64_t key,
                               uint32_t sample, F3 o_off, F3 &neg, float4 *so, float4 *sd, float4 *sc) {
  uint32_t cnt = 0, sidx = 0;
  for (uint32_t k = 0; k < sv.first_point; ++k) {
    DevLight L = sv.lights[k];
    if (L.type != CKR_LIGHT_MESH) continue;
    const float w_area = L.area / (float)prm.n_light;
    for (uint32_t i = 0; i < prm.n_light; ++i, ++sidx) {
      float e0 = ckr_draw_f(key, ctr(sample, 0, 3 * sidx));
      float e1 = ckr_draw_f(key, ctr(sample, 0, 3 * sidx + 1));
      float e2 = ckr_draw_f(key, ctr(sample, 0, 3 * sidx + 2));
      uint32_t b = (uint32_t)(e0 * (float)kInvCdfBins);
      b = b >= kInvCdfBins ? kInvCdfBins - 1 : b;
      const uint32_t tri = L.first + __ldg(&sv.cdf[L.cdf + b]);
      const float *t9 = sv.tri9 + 9 * (size_t)tri;
      F3 A = f3(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2));
      F3 B = f3(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5));
      F3 C = f3(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8));
      F3 Pl = sample_triangle(A, B, C, e1, e2);
      F3 dv = Pl - S.x;
      float d2 = dot(dv, dv), d = sqrtf(d2);
      F3 w = dv * (1.0f / d);
      float c = dot(w, S.n);
      if (c < 0.f) continue;
      float c1 = fabsf(dot(w, tri_normal(sv, tri)));
      float g = c * c1 / d2 * w_area;
      F3 Le = mat_radiance(sv, sv.tri_mat[tri]);
      float fa = brdf_eval(M, S.n, S.wo_ref, S.wo, w) * refl;
      if (!WRITE) {
        float fl = (ltc_on ? brdf_ltc(M, Lk, minv, S.n, w) : brdf_eval(M, S.n, S.wo_ref, S.wo, w)) * refl;
        neg = neg - Le * (fl * g);
      }
      if (fa > 0.f) {
        if (WRITE) {
          F3 contrib = mulc(col, Le) * (fa * g);
          so[cnt] = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
          sd[cnt] = shadow_dir(o_off, Pl);
          sc[cnt] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
        }
        ++cnt;
      }
    }
  }
  return cnt;
}

// Continuation dims of CKR_SHADER_EXPLICIT: RR at kDimRR, redraws r < kExplicitTries
// of the hemisphere direction at kDimHemi + 2r, + 2r + 1.
constexpr uint32_t kDimHemi = 1004, kExplicitTries = 8;

template <uint32_t SHADER, int TPB, uint32_t LF = kLightsAll>
__device__ __forceinline__ void shade(ShadeView sv0, Paths P, Params prm, int cur, int depth,
                                      const LtcEntry *__restrict__ ltc, SceneView scene, int stack_depth) {
  const uint32_t n = P.counts[cur];
  const uint32_t *q = cur ? P.q1 : P.q0;
  uint32_t *qn = cur ? P.q0 : P.q1;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (TPB / 32);
  const uint32_t warp_id = blockIdx.x * (TPB / 32) + (threadIdx.x >> 5);
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
    ShadeView sv = sv0;  // a batch job's materials replace the scene's
    PathCtx pc = path_ctx(prm, 0u);
    uint64_t key = 0;
    F3 o_off = f3(0, 0, 0);
    bool surface = false;
    if (valid) {
      uint32_t id = P.hit_id[slot];
      meta = P.meta[slot];
      pc = path_ctx(prm, meta.w);
      sv.mats = sv0.mats + pc.mat_off;
      if ((LF & kLightEnv) && id == kMiss && SHADER == CKR_SHADER_PATH && sv.env_n && meta.z > 0) {
        // A BRDF-sampled ray left the scene: the environment, with its MIS weight.
        const float4 rd = P.ray_d[slot], b4 = P.beta[slot];
        const float4 e = env_lookup(sv, f3(rd.x, rd.y, rd.z));
        add_px(P.accum, meta.x, mulc(f3(b4.x, b4.y, b4.z), f3(e.x, e.y, e.z)) * b4.w);
      }
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
          key = ckr_key(pc.seed, meta.x - pc.px_base);
          o_off = offset_origin(S.x, S.n);
        }
      }
    }
    // ---- direct light: count the shadow rays, reserve, then write them ----
    LtcLookup Lk{};
    M3f minv{};
    bool ltc_on = false;
    F3 cv_neg = f3(0, 0, 0);
    if (surface && (SHADER == CKR_SHADER_DIRECT_MISCV || SHADER == CKR_SHADER_DIRECT_CV ||
                    SHADER == CKR_SHADER_EXPLICIT)) {
      auto tab = [&](int idx) { return ltc[idx]; };
      float theta = acosf(fminf(1.0f, fmaxf(-1.0f, dot(S.n, S.wo))));
      Lk = ltc_lookup(tab, theta, M.alpha);
      minv = ltc_minv_world(Lk, S.n, S.wo);
      ltc_on = M.brdf == kGGX || M.brdf == kGGXApprox;
    }
    if (surface && SHADER == CKR_SHADER_DIRECT_CV)
      nshadow = cv_samples<false>(sv, prm, S, M, sv.mats[S.mat].reflectance, Lk, minv, ltc_on,
                                  f3(sv.mats[S.mat].color[0], sv.mats[S.mat].color[1], sv.mats[S.mat].color[2]), key,
                                  meta.y, o_off, cv_neg, nullptr, nullptr, nullptr);
    else if (surface && SHADER != CKR_SHADER_DIRECT_MISCV && SHADER != CKR_SHADER_EXPLICIT)
      nshadow = light_samples<SHADER == CKR_SHADER_DIRECT_MIS, LF>(sv, prm, S, M, fcol, beta, key, meta.y, meta.z,
                                                                   o_off, nullptr, nullptr, nullptr, false);
    uint32_t sbase = warp_reserve(&P.counts[2], nshadow);
    nshadow = shadow_fit(P, sbase, nshadow);
    if (nshadow) {
      if (SHADER == CKR_SHADER_DIRECT_CV) {
        F3 unused = f3(0, 0, 0);
        cv_samples<true>(sv, prm, S, M, sv.mats[S.mat].reflectance, Lk, minv, ltc_on,
                         f3(sv.mats[S.mat].color[0], sv.mats[S.mat].color[1], sv.mats[S.mat].color[2]), key, meta.y,
                         o_off, unused, P.sh_o + sbase, P.sh_d + sbase, P.sh_c + sbase);
      } else {
        light_samples<SHADER == CKR_SHADER_DIRECT_MIS, LF>(sv, prm, S, M, fcol, beta, key, meta.y, meta.z, o_off,
                                                       P.sh_o + sbase, P.sh_d + sbase, P.sh_c + sbase, true);
      }
      for (uint32_t k = 0; k < nshadow; ++k) P.sh_px[sbase + k] = meta.x;
    }
    if (surface && SHADER == CKR_SHADER_DIRECT_CV) {
      // getLightFromMeshSource_AnalyticCV: the LTC term plus the unoccluded part of
      // the sampled residual; the occluded part arrives through the shadow rays.
      const ckr_material &mm = sv.mats[S.mat];
      F3 col = f3(mm.color[0], mm.color[1], mm.color[2]);
      add_px(P.accum, meta.x, mulc(col, ltc_term(sv, S, M, Lk, minv, ltc_on) + cv_neg));
    }
    if (surface && (SHADER == CKR_SHADER_DIRECT_MISCV || SHADER == CKR_SHADER_EXPLICIT)) {
      // getLightFromMeshSource_Analytic_MISCV (src/lightSources_CV.cpp:399-450); at
      // every vertex of the explicit path loop (shadeDI, src/shader.cpp:100-109).
      F3 G = ltc_term(sv, S, M, Lk, minv, ltc_on);
      // MIS residual over the getSamples set; visibility is 1 in the reference.
      F3 res = f3(0, 0, 0);
      const uint32_t nb = prm.n_brdf, nlobe = (uint32_t)((float)nb * M.spec);
      const uint32_t nls = sv.first_point * prm.n_light;
      for (uint32_t si = 0; si < nls + nb; ++si) {
        float e0 = ckr_draw_f(key, ctr(meta.y, meta.z, 3 * si));
        float e1 = ckr_draw_f(key, ctr(meta.y, meta.z, 3 * si + 1));
        float e2 = ckr_draw_f(key, ctr(meta.y, meta.z, 3 * si + 2));
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
      add_px(P.accum, meta.x, mulc(beta, mulc(col, res + G)));
    }
    // ---- continuation of the explicit path loop (shadeExplicit, src/shader.cpp:111-207):
    // Russian roulette 0.3 after the vertex's direct light, then a uniform hemisphere
    // direction, redrawn while it meets an emitter (emitters only count through the
    // direct term), traced here; beta *= c 2 pi cos f / 0.7.
    if (SHADER == CKR_SHADER_EXPLICIT) {
      extern __shared__ uint2 smem_trav[];
      uint32_t hit = kMiss;
      float th = 0.f;
      F3 wn = f3(0, 0, 0);
      const bool go = surface && meta.z + 1 < pc.max_depth &&
                      ckr_draw_f(key, ctr(meta.y, meta.z, kDimRR)) >= prm.rr_prob;
      // Every lane runs the same number of traversals (the stack is per thread, the
      // loop has no barrier, but keeping lanes together keeps the warp converged).
      bool done = !go;
      for (uint32_t r = 0; r < kExplicitTries; ++r) {
        if (!done) {
          wn = sample_hemisphere(S.n, ckr_draw_f(key, ctr(meta.y, meta.z, kDimHemi + 2 * r)),
                                 ckr_draw_f(key, ctr(meta.y, meta.z, kDimHemi + 2 * r + 1)));
          RayPre rp = ray_pre(o_off, wn, 0.f);
          th = 3.0e38f;
          hit = trace_ray<false>(scene, rp, th, smem_trav + threadIdx.x, TPB, stack_depth);
          if (hit == kMiss) {
            done = true;  // escapes the scene
          } else {
            const uint32_t hm = (hit & kSphereBit) ? __ldg(&sv.sph_mat[hit & ~kSphereBit]) : __ldg(&sv.tri_mat[hit]);
            if (sv.mats[hm].light_type == 0) done = true;  // accepted
            else hit = kMiss;                              // an emitter: draw again
          }
        }
      }
      if (go && hit != kMiss) {
        const ckr_material &mm = sv.mats[S.mat];
        float f = brdf_eval(M, S.n, S.wo_ref, S.wo, wn) * mm.reflectance;
        float k = 2.0f * kPi * dot(wn, S.n) * f / (1.0f - prm.rr_prob);
        F3 nb = mulc(beta, f3(mm.color[0], mm.color[1], mm.color[2])) * k;
        cont = true;
        next_o = o_off;
        next_d = make_float4(wn.x, wn.y, wn.z, 3.0e38f);
        next_b = make_float4(nb.x, nb.y, nb.z, 1.f);
        P.hit_id[slot] = hit;
        P.hit_t[slot] = th;
      }
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
          LightQuery lq = query_lights<true, LF>(sv, S.x, o_off, w, prm.n_light);
          float wb = (float)prm.n_brdf * pb / ((float)prm.n_brdf * pb + lq.pdf_sum);
          F3 nb = mulc(beta, fcol) * (f * c / (pb * (1.0f - prm.rr_prob)));
          cont = true;
          next_o = o_off;
          next_d = make_float4(w.x, w.y, w.z, 3.0e38f);
          next_b = make_float4(nb.x, nb.y, nb.z, wb);
        }
      }
    }
    const bool fresh = regenerate(prm, P, valid && !cont, slot);
    uint32_t cbase = warp_reserve(&P.counts[cur ^ 1], cont || fresh ? 1u : 0u);
    if (cont) {
      // Continue in place: the path keeps its slot.  tmin = -1 marks a ray the
      // explicit loop has traced already.
      P.ray_o[slot] = make_float4(next_o.x, next_o.y, next_o.z, SHADER == CKR_SHADER_EXPLICIT ? -1.f : 0.f);
      P.ray_d[slot] = next_d;
      P.beta[slot] = next_b;
      uint32_t nd = meta.z + 1;
      P.meta[slot] = make_uint4(meta.x, meta.y, nd, (meta.w & ~1u) | (nd >= pc.max_depth ? 1u : 0u));
    }
    if (cont || fresh) qn[cbase] = slot;
  }
}

// Shading kernels.  The MIS path tracer's vertex is register hungry but short: at
// 640 / TPB resident blocks (96 registers at 128 threads, with some spills) the box
// frame took 1.50 ms against 1.65 ms at the default 149 registers.  The direct-light
// shaders run at 1024 / TPB resident blocks (64 registers at 128 threads): box
// 512^2 x 4 spp, 10 light + 60 BRDF samples, DIRECT_MIS 10.0 -> 7.8 ms, DIRECT_CV
// 2.46 -> 2.40 ms against the compiler's choice.  The explicit path loop, which
// traverses inside the kernel, at 512 / TPB (128 registers; box 256^2 x 4 spp,
// depth 4: 7.01 ms at the compiler's 195 registers, 4.81 ms, 5.06 ms at 640 / TPB).
constexpr int shade_blocks(uint32_t shader, int tpb) {
  return shader == CKR_SHADER_EXPLICIT ? (512 / tpb > 1 ? 512 / tpb : 1) : (1024 / tpb > 1 ? 1024 / tpb : 1);
}

template <uint32_t SHADER, int TPB>
__global__ void __launch_bounds__(TPB, shade_blocks(SHADER, TPB)) k_shade(ShadeView sv0, Paths P, Params prm, int cur, int depth,
                                                 const LtcEntry *__restrict__ ltc, SceneView scene = SceneView{},
                                                 int stack_depth = 0) {
  shade<SHADER, TPB>(sv0, P, prm, cur, depth, ltc, scene, stack_depth);
}

// LF: the light kinds compiled in (kLightsMeshOnly for scenes whose lights are all
// MESH / TRI lights, see light_kinds_of).
template <int TPB, uint32_t LF = kLightsAll>
__global__ void __launch_bounds__(TPB, (640 / TPB > 1 ? 640 / TPB : 1))
    k_shade_path(ShadeView sv0, Paths P, Params prm, int cur, int depth, const LtcEntry *__restrict__ ltc) {
  shade<CKR_SHADER_PATH, TPB, LF>(sv0, P, prm, cur, depth, ltc, SceneView{}, 0);
}

// Whether a scene's lights are all MESH / TRI lights (no point or sphere light, no
// environment): its path shader can leave the other kinds' code out.
inline bool mesh_lights_only(const ckr_scene *s) {
  if (s->env_n) return false;
  for (const DevLight &L : s->host_lights)
    if (L.type != CKR_LIGHT_MESH && L.type != CKR_LIGHT_TRI) return false;
  return true;
}

// The reference's default shader (MISCV) at 1024 / TPB resident blocks (64
// registers at 128 threads, with spills): box, 512^2 x 4 spp, 10 light + 60 BRDF
// samples: 6.13 ms at 512 / TPB (128 registers), 6.24 at 640, 5.89 at 768, 5.51 at
// 1024, 5.83 at 1280, 5.78 at 1536; at 154 spill-free registers it was slower still.
template <int TPB>
__global__ void __launch_bounds__(TPB, (1024 / TPB > 1 ? 1024 / TPB : 1))
    k_shade_miscv(ShadeView sv0, Paths P, Params prm, int cur, int depth, const LtcEntry *__restrict__ ltc) {
  shade<CKR_SHADER_DIRECT_MISCV, TPB>(sv0, P, prm, cur, depth, ltc, SceneView{}, 0);
}

// CKR_SHADER_PATH_NEE: one light sample and one BRDF sample per vertex over many
// lights.  The light technique draws an emitter light from the selection
// distribution, one of its triangles in proportion to power and a uniform point
// on it; the BRDF sample continues the path and, if it meets an emitter, is
// weighted at the next vertex with the light technique's pdf of the previous
// vertex (its pdf is carried in beta.w).  Balance heuristic throughout.  Launched
// with 1024 / TPB resident blocks (64 registers at 128 threads, some spills): the
// many-light frame at 640 / 768 / 896 / 1024 was 0.3135 / 0.3110 / 0.3042 /
// 0.3040 s, the extra resident warps hiding the vertex's dependent loads.
template <int TPB>
__global__ void __launch_bounds__(TPB, (1024 / TPB > 1 ? 1024 / TPB : 1))
    k_shade_nee(ShadeView sv0, Paths P, Params prm, int cur, Learn lr) {
  const uint32_t n = P.counts[cur];
  const uint32_t *q = cur ? P.q1 : P.q0;
  uint32_t *qn = cur ? P.q0 : P.q1;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (TPB / 32);
  const uint32_t warp_id = blockIdx.x * (TPB / 32) + (threadIdx.x >> 5);
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
    ShadeView sv = sv0;  // a batch job's materials replace the scene's
    PathCtx pc = path_ctx(prm, 0u);
    if (valid) {
      uint32_t id = P.hit_id[slot];
      meta = P.meta[slot];
      pc = path_ctx(prm, meta.w);
      sv.mats = sv0.mats + pc.mat_off;
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
          uint64_t key = ckr_key(pc.seed, meta.x - pc.px_base);
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
              sd = shadow_dir(o_off, Pl);
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
          if (meta.z + 1 <= pc.max_depth) {
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
    nshadow = shadow_fit(P, sbase, nshadow);
    if (nshadow) {
      P.sh_o[sbase] = so;
      P.sh_d[sbase] = sd;
      P.sh_c[sbase] = sc;
      P.sh_px[sbase] = meta.x;
      if (lr.rec) P.sh_rec[sbase] = rbase;
    }
    const bool fresh = regenerate(prm, P, valid && !cont, slot);
    uint32_t cbase = warp_reserve(&P.counts[cur ^ 1], cont || fresh ? 1u : 0u);
    if (cont) {
      P.ray_o[slot] = make_float4(next_o.x, next_o.y, next_o.z, 0.f);
      P.ray_d[slot] = next_d;
      P.beta[slot] = next_b;
      uint32_t nd = meta.z + 1;
      P.meta[slot] = make_uint4(meta.x, meta.y, nd, (meta.w & ~1u) | (nd >= pc.max_depth ? 1u : 0u));
      if (lr.sel) P.prev_row[slot] = i;
    }
    if (cont || fresh) qn[cbase] = slot;
  }
}

// Batched resolve: accumulation row p belongs to the job whose rows contain it.
__global__ void k_resolve_jobs(const double *accum, const JobDev *jobs, uint32_t njobs, uint32_t npix_total) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix_total; p += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = njobs - 1;
    while (lo < hi) {
      uint32_t mid = (lo + hi + 1) >> 1;
      if (jobs[mid].accum_off <= p) lo = mid;
      else hi = mid - 1;
    }
    const JobDev &J = jobs[lo];
    const double inv = 1.0 / J.spp;
    const uint32_t q = p - J.accum_off;
    for (int c = 0; c < 3; ++c) J.rgb[3 * (size_t)q + c] = (float)(accum[3 * (size_t)p + c] * inv);
  }
}

__global__ void k_resolve(const double *accum, float *rgb, uint32_t n3, double inv_spp) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x)
    rgb[i] = (float)(accum[i] * inv_spp);
}


int grid_for(const void *fn, size_t smem, int tpb) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, tpb, smem);
  return std::max(1, sms * std::max(1, per));
}

}  // namespace
}  // namespace ckr
