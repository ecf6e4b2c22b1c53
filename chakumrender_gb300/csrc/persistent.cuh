// persistent.cuh — batched path tracing in one persistent launch.
//
// The wavefront renderer (wavefront.cuh) runs every bounce as three launches over
// queues in global memory.  For a batch of many jobs over a small scene that is a
// long fixed launch sequence whose stages each read and write the whole path
// state.  Here one persistent grid (the SMs x resident blocks) renders the whole
// batch: every lane owns one path at a time and runs its bounce loop --
// closest hit, the shading vertex, its shadow rays (any hit) and the continuation
// -- in registers, with the traversal stack in shared memory.  A lane whose path
// ends takes the next camera path of the batch: the paths of all jobs are numbered
// consecutively, and each warp draws as many path indices as it has idle lanes
// from one 64-bit counter (one atomicAdd per refill), so jobs of any resolution,
// spp and depth share the grid until the last path has started.
//
// A path draws the same random numbers and runs the same device functions as in
// the wavefront shaders (camera_ray, make_surface, light_samples, sample_brdf,
// pdf_eval, brdf_eval, query_lights, select/nee_pdf, trace_ray), so each job's
// image equals ckr_render of that job up to the order of the FP64 sums.
#pragma once
#include "wavefront.cuh"

namespace ckr {
namespace {

// Shadow rays a vertex may need (lights x samples); larger batches use the
// wavefront renderer.
constexpr uint32_t kInlineShadow = 4;

struct LaneShadow {
  float4 o[kInlineShadow], d[kInlineShadow], c[kInlineShadow];
  uint32_t n;
};

// One vertex of CKR_SHADER_PATH for the path in (ro, rd, b4, meta) that met `id`
// at `t` (the per-lane form of shade<CKR_SHADER_PATH>): emission and environment
// into the accumulation buffer, the light-technique shadow rays into `sh`, and the
// continuation in place.  Returns whether the path continues.
template <uint32_t LF>
__device__ __noinline__ bool vertex_path(const ShadeView &sv0, const Params &prm, double *accum, uint32_t id,
                                         float t, float4 &ro, float4 &rd, float4 &b4, uint4 &meta,
                                         LaneShadow &sh) {
  sh.n = 0;
  const PathCtx pc = path_ctx(prm, meta.w);
  ShadeView sv = sv0;
  sv.mats = sv0.mats + pc.mat_off;
  if (id == kMiss) {
    if ((LF & kLightEnv) && sv.env_n && meta.z > 0) {
      // A BRDF-sampled ray left the scene: the environment, with its MIS weight.
      const float4 e = env_lookup(sv, f3(rd.x, rd.y, rd.z));
      add_px(accum, meta.x, mulc(f3(b4.x, b4.y, b4.z), f3(e.x, e.y, e.z)) * b4.w);
    }
    return false;
  }
  const F3 beta = f3(b4.x, b4.y, b4.z);
  const Surface S = make_surface(sv, f3(ro.x, ro.y, ro.z), f3(rd.x, rd.y, rd.z), id, t);
  const ckr_material &mm = sv.mats[S.mat];
  if (mm.light_type != 0) {
    const F3 Le = f3(mm.radiance[0], mm.radiance[1], mm.radiance[2]);
    if (meta.z == 0) {
      float mx = Le.x;  // Vec::maxnorm, as the wavefront shaders
      if (mx < Le.y) mx = Le.y;
      if (mx < Le.z) mx = Le.z;
      add_px(accum, meta.x, Le * (1.0f / mx));
    } else {
      add_px(accum, meta.x, mulc(beta, Le) * b4.w);
    }
    return false;
  }
  if (meta.w & 1u) return false;  // the last depth only adds emission
  const Material M = material_of(mm);
  const F3 fcol = f3(mm.color[0], mm.color[1], mm.color[2]) * mm.reflectance;
  const uint64_t key = ckr_key(pc.seed, meta.x - pc.px_base);
  const F3 o_off = offset_origin(S.x, S.n);
  sh.n = light_samples<false, LF>(sv, prm, S, M, fcol, beta, key, meta.y, meta.z, o_off, sh.o, sh.d, sh.c, true);
  const float e0 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf));
  const float e1 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 1));
  const float e2 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 2));
  const F3 w = sample_brdf(M, S.n, S.wo_ref, S.wo, e0, e1, e2);
  const float c = dot(w, S.n);
  const float err = ckr_draw_f(key, ctr(meta.y, meta.z, kDimRR));
  if (!(c > 0.f && err >= prm.rr_prob)) return false;
  const float pb = pdf_eval(M, S.n, S.wo_ref, S.wo, w);
  const float f = brdf_eval(M, S.n, S.wo_ref, S.wo, w);
  if (!(pb > 0.f && f > 0.f)) return false;
  const LightQuery lq = query_lights<true, LF>(sv, S.x, o_off, w, prm.n_light);
  const float wb = (float)prm.n_brdf * pb / ((float)prm.n_brdf * pb + lq.pdf_sum);
  const F3 nb = mulc(beta, fcol) * (f * c / (pb * (1.0f - prm.rr_prob)));
  ro = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
  rd = make_float4(w.x, w.y, w.z, 3.0e38f);
  b4 = make_float4(nb.x, nb.y, nb.z, wb);
  const uint32_t nd = meta.z + 1;
  meta = make_uint4(meta.x, meta.y, nd, (meta.w & ~1u) | (nd >= pc.max_depth ? 1u : 0u));
  return true;
}

// One vertex of CKR_SHADER_PATH_NEE with lights selected in proportion to power
// (the per-lane form of k_shade_nee without a proposal network).
__device__ __noinline__ bool vertex_nee(const ShadeView &sv0, const Params &prm, double *accum, uint32_t id,
                                        float t, float4 &ro, float4 &rd, float4 &b4, uint4 &meta,
                                        LaneShadow &sh) {
  sh.n = 0;
  if (id == kMiss) return false;
  const PathCtx pc = path_ctx(prm, meta.w);
  ShadeView sv = sv0;
  sv.mats = sv0.mats + pc.mat_off;
  const F3 beta = f3(b4.x, b4.y, b4.z);
  const Surface S = make_surface(sv, f3(ro.x, ro.y, ro.z), f3(rd.x, rd.y, rd.z), id, t);
  const ckr_material &mm = sv.mats[S.mat];
  const Select none{nullptr};
  if (mm.light_type != 0) {
    const F3 Le = f3(mm.radiance[0], mm.radiance[1], mm.radiance[2]);
    if (meta.z == 0) {
      float mx = Le.x;
      if (mx < Le.y) mx = Le.y;
      if (mx < Le.z) mx = Le.z;
      add_px(accum, meta.x, Le * (1.0f / mx));
    } else {
      float wb = 1.0f;
      const uint32_t k = (id & kSphereBit) ? kNoLight : __ldg(&sv.tri_light[id]);
      if (k != kNoLight && b4.w > 0.f) {
        const DevLight L = sv.lights[k];
        const float *t9 = sv.tri9 + 9 * (size_t)id;
        const F3 A = f3(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2));
        const F3 B = f3(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5));
        const F3 C = f3(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8));
        const F3 nrm = cross_rn(C - A, B - A);
        const float len = length(nrm);
        const float cl = fabsf(dot(nrm, f3(rd.x, rd.y, rd.z))) / len;
        const float pl = nee_pdf(sv, select_prob(sv, none, k - sv.first_emit), L, id, t, 0.5f * len, cl);
        if (pl > 0.f && pl < 3.0e38f) wb = b4.w / (b4.w + pl);
      }
      add_px(accum, meta.x, mulc(beta, Le) * wb);
    }
    return false;
  }
  if (meta.w & 1u) return false;
  const Material M = material_of(mm);
  const F3 fcol = f3(mm.color[0], mm.color[1], mm.color[2]) * mm.reflectance;
  const uint64_t key = ckr_key(pc.seed, meta.x - pc.px_base);
  const F3 o_off = offset_origin(S.x, S.n);
  // ---- light technique: one sample ----
  {
    const float e0 = ckr_draw_f(key, ctr(meta.y, meta.z, 0)), e1 = ckr_draw_f(key, ctr(meta.y, meta.z, 1));
    const float e2 = ckr_draw_f(key, ctr(meta.y, meta.z, 2)), e3 = ckr_draw_f(key, ctr(meta.y, meta.z, 3));
    const uint32_t j = select_pick(sv, none, e0);
    const DevLight L = sv.lights[sv.first_emit + j];
    const uint32_t tri = L.first + cdf_pick(sv.pcdf + L.pcdf, L.count, e1);
    const float *t9 = sv.tri9 + 9 * (size_t)tri;
    const F3 A = f3(__ldg(t9), __ldg(t9 + 1), __ldg(t9 + 2));
    const F3 B = f3(__ldg(t9 + 3), __ldg(t9 + 4), __ldg(t9 + 5));
    const F3 C = f3(__ldg(t9 + 6), __ldg(t9 + 7), __ldg(t9 + 8));
    const F3 Pl = sample_triangle(A, B, C, e2, e3);
    const F3 dv = Pl - S.x;
    const float dist = length(dv);
    const F3 w = dv * (1.0f / dist);
    const float c = dot(w, S.n);
    const F3 nrm = cross_rn(C - A, B - A);
    const float len = length(nrm);
    const float cl = fabsf(dot(nrm, w)) / len;
    if (c > 0.f && cl > 0.f && len > 0.f && dist > 0.f) {
      const float pl = nee_pdf(sv, select_prob(sv, none, j), L, tri, dist, 0.5f * len, cl);
      const float f = brdf_eval(M, S.n, S.wo_ref, S.wo, w);
      if (pl > 0.f && f > 0.f) {
        const float pb = pdf_eval(M, S.n, S.wo_ref, S.wo, w);
        const F3 Le = mat_radiance(sv, sv.tri_mat[tri]);
        const float g = f * c / pl;
        const F3 contrib = mulc(beta, mulc(fcol, Le)) * (g * (pl / (pl + pb)));
        sh.n = 1;
        sh.o[0] = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
        sh.d[0] = shadow_dir(o_off, Pl);
        sh.c[0] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
      }
    }
  }
  // ---- BRDF technique: continues the path ----
  if (meta.z + 1 > pc.max_depth) return false;
  const float b0 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf));
  const float b1 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 1));
  const float b2 = ckr_draw_f(key, ctr(meta.y, meta.z, kDimBrdf + 2));
  const F3 wn = sample_brdf(M, S.n, S.wo_ref, S.wo, b0, b1, b2);
  const float cn = dot(wn, S.n);
  const float err = ckr_draw_f(key, ctr(meta.y, meta.z, kDimRR));
  if (!(cn > 0.f && err >= prm.rr_prob)) return false;
  const float pb = pdf_eval(M, S.n, S.wo_ref, S.wo, wn);
  const float f = brdf_eval(M, S.n, S.wo_ref, S.wo, wn);
  if (!(pb > 0.f && f > 0.f)) return false;
  const F3 nb = mulc(beta, fcol) * (f * cn / (pb * (1.0f - prm.rr_prob)));
  ro = make_float4(o_off.x, o_off.y, o_off.z, 0.f);
  rd = make_float4(wn.x, wn.y, wn.z, 3.0e38f);
  b4 = make_float4(nb.x, nb.y, nb.z, pb);
  const uint32_t nd = meta.z + 1;
  meta = make_uint4(meta.x, meta.y, nd, (meta.w & ~1u) | (nd >= pc.max_depth ? 1u : 0u));
  return true;
}

// Resident blocks of the persistent kernel: 512 / TPB (128 registers at 128
// threads, 16 warps per SM).
constexpr int persist_blocks(int tpb) { return 512 / tpb > 1 ? 512 / tpb : 1; }

// Renders the batch's paths [first, first + count) (global path indices; `next`
// counts from 0 and is zeroed before the launch).  Every lane of every warp runs
// the loop (the refill votes over full warps).
// LF: the light kinds compiled into the path vertex (kLightsMeshOnly for scenes whose
// lights are all MESH / TRI lights).
template <uint32_t SHADER, int TPB, uint32_t LF = kLightsAll>
__global__ void __launch_bounds__(TPB, persist_blocks(TPB))
    k_render_persistent(SceneView scene, ShadeView sv, Params prm, Paths P, uint64_t first, uint64_t count,
                        unsigned long long *next, int stack_depth) {
  extern __shared__ uint2 smem_trav[];
  uint2 *const stack = smem_trav + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u;
  float4 ro = make_float4(0, 0, 0, 0), rd = ro, b4 = ro;
  uint4 meta = make_uint4(0, 0, 0, 0);
  bool active = false, more = true;
  unsigned long long n_closest = 0, n_shadow = 0;
  LaneShadow sh;
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !active);
    if (more && idle) {
      const uint32_t want = (uint32_t)__popc(idle);
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(next, (unsigned long long)want);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + want >= count) more = false;
      if (!active) {
        const uint64_t g = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
        if (g < count) {
          camera_ray(Cam{}, prm, first + g, ro, rd, b4, meta);
          active = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) {
      if (!more) break;
      continue;
    }
    if (!active) continue;
    // Closest hit, the vertex, its shadow rays.
    float t = rd.w;
    const uint32_t id = trace_ray_rt(scene, make_ray(ro, rd), t, stack, TPB, stack_depth, false);
    ++n_closest;
    const uint32_t px = meta.x;
    active = SHADER == CKR_SHADER_PATH_NEE ? vertex_nee(sv, prm, P.accum, id, t, ro, rd, b4, meta, sh)
                                           : vertex_path<LF>(sv, prm, P.accum, id, t, ro, rd, b4, meta, sh);
    n_shadow += sh.n;
    for (uint32_t k = 0; k < sh.n; ++k) {
      float ts = sh.d[k].w;
      if (trace_ray_rt(scene, make_ray(sh.o[k], sh.d[k]), ts, stack, TPB, stack_depth, true) == kMiss)
        add_px(P.accum, px, f3(sh.c[k].x, sh.c[k].y, sh.c[k].z));
    }
  }
  // Ray statistics: closest-hit and shadow rays, one atomic per warp.
  for (int off = 16; off > 0; off >>= 1) {
    n_closest += __shfl_down_sync(0xffffffffu, n_closest, off);
    n_shadow += __shfl_down_sync(0xffffffffu, n_shadow, off);
  }
  if (lane == 0) {
    atomicAdd(&P.stats[0], n_closest);
    atomicAdd(&P.stats[1], n_shadow);
  }
}

}  // namespace
}  // namespace ckr
