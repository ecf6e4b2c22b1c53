// render.cu — wavefront renderer: camera rays -> closest hit -> shade (MIS light
// sampling, BRDF-sampled continuation) -> shadow rays -> FP64 accumulation.
//
// Paths live in up to `wave` path slots.  Each step runs three persistent kernels
// over device-side queues: k_extend (closest hit), k_shade (emits shadow rays and
// the continuation ray into queues whose slots are reserved once per warp: a
// warp-wide prefix sum of the per-lane counts and one atomicAdd by lane 31),
// k_shadow (any hit, adds unoccluded contributions).  Path tracers of more than
// one wave regenerate: a path that ends hands its slot to the next camera path,
// and the host stops on an empty queue.  Otherwise (direct-light shaders, single
// waves, inside stream capture) paths run in waves of one step per bounce, a
// fixed launch sequence with no host synchronisation (capturable in a CUDA graph).
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
#include "ckr_test.h"
#include "ltc_table.h"
#include "mlp.h"
#include "proposal.h"
#include "wavefront.cuh"

namespace ckr {
namespace {

constexpr int kRTPB = 128;  // block size of the single-render kernels

uint32_t mesh_lights_of(const ckr_scene *s) {
  uint32_t n = 0;
  for (const DevLight &L : s->host_lights) n += L.type == CKR_LIGHT_MESH;
  return n;
}

// Per triangle: the geometric normal and the material index, which a surface hit
// needs (make_surface) -- one 16-byte load instead of nine vertex loads and a
// dependent material load.
__global__ void k_tri_nm(const float *__restrict__ tri9, const uint32_t *__restrict__ tri_mat, uint32_t ntri,
                         float4 *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntri) return;
  const float *t9 = tri9 + 9 * (size_t)i;
  const F3 A = f3(t9[0], t9[1], t9[2]), B = f3(t9[3], t9[4], t9[5]), C = f3(t9[6], t9[7], t9[8]);
  const F3 n = normalize(cross_rn(C - A, B - A));
  out[i] = make_float4(n.x, n.y, n.z, __uint_as_float(tri_mat[i]));
}

struct Workspace {
  DevBuf<float4> ray_o, ray_d, beta, sh_o, sh_d, sh_c;
  DevBuf<uint4> meta;
  DevBuf<uint32_t> hit_id, q0, q1, sh_px, counts;
  DevBuf<unsigned long long> stats;
  DevBuf<float> hit_t;
  DevBuf<double> accum;
  size_t wave = 0, shadow = 0, pixels = 0;
  uint32_t *h_count = nullptr;  // pinned: queue lengths read back under regeneration
  cudaEvent_t ev[2] = {nullptr, nullptr};
  Workspace() = default;
  Workspace(const Workspace &) = delete;
  Workspace &operator=(const Workspace &) = delete;
  ~Workspace() {
    if (h_count) cudaFreeHost(h_count);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
};


}  // namespace
}  // namespace ckr

using namespace ckr;

namespace {
void free_ws(void *p) { delete static_cast<Workspace *>(p); }
}  // namespace

namespace {

int render_impl(ckr_scene *s, ckr_proposal *prop, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb,
                double *accum, void *stream_, const ckr_ray *rays = nullptr) {
  if (!s || !cam || !cfg || !rgb || cam->width == 0 || cam->height == 0 || cfg->spp == 0 || cfg->shader > 5)
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
  Params prm{};
  prm.shader = cfg->shader;
  prm.spp = cfg->spp;
  const bool path = cfg->shader == CKR_SHADER_PATH || cfg->shader == CKR_SHADER_PATH_NEE ||
                    cfg->shader == CKR_SHADER_EXPLICIT;
  if (cfg->shader == CKR_SHADER_PATH_NEE && s->n_emit == 0) return CKR_ERR_INVALID_ARGUMENT;
  prm.max_depth = path ? std::max(1u, cfg->max_depth) : 1u;
  prm.n_light = cfg->n_light_samples;
  prm.n_brdf = path && cfg->shader != CKR_SHADER_EXPLICIT ? 1u : cfg->n_brdf_samples;
  prm.rr_prob = path ? cfg->rr_prob : 0.f;
  prm.seed = cfg->seed;
  prm.npix = cam->width * cam->height;
  prm.rays = reinterpret_cast<const float4 *>(rays);
  uint32_t area_lights = 0, point_lights = 0;
  for (const DevLight &L : s->host_lights) (L.type == CKR_LIGHT_POINT ? point_lights : area_lights)++;
  uint32_t per_path = cfg->shader == CKR_SHADER_PATH_NEE
                          ? 1u
                          : point_lights + area_lights * prm.n_light + (cfg->shader == CKR_SHADER_DIRECT_MIS ? prm.n_brdf : 0) +
                                (cfg->shader == CKR_SHADER_DIRECT_MIS || cfg->shader == CKR_SHADER_PATH ? s->env_n : 0);
  if (cfg->shader == CKR_SHADER_DIRECT_CV) per_path = mesh_lights_of(s) * prm.n_light;
  if (cfg->shader == CKR_SHADER_EXPLICIT) per_path = 0;  // the MISCV direct term traces no shadow rays
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
  CKR_CUDA_TRY(W.counts.reserve(8));
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
  P.sh_cap = (uint32_t)std::min<size_t>(shadow, 0xFFFFFFFFu);
  P.status = s->status.ptr;
  if (s->test_shadow_cap) {
    P.sh_cap = std::min(P.sh_cap, s->test_shadow_cap);
    s->test_shadow_cap = 0;
  }
  bool train = prop && prop->train && (!prop->max_steps || prop->net.step < prop->max_steps);
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  CKR_CUDA_TRY(cudaStreamIsCapturing(stream, &capture));
  // Training overlaps rendering outside stream capture (see ckr_proposal).
  const bool overlap = train && capture == cudaStreamCaptureStatusNone;
  bool pending[2] = {false, false};  // a training whose `done` event the stream has not waited for
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
  if (overlap) {
    if (!prop->train_stream) {
      // Highest priority: the training CTAs take SMs as the renderer's blocks retire.
      int lo = 0, hi = 0;
      CKR_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      CKR_CUDA_TRY(cudaStreamCreateWithPriority(&prop->train_stream, cudaStreamNonBlocking, hi));
    }
    for (int b = 0; b < 2; ++b) {
      if (!prop->rec_ready[b]) CKR_CUDA_TRY(cudaEventCreateWithFlags(&prop->rec_ready[b], cudaEventDisableTiming));
      if (!prop->done[b]) CKR_CUDA_TRY(cudaEventCreateWithFlags(&prop->done[b], cudaEventDisableTiming));
      CKR_CUDA_TRY(prop->rec_k[b].reserve(3 * (size_t)prop->batch));
      CKR_CUDA_TRY(prop->rec_count_k[b].reserve(1));
      CKR_CUDA_TRY(prop->img_pub[b].reserve(mlp::kImgBytes));
      CKR_CUDA_TRY(cudaMemsetAsync(prop->rec_count_k[b].ptr, 0, 4, stream));
      CKR_CUDA_TRY(cudaMemcpyAsync(prop->img_pub[b].ptr, prop->net.img, mlp::kImgBytes, cudaMemcpyDeviceToDevice,
                                   stream));
    }
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
  size_t smem = (size_t)depth * kRTPB * sizeof(uint2);
  smem += shear_smem_bytes(kRTPB);  // the triangle test's ray data (dynamic fetching)
  // Deep trees: dynamic fetching; one or two levels: one ray per thread.
  const bool dyn = s->max_depth >= kDynamicDepth;
  void (*const extend_fn)(SceneView, Paths, int, int) = dyn ? k_extend<kRTPB, true> : k_extend<kRTPB, false>;
  void (*const shadow_fn)(SceneView, Paths, int, int, float4 *) =
      dyn ? k_shadow<kRTPB, true> : k_shadow<kRTPB, false>;
  if (smem > 48 * 1024) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(extend_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CKR_CUDA_TRY(cudaFuncSetAttribute(shadow_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int g_ext = grid_for((const void *)extend_fn, smem, kRTPB);
  const int g_sh = grid_for((const void *)shadow_fn, smem, kRTPB);
  if (cfg->shader == CKR_SHADER_EXPLICIT && smem > 48 * 1024)
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_shade<CKR_SHADER_EXPLICIT, kRTPB>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // The path shader without the code of light kinds the scene does not have.
  void (*const path_fn)(ShadeView, Paths, Params, int, int, const LtcEntry *) =
      mesh_lights_only(s) ? k_shade_path<kRTPB, kLightsMeshOnly> : k_shade_path<kRTPB, kLightsAll>;
  const void *shade_fn = cfg->shader == CKR_SHADER_EXPLICIT ? (const void *)k_shade<CKR_SHADER_EXPLICIT, kRTPB>
                         : cfg->shader == CKR_SHADER_PATH_NEE ? (const void *)k_shade_nee<kRTPB>
                         : cfg->shader == CKR_SHADER_PATH      ? (const void *)path_fn
                         : cfg->shader == CKR_SHADER_DIRECT_CV  ? (const void *)k_shade<CKR_SHADER_DIRECT_CV, kRTPB>
                         : cfg->shader == CKR_SHADER_DIRECT_MIS ? (const void *)k_shade<CKR_SHADER_DIRECT_MIS, kRTPB>
                                                                : (const void *)k_shade_miscv<kRTPB>;
  const int g_shade = grid_for(shade_fn, cfg->shader == CKR_SHADER_EXPLICIT ? smem : 0, kRTPB);
  // One step of the wavefront over queue `cur`: closest hit, [learned selection],
  // shading, shadow rays, [training].  k: the step's index within the wave (or the
  // render, with regeneration) -- it picks the selection buffer, and k = 0 has no
  // previous one; nee: the step's vertices may draw light samples.
  int cur = 0;
  auto step = [&](uint64_t k, bool nee) -> int {
    // Work counters of k_extend and k_shadow (P.counts[3], [4]).
    CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 3, 0, 2 * sizeof(uint32_t), stream));
    extend_fn<<<g_ext, kRTPB, smem, stream>>>(sv, P, cur, depth);
    CKR_CUDA_TRY(cudaMemsetAsync(P.counts + (cur ^ 1), 0, sizeof(uint32_t), stream));
    CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 2, 0, sizeof(uint32_t), stream));
    Learn lr{};
    if (prop) lr.sel_prev = k ? prop->sel[(k - 1) & 1].ptr : nullptr;
    // Overlapped training: this step uses record buffer and weight copy b, which the
    // training of step k - 2 used and wrote; wait for it.  Once training has
    // stopped, every pending training is waited for and the final weights used.
    const int b = (int)(k & 1);
    const uint8_t *img = nullptr;
    float4 *rec = prop ? prop->rec.ptr : nullptr;
    uint32_t *rec_count = prop ? prop->rec_count.ptr : nullptr;
    if (overlap) {
      for (int i = 0; i < 2; ++i)
        if (pending[i] && (i == b || !train)) {
          CKR_CUDA_TRY(cudaStreamWaitEvent(stream, prop->done[i], 0));
          pending[i] = false;
        }
      if (train) {
        img = prop->img_pub[b].ptr;
        rec = prop->rec_k[b].ptr;
        rec_count = prop->rec_count_k[b].ptr;
      }
    }
    if (prop && nee) {
      // Light distributions at this step's vertices.
      mlp::PathRows pr;
      pr.queue = cur ? P.q1 : P.q0;
      pr.hit_id = P.hit_id;
      pr.ray_o = P.ray_o;
      pr.ray_d = P.ray_d;
      pr.hit_t = P.hit_t;
      pr.meta = P.meta;
      pr.sv = shv;
      int ms = mlp::infer_paths(prop->net, pr, (uint32_t)wave, P.counts + cur, prop->sel[k & 1].ptr,
                                prop->defensive, stream, img);
      if (ms != CKR_OK) return ms;
      lr.sel = prop->sel[k & 1].ptr;
      if (train) {
        lr.rec = rec;
        lr.rec_count = rec_count;
        lr.rec_cap = prop->batch;
      }
    }
    const int d = (int)std::min<uint64_t>(k, prm.max_depth);
    if (cfg->shader == CKR_SHADER_EXPLICIT)
      k_shade<CKR_SHADER_EXPLICIT, kRTPB><<<g_shade, kRTPB, smem, stream>>>(shv, P, prm, cur, d, ltc, sv, depth);
    else if (cfg->shader == CKR_SHADER_PATH_NEE)
      k_shade_nee<kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, lr);
    else if (cfg->shader == CKR_SHADER_PATH)
      path_fn<<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, d, ltc);
    else if (cfg->shader == CKR_SHADER_DIRECT_CV)
      k_shade<CKR_SHADER_DIRECT_CV, kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, d, ltc);
    else if (cfg->shader == CKR_SHADER_DIRECT_MIS)
      k_shade<CKR_SHADER_DIRECT_MIS, kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, d, ltc);
    else
      k_shade_miscv<kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, d, ltc);
    shadow_fn<<<g_sh, kRTPB, smem, stream>>>(sv, P, depth, cur, train && nee ? rec : nullptr);
    if (train && nee) {
      // Adam steps on this step's light samples (visibility applied above),
      // minibatch by minibatch; steps past the records actually written are no-ops.
      // Overlapped: on the training stream once the records are complete, then the
      // new weights are published for step k + 2.
      cudaStream_t ts_stream = stream;
      if (overlap) {
        CKR_CUDA_TRY(cudaEventRecord(prop->rec_ready[b], stream));
        CKR_CUDA_TRY(cudaStreamWaitEvent(prop->train_stream, prop->rec_ready[b], 0));
        ts_stream = prop->train_stream;
      }
      for (uint32_t off = 0; off < prop->batch; off += prop->minibatch) {
        int ts = mlp::train_step(prop->net, rec + 3 * (size_t)off, std::min(prop->minibatch, prop->batch - off),
                                 rec_count, off, ts_stream);
        if (ts != CKR_OK) return ts;
      }
      CKR_CUDA_TRY(cudaMemsetAsync(rec_count, 0, 4, ts_stream));
      if (overlap) {
        CKR_CUDA_TRY(cudaMemcpyAsync(prop->img_pub[b].ptr, prop->net.img, mlp::kImgBytes, cudaMemcpyDeviceToDevice,
                                     ts_stream));
        CKR_CUDA_TRY(cudaEventRecord(prop->done[b], ts_stream));
        pending[b] = true;
      }
      if (prop->max_steps && prop->net.step >= prop->max_steps) train = false;  // converged: inference only
    }
    cur ^= 1;
    return CKR_OK;
  };
  // Path regeneration for path tracers of more than one wave (outside stream
  // capture, whose launch sequence must be fixed): one wave of slots, and a
  // shading step that ends a path starts the next camera path in its slot, so
  // every step runs a full queue until the last paths have started.  The host
  // stops when the queue is empty, reading its length one step behind so that the
  // device always has the next step queued.  It pays where traversal is long
  // (trees of kDynamicDepth levels or more: many-light frame 0.364 -> 0.312 s);
  // on shallow trees a step is short and mixing camera rays with bounce rays in
  // one queue costs more than the drained waves' tails (box, 1024^2 x 64 spp:
  // 111 ms against 98 ms with waves), so those keep the waves.
  const bool regen = (cfg->shader == CKR_SHADER_PATH || cfg->shader == CKR_SHADER_PATH_NEE) && total > wave &&
                     dyn && capture == cudaStreamCaptureStatusNone && total + 64ull * wave < (1ull << 32);
  if (regen) {
    if (!W.h_count) CKR_CUDA_TRY(cudaMallocHost((void **)&W.h_count, 2 * sizeof(uint32_t)));
    for (cudaEvent_t &e : W.ev)
      if (!e) CKR_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    prm.regen_total = (uint32_t)total;
    prm.cam = c;
    k_camera<kRTPB><<<std::min<int>(g_ext, ceil_div(wave, kRTPB)), kRTPB, 0, stream>>>(c, P, prm, 0, (uint32_t)wave);
    // While paths start, every step runs `wave` vertices, and a path has at most
    // max_depth + 1: a bound on the steps in case the read-back never sees zero.
    const uint64_t max_steps = ceil_div(total, wave) * (uint64_t)(prm.max_depth + 1) + prm.max_depth + 2;
    for (uint64_t k = 0; k < max_steps; ++k) {
      int st = step(k, true);
      if (st != CKR_OK) return st;
      CKR_CUDA_TRY(cudaMemcpyAsync(W.h_count + (k & 1), P.counts + cur, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                   stream));
      CKR_CUDA_TRY(cudaEventRecord(W.ev[k & 1], stream));
      if (k >= 1) {
        CKR_CUDA_TRY(cudaEventSynchronize(W.ev[(k - 1) & 1]));
        if (W.h_count[(k - 1) & 1] == 0) break;
      }
    }
  } else {
    for (uint64_t base = 0; base < total; base += wave) {
      uint32_t n = (uint32_t)std::min<uint64_t>(wave, total - base);
      k_camera<kRTPB><<<std::min<int>(g_ext, ceil_div(n, kRTPB)), kRTPB, 0, stream>>>(c, P, prm, base, n);
      cur = 0;
      for (uint32_t d = 0; d <= prm.max_depth; ++d) {
        // The vertices at the last depth only add emission: no light sample, so
        // neither a light distribution nor training records there.
        int st = step(d, d < prm.max_depth);
        if (st != CKR_OK) return st;
        if (!path) break;
      }
    }
  }
  // The render completes (on `stream`) after its trainings.
  for (int i = 0; i < 2; ++i)
    if (pending[i]) CKR_CUDA_TRY(cudaStreamWaitEvent(stream, prop->done[i], 0));
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

extern "C" int ckr_shade_rays(ckr_scene *s, const ckr_ray *rays, uint32_t n, const ckr_render_cfg *cfg, float *rgb,
                              void *stream) {
  if (!s || !rays || !cfg || !rgb || n == 0 || (reinterpret_cast<uintptr_t>(rays) & 15u))
    return CKR_ERR_INVALID_ARGUMENT;
  ckr_camera cam{};
  cam.width = n;  // one output row per ray: key (seed, i), pixel i of an n x 1 image
  cam.height = 1;
  return render_impl(s, nullptr, &cam, cfg, rgb, nullptr, stream, rays);
}

extern "C" int ckr_shade_rays_host(ckr_scene *s, const ckr_ray *rays, uint32_t n, const ckr_render_cfg *cfg,
                                   float *rgb, void *stream) {
  if (!s || !rays || !cfg || !rgb || n == 0) return CKR_ERR_INVALID_ARGUMENT;
  cudaStream_t st_ = (cudaStream_t)stream;
  ckr_ray *d_rays = nullptr;
  float *d_rgb = nullptr;
  CKR_CUDA_TRY(cudaMalloc((void **)&d_rays, n * sizeof(ckr_ray)));
  int st = CKR_OK;
  if (cudaMalloc((void **)&d_rgb, 3 * sizeof(float) * (size_t)n) != cudaSuccess) st = CKR_ERR_OUT_OF_MEMORY;
  if (st == CKR_OK &&
      cudaMemcpyAsync(d_rays, rays, n * sizeof(ckr_ray), cudaMemcpyHostToDevice, st_) != cudaSuccess)
    st = CKR_ERR_CUDA;
  if (st == CKR_OK) st = ckr_shade_rays(s, d_rays, n, cfg, d_rgb, stream);
  if (st == CKR_OK) {
    cudaError_t e = cudaMemcpyAsync(rgb, d_rgb, 3 * sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) st = CKR_ERR_CUDA;
  }
  cudaFree(d_rays);
  cudaFree(d_rgb);
  if (st == CKR_OK) {
    int h = ckr_scene_check(s, stream);
    if (h != 0) st = h;
  }
  return st;
}

extern "C" int ckr_internal_limit_shadow_queue(ckr_scene *s, uint32_t capacity) {
  if (!s || capacity == 0) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->host_mu);
  s->test_shadow_cap = capacity;
  return CKR_OK;
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
// For callers that cannot call cudaMalloc while they render: renderers embedded
// in a host application whose device memory comes only from the host's own pool,
// frame loops that cannot afford the device-wide synchronisation an allocation
// or a free may cause, and processes so close to the memory limit that an
// allocation in the middle of a frame could fail.  ckr_render_noalloc runs the same kernels as ckr_render,
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
  if (!s || !cam || !cfg || !rgb || cam->width == 0 || cam->height == 0 || cfg->spp == 0 || cfg->shader > 5)
    return CKR_ERR_INVALID_ARGUMENT;
  if (!s->has_shading) return CKR_ERR_INVALID_ARGUMENT;
  if (cfg->max_depth > 60 || cfg->spp > 65536 || cfg->n_light_samples > 256 || cfg->n_brdf_samples > 256)
    return CKR_ERR_TOO_LARGE;
  if ((uint64_t)cam->width * cam->height > kNoAllocMaxPixels) return CKR_ERR_TOO_LARGE;
  cudaStream_t stream = (cudaStream_t)stream_;
  std::lock_guard<std::mutex> scene_lock(s->host_mu);
  int dev = 0;
  CKR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return CKR_ERR_INVALID_ARGUMENT;
  int st = noalloc_setup(dev);
  if (st != CKR_OK) return st;
  Params prm{};
  prm.shader = cfg->shader;
  prm.spp = cfg->spp;
  const bool path = cfg->shader == CKR_SHADER_PATH || cfg->shader == CKR_SHADER_PATH_NEE ||
                    cfg->shader == CKR_SHADER_EXPLICIT;
  if (cfg->shader == CKR_SHADER_PATH_NEE && s->n_emit == 0) return CKR_ERR_INVALID_ARGUMENT;
  prm.max_depth = path ? std::max(1u, cfg->max_depth) : 1u;
  prm.n_light = cfg->n_light_samples;
  prm.n_brdf = path && cfg->shader != CKR_SHADER_EXPLICIT ? 1u : cfg->n_brdf_samples;
  prm.rr_prob = path ? cfg->rr_prob : 0.f;
  prm.seed = cfg->seed;
  prm.npix = cam->width * cam->height;
  uint32_t area_lights = 0, point_lights = 0;
  for (const DevLight &L : s->host_lights) (L.type == CKR_LIGHT_POINT ? point_lights : area_lights)++;
  uint64_t per_path = cfg->shader == CKR_SHADER_PATH_NEE
                          ? 1u
                          : (uint64_t)point_lights + (uint64_t)area_lights * prm.n_light +
                                (cfg->shader == CKR_SHADER_DIRECT_MIS ? prm.n_brdf : 0) +
                                (cfg->shader == CKR_SHADER_DIRECT_MIS || cfg->shader == CKR_SHADER_PATH ? s->env_n : 0);
  if (cfg->shader == CKR_SHADER_DIRECT_CV) per_path = (uint64_t)mesh_lights_of(s) * prm.n_light;
  if (cfg->shader == CKR_SHADER_EXPLICIT) per_path = 0;  // the MISCV direct term traces no shadow rays
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
  P.counts = reinterpret_cast<uint32_t *>(take(32));
  P.stats = reinterpret_cast<unsigned long long *>(take(16));
  P.accum = reinterpret_cast<double *>(take(24ull * kNoAllocMaxPixels));
  P.sh_cap = kNoAllocShadow;
  P.status = s->status.ptr;
  // The arena keeps the previous call's contents: clear what must start at zero.
  CKR_CUDA_TRY(cudaMemsetAsync(P.counts, 0, 32, stream));
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
  size_t smem = (size_t)depth * kRTPB * sizeof(uint2);
  smem += shear_smem_bytes(kRTPB);  // the triangle test's ray data (dynamic fetching)
  // Deep trees: dynamic fetching; one or two levels: one ray per thread.
  const bool dyn = s->max_depth >= kDynamicDepth;
  void (*const extend_fn)(SceneView, Paths, int, int) = dyn ? k_extend<kRTPB, true> : k_extend<kRTPB, false>;
  void (*const shadow_fn)(SceneView, Paths, int, int, float4 *) =
      dyn ? k_shadow<kRTPB, true> : k_shadow<kRTPB, false>;
  if (smem > 48 * 1024) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(extend_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CKR_CUDA_TRY(cudaFuncSetAttribute(shadow_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int g_ext = grid_for((const void *)extend_fn, smem, kRTPB);
  const int g_sh = grid_for((const void *)shadow_fn, smem, kRTPB);
  if (cfg->shader == CKR_SHADER_EXPLICIT && smem > 48 * 1024)
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_shade<CKR_SHADER_EXPLICIT, kRTPB>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // The path shader without the code of light kinds the scene does not have.
  void (*const path_fn)(ShadeView, Paths, Params, int, int, const LtcEntry *) =
      mesh_lights_only(s) ? k_shade_path<kRTPB, kLightsMeshOnly> : k_shade_path<kRTPB, kLightsAll>;
  const void *shade_fn = cfg->shader == CKR_SHADER_EXPLICIT ? (const void *)k_shade<CKR_SHADER_EXPLICIT, kRTPB>
                         : cfg->shader == CKR_SHADER_PATH_NEE ? (const void *)k_shade_nee<kRTPB>
                         : cfg->shader == CKR_SHADER_PATH      ? (const void *)path_fn
                         : cfg->shader == CKR_SHADER_DIRECT_CV  ? (const void *)k_shade<CKR_SHADER_DIRECT_CV, kRTPB>
                         : cfg->shader == CKR_SHADER_DIRECT_MIS ? (const void *)k_shade<CKR_SHADER_DIRECT_MIS, kRTPB>
                                                                : (const void *)k_shade_miscv<kRTPB>;
  const int g_shade = grid_for(shade_fn, cfg->shader == CKR_SHADER_EXPLICIT ? smem : 0, kRTPB);
  for (uint64_t base = 0; base < total; base += wave) {
    uint32_t n = (uint32_t)std::min<uint64_t>(wave, total - base);
    k_camera<kRTPB><<<std::min<int>(g_ext, ceil_div(n, kRTPB)), kRTPB, 0, stream>>>(c, P, prm, base, n);
    int cur = 0;
    for (uint32_t d = 0; d <= prm.max_depth; ++d) {
      // Work counters of k_extend and k_shadow (P.counts[3], [4]).
      CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 3, 0, 2 * sizeof(uint32_t), stream));
      extend_fn<<<g_ext, kRTPB, smem, stream>>>(sv, P, cur, depth);
      CKR_CUDA_TRY(cudaMemsetAsync(P.counts + (cur ^ 1), 0, sizeof(uint32_t), stream));
      CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 2, 0, sizeof(uint32_t), stream));
      if (cfg->shader == CKR_SHADER_EXPLICIT)
        k_shade<CKR_SHADER_EXPLICIT, kRTPB><<<g_shade, kRTPB, smem, stream>>>(shv, P, prm, cur, (int)d, ltc, sv,
                                                                              depth);
      else if (cfg->shader == CKR_SHADER_PATH_NEE)
        k_shade_nee<kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, Learn{});
      else if (cfg->shader == CKR_SHADER_PATH)
        path_fn<<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      else if (cfg->shader == CKR_SHADER_DIRECT_CV)
        k_shade<CKR_SHADER_DIRECT_CV, kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      else if (cfg->shader == CKR_SHADER_DIRECT_MIS)
        k_shade<CKR_SHADER_DIRECT_MIS, kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      else
        k_shade_miscv<kRTPB><<<g_shade, kRTPB, 0, stream>>>(shv, P, prm, cur, (int)d, ltc);
      shadow_fn<<<g_sh, kRTPB, smem, stream>>>(sv, P, depth, cur, nullptr);
      cur ^= 1;
      if (!path) break;
    }
  }
  uint32_t n3 = prm.npix * 3;
  k_resolve<<<std::min<unsigned>(1024, ceil_div(n3, 256)), 256, 0, stream>>>(P.accum, rgb, n3, 1.0 / prm.spp);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}

namespace ckr {
int build_tri_nm(ckr_scene *s) {
  if (s->ntri == 0) return CKR_OK;
  CKR_CUDA_TRY(s->tri_nm.reserve(s->ntri));
  k_tri_nm<<<ceil_div(s->ntri, 256), 256>>>(s->tri9.ptr, s->tri_mat.ptr, s->ntri, s->tri_nm.ptr);
  CKR_CUDA_TRY(cudaGetLastError());
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  return CKR_OK;
}
}  // namespace ckr
