// batch.cu — batched rendering: many jobs of uneven resolution, spp and depth in
// one pass, captured as a CUDA graph, with an autotuner for the renderer, the
// block size and the number of paths in flight.
//
// Paths of all jobs are numbered consecutively (job by job, sample-major inside a
// job); a path finds its job by binary search over the jobs' first path indices
// and carries it in meta.w >> 8, so shading picks the job's materials, seed and
// depth.  Two renderers:
//  - persistent (persistent.cuh): one launch of a persistent grid whose lanes
//    each run a path's whole bounce loop and take the next path of the batch when
//    theirs ends; the graph is a memset of the sums and the counter, that launch
//    and the resolve;
//  - wavefront (wavefront.cuh): waves of paths that cross job boundaries, three
//    launches per bounce over device-side queues; a fixed launch sequence.
// The pass is captured once with stream capture and replayed with cudaGraphLaunch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <vector>

#include "ckr_test.h"
#include "persistent.cuh"
#include "scene.h"

namespace ckr {
namespace {

// Test hook (ckr_internal_batch_workspace_cap): wave workspaces larger than this
// many bytes fail as if device memory had run out; 0 = no cap.
std::atomic<size_t> g_test_ws_cap{0};

struct BatchWs {
  DevBuf<float4> ray_o, ray_d, beta, sh_o, sh_d, sh_c;
  DevBuf<uint4> meta;
  DevBuf<uint32_t> hit_id, q0, q1, sh_px, counts;
  DevBuf<unsigned long long> stats;
  DevBuf<float> hit_t;
  size_t wave = 0, shadow = 0;
  // Frees the per-wave buffers (after a reserve that did not fit, so that a smaller
  // wave is tried against all of device memory).
  void release_waves() {
    ray_o.release(), ray_d.release(), beta.release(), meta.release(), hit_id.release(), hit_t.release();
    q0.release(), q1.release(), sh_o.release(), sh_d.release(), sh_c.release(), sh_px.release();
    wave = shadow = 0;
  }
  // Bytes of the per-wave buffers for `w` paths: path state 72 B a path (ray_o,
  // ray_d, beta, meta, hit_id, hit_t, two queue entries), shadow rays 52 B each.
  static size_t bytes_for(size_t w, size_t per_path) { return 72 * w + 52 * w * per_path; }
  int reserve(size_t w, size_t per_path) {
    size_t sh = w * per_path;
    const size_t cap = g_test_ws_cap.load();
    if (cap && bytes_for(w, per_path) > cap) return CKR_ERR_OUT_OF_MEMORY;
    if (ray_o.reserve(w) || ray_d.reserve(w) || beta.reserve(w) || meta.reserve(w) || hit_id.reserve(w) ||
        hit_t.reserve(w) || q0.reserve(w) || q1.reserve(w) || sh_o.reserve(sh) || sh_d.reserve(sh) ||
        sh_c.reserve(sh) || sh_px.reserve(sh) || counts.reserve(8) || stats.reserve(2))
      return CKR_ERR_OUT_OF_MEMORY;
    wave = w;
    shadow = sh;
    return CKR_OK;
  }
  Paths paths(double *accum) {
    Paths P{};
    P.ray_o = ray_o.ptr; P.ray_d = ray_d.ptr; P.beta = beta.ptr; P.meta = meta.ptr;
    P.hit_id = hit_id.ptr; P.hit_t = hit_t.ptr; P.q0 = q0.ptr; P.q1 = q1.ptr;
    P.sh_o = sh_o.ptr; P.sh_d = sh_d.ptr; P.sh_c = sh_c.ptr; P.sh_px = sh_px.ptr;
    P.counts = counts.ptr;
    P.stats = stats.ptr;
    P.accum = accum;
    P.sh_cap = (uint32_t)std::min<size_t>(shadow, 0xFFFFFFFFu);
    return P;
  }
};

Cam cam_of(const ckr_camera &c) {
  Cam k;
  k.pos = f3(c.pos[0], c.pos[1], c.pos[2]);
  k.dir = f3(c.dir[0], c.dir[1], c.dir[2]);
  k.cx = f3(c.cx[0], c.cx[1], c.cx[2]);
  k.cy = f3(c.cy[0], c.cy[1], c.cy[2]);
  k.w = c.width;
  k.h = c.height;
  return k;
}

// A job list on the device plus the host copy the launch sequence is built from.
struct JobSet {
  std::vector<JobDev> host;
  DevBuf<JobDev> dev;
  uint64_t paths = 0;
  uint32_t pixels = 0;
  int build(const ckr_job *jobs, uint32_t njobs, uint32_t nmat, uint32_t spp_cap, float *const *rgb_override) {
    host.resize(njobs);
    paths = 0;
    pixels = 0;
    for (uint32_t j = 0; j < njobs; ++j) {
      JobDev &J = host[j];
      J.cam = cam_of(jobs[j].cam);
      J.npix = jobs[j].cam.width * jobs[j].cam.height;
      J.spp = spp_cap ? std::min(jobs[j].spp, spp_cap) : jobs[j].spp;
      J.max_depth = std::max(1u, jobs[j].max_depth);
      J.mat_off = jobs[j].material_set * nmat;
      J.seed = jobs[j].seed;
      J.path_begin = paths;
      J.accum_off = pixels;
      J.rgb = rgb_override ? rgb_override[j] : jobs[j].rgb;
      paths += (uint64_t)J.npix * J.spp;
      pixels += J.npix;
    }
    if (dev.reserve(njobs) != cudaSuccess) return CKR_ERR_OUT_OF_MEMORY;
    CKR_CUDA_TRY(cudaMemcpy(dev.ptr, host.data(), njobs * sizeof(JobDev), cudaMemcpyHostToDevice));
    return CKR_OK;
  }
};

// Deepest job among the paths [a, b).
uint32_t depth_of_range(const std::vector<JobDev> &jobs, uint64_t a, uint64_t b) {
  uint32_t d = 1;
  for (const JobDev &J : jobs) {
    uint64_t e = J.path_begin + (uint64_t)J.npix * J.spp;
    if (J.path_begin < b && e > a) d = std::max(d, J.max_depth);
  }
  return d;
}

}  // namespace
}  // namespace ckr

using namespace ckr;

struct ckr_batch {
  ckr_scene *scene = nullptr;
  DevBuf<unsigned long long> next;  // path counter of the persistent renderer
  uint32_t shader = CKR_SHADER_PATH, n_light = 1;
  float rr_prob = 0.3f;
  uint32_t nmat = 0, nsets = 0;
  DevBuf<ckr_material> mats;
  JobSet jobs;
  std::vector<ckr_job> job_in;
  BatchWs ws;
  DevBuf<double> accum;
  ckr_batch_tuning tuning{};
  uint32_t per_path = 1;
  bool persistent_ok = false;  // shadow rays per vertex fit the persistent kernel's lanes
  uint32_t launches = 0;
  cudaStream_t capture = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~ckr_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (capture) cudaStreamDestroy(capture);
  }
};

namespace {

// Enqueues one render of `set` on `stream`: waves over [first, last) path ranges;
// `pack` = waves cross job boundaries (else each job has its own waves).
template <int TPB>
int enqueue(ckr_batch *b, JobSet &set, bool pack, size_t wave, cudaStream_t stream, uint32_t *launches) {
  ckr_scene *s = b->scene;
  const int depth = (int)stack_depth_of(s);
  size_t smem = (size_t)depth * TPB * sizeof(uint2);
  smem += shear_smem_bytes(TPB);  // the triangle test's ray data (dynamic fetching)
  // Deep trees: dynamic fetching; one or two levels: one ray per thread.
  const bool dyn = s->max_depth >= kDynamicDepth;
  void (*const extend_fn)(SceneView, Paths, int, int) = dyn ? k_extend<TPB, true> : k_extend<TPB, false>;
  void (*const shadow_fn)(SceneView, Paths, int, int, float4 *) =
      dyn ? k_shadow<TPB, true> : k_shadow<TPB, false>;
  if (smem > 48 * 1024) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(extend_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CKR_CUDA_TRY(cudaFuncSetAttribute(shadow_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int g_ext = grid_for((const void *)extend_fn, smem, TPB);
  const int g_sh = grid_for((const void *)shadow_fn, smem, TPB);
  const bool nee = b->shader == CKR_SHADER_PATH_NEE;
  void (*const path_fn)(ShadeView, Paths, Params, int, int, const LtcEntry *) =
      mesh_lights_only(s) ? k_shade_path<TPB, kLightsMeshOnly> : k_shade_path<TPB, kLightsAll>;
  const int g_shade = grid_for(nee ? (const void *)k_shade_nee<TPB> : (const void *)path_fn, 0, TPB);
  Params prm{};
  prm.shader = b->shader;
  prm.n_light = b->n_light;
  prm.n_brdf = 1;
  prm.rr_prob = b->rr_prob;
  prm.shadow_per_path = b->per_path;
  prm.jobs = set.dev.ptr;
  prm.njobs = (uint32_t)set.host.size();
  prm.spp = 1;
  prm.npix = 1;
  SceneView sv = view_of(s);
  ShadeView shv = shade_view_of(s);
  shv.mats = b->mats.ptr;
  Paths P = b->ws.paths(b->accum.ptr);
  P.status = b->scene->status.ptr;
  uint32_t n_launch = 0;
  CKR_CUDA_TRY(cudaMemsetAsync(b->accum.ptr, 0, sizeof(double) * 3 * (size_t)set.pixels, stream));
  // Path ranges: the whole batch, or one range per job.
  std::vector<std::pair<uint64_t, uint64_t>> ranges;
  if (pack) {
    ranges.push_back({0, set.paths});
  } else {
    for (const JobDev &J : set.host) ranges.push_back({J.path_begin, J.path_begin + (uint64_t)J.npix * J.spp});
  }
  for (auto [first, last] : ranges) {
    for (uint64_t base = first; base < last; base += wave) {
      const uint32_t n = (uint32_t)std::min<uint64_t>(wave, last - base);
      const uint32_t dmax = depth_of_range(set.host, base, base + n);
      k_camera<TPB><<<std::min<int>(g_ext, ceil_div(n, TPB)), TPB, 0, stream>>>(Cam{}, P, prm, base, n);
      ++n_launch;
      int cur = 0;
      for (uint32_t d = 0; d <= dmax; ++d) {
        // Work counters of k_extend and k_shadow (P.counts[3], [4]).
        CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 3, 0, 2 * sizeof(uint32_t), stream));
        extend_fn<<<g_ext, TPB, smem, stream>>>(sv, P, cur, depth);
        CKR_CUDA_TRY(cudaMemsetAsync(P.counts + (cur ^ 1), 0, sizeof(uint32_t), stream));
        CKR_CUDA_TRY(cudaMemsetAsync(P.counts + 2, 0, sizeof(uint32_t), stream));
        if (nee) k_shade_nee<TPB><<<g_shade, TPB, 0, stream>>>(shv, P, prm, cur, Learn{});
        else path_fn<<<g_shade, TPB, 0, stream>>>(shv, P, prm, cur, (int)d, nullptr);
        shadow_fn<<<g_sh, TPB, smem, stream>>>(sv, P, depth, cur, nullptr);
        n_launch += 3;
        cur ^= 1;
      }
    }
  }
  k_resolve_jobs<<<std::min<unsigned>(2048, ceil_div(set.pixels, 256)), 256, 0, stream>>>(
      b->accum.ptr, set.dev.ptr, (uint32_t)set.host.size(), set.pixels);
  ++n_launch;
  CKR_CUDA_TRY(cudaGetLastError());
  if (launches) *launches = n_launch;
  return CKR_OK;
}

// The persistent renderer: `lanes` paths in flight (the grid's threads, a
// multiple of TPB); pack = one launch for the whole batch, else one per job.
template <int TPB>
int enqueue_persistent(ckr_batch *b, JobSet &set, bool pack, uint32_t lanes, cudaStream_t stream,
                       uint32_t *launches) {
  ckr_scene *s = b->scene;
  const int depth = (int)stack_depth_of(s);
  const size_t smem = (size_t)std::max(1, depth) * TPB * sizeof(uint2);
  const bool nee = b->shader == CKR_SHADER_PATH_NEE;
  void (*const fn)(SceneView, ShadeView, Params, Paths, uint64_t, uint64_t, unsigned long long *, int) =
      nee                    ? k_render_persistent<CKR_SHADER_PATH_NEE, TPB>
      : mesh_lights_only(s) ? k_render_persistent<CKR_SHADER_PATH, TPB, kLightsMeshOnly>
                             : k_render_persistent<CKR_SHADER_PATH, TPB, kLightsAll>;
  if (smem > 48 * 1024) CKR_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uint32_t grid = std::max<uint32_t>(1, lanes / TPB);
  Params prm{};
  prm.shader = b->shader;
  prm.n_light = b->n_light;
  prm.n_brdf = 1;
  prm.rr_prob = b->rr_prob;
  prm.shadow_per_path = b->per_path;
  prm.jobs = set.dev.ptr;
  prm.njobs = (uint32_t)set.host.size();
  prm.spp = 1;
  prm.npix = 1;
  SceneView sv = view_of(s);
  ShadeView shv = shade_view_of(s);
  shv.mats = b->mats.ptr;
  Paths P = b->ws.paths(b->accum.ptr);
  P.status = s->status.ptr;
  uint32_t n_launch = 0;
  CKR_CUDA_TRY(cudaMemsetAsync(b->accum.ptr, 0, sizeof(double) * 3 * (size_t)set.pixels, stream));
  std::vector<std::pair<uint64_t, uint64_t>> ranges;
  if (pack) ranges.push_back({0, set.paths});
  else
    for (const JobDev &J : set.host) ranges.push_back({J.path_begin, (uint64_t)J.npix * J.spp});
  for (auto [first, count] : ranges) {
    CKR_CUDA_TRY(cudaMemsetAsync(b->next.ptr, 0, sizeof(unsigned long long), stream));
    fn<<<grid, TPB, smem, stream>>>(sv, shv, prm, P, first, count, b->next.ptr, depth);
    ++n_launch;
  }
  k_resolve_jobs<<<std::min<unsigned>(2048, ceil_div(set.pixels, 256)), 256, 0, stream>>>(
      b->accum.ptr, set.dev.ptr, (uint32_t)set.host.size(), set.pixels);
  ++n_launch;
  CKR_CUDA_TRY(cudaGetLastError());
  if (launches) *launches = n_launch;
  return CKR_OK;
}

int enqueue_any(ckr_batch *b, JobSet &set, bool pack, const ckr_batch_tuning &t, cudaStream_t stream,
                uint32_t *launches) {
  if (t.mode == CKR_BATCH_PERSISTENT) {
    if (t.block == 64) return enqueue_persistent<64>(b, set, pack, t.wave, stream, launches);
    if (t.block == 256) return enqueue_persistent<256>(b, set, pack, t.wave, stream, launches);
    return enqueue_persistent<128>(b, set, pack, t.wave, stream, launches);
  }
  if (t.block == 64) return enqueue<64>(b, set, pack, t.wave, stream, launches);
  if (t.block == 256) return enqueue<256>(b, set, pack, t.wave, stream, launches);
  return enqueue<128>(b, set, pack, t.wave, stream, launches);
}

// Resident lanes of the persistent kernel at block size TPB: SMs x resident blocks
// x TPB.
template <int TPB>
uint32_t persistent_lanes(ckr_batch *b) {
  const int depth = (int)stack_depth_of(b->scene);
  const size_t smem = (size_t)std::max(1, depth) * TPB * sizeof(uint2);
  const void *fn = b->shader == CKR_SHADER_PATH_NEE ? (const void *)k_render_persistent<CKR_SHADER_PATH_NEE, TPB>
                   : mesh_lights_only(b->scene)      ? (const void *)k_render_persistent<CKR_SHADER_PATH, TPB, kLightsMeshOnly>
                                                     : (const void *)k_render_persistent<CKR_SHADER_PATH, TPB, kLightsAll>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return (uint32_t)grid_for(fn, smem, TPB) * TPB;
}

uint32_t persistent_lanes_of(ckr_batch *b, uint32_t block) {
  if (block == 64) return persistent_lanes<64>(b);
  if (block == 256) return persistent_lanes<256>(b);
  return persistent_lanes<128>(b);
}

// Times block x wave candidates on the batch with spp capped at 1 (outputs to a
// scratch image) and keeps the fastest.  A wave whose workspace does not fit in
// device memory ends that block size's sweep (larger waves need more); the
// tuner fails only when no candidate fits at all.
int autotune(ckr_batch *b, ckr_batch_tuning *best) {
  std::vector<float *> scratch(b->job_in.size(), nullptr);
  uint32_t maxpix = 0;
  for (const ckr_job &j : b->job_in) maxpix = std::max(maxpix, j.cam.width * j.cam.height);
  DevBuf<float> img;
  if (img.reserve(3 * (size_t)maxpix) != cudaSuccess) return CKR_ERR_OUT_OF_MEMORY;
  for (auto &p : scratch) p = img.ptr;  // jobs overwrite each other's pixels: timing only
  JobSet small;
  int st = small.build(b->job_in.data(), (uint32_t)b->job_in.size(), b->nmat, 1, scratch.data());
  if (st != CKR_OK) return st;
  cudaStream_t s = b->capture;
  cudaEvent_t e0, e1;
  CKR_CUDA_TRY(cudaEventCreate(&e0));
  CKR_CUDA_TRY(cudaEventCreate(&e1));
  const uint32_t blocks[3] = {64, 128, 256};
  best->ms = 3.0e38f;
  best->candidates = 0;
  auto time_one = [&](const ckr_batch_tuning &t) -> int {
    int r;
    if ((r = enqueue_any(b, small, true, t, s, nullptr)) != CKR_OK) return r;  // warm-up
    CKR_CUDA_TRY(cudaEventRecord(e0, s));
    if ((r = enqueue_any(b, small, true, t, s, nullptr)) != CKR_OK) return r;
    CKR_CUDA_TRY(cudaEventRecord(e1, s));
    CKR_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    CKR_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    ++best->candidates;
    if (ms < best->ms) {
      best->ms = ms;
      best->block = t.block;
      best->wave = t.wave;
      best->mode = t.mode;
    }
    return CKR_OK;
  };
  // Persistent renderer: the resident grid or half of it, per block size.
  if (b->persistent_ok) {
    for (uint32_t blk : blocks) {
      const uint32_t full = persistent_lanes_of(b, blk);
      for (uint32_t lanes : {full, std::max(blk, (full / 2) / blk * blk)}) {
        ckr_batch_tuning t{blk, lanes, 0.f, 0, CKR_BATCH_PERSISTENT};
        if ((st = time_one(t)) != CKR_OK) break;
      }
      if (st != CKR_OK) break;
    }
  }
  for (uint32_t blk : blocks) {
    if (st != CKR_OK) break;
    for (uint32_t w = 1u << 17; w <= (1u << 21); w <<= 1) {
      if (w > 2 * small.paths && w > (1u << 17)) break;
      ckr_batch_tuning t{blk, w, 0.f, 0, CKR_BATCH_WAVEFRONT};
      if ((st = b->ws.reserve(w, b->per_path)) != CKR_OK) {
        if (st != CKR_ERR_OUT_OF_MEMORY) break;
        (void)cudaGetLastError();  // the failed allocation's error is not sticky
        b->ws.release_waves();
        st = CKR_OK;
        break;  // next block size
      }
      if ((st = time_one(t)) != CKR_OK) break;
    }
    if (st != CKR_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == CKR_OK && best->candidates == 0) st = CKR_ERR_OUT_OF_MEMORY;
  return st;
}

}  // namespace

extern "C" int ckr_batch_create(ckr_scene *s, uint32_t shader, float rr_prob, uint32_t n_light_samples,
                                const ckr_material *materials, uint32_t nsets, const ckr_job *jobs, uint32_t njobs,
                                const ckr_batch_tuning *tuning, ckr_batch **out) {
  if (!s || !out || !jobs || njobs == 0 || !s->has_shading ||
      (shader != CKR_SHADER_PATH && shader != CKR_SHADER_PATH_NEE) || !(rr_prob >= 0.f && rr_prob < 1.f) ||
      (nsets && !materials) || njobs > (1u << 16))
    return CKR_ERR_INVALID_ARGUMENT;
  if (shader == CKR_SHADER_PATH_NEE && s->n_emit == 0) return CKR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const uint32_t nmat = (uint32_t)s->host_mats.size();
  const uint32_t sets = nsets ? nsets : 1;
  uint64_t pixels = 0;
  for (uint32_t j = 0; j < njobs; ++j) {
    const ckr_job &J = jobs[j];
    if (!J.rgb || J.cam.width == 0 || J.cam.height == 0 || J.spp == 0 || J.material_set >= sets)
      return CKR_ERR_INVALID_ARGUMENT;
    if (J.max_depth > 60 || J.spp > 65536) return CKR_ERR_TOO_LARGE;
    pixels += (uint64_t)J.cam.width * J.cam.height;
  }
  if (pixels > 0xFFFFFFF0ull / 3) return CKR_ERR_TOO_LARGE;
  uint32_t area = 0, points = 0;
  for (const DevLight &L : s->host_lights) (L.type == CKR_LIGHT_POINT ? points : area)++;
  ckr_batch *b = new (std::nothrow) ckr_batch();
  if (!b) return CKR_ERR_OUT_OF_MEMORY;
  auto fail = [&](int st) {
    delete b;
    return st;
  };
  b->scene = s;
  b->shader = shader;
  b->rr_prob = rr_prob;
  b->n_light = std::max(1u, n_light_samples);
  b->per_path = shader == CKR_SHADER_PATH_NEE ? 1u : std::max(1u, points + area * b->n_light + s->env_n);
  b->nmat = nmat;
  b->nsets = sets;
  b->job_in.assign(jobs, jobs + njobs);
  if (b->mats.reserve((size_t)sets * nmat) != cudaSuccess) return fail(CKR_ERR_OUT_OF_MEMORY);
  const ckr_material *src = nsets ? materials : s->host_mats.data();
  if (cudaMemcpy(b->mats.ptr, src, (size_t)sets * nmat * sizeof(ckr_material), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(CKR_ERR_CUDA);
  int st = b->jobs.build(jobs, njobs, nmat, 0, nullptr);
  if (st != CKR_OK) return fail(st);
  if (b->accum.reserve(3 * (size_t)b->jobs.pixels) != cudaSuccess) return fail(CKR_ERR_OUT_OF_MEMORY);
  if (cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking) != cudaSuccess) return fail(CKR_ERR_CUDA);
  if (b->next.reserve(1) != cudaSuccess || b->ws.stats.reserve(2) != cudaSuccess) return fail(CKR_ERR_OUT_OF_MEMORY);
  if (cudaMemset(b->ws.stats.ptr, 0, 2 * sizeof(unsigned long long)) != cudaSuccess) return fail(CKR_ERR_CUDA);
  b->persistent_ok = b->per_path <= kInlineShadow;
  std::lock_guard<std::mutex> lock(s->host_mu);
  if (tuning) {
    b->tuning = *tuning;
    if (b->tuning.block != 64 && b->tuning.block != 128 && b->tuning.block != 256) return fail(CKR_ERR_INVALID_ARGUMENT);
    if (b->tuning.mode == CKR_BATCH_PERSISTENT) {
      if (!b->persistent_ok || b->tuning.wave < b->tuning.block) return fail(CKR_ERR_INVALID_ARGUMENT);
      b->tuning.wave = b->tuning.wave / b->tuning.block * b->tuning.block;
    } else if (b->tuning.mode != CKR_BATCH_WAVEFRONT || b->tuning.wave < 1024) {
      return fail(CKR_ERR_INVALID_ARGUMENT);
    }
  } else if ((st = autotune(b, &b->tuning)) != CKR_OK) {
    return fail(st);
  }
  if (b->tuning.mode == CKR_BATCH_WAVEFRONT) {
    b->tuning.wave = (uint32_t)std::min<uint64_t>(b->tuning.wave, std::max<uint64_t>(1024, b->jobs.paths));
    if ((st = b->ws.reserve(b->tuning.wave, b->per_path)) != CKR_OK) return fail(st);
  } else {
    b->ws.release_waves();  // the autotuner's wavefront candidates
  }
  if (cudaMemset(b->ws.stats.ptr, 0, 2 * sizeof(unsigned long long)) != cudaSuccess) return fail(CKR_ERR_CUDA);
  // One uncaptured pass first: kernel attributes are set and the kernels loaded
  // outside the capture.
  if ((st = enqueue_any(b, b->jobs, true, b->tuning, b->capture, nullptr)) != CKR_OK) return fail(st);
  if (cudaStreamSynchronize(b->capture) != cudaSuccess) return fail(CKR_ERR_CUDA);
  // Capture the pass once.
  if (cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fail(CKR_ERR_CUDA);
  st = enqueue_any(b, b->jobs, true, b->tuning, b->capture, &b->launches);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->capture, &g);
  if (st != CKR_OK) {
    if (g) cudaGraphDestroy(g);
    return fail(st);
  }
  if (e != cudaSuccess) return fail(CKR_ERR_CUDA);
  b->graph = g;
  if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) return fail(CKR_ERR_CUDA);
  *out = b;
  return CKR_OK;
}

extern "C" int ckr_internal_batch_workspace_cap(uint64_t bytes) {
  g_test_ws_cap.store((size_t)bytes);
  return CKR_OK;
}

extern "C" int ckr_batch_render(ckr_batch *b, void *stream) {
  if (!b || !b->exec) return CKR_ERR_INVALID_ARGUMENT;
  CKR_CUDA_TRY(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  return CKR_OK;
}

extern "C" int ckr_batch_render_sequential(ckr_batch *b, void *stream) {
  if (!b) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(b->scene->host_mu);
  return enqueue_any(b, b->jobs, false, b->tuning, (cudaStream_t)stream, nullptr);
}

extern "C" int ckr_batch_get_tuning(const ckr_batch *b, ckr_batch_tuning *out) {
  if (!b || !out) return CKR_ERR_INVALID_ARGUMENT;
  *out = b->tuning;
  return CKR_OK;
}

extern "C" int ckr_batch_get_stats(const ckr_batch *b, uint64_t *paths, uint32_t *launches) {
  if (!b || !paths || !launches) return CKR_ERR_INVALID_ARGUMENT;
  *paths = b->jobs.paths;
  *launches = b->launches;
  return CKR_OK;
}

extern "C" int ckr_batch_destroy(ckr_batch *b) {
  if (!b) return CKR_ERR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  delete b;
  return CKR_OK;
}
