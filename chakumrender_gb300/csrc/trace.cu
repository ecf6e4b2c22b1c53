// trace.cu — scene upload and the closest-hit / any-hit traversal kernels.
//
// A persistent grid (the SMs x the blocks that fit) fetches rays dynamically
// (trace_dynamic): a lane takes a new ray when its own is finished.  Each lane
// keeps its traversal stack of node groups in shared memory, laid out level-major
// ([level][thread]) so stack traffic is bank-conflict free.  Wide nodes (80 B:
// eight quantised child boxes) and triangles (48 B) are read with 16-byte
// read-only loads.  The host-buffer entry points pipeline uploads, traversal and
// downloads over internal streams.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <vector>

#include "bvh_build.h"
#include "ckr_internal.h"
#include "scene.h"
#include "trace_device.cuh"

namespace ckr {

SceneView view_of(const ckr_scene *s) {
  SceneView v;
  v.nodes = s->nodes.ptr;
  v.tris = s->tris.ptr;
  v.spheres = s->spheres.ptr;
  v.root = s->root;
  v.nsph = s->nsph;
  v.status = s->status.ptr;
  v.slot_bits = s->slot_bits.ptr;
  return v;
}

uint32_t stack_depth_of(const ckr_scene *s) { return std::max<uint32_t>(1, s->max_depth); }

namespace {

constexpr int kTPB = 128;

// The triangle test's ray data in shared memory after the stacks (TriShearSmem,
// trace_device.cuh): 64 registers and eight CTAs per SM instead of 72 and seven
// (closest hit 2.194 -> 2.148 ms per 2^23 rays, any hit 1.621 -> 1.580 ms).  Capping
// the kernel at 56 or 48 registers (nine or ten CTAs) spilled and was 3 % and 7 %
// slower.  After them, the 2 KB octant table of the slot bits (slot_lut): the hit
// bits of each child come from the scene's slot_bits array (2.145 -> 2.105 ms, any
// hit 1.576 -> 1.546 ms).
constexpr size_t kAfterStacksBytes = shear_smem_bytes(kTPB) + kSlotLutBytes;

// Closest / any hit over a ray array, with dynamic ray fetching (trace_dynamic).
template <bool ANY>
__global__ void __launch_bounds__(kTPB) k_trace_dyn(SceneView s, const float4 *__restrict__ rays, uint32_t n,
                                                    uint32_t *__restrict__ hit_id, float *__restrict__ hit_t,
                                                    uint8_t *__restrict__ occluded, int depth, uint32_t *next) {
  extern __shared__ uint2 smem_trav[];
  float4 *col = shear_column<kTPB>(smem_trav, depth);
  const uint8_t *lut = fill_slot_lut<kTPB>(reinterpret_cast<uint8_t *>(col - threadIdx.x + 3 * kTPB));
  const TriShearSmem<kTPB, true, true> tri_pol{col, lut};
  trace_dynamic<ANY>(
      s, n, next, smem_trav + threadIdx.x, kTPB, depth,
      [&](uint32_t i, RayPre &r, float &tmax) {
        const float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
        r = make_ray(a, b);
        tmax = b.w;
        store_shear<kTPB>(col, r);
        return true;
      },
      [&](uint32_t i, uint32_t best, float t) {
        if (ANY) {
          occluded[i] = best != kMiss ? 1 : 0;
        } else {
          hit_id[i] = best;
          hit_t[i] = t;
        }
      },
      tri_pol);
}

struct LaunchShape {
  int grid;
  size_t smem;
};

// Persistent grid of the traversal kernel for scene s: as many blocks as fit on
// the device at once.
template <bool ANY>
cudaError_t launch_shape(const ckr_scene *s, LaunchShape &ls) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  ls.smem = (size_t)stack_depth_of(s) * kTPB * sizeof(uint2) + kAfterStacksBytes;
  if (ls.smem > 48 * 1024) {
    e = cudaFuncSetAttribute(k_trace_dyn<ANY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ls.smem);
    if (e != cudaSuccess) return e;
  }
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_dyn<ANY>, kTPB, ls.smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  ls.grid = sms * per_sm;
  return cudaSuccess;
}

// Launches the traversal of rays[0, n).  `next` is a zeroed-per-launch ray counter
// owned by the caller (one per concurrently used stream), or null to allocate one
// in stream order for this call.
template <bool ANY>
int launch_trace(const ckr_scene *s, const ckr_ray *rays, uint32_t n, uint32_t *hit_id, float *hit_t,
                 uint8_t *occluded, cudaStream_t stream, uint32_t *next = nullptr) {
  if (n == 0) return CKR_OK;
  const int grid = s->trace_grid[ANY ? 1 : 0];
  const size_t smem = s->trace_smem;
  // The attribute is per kernel: set it for this scene's stack before each launch.
  if (smem > 48 * 1024)
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_trace_dyn<ANY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // Launches cover at most 2^31 rays so that the counter, which overshoots n by at
  // most one refill per warp, cannot wrap.
  const bool own = next == nullptr;
  if (own) CKR_CUDA_TRY(cudaMallocAsync((void **)&next, sizeof(uint32_t), stream));
  cudaError_t e = cudaSuccess;
  constexpr uint32_t kChunk = 1u << 31;
  for (uint32_t off = 0; off < n && e == cudaSuccess; off += std::min(n - off, kChunk)) {
    const uint32_t m = std::min(n - off, kChunk);
    e = cudaMemsetAsync(next, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) break;
    k_trace_dyn<ANY><<<grid, kTPB, smem, stream>>>(
        view_of(s), reinterpret_cast<const float4 *>(rays + off), m, ANY ? nullptr : hit_id + off,
        ANY ? nullptr : hit_t + off, ANY ? occluded + off : nullptr, (int)stack_depth_of(s), next);
    e = cudaGetLastError();
    if (n - off <= kChunk) break;
  }
  if (own) cudaFreeAsync(next, stream);
  CKR_CUDA_TRY(e);
  return CKR_OK;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace
}  // namespace ckr

using namespace ckr;

extern "C" int ckr_scene_create(const float *tri9, uint32_t ntri, const float *sph4, uint32_t nsph,
                                const ckr_build_params *params, ckr_scene **out) {
  if (!out || (ntri && !tri9) || (nsph && !sph4)) return CKR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CKR_ERR_NO_DEVICE;
  ckr_build_params p = params ? *params : ckr_build_params{0, 0, 0};
  auto t0 = std::chrono::steady_clock::now();
  FlatBvh bvh;
  int st = build_bvh(tri9, ntri, p, bvh);
  if (st != CKR_OK) return st;
  auto t1 = std::chrono::steady_clock::now();
  ckr_scene *s = new (std::nothrow) ckr_scene();
  if (!s) return CKR_ERR_OUT_OF_MEMORY;
  auto fail = [&](int code) {
    delete s;
    return code;
  };
  if (cudaGetDevice(&s->device) != cudaSuccess) return fail(CKR_ERR_CUDA);
  s->ntri = ntri;
  s->nsph = nsph;
  s->root = bvh.root;
  s->nnodes = bvh.nnodes;
  s->nleaves = bvh.nleaves;
  s->max_depth = bvh.max_depth;
  s->nnodes_binary = bvh.nnodes_binary;
  s->build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  size_t nn = std::max<size_t>(1, bvh.nodes.size() / 4), nt = std::max<size_t>(1, bvh.tris.size() / 4);
  if (s->nodes.reserve(nn) != cudaSuccess || s->tris.reserve(nt) != cudaSuccess ||
      s->spheres.reserve(std::max<uint32_t>(1, nsph)) != cudaSuccess || s->status.reserve(1) != cudaSuccess)
    return fail(CKR_ERR_OUT_OF_MEMORY);
  if (!bvh.nodes.empty() && cudaMemcpy(s->nodes.ptr, bvh.nodes.data(), bvh.nodes.size() * sizeof(uint32_t),
                                        cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(CKR_ERR_CUDA);
  if (!bvh.tris.empty() &&
      cudaMemcpy(s->tris.ptr, bvh.tris.data(), bvh.tris.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(CKR_ERR_CUDA);
  {
    // Each slot's hit bits from its meta byte (pattern << position), interior slots at
    // 24 + slot (the traversal permutes them for the ray's octant).
    std::vector<uint32_t> bits(8 * std::max<size_t>(1, bvh.nnodes), 0u);
    for (size_t n = 0; n < bvh.nnodes; ++n)
      for (int k = 0; k < 8; ++k) {
        const uint32_t m = (bvh.nodes[kWideWords * n + 6 + (k >> 2)] >> (8 * (k & 3))) & 0xffu;
        bits[8 * n + k] = m ? (m >> 5) << (m & 31u) : 0u;
      }
    if (s->slot_bits.reserve(bits.size() / 4) != cudaSuccess) return fail(CKR_ERR_OUT_OF_MEMORY);
    if (cudaMemcpy(s->slot_bits.ptr, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice) !=
        cudaSuccess)
      return fail(CKR_ERR_CUDA);
  }
  if (nsph) {
    s->host_spheres.assign(sph4, sph4 + 4 * (size_t)nsph);
    if (cudaMemcpy(s->spheres.ptr, sph4, 4 * sizeof(float) * nsph, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(CKR_ERR_CUDA);
  }
  if (cudaMemset(s->status.ptr, 0, sizeof(int)) != cudaSuccess) return fail(CKR_ERR_CUDA);
  LaunchShape l0, l1;
  if (launch_shape<false>(s, l0) != cudaSuccess || launch_shape<true>(s, l1) != cudaSuccess) return fail(CKR_ERR_CUDA);
  s->trace_grid[0] = l0.grid;
  s->trace_grid[1] = l1.grid;
  s->trace_smem = l0.smem;
  s->host_nodes.swap(bvh.nodes);
  s->host_tris.swap(bvh.tris);
  *out = s;
  return CKR_OK;
}

extern "C" int ckr_scene_destroy(ckr_scene *scene) {
  if (!scene) return CKR_ERR_INVALID_ARGUMENT;
  for (auto &st : scene->pipe)
    if (st) cudaStreamDestroy(st);
  for (auto &e : scene->pipe_done)
    if (e) cudaEventDestroy(e);
  if (scene->user_ready) cudaEventDestroy(scene->user_ready);
  if (scene->h_status) cudaFreeHost(scene->h_status);
  if (scene->render_ws && scene->render_ws_free) scene->render_ws_free(scene->render_ws);
  delete scene;
  return CKR_OK;
}

extern "C" int ckr_scene_get_info(const ckr_scene *s, ckr_scene_info *out) {
  if (!s || !out) return CKR_ERR_INVALID_ARGUMENT;
  std::memset(out, 0, sizeof(*out));
  out->ntri = s->ntri;
  out->nsph = s->nsph;
  out->nnodes = s->nnodes;
  out->nleaves = s->nleaves;
  out->max_depth = s->max_depth;
  out->nnodes_binary = s->nnodes_binary;
  out->device_bytes = s->nodes.bytes() + s->tris.bytes() + s->spheres.bytes();
  out->build_ms = s->build_ms;
  return CKR_OK;
}

extern "C" int ckr_scene_check(ckr_scene *s, void *stream) {
  if (!s) return CKR_ERR_INVALID_ARGUMENT;
  int h = 0;
  CKR_CUDA_TRY(cudaMemcpyAsync(&h, s->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  CKR_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  if (h != 0) CKR_CUDA_TRY(cudaMemset(s->status.ptr, 0, sizeof(int)));
  return h;
}

extern "C" int ckr_trace_closest(const ckr_scene *s, const ckr_ray *rays, uint32_t n, uint32_t *hit_id,
                                 float *hit_t, void *stream) {
  if (!s || (n && (!rays || !hit_id || !hit_t)) || !aligned16(rays)) return CKR_ERR_INVALID_ARGUMENT;
  return launch_trace<false>(s, rays, n, hit_id, hit_t, nullptr, (cudaStream_t)stream);
}

extern "C" int ckr_trace_any(const ckr_scene *s, const ckr_ray *rays, uint32_t n, uint8_t *occluded,
                             void *stream) {
  if (!s || (n && (!rays || !occluded)) || !aligned16(rays)) return CKR_ERR_INVALID_ARGUMENT;
  return launch_trace<true>(s, rays, n, nullptr, nullptr, occluded, (cudaStream_t)stream);
}

namespace {

// Host-buffer path: kPipes internal streams take turns over chunks of kHostChunk
// rays, so that the host-to-device copy of one chunk (rays in pageable memory; rays
// in pinned memory are read in place) and the device-to-host copy of another
// overlap the traversal of a third; each stream has its own staging slot and ray
// counter.  Swept on the 2^23-ray workload with uploads (e2e Mrays/s): 2 x 2^19
// 2530, 2 x 2^20 2899, 2 x 2^21 2983, 3 x 2^19 2999, 3 x 2^20 3089, 3 x 2^21 2987,
// 4 x 2^20 3086.
constexpr int kPipes = 3;
constexpr uint32_t kHostChunk = 1u << 20;

// True when the device can load [p, p + bytes) at the same address: pinned host
// memory (which unified addressing maps into the device's address space), managed
// or device memory.  Both ends are checked, so a range that runs past its
// allocation is refused.
bool device_addressable(const void *p, size_t bytes) {
  for (const char *q : {static_cast<const char *>(p), static_cast<const char *>(p) + bytes - 1}) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const bool ok = a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged ||
                    (a.type == cudaMemoryTypeHost && a.devicePointer == q);
    if (!ok) return false;
  }
  return true;
}

template <bool ANY>
int trace_host(ckr_scene *s, const ckr_ray *rays, uint32_t n, uint32_t *hit_id, float *hit_t, uint8_t *occ,
               cudaStream_t user) {
  static_assert(kPipes <= ckr_scene::kMaxPipes, "pipeline streams");
  if (n == 0) return CKR_OK;
  std::lock_guard<std::mutex> lock(s->host_mu);
  // Rays the device can address in place (pinned host memory): the kernels read
  // them there and no upload is issued (2^23 rays: 3115 -> 3175 Mrays/s end to
  // end); the results are still staged and copied back chunk by chunk.
  const bool in_place = aligned16(rays) && device_addressable(rays, (size_t)n * sizeof(ckr_ray));
  const uint32_t chunk = kHostChunk;
  uint32_t cap = (uint32_t)std::min<uint64_t>(n, (uint64_t)kPipes * chunk);
  if (!in_place) CKR_CUDA_TRY(s->st_rays.reserve(cap));
  CKR_CUDA_TRY(s->st_next.reserve(kPipes));
  if (ANY) {
    CKR_CUDA_TRY(s->st_occ.reserve(cap));
  } else {
    CKR_CUDA_TRY(s->st_id.reserve(cap));
    CKR_CUDA_TRY(s->st_t.reserve(cap));
  }
  for (int k = 0; k < kPipes; ++k) {
    if (!s->pipe[k]) CKR_CUDA_TRY(cudaStreamCreateWithFlags(&s->pipe[k], cudaStreamNonBlocking));
    if (!s->pipe_done[k]) CKR_CUDA_TRY(cudaEventCreateWithFlags(&s->pipe_done[k], cudaEventDisableTiming));
  }
  if (!s->user_ready) CKR_CUDA_TRY(cudaEventCreateWithFlags(&s->user_ready, cudaEventDisableTiming));
  // Order after prior work on the caller's stream.
  CKR_CUDA_TRY(cudaEventRecord(s->user_ready, user));
  for (int k = 0; k < kPipes; ++k) CKR_CUDA_TRY(cudaStreamWaitEvent(s->pipe[k], s->user_ready, 0));
  // Chunks grow from kHostChunk / 8 to kHostChunk, so that the first upload, which
  // nothing overlaps, is short (e2e 3088 -> 3118 Mrays/s; shrinking the last chunks
  // as well was slower, 3035).
  // Rays read in place have no first upload to hide: full chunks from the start.
  uint32_t k = 0, size = in_place ? chunk : chunk >> 3;
  for (uint32_t off = 0; off < n; ++k) {
    const uint32_t m = std::min(size, n - off);
    size = std::min(size * 2, chunk);
    int slot = (int)(k % kPipes);
    cudaStream_t st = s->pipe[slot];
    size_t base = (size_t)slot * chunk;
    if (!in_place)
      CKR_CUDA_TRY(cudaMemcpyAsync(s->st_rays.ptr + base, rays + off, (size_t)m * sizeof(ckr_ray),
                                   cudaMemcpyHostToDevice, st));
    const ckr_ray *src = in_place ? rays + off : s->st_rays.ptr + base;
    int rc = ANY ? launch_trace<true>(s, src, m, nullptr, nullptr, s->st_occ.ptr + base, st, s->st_next.ptr + slot)
                 : launch_trace<false>(s, src, m, s->st_id.ptr + base, s->st_t.ptr + base, nullptr, st,
                                       s->st_next.ptr + slot);
    if (rc != CKR_OK) return rc;
    if (ANY) {
      CKR_CUDA_TRY(cudaMemcpyAsync(occ + off, s->st_occ.ptr + base, m, cudaMemcpyDeviceToHost, st));
    } else {
      CKR_CUDA_TRY(cudaMemcpyAsync(hit_id + off, s->st_id.ptr + base, (size_t)m * 4, cudaMemcpyDeviceToHost, st));
      CKR_CUDA_TRY(cudaMemcpyAsync(hit_t + off, s->st_t.ptr + base, (size_t)m * 4, cudaMemcpyDeviceToHost, st));
    }
    off += m;
  }
  for (int k = 0; k < kPipes; ++k) {
    CKR_CUDA_TRY(cudaEventRecord(s->pipe_done[k], s->pipe[k]));
    CKR_CUDA_TRY(cudaStreamWaitEvent(user, s->pipe_done[k], 0));
  }
  // The status word comes back in the same stream order, so one synchronisation
  // covers the traversal, the results and the status.
  if (!s->h_status) CKR_CUDA_TRY(cudaMallocHost((void **)&s->h_status, sizeof(int)));
  CKR_CUDA_TRY(cudaMemcpyAsync(s->h_status, s->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, user));
  CKR_CUDA_TRY(cudaStreamSynchronize(user));
  const int h = *s->h_status;
  if (h != 0) {
    CKR_CUDA_TRY(cudaMemset(s->status.ptr, 0, sizeof(int)));
    return h;
  }
  return CKR_OK;
}

}  // namespace

extern "C" int ckr_trace_closest_host(ckr_scene *s, const ckr_ray *rays, uint32_t n, uint32_t *hit_id,
                                      float *hit_t, void *stream) {
  if (!s || (n && (!rays || !hit_id || !hit_t))) return CKR_ERR_INVALID_ARGUMENT;
  return trace_host<false>(s, rays, n, hit_id, hit_t, nullptr, (cudaStream_t)stream);
}

extern "C" int ckr_trace_any_host(ckr_scene *s, const ckr_ray *rays, uint32_t n, uint8_t *occluded,
                                  void *stream) {
  if (!s || (n && (!rays || !occluded))) return CKR_ERR_INVALID_ARGUMENT;
  return trace_host<true>(s, rays, n, nullptr, nullptr, occluded, (cudaStream_t)stream);
}

namespace ckr {
// Accessors for the host statistics replay (trace_stats.cpp).
void scene_host_arrays(const ckr_scene *s, const uint32_t **nodes, const float **tris, const float **spheres,
                       int32_t *root, uint32_t *nsph, uint32_t *depth) {
  *nodes = s->host_nodes.data();
  *tris = s->host_tris.data();
  *spheres = s->host_spheres.data();
  *root = s->root;
  *nsph = s->nsph;
  *depth = s->max_depth;
}
}  // namespace ckr
