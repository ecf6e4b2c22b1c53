// scene.h — the library-owned scene (geometry, BVH, shading data) shared by the
// traversal and rendering translation units.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "ckr_internal.h"
#include "trace_device.cuh"

namespace ckr {

// Device form of one light source (ckr_light + precomputed sampling data).
struct DevLight {
  int32_t type;      // CKR_LIGHT_*
  uint32_t first;    // MESH/TRI: first emitter triangle; SPHERE: sphere index
  uint32_t count;    // MESH: emitter triangles
  uint32_t cdf;      // MESH: offset of its 300-entry inverse CDF in the cdf table
  float area;        // MESH/TRI: total emitter area (the pdf's 1/area)
  float px, py, pz;  // POINT: position; SPHERE: centre
  float radius;      // SPHERE
  float pr, pg, pb;  // POINT: power
  uint32_t pcdf;     // MESH/TRI: offset of its per-triangle power CDF (one-sample NEE)
  float power;       // MESH/TRI: emitted power sum of luminance(radiance) x area
  float sel;         // MESH/TRI: power / total power of all MESH/TRI lights
  float pad_;
};

constexpr uint32_t kNoLight = 0xFFFFFFFFu;

constexpr uint32_t kInvCdfBins = 300;  // MeshLight::invCDFBins (headers/lightSources.h:150)

struct ShadeView {
  const ckr_material *mats;
  const uint32_t *tri_mat;   // per input triangle
  const float *tri9;         // input-order vertices (light sampling)
  const float4 *tri_nm;      // per input triangle: geometric normal, material index (bits)
  const uint32_t *sph_mat;
  const float4 *sph;         // centre, radius
  const DevLight *lights;     // sorted: sphere, mesh, triangle, point lights
  uint32_t nlights;
  uint32_t first_point;      // index of the first point light (= number of area/sphere lights)
  const uint32_t *cdf;       // mesh-light inverse CDFs (triangle offsets within the light)
  // One-sample NEE over many lights (CKR_SHADER_PATH_NEE).
  const uint32_t *tri_light;  // per triangle: its MESH/TRI light, or kNoLight
  const float *pcdf;          // per-light triangle power CDFs (DevLight::pcdf)
  const float *sel_cdf;       // power CDF over the emitter lights [first_emit, first_emit + n_emit)
  uint32_t first_emit, n_emit;
  // Environment light (ckr_env_light); env_n = 0 when there is none.
  const float4 *env;         // per pixel: radiance rgb, luminance
  const float *env_marg;     // env_h + 1: CDF over rows (luminance x solid angle)
  const float *env_cond;     // env_h x (env_w + 1): CDF over the columns of each row
  const float *env_cos;      // env_h + 1: cos(r pi / env_h)
  uint32_t env_w, env_h, env_axis, env_n;
  float env_inv_area;        // 1 / integral of the luminance over the sphere
};

}  // namespace ckr

struct ckr_scene {
  int device = 0;
  ckr::DevBuf<float4> nodes, tris, spheres;
  ckr::DevBuf<uint4> slot_bits;  // per wide node: each slot's hit bits (trace_device.cuh)
  ckr::DevBuf<int> status;
  int32_t root = ckr::kDone;
  uint32_t ntri = 0, nsph = 0, nnodes = 0, nleaves = 0, max_depth = 0, nnodes_binary = 0;
  double build_ms = 0.0;
  std::vector<uint32_t> host_nodes;          // wide nodes, kept for the host statistics replay
  std::vector<float> host_tris;
  std::vector<float> host_spheres;
  // Shading data (ckr_scene_create_ex only).
  bool has_shading = false;
  ckr::DevBuf<ckr_material> mats;
  ckr::DevBuf<uint32_t> tri_mat, sph_mat, cdf;
  ckr::DevBuf<float> tri9;
  ckr::DevBuf<float4> tri_nm;  // per triangle: geometric normal, material index (bits)
  ckr::DevBuf<ckr::DevLight> lights;
  ckr::DevBuf<uint32_t> tri_light;
  ckr::DevBuf<float> pcdf, sel_cdf;
  uint32_t nlights = 0, first_point = 0, first_emit = 0, n_emit = 0;
  ckr::DevBuf<float4> env;
  ckr::DevBuf<float> env_marg, env_cond, env_cos;
  uint32_t env_w = 0, env_h = 0, env_axis = 1, env_n = 0;
  float env_inv_area = 0.f;
  float bounds[6] = {0, 0, 0, 0, 0, 0};  // scene box (lo.xyz, hi.xyz) of triangles and spheres
  std::vector<ckr_material> host_mats;
  std::vector<ckr::DevLight> host_lights;
  // Renderer work buffers (path state, queues), grown on demand, owned here.
  void *render_ws = nullptr;
  void (*render_ws_free)(void *) = nullptr;
  // Staging for the host-buffer entry points.
  std::mutex host_mu;
  ckr::DevBuf<ckr_ray> st_rays;
  ckr::DevBuf<uint32_t> st_id;
  ckr::DevBuf<float> st_t;
  ckr::DevBuf<uint8_t> st_occ;
  ckr::DevBuf<uint32_t> st_next;  // ray counters of the pipeline streams
  int trace_grid[2] = {1, 1};     // persistent grids of the closest / any-hit kernels
  size_t trace_smem = 0;          // their traversal stacks
  static constexpr int kMaxPipes = 4;
  cudaStream_t pipe[kMaxPipes] = {};
  cudaEvent_t pipe_done[kMaxPipes] = {};
  cudaEvent_t user_ready = nullptr;
  int *h_status = nullptr;  // pinned: the status word read back at the end of a host-buffer query
  // Test hook (ckr_internal_limit_shadow_queue): a shadow-queue capacity for the
  // next render only; 0 = the size the renderer computes.
  uint32_t test_shadow_cap = 0;
};

namespace ckr {
SceneView view_of(const ckr_scene *s);
uint32_t stack_depth_of(const ckr_scene *s);
ShadeView shade_view_of(const ckr_scene *s);
// Fills s->tri_nm from the uploaded vertices and materials (synchronous).
int build_tri_nm(ckr_scene *s);
}  // namespace ckr
