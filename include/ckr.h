/*
 * ckr.h — C ABI of chakumrender_gb300, a GB300 (sm_103a) implementation of the
 * path-tracing hot path of Sayantan2048/ChakumRender.
 *
 * Conventions (every entry point):
 *   - returns int status: CKR_OK (0) or a negative CKR_ERR_* code; no C++
 *     exception crosses this boundary; ckr_status_string() names a code;
 *   - plain pointers and sizes; "device" pointers are CUDA device memory on
 *     the current device, "host" pointers are ordinary (ideally pinned) memory;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream);
 *     entry points that take device buffers are asynchronous on that stream,
 *     entry points suffixed _host are synchronous and copy inside;
 *   - scene handles are library-owned device state: create once, query from any
 *     number of host threads, destroy once.
 *
 * Each declaration names the reference interface it replaces (file:line in
 * the reference repository).
 */
#ifndef CKR_H
#define CKR_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
/* The library is built with hidden visibility; what this header declares is
 * its exported interface. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- status codes ------------------------------------------------------ */
#define CKR_OK 0
#define CKR_ERR_INVALID_ARGUMENT -1
#define CKR_ERR_CUDA -2
#define CKR_ERR_OUT_OF_MEMORY -3
#define CKR_ERR_STACK_OVERFLOW -4 /* traversal stack deeper than the BVH allows */
#define CKR_ERR_QUEUE_OVERFLOW -5 /* wavefront queue capacity exceeded */
#define CKR_ERR_ITERATION_LIMIT -6 /* a bounded device loop gave up */
#define CKR_ERR_NO_DEVICE -7
#define CKR_ERR_PARSE -8
#define CKR_ERR_IO -9
#define CKR_ERR_TOO_LARGE -10

/* Writes a NUL-terminated description of `status` into buf[0..len). */
int ckr_status_string(int status, char *buf, size_t len);

/* ---- rays and hits ----------------------------------------------------- */
/* One ray: 32 bytes, two 16-byte loads on the device.  The reference's Ray
 * (headers/mathPrimitives.h:39-44) is origin + direction in FP64 with no
 * range; here a ray carries its own (tmin, tmax) interval. */
typedef struct ckr_ray {
  float ox, oy, oz, tmin;
  float dx, dy, dz, tmax;
} ckr_ray;

/* Hit ids: CKR_MISS on a miss (the reference's id = 0xFFFFFFFF,
 * src/bvhAccel.cpp:213), the input index of a triangle, or CKR_SPHERE_BIT |
 * the input index of a sphere.  Ids are in INPUT order; the reference returns
 * BVH order and reorders its primitive list (src/bvhAccel.cpp:95-124). */
#define CKR_MISS 0xFFFFFFFFu
#define CKR_SPHERE_BIT 0x80000000u

/* ---- scene: geometry + BVH in device memory ---------------------------- */
typedef struct ckr_scene ckr_scene;

typedef struct ckr_build_params {
  uint32_t max_leaf_size; /* triangles per leaf of the wide tree, 1..8 accepted, capped at 3;
                             0 = default (3) */
  uint32_t sah_bins;      /* binned-SAH bins, 4..64; 0 = default (16) */
  uint32_t threads;       /* host build threads; 0 = all cores */
} ckr_build_params;

typedef struct ckr_scene_info {
  uint32_t ntri, nsph;
  uint32_t nnodes;     /* wide nodes (each holds up to eight child boxes) */
  uint32_t nleaves;    /* leaf children (runs of 1..3 triangles) */
  uint32_t max_depth;  /* levels of wide nodes = traversal stack entries needed */
  uint32_t nnodes_binary; /* interior nodes of the binary SAH tree before collapsing */
  uint64_t device_bytes;
  double build_ms;
} ckr_scene_info;

/* Replaces loadAccels() (headers/objects.h:17, src/objects.cpp:38-56), which
 * builds the two BVHs (BvhAccel::initAccel, src/bvhAccel.cpp:13-22) over the
 * global triangle and sphere lists.  tri9: ntri x (A.xyz, B.xyz, C.xyz);
 * sph4: nsph x (centre.xyz, radius).  Builds a binned-SAH BVH on the host and
 * uploads it.  Either list may be empty (NULL, 0). */
int ckr_scene_create(const float *tri9, uint32_t ntri, const float *sph4, uint32_t nsph,
                     const ckr_build_params *params, ckr_scene **out);
int ckr_scene_destroy(ckr_scene *scene);
int ckr_scene_get_info(const ckr_scene *scene, ckr_scene_info *out);

/* Device status word of the scene: the first error a traversal kernel hit
 * (CKR_ERR_STACK_OVERFLOW); synchronises `stream`, returns and clears it. */
int ckr_scene_check(ckr_scene *scene, void *stream);

/* Closest hit.  Replaces BvhAccel::intersectT / intersectS
 * (headers/bvhAccel.h:73-74, src/bvhAccel.cpp:151-248) and the
 * intersectTriangle / intersectSphere pair of src/shader.cpp:16-73, which
 * shade() combines as "sphere if tS < tT".  Device buffers: rays[n] in,
 * hit_id[n] and hit_t[n] out (hit_t = tmax on a miss).  A triangle is hit
 * when tmin < t < best-so-far, both faces, edges inclusive, with the
 * reference's near-parallel rejection (d.n)^2 <= 1e-10 (n the unit normal);
 * the test itself is watertight (Woop, Benthin, Wald 2013).  A
 * sphere is hit at the nearest root above max(tmin, 1e-4)
 * (src/geometryPrimitives.cpp:12-27). */
int ckr_trace_closest(const ckr_scene *scene, const ckr_ray *rays, uint32_t n,
                      uint32_t *hit_id, float *hit_t, void *stream);

/* Any hit.  Replaces shadow(ray, dist) (headers/shader.h:6,
 * src/shader.cpp:76-97): occluded[i] = 1 iff some primitive is hit with
 * tmin < t < tmax; the caller folds the reference's 1e-5 slack into tmax
 * (tmax = dist - 1e-5).  Stops at the first hit. */
int ckr_trace_any(const ckr_scene *scene, const ckr_ray *rays, uint32_t n,
                  uint8_t *occluded, void *stream);

/* Host-buffer forms of the two queries (the drop-in for callers that hold
 * rays in host memory, as every reference caller does): copy rays in, trace,
 * copy results out, in chunks that overlap copies with traversal.  Rays in
 * pinned memory whose address is 16-byte aligned are read in place by the
 * kernels instead of being copied in.  Staging buffers are owned by the scene
 * and reused. */
int ckr_trace_closest_host(ckr_scene *scene, const ckr_ray *rays, uint32_t n,
                           uint32_t *hit_id, float *hit_t, void *stream);
int ckr_trace_any_host(ckr_scene *scene, const ckr_ray *rays, uint32_t n,
                       uint8_t *occluded, void *stream);

/* Host replay of the device traversal in the same FP32 arithmetic: mean wide
 * nodes visited (80 bytes each, eight child boxes) and triangles tested per ray
 * (closest-hit mode), used for the algorithmic-bytes roofline.  rays are host
 * memory. */
int ckr_trace_stats(const ckr_scene *scene, const ckr_ray *rays, uint32_t n,
                    double *mean_nodes, double *mean_tris);

/* ---- full scenes: materials, lights, rendering --------------------------- */
/* MaterialType + BasePrimitive colour/reflectance (headers/materialTypes.h:21-98,
 * headers/geometryPrimitives.h:22-34).  brdf uses the reference's BRDFType
 * numbering (0 NONE, 1 CLASSIC_PHONG, 2 GGX, 3 BECKMANN, 4 PHONG, 5 GGXAPPROX);
 * light_type its LightType (0 NONE, 1 POINT, 2 VOLUME, 3 PLANAR, 4 MESH); a
 * primitive whose material has light_type != 0 is an emitter of `radiance`. */
typedef struct ckr_material {
  int32_t brdf;
  int32_t light_type;
  float alpha;       /* GGX/Beckmann roughness, microfacet-Phong exponent */
  float phong_exp;   /* CLASSIC_PHONG exponent */
  float spec;        /* specularCoef in [0, 1] */
  float int_ior, ext_ior;
  float reflectance;
  float color[3];    /* primitive colour c (multiplies shaded light) */
  float radiance[3]; /* emitters */
  float pad[2];
} ckr_material;

#define CKR_LIGHT_MESH 0   /* MeshLight: emitter triangles [first, first+count) */
#define CKR_LIGHT_TRI 1    /* TriLight: one emitter triangle `first` */
#define CKR_LIGHT_SPHERE 2 /* SphereSource: emitter sphere `first` */
#define CKR_LIGHT_POINT 3  /* PointSource at pos with power `power` */

/* One entry of the reference's LightSource lists (headers/lightSources.h:155-249). */
typedef struct ckr_light {
  int32_t type;
  uint32_t first, count;
  float pos[3];
  float power[3];
  float pad;
} ckr_light;

/* Environment light (EnvSource, headers/lightSources.h:33-109, attached by
 * LightSource::addESource; the reference's call, src/prepareScene.cpp:149-153, is
 * commented out and its image env1.ppm is missing).  An equirectangular RGB image
 * about the up axis: row r covers theta in [r, r + 1) pi / height, column c covers
 * phi in [c, c + 1) 2 pi / width, looked up as EnvSource::getRadiance does; the
 * radiance is image x color / max(color) x intensity (BaseSource).  Directions are
 * sampled in proportion to the luminance 0.3 r + 0.59 g + 0.11 b (to_greyScale)
 * over the sphere, with pdf(w) = luminance(L(w)) / A, A the luminance integral
 * (EnvSource::calcArea, computed exactly here and numerically there).
 * CKR_SHADER_DIRECT_MIS draws n_samples environment samples per point (MIS::nEnMpIS,
 * default 10) into the MIS set, and a sample direction that meets no other light
 * sees the environment when unoccluded (src/lightSources.cpp:103-106);
 * CKR_SHADER_PATH does the same at every vertex, and its BRDF-sampled rays that
 * leave the scene see the environment with their MIS weight.  The other shaders
 * ignore it, as the reference's analytic (LTC) estimators do; camera rays that
 * leave the scene are black, as in the reference. */
typedef struct ckr_env_light {
  const float *rgb;  /* width x height x 3 floats, host memory, read at scene creation */
  uint32_t width, height;
  uint32_t axis;     /* up axis: 0 x, 1 y, 2 z (EnvSource::axis) */
  float color[3];
  float intensity;
  uint32_t n_samples; /* 0: 10 */
} ckr_env_light;

typedef struct ckr_scene_desc {
  const float *tri9;            /* ntri x (A, B, C), emitter triangles included */
  const uint32_t *tri_material; /* ntri material indices (NULL: all 0) */
  uint32_t ntri;
  const float *sph4;            /* nsph x (centre, radius) */
  const uint32_t *sph_material;
  uint32_t nsph;
  const ckr_material *materials;
  uint32_t nmaterials;
  const ckr_light *lights;
  uint32_t nlights;
  ckr_build_params build;
  const ckr_env_light *env;     /* NULL: no environment light */
} ckr_scene_desc;

/* Scene with shading data (prepareObjects + prepareLightSources + loadAccels +
 * loadLightSampler, src/prepareScene.cpp:54-280, src/mis.cpp:225-233).  Mesh
 * lights keep the reference's 300-bin area CDF (src/lightSources.cpp:784-807). */
int ckr_scene_create_ex(const ckr_scene_desc *desc, ckr_scene **out);

/* Camera of src/main.cpp:77 and src/prepareScene.cpp:12-36: the ray through
 * pixel (x, y) with sub-pixel offset (jx, jy) has direction
 * normalize(cx ((x + jx)/w - .5) + cy ((y + jy)/h - .5) + dir); y = 0 is the
 * bottom row; output pixel index (h - 1 - y) w + x (top row first). */
typedef struct ckr_camera {
  float pos[3], dir[3], cx[3], cy[3];
  uint32_t width, height;
} ckr_camera;

#define CKR_SHADER_DIRECT_MISCV 0 /* shadeDirectOnly + getLightFromMeshSource_Analytic_MISCV (reference default) */
#define CKR_SHADER_DIRECT_MIS 1   /* shadeDirectOnly + getLightFromAllSources_MIS */
#define CKR_SHADER_PATH 2         /* path tracer: MIS light/BRDF at every vertex, BRDF-sampled continuation */
/* Many-light path tracer (no reference counterpart: the reference's
 * getLightFromAllSources_MIS samples every light, src/mis.cpp:100-146): at every
 * vertex ONE light sample -- an emitter light (MESH/TRI; "cluster") drawn from the
 * selection distribution, one of its triangles in proportion to power
 * (luminance x area), a uniform point on it -- and one BRDF sample
 * (getBrdfDirectionSampleRandomized) that also continues the path; balance
 * heuristic between the two; Russian roulette with rr_prob.  ckr_render selects
 * lights in proportion to power; ckr_render_learned with a proposal network. */
#define CKR_SHADER_PATH_NEE 3
/* shadeDirectOnly + getLightFromMeshSource_AnalyticCV (src/lightSources_CV.cpp:335-397):
 * the LTC analytic term plus a control-variate residual over n_light_samples area
 * samples per mesh light, sum Le (V f - f_ltc) cos cos_l / d^2 * area / n, with
 * shadow rays for V. */
#define CKR_SHADER_DIRECT_CV 4
/* shadeExplicit (src/shader.cpp:111-207): at every vertex the MISCV direct term
 * (n_light_samples / n_brdf_samples as in DIRECT_MISCV), then Russian roulette with
 * rr_prob and a uniform hemisphere continuation redrawn (up to 8 times) while it
 * meets an emitter; up to max_depth vertices (the reference allows 100). */
#define CKR_SHADER_EXPLICIT 5

typedef struct ckr_render_cfg {
  uint32_t shader;           /* CKR_SHADER_* */
  uint32_t spp;              /* samples per pixel; sample k < 8 uses the reference's fixed
                                sub-pixel offsets (src/main.cpp:23-24), later ones (0, 0) */
  uint32_t max_depth;        /* path vertices (CKR_SHADER_PATH) */
  uint32_t n_light_samples;  /* MIS samples per area/sphere light (reference: 10) */
  uint32_t n_brdf_samples;   /* MIS BRDF samples (reference: 60; the path tracer uses 1) */
  float rr_prob;             /* Russian-roulette termination probability (reference: 0.3) */
  uint64_t seed;             /* per-pixel stream key = hash(seed, pixel index) */
  uint32_t flags;            /* reserved, 0 */
  uint32_t reserved;
} ckr_render_cfg;

/* Renders linear RGB (3 floats per pixel, top row first) into rgb (device),
 * the mean over spp; accum (device, nullable) receives the FP64 per-pixel sums.
 * Replaces the OpenMP pixel loop of src/main.cpp:62-94 over shade(). */
int ckr_render(ckr_scene *scene, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb, double *accum,
               void *stream);

/* Shades caller rays: radiance along each ray by the configured shader, the
 * mean over cfg->spp samples, 3 floats per ray into rgb (device).  This is
 * shade() (headers/shader.h:4, src/shader.cpp:363-378) over a batch: ray i
 * draws from the stream (cfg->seed, i) exactly as pixel i of ckr_render does,
 * so rays equal to a camera's give that camera's image.  Directions are
 * normalised on the device; rays (device) must be 16-byte aligned; tmin < 0
 * counts as 0. */
int ckr_shade_rays(ckr_scene *scene, const ckr_ray *rays, uint32_t n, const ckr_render_cfg *cfg, float *rgb,
                   void *stream);
/* The same with host buffers: copies in, shades, copies out, synchronises and
 * returns the scene's device status (ckr_scene_check). */
int ckr_shade_rays_host(ckr_scene *scene, const ckr_ray *rays, uint32_t n, const ckr_render_cfg *cfg, float *rgb,
                        void *stream);

/* Rendering that allocates no device memory.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc while they render: a
 * renderer embedded in a host application (an engine or a content tool) whose
 * device memory is handed out only by the host's own pool, real-time frame
 * loops that cannot take the device-wide synchronisation a cudaMalloc or
 * cudaFree may cause, and processes running so close to the memory limit that
 * an allocation in the middle of a frame could fail.  Same result as ckr_render with accum = NULL (up to the order of
 * the FP64 sums), for every shader; the scene must already exist.  Path
 * tracers run in fixed waves here (ckr_render may regenerate paths instead),
 * which changes only the order of the FP64 sums.  Like ckr_render it does not
 * wait for the GPU: traversal errors (a stack overflow, an iteration limit)
 * land in the scene's device status word, which the caller reads with
 * ckr_scene_check after the stream has run the call.  All scratch memory (path
 * state, queues, shadow rays, FP64 sums, an LTC table copy) lives in one
 * static device arena of 16 MiB plus 192 KiB, which every GPU that loads the
 * library holds until the process exits.  Limits: width * height <= 262144
 * pixels and <= 131072 shadow rays per path sample, else CKR_ERR_TOO_LARGE.
 * The first call on a device looks up the arena's device address and uploads
 * the LTC table with synchronous copies: make that first call before any
 * stream capture.  Every call uses the same arena, so calls that overlap on
 * the GPU (other streams or host threads) race: serialise them. */
int ckr_render_noalloc(ckr_scene *scene, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb,
                       void *stream);

/* ---- batched rendering (no reference counterpart) -------------------------
 * Many jobs of uneven resolution, spp and depth over one scene's geometry are
 * rendered in one pass: their paths are numbered consecutively, so the GPU stays
 * full across job boundaries.  Two renderers: PERSISTENT, one launch of a
 * persistent grid whose lanes each run a path's bounce loop (closest hit,
 * shading, shadow rays) and take the next path of the batch when theirs ends;
 * and WAVEFRONT, waves of paths with three launches per bounce over device-side
 * queues.  The pass (memsets, launches, resolve) has no host synchronisation; it
 * is captured once into a CUDA graph and replayed.  Each job may use its own
 * material table (same layout as the scene's, e.g. other sphere BRDFs).  The
 * renderer, block size and paths in flight come from an autotuner that times
 * candidates on a reduced copy of the batch (spp capped at 1). */
typedef struct ckr_job {
  ckr_camera cam;        /* resolution: cam.width x cam.height */
  uint32_t spp, max_depth;
  uint64_t seed;         /* per-pixel stream key = hash(seed, pixel) as in ckr_render */
  uint32_t material_set; /* index of the batch material table the job uses */
  uint32_t reserved;
  float *rgb;            /* device output, width x height x 3 floats, top row first */
} ckr_job;

#define CKR_BATCH_WAVEFRONT 0
#define CKR_BATCH_PERSISTENT 1 /* needs <= 4 shadow rays per vertex (lights x samples) */

typedef struct ckr_batch_tuning {
  uint32_t block;  /* threads per block: 64, 128 or 256 */
  uint32_t wave;   /* WAVEFRONT: paths per wave (queue capacity), >= 1024;
                      PERSISTENT: paths in flight (the grid's threads) */
  float ms;        /* autotuner: time of the reduced batch with these values */
  uint32_t candidates; /* autotuner: configurations timed */
  uint32_t mode;   /* CKR_BATCH_WAVEFRONT or CKR_BATCH_PERSISTENT */
} ckr_batch_tuning;

typedef struct ckr_batch ckr_batch;
/* shader: CKR_SHADER_PATH (n_light_samples per light, one BRDF sample) or
 * CKR_SHADER_PATH_NEE; rr_prob as in ckr_render_cfg.  materials: nsets tables of
 * the scene's material count each (NULL, 0: the scene's own, set 0).  tuning NULL:
 * autotune.  Jobs' rgb buffers are recorded in the graph: keep them alive. */
int ckr_batch_create(ckr_scene *scene, uint32_t shader, float rr_prob, uint32_t n_light_samples,
                     const ckr_material *materials, uint32_t nsets, const ckr_job *jobs, uint32_t njobs,
                     const ckr_batch_tuning *tuning, ckr_batch **out);
/* One replay of the captured graph on `stream` (asynchronous). */
int ckr_batch_render(ckr_batch *batch, void *stream);
/* The same jobs one after another with the batch's renderer, each with its own
 * launches (no packing across jobs, no graph): the baseline the batch is
 * measured against. */
int ckr_batch_render_sequential(ckr_batch *batch, void *stream);
int ckr_batch_get_tuning(const ckr_batch *batch, ckr_batch_tuning *out);
/* Paths (samples) per replay and launches in the captured graph. */
int ckr_batch_get_stats(const ckr_batch *batch, uint64_t *paths, uint32_t *launches);
int ckr_batch_destroy(ckr_batch *batch);

/* ---- learned light selection (no reference counterpart) -------------------
 * A proposal is a small network that maps a shading point (position, normal,
 * outgoing direction, GGX roughness) to a distribution over the scene's emitter
 * lights ("clusters", at most 64): 96 inputs (12-frequency sin/cos encoding of
 * the position normalised to the scene box, n, wo, alpha, 1), three hidden
 * layers of 64 with ReLU, softmax.  BF16 weights and activations, FP32
 * accumulation, evaluated and trained on the tensor cores.  The renderer draws
 * lights from (1 - defensive) * network + defensive * uniform and weights the
 * light sample against the BRDF sample by the balance heuristic, so estimates
 * stay unbiased whatever the network says.  Training is online: every bounce's
 * light samples (position, cluster, luminance of the unoccluded contribution /
 * pdf) feed one Adam step minimising the cross-entropy between the clusters'
 * contributions and the network's distribution. */
typedef struct ckr_proposal ckr_proposal;
typedef struct ckr_proposal_cfg {
  uint64_t seed;      /* weight initialisation stream */
  float lr;           /* Adam learning rate (1e-3) */
  float defensive;    /* uniform fraction of the selection mixture, (0, 1] (0.2) */
  uint32_t batch;     /* training records kept per bounce (65536) */
  uint32_t train;     /* 1: train while rendering */
  uint32_t minibatch; /* records per Adam step, batch / minibatch steps per bounce (16384; 0: batch) */
  uint32_t max_steps; /* training stops after this many Adam steps in total (0: never) */
} ckr_proposal_cfg;
#define CKR_PROPOSAL_NPARAMS 18624 /* W1[64][96], W2[64][64], b2, W3, b3, W4, b4 */

/* cfg NULL: the defaults above.  CKR_ERR_TOO_LARGE if the scene has more than 64
 * MESH/TRI lights, CKR_ERR_INVALID_ARGUMENT if it has none. */
int ckr_proposal_create(const ckr_scene *scene, const ckr_proposal_cfg *cfg, ckr_proposal **out);
int ckr_proposal_destroy(ckr_proposal *p);
int ckr_proposal_set_training(ckr_proposal *p, int train);
/* FP32 master weights (host buffers of CKR_PROPOSAL_NPARAMS floats); setting
 * them resets the optimiser state. */
int ckr_proposal_get_params(ckr_proposal *p, float *params);
int ckr_proposal_set_params(ckr_proposal *p, const float *params);
/* The position normalisation (p - centre) * scale and the number of clusters. */
int ckr_proposal_encoding(const ckr_proposal *p, float centre[3], float *scale, uint32_t *nclusters);
/* Direct use on caller records (device, 16-byte aligned, 12 floats each:
 * x.xyz, alpha, n.xyz, weight, wo.xyz, cluster index as uint32 bits): network
 * probabilities (FP16 bits, 64 per record), or one training step. */
int ckr_proposal_infer(ckr_proposal *p, const float *rec12, uint32_t n, uint16_t *probs, void *stream);
int ckr_proposal_train_step(ckr_proposal *p, const float *rec12, uint32_t n, void *stream);
/* Synchronises; Adam steps taken and the last step's loss.  Returns a device
 * error recorded by the network kernels (CKR_ERR_ITERATION_LIMIT), then clears it. */
int ckr_proposal_status(ckr_proposal *p, uint32_t *steps, float *last_loss);

/* ckr_render with cfg->shader = CKR_SHADER_PATH_NEE and lights drawn from the
 * proposal (trained online while rendering if its training flag is set). */
int ckr_render_learned(ckr_scene *scene, ckr_proposal *proposal, const ckr_camera *cam, const ckr_render_cfg *cfg,
                       float *rgb, double *accum, void *stream);

/* Rays traced by ckr_render on this scene since the last reset: closest-hit
 * rays (camera + continuation) and shadow rays.  Synchronises the device. */
int ckr_render_stats(ckr_scene *scene, uint64_t *closest_rays, uint64_t *shadow_rays, int reset);

/* Host form: rgb is host memory (w * h * 3 floats). */
int ckr_render_host(ckr_scene *scene, const ckr_camera *cam, const ckr_render_cfg *cfg, float *rgb, void *stream);

/* Scene XML (the reference's schema: SCREEN, CAMERA, MESHOBJECT, SPHEREOBJECT,
 * MESHSOURCE, TRISOURCE, POINTSOURCE, SPHERESOURCE).  Replaces
 * initSceneParser + prepareScreenCamera + prepareObjects + prepareLightSources
 * (headers/prepareScene.h:7-10, src/prepareScene.cpp, src/sceneParser.cpp):
 * objects first (with the reference's dummy sphere and degenerate dummy
 * triangle), then light sources, whose emitters are also visible primitives.
 * ckr_xml_get fills a ckr_scene_desc pointing into the loaded scene's arrays
 * (valid until ckr_xml_free) and the camera. */
typedef struct ckr_xml_scene ckr_xml_scene;
int ckr_xml_load(const char *path, ckr_xml_scene **out);
int ckr_xml_get(const ckr_xml_scene *scene, ckr_scene_desc *desc, ckr_camera *cam);
int ckr_xml_free(ckr_xml_scene *scene);

/* P3 PPM of src/main.cpp:98-117: clamp to [0, 1], gamma 1/2.2, int(x*255+.5). */
int ckr_write_ppm(const char *path, const float *rgb, uint32_t width, uint32_t height);

/* Binary P6 PPM, replacing readImage / writeImage (headers/ppm.h:6-7,
 * src/ppm.cpp:36-152; the reference reads and writes the fixed names env1.ppm
 * and env1_cpy.ppm).  Read: "P6", comment lines, width, height, maxval 255 (else
 * CKR_ERR_PARSE), then bytes b -> b / 255 into rgb (w * h * 3 floats, row 0 first);
 * rgb = NULL returns the size only, capacity_px < w * h gives CKR_ERR_TOO_LARGE.
 * Write: clamp to [0, 1] and truncate x * 255 (no gamma, as writeImage). */
int ckr_read_ppm_p6(const char *path, float *rgb, uint32_t capacity_px, uint32_t *width, uint32_t *height);
int ckr_write_ppm_p6(const char *path, const float *rgb, uint32_t width, uint32_t height);

/* HDR output (no reference counterpart; the reference writes only 8-bit P3):
 * linear FP32 PFM ("PF", little- or big-endian by the host, rows bottom to top)
 * of the same rgb layout as ckr_write_ppm (row 0 = top of the image). */
int ckr_write_pfm(const char *path, const float *rgb, uint32_t width, uint32_t height);

/* Wavefront OBJ geometry, written from the public format (the reference carries
 * an unused loader, externLib/objectLoader, and no OBJ asset): `v` vertices and
 * `f` polygons (corners v, v/vt, v//vn, v/vt/vn; 1-based or negative indices),
 * triangulated as fans; other statements skipped.  tri9 = NULL returns the
 * triangle count in *ntri; else up to `capacity` triangles (A.xyz B.xyz C.xyz)
 * are written and CKR_ERR_TOO_LARGE reports a short buffer.  CKR_ERR_IO: the file
 * cannot be read; CKR_ERR_PARSE: a malformed v or f line or an index out of range. */
int ckr_obj_load(const char *path, float *tri9, uint32_t capacity, uint32_t *ntri);

/* ---- LTC polygon-light shading ------------------------------------------ */
/* Loads the GGX LTC fit table (the reference's headers/ltc.inc, converted to
 * data/ltc_ggx.bin).  NULL: the copy beside libckr.so.  Optional: the first
 * shading call loads the default; call before it to use another file. */
int ckr_ltc_init(const char *table_path);

/* LTC shading of a G-buffer.  Replaces, per pixel,
 * LightSource::getLightFromMeshSource_Analytic (src/lightSources_CV.cpp:323-333)
 * with its helpers getLightAnalytic / getLightAnalyticDiffuse / clipTriangle /
 * integrateEdge (:8-321) and M_GGX + getBrdfApproxParam
 * (headers/ltc.h:18-61, src/materialTypes.cpp:52-74), for a GGX material with
 * specularCoef `spec`:
 *   rgb = spec * amplitude * sum_i L_i |I_ltc,i| / 2pi + (1 - spec) * sum_i L_i |I_cos,i| / 2pi
 * over the emitter triangles i of one mesh light.  Device buffers:
 * gbuf[npx] = 12 floats per pixel (pos.xyz, alpha, n.xyz, f0, v.xyz, spec),
 * v the unit direction towards the viewer (-ray.d), 16-byte aligned;
 * light_tri9[nlight] (A, B, C), light_rgb[nlight] radiance; rgb[npx] out
 * (3 floats).  f0 is not used by the LTC (the fit has no Fresnel term). */
int ckr_ltc_shade(const float *gbuf, uint32_t npx, const float *light_tri9, const float *light_rgb,
                  uint32_t nlight, float *rgb, void *stream);

/* Monte Carlo estimate of the integral ckr_ltc_shade approximates, per pixel of
 * the same G-buffer: the integral over the emitter triangles (two-sided and
 * unoccluded, as the LTC integral treats them) of MaterialType::brdf x cos x
 * radiance for the GGX material (alpha, spec) of the pixel.  spp samples
 * (even, >= 2): half pick an emitter point by area, half follow
 * getBrdfDirectionSampleRandomized; balance-heuristic MIS; FP32 arithmetic,
 * FP64 per-pixel sums.  fresnel = 0 sets F = 1 (IOR 1e5), the lobe the LTC fit
 * models; fresnel = 1 takes the IOR from f0: (1 + sqrt f0) / (1 - sqrt f0).
 * Random numbers: counter 4s..4s+2 of the stream (seed, pixel).  rgb receives
 * npx x 3 doubles (device).  nlight <= 256 (CKR_ERR_TOO_LARGE above).
 * No reference counterpart: the LTC's high-spp reference. */
int ckr_ltc_mc(const float *gbuf, uint32_t npx, const float *light_tri9, const float *light_rgb, uint32_t nlight,
               uint32_t spp, uint64_t seed, int fresnel, double *rgb, void *stream);

/* ---- synthetic workloads (deterministic; no reference counterpart) ----- */
/* G-buffer for LTC shading (12 floats per pixel as ckr_ltc_shade reads them):
 * pos uniform in [-1,1]^3, n uniform on the +z hemisphere, v cosine-distributed
 * about n, alpha uniform in [0.05,1], f0 uniform in [0.02,0.9], spec uniform
 * in [0,1). */
int ckr_workload_gbuffer(uint64_t seed, uint32_t npx, float *out12);

/* Axis-aligned square emitters facing -z: side uniform in [side_lo, side_hi],
 * centre uniform in [-2,2]^2 x [1,3]; two triangles per quad (tri9_out gets
 * 2*nquads rows), each with radiance (r, r, r). */
int ckr_workload_quad_lights(uint64_t seed, uint32_t nquads, float side_lo, float side_hi, float radiance,
                             float *tri9_out, float *rgb_out);

/* Icosphere: the 20-face icosahedron, `subdiv` midpoint subdivisions
 * (20 * 4^subdiv triangles), vertices pushed to radius
 * 1 + noise_amp * fbm(p), fbm = `octaves` octaves of seeded 3-D value noise
 * (base frequency 2, lacunarity 2, gain 0.5) normalised to [-1, 1]. */
int ckr_workload_icosphere(uint32_t subdiv, float noise_amp, uint32_t octaves,
                           uint64_t seed, float *tri9_out, uint32_t capacity,
                           uint32_t *ntri_out);

/* Pinhole camera rays through pixel centres, row-major from the top-left
 * pixel, vertical field of view vfov_deg, square pixels; tmin 0. */
int ckr_workload_rays_pinhole(const float eye[3], const float target[3], const float up[3],
                              float vfov_deg, uint32_t width, uint32_t height, float tmax,
                              ckr_ray *out);

/* Incoherent rays: origins uniform in the box [lo, hi], directions uniform on
 * the unit sphere (Marsaglia 1972), tmax uniform in [tmax_lo, tmax_hi];
 * ray i is a function of (seed, i) only. */
int ckr_workload_rays_incoherent(const float lo[3], const float hi[3], uint64_t seed,
                                 uint32_t n, float tmax_lo, float tmax_hi, ckr_ray *out);

/* Many-light scene: the displaced icosphere of ckr_workload_icosphere
 * (GGX, F = 1, specularCoef mesh_spec, roughness uniform in [alpha_lo, alpha_hi]
 * per triangle from stream rough_seed) inside the room [-5,5] x
 * [floor_y, floor_y + 10] x [-5,5] (Lambertian, albedo room_albedo).  nemit
 * equilateral emitters of side emit_side lie 1e-3 inside the ceiling and the four
 * walls (face, position, rotation from stream (emit_seed, i)), radiance
 * log-uniform in [radiance_lo, radiance_hi], grouped by 20 Lloyd iterations of
 * k-means on their centroids into nclusters mesh lights.  Triangle order: mesh,
 * room (12), emitters by cluster.  Materials: one per mesh triangle, the room,
 * one per emitter.  counts receives (ntri, nmaterials, nlights); with tri9 NULL
 * only counts is written (size query). */
typedef struct ckr_manylight_spec {
  uint32_t subdiv, octaves;
  float noise_amp;
  uint64_t mesh_seed, rough_seed, emit_seed;
  float alpha_lo, alpha_hi, mesh_spec, mesh_albedo, room_albedo, floor_y;
  uint32_t nemit, nclusters;
  float emit_side, radiance_lo, radiance_hi;
  float cam_pos[3], cam_target[3], fov_deg;
  uint32_t width, height;
} ckr_manylight_spec;
int ckr_workload_manylight(const ckr_manylight_spec *spec, float *tri9, uint32_t *tri_material,
                           ckr_material *materials, ckr_light *lights, ckr_camera *cam, uint32_t counts[3]);

/* The library's counter-based stream (see csrc/ckr_rng.h), for checkers. */
float ckr_rng_uniform(uint64_t seed, uint64_t index, uint32_t counter);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
