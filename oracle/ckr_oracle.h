/*
 * ckr_oracle.h — CPU oracle for the ChakumRender path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code: it is the checker that the parity tests, the smoke check
 * and the CPU-baseline leg of bench.py compare the CUDA path against.
 *
 * Everything here is a plain-C FP64 restatement of the reference renderer
 * (Sayantan2048/ChakumRender, C++98, FP64).  Each function names the
 * reference file:line it follows.  The restatement is pinned against the
 * reference itself: oracle/Makefile compiles the reference's own sources
 * into oracle/_ref/libckr_ref.so and tests/test_oracle_pin.py checks that
 * both give identical answers (bit-identical hit ids and t for traversal).
 *
 * Build with -ffp-contract=off so that x86-64 and aarch64 round identically.
 */
#ifndef CKR_ORACLE_H
#define CKR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INF 1e20 /* headers/mathPrimitives.h:5 */
#define ORC_MISS 0xFFFFFFFFu

/* ---------------------------------------------------------------------- */
/* Traversal: midpoint BVH over FP64 triangles (src/bvhAccel.cpp).        */
/* ---------------------------------------------------------------------- */
typedef struct orc_bvh orc_bvh;

/* Build the reference's BVH (centroid-midpoint split, one primitive per leaf,
 * src/bvhAccel.cpp:13-149) over ntri triangles given as 9 floats each
 * (A.xyz, B.xyz, C.xyz).  Returns NULL on allocation failure. */
orc_bvh *orc_bvh_build(const float *tri9, uint32_t ntri);
void orc_bvh_free(orc_bvh *b);
uint32_t orc_bvh_node_count(const orc_bvh *b);

/* Rays are 8 floats: ox oy oz tmin dx dy dz tmax (tmin/tmax are ignored by the
 * closest-hit query, which, like BvhAccel::intersectT, has no t range).
 * hit_id receives the ORIGINAL triangle index (ORC_MISS on a miss) and hit_t
 * the FP64 distance (ORC_INF on a miss).  nodes/tris, when non-NULL, receive
 * per-ray counts of node visits and triangle tests.  threads<=0: all cores. */
void orc_trace_closest(const orc_bvh *b, const float *rays8, uint32_t nrays,
                       uint32_t *hit_id, double *hit_t,
                       uint32_t *nodes, uint32_t *tris, int threads);

/* BvhAccel::intersectT for one FP64 ray: input triangle index or ORC_MISS. */
uint32_t orc_bvh_closest1(const orc_bvh *b, const double *o3, const double *d3, double *t);

/* shadow() semantics (src/shader.cpp:76-97) for a triangle-only scene:
 * occluded[i] = 1 iff the closest triangle hit t satisfies t + 1e-5 < dist,
 * with dist = tmax + 1e-5 so that "occluded" means a hit with t < tmax. */
void orc_trace_shadow(const orc_bvh *b, const float *rays8, uint32_t nrays,
                      uint8_t *occluded, int threads);

/* Triangle::intersect (src/geometryPrimitives.cpp:29-71) on one triangle, plus
 * the barycentric margin min(beta, gamma, 1-beta-gamma) (negative: outside)
 * and |d.n| (the reference rejects rays with (d.n)^2 <= 1e-10). */
double orc_tri_intersect(const float *tri9, const float *ray8, double *margin,
                         double *ddotn);

/* Sphere::intersect (src/geometryPrimitives.cpp:12-27). */
double orc_sphere_intersect(const double *c3, double r, const double *o3,
                            const double *d3);

/* Signed distance from the ray's plane hit point to the triangle boundary
 * (negative inside); t_plane receives the plane distance. */
double orc_tri_edge_distance(const float *tri9, const float *ray8, double *t_plane);

/* Nearest sphere per ray (sph4: centre.xyz, radius); ORC_MISS / ORC_INF on a miss. */
void orc_spheres_closest(const float *sph4, uint32_t nsph, const float *rays8, uint32_t nrays,
                         uint32_t *hit_id, double *hit_t);

/* ---------------------------------------------------------------------- */
/* Materials, samplers and LTC shading (orc_shading.c).                   */
/* ---------------------------------------------------------------------- */
/* MaterialType (headers/materialTypes.h:21-98); brdf uses the reference's
 * BRDFType numbering: 0 NONE, 1 CLASSIC_PHONG, 2 GGX, 3 BECKMANN, 4 PHONG,
 * 5 GGXAPPROX.  `spec` is specularCoef. */
typedef struct orc_material {
  int32_t brdf;
  int32_t pad;
  double alpha, phong_exp, spec, int_ior, ext_ior;
} orc_material;

/* Loads the LTC fit table (chakumrender_gb300/data/ltc_ggx.bin). 0 on success. */
int orc_ltc_load(const char *path);
/* M_GGX (headers/ltc.h:18-61): lerped M (row-major, stale det of the lower
 * theta entry), lerped Minv, lerped amplitude. */
void orc_m_ggx(float theta, float alpha, double *M9, double *detM, double *Minv9, double *amplitude);
/* MaterialType::brdf and ::pdfEval per row (vectors are 3 doubles per row).
 * use_ltc: evaluate the LTC-approximate branch with getBrdfApproxParam(force). */
void orc_brdf_batch(const orc_material *m, uint32_t count, const double *n, const double *wo_ref, const double *wo,
                    const double *wi, int use_ltc, double *brdf_out, double *pdf_out);
/* getLightFromMeshSource_Analytic for one shading point (x, n, v = -r.d). */
void orc_ltc_shade(const orc_material *m, const double *x3, const double *n3, const double *v3,
                   const float *light_tri9, const float *light_rgb, uint32_t nlight, double *rgb);
void orc_ltc_shade_batch(const orc_material *m, uint32_t count, const double *x, const double *n, const double *v,
                         const float *light_tri9, const float *light_rgb, uint32_t nlight, double *rgb, int threads);
/* Monte Carlo reference for the LTC integral (ckr_ltc_mc of the library in FP64):
 * spp samples per point (even: emitter area, odd: BRDF), balance heuristic,
 * random stream (seed, pixel_index[i] or i).  rgb: count x 3 doubles. */
void orc_ltc_mc(const orc_material *m, uint32_t count, const double *x, const double *n, const double *v,
                const float *light_tri9, const float *light_rgb, uint32_t nlight, uint32_t spp, uint64_t seed,
                const uint32_t *pixel_index, double *rgb, int threads);
/* Renders with the reference's shaders restated in FP64 (see orc_render.inc):
 * desc/cam/cfg are the library's ABI structs (include/ckr.h); rgb receives
 * width*height*3 doubles, top row first, the mean over cfg->spp. */
struct ckr_scene_desc;
struct ckr_camera;
struct ckr_render_cfg;
void orc_render(const struct ckr_scene_desc *desc, const struct ckr_camera *cam, const struct ckr_render_cfg *cfg,
                double *rgb, int threads);

/* Environment light (EnvSource restated): radiance + luminance per direction and
 * the luminance integral; directions drawn from uniforms (3 per sample). */
struct ckr_env_light;
void orc_env_eval(const struct ckr_env_light *e, const double *dirs, uint32_t n, double *rgbl, double *area);
void orc_env_sample(const struct ckr_env_light *e, const double *u, uint32_t n, double *dirs);

/* ---------------------------------------------------------------------- */
/* Learned light-selection network (orc_mlp.c; no reference counterpart).  */
/* ---------------------------------------------------------------------- */
#define ORC_MLP_IN 96
#define ORC_MLP_HIDDEN 64
#define ORC_MLP_OUT 64
#define ORC_MLP_FREQS 12
#define ORC_MLP_NPARAMS (64 * 96 + 3 * (64 * 64 + 64))
/* The 96 input features of one 12-float record. */
void orc_mlp_features(const float *rec12, const double *centre, double scale, double *f96);
/* probs: n x 64, softmax over the first nclusters outputs (the rest 0). */
void orc_mlp_forward(const double *params, const float *rec12, uint32_t n, const double *centre, double scale,
                     uint32_t nclusters, double *probs);
/* Loss and its gradient over n records; returns 0 (and zeros) when the weights sum to 0. */
int orc_mlp_loss_grad(const double *params, const float *rec12, uint32_t n, const double *centre, double scale,
                      uint32_t nclusters, double *grad, double *loss);
/* One Adam step (step = 1, 2, ...). */
void orc_mlp_adam(double *params, double *m, double *v, const double *grad, uint32_t n, uint32_t step, double lr,
                  double beta1, double beta2, double eps);

/* ---------------------------------------------------------------------- */
/* The synthetic traversal workload (orc_workload.c; no reference          */
/* counterpart): byte-identical to the library's ckr_workload_* outputs.   */
/* ---------------------------------------------------------------------- */
/* Icosphere with subdiv levels, radially displaced by fractal value noise;
 * tri9_out NULL: size query.  0 on success, negative on error. */
int orc_workload_icosphere(uint32_t subdiv, float noise_amp, uint32_t octaves, uint64_t seed, float *tri9_out,
                           uint32_t capacity, uint32_t *ntri_out);
/* width x height pinhole rays (8 floats each), top row first. */
int orc_workload_rays_pinhole(const float eye[3], const float target[3], const float up[3], float vfov_deg,
                              uint32_t width, uint32_t height, float tmax, float *rays8);
/* n rays with origins uniform in [lo, hi] and directions uniform on the sphere. */
int orc_workload_rays_incoherent(const float lo[3], const float hi[3], uint64_t seed, uint32_t n, float tmax_lo,
                                 float tmax_hi, float *rays8);

/* One direction sample from uniforms (e1, e2); see orc_shading.c for `kind`. */
void orc_sample_dir(int kind, const double *n3, const double *w3, double param, double e1, double e2, double *out3);

#ifdef __cplusplus
}
#endif
#endif
