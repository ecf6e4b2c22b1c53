/*
 * ckr_test.h — test hooks of libckr.so.  Not part of the drop-in interface and
 * with no counterpart in the reference: the library's parity tests call these
 * to check host-side restatements of device code (BRDF, LTC shading, BVH
 * replay) and the network's gradients against the CPU oracle.  Same
 * conventions as ckr.h (int status, plain pointers, no exceptions).
 */
#ifndef CKR_TEST_H
#define CKR_TEST_H
#include "ckr.h"

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* BVH build + traversal replayed on the host: per-ray hit id / t (any: occlusion
 * only) and the mean wide nodes / triangles visited. */
int ckr_internal_replay(const float *tri9, uint32_t ntri, uint32_t max_leaf, const ckr_ray *rays, uint32_t n,
                        int any, uint32_t *hit_id, float *hit_t, double *mean_nodes, double *mean_tris);

/* 64-bit digest of the built BVH (nodes + triangle order) with `threads` build
 * threads: the build must not depend on the thread count. */
int ckr_internal_bvh_digest(const float *tri9, uint32_t ntri, uint32_t max_leaf, uint32_t threads, uint64_t *digest,
                            uint32_t *nnodes);

/* The device BRDF / pdf code compiled for the host, per row. */
int ckr_internal_brdf_host(const ckr_material *mats, uint32_t count, const float *n, const float *wo_ref,
                           const float *wo, const float *wi, float *brdf, float *pdf);
/* The LTC-approximate BRDF branch on the host, per row. */
int ckr_internal_brdf_ltc_host(const ckr_material *mats, uint32_t count, const float *n, const float *wo,
                               const float *wi, float *brdf);
/* LTC polygon-light shading on the host (the device kernel's per-pixel code). */
int ckr_internal_ltc_shade_host(const float *gbuf, uint32_t npx, const float *light_tri9, const float *light_rgb,
                                uint32_t nlight, float *rgb);
/* The edge integral's theta / sin(theta) at theta = acos(c) (the polynomial of
 * theta_over_sin) on the host, per value. */
int ckr_internal_theta_over_sin_host(const float *c, uint32_t n, float *out);

/* The network's loss and gradients on n 12-float records in device memory,
 * computed by the tensor-core training kernels without an Adam step. */
int ckr_internal_proposal_gradients(ckr_proposal *p, const float *rec12, uint32_t n, float *grad, float *loss);

/* Failure paths, driven without a GPU fault.  The next ckr_render on `scene`
 * runs with a shadow queue of at most `capacity` rays: shading steps that need
 * more drop their rays and the scene's status word reports
 * CKR_ERR_QUEUE_OVERFLOW (ckr_scene_check); later renders size the queue
 * normally. */
int ckr_internal_limit_shadow_queue(ckr_scene *scene, uint32_t capacity);

/* One inference over n records whose first layer's MMAs are never issued, so
 * every tile waits on an mbarrier phase that nothing completes; each wait gives
 * up after `wait_tries` polls, the kernel records CKR_ERR_ITERATION_LIMIT
 * (ckr_proposal_status) and frees its tensor memory.  The next call runs
 * normally. */
int ckr_internal_proposal_infer_stalled(ckr_proposal *p, const float *rec12, uint32_t n, uint16_t *probs,
                                        uint32_t wait_tries, void *stream);

/* Batch autotuner under scarce device memory: from now on (process-wide), a
 * wavefront workspace of more than `bytes` fails as if cudaMalloc had run out
 * (0 removes the cap).  The autotuner must then keep the best candidate that fits,
 * and fail with CKR_ERR_OUT_OF_MEMORY only when none does. */
int ckr_internal_batch_workspace_cap(uint64_t bytes);

/* Draws `count` samples from the renderer's device samplers (the functions the
 * shading kernels call), sample i from the stream (seed, i), into out4 (device,
 * 16-byte aligned, 4 floats per sample): direction and its density for the
 * direction samplers, the point and 0 for the triangle.
 *   CKR_PROBE_BRDF        sample_brdf for material `mat` at normal n, outgoing wo
 *                         (mirror direction 2(n.wo)n - wo); density pdf_eval
 *   CKR_PROBE_COSINE      cosine-weighted about n; cos / pi
 *   CKR_PROBE_HEMISPHERE  uniform on n's hemisphere; 1 / 2 pi
 *   CKR_PROBE_CONE        uniform in the cone about n with cos(theta_max) = param
 *   CKR_PROBE_TRIANGLE    uniform point on tri9 (A, B, C) */
#define CKR_PROBE_BRDF 0
#define CKR_PROBE_COSINE 1
#define CKR_PROBE_HEMISPHERE 2
#define CKR_PROBE_CONE 3
#define CKR_PROBE_TRIANGLE 4
int ckr_internal_sample_probe(int kind, const ckr_material *mat, const float n[3], const float wo[3],
                              const float tri9[9], float param, uint64_t seed, uint32_t count, float *out4,
                              void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
