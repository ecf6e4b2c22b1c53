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

/* The network's loss and gradients on n 12-float records in device memory,
 * computed by the tensor-core training kernels without an Adam step. */
int ckr_internal_proposal_gradients(ckr_proposal *p, const float *rec12, uint32_t n, float *grad, float *loss);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
