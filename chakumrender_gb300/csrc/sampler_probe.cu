// sampler_probe.cu — draws directions from the renderer's device samplers for the
// statistical tests (test hook, declared in include/ckr_test.h).
//
// Each draw i uses the renderer's counter-based stream (seed, i) for its three
// uniforms and calls the same device functions the shading kernels call
// (shading_device.cuh): sample_brdf (the one-sample mixture of the specular lobe
// and cosine sampling, getBrdfDirectionSampleRandomized), sample_cosine,
// sample_hemisphere, sample_cone and sample_triangle.  For direction samplers the
// output row is (direction, pdf_eval of that direction); for the triangle it is
// (point, 0).
#include "ckr_internal.h"
#include "ckr_rng.h"
#include "ckr_test.h"
#include "shading_device.cuh"

namespace ckr {
namespace {

__global__ void k_sample_probe(int kind, Material m, F3 n, F3 wo, F3 a, F3 b, F3 c, float param, uint64_t seed,
                               uint32_t count, float4 *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint64_t key = ckr_key(seed, i);
    const float e0 = ckr_draw_f(key, 0), e1 = ckr_draw_f(key, 1), e2 = ckr_draw_f(key, 2);
    F3 w = f3(0, 0, 0);
    float pdf = 0.f;
    const F3 wo_ref = n * (2.0f * dot(n, wo)) - wo;
    switch (kind) {
      case CKR_PROBE_BRDF:
        w = sample_brdf(m, n, wo_ref, wo, e0, e1, e2);
        pdf = pdf_eval(m, n, wo_ref, wo, w);
        break;
      case CKR_PROBE_COSINE:
        w = sample_cosine(n, e1, e2);
        pdf = dot(w, n) / kPi;
        break;
      case CKR_PROBE_HEMISPHERE:
        w = sample_hemisphere(n, e1, e2);
        pdf = 1.0f / (2.0f * kPi);
        break;
      case CKR_PROBE_CONE:
        w = sample_cone(n, param, e1, e2);
        pdf = 1.0f / (2.0f * kPi * (1.0f - param));
        break;
      default:  // CKR_PROBE_TRIANGLE
        w = sample_triangle(a, b, c, e1, e2);
        break;
    }
    out[i] = make_float4(w.x, w.y, w.z, pdf);
  }
}

}  // namespace
}  // namespace ckr

extern "C" int ckr_internal_sample_probe(int kind, const ckr_material *mat, const float n[3], const float wo[3],
                                         const float tri9[9], float param, uint64_t seed, uint32_t count,
                                         float *out4, void *stream) {
  using namespace ckr;
  if (kind < CKR_PROBE_BRDF || kind > CKR_PROBE_TRIANGLE || !out4 || count == 0 ||
      (reinterpret_cast<uintptr_t>(out4) & 15u))
    return CKR_ERR_INVALID_ARGUMENT;
  if ((kind == CKR_PROBE_BRDF && (!mat || !n || !wo)) || (kind == CKR_PROBE_TRIANGLE && !tri9) ||
      (kind != CKR_PROBE_TRIANGLE && !n))
    return CKR_ERR_INVALID_ARGUMENT;
  Material m{};
  if (mat) {
    m.brdf = mat->brdf;
    m.alpha = mat->alpha;
    m.phong_exp = mat->phong_exp;
    m.spec = mat->spec;
    m.int_ior = mat->int_ior;
    m.ext_ior = mat->ext_ior;
  }
  const F3 nn = n ? f3(n[0], n[1], n[2]) : f3(0, 0, 1), ww = wo ? f3(wo[0], wo[1], wo[2]) : f3(0, 0, 1);
  const F3 A = tri9 ? f3(tri9[0], tri9[1], tri9[2]) : f3(0, 0, 0), B = tri9 ? f3(tri9[3], tri9[4], tri9[5]) : A,
           C = tri9 ? f3(tri9[6], tri9[7], tri9[8]) : A;
  const unsigned grid = std::min<unsigned>(4096, ceil_div(count, 256));
  k_sample_probe<<<grid, 256, 0, (cudaStream_t)stream>>>(kind, m, nn, ww, A, B, C, param, seed, count,
                                                         reinterpret_cast<float4 *>(out4));
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}
