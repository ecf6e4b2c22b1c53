// ltc.cu — LTC polygon-light shading of a G-buffer (getLightFromMeshSource_Analytic,
// src/lightSources_CV.cpp:323-333, per pixel).
//
// The kernel is FP32-ALU bound (per pixel and emitter triangle: three
// transformed vertices, horizon clipping, 3-4 edge integrals with acos/sin,
// for both the specular LTC lobe and the diffuse cosine lobe).  The 64x64 LTC
// table (Minv's five non-zeros + amplitude, 96 KB) is staged once per CTA into
// shared memory; CTAs are persistent (one or two per SM) and stride over pixels.
// Emitter triangles are read through the read-only path (every thread of a warp
// reads the same triangle, a broadcast).
#include <algorithm>

#include "ckr_internal.h"
#include "ltc_table.h"
#include "shading_device.cuh"

namespace ckr {
namespace {

constexpr int kLtcTPB = 256;

struct SmemTable {
  const float4 *a;  // mi0 mi2 mi4 mi6
  const float2 *b;  // mi8 amp
  SHD LtcEntry operator()(int i) const {
    float4 x = a[i];
    float2 y = b[i];
    LtcEntry e;
    e.mi0 = x.x; e.mi2 = x.y; e.mi4 = x.z; e.mi6 = x.w; e.mi8 = y.x; e.amp = y.y;
    e.m0 = e.m2 = e.m4 = e.m6 = e.m8 = e.det = 0.f;
    return e;
  }
};

__global__ void __launch_bounds__(kLtcTPB, 2) k_ltc_shade(const float4 *__restrict__ gbuf, uint32_t npx,
                                                       const float *__restrict__ light_tri9,
                                                       const float *__restrict__ light_rgb, uint32_t nlight,
                                                       float *__restrict__ rgb, const LtcEntry *__restrict__ table) {
  extern __shared__ float4 smem[];
  float4 *sa = smem;
  float2 *sb = reinterpret_cast<float2 *>(smem + 4096);
  for (int i = threadIdx.x; i < 4096; i += kLtcTPB) {
    const LtcEntry &e = table[i];
    sa[i] = make_float4(e.mi0, e.mi2, e.mi4, e.mi6);
    sb[i] = make_float2(e.mi8, e.amp);
  }
  __syncthreads();
  SmemTable tab{sa, sb};
  auto light = [&](uint32_t k, F3 &A, F3 &B, F3 &C, float *c) {
    const float *t = light_tri9 + 9 * (size_t)k;
    A = f3(__ldg(t), __ldg(t + 1), __ldg(t + 2));
    B = f3(__ldg(t + 3), __ldg(t + 4), __ldg(t + 5));
    C = f3(__ldg(t + 6), __ldg(t + 7), __ldg(t + 8));
    c[0] = __ldg(light_rgb + 3 * k);
    c[1] = __ldg(light_rgb + 3 * k + 1);
    c[2] = __ldg(light_rgb + 3 * k + 2);
  };
  for (uint32_t p = blockIdx.x * kLtcTPB + threadIdx.x; p < npx; p += gridDim.x * kLtcTPB) {
    float4 g0 = gbuf[3 * (size_t)p], g1 = gbuf[3 * (size_t)p + 1], g2 = gbuf[3 * (size_t)p + 2];
    float out[3];
    ltc_shade_point(tab, f3(g0.x, g0.y, g0.z), f3(g1.x, g1.y, g1.z), f3(g2.x, g2.y, g2.z), g0.w, g2.w, nlight,
                    light, out);
    rgb[3 * (size_t)p] = out[0];
    rgb[3 * (size_t)p + 1] = out[1];
    rgb[3 * (size_t)p + 2] = out[2];
  }
}

}  // namespace
}  // namespace ckr

using namespace ckr;

extern "C" int ckr_ltc_shade(const float *gbuf, uint32_t npx, const float *light_tri9, const float *light_rgb,
                             uint32_t nlight, float *rgb, void *stream) {
  if ((npx && (!gbuf || !rgb)) || (nlight && (!light_tri9 || !light_rgb)) || ((uintptr_t)gbuf & 15u))
    return CKR_ERR_INVALID_ARGUMENT;
  if (npx == 0) return CKR_OK;
  int st = CKR_OK;
  const LtcEntry *table = device_ltc_table(&st);
  if (!table) return st;
  const size_t smem = 4096 * (sizeof(float4) + sizeof(float2));
  static bool attr_set[64] = {false};
  int dev = 0, sms = 0, per_sm = 0;
  CKR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(k_ltc_shade, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set[dev] = true;
  }
  CKR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CKR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ltc_shade, kLtcTPB, smem));
  if (per_sm < 1) return CKR_ERR_CUDA;
  int grid = (int)std::min<uint64_t>(ceil_div(npx, kLtcTPB), (uint64_t)sms * per_sm);
  k_ltc_shade<<<grid, kLtcTPB, smem, (cudaStream_t)stream>>>(reinterpret_cast<const float4 *>(gbuf), npx, light_tri9,
                                                               light_rgb, nlight, rgb, table);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}
