// mlp.cu — the learned light-selection network on the fifth-generation tensor
// cores: inference (k_mlp_infer), training forward + backward (k_mlp_train) and
// the Adam update (k_mlp_adam), all for tiles of 128 rows.
//
// One CTA of 128 threads owns a tile: thread t computes row t's features and
// epilogues, thread 0 issues the tcgen05.mma chain of each layer (M = 128 rows,
// N = 64 outputs, K = 96 or 64 in steps of 16) into tensor memory and commits it
// to an mbarrier that the CTA waits on with a bounded poll.  Row t of the
// accumulator lives in TMEM lane t, which warp t / 32 reads with tcgen05.ld.
//
// Backward pass, per layer l with input activations X (rows b) and output
// gradient G (rows b):  dW^T = X^T G  (M = input features padded to 128,
// N = 64, K = the 128 rows of the tile), accumulated in TMEM across all tiles a
// CTA processes, and dX = G W  (M = 128 rows, N = 64, K = 64) for the layer
// below.  The transposed operands X^T and G^T are written to shared memory by
// the epilogues.  Row 64 of X^T is all ones, so row 64 of dW^T is the bias
// gradient (the first layer's bias is the weight of its constant feature).
//
// Bounds: every mbarrier wait gives up after kWaitTries polls, records
// CKR_ERR_ITERATION_LIMIT, waits once more (bounded) for the MMAs in flight,
// frees the CTA's tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ckr_internal.h"
#include "ckr_rng.h"
#include "mlp.h"
#include "tc05.cuh"

namespace ckr {
namespace mlp {
namespace {

constexpr uint32_t kTPB = 128;
constexpr uint32_t kWaitTries = 1u << 22;
constexpr uint32_t kIdesc = tc::idesc_bf16(128, 64);

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&h);
}
__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xFFFF0000u); }

// Writes 8 consecutive K entries (k0 % 8 == 0) of row r of a K-major operand.
__device__ __forceinline__ void st8(uint8_t *op, uint32_t r, uint32_t k0, uint32_t K, const float *v) {
  uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
  *reinterpret_cast<uint4 *>(op + tc::kmaj(r, k0, K)) = q;
}
__device__ __forceinline__ void ld8(const uint8_t *op, uint32_t r, uint32_t k0, uint32_t K, float *v) {
  uint4 q = *reinterpret_cast<const uint4 *>(op + tc::kmaj(r, k0, K));
  v[0] = bf16_lo(q.x); v[1] = bf16_hi(q.x); v[2] = bf16_lo(q.y); v[3] = bf16_hi(q.y);
  v[4] = bf16_lo(q.z); v[5] = bf16_hi(q.z); v[6] = bf16_lo(q.w); v[7] = bf16_hi(q.w);
}
__device__ __forceinline__ void st1(uint8_t *op, uint32_t r, uint32_t k, uint32_t K, float v) {
  *reinterpret_cast<__nv_bfloat16 *>(op + tc::kmaj(r, k, K)) = __float2bfloat16_rn(v);
}

// Rows to process: n_max, or what the device count leaves after n_off.
__device__ __forceinline__ uint32_t rows(uint32_t n_max, const uint32_t *n_dev, uint32_t n_off) {
  if (!n_dev) return n_max;
  const uint32_t c = *n_dev;
  return c > n_off ? min(c - n_off, n_max) : 0u;
}

struct Params {
  float cx, cy, cz, scale;
  uint32_t nclusters;
};

// Row features into the first-layer operand (K = 96).
__device__ __forceinline__ void write_features(uint8_t *x0, uint32_t t, float4 r0, float4 r1, float4 r2,
                                               const Params &p) {
  float f[kIn];
  const float pc[3] = {(r0.x - p.cx) * p.scale, (r0.y - p.cy) * p.scale, (r0.z - p.cz) * p.scale};
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int k = 0; k < (int)kFreqs; ++k) sincospif(ldexpf(pc[c], k), &f[24 * c + 2 * k], &f[24 * c + 2 * k + 1]);
  f[72] = r1.x; f[73] = r1.y; f[74] = r1.z;
  f[75] = r2.x; f[76] = r2.y; f[77] = r2.z;
  f[78] = r0.w;
  f[79] = 1.0f;
#pragma unroll
  for (int j = 80; j < (int)kIn; ++j) f[j] = 0.f;
#pragma unroll
  for (int q = 0; q < (int)kIn / 8; ++q) st8(x0, t, 8 * q, kIn, f + 8 * q);
}

// Accumulator row (64 columns) + bias, ReLU, into row t of a K = 64 operand.
__device__ __forceinline__ void epilogue_relu(uint32_t taddr, const float *bias, uint8_t *dst, uint32_t t) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[32];
    tc::tmem_ld32(taddr + 32 * h, v);
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j] + (bias ? bias[32 * h + j] : 0.f), 0.f);
#pragma unroll
    for (int q = 0; q < 4; ++q) st8(dst, t, 32 * h + 8 * q, 64, v + 8 * q);
  }
}

// Softmax over the first C logits (accumulator + bias) of row t.
__device__ __forceinline__ void softmax_row(uint32_t taddr, const float *bias, uint32_t C, float *p) {
  tc::tmem_ld32(taddr, p);
  tc::tmem_ld32(taddr + 32, p + 32);
  float mx = -3.0e38f;
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    p[j] += bias[j];
    if ((uint32_t)j < C) mx = fmaxf(mx, p[j]);
  }
  float sum = 0.f;
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    p[j] = (uint32_t)j < C ? __expf(p[j] - mx) : 0.f;
    sum += p[j];
  }
  const float inv = 1.0f / sum;
#pragma unroll
  for (int j = 0; j < 64; ++j) p[j] *= inv;
}

__device__ __forceinline__ void issue(uint32_t d, uint32_t a, uint32_t b, uint32_t K, uint32_t accumulate_first) {
  for (uint32_t s = 0; s < K / 16; ++s)
    tc::mma_bf16(d, tc::sdesc(a, K, s), tc::sdesc(b, K, s), kIdesc, (s > 0 || accumulate_first) ? 1u : 0u);
}

// Every thread: shared-memory writes visible to the tensor core, TMEM reads done.
__device__ __forceinline__ void sync_for_mma() {
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
}

// Waits for the committed MMAs; false (uniformly) when the wait gave up.
__device__ __forceinline__ bool wait_mma(uint32_t mbar, uint32_t &phase, int *abort, int *err) {
  if (!tc::mbar_wait(mbar, phase, kWaitTries)) {
    *abort = 1;
    atomicExch(err, CKR_ERR_ITERATION_LIMIT);
  }
  __syncthreads();
  if (*abort) {
    tc::mbar_wait(mbar, phase, kWaitTries);  // let the MMAs in flight land before TMEM is freed
    return false;
  }
  phase ^= 1u;
  tc::fence_after_sync();
  return true;
}

// ---- inference ------------------------------------------------------------------
struct SmemInfer {
  uint8_t w[kImgForward];
  uint8_t a[128 * kIn * 2];
  float b[3][64];
  uint64_t mbar;
  uint32_t tmem;
  int abort;
};

__global__ void __launch_bounds__(kTPB) k_mlp_infer(const float4 *__restrict__ rec, uint32_t n_max,
                                                    const uint32_t *n_dev, uint32_t n_off,
                                                    const uint8_t *__restrict__ img,
                                                    const float *__restrict__ params, Params p,
                                                    __half *__restrict__ probs, int *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  SmemInfer &S = *reinterpret_cast<SmemInfer *>(smem_raw);
  const uint32_t t = threadIdx.x, warp = t >> 5;
  for (uint32_t i = t; i < kImgForward / 16; i += kTPB)
    reinterpret_cast<uint4 *>(S.w)[i] = reinterpret_cast<const uint4 *>(img)[i];
  for (uint32_t i = t; i < 64; i += kTPB) {
    S.b[0][i] = params[kOffB2 + i];
    S.b[1][i] = params[kOffB3 + i];
    S.b[2][i] = params[kOffB4 + i];
  }
  const uint32_t mbar = tc::smem_u32(&S.mbar);
  if (t == 0) {
    tc::mbar_init(mbar, 1);
    S.abort = 0;
  }
  if (warp == 0) tc::tmem_alloc(&S.tmem, 64);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem, lane_addr = tmem + ((warp * 32u) << 16);
  const uint32_t n = rows(n_max, n_dev, n_off);
  const uint32_t a_addr = tc::smem_u32(S.a), w_addr = tc::smem_u32(S.w);
  uint32_t phase = 0;
  for (uint32_t tile = blockIdx.x; tile * 128u < n; tile += gridDim.x) {
    const uint32_t row = tile * 128u + t;
    float4 r0 = make_float4(0, 0, 0, 0), r1 = r0, r2 = r0;
    if (row < n) {
      r0 = rec[3 * (size_t)row];
      r1 = rec[3 * (size_t)row + 1];
      r2 = rec[3 * (size_t)row + 2];
    }
    write_features(S.a, t, r0, r1, r2, p);
    sync_for_mma();
    if (t == 0) {
      tc::fence_after_sync();
      issue(tmem, a_addr, w_addr + kImgW1, kIn, 0);
      tc::mma_commit(mbar);
    }
    if (!wait_mma(mbar, phase, &S.abort, err)) break;
    epilogue_relu(lane_addr, nullptr, S.a, t);
    bool ok = true;
    for (int l = 0; l < 3 && ok; ++l) {
      sync_for_mma();
      if (t == 0) {
        tc::fence_after_sync();
        issue(tmem, a_addr, w_addr + kImgW2 + 8192u * l, 64, 0);
        tc::mma_commit(mbar);
      }
      ok = wait_mma(mbar, phase, &S.abort, err);
      if (ok && l < 2) epilogue_relu(lane_addr, S.b[l], S.a, t);
    }
    if (!ok) break;
    float pr[64];
    softmax_row(lane_addr, S.b[2], p.nclusters, pr);
    if (row < n) {
      uint4 *dst = reinterpret_cast<uint4 *>(probs + 64 * (size_t)row);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        __half2 h0 = __floats2half2_rn(pr[8 * q], pr[8 * q + 1]), h1 = __floats2half2_rn(pr[8 * q + 2], pr[8 * q + 3]);
        __half2 h2 = __floats2half2_rn(pr[8 * q + 4], pr[8 * q + 5]), h3 = __floats2half2_rn(pr[8 * q + 6], pr[8 * q + 7]);
        dst[q] = make_uint4(*reinterpret_cast<uint32_t *>(&h0), *reinterpret_cast<uint32_t *>(&h1),
                            *reinterpret_cast<uint32_t *>(&h2), *reinterpret_cast<uint32_t *>(&h3));
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// ---- training -------------------------------------------------------------------
struct SmemTrain {
  uint8_t w[kImgBytes];
  uint8_t x0[128 * kIn * 2];
  uint8_t h[3][128 * 64 * 2];
  uint8_t g[128 * 64 * 2];   // G [128 rows x K 64]
  uint8_t gt[64 * 128 * 2];  // G^T [64 x K 128]
  uint8_t ht[128 * 128 * 2]; // X^T [128 (features, padded) x K 128]
  float b[3][64];
  float loss[kTPB / 32];
  uint64_t mbar;
  uint32_t tmem;
  int abort;
};

constexpr uint32_t kColD = 0;
// TMEM column of the dW^T accumulator of layer l = 0..3 (dW1..dW4).
__device__ __forceinline__ uint32_t col_w(int l) { return 256u - 64u * (uint32_t)l; }

__global__ void __launch_bounds__(kTPB) k_mlp_train(const float4 *__restrict__ rec, uint32_t n_max,
                                                    const uint32_t *n_dev, uint32_t n_off,
                                                    const uint8_t *__restrict__ img,
                                                    const float *__restrict__ params, const float *scalars,
                                                    Params p, float *__restrict__ part, float *loss_part,
                                                    int *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  SmemTrain &S = *reinterpret_cast<SmemTrain *>(smem_raw);
  const uint32_t t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (uint32_t i = t; i < kImgBytes / 16; i += kTPB)
    reinterpret_cast<uint4 *>(S.w)[i] = reinterpret_cast<const uint4 *>(img)[i];
  for (uint32_t i = t; i < sizeof(S.ht) / 16; i += kTPB) reinterpret_cast<uint4 *>(S.ht)[i] = make_uint4(0, 0, 0, 0);
  for (uint32_t i = t; i < 64; i += kTPB) {
    S.b[0][i] = params[kOffB2 + i];
    S.b[1][i] = params[kOffB3 + i];
    S.b[2][i] = params[kOffB4 + i];
  }
  const uint32_t mbar = tc::smem_u32(&S.mbar);
  if (t == 0) {
    tc::mbar_init(mbar, 1);
    S.abort = 0;
  }
  if (warp == 0) tc::tmem_alloc(&S.tmem, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem, lane_addr = tmem + ((warp * 32u) << 16);
  const uint32_t n = rows(n_max, n_dev, n_off);
  const float wsum = scalars[0];
  const uint32_t w_addr = tc::smem_u32(S.w), x0_addr = tc::smem_u32(S.x0), g_addr = tc::smem_u32(S.g),
                 gt_addr = tc::smem_u32(S.gt), ht_addr = tc::smem_u32(S.ht);
  const uint32_t h0_addr = tc::smem_u32(S.h[0]);  // H1, H2, H3 are 16 KB apart
  uint32_t phase = 0, tiles = 0;
  float loss = 0.f;
  bool ok = wsum > 0.f;
  for (uint32_t tile = blockIdx.x; ok && tile * 128u < n; tile += gridDim.x, ++tiles) {
    const uint32_t row = tile * 128u + t;
    float4 r0 = make_float4(0, 0, 0, 0), r1 = r0, r2 = r0;
    if (row < n) {
      r0 = rec[3 * (size_t)row];
      r1 = rec[3 * (size_t)row + 1];
      r2 = rec[3 * (size_t)row + 2];
    }
    const float a = (row < n && r1.w > 0.f) ? r1.w / wsum : 0.f;
    const uint32_t k = min(__float_as_uint(r2.w), 63u);
    const uint32_t acc = tiles ? 1u : 0u;
    // ---- forward ----
    write_features(S.x0, t, r0, r1, r2, p);
    sync_for_mma();
    if (t == 0) {
      tc::fence_after_sync();
      issue(tmem + kColD, x0_addr, w_addr + kImgW1, kIn, 0);
      tc::mma_commit(mbar);
    }
    if (!(ok = wait_mma(mbar, phase, &S.abort, err))) break;
    epilogue_relu(lane_addr + kColD, nullptr, S.h[0], t);
    for (int l = 0; l < 3 && ok; ++l) {
      sync_for_mma();
      if (t == 0) {
        tc::fence_after_sync();
        issue(tmem + kColD, h0_addr + 16384u * l, w_addr + kImgW2 + 8192u * l, 64, 0);
        tc::mma_commit(mbar);
      }
      ok = wait_mma(mbar, phase, &S.abort, err);
      if (ok && l < 2) epilogue_relu(lane_addr + kColD, S.b[l], S.h[l + 1], t);
    }
    if (!ok) break;
    // ---- loss gradient at the logits ----
    {
      float pr[64];
      softmax_row(lane_addr + kColD, S.b[2], p.nclusters, pr);
      float pk = 0.f;
#pragma unroll
      for (int j = 0; j < 64; ++j) pk = (uint32_t)j == k ? pr[j] : pk;
      if (a > 0.f) loss -= a * __logf(fmaxf(pk, 1e-30f));
#pragma unroll
      for (int j = 0; j < 64; ++j) pr[j] = (uint32_t)j < p.nclusters ? a * (pr[j] - ((uint32_t)j == k ? 1.f : 0.f)) : 0.f;
#pragma unroll
      for (int q = 0; q < 8; ++q) st8(S.g, t, 8 * q, 64, pr + 8 * q);
#pragma unroll
      for (int j = 0; j < 64; ++j) st1(S.gt, j, t, 128, pr[j]);
    }
    // ---- backward, layers 4, 3, 2 ----
    for (int l = 2; l >= 0 && ok; --l) {
      // X^T of this layer's input (H3, H2, H1) with the ones row for the bias.
      {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          ld8(S.h[l], t, 8 * q, 64, v);
#pragma unroll
          for (int j = 0; j < 8; ++j) st1(S.ht, 8 * q + j, t, 128, v[j]);
        }
        st1(S.ht, 64, t, 128, 1.0f);
      }
      sync_for_mma();
      if (t == 0) {
        tc::fence_after_sync();
        issue(tmem + col_w(l + 1), ht_addr, gt_addr, 128, acc);  // dW^T += X^T G
        issue(tmem + kColD, g_addr, w_addr + kImgW2t + 8192u * l, 64, 0);  // dX = G W
        tc::mma_commit(mbar);
      }
      if (!(ok = wait_mma(mbar, phase, &S.abort, err))) break;
      // G of the layer below: dX masked by its ReLU.
      float d[64], hv[64];
      tc::tmem_ld32(lane_addr + kColD, d);
      tc::tmem_ld32(lane_addr + kColD + 32, d + 32);
#pragma unroll
      for (int q = 0; q < 8; ++q) ld8(S.h[l], t, 8 * q, 64, hv + 8 * q);
#pragma unroll
      for (int j = 0; j < 64; ++j) d[j] = hv[j] > 0.f ? d[j] : 0.f;
      if (l > 0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) st8(S.g, t, 8 * q, 64, d + 8 * q);
      }
#pragma unroll
      for (int j = 0; j < 64; ++j) st1(S.gt, j, t, 128, d[j]);
    }
    if (!ok) break;
    // ---- layer 1: dW1^T += X0^T G1 ----
    {
      float v[8];
#pragma unroll
      for (int q = 0; q < (int)kIn / 8; ++q) {
        ld8(S.x0, t, 8 * q, kIn, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) st1(S.ht, 8 * q + j, t, 128, v[j]);
      }
    }
    sync_for_mma();
    if (t == 0) {
      tc::fence_after_sync();
      issue(tmem + col_w(0), ht_addr, gt_addr, 128, acc);
      tc::mma_commit(mbar);
    }
    if (!(ok = wait_mma(mbar, phase, &S.abort, err))) break;
    tc::fence_before_sync();
    __syncthreads();
  }
  // ---- per-CTA partial sums ----
  for (int o = 16; o; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if (lane == 0) S.loss[warp] = loss;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  float *my = part + (size_t)blockIdx.x * kNParams;
  const bool have = ok && tiles > 0;
  if (t == 0) loss_part[blockIdx.x] = have ? S.loss[0] + S.loss[1] + S.loss[2] + S.loss[3] : 0.f;
  // Row i = 32 * warp + lane of each dW^T accumulator: weights of input i, or
  // (row 64 of layers 2-4) the bias.
  const uint32_t i = warp * 32u + lane;
  for (int l = 0; l < 4; ++l) {
    const uint32_t fan = l == 0 ? kIn : 64;
    float v[64];
    if (have) {
      tc::tmem_ld32(lane_addr + col_w(l), v);
      tc::tmem_ld32(lane_addr + col_w(l) + 32, v + 32);
    } else {
#pragma unroll
      for (int j = 0; j < 64; ++j) v[j] = 0.f;
    }
    const uint32_t offW = l == 0 ? kOffW1 : l == 1 ? kOffW2 : l == 2 ? kOffW3 : kOffW4;
    const uint32_t offB = l == 1 ? kOffB2 : l == 2 ? kOffB3 : kOffB4;
    if (i < fan) {
#pragma unroll
      for (int o = 0; o < 64; ++o) my[offW + o * fan + i] = v[o];
    } else if (l > 0 && i == 64) {
#pragma unroll
      for (int o = 0; o < 64; ++o) my[offB + o] = v[o];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// Weight sum of the batch (one CTA; deterministic order).
__global__ void k_mlp_wsum(const float4 *__restrict__ rec, uint32_t n_max, const uint32_t *n_dev, uint32_t n_off,
                           float *scalars) {
  __shared__ float red[32];
  const uint32_t n = rows(n_max, n_dev, n_off);
  float s = 0.f;
  for (uint32_t r = threadIdx.x; r < n; r += blockDim.x) {
    float w = rec[3 * (size_t)r + 1].w;
    s += w > 0.f ? w : 0.f;
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tot = 0.f;
    for (uint32_t w = 0; w < blockDim.x / 32; ++w) tot += red[w];
    scalars[0] = tot;
  }
}

// Image slots of parameter j (kmaj offsets in bytes; -1: none).
__device__ __forceinline__ void image_slots(uint32_t j, int &a, int &b) {
  a = b = -1;
  if (j < kOffW2) {
    uint32_t o = j / kIn, i = j % kIn;
    a = kImgW1 + tc::kmaj(o, i, kIn);
  } else {
    const uint32_t offs[3] = {kOffW2, kOffW3, kOffW4}, img[3] = {kImgW2, kImgW3, kImgW4},
                   imgt[3] = {kImgW2t, kImgW3t, kImgW4t};
    for (int l = 0; l < 3; ++l)
      if (j >= offs[l] && j < offs[l] + 4096) {
        uint32_t o = (j - offs[l]) / 64, i = (j - offs[l]) % 64;
        a = img[l] + tc::kmaj(o, i, 64);
        b = imgt[l] + tc::kmaj(i, o, 64);
      }
  }
}

// Sums the per-CTA gradients, applies Adam (when the batch had weight) and
// rewrites the BF16 images.  update = 0: images only.
__global__ void k_mlp_adam(float *params, float *m, float *v, const float *part, uint32_t grid,
                           const float *loss_part, float *scalars, uint8_t *img, int update, float lr, float b1,
                           float b2, float eps, float c1, float c2) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (update && blockIdx.x == 0 && threadIdx.x == 0 && scalars[0] > 0.f) {
    float l = 0.f;
    for (uint32_t c = 0; c < grid; ++c) l += loss_part[c];
    scalars[1] = l;
  }
  if (j >= kNParams) return;
  float w = params[j];
  if (update && scalars[0] > 0.f) {
    float g = 0.f;
    for (uint32_t c = 0; c < grid; ++c) g += part[(size_t)c * kNParams + j];
    float mj = b1 * m[j] + (1.f - b1) * g, vj = b2 * v[j] + (1.f - b2) * g * g;
    m[j] = mj;
    v[j] = vj;
    w -= lr * (mj / c1) / (sqrtf(vj / c2) + eps);
    params[j] = w;
  }
  int a, b;
  image_slots(j, a, b);
  __nv_bfloat16 h = __float2bfloat16_rn(w);
  if (a >= 0) *reinterpret_cast<__nv_bfloat16 *>(img + a) = h;
  if (b >= 0) *reinterpret_cast<__nv_bfloat16 *>(img + b) = h;
}

Params params_of(const Net &net) {
  Params p;
  p.cx = net.centre[0];
  p.cy = net.centre[1];
  p.cz = net.centre[2];
  p.scale = net.scale;
  p.nclusters = net.nclusters;
  return p;
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, sms);
}

}  // namespace

int create(Net &net, uint64_t seed) {
  std::vector<float> w(kNParams, 0.f);
  // He-uniform initialisation from the counter stream (seed, layer); the output
  // layer is scaled by 0.1 so that the first proposals are close to uniform.
  auto init = [&](uint32_t off, uint32_t nout, uint32_t nin, uint32_t fan, uint32_t layer, double gain) {
    uint64_t key = ckr_key(seed, layer);
    double lim = gain * std::sqrt(6.0 / fan);
    for (uint32_t o = 0; o < nout; ++o)
      for (uint32_t i = 0; i < nin; ++i)
        w[off + o * (nin == 79 ? kIn : nin) + i] =
            (float)((2.0 * ckr_draw_f(key, o * 128 + i) - 1.0) * lim);
  };
  init(kOffW1, kHid, 79, 79, 1, 1.0);  // features 0..78; the bias column 79 and padding stay 0
  init(kOffW2, kHid, kHid, kHid, 2, 1.0);
  init(kOffW3, kHid, kHid, kHid, 3, 1.0);
  init(kOffW4, kOut, kHid, kHid, 4, 0.1);
  net.grid = (uint32_t)sm_count();
  if (cudaMalloc((void **)&net.params, kNParams * 4) != cudaSuccess ||
      cudaMalloc((void **)&net.m, kNParams * 4) != cudaSuccess ||
      cudaMalloc((void **)&net.v, kNParams * 4) != cudaSuccess ||
      cudaMalloc((void **)&net.part, (size_t)net.grid * kNParams * 4) != cudaSuccess ||
      cudaMalloc((void **)&net.loss_part, net.grid * 4) != cudaSuccess ||
      cudaMalloc((void **)&net.scalars, 16) != cudaSuccess || cudaMalloc((void **)&net.img, kImgBytes) != cudaSuccess ||
      cudaMalloc((void **)&net.err, 4) != cudaSuccess) {
    destroy(net);
    return CKR_ERR_OUT_OF_MEMORY;
  }
  CKR_CUDA_TRY(cudaMemcpy(net.params, w.data(), kNParams * 4, cudaMemcpyHostToDevice));
  CKR_CUDA_TRY(cudaMemset(net.m, 0, kNParams * 4));
  CKR_CUDA_TRY(cudaMemset(net.v, 0, kNParams * 4));
  CKR_CUDA_TRY(cudaMemset(net.img, 0, kImgBytes));
  CKR_CUDA_TRY(cudaMemset(net.scalars, 0, 16));
  CKR_CUDA_TRY(cudaMemset(net.err, 0, 4));
  int dev = 0;
  CKR_CUDA_TRY(cudaGetDevice(&dev));
  CKR_CUDA_TRY(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemInfer)));
  CKR_CUDA_TRY(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemTrain)));
  int st = pack(net, nullptr);
  if (st != CKR_OK) return st;
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  return CKR_OK;
}

void destroy(Net &net) {
  cudaFree(net.params);
  cudaFree(net.m);
  cudaFree(net.v);
  cudaFree(net.part);
  cudaFree(net.loss_part);
  cudaFree(net.scalars);
  cudaFree(net.img);
  cudaFree(net.err);
  net = Net();
}

int pack(Net &net, cudaStream_t stream) {
  k_mlp_adam<<<ceil_div(kNParams, 256), 256, 0, stream>>>(net.params, net.m, net.v, net.part, net.grid,
                                                           net.loss_part, net.scalars, net.img, 0, 0.f, 0.f, 0.f,
                                                           0.f, 1.f, 1.f);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}

int infer(const Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, __half *probs,
          cudaStream_t stream) {
  if (n_max == 0) return CKR_OK;
  int per = 0;
  CKR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mlp_infer, kTPB, sizeof(SmemInfer)));
  uint32_t grid = std::min<uint32_t>(ceil_div(n_max, 128), (uint32_t)sm_count() * std::max(1, per));
  k_mlp_infer<<<grid, kTPB, sizeof(SmemInfer), stream>>>(rec, n_max, n_dev, 0, net.img, net.params, params_of(net),
                                                        probs, net.err);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}

int gradients(Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, uint32_t n_off,
              cudaStream_t stream) {
  k_mlp_wsum<<<1, 1024, 0, stream>>>(rec, n_max, n_dev, n_off, net.scalars);
  k_mlp_train<<<net.grid, kTPB, sizeof(SmemTrain), stream>>>(rec, n_max, n_dev, n_off, net.img, net.params,
                                                            net.scalars,
                                                            params_of(net), net.part, net.loss_part, net.err);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}

int train_step(Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, uint32_t n_off,
               cudaStream_t stream) {
  if (n_max == 0) return CKR_OK;
  int st = gradients(net, rec, n_max, n_dev, n_off, stream);
  if (st != CKR_OK) return st;
  net.step += 1;
  const float c1 = 1.0f - std::pow(net.beta1, (float)net.step), c2 = 1.0f - std::pow(net.beta2, (float)net.step);
  k_mlp_adam<<<ceil_div(kNParams, 256), 256, 0, stream>>>(net.params, net.m, net.v, net.part, net.grid,
                                                           net.loss_part, net.scalars, net.img, 1, net.lr, net.beta1,
                                                           net.beta2, net.eps, c1, c2);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}

}  // namespace mlp
}  // namespace ckr
