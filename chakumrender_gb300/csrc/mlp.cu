// mlp.cu — the learned light-selection network on the fifth-generation tensor
// cores: inference (k_mlp_infer), training forward + backward (k_mlp_train) and
// the Adam update (k_mlp_adam), all for tiles of 128 rows.
//
// A group of 128 threads owns a tile: thread t computes row t's features and
// epilogues, thread 0 issues the tcgen05.mma chain of each layer (M = 128 rows,
// N = 64 outputs, K = 96, or 80 for the hidden layers whose operands carry a
// constant 1 that multiplies the bias) into tensor memory and commits it to an
// mbarrier that the group waits on with a bounded poll.  Row t of the
// accumulator lives in TMEM lane t, which warp (t / 32) % 4 reads with
// tcgen05.ld.  Inference runs two groups per CTA over the same weights, so one
// group's epilogue overlaps the other's MMAs; training runs one.
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
#include "render_device.cuh"
#include "tc05.cuh"

namespace ckr {
namespace mlp {
namespace {

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
  // Test hook: when non-zero, the first layer's MMAs are not issued and every
  // mbarrier wait gives up after this many polls (a phase nothing completes).
  uint32_t stall_tries;
};

// Row features into the first-layer operand (K = 96).
__device__ __forceinline__ void write_features(uint8_t *x0, uint32_t t, float4 r0, float4 r1, float4 r2,
                                               const Params &p) {
  float f[kIn];
  const float pc[3] = {(r0.x - p.cx) * p.scale, (r0.y - p.cy) * p.scale, (r0.z - p.cz) * p.scale};
  // sin, cos of 2^k pi p: the base frequency, then the double-angle recurrences
  // sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a); the error
  // (about 1e-6 at the base) roughly doubles per octave, a few 1e-3 after eleven,
  // at the level of BF16's rounding of the features.
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float sn, cs;
    __sincosf(3.14159265358979f * pc[c], &sn, &cs);  // |argument| <= pi inside the scene box
#pragma unroll
    for (int k = 0; k < (int)kFreqs; ++k) {
      f[24 * c + 2 * k] = sn;
      f[24 * c + 2 * k + 1] = cs;
      const float s2 = 2.0f * sn * cs;
      cs = (cs - sn) * (cs + sn);
      sn = s2;
    }
  }
  f[72] = r1.x; f[73] = r1.y; f[74] = r1.z;
  f[75] = r2.x; f[76] = r2.y; f[77] = r2.z;
  f[78] = r0.w;
  f[79] = 1.0f;
#pragma unroll
  for (int j = 80; j < (int)kIn; ++j) f[j] = 0.f;
#pragma unroll
  for (int q = 0; q < (int)kIn / 8; ++q) st8(x0, t, 8 * q, kIn, f + 8 * q);
}

// Two FP32 values to a BF16 pair with ReLU (lower half = first value).
__device__ __forceinline__ uint32_t pack_relu_bf16(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// Accumulator row t (64 columns, bias included by the MMA) through ReLU into row t
// of a hidden-layer operand (K = 80): columns 0..63, then the constant 1 at 64 and
// zeros to 79.
__device__ __forceinline__ void epilogue_relu(uint32_t taddr, uint8_t *dst, uint32_t t) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[32];
    tc::tmem_ld32(taddr + 32 * h, v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float *x = v + 8 * q;
      *reinterpret_cast<uint4 *>(dst + tc::kmaj(t, 32 * h + 8 * q, kHidK)) =
          make_uint4(pack_relu_bf16(x[0], x[1]), pack_relu_bf16(x[2], x[3]), pack_relu_bf16(x[4], x[5]),
                     pack_relu_bf16(x[6], x[7]));
    }
  }
  *reinterpret_cast<uint4 *>(dst + tc::kmaj(t, 64, kHidK)) = make_uint4(0x3F80u, 0u, 0u, 0u);  // BF16 1.0
  *reinterpret_cast<uint4 *>(dst + tc::kmaj(t, 72, kHidK)) = make_uint4(0u, 0u, 0u, 0u);
}

// exp(z) over the logits of row t when all 64 are clusters, with z clamped to
// [-80, 80] so that neither the terms nor their sum leave FP32's range (the
// softmax does not change for logits inside that range); returns the sum.
__device__ __forceinline__ float softmax_exp64(uint32_t taddr, float *p) {
  tc::tmem_ld32(taddr, p);
  tc::tmem_ld32(taddr + 32, p + 32);
  float sum = 0.f;
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    p[j] = __expf(fminf(fmaxf(p[j], -80.f), 80.f));
    sum += p[j];
  }
  return sum;
}

// exp(z - max) over the first C logits of row t (0 beyond); returns their sum.
__device__ __forceinline__ float softmax_exp(uint32_t taddr, uint32_t C, float *p) {
  tc::tmem_ld32(taddr, p);
  tc::tmem_ld32(taddr + 32, p + 32);
  float mx = -3.0e38f;
#pragma unroll
  for (int j = 0; j < 64; ++j)
    if ((uint32_t)j < C) mx = fmaxf(mx, p[j]);
  float sum = 0.f;
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    p[j] = (uint32_t)j < C ? __expf(p[j] - mx) : 0.f;
    sum += p[j];
  }
  return sum;
}

__device__ __forceinline__ void issue(uint32_t d, uint32_t a, uint32_t b, uint32_t K, uint32_t accumulate_first) {
  for (uint32_t s = 0; s < K / 16; ++s)
    tc::mma_bf16(d, tc::sdesc(a, K, s), tc::sdesc(b, K, s), kIdesc, (s > 0 || accumulate_first) ? 1u : 0u);
}

// Barrier of one 128-thread group (named barrier 1 + g; 0 is __syncthreads).
// Immediate ids, so that the kernel reserves only the barriers it uses.
__device__ __forceinline__ void group_sync(uint32_t g) {
  if (g == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
  else asm volatile("bar.sync 2, 128;" ::: "memory");
}

// Every thread of the group: shared-memory writes visible to the tensor core,
// TMEM reads done before the next MMA overwrites the accumulator.
__device__ __forceinline__ void sync_for_mma(uint32_t g) {
  tc::fence_proxy_async();
  tc::fence_before_sync();
  group_sync(g);
}

// Waits for the group's committed MMAs; false (uniformly within the group) when
// the wait gave up.
__device__ __forceinline__ bool wait_mma(uint32_t g, uint32_t mbar, uint32_t &phase, int *abort, int *err,
                                         uint32_t tries = kWaitTries) {
  if (!tc::mbar_wait(mbar, phase, tries)) {
    *abort = 1;
    atomicExch(err, CKR_ERR_ITERATION_LIMIT);
  }
  group_sync(g);
  if (*abort) {
    tc::mbar_wait(mbar, phase, tries);  // let the MMAs in flight land before TMEM is freed
    return false;
  }
  phase ^= 1u;
  tc::fence_after_sync();
  return true;
}

// ---- inference ------------------------------------------------------------------
// kGroups independent 128-thread groups per CTA share the weights in shared memory;
// each owns a 128-row tile, an activation buffer, an mbarrier and 64 TMEM columns,
// so one group's epilogue overlaps another's MMAs.
constexpr uint32_t kGroups = 2, kInferTPB = 128 * kGroups;

struct SmemInfer {
  uint8_t w[kImgForward];
  uint8_t a[kGroups][128 * kIn * 2];
  uint64_t mbar[kGroups];
  uint32_t tmem;
  int abort[kGroups];
};

// A queue entry's path state, gathered in three dependent steps (the path slot from
// the queue, the slot's hit and ray, the hit triangle's normal and alpha) so that
// each step's latency can overlap other work of the tile before it.
struct PathGather {
  uint32_t slot, id, flags;
  float4 ro, rd;
  float t;
  float4 na;
};

__device__ __forceinline__ void gather_slot(const PathRows &pr, uint32_t row, uint32_t n, PathGather &g) {
  g.slot = row < n ? pr.queue[row] : 0xFFFFFFFFu;
}

__device__ __forceinline__ void gather_hit(const PathRows &pr, PathGather &g) {
  g.id = kMiss;
  if (g.slot == 0xFFFFFFFFu) return;
  g.id = pr.hit_id[g.slot];
  g.flags = pr.meta[g.slot].w;
  g.ro = pr.ray_o[g.slot];
  g.rd = pr.ray_d[g.slot];
  g.t = pr.hit_t[g.slot];
}

// The hit triangle's normal and material index (ShadeView::tri_nm, a third
// dependent step).
__device__ __forceinline__ void gather_na(const PathRows &pr, PathGather &g) {
  if (g.id != kMiss && !(g.id & kSphereBit)) g.na = pr.sv.tri_nm[g.id];
}

// Network input of a gathered queue entry: its shading point (zeros where the entry is
// not a shaded surface).
__device__ __forceinline__ void path_row(const PathRows &pr, const PathGather &g, float4 &r0, float4 &r1,
                                         float4 &r2) {
  r0 = r1 = r2 = make_float4(0, 0, 0, 0);
  if (g.id == kMiss || (g.flags & 1u)) return;
  if (!(g.id & kSphereBit)) {
    const ckr_material &mm = pr.sv.mats[__float_as_uint(g.na.w)];
    if (mm.light_type != 0) return;  // an emitter
    const F3 d = f3(g.rd.x, g.rd.y, g.rd.z), x = f3(g.ro.x, g.ro.y, g.ro.z) + d * g.t;
    F3 nn = f3(g.na.x, g.na.y, g.na.z);
    if (dot(d, nn) > 0.f) nn = -nn;
    r0 = make_float4(x.x, x.y, x.z, mm.alpha);
    r1 = make_float4(nn.x, nn.y, nn.z, 0.f);
    r2 = make_float4(-d.x, -d.y, -d.z, 0.f);
    return;
  }
  Surface S = make_surface(pr.sv, f3(g.ro.x, g.ro.y, g.ro.z), f3(g.rd.x, g.rd.y, g.rd.z), g.id, g.t);
  const ckr_material &mm = pr.sv.mats[S.mat];
  if (mm.light_type != 0) return;
  r0 = make_float4(S.x.x, S.x.y, S.x.z, mm.alpha);
  r1 = make_float4(S.n.x, S.n.y, S.n.z, 0.f);
  r2 = make_float4(S.wo.x, S.wo.y, S.wo.z, 0.f);
}

template <bool PATHS>
__global__ void __launch_bounds__(kInferTPB, 2) k_mlp_infer(const float4 *__restrict__ rec, PathRows pr, uint32_t n_max,
                                                         const uint32_t *n_dev, uint32_t n_off,
                                                         const uint8_t *__restrict__ img, Params p, float delta,
                                                         __half *__restrict__ probs, uint16_t *__restrict__ cdf16,
                                                         int *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  SmemInfer &S = *reinterpret_cast<SmemInfer *>(smem_raw);
  const uint32_t g = threadIdx.x >> 7, t = threadIdx.x & 127u, warp = threadIdx.x >> 5;
  for (uint32_t i = threadIdx.x; i < kImgForward / 16; i += kInferTPB)
    reinterpret_cast<uint4 *>(S.w)[i] = reinterpret_cast<const uint4 *>(img)[i];
  const uint32_t mbar = tc::smem_u32(&S.mbar[g]);
  if (t == 0) {
    tc::mbar_init(mbar, 1);
    S.abort[g] = 0;
  }
  if (warp == 0) tc::tmem_alloc(&S.tmem, 64 * kGroups);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // Warp w reads TMEM lanes 32 (w % 4) .. +31; group g owns columns 64 g .. +63.
  const uint32_t tmem = S.tmem + 64u * g, lane_addr = tmem + (((warp & 3u) * 32u) << 16);
  const uint32_t n = rows(n_max, n_dev, n_off);
  uint8_t *A = S.a[g];
  const uint32_t a_addr = tc::smem_u32(A), w_addr = tc::smem_u32(S.w);
  uint32_t phase = 0;
  const uint32_t stride = gridDim.x * kGroups;
  // PATHS: the gather of the next tile's rows runs one tile ahead -- its queue load
  // from the start of this tile's MMA chain, its hit and ray loads from the second
  // layer, its triangle's normal and material (ShadeView::tri_nm) during the softmax --
  // so that a row's inputs are in registers when its tile starts (spheres still
  // read the scene through make_surface).  Two CTAs per SM: 128 registers.
  PathGather cur{}, nxt{};
  if (PATHS) {
    gather_slot(pr, (blockIdx.x * kGroups + g) * 128u + t, n, cur);
    gather_hit(pr, cur);
    gather_na(pr, cur);
  }
  for (uint32_t tile = blockIdx.x * kGroups + g; tile * 128u < n; tile += stride) {
    const uint32_t row = tile * 128u + t;
    float4 r0 = make_float4(0, 0, 0, 0), r1 = r0, r2 = r0;
    if (PATHS) {
      path_row(pr, cur, r0, r1, r2);
      gather_slot(pr, (tile + stride) * 128u + t, n, nxt);
    } else if (row < n) {
      r0 = rec[3 * (size_t)row];
      r1 = rec[3 * (size_t)row + 1];
      r2 = rec[3 * (size_t)row + 2];
    }
    write_features(A, t, r0, r1, r2, p);
    bool ok = true;
    for (int l = 0; l < 4 && ok; ++l) {
      sync_for_mma(g);
      if (t == 0 && !(p.stall_tries && l == 0)) {
        tc::fence_after_sync();
        if (l == 0) issue(tmem, a_addr, w_addr + kImgW1, kIn, 0);
        else issue(tmem, a_addr, w_addr + kImgW2 + 10240u * (l - 1), kHidK, 0);
        tc::mma_commit(mbar);
      }
      ok = wait_mma(g, mbar, phase, &S.abort[g], err, p.stall_tries ? p.stall_tries : kWaitTries);
      if (ok && l < 3) epilogue_relu(lane_addr, A, t);
      if (PATHS && l == 1) gather_hit(pr, nxt);
    }
    if (!ok) break;
    if (PATHS) gather_na(pr, nxt);
    float e[64];
    const bool full = p.nclusters == 64;
    const float sum = full ? softmax_exp64(lane_addr, e) : softmax_exp(lane_addr, p.nclusters, e);
    if (row < n && cdf16 && full) {
      const float unif = delta / 64.0f, keep = (1.0f - delta) / sum;
      float run = 0.f;
      uint32_t w[32];
#pragma unroll
      for (int j = 0; j < 64; j += 2) {
        run += fmaf(keep, e[j], unif);
        const uint32_t c0 = min(65535u, __float2uint_rn(65535.0f * run));
        run += fmaf(keep, e[j + 1], unif);
        const uint32_t c1 = j + 2 == 64 ? 65535u : min(65535u, __float2uint_rn(65535.0f * run));
        w[j / 2] = c0 | (c1 << 16);
      }
      uint4 *dst = reinterpret_cast<uint4 *>(cdf16 + 64 * (size_t)row);
#pragma unroll
      for (int q = 0; q < 8; ++q) dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    } else if (row < n && cdf16) {
      // Selection mixture (1 - delta) softmax + delta / C as a 16-bit cumulative
      // table: entry j = round(65535 * sum_{i <= j} q_i), the last cluster's 65535.
      const float unif = delta / (float)p.nclusters, keep = (1.0f - delta) / sum;
      float run = 0.f;
      uint32_t w[32];
#pragma unroll
      for (int j = 0; j < 64; j += 2) {
        run += (uint32_t)j < p.nclusters ? keep * e[j] + unif : 0.f;
        uint32_t c0 = (uint32_t)j + 1 >= p.nclusters ? 65535u : min(65535u, __float2uint_rn(65535.0f * run));
        run += (uint32_t)j + 1 < p.nclusters ? keep * e[j + 1] + unif : 0.f;
        uint32_t c1 = (uint32_t)j + 2 >= p.nclusters ? 65535u : min(65535u, __float2uint_rn(65535.0f * run));
        w[j / 2] = c0 | (c1 << 16);
      }
      uint4 *dst = reinterpret_cast<uint4 *>(cdf16 + 64 * (size_t)row);
#pragma unroll
      for (int q = 0; q < 8; ++q) dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    }
    if (row < n && probs) {
      const float inv = 1.0f / sum;
      uint4 *dst = reinterpret_cast<uint4 *>(probs + 64 * (size_t)row);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float *x = e + 8 * q;
        __half2 h0 = __floats2half2_rn(x[0] * inv, x[1] * inv), h1 = __floats2half2_rn(x[2] * inv, x[3] * inv);
        __half2 h2 = __floats2half2_rn(x[4] * inv, x[5] * inv), h3 = __floats2half2_rn(x[6] * inv, x[7] * inv);
        dst[q] = make_uint4(*reinterpret_cast<uint32_t *>(&h0), *reinterpret_cast<uint32_t *>(&h1),
                            *reinterpret_cast<uint32_t *>(&h2), *reinterpret_cast<uint32_t *>(&h3));
      }
    }
    if (PATHS) cur = nxt;
    tc::fence_before_sync();
    group_sync(g);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(S.tmem, 64 * kGroups);
}

// ---- training -------------------------------------------------------------------
constexpr uint32_t kTrainTPB = 128;

struct SmemTrain {
  uint8_t w[kImgBytes];
  uint8_t x0[128 * kIn * 2];
  uint8_t h[3][128 * kHidK * 2];  // H1, H2, H3 with the constant-1 column (K = 80)
  uint8_t g[128 * 64 * 2];        // G [128 rows x K 64]
  uint8_t gt[64 * 128 * 2];       // G^T [64 x K 128]
  uint8_t ht[128 * 128 * 2];      // X^T [128 (features, padded) x K 128]
  float loss[kTrainTPB / 32];
  uint64_t mbar;
  uint32_t tmem;
  int abort;
};

constexpr uint32_t kColD = 0;
// TMEM column of the dW^T accumulator of layer l = 0..3 (dW1..dW4).
__device__ __forceinline__ uint32_t col_w(int l) { return 256u - 64u * (uint32_t)l; }

__global__ void __launch_bounds__(kTrainTPB) k_mlp_train(const float4 *__restrict__ rec, uint32_t n_max,
                                                         const uint32_t *n_dev, uint32_t n_off,
                                                         const uint8_t *__restrict__ img, const float *scalars,
                                                         Params p, float *__restrict__ part, float *loss_part,
                                                         int *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  SmemTrain &S = *reinterpret_cast<SmemTrain *>(smem_raw);
  const uint32_t t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (uint32_t i = t; i < kImgBytes / 16; i += kTrainTPB)
    reinterpret_cast<uint4 *>(S.w)[i] = reinterpret_cast<const uint4 *>(img)[i];
  for (uint32_t i = t; i < sizeof(S.ht) / 16; i += kTrainTPB)
    reinterpret_cast<uint4 *>(S.ht)[i] = make_uint4(0, 0, 0, 0);
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
  const uint32_t h0_addr = tc::smem_u32(S.h[0]);  // H1, H2, H3 are 20 KB apart
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
    for (int l = 0; l < 4 && ok; ++l) {
      sync_for_mma(0);
      if (t == 0) {
        tc::fence_after_sync();
        if (l == 0) issue(tmem + kColD, x0_addr, w_addr + kImgW1, kIn, 0);
        else issue(tmem + kColD, h0_addr + 20480u * (l - 1), w_addr + kImgW2 + 10240u * (l - 1), kHidK, 0);
        tc::mma_commit(mbar);
      }
      ok = wait_mma(0, mbar, phase, &S.abort, err);
      if (ok && l < 3) epilogue_relu(lane_addr + kColD, S.h[l], t);
    }
    if (!ok) break;
    // ---- loss gradient at the logits: a (softmax - onehot(k)) ----
    {
      float pr[64];
      const float inv = 1.0f / softmax_exp(lane_addr + kColD, p.nclusters, pr);
      float pk = 0.f;
#pragma unroll
      for (int j = 0; j < 64; ++j) {
        pr[j] *= inv;
        pk = (uint32_t)j == k ? pr[j] : pk;
      }
      if (a > 0.f) loss -= a * __logf(fmaxf(pk, 1e-30f));
#pragma unroll
      for (int j = 0; j < 64; ++j) pr[j] = (uint32_t)j < p.nclusters ? a * (pr[j] - ((uint32_t)j == k ? 1.f : 0.f)) : 0.f;
#pragma unroll
      for (int q = 0; q < 8; ++q) st8(S.g, t, 8 * q, 64, pr + 8 * q);
#pragma unroll
      for (int j = 0; j < 64; ++j) st1(S.gt, j, t, 128, pr[j]);
    }
    // ---- backward, layers 4, 3, 2 (input H3, H2, H1) ----
    for (int l = 2; l >= 0 && ok; --l) {
      // X^T of the layer's input with the ones row (64) for the bias.
      {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          ld8(S.h[l], t, 8 * q, kHidK, v);
#pragma unroll
          for (int j = 0; j < 8; ++j) st1(S.ht, 8 * q + j, t, 128, v[j]);
        }
        st1(S.ht, 64, t, 128, 1.0f);
      }
      sync_for_mma(0);
      if (t == 0) {
        tc::fence_after_sync();
        issue(tmem + col_w(l + 1), ht_addr, gt_addr, 128, acc);            // dW^T += X^T G
        issue(tmem + kColD, g_addr, w_addr + kImgW2t + 8192u * l, 64, 0);  // dX = G W
        tc::mma_commit(mbar);
      }
      if (!(ok = wait_mma(0, mbar, phase, &S.abort, err))) break;
      // G of the layer below: dX masked by its ReLU.
      float d[64], hv[64];
      tc::tmem_ld32(lane_addr + kColD, d);
      tc::tmem_ld32(lane_addr + kColD + 32, d + 32);
#pragma unroll
      for (int q = 0; q < 8; ++q) ld8(S.h[l], t, 8 * q, kHidK, hv + 8 * q);
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
    sync_for_mma(0);
    if (t == 0) {
      tc::fence_after_sync();
      issue(tmem + col_w(0), ht_addr, gt_addr, 128, acc);
      tc::mma_commit(mbar);
    }
    if (!(ok = wait_mma(0, mbar, phase, &S.abort, err))) break;
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
    for (int l = 0; l < 3; ++l) {
      if (j >= offs[l] && j < offs[l] + 4096) {
        uint32_t o = (j - offs[l]) / 64, i = (j - offs[l]) % 64;
        a = img[l] + tc::kmaj(o, i, kHidK);
        b = imgt[l] + tc::kmaj(i, o, 64);
      } else if (j >= offs[l] + 4096 && j < offs[l] + 4096 + 64) {  // bias of output o at K = 64
        a = img[l] + tc::kmaj(j - offs[l] - 4096, 64, kHidK);
      }
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
  p.stall_tries = net.stall_tries;
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
  for (const void *fn : {(const void *)k_mlp_infer<false>, (const void *)k_mlp_infer<true>}) {
    CKR_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemInfer)));
    CKR_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  }
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

namespace {
template <bool PATHS>
int launch_infer(const Net &net, const float4 *rec, const PathRows &pr, uint32_t n_max, const uint32_t *n_dev,
                 __half *probs, uint16_t *cdf16, float delta, cudaStream_t stream, const uint8_t *img = nullptr) {
  if (n_max == 0) return CKR_OK;
  // CTAs resident per SM: shared memory (the opt-in maximum over the CTA's
  // footprint plus the 1 KB the driver reserves per CTA) or 4.
  static int per_sm = 0;
  if (!per_sm) {
    int dev = 0, smem = 0;
    CKR_CUDA_TRY(cudaGetDevice(&dev));
    CKR_CUDA_TRY(cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    per_sm = std::max(1, std::min(4, smem / (int)(sizeof(SmemInfer) + 1024)));
  }
  uint32_t grid = std::min<uint32_t>(ceil_div(n_max, 128 * kGroups), (uint32_t)sm_count() * per_sm);
  k_mlp_infer<PATHS><<<grid, kInferTPB, sizeof(SmemInfer), stream>>>(rec, pr, n_max, n_dev, 0, img ? img : net.img,
                                                                    params_of(net), delta, probs, cdf16, net.err);
  CKR_CUDA_TRY(cudaGetLastError());
  return CKR_OK;
}
}  // namespace

int infer(const Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, __half *probs, uint16_t *cdf16,
          float delta, cudaStream_t stream) {
  return launch_infer<false>(net, rec, PathRows{}, n_max, n_dev, probs, cdf16, delta, stream);
}

int infer_paths(const Net &net, const PathRows &rows, uint32_t n_max, const uint32_t *n_dev, uint16_t *cdf16,
                float delta, cudaStream_t stream, const uint8_t *img) {
  return launch_infer<true>(net, nullptr, rows, n_max, n_dev, nullptr, cdf16, delta, stream, img);
}

int gradients(Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, uint32_t n_off,
              cudaStream_t stream) {
  k_mlp_wsum<<<1, 1024, 0, stream>>>(rec, n_max, n_dev, n_off, net.scalars);
  k_mlp_train<<<net.grid, kTrainTPB, sizeof(SmemTrain), stream>>>(rec, n_max, n_dev, n_off, net.img, net.scalars,
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
