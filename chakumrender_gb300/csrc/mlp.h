// mlp.h — the learned light-selection network (internal interface).
//
// A 96 -> 64 -> 64 -> 64 -> 64 MLP (ReLU, softmax over the scene's emitter
// lights) evaluated and trained on the tensor cores (tcgen05, BF16 operands,
// FP32 accumulation in tensor memory).  Inputs are 12-float records:
// (x.xyz, alpha), (n.xyz, weight), (wo.xyz, cluster bits); features are the
// 12-frequency sin/cos encoding of the normalised position, n, wo, alpha and a
// constant 1 (the first layer's bias).  Parameters are FP32 master copies (the
// order of the oracle's orc_mlp.c) with BF16 operand images for the kernels.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "scene.h"

namespace ckr {
namespace mlp {

// Network input straight from the renderer's path state: queue entry i is path
// slot queue[i]; its shading point comes from the hit record and the scene.
struct PathRows {
  const uint32_t *queue = nullptr, *hit_id = nullptr;
  const float4 *ray_o = nullptr, *ray_d = nullptr;
  const float *hit_t = nullptr;
  const uint4 *meta = nullptr;
  ShadeView sv{};
};

constexpr uint32_t kIn = 96, kHid = 64, kOut = 64, kFreqs = 12;
constexpr uint32_t kOffW1 = 0, kOffW2 = kOffW1 + kHid * kIn, kOffB2 = kOffW2 + kHid * kHid,
                   kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kHid, kOffW4 = kOffB3 + kHid,
                   kOffB4 = kOffW4 + kOut * kHid, kNParams = kOffB4 + kOut;
// BF16 operand images (K-major core-matrix layout): W1 [64 x 96] (its bias is the
// weight of the constant feature 79); W2, W3, W4 [64 x 80]: the 64 weights of an
// output, its bias at K = 64 (the activations carry a constant 1 there) and zeros;
// then the transposes W2t, W3t, W4t [64 x 64] used by the backward pass.
constexpr uint32_t kHidK = 80;  // K of the hidden-layer operands
constexpr uint32_t kImgW1 = 0, kImgW2 = 12288, kImgW3 = 22528, kImgW4 = 32768, kImgW2t = 43008, kImgW3t = 51200,
                   kImgW4t = 59392, kImgForward = 43008, kImgBytes = 67584;

struct Net {
  float *params = nullptr, *m = nullptr, *v = nullptr;  // FP32 master weights and Adam moments
  float *part = nullptr;     // per-CTA gradient partial sums [grid x kNParams]
  float *loss_part = nullptr;  // per-CTA loss partial sums [grid]
  float *scalars = nullptr;  // [0] weight sum of the batch, [1] loss of the last step
  uint8_t *img = nullptr;    // kImgBytes
  int *err = nullptr;
  uint32_t grid = 0;         // CTAs of the training kernel
  float centre[3] = {0, 0, 0}, scale = 1.0f;
  uint32_t nclusters = 0;
  uint32_t step = 0;
  float lr = 1e-3f, beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  uint32_t stall_tries = 0;  // test hook of the bounded waits (0: off); see Params in mlp.cu
};

int create(Net &net, uint64_t seed);
void destroy(Net &net);
// Network output for rows [0, n), n = min(*n_dev, n_max) when n_dev is not null,
// else n_max; rec: 3 float4 per row.  probs (nullable): the softmax, FP16, 64 per
// row.  cdf16 (nullable): the selection mixture (1 - delta) softmax + delta / C as
// 64 cumulative 16-bit entries per row, pmf(j) = (cdf[j] - cdf[j-1]) / 65535.
int infer(const Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, __half *probs, uint16_t *cdf16,
          float delta, cudaStream_t stream);
// The selection CDFs for the renderer's queue entries [0, min(*n_dev, n_max)), with
// the weights of `img` (a copy of Net::img; nullptr: Net::img itself).
int infer_paths(const Net &net, const PathRows &rows, uint32_t n_max, const uint32_t *n_dev, uint16_t *cdf16,
                float delta, cudaStream_t stream, const uint8_t *img = nullptr);
// One Adam step on the records [0, n) of rec, n = min(*n_dev - n_off, n_max) (rec
// already advanced by n_off rows) or n_max; skipped (no update) when their weights
// sum to 0.
int train_step(Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, uint32_t n_off,
               cudaStream_t stream);
// The batch's weight sum, per-CTA gradient partials (part) and loss partials,
// without an update (for checking the backward pass).
int gradients(Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, uint32_t n_off,
              cudaStream_t stream);
// Rewrites the BF16 images from the FP32 master weights.
int pack(Net &net, cudaStream_t stream);

}  // namespace mlp
}  // namespace ckr
