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

namespace ckr {
namespace mlp {

constexpr uint32_t kIn = 96, kHid = 64, kOut = 64, kFreqs = 12;
constexpr uint32_t kOffW1 = 0, kOffW2 = kOffW1 + kHid * kIn, kOffB2 = kOffW2 + kHid * kHid,
                   kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kHid, kOffW4 = kOffB3 + kHid,
                   kOffB4 = kOffW4 + kOut * kHid, kNParams = kOffB4 + kOut;
// BF16 operand images (K-major core-matrix layout): W1 [64 x 96], W2, W3, W4
// [64 x 64], then the transposes W2t, W3t, W4t used by the backward pass.
constexpr uint32_t kImgW1 = 0, kImgW2 = 12288, kImgW3 = 20480, kImgW4 = 28672, kImgW2t = 36864, kImgW3t = 45056,
                   kImgW4t = 53248, kImgForward = 36864, kImgBytes = 61440;

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
};

int create(Net &net, uint64_t seed);
void destroy(Net &net);
// Probabilities (FP16, 64 per row) for rows [0, n), n = min(*n_dev, n_max) when
// n_dev is not null, else n_max.  rec: 3 float4 per row.
int infer(const Net &net, const float4 *rec, uint32_t n_max, const uint32_t *n_dev, __half *probs,
          cudaStream_t stream);
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
