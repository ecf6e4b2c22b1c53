// proposal.cu — C ABI of the learned light-selection proposal (no reference
// counterpart): creation from a scene, parameters, direct network evaluation and
// training steps on caller records.  Rendering with it is ckr_render_learned
// (render.cu).
#include <algorithm>
#include <cstring>
#include <vector>

#include "ckr_test.h"
#include "proposal.h"
#include "scene.h"

using namespace ckr;

extern "C" int ckr_proposal_create(const ckr_scene *s, const ckr_proposal_cfg *cfg, ckr_proposal **out) {
  if (!s || !out || !s->has_shading) return CKR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (s->n_emit == 0) return CKR_ERR_INVALID_ARGUMENT;
  if (s->n_emit > mlp::kOut) return CKR_ERR_TOO_LARGE;
  ckr_proposal_cfg c = cfg ? *cfg : ckr_proposal_cfg{1, 1e-3f, 0.2f, 65536, 1, 16384, 0};
  if (c.minibatch == 0) c.minibatch = c.batch;
  if (!(c.lr > 0.f) || !(c.defensive > 0.f) || c.defensive > 1.f || c.batch == 0 || c.batch > (1u << 22) ||
      c.minibatch > c.batch)
    return CKR_ERR_INVALID_ARGUMENT;
  ckr_proposal *p = new (std::nothrow) ckr_proposal();
  if (!p) return CKR_ERR_OUT_OF_MEMORY;
  if (cudaGetDevice(&p->device) != cudaSuccess) {
    delete p;
    return CKR_ERR_CUDA;
  }
  // Position encoding: the scene box mapped to [-1, 1] along its longest side.
  float ext = 0.f;
  for (int k = 0; k < 3; ++k) {
    p->net.centre[k] = 0.5f * (s->bounds[k] + s->bounds[3 + k]);
    ext = std::max(ext, s->bounds[3 + k] - s->bounds[k]);
  }
  p->net.scale = ext > 0.f ? 2.0f / ext : 1.0f;
  p->net.nclusters = s->n_emit;
  p->net.lr = c.lr;
  p->defensive = c.defensive;
  p->batch = c.batch;
  p->minibatch = c.minibatch;
  p->max_steps = c.max_steps;
  p->train = c.train ? 1 : 0;
  int st = mlp::create(p->net, c.seed);
  if (st == CKR_OK && p->rec_count.reserve(1) != cudaSuccess) st = CKR_ERR_OUT_OF_MEMORY;
  if (st == CKR_OK && cudaMemset(p->rec_count.ptr, 0, 4) != cudaSuccess) st = CKR_ERR_CUDA;
  if (st != CKR_OK) {
    mlp::destroy(p->net);
    delete p;
    return st;
  }
  *out = p;
  return CKR_OK;
}

extern "C" int ckr_proposal_destroy(ckr_proposal *p) {
  if (!p) return CKR_ERR_INVALID_ARGUMENT;
  mlp::destroy(p->net);
  delete p;
  return CKR_OK;
}

extern "C" int ckr_proposal_set_training(ckr_proposal *p, int train) {
  if (!p) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  p->train = train ? 1 : 0;
  return CKR_OK;
}

extern "C" int ckr_proposal_get_params(ckr_proposal *p, float *params) {
  if (!p || !params) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  CKR_CUDA_TRY(cudaMemcpy(params, p->net.params, mlp::kNParams * 4, cudaMemcpyDeviceToHost));
  return CKR_OK;
}

extern "C" int ckr_proposal_set_params(ckr_proposal *p, const float *params) {
  if (!p || !params) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  CKR_CUDA_TRY(cudaMemcpy(p->net.params, params, mlp::kNParams * 4, cudaMemcpyHostToDevice));
  CKR_CUDA_TRY(cudaMemset(p->net.m, 0, mlp::kNParams * 4));
  CKR_CUDA_TRY(cudaMemset(p->net.v, 0, mlp::kNParams * 4));
  p->net.step = 0;
  int st = mlp::pack(p->net, nullptr);
  if (st != CKR_OK) return st;
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  return CKR_OK;
}

extern "C" int ckr_proposal_encoding(const ckr_proposal *p, float centre[3], float *scale, uint32_t *nclusters) {
  if (!p || !centre || !scale || !nclusters) return CKR_ERR_INVALID_ARGUMENT;
  for (int k = 0; k < 3; ++k) centre[k] = p->net.centre[k];
  *scale = p->net.scale;
  *nclusters = p->net.nclusters;
  return CKR_OK;
}

extern "C" int ckr_proposal_infer(ckr_proposal *p, const float *rec12, uint32_t n, uint16_t *probs, void *stream) {
  if (!p || (n && (!rec12 || !probs)) || ((uintptr_t)rec12 & 15u) || ((uintptr_t)probs & 15u))
    return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  return mlp::infer(p->net, reinterpret_cast<const float4 *>(rec12), n, nullptr, reinterpret_cast<__half *>(probs),
                    nullptr, p->defensive, (cudaStream_t)stream);
}

extern "C" int ckr_internal_proposal_infer_stalled(ckr_proposal *p, const float *rec12, uint32_t n, uint16_t *probs,
                                                   uint32_t wait_tries, void *stream) {
  if (!p || !n || !rec12 || !probs || wait_tries == 0 || ((uintptr_t)rec12 & 15u) || ((uintptr_t)probs & 15u))
    return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  p->net.stall_tries = wait_tries;
  int st = mlp::infer(p->net, reinterpret_cast<const float4 *>(rec12), n, nullptr, reinterpret_cast<__half *>(probs),
                      nullptr, p->defensive, (cudaStream_t)stream);
  p->net.stall_tries = 0;
  return st;
}

extern "C" int ckr_proposal_train_step(ckr_proposal *p, const float *rec12, uint32_t n, void *stream) {
  if (!p || (n && !rec12) || ((uintptr_t)rec12 & 15u)) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  return mlp::train_step(p->net, reinterpret_cast<const float4 *>(rec12), n, nullptr, 0, (cudaStream_t)stream);
}

extern "C" int ckr_proposal_status(ckr_proposal *p, uint32_t *steps, float *last_loss) {
  if (!p || !steps || !last_loss) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  float sc[2];
  int err = 0;
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  CKR_CUDA_TRY(cudaMemcpy(sc, p->net.scalars, 8, cudaMemcpyDeviceToHost));
  CKR_CUDA_TRY(cudaMemcpy(&err, p->net.err, 4, cudaMemcpyDeviceToHost));
  *steps = p->net.step;
  *last_loss = sc[1];
  if (err) {
    CKR_CUDA_TRY(cudaMemset(p->net.err, 0, 4));
    return err;
  }
  return CKR_OK;
}

// Host sum of the per-CTA gradient partials of one batch (no update), for the
// CPU-oracle comparison of the backward pass.  Not part of the public ABI.
extern "C" int ckr_internal_proposal_gradients(ckr_proposal *p, const float *rec12, uint32_t n, float *grad,
                                               float *loss) {
  if (!p || !rec12 || !grad || !loss) return CKR_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(p->mu);
  int st = mlp::gradients(p->net, reinterpret_cast<const float4 *>(rec12), n, nullptr, 0, nullptr);
  if (st != CKR_OK) return st;
  CKR_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<float> part((size_t)p->net.grid * mlp::kNParams), lp(p->net.grid);
  CKR_CUDA_TRY(cudaMemcpy(part.data(), p->net.part, part.size() * 4, cudaMemcpyDeviceToHost));
  CKR_CUDA_TRY(cudaMemcpy(lp.data(), p->net.loss_part, lp.size() * 4, cudaMemcpyDeviceToHost));
  for (uint32_t j = 0; j < mlp::kNParams; ++j) {
    double g = 0;
    for (uint32_t c = 0; c < p->net.grid; ++c) g += part[(size_t)c * mlp::kNParams + j];
    grad[j] = (float)g;
  }
  double l = 0;
  for (float v : lp) l += v;
  *loss = (float)l;
  int err = 0;
  CKR_CUDA_TRY(cudaMemcpy(&err, p->net.err, 4, cudaMemcpyDeviceToHost));
  return err ? err : CKR_OK;
}
