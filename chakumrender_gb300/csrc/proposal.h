// proposal.h — the learned light-selection proposal object behind the C ABI
// (ckr_proposal_*, ckr_render_learned): the network and the renderer's buffers
// for it.
#pragma once
#include <cuda_fp16.h>

#include <mutex>

#include "ckr_internal.h"
#include "mlp.h"

struct ckr_proposal {
  int device = 0;
  ckr::mlp::Net net;
  float defensive = 0.2f;   // uniform fraction of the selection mixture
  uint32_t batch = 65536;      // training records kept per bounce
  uint32_t minibatch = 16384;  // records per Adam step (batch / minibatch steps per bounce)
  uint32_t max_steps = 0;      // training stops after this many Adam steps (0: never)
  int train = 1;
  std::mutex mu;
  // Renderer buffers, grown on demand.
  ckr::DevBuf<uint16_t> sel[2];   // selection CDFs of the current / previous bounce (64 x u16 per row)
  ckr::DevBuf<float4> rec;        // training records (3 float4 each)
  ckr::DevBuf<uint32_t> rec_count;
  ckr::DevBuf<uint32_t> prev_row, sh_rec;
  // Training that overlaps rendering (ckr_render_learned): step k's records
  // (rec_k[k & 1]) are trained on `train_stream` while the renderer runs step
  // k + 1; each training publishes the weights it produced (img_pub[k & 1]), and
  // step k + 2's inference waits for them (done[k & 1]) before it reads that copy
  // and before its shading refills rec_k[k & 1].
  cudaStream_t train_stream = nullptr;
  cudaEvent_t rec_ready[2] = {}, done[2] = {};
  ckr::DevBuf<float4> rec_k[2];
  ckr::DevBuf<uint32_t> rec_count_k[2];
  ckr::DevBuf<uint8_t> img_pub[2];
  ~ckr_proposal() {
    for (int i = 0; i < 2; ++i) {
      if (rec_ready[i]) cudaEventDestroy(rec_ready[i]);
      if (done[i]) cudaEventDestroy(done[i]);
    }
    if (train_stream) cudaStreamDestroy(train_stream);
  }
};
