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
};
