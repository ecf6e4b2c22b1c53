// abi.cpp — status strings and CUDA error bookkeeping for the C ABI.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "ckr_internal.h"

namespace ckr {
namespace {
std::mutex g_mu;
std::string g_last_cuda;
}  // namespace

void note_cuda_error(cudaError_t err, const char *what, const char *file, int line) {
  std::lock_guard<std::mutex> lock(g_mu);
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s (%s) at %s:%d: %s", cudaGetErrorName(err), cudaGetErrorString(err), file, line,
                what);
  g_last_cuda = buf;
}
}  // namespace ckr

extern "C" int ckr_status_string(int status, char *buf, size_t len) {
  if (!buf || len == 0) return CKR_ERR_INVALID_ARGUMENT;
  std::string s;
  switch (status) {
    case CKR_OK: s = "ok"; break;
    case CKR_ERR_INVALID_ARGUMENT: s = "invalid argument"; break;
    case CKR_ERR_CUDA: {
      std::lock_guard<std::mutex> lock(ckr::g_mu);
      s = "CUDA error: " + (ckr::g_last_cuda.empty() ? std::string("unknown") : ckr::g_last_cuda);
      break;
    }
    case CKR_ERR_OUT_OF_MEMORY: s = "out of device memory"; break;
    case CKR_ERR_STACK_OVERFLOW: s = "traversal stack overflow"; break;
    case CKR_ERR_QUEUE_OVERFLOW: s = "wavefront queue overflow"; break;
    case CKR_ERR_ITERATION_LIMIT: s = "device loop iteration limit reached"; break;
    case CKR_ERR_NO_DEVICE: s = "no CUDA device"; break;
    case CKR_ERR_PARSE: s = "scene parse error"; break;
    case CKR_ERR_IO: s = "I/O error"; break;
    case CKR_ERR_TOO_LARGE: s = "size exceeds a limit"; break;
    default: s = "unknown status " + std::to_string(status); break;
  }
  std::snprintf(buf, len, "%s", s.c_str());
  return CKR_OK;
}
