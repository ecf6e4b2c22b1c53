// ckr_internal.h — helpers shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>

#include "../../include/ckr.h"

#define CKR_CUDA_TRY(expr)                                                        \
  do {                                                                            \
    cudaError_t ckr_err_ = (expr);                                                \
    if (ckr_err_ != cudaSuccess) {                                                \
      ckr::note_cuda_error(ckr_err_, #expr, __FILE__, __LINE__);                  \
      return ckr_err_ == cudaErrorMemoryAllocation ? CKR_ERR_OUT_OF_MEMORY        \
                                                   : CKR_ERR_CUDA;                \
    }                                                                             \
  } while (0)

namespace ckr {

// Records the last CUDA failure (readable via ckr_status_string(CKR_ERR_CUDA)).
void note_cuda_error(cudaError_t err, const char *what, const char *file, int line);

// Device allocation owned by the library; freed on destruction.
template <typename T>
struct DevBuf {
  T *ptr = nullptr;
  size_t count = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
  cudaError_t reserve(size_t n) {
    if (n <= count) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc((void **)&ptr, n * sizeof(T) + 16);
    if (e == cudaSuccess) count = n;
    return e;
  }
  size_t bytes() const { return count * sizeof(T); }
};

inline unsigned ceil_div(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

}  // namespace ckr
