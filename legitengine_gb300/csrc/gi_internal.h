// gi_internal.h -- host-side helpers shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>

#include "../../include/legit_gi.h"

namespace gi {

// Records `msg` as the calling thread's last error and returns `status`.
int fail(int status, const std::string& msg);
// Converts a CUDA error into GI_ERR_CUDA (or GI_OK) with a message naming `what`.
int check_cuda(cudaError_t e, const char* what);
// Counts kernel launches issued by the library.
void count_launches(uint64_t n);

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Every device allocation of the library goes through these: they count the
// live allocations (gi_debug_live_allocations) and honour the test hook that
// makes allocations fail (gi_debug_fail_allocations).  Same results as
// cudaMalloc / cudaFree / cudaMallocMipmappedArray / cudaFreeMipmappedArray.
cudaError_t device_alloc(void** p, size_t bytes);
void device_free(void* p);
cudaError_t device_alloc_mipmapped(cudaMipmappedArray_t* a, const cudaChannelFormatDesc* desc, cudaExtent extent,
                                   unsigned levels, unsigned flags);
void device_free_mipmapped(cudaMipmappedArray_t a);
template <class T> inline cudaError_t dmalloc(T** p, size_t bytes) {
  return device_alloc(reinterpret_cast<void**>(p), bytes);
}
inline void dfree(const void* p) { device_free(const_cast<void*>(p)); }

// Level geometry of the mip chain: level k is floor(size / 2^k).
inline int level_dim(int size, int level) { return size >> level; }

}  // namespace gi

#define GI_CHECK_ARG(cond, msg)                                   \
  do {                                                            \
    if (!(cond)) return ::gi::fail(GI_ERR_INVALID_ARGUMENT, msg); \
  } while (0)

#define GI_CHECK_LAUNCH(what)                                              \
  do {                                                                     \
    cudaError_t e_ = cudaGetLastError();                                   \
    if (e_ != cudaSuccess) return ::gi::check_cuda(e_, what);              \
  } while (0)
