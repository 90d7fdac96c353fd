// Internal helpers shared by the host and device translation units.
#pragma once

#include <cstdint>
#include <cstdio>
#include <exception>
#include <new>
#include <string>

#include "../../include/esr_gb300.h"

namespace esr {

// Records a message for esr_last_error() on this host thread and returns code.
int fail(int code, const std::string &msg);

}  // namespace esr

// Body guard of the host-side extern "C" entry points: a C++ exception
// (host memory exhausted, a thread that cannot be created) becomes an
// error status instead of crossing the C boundary.
#define ESR_HOST_TRY try {
#define ESR_HOST_CATCH                                                        \
  }                                                                           \
  catch (const std::bad_alloc &) {                                            \
    return esr::fail(ESR_ERR_ARG, "out of host memory");                      \
  }                                                                           \
  catch (const std::exception &ex) {                                          \
    return esr::fail(ESR_ERR_ARG, std::string("host error: ") + ex.what()); \
  }

#ifdef __CUDACC__
#include <cuda_runtime.h>

namespace esr {

// Returns ESR_ERR_CUDA with the CUDA error text if `e` is an error.
int cuda_check(cudaError_t e, const char *where);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Every device translation unit has its own status word (internal linkage,
// no relocatable device code needed); esr_device_status() ORs them all.
namespace {
__device__ int g_status;
}

__device__ __forceinline__ void raise_status(int bits) { atomicOr(&g_status, bits); }

}  // namespace esr

// Host reader of this translation unit's status word.
#define ESR_DEFINE_STATUS_READER(fn)                                          \
  int fn(int *bits, int clear, cudaStream_t s) {                              \
    int v = 0;                                                                \
    cudaError_t e = cudaMemcpyFromSymbolAsync(&v, esr::g_status, sizeof(int), \
                                              0, cudaMemcpyDeviceToHost, s);  \
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);                       \
    if (e == cudaSuccess && clear) {                                          \
      int z = 0;                                                              \
      e = cudaMemcpyToSymbolAsync(esr::g_status, &z, sizeof(int), 0,          \
                                  cudaMemcpyHostToDevice, s);                 \
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);                     \
    }                                                                         \
    if (e != cudaSuccess) return esr::cuda_check(e, #fn);                     \
    *bits |= v;                                                               \
    return ESR_OK;                                                            \
  }

#define ESR_LAUNCH_CHECK(where)                               \
  do {                                                        \
    cudaError_t _e = cudaGetLastError();                      \
    if (_e != cudaSuccess) return esr::cuda_check(_e, where); \
  } while (0)

#endif
