// Library-wide runtime pieces: CUDA error mapping, the device status word
// reader, and small vector kernels the mixed-precision solvers compose.
#include <cstdint>
#include <string>

#include "esr_internal.h"

// status readers of the other device translation units
int esr_status_gather_reduce(int *bits, int clear, cudaStream_t s);
int esr_status_swe(int *bits, int clear, cudaStream_t s);
int esr_status_cg(int *bits, int clear, cudaStream_t s);
int esr_status_gnn(int *bits, int clear, cudaStream_t s);
int esr_status_mesh_gpu(int *bits, int clear, cudaStream_t s);

namespace esr {
int cuda_check(cudaError_t e, const char *where) {
  return fail(ESR_ERR_CUDA, std::string(where) + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e));
}
}  // namespace esr

ESR_DEFINE_STATUS_READER(esr_status_runtime)

extern "C" int esr_device_status(int *status_out, int clear, void *stream) {
  if (!status_out) return esr::fail(ESR_ERR_ARG, "null status pointer");
  cudaStream_t s = esr::as_stream(stream);
  int bits = 0, st;
  if ((st = esr_status_gather_reduce(&bits, clear, s))) return st;
  if ((st = esr_status_swe(&bits, clear, s))) return st;
  if ((st = esr_status_cg(&bits, clear, s))) return st;
  if ((st = esr_status_gnn(&bits, clear, s))) return st;
  if ((st = esr_status_mesh_gpu(&bits, clear, s))) return st;
  if ((st = esr_status_runtime(&bits, clear, s))) return st;
  *status_out = bits;
  return ESR_OK;
}

namespace {

template <typename TI, typename TO>
__global__ void convert_kernel(const TI *__restrict__ in, TO *__restrict__ out, int64_t n, double scale) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = (TO)(scale * (double)in[i]);
}

template <typename TD>
__global__ void axpy_f64_kernel(double *__restrict__ x, const TD *__restrict__ d, double scale, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    x[i] = fma(scale, (double)d[i], x[i]);
}

int vec_grid(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152 * 8) g = 152 * 8;
  return (int)g;
}

}  // namespace

extern "C" int esr_convert(int dtype_in, const void *in, int dtype_out, void *out, int64_t n, double scale,
                           void *stream) {
  if (n < 0) return esr::fail(ESR_ERR_ARG, "negative size");
  if (n == 0) return ESR_OK;
  if (!in || !out) return esr::fail(ESR_ERR_ARG, "null pointer");
  cudaStream_t s = esr::as_stream(stream);
  const int g = vec_grid(n);
  if (dtype_in == ESR_F64 && dtype_out == ESR_F32)
    convert_kernel<double, float><<<g, 256, 0, s>>>((const double *)in, (float *)out, n, scale);
  else if (dtype_in == ESR_F32 && dtype_out == ESR_F64)
    convert_kernel<float, double><<<g, 256, 0, s>>>((const float *)in, (double *)out, n, scale);
  else if (dtype_in == ESR_F64 && dtype_out == ESR_F64)
    convert_kernel<double, double><<<g, 256, 0, s>>>((const double *)in, (double *)out, n, scale);
  else if (dtype_in == ESR_F32 && dtype_out == ESR_F32)
    convert_kernel<float, float><<<g, 256, 0, s>>>((const float *)in, (float *)out, n, scale);
  else
    return esr::fail(ESR_ERR_UNSUPPORTED, "esr_convert: dtype pair");
  ESR_LAUNCH_CHECK("esr_convert");
  return ESR_OK;
}

extern "C" int esr_axpy_f64(double *x, int dtype_d, const void *d, double scale, int64_t n, void *stream) {
  if (n < 0) return esr::fail(ESR_ERR_ARG, "negative size");
  if (n == 0) return ESR_OK;
  if (!x || !d) return esr::fail(ESR_ERR_ARG, "null pointer");
  cudaStream_t s = esr::as_stream(stream);
  const int g = vec_grid(n);
  if (dtype_d == ESR_F32) axpy_f64_kernel<float><<<g, 256, 0, s>>>(x, (const float *)d, scale, n);
  else if (dtype_d == ESR_F64) axpy_f64_kernel<double><<<g, 256, 0, s>>>(x, (const double *)d, scale, n);
  else return esr::fail(ESR_ERR_UNSUPPORTED, "esr_axpy_f64: dtype");
  ESR_LAUNCH_CHECK("esr_axpy_f64");
  return ESR_OK;
}
