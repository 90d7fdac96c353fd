/* The C ABI from plain C (C99) on the device: a shallow-water style edge
 * exchange on the tutorial mesh -- Selector gather of a cell field to the
 * edges' sources (esr_gather), then the Reducer's in-order segment sum over
 * destinations (esr_segreduce with the stable CSR of the index) -- on the
 * caller's stream, checked bitwise against the same loops on the host.
 * Usage: c_abi_device <n>; exit 0 and "ok" on success. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime_api.h>

#include "esr_gb300.h"

#define CHECK(call)                                                    \
  do {                                                                 \
    if ((call) != ESR_OK) {                                            \
      fprintf(stderr, "%s failed: %s\n", #call, esr_last_error());     \
      return 1;                                                        \
    }                                                                  \
  } while (0)
#define CUDA(call)                                                                  \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      fprintf(stderr, "%s failed: %s\n", #call, cudaGetErrorString(e_));            \
      return 1;                                                                     \
    }                                                                               \
  } while (0)

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  const int64_t n = atoll(argv[1]);
  int64_t nc, ne, nbc, np;
  CHECK(esr_mesh_sizes(n, &nc, &ne, &nbc, &np));
  int64_t *src = malloc(ne * sizeof *src), *dst = malloc(ne * sizeof *dst);
  int64_t *cells = malloc(3 * nc * sizeof *cells), *bcells = malloc(nbc * sizeof *bcells);
  int64_t *bpoints = malloc(2 * nbc * sizeof *bpoints);
  double *points = malloc(2 * np * sizeof *points);
  int64_t *rowptr = malloc((nc + 1) * sizeof *rowptr), *perm = malloc(ne * sizeof *perm);
  int32_t *src32 = malloc(ne * sizeof *src32), *rowptr32 = malloc((nc + 1) * sizeof *rowptr32);
  int32_t *perm32 = malloc(ne * sizeof *perm32);
  double *x = malloc(nc * sizeof *x), *y = malloc(ne * sizeof *y), *out = malloc(nc * sizeof *out);
  if (!src || !dst || !cells || !bcells || !bpoints || !points || !rowptr || !perm || !src32 || !rowptr32 ||
      !perm32 || !x || !y || !out)
    return 1;
  CHECK(esr_mesh_triangular(n, src, dst, cells, bcells, bpoints, points));
  CHECK(esr_csr_from_index(dst, ne, nc, rowptr, perm));
  for (int64_t e = 0; e < ne; ++e) {
    src32[e] = (int32_t)src[e];
    perm32[e] = (int32_t)perm[e];
  }
  for (int64_t i = 0; i <= nc; ++i) rowptr32[i] = (int32_t)rowptr[i];
  for (int64_t c = 0; c < nc; ++c) x[c] = sin(0.37 * (double)c) + 1e-3 * (double)c;

  cudaStream_t s;
  CUDA(cudaStreamCreate(&s));
  double *dx, *dy, *dout;
  int32_t *dsrc, *drow, *dperm;
  CUDA(cudaMalloc((void **)&dx, nc * sizeof(double)));
  CUDA(cudaMalloc((void **)&dy, ne * sizeof(double)));
  CUDA(cudaMalloc((void **)&dout, nc * sizeof(double)));
  CUDA(cudaMalloc((void **)&dsrc, ne * sizeof(int32_t)));
  CUDA(cudaMalloc((void **)&drow, (nc + 1) * sizeof(int32_t)));
  CUDA(cudaMalloc((void **)&dperm, ne * sizeof(int32_t)));
  CUDA(cudaMemcpyAsync(dx, x, nc * sizeof(double), cudaMemcpyHostToDevice, s));
  CUDA(cudaMemcpyAsync(dsrc, src32, ne * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  CUDA(cudaMemcpyAsync(drow, rowptr32, (nc + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  CUDA(cudaMemcpyAsync(dperm, perm32, ne * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  CUDA(cudaMemsetAsync(dout, 0, nc * sizeof(double), s));
  CHECK(esr_gather(dx, nc, sizeof(double), dsrc, ne, dy, (void *)s));
  CHECK(esr_segreduce(ESR_F64, ESR_REDUCE_SUM, dy, 1, drow, dperm, nc, dout, (void *)s));
  CUDA(cudaMemcpyAsync(y, dy, ne * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUDA(cudaMemcpyAsync(out, dout, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUDA(cudaStreamSynchronize(s));
  int status = 0;
  CHECK(esr_device_status(&status, 1, (void *)s));

  int bad = status != 0;
  for (int64_t e = 0; e < ne && !bad; ++e) bad = y[e] != x[src[e]];
  for (int64_t i = 0; i < nc && !bad; ++i) {
    double acc = 0.0;
    int first = 1;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      acc = first ? x[src[perm[k]]] : acc + x[src[perm[k]]];
      first = 0;
    }
    bad = out[i] != acc;
  }
  cudaFree(dx); cudaFree(dy); cudaFree(dout); cudaFree(dsrc); cudaFree(drow); cudaFree(dperm);
  cudaStreamDestroy(s);
  free(src); free(dst); free(cells); free(bcells); free(bpoints); free(points); free(rowptr); free(perm);
  free(src32); free(rowptr32); free(perm32); free(x); free(y); free(out);
  if (bad) {
    fprintf(stderr, "mismatch\n");
    return 1;
  }
  printf("ok\n");
  return 0;
}
