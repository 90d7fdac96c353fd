// Arithmetic with explicit rounding and deterministic block reductions.
#pragma once

#include <cstdint>

// ops<T>: one IEEE operation each, round-to-nearest, never contracted into
// an FMA.  Integer types wrap like the reference's int64 torch ops.
template <typename T>
struct ops;

template <>
struct ops<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double div_count(double a, int64_t c) { return __ddiv_rn(a, (double)c); }
};

template <>
struct ops<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float div_count(float a, int64_t c) { return __fdiv_rn(a, (float)c); }
};

template <typename I, typename U>
struct int_ops {
  static __device__ __forceinline__ I add(I a, I b) { return (I)((U)a + (U)b); }
  static __device__ __forceinline__ I sub(I a, I b) { return (I)((U)a - (U)b); }
  static __device__ __forceinline__ I mul(I a, I b) { return (I)((U)a * (U)b); }
  // floor division, as torch's scatter_reduce 'mean' on integer tensors
  static __device__ __forceinline__ I div_count(I a, int64_t c) {
    int64_t q = (int64_t)a / c;
    if (((int64_t)a % c != 0) && ((a < 0) != (c < 0))) q -= 1;
    return (I)q;
  }
};

template <>
struct ops<int32_t> : int_ops<int32_t, uint32_t> {};
template <>
struct ops<int64_t> : int_ops<int64_t, uint64_t> {};

namespace esr {

// Sum of one double per thread over the block, in a fixed order (warp
// shuffle tree, then the warp totals in warp order).  Result valid in
// every thread.  `s_red` holds blockDim/32 doubles.
template <int THREADS>
__device__ __forceinline__ double block_sum_fixed(double v, double *s_red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = (lane < THREADS / 32) ? s_red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) s_red[0] = t;
  }
  __syncthreads();
  t = s_red[0];
  __syncthreads();
  return t;
}

// Publishes this block's partial and returns true in every thread of the
// block that finished last (which then owns the final combine).  The
// combine reads the partials in block order, so the result does not depend
// on which block finished last.
__device__ __forceinline__ bool last_block_done(double block_total, double *partial, unsigned int *counter) {
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = block_total;
    __threadfence();
    unsigned int ticket = atomicAdd(counter, 1u);
    s_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

}  // namespace esr
