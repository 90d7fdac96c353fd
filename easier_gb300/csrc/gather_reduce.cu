// Selector gather, Reducer segmented reduce, aggregators and dot products.
//
// Everything here is deterministic: there are no floating-point atomics.
// Segmented reductions run one thread per (row, column) and walk the segment
// in ascending order, which is the order the reference's CPU
// scatter_reduce_ accumulates in, so sums are bitwise equal to it.
#include <cmath>
#include <cstdint>
#include <mutex>

#include "esr_internal.h"
#include "reduce_util.cuh"

namespace {

constexpr int kThreads = 256;

int grid_for(int64_t work, int threads = kThreads) {
  int64_t g = (work + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;  // grid-stride beyond 32 CTAs per SM
  return (int)g;
}

// ---------------------------------------------------------------- gather --
template <typename V>
__global__ void __launch_bounds__(kThreads)
gather_kernel(const V *__restrict__ x, int64_t n_in, int64_t vpr,
              const int32_t *__restrict__ idx, int64_t m, V *__restrict__ y) {
  const int64_t total = m * vpr;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
    int64_t e, c;
    if (vpr == 1) {
      e = t;
      c = 0;
    } else {
      e = t / vpr;
      c = t - e * vpr;
    }
    const int32_t s = __ldg(idx + e);
    if (s < 0 || (int64_t)s >= n_in) {
      esr::raise_status(ESR_DEV_IDX_RANGE);
      continue;
    }
    y[t] = x[(int64_t)s * vpr + c];
  }
}

template <typename V>
int launch_gather(const void *x, int64_t n_in, int64_t row_bytes, const int32_t *idx, int64_t m,
                  void *y, cudaStream_t st) {
  const int64_t vpr = row_bytes / (int64_t)sizeof(V);
  gather_kernel<V><<<grid_for(m * vpr), kThreads, 0, st>>>((const V *)x, n_in, vpr, idx, m, (V *)y);
  ESR_LAUNCH_CHECK("esr_gather");
  return ESR_OK;
}

// ----------------------------------------------------------- segreduce --
template <typename T>
struct Acc {  // accumulation type
  using type = T;
};

template <typename T>
__device__ __forceinline__ bool is_nan(T v) {
  return v != v;
}

template <typename T, int OP>
__global__ void __launch_bounds__(kThreads)
segreduce_kernel(const T *__restrict__ t, int64_t cols, const int32_t *__restrict__ rowptr,
                 const int32_t *__restrict__ perm, int64_t n, T *__restrict__ out) {
  const int64_t total = n * cols;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += stride) {
    int64_t i, c;
    if (cols == 1) {
      i = g;
      c = 0;
    } else {
      i = g / cols;
      c = g - i * cols;
    }
    const int32_t b = __ldg(rowptr + i), e = __ldg(rowptr + i + 1);
    if (b >= e) continue;  // unreferenced row keeps `out`
    T acc;
    if (OP == ESR_REDUCE_SUM || OP == ESR_REDUCE_MEAN) acc = T(0);
    else if (OP == ESR_REDUCE_PROD) acc = T(1);
    for (int32_t k = b; k < e; ++k) {
      const int64_t src = perm ? (int64_t)__ldg(perm + k) : (int64_t)k;
      const T v = t[src * cols + c];
      if (OP == ESR_REDUCE_SUM || OP == ESR_REDUCE_MEAN) acc = ops<T>::add(acc, v);
      else if (OP == ESR_REDUCE_PROD) acc = ops<T>::mul(acc, v);
      else if (OP == ESR_REDUCE_AMAX) {
        if (k == b) acc = v;
        else acc = is_nan(v) ? v : ((acc < v) ? v : acc);
      } else {
        if (k == b) acc = v;
        else acc = is_nan(v) ? v : ((v < acc) ? v : acc);
      }
    }
    if (OP == ESR_REDUCE_MEAN) acc = ops<T>::div_count(acc, (int64_t)(e - b));
    out[i * cols + c] = acc;
  }
}

template <typename T>
int launch_segreduce(int op, const void *t, int64_t cols, const int32_t *rowptr, const int32_t *perm,
                     int64_t n, void *out, cudaStream_t st) {
  const int g = grid_for(n * cols);
  switch (op) {
    case ESR_REDUCE_SUM:
      segreduce_kernel<T, ESR_REDUCE_SUM><<<g, kThreads, 0, st>>>((const T *)t, cols, rowptr, perm, n, (T *)out);
      break;
    case ESR_REDUCE_PROD:
      segreduce_kernel<T, ESR_REDUCE_PROD><<<g, kThreads, 0, st>>>((const T *)t, cols, rowptr, perm, n, (T *)out);
      break;
    case ESR_REDUCE_MEAN:
      segreduce_kernel<T, ESR_REDUCE_MEAN><<<g, kThreads, 0, st>>>((const T *)t, cols, rowptr, perm, n, (T *)out);
      break;
    case ESR_REDUCE_AMAX:
      segreduce_kernel<T, ESR_REDUCE_AMAX><<<g, kThreads, 0, st>>>((const T *)t, cols, rowptr, perm, n, (T *)out);
      break;
    case ESR_REDUCE_AMIN:
      segreduce_kernel<T, ESR_REDUCE_AMIN><<<g, kThreads, 0, st>>>((const T *)t, cols, rowptr, perm, n, (T *)out);
      break;
    default:
      return esr::fail(ESR_ERR_ARG, "unknown reduce op");
  }
  ESR_LAUNCH_CHECK("esr_segreduce");
  return ESR_OK;
}

// ---------------------------------------------------------- aggregate --
// Two launches: blocks reduce fixed row ranges into partials, then one
// block per column reduces the partials in block order.
constexpr int64_t kAggRowsPerBlock = 8192;
constexpr int kAggMaxBlocks = 1024;

int64_t agg_blocks(int64_t n) {
  int64_t b = (n + kAggRowsPerBlock - 1) / kAggRowsPerBlock;
  if (b < 1) b = 1;
  if (b > kAggMaxBlocks) b = kAggMaxBlocks;
  return b;
}

template <typename T>
struct AggTraits {
  using acc_t = double;
};
template <>
struct AggTraits<int32_t> {
  using acc_t = int64_t;
};
template <>
struct AggTraits<int64_t> {
  using acc_t = int64_t;
};

template <typename A, int AGG>
__device__ __forceinline__ A agg_identity() {
  if (AGG == ESR_AGG_PROD) return A(1);
  if (AGG == ESR_AGG_MAX || AGG == ESR_AGG_MIN) return A(0);  // replaced by first value
  return A(0);
}

template <typename A, int AGG>
__device__ __forceinline__ A agg_combine(A a, A b, bool a_valid) {
  if (!a_valid) {
    if (AGG == ESR_AGG_SUM || AGG == ESR_AGG_NORM) return b;
    if (AGG == ESR_AGG_PROD) return b;
    return b;
  }
  if (AGG == ESR_AGG_SUM || AGG == ESR_AGG_NORM) return ops<A>::add(a, b);
  if (AGG == ESR_AGG_PROD) return ops<A>::mul(a, b);
  if (AGG == ESR_AGG_MAX) return is_nan(b) ? b : (is_nan(a) ? a : ((a < b) ? b : a));
  return is_nan(b) ? b : (is_nan(a) ? a : ((b < a) ? b : a));
}

// Block-wide fixed-order combine of one value per thread; result in lane 0
// of warp 0.  `valid` marks threads that saw at least one element.
template <typename A, int AGG>
__device__ A block_combine(A v, bool valid, bool &any_valid) {
  __shared__ A s_val[kThreads];
  __shared__ int s_ok[kThreads];
  s_val[threadIdx.x] = v;
  s_ok[threadIdx.x] = valid ? 1 : 0;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      const int o = threadIdx.x + w;
      if (s_ok[o]) {
        s_val[threadIdx.x] = agg_combine<A, AGG>(s_val[threadIdx.x], s_val[o], s_ok[threadIdx.x] != 0);
        s_ok[threadIdx.x] = 1;
      }
    }
    __syncthreads();
  }
  A r = s_val[0];
  any_valid = s_ok[0] != 0;
  __syncthreads();
  return r;
}

template <typename T, int AGG>
__global__ void __launch_bounds__(kThreads)
agg_partial_kernel(const T *__restrict__ t, int64_t n, int64_t cols, int64_t rows_per_block,
                   typename AggTraits<T>::acc_t *__restrict__ partial, int *__restrict__ partial_ok) {
  using A = typename AggTraits<T>::acc_t;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  int64_t r1 = r0 + rows_per_block;
  if (r1 > n) r1 = n;
  for (int64_t c = 0; c < cols; ++c) {
    A acc = agg_identity<A, AGG>();
    bool valid = false;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      A v = (A)t[r * cols + c];
      if (AGG == ESR_AGG_NORM) v = ops<A>::mul(v, v);
      acc = agg_combine<A, AGG>(acc, v, valid);
      valid = true;
    }
    bool any = false;
    A tot = block_combine<A, AGG>(acc, valid, any);
    if (threadIdx.x == 0) {
      partial[(int64_t)blockIdx.x * cols + c] = tot;
      partial_ok[(int64_t)blockIdx.x * cols + c] = any ? 1 : 0;
    }
  }
}

template <typename T, int AGG>
__global__ void __launch_bounds__(kThreads)
agg_final_kernel(const typename AggTraits<T>::acc_t *__restrict__ partial, const int *__restrict__ partial_ok,
                 int64_t nblocks, int64_t cols, T *__restrict__ out) {
  using A = typename AggTraits<T>::acc_t;
  const int64_t c = blockIdx.x;
  A acc = agg_identity<A, AGG>();
  bool valid = false;
  for (int64_t b = threadIdx.x; b < nblocks; b += blockDim.x) {
    if (partial_ok[b * cols + c]) {
      acc = agg_combine<A, AGG>(acc, partial[b * cols + c], valid);
      valid = true;
    }
  }
  bool any = false;
  A tot = block_combine<A, AGG>(acc, valid, any);
  if (threadIdx.x == 0) {
    if (!any) {
      // empty input: sum/norm -> 0, prod -> 1, max/min -> NaN (torch raises;
      // the host rejects empty max/min before calling)
      if (AGG == ESR_AGG_PROD) tot = A(1);
      else tot = A(0);
    }
    if (AGG == ESR_AGG_NORM) out[c] = (T)sqrt((double)tot);
    else out[c] = (T)tot;
  }
}

template <typename T, int AGG>
int launch_agg_t(const void *t, int64_t n, int64_t cols, void *out, void *ws, cudaStream_t st) {
  using A = typename AggTraits<T>::acc_t;
  const int64_t nb = agg_blocks(n);
  const int64_t rpb = (n + nb - 1) / nb;
  A *partial = (A *)ws;
  int *ok = (int *)((char *)ws + nb * cols * sizeof(double));
  agg_partial_kernel<T, AGG><<<(int)nb, kThreads, 0, st>>>((const T *)t, n, cols, rpb < 1 ? 1 : rpb, partial, ok);
  ESR_LAUNCH_CHECK("esr_aggregate/partial");
  agg_final_kernel<T, AGG><<<(int)cols, kThreads, 0, st>>>(partial, ok, nb, cols, (T *)out);
  ESR_LAUNCH_CHECK("esr_aggregate/final");
  return ESR_OK;
}

template <typename T>
int launch_agg(int agg, const void *t, int64_t n, int64_t cols, void *out, void *ws, cudaStream_t st) {
  switch (agg) {
    case ESR_AGG_SUM: return launch_agg_t<T, ESR_AGG_SUM>(t, n, cols, out, ws, st);
    case ESR_AGG_PROD: return launch_agg_t<T, ESR_AGG_PROD>(t, n, cols, out, ws, st);
    case ESR_AGG_NORM: return launch_agg_t<T, ESR_AGG_NORM>(t, n, cols, out, ws, st);
    case ESR_AGG_MAX: return launch_agg_t<T, ESR_AGG_MAX>(t, n, cols, out, ws, st);
    case ESR_AGG_MIN: return launch_agg_t<T, ESR_AGG_MIN>(t, n, cols, out, ws, st);
    default: return esr::fail(ESR_ERR_ARG, "unknown aggregator");
  }
}

// ----------------------------------------------------------------- dot --
template <typename T>
__global__ void __launch_bounds__(kThreads)
dot_kernel(const T *__restrict__ a, const T *__restrict__ b, int64_t n, double *__restrict__ partial,
           unsigned int *__restrict__ counter, double *__restrict__ out) {
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    acc = fma((double)a[i], (double)b[i], acc);
  __shared__ double s_red[kThreads / 32];
  double tot = esr::block_sum_fixed<kThreads>(acc, s_red);
  if (esr::last_block_done(tot, partial, counter)) {
    double v = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) v += __ldcg(partial + k);
    double all = esr::block_sum_fixed<kThreads>(v, s_red);
    if (threadIdx.x == 0) {
      *out = all;
      *counter = 0u;
    }
  }
}

constexpr int kDotMaxBlocks = 152 * 4;

int dot_blocks(int64_t n) {
  int64_t g = (n + kThreads - 1) / kThreads;
  if (g < 1) g = 1;
  if (g > kDotMaxBlocks) g = kDotMaxBlocks;
  return (int)g;
}

}  // namespace

ESR_DEFINE_STATUS_READER(esr_status_gather_reduce)

extern "C" int esr_gather(const void *x, int64_t n_in, int64_t row_bytes, const int32_t *idx, int64_t m,
                          void *y, void *stream) {
  if (m < 0 || n_in < 0 || row_bytes < 0) return esr::fail(ESR_ERR_ARG, "esr_gather: negative size");
  if (m == 0 || row_bytes == 0) return ESR_OK;
  if (!x || !idx || !y) return esr::fail(ESR_ERR_ARG, "esr_gather: null pointer");
  cudaStream_t st = esr::as_stream(stream);
  const uintptr_t al = (uintptr_t)x | (uintptr_t)y;
  if (row_bytes % 16 == 0 && al % 16 == 0) return launch_gather<uint4>(x, n_in, row_bytes, idx, m, y, st);
  if (row_bytes % 8 == 0 && al % 8 == 0) return launch_gather<uint2>(x, n_in, row_bytes, idx, m, y, st);
  if (row_bytes % 4 == 0 && al % 4 == 0) return launch_gather<uint32_t>(x, n_in, row_bytes, idx, m, y, st);
  return launch_gather<uint8_t>(x, n_in, row_bytes, idx, m, y, st);
}

extern "C" int esr_segreduce(int dtype, int op, const void *t, int64_t row_elems, const int32_t *rowptr,
                             const int32_t *perm, int64_t n, void *out, void *stream) {
  if (n < 0 || row_elems < 0) return esr::fail(ESR_ERR_ARG, "esr_segreduce: negative size");
  if (n == 0 || row_elems == 0) return ESR_OK;
  if (!rowptr || !out) return esr::fail(ESR_ERR_ARG, "esr_segreduce: null pointer");
  cudaStream_t st = esr::as_stream(stream);
  switch (dtype) {
    case ESR_F32: return launch_segreduce<float>(op, t, row_elems, rowptr, perm, n, out, st);
    case ESR_F64: return launch_segreduce<double>(op, t, row_elems, rowptr, perm, n, out, st);
    case ESR_I32: return launch_segreduce<int32_t>(op, t, row_elems, rowptr, perm, n, out, st);
    case ESR_I64: return launch_segreduce<int64_t>(op, t, row_elems, rowptr, perm, n, out, st);
    default: return esr::fail(ESR_ERR_UNSUPPORTED, "esr_segreduce: dtype");
  }
}

extern "C" int64_t esr_aggregate_workspace_bytes(int64_t n, int64_t cols) {
  if (n < 0 || cols < 0) return -1;
  return agg_blocks(n) * (cols < 1 ? 1 : cols) * (int64_t)(sizeof(double) + sizeof(int));
}

extern "C" int esr_aggregate(int dtype, int agg, const void *t, int64_t n, int64_t cols, void *out,
                             void *workspace, void *stream) {
  if (n < 0 || cols < 0) return esr::fail(ESR_ERR_ARG, "esr_aggregate: negative size");
  if (cols == 0) return ESR_OK;
  if (!out || !workspace || (n && !t)) return esr::fail(ESR_ERR_ARG, "esr_aggregate: null pointer");
  if (cols > 65535) return esr::fail(ESR_ERR_UNSUPPORTED, "esr_aggregate: too many columns");
  cudaStream_t st = esr::as_stream(stream);
  switch (dtype) {
    case ESR_F32: return launch_agg<float>(agg, t, n, cols, out, workspace, st);
    case ESR_F64: return launch_agg<double>(agg, t, n, cols, out, workspace, st);
    case ESR_I32:
      if (agg == ESR_AGG_NORM) return esr::fail(ESR_ERR_UNSUPPORTED, "norm of an integer tensor");
      return launch_agg<int32_t>(agg, t, n, cols, out, workspace, st);
    case ESR_I64:
      if (agg == ESR_AGG_NORM) return esr::fail(ESR_ERR_UNSUPPORTED, "norm of an integer tensor");
      return launch_agg<int64_t>(agg, t, n, cols, out, workspace, st);
    default: return esr::fail(ESR_ERR_UNSUPPORTED, "esr_aggregate: dtype");
  }
}

extern "C" int64_t esr_dot_workspace_bytes(int64_t n) {
  if (n < 0) return -1;
  return (int64_t)kDotMaxBlocks * sizeof(double) + 64;
}

extern "C" int esr_dot(int dtype, const void *a, const void *b, int64_t n, double *out_f64, void *workspace,
                       void *stream) {
  if (n < 0) return esr::fail(ESR_ERR_ARG, "esr_dot: negative size");
  if (!out_f64 || !workspace || (n && (!a || !b))) return esr::fail(ESR_ERR_ARG, "esr_dot: null pointer");
  cudaStream_t st = esr::as_stream(stream);
  double *partial = (double *)workspace;
  unsigned int *counter = (unsigned int *)((char *)workspace + kDotMaxBlocks * sizeof(double));
  const int g = dot_blocks(n);
  switch (dtype) {
    case ESR_F32:
      dot_kernel<float><<<g, kThreads, 0, st>>>((const float *)a, (const float *)b, n, partial, counter, out_f64);
      break;
    case ESR_F64:
      dot_kernel<double><<<g, kThreads, 0, st>>>((const double *)a, (const double *)b, n, partial, counter, out_f64);
      break;
    default: return esr::fail(ESR_ERR_UNSUPPORTED, "esr_dot: dtype");
  }
  ESR_LAUNCH_CHECK("esr_dot");
  return ESR_OK;
}

// ------------------------------------------------------ allocation-free --
// esr_aggregate_noalloc runs the same two launches as esr_aggregate, but its
// block partials live in the file-scope device array below instead of a
// workspace the caller allocates.  It exists for callers that cannot call
// cudaMalloc at the point where they need an aggregate: cudaMalloc/cudaFree
// synchronise the whole device (stalling every other stream of a time-step
// loop or solver), they can fail with out-of-memory in the middle of a run,
// and some host applications hand all device memory to their own pool and
// forbid libraries from allocating.  The array is a fixed 1 MiB per device
// that loaded this library, held until the process exits.
static __device__ __align__(256) unsigned char g_agg_noalloc_scratch[ESR_AGG_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kNoAllocMaxDevices = 64;
// The array's device address belongs to one CUDA context: the primary
// context of a device, recreated with a new address after cudaDeviceReset,
// or a context the caller created with the driver API.  It is cached per
// device together with the unique ID (cuCtxGetId) of the context it was
// looked up in, and looked up again whenever the current context's ID
// differs.
std::mutex g_noalloc_mu;
struct NoAllocAddr {
  unsigned long long ctx_id;
  void *addr;
};
NoAllocAddr g_noalloc_addr[kNoAllocMaxDevices];

using CtxGetCurrentFn = int (*)(void **);
using CtxGetIdFn = int (*)(void *, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current;
CtxGetIdFn g_ctx_get_id;

// Driver entry points through the runtime (no link against libcuda).
cudaError_t noalloc_driver_fns() {
  if (g_ctx_get_current && g_ctx_get_id) return cudaSuccess;
  void *a = nullptr, *b = nullptr;
  cudaDriverEntryPointQueryResult qa, qb;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa);
  if (e != cudaSuccess) return e;
  e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb);
  if (e != cudaSuccess) return e;
  if (qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
    return cudaErrorSymbolNotFound;
  g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(a);
  g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(b);
  return cudaSuccess;
}

// ID of the context current on this thread; 0 when there is none yet.
cudaError_t noalloc_ctx_id(unsigned long long *id) {
  *id = 0;
  void *ctx = nullptr;
  if (g_ctx_get_current(&ctx) != 0) return cudaErrorDeviceUninitialized;
  if (!ctx) return cudaSuccess;
  if (g_ctx_get_id(ctx, id) != 0) return cudaErrorDeviceUninitialized;
  return cudaSuccess;
}
}  // namespace

extern "C" int esr_aggregate_noalloc(int dtype, int agg, const void *t, int64_t n, int64_t cols, void *out,
                                     void *stream) {
  if (n < 0 || cols < 0) return esr::fail(ESR_ERR_ARG, "esr_aggregate_noalloc: negative size");
  if (cols == 0) return ESR_OK;
  if (!out || (n && !t)) return esr::fail(ESR_ERR_ARG, "esr_aggregate_noalloc: null pointer");
  const int64_t need = esr_aggregate_workspace_bytes(n, cols);
  if (need > (int64_t)ESR_AGG_NOALLOC_SCRATCH_BYTES)
    return esr::fail(ESR_ERR_ARG, "esr_aggregate_noalloc: n=" + std::to_string(n) + ", cols=" +
                                      std::to_string(cols) + " needs " + std::to_string(need) +
                                      " bytes of scratch, more than the " +
                                      std::to_string((long long)ESR_AGG_NOALLOC_SCRATCH_BYTES) +
                                      " bytes of the static array (any cols <= " +
                                      std::to_string(ESR_AGG_NOALLOC_MAX_COLS) +
                                      " fits); use esr_aggregate with a workspace");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_aggregate_noalloc/cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices) return esr::fail(ESR_ERR_UNSUPPORTED, "esr_aggregate_noalloc: device ordinal");
  void *ws = nullptr;
  {
    // Set-up, on the first call in a context: look up the array's device
    // address (this may load the module, so it must not be the first call
    // inside a stream capture).
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    e = noalloc_driver_fns();
    if (e != cudaSuccess) return esr::cuda_check(e, "esr_aggregate_noalloc/driver entry points");
    unsigned long long id = 0;
    e = noalloc_ctx_id(&id);
    if (e != cudaSuccess) return esr::cuda_check(e, "esr_aggregate_noalloc/current context");
    NoAllocAddr &slot = g_noalloc_addr[dev];
    if (id == 0 || slot.addr == nullptr || slot.ctx_id != id) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_agg_noalloc_scratch);
      if (e != cudaSuccess) return esr::cuda_check(e, "esr_aggregate_noalloc/cudaGetSymbolAddress");
      if (id == 0) {  // the lookup made the device's primary context current
        e = noalloc_ctx_id(&id);
        if (e != cudaSuccess) return esr::cuda_check(e, "esr_aggregate_noalloc/current context");
      }
      slot.ctx_id = id;
      slot.addr = p;
    }
    ws = slot.addr;
  }
  // Every partial slot the second launch reads is written by the first one,
  // so nothing needs clearing between calls.
  cudaStream_t st = esr::as_stream(stream);
  switch (dtype) {
    case ESR_F32: return launch_agg<float>(agg, t, n, cols, out, ws, st);
    case ESR_F64: return launch_agg<double>(agg, t, n, cols, out, ws, st);
    case ESR_I32:
      if (agg == ESR_AGG_NORM) return esr::fail(ESR_ERR_UNSUPPORTED, "norm of an integer tensor");
      return launch_agg<int32_t>(agg, t, n, cols, out, ws, st);
    case ESR_I64:
      if (agg == ESR_AGG_NORM) return esr::fail(ESR_ERR_UNSUPPORTED, "norm of an integer tensor");
      return launch_agg<int64_t>(agg, t, n, cols, out, ws, st);
    default: return esr::fail(ESR_ERR_UNSUPPORTED, "esr_aggregate_noalloc: dtype");
  }
}
