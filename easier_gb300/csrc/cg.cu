// Linsys SpMV and fused preconditioned CG.
//
// Matrix layout: SELL-32 (slices of 32 consecutive rows, each slice stored
// slot-major: element (slice s, slot k, lane l) at slice_ptr[s] + 32*k + l,
// col = -1 marks padding).  A warp reads one slot of 32 rows with one
// coalesced 128-byte load; each thread still walks its own row's entries in
// the reference's edge order, so the exact SpMV is bitwise the reference's
//   y = reducer(selector(x) * Ae) + x * Av      (easier/numeric/linsys.py:23-24)
//
// PCG follows easier/numeric/solver/cg.py:
//   Init   :49-53   r = b - A x; z = M r; p = z; bnorm = ||b||
//   Step   :68-76   Ap = A p; alpha = r.z / p.Ap; r -= alpha Ap; x += alpha p
//   test   :150-153 stop when rnorm <= tol (or the iteration cap)
//   Update :90-95   z = M r; beta = r.z_new / r.z; p = z + beta p
// Native precision: three launches per iteration (spmv + p.Ap; update +
// r.r + r.z; p update).  Mixed precision: two launches per iteration (the p
// update is folded into the SpMV, recomputing z + beta p for the gathered
// columns on the FP32 pipes), plus an FP64 true-residual replacement every
// k iterations.  Every global dot is finished by the last block to arrive,
// reading the block partials in block order (deterministic, no floating
// atomics).  The stopping test runs on the device; launches after
// convergence return at once, so the host can enqueue iterations in chunks
// and poll.
#include <cmath>
#include <cstdint>

#include "esr_internal.h"
#include "reduce_util.cuh"

namespace {

constexpr int kCgThreads = 256;
constexpr int kCgMaxBlocks = 152 * 8;

struct CgWork {
  esr_cg_scalars s;
  unsigned int counter[8];
  double partial[3][kCgMaxBlocks];
};
static_assert(sizeof(esr_cg_scalars) == 96, "scalars layout");

int cg_blocks(int64_t n) {
  int64_t g = (n + kCgThreads - 1) / kCgThreads;
  if (g < 1) g = 1;
  if (g > kCgMaxBlocks) g = kCgMaxBlocks;
  return (int)g;
}

// Dot-product accumulator.  double: FMA in FP64.  float: the product's exact
// error (fmaf) and a two-sum keep a (hi, lo) pair, i.e. FP64-class
// accumulation on the FP32 pipes (GB300's FP64 rate is 1/59 of FP32).
template <typename T>
struct DotAcc;
template <>
struct DotAcc<double> {
  double v = 0.0;
  __device__ __forceinline__ void add(double a, double b) { v = fma(a, b, v); }
  __device__ __forceinline__ double value() const { return v; }
};
template <>
struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);
    const float s = hi + p;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (p - bb);
    hi = s;
    lo += err + pe;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// sum_k x[col]*val in slot order; EXACT: separate rounded mul and add.
// Slices up to 8 slots wide take an unrolled path that issues every column
// and value load before the dependent gathers (memory-level parallelism);
// wider slices loop.
template <typename T, bool EXACT>
__device__ __forceinline__ T sell_row(int64_t i, int64_t n, const int64_t *__restrict__ slice_ptr,
                                      const int32_t *__restrict__ col, const T *__restrict__ val,
                                      const T *__restrict__ x) {
  const int64_t s = i >> 5;
  const int lane = (int)(i & 31);
  const int64_t b = __ldg(slice_ptr + s);
  const int w = (int)((__ldg(slice_ptr + s + 1) - b) >> 5);
  const int32_t *cp = col + b + lane;
  const T *vp = val + b + lane;
  T acc = T(0);
  if (w <= 8) {
    int32_t c[8];
    T v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      c[k] = k < w ? __ldg(cp + 32 * k) : -1;
      v[k] = k < w ? __ldg(vp + 32 * k) : T(0);
    }
    T xc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) xc[k] = (c[k] >= 0 && (int64_t)c[k] < n) ? __ldg(x + c[k]) : T(0);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (c[k] >= 0 && (int64_t)c[k] < n) {  // -1 = padding
        if (EXACT) acc = ops<T>::add(acc, ops<T>::mul(xc[k], v[k]));
        else acc = fma(xc[k], v[k], acc);
      }
    }
    return acc;
  }
  for (int k = 0; k < w; ++k) {
    const int32_t c = __ldg(cp + 32 * k);
    if (c >= 0 && (int64_t)c < n) {
      const T vv = __ldg(vp + 32 * k);
      const T xc = __ldg(x + c);
      if (EXACT) acc = ops<T>::add(acc, ops<T>::mul(xc, vv));
      else acc = fma(xc, vv, acc);
    }
  }
  return acc;
}

template <typename T>
__global__ void __launch_bounds__(kCgThreads)
spmv_exact_kernel(int64_t n, const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ col,
                  const T *__restrict__ val, const T *__restrict__ diag, const T *__restrict__ x,
                  T *__restrict__ y) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T off = sell_row<T, true>(i, n, slice_ptr, col, val, x);
    y[i] = ops<T>::add(off, ops<T>::mul(x[i], diag[i]));
  }
}

__device__ __forceinline__ void finish_two(double a, double b, double *pa, double *pb, unsigned int *counter,
                                           double &ta, double &tb, bool &last) {
  __shared__ double s_red[kCgThreads / 32];
  const double ba = esr::block_sum_fixed<kCgThreads>(a, s_red);
  const double bb = esr::block_sum_fixed<kCgThreads>(b, s_red);
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    pa[blockIdx.x] = ba;
    pb[blockIdx.x] = bb;
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  last = s_last;
  if (!last) return;
  __threadfence();
  double va = 0.0, vb = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    va += __ldcg(pa + k);
    vb += __ldcg(pb + k);
  }
  ta = esr::block_sum_fixed<kCgThreads>(va, s_red);
  tb = esr::block_sum_fixed<kCgThreads>(vb, s_red);
}

__device__ __forceinline__ void reset_scalars(esr_cg_scalars &s, double bnorm, double rz, double rr, double rtol,
                                              double atol, int has_atol, int maxiter) {
  s.bnorm = bnorm;
  double tol = rtol * s.bnorm;
  if (has_atol && atol > tol) tol = atol;
  s.tol = tol;
  s.rz = rz;
  s.rz_new = rz;
  s.rz_prev = rz;
  s.pq = 0;
  s.alpha = 0;
  s.beta = 0;
  s.rr = rr;
  s.true_rr = rr;
  s.iters = 0;
  s.done = 0;
  s.maxiter = maxiter;
  s.replacements = 0;
}

// ---- init: r = b - A x, z = M r, p = z, b.b, r.z
template <typename T>
__global__ void __launch_bounds__(kCgThreads)
cg_init_kernel(int64_t n, const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ col,
               const T *__restrict__ val, const T *__restrict__ diag, const T *__restrict__ b,
               const T *__restrict__ x, T *__restrict__ r, T *__restrict__ z, T *__restrict__ p,
               const T *__restrict__ invdiag, double rtol, double atol, int has_atol, int maxiter,
               CgWork *__restrict__ w) {
  DotAcc<T> bb, rz;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T ax = ops<T>::add(sell_row<T, true>(i, n, slice_ptr, col, val, x), ops<T>::mul(x[i], diag[i]));
    const T ri = ops<T>::sub(b[i], ax);
    const T zi = invdiag ? ri * invdiag[i] : ri;
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    bb.add(b[i], b[i]);
    rz.add(ri, zi);
  }
  double tb = 0, trz = 0;
  bool last = false;
  finish_two(bb.value(), rz.value(), w->partial[0], w->partial[1], &w->counter[0], tb, trz, last);
  if (last && threadIdx.x == 0) {
    reset_scalars(w->s, sqrt(tb), trz, 0.0, rtol, atol, has_atol, maxiter);
    w->counter[0] = 0u;
  }
}

// ---- step part 1: q = A p, p.q, alpha
template <typename T>
__global__ void __launch_bounds__(kCgThreads)
cg_spmv_kernel(int64_t n, const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ col,
               const T *__restrict__ val, const T *__restrict__ diag, const T *__restrict__ p,
               T *__restrict__ q, CgWork *__restrict__ w) {
  if (w->s.done) return;
  DotAcc<T> pq;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T pi = p[i];
    const T qi = fma(pi, diag[i], sell_row<T, false>(i, n, slice_ptr, col, val, p));
    q[i] = qi;
    pq.add(pi, qi);
  }
  double tpq = 0, unused = 0;
  bool last = false;
  finish_two(pq.value(), 0.0, w->partial[0], w->partial[2], &w->counter[1], tpq, unused, last);
  if (last && threadIdx.x == 0) {
    w->s.pq = tpq;
    w->s.alpha = w->s.rz / tpq;
    w->counter[1] = 0u;
  }
}

// ---- step part 2 + update: x += a p; r -= a q; z = M r; r.r; r.z; test
template <typename T, typename XT>
__global__ void __launch_bounds__(kCgThreads)
cg_update_kernel(int64_t n, XT *__restrict__ x, T *__restrict__ r, T *__restrict__ z, const T *__restrict__ p,
                 const T *__restrict__ q, const T *__restrict__ invdiag, CgWork *__restrict__ w) {
  if (w->s.done) return;
  const double ad = w->s.alpha;
  const T a = (T)ad;
  DotAcc<T> rr, rz;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] = fma((XT)ad, (XT)p[i], x[i]);
    const T ri = fma(-a, q[i], r[i]);
    r[i] = ri;
    const T zi = invdiag ? ri * invdiag[i] : ri;
    z[i] = zi;
    rr.add(ri, ri);
    rz.add(ri, zi);
  }
  double trr = 0, trz = 0;
  bool last = false;
  finish_two(rr.value(), rz.value(), w->partial[0], w->partial[1], &w->counter[2], trr, trz, last);
  if (last && threadIdx.x == 0) {
    esr_cg_scalars &s = w->s;
    s.iters += 1;
    s.rr = trr;
    s.rz_new = trz;
    s.rz_prev = s.rz;
    const double rnorm = sqrt(trr);
    if (!isnan(rnorm) && rnorm <= s.tol) {
      s.done = 1;
    } else if (s.maxiter >= 0 && s.iters - 1 >= s.maxiter) {
      s.done = 2;
    } else if (!isfinite(rnorm) || !isfinite(trz) || s.rz == 0.0) {
      s.done = 3;
    } else {
      s.beta = trz / s.rz;
      s.rz = trz;
    }
    w->counter[2] = 0u;
  }
}

// ---- update part 2 (native path): p = z + beta p
template <typename T>
__global__ void __launch_bounds__(kCgThreads)
cg_pupdate_kernel(int64_t n, const T *__restrict__ z, T *__restrict__ p, const CgWork *__restrict__ w) {
  if (w->s.done) return;
  const T beta = (T)w->s.beta;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    p[i] = fma(beta, p[i], z[i]);
}

// ---- mixed step part 1: q = A32 p32 on the FP32 pipes (FP32 matrix and an
// FP32 copy of p for the gathers), p.q accumulated in FP64
__global__ void __launch_bounds__(kCgThreads)
cg_spmv_mixed_kernel(int64_t n, const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ col,
                     const float *__restrict__ val32, const float *__restrict__ diag32,
                     const double *__restrict__ p, const float *__restrict__ p32, double *__restrict__ q,
                     CgWork *__restrict__ w) {
  if (w->s.done) return;
  DotAcc<double> pq;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float qf = fmaf(p32[i], diag32[i], sell_row<float, false>(i, n, slice_ptr, col, val32, p32));
    const double qi = (double)qf;
    q[i] = qi;
    pq.add(p[i], qi);
  }
  double tpq = 0, unused = 0;
  bool last = false;
  finish_two(pq.value(), 0.0, w->partial[0], w->partial[2], &w->counter[1], tpq, unused, last);
  if (last && threadIdx.x == 0) {
    w->s.pq = tpq;
    w->s.alpha = w->s.rz / tpq;
    w->counter[1] = 0u;
  }
}

// ---- mixed update part 2: p = z + beta p, and its FP32 gather copy
__global__ void __launch_bounds__(kCgThreads)
cg_pupdate_mixed_kernel(int64_t n, const double *__restrict__ z, double *__restrict__ p, float *__restrict__ p32,
                        const CgWork *__restrict__ w) {
  if (w->s.done) return;
  const double beta = w->s.beta;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double pi = fma(beta, p[i], z[i]);
    p[i] = pi;
    p32[i] = (float)pi;
  }
}

__global__ void cg_to_f32_kernel(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) b[i] = (float)a[i];
}

// ---- mixed: the FP64 true residual b - A64 x replaces the recurrence
// residual (z = M r recomputed, beta rescaled) and decides convergence
__global__ void __launch_bounds__(kCgThreads)
cg_replace_kernel(int64_t n, const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ col,
                  const double *__restrict__ val64, const double *__restrict__ diag64, const double *__restrict__ b,
                  const double *__restrict__ x, double *__restrict__ r, double *__restrict__ z,
                  const double *__restrict__ invdiag, CgWork *__restrict__ w) {
  if (w->s.done > 1) return;  // maxiter / breakdown: leave as is
  DotAcc<double> rr, rz;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double ri = b[i] - fma(x[i], diag64[i], sell_row<double, false>(i, n, slice_ptr, col, val64, x));
    const double zi = invdiag ? ri * invdiag[i] : ri;
    r[i] = ri;
    z[i] = zi;
    rr.add(ri, ri);
    rz.add(ri, zi);
  }
  double trr = 0, trz = 0;
  bool last = false;
  finish_two(rr.value(), rz.value(), w->partial[0], w->partial[1], &w->counter[3], trr, trz, last);
  if (last && threadIdx.x == 0) {
    esr_cg_scalars &s = w->s;
    s.replacements += 1;
    s.rr = trr;
    s.true_rr = trr;
    // rz_prev = r.z before this iteration's update: beta from the true residual
    if (s.rz_prev != 0.0) s.beta = trz / s.rz_prev;
    s.rz = trz;
    const double rnorm = sqrt(trr);
    s.done = (!isnan(rnorm) && rnorm <= s.tol) ? 1 : 0;
    w->counter[3] = 0u;
  }
}

// ---- true residual ||b - A x|| (exact SpMV, FP64 accumulation)
template <typename T>
__global__ void __launch_bounds__(kCgThreads)
true_residual_kernel(int64_t n, const int64_t *__restrict__ slice_ptr, const int32_t *__restrict__ col,
                     const T *__restrict__ val, const T *__restrict__ diag, const T *__restrict__ b,
                     const T *__restrict__ x, T *__restrict__ r, double *__restrict__ out, CgWork *__restrict__ w) {
  DotAcc<T> rr;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T ax = ops<T>::add(sell_row<T, true>(i, n, slice_ptr, col, val, x), ops<T>::mul(x[i], diag[i]));
    const T ri = ops<T>::sub(b[i], ax);
    r[i] = ri;
    rr.add(ri, ri);
  }
  double t = 0, unused = 0;
  bool last = false;
  finish_two(rr.value(), 0.0, w->partial[0], w->partial[2], &w->counter[5], t, unused, last);
  if (last && threadIdx.x == 0) {
    *out = sqrt(t);
    w->counter[5] = 0u;
  }
}

int check_sell(const esr_sell *A) {
  if (!A) return esr::fail(ESR_ERR_ARG, "null matrix");
  if (A->n <= 0) return esr::fail(ESR_ERR_ARG, "matrix has no rows");
  if (A->dtype != ESR_F32 && A->dtype != ESR_F64) return esr::fail(ESR_ERR_UNSUPPORTED, "matrix dtype");
  if (!A->slice_ptr || !A->diag || (A->nslots && (!A->col || !A->val))) return esr::fail(ESR_ERR_ARG, "null matrix array");
  return ESR_OK;
}

int check_pair(const esr_sell *A64, const esr_sell *A32) {
  int st = check_sell(A64);
  if (st) return st;
  if ((st = check_sell(A32))) return st;
  if (A64->dtype != ESR_F64 || A32->dtype != ESR_F32) return esr::fail(ESR_ERR_ARG, "mixed CG needs an FP64 and an FP32 matrix");
  if (A64->n != A32->n || A64->nslots != A32->nslots || A64->slice_ptr != A32->slice_ptr || A64->col != A32->col)
    return esr::fail(ESR_ERR_ARG, "mixed CG: the two matrices must share one SELL layout");
  return ESR_OK;
}

}  // namespace

ESR_DEFINE_STATUS_READER(esr_status_cg)

extern "C" int esr_spmv(const esr_sell *A, const void *x, void *y, void *stream) {
  int st = check_sell(A);
  if (st) return st;
  if (!x || !y) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  const int g = cg_blocks(A->n);
  if (A->dtype == ESR_F64)
    spmv_exact_kernel<double><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const double *)A->val,
                                                       (const double *)A->diag, (const double *)x, (double *)y);
  else
    spmv_exact_kernel<float><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const float *)A->val,
                                                      (const float *)A->diag, (const float *)x, (float *)y);
  ESR_LAUNCH_CHECK("esr_spmv");
  return ESR_OK;
}

extern "C" int64_t esr_cg_workspace_bytes(int64_t n) {
  (void)n;
  return (int64_t)sizeof(CgWork);
}

extern "C" int esr_cg_init(const esr_sell *A, const void *b, void *x, void *r, void *z, void *p,
                           const void *invdiag, double rtol, double atol, int32_t maxiter, void *workspace,
                           void *stream) {
  int st = check_sell(A);
  if (st) return st;
  if (!b || !x || !r || !z || !p || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  CgWork *w = (CgWork *)workspace;
  cudaError_t e = cudaMemsetAsync(w->counter, 0, sizeof(w->counter), s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_cg_init/memset");
  const int g = cg_blocks(A->n);
  const int has_atol = (atol > 0.0) ? 1 : 0;
  if (A->dtype == ESR_F64)
    cg_init_kernel<double><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const double *)A->val,
                                                    (const double *)A->diag, (const double *)b, (const double *)x,
                                                    (double *)r, (double *)z, (double *)p, (const double *)invdiag,
                                                    rtol, atol, has_atol, maxiter, w);
  else
    cg_init_kernel<float><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const float *)A->val,
                                                   (const float *)A->diag, (const float *)b, (const float *)x,
                                                   (float *)r, (float *)z, (float *)p, (const float *)invdiag, rtol,
                                                   atol, has_atol, maxiter, w);
  ESR_LAUNCH_CHECK("esr_cg_init");
  return ESR_OK;
}

extern "C" int esr_cg_iterate(const esr_sell *A, void *x, void *r, void *z, void *p, void *q, const void *invdiag,
                              int32_t k, void *workspace, void *stream) {
  int st = check_sell(A);
  if (st) return st;
  if (!x || !r || !z || !p || !q || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  if (k < 0) return esr::fail(ESR_ERR_ARG, "negative iteration count");
  cudaStream_t s = esr::as_stream(stream);
  CgWork *w = (CgWork *)workspace;
  const int g = cg_blocks(A->n);
  for (int32_t it = 0; it < k; ++it) {
    if (A->dtype == ESR_F64) {
      cg_spmv_kernel<double><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const double *)A->val,
                                                      (const double *)A->diag, (const double *)p, (double *)q, w);
      cg_update_kernel<double, double><<<g, kCgThreads, 0, s>>>(A->n, (double *)x, (double *)r, (double *)z,
                                                                (const double *)p, (const double *)q,
                                                                (const double *)invdiag, w);
      cg_pupdate_kernel<double><<<g, kCgThreads, 0, s>>>(A->n, (const double *)z, (double *)p, w);
    } else {
      cg_spmv_kernel<float><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const float *)A->val,
                                                     (const float *)A->diag, (const float *)p, (float *)q, w);
      cg_update_kernel<float, float><<<g, kCgThreads, 0, s>>>(A->n, (float *)x, (float *)r, (float *)z,
                                                              (const float *)p, (const float *)q,
                                                              (const float *)invdiag, w);
      cg_pupdate_kernel<float><<<g, kCgThreads, 0, s>>>(A->n, (const float *)z, (float *)p, w);
    }
  }
  ESR_LAUNCH_CHECK("esr_cg_iterate");
  return ESR_OK;
}

extern "C" int esr_cg_mixed_init(const esr_sell *A64, const esr_sell *A32, const double *b, double *x, double *r,
                                 double *z, double *p, float *p32, const double *invdiag, double rtol, double atol,
                                 int32_t maxiter, void *workspace, void *stream) {
  int st = check_pair(A64, A32);
  if (st) return st;
  if (!p32) return esr::fail(ESR_ERR_ARG, "null p32");
  if ((st = esr_cg_init(A64, b, x, r, z, p, invdiag, rtol, atol, maxiter, workspace, stream))) return st;
  cg_to_f32_kernel<<<cg_blocks(A64->n), kCgThreads, 0, esr::as_stream(stream)>>>(A64->n, p, p32);
  ESR_LAUNCH_CHECK("esr_cg_mixed_init");
  return ESR_OK;
}

extern "C" int esr_cg_mixed_iterate(const esr_sell *A64, const esr_sell *A32, const double *b, double *x, double *r,
                                    double *z, double *p, float *p32, double *q, const double *invdiag, int32_t k,
                                    void *workspace, void *stream) {
  int st = check_pair(A64, A32);
  if (st) return st;
  if (!b || !x || !r || !z || !p || !p32 || !q || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  if (k < 1) return esr::fail(ESR_ERR_ARG, "mixed CG iterates in chunks >= 1");
  cudaStream_t s = esr::as_stream(stream);
  CgWork *w = (CgWork *)workspace;
  const int g = cg_blocks(A64->n);
  for (int32_t it = 0; it < k; ++it) {
    cg_spmv_mixed_kernel<<<g, kCgThreads, 0, s>>>(A32->n, A32->slice_ptr, A32->col, (const float *)A32->val,
                                                  (const float *)A32->diag, p, p32, q, w);
    cg_update_kernel<double, double><<<g, kCgThreads, 0, s>>>(A64->n, x, r, z, p, q, invdiag, w);
    // the last iteration of the chunk replaces r (and z, beta) by the true
    // residual before the search direction is updated from them
    if (it == k - 1)
      cg_replace_kernel<<<g, kCgThreads, 0, s>>>(A64->n, A64->slice_ptr, A64->col, (const double *)A64->val,
                                                 (const double *)A64->diag, b, x, r, z, invdiag, w);
    cg_pupdate_mixed_kernel<<<g, kCgThreads, 0, s>>>(A64->n, z, p, p32, w);
  }
  ESR_LAUNCH_CHECK("esr_cg_mixed_iterate");
  return ESR_OK;
}

extern "C" int esr_cg_read_scalars(const void *workspace, esr_cg_scalars *out, void *stream) {
  if (!workspace || !out) return esr::fail(ESR_ERR_ARG, "null pointer");
  cudaStream_t s = esr::as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(out, workspace, sizeof(esr_cg_scalars), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_cg_read_scalars");
  return ESR_OK;
}

extern "C" int esr_true_residual(const esr_sell *A, const void *b, const void *x, void *r, double *out_f64,
                                 void *workspace, void *stream) {
  int st = check_sell(A);
  if (st) return st;
  if (!b || !x || !r || !out_f64 || !workspace) return esr::fail(ESR_ERR_ARG, "null pointer");
  cudaStream_t s = esr::as_stream(stream);
  CgWork *w = (CgWork *)workspace;
  const int g = cg_blocks(A->n);
  if (A->dtype == ESR_F64)
    true_residual_kernel<double><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const double *)A->val,
                                                          (const double *)A->diag, (const double *)b,
                                                          (const double *)x, (double *)r, out_f64, w);
  else
    true_residual_kernel<float><<<g, kCgThreads, 0, s>>>(A->n, A->slice_ptr, A->col, (const float *)A->val,
                                                         (const float *)A->diag, (const float *)b, (const float *)x,
                                                         (float *)r, out_f64, w);
  ESR_LAUNCH_CHECK("esr_true_residual");
  return ESR_OK;
}
