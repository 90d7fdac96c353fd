// Batched preconditioned CG: many independent Linsys instances packed as
// one block-diagonal SELL-32 system, iterated in lockstep with per-instance
// scalars and per-instance stopping.  A single system is a batch of one.
//
// Iteration per instance (easier/numeric/solver/cg.py:68-95, Jacobi M):
//   q = A p; alpha = r.z / p.q; x += alpha p; r -= alpha q; z = M r;
//   stop when ||r|| <= tol; beta = r.z_new / r.z; p = z + beta p
//
// Work decomposition.  Every instance is padded to whole 256-row tiles
// (identity rows), so no tile spans two instances.  Consecutive tiles of an
// instance form chunks of up to `tiles_per_chunk` tiles: the unit of work
// of one CTA iteration in the three per-iteration kernels, which are
// persistent (a fixed grid loops over the chunk list).  A one-CTA compaction
// kernel at the start of every esr_bcg_iterate call lists the chunks of the
// instances still running, so finished instances cost nothing afterwards.
// Each dot product is finished per instance by the instance's last chunk to
// arrive (atomic ticket), which adds the instance's chunk partials in chunk
// order: deterministic, no floating-point atomics, no CTA ever waits for
// another.
//
// Arithmetic policies:
//   PolF64  FP64 vectors and matrix (the reference's precision);
//   PolDF   double-float (df64.cuh): the same algorithm on FP32 pairs, ~48
//           significand bits on the FP32 pipes (GB300's FP64 rate is 1/59 of
//           its FP32 rate, and the FP64 CG saturates the FP64 pipe before
//           HBM).
// Convergence is re-checked on the FP64 true residual b - A x computed from
// an FP64 copy of the matrix (esr_bcg_verify).  An instance whose true
// residual misses the tolerance continues from it: r = b - A x replaces the
// recurrence residual and p keeps its direction (a residual replacement,
// not a restart).
#include <cmath>
#include <cstdint>

#include "df64.cuh"
#include "esr_internal.h"
#include "reduce_util.cuh"

namespace {

constexpr int kBThreads = 256;  // rows per tile: one row per thread per tile
constexpr int kBSums = 3;       // partial arrays

struct BcgHead {
  int32_t active;  // instances with done == 0
  int32_t acount;  // entries of the active chunk list
  int32_t pad[62];
};

struct BcgLayout {
  BcgHead *head;
  esr_bcg_inst *inst;
  unsigned int *counter;  // [ninst] arrival tickets
  int32_t *alist;         // [nchunks] active chunk list
  double *partial;        // [kBSums][nblocks] (chunk or tile partials)
};

inline int64_t round256(int64_t v) { return (v + 255) / 256 * 256; }

BcgLayout layout_of(void *ws, int32_t ninst, int32_t nchunks) {
  char *p = (char *)ws;
  BcgLayout L;
  L.head = (BcgHead *)p;
  p += round256(sizeof(BcgHead));
  L.inst = (esr_bcg_inst *)p;
  p += round256(ninst * (int64_t)sizeof(esr_bcg_inst));
  L.counter = (unsigned int *)p;
  p += round256(ninst * (int64_t)sizeof(unsigned int));
  L.alist = (int32_t *)p;
  p += round256(nchunks * (int64_t)sizeof(int32_t));
  L.partial = (double *)p;
  return L;
}

int64_t workspace_bytes(int32_t ninst, int32_t nblocks, int32_t nchunks) {
  return round256(sizeof(BcgHead)) + round256(ninst * (int64_t)sizeof(esr_bcg_inst)) +
         round256(ninst * (int64_t)sizeof(unsigned int)) + round256(nchunks * (int64_t)sizeof(int32_t)) +
         kBSums * (int64_t)nblocks * (int64_t)sizeof(double);
}

// ---- arithmetic policies
struct DotAccD {
  double v = 0.0;
  __device__ __forceinline__ void add(double a, double b) { v = fma(a, b, v); }
  __device__ __forceinline__ double value() const { return v; }
};

struct DotAccDF {  // hi*hi products exactly (two-prod + two-sum), cross terms in lo
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(df64::df a, df64::df b) {
    const df64::df p = df64::two_prod(a.hi, b.hi);
    const df64::df s = df64::two_sum(hi, p.hi);
    hi = s.hi;
    lo = __fadd_rn(lo, __fadd_rn(s.lo, __fadd_rn(p.lo, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi)))));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

struct PolF64 {
  using V = double;
  using Acc = DotAccD;
  static __device__ __forceinline__ V fma(V a, V b, V c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
  static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
  static __device__ __forceinline__ V of(double d) { return d; }
  static __device__ __forceinline__ V zero() { return 0.0; }
  static __device__ __forceinline__ double dbl(V a) { return a; }
};

struct PolDF {
  using V = df64::df;
  using Acc = DotAccDF;
  static __device__ __forceinline__ V fma(V a, V b, V c) { return df64::fma(a, b, c); }
  static __device__ __forceinline__ V mul(V a, V b) { return df64::mul(a, b); }
  static __device__ __forceinline__ V sub(V a, V b) { return df64::add(a, df64::neg(b)); }
  static __device__ __forceinline__ V of(double d) { return df64::from_double(d); }
  static __device__ __forceinline__ V zero() { return V{0.f, 0.f}; }
  static __device__ __forceinline__ double dbl(V a) { return df64::to_double(a); }
};

// sum over the row's SELL slots of val * x, in slot order
template <class P>
__device__ __forceinline__ typename P::V bsell_row(int64_t i, int64_t n, const int64_t *__restrict__ slice_ptr,
                                                   const int32_t *__restrict__ col,
                                                   const typename P::V *__restrict__ val,
                                                   const typename P::V *__restrict__ x) {
  using V = typename P::V;
  const int64_t s = i >> 5;
  const int lane = (int)(i & 31);
  const int64_t b = __ldg(slice_ptr + s);
  const int w = (int)((__ldg(slice_ptr + s + 1) - b) >> 5);
  const int32_t *cp = col + b + lane;
  const V *vp = val + b + lane;
  V acc = P::zero();
  if (w <= 8) {
    int32_t c[8];
    V v[8], xc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      c[k] = k < w ? __ldg(cp + 32 * k) : -1;
      if ((int64_t)c[k] >= n) c[k] = -1;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (c[k] >= 0) {
        v[k] = vp[32 * k];
        xc[k] = x[c[k]];
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (c[k] >= 0) acc = P::fma(v[k], xc[k], acc);
    return acc;
  }
  for (int k = 0; k < w; ++k) {
    const int32_t c = __ldg(cp + 32 * k);
    if (c >= 0 && (int64_t)c < n) acc = P::fma(vp[32 * k], x[c], acc);
  }
  return acc;
}

// FP64 row of the true residual
__device__ __forceinline__ double bsell_row64(int64_t i, int64_t n, const int64_t *__restrict__ slice_ptr,
                                              const int32_t *__restrict__ col, const double *__restrict__ val,
                                              const double *__restrict__ x) {
  const int64_t s = i >> 5;
  const int lane = (int)(i & 31);
  const int64_t b = __ldg(slice_ptr + s);
  const int w = (int)((__ldg(slice_ptr + s + 1) - b) >> 5);
  double acc = 0.0;
  for (int k = 0; k < w; ++k) {
    const int64_t e = b + 32 * k + lane;
    const int32_t c = __ldg(col + e);
    if (c >= 0 && (int64_t)c < n) acc = fma(__ldg(val + e), __ldg(x + c), acc);
  }
  return acc;
}

// Per-instance finish of K sums.  The calling CTA publishes its K block
// sums at partial[k][slot] and takes an arrival ticket on the instance's
// counter; the CTA holding the last of `expected` tickets (returns true in
// all its threads) adds partial[k][p0..p1) in order into tot and resets the
// counter.  Never waits on another CTA.
template <int K>
__device__ __forceinline__ bool inst_finish(const double (&v)[K], int slot, int p0, int p1, int expected,
                                            int nblocks, double *partial, unsigned int *counter, double (&tot)[K]) {
  __shared__ double s_red[kBThreads / 32];
  __shared__ bool s_last;
  double bs[K];
#pragma unroll
  for (int k = 0; k < K; ++k) bs[k] = esr::block_sum_fixed<kBThreads>(v[k], s_red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) partial[k * (int64_t)nblocks + slot] = bs[k];
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    s_last = (t == (unsigned int)(expected - 1));
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double acc = 0.0;
    for (int q = p0 + threadIdx.x; q < p1; q += kBThreads) acc += __ldcg(partial + k * (int64_t)nblocks + q);
    tot[k] = esr::block_sum_fixed<kBThreads>(acc, s_red);
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

struct BArgs {
  int64_t n;
  int32_t nblocks;
  int32_t ninst;
  int32_t nchunks;
  const int64_t *slice_ptr;
  const int32_t *col;
  const int32_t *block_inst;
  const int32_t *inst_block0;
  const int32_t *chunk_tile0;
  const int32_t *chunk_inst;
  const int32_t *inst_chunk0;
};

inline BArgs bargs(const esr_batch *B) {
  return BArgs{B->n,         B->nblocks,     B->ninst,       B->nchunks,     B->slice_ptr, B->col,
               B->block_inst, B->inst_block0, B->chunk_tile0, B->chunk_inst, B->inst_chunk0};
}

__device__ __forceinline__ void retire(BcgLayout L) { atomicSub(&L.head->active, 1); }

// tile-grid finish (init / verify kernels: one CTA per tile)
template <int K>
__device__ __forceinline__ bool tile_finish(const BArgs &a, int inst, const double (&v)[K], BcgLayout L,
                                            double (&tot)[K]) {
  const int b0 = a.inst_block0[inst], b1 = a.inst_block0[inst + 1];
  return inst_finish<K>(v, blockIdx.x, b0, b1, b1 - b0, a.nblocks, L.partial, L.counter + inst, tot);
}

// chunk finish (persistent kernels)
template <int K>
__device__ __forceinline__ bool chunk_finish(const BArgs &a, int chunk, int inst, const double (&v)[K],
                                             BcgLayout L, double (&tot)[K]) {
  const int c0 = a.inst_chunk0[inst], c1 = a.inst_chunk0[inst + 1];
  return inst_finish<K>(v, chunk, c0, c1, c1 - c0, a.nblocks, L.partial, L.counter + inst, tot);
}

// ---- compaction: list the chunks of running instances (one CTA)
__global__ void __launch_bounds__(1024) bcg_compact_kernel(BArgs a, BcgLayout L) {
  __shared__ int32_t s_scan[1024];
  __shared__ int32_t s_base;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (int i0 = 0; i0 < a.ninst; i0 += 1024) {
    const int i = i0 + threadIdx.x;
    int cnt = 0;
    if (i < a.ninst && L.inst[i].done == 0) cnt = a.inst_chunk0[i + 1] - a.inst_chunk0[i];
    s_scan[threadIdx.x] = cnt;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
      const int t = threadIdx.x >= off ? s_scan[threadIdx.x - off] : 0;
      __syncthreads();
      s_scan[threadIdx.x] += t;
      __syncthreads();
    }
    const int pos = s_base + s_scan[threadIdx.x] - cnt;
    const int c0 = cnt ? a.inst_chunk0[i] : 0;
    for (int j = 0; j < cnt; ++j) L.alist[pos + j] = c0 + j;
    __syncthreads();
    if (threadIdx.x == 1023) s_base += s_scan[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) L.head->acount = s_base;
}

// ---- init: r = b - A x; z = M r; p = z; ||b|| (FP64 b); r.z; r.r
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_init_kernel(BArgs a, const typename P::V *__restrict__ val, const typename P::V *__restrict__ diag,
                const typename P::V *__restrict__ invdiag, const double *__restrict__ b64,
                const typename P::V *__restrict__ b, const typename P::V *__restrict__ x, typename P::V *__restrict__ r,
                typename P::V *__restrict__ z, typename P::V *__restrict__ p, double rtol, double atol, int has_atol,
                int maxiter, BcgLayout L) {
  using V = typename P::V;
  const int inst = a.block_inst[blockIdx.x];
  const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
  typename P::Acc rz, rr;
  double bb = 0.0;
  if (i < a.n) {
    const V ax = P::fma(diag[i], x[i], bsell_row<P>(i, a.n, a.slice_ptr, a.col, val, x));
    const V ri = P::sub(b[i], ax);
    const V zi = invdiag ? P::mul(ri, invdiag[i]) : ri;
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    bb = b64[i] * b64[i];
    rz.add(ri, zi);
    rr.add(ri, ri);
  }
  const double v[3] = {bb, rz.value(), rr.value()};
  double tot[3];
  if (tile_finish<3>(a, inst, v, L, tot) && threadIdx.x == 0) {
    esr_bcg_inst &s = L.inst[inst];
    s.bnorm = sqrt(tot[0]);
    double tol = rtol * s.bnorm;
    if (has_atol && atol > tol) tol = atol;
    s.tol = tol;
    s.rz = tot[1];
    s.rr = tot[2];
    s.pq = s.alpha = s.beta = 0.0;
    s.true_rr = -1.0;
    s.iters = 0;
    s.verified = 0;
    s.restarts = 0;
    s.maxiter = maxiter;
    s.done = 0;  // the reference always takes a first step (cg.py:143-153)
    atomicAdd(&L.head->active, 1);
  }
}

// ---- step part 1: q = A p; p.q; alpha
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_spmv_kernel(BArgs a, const typename P::V *__restrict__ val, const typename P::V *__restrict__ diag,
                const typename P::V *__restrict__ p, typename P::V *__restrict__ q, BcgLayout L) {
  using V = typename P::V;
  const int count = L.head->acount;
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = L.alist[w];
    const int inst = a.chunk_inst[c];
    if (L.inst[inst].done) continue;
    typename P::Acc pq;
    const int t1 = a.chunk_tile0[c + 1];
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      const V pi = p[i];
      const V qi = P::fma(diag[i], pi, bsell_row<P>(i, a.n, a.slice_ptr, a.col, val, p));
      q[i] = qi;
      pq.add(pi, qi);
    }
    const double v[1] = {pq.value()};
    double tot[1];
    if (chunk_finish<1>(a, c, inst, v, L, tot) && threadIdx.x == 0) {
      esr_bcg_inst &s = L.inst[inst];
      s.pq = tot[0];
      if (!(tot[0] != 0.0) || !isfinite(tot[0])) {
        s.done = 3;  // breakdown
        retire(L);
      } else {
        s.alpha = s.rz / tot[0];
      }
    }
  }
}

// ---- step part 2 + update: x += a p; r -= a q; z = M r; r.r; r.z; test
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_update_kernel(BArgs a, const typename P::V *__restrict__ invdiag, typename P::V *__restrict__ x,
                  typename P::V *__restrict__ r, typename P::V *__restrict__ z, const typename P::V *__restrict__ p,
                  const typename P::V *__restrict__ q, BcgLayout L) {
  using V = typename P::V;
  const int count = L.head->acount;
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = L.alist[w];
    const int inst = a.chunk_inst[c];
    if (L.inst[inst].done) continue;
    const double ad = L.inst[inst].alpha;
    const V av = P::of(ad), nav = P::of(-ad);
    typename P::Acc rr, rz;
    const int t1 = a.chunk_tile0[c + 1];
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      x[i] = P::fma(av, p[i], x[i]);
      const V ri = P::fma(nav, q[i], r[i]);
      r[i] = ri;
      const V zi = invdiag ? P::mul(ri, invdiag[i]) : ri;
      z[i] = zi;
      rr.add(ri, ri);
      rz.add(ri, zi);
    }
    const double v[2] = {rr.value(), rz.value()};
    double tot[2];
    if (chunk_finish<2>(a, c, inst, v, L, tot) && threadIdx.x == 0) {
      esr_bcg_inst &s = L.inst[inst];
      s.iters += 1;
      s.rr = tot[0];
      const double rnorm = sqrt(tot[0]);
      if (!isnan(rnorm) && rnorm <= s.tol) {
        s.done = 1;
        retire(L);
      } else if (s.maxiter >= 0 && s.iters - 1 >= s.maxiter) {
        s.done = 2;
        retire(L);
      } else if (!isfinite(rnorm) || !isfinite(tot[1]) || s.rz == 0.0) {
        s.done = 3;
        retire(L);
      } else {
        s.beta = tot[1] / s.rz;
        s.rz = tot[1];
      }
    }
  }
}

// ---- update part 2: p = z + beta p
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_pupdate_kernel(BArgs a, const typename P::V *__restrict__ z, typename P::V *__restrict__ p, BcgLayout L) {
  using V = typename P::V;
  const int count = L.head->acount;
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = L.alist[w];
    const int inst = a.chunk_inst[c];
    if (L.inst[inst].done) continue;
    const V beta = P::of(L.inst[inst].beta);
    const int t1 = a.chunk_tile0[c + 1];
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      p[i] = P::fma(beta, p[i], z[i]);
    }
  }
}

// ---- verification, pass 1: x64 = x for the instances to verify (its own
// launch: the residual of a row reads x64 of other CTAs' rows)
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_export_kernel(BArgs a, const typename P::V *__restrict__ x, double *__restrict__ x64, BcgLayout L) {
  const int inst = a.block_inst[blockIdx.x];
  const esr_bcg_inst &st = L.inst[inst];
  if (st.done != 1 || st.verified) return;
  const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
  if (i < a.n) x64[i] = P::dbl(x[i]);
}

// ---- pass 2: r64 = b64 - A64 x64; true ||r|| per instance
__global__ void __launch_bounds__(kBThreads)
bcg_residual_kernel(BArgs a, const double *__restrict__ val64, const double *__restrict__ diag64,
                    const double *__restrict__ b64, const double *__restrict__ x64, double *__restrict__ r64,
                    BcgLayout L) {
  const int inst = a.block_inst[blockIdx.x];
  esr_bcg_inst &st = L.inst[inst];
  if (st.done != 1 || st.verified) return;
  const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
  double rr = 0.0;
  if (i < a.n) {
    const double ri = b64[i] - fma(diag64[i], x64[i], bsell_row64(i, a.n, a.slice_ptr, a.col, val64, x64));
    r64[i] = ri;
    rr = ri * ri;
  }
  const double v[1] = {rr};
  double tot[1];
  if (tile_finish<1>(a, inst, v, L, tot) && threadIdx.x == 0) {
    st.true_rr = tot[0];
    const double rn = sqrt(tot[0]);
    st.verified = (!isnan(rn) && rn <= st.tol) ? 1 : -1;
  }
}

// ---- pass 3, instances whose true residual missed: residual replacement
// r = r64, z = M r, beta = r.z / r.z_old, p = z + beta p; running again
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_replace_kernel(BArgs a, const typename P::V *__restrict__ invdiag, const double *__restrict__ r64,
                   typename P::V *__restrict__ r, typename P::V *__restrict__ z, BcgLayout L) {
  using V = typename P::V;
  const int inst = a.block_inst[blockIdx.x];
  esr_bcg_inst &st = L.inst[inst];
  if (st.verified != -1) return;
  const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
  typename P::Acc rz;
  if (i < a.n) {
    const V ri = P::of(r64[i]);
    const V zi = invdiag ? P::mul(ri, invdiag[i]) : ri;
    r[i] = ri;
    z[i] = zi;
    rz.add(ri, zi);
  }
  const double v[1] = {rz.value()};
  double tot[1];
  if (tile_finish<1>(a, inst, v, L, tot) && threadIdx.x == 0) {
    st.beta = (st.rz != 0.0) ? tot[0] / st.rz : 0.0;
    st.rz = tot[0];
    st.rr = st.true_rr;
    st.verified = -2;  // p update pending
  }
}

template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_replace_p_kernel(BArgs a, const typename P::V *__restrict__ z, typename P::V *__restrict__ p, BcgLayout L) {
  const int inst = a.block_inst[blockIdx.x];
  esr_bcg_inst &st = L.inst[inst];
  if (st.verified != -2) return;
  const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
  if (i < a.n) p[i] = P::fma(P::of(st.beta), p[i], z[i]);
  // the instance's tiles all pass the test above before any of them
  // re-arms it: the ticket counter orders them
  const double v[1] = {0.0};
  double tot[1];
  if (tile_finish<1>(a, inst, v, L, tot) && threadIdx.x == 0) {
    st.verified = 0;
    st.restarts += 1;
    st.done = 0;
    atomicAdd(&L.head->active, 1);
  }
}

int check_batch(const esr_batch *B) {
  if (!B) return esr::fail(ESR_ERR_ARG, "null batch");
  if (B->n <= 0 || B->ninst <= 0 || B->nblocks <= 0 || B->nchunks <= 0) return esr::fail(ESR_ERR_ARG, "empty batch");
  if (B->rows_per_block != kBThreads) return esr::fail(ESR_ERR_ARG, "rows_per_block must be 256");
  if (B->n != (int64_t)B->nblocks * kBThreads) return esr::fail(ESR_ERR_ARG, "n must be nblocks * 256");
  if (B->nchunks > B->nblocks || B->nchunks < B->ninst) return esr::fail(ESR_ERR_ARG, "bad chunk count");
  if (B->grid <= 0) return esr::fail(ESR_ERR_ARG, "grid must be positive");
  if (!B->slice_ptr || !B->col || !B->val || !B->diag || !B->val64 || !B->diag64 || !B->block_inst ||
      !B->inst_block0 || !B->chunk_tile0 || !B->chunk_inst || !B->inst_chunk0)
    return esr::fail(ESR_ERR_ARG, "null batch array");
  return ESR_OK;
}

template <class P>
int run_init(const esr_batch *B, const double *b64, const void *b, void *x, void *r, void *z, void *p, double rtol,
             double atol, int32_t maxiter, void *ws, cudaStream_t s) {
  using V = typename P::V;
  BcgLayout L = layout_of(ws, B->ninst, B->nchunks);
  cudaError_t e = cudaMemsetAsync(ws, 0, workspace_bytes(B->ninst, B->nblocks, B->nchunks), s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_init/memset");
  bcg_init_kernel<P><<<B->nblocks, kBThreads, 0, s>>>(bargs(B), (const V *)B->val, (const V *)B->diag,
                                                      (const V *)B->invdiag, b64, (const V *)b, (const V *)x,
                                                      (V *)r, (V *)z, (V *)p, rtol, atol, atol > 0.0 ? 1 : 0,
                                                      maxiter, L);
  ESR_LAUNCH_CHECK("esr_bcg_init");
  return ESR_OK;
}

template <class P>
int run_iterate(const esr_batch *B, void *x, void *r, void *z, void *p, void *q, int32_t k, void *ws,
                cudaStream_t s) {
  using V = typename P::V;
  BcgLayout L = layout_of(ws, B->ninst, B->nchunks);
  const BArgs a = bargs(B);
  bcg_compact_kernel<<<1, 1024, 0, s>>>(a, L);
  for (int32_t it = 0; it < k; ++it) {
    bcg_spmv_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->val, (const V *)B->diag, (const V *)p,
                                                     (V *)q, L);
    bcg_update_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->invdiag, (V *)x, (V *)r, (V *)z,
                                                       (const V *)p, (const V *)q, L);
    bcg_pupdate_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)z, (V *)p, L);
  }
  ESR_LAUNCH_CHECK("esr_bcg_iterate");
  return ESR_OK;
}

template <class P>
int run_verify(const esr_batch *B, const double *b64, void *x, double *x64, double *r64, void *r, void *z, void *p,
               void *ws, cudaStream_t s) {
  using V = typename P::V;
  BcgLayout L = layout_of(ws, B->ninst, B->nchunks);
  const BArgs a = bargs(B);
  bcg_export_kernel<P><<<B->nblocks, kBThreads, 0, s>>>(a, (const V *)x, x64, L);
  bcg_residual_kernel<<<B->nblocks, kBThreads, 0, s>>>(a, B->val64, B->diag64, b64, x64, r64, L);
  bcg_replace_kernel<P><<<B->nblocks, kBThreads, 0, s>>>(a, (const V *)B->invdiag, r64, (V *)r, (V *)z, L);
  bcg_replace_p_kernel<P><<<B->nblocks, kBThreads, 0, s>>>(a, (const V *)z, (V *)p, L);
  ESR_LAUNCH_CHECK("esr_bcg_verify");
  return ESR_OK;
}

}  // namespace

extern "C" int64_t esr_bcg_workspace_bytes(int32_t ninst, int32_t nblocks, int32_t nchunks) {
  if (ninst <= 0 || nblocks <= 0 || nchunks <= 0) return -1;
  return workspace_bytes(ninst, nblocks, nchunks);
}

extern "C" int esr_bcg_init(const esr_batch *B, const double *b64, const void *b, void *x, void *r, void *z, void *p,
                            double rtol, double atol, int32_t maxiter, void *workspace, void *stream) {
  int st = check_batch(B);
  if (st) return st;
  if (!b64 || !b || !x || !r || !z || !p || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  return B->df64 ? run_init<PolDF>(B, b64, b, x, r, z, p, rtol, atol, maxiter, workspace, s)
                 : run_init<PolF64>(B, b64, b, x, r, z, p, rtol, atol, maxiter, workspace, s);
}

extern "C" int esr_bcg_iterate(const esr_batch *B, void *x, void *r, void *z, void *p, void *q, int32_t k,
                               void *workspace, void *stream) {
  int st = check_batch(B);
  if (st) return st;
  if (!x || !r || !z || !p || !q || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  if (k < 0) return esr::fail(ESR_ERR_ARG, "negative iteration count");
  cudaStream_t s = esr::as_stream(stream);
  return B->df64 ? run_iterate<PolDF>(B, x, r, z, p, q, k, workspace, s)
                 : run_iterate<PolF64>(B, x, r, z, p, q, k, workspace, s);
}

extern "C" int esr_bcg_verify(const esr_batch *B, const double *b64, void *x, double *x64, double *r64, void *r,
                              void *z, void *p, void *workspace, void *stream) {
  int st = check_batch(B);
  if (st) return st;
  if (!b64 || !x || !x64 || !r64 || !r || !z || !p || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  return B->df64 ? run_verify<PolDF>(B, b64, x, x64, r64, r, z, p, workspace, s)
                 : run_verify<PolF64>(B, b64, x, x64, r64, r, z, p, workspace, s);
}

extern "C" int esr_bcg_status(const void *workspace, int32_t ninst, int32_t nchunks, int32_t *active,
                              esr_bcg_inst *inst_out, void *stream) {
  if (!workspace || ninst <= 0 || nchunks <= 0 || !active) return esr::fail(ESR_ERR_ARG, "bad status query");
  cudaStream_t s = esr::as_stream(stream);
  BcgLayout L = layout_of(const_cast<void *>(workspace), ninst, nchunks);
  cudaError_t e = cudaMemcpyAsync(active, &L.head->active, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && inst_out)
    e = cudaMemcpyAsync(inst_out, L.inst, ninst * sizeof(esr_bcg_inst), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_status");
  return ESR_OK;
}
