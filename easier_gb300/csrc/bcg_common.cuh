// Shared pieces of the batched PCG (bcg.cu) and of the GNN preconditioner
// kernels that run inside it (gnn.cu): workspace layout, arithmetic
// policies, SELL rows, and the per-instance deterministic finish of dot
// products.  Everything lives in an anonymous namespace: each translation
// unit gets its own copy.
#pragma once

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
  int32_t bodies;  // loop bodies run by the one-launch graph
  int32_t pad[61];
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

// alpha and beta of an instance, kept in both forms (set once per
// iteration by the finishing thread; the df64 kernels read the float pair)
__device__ __forceinline__ void split_df(double v, float (&out)[2]) {
  const float hi = __double2float_rn(v);
  out[0] = hi;
  out[1] = __double2float_rn(v - (double)hi);
}
__device__ __forceinline__ void set_alpha(esr_bcg_inst &s, double a) {
  s.alpha = a;
  split_df(a, s.alpha_df);
}
__device__ __forceinline__ void set_beta(esr_bcg_inst &s, double b) {
  s.beta = b;
  split_df(b, s.beta_df);
}

// Block sum of a per-thread dot accumulator (identical result in every
// thread, fixed order).  FP64: shuffles of doubles.  df64: the (hi, lo)
// pairs are added with the double-float add on the FP32 pipes and only the
// block total is widened to double, so the df64 kernels issue no FP64
// arithmetic per chunk.
template <int THREADS>
__device__ __forceinline__ double bsum(const DotAccD &a) {
  __shared__ double s_red[THREADS / 32];
  return esr::block_sum_fixed<THREADS>(a.v, s_red);
}

__device__ __forceinline__ df64::df warp_sum_df(df64::df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const df64::df w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
    v = df64::add(v, w);
  }
  return v;
}

template <int THREADS>
__device__ __forceinline__ double bsum(const DotAccDF &a) {
  __shared__ float2 s_red[THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  df64::df v = df64::quick_two_sum(a.hi, a.lo);
  v = warp_sum_df(v);
  if (lane == 0) s_red[warp] = make_float2(v.hi, v.lo);
  __syncthreads();
  if (warp == 0) {
    const float2 t = lane < THREADS / 32 ? s_red[lane] : make_float2(0.f, 0.f);
    v = warp_sum_df(df64::df{t.x, t.y});
    if (lane == 0) s_red[0] = make_float2(v.hi, v.lo);
  }
  __syncthreads();
  const float2 t = s_red[0];
  __syncthreads();
  return (double)t.x + (double)t.y;
}

struct PolF64 {
  using V = double;
  using Acc = DotAccD;
  // FP64 iterations are bound by the FP64 pipe: the direction sweep of the
  // double-float policy (q = A z + beta q, one more FMA a row) costs more
  // than the separate p-update sweep it saves
  static constexpr bool kFusedDirection = false;
  static __device__ __forceinline__ V alpha(const esr_bcg_inst &s) { return s.alpha; }
  static __device__ __forceinline__ V beta(const esr_bcg_inst &s) { return s.beta; }
  static __device__ __forceinline__ V neg(V a) { return -a; }
  static __device__ __forceinline__ V fma(V a, V b, V c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
  static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
  static __device__ __forceinline__ V of(double d) { return d; }
  static __device__ __forceinline__ V zero() { return 0.0; }
  static __device__ __forceinline__ double dbl(V a) { return a; }
  static __device__ __forceinline__ float flt(V a) { return (float)a; }
  static __device__ __forceinline__ V off(float f) { return (double)f; }
};

struct PolDF {
  using V = df64::df;
  using Acc = DotAccDF;
  static constexpr bool kFusedDirection = true;
  static __device__ __forceinline__ V alpha(const esr_bcg_inst &s) { return V{s.alpha_df[0], s.alpha_df[1]}; }
  static __device__ __forceinline__ V beta(const esr_bcg_inst &s) { return V{s.beta_df[0], s.beta_df[1]}; }
  static __device__ __forceinline__ V neg(V a) { return df64::neg(a); }
  static __device__ __forceinline__ V fma(V a, V b, V c) { return df64::fma(a, b, c); }
  static __device__ __forceinline__ V mul(V a, V b) { return df64::mul(a, b); }
  static __device__ __forceinline__ V sub(V a, V b) { return df64::add(a, df64::neg(b)); }
  static __device__ __forceinline__ V of(double d) { return df64::from_double(d); }
  static __device__ __forceinline__ V zero() { return V{0.f, 0.f}; }
  static __device__ __forceinline__ double dbl(V a) { return df64::to_double(a); }
  static __device__ __forceinline__ float flt(V a) { return __fadd_rn(a.hi, a.lo); }
  static __device__ __forceinline__ V off(float f) { return V{f, 0.f}; }
};

// sum over the row's SELL slots of val * x(col), in slot order; `x` maps a
// column to its value (a vector load, or a value formed from several)
// (WIDE: rows of <= 8 slots issue all their loads at once; otherwise, or for
// a costly x, one slot after the other)
template <class P, bool WIDE = true, class X>
__device__ __forceinline__ typename P::V bsell_row_of(int64_t i, int64_t n, const int64_t *__restrict__ slice_ptr,
                                                      const int32_t *__restrict__ col,
                                                      const typename P::V *__restrict__ val, const X &x) {
  using V = typename P::V;
  const int64_t s = i >> 5;
  const int lane = (int)(i & 31);
  const int64_t b = __ldg(slice_ptr + s);
  const int w = (int)((__ldg(slice_ptr + s + 1) - b) >> 5);
  const int32_t *cp = col + b + lane;
  const V *vp = val + b + lane;
  V acc = P::zero();
  if (WIDE && w <= 8) {
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
        xc[k] = x(c[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (c[k] >= 0) acc = P::fma(v[k], xc[k], acc);
    return acc;
  }
  for (int k = 0; k < w; ++k) {
    const int32_t c = __ldg(cp + 32 * k);
    if (c >= 0 && (int64_t)c < n) acc = P::fma(vp[32 * k], x(c), acc);
  }
  return acc;
}

template <class P>
__device__ __forceinline__ typename P::V bsell_row(int64_t i, int64_t n, const int64_t *__restrict__ slice_ptr,
                                                   const int32_t *__restrict__ col,
                                                   const typename P::V *__restrict__ val,
                                                   const typename P::V *__restrict__ x) {
  return bsell_row_of<P>(i, n, slice_ptr, col, val, [x](int64_t j) { return x[j]; });
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
// `bs` are the block's sums (bsum above, the same in every thread).
template <int K, int THREADS = kBThreads>
__device__ __forceinline__ bool inst_finish(const double (&bs)[K], int slot, int p0, int p1, int expected,
                                            int nblocks, double *partial, unsigned int *counter, double (&tot)[K]) {
  __shared__ double s_red[THREADS / 32];
  __shared__ bool s_last;
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
    for (int q = p0 + threadIdx.x; q < p1; q += THREADS) acc += __ldcg(partial + k * (int64_t)nblocks + q);
    tot[k] = esr::block_sum_fixed<THREADS>(acc, s_red);
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
  const int32_t *inst_rows;  // GNN only: rows before padding
  int32_t use_gnn;
  int32_t stall_window;
  int32_t poly;  // polynomial-Jacobi: z, r.z and beta come from bcg_poly_kernel
};

inline BArgs bargs(const esr_batch *B) {
  BArgs a{B->n,         B->nblocks,     B->ninst,       B->nchunks,     B->slice_ptr, B->col,
          B->block_inst, B->inst_block0, B->chunk_tile0, B->chunk_inst, B->inst_chunk0,
          nullptr,      0,              0,              B->poly_degree > 0 ? 1 : 0};
  if (B->gnn) {
    a.inst_rows = B->gnn->inst_rows;
    a.use_gnn = 1;
    a.stall_window = B->gnn->stall_window;
  }
  return a;
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
template <int K, int THREADS = kBThreads>
__device__ __forceinline__ bool chunk_finish(const BArgs &a, int chunk, int inst, const double (&v)[K],
                                             BcgLayout L, double (&tot)[K]) {
  const int c0 = a.inst_chunk0[inst], c1 = a.inst_chunk0[inst + 1];
  return inst_finish<K, THREADS>(v, chunk, c0, c1, c1 - c0, a.nblocks, L.partial, L.counter + inst, tot);
}

// Flexible-CG (GNN preconditioner) modes of an instance
constexpr int kModeJacobi = 0;
constexpr int kModeGnn = 1;


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
  if (B->gnn) {
    const esr_gnn *G = B->gnn;
    if (!B->invdiag) return esr::fail(ESR_ERR_ARG, "the GNN preconditioner needs invdiag");
    if (!G->node_lk || !G->edge_feat || !G->inst_rows || !G->h0 || !G->h1 || !G->enc_w || !G->enc_b ||
        !G->layer_w || !G->layer_b || !G->dec_w)
      return esr::fail(ESR_ERR_ARG, "null GNN array");
    if (G->grid <= 0 || G->stall_window <= 0) return esr::fail(ESR_ERR_ARG, "bad GNN grid or stall window");
  }
  if (B->poly_degree != 0) {
    if (B->poly_degree < 2 || B->poly_degree > 16) return esr::fail(ESR_ERR_ARG, "poly_degree must be 0 or in [2, 16]");
    if (B->gnn) return esr::fail(ESR_ERR_ARG, "the polynomial and GNN preconditioners exclude each other");
    if (!B->invdiag || !B->poly_tmp) return esr::fail(ESR_ERR_ARG, "the polynomial preconditioner needs invdiag and poly_tmp");
  }
  return ESR_OK;
}


}  // namespace

namespace esr {
// GNN preconditioner layers of one flexible-CG iteration (gnn.cu): z = M(r)
// for the running GNN-mode instances, then z.r and z.q and the direction
// coefficient beta per instance.
int gnn_layers(const esr_batch *B, const void *r, const void *q, void *z, void *workspace, cudaStream_t s);
}  // namespace esr
