// Batched preconditioned CG: many independent Linsys instances packed as
// one block-diagonal SELL-32 system, iterated in lockstep with per-instance
// scalars and per-instance stopping.  A single system is a batch of one.
//
// Iteration per instance (easier/numeric/solver/cg.py:68-95, Jacobi M):
//   q = A p; alpha = r.z / p.q; x += alpha p; r -= alpha q; z = M r;
//   stop when ||r|| <= tol; beta = r.z_new / r.z; p = z + beta p
// With the GNN preconditioner (esr_batch.gnn, gnn.cu) the iteration is
// flexible CG: z = M(r) is the network's output and beta takes the
// Polak-Ribiere form z.(r - r_old) / z_old.r_old = -alpha z.q / z_old.r_old.
//
// Work decomposition.  Every instance is padded to whole 256-row tiles
// (identity rows), so no tile spans two instances.  Consecutive tiles of an
// instance form chunks of up to `tiles_per_chunk` tiles: the unit of work
// of one CTA iteration in the per-iteration kernels, which are persistent
// (a fixed grid loops over the chunk list): the direction sweep (p, q = A p,
// p.q) and the update sweep (x, r, z, r.r, r.z), plus the GNN layers and a
// z fix-up in GNN batches.  The double-float policy forms the direction in
// one sweep (q = A z + beta q); the FP64 policy, bound by the FP64 pipe,
// keeps q = A p and a separate p-update sweep at the end of the iteration.  A one-CTA compaction
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
// Polynomial-Jacobi preconditioner (esr_batch.poly_degree = d > 0; a
// classical control for the GNN, no reference counterpart): z = M r is the
// result of d+1 damped Jacobi sweeps on A z = r from z = 0 (a Neumann
// polynomial of degree d in W A, W = omega/diag, held in invdiag).  The
// kernels that write r (init, update, replacement) write the first sweep
// z = W r; bcg_poly_kernel runs the other d at the start of the next
// iteration, the last of them finishing r.z and beta.
// Convergence is re-checked on the FP64 true residual b - A x computed from
// an FP64 copy of the matrix (esr_bcg_verify).  An instance whose true
// residual misses the tolerance continues from it: r = b - A x replaces the
// recurrence residual and p keeps its direction (a residual replacement,
// not a restart).
#include <vector>

#include "bcg_common.cuh"

namespace {

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
  const double v[3] = {bsum<kBThreads>(DotAccD{bb}), bsum<kBThreads>(rz), bsum<kBThreads>(rr)};
  double tot[3];
  if (tile_finish<3>(a, inst, v, L, tot) && threadIdx.x == 0) {
    esr_bcg_inst &s = L.inst[inst];
    s.bnorm = sqrt(tot[0]);
    double tol = rtol * s.bnorm;
    if (has_atol && atol > tol) tol = atol;
    s.tol = tol;
    s.rz = tot[1];
    s.rr = tot[2];
    s.pq = 0.0;
    set_alpha(s, 0.0);
    set_beta(s, 0.0);
    s.true_rr = -1.0;
    s.iters = 0;
    s.verified = 0;
    s.restarts = 0;
    s.maxiter = maxiter;
    s.mode = a.use_gnn ? kModeGnn : kModeJacobi;
    s.refresh = 2;  // the first direction: p = z, q = A z
    s.fallbacks = 0;
    s.gnn_iters = 0;
    s.clips = 0;
    s.clips_mark = 0;
    s.theta = 1.0;
    s.nrows = a.use_gnn ? a.inst_rows[inst] : 0;
    s.sigma = s.nrows > 0 ? sqrt(tot[2] / s.nrows) : 0.0;
    s.rr_mark = tot[2];
    s.rz_jac = tot[1];
    s.done = 0;  // the reference always takes a first step (cg.py:143-153)
    atomicAdd(&L.head->active, 1);
  }
}

// ---- step part 1: the direction and its product with A.
// p = z + beta p and q = A p, formed as q = A z + beta q (A p_new =
// A z + beta A p_old): the SpMV reads z, which the previous sweep finished,
// so the p-update needs no sweep of its own; then p.q -> alpha.  Each row
// reads other rows' z (never written here) and writes only its own p and q.
// A first direction (refresh != 0: after init or a residual replacement,
// and the GNN's fallback to Jacobi) is p = z, q = A z.  The GNN's clipped
// correction is folded into z by bcg_zfix_kernel before.
template <class P>
__global__ void __launch_bounds__(kBThreads, 4)
bcg_pq_kernel(BArgs a, const typename P::V *__restrict__ val, const typename P::V *__restrict__ diag,
              const typename P::V *__restrict__ z, typename P::V *__restrict__ p, typename P::V *__restrict__ q,
              BcgLayout L) {
  using V = typename P::V;
  const int count = L.head->acount;
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = L.alist[w];
    const int inst = a.chunk_inst[c];
    if (L.inst[inst].done) continue;
    const bool first = L.inst[inst].refresh != 0;
    const V beta = P::beta(L.inst[inst]);
    typename P::Acc pq;
    const int t1 = a.chunk_tile0[c + 1];
#pragma unroll 2
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      const V zi = z[i];
      const V w = P::fma(diag[i], zi, bsell_row<P>(i, a.n, a.slice_ptr, a.col, val, z));
      const V pi = first ? zi : P::fma(beta, p[i], zi);
      const V qi = first ? w : P::fma(beta, q[i], w);
      p[i] = pi;
      q[i] = qi;
      pq.add(pi, qi);
    }
    const double v[1] = {bsum<kBThreads>(pq)};
    double tot[1];
    if (chunk_finish<1>(a, c, inst, v, L, tot) && threadIdx.x == 0) {
      esr_bcg_inst &s = L.inst[inst];
      s.pq = tot[0];
      if (!(tot[0] != 0.0) || !isfinite(tot[0])) {
        s.done = 3;  // breakdown
        retire(L);
      } else {
        set_alpha(s, s.rz / tot[0]);
      }
    }
  }
}

// ---- the same as two sweeps (FP64 policy): q = A p; p.q; alpha ...
template <class P>
__global__ void __launch_bounds__(kBThreads, 4)
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
#pragma unroll 2
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      const V pi = p[i];
      const V qi = P::fma(diag[i], pi, bsell_row<P>(i, a.n, a.slice_ptr, a.col, val, p));
      q[i] = qi;
      pq.add(pi, qi);
    }
    const double v[1] = {bsum<kBThreads>(pq)};
    double tot[1];
    if (chunk_finish<1>(a, c, inst, v, L, tot) && threadIdx.x == 0) {
      esr_bcg_inst &s = L.inst[inst];
      s.pq = tot[0];
      if (!(tot[0] != 0.0) || !isfinite(tot[0])) {
        s.done = 3;  // breakdown
        retire(L);
      } else {
        set_alpha(s, s.rz / tot[0]);
      }
    }
  }
}

// ... and, at the end of the iteration, p = z + beta p (p = z for a first
// direction: the GNN's fallback; init and replacement set p themselves)
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_pupdate_kernel(BArgs a, const typename P::V *__restrict__ z, typename P::V *__restrict__ p, BcgLayout L) {
  using V = typename P::V;
  const int count = L.head->acount;
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = L.alist[w];
    const int inst = a.chunk_inst[c];
    if (L.inst[inst].done) continue;
    const bool first = L.inst[inst].refresh != 0;
    const V beta = P::beta(L.inst[inst]);
    const int t1 = a.chunk_tile0[c + 1];
#pragma unroll 2
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      p[i] = first ? z[i] : P::fma(beta, p[i], z[i]);
    }
  }
}

// ---- GNN iterations, after the layers: the z the next direction uses.
//   refresh == 1 (fallback to Jacobi; beta = 0): z = invdiag r
//   GNN with a clipped correction (theta < 1): the layers stored
//   z = zJ + zN; z = zJ + theta zN = theta z + (1 - theta) invdiag r
template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_zfix_kernel(BArgs a, const typename P::V *__restrict__ invdiag, const typename P::V *__restrict__ r,
                typename P::V *__restrict__ z, BcgLayout L) {
  using V = typename P::V;
  const int count = L.head->acount;
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = L.alist[w];
    const int inst = a.chunk_inst[c];
    const esr_bcg_inst &st = L.inst[inst];
    if (st.done) continue;
    const bool refresh = st.refresh == 1;
    if (!refresh && !(st.mode == kModeGnn && st.theta != 1.0)) continue;
    const V th = P::of(st.theta), omth = P::of(1.0 - st.theta);
    const int t1 = a.chunk_tile0[c + 1];
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      const V zj = invdiag ? P::mul(r[i], invdiag[i]) : r[i];
      z[i] = refresh ? zj : P::fma(th, z[i], P::mul(omth, zj));
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
    const bool gnn = L.inst[inst].mode == kModeGnn;  // z comes from the GNN layers
    const V av = P::alpha(L.inst[inst]), nav = P::neg(av);
    typename P::Acc rr, rz;
    const int t1 = a.chunk_tile0[c + 1];
#pragma unroll 2
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      x[i] = P::fma(av, p[i], x[i]);
      const V ri = P::fma(nav, q[i], r[i]);
      r[i] = ri;
      const V zi = invdiag ? P::mul(ri, invdiag[i]) : ri;
      if (!gnn) z[i] = zi;
      rr.add(ri, ri);
      rz.add(ri, zi);
    }
    const double v[2] = {bsum<kBThreads>(rr), bsum<kBThreads>(rz)};
    double tot[2];
    if (chunk_finish<2>(a, c, inst, v, L, tot) && threadIdx.x == 0) {
      esr_bcg_inst &s = L.inst[inst];
      s.iters += 1;
      s.rr = tot[0];
      s.rz_jac = tot[1];
      s.refresh = 0;
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
      } else if (s.mode == kModeGnn) {
        // beta follows from the GNN output (gnn.cu); here: input scale and
        // the stall test (no decrease of r.r over a window -> Jacobi)
        s.sigma = s.nrows > 0 ? sqrt(tot[0] / s.nrows) : 0.0;
        if (a.stall_window > 0 && s.iters % a.stall_window == 0) {
          const bool clipped = 2 * (s.clips - s.clips_mark) > a.stall_window;
          s.clips_mark = s.clips;
          if (!(tot[0] < s.rr_mark) || clipped) {
            s.mode = kModeJacobi;
            s.refresh = 1;
            s.fallbacks += 1;
            s.gnn_iters = s.iters;
            set_beta(s, 0.0);
            s.rz = tot[1];
          } else {
            s.rr_mark = tot[0];
          }
        }
      } else if (!a.poly) {  // polynomial: beta and r.z follow the sweeps
        set_beta(s, tot[1] / s.rz);
        s.rz = tot[1];
      }
    }
  }
}

// ---- polynomial-Jacobi sweep: y_out = y_in + W (r - A y_in), persistent
// over the running chunks.  Each row reads other rows' y_in (never written
// here) and writes only its own y_out.  The last sweep (y_out = z) adds r.z
// per instance and sets beta = r.z / r.z_old, except for a first direction
// (refresh != 0: after init), which only takes r.z.  After a residual
// replacement the direction continues (refresh == 0) with the r.z_old of
// the iteration before it.
template <class P, bool LAST>
__global__ void __launch_bounds__(kBThreads, 4)
bcg_poly_kernel(BArgs a, const typename P::V *__restrict__ val, const typename P::V *__restrict__ diag,
                const typename P::V *__restrict__ w, const typename P::V *__restrict__ r,
                const typename P::V *__restrict__ y_in, typename P::V *__restrict__ y_out, BcgLayout L) {
  using V = typename P::V;
  const int count = L.head->acount;
  for (int u = blockIdx.x; u < count; u += gridDim.x) {
    const int c = L.alist[u];
    const int inst = a.chunk_inst[c];
    if (L.inst[inst].done) continue;
    typename P::Acc rz;
    const int t1 = a.chunk_tile0[c + 1];
#pragma unroll 2
    for (int t = a.chunk_tile0[c]; t < t1; ++t) {
      const int64_t i = (int64_t)t * kBThreads + threadIdx.x;
      const V yi = y_in[i];
      const V ri = r[i];
      const V ay = P::fma(diag[i], yi, bsell_row<P>(i, a.n, a.slice_ptr, a.col, val, y_in));
      const V yo = P::fma(w[i], P::sub(ri, ay), yi);
      y_out[i] = yo;
      if constexpr (LAST) rz.add(ri, yo);
    }
    if constexpr (LAST) {
      const double v[1] = {bsum<kBThreads>(rz)};
      double tot[1];
      if (chunk_finish<1>(a, c, inst, v, L, tot) && threadIdx.x == 0) {
        esr_bcg_inst &s = L.inst[inst];
        if (!(tot[0] != 0.0) || !isfinite(tot[0])) {
          s.done = 3;  // breakdown (M r = 0 or not finite)
          retire(L);
        } else {
          if (s.refresh == 0) set_beta(s, tot[0] / s.rz);
          s.rz = tot[0];
        }
      }
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
  const double v[1] = {bsum<kBThreads>(DotAccD{rr})};
  double tot[1];
  if (tile_finish<1>(a, inst, v, L, tot) && threadIdx.x == 0) {
    st.true_rr = tot[0];
    const double rn = sqrt(tot[0]);
    st.verified = (!isnan(rn) && rn <= st.tol) ? 1 : -1;
  }
}

// ---- pass 3, instances whose true residual missed: residual replacement
// r = r64, z = M r, then p = z + beta p with beta = r.z / r.z_old while the
// true residual is within twice the recurrence residual (rounding drift:
// the direction stays conjugate enough to keep), else a restart, p = z (a
// residual far from the recurrence's makes beta huge and the continued
// direction useless); running again
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
  const double v[1] = {bsum<kBThreads>(rz)};
  double tot[1];
  if (tile_finish<1>(a, inst, v, L, tot) && threadIdx.x == 0) {
    // GNN mode: p restarts from the Jacobi direction
    const bool restart = st.mode == kModeGnn || st.rz == 0.0 || !(st.true_rr <= 4.0 * st.rr);
    if (!a.poly) {  // polynomial: z = W r is the first sweep; r.z_old stays for the last
      set_beta(st, restart ? 0.0 : tot[0] / st.rz);
      st.rz = tot[0];
      st.rz_jac = tot[0];
    }
    st.rr = st.true_rr;
    st.verified = restart ? -3 : -2;  // p update pending
  }
}

template <class P>
__global__ void __launch_bounds__(kBThreads)
bcg_replace_p_kernel(BArgs a, typename P::V *__restrict__ z, typename P::V *__restrict__ p, BcgLayout L) {
  const int inst = a.block_inst[blockIdx.x];
  esr_bcg_inst &st = L.inst[inst];
  if (st.verified != -2 && st.verified != -3) return;
  const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
  // the continued direction p_new = z + beta p (beta = 0 on a restart), in
  // p (for bcg_spmv_kernel) and in z (for bcg_pq_kernel's first direction),
  // so the next product is q = A p_new exactly (the update recomputes z
  // from r before anything else reads it)
  // (polynomial: p stays; the sweeps finish z and beta, and the next
  // direction continues from p as in any iteration, or starts at p = z)
  if (i < a.n && !a.poly) {
    const typename P::V pn = P::fma(P::beta(st), p[i], z[i]);
    p[i] = pn;
    z[i] = pn;
  }
  // the instance's tiles all pass the test above before any of them
  // re-arms it: the ticket counter orders them
  const double v[1] = {0.0};
  double tot[1];
  if (tile_finish<1>(a, inst, v, L, tot) && threadIdx.x == 0) {
    st.refresh = (a.poly && st.verified == -2) ? 0 : 2;
    st.verified = 0;
    st.restarts += 1;
    st.done = 0;
    atomicAdd(&L.head->active, 1);
  }
}

// ---- standalone preconditioner application: every instance in GNN mode
// with sigma = rms of r
template <class P>
__global__ void __launch_bounds__(kBThreads)
gnn_prep_kernel(BArgs a, const typename P::V *__restrict__ r, BcgLayout L) {
  const int inst = a.block_inst[blockIdx.x];
  const int64_t i = (int64_t)blockIdx.x * kBThreads + threadIdx.x;
  typename P::Acc rr;
  if (i < a.n) rr.add(r[i], r[i]);
  const double v[1] = {bsum<kBThreads>(rr)};
  double tot[1];
  if (tile_finish<1>(a, inst, v, L, tot) && threadIdx.x == 0) {
    esr_bcg_inst &s = L.inst[inst];
    s.nrows = a.inst_rows[inst];
    s.sigma = s.nrows > 0 ? sqrt(tot[0] / s.nrows) : 0.0;
    s.rr = tot[0];
    s.rz = 1.0;
    set_alpha(s, 0.0);
    s.mode = kModeGnn;
    s.done = 0;
  }
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
  const int d = B->poly_degree;
  V *const tmp0 = (V *)B->poly_tmp, *const tmp1 = tmp0 ? tmp0 + B->n : nullptr;
  for (int32_t it = 0; it < k; ++it) {
    if (d > 0) {  // z = M r: sweeps 2..d+1 (z -> tmp0 -> tmp1 -> tmp0 ... -> z)
      const V *src = (const V *)z;
      for (int j = 1; j <= d; ++j) {
        V *dst = j == d ? (V *)z : ((j & 1) ? tmp0 : tmp1);
        if (j == d)
          bcg_poly_kernel<P, true><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->val, (const V *)B->diag,
                                                                 (const V *)B->invdiag, (const V *)r, src, dst, L);
        else
          bcg_poly_kernel<P, false><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->val, (const V *)B->diag,
                                                                  (const V *)B->invdiag, (const V *)r, src, dst, L);
        src = dst;
      }
      if constexpr (!P::kFusedDirection)
        bcg_pupdate_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)z, (V *)p, L);
    }
    if constexpr (P::kFusedDirection)
      bcg_pq_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->val, (const V *)B->diag, (const V *)z, (V *)p,
                                                     (V *)q, L);
    else
      bcg_spmv_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->val, (const V *)B->diag, (const V *)p,
                                                       (V *)q, L);
    bcg_update_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->invdiag, (V *)x, (V *)r, (V *)z,
                                                       (const V *)p, (const V *)q, L);
    if (B->gnn) {
      const int st = esr::gnn_layers(B, r, q, z, ws, s);
      if (st) return st;
      bcg_zfix_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)B->invdiag, (const V *)r, (V *)z, L);
    }
    if constexpr (!P::kFusedDirection)
      if (d == 0) bcg_pupdate_kernel<P><<<B->grid, kBThreads, 0, s>>>(a, (const V *)z, (V *)p, L);
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
  bcg_replace_p_kernel<P><<<B->nblocks, kBThreads, 0, s>>>(a, (V *)z, (V *)p, L);
  ESR_LAUNCH_CHECK("esr_bcg_verify");
  return ESR_OK;
}

template <class P>
int run_gnn_apply(const esr_batch *B, const void *r, void *z, void *ws, cudaStream_t s) {
  BcgLayout L = layout_of(ws, B->ninst, B->nchunks);
  const BArgs a = bargs(B);
  cudaError_t e = cudaMemsetAsync(ws, 0, workspace_bytes(B->ninst, B->nblocks, B->nchunks), s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_gnn_apply/memset");
  gnn_prep_kernel<P><<<B->nblocks, kBThreads, 0, s>>>(a, (const typename P::V *)r, L);
  bcg_compact_kernel<<<1, 1024, 0, s>>>(a, L);
  ESR_LAUNCH_CHECK("esr_gnn_apply");
  return esr::gnn_layers(B, r, r, z, ws, s);
}

// ------------------------------------------------------------------------
// The whole solve as ONE CUDA graph launch: [workspace memset, init] then a
// device-side WHILE node whose body is [compaction + k iterations,
// verification of the instances that converged in it, condition].  The
// condition kernel keeps looping while instances run and stops after
// max_bodies bodies whatever happens, so the graph always terminates.
__global__ void bcg_graph_cond_kernel(cudaGraphConditionalHandle h, BcgHead *head, int max_bodies) {
  const int bodies = head->bodies + 1;
  head->bodies = bodies;
  cudaGraphSetConditional(h, (head->active > 0 && bodies < max_bodies) ? 1u : 0u);
}

struct BcgGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
};

template <class P>
int build_graph(const esr_batch *B, const double *b64, const void *b, void *x, void *r, void *z, void *p, void *q,
                double *x64, double *r64, double rtol, double atol, int32_t maxiter, int32_t k, void *ws,
                BcgGraph *G) {
  cudaError_t e = cudaStreamCreateWithFlags(&G->capture, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaGraphCreate(&G->graph, 0);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create");
  cudaStream_t s = G->capture;
  // [memset, init]
  e = cudaStreamBeginCaptureToGraph(s, G->graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/capture init");
  int st = run_init<P>(B, b64, b, x, r, z, p, rtol, atol, maxiter, ws, s);
  cudaGraph_t tmp = nullptr;
  e = cudaStreamEndCapture(s, &tmp);
  if (st) return st;
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/end init");
  // the WHILE node after the init's last node
  size_t nn = 0;
  e = cudaGraphGetNodes(G->graph, nullptr, &nn);
  if (e != cudaSuccess || nn == 0) return esr::cuda_check(e, "esr_bcg_graph_create/nodes");
  std::vector<cudaGraphNode_t> nodes(nn), leaves;
  e = cudaGraphGetNodes(G->graph, nodes.data(), &nn);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/nodes");
  for (cudaGraphNode_t n : nodes) {
    size_t nd = 0;
    e = cudaGraphNodeGetDependentNodes(n, nullptr, nullptr, &nd);
    if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/dependents");
    if (nd == 0) leaves.push_back(n);
  }
  cudaGraphConditionalHandle h;
  e = cudaGraphConditionalHandleCreate(&h, G->graph, 1u, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/handle");
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t cnode;
  e = cudaGraphAddNode(&cnode, G->graph, leaves.data(), nullptr, leaves.size(), &np);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/while node");
  cudaGraph_t body = np.conditional.phGraph_out[0];
  // the body
  e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/capture body");
  st = run_iterate<P>(B, x, r, z, p, q, k, ws, s);
  if (!st) st = run_verify<P>(B, b64, x, x64, r64, r, z, p, ws, s);
  const int max_bodies = (int)((maxiter + (int64_t)k) / k) * 2 + 16;  // replacements restart instances
  if (!st) {
    BcgLayout L = layout_of(ws, B->ninst, B->nchunks);
    bcg_graph_cond_kernel<<<1, 1, 0, s>>>(h, L.head, max_bodies);
  }
  cudaGraph_t tmp2 = nullptr;
  e = cudaStreamEndCapture(s, &tmp2);
  if (st) return st;
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/end body");
  e = cudaGraphInstantiate(&G->exec, G->graph, 0);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_create/instantiate");
  return ESR_OK;
}

void destroy_graph(BcgGraph *G) {
  if (!G) return;
  if (G->exec) cudaGraphExecDestroy(G->exec);
  if (G->graph) cudaGraphDestroy(G->graph);
  if (G->capture) cudaStreamDestroy(G->capture);
  delete G;
}

}  // namespace

extern "C" int esr_bcg_graph_create(const esr_batch *B, const double *b64, const void *b, void *x, void *r, void *z,
                                    void *p, void *q, double *x64, double *r64, double rtol, double atol,
                                    int32_t maxiter, int32_t k, void *workspace, void **graph_out) {
  int st = check_batch(B);
  if (st) return st;
  if (!b64 || !b || !x || !r || !z || !p || !q || !x64 || !r64 || !workspace || !graph_out)
    return esr::fail(ESR_ERR_ARG, "null argument");
  if (maxiter < 0 || maxiter > (1 << 26)) return esr::fail(ESR_ERR_ARG, "the one-launch graph needs a finite maxiter");
  if (k < 1 || k > 1024) return esr::fail(ESR_ERR_ARG, "iterations per body must be in [1, 1024]");
  BcgGraph *G = new (std::nothrow) BcgGraph();
  if (!G) return esr::fail(ESR_ERR_ARG, "out of host memory");
  try {
    st = B->df64 ? build_graph<PolDF>(B, b64, b, x, r, z, p, q, x64, r64, rtol, atol, maxiter, k, workspace, G)
                 : build_graph<PolF64>(B, b64, b, x, r, z, p, q, x64, r64, rtol, atol, maxiter, k, workspace, G);
  } catch (const std::bad_alloc &) {
    st = esr::fail(ESR_ERR_ARG, "out of host memory");
  }
  if (st) {
    destroy_graph(G);
    return st;
  }
  *graph_out = G;
  return ESR_OK;
}

extern "C" int esr_bcg_graph_launch(void *graph, void *stream) {
  if (!graph) return esr::fail(ESR_ERR_ARG, "null graph");
  cudaError_t e = cudaGraphLaunch(((BcgGraph *)graph)->exec, esr::as_stream(stream));
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bcg_graph_launch");
  return ESR_OK;
}

extern "C" int esr_bcg_graph_destroy(void *graph) {
  destroy_graph((BcgGraph *)graph);
  return ESR_OK;
}

extern "C" int esr_gnn_apply(const esr_batch *B, const void *r, void *z, void *workspace, void *stream) {
  int st = check_batch(B);
  if (st) return st;
  if (!B->gnn) return esr::fail(ESR_ERR_ARG, "esr_gnn_apply needs batch.gnn");
  if (!r || !z || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  return B->df64 ? run_gnn_apply<PolDF>(B, r, z, workspace, s) : run_gnn_apply<PolF64>(B, r, z, workspace, s);
}

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
