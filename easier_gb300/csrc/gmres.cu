// Fused restarted GMRES on a SELL-32 Linsys, easier/numeric/solver/gmres.py.
//
// One restart cycle (gmres.py:235-261) on the device, enqueued as a fixed
// sequence of launches (the host captures it in a CUDA graph):
//   initv       V_0 = r / ||r||
//   for j < restart:
//     matvec(j) V_j = w_prev / H[j][j-1] (j >= 1, written for own rows and
//               formed on the fly for gathered columns), w = A M V_j,
//               H[0][j] = V_0 . w
//     mgs(i, j) for i = 0..j: w -= H[i][j] V_i, then H[i+1][j] = V_{i+1} . w
//               (i < j) or H[j+1][j] = ||w|| (i == j): modified Gram-Schmidt
//               in the reference's order, each dot fused into the preceding
//               axpy's pass
//   lsq         y = argmin || ||r|| e_1 - H y || by Givens rotations (one
//               thread; the reference takes the SVD pseudo-inverse with
//               singular values clamped at 1e-8: the same y for a full-rank H)
//   updatex     x += M (V[:, :k] y)
//   residual    r = b - A x, ||r|| for the host's stopping test
// A breakdown (H[j+1][j] < 1e-15) ends the Arnoldi loop: the remaining
// matvec/mgs launches of the cycle see the flag and return.  Dots
// accumulate in FP64 per thread and are combined by the grid's last block
// in block order (deterministic).  V is column-contiguous: V_c = V + c*n.
#include <cmath>
#include <cstdint>

#include "esr_internal.h"
#include "reduce_util.cuh"

namespace {

constexpr int kGmThreads = 256;
constexpr int kGmMaxBlocks = 1216;
constexpr int kGmMaxRestart = 64;

struct GmState {
  double rnorm, bnorm, tol, pad0;
  double H[(kGmMaxRestart + 1) * kGmMaxRestart];  // [i][j] at i * kGmMaxRestart + j
  double y[kGmMaxRestart];
  int32_t jend;    // Arnoldi columns of the current cycle
  int32_t broken;  // breakdown in the current cycle
  int32_t cycles;
  int32_t pad1;
};

struct GmWork {
  GmState s;
  unsigned int counter[4];
  double partial[kGmMaxBlocks];
};

inline int grid_for(int64_t n) {
  int64_t g = (n + kGmThreads - 1) / kGmThreads;
  return (int)(g < 1 ? 1 : (g > kGmMaxBlocks ? kGmMaxBlocks : g));
}

// sum over the row's SELL slots of val * f(col), in slot order
template <typename T, class F>
__device__ __forceinline__ double gm_row(int64_t i, int64_t n, const int64_t *__restrict__ slice_ptr,
                                         const int32_t *__restrict__ col, const T *__restrict__ val, F f) {
  const int64_t s = i >> 5;
  const int lane = (int)(i & 31);
  const int64_t b = __ldg(slice_ptr + s);
  const int w = (int)((__ldg(slice_ptr + s + 1) - b) >> 5);
  double acc = 0.0;
  for (int k = 0; k < w; ++k) {
    const int64_t e = b + 32 * k + lane;
    const int32_t c = __ldg(col + e);
    if (c >= 0 && (int64_t)c < n) acc = fma((double)__ldg(val + e), f(c), acc);
  }
  return acc;
}

// block partial -> last block writes the grid total through `store`
template <class S>
__device__ __forceinline__ void gm_finish(double v, GmWork *w, S store) {
  __shared__ double s_red[kGmThreads / 32];
  const double bs = esr::block_sum_fixed<kGmThreads>(v, s_red);
  if (esr::last_block_done(bs, w->partial, &w->counter[0])) {
    double acc = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += kGmThreads) acc += __ldcg(w->partial + q);
    const double tot = esr::block_sum_fixed<kGmThreads>(acc, s_red);
    if (threadIdx.x == 0) {
      store(tot);
      w->counter[0] = 0u;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kGmThreads) gm_norm_kernel(int64_t n, const T *__restrict__ b, double rtol,
                                                             double atol, int has_atol, GmWork *w) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kGmThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kGmThreads) {
    const double v = (double)b[i];
    acc = fma(v, v, acc);
  }
  gm_finish(acc, w, [&](double tot) {
    GmState &s = w->s;
    s.bnorm = sqrt(tot);
    double tol = rtol * s.bnorm;
    if (has_atol && atol > tol) tol = atol;
    s.tol = tol;
    s.cycles = 0;
  });
}

// r = b - A x; ||r||
template <typename T>
__global__ void __launch_bounds__(kGmThreads)
gm_resid_kernel(esr_sell A, const T *__restrict__ b, const T *__restrict__ x, T *__restrict__ r, GmWork *w) {
  const T *val = (const T *)A.val, *diag = (const T *)A.diag;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kGmThreads + threadIdx.x; i < A.n;
       i += (int64_t)gridDim.x * kGmThreads) {
    const double ax = fma((double)diag[i], (double)x[i],
                          gm_row<T>(i, A.n, A.slice_ptr, A.col, val, [&](int32_t c) { return (double)x[c]; }));
    const T ri = (T)((double)b[i] - ax);
    r[i] = ri;
    acc = fma((double)ri, (double)ri, acc);
  }
  gm_finish(acc, w, [&](double tot) {
    w->s.rnorm = sqrt(tot);
    w->s.broken = 0;
    w->s.jend = 0;
  });
}

template <typename T>
__global__ void __launch_bounds__(kGmThreads) gm_initv_kernel(int64_t n, const T *__restrict__ r, T *__restrict__ v0,
                                                              const GmWork *w) {
  const double rn = w->s.rnorm;
  const double inv = rn > 0.0 ? 1.0 / rn : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kGmThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kGmThreads)
    v0[i] = (T)((double)r[i] * inv);
}

// V_j (j >= 1: from w_prev), w = A M V_j, H[0][j] = V_0 . w
template <typename T>
__global__ void __launch_bounds__(kGmThreads)
gm_matvec_kernel(esr_sell A, const T *__restrict__ invdiag, T *__restrict__ V, const T *__restrict__ w_prev,
                 T *__restrict__ w_out, int j, GmWork *w) {
  if (w->s.broken) return;
  const int64_t n = A.n;
  const T *val = (const T *)A.val, *diag = (const T *)A.diag;
  T *vj = V + (int64_t)j * n;
  const T *v0 = V;
  const double inv_h = j >= 1 ? 1.0 / w->s.H[j * kGmMaxRestart + (j - 1)] : 1.0;
  auto vcol = [&](int64_t c) -> double {  // V_j[c] without reading V_j
    return j >= 1 ? (double)(T)((double)w_prev[c] * inv_h) : (double)vj[c];
  };
  auto zcol = [&](int64_t c) -> double {  // (M V_j)[c]
    const double v = vcol(c);
    return invdiag ? (double)(T)(v * (double)invdiag[c]) : v;
  };
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kGmThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kGmThreads) {
    if (j >= 1) vj[i] = (T)((double)w_prev[i] * inv_h);
    const double wi =
        fma((double)diag[i], zcol(i), gm_row<T>(i, n, A.slice_ptr, A.col, val, [&](int32_t c) { return zcol(c); }));
    const T wt = (T)wi;
    w_out[i] = wt;
    acc = fma((double)v0[i], (double)wt, acc);
  }
  gm_finish(acc, w, [&](double tot) { w->s.H[0 * kGmMaxRestart + j] = tot; });
}

// w -= H[i][j] V_i; then H[i+1][j] = V_{i+1} . w (i < j) or ||w|| (i == j)
template <typename T>
__global__ void __launch_bounds__(kGmThreads)
gm_mgs_kernel(int64_t n, const T *__restrict__ V, T *__restrict__ wv, int i, int j, int restart, GmWork *w) {
  if (w->s.broken) return;
  const double h = w->s.H[i * kGmMaxRestart + j];
  const T *vi = V + (int64_t)i * n;
  const T *vn = (i < j) ? V + (int64_t)(i + 1) * n : nullptr;
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * kGmThreads + threadIdx.x; r < n; r += (int64_t)gridDim.x * kGmThreads) {
    const T nw = (T)((double)wv[r] - h * (double)vi[r]);
    wv[r] = nw;
    acc = vn ? fma((double)vn[r], (double)nw, acc) : fma((double)nw, (double)nw, acc);
  }
  gm_finish(acc, w, [&](double tot) {
    GmState &s = w->s;
    if (i < j) {
      s.H[(i + 1) * kGmMaxRestart + j] = tot;
    } else {
      const double hn = sqrt(tot);
      s.H[(j + 1) * kGmMaxRestart + j] = hn;
      s.jend = j + 1;
      if (!(hn >= 1e-15)) s.broken = 1;
    }
  });
  (void)restart;
}

// y = argmin || rnorm e_1 - H[:k+1, :k] y ||, k = jend (one thread)
__global__ void gm_lsq_kernel(GmWork *w) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  GmState &s = w->s;
  const int k = s.jend;
  double R[(kGmMaxRestart + 1) * kGmMaxRestart];  // local copy, column j of row i at i*k + j
  double g[kGmMaxRestart + 1];
  for (int i = 0; i <= k; ++i) {
    g[i] = i == 0 ? s.rnorm : 0.0;
    for (int j = 0; j < k; ++j) R[i * kGmMaxRestart + j] = s.H[i * kGmMaxRestart + j];
  }
  for (int j = 0; j < k; ++j) {  // rotate rows j, j+1 to zero R[j+1][j]
    const double a = R[j * kGmMaxRestart + j], b = R[(j + 1) * kGmMaxRestart + j];
    const double rr = hypot(a, b);
    const double c = rr > 0.0 ? a / rr : 1.0, sn = rr > 0.0 ? b / rr : 0.0;
    for (int q = j; q < k; ++q) {
      const double u = R[j * kGmMaxRestart + q], v = R[(j + 1) * kGmMaxRestart + q];
      R[j * kGmMaxRestart + q] = c * u + sn * v;
      R[(j + 1) * kGmMaxRestart + q] = -sn * u + c * v;
    }
    const double u = g[j], v = g[j + 1];
    g[j] = c * u + sn * v;
    g[j + 1] = -sn * u + c * v;
  }
  for (int j = k - 1; j >= 0; --j) {  // back substitution; a zero pivot keeps y_j = 0
    double t = g[j];
    for (int q = j + 1; q < k; ++q) t -= R[j * kGmMaxRestart + q] * s.y[q];
    const double d = R[j * kGmMaxRestart + j];
    s.y[j] = fabs(d) > 1e-300 ? t / d : 0.0;
  }
  s.cycles += 1;
}

// x += M (sum_{c < k} y_c V_c)
template <typename T>
__global__ void __launch_bounds__(kGmThreads)
gm_updatex_kernel(int64_t n, const T *__restrict__ V, const T *__restrict__ invdiag, T *__restrict__ x,
                  const GmWork *w) {
  __shared__ double sy[kGmMaxRestart];
  const int k = w->s.jend;
  for (int c = threadIdx.x; c < k; c += kGmThreads) sy[c] = w->s.y[c];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * kGmThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kGmThreads) {
    double dx = 0.0;
    for (int c = 0; c < k; ++c) dx = fma((double)V[(int64_t)c * n + i], sy[c], dx);
    const T d = (T)dx;
    x[i] = (T)((double)x[i] + (invdiag ? (double)(T)((double)d * (double)invdiag[i]) : (double)d));
  }
}

int check(const esr_sell *A, int32_t restart) {
  if (!A || A->n <= 0) return esr::fail(ESR_ERR_ARG, "empty Linsys");
  if (A->dtype != ESR_F32 && A->dtype != ESR_F64) return esr::fail(ESR_ERR_UNSUPPORTED, "GMRES needs F32 or F64");
  if (restart < 1 || restart > kGmMaxRestart) return esr::fail(ESR_ERR_ARG, "restart must be in [1, 64]");
  if (!A->slice_ptr || !A->col || !A->val || !A->diag) return esr::fail(ESR_ERR_ARG, "null SELL array");
  return ESR_OK;
}

template <typename T>
int run_cycle(const esr_sell *A, const T *invdiag, const T *b, T *x, T *r, T *V, T *w2, int32_t restart, GmWork *w,
              cudaStream_t s) {
  const int64_t n = A->n;
  const int g = grid_for(n);
  gm_initv_kernel<T><<<g, kGmThreads, 0, s>>>(n, r, V, w);
  for (int j = 0; j < restart; ++j) {
    T *wout = w2 + (int64_t)(j & 1) * n;
    const T *wprev = w2 + (int64_t)((j + 1) & 1) * n;
    gm_matvec_kernel<T><<<g, kGmThreads, 0, s>>>(*A, invdiag, V, wprev, wout, j, w);
    for (int i = 0; i <= j; ++i) gm_mgs_kernel<T><<<g, kGmThreads, 0, s>>>(n, V, wout, i, j, restart, w);
  }
  gm_lsq_kernel<<<1, 32, 0, s>>>(w);
  gm_updatex_kernel<T><<<g, kGmThreads, 0, s>>>(n, V, invdiag, x, w);
  gm_resid_kernel<T><<<g, kGmThreads, 0, s>>>(*A, b, x, r, w);
  ESR_LAUNCH_CHECK("esr_gmres_cycle");
  return ESR_OK;
}

}  // namespace

extern "C" int64_t esr_gmres_workspace_bytes(int64_t n, int32_t restart) {
  if (n <= 0 || restart < 1 || restart > kGmMaxRestart) return -1;
  return (int64_t)sizeof(GmWork);
}

extern "C" int esr_gmres_init(const esr_sell *A, const void *b, double rtol, double atol, void *workspace,
                              void *stream) {
  int st = check(A, 1);
  if (st) return st;
  if (!b || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  cudaError_t e = cudaMemsetAsync(workspace, 0, sizeof(GmWork), s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_gmres_init/memset");
  GmWork *w = (GmWork *)workspace;
  const int g = grid_for(A->n);
  if (A->dtype == ESR_F64)
    gm_norm_kernel<double><<<g, kGmThreads, 0, s>>>(A->n, (const double *)b, rtol, atol, atol > 0.0, w);
  else
    gm_norm_kernel<float><<<g, kGmThreads, 0, s>>>(A->n, (const float *)b, rtol, atol, atol > 0.0, w);
  ESR_LAUNCH_CHECK("esr_gmres_init");
  return ESR_OK;
}

extern "C" int esr_gmres_residual(const esr_sell *A, const void *b, const void *x, void *r, void *workspace,
                                  void *stream) {
  int st = check(A, 1);
  if (st) return st;
  if (!b || !x || !r || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  GmWork *w = (GmWork *)workspace;
  const int g = grid_for(A->n);
  if (A->dtype == ESR_F64)
    gm_resid_kernel<double><<<g, kGmThreads, 0, s>>>(*A, (const double *)b, (const double *)x, (double *)r, w);
  else
    gm_resid_kernel<float><<<g, kGmThreads, 0, s>>>(*A, (const float *)b, (const float *)x, (float *)r, w);
  ESR_LAUNCH_CHECK("esr_gmres_residual");
  return ESR_OK;
}

extern "C" int esr_gmres_cycle(const esr_sell *A, const void *invdiag, const void *b, void *x, void *r, void *V,
                               void *w2, int32_t restart, void *workspace, void *stream) {
  int st = check(A, restart);
  if (st) return st;
  if (!b || !x || !r || !V || !w2 || !workspace) return esr::fail(ESR_ERR_ARG, "null vector");
  cudaStream_t s = esr::as_stream(stream);
  GmWork *w = (GmWork *)workspace;
  if (A->dtype == ESR_F64)
    return run_cycle<double>(A, (const double *)invdiag, (const double *)b, (double *)x, (double *)r, (double *)V,
                             (double *)w2, restart, w, s);
  return run_cycle<float>(A, (const float *)invdiag, (const float *)b, (float *)x, (float *)r, (float *)V,
                          (float *)w2, restart, w, s);
}

extern "C" int esr_gmres_read(const void *workspace, esr_gmres_scalars *out, void *stream) {
  if (!workspace || !out) return esr::fail(ESR_ERR_ARG, "null argument");
  cudaStream_t s = esr::as_stream(stream);
  const GmWork *w = (const GmWork *)workspace;
  GmState h;
  cudaError_t e = cudaMemcpyAsync(&h, &w->s, sizeof(GmState), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_gmres_read");
  out->rnorm = h.rnorm;
  out->bnorm = h.bnorm;
  out->tol = h.tol;
  out->jend = h.jend;
  out->broken = h.broken;
  out->cycles = h.cycles;
  out->pad_ = 0;
  return ESR_OK;
}
