// Fused shallow-water step: gather of neighbour state, face reconstruction,
// central flux, per-cell face sum, wall pressure term, division by area and
// the stage combination, in one kernel per stage (4 per step).
//
// Reference: tutorial/shallow_water_equation/swe_main.py
//   face_reconstruct  :83-85   phi_f = (1 - alpha) * phi[src] + alpha * phi[dst]
//   delta             :87-119  fluxes, scatter(dst), scatter_b(bcells), / area
//   forward           :121-141 stage states s + c*delta_k, s += dt/6 * sum_k
//
// Layout (all of it stays in HBM between launches):
//   state  [nc][4]  (h, uh, vh, 0)   16 B (FP32) / 32 B (FP64) per cell
//   slots  [width][nc] nbr:int32, sx, sy, alpha   slot-major -> coalesced
//   area   [nc]
// One thread owns one cell and walks its face slots in order: interior edges
// in the reference's edge order, then wall faces.  The per-cell sums are
// therefore the reference's in-order Reducer sums, and every arithmetic
// operation is one round-to-nearest IEEE op in the reference's order, so the
// result is bitwise the reference's CPU result.
//
// Stages (c1 = 0.5*dt, c3 = dt, c4 = dt/6, rounded to T like torch does):
//   1: D1 = delta(s0);           S1 = s0 + c1*D1;  A = D1
//   2: D2 = delta(S1);           S2 = s0 + c1*D2;  A = A + D2
//   3: D3 = delta(S2);           S1 = s0 + c3*D3;  A = A + D3
//   4: D4 = delta(S1);           s0 = s0 + c4*(A + D4)
// Stage 4 writes s0 in place: it gathers neighbours from S1 and reads s0
// only at its own cell.
#include <cstdint>

#include "esr_internal.h"
#include "reduce_util.cuh"

namespace {

constexpr int kSweThreads = 256;

template <typename T>
struct alignas(4 * sizeof(T)) Vec4 {
  T x, y, z, w;
};

template <typename T>
__device__ __forceinline__ Vec4<T> load4(const T *p) {
  return *reinterpret_cast<const Vec4<T> *>(p);
}
template <>
__device__ __forceinline__ Vec4<double> load4<double>(const double *p) {
  const double2 a = reinterpret_cast<const double2 *>(p)[0];
  const double2 b = reinterpret_cast<const double2 *>(p)[1];
  return Vec4<double>{a.x, a.y, b.x, b.y};
}
template <typename T>
__device__ __forceinline__ void store4(T *p, Vec4<T> v) {
  *reinterpret_cast<Vec4<T> *>(p) = v;
}
template <>
__device__ __forceinline__ void store4<double>(double *p, Vec4<double> v) {
  reinterpret_cast<double2 *>(p)[0] = make_double2(v.x, v.y);
  reinterpret_cast<double2 *>(p)[1] = make_double2(v.z, v.w);
}

// delta (swe_main.py:87-119) of cell i given the stage state `s`.
template <typename T, int W>
__device__ __forceinline__ Vec4<T> cell_delta(int64_t i, int64_t nc, const int32_t *__restrict__ nbr,
                                              const T *__restrict__ sx, const T *__restrict__ sy,
                                              const T *__restrict__ alpha, const T *__restrict__ area,
                                              const T *__restrict__ s, const Vec4<T> own) {
  using O = ops<T>;
  const T half = T(0.5);
  T Sh = T(0), Su = T(0), Sv = T(0);  // scatter(...) over interior edges
  T Bu = T(0), Bv = T(0);             // scatter_b(...) over wall faces
#pragma unroll
  for (int k = 0; k < W; ++k) {
    const int32_t j = __ldg(nbr + k * nc + i);
    if (j >= 0) {
      if ((int64_t)j >= nc) {  // corrupt slot: flag it, never read out of bounds
        esr::raise_status(ESR_DEV_IDX_RANGE);
        continue;
      }
      const T a = __ldg(alpha + k * nc + i);
      const T fx = __ldg(sx + k * nc + i);
      const T fy = __ldg(sy + k * nc + i);
      const Vec4<T> nb = load4(s + 4 * (int64_t)j);
      const T om = O::sub(T(1), a);
      // face_reconstruct: (1 - alpha) * gather_src + alpha * gather_dst
      const T hf = O::add(O::mul(om, nb.x), O::mul(a, own.x));
      const T uhf = O::add(O::mul(om, nb.y), O::mul(a, own.y));
      const T vhf = O::add(O::mul(om, nb.z), O::mul(a, own.z));
      const T uf = O::div(uhf, hf);
      const T vf = O::div(vhf, hf);
      const T hfs = O::mul(O::mul(half, hf), hf);  // 0.5 * h_f * h_f
      const T uhsx = O::mul(uhf, fx);               // uh_f * sx
      const T vhsy = O::mul(vhf, fy);               // vh_f * sy
      const T Fh = O::add(uhsx, vhsy);
      const T Fu = O::add(O::mul(O::add(O::mul(uf, uhf), hfs), fx), O::mul(uf, vhsy));
      const T Fv = O::add(O::mul(vf, uhsx), O::mul(O::add(O::mul(vf, vhf), hfs), fy));
      Sh = O::add(Sh, Fh);
      Su = O::add(Su, Fu);
      Sv = O::add(Sv, Fv);
    } else if (j == -1) {
      // wall face: 0.5 * gather_b(h)**2 * (bsx, bsy)
      const T fx = __ldg(sx + k * nc + i);
      const T fy = __ldg(sy + k * nc + i);
      const T gb = O::mul(half, O::mul(own.x, own.x));
      Bu = O::add(Bu, O::mul(gb, fx));
      Bv = O::add(Bv, O::mul(gb, fy));
    }
  }
  const T ar = __ldg(area + i);
  Vec4<T> d;
  d.x = O::div(-Sh, ar);
  d.y = O::div(-O::add(Su, Bu), ar);
  d.z = O::div(-O::add(Sv, Bv), ar);
  d.w = T(0);
  return d;
}

template <typename T, int W, int STAGE>
__global__ void __launch_bounds__(kSweThreads)
swe_stage_kernel(int64_t nc, const int32_t *__restrict__ nbr, const T *__restrict__ sx,
                 const T *__restrict__ sy, const T *__restrict__ alpha, const T *__restrict__ area,
                 const T *__restrict__ sin, const T *s0, T *__restrict__ acc, T *sout, T c) {
  using O = ops<T>;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const Vec4<T> own_in = load4(sin + 4 * i);
  const Vec4<T> d = cell_delta<T, W>(i, nc, nbr, sx, sy, alpha, area, sin, own_in);
  const Vec4<T> base = (STAGE == 1) ? own_in : load4(s0 + 4 * i);
  Vec4<T> out;
  if (STAGE < 4) {
    out.x = O::add(base.x, O::mul(c, d.x));
    out.y = O::add(base.y, O::mul(c, d.y));
    out.z = O::add(base.z, O::mul(c, d.z));
    out.w = T(0);
    Vec4<T> a;
    if (STAGE == 1) {
      a = d;
    } else {
      const Vec4<T> prev = load4(acc + 4 * i);
      a.x = O::add(prev.x, d.x);
      a.y = O::add(prev.y, d.y);
      a.z = O::add(prev.z, d.z);
      a.w = T(0);
    }
    store4(acc + 4 * i, a);
  } else {
    const Vec4<T> prev = load4(acc + 4 * i);
    out.x = O::add(base.x, O::mul(c, O::add(prev.x, d.x)));
    out.y = O::add(base.y, O::mul(c, O::add(prev.y, d.y)));
    out.z = O::add(base.z, O::mul(c, O::add(prev.z, d.z)));
    out.w = base.w;
  }
  store4(sout + 4 * i, out);
}

template <typename T, int W>
__global__ void __launch_bounds__(kSweThreads)
swe_delta_kernel(int64_t nc, const int32_t *__restrict__ nbr, const T *__restrict__ sx,
                 const T *__restrict__ sy, const T *__restrict__ alpha, const T *__restrict__ area,
                 const T *__restrict__ s, T *__restrict__ dout) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const Vec4<T> own = load4(s + 4 * i);
  store4(dout + 4 * i, cell_delta<T, W>(i, nc, nbr, sx, sy, alpha, area, s, own));
}

int check_mesh(const esr_swe_mesh *m) {
  if (!m) return esr::fail(ESR_ERR_ARG, "null mesh");
  if (m->nc <= 0) return esr::fail(ESR_ERR_ARG, "mesh has no cells");
  if (m->nc > ((int64_t)1 << 31) - 1) return esr::fail(ESR_ERR_UNSUPPORTED, "more than 2^31-1 cells");
  if (m->width != 3 && m->width != 4) return esr::fail(ESR_ERR_UNSUPPORTED, "face-slot width must be 3 or 4");
  if (m->dtype != ESR_F32 && m->dtype != ESR_F64) return esr::fail(ESR_ERR_UNSUPPORTED, "mesh dtype");
  if (!m->nbr || !m->sx || !m->sy || !m->alpha || !m->area) return esr::fail(ESR_ERR_ARG, "null mesh array");
  return ESR_OK;
}

template <typename T, int W>
int run_steps(const esr_swe_mesh *m, double dt, T *state, int64_t steps, T *ws, cudaStream_t st) {
  const int64_t nc = m->nc;
  const int grid = (int)((nc + kSweThreads - 1) / kSweThreads);
  T *S1 = ws;
  T *S2 = ws + 4 * nc;
  T *A = ws + 8 * nc;
  const int32_t *nbr = m->nbr;
  const T *sx = (const T *)m->sx, *sy = (const T *)m->sy, *al = (const T *)m->alpha, *ar = (const T *)m->area;
  // scalar constants exactly as the reference forms them in Python (double)
  // and as torch rounds a Python scalar into a tensor op of dtype T
  const T c1 = (T)(0.5 * dt);
  const T c3 = (T)dt;
  const T c4 = (T)(dt / 6);
  for (int64_t s = 0; s < steps; ++s) {
    swe_stage_kernel<T, W, 1><<<grid, kSweThreads, 0, st>>>(nc, nbr, sx, sy, al, ar, state, state, A, S1, c1);
    swe_stage_kernel<T, W, 2><<<grid, kSweThreads, 0, st>>>(nc, nbr, sx, sy, al, ar, S1, state, A, S2, c1);
    swe_stage_kernel<T, W, 3><<<grid, kSweThreads, 0, st>>>(nc, nbr, sx, sy, al, ar, S2, state, A, S1, c3);
    swe_stage_kernel<T, W, 4><<<grid, kSweThreads, 0, st>>>(nc, nbr, sx, sy, al, ar, S1, state, A, state, c4);
  }
  ESR_LAUNCH_CHECK("esr_swe_step");
  return ESR_OK;
}

template <typename T, int W>
int run_delta(const esr_swe_mesh *m, const T *s, T *d, cudaStream_t st) {
  const int64_t nc = m->nc;
  const int grid = (int)((nc + kSweThreads - 1) / kSweThreads);
  swe_delta_kernel<T, W><<<grid, kSweThreads, 0, st>>>(nc, m->nbr, (const T *)m->sx, (const T *)m->sy,
                                                       (const T *)m->alpha, (const T *)m->area, s, d);
  ESR_LAUNCH_CHECK("esr_swe_delta");
  return ESR_OK;
}

}  // namespace

ESR_DEFINE_STATUS_READER(esr_status_swe)

extern "C" int64_t esr_swe_workspace_bytes(const esr_swe_mesh *mesh) {
  if (check_mesh(mesh)) return -1;
  const int64_t es = mesh->dtype == ESR_F64 ? 8 : 4;
  return 3 * 4 * mesh->nc * es;
}

extern "C" int esr_swe_step(const esr_swe_mesh *mesh, double dt, void *state, int64_t steps, void *workspace,
                            void *stream) {
  int st = check_mesh(mesh);
  if (st) return st;
  if (steps < 0) return esr::fail(ESR_ERR_ARG, "negative step count");
  if (steps == 0) return ESR_OK;
  if (!state || !workspace) return esr::fail(ESR_ERR_ARG, "null state/workspace");
  if (((uintptr_t)state | (uintptr_t)workspace) % 32) return esr::fail(ESR_ERR_ARG, "state/workspace must be 32-byte aligned");
  cudaStream_t s = esr::as_stream(stream);
  if (mesh->dtype == ESR_F64) {
    if (mesh->width == 3) return run_steps<double, 3>(mesh, dt, (double *)state, steps, (double *)workspace, s);
    return run_steps<double, 4>(mesh, dt, (double *)state, steps, (double *)workspace, s);
  }
  if (mesh->width == 3) return run_steps<float, 3>(mesh, dt, (float *)state, steps, (float *)workspace, s);
  return run_steps<float, 4>(mesh, dt, (float *)state, steps, (float *)workspace, s);
}

extern "C" int esr_swe_delta(const esr_swe_mesh *mesh, const void *state, void *delta, void *stream) {
  int st = check_mesh(mesh);
  if (st) return st;
  if (!state || !delta) return esr::fail(ESR_ERR_ARG, "null state/delta");
  if (((uintptr_t)state | (uintptr_t)delta) % 32) return esr::fail(ESR_ERR_ARG, "state/delta must be 32-byte aligned");
  cudaStream_t s = esr::as_stream(stream);
  if (mesh->dtype == ESR_F64) {
    if (mesh->width == 3) return run_delta<double, 3>(mesh, (const double *)state, (double *)delta, s);
    return run_delta<double, 4>(mesh, (const double *)state, (double *)delta, s);
  }
  if (mesh->width == 3) return run_delta<float, 3>(mesh, (const float *)state, (float *)delta, s);
  return run_delta<float, 4>(mesh, (const float *)state, (float *)delta, s);
}
