// Fused shallow-water step: gather of neighbour state, face reconstruction,
// central flux, per-cell face sum, wall pressure term, division by area and
// the stage combination.
//
// Reference: tutorial/shallow_water_equation/swe_main.py
//   face_reconstruct  :83-85   phi_f = (1 - alpha) * phi[src] + alpha * phi[dst]
//   delta             :87-119  fluxes, scatter(dst), scatter_b(bcells), / area
//   forward           :121-141 stage states s + c*delta_k, s += dt/6 * sum_k
//
// Two kernels with the same per-cell arithmetic:
//   * swe_stage_kernel: one launch per stage (4 per step), stage states in
//     HBM.  Layout: state [nc][4] (h, uh, vh, 0); face slots [width][nc]
//     (nbr int32, sx, sy, alpha) slot-major; area [nc].
//   * swe_tile_step_kernel (FP32): one launch per step; a CTA keeps a tile
//     plus the 4 rings of in-neighbours in shared memory and recomputes the
//     halo's stage values instead of exchanging them through HBM.
// One thread owns one cell and walks its face slots in order: interior edges
// in the reference's edge order, then wall faces, so the per-cell sums are
// the reference's in-order Reducer sums.
//
// Arithmetic policy (template flag EXACT):
//   EXACT: every operation is one round-to-nearest IEEE op in the
//          reference's order (explicit _rn intrinsics: no FMA contraction,
//          IEEE division) -> bitwise the reference's CPU backend.
//   fast:  the same formulas with FMA contraction, one reciprocal of h_f per
//          face for u_f = uh_f/h_f and v_f = vh_f/h_f, and a multiply by a
//          precomputed 1/area (the tiled kernel: face records whose sx, sy
//          are already divided by the cell's area, the fluxes being linear
//          in them).
//
// Stages (c1 = 0.5*dt, c3 = dt, c4 = dt/6, rounded to T like torch does):
//   1: D1 = delta(s0);           S1 = s0 + c1*D1;  A = D1
//   2: D2 = delta(S1);           S2 = s0 + c1*D2;  A = A + D2
//   3: D3 = delta(S2);           S1 = s0 + c3*D3;  A = A + D3
//   4: D4 = delta(S1);           s0 = s0 + c4*(A + D4)
#include <algorithm>
#include <cstdint>
#include <vector>

#include "esr_internal.h"
#include "reduce_util.cuh"

namespace {

constexpr int kSweThreads = 256;

template <typename T, bool EXACT>
struct Ar;

template <typename T>
struct Ar<T, true> {
  using O = ops<T>;
  static __device__ __forceinline__ T mul(T a, T b) { return O::mul(a, b); }
  static __device__ __forceinline__ T add(T a, T b) { return O::add(a, b); }
  static __device__ __forceinline__ T sub(T a, T b) { return O::sub(a, b); }
  // a*b + c, two roundings
  static __device__ __forceinline__ T madd(T a, T b, T c) { return O::add(O::mul(a, b), c); }
  static __device__ __forceinline__ T recip(T) { return T(0); }
  static __device__ __forceinline__ T quot(T x, T y, T) { return O::div(x, y); }
};

template <>
struct Ar<float, false> {
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
  static __device__ __forceinline__ float madd(float a, float b, float c) { return fmaf(a, b, c); }
  // approximate reciprocal (one MUFU op, ~1 ulp; flushes subnormals)
  static __device__ __forceinline__ float recip(float y) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
    return r;
  }
  static __device__ __forceinline__ float quot(float x, float, float yinv) { return x * yinv; }
};

template <>
struct Ar<double, false> {
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double madd(double a, double b, double c) { return fma(a, b, c); }
  static __device__ __forceinline__ double recip(double y) { return 1.0 / y; }
  static __device__ __forceinline__ double quot(double x, double, double yinv) { return x * yinv; }
};

template <typename T>
struct Acc3 {
  T Sh, Su, Sv;  // scatter(...) over interior edges
  T Bu, Bv;      // scatter_b(...) over wall faces
};

// One interior face of a cell: flux terms of swe_main.py:87-117 added to the
// cell's sums.  own/nb = (h, uh, vh) of the destination (this cell) and the
// source (neighbour).
//   exact: the reference's operations in its order;
//   fast:  the same quantities regrouped, with F_h = uh_f sx + vh_f sy:
//          phi_f = phi_src + alpha (phi_dst - phi_src)
//          F_uh  = (uh_f / h_f) F_h + h_f^2 / 2 sx
//          F_vh  = (vh_f / h_f) F_h + h_f^2 / 2 sy
//          (u_f uh_f sx + u_f vh_f sy = u_f F_h), each term an FMA into the
//          sum, and the wall terms go straight into the same sums.
template <typename T, bool EXACT>
__device__ __forceinline__ void add_face(Acc3<T> &s, T oh, T ou, T ov, T nh, T nu, T nv, T a, T fx, T fy) {
  using A = Ar<T, EXACT>;
  if constexpr (!EXACT) {
    const T hf = A::madd(a, A::sub(oh, nh), nh);
    const T uhf = A::madd(a, A::sub(ou, nu), nu);
    const T vhf = A::madd(a, A::sub(ov, nv), nv);
    const T Fh = A::madd(uhf, fx, A::mul(vhf, fy));
    const T Fi = A::mul(Fh, A::recip(hf));
    const T hfs = A::mul(A::mul(T(0.5), hf), hf);
    s.Sh = A::add(s.Sh, Fh);
    s.Su = A::madd(uhf, Fi, A::madd(hfs, fx, s.Su));
    s.Sv = A::madd(vhf, Fi, A::madd(hfs, fy, s.Sv));
    return;
  }
  const T half = T(0.5);
  const T om = A::sub(T(1), a);
  const T hf = A::madd(om, nh, A::mul(a, oh));   // (1 - alpha)*h[src] + alpha*h[dst]
  const T uhf = A::madd(om, nu, A::mul(a, ou));
  const T vhf = A::madd(om, nv, A::mul(a, ov));
  const T ih = A::recip(hf);
  const T uf = A::quot(uhf, hf, ih);
  const T vf = A::quot(vhf, hf, ih);
  const T hfs = A::mul(A::mul(half, hf), hf);    // 0.5 * h_f * h_f
  const T uhsx = A::mul(uhf, fx);                // uh_f * sx
  const T vhsy = A::mul(vhf, fy);                // vh_f * sy
  const T Fh = A::add(uhsx, vhsy);
  const T Fu = A::madd(A::madd(uf, uhf, hfs), fx, A::mul(uf, vhsy));
  const T Fv = A::madd(vf, uhsx, A::mul(A::madd(vf, vhf, hfs), fy));
  s.Sh = A::add(s.Sh, Fh);
  s.Su = A::add(s.Su, Fu);
  s.Sv = A::add(s.Sv, Fv);
}

// A wall face: 0.5 * gather_b(h)**2 * (bsx, bsy)
template <typename T, bool EXACT>
__device__ __forceinline__ void add_wall(Acc3<T> &s, T oh, T fx, T fy) {
  using A = Ar<T, EXACT>;
  const T gb = A::mul(T(0.5), A::mul(oh, oh));
  if constexpr (EXACT) {
    s.Bu = A::madd(gb, fx, s.Bu);
    s.Bv = A::madd(gb, fy, s.Bv);
  } else {
    s.Su = A::madd(gb, fx, s.Su);
    s.Sv = A::madd(gb, fy, s.Sv);
  }
}

// delta = -(sums) / area
template <typename T, bool EXACT>
__device__ __forceinline__ void finish(const Acc3<T> &s, T ar, T iar, T &dh, T &du, T &dv) {
  using A = Ar<T, EXACT>;
  dh = A::quot(-s.Sh, ar, iar);
  if constexpr (EXACT) {
    du = A::quot(-A::add(s.Su, s.Bu), ar, iar);
    dv = A::quot(-A::add(s.Sv, s.Bv), ar, iar);
  } else {  // wall terms are in Su, Sv
    du = A::quot(-s.Su, ar, iar);
    dv = A::quot(-s.Sv, ar, iar);
  }
}

// ----------------------------------------------------------- staged --
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

template <typename T>
struct SlotsG {  // face slots in global memory, [width][nc]
  const int32_t *nbr;
  const T *sx, *sy, *alpha, *area, *inv_area;
};

// delta (swe_main.py:87-119) of cell i given the stage state `s`.
template <typename T, int W, bool EXACT>
__device__ __forceinline__ Vec4<T> cell_delta(int64_t i, int64_t nc, const SlotsG<T> &g, const T *s,
                                              const Vec4<T> own) {
  Acc3<T> acc{T(0), T(0), T(0), T(0), T(0)};
#pragma unroll
  for (int k = 0; k < W; ++k) {
    const int32_t j = __ldg(g.nbr + k * nc + i);
    if (j >= 0) {
      if ((int64_t)j >= nc) {  // corrupt slot: flag it, never read out of bounds
        esr::raise_status(ESR_DEV_IDX_RANGE);
        continue;
      }
      const Vec4<T> nb = load4(s + 4 * (int64_t)j);
      add_face<T, EXACT>(acc, own.x, own.y, own.z, nb.x, nb.y, nb.z, __ldg(g.alpha + k * nc + i),
                         __ldg(g.sx + k * nc + i), __ldg(g.sy + k * nc + i));
    } else if (j == -1) {
      add_wall<T, EXACT>(acc, own.x, __ldg(g.sx + k * nc + i), __ldg(g.sy + k * nc + i));
    }
  }
  Vec4<T> d;
  finish<T, EXACT>(acc, __ldg(g.area + i), EXACT ? T(0) : __ldg(g.inv_area + i), d.x, d.y, d.z);
  d.w = T(0);
  return d;
}

template <typename T, int W, int STAGE, bool EXACT>
__global__ void __launch_bounds__(kSweThreads)
swe_stage_kernel(int64_t nc, SlotsG<T> g, const T *__restrict__ sin, const T *s0, T *__restrict__ acc, T *sout,
                 T c) {
  using A = Ar<T, EXACT>;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const Vec4<T> own_in = load4(sin + 4 * i);
  const Vec4<T> d = cell_delta<T, W, EXACT>(i, nc, g, sin, own_in);
  const Vec4<T> base = (STAGE == 1) ? own_in : load4(s0 + 4 * i);
  Vec4<T> out;
  if (STAGE < 4) {
    out.x = A::madd(c, d.x, base.x);
    out.y = A::madd(c, d.y, base.y);
    out.z = A::madd(c, d.z, base.z);
    out.w = T(0);
    Vec4<T> a;
    if (STAGE == 1) {
      a = d;
    } else {
      const Vec4<T> prev = load4(acc + 4 * i);
      a.x = A::add(prev.x, d.x);
      a.y = A::add(prev.y, d.y);
      a.z = A::add(prev.z, d.z);
      a.w = T(0);
    }
    store4(acc + 4 * i, a);
  } else {
    const Vec4<T> prev = load4(acc + 4 * i);
    out.x = A::madd(c, A::add(prev.x, d.x), base.x);
    out.y = A::madd(c, A::add(prev.y, d.y), base.y);
    out.z = A::madd(c, A::add(prev.z, d.z), base.z);
    out.w = base.w;
  }
  store4(sout + 4 * i, out);
}

template <typename T, int W, bool EXACT>
__global__ void __launch_bounds__(kSweThreads)
swe_delta_kernel(int64_t nc, SlotsG<T> g, const T *__restrict__ s, T *__restrict__ dout) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const Vec4<T> own = load4(s + 4 * i);
  store4(dout + 4 * i, cell_delta<T, W, EXACT>(i, nc, g, s, own));
}

int check_mesh(const esr_swe_mesh *m) {
  if (!m) return esr::fail(ESR_ERR_ARG, "null mesh");
  if (m->nc <= 0) return esr::fail(ESR_ERR_ARG, "mesh has no cells");
  if (m->nc > ((int64_t)1 << 31) - 1) return esr::fail(ESR_ERR_UNSUPPORTED, "more than 2^31-1 cells");
  if (m->width != 3 && m->width != 4) return esr::fail(ESR_ERR_UNSUPPORTED, "face-slot width must be 3 or 4");
  if (m->dtype != ESR_F32 && m->dtype != ESR_F64) return esr::fail(ESR_ERR_UNSUPPORTED, "mesh dtype");
  if (!m->nbr || !m->sx || !m->sy || !m->alpha || !m->area) return esr::fail(ESR_ERR_ARG, "null mesh array");
  if (!m->exact && !m->inv_area) return esr::fail(ESR_ERR_ARG, "fast arithmetic needs inv_area");
  return ESR_OK;
}

template <typename T>
SlotsG<T> slots_of(const esr_swe_mesh *m) {
  return SlotsG<T>{m->nbr, (const T *)m->sx, (const T *)m->sy, (const T *)m->alpha, (const T *)m->area,
                   (const T *)m->inv_area};
}

template <typename T, int W, bool EXACT>
int run_steps(const esr_swe_mesh *m, double dt, T *state, int64_t steps, T *ws, cudaStream_t st) {
  const int64_t nc = m->nc;
  const int grid = (int)((nc + kSweThreads - 1) / kSweThreads);
  T *S1 = ws;
  T *S2 = ws + 4 * nc;
  T *A = ws + 8 * nc;
  const SlotsG<T> g = slots_of<T>(m);
  // scalar constants exactly as the reference forms them in Python (double)
  // and as torch rounds a Python scalar into a tensor op of dtype T
  const T c1 = (T)(0.5 * dt);
  const T c3 = (T)dt;
  const T c4 = (T)(dt / 6);
  for (int64_t s = 0; s < steps; ++s) {
    swe_stage_kernel<T, W, 1, EXACT><<<grid, kSweThreads, 0, st>>>(nc, g, state, state, A, S1, c1);
    swe_stage_kernel<T, W, 2, EXACT><<<grid, kSweThreads, 0, st>>>(nc, g, S1, state, A, S2, c1);
    swe_stage_kernel<T, W, 3, EXACT><<<grid, kSweThreads, 0, st>>>(nc, g, S2, state, A, S1, c3);
    swe_stage_kernel<T, W, 4, EXACT><<<grid, kSweThreads, 0, st>>>(nc, g, S1, state, A, state, c4);
  }
  ESR_LAUNCH_CHECK("esr_swe_step");
  return ESR_OK;
}

template <typename T, int W, bool EXACT>
int run_delta(const esr_swe_mesh *m, const T *s, T *d, cudaStream_t st) {
  const int64_t nc = m->nc;
  const int grid = (int)((nc + kSweThreads - 1) / kSweThreads);
  swe_delta_kernel<T, W, EXACT><<<grid, kSweThreads, 0, st>>>(nc, slots_of<T>(m), s, d);
  ESR_LAUNCH_CHECK("esr_swe_delta");
  return ESR_OK;
}

template <typename T, bool EXACT>
int dispatch_steps(const esr_swe_mesh *m, double dt, void *state, int64_t steps, void *ws, cudaStream_t s) {
  if (m->width == 3) return run_steps<T, 3, EXACT>(m, dt, (T *)state, steps, (T *)ws, s);
  return run_steps<T, 4, EXACT>(m, dt, (T *)state, steps, (T *)ws, s);
}

template <typename T, bool EXACT>
int dispatch_delta(const esr_swe_mesh *m, const void *state, void *delta, cudaStream_t s) {
  if (m->width == 3) return run_delta<T, 3, EXACT>(m, (const T *)state, (T *)delta, s);
  return run_delta<T, 4, EXACT>(m, (const T *)state, (T *)delta, s);
}

// ------------------------------------------------ temporally blocked step --
// One launch per step.  Cells are grouped in compact tiles; a CTA loads its
// tile plus the 4 rings of in-neighbours around it into shared memory and
// runs all 4 stages there:
//   stage 1 on cells of level <= 3 (reads s0 of levels <= 4)
//   stage 2 on levels <= 2, stage 3 on levels <= 1, stage 4 on the tile.
// In exact arithmetic every cell value is computed with the operations of
// swe_stage_kernel, so the result is bitwise the same; in fast arithmetic
// the face records carry sx/area, sy/area and a cell's faces are summed in
// neighbour order (within rounding of the staged fast step).  HBM traffic
// per step is the tile's geometry (plus the halo's), s0 of tile + halo, and
// the new state; the stage states never leave the SM.
// The CTA size TT is 1024, 512 or 256 threads with 1024 / TT CTAs per SM
// (64 registers a thread either way): the largest tiles use one CTA per SM,
// tiles of half or a quarter the size run two or four CTAs per SM, so one
// CTA's state loads and barriers overlap another's compute.
constexpr int kTileIters = 6;     // cells of level <= 3 per thread: <= 6 * TT
constexpr int kTileOwnIters = 4;  // tile cells per thread: <= 4 * TT
constexpr int kTileGroup = 2;     // cells whose geometry loads are issued together
constexpr int kTileMaxThreads = 1024;

struct SlotsT {  // one tile's face slots, [3][n3] records {sx, sy, alpha, lnbr}
  const float4 *slot;
  const float *area;  // exact arithmetic only (fast: sx, sy hold sx/area, sy/area)
  int n3, nL;
};

// geometry of one tile cell's three face slots
struct CellGeom {
  int32_t nb[3];
  float al[3], sx[3], sy[3];
  float area;
};

// The cell's geometry: three 16-byte face records (and, exact, its area),
// all loads issued together.
template <bool EXACT>
__device__ __forceinline__ void load_geom(int j, const SlotsT &g, CellGeom &c) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 f = __ldg(g.slot + k * g.n3 + j);
    c.sx[k] = f.x;
    c.sy[k] = f.y;
    c.al[k] = f.z;
    c.nb[k] = __float_as_int(f.w);
  }
  c.area = EXACT ? __ldg(g.area + j) : 1.f;
}

// Stage state of a tile in shared memory.  Fast arithmetic: (h, uh) pairs
// and vh, so a neighbour's state is two loads; exact: h, uh, vh arrays (the
// paired layout costs the exact kernel registers and spills).
template <bool EXACT>
struct TileState;

template <>
struct TileState<false> {
  float2 *hu;
  float *v;
  // the layout's arrays over a shared buffer of `cells` entries at `base`
  static __device__ __forceinline__ TileState at(float *smem, int total, int base) {
    return TileState{reinterpret_cast<float2 *>(smem) + base, smem + 2 * total + base};
  }
  __device__ __forceinline__ void load(int j, float &h, float &u, float &w) const {
    const float2 a = hu[j];
    h = a.x;
    u = a.y;
    w = v[j];
  }
  __device__ __forceinline__ void store(int j, float h, float u, float w) const {
    hu[j] = make_float2(h, u);
    v[j] = w;
  }
};

template <>
struct TileState<true> {
  float *h, *u, *v;
  static __device__ __forceinline__ TileState at(float *smem, int total, int base) {
    return TileState{smem + base, smem + total + base, smem + 2 * total + base};
  }
  __device__ __forceinline__ void load(int j, float &a, float &b, float &c) const {
    a = h[j];
    b = u[j];
    c = v[j];
  }
  __device__ __forceinline__ void store(int j, float a, float b, float c) const {
    h[j] = a;
    u[j] = b;
    v[j] = c;
  }
};

template <bool EXACT>
__device__ __forceinline__ void tile_delta(int j, const CellGeom &c, int nL, const TileState<EXACT> &s, float &dh,
                                           float &du, float &dv) {
  float oh, ou, ov;
  s.load(j, oh, ou, ov);
  Acc3<float> acc{0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int32_t q = c.nb[k];
    if ((uint32_t)q < (uint32_t)nL) {  // one compare: 0 <= q < nL
      float nh, nu, nv;
      s.load(q, nh, nu, nv);
      add_face<float, EXACT>(acc, oh, ou, ov, nh, nu, nv, c.al[k], c.sx[k], c.sy[k]);
    } else if (q == -1) {
      add_wall<float, EXACT>(acc, oh, c.sx[k], c.sy[k]);
    } else if (q >= 0) {  // corrupt layout: flag, never read outside the tile's list
      esr::raise_status(ESR_DEV_IDX_RANGE);
    }
  }
  if (EXACT) {
    finish<float, true>(acc, c.area, 0.f, dh, du, dv);
  } else {  // the area is in the records, the wall terms in Su, Sv
    dh = -acc.Sh;
    du = -acc.Su;
    dv = -acc.Sv;
  }
}

template <int STAGE, bool EXACT>
__device__ __forceinline__ void tile_cell(int r, int j, int n0, const CellGeom &cg, int nL,
                                          const TileState<EXACT> &in, const TileState<EXACT> &s0,
                                          const TileState<EXACT> &out,
                                          float (&acc)[kTileOwnIters][3], float c, float4 *sout, int64_t cell_off) {
  using A = Ar<float, EXACT>;
  float dh, du, dv;
  tile_delta<EXACT>(j, cg, nL, in, dh, du, dv);
  float h0, u0, v0;
  s0.load(j, h0, u0, v0);
  if (STAGE < 4) {
    out.store(j, A::madd(c, dh, h0), A::madd(c, du, u0), A::madd(c, dv, v0));
    if (r < kTileOwnIters && j < n0) {
      if (STAGE == 1) {
        acc[r][0] = dh;
        acc[r][1] = du;
        acc[r][2] = dv;
      } else {
        acc[r][0] = A::add(acc[r][0], dh);
        acc[r][1] = A::add(acc[r][1], du);
        acc[r][2] = A::add(acc[r][2], dv);
      }
    }
  } else if (r < kTileOwnIters) {
    float4 o;
    o.x = A::madd(c, A::add(acc[r][0], dh), h0);
    o.y = A::madd(c, A::add(acc[r][1], du), u0);
    o.z = A::madd(c, A::add(acc[r][2], dv), v0);
    o.w = 0.f;
    sout[cell_off + j] = o;
  }
}

// Cells j = tid + r * TT in groups of kTileGroup consecutive r:
// the geometry of the whole group is requested before any of its cells is
// computed, so the group's loads are in flight together (the kernel is
// latency-bound on these L1/L2 loads otherwise).
template <int TT, int STAGE, bool EXACT>
__device__ __forceinline__ void tile_stage(int count, int n0, const SlotsT &g, const TileState<EXACT> &in,
                                           const TileState<EXACT> &s0, const TileState<EXACT> &out,
                                           float (&acc)[kTileOwnIters][3], float c, float4 *sout, int64_t cell_off) {
  constexpr int kIters = STAGE == 4 ? kTileOwnIters : kTileIters;
#pragma unroll
  for (int r0 = 0; r0 < kIters; r0 += kTileGroup) {
    CellGeom cg[kTileGroup];
#pragma unroll
    for (int u = 0; u < kTileGroup; ++u) {
      const int j = threadIdx.x + (r0 + u) * TT;
      if (r0 + u < kIters && j < count) load_geom<EXACT>(j, g, cg[u]);
    }
#pragma unroll
    for (int u = 0; u < kTileGroup; ++u) {
      const int j = threadIdx.x + (r0 + u) * TT;
      if (r0 + u < kIters && j < count)
        tile_cell<STAGE, EXACT>(r0 + u, j, n0, cg[u], g.nL, in, s0, out, acc, c, sout, cell_off);
    }
  }
}

template <bool EXACT, int TT>
__global__ void __launch_bounds__(TT, kTileMaxThreads / TT)
swe_tile_step_kernel(const int32_t *__restrict__ meta, const int64_t *__restrict__ off3,
                     const int64_t *__restrict__ offh, const int32_t *__restrict__ halo,
                     const float4 *__restrict__ gslot, const float *__restrict__ garea, const float4 *__restrict__ sin,
                     float4 *__restrict__ sout, int64_t nc, int max_local, int max_l3, float c1, float c3,
                     float c4) {
  extern __shared__ float smem[];
  const int t = blockIdx.x;
  const int32_t *mt = meta + 8 * (int64_t)t;
  const int cell_off = mt[0], n0 = mt[1], n1 = mt[2], n2 = mt[3], n3 = mt[4], nL = mt[5];
  // s0 of the local list, then the two stage buffers of the level-<=3 cells
  const int total = max_local + 2 * max_l3;
  using TS = TileState<EXACT>;
  const TS S0 = TS::at(smem, total, 0), SA = TS::at(smem, total, max_local),
           SB = TS::at(smem, total, max_local + max_l3);
  const int64_t hb = offh[t];
  for (int j = threadIdx.x; j < nL; j += TT) {
    const int64_t gcell = j < n0 ? (int64_t)cell_off + j : (int64_t)__ldg(halo + hb + (j - n0));
    if (gcell < 0 || gcell >= nc) {  // corrupt layout: flag, never read out of bounds
      esr::raise_status(ESR_DEV_IDX_RANGE);
      S0.store(j, 1.f, 0.f, 0.f);
      continue;
    }
    const float4 s = sin[gcell];
    S0.store(j, s.x, s.y, s.z);
  }
  __syncthreads();
  const int64_t o3 = off3[t];
  const SlotsT g{gslot + 3 * o3, EXACT ? garea + o3 : nullptr, n3, nL};
  float acc[kTileOwnIters][3];
#pragma unroll
  for (int r = 0; r < kTileOwnIters; ++r) acc[r][0] = acc[r][1] = acc[r][2] = 0.f;
  tile_stage<TT, 1, EXACT>(n3, n0, g, S0, S0, SA, acc, c1, sout, cell_off);
  __syncthreads();
  tile_stage<TT, 2, EXACT>(n2, n0, g, SA, S0, SB, acc, c1, sout, cell_off);
  __syncthreads();
  tile_stage<TT, 3, EXACT>(n1, n0, g, SB, S0, SA, acc, c3, sout, cell_off);
  __syncthreads();
  tile_stage<TT, 4, EXACT>(n0, n0, g, SA, S0, SA, acc, c4, sout, cell_off);
}

int64_t tile_smem_bytes(const esr_swe_tiles *T) {
  return (int64_t)(3 * (int64_t)T->max_local + 6 * (int64_t)T->max_l3) * (int64_t)sizeof(float);
}
// (3 floats a cell; the paired layout puts its float2 array first, so it is
// 8-byte aligned at any max_local, max_l3)

int check_tiles(const esr_swe_tiles *T) {
  if (!T) return esr::fail(ESR_ERR_ARG, "null tile layout");
  if (T->dtype != ESR_F32) return esr::fail(ESR_ERR_UNSUPPORTED, "tiled step is FP32 only");
  if (T->nc <= 0 || T->ntiles <= 0) return esr::fail(ESR_ERR_ARG, "empty tile layout");
  if (T->max_own > kTileOwnIters * kTileMaxThreads)
    return esr::fail(ESR_ERR_UNSUPPORTED, "a tile has more than 4096 cells");
  if (T->max_l3 > kTileIters * kTileMaxThreads)
    return esr::fail(ESR_ERR_UNSUPPORTED, "a tile plus 3 halo rings has more than 6144 cells");
  if (T->max_local < T->max_l3 || T->max_l3 < T->max_own) return esr::fail(ESR_ERR_ARG, "inconsistent tile maxima");
  if (tile_smem_bytes(T) > 227 * 1024) return esr::fail(ESR_ERR_UNSUPPORTED, "tile needs more than 227 KB shared memory");
  if (!T->meta || !T->off3 || !T->offh || !T->slots || !T->area) return esr::fail(ESR_ERR_ARG, "null tile array");
  if (reinterpret_cast<uintptr_t>(T->slots) % 16 != 0) return esr::fail(ESR_ERR_ARG, "slots must be 16-byte aligned");
  return ESR_OK;
}

// CTA size for a tile layout: the smallest that holds the largest tile
// (4 own cells and 6 level-<=3 cells a thread) and whose 1024 / TT CTAs fit
// one SM's shared memory together (228 KB, 1 KB of it reserved per CTA).
int tile_threads(const esr_swe_tiles *T) {
  const int64_t smem = tile_smem_bytes(T);
  for (int tt = 256; tt < kTileMaxThreads; tt *= 2) {
    const int64_t ctas = kTileMaxThreads / tt;
    if (T->max_own <= kTileOwnIters * tt && T->max_l3 <= kTileIters * tt && ctas * (smem + 1024) <= 228 * 1024)
      return tt;
  }
  return kTileMaxThreads;
}

template <bool EXACT, int TT>
int run_tiles_tt(const esr_swe_tiles *tiles, double dt, void *state_a, void *state_b, int64_t steps,
                 cudaStream_t s) {
  const int64_t smem = tile_smem_bytes(tiles);
  cudaError_t e = cudaFuncSetAttribute(swe_tile_step_kernel<EXACT, TT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_tile_step/smem attribute");
  const float c1 = (float)(0.5 * dt), c3 = (float)dt, c4 = (float)(dt / 6);
  float4 *buf[2] = {(float4 *)state_a, (float4 *)state_b};
  for (int64_t k = 0; k < steps; ++k) {
    swe_tile_step_kernel<EXACT, TT><<<tiles->ntiles, TT, smem, s>>>(
        tiles->meta, tiles->off3, tiles->offh, tiles->halo, (const float4 *)tiles->slots,
        (const float *)tiles->area, buf[k & 1], buf[(k + 1) & 1], tiles->nc,
        tiles->max_local, tiles->max_l3, c1, c3, c4);
  }
  ESR_LAUNCH_CHECK("esr_swe_tile_step");
  return ESR_OK;
}

template <bool EXACT>
int run_tiles(const esr_swe_tiles *tiles, double dt, void *state_a, void *state_b, int64_t steps, cudaStream_t s) {
  switch (tile_threads(tiles)) {
    case 256: return run_tiles_tt<EXACT, 256>(tiles, dt, state_a, state_b, steps, s);
    case 512: return run_tiles_tt<EXACT, 512>(tiles, dt, state_a, state_b, steps, s);
    default: return run_tiles_tt<EXACT, 1024>(tiles, dt, state_a, state_b, steps, s);
  }
}

// ------------------------------------- pipelined tile step (fast FP32) --
// Same tiles, same arithmetic and order as swe_tile_step_kernel<fast>, so
// the result is bitwise the same; organised for GB300's latency and issue
// limits instead of one CTA per tile:
//   * persistent: one CTA per SM walks tiles t, t + grid, ...;
//   * thread x of a TT-thread CTA computes the local cells j = x + r*TT,
//     r < CELLS, whatever their level (tile cells first, then the halo of
//     levels 1..3), as CELLS/2 pairs: every thread has the same number of
//     cells in a stage, so no warp waits at the stage barriers for another
//     one's extra halo cell;
//   * the face records of those cells are loaded into registers once per
//     step and kept through the four stages (the stages touch shared memory
//     only); local cells past CELLS*TT (large halos) read theirs per stage;
//   * the next tile's state (own cells and halo) is copied into a second
//     shared-memory buffer with cp.async while this tile computes, and its
//     face records are prefetched into L2 with one bulk prefetch;
//   * the two cells of a pair are computed in lock step with the packed
//     FP32x2 instructions (__ffma2_rn, __fadd2_rn, __fmul2_rn: per lane the
//     IEEE operations of the scalar kernel), halving the FP instructions;
//   * stage states live in shared memory as three float arrays (h, uh, vh)
//     at fixed offsets, so a neighbour's state is three 4-byte loads from
//     one address register.
namespace pipe {
constexpr int kMaxLocal = 4096;             // nL
constexpr int kBuf = 3 * kMaxLocal;         // floats of one (h, uh, vh) buffer
constexpr int kSmemBytes = 4 * kBuf * 4;    // S0 x 2, SA, SB: 192 KB
static_assert(kSmemBytes <= 227 * 1024, "shared memory of one CTA");

struct Geo {  // one cell's three faces
  float sx[3], sy[3], al[3];
  int nb[3];
};

__device__ __forceinline__ void load_geo(const float4 *slot, int n3, int j, bool valid, Geo &g) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (valid) {
      const float4 f = __ldg(slot + k * n3 + j);
      g.sx[k] = f.x;
      g.sy[k] = f.y;
      g.al[k] = f.z;
      g.nb[k] = __float_as_int(f.w);
    } else {
      g.sx[k] = g.sy[k] = g.al[k] = 0.f;
      g.nb[k] = -2;
    }
  }
}

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
// a - b with one rounding (the product -1 * b is exact)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f, -1.f), a); }
__device__ __forceinline__ float rcpf(float y) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
  return r;
}

// (h, uh, vh) arrays of one buffer at fixed offsets
struct Buf {
  float *p;
  __device__ __forceinline__ float h(int j) const { return p[j]; }
  __device__ __forceinline__ float u(int j) const { return p[kMaxLocal + j]; }
  __device__ __forceinline__ float v(int j) const { return p[2 * kMaxLocal + j]; }
  __device__ __forceinline__ void put(int j, float a, float b, float c) const {
    p[j] = a;
    p[kMaxLocal + j] = b;
    p[2 * kMaxLocal + j] = c;
  }
};

// One face of one cell, scalar (swe_tile_step_kernel's fast add_face / add_wall).
__device__ __forceinline__ void face1(float &Sh, float &Su, float &Sv, float oh, float ou, float ov, const Buf &in,
                                      int q, int nL, float a, float fx, float fy) {
  if ((unsigned)q < (unsigned)nL) {
    const float nh = in.h(q), nu = in.u(q), nv = in.v(q);
    const float hf = fmaf(a, oh - nh, nh);
    const float uhf = fmaf(a, ou - nu, nu);
    const float vhf = fmaf(a, ov - nv, nv);
    const float Fh = fmaf(uhf, fx, vhf * fy);
    const float Fi = Fh * rcpf(hf);
    const float hfs = (0.5f * hf) * hf;
    Sh = Sh + Fh;
    Su = fmaf(uhf, Fi, fmaf(hfs, fx, Su));
    Sv = fmaf(vhf, Fi, fmaf(hfs, fy, Sv));
  } else if (q == -1) {
    const float gb = 0.5f * (oh * oh);
    Su = fmaf(gb, fx, Su);
    Sv = fmaf(gb, fy, Sv);
  } else if (q >= 0) {  // corrupt layout: flag, never read outside the tile's list
    esr::raise_status(ESR_DEV_IDX_RANGE);
  }
}

// Face records of two cells A, B, held as the lanes of float2 values so the
// packed arithmetic takes them without re-pairing registers in every stage.
struct GeoPair {
  float2 sx[3], sy[3], al[3];
  int nbA[3], nbB[3];
};

// Slots 1 and 2 of a cell are interior faces (the layout's slot_info
// promise; walls and empty slots sort into slot 0): a cell past the tile's
// end gets faces there that contribute nothing (neighbour 0, zero normal),
// and a slot that breaks the promise is flagged and gets the same.
__device__ __forceinline__ void interior_slots(Geo &g, int nL, bool valid) {
#pragma unroll
  for (int k = 1; k < 3; ++k) {
    if ((unsigned)g.nb[k] >= (unsigned)nL) {
      if (valid) esr::raise_status(ESR_DEV_IDX_RANGE);
      g.nb[k] = 0;
      g.sx[k] = g.sy[k] = g.al[k] = 0.f;
    }
  }
}

__device__ __forceinline__ void load_pair(const float4 *slot, int n3, int nL, int jA, bool vA, int jB, bool vB,
                                          GeoPair &g) {
  Geo a, b;
  load_geo(slot, n3, jA, vA, a);
  load_geo(slot, n3, jB, vB, b);
  interior_slots(a, nL, vA);
  interior_slots(b, nL, vB);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    g.sx[k] = f2(a.sx[k], b.sx[k]);
    g.sy[k] = f2(a.sy[k], b.sy[k]);
    g.al[k] = f2(a.al[k], b.al[k]);
    g.nbA[k] = a.nb[k];
    g.nbB[k] = b.nb[k];
  }
}

// one interior face of two cells A, B (the lanes of every float2)
__device__ __forceinline__ void face2(float2 &Sh, float2 &Su, float2 &Sv, float2 oh, float2 ou, float2 ov,
                                      const Buf &in, int qA, int qB, float2 a, float2 fx, float2 fy) {
  const float2 nh = f2(in.h(qA), in.h(qB));
  const float2 nu = f2(in.u(qA), in.u(qB));
  const float2 nv = f2(in.v(qA), in.v(qB));
  const float2 hf = fma2(a, sub2(oh, nh), nh);
  const float2 uhf = fma2(a, sub2(ou, nu), nu);
  const float2 vhf = fma2(a, sub2(ov, nv), nv);
  const float2 Fh = fma2(uhf, fx, mul2(vhf, fy));
  const float2 Fi = mul2(Fh, f2(rcpf(hf.x), rcpf(hf.y)));
  const float2 hfs = mul2(mul2(f2(0.5f, 0.5f), hf), hf);
  Sh = add2(Sh, Fh);
  Su = fma2(uhf, Fi, fma2(hfs, fx, Su));
  Sv = fma2(vhf, Fi, fma2(hfs, fy, Sv));
}

// The face sums S of two cells A, B from buffer `in` (delta = -S; the
// callers fold the sign into their coefficients, which is exact).  Slot 0
// may be a wall or empty; slots 1 and 2 are interior (interior_slots).
__device__ __forceinline__ void sums2(const GeoPair &g, float2 oh, float2 ou, float2 ov, const Buf &in, int nL,
                                      float2 &Sh, float2 &Su, float2 &Sv) {
  Sh = f2(0.f, 0.f);
  Su = f2(0.f, 0.f);
  Sv = f2(0.f, 0.f);
  const int qA = g.nbA[0], qB = g.nbB[0];
  if (((unsigned)qA < (unsigned)nL) & ((unsigned)qB < (unsigned)nL)) {
    face2(Sh, Su, Sv, oh, ou, ov, in, qA, qB, g.al[0], g.sx[0], g.sy[0]);
  } else {
    face1(Sh.x, Su.x, Sv.x, oh.x, ou.x, ov.x, in, qA, nL, g.al[0].x, g.sx[0].x, g.sy[0].x);
    face1(Sh.y, Su.y, Sv.y, oh.y, ou.y, ov.y, in, qB, nL, g.al[0].y, g.sx[0].y, g.sy[0].y);
  }
#pragma unroll
  for (int k = 1; k < 3; ++k) face2(Sh, Su, Sv, oh, ou, ov, in, g.nbA[k], g.nbB[k], g.al[k], g.sx[k], g.sy[k]);
}

// 4-byte cp.async global -> shared
__device__ __forceinline__ void cp4(float *dst, const float *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// state (h, uh, vh) of global cell g into buffer slot j
__device__ __forceinline__ void fetch_state(const Buf &b, int j, const float4 *sin, int64_t g) {
  const float *s = reinterpret_cast<const float *>(sin + g);
  cp4(b.p + j, s);
  cp4(b.p + kMaxLocal + j, s + 1);
  cp4(b.p + 2 * kMaxLocal + j, s + 2);
}

struct TileMeta {
  int cell_off, n0, n1, n2, n3, nL;
  int64_t o3, oh;
};

__device__ __forceinline__ TileMeta tile_meta(const int32_t *meta, const int64_t *off3, const int64_t *offh, int t) {
  const int32_t *m = meta + 8 * (int64_t)t;
  return TileMeta{m[0], m[1], m[2], m[3], m[4], m[5], off3[t], offh[t]};
}

__device__ __forceinline__ bool tile_fits(const TileMeta &m, int64_t nc, int max_own) {
  return m.cell_off >= 0 && (int64_t)m.cell_off + m.n0 <= nc && m.n0 >= 0 && m.n0 <= max_own &&
         m.nL <= kMaxLocal && m.n0 <= m.n1 && m.n1 <= m.n2 && m.n2 <= m.n3 && m.n3 <= m.nL;
}

// the own cells' state of tile m into buffer b (cp.async); the halo part
// needs its indices first (fetch_halo)
template <int TT>
__device__ __forceinline__ void fetch_own(const Buf &b, const TileMeta &m, const float4 *sin) {
  for (int j = threadIdx.x; j < m.n0; j += TT) fetch_state(b, j, sin, (int64_t)m.cell_off + j);
}

__device__ __forceinline__ void fetch_halo1(const Buf &b, int j, const float4 *sin, int64_t nc, int g) {
  if (g < 0 || (int64_t)g >= nc) {  // corrupt layout: flag, never read out of bounds
    esr::raise_status(ESR_DEV_IDX_RANGE);
    b.put(j, 1.f, 0.f, 0.f);
  } else {
    fetch_state(b, j, sin, g);
  }
}

// the halo's state: the first two cells of this thread from the indices
// halo_index() loaded earlier, any further ones (large halos) index and copy
// here
template <int TT>
__device__ __forceinline__ void fetch_halo(const Buf &b, const TileMeta &m, const float4 *sin, int64_t nc,
                                           const int32_t *halo, const int (&hidx)[2]) {
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int j = m.n0 + threadIdx.x + r * TT;
    if (j < m.nL) fetch_halo1(b, j, sin, nc, hidx[r]);
  }
  for (int j = m.n0 + threadIdx.x + 2 * TT; j < m.nL; j += TT)
    fetch_halo1(b, j, sin, nc, __ldg(halo + m.oh + (j - m.n0)));
}

template <int TT>
__device__ __forceinline__ void halo_index(const TileMeta &m, const int32_t *halo, int (&hidx)[2]) {
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int j = m.n0 + threadIdx.x + r * TT;
    hidx[r] = j < m.nL ? __ldg(halo + m.oh + (j - m.n0)) : -1;
  }
}

// records of the local cells x + r*TT, r < CELLS, of level <= 3
template <int TT, int CELLS>
__device__ __forceinline__ void load_tile_geo(const TileMeta &m, const float4 *gslot, GeoPair (&gp)[CELLS / 2]) {
  const float4 *slot = gslot + 3 * m.o3;
#pragma unroll
  for (int p = 0; p < CELLS / 2; ++p) {
    const int jA = threadIdx.x + 2 * p * TT, jB = jA + TT;
    load_pair(slot, m.n3, m.nL, jA, jA < m.n3, jB, jB < m.n3, gp[p]);
  }
}

// a local cell past CELLS*TT (a large halo): its records from global memory
// (L1 / L2), scalar
template <int STAGE>
__device__ __forceinline__ void extra_cell(int j, const TileMeta &m, const float4 *gslot, const Buf &in,
                                           const Buf &s0, const Buf &out, float c) {
  Geo g;
  load_geo(gslot + 3 * m.o3, m.n3, j, true, g);
  const float oh = in.h(j), ou = in.u(j), ov = in.v(j);
  float Sh = 0.f, Su = 0.f, Sv = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) face1(Sh, Su, Sv, oh, ou, ov, in, g.nb[k], m.nL, g.al[k], g.sx[k], g.sy[k]);
  const float h0 = STAGE == 1 ? oh : s0.h(j), u0 = STAGE == 1 ? ou : s0.u(j), v0 = STAGE == 1 ? ov : s0.v(j);
  out.put(j, fmaf(c, -Sh, h0), fmaf(c, -Su, u0), fmaf(c, -Sv, v0));
}

// One stage: cells j < lim (n3, n2, n1 for stages 1-3; the tile, j < n0,
// for stage 4).  Tile cells add their delta to `acc` (stages 1-3) and
// combine it into the new state (stage 4); halo cells only give their stage
// value.  acc lanes of halo cells hold values nobody reads.
template <int STAGE, int TT, int CELLS>
__device__ __forceinline__ void stage(const TileMeta &m, const GeoPair (&gp)[CELLS / 2], const Buf &in,
                                      const Buf &s0, const Buf &out, float2 (&acc)[CELLS / 2][3], float c,
                                      float4 *sout, const float4 *gslot) {
  const float2 nc2 = f2(-c, -c);  // delta = -S: c*delta = (-c)*S exactly
  const int lim = STAGE == 1 ? m.n3 : STAGE == 2 ? m.n2 : STAGE == 3 ? m.n1 : m.n0;
#pragma unroll
  for (int p = 0; p < CELLS / 2; ++p) {
    const int jA = threadIdx.x + 2 * p * TT;
    const int jB0 = jA + TT;
    if (jA >= lim) break;
    const bool vB = jB0 < lim;
    const int jB = vB ? jB0 : jA;
    const float2 oh = f2(in.h(jA), in.h(jB)), ou = f2(in.u(jA), in.u(jB)), ov = f2(in.v(jA), in.v(jB));
    float2 Sh, Su, Sv;
    sums2(gp[p], oh, ou, ov, in, m.nL, Sh, Su, Sv);
    const float2 h0 = STAGE == 1 ? oh : f2(s0.h(jA), s0.h(jB));
    const float2 u0 = STAGE == 1 ? ou : f2(s0.u(jA), s0.u(jB));
    const float2 v0 = STAGE == 1 ? ov : f2(s0.v(jA), s0.v(jB));
    // acc holds the sum of the stages' S (the negated sum of their deltas:
    // rounding is symmetric, so the same values up to sign)
    if (STAGE < 4) {
      const float2 xh = fma2(nc2, Sh, h0), xu = fma2(nc2, Su, u0), xv = fma2(nc2, Sv, v0);
      out.put(jA, xh.x, xu.x, xv.x);
      if (vB) out.put(jB, xh.y, xu.y, xv.y);
      if (STAGE == 1) {
        acc[p][0] = Sh;
        acc[p][1] = Su;
        acc[p][2] = Sv;
      } else {
        acc[p][0] = add2(acc[p][0], Sh);
        acc[p][1] = add2(acc[p][1], Su);
        acc[p][2] = add2(acc[p][2], Sv);
      }
    } else {
      const float2 xh = fma2(nc2, add2(acc[p][0], Sh), h0);
      const float2 xu = fma2(nc2, add2(acc[p][1], Su), u0);
      const float2 xv = fma2(nc2, add2(acc[p][2], Sv), v0);
      sout[(int64_t)m.cell_off + jA] = make_float4(xh.x, xu.x, xv.x, 0.f);
      if (vB) sout[(int64_t)m.cell_off + jB] = make_float4(xh.y, xu.y, xv.y, 0.f);
    }
  }
  if (STAGE < 4)  // local cells beyond the register-held ones (the tile's fit in them)
    for (int j = threadIdx.x + CELLS * TT; j < lim; j += TT) extra_cell<STAGE>(j, m, gslot, in, s0, out, c);
}

}  // namespace pipe

template <int TT, int CELLS>
__global__ void __launch_bounds__(TT, 1)
swe_tile_pipe_kernel(const int32_t *__restrict__ meta, const int64_t *__restrict__ off3,
                     const int64_t *__restrict__ offh, const int32_t *__restrict__ halo,
                     const float4 *__restrict__ gslot, const float4 *__restrict__ sin, float4 *__restrict__ sout,
                     int64_t nc, int ntiles, float c1, float c3, float c4, const int32_t *__restrict__ tile_ids) {
  // tile_ids (optional): the tiles this launch walks, ntiles of them
  using namespace pipe;
  extern __shared__ float smem[];
  const Buf SA{smem + 2 * kBuf}, SB{smem + 3 * kBuf};
  int t = blockIdx.x;
  if (t >= ntiles) return;
  TileMeta m = tile_meta(meta, off3, offh, tile_ids ? __ldg(tile_ids + t) : t);
  constexpr int kMaxOwnT = TT * CELLS;  // the tile's cells are among the register-held ones
  bool fits = tile_fits(m, nc, kMaxOwnT);
  int cur = 0;
  GeoPair gp[CELLS / 2];
  int hidx[2];
  if (fits) {  // prologue: the first tile's state and geometry
    halo_index<TT>(m, halo, hidx);
    fetch_own<TT>(Buf{smem}, m, sin);
    fetch_halo<TT>(Buf{smem}, m, sin, nc, halo, hidx);
    load_tile_geo<TT, CELLS>(m, gslot, gp);
  } else {
    esr::raise_status(ESR_DEV_IDX_RANGE);
  }
  cp_commit();
  while (true) {
    const int tn = t + gridDim.x;
    TileMeta mn{};
    bool next = tn < ntiles;
    if (next) {
      mn = tile_meta(meta, off3, offh, tile_ids ? __ldg(tile_ids + tn) : tn);
      if (!tile_fits(mn, nc, kMaxOwnT)) {  // outside the kernel's limits: flag it, leave its cells unwritten
        esr::raise_status(ESR_DEV_IDX_RANGE);
      }
    }
    cp_wait_all();
    __syncthreads();  // this tile's state is in buffer `cur`; the other buffer is free
    const Buf S0{smem + cur * kBuf}, S0n{smem + (cur ^ 1) * kBuf};
    const bool nfit = next && tile_fits(mn, nc, kMaxOwnT);
    if (nfit) {
      if (threadIdx.x == 0) {  // the next tile's face records into L2
        const float4 *g = gslot + 3 * mn.o3;
        const unsigned bytes = (unsigned)(3 * (int64_t)mn.n3 * 16);
        if (bytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(g), "r"(bytes) : "memory");
      }
      halo_index<TT>(mn, halo, hidx);
      fetch_own<TT>(S0n, mn, sin);
    }
    if (fits) {
      float2 acc[CELLS / 2][3];
      stage<1, TT, CELLS>(m, gp, S0, S0, SA, acc, c1, sout, gslot);
      if (nfit) fetch_halo<TT>(S0n, mn, sin, nc, halo, hidx);
      cp_commit();
      __syncthreads();
      stage<2, TT, CELLS>(m, gp, SA, S0, SB, acc, c1, sout, gslot);
      __syncthreads();
      stage<3, TT, CELLS>(m, gp, SB, S0, SA, acc, c3, sout, gslot);
      __syncthreads();
      stage<4, TT, CELLS>(m, gp, SA, S0, SA, acc, c4, sout, gslot);
    } else {
      if (nfit) fetch_halo<TT>(S0n, mn, sin, nc, halo, hidx);
      cp_commit();
    }
    if (!next) break;
    // the next tile's geometry: this thread is done with the current one
    if (nfit) load_tile_geo<TT, CELLS>(mn, gslot, gp);
    m = mn;
    fits = nfit;
    t = tn;
    cur ^= 1;
  }
  cp_wait_all();
}

// CTA shapes of the pipelined kernel: 512 threads x 4 tile cells (what
// PIPELINED and AUTO run; measured fastest at N=2000 with 1,900-cell tiles)
// and 768 threads x 2 (n0 <= 1536; on request)
constexpr int kPipeSmall = 768 * 2, kPipeLarge = 512 * 4;

bool pipe_fits(const esr_swe_tiles *T, int shape) {
  const int max_own = shape == ESR_SWE_TILE_PIPELINED_768 ? kPipeSmall : kPipeLarge;
  return !T->exact && T->max_own <= max_own && T->max_local <= pipe::kMaxLocal && T->slot_info == 1;
}

int pipe_shape(const esr_swe_tiles *) { return ESR_SWE_TILE_PIPELINED_512; }

// (tile_ids: the launch walks those `count` tiles only)
template <int TT, int CELLS>
int run_pipe_shape(const esr_swe_tiles *tiles, double dt, void *state_a, void *state_b, int64_t steps,
                   cudaStream_t s, const int32_t *tile_ids = nullptr, int count = 0) {
  cudaError_t e = cudaFuncSetAttribute(swe_tile_pipe_kernel<TT, CELLS>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, pipe::kSmemBytes);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_tile_step/pipelined smem attribute");
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_tile_step/SM count");
  const int nt = tile_ids ? count : tiles->ntiles;
  if (nt <= 0) return ESR_OK;
  const int grid = nt < sms ? nt : sms;
  const float c1 = (float)(0.5 * dt), c3 = (float)dt, c4 = (float)(dt / 6);
  float4 *buf[2] = {(float4 *)state_a, (float4 *)state_b};
  for (int64_t k = 0; k < steps; ++k) {
    swe_tile_pipe_kernel<TT, CELLS><<<grid, TT, pipe::kSmemBytes, s>>>(
        tiles->meta, tiles->off3, tiles->offh, tiles->halo, (const float4 *)tiles->slots, buf[k & 1],
        buf[(k + 1) & 1], tiles->nc, nt, c1, c3, c4, tile_ids);
  }
  ESR_LAUNCH_CHECK("esr_swe_tile_step/pipelined");
  return ESR_OK;
}

int run_pipe(const esr_swe_tiles *tiles, int shape, double dt, void *state_a, void *state_b, int64_t steps,
             cudaStream_t s) {
  if (shape == ESR_SWE_TILE_PIPELINED_768)
    return run_pipe_shape<768, 2>(tiles, dt, state_a, state_b, steps, s);
  return run_pipe_shape<512, 4>(tiles, dt, state_a, state_b, steps, s);
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
  if (mesh->dtype == ESR_F64)
    return mesh->exact ? dispatch_steps<double, true>(mesh, dt, state, steps, workspace, s)
                       : dispatch_steps<double, false>(mesh, dt, state, steps, workspace, s);
  return mesh->exact ? dispatch_steps<float, true>(mesh, dt, state, steps, workspace, s)
                     : dispatch_steps<float, false>(mesh, dt, state, steps, workspace, s);
}

extern "C" int esr_swe_delta(const esr_swe_mesh *mesh, const void *state, void *delta, void *stream) {
  int st = check_mesh(mesh);
  if (st) return st;
  if (!state || !delta) return esr::fail(ESR_ERR_ARG, "null state/delta");
  if (((uintptr_t)state | (uintptr_t)delta) % 32) return esr::fail(ESR_ERR_ARG, "state/delta must be 32-byte aligned");
  cudaStream_t s = esr::as_stream(stream);
  if (mesh->dtype == ESR_F64)
    return mesh->exact ? dispatch_delta<double, true>(mesh, state, delta, s)
                       : dispatch_delta<double, false>(mesh, state, delta, s);
  return mesh->exact ? dispatch_delta<float, true>(mesh, state, delta, s)
                     : dispatch_delta<float, false>(mesh, state, delta, s);
}

extern "C" int64_t esr_swe_tile_smem_bytes(const esr_swe_tiles *tiles) {
  if (check_tiles(tiles)) return -1;
  return tile_smem_bytes(tiles);
}

extern "C" int esr_swe_tile_threads(const esr_swe_tiles *tiles) {
  if (check_tiles(tiles)) return -1;
  return tile_threads(tiles);
}

extern "C" int esr_swe_tile_kernel(const esr_swe_tiles *tiles) {
  if (check_tiles(tiles)) return -1;
  return pipe_fits(tiles, ESR_SWE_TILE_PIPELINED_512) ? pipe_shape(tiles) : ESR_SWE_TILE_BLOCKED;
}

extern "C" int esr_swe_tile_step_with(const esr_swe_tiles *tiles, int kernel, double dt, void *state_a,
                                      void *state_b, int64_t steps, void *stream) {
  int st = check_tiles(tiles);
  if (st) return st;
  if (steps < 0) return esr::fail(ESR_ERR_ARG, "negative step count");
  if (!state_a || !state_b || state_a == state_b) return esr::fail(ESR_ERR_ARG, "need two distinct state buffers");
  if (((uintptr_t)state_a | (uintptr_t)state_b) % 16) return esr::fail(ESR_ERR_ARG, "state buffers must be 16-byte aligned");
  if (kernel == ESR_SWE_TILE_AUTO) kernel = esr_swe_tile_kernel(tiles);
  if (kernel == ESR_SWE_TILE_PIPELINED) kernel = pipe_shape(tiles);
  if (kernel == ESR_SWE_TILE_PIPELINED_512 || kernel == ESR_SWE_TILE_PIPELINED_768) {
    if (!pipe_fits(tiles, kernel))
      return esr::fail(ESR_ERR_UNSUPPORTED, "the pipelined tile kernel needs fast arithmetic, slot_info == 1, <= 4096 "
                                            "local cells a tile and <= 2048 own cells (512-thread shape) or <= 1536 "
                                            "(768-thread)");
  } else if (kernel != ESR_SWE_TILE_BLOCKED) {
    return esr::fail(ESR_ERR_ARG, "unknown tile kernel");
  }
  if (steps == 0) return ESR_OK;
  cudaStream_t s = esr::as_stream(stream);
  if (kernel != ESR_SWE_TILE_BLOCKED) return run_pipe(tiles, kernel, dt, state_a, state_b, steps, s);
  return tiles->exact ? run_tiles<true>(tiles, dt, state_a, state_b, steps, s)
                      : run_tiles<false>(tiles, dt, state_a, state_b, steps, s);
}

extern "C" int esr_swe_tile_step(const esr_swe_tiles *tiles, double dt, void *state_a, void *state_b, int64_t steps,
                                 void *stream) {
  return esr_swe_tile_step_with(tiles, ESR_SWE_TILE_AUTO, dt, state_a, state_b, steps, stream);
}

// ------------------------------------------------------------------------
// A state held in host memory, stepped on the GPU.  Per step the FP32
// (h, uh, vh) [nc][3] state goes up in chunks (copy stream `up`), each chunk
// is unpacked into the [nc] float4 engine layout as it lands, the step runs
// on the caller's stream, and each chunk is packed and brought back (copy
// stream `down`) as soon as it is packed.  The next step's upload of a
// chunk waits only for that chunk's download, so while chunk c of a result
// comes home chunk c - 1 of the next step's input goes up: the link carries
// both directions at once.
namespace {

__global__ void unpack3_kernel(const float *__restrict__ stage, float4 *__restrict__ a, int64_t off, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float *q = stage + 3 * (off + i);
    a[off + i] = make_float4(q[0], q[1], q[2], 0.f);
  }
}

__global__ void pack3_kernel(const float4 *__restrict__ b, float *__restrict__ stage, int64_t off, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float4 v = b[off + i];
    float *q = stage + 3 * (off + i);
    q[0] = v.x;
    q[1] = v.y;
    q[2] = v.z;
  }
}

struct SweHostPlan {
  esr_swe_tiles tiles{};
  float4 *a = nullptr, *b = nullptr;
  float *stage = nullptr;
  int chunks = 0;
  int grid = 0;
  std::vector<int64_t> off;  // [chunks + 1] cell offsets, multiples of 4
  cudaStream_t up = nullptr, down = nullptr;
  cudaEvent_t entry = nullptr;
  std::vector<cudaEvent_t> ev_up, ev_pack, ev_down;
  // grouped schedule (pipelined kernel): the tiles whose local cells all lie
  // in chunks <= g form group g (tile_list[group_off[g] .. group_off[g+1]])
  // and run as soon as chunk g has landed; chunk c goes home after group
  // ready[c], the last one holding tiles that own cells of chunk c
  const int32_t *tile_list = nullptr;
  std::vector<int32_t> group_off, ready;
};

// the grouped schedule of a plan from the layout (read back once)
int plan_groups(SweHostPlan *P, int32_t *tile_list) {
  const esr_swe_tiles &T = P->tiles;
  const int C = P->chunks;
  const int nt = T.ntiles;
  std::vector<int32_t> meta(8 * (size_t)nt);
  std::vector<int64_t> offh(nt);
  cudaError_t e = cudaMemcpy(meta.data(), T.meta, meta.size() * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(offh.data(), T.offh, offh.size() * 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_host_plan_create/layout");
  int64_t th = 0;
  for (int t = 0; t < nt; ++t) th = std::max(th, offh[t] + (int64_t)(meta[8 * t + 5] - meta[8 * t + 1]));
  std::vector<int32_t> halo(th > 0 ? th : 1);
  if (th > 0) e = cudaMemcpy(halo.data(), T.halo, th * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_host_plan_create/halo");
  const int64_t per = P->off[1];  // every chunk but the last has `per` cells
  auto chunk = [&](int64_t cell) { return (int)std::min<int64_t>(cell / per, C - 1); };
  std::vector<int32_t> group(nt);
  P->ready.assign(C, 0);
  for (int t = 0; t < nt; ++t) {
    const int64_t c0 = meta[8 * t], n0 = meta[8 * t + 1], nl = meta[8 * t + 5];
    if (n0 <= 0) {
      group[t] = 0;
      continue;
    }
    int g = chunk(c0 + n0 - 1);
    for (int64_t j = 0; j < nl - n0; ++j) {
      const int64_t cell = halo[offh[t] + j];
      if (cell >= 0 && cell < T.nc) g = std::max(g, chunk(cell));
    }
    group[t] = g;
    for (int c = chunk(c0); c <= chunk(c0 + n0 - 1); ++c) P->ready[c] = std::max(P->ready[c], g);
  }
  P->group_off.assign(C + 1, 0);
  for (int t = 0; t < nt; ++t) P->group_off[group[t] + 1]++;
  for (int g = 0; g < C; ++g) P->group_off[g + 1] += P->group_off[g];
  std::vector<int32_t> list(nt), fill(P->group_off.begin(), P->group_off.end() - 1);
  for (int t = 0; t < nt; ++t) list[fill[group[t]]++] = t;
  e = cudaMemcpy(tile_list, list.data(), (size_t)nt * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_host_plan_create/tile list");
  P->tile_list = tile_list;
  return ESR_OK;
}

void destroy_host_plan(SweHostPlan *P) {
  if (!P) return;
  for (auto *v : {&P->ev_up, &P->ev_pack, &P->ev_down})
    for (cudaEvent_t e : *v)
      if (e) cudaEventDestroy(e);
  if (P->entry) cudaEventDestroy(P->entry);
  if (P->up) cudaStreamDestroy(P->up);
  if (P->down) cudaStreamDestroy(P->down);
  delete P;
}

}  // namespace

extern "C" int esr_swe_host_plan_create(const esr_swe_tiles *tiles, void *state_a, void *state_b, void *staging,
                                        int32_t *tile_list, int32_t chunks, void **plan_out) {
  int st = check_tiles(tiles);
  if (st) return st;
  if (!state_a || !state_b || !staging || !plan_out || state_a == state_b)
    return esr::fail(ESR_ERR_ARG, "need two distinct state buffers, a staging buffer and an output pointer");
  if (((uintptr_t)state_a | (uintptr_t)state_b) % 16 || (uintptr_t)staging % 16)
    return esr::fail(ESR_ERR_ARG, "state and staging buffers must be 16-byte aligned");
  if (chunks < 1 || chunks > 64) return esr::fail(ESR_ERR_ARG, "chunks must be in [1, 64]");
  SweHostPlan *P = new (std::nothrow) SweHostPlan();
  if (!P) return esr::fail(ESR_ERR_ARG, "out of host memory");
  try {
    P->tiles = *tiles;
    P->a = (float4 *)state_a;
    P->b = (float4 *)state_b;
    P->stage = (float *)staging;
    const int64_t nc = tiles->nc;
    const int64_t per = ((nc + chunks - 1) / chunks + 3) / 4 * 4;
    P->off.push_back(0);
    while (P->off.back() < nc) P->off.push_back(std::min(nc, P->off.back() + per));
    P->chunks = (int)P->off.size() - 1;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->down, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->entry, cudaEventDisableTiming);
    P->grid = 4 * (sms > 0 ? sms : 1);
    for (auto *v : {&P->ev_up, &P->ev_pack, &P->ev_down}) {
      v->assign(P->chunks, nullptr);
      for (int c = 0; c < P->chunks && e == cudaSuccess; ++c) e = cudaEventCreateWithFlags(&(*v)[c], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
      destroy_host_plan(P);
      return esr::cuda_check(e, "esr_swe_host_plan_create");
    }
    if (tile_list && P->chunks > 1 && pipe_fits(tiles, ESR_SWE_TILE_PIPELINED_512)) {
      const int gst = plan_groups(P, tile_list);
      if (gst) {
        destroy_host_plan(P);
        return gst;
      }
    }
  } catch (const std::bad_alloc &) {
    destroy_host_plan(P);
    return esr::fail(ESR_ERR_ARG, "out of host memory");
  }
  *plan_out = P;
  return ESR_OK;
}

extern "C" int esr_swe_host_step(void *plan, double dt, float *host_state, int64_t steps, void *stream) {
  if (!plan || !host_state) return esr::fail(ESR_ERR_ARG, "null plan or host state");
  if (steps < 0) return esr::fail(ESR_ERR_ARG, "negative step count");
  if (steps == 0) return ESR_OK;
  SweHostPlan *P = (SweHostPlan *)plan;
  cudaStream_t s = esr::as_stream(stream);
  const int C = P->chunks;
  // the uploads overwrite the staging buffer: after the caller's earlier work
  cudaError_t e = cudaEventRecord(P->entry, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(P->up, P->entry, 0);
  for (int64_t k = 0; k < steps && e == cudaSuccess; ++k) {
    for (int c = 0; c < C && e == cudaSuccess; ++c) {
      const int64_t o = P->off[c], n = P->off[c + 1] - o;
      if (k > 0) e = cudaStreamWaitEvent(P->up, P->ev_down[c], 0);  // chunk c of the last result is home
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(P->stage + 3 * o, host_state + 3 * o, 12 * n, cudaMemcpyHostToDevice, P->up);
      if (e == cudaSuccess) e = cudaEventRecord(P->ev_up[c], P->up);
    }
    auto unpack = [&](int c) {
      const int64_t o = P->off[c], n = P->off[c + 1] - o;
      cudaError_t r = cudaStreamWaitEvent(s, P->ev_up[c], 0);
      if (r == cudaSuccess) {
        unpack3_kernel<<<P->grid, 256, 0, s>>>(P->stage, P->a, o, n);
        r = cudaGetLastError();
      }
      return r;
    };
    auto pack = [&](int c) {
      const int64_t o = P->off[c], n = P->off[c + 1] - o;
      pack3_kernel<<<P->grid, 256, 0, s>>>(P->b, P->stage, o, n);
      cudaError_t r = cudaGetLastError();
      if (r == cudaSuccess) r = cudaEventRecord(P->ev_pack[c], s);
      return r;
    };
    if (P->tile_list) {  // each group of tiles as soon as its chunks have landed
      for (int g = 0; g < C && e == cudaSuccess; ++g) {
        e = unpack(g);
        if (e != cudaSuccess) break;
        const int st = run_pipe_shape<512, 4>(&P->tiles, dt, P->a, P->b, 1, s, P->tile_list + P->group_off[g],
                                              P->group_off[g + 1] - P->group_off[g]);
        if (st) return st;
        for (int c = 0; c < C && e == cudaSuccess; ++c)
          if (P->ready[c] == g) e = pack(c);
      }
    } else {
      for (int c = 0; c < C && e == cudaSuccess; ++c) e = unpack(c);
      if (e != cudaSuccess) break;
      const int st = esr_swe_tile_step_with(&P->tiles, ESR_SWE_TILE_AUTO, dt, P->a, P->b, 1, s);
      if (st) return st;
      for (int c = 0; c < C && e == cudaSuccess; ++c) e = pack(c);
    }
    for (int c = 0; c < C && e == cudaSuccess; ++c) {
      const int64_t o = P->off[c], n = P->off[c + 1] - o;
      e = cudaStreamWaitEvent(P->down, P->ev_pack[c], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_state + 3 * o, P->stage + 3 * o, 12 * n, cudaMemcpyDeviceToHost, P->down);
      if (e == cudaSuccess) e = cudaEventRecord(P->ev_down[c], P->down);
    }
  }
  // the caller's stream sees the last result home
  for (int c = 0; c < C && e == cudaSuccess; ++c) e = cudaStreamWaitEvent(s, P->ev_down[c], 0);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_host_step");
  return ESR_OK;
}

extern "C" int esr_swe_host_plan_destroy(void *plan) {
  if (!plan) return ESR_OK;
  SweHostPlan *P = (SweHostPlan *)plan;
  cudaError_t e = cudaStreamSynchronize(P->up);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->down);
  destroy_host_plan(P);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_swe_host_plan_destroy");
  return ESR_OK;
}
