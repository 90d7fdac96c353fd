// Mesh generation, shallow-water geometry and FV Poisson assembly on the
// GPU: the same outputs as host_mesh.cpp, one thread per square / cell /
// edge / wall face.
//
// Reference: csrc/triangular_mesh.cpp:10-143 (get_mesh),
// tutorial/shallow_water_equation/assemble_shallow_water.py:154-253,
// tutorial/poisson/assemble_poisson.py:160-230.
//
// Every floating operation is one IEEE double operation in the reference's
// order, written with the explicit round-to-nearest intrinsics (__dadd_rn,
// __dmul_rn, __ddiv_rn, ...) so that nothing is contracted into an FMA: the
// integer outputs are index-for-index the reference's and the floating ones
// bit for bit, except rho and b of the Poisson assembly, which go through
// CUDA's exp (a few ulp from the host's).
#include <cstdint>

#include "esr_internal.h"

namespace {

constexpr int kMeshThreads = 256;

struct P2 {
  double x, y;
};

__device__ __forceinline__ P2 pt(const double *points, int64_t p) { return P2{points[2 * p], points[2 * p + 1]}; }

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double sign_of(double v) {  // torch.sign
  if (v > 0.0) return 1.0;
  if (v < 0.0) return -1.0;
  return v;
}

// get_face_norm (assemble_shallow_water.py:173-183): normal of (b, c) away
// from a, scaled by the segment length
__device__ __forceinline__ P2 face_normal(P2 a, P2 b, P2 c) {
  const double bcx = sub(b.x, c.x), bcy = sub(b.y, c.y);
  const double acx = sub(a.x, c.x), acy = sub(a.y, c.y);
  const double cross = sub(mul(bcx, acy), mul(bcy, acx));
  const double s = sign_of(cross);
  return P2{mul(s, bcy), mul(-s, bcx)};
}

// get_alpha (assemble_shallow_water.py:154-171)
__device__ __forceinline__ double line_alpha(P2 sc, P2 dc, P2 p0, P2 p1) {
  const double y21 = sub(dc.y, sc.y), y43 = sub(p1.y, p0.y), y31 = sub(p0.y, sc.y);
  const double x31 = sub(p0.x, sc.x), x21 = sub(dc.x, sc.x), x43 = sub(p1.x, p0.x);
  const double num = sub(mul(x31, y43), mul(y31, x43));
  const double den = sub(mul(x21, y43), mul(y21, x43));
  return dvd(num, den);
}

__device__ __forceinline__ P2 centroid3(P2 a, P2 b, P2 c) {
  return P2{dvd(add(add(a.x, b.x), c.x), 3.0), dvd(add(add(a.y, b.y), c.y), 3.0)};
}

__device__ __forceinline__ double tri_area(P2 p0, P2 p1, P2 p2) {
  const double t0 = mul(p0.x, sub(p1.y, p2.y));
  const double t1 = mul(p1.x, sub(p2.y, p0.y));
  const double t2 = mul(p2.x, sub(p0.y, p1.y));
  return mul(0.5, fabs(add(add(t0, t1), t2)));
}

struct Sel {
  double nx, ny, alpha;
};

// the face of the src triangle the dst centroid lies beyond
// (assemble_shallow_water.py:199-223, assemble_poisson.py:174-192)
__device__ __forceinline__ Sel select_face(const P2 (&sp)[3], P2 sc, P2 dc, bool want_alpha) {
  const int kA[3] = {2, 0, 1}, kB[3] = {0, 1, 2}, kC[3] = {1, 2, 0};
  Sel out{0., 0., 0.};
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const P2 own = face_normal(sp[kA[f]], sp[kB[f]], sp[kC[f]]);
    const P2 dn = face_normal(dc, sp[kB[f]], sp[kC[f]]);
    const double dot = add(mul(own.x, dn.x), mul(own.y, dn.y));
    if (dot < 0) {
      out.nx = own.x;
      out.ny = own.y;
      if (want_alpha) out.alpha = line_alpha(sc, dc, sp[kB[f]], sp[kC[f]]);
    }
  }
  return out;
}

__device__ __forceinline__ void cell_points(const int64_t *cells, const double *points, int64_t c, P2 (&p)[3]) {
#pragma unroll
  for (int v = 0; v < 3; ++v) p[v] = pt(points, cells[3 * c + v]);
}

// ---------------------------------------------------------------- mesh --
// corner (i, j) of the (n+1)^2 grid, then the n^2 square centres
__global__ void __launch_bounds__(kMeshThreads) mesh_points_kernel(int64_t n, double *points) {
  const int64_t ncorner = (n + 1) * (n + 1);
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ncorner + n * n) return;
  const double d = dvd(1.0, (double)n);
  double x, y;
  if (p < ncorner) {
    const int64_t j = p / (n + 1), i = p % (n + 1);
    x = i < n ? mul((double)i, d) : add(mul((double)(n - 1), d), d);
    y = j < n ? mul((double)j, d) : add(mul((double)(n - 1), d), d);
  } else {
    const int64_t c = p - ncorner, j = c / n, i = c % n;
    x = add(mul((double)i, d), dvd(d, 2.0));
    y = add(mul((double)j, d), dvd(d, 2.0));
  }
  points[2 * p] = x;
  points[2 * p + 1] = y;
}

// one square: its 4 triangles, 8 internal directed edges, and the edge or
// wall face towards each of its 4 neighbours (triangular_mesh.cpp layout)
__global__ void __launch_bounds__(kMeshThreads)
mesh_squares_kernel(int64_t n, int64_t *src, int64_t *dst, int64_t *cells, int64_t *bcells, int64_t *bpoints) {
  const int64_t sq = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (sq >= n * n) return;
  const int64_t j = sq / n, i = sq % n;
  const int64_t ncorner = (n + 1) * (n + 1), base = 8 * n * n;
  const int64_t c0 = 4 * sq;
  const int64_t bl = j * (n + 1) + i, tl = (j + 1) * (n + 1) + i, tr = tl + 1, br = bl + 1;
  const int64_t ce = ncorner + n * j + i;
  const int64_t tri[4][3] = {{bl, br, ce}, {tr, ce, br}, {tr, tl, ce}, {bl, ce, tl}};
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int v = 0; v < 3; ++v) cells[3 * (c0 + k) + v] = tri[k][v];
#pragma unroll
  for (int64_t k = 0; k < 4; ++k) {
    const int64_t a = c0 + k, b = c0 + (k + 1) % 4;
    src[8 * sq + 2 * k] = a;
    dst[8 * sq + 2 * k] = b;
    src[8 * sq + 2 * k + 1] = b;
    dst[8 * sq + 2 * k + 1] = a;
  }
  if (j > 0) {
    const int64_t e = base + n * (j - 1) + i;
    src[e] = c0;
    dst[e] = c0 - 4 * n + 2;
  } else {
    bcells[i] = c0;
    bpoints[2 * i] = bl;
    bpoints[2 * i + 1] = br;
  }
  if (j < n - 1) {
    const int64_t e = base + n * (n - 1) + n * j + i;
    src[e] = c0 + 2;
    dst[e] = c0 + 4 * n;
  } else {
    bcells[n + i] = c0 + 2;
    bpoints[2 * (n + i)] = tl;
    bpoints[2 * (n + i) + 1] = tr;
  }
  if (i > 0) {
    const int64_t e = base + 2 * n * (n - 1) + (n - 1) * j + i - 1;
    src[e] = c0 + 3;
    dst[e] = c0 - 3;
  } else {
    bcells[2 * n + j] = c0 + 3;
    bpoints[2 * (2 * n + j)] = bl;
    bpoints[2 * (2 * n + j) + 1] = tl;
  }
  if (i < n - 1) {
    const int64_t e = base + 3 * n * (n - 1) + (n - 1) * j + i;
    src[e] = c0 + 1;
    dst[e] = c0 + 7;
  } else {
    bcells[3 * n + j] = c0 + 1;
    bpoints[2 * (3 * n + j)] = tr;
    bpoints[2 * (3 * n + j) + 1] = br;
  }
}

// ------------------------------------------------------------ geometry --
__global__ void __launch_bounds__(kMeshThreads)
geo_cells_kernel(int64_t nc, int64_t np, const int64_t *cells, const double *points, double *area, double *x,
                 double *y) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  if (cells[3 * c] < 0 || cells[3 * c] >= np || cells[3 * c + 1] < 0 || cells[3 * c + 1] >= np ||
      cells[3 * c + 2] < 0 || cells[3 * c + 2] >= np) {
    esr::raise_status(ESR_DEV_IDX_RANGE);
    return;
  }
  P2 p[3];
  cell_points(cells, points, c, p);
  area[c] = tri_area(p[0], p[1], p[2]);
  const P2 g = centroid3(p[0], p[1], p[2]);
  x[c] = g.x;
  y[c] = g.y;
}

__device__ __forceinline__ bool cell_ok(const int64_t *cells, int64_t np, int64_t c) {
  return cells[3 * c] >= 0 && cells[3 * c] < np && cells[3 * c + 1] >= 0 && cells[3 * c + 1] < np &&
         cells[3 * c + 2] >= 0 && cells[3 * c + 2] < np;
}

// POISSON: Af = (dist / |dist|^2) . n instead of (sx, sy, alpha)
template <bool POISSON>
__global__ void __launch_bounds__(kMeshThreads)
geo_edges_kernel(int64_t ne, int64_t nc, int64_t np, const int64_t *src, const int64_t *dst, const int64_t *cells,
                 const double *points, double *sx, double *sy, double *alpha) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int64_t s = src[e], t = dst[e];
  if (s < 0 || s >= nc || t < 0 || t >= nc || !cell_ok(cells, np, s) || !cell_ok(cells, np, t)) {
    esr::raise_status(ESR_DEV_IDX_RANGE);
    return;
  }
  P2 sp[3], dp[3];
  cell_points(cells, points, s, sp);
  cell_points(cells, points, t, dp);
  const P2 sc = centroid3(sp[0], sp[1], sp[2]);
  const P2 dc = centroid3(dp[0], dp[1], dp[2]);
  if (POISSON) {
    const double distx = sub(dc.x, sc.x), disty = sub(dc.y, sc.y);
    const Sel f = select_face(sp, sc, dc, false);
    const double d2 = add(mul(distx, distx), mul(disty, disty));
    const double ux = dvd(distx, d2), uy = dvd(disty, d2);
    sx[e] = add(mul(ux, f.nx), mul(uy, f.ny));  // Af
  } else {
    const Sel f = select_face(sp, sc, dc, true);
    sx[e] = f.nx;
    sy[e] = f.ny;
    alpha[e] = f.alpha;
  }
}

__global__ void __launch_bounds__(kMeshThreads)
geo_walls_kernel(int64_t nbc, int64_t nc, int64_t np, const int64_t *bcells, const int64_t *bpoints,
                 const int64_t *cells, const double *points, double *bsx, double *bsy) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbc) return;
  const int64_t c = bcells[b], q0 = bpoints[2 * b], q1 = bpoints[2 * b + 1];
  if (c < 0 || c >= nc || q0 < 0 || q0 >= np || q1 < 0 || q1 >= np || !cell_ok(cells, np, c)) {
    esr::raise_status(ESR_DEV_IDX_RANGE);
    return;
  }
  P2 p[3];
  cell_points(cells, points, c, p);
  const P2 bn = face_normal(centroid3(p[0], p[1], p[2]), pt(points, q0), pt(points, q1));
  bsx[b] = -bn.x;
  bsy[b] = -bn.y;
}

// ------------------------------------------------------------- Poisson --
// Ac[c] = -(in-order sum of Af over the edges with src c) - (in-order sum of
// the boundary terms of c's wall faces); rho, b per cell.  rowptr/perm: the
// stable CSR of src (the reference Reducer's order), brow/bperm that of
// bcells.
__global__ void __launch_bounds__(kMeshThreads)
fv_cells_kernel(int64_t nc, int64_t np, const int32_t *rowptr, const int32_t *perm, const int32_t *brow,
                const int32_t *bperm, const int64_t *cells, const int64_t *bpoints, const double *points,
                const double *Af, double *Ac, double *b, double *rho, double *centroid) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  if (!cell_ok(cells, np, c)) {
    esr::raise_status(ESR_DEV_IDX_RANGE);
    return;
  }
  P2 p[3];
  cell_points(cells, points, c, p);
  const double ar = tri_area(p[0], p[1], p[2]);
  const P2 g = centroid3(p[0], p[1], p[2]);
  centroid[2 * c] = g.x;
  centroid[2 * c + 1] = g.y;
  double acc = 0.0;
  for (int32_t k = rowptr[c]; k < rowptr[c + 1]; ++k) acc = add(acc, Af[perm[k]]);
  double bacc = 0.0;
  for (int32_t k = brow[c]; k < brow[c + 1]; ++k) {
    const int32_t w = bperm[k];
    const int64_t q0 = bpoints[2 * w], q1 = bpoints[2 * w + 1];
    if (q0 < 0 || q0 >= np || q1 < 0 || q1 >= np) {
      esr::raise_status(ESR_DEV_IDX_RANGE);
      continue;
    }
    const P2 b0 = pt(points, q0), b1 = pt(points, q1);
    const P2 fc{dvd(add(b0.x, b1.x), 2.0), dvd(add(b0.y, b1.y), 2.0)};
    const P2 bn = face_normal(g, b0, b1);
    const double dx = sub(fc.x, g.x), dy = sub(fc.y, g.y);
    const double d2 = add(mul(dx, dx), mul(dy, dy));
    const double ux = dvd(dx, d2), uy = dvd(dy, d2);
    bacc = add(bacc, add(mul(ux, bn.x), mul(uy, bn.y)));
  }
  Ac[c] = sub(-acc, bacc);
  const double dx = sub(g.x, 0.5), dy = sub(g.y, 0.5);
  const double r2 = add(mul(dx, dx), mul(dy, dy));
  const double rh = exp(mul(-200.0, r2));
  rho[c] = rh;
  b[c] = mul(rh, ar);
}

int grid_for(int64_t n) { return (int)((n + kMeshThreads - 1) / kMeshThreads); }

}  // namespace

ESR_DEFINE_STATUS_READER(esr_status_mesh_gpu)

extern "C" int esr_mesh_triangular_device(int64_t n, int64_t *src, int64_t *dst, int64_t *cells, int64_t *bcells,
                                          int64_t *bpoints, double *points, void *stream) {
  int64_t nc, ne, nbc, np;
  int st = esr_mesh_sizes(n, &nc, &ne, &nbc, &np);
  if (st) return st;
  if (!src || !dst || !cells || !bcells || !bpoints || !points)
    return esr::fail(ESR_ERR_ARG, "esr_mesh_triangular_device: null output");
  cudaStream_t s = esr::as_stream(stream);
  mesh_points_kernel<<<grid_for(np), kMeshThreads, 0, s>>>(n, points);
  mesh_squares_kernel<<<grid_for(n * n), kMeshThreads, 0, s>>>(n, src, dst, cells, bcells, bpoints);
  ESR_LAUNCH_CHECK("esr_mesh_triangular_device");
  return ESR_OK;
}

extern "C" int esr_swe_geometry_device(int64_t nc, int64_t ne, int64_t nbc, int64_t np, const int64_t *src,
                                       const int64_t *dst, const int64_t *cells, const int64_t *bcells,
                                       const int64_t *bpoints, const double *points, double *sx, double *sy,
                                       double *alpha, double *area, double *x, double *y, double *bsx, double *bsy,
                                       void *stream) {
  if (nc <= 0 || ne < 0 || nbc < 0 || np <= 0) return esr::fail(ESR_ERR_ARG, "esr_swe_geometry_device: sizes");
  if (!src || !dst || !cells || !points || !sx || !sy || !alpha || !area || !x || !y ||
      (nbc && (!bcells || !bpoints || !bsx || !bsy)))
    return esr::fail(ESR_ERR_ARG, "esr_swe_geometry_device: null array");
  cudaStream_t s = esr::as_stream(stream);
  geo_cells_kernel<<<grid_for(nc), kMeshThreads, 0, s>>>(nc, np, cells, points, area, x, y);
  if (ne) geo_edges_kernel<false><<<grid_for(ne), kMeshThreads, 0, s>>>(ne, nc, np, src, dst, cells, points, sx, sy, alpha);
  if (nbc) geo_walls_kernel<<<grid_for(nbc), kMeshThreads, 0, s>>>(nbc, nc, np, bcells, bpoints, cells, points, bsx, bsy);
  ESR_LAUNCH_CHECK("esr_swe_geometry_device");
  return ESR_OK;
}

extern "C" int esr_poisson_fv_assemble_device(int64_t nc, int64_t ne, int64_t nbc, int64_t np, const int64_t *src,
                                              const int64_t *dst, const int64_t *cells, const int64_t *bcells,
                                              const int64_t *bpoints, const double *points, const int32_t *rowptr,
                                              const int32_t *perm, const int32_t *brow, const int32_t *bperm,
                                              double *Af, double *Ac, double *b, double *rho, double *centroid,
                                              void *stream) {
  if (nc <= 0 || ne < 0 || nbc < 0 || np <= 0) return esr::fail(ESR_ERR_ARG, "esr_poisson_fv_assemble_device: sizes");
  if (!src || !dst || !cells || !points || !rowptr || !perm || !brow || !Af || !Ac || !b || !rho || !centroid ||
      (nbc && (!bcells || !bpoints || !bperm)))
    return esr::fail(ESR_ERR_ARG, "esr_poisson_fv_assemble_device: null array");
  cudaStream_t s = esr::as_stream(stream);
  if (ne) geo_edges_kernel<true><<<grid_for(ne), kMeshThreads, 0, s>>>(ne, nc, np, src, dst, cells, points, Af, nullptr, nullptr);
  fv_cells_kernel<<<grid_for(nc), kMeshThreads, 0, s>>>(nc, np, rowptr, perm, brow, bperm, cells, bpoints, points, Af,
                                                         Ac, b, rho, centroid);
  ESR_LAUNCH_CHECK("esr_poisson_fv_assemble_device");
  return ESR_OK;
}
