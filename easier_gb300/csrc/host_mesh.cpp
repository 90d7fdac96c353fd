// Host-side mesh generation, geometry and assembly for the sparse-mesh path.
//
// Integer outputs are index-for-index those of the reference; floating
// outputs follow the reference's operation order one IEEE operation at a
// time.  This file must be compiled with -ffp-contract=off (no fused
// multiply-add), otherwise aarch64 compilers contract a*b+c and the values
// drift by an ulp from the reference's CPU run.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "esr_internal.h"

namespace {

struct Pt {
  double x, y;
};

inline Pt pt_at(const double *points, int64_t p) {
  return Pt{points[2 * p], points[2 * p + 1]};
}

// sign() as torch.sign: -1, 0, +1 (NaN propagates).
inline double sign_of(double v) {
  if (v > 0.0) return 1.0;
  if (v < 0.0) return -1.0;
  return v;  // +0, -0 or NaN
}

// Outward-facing normal of the segment (b, c) seen from a, scaled by the
// segment length: tutorial/shallow_water_equation/assemble_shallow_water.py
// :173-183 (get_face_norm).  Returns (s*(b.y-c.y), -s*(b.x-c.x)).
inline Pt face_normal(Pt a, Pt b, Pt c) {
  double bcx = b.x - c.x;
  double bcy = b.y - c.y;
  double acx = a.x - c.x;
  double acy = a.y - c.y;
  double cross = bcx * acy - bcy * acx;
  double s = sign_of(cross);
  double ms = -s;
  return Pt{s * bcy, ms * bcx};
}

// Fraction along (sc -> dc) where it crosses the line (p0, p1):
// assemble_shallow_water.py:154-171 (get_alpha).
inline double line_alpha(Pt sc, Pt dc, Pt p0, Pt p1) {
  double y21 = dc.y - sc.y;
  double y43 = p1.y - p0.y;
  double y31 = p0.y - sc.y;
  double x31 = p0.x - sc.x;
  double x21 = dc.x - sc.x;
  double x43 = p1.x - p0.x;
  double num = x31 * y43 - y31 * x43;
  double den = x21 * y43 - y21 * x43;
  return num / den;
}

// ((a + b) + c) / 3, the reference's centroid expression.
inline Pt centroid3(Pt a, Pt b, Pt c) {
  double sx = a.x + b.x;
  sx = sx + c.x;
  double sy = a.y + b.y;
  sy = sy + c.y;
  return Pt{sx / 3., sy / 3.};
}

inline double tri_area(Pt p0, Pt p1, Pt p2) {
  double t0 = p0.x * (p1.y - p2.y);
  double t1 = p1.x * (p2.y - p0.y);
  double t2 = p2.x * (p0.y - p1.y);
  double s = t0 + t1;
  s = s + t2;
  return 0.5 * std::fabs(s);
}

// Face selection shared by the shallow-water and Poisson assemblies: for the
// directed edge src -> dst, pick the face of the src triangle that the dst
// centroid lies beyond (assemble_shallow_water.py:199-223,
// assemble_poisson.py:174-192).  Outputs the selected normal and alpha.
struct FaceSel {
  double nx, ny, alpha;
};

inline FaceSel select_face(const Pt sp[3], Pt sc, Pt dc, bool want_alpha) {
  static const int kA[3] = {2, 0, 1};  // third vertex of faces 01, 12, 20
  static const int kB[3] = {0, 1, 2};
  static const int kC[3] = {1, 2, 0};
  FaceSel out{0., 0., 0.};
  for (int f = 0; f < 3; ++f) {
    Pt own = face_normal(sp[kA[f]], sp[kB[f]], sp[kC[f]]);
    Pt dstn = face_normal(dc, sp[kB[f]], sp[kC[f]]);
    double dot = own.x * dstn.x + own.y * dstn.y;
    if (dot < 0) {
      out.nx = own.x;
      out.ny = own.y;
      if (want_alpha) out.alpha = line_alpha(sc, dc, sp[kB[f]], sp[kC[f]]);
    }
  }
  return out;
}

}  // namespace

extern "C" int esr_mesh_sizes(int64_t n, int64_t *nc, int64_t *ne,
                              int64_t *nbc, int64_t *np) {
  if (n < 1 || n > (int64_t)1 << 20) return esr::fail(ESR_ERR_ARG, "mesh size n out of range");
  if (nc) *nc = 4 * n * n;
  if (ne) *ne = 12 * n * n - 4 * n;
  if (nbc) *nbc = 4 * n;
  if (np) *np = (n + 1) * (n + 1) + n * n;
  return ESR_OK;
}

// Unit-square mesh, 4 triangles per square around the square's centre.
// Index layout identical to csrc/triangular_mesh.cpp:10-143 (get_mesh).
// The reference writes shared corner points once per adjacent square inside
// an OpenMP loop; the coordinates here are the ones its sequential order
// leaves behind (the last square to touch a corner wins).
extern "C" int esr_mesh_triangular(int64_t n, int64_t *src, int64_t *dst,
                                   int64_t *cells, int64_t *bcells,
                                   int64_t *bpoints, double *points) {
  ESR_HOST_TRY
  int64_t nc, ne, nbc, np;
  int st = esr_mesh_sizes(n, &nc, &ne, &nbc, &np);
  if (st) return st;
  if (!src || !dst || !cells || !bcells || !bpoints || !points)
    return esr::fail(ESR_ERR_ARG, "esr_mesh_triangular: null output");
  const double d = 1. / n;
  const int64_t ncorner = (n + 1) * (n + 1);

  // corner points: (i, j) -> j*(n+1) + i
  for (int64_t j = 0; j <= n; ++j) {
    for (int64_t i = 0; i <= n; ++i) {
      double x, y;
      if (i < n) x = i * d; else x = (n - 1) * d + d;
      if (j < n) y = j * d; else y = (n - 1) * d + d;
      points[2 * (j * (n + 1) + i)] = x;
      points[2 * (j * (n + 1) + i) + 1] = y;
    }
  }
  // square centres
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < n; ++i) {
      int64_t c = ncorner + n * j + i;
      points[2 * c] = i * d + d / 2;
      points[2 * c + 1] = j * d + d / 2;
    }
  }

  const int64_t base = 8 * n * n;
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < n; ++i) {
      const int64_t sq = i + j * n;
      const int64_t c0 = 4 * sq;
      const int64_t bl = j * (n + 1) + i;        // bottom-left corner
      const int64_t tl = (j + 1) * (n + 1) + i;  // top-left
      const int64_t tr = tl + 1;                 // top-right
      const int64_t br = bl + 1;                 // bottom-right
      const int64_t ce = ncorner + n * j + i;    // centre
      const int64_t tri[4][3] = {{bl, br, ce}, {tr, ce, br}, {tr, tl, ce}, {bl, ce, tl}};
      for (int k = 0; k < 4; ++k)
        for (int v = 0; v < 3; ++v) cells[3 * (c0 + k) + v] = tri[k][v];

      // the 8 directed edges between the 4 triangles of this square
      for (int64_t k = 0; k < 4; ++k) {
        int64_t a = c0 + k, b = c0 + (k + 1) % 4;
        src[8 * sq + 2 * k] = a;
        dst[8 * sq + 2 * k] = b;
        src[8 * sq + 2 * k + 1] = b;
        dst[8 * sq + 2 * k + 1] = a;
      }
      // towards the square below (or the bottom wall)
      if (j > 0) {
        int64_t e = base + n * (j - 1) + i;
        src[e] = c0;
        dst[e] = c0 - 4 * n + 2;
      } else {
        bcells[i] = c0;
        bpoints[2 * i] = bl;
        bpoints[2 * i + 1] = br;
      }
      // towards the square above (or the top wall)
      if (j < n - 1) {
        int64_t e = base + n * (n - 1) + n * j + i;
        src[e] = c0 + 2;
        dst[e] = c0 + 4 * n;
      } else {
        bcells[n + i] = c0 + 2;
        bpoints[2 * (n + i)] = tl;
        bpoints[2 * (n + i) + 1] = tr;
      }
      // towards the square on the left (or the left wall)
      if (i > 0) {
        int64_t e = base + 2 * n * (n - 1) + (n - 1) * j + i - 1;
        src[e] = c0 + 3;
        dst[e] = c0 - 3;
      } else {
        bcells[2 * n + j] = c0 + 3;
        bpoints[2 * (2 * n + j)] = bl;
        bpoints[2 * (2 * n + j) + 1] = tl;
      }
      // towards the square on the right (or the right wall)
      if (i < n - 1) {
        int64_t e = base + 3 * n * (n - 1) + (n - 1) * j + i;
        src[e] = c0 + 1;
        dst[e] = c0 + 7;
      } else {
        bcells[3 * n + j] = c0 + 1;
        bpoints[2 * (3 * n + j)] = tr;
        bpoints[2 * (3 * n + j) + 1] = br;
      }
    }
  }
  return ESR_OK;
  ESR_HOST_CATCH
}

static int check_mesh_args(int64_t nc, int64_t ne, int64_t nbc, const int64_t *src,
                           const int64_t *dst, const int64_t *cells,
                           const int64_t *bcells, const int64_t *bpoints,
                           const double *points) {
  if (nc <= 0 || ne < 0 || nbc < 0) return esr::fail(ESR_ERR_ARG, "negative mesh size");
  if (!src || !dst || !cells || !points || (nbc && (!bcells || !bpoints)))
    return esr::fail(ESR_ERR_ARG, "null mesh array");
  for (int64_t e = 0; e < ne; ++e)
    if (src[e] < 0 || src[e] >= nc || dst[e] < 0 || dst[e] >= nc)
      return esr::fail(ESR_ERR_ARG, "edge index out of range");
  for (int64_t b = 0; b < nbc; ++b)
    if (bcells[b] < 0 || bcells[b] >= nc) return esr::fail(ESR_ERR_ARG, "bcells out of range");
  return ESR_OK;
}

extern "C" int esr_swe_geometry(int64_t nc, int64_t ne, int64_t nbc,
                                const int64_t *src, const int64_t *dst,
                                const int64_t *cells, const int64_t *bcells,
                                const int64_t *bpoints, const double *points,
                                double *sx, double *sy, double *alpha,
                                double *area, double *x, double *y,
                                double *bsx, double *bsy) {
  ESR_HOST_TRY
  int st = check_mesh_args(nc, ne, nbc, src, dst, cells, bcells, bpoints, points);
  if (st) return st;
  // per cell: centroid and area (assemble_shallow_water.py:225-240)
  std::vector<Pt> cent(nc);
  for (int64_t c = 0; c < nc; ++c) {
    Pt p0 = pt_at(points, cells[3 * c]);
    Pt p1 = pt_at(points, cells[3 * c + 1]);
    Pt p2 = pt_at(points, cells[3 * c + 2]);
    area[c] = tri_area(p0, p1, p2);
    cent[c] = centroid3(p0, p1, p2);
    x[c] = cent[c].x;
    y[c] = cent[c].y;
  }
  // per edge: face normal of the src triangle towards dst, and alpha
  // (assemble_shallow_water.py:186-223)
  for (int64_t e = 0; e < ne; ++e) {
    const int64_t s = src[e], t = dst[e];
    Pt sp[3] = {pt_at(points, cells[3 * s]), pt_at(points, cells[3 * s + 1]),
                pt_at(points, cells[3 * s + 2])};
    Pt dp0 = pt_at(points, cells[3 * t]), dp1 = pt_at(points, cells[3 * t + 1]),
       dp2 = pt_at(points, cells[3 * t + 2]);
    Pt sc = centroid3(sp[0], sp[1], sp[2]);
    Pt dc = centroid3(dp0, dp1, dp2);
    FaceSel f = select_face(sp, sc, dc, true);
    sx[e] = f.nx;
    sy[e] = f.ny;
    alpha[e] = f.alpha;
  }
  // boundary faces (assemble_shallow_water.py:246-253)
  for (int64_t b = 0; b < nbc; ++b) {
    Pt bp0 = pt_at(points, bpoints[2 * b]);
    Pt bp1 = pt_at(points, bpoints[2 * b + 1]);
    Pt bn = face_normal(cent[bcells[b]], bp0, bp1);
    bsx[b] = -bn.x;
    bsy[b] = -bn.y;
  }
  return ESR_OK;
  ESR_HOST_CATCH
}

extern "C" int esr_poisson_fv_assemble(int64_t nc, int64_t ne, int64_t nbc,
                                       const int64_t *src, const int64_t *dst,
                                       const int64_t *cells,
                                       const int64_t *bcells,
                                       const int64_t *bpoints,
                                       const double *points, double *Af,
                                       double *Ac, double *b, double *rho,
                                       double *centroid) {
  ESR_HOST_TRY
  int st = check_mesh_args(nc, ne, nbc, src, dst, cells, bcells, bpoints, points);
  if (st) return st;
  std::vector<Pt> cent(nc);
  std::vector<double> area(nc);
  for (int64_t c = 0; c < nc; ++c) {
    Pt p0 = pt_at(points, cells[3 * c]);
    Pt p1 = pt_at(points, cells[3 * c + 1]);
    Pt p2 = pt_at(points, cells[3 * c + 2]);
    area[c] = tri_area(p0, p1, p2);
    cent[c] = centroid3(p0, p1, p2);
    centroid[2 * c] = cent[c].x;
    centroid[2 * c + 1] = cent[c].y;
  }
  // Af per edge (assemble_poisson.py:161-195)
  for (int64_t e = 0; e < ne; ++e) {
    const int64_t s = src[e], t = dst[e];
    Pt sp[3] = {pt_at(points, cells[3 * s]), pt_at(points, cells[3 * s + 1]),
                pt_at(points, cells[3 * s + 2])};
    Pt dp0 = pt_at(points, cells[3 * t]), dp1 = pt_at(points, cells[3 * t + 1]),
       dp2 = pt_at(points, cells[3 * t + 2]);
    Pt sc = centroid3(sp[0], sp[1], sp[2]);
    Pt dc = centroid3(dp0, dp1, dp2);
    double distx = dc.x - sc.x, disty = dc.y - sc.y;
    FaceSel f = select_face(sp, sc, dc, false);
    double d2 = distx * distx + disty * disty;
    double ux = distx / d2, uy = disty / d2;
    Af[e] = ux * f.nx + uy * f.ny;
  }
  // Ac = -reducer(Af), reducer idx = src, in-order segment sums
  // (assemble_poisson.py:91, 196); rows never referenced stay 0 -> -0 = -0.
  std::vector<double> acc(nc, 0.0);
  std::vector<char> hit(nc, 0);
  for (int64_t e = 0; e < ne; ++e) {
    acc[src[e]] = acc[src[e]] + Af[e];
    hit[src[e]] = 1;
  }
  for (int64_t c = 0; c < nc; ++c) Ac[c] = -acc[c];
  // rho and b (assemble_poisson.py:212-216)
  for (int64_t c = 0; c < nc; ++c) {
    double dx = cent[c].x - 0.5, dy = cent[c].y - 0.5;
    double r2 = dx * dx + dy * dy;
    rho[c] = std::exp(-200.0 * r2);
    b[c] = rho[c] * area[c];
  }
  // boundary term (assemble_poisson.py:219-230)
  std::vector<double> bacc(nc, 0.0);
  for (int64_t k = 0; k < nbc; ++k) {
    Pt bp0 = pt_at(points, bpoints[2 * k]);
    Pt bp1 = pt_at(points, bpoints[2 * k + 1]);
    Pt cc = cent[bcells[k]];
    Pt fc{(bp0.x + bp1.x) / 2., (bp0.y + bp1.y) / 2.};
    Pt bn = face_normal(cc, bp0, bp1);
    double dx = fc.x - cc.x, dy = fc.y - cc.y;
    double d2 = dx * dx + dy * dy;
    double ux = dx / d2, uy = dy / d2;
    double v = ux * bn.x + uy * bn.y;
    bacc[bcells[k]] = bacc[bcells[k]] + v;
  }
  for (int64_t c = 0; c < nc; ++c) Ac[c] = Ac[c] - bacc[c];
  (void)hit;
  return ESR_OK;
  ESR_HOST_CATCH
}

// ---------------------------------------------------------------------------
// P1 finite elements on the n x n square grid, 2 right triangles per square
// split along the (i,j)-(i+1,j+1) diagonal, zero Dirichlet boundary.
// Element stiffness of a right isosceles triangle with right-angle vertex R
// and the other vertices A, B (any leg length, 2-D):
//   K_RR = k, K_AA = K_BB = k/2, K_RA = K_RB = -k/2, K_AB = 0.
// ---------------------------------------------------------------------------
extern "C" int esr_p1_sizes(int64_t n, int64_t *nunk, int64_t *nnz_off) {
  if (n < 2 || n > 65536) return esr::fail(ESR_ERR_ARG, "P1 grid size out of range");
  int64_t m = n - 1;  // interior nodes per side
  if (nunk) *nunk = m * m;
  // directed couplings: W/E pairs, S/N pairs, SW/NE pairs
  if (nnz_off) *nnz_off = 2 * (m * (m - 1)) * 2 + 2 * (m - 1) * (m - 1);
  return ESR_OK;
}

extern "C" int esr_p1_assemble(int64_t n, const double *kappa, int64_t *row,
                               int64_t *col, double *Ae, double *Av) {
  ESR_HOST_TRY
  int64_t nunk, nnz;
  int st = esr_p1_sizes(n, &nunk, &nnz);
  if (st) return st;
  if (!row || !col || !Ae || !Av) return esr::fail(ESR_ERR_ARG, "esr_p1_assemble: null output");
  const int64_t m = n - 1;
  auto kap = [&](int64_t i, int64_t j, int up) -> double {
    return kappa ? kappa[2 * (j * n + i) + up] : 1.0;
  };
  // Stencil per node (i, j), 1 <= i, j <= n-1:
  //   diag  = sum over the 6 incident triangles of their K_vv
  //   W/E/S/N couplings = -(k_t1 + k_t2)/2 over the two triangles sharing
  //   the leg; SW/NE (hypotenuse) = 0.
  // Accumulate in a fixed order so the values are reproducible.
  int64_t k = 0;
  for (int64_t j = 1; j <= m; ++j) {
    for (int64_t i = 1; i <= m; ++i) {
      const int64_t u = (j - 1) * m + (i - 1);
      // incident triangles:
      //  square (i-1, j-1): upper? node (i,j) is its top-right corner ->
      //     lower tri {(i-1,j-1),(i,j-1),(i,j)}: node is A/B (k/2)
      //     upper tri {(i-1,j-1),(i,j),(i-1,j)}: node is A/B (k/2)
      //  square (i, j-1): node is its top-left corner -> upper tri
      //     {(i,j-1),(i+1,j),(i,j)}, right angle at (i,j): R (k)
      //  square (i-1, j): node is its bottom-right corner -> lower tri
      //     {(i-1,j),(i,j),(i,j+1)}, right angle at (i,j): R (k)
      //  square (i, j): node is its bottom-left corner ->
      //     lower {(i,j),(i+1,j),(i+1,j+1)}: A/B (k/2)
      //     upper {(i,j),(i+1,j+1),(i,j+1)}: A/B (k/2)
      double kl_sw = kap(i - 1, j - 1, 0), ku_sw = kap(i - 1, j - 1, 1);
      double ku_s = kap(i, j - 1, 1);
      double kl_w = kap(i - 1, j, 0);
      double kl_c = kap(i, j, 0), ku_c = kap(i, j, 1);
      double diag = kl_sw / 2;
      diag = diag + ku_sw / 2;
      diag = diag + ku_s;
      diag = diag + kl_w;
      diag = diag + kl_c / 2;
      diag = diag + ku_c / 2;
      Av[u] = diag;
      // couplings, ascending column: SW, S, W, E, N, NE
      // S edge (i,j)-(i,j-1): lower tri of square (i-1,j-1) [right angle at
      //   (i,j-1)] and upper tri of square (i,j-1) [right angle at (i,j)]
      double cS = -(kl_sw + ku_s) / 2;
      // W edge (i,j)-(i-1,j): upper tri of square (i-1,j-1) [right angle at
      //   (i-1,j)] and lower tri of square (i-1,j) [right angle at (i,j)]
      double cW = -(ku_sw + kl_w) / 2;
      // E edge (i,j)-(i+1,j): lower tri of square (i,j) [R at (i+1,j)] and
      //   upper tri of square (i,j-1) [R at (i,j)]
      double cE = -(kl_c + ku_s) / 2;
      // N edge (i,j)-(i,j+1): upper tri of square (i,j) [R at (i,j+1)] and
      //   lower tri of square (i-1,j) [R at (i,j)]
      double cN = -(ku_c + kl_w) / 2;
      struct {
        int64_t di, dj;
        double v;
      } nb[6] = {{-1, -1, 0.0}, {0, -1, cS}, {-1, 0, cW}, {1, 0, cE}, {0, 1, cN}, {1, 1, 0.0}};
      for (int q = 0; q < 6; ++q) {
        int64_t ii = i + nb[q].di, jj = j + nb[q].dj;
        if (ii < 1 || ii > m || jj < 1 || jj > m) continue;
        row[k] = u;
        col[k] = (jj - 1) * m + (ii - 1);
        Ae[k] = nb[q].v;
        ++k;
      }
    }
  }
  if (k != nnz) return esr::fail(ESR_ERR_ARG, "P1 assembly count mismatch");
  return ESR_OK;
  ESR_HOST_CATCH
}
