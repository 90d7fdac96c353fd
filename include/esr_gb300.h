/*
 * esr_gb300.h -- C ABI of the GB300 (sm_103a) sparse-mesh hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns an int status (ESR_OK == 0).  On a non-zero status,
 * esr_last_error() returns a message for the calling host thread.
 *
 * Device entry points are stream-ordered on the caller's `stream`
 * (a cudaStream_t passed as void*; NULL = legacy default stream) and never
 * synchronise the host.  The library never allocates device memory: any
 * scratch a kernel needs is passed in by the caller, sized by the matching
 * *_workspace_bytes() query.
 *
 * Index arrays on the device are int32 (the reference stores int64; the host
 * side narrows them once, after checking every value fits).
 *
 * Citations name the reference function each entry point replaces
 * (paths relative to the EASIER source tree).
 */
#ifndef ESR_GB300_H
#define ESR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ESR_GB300_ABI_VERSION 11

/* element types */
enum {
  ESR_F32 = 0,
  ESR_F64 = 1,
  ESR_I32 = 2,
  ESR_I64 = 3
};

/* Reducer reduce ops: easier/core/module.py:386 (ReduceOp) */
enum {
  ESR_REDUCE_SUM = 0,
  ESR_REDUCE_PROD = 1,
  ESR_REDUCE_MEAN = 2,
  ESR_REDUCE_AMAX = 3,
  ESR_REDUCE_AMIN = 4
};

/* aggregators: easier/core/module.py:825-884 (sum, prod, norm, max, min) */
enum {
  ESR_AGG_SUM = 0,
  ESR_AGG_PROD = 1,
  ESR_AGG_NORM = 2,
  ESR_AGG_MAX = 3,
  ESR_AGG_MIN = 4
};

/* status codes */
enum {
  ESR_OK = 0,
  ESR_ERR_ARG = 1,        /* bad argument (size, dtype, null pointer)      */
  ESR_ERR_CUDA = 2,       /* a CUDA runtime call or launch failed          */
  ESR_ERR_DEVICE = 3,     /* a kernel reported an error (e.g. idx range)   */
  ESR_ERR_UNSUPPORTED = 4 /* shape/type combination not implemented        */
};

/* device-side error bits, OR-ed into the library's device status word */
enum {
  ESR_DEV_IDX_RANGE = 1,  /* an index was outside [0, n_in)                */
  ESR_DEV_NONFINITE = 2,  /* a solver produced NaN/Inf                     */
  ESR_DEV_WAIT_TIMEOUT = 4 /* a bounded device wait gave up                */
};

const char *esr_last_error(void);
int esr_abi_version(void);

/* Read (and optionally clear) the device status word of the current device.
 * Synchronises `stream` first. */
int esr_device_status(int *status_out, int clear, void *stream);

/* ------------------------------------------------------------------------ *
 * Host-side mesh, geometry and ordering (integer work is bit-exact).
 * ------------------------------------------------------------------------ */

/* Sizes of the unit-square triangular mesh with 4 triangles per square.
 * Replaces csrc/triangular_mesh.cpp:10-16 (get_mesh size formulas). */
int esr_mesh_sizes(int64_t n, int64_t *nc, int64_t *ne, int64_t *nbc,
                   int64_t *np);

/* Unit-square triangular mesh: src/dst [ne], cells [nc*3], bcells [nbc],
 * bpoints [nbc*2], points [np*2].  Index-for-index identical to
 * csrc/triangular_mesh.cpp:10-143 (get_mesh). */
int esr_mesh_triangular(int64_t n, int64_t *src, int64_t *dst, int64_t *cells,
                        int64_t *bcells, int64_t *bpoints, double *points);

/* Shallow-water geometry: per edge sx, sy, alpha [ne]; per cell area, x, y
 * [nc]; per boundary face bsx, bsy [nbc].  Same operation order as
 * tutorial/shallow_water_equation/assemble_shallow_water.py:154-253
 * (ShallowWaterInitializer.get_alpha/get_face_norm/forward), so the values
 * are bit-identical to the reference's CPU run. */
int esr_swe_geometry(int64_t nc, int64_t ne, int64_t nbc, const int64_t *src,
                     const int64_t *dst, const int64_t *cells,
                     const int64_t *bcells, const int64_t *bpoints,
                     const double *points, double *sx, double *sy,
                     double *alpha, double *area, double *x, double *y,
                     double *bsx, double *bsy);

/* Cell-centred finite-volume Poisson assembly: Af [ne], Ac, b, rho [nc],
 * centroid [nc*2].  Follows tutorial/poisson/assemble_poisson.py:160-230
 * (PoissonInitializer.forward); Ac uses an in-order segment sum like the
 * reference's Reducer. */
int esr_poisson_fv_assemble(int64_t nc, int64_t ne, int64_t nbc,
                            const int64_t *src, const int64_t *dst,
                            const int64_t *cells, const int64_t *bcells,
                            const int64_t *bpoints, const double *points,
                            double *Af, double *Ac, double *b, double *rho,
                            double *centroid);

/* esr_mesh_triangular on the GPU: every array device memory, stream-ordered
 * on `stream`; one thread per point and per square.  Index for index and
 * bit for bit the host generator's (csrc/triangular_mesh.cpp:10-143,
 * get_mesh). */
int esr_mesh_triangular_device(int64_t n, int64_t *src, int64_t *dst,
                               int64_t *cells, int64_t *bcells,
                               int64_t *bpoints, double *points, void *stream);

/* esr_swe_geometry on the GPU (device arrays; np = number of points): one
 * thread per cell, edge and wall face, the reference's operation order one
 * IEEE operation at a time, so bit for bit the host's values
 * (assemble_shallow_water.py:154-253).  An index out of range sets
 * ESR_DEV_IDX_RANGE and leaves that entry unwritten. */
int esr_swe_geometry_device(int64_t nc, int64_t ne, int64_t nbc, int64_t np,
                            const int64_t *src, const int64_t *dst,
                            const int64_t *cells, const int64_t *bcells,
                            const int64_t *bpoints, const double *points,
                            double *sx, double *sy, double *alpha,
                            double *area, double *x, double *y, double *bsx,
                            double *bsy, void *stream);

/* esr_poisson_fv_assemble on the GPU (device arrays), given the stable CSR
 * of src (rowptr [nc+1], perm [ne]) and of bcells (brow [nc+1], bperm
 * [nbc]), int32: the in-order sums of the reference's Reducer.  Af, Ac and
 * centroid bit for bit the host's; rho and b go through CUDA's exp (within
 * a few ulp).  assemble_poisson.py:160-230. */
int esr_poisson_fv_assemble_device(int64_t nc, int64_t ne, int64_t nbc,
                                   int64_t np, const int64_t *src,
                                   const int64_t *dst, const int64_t *cells,
                                   const int64_t *bcells,
                                   const int64_t *bpoints,
                                   const double *points,
                                   const int32_t *rowptr, const int32_t *perm,
                                   const int32_t *brow, const int32_t *bperm,
                                   double *Af, double *Ac, double *b,
                                   double *rho, double *centroid,
                                   void *stream);

/* Sizes of the P1 finite-element Poisson system on an n x n square grid
 * split into 2 right triangles per square (diagonal (i,j)-(i+1,j+1)), zero
 * Dirichlet boundary: unknowns = (n-1)^2 interior nodes, nnz_off = number
 * of directed off-diagonal couplings (6 per interior node minus the ones
 * that reach the boundary). */
int esr_p1_sizes(int64_t n, int64_t *nunk, int64_t *nnz_off);

/* P1 stiffness in Linsys form (easier/numeric/linsys.py:10-24): row/col
 * [nnz_off] (row sorted ascending, the Reducer/Selector idx), Ae [nnz_off]
 * off-diagonal values, Av [nunk] diagonal.  kappa [2*n*n] is the
 * per-triangle coefficient (lower triangle of square (i,j) at 2*(j*n+i),
 * upper at 2*(j*n+i)+1); NULL means kappa = 1.  No reference counterpart
 * (the reference ships only the FV discretisation). */
int esr_p1_assemble(int64_t n, const double *kappa, int64_t *row, int64_t *col,
                    double *Ae, double *Av);

/* Stable counting sort of idx[m] (values in [0, n)): rowptr [n+1] and
 * perm [m] with perm[k] = original position of the k-th element in
 * ascending-key, original-order-within-key order.  This is the edge order
 * the reference's reorder produces at world size 1:
 * easier/core/passes/sparse_encoding/sparse_encoding.py:244-338
 * (reorder_input_by_reducer) + easier/core/passes/utils.py:301-336
 * (zipsort_using_order, stable=True).  Returns ESR_ERR_ARG if any value is
 * out of range (easier/core/passes/collective_initialization.py:76-106). */
int esr_csr_from_index(const int64_t *idx, int64_t m, int64_t n,
                       int64_t *rowptr, int64_t *perm);

/* Reverse Cuthill-McKee ordering of an undirected graph given by directed
 * edge lists (both directions need not be present; self loops ignored).
 * order[k] = old vertex placed at new position k.  Deterministic: start of
 * each component = pseudo-peripheral vertex found from the lowest-degree,
 * lowest-index unvisited vertex; neighbours visited by (degree, index). */
int esr_rcm_order(int64_t n, int64_t m, const int64_t *src, const int64_t *dst,
                  int64_t *order);

/* ------------------------------------------------------------------------ *
 * Selector / Reducer / aggregators (device).
 * ------------------------------------------------------------------------ */

/* y[e, :] = x[idx[e], :] for e in [0, m); a row is row_bytes bytes.
 * Replaces easier/core/module.py:364-371 (Selector.forward).  Indices out
 * of [0, n_in) set ESR_DEV_IDX_RANGE in the device status word and that row
 * is left unwritten. */
int esr_gather(const void *x, int64_t n_in, int64_t row_bytes,
               const int32_t *idx, int64_t m, void *y, void *stream);

/* Deterministic segmented reduce over a CSR segmentation:
 *   out[i, c] = op over k in [rowptr[i], rowptr[i+1]) of t[perm ? perm[k] : k, c]
 * in ascending k (the reference's in-segment edge order).  Rows with an empty
 * segment keep `out` unchanged (scatter_reduce_ with include_self=False).
 * Replaces easier/core/module.py:441-461 (Reducer.forward).
 * dtype: ESR_F32/F64/I32/I64; op: ESR_REDUCE_*. */
int esr_segreduce(int dtype, int op, const void *t, int64_t row_elems,
                  const int32_t *rowptr, const int32_t *perm, int64_t n,
                  void *out, void *stream);

/* Bytes of scratch esr_aggregate needs for an [n, cols] input. */
int64_t esr_aggregate_workspace_bytes(int64_t n, int64_t cols);

/* out[c] = agg over rows r of t[r, c] (dim 0, keepdim).  Floating inputs
 * accumulate in FP64 with a fixed two-level tree (deterministic); the
 * result is stored in the input dtype.  Replaces the local part of
 * easier/core/module.py:825-884 (esr.sum/prod/norm/max/min); at world size
 * 1 the allgather that dataflow_distribution.py:197-289 inserts is the
 * identity, so this is the whole aggregator. */
int esr_aggregate(int dtype, int agg, const void *t, int64_t n, int64_t cols,
                  void *out, void *workspace, void *stream);

/* Aggregate that allocates nothing and takes no workspace: same result,
 * bit for bit, as esr_aggregate.  No counterpart in the reference.  Meant
 * for callers that cannot call cudaMalloc where they aggregate (it
 * synchronises the device, can fail mid-run, or the host application owns
 * all device memory).  Its scratch is a static 1 MiB device array per
 * device, kept until the process exits; sizes needing more
 * (esr_aggregate_workspace_bytes(n, cols) > ESR_AGG_NOALLOC_SCRATCH_BYTES;
 * every cols <= ESR_AGG_NOALLOC_MAX_COLS fits) are rejected with
 * ESR_ERR_ARG.  The first call in a CUDA context looks up the array's
 * address in that context (make that call before any stream capture); the
 * address is kept with the context's unique ID, so a call after
 * cudaDeviceReset, or under another context of the same device, looks it
 * up again instead of using a stale one.  All calls share the array:
 * calls that overlap on the GPU (different streams, no ordering) race. */
#define ESR_AGG_NOALLOC_SCRATCH_BYTES (1 << 20)
#define ESR_AGG_NOALLOC_MAX_COLS 64
int esr_aggregate_noalloc(int dtype, int agg, const void *t, int64_t n,
                          int64_t cols, void *out, void *stream);

/* Bytes of scratch esr_dot needs for length-n vectors. */
int64_t esr_dot_workspace_bytes(int64_t n);

/* out_f64[0] = sum_i a[i]*b[i], FP64 accumulation, fixed tree order.
 * The CG dot product (easier/numeric/solver/cg.py:70-71, 92). */
int esr_dot(int dtype, const void *a, const void *b, int64_t n,
            double *out_f64, void *workspace, void *stream);

/* ------------------------------------------------------------------------ *
 * Fused shallow-water step (ELL face-slot layout, see esr_swe_mesh).
 * ------------------------------------------------------------------------ */

/* Face-slot mesh: every cell has `width` face slots stored slot-major
 * ([slot][cell]).  nbr = neighbour cell (>= 0, an interior edge
 * src -> this cell), -1 = boundary face, -2 = empty.  Interior slots come
 * first, in the reference's edge order; then boundary faces.  For an
 * interior slot sx/sy/alpha are the edge's values; for a boundary slot
 * sx/sy hold bsx/bsy and alpha is unused. */
typedef struct {
  int64_t nc;
  int32_t width;     /* 3 or 4 */
  int32_t dtype;     /* ESR_F32 or ESR_F64 (of sx/sy/alpha/area) */
  const int32_t *nbr;
  const void *sx;
  const void *sy;
  const void *alpha;
  const void *area;
  const void *inv_area; /* 1/area, used when exact == 0 (may be NULL otherwise) */
  int32_t exact;     /* 1: bitwise the reference; 0: fast arithmetic (see esr_swe_step) */
  int32_t pad_;
} esr_swe_mesh;

/* Scratch bytes for esr_swe_step: two stage states + one accumulator, each
 * nc x 4 elements. */
int64_t esr_swe_workspace_bytes(const esr_swe_mesh *mesh);

/* `steps` explicit steps of the reference scheme
 * (tutorial/shallow_water_equation/swe_main.py:86-141: face_reconstruct,
 * delta, forward with stage weights 1/6 each) on the cell state
 * `state` [nc][4] = (h, uh, vh, unused), updated in place.
 * With mesh->exact, every floating operation is issued in the reference's
 * order with round-to-nearest and no contraction, so FP64/FP32 results are
 * bitwise those of the reference's CPU backend on the same (reordered)
 * inputs.  With exact == 0 the same formulas run with FMA contraction, one
 * reciprocal per face for u = uh/h, v = vh/h and a multiply by inv_area
 * (fewer instructions; FP32 within 1e-5, FP64 within 1e-10 relative of the
 * reference after 1,000 steps). */
int esr_swe_step(const esr_swe_mesh *mesh, double dt, void *state,
                 int64_t steps, void *workspace, void *stream);

/* One `delta` evaluation (swe_main.py:90-119) on state [nc][4]; writes
 * delta [nc][4] = (delta_h, delta_uh, delta_vh, 0). */
int esr_swe_delta(const esr_swe_mesh *mesh, const void *state, void *delta,
                  void *stream);

/* Temporally blocked layout of the same step (FP32, 3 face slots per
 * cell).  Cells are numbered tile-major: tile t owns cells
 * [cell_off, cell_off + n0).  Its local list is the tile followed by the
 * rings of in-neighbours at distance 1..4 (the cells a 4-stage step of the
 * tile depends on), sorted by ring: local j < n1 are levels <= 1, j < n2
 * levels <= 2, j < n3 levels <= 3, j < nL all.  Per tile:
 *   meta[8t..8t+5] = cell_off, n0, n1, n2, n3, nL
 *   halo[offh[t] + j - n0] = global cell of local j >= n0
 *   per local cell j < n3 and slot k: slots[3*off3[t] + k*n3 + j] = one
 *   16-byte record {float sx, float sy, float alpha, int32 lnbr} (lnbr =
 *   local index of the neighbour, -1 wall, -2 empty; one vector load per
 *   face), area[off3[t] + j].  With exact == 0 the records hold sx / area
 *   and sy / area of their cell (the fluxes are linear in sx, sy) and
 *   area / inv_area are not read.
 * Limits: n0 <= 4096, n3 <= 6144, 12*nL + 24*n3 bytes <= 227 KB. */
typedef struct {
  int64_t nc;
  int32_t ntiles;
  int32_t dtype;     /* ESR_F32 */
  int32_t max_local; /* max nL */
  int32_t max_l3;    /* max n3 */
  int32_t max_own;   /* max n0 */
  int32_t max_halo3; /* max n3 - n0 (informational; not read) */
  const int32_t *meta;
  const int64_t *off3;
  const int64_t *offh;
  const int32_t *halo;
  const void *slots;  /* 16-byte aligned face-slot records, see above */
  const void *area;     /* [sum(n3)], read when exact != 0 */
  const void *inv_area; /* not read (reserved) */
  int32_t exact;        /* as in esr_swe_mesh */
  int32_t slot_info;    /* 1: no cell has more than one wall or empty face
                         * slot, so with exact == 0 (each cell's records
                         * sorted by lnbr) slots 1 and 2 are interior
                         * faces; else 0.  The pipelined kernel needs 1. */
} esr_swe_tiles;

/* Shared memory one CTA of esr_swe_tile_step uses, or -1 if the layout is
 * outside the limits. */
int64_t esr_swe_tile_smem_bytes(const esr_swe_tiles *tiles);

/* Threads per CTA esr_swe_tile_step launches for this layout (1024, 512 or
 * 256, with 1024 / threads CTAs resident per SM), or -1 if the layout is
 * outside the limits. */
int esr_swe_tile_threads(const esr_swe_tiles *tiles);

/* `steps` steps of swe_main.py:121-141, one launch per step; with exact != 0
 * bitwise equal to esr_swe_step (exact), else within rounding of it.  Step k reads buffer k%2 and writes the other
 * ([nc][4] FP32 each, tile-major numbering): the result is in state_a when
 * `steps` is even, in state_b when odd. */
int esr_swe_tile_step(const esr_swe_tiles *tiles, double dt, void *state_a,
                      void *state_b, int64_t steps, void *stream);

/* The two kernels behind esr_swe_tile_step, same results bit for bit:
 *   BLOCKED: one CTA per tile (1024, 512 or 256 threads), the face records
 *     read from global memory in every stage; any layout within the limits
 *     above, exact or fast arithmetic;
 *   PIPELINED: fast arithmetic only; one persistent CTA per SM, each
 *     thread's tile-cell face records held in registers through the four
 *     stages, the next tile's state copied into shared memory (cp.async)
 *     and its records prefetched into L2 while the current tile computes,
 *     cells (tile and halo alike) assigned round-robin and computed in
 *     pairs with packed FP32x2 arithmetic.  Two CTA shapes, by the cells a
 *     thread keeps in registers: PIPELINED_512 (512 threads x 4 cells,
 *     n0 <= 2048) and PIPELINED_768 (768 threads x 2, n0 <= 1536); cells
 *     of level <= 3 past those read their records per stage.  PIPELINED is
 *     the 512-thread shape.  Needs nL <= 4096 in every tile and
 *     slot_info == 1.
 * AUTO picks a pipelined shape when the layout allows it. */
#define ESR_SWE_TILE_AUTO 0
#define ESR_SWE_TILE_BLOCKED 1
#define ESR_SWE_TILE_PIPELINED 2
#define ESR_SWE_TILE_PIPELINED_512 3
#define ESR_SWE_TILE_PIPELINED_768 4

/* The kernel AUTO runs for this layout (BLOCKED, PIPELINED_512 or
 * PIPELINED_768), or -1 if the layout is outside the limits.  No reference
 * counterpart. */
int esr_swe_tile_kernel(const esr_swe_tiles *tiles);

/* esr_swe_tile_step on a chosen kernel (ESR_ERR_UNSUPPORTED if the layout
 * does not fit it).  No reference counterpart. */
int esr_swe_tile_step_with(const esr_swe_tiles *tiles, int kernel, double dt,
                           void *state_a, void *state_b, int64_t steps,
                           void *stream);

/* A shallow-water state held in host memory, stepped on the GPU (no
 * reference counterpart; the round trip of a user who keeps the state on
 * the host).  host_state is FP32 (h, uh, vh) [nc][3] in the tiled layout's
 * cell numbering (pinned memory for overlap).  Per step the state goes up
 * in `chunks` pieces (each unpacked into state_a, [nc] x 16 bytes, as it
 * lands), esr_swe_tile_step advances state_a into state_b, and each piece
 * is packed and brought back as soon as it is ready; a piece's upload for
 * the next step waits only for its own download, so uploads and downloads
 * share the host link in both directions.  staging: [nc][3] FP32 device
 * scratch.  tile_list (optional, [ntiles] int32 device scratch): when the
 * pipelined kernel takes the layout, the step itself overlaps the copies --
 * the tiles whose local cells all lie in the first g+1 chunks run as soon as
 * chunk g has landed, and a chunk goes home as soon as the tiles owning its
 * cells have run (results bitwise those of esr_swe_tile_step); the plan
 * reads the layout's meta, offh and halo back once to group the tiles.
 * The plan keeps a copy of *tiles (its arrays must outlive it) and owns two
 * copy streams and per-chunk events.  esr_swe_host_step returns with the
 * work enqueued: host_state holds the result once `stream` is
 * synchronised. */
int esr_swe_host_plan_create(const esr_swe_tiles *tiles, void *state_a,
                             void *state_b, void *staging, int32_t *tile_list,
                             int32_t chunks, void **plan_out);
int esr_swe_host_step(void *plan, double dt, float *host_state, int64_t steps,
                      void *stream);
int esr_swe_host_plan_destroy(void *plan);

/* Host: partition an undirected graph (directed edge lists) into parts of at
 * most max_part vertices by recursive BFS bisection: a set is ordered by
 * (BFS distance from the vertex farthest from its first vertex -- largest
 * distance, then smallest id --, id), unreached vertices last by id, and a
 * set due to end as k = ceil(size / max_part) parts keeps its first
 * size * floor(k/2) / k vertices on the left; ceil(n / max_part) compact
 * parts of nearly equal size, numbered depth first; part[v] in
 * [0, *nparts).  No reference counterpart. */
int esr_bisect_partition(int64_t n, int64_t m, const int64_t *src,
                         const int64_t *dst, int64_t max_part, int64_t *part,
                         int64_t *nparts);

/* Device: the same partition on the GPU, vertex for vertex (src, dst, part
 * device arrays; n and 2m below 2^31).  Workspace of
 * esr_bisect_device_workspace_bytes(n, m, max_part) bytes (-1: sizes out of
 * range).  Reads the error count and the largest degree back (synchronises
 * the stream once).  No reference counterpart. */
int64_t esr_bisect_device_workspace_bytes(int64_t n, int64_t m,
                                          int64_t max_part);
int esr_bisect_partition_device(int64_t n, int64_t m, const int64_t *src,
                                const int64_t *dst, int64_t max_part,
                                int32_t *part, int64_t *nparts,
                                void *workspace, int64_t workspace_bytes,
                                void *stream);

/* Host: the arrays of esr_swe_tiles from face slots nbr [3][nc] in a
 * tile-major numbering and the non-decreasing tile id of every cell.  Call
 * once with halo == NULL (fills meta [ntiles*8], *total_halo, *total_l3),
 * then with off3/offh [ntiles], halo [total_halo], lnbr/slot_src
 * [3*total_l3] and area_src [total_l3] allocated.  slot_src/area_src give
 * the source index of each tile slot in the [3][nc] face-slot arrays and in
 * the per-cell area array.  No reference counterpart. */
int esr_swe_tile_layout(int64_t nc, const int32_t *nbr, const int64_t *part,
                        int64_t ntiles, int32_t *meta, int64_t *total_halo,
                        int64_t *total_l3, int64_t *off3, int64_t *offh,
                        int32_t *halo, int32_t *lnbr, int64_t *slot_src,
                        int64_t *area_src);

/* ------------------------------------------------------------------------ *
 * Linsys SpMV and fused (P)CG.
 * ------------------------------------------------------------------------ */

/* SELL-32 form of Linsys (easier/numeric/linsys.py:23-24):
 *   y[i] = (sum_k x[col[k]] * val[k], k in row i, in order) + x[i] * diag[i].
 * Rows are grouped in slices of 32; slice s stores its entries slot-major:
 * entry (slot k, lane l) of slice s lives at slice_ptr[s] + 32*k + l and
 * belongs to row 32*s + l.  col = -1 marks padding.  Within a row the slots
 * keep the reference's edge order. */
typedef struct {
  int64_t n;                 /* rows (= columns)                        */
  int64_t nslots;            /* stored entries incl. padding            */
  int32_t dtype;             /* of val/diag: ESR_F32 or ESR_F64         */
  int32_t pad_;
  const int64_t *slice_ptr;  /* [ceil(n/32) + 1]                        */
  const int32_t *col;        /* [nslots]                                */
  const void *val;           /* [nslots]                                */
  const void *diag;          /* [n]                                     */
} esr_sell;

/* Host: SELL-32 layout of a Linsys.  rowptr/perm = esr_csr_from_index of
 * the Reducer idx (rows), colidx [m] = the Selector idx (columns, original
 * edge order).  Always fills slice_ptr; when col and src_pos are non-NULL
 * also fills col [nslots] and src_pos [nslots] (original edge index of each
 * slot, -1 for padding) so the caller can gather Ae into val.  Replaces the
 * layout work of easier/core/passes/sparse_encoding/sparse_encoding.py
 * :383-434 (rewrite_reducer_instance) at world size 1. */
int esr_sell_build(int64_t n, const int64_t *rowptr, const int64_t *perm,
                   const int64_t *colidx, int64_t ncols, int64_t *slice_ptr,
                   int32_t *col, int64_t *src_pos);

/* y = A x; dtype of x/y = A's dtype. Bit-identical to the reference's
 * index-multiply-scatter-add sequence (no contraction). */
int esr_spmv(const esr_sell *A, const void *x, void *y, void *stream);

/* Scratch bytes for esr_cg_* on an n-row system. */
int64_t esr_cg_workspace_bytes(int64_t n);

/* Device-side scalars of a fused CG run (FP64), inside the workspace. */
typedef struct {
  double rz;       /* r.z of the current iterate                    */
  double pq;       /* p.Ap                                           */
  double alpha;
  double beta;
  double rr;       /* r.r  (rnorm^2)                                 */
  double bnorm;
  double tol;      /* absolute stopping tolerance on ||r||           */
  double rz_new;
  double rz_prev;  /* r.z before the last update (for replacements)  */
  double true_rr;  /* ||b - A x||^2 at the last replacement (mixed)  */
  int32_t iters;   /* completed step() calls                        */
  int32_t done;    /* 1 = converged, 2 = maxiter, 3 = breakdown/NaN  */
  int32_t maxiter; /* < 0: unlimited                                 */
  int32_t replacements; /* true-residual replacements (mixed)        */
} esr_cg_scalars;

/* PCG set-up (easier/numeric/solver/cg.py:49-53 Init + :136-139):
 * r = b - A x, z = M r (invdiag == NULL: identity, else z = r * invdiag),
 * p = z, bnorm = ||b||, tol = max(rtol*bnorm, atol), rz = r.z. */
int esr_cg_init(const esr_sell *A, const void *b, void *x, void *r, void *z,
                void *p, const void *invdiag, double rtol, double atol,
                int32_t maxiter, void *workspace, void *stream);

/* `k` PCG iterations (cg.py:68-95 Step + Update, with the stopping test of
 * cg.py:150-153 evaluated on the device).  Iterations after convergence are
 * no-ops, so the host may launch in chunks and poll
 * esr_cg_read_scalars(). Vectors q and p2 are scratch of length n. */
int esr_cg_iterate(const esr_sell *A, void *x, void *r, void *z, void *p,
                   void *q, const void *invdiag, int32_t k, void *workspace,
                   void *stream);

/* Copy the device scalars to host memory (synchronises `stream`). */
int esr_cg_read_scalars(const void *workspace, esr_cg_scalars *out,
                        void *stream);

/* Mixed-precision PCG: the SpMV runs on the FP32 pipes (FP32 matrix values
 * A32 and an FP32 copy p32 of the search direction for the gathers), the
 * vectors x, r, z, p, q and every dot product stay FP64, and after every
 * chunk of k iterations the FP64 true residual b - A64 x replaces r (the
 * search direction is kept: no restart) and decides convergence, so a
 * converged solve is FP64-verified.  A64/A32 share one SELL layout.
 * No reference counterpart (the reference CG is FP64 only). */
int esr_cg_mixed_init(const esr_sell *A64, const esr_sell *A32, const double *b,
                      double *x, double *r, double *z, double *p, float *p32,
                      const double *invdiag, double rtol, double atol,
                      int32_t maxiter, void *workspace, void *stream);

/* `k` (>= 1) mixed iterations followed by one true-residual replacement;
 * iterations after convergence are no-ops. */
int esr_cg_mixed_iterate(const esr_sell *A64, const esr_sell *A32,
                         const double *b, double *x, double *r, double *z,
                         double *p, float *p32, double *q,
                         const double *invdiag, int32_t k, void *workspace,
                         void *stream);

/* ||b - A x||_2 in FP64 (true residual); out_f64 on the device.
 * `r` is scratch of length n (receives b - A x). */
int esr_true_residual(const esr_sell *A, const void *b, const void *x, void *r,
                      double *out_f64, void *workspace, void *stream);

/* out[i] = (dtype_out)(scale * (double)in[i]); F32/F64 in either direction.
 * Used by mixed-precision iterative refinement (no reference counterpart). */
int esr_convert(int dtype_in, const void *in, int dtype_out, void *out,
                int64_t n, double scale, void *stream);

/* x[i] += scale * (double)d[i] with x FP64 and d F32 or F64: the refinement
 * correction of mixed-precision CG (no reference counterpart). */
int esr_axpy_f64(double *x, int dtype_d, const void *d, double scale,
                 int64_t n, void *stream);

/* ------------------------------------------------------------------------
 * Fused restarted GMRES (easier/numeric/solver/gmres.py:139-266) on a
 * SELL-32 Linsys, F32 or F64, M = Jacobi (invdiag) or identity (NULL).
 * ------------------------------------------------------------------------ */
typedef struct {
  double rnorm;    /* ||b - A x|| after the last residual evaluation        */
  double bnorm;
  double tol;      /* max(rtol * bnorm, atol)                              */
  int32_t jend;    /* Arnoldi columns of the last cycle                    */
  int32_t broken;  /* the last cycle stopped on H[j+1][j] < 1e-15          */
  int32_t cycles;  /* restart cycles run since esr_gmres_init             */
  int32_t pad_;
} esr_gmres_scalars;

/* Scratch bytes (restart <= 64). */
int64_t esr_gmres_workspace_bytes(int64_t n, int32_t restart);

/* bnorm = ||b||, tol = max(rtol * bnorm, atol) (gmres.py:232-234);
 * zeroes the workspace. */
int esr_gmres_init(const esr_sell *A, const void *b, double rtol, double atol,
                   void *workspace, void *stream);

/* r = b - A x, rnorm = ||r|| (UpdateRnorm, gmres.py:21-24). */
int esr_gmres_residual(const esr_sell *A, const void *b, const void *x, void *r,
                       void *workspace, void *stream);

/* One restart cycle (gmres.py:245-261): V_0 = r / rnorm, `restart` Arnoldi
 * steps with modified Gram-Schmidt in the reference's order (stopping early
 * on H[j+1][j] < 1e-15), the Hessenberg least squares on the device (Givens
 * rotations; the reference's clamped SVD gives the same y for a full-rank
 * H), x += M (V y), then the residual for the next stopping test.  V is
 * [restart][n] (column-contiguous), w2 is [2][n] scratch.  A fixed launch
 * sequence: capturable in a CUDA graph. */
int esr_gmres_cycle(const esr_sell *A, const void *invdiag, const void *b,
                    void *x, void *r, void *V, void *w2, int32_t restart,
                    void *workspace, void *stream);

/* Copy the scalars to host memory (synchronises `stream`). */
int esr_gmres_read(const void *workspace, esr_gmres_scalars *out, void *stream);

/* ------------------------------------------------------------------------
 * Batched (P)CG: `ninst` independent Linsys instances packed as one
 * block-diagonal SELL-32 system and iterated in lockstep, each with its own
 * scalars and stopping test (easier/numeric/solver/cg.py:68-161 per
 * instance).  A single system is a batch of one.  No reference counterpart
 * for batching or df64: the reference runs one FP64 system per call.
 *
 * Layout: instance i owns the 256-row tiles [inst_block0[i],
 * inst_block0[i+1]) (padded with identity rows: diag 1, b 0), and no column
 * of an instance points into another.  Consecutive tiles of an instance are
 * grouped into chunks (chunk c = tiles [chunk_tile0[c], chunk_tile0[c+1]),
 * all of instance chunk_inst[c]; instance i owns chunks [inst_chunk0[i],
 * inst_chunk0[i+1])).  The per-iteration kernels run `grid` persistent CTAs
 * of 256 threads that loop over the chunks of the running instances.
 *
 * df64 = 0: val/diag/invdiag and the vectors x, r, z, p, q are FP64.
 * df64 = 1: they are double-float pairs {float hi, lo} (8 bytes per value,
 *           hi + lo), the arithmetic runs on the FP32 pipes with ~48
 *           significand bits; val64/diag64 (FP64) serve the true-residual
 *           check of esr_bcg_verify. */
/* GNN preconditioner of the batched flexible CG (no reference counterpart).
 * Per node i of an instance, with sigma = rms of the instance's residual:
 *   h0_i = relu(enc_w [r_i / sigma, lk_i] + enc_b)                  (32)
 *   4 layers l: A_i = sum_j w_ij h_j, L_i = sum_j len_ij h_j over the
 *     SELL slots of row i; h_i += relu(W_l [h_i, A_i, L_i] + b_l)     (96 -> 32)
 *   y_i = dec_w . h_i + dec_b;  z_i = invdiag_i (r_i + theta sigma y_i)
 * theta = 1 unless the correction would push z.r below half the Jacobi
 * value r.(invdiag r); then theta is cut to hold z.r at that half.
 * h and the MLP inputs are BF16, the MLP runs on the tensor cores
 * (tcgen05, FP32 accumulation in tensor memory), aggregation in FP32.
 * Instances fall back to Jacobi (z = invdiag r, direction restart) when the
 * preconditioned direction breaks down (z.r <= 0 or non-finite), or at a
 * check every `stall_window` iterations when r.r has not decreased since
 * the last check or theta was cut in more than half of the window's
 * iterations. */
typedef struct {
  const float *node_lk;     /* [n] node input (log kappa); 0 on padding rows */
  const float *edge_feat;   /* [nslots][2] (w, len) per SELL slot            */
  const int32_t *inst_rows; /* [ninst] rows of each instance before padding  */
  void *h0;                 /* [n][32] BF16 scratch                          */
  void *h1;                 /* [n][32] BF16 scratch                          */
  const float *enc_w;       /* [32][2]                                       */
  const float *enc_b;       /* [32]                                          */
  const uint16_t *layer_w;  /* [4][32][96] BF16 bits, [out][in]              */
  const float *layer_b;     /* [4][32]                                       */
  const float *dec_w;       /* [32]                                          */
  float dec_b;
  int32_t grid;             /* persistent CTAs of the GNN layer kernels      */
  int32_t stall_window;     /* iterations                                    */
  int32_t pad_;
} esr_gnn;

typedef struct {
  int64_t n;               /* packed rows = 256 * nblocks                  */
  int32_t ninst;
  int32_t nblocks;         /* 256-row tiles                                */
  int32_t rows_per_block;  /* must be 256                                  */
  int32_t df64;
  int32_t nchunks;
  int32_t grid;            /* persistent CTAs of the iteration kernels     */
  const int64_t *slice_ptr;  /* [n/32 + 1]                                 */
  const int32_t *col;        /* [nslots], -1 = padding                     */
  const void *val;           /* [nslots] FP64 or df64                      */
  const void *diag;          /* [n]                                        */
  const void *invdiag;       /* [n] Jacobi 1/diag, NULL = no preconditioner */
  const double *val64;       /* [nslots] FP64 (verification)               */
  const double *diag64;      /* [n]                                        */
  const int32_t *block_inst; /* [nblocks] instance of each tile            */
  const int32_t *inst_block0;/* [ninst + 1] first tile of each instance    */
  const int32_t *chunk_tile0;/* [nchunks + 1] first tile of each chunk     */
  const int32_t *chunk_inst; /* [nchunks] instance of each chunk           */
  const int32_t *inst_chunk0;/* [ninst + 1] first chunk of each instance   */
  const esr_gnn *gnn;        /* NULL: Jacobi (or no) PCG; else flexible CG
                                with the GNN preconditioner                */
  /* Polynomial-Jacobi preconditioner (0 = off; needs gnn == NULL):
   * z = sum_{j<=d} (I - W A)^j W r, the result of d+1 damped Jacobi sweeps
   * on A z = r from z = 0, with W = invdiag, which then holds the damped
   * weights omega/diag.  d in [2, 16]; an even d gives an SPD M for any
   * omega > 0, an odd d needs omega * lambda_max(D^-1 A) < 2. */
  void *poly_tmp;            /* [2][n] scratch (FP64 or df64), d > 0       */
  int32_t poly_degree;       /* d: SpMV sweeps per application             */
  int32_t pad_poly_;
} esr_batch;

/* Per-instance device scalars. */
typedef struct {
  double rz, pq, alpha, beta, rr, bnorm, tol;
  double true_rr;    /* FP64 ||b - A x||^2 of the last verification, -1 none */
  double sigma;      /* rms of r (GNN input scale)                          */
  double rr_mark;    /* r.r at the last stall check                         */
  double rz_jac;     /* r.(invdiag r) of the current residual               */
  double theta;      /* weight of the network's correction in z (GNN mode)  */
  int32_t iters;     /* completed step() calls                              */
  int32_t done;      /* 0 running, 1 converged, 2 maxiter, 3 breakdown/NaN  */
  int32_t verified;  /* 1 = FP64 true residual <= tol                       */
  int32_t restarts;  /* residual replacements after a failed verification   */
  int32_t maxiter;
  int32_t mode;      /* 0 Jacobi, 1 GNN                                     */
  int32_t refresh;   /* next direction: 1 restarts with p = invdiag r,       *
                      * 2 keeps the p already set (q = A p)                 */
  int32_t fallbacks; /* GNN -> Jacobi switches                              */
  int32_t nrows;     /* rows before padding                                 */
  int32_t gnn_iters; /* iteration of the last GNN -> Jacobi switch (0 none) */
  int32_t clips;     /* iterations with theta < 1                           */
  int32_t clips_mark;/* clips at the last stall check                       */
  float alpha_df[2]; /* alpha and beta as double-float pairs (hi, lo), set   */
  float beta_df[2];  /* with alpha/beta so the df64 kernels need no FP64 op */
} esr_bcg_inst;

int64_t esr_bcg_workspace_bytes(int32_t ninst, int32_t nblocks,
                                int32_t nchunks);

/* Per instance: r = b - A x, z = M r, p = z, bnorm = ||b64||,
 * tol = max(rtol*bnorm, atol); counts every instance as running.  Zeroes
 * the workspace. */
int esr_bcg_init(const esr_batch *B, const double *b64, const void *b, void *x,
                 void *r, void *z, void *p, double rtol, double atol,
                 int32_t maxiter, void *workspace, void *stream);

/* One compaction launch (lists the chunks of running instances) and `k`
 * lockstep iterations of 2 (df64) or 3 (FP64) persistent launches each,
 * plus poly_degree polynomial sweeps and 5 GNN launches where those
 * preconditioners are on.  Instances that stop
 * inside the call skip their chunks; the host enqueues calls (e.g. as CUDA
 * graphs) and polls esr_bcg_status between them.  q is scratch [n]. */
int esr_bcg_iterate(const esr_batch *B, void *x, void *r, void *z, void *p,
                    void *q, int32_t k, void *workspace, void *stream);

/* For every converged, unverified instance: x64 = x, r64 = b64 - A64 x64 in
 * FP64; verified = 1 when ||r64|| <= tol.  Otherwise r = r64 replaces the
 * recurrence residual (z = M r, and p = z + (r.z / r.z_old) p while
 * ||r64|| <= 2 ||r||, else p = z; with the polynomial preconditioner the
 * next iteration's sweeps form z and beta) and the instance runs again.
 * 4 launches. */
int esr_bcg_verify(const esr_batch *B, const double *b64, void *x, double *x64,
                   double *r64, void *r, void *z, void *p, void *workspace,
                   void *stream);

/* The whole batched solve as ONE CUDA graph launch: workspace reset and
 * esr_bcg_init, then a device-side WHILE node whose body is
 * esr_bcg_iterate(k) + esr_bcg_verify and sets the loop condition on the
 * device (instances still running).  maxiter must be finite: the loop also
 * stops after 2*ceil(maxiter/k) + 16 bodies, so the graph always ends.
 * Pointers and rtol/atol/maxiter are baked in at creation; launch with
 * esr_bcg_graph_launch on any stream, free with esr_bcg_graph_destroy. */
int esr_bcg_graph_create(const esr_batch *B, const double *b64, const void *b,
                         void *x, void *r, void *z, void *p, void *q,
                         double *x64, double *r64, double rtol, double atol,
                         int32_t maxiter, int32_t k, void *workspace,
                         void **graph_out);
int esr_bcg_graph_launch(void *graph, void *stream);
int esr_bcg_graph_destroy(void *graph);

/* The GNN preconditioner alone: z = M(r) for every instance of a batch
 * with batch.gnn set (sigma = rms of each instance's r), zero on padding
 * rows.  Uses (and overwrites) the workspace.  6 launches. */
int esr_gnn_apply(const esr_batch *B, const void *r, void *z, void *workspace,
                  void *stream);

/* Self-test of the bounded device wait used by the GNN kernels: one warp
 * allocates tensor memory, waits at most `limit_polls` polls on an mbarrier
 * that nothing arrives on, frees the tensor memory, writes 1 to
 * *gave_up_dev and raises ESR_DEV_WAIT_TIMEOUT.  The context stays usable.
 * Test hook (no reference counterpart). */
int esr_wait_selftest(int32_t limit_polls, int32_t *gave_up_dev, void *stream);

/* Running-instance count and (if inst_out) the per-instance scalars, to
 * host memory; synchronises `stream`. */
int esr_bcg_status(const void *workspace, int32_t ninst, int32_t nchunks,
                   int32_t *active, esr_bcg_inst *inst_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ESR_GB300_H */
