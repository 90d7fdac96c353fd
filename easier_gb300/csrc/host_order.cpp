// Host-side integer work: error reporting, CSR construction from a Reducer
// index, and reverse Cuthill-McKee ordering.  All of it is exact integer
// arithmetic and deterministic.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <exception>
#include <string>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include "esr_internal.h"

namespace {
thread_local std::string t_last_error;
}

namespace esr {
int fail(int code, const std::string &msg) {
  t_last_error = msg;
  return code;
}
}  // namespace esr

extern "C" const char *esr_last_error(void) { return t_last_error.c_str(); }

extern "C" int esr_abi_version(void) { return ESR_GB300_ABI_VERSION; }

// Stable counting sort: the edge order the reference's reorder pass gives a
// Reducer at world size 1 (sparse_encoding.py:244-338 with the stable
// zipsort of passes/utils.py:301-336), plus the CSR row pointer.
extern "C" int esr_csr_from_index(const int64_t *idx, int64_t m, int64_t n,
                                  int64_t *rowptr, int64_t *perm) {
  ESR_HOST_TRY
  if (m < 0 || n < 0) return esr::fail(ESR_ERR_ARG, "negative size");
  if (!rowptr || (m && (!idx || !perm))) return esr::fail(ESR_ERR_ARG, "null pointer");
  std::fill(rowptr, rowptr + n + 1, 0);
  for (int64_t k = 0; k < m; ++k) {
    int64_t v = idx[k];
    if (v < 0 || v >= n)
      return esr::fail(ESR_ERR_ARG, "index " + std::to_string(v) + " at position " +
                                        std::to_string(k) + " is out of range [0, " +
                                        std::to_string(n) + ")");
    rowptr[v + 1] += 1;
  }
  for (int64_t i = 0; i < n; ++i) rowptr[i + 1] += rowptr[i];
  std::vector<int64_t> fill(rowptr, rowptr + n);
  for (int64_t k = 0; k < m; ++k) perm[fill[idx[k]]++] = k;
  return ESR_OK;
  ESR_HOST_CATCH
}

// Reverse Cuthill-McKee.
//  1. Build the undirected simple graph (both directions, no self loops,
//     no duplicate neighbours); neighbour lists sorted by (degree, index).
//  2. For each component, in order of its lowest-degree lowest-index
//     unvisited vertex: find a pseudo-peripheral start by repeated BFS
//     (move to the lowest-degree vertex of the last level while the
//     eccentricity grows, at most 16 rounds), then Cuthill-McKee BFS.
//  3. Reverse the concatenated order.
extern "C" int esr_rcm_order(int64_t n, int64_t m, const int64_t *src,
                             const int64_t *dst, int64_t *order) {
  ESR_HOST_TRY
  if (n < 0 || m < 0) return esr::fail(ESR_ERR_ARG, "negative size");
  if (!order || (m && (!src || !dst))) return esr::fail(ESR_ERR_ARG, "null pointer");
  if (n == 0) return ESR_OK;
  for (int64_t e = 0; e < m; ++e)
    if (src[e] < 0 || src[e] >= n || dst[e] < 0 || dst[e] >= n)
      return esr::fail(ESR_ERR_ARG, "edge endpoint out of range");

  // undirected adjacency in CSR
  std::vector<int64_t> deg(n + 1, 0);
  for (int64_t e = 0; e < m; ++e) {
    if (src[e] == dst[e]) continue;
    deg[src[e] + 1]++;
    deg[dst[e] + 1]++;
  }
  for (int64_t i = 0; i < n; ++i) deg[i + 1] += deg[i];
  std::vector<int64_t> adj(deg[n]);
  {
    std::vector<int64_t> pos(deg.begin(), deg.end() - 1);
    for (int64_t e = 0; e < m; ++e) {
      if (src[e] == dst[e]) continue;
      adj[pos[src[e]]++] = dst[e];
      adj[pos[dst[e]]++] = src[e];
    }
  }
  // dedupe each list
  std::vector<int64_t> ptr(n + 1, 0);
  {
    int64_t w = 0;
    for (int64_t i = 0; i < n; ++i) {
      int64_t b = deg[i], e = deg[i + 1];
      std::sort(adj.begin() + b, adj.begin() + e);
      ptr[i] = w;
      for (int64_t k = b; k < e; ++k)
        if (k == b || adj[k] != adj[k - 1]) adj[w++] = adj[k];
    }
    ptr[n] = w;
    adj.resize(w);
  }
  std::vector<int64_t> degree(n);
  for (int64_t i = 0; i < n; ++i) degree[i] = ptr[i + 1] - ptr[i];
  auto by_degree = [&](int64_t a, int64_t b) {
    return degree[a] != degree[b] ? degree[a] < degree[b] : a < b;
  };
  for (int64_t i = 0; i < n; ++i) std::sort(adj.begin() + ptr[i], adj.begin() + ptr[i + 1], by_degree);

  // candidate roots in (degree, index) order: a counting sort by degree
  // (stable, so equal degrees stay in index order)
  std::vector<int64_t> roots(n);
  {
    int64_t maxd = 0;
    for (int64_t i = 0; i < n; ++i) maxd = std::max(maxd, degree[i]);
    std::vector<int64_t> start(maxd + 2, 0);
    for (int64_t i = 0; i < n; ++i) start[degree[i] + 1]++;
    for (int64_t d = 0; d <= maxd; ++d) start[d + 1] += start[d];
    for (int64_t i = 0; i < n; ++i) roots[start[degree[i]]++] = i;
  }

  std::vector<int64_t> level(n, -1);  // scratch for the peripheral search
  std::vector<int64_t> touched;
  std::vector<char> placed(n, 0);
  int64_t out = 0;

  auto bfs_last_level = [&](int64_t s, int64_t &ecc) -> int64_t {
    // BFS limited to s's component; returns the lowest (degree, index)
    // vertex of the deepest level.
    touched.clear();
    std::vector<int64_t> q;
    q.push_back(s);
    level[s] = 0;
    touched.push_back(s);
    size_t h = 0;
    int64_t maxl = 0;
    while (h < q.size()) {
      int64_t v = q[h++];
      for (int64_t k = ptr[v]; k < ptr[v + 1]; ++k) {
        int64_t w = adj[k];
        if (level[w] < 0) {
          level[w] = level[v] + 1;
          maxl = std::max(maxl, level[w]);
          q.push_back(w);
          touched.push_back(w);
        }
      }
    }
    int64_t best = -1;
    for (int64_t v : q)
      if (level[v] == maxl && (best < 0 || by_degree(v, best))) best = v;
    for (int64_t v : touched) level[v] = -1;
    ecc = maxl;
    return best;
  };

  for (int64_t ri = 0; ri < n; ++ri) {
    int64_t r = roots[ri];
    if (placed[r]) continue;
    // pseudo-peripheral vertex
    int64_t start = r, ecc = 0;
    int64_t cand = bfs_last_level(start, ecc);
    for (int round = 0; round < 16; ++round) {
      int64_t ecc2 = 0;
      int64_t cand2 = bfs_last_level(cand, ecc2);
      if (ecc2 <= ecc) break;
      start = cand;
      ecc = ecc2;
      cand = cand2;
    }
    // Cuthill-McKee BFS
    int64_t head = out;
    order[out++] = start;
    placed[start] = 1;
    while (head < out) {
      int64_t v = order[head++];
      for (int64_t k = ptr[v]; k < ptr[v + 1]; ++k) {
        int64_t w = adj[k];
        if (!placed[w]) {
          placed[w] = 1;
          order[out++] = w;
        }
      }
    }
  }
  std::reverse(order, order + n);
  return ESR_OK;
  ESR_HOST_CATCH
}

// SELL-32 layout of a Linsys.  Slices of 32 consecutive rows; a slice is as
// wide as its longest row; entries stored slot-major so a warp reads one
// slot of 32 rows contiguously.  Row entries keep the CSR (= reference edge)
// order.
extern "C" int esr_sell_build(int64_t n, const int64_t *rowptr, const int64_t *perm,
                              const int64_t *colidx, int64_t ncols, int64_t *slice_ptr,
                              int32_t *col, int64_t *src_pos) {
  ESR_HOST_TRY
  if (n < 0 || ncols < 0) return esr::fail(ESR_ERR_ARG, "negative size");
  if (!rowptr || !slice_ptr) return esr::fail(ESR_ERR_ARG, "null pointer");
  if (ncols > ((int64_t)1 << 31) - 1) return esr::fail(ESR_ERR_UNSUPPORTED, "more than 2^31-1 columns");
  const int64_t nslices = (n + 31) / 32;
  slice_ptr[0] = 0;
  for (int64_t s = 0; s < nslices; ++s) {
    int64_t w = 0;
    for (int64_t r = 32 * s; r < 32 * s + 32 && r < n; ++r) w = std::max(w, rowptr[r + 1] - rowptr[r]);
    slice_ptr[s + 1] = slice_ptr[s] + 32 * w;
  }
  if (!col || !src_pos) return ESR_OK;
  if (rowptr[n] > 0 && (!perm || !colidx)) return esr::fail(ESR_ERR_ARG, "null perm/colidx");
  for (int64_t s = 0; s < nslices; ++s) {
    const int64_t w = (slice_ptr[s + 1] - slice_ptr[s]) / 32;
    for (int64_t l = 0; l < 32; ++l) {
      const int64_t r = 32 * s + l;
      const int64_t len = r < n ? rowptr[r + 1] - rowptr[r] : 0;
      for (int64_t k = 0; k < w; ++k) {
        const int64_t pos = slice_ptr[s] + 32 * k + l;
        if (k < len) {
          const int64_t e = perm[rowptr[r] + k];
          const int64_t c = colidx[e];
          if (c < 0 || c >= ncols)
            return esr::fail(ESR_ERR_ARG, "selector index " + std::to_string(c) + " out of range [0, " +
                                              std::to_string(ncols) + ")");
          col[pos] = (int32_t)c;
          src_pos[pos] = e;
        } else {
          col[pos] = -1;
          src_pos[pos] = -1;
        }
      }
    }
  }
  return ESR_OK;
  ESR_HOST_CATCH
}

// Recursive BFS bisection: split a vertex set in two along the BFS
// distances from a pseudo-peripheral vertex of the set, recurse until every
// part has at most max_part vertices.  The pseudo-peripheral vertex is the
// one farthest (largest distance, then smallest id) from the set's first
// vertex; the set is then ordered by (distance from it, id), unreached
// vertices (another component) last by id, and a set due to end as
// k = ceil(size / max_part) parts keeps its first size * floor(k/2) / k
// vertices on the left.  Parts are compact and equal-sized within one
// vertex; part ids are numbered in depth-first order.  Deterministic, and
// the same partition as esr_bisect_partition_device (partition_gpu.cu),
// which computes the same distances and order on the GPU.
namespace {

constexpr int64_t kUnreached = INT64_MAX;

// Recursive BFS bisection over disjoint ranges of `verts`.  A range's
// vertices carry its label; ranges of one level touch disjoint vertices, so
// subtrees run on separate threads: label is read across ranges (a
// neighbour's) while its owner relabels it, hence relaxed atomic accesses
// (the value read is never the reader's own id either way).  Labels are
// heap-numbered (children of id: 2 id + 1, 2 id + 2), so no counter is
// shared; part ids come from each range's first part and part count, in
// left-to-right order.
struct Bisector {
  const std::vector<int64_t> &ptr, &adj;
  std::vector<int64_t> &label, &dist, &verts;
  int64_t *part;
  int64_t max_part;
  int par_depth;

  static int64_t ld(const int64_t *p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
  static void st(int64_t *p, int64_t v) { __atomic_store_n(p, v, __ATOMIC_RELAXED); }

  // BFS distances from start over the vertices labelled id (verts[b:e]);
  // the others of the range stay kUnreached.  `queue` is scratch.
  void distances(int64_t b, int64_t e, int64_t id, int64_t start, std::vector<int64_t> &queue) const {
    for (int64_t i = b; i < e; ++i) dist[verts[i]] = kUnreached;
    queue.clear();
    queue.push_back(start);
    dist[start] = 0;
    for (size_t h = 0; h < queue.size(); ++h) {
      const int64_t v = queue[h];
      for (int64_t k = ptr[v]; k < ptr[v + 1]; ++k) {
        const int64_t w = adj[k];
        if (ld(&label[w]) == id && dist[w] == kUnreached) {
          dist[w] = dist[v] + 1;
          queue.push_back(w);
        }
      }
    }
  }

  void run(int64_t b, int64_t e, int64_t id, int64_t first_part, int depth) {
    const int64_t sz = e - b;
    if (sz <= max_part) {
      for (int64_t i = b; i < e; ++i) part[verts[i]] = first_part;
      return;
    }
    // one sweep: the reached vertex farthest from the first one (largest
    // distance, then smallest id); the distances from there order the set
    std::vector<int64_t> queue;
    queue.reserve(sz);
    distances(b, e, id, verts[b], queue);
    int64_t far = verts[b], fd = 0;
    for (int64_t i = b; i < e; ++i) {
      const int64_t v = verts[i], d = dist[v];
      if (d != kUnreached && (d > fd || (d == fd && v < far))) {
        far = v;
        fd = d;
      }
    }
    distances(b, e, id, far, queue);
    std::sort(verts.begin() + b, verts.begin() + e, [this](int64_t x, int64_t y) {
      const int64_t dx = dist[x], dy = dist[y];
      return dx != dy ? dx < dy : x < y;
    });
    // the set ends as k = ceil(sz / max_part) parts: the first floor(k/2)
    // parts' share of it goes left, so every final part has about sz / k
    // vertices (not sz / 2^j: tiles come out close to max_part)
    const int64_t k = (sz + max_part - 1) / max_part;
    const int64_t half = b + sz * (k / 2) / k;
    const int64_t ida = 2 * id + 1, idb = 2 * id + 2;
    for (int64_t i = b; i < half; ++i) st(&label[verts[i]], ida);
    for (int64_t i = half; i < e; ++i) st(&label[verts[i]], idb);
    std::thread left;
    std::exception_ptr err_left, err_right;  // whatever either half threw
    if (depth < par_depth) {
      try {
        left = std::thread([&] {
          try {
            run(b, half, ida, first_part, depth + 1);
          } catch (...) {
            err_left = std::current_exception();
          }
        });
      } catch (const std::system_error &) {  // no thread to be had: this one does both halves
      }
    }
    if (left.joinable()) {
      // the worker is always joined before anything leaves this scope
      try {
        run(half, e, idb, first_part + k / 2, depth + 1);
      } catch (...) {
        err_right = std::current_exception();
      }
      left.join();
      if (err_left) std::rethrow_exception(err_left);
      if (err_right) std::rethrow_exception(err_right);
    } else {
      run(b, half, ida, first_part, depth + 1);
      run(half, e, idb, first_part + k / 2, depth + 1);
    }
  }
};

}  // namespace

extern "C" int esr_bisect_partition(int64_t n, int64_t m, const int64_t *src, const int64_t *dst,
                                    int64_t max_part, int64_t *part, int64_t *nparts) {
  if (n < 0 || m < 0 || max_part < 1) return esr::fail(ESR_ERR_ARG, "bad size");
  if (!part || !nparts || (m && (!src || !dst))) return esr::fail(ESR_ERR_ARG, "null pointer");
  for (int64_t e = 0; e < m; ++e)
    if (src[e] < 0 || src[e] >= n || dst[e] < 0 || dst[e] >= n)
      return esr::fail(ESR_ERR_ARG, "edge endpoint out of range");
  ESR_HOST_TRY
  std::vector<int64_t> ptr(n + 1, 0);
  for (int64_t e = 0; e < m; ++e) {
    if (src[e] == dst[e]) continue;
    ptr[src[e] + 1]++;
    ptr[dst[e] + 1]++;
  }
  for (int64_t i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  std::vector<int64_t> adj(ptr[n]);
  {
    std::vector<int64_t> pos(ptr.begin(), ptr.end() - 1);
    for (int64_t e = 0; e < m; ++e) {
      if (src[e] == dst[e]) continue;
      adj[pos[src[e]]++] = dst[e];
      adj[pos[dst[e]]++] = src[e];
    }
  }
  std::vector<int64_t> label(n, 0), dist(n, kUnreached), verts(n);
  for (int64_t i = 0; i < n; ++i) verts[i] = i;
  // subtrees in parallel down to ~2 per hardware thread
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  int par_depth = 0;
  while ((1u << par_depth) < 2 * hw && par_depth < 8) ++par_depth;
  Bisector bs{ptr, adj, label, dist, verts, part, max_part, par_depth};
  if (n > 0) bs.run(0, n, 0, 0, 0);
  *nparts = n > 0 ? (n + max_part - 1) / max_part : 0;
  return ESR_OK;
  ESR_HOST_CATCH
}


// Tiled face-slot layout of the shallow-water step (see esr_swe_tiles).
// Two calls: with halo == NULL it fills meta and the totals; then with the
// arrays allocated (halo [total_halo], lnbr/slot_src [3*total_l3],
// area_src/off3 [..]) it fills them.  Per tile the local list is the tile's
// cells (ascending), then the rings of in-neighbours at distance 1..4, each
// ring sorted ascending.  nbr [3][nc] is in tile-major numbering; part[c]
// must be non-decreasing.
extern "C" int esr_swe_tile_layout(int64_t nc, const int32_t *nbr, const int64_t *part, int64_t ntiles,
                                   int32_t *meta, int64_t *total_halo, int64_t *total_l3, int64_t *off3,
                                   int64_t *offh, int32_t *halo, int32_t *lnbr, int64_t *slot_src,
                                   int64_t *area_src) {
  ESR_HOST_TRY
  if (nc <= 0 || ntiles <= 0) return esr::fail(ESR_ERR_ARG, "empty layout");
  if (!nbr || !part || !meta || !total_halo || !total_l3) return esr::fail(ESR_ERR_ARG, "null pointer");
  const bool fill = halo != nullptr;
  if (fill && (!off3 || !offh || !lnbr || !slot_src || !area_src)) return esr::fail(ESR_ERR_ARG, "null output");
  for (int64_t c = 0; c < nc; ++c) {
    if (part[c] < 0 || part[c] >= ntiles || (c && part[c] < part[c - 1]))
      return esr::fail(ESR_ERR_ARG, "part must be non-decreasing tile ids");
    for (int k = 0; k < 3; ++k) {
      const int32_t g = nbr[k * nc + c];
      if (g < -2 || g >= nc) return esr::fail(ESR_ERR_ARG, "face slot out of range");
    }
  }
  std::vector<int64_t> mark(nc, -1), lpos(nc, 0);
  std::vector<int64_t> list, next;
  int64_t tot_h = 0, tot_3 = 0;
  int64_t t_begin = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    int64_t t_end = t_begin;
    while (t_end < nc && part[t_end] == t) ++t_end;
    const int64_t n0 = t_end - t_begin;
    list.clear();
    for (int64_t c = t_begin; c < t_end; ++c) {
      mark[c] = t;
      lpos[c] = (int64_t)list.size();
      list.push_back(c);
    }
    int64_t cum[5];
    cum[0] = n0;
    size_t fb = 0, fe = list.size();
    for (int level = 1; level <= 4; ++level) {
      next.clear();
      for (size_t q = fb; q < fe; ++q) {
        const int64_t c = list[q];
        for (int k = 0; k < 3; ++k) {
          const int32_t g = nbr[k * nc + c];
          if (g >= 0 && mark[g] != t) {
            mark[g] = t;
            next.push_back(g);
          }
        }
      }
      std::sort(next.begin(), next.end());
      fb = list.size();
      for (int64_t g : next) {
        lpos[g] = (int64_t)list.size();
        list.push_back(g);
      }
      fe = list.size();
      cum[level] = (int64_t)list.size();
    }
    int32_t *mt = meta + 8 * t;
    mt[0] = (int32_t)t_begin;
    for (int q = 0; q < 5; ++q) mt[1 + q] = (int32_t)cum[q];
    mt[6] = mt[7] = 0;
    const int64_t n3 = cum[3], nL = cum[4];
    if (fill) {
      off3[t] = tot_3;
      offh[t] = tot_h;
      for (int64_t j = n0; j < nL; ++j) halo[tot_h + (j - n0)] = (int32_t)list[j];
      for (int64_t j = 0; j < n3; ++j) {
        const int64_t c = list[j];
        for (int k = 0; k < 3; ++k) {
          const int32_t g = nbr[k * nc + c];
          const int64_t dst = 3 * tot_3 + k * n3 + j;
          lnbr[dst] = g >= 0 ? (int32_t)lpos[g] : g;
          slot_src[dst] = k * nc + c;
        }
        area_src[tot_3 + j] = c;
      }
    }
    tot_h += nL - n0;
    tot_3 += n3;
    t_begin = t_end;
  }
  if (t_begin != nc) return esr::fail(ESR_ERR_ARG, "tile ids skip a value");
  *total_halo = tot_h;
  *total_l3 = tot_3;
  return ESR_OK;
  ESR_HOST_CATCH
}
