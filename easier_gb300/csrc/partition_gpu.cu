// Tile partition on the GPU: recursive BFS bisection of a graph, the
// contract of esr_bisect_partition (host_order.cpp) -- a set due to end as
// k = ceil(size / max_part) parts splits floor(k/2) : ceil(k/2) by size
// along the BFS order from a pseudo-peripheral vertex, and the parts are
// numbered left to right, i.e. in depth-first order.  The pseudo-peripheral
// vertex comes from one sweep (the vertex farthest from the set's first
// one; two sweeps gave no more compact tiles on the tutorial meshes --
// level-<=3 cells per tile cell 1.205 vs 1.208 at N=1000 -- for 50% more
// BFS levels).
//
// GPU shape.  All sets ("segments") of one recursion depth are processed by
// one launch, one thread-block cluster per segment (clusters of up to 8 CTAs
// while the segments are few and large, single CTAs once there are more
// segments than SMs).  A BFS is level-synchronous inside its cluster: the
// frontier lives in global memory, a warp reserves room for its
// discoveries with one atomic per neighbour step, and one cluster barrier
// separates the levels.  Nothing waits on a flag: the barriers are hardware
// barriers, and a BFS ends when its frontier is empty (every vertex enters
// it once).  A level costs a chain of dependent memory accesses, so the
// data is shaped to keep the chain short: a vertex's segment and BFS
// distance share one 64-bit word (one load tests a neighbour, one CAS
// claims it), and graphs of degree <= 8 (meshes) keep their neighbours in
// fixed-width rows (no row-offset load).  That word is also the sort key:
// each depth orders every segment's vertices by (segment, distance) with one
// radix sort, stable over vertex ids, and cuts the segments.  The result
// depends only on BFS distances and ids, never on the order in which
// threads discover vertices: it is deterministic and vertex for vertex the
// host function's, which takes the same steps serially.
#include <cooperative_groups.h>

#include <cstdint>
#include <cub/cub.cuh>

#include "esr_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int kPartThreads = 1024;
constexpr uint32_t kInf = 0xFFFFFFFFu;  // not reached
constexpr int kMaxCluster = 8;
constexpr int kEllMax = 8;  // widest fixed-width neighbour rows

inline int64_t al256(int64_t v) { return (v + 255) / 256 * 256; }

struct PartWs {
  int32_t *ptr;       // [n + 1] degrees, then CSR row offsets
  int32_t *adj;       // [max(2 m, kEllMax n)] CSR neighbours or fixed-width rows
  int32_t *cursor;    // [n] fill cursors
  unsigned long long *word;  // [n] (segment << 32) | BFS distance
  unsigned long long *key2;  // [n] sorted words
  int32_t *ids;       // [n] 0..n-1
  int32_t *verts;     // [n] vertices in segment order
  int32_t *fa, *fb;   // [n] frontiers (a segment uses its own range)
  int32_t *seg, *seg2;  // [P + 1] segment boundaries in `verts`
  int32_t *info;      // [4]: segment count, bad edges, largest degree
  int32_t *start;     // [P] BFS start of each segment
  unsigned long long *far;  // [P] (distance, ~id) maximum of a sweep
  int32_t *cnt;       // [3 P] rotating frontier counters
  void *tmp;          // CUB scratch
  size_t tmp_bytes;
  int64_t total;
};

size_t cub_bytes(int64_t n) {
  size_t a = 0, b = 0, c = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, a, (const unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                  (const int32_t *)nullptr, (int32_t *)nullptr, (int)n);
  cub::DeviceScan::ExclusiveSum(nullptr, b, (const int32_t *)nullptr, (int32_t *)nullptr, (int)(n + 1));
  cub::DeviceReduce::Max(nullptr, c, (const int32_t *)nullptr, (int32_t *)nullptr, (int)n);
  return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

PartWs layout(void *base, int64_t n, int64_t m, int64_t P) {
  PartWs w{};
  char *p = (char *)base;
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    char *r = p ? p + off : nullptr;
    off += al256(bytes > 0 ? bytes : 1);
    return r;
  };
  const int64_t nadj = 2 * m > kEllMax * n ? 2 * m : kEllMax * n;
  w.ptr = (int32_t *)take(4 * (n + 1));
  w.adj = (int32_t *)take(4 * nadj);
  w.cursor = (int32_t *)take(4 * n);
  w.word = (unsigned long long *)take(8 * n);
  w.key2 = (unsigned long long *)take(8 * n);
  w.ids = (int32_t *)take(4 * n);
  w.verts = (int32_t *)take(4 * n);
  w.fa = (int32_t *)take(4 * n);
  w.fb = (int32_t *)take(4 * n);
  w.seg = (int32_t *)take(4 * (P + 1));
  w.seg2 = (int32_t *)take(4 * (P + 1));
  w.info = (int32_t *)take(16);
  w.start = (int32_t *)take(4 * P);
  w.far = (unsigned long long *)take(8 * P);
  w.cnt = (int32_t *)take(12 * P);
  w.tmp_bytes = cub_bytes(n);
  w.tmp = take((int64_t)w.tmp_bytes);
  w.total = off;
  return w;
}

__global__ void degree_kernel(int64_t n, int64_t m, const int64_t *__restrict__ src, const int64_t *__restrict__ dst,
                              int32_t *__restrict__ deg, int32_t *__restrict__ info) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += stride) {
    const int64_t s = src[e], d = dst[e];
    if (s < 0 || s >= n || d < 0 || d >= n) {
      atomicAdd(info + 1, 1);
      continue;
    }
    if (s == d) continue;
    atomicAdd(deg + s, 1);
    atomicAdd(deg + d, 1);
  }
}

// neighbours of s and d: CSR rows (ell == 0, ptr = row offsets) or
// fixed-width rows of `ell` entries, -1 padded
__global__ void fill_kernel(int64_t n, int64_t m, const int64_t *__restrict__ src, const int64_t *__restrict__ dst,
                            const int32_t *__restrict__ ptr, int ell, int32_t *__restrict__ cursor,
                            int32_t *__restrict__ adj) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += stride) {
    const int64_t s = src[e], d = dst[e];
    if (s < 0 || s >= n || d < 0 || d >= n || s == d) continue;
    const int64_t rs = ell ? s * ell : ptr[s], rd = ell ? d * ell : ptr[d];
    adj[rs + atomicAdd(cursor + s, 1)] = (int32_t)d;
    adj[rd + atomicAdd(cursor + d, 1)] = (int32_t)s;
  }
}

__global__ void init_kernel(int64_t n, unsigned long long *__restrict__ word, int32_t *__restrict__ ids,
                            int32_t *__restrict__ verts, int32_t *__restrict__ seg, int32_t *__restrict__ info) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    word[v] = 0ull;  // segment 0, distance 0
    ids[v] = (int32_t)v;
    verts[v] = (int32_t)v;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    seg[0] = 0;
    seg[1] = (int32_t)n;
    info[0] = 1;
  }
}

// One BFS pass over every segment still to split (one cluster each).
// Pass 0 starts at the segment's first vertex and records the farthest
// vertex it reached (largest distance, then smallest id); pass 1 starts
// there and leaves the distances the cut follows.  ELL: rows of `width`
// neighbours at adj + v * width (-1 padding); else CSR rows ptr[v]..ptr[v+1].
template <bool ELL>
__global__ void __launch_bounds__(kPartThreads, 1)
bfs_kernel(const int32_t *__restrict__ ptr, const int32_t *__restrict__ adj, int width,
           const int32_t *__restrict__ verts, unsigned long long *__restrict__ word, const int32_t *__restrict__ seg,
           const int32_t *__restrict__ info, int64_t max_part, int32_t *__restrict__ start,
           unsigned long long *__restrict__ far, int32_t *__restrict__ cnt, int32_t *__restrict__ fa,
           int32_t *__restrict__ fb, int pass) {
  __shared__ unsigned long long s_red[kPartThreads / 32];
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int s = (int)(blockIdx.x / C);
  if (s >= info[0]) return;  // the whole cluster leaves together
  const int32_t b = seg[s], e = seg[s + 1];
  if ((int64_t)(e - b) <= max_part) return;
  const unsigned long long mine = (unsigned long long)(uint32_t)s << 32;
  const int gt = rank * kPartThreads + threadIdx.x, gs = C * kPartThreads;
  int32_t *c3 = cnt + 3 * (int64_t)s;
  for (int32_t p = b + gt; p < e; p += gs) word[verts[p]] = mine | kInf;
  if (gt == 0) {
    far[s] = 0ull;
    c3[1] = 0;
    c3[2] = 0;
  }
  cl.sync();
  if (gt == 0) {
    const int32_t src = pass == 0 ? verts[b] : start[s];
    word[src] = mine;
    fa[b] = src;
    c3[0] = 1;
  }
  cl.sync();
  const int32_t *cur = fa + b;
  int32_t *nxt = fb + b;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const unsigned long long unseen = mine | kInf;
  uint32_t level = 0;
  while (true) {
    const int32_t count = __ldcg(c3 + level % 3);
    if (count == 0) break;
    const uint32_t nl = level + 1;
    int32_t *ncnt = c3 + nl % 3;
    // whole warps step through the frontier together (the appends are
    // aggregated per warp: one atomic per neighbour step)
    for (int32_t i0 = gt - lane; i0 < count; i0 += gs) {
      const int32_t i = i0 + lane;
      int64_t k = 0, k1 = 0;
      if (i < count) {
        const int32_t v = __ldcg(cur + i);
        if (ELL) {
          k = (int64_t)v * width;
          k1 = k + width;
        } else {
          k = ptr[v];
          k1 = ptr[v + 1];
        }
      }
      while (__any_sync(0xffffffffu, k < k1)) {
        bool found = false;
        int32_t w = -1;
        if (k < k1) w = adj[k++];
        // in this segment and not reached: the whole word says both
        if (w >= 0 && __ldcg(word + w) == unseen) found = atomicCAS(word + w, unseen, mine | nl) == unseen;
        const unsigned mask = __ballot_sync(0xffffffffu, found);
        if (mask) {
          int32_t base = 0;
          if (lane == __ffs(mask) - 1) base = atomicAdd(ncnt, __popc(mask));
          base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
          if (found) nxt[base + __popc(mask & below)] = w;
        }
      }
    }
    // the counter of level + 2 was last read at level - 1: every CTA has
    // passed the barrier after that
    if (gt == 0) c3[(level + 2) % 3] = 0;
    cl.sync();
    const int32_t *t = cur;
    cur = nxt;
    nxt = const_cast<int32_t *>(t);
    level = nl;
  }
  if (pass == 1) return;
  // the farthest reached vertex: largest distance, then smallest id
  unsigned long long best = 0ull;
  for (int32_t p = b + gt; p < e; p += gs) {
    const int32_t v = verts[p];
    const uint32_t d = (uint32_t)__ldcg(word + v);
    if (d != kInf) {
      const unsigned long long kv = ((unsigned long long)d << 32) | (unsigned long long)(~(uint32_t)v);
      best = kv > best ? kv : best;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_down_sync(0xffffffffu, best, o);
    best = x > best ? x : best;
  }
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x < 32) {
    best = s_red[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_down_sync(0xffffffffu, best, o);
      best = x > best ? x : best;
    }
    if (threadIdx.x == 0) atomicMax(far + s, best);
  }
  cl.sync();
  if (gt == 0) start[s] = (int32_t)(~(uint32_t)(__ldcg(far + s) & 0xFFFFFFFFull));
}

// new segment boundaries (one CTA): a segment of size sz ending as
// k = ceil(sz / max_part) parts keeps its first sz * floor(k/2) / k
// vertices (in the sorted order) on the left
__global__ void __launch_bounds__(kPartThreads)
split_kernel(int64_t n, const int32_t *__restrict__ seg, int32_t *__restrict__ seg2, int32_t *__restrict__ info,
             int64_t max_part) {
  using Scan = cub::BlockScan<int32_t, kPartThreads>;
  __shared__ typename Scan::TempStorage tmp;
  __shared__ int32_t s_off;
  const int32_t S = info[0];
  if (threadIdx.x == 0) s_off = 0;
  __syncthreads();
  for (int32_t s0 = 0; s0 < S; s0 += kPartThreads) {
    const int32_t s = s0 + threadIdx.x;
    int32_t b = 0, sz = 0, kids = 0;
    if (s < S) {
      b = seg[s];
      sz = seg[s + 1] - b;
      kids = (int64_t)sz > max_part ? 2 : 1;
    }
    int32_t pos, total;
    Scan(tmp).ExclusiveSum(kids, pos, total);
    const int32_t o = s_off;
    if (s < S) {
      seg2[o + pos] = b;
      if (kids == 2) {
        const int64_t k = ((int64_t)sz + max_part - 1) / max_part;
        seg2[o + pos + 1] = b + (int32_t)((int64_t)sz * (k / 2) / k);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) s_off = o + total;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    seg2[s_off] = (int32_t)n;
    info[0] = s_off;
  }
}

// word[v] = (the segment holding v's position in the new order, 0)
__global__ void label_kernel(int64_t n, const int32_t *__restrict__ verts, const int32_t *__restrict__ seg,
                             const int32_t *__restrict__ info, unsigned long long *__restrict__ word) {
  const int32_t S = info[0];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    int32_t lo = 0, hi = S - 1;  // largest i with seg[i] <= p
    while (lo < hi) {
      const int32_t mid = (lo + hi + 1) >> 1;
      if ((int64_t)seg[mid] <= p) lo = mid;
      else hi = mid - 1;
    }
    word[verts[p]] = (unsigned long long)(uint32_t)lo << 32;
  }
}

__global__ void part_kernel(int64_t n, const unsigned long long *__restrict__ word, int32_t *__restrict__ part) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride)
    part[v] = (int32_t)(word[v] >> 32);
}

int grid_for(int64_t items, int sms) {
  const int64_t g = (items + 255) / 256;
  return (int)(g < 8LL * sms ? (g > 0 ? g : 1) : 8LL * sms);
}

template <bool ELL>
cudaError_t launch_bfs(const cudaLaunchConfig_t &cfg, const PartWs &w, int width, const int32_t *seg,
                       int64_t max_part, int pass) {
  return cudaLaunchKernelEx(&cfg, bfs_kernel<ELL>, (const int32_t *)w.ptr, (const int32_t *)w.adj, width,
                            (const int32_t *)w.verts, w.word, seg, (const int32_t *)w.info, max_part, w.start, w.far,
                            w.cnt, w.fa, w.fb, pass);
}

}  // namespace

extern "C" int64_t esr_bisect_device_workspace_bytes(int64_t n, int64_t m, int64_t max_part) {
  if (n <= 0 || m < 0 || max_part < 1 || n >= (1LL << 31) - 1 || 2 * m >= (1LL << 31) - 1) return -1;
  const int64_t P = (n + max_part - 1) / max_part;
  return layout(nullptr, n, m, P).total;
}

extern "C" int esr_bisect_partition_device(int64_t n, int64_t m, const int64_t *src, const int64_t *dst,
                                           int64_t max_part, int32_t *part, int64_t *nparts, void *workspace,
                                           int64_t workspace_bytes, void *stream) {
  if (n <= 0 || m < 0 || max_part < 1) return esr::fail(ESR_ERR_ARG, "bad size");
  if (n >= (1LL << 31) - 1 || 2 * m >= (1LL << 31) - 1) return esr::fail(ESR_ERR_ARG, "graph too large for 32-bit ids");
  if (!part || !nparts || !workspace || (m && (!src || !dst))) return esr::fail(ESR_ERR_ARG, "null pointer");
  const int64_t P = (n + max_part - 1) / max_part;
  PartWs w = layout(workspace, n, m, P);
  if (workspace_bytes < w.total) return esr::fail(ESR_ERR_ARG, "workspace too small");
  cudaStream_t s = esr::as_stream(stream);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.ptr, 0, 4 * (n + 1), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.cursor, 0, 4 * n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.info, 0, 16, s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bisect_partition_device/setup");
  // degrees (self loops left out), the largest one, and bad endpoints
  if (m) degree_kernel<<<grid_for(m, sms), 256, 0, s>>>(n, m, src, dst, w.ptr, w.info);
  ESR_LAUNCH_CHECK("esr_bisect_partition_device/degree");
  size_t tb = w.tmp_bytes;
  e = cub::DeviceReduce::Max(w.tmp, tb, w.ptr, w.info + 2, (int)n, s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bisect_partition_device/max degree");
  int32_t hinfo[3] = {0, 0, 0};
  e = cudaMemcpyAsync(hinfo, w.info, 12, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bisect_partition_device/degrees");
  if (hinfo[1]) return esr::fail(ESR_ERR_ARG, "edge endpoint out of range");
  // meshes (degree <= 8): fixed-width rows; else CSR
  const int width = hinfo[2] <= kEllMax ? (hinfo[2] > 0 ? hinfo[2] : 1) : 0;
  if (width) {
    e = cudaMemsetAsync(w.adj, 0xFF, 4 * (int64_t)width * n, s);
  } else {
    tb = w.tmp_bytes;
    e = cub::DeviceScan::ExclusiveSum(w.tmp, tb, w.ptr, w.ptr, (int)(n + 1), s);
  }
  if (e != cudaSuccess) return esr::cuda_check(e, "esr_bisect_partition_device/rows");
  if (m) fill_kernel<<<grid_for(m, sms), 256, 0, s>>>(n, m, src, dst, w.ptr, width, w.cursor, w.adj);
  init_kernel<<<grid_for(n, sms), 256, 0, s>>>(n, w.word, w.ids, w.verts, w.seg, w.info);
  ESR_LAUNCH_CHECK("esr_bisect_partition_device/init");
  int depths = 0;
  while ((1LL << depths) < P) ++depths;
  int32_t *seg = w.seg, *seg2 = w.seg2;
  for (int d = 0; d < depths; ++d) {
    const int64_t smax = (1LL << d) < P ? (1LL << d) : P;  // segments at this depth, at most
    int C = 1;
    while (C < kMaxCluster && smax * C * 2 <= 2LL * sms) C *= 2;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(smax * C));
    cfg.blockDim = dim3(kPartThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    for (int pass = 0; pass < 2; ++pass) {
      e = width ? launch_bfs<true>(cfg, w, width, seg, max_part, pass)
                : launch_bfs<false>(cfg, w, 0, seg, max_part, pass);
      if (e != cudaSuccess) return esr::cuda_check(e, "esr_bisect_partition_device/bfs");
    }
    // (segment, distance) words sorted, stable over the vertex ids; finished
    // segments keep distance 0, so their vertices stay in id order
    int bits = 1;
    while ((1LL << bits) < smax) ++bits;
    tb = w.tmp_bytes;
    e = cub::DeviceRadixSort::SortPairs(w.tmp, tb, w.word, w.key2, w.ids, w.verts, (int)n, 0, 32 + bits, s);
    if (e != cudaSuccess) return esr::cuda_check(e, "esr_bisect_partition_device/sort");
    split_kernel<<<1, kPartThreads, 0, s>>>(n, seg, seg2, w.info, max_part);
    label_kernel<<<grid_for(n, sms), 256, 0, s>>>(n, w.verts, seg2, w.info, w.word);
    ESR_LAUNCH_CHECK("esr_bisect_partition_device/depth");
    int32_t *t = seg;
    seg = seg2;
    seg2 = t;
  }
  part_kernel<<<grid_for(n, sms), 256, 0, s>>>(n, w.word, part);
  ESR_LAUNCH_CHECK("esr_bisect_partition_device/part");
  *nparts = P;
  return ESR_OK;
}
