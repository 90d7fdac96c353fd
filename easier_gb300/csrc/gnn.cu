// GNN preconditioner of the batched flexible CG (bcg.cu): four message-
// passing layers, hidden width 32, BF16 features, MLPs on the 5th-generation
// tensor cores (tcgen05.mma, FP32 accumulator in tensor memory).
//
// One launch per layer.  Each is persistent over the active chunk list of
// the batch and walks a chunk in 128-node tiles:
//   1. aggregation (CUDA cores, FP32): 4 threads per node (512 threads, one
//      pass per tile), 8 channels each,
//      gather the neighbours' BF16 features over the node's SELL slots and
//      form u = [h_i, sum_j w_ij h_j, sum_j len_ij h_j] (96 BF16) in shared
//      memory, in the K-major core-matrix layout of the MMA (8 rows x 16 B
//      core matrices; 128 B between core matrices along K, 1536 B between
//      8-row groups);
//   2. one thread issues 6 tcgen05.mma (M=128, N=32, K=16 each, BF16 in,
//      FP32 accumulate) against the layer's weights, staged once per CTA in
//      the same layout, and commits to an mbarrier;
//   3. each of the 16 warps reads 8 accumulator columns of the 32 lanes it
//      may access (tcgen05.ld 32x32b.x8), adds bias, ReLU and the residual
//      h_i and stores BF16 h (layers 1-3),
//      or (layer 4) decodes y_i = dec_w . h_i + dec_b and writes
//      z_i = invdiag_i (r_i + sigma y_i), accumulating the dots that fix the
//      instance's correction weight theta (z.r >= half the Jacobi r.z; the
//      p-update applies theta) and its Polak-Ribiere beta.
// Layer 1 evaluates the encoder h0 = relu(enc_w [r/sigma, lk] + enc_b) on
// the fly for the node and its neighbours instead of storing h0.
//
// The mbarrier wait is bounded: on time-out the kernel raises
// ESR_DEV_WAIT_TIMEOUT, stops, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include "bcg_common.cuh"

namespace {

constexpr int kGThreads = 512;                    // CTA threads: 4 per node of a tile
constexpr int kGRows = 128;                       // nodes per MMA tile (M)
constexpr int kHid = 32;                          // hidden width (N)
constexpr int kIn = 96;                           // MLP input (K) = [h, A, L]
constexpr int kKChunks = kIn / 8;                 // 16-byte columns along K
constexpr int kCoreBytes = 128;                   // one 8 x 16 B core matrix
constexpr int kSBO = kKChunks * kCoreBytes;       // bytes between 8-row groups
constexpr uint32_t kTmemCols = 32;                // FP32 accumulator columns
constexpr int kWaitLimit = 1 << 22;               // mbarrier polls before giving up

static_assert(kGThreads == 4 * kGRows, "4 aggregation threads per node");
static_assert(kGThreads / 32 == 4 * (kHid / 8), "16 warps: 4 TMEM lane groups x 4 column groups");
static_assert(kBThreads % kGRows == 0, "tiles split into whole MMA tiles");

// instruction descriptor, kind::f16: D F32 (bits 4-5 = 1), A BF16 (bits 7-9
// = 1), B BF16 (bits 10-12 = 1), A and B K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kHid >> 3) << 17) |
                            ((uint32_t)(kGRows >> 4) << 24);

struct GArgs {
  const float *node_lk;
  const float2 *edge_feat;
  const float *enc_w;
  const float *enc_b;
  const uint16_t *layer_w;
  const float *layer_b;
  const float *dec_w;
  float dec_b;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, LBO = 128 B (next core
// matrix along K), SBO = 1536 B (next 8-row group), version 1 (bits 46-47),
// base offset 0, no swizzle
__device__ __forceinline__ uint64_t mma_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(kCoreBytes >> 4) << 16) |
         ((uint64_t)(kSBO >> 4) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint64_t *mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of an mbarrier: at most `limit` polls
// (each try_wait may suspend briefly); false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *mbar, uint32_t parity, int limit) {
  bool ok = false;
  for (int tries = 0; tries < limit && !ok; ++tries) ok = mbar_try_wait(mbar, parity);
  return ok;
}

// 8 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
  uint4 u;
  __nv_bfloat162 t;
  t = __floats2bfloat162_rn(f[0], f[1]);
  u.x = *reinterpret_cast<uint32_t *>(&t);
  t = __floats2bfloat162_rn(f[2], f[3]);
  u.y = *reinterpret_cast<uint32_t *>(&t);
  t = __floats2bfloat162_rn(f[4], f[5]);
  u.z = *reinterpret_cast<uint32_t *>(&t);
  t = __floats2bfloat162_rn(f[6], f[7]);
  u.w = *reinterpret_cast<uint32_t *>(&t);
  return u;
}

__device__ __forceinline__ void unpack8(uint4 u, float (&f)[8]) {
  const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    f[2 * k] = __uint_as_float(w[k] << 16);
    f[2 * k + 1] = __uint_as_float(w[k] & 0xFFFF0000u);
  }
}

__device__ __forceinline__ int sU_off(int m, int chunk) { return (m >> 3) * kSBO + chunk * kCoreBytes + (m & 7) * 16; }

template <int LAYER, class P>
__global__ void __launch_bounds__(kGThreads, 2)
gnn_layer_kernel(BArgs a, GArgs g, const typename P::V *__restrict__ r, const typename P::V *__restrict__ q,
                 const typename P::V *__restrict__ invdiag, typename P::V *__restrict__ z,
                 const uint4 *__restrict__ h_in, uint4 *__restrict__ h_out, BcgLayout L) {
  using V = typename P::V;
  __shared__ __align__(1024) uint8_t sU[kGRows * kIn * 2];
  __shared__ __align__(1024) uint8_t sW[kHid * kIn * 2];
  __shared__ float sBias[kHid];
  __shared__ float sDec[kHid];
  __shared__ float sY[kHid / 8][kGRows];  // layer 4: decoder partial sums per channel group
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_err;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // aggregation: node m_agg, channels 8*part .. 8*part+7
  const int m_agg = tid >> 2, part = tid & 3;
  // epilogue: TMEM lanes 32*(warp%4) (the lanes this warp may read), row
  // m_epi of the tile, accumulator columns 8*cgrp .. 8*cgrp+7
  const int lgrp = warp & 3, cgrp = warp >> 2;
  const int m_epi = 32 * lgrp + lane;
  {
    const uint16_t *W = g.layer_w + (LAYER - 1) * kHid * kIn;
    for (int e = tid; e < kHid * kKChunks; e += kGThreads) {
      const int n = e / kKChunks, c = e % kKChunks;
      *reinterpret_cast<uint4 *>(sW + sU_off(n, c)) = *reinterpret_cast<const uint4 *>(W + n * kIn + c * 8);
    }
    if (tid < kHid) {
      sBias[tid] = g.layer_b[(LAYER - 1) * kHid + tid];
      sDec[tid] = g.dec_w[tid];
    }
  }
  if (tid == 0) {
    mbar_init(&s_mbar);
    s_err = 0;
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, kTmemCols);
    tmem_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t tmem_epi = tmem + ((uint32_t)(32 * lgrp) << 16) + (uint32_t)(8 * cgrp);

  float ew0[8], ew1[8], eb[8];  // encoder rows of this thread's channels
  if (LAYER == 1) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      ew0[k] = g.enc_w[(8 * part + k) * 2];
      ew1[k] = g.enc_w[(8 * part + k) * 2 + 1];
      eb[k] = g.enc_b[8 * part + k];
    }
  }
  float bias[8], dec[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    bias[k] = sBias[8 * cgrp + k];
    dec[k] = sDec[8 * cgrp + k];
  }

  uint32_t phase = 0;
  const int count = L.head->acount;
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = L.alist[w];
    const int inst = a.chunk_inst[c];
    const esr_bcg_inst &st = L.inst[inst];
    if (st.done || st.mode != kModeGnn) continue;
    const float sigma = (float)st.sigma;
    const float inv_sigma = sigma > 0.f ? 1.f / sigma : 0.f;
    const int64_t real_end = (int64_t)a.inst_block0[inst] * kBThreads + st.nrows;
    typename P::Acc nr, nq, jq;  // zN.r, zN.q, zJ.q (zJ = invdiag r, zN = invdiag sigma y)
    const int64_t row1 = (int64_t)a.chunk_tile0[c + 1] * kBThreads;
    bool stop = false;
    for (int64_t s0 = (int64_t)a.chunk_tile0[c] * kBThreads; s0 < row1; s0 += kGRows) {
      // ---- 1. aggregation into sU: 4 threads per node, one node per quad
      {
        const int64_t i = s0 + m_agg;
        float hs[8], accA[8], accL[8];
        if (LAYER == 1) {
          const float rh = P::flt(r[i]) * inv_sigma, lk = g.node_lk[i];
#pragma unroll
          for (int k = 0; k < 8; ++k) hs[k] = bf16r(fmaxf(fmaf(ew0[k], rh, fmaf(ew1[k], lk, eb[k])), 0.f));
        } else {
          unpack8(h_in[i * 4 + part], hs);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) accA[k] = accL[k] = 0.f;
        const int64_t sl = i >> 5;
        const int ln = (int)(i & 31);
        const int64_t base = a.slice_ptr[sl];
        const int wd = (int)((a.slice_ptr[sl + 1] - base) >> 5);
        for (int k = 0; k < wd; ++k) {
          const int64_t e = base + 32 * k + ln;
          const int32_t j = a.col[e];
          if (j < 0 || (int64_t)j >= a.n) continue;
          const float2 ef = g.edge_feat[e];
          float hj[8];
          if (LAYER == 1) {
            const float rj = P::flt(r[j]) * inv_sigma, lj = g.node_lk[j];
#pragma unroll
            for (int t = 0; t < 8; ++t) hj[t] = bf16r(fmaxf(fmaf(ew0[t], rj, fmaf(ew1[t], lj, eb[t])), 0.f));
          } else {
            unpack8(h_in[(int64_t)j * 4 + part], hj);
          }
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            accA[t] = fmaf(ef.x, hj[t], accA[t]);
            accL[t] = fmaf(ef.y, hj[t], accL[t]);
          }
        }
        *reinterpret_cast<uint4 *>(sU + sU_off(m_agg, part)) = pack8(hs);
        *reinterpret_cast<uint4 *>(sU + sU_off(m_agg, 4 + part)) = pack8(accA);
        *reinterpret_cast<uint4 *>(sU + sU_off(m_agg, 8 + part)) = pack8(accL);
      }
      // ---- 2. MLP on the tensor cores
      fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t ua = smem_u32(sU), wa = smem_u32(sW);
#pragma unroll
        for (int k = 0; k < kIn / 16; ++k)
          mma_bf16(tmem, mma_desc(ua + k * 2 * kCoreBytes), mma_desc(wa + k * 2 * kCoreBytes), k > 0 ? 1u : 0u);
        mma_commit(&s_mbar);
      }
      if (!mbar_wait_bounded(&s_mbar, phase, kWaitLimit)) s_err = 1;
      phase ^= 1u;
      tc_fence_after();
      __syncthreads();
      if (s_err) {
        stop = true;
        break;
      }
      // ---- 3. epilogue: row m_epi, channels 8*cgrp .. 8*cgrp+7
      float acc[8];
      tmem_ld8(tmem_epi, acc);
      const int64_t i = s0 + m_epi;
      float o[8];
      {
        float hv[8];
        unpack8(*reinterpret_cast<const uint4 *>(sU + sU_off(m_epi, cgrp)), hv);
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = bf16r(hv[k] + fmaxf(acc[k] + bias[k], 0.f));
      }
      if (LAYER < 4) {
        h_out[i * 4 + cgrp] = pack8(o);
      } else {
        float yp = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) yp = fmaf(dec[k], o[k], yp);
        sY[cgrp][m_epi] = yp;
        __syncthreads();
        if (cgrp == 0) {
          const float y = g.dec_b + ((sY[0][m_epi] + sY[1][m_epi]) + (sY[2][m_epi] + sY[3][m_epi]));
          V zi = P::zero();
          const V ri = r[i], qi = q[i];
          if (i < real_end) {
            const V d = invdiag[i];
            const V zn = P::mul(d, P::off(sigma * y));
            const V zj = P::mul(d, ri);
            zi = P::fma(d, ri, zn);
            nr.add(zn, ri);
            nq.add(zn, qi);
            jq.add(zj, qi);
          }
          z[i] = zi;
        }
      }
      tc_fence_before();
      __syncthreads();  // sU, sY and the accumulator are reused by the next tile
    }
    if (stop) break;
    if (LAYER == 4) {
      const double v[3] = {bsum<kGThreads>(nr), bsum<kGThreads>(nq), bsum<kGThreads>(jq)};
      double tot[3];
      if (chunk_finish<3, kGThreads>(a, c, inst, v, L, tot) && tid == 0) {
        esr_bcg_inst &s = L.inst[inst];
        // z = zJ + theta zN with z.r >= zJ.r / 2 (zJ.r = rz_jac > 0)
        const double jr = s.rz_jac;
        double theta = 1.0;
        if (tot[0] < -0.5 * jr) {
          theta = 0.5 * jr / -tot[0];
          s.clips += 1;
        }
        const double zr = jr + theta * tot[0], zq = tot[2] + theta * tot[1];
        s.theta = theta;
        if (!(zr > 0.0) || !isfinite(zr) || !isfinite(zq) || s.rz == 0.0) {
          // the network's direction is unusable: Jacobi from here on
          s.mode = kModeJacobi;
          s.refresh = 1;
          s.fallbacks += 1;
          s.gnn_iters = s.iters;
          set_beta(s, 0.0);
          s.rz = s.rz_jac;
        } else {
          set_beta(s, -s.alpha * zq / s.rz);
          s.rz = zr;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
  if (tid == 0 && s_err) esr::raise_status(ESR_DEV_WAIT_TIMEOUT);
}

template <class P>
int launch_layers(const esr_batch *B, const void *r, const void *q, void *z, void *ws, cudaStream_t s) {
  using V = typename P::V;
  const esr_gnn *G = B->gnn;
  BcgLayout L = layout_of(ws, B->ninst, B->nchunks);
  const BArgs a = bargs(B);
  const GArgs g{G->node_lk, reinterpret_cast<const float2 *>(G->edge_feat), G->enc_w, G->enc_b, G->layer_w,
                G->layer_b, G->dec_w, G->dec_b};
  const uint4 *h0 = (const uint4 *)G->h0;
  const uint4 *h1 = (const uint4 *)G->h1;
  const V *rv = (const V *)r, *qv = (const V *)q, *dv = (const V *)B->invdiag;
  gnn_layer_kernel<1, P><<<G->grid, kGThreads, 0, s>>>(a, g, rv, qv, dv, (V *)z, nullptr, (uint4 *)G->h0, L);
  gnn_layer_kernel<2, P><<<G->grid, kGThreads, 0, s>>>(a, g, rv, qv, dv, (V *)z, h0, (uint4 *)G->h1, L);
  gnn_layer_kernel<3, P><<<G->grid, kGThreads, 0, s>>>(a, g, rv, qv, dv, (V *)z, h1, (uint4 *)G->h0, L);
  gnn_layer_kernel<4, P><<<G->grid, kGThreads, 0, s>>>(a, g, rv, qv, dv, (V *)z, h0, nullptr, L);
  ESR_LAUNCH_CHECK("esr_bcg_iterate/gnn");
  return ESR_OK;
}

// Self-test of the bounded wait: allocates tensor memory like the layer
// kernel, waits on an mbarrier that nothing arrives on, and must give up,
// raise ESR_DEV_WAIT_TIMEOUT, free the tensor memory and return.
__global__ void __launch_bounds__(32) gnn_wait_selftest_kernel(int limit, int *gave_up) {
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ uint32_t s_tmem;
  if (threadIdx.x == 0) mbar_init(&s_mbar);
  tmem_alloc(&s_tmem, kTmemCols);
  tmem_relinquish();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const bool ok = mbar_wait_bounded(&s_mbar, 0u, limit);
  __syncthreads();
  tc_fence_after();
  tmem_dealloc(s_tmem, kTmemCols);
  if (threadIdx.x == 0) {
    *gave_up = ok ? 0 : 1;
    if (!ok) esr::raise_status(ESR_DEV_WAIT_TIMEOUT);
  }
}

}  // namespace

ESR_DEFINE_STATUS_READER(esr_status_gnn)

extern "C" int esr_wait_selftest(int32_t limit_polls, int32_t *gave_up_dev, void *stream) {
  if (limit_polls <= 0 || limit_polls > kWaitLimit || !gave_up_dev)
    return esr::fail(ESR_ERR_ARG, "esr_wait_selftest: limit in [1, 2^22] and a device flag");
  gnn_wait_selftest_kernel<<<1, 32, 0, esr::as_stream(stream)>>>(limit_polls, gave_up_dev);
  ESR_LAUNCH_CHECK("esr_wait_selftest");
  return ESR_OK;
}

namespace esr {
int gnn_layers(const esr_batch *B, const void *r, const void *q, void *z, void *workspace, cudaStream_t s) {
  return B->df64 ? launch_layers<PolDF>(B, r, q, z, workspace, s) : launch_layers<PolF64>(B, r, q, z, workspace, s);
}
}  // namespace esr
