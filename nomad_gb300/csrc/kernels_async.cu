// kernels_async.cu -- the pipelined asynchronous NOMAD kernel for sm_103a.
//
// Same algorithm as Code/nomad/nb_main.cpp:480-572: persistent workers own row blocks,
// column tokens move between workers through per-worker queues, each visit runs SGD over
// the (worker rows x column) ratings, and the step size of a visit follows the token's
// pass count.  What makes a hop cheap on this GPU:
//
//  1. Ring queues with sequence-tagged 64-bit entries.  A producer takes a slot with one
//     atomic add and writes (sequence << 32 | token); a consumer owns its head counter and
//     takes a token with one acquire load of the slot it expects.  Heads and tails never
//     reset, so an entry left from an earlier pass can never match.
//  2. Warp roles inside a thread block: compute warps (one per worker) only compute; a pop
//     warp moves tokens from their rings into shared-memory inboxes, a push warp moves
//     processed tokens from shared-memory outboxes into the rings behind one gpu-scope
//     release fence per batch.  Compute warps synchronise at block scope only.
//  3. A per-token mailbox: the producer of a hop writes the next visit (rating run, route
//     position, pass count, route, first four ratings) next to the token, so the consumer
//     can load its first rows as soon as the mailbox lands.
//  4. A two-slot token pipeline per compute warp: a taken token's mailbox and held column
//     are copied into shared memory by cp.async (D); next iteration its first rows are
//     loaded into registers and its rating indices copied (W, R); then it is processed.
//  5. Long visits run in blocks of 7 ratings with the chain rewritten exactly: with
//     c = 1 - eta*lambda and b_j = <h_t, w_j> for the block's (distinct, old) rows,
//        e_t = b_t - v_t,   b_j <- c b_j - eta e_t <w_t, w_j>   (j > t),
//     so one reduce-scatter of the 7 <h, w_t> and 21 <w_s, w_t> replaces 7 dependent warp
//     reductions; then w_t' = c w_t - eta e_t h_t and h_{t+1} = c h_t - eta e_t w_t are
//     lane-local.  Rows are staged kRing-1 blocks ahead in shared memory by cp.async (a TMA
//     bulk-copy variant is kept behind NOMAD_STAGE_TMA).
//  6. Columns long enough to set the epoch time visit whole thread blocks instead of
//     workers; the block's compute warps process such a visit together (below).
#include <cuda_bf16.h>

#include <algorithm>
#include <cstddef>

#include "device_common.cuh"
#include "launch.h"

namespace {

using nd::kFull;
using nd::Vec;

constexpr int kPF = 4;       // rows prefetched in registers on the short-visit path
constexpr int kBlk = 7;      // ratings per block on the long-visit path
constexpr int kChunk = 28;   // ratings indexed per register chunk (4 blocks)
constexpr int kRing = 3;     // staged blocks per warp on the long-visit path
constexpr int kBarBytes = (8 * kRing + 15) / 16 * 16;  // mbarriers, padded to keep 16-byte alignment

#ifndef NOMAD_STAGE_TMA
#define NOMAD_STAGE_TMA 0
#endif

// ---- PTX helpers ---------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// 1-D bulk copy global -> shared (the TMA engine), completion counted on `bar`.
__device__ __forceinline__ void tma_row(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
// Bulk prefetch of [p, p + bytes) into L2 (p and bytes multiples of 16).
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// Per-lane asynchronous global -> shared copies (completion by commit groups).  The
// 16-byte form bypasses L1 (.cg), so it also suits data that other SMs write.
__device__ __forceinline__ void cp16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp8(uint32_t dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
template <int BYTES>
__device__ __forceinline__ void cp_async(uint32_t dst, const void* src) {
  if (BYTES == 16) cp16(dst, src); else cp8(dst, src);
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// ---- shared-memory slot of one pipelined token ----------------------------------------
// Mailbox (64 bytes, written by the producer of the hop):
//   a = {start lo, start hi, len, pos}           the visit's rating run and route position
//   b = {ep, nseg | priority bit, vb lo, vb hi}  pass count, route length, route start
//   c, d = the visit's first four ratings {row, value bits}
struct SlotHdr {
  int4 a;
  int4 b;
  int4 c;              // the visit's first ratings {r0, v0, r1, v1}
  int4 d;              //                           {r2, v2, r3, v3}
  int4 nxt[3];         // the route's next visit {start lo, start hi, len, worker} and its first ratings
  int4 pad;
  int2 rv[kChunk];     // the visit's first rating indices {row, value bits}
};
static_assert(sizeof(SlotHdr) == 128 + 8 * kChunk, "slot header layout");

struct Shape {
  int nvec, red_width, row_bytes, heavy_min, slot_bytes;
};

__device__ __forceinline__ int64_t lo_hi(int lo, int hi) {
  return static_cast<int64_t>(static_cast<uint32_t>(lo)) | (static_cast<int64_t>(hi) << 32);
}

template <typename Store, int NV>
__device__ __forceinline__ void store_row(void* W, int r, const Shape& s, int lane,
                                          const float (&x)[NV][Vec<Store>::E], uint32_t key) {
  Store* row = reinterpret_cast<Store*>(static_cast<char*>(W) + static_cast<int64_t>(r) * s.row_bytes);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    if (v < s.nvec) nd::store_vec<Store, false>(row, v, x[q], key + 4u * static_cast<uint32_t>(v));
  }
}

template <typename Store, int NV>
__device__ __forceinline__ void load_row_regs(const void* W, int r, const Shape& s, int lane,
                                              typename Vec<Store>::Raw (&x)[NV]) {
  using Raw = typename Vec<Store>::Raw;
  const Raw* row = reinterpret_cast<const Raw*>(static_cast<const char*>(W) + static_cast<int64_t>(r) * s.row_bytes);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    x[q] = v < s.nvec ? row[v] : nd::zero_raw<Raw>();
  }
}

// The visit's rating i < 4 as carried by the mailbox.
__device__ __forceinline__ int2 first_rating(const SlotHdr* hd, int i) {
  const int4 q = i < 2 ? hd->c : hd->d;
  return (i & 1) ? make_int2(q.z, q.w) : make_int2(q.x, q.y);
}

// ---- short visit: one warp reduction per rating, rows kPF ahead in registers ----------
template <typename Store, int NV>
__device__ __forceinline__ float visit_short(const SlotHdr* hd, int len, float (&h)[NV][Vec<Store>::E], void* W,
                                             const Shape& s, float step, float lambda, uint32_t colkey, int lane) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  Raw wb[kPF][NV];  // rows kPF ahead (the first ones were prefetched into L1 and L2)
#pragma unroll
  for (int i = 0; i < kPF; ++i)
    if (i < len) load_row_regs<Store, NV>(W, first_rating(hd, i).x, s, lane, wb[i]);
  float err2 = 0.f;
  for (int t0 = 0; t0 < len; t0 += kPF) {
#pragma unroll
    for (int i = 0; i < kPF; ++i) {
      const int t = t0 + i;
      if (t < len) {
        const int2 rt = t0 == 0 ? first_rating(hd, i) : hd->rv[t];  // t0 == 0: t == i < 4
        float w[NV][E];
#pragma unroll
        for (int q = 0; q < NV; ++q) nd::unpack(wb[i][q], w[q]);
        float part = 0.f;
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
          for (int e = 0; e < E; ++e) part = fmaf(h[q][e], w[q][e], part);
        const float err = nd::warp_allreduce(part, s.red_width) - __int_as_float(rt.y);
        err2 += err * err;
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const float wo = w[q][e], ho = h[q][e];
            w[q][e] = fmaf(-step, fmaf(err, ho, lambda * wo), wo);
            h[q][e] = fmaf(-step, fmaf(err, wo, lambda * ho), ho);
          }
        store_row<Store, NV>(W, rt.x, s, lane, w, nd::row_key(rt.x, colkey));
        const int tn = t + kPF;
        if (tn < len) load_row_regs<Store, NV>(W, hd->rv[tn].x, s, lane, wb[i]);
      }
    }
  }
  return err2;
}

// ---- long visit ------------------------------------------------------------------------
struct Ring {
  char* rows;       // kRing slots x kBlk rows x row_bytes
  uint32_t bars;    // shared address of kRing mbarriers (TMA variant)
  float* gather;    // 32 floats
  uint32_t phase;   // mbarrier parity bits (TMA variant)
};

// Copies of block `b` of the visit; VB = bytes per lane vector (16 fp32, 8 bf16).
template <int VB>
__device__ __forceinline__ void issue_block(const Ring& R, int b, int len, int chunk_base, int2 rv_cur,
                                            int2 rv_nxt, const void* W, int row_bytes, int lane) {
  const int first = b * kBlk;
  const int nr = min(kBlk, len - first);
  const int slot = b % kRing;
  const int r = lane < nr ? first + lane - chunk_base : 0;  // index into the cur|nxt chunks
  const int a_row = __shfl_sync(kFull, rv_cur.x, min(max(r, 0), 31));
  const int b_row = __shfl_sync(kFull, rv_nxt.x, min(max(r - kChunk, 0), 31));
  const int row = r < kChunk ? a_row : b_row;
#if NOMAD_STAGE_TMA
  if (lane == 0) {
    fence_proxy_async_shared();
    mbar_expect_tx(R.bars + 8u * slot, static_cast<uint32_t>(nr * row_bytes));
  }
  __syncwarp();
  if (lane < nr) {
    const uint32_t dst = smem_u32(R.rows + (static_cast<size_t>(slot) * kBlk + lane) * row_bytes);
    tma_row(dst, static_cast<const char*>(W) + static_cast<int64_t>(row) * row_bytes,
            static_cast<uint32_t>(row_bytes), R.bars + 8u * slot);
  }
#else
  // each lane stages, and later reads, only its own slice of every row
  const uint32_t base = smem_u32(R.rows + static_cast<size_t>(slot) * kBlk * row_bytes);
#pragma unroll
  for (int t = 0; t < kBlk; ++t) {
    const int rt = __shfl_sync(kFull, row, t);
    if (t < nr) {
      const char* src = static_cast<const char*>(W) + static_cast<int64_t>(rt) * row_bytes;
      for (int v = lane; v * VB < row_bytes; v += 32) cp_async<VB>(base + t * row_bytes + v * VB, src + v * VB);
    }
  }
#endif
}

__device__ __forceinline__ bool wait_block(Ring& R, int slot, int* ctrl, int64_t budget_ns) {
#if !NOMAD_STAGE_TMA
  cp_async_wait<kRing - 1>();  // one commit group per block
  return true;
#else
  const uint32_t bar = R.bars + 8u * slot;
  const uint32_t par = (R.phase >> slot) & 1u;
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, par)) break;
    if ((it & 255u) == 0) {
      const uint64_t now = nd::globaltimer();
      if (it == 0) t0 = now;
      else if (static_cast<int64_t>(now - t0) > budget_ns) {
        atomicCAS(&ctrl[1], 0, nd::kDevErrTimeout);
        return false;
      }
    }
  }
  R.phase ^= 1u << slot;
  return true;
#endif
}

// Reduce-scatter of 32 per-lane partials: lane l ends with the warp total of index l.
__device__ __forceinline__ float reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
  for (int lvl = 0; lvl < 5; ++lvl) {
    const int half = 16 >> lvl;
    const bool up = (lane & half) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = up ? v[i] : v[i + half];
      const float keep = up ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, half);
    }
  }
  return v[0];
}

template <typename Store, int NV>
__device__ __forceinline__ float visit_long(const SlotHdr* hd, int64_t start, int len, float (&h)[NV][Vec<Store>::E],
                                            void* W, const Shape& s, Ring& R, const int2* __restrict__ ratings,
                                            float step, float lambda, uint32_t colkey, int lane, int* ctrl,
                                            int64_t budget_ns, bool& failed) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  constexpr int VB = static_cast<int>(sizeof(Raw));
  const int nblocks = (len + kBlk - 1) / kBlk;
  const float c = 1.f - step * lambda;
  float err2 = 0.f;
#if NOMAD_STAGE_TMA
  fence_proxy_async_global();  // earlier generic row stores precede the TMA reads
  __syncwarp();
#endif
  int2 rv_cur = lane < kChunk ? hd->rv[lane] : make_int2(0, 0);
  int2 rv_nxt = lane < kChunk && kChunk + lane < len ? __ldg(&ratings[start + kChunk + lane]) : make_int2(0, 0);
  int chunk_base = 0;
  for (int b = 0; b < kRing - 1; ++b) {
    if (b < nblocks) issue_block<VB>(R, b, len, chunk_base, rv_cur, rv_nxt, W, s.row_bytes, lane);
    if (!NOMAD_STAGE_TMA) cp_async_commit();
  }
  for (int b = 0; b < nblocks; ++b) {
    if (b + kRing - 1 < nblocks) issue_block<VB>(R, b + kRing - 1, len, chunk_base, rv_cur, rv_nxt, W, s.row_bytes, lane);
    if (!NOMAD_STAGE_TMA) cp_async_commit();
    const int slot = b % kRing;
    if (!wait_block(R, slot, ctrl, budget_ns)) {
      failed = true;
      return err2;
    }
    const int first = b * kBlk;
    const int nr = min(kBlk, len - first);
    const char* srow = R.rows + static_cast<size_t>(slot) * kBlk * s.row_bytes;
    int rr[kBlk];
    float vv[kBlk];
#pragma unroll
    for (int t = 0; t < kBlk; ++t) {
      const int idx = first + t - chunk_base;
      const int x1 = __shfl_sync(kFull, rv_cur.x, min(max(idx, 0), 31));
      const int y1 = __shfl_sync(kFull, rv_cur.y, min(max(idx, 0), 31));
      const int x2 = __shfl_sync(kFull, rv_nxt.x, min(max(idx - kChunk, 0), 31));
      const int y2 = __shfl_sync(kFull, rv_nxt.y, min(max(idx - kChunk, 0), 31));
      rr[t] = idx < kChunk ? x1 : x2;
      vv[t] = t < nr ? __int_as_float(idx < kChunk ? y1 : y2) : 0.f;
    }
    float p[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) p[i] = 0.f;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int v = lane + 32 * q;
      if (v < s.nvec) {
        float w[kBlk][E];
#pragma unroll
        for (int t = 0; t < kBlk; ++t) {
          if (t < nr)
            nd::unpack(reinterpret_cast<const Raw*>(srow + t * s.row_bytes)[v], w[t]);
          else
#pragma unroll
            for (int e = 0; e < E; ++e) w[t][e] = 0.f;
        }
#pragma unroll
        for (int t = 0; t < kBlk; ++t) {
#pragma unroll
          for (int e = 0; e < E; ++e) p[t] = fmaf(h[q][e], w[t][e], p[t]);
#pragma unroll
          for (int u = 0; u < t; ++u)
#pragma unroll
            for (int e = 0; e < E; ++e)
              p[kBlk + t * (t - 1) / 2 + u] = fmaf(w[u][e], w[t][e], p[kBlk + t * (t - 1) / 2 + u]);
        }
      }
    }
    R.gather[lane] = reduce_scatter32(p, lane);
    __syncwarp();
    float S[28];
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const float4 g = reinterpret_cast<const float4*>(R.gather)[i];
      S[4 * i] = g.x; S[4 * i + 1] = g.y; S[4 * i + 2] = g.z; S[4 * i + 3] = g.w;
    }
    __syncwarp();
    float bb[kBlk], ee[kBlk];
#pragma unroll
    for (int t = 0; t < kBlk; ++t) bb[t] = S[t];
#pragma unroll
    for (int t = 0; t < kBlk; ++t) {
      ee[t] = bb[t] - vv[t];
      const float ne = -step * ee[t];
#pragma unroll
      for (int j = t + 1; j < kBlk; ++j) bb[j] = fmaf(ne, S[kBlk + j * (j - 1) / 2 + t], c * bb[j]);
    }
#pragma unroll
    for (int t = 0; t < kBlk; ++t) {
      if (t < nr) {
        const float ne = -step * ee[t];
        err2 += ee[t] * ee[t];
        float wn[NV][E];
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          const int v = lane + 32 * q;
          float wo[E];
          if (v < s.nvec)
            nd::unpack(reinterpret_cast<const Raw*>(srow + t * s.row_bytes)[v], wo);
          else
#pragma unroll
            for (int e = 0; e < E; ++e) wo[e] = 0.f;
#pragma unroll
          for (int e = 0; e < E; ++e) {
            wn[q][e] = fmaf(ne, h[q][e], c * wo[e]);
            h[q][e] = fmaf(ne, wo[e], c * h[q][e]);
          }
        }
        store_row<Store, NV>(W, rr[t], s, lane, wn, nd::row_key(rr[t], colkey));
      }
    }
    if ((b & 3) == 3) {  // after the fourth block of a chunk: the next rating chunk
      rv_cur = rv_nxt;
      chunk_base += kChunk;
      const int nx = chunk_base + kChunk + lane;
      rv_nxt = lane < kChunk && nx < len ? __ldg(&ratings[start + nx]) : make_int2(0, 0);
    }
  }
#if !NOMAD_STAGE_TMA
  cp_async_wait<0>();
#endif
  return err2;
}

// ---- visits of priority tokens: all warps of a thread block together ---------------------
// A priority column visits thread blocks instead of workers; the rows of a block's warps
// form one run of the column, and while the warps process it together nobody else
// touches those rows.  The visit runs in blocks of kHB ratings with the chain rewritten
// exactly, as on the long-visit path:
//   G = X X^T over the block's (distinct, old) rows X -- tensor cores, 3xTF32 for fp32
//       rows (split into tf32 parts once per block), exact bf16 products for bf16 rows;
//       b = X h -- four warps;
//   e_t = b_t - v_t,  b_j <- c b_j - eta e_t G_jt (j > t) -- one warp, lane j holds b_j;
//   w_t' = c w_t - eta e_t h_t,  h_{t+1} = c h_t - eta e_t w_t -- each warp for its rows,
//       from h_t = c^t (h_0 + sum_{s<t} k_s w_s), k_s = -eta e_s c^-(s+1), summed over the
//       rows before them.
constexpr int kHB = 32;          // ratings per block
constexpr int kHStages = 3;      // row blocks in shared memory (one in use, two in flight)
constexpr int kHRv = 8;          // rating-index blocks in shared memory (ring)
constexpr int kGStride = kHB + 1;
constexpr int kCtaHdrBytes = 16;

struct CtaHdr {
  int hv_tok;                // priority token the block processes next (-1: none)
  int stop;                  // the launch is over (every token retired, or an error)
  unsigned long long join;   // mbarrier, one arrival per live compute warp
};
static_assert(sizeof(CtaHdr) == kCtaHdrBytes, "block header layout");

// Words per shared-memory row of a block visit: at least the row (fp32 rows rounded up to
// the k8 tile, padding zero), and == 4 (mod 8) so the 8 rows of an mma fragment load
// fall in distinct banks.
__host__ __device__ inline int cta_row_words(int kpad, int esz) {
  int sw = esz == 2 ? kpad / 2 : (kpad + 7) / 8 * 8;
  if (sw % 8 == 0) sw += 4;
  return sw;
}
__host__ __device__ inline size_t cta_region_bytes(int kpad, int esz) {
  // fp32 rows: kHStages staged blocks plus the tf32 high and low parts of one block
  const size_t rows = static_cast<size_t>(kHStages + (esz == 4 ? 2 : 0)) * kHB * cta_row_words(kpad, esz) * 4;
  const size_t gram = static_cast<size_t>(kHB) * kGStride * 4;
  const size_t h = (static_cast<size_t>(2) * kpad * 4 + 15) / 16 * 16;
  return rows + gram + h + 3 * kHB * 4 + static_cast<size_t>(kHRv) * kHB * 8 + 80 * 4;
}

struct CtaRegion {
  char* rows;   // kHStages x kHB rows of sw words
  float* xhi;   // fp32 rows: kHB rows of sw words, tf32 high parts of the block the next
  float* xlo;   //   Gram tiles read; low parts (x - hi rounded to tf32) in xlo
  float* G;     // kHB x kGStride
  float* h;     // 2 x kpad, the held column (fp32) before and after a block
  float* bsh;   // kHB
  float* nesh;  // kHB: -eta e_t
  float* ksh;   // kHB: k_t = -eta e_t c^-(t+1)
  int2* rv;     // kHRv x kHB rating indices
  float* cpow;  // kHB + 1: c^k
  float* cinv;  // kHB: c^-(k+1)
  int sw;
};

__device__ __forceinline__ CtaRegion cta_region(char* base, int kpad, int esz) {
  CtaRegion C;
  C.sw = cta_row_words(kpad, esz);
  C.rows = base;
  char* p = base + static_cast<size_t>(kHStages) * kHB * C.sw * 4;
  C.xhi = reinterpret_cast<float*>(p);
  C.xlo = C.xhi + kHB * C.sw;
  if (esz == 4) p += static_cast<size_t>(2) * kHB * C.sw * 4;
  C.G = reinterpret_cast<float*>(p);
  p += static_cast<size_t>(kHB) * kGStride * 4;
  C.h = reinterpret_cast<float*>(p);
  p += (static_cast<size_t>(2) * kpad * 4 + 15) / 16 * 16;
  C.bsh = reinterpret_cast<float*>(p);
  C.nesh = C.bsh + kHB;
  C.ksh = C.nesh + kHB;
  C.rv = reinterpret_cast<int2*>(C.ksh + kHB);
  C.cpow = reinterpret_cast<float*>(C.rv + kHRv * kHB);
  C.cinv = C.cpow + 36;
  return C;
}

// Non-blocking test of phase `parity` of mbarrier `bar` (acquire, cta scope).
__device__ __forceinline__ bool mbar_test_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Polls phase `parity` of `bar` until it completes (true) or the launch's budget runs
// out (false).  The clock is read only after 1,024 unsuccessful polls, and then every
// 1,024, so a short wait costs no %globaltimer read; the budget counts from the first.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, const nomad::AsyncArgs& a) {
  uint64_t t0 = 0;
  for (uint32_t it = 1;; ++it) {
    if (mbar_test_wait(bar, parity)) return true;
    if ((it & 1023u) == 0) {
      const uint64_t now = nd::globaltimer();
      if (t0 == 0) t0 = now;
      else if (static_cast<int64_t>(now - t0) > a.budget_ns) return false;
    }
  }
}

// Barrier of the block's live compute warps between the phases of a block visit (named
// barrier 1 over their nthreads threads).  It cannot wait forever: every live compute
// warp enters a visit or none does (cta_join), and a visit has no early exit and no
// wait on another agent -- its only other waits are cp.async.wait_group on its own
// copies -- so every warp reaches every barrier after a bounded amount of work.  (An
// mbarrier-based barrier in its place measured about twice the epoch time.)
__device__ __forceinline__ void bar_sync_named(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

__device__ __forceinline__ int ld_volatile_shared(const int* p) { return *reinterpret_cast<const volatile int*>(p); }
__device__ __forceinline__ void st_volatile_shared(int* p, int v) { *reinterpret_cast<volatile int*>(p) = v; }

__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ void mma_bf16_k16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ void mma_bf16_k8(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t b0) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(b0));
}

// x = hi + lo with hi the TF32 rounding of x and lo the TF32 rounding of the rest: the
// split of the 3xTF32 scheme (products hi*hi + hi*lo + lo*hi, the lo*lo term dropped),
// which keeps about fp32 accuracy on the TF32 tensor-core path.
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_bits(x);
  lo = tf32_bits(x - __uint_as_float(hi));
}

// Fragments by ldmatrix: each 8x8 b16 matrix is 8 rows of 16 bytes, so for 32-bit data it
// is 8 rows x 4 words and thread l receives row l/4, word l%4 -- the layout of the mma
// fragments below for tf32 (words) and bf16 (pairs).  One instruction replaces four (x4)
// or two (x2) shared-memory loads per lane; lanes 0-7, 8-15, 16-23, 24-31 give the row
// addresses of matrices 0..3 (16-byte aligned: rows are multiples of 16 bytes apart and
// start at multiples of 4 words).
__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t (&r)[4]) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr)
               : "memory");
}
__device__ __forceinline__ void ldsm_x2(uint32_t addr, uint32_t (&r)[2]) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(addr)
               : "memory");
}

// One 16x8 tile of G = X X^T: rows r0.., columns n0.. (fragment layouts of mma.m16n8k8 /
// m16n8k16: g = lane / 4 selects the row, t = lane % 4 the k pair or k element).  fp32
// rows: 3xTF32 from the block's rows split once into tf32 high and low parts (Xh, Xl),
// three mma per k step (hi*hi into one accumulator, hi*lo + lo*hi into another, summed at
// the end), so G carries close to fp32 precision like the rest of the fp32 form; b = X h
// is computed separately in fp32.
__device__ __forceinline__ void gram_tile(const float* Xh, const float* Xl, int sw, int kpad, int r0, int n0,
                                          float (&d)[4], int lane) {
  const int rr = lane & 7, mi = lane >> 3;
  // A: matrices (rows r0.., words k0..), (rows r0+8.., k0..), (r0.., k0+4..), (r0+8.., k0+4..)
  const uint32_t a_off = 4u * ((r0 + rr + (mi & 1) * 8) * sw + (mi >> 1) * 4);
  // B: matrices (rows n0.., words k0..), (rows n0.., k0+4..) from lanes 0..15
  const uint32_t b_off = 4u * ((n0 + rr) * sw + (mi & 1) * 4);
  const uint32_t hs = smem_u32(Xh), ls = smem_u32(Xl);
  float d2[4] = {0.f, 0.f, 0.f, 0.f};  // the cross terms hi*lo + lo*hi
  const int kmma = (kpad + 7) / 8 * 8;  // the row padded with zeros to whole k8 steps
#pragma unroll 2
  for (int k0 = 0; k0 < kmma; k0 += 8) {
    uint32_t ah[4], al[4], bh[2], bl[2];
    ldsm_x4(hs + a_off + 4u * k0, ah);
    ldsm_x4(ls + a_off + 4u * k0, al);
    ldsm_x2(hs + b_off + 4u * k0, bh);
    ldsm_x2(ls + b_off + 4u * k0, bl);
    mma_tf32(d2, ah, bl);
    mma_tf32(d2, al, bh);
    mma_tf32(d, ah, bh);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] += d2[i];
}
__device__ __forceinline__ void gram_tile(const __nv_bfloat16* X, int sw, int kpad, int r0, int n0, float (&d)[4],
                                          int lane) {
  const int g = lane >> 2, t = lane & 3, rr = lane & 7, mi = lane >> 3;
  const uint32_t* Xw = reinterpret_cast<const uint32_t*>(X);
  const uint32_t a_addr = smem_u32(Xw + (r0 + rr + (mi & 1) * 8) * sw + (mi >> 1) * 4);
  const uint32_t b_addr = smem_u32(Xw + (n0 + rr) * sw + (mi & 1) * 4);
  const int kw = kpad / 2;  // words per row; a multiple of 4
  float d2[4] = {0.f, 0.f, 0.f, 0.f};
  int k = 0;
#pragma unroll 2
  for (; k + 16 <= kw; k += 16) {
    uint32_t a[4], b[2], a2[4], b2[2];
    ldsm_x4(a_addr + 4u * k, a);
    ldsm_x2(b_addr + 4u * k, b);
    ldsm_x4(a_addr + 4u * (k + 8), a2);
    ldsm_x2(b_addr + 4u * (k + 8), b2);
    mma_bf16_k16(d, a, b);
    mma_bf16_k16(d2, a2, b2);
  }
  if (k + 8 <= kw) {
    uint32_t a[4], b[2];
    ldsm_x4(a_addr + 4u * k, a);
    ldsm_x2(b_addr + 4u * k, b);
    mma_bf16_k16(d, a, b);
    k += 8;
  }
  if (k < kw) {
    const uint32_t* A0 = Xw + (r0 + g) * sw;
    const uint32_t* B = Xw + (n0 + g) * sw;
    mma_bf16_k8(d2, A0[k + t], A0[8 * sw + k + t], B[k + t]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] += d2[i];
}

// The Gram tile of a block's rows in either form.
__device__ __forceinline__ void block_gram_tile(const CtaRegion& C, const char* X, const float*, int kpad, int r0,
                                                int n0, float (&d)[4], int lane) {
  gram_tile(C.xhi, C.xlo, C.sw, kpad, r0, n0, d, lane);
  (void)X;
}
__device__ __forceinline__ void block_gram_tile(const CtaRegion& C, const char* X, const __nv_bfloat16*, int kpad,
                                                int r0, int n0, float (&d)[4], int lane) {
  gram_tile(reinterpret_cast<const __nv_bfloat16*>(X), C.sw, kpad, r0, n0, d, lane);
}

// Reduce-scatter of 8 per-lane partials: lane l ends with the warp total of index l % 8.
__device__ __forceinline__ float reduce_scatter8(float (&v)[8], int lane) {
#pragma unroll
  for (int lvl = 0; lvl < 3; ++lvl) {
    const int half = 4 >> lvl;
    const bool up = (lane & half) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = up ? v[i] : v[i + half];
      const float keep = up ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, half);
    }
  }
  const float x = v[0] + __shfl_xor_sync(kFull, v[0], 8);
  return x + __shfl_xor_sync(kFull, x, 16);
}

// b_j = <h, x_j> for 8 rows x_j of a block, one warp; lane j ends with b_{j % 8}.  Four
// warps cover a block's 32 rows, beside the six warps of its Gram tiles.
template <typename Store, int NV>
__device__ __forceinline__ float cta_dots8(const char* X, int sw, const float* h, const Shape& s, int lane) {
  using Raw = typename Vec<Store>::Raw;
  float p[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) p[j] = 0.f;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    if (v < s.nvec) {
      const float4 hv = reinterpret_cast<const float4*>(h)[v];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float w[4];
        nd::unpack(reinterpret_cast<const Raw*>(X + static_cast<size_t>(j) * sw * 4)[v], w);
        p[j] = fmaf(hv.x, w[0], p[j]);
        p[j] = fmaf(hv.y, w[1], p[j]);
        p[j] = fmaf(hv.z, w[2], p[j]);
        p[j] = fmaf(hv.w, w[3], p[j]);
      }
    }
  }
  return reduce_scatter8(p, lane);
}

// The serial part of a block, lane j holding row j.  With b_j = c^t beta_j after step t,
//   e_t = c^t beta_t - v_t,   beta_j += k_t G_jt  (j > t),   k_t = -eta e_t c^-(t+1),
// and lane j can form its own k_j as soon as step j - 1 is applied:
//   k_j = beta_j (-eta / c) + eta v_j c^-(j+1),
// so a step is one shuffle (k_t from lane t) and two FMAs on the dependent path -- the
// broadcast k_t updates every lane's beta, and lane t + 1's k is then final.  (Lanes at
// or below t keep updating values nothing reads again.)  Returns this lane's squared
// error and leaves -eta e_t in nesh[t] and k_t = -eta e_t c^-(t+1) in ksh[t] (both 0 past
// the block's last rating).
__device__ __forceinline__ float cta_chain(const float* G, const float* bsh, const int2* rvb, float* nesh,
                                           float* ksh, const float* cpow, const float* cinv, int nr, float step,
                                           float c, int lane) {
  float beta = bsh[lane];
  const float v = __int_as_float(rvb[lane].y);  // unused past the block's last rating
  const float a = -step / c;
  const float bj = step * v * cinv[lane];
  const float cp = cpow[lane];
  float k = fmaf(beta, a, bj);  // final for lane 0
  float my_e = 0.f;
  // All kHB steps run, without a branch per step: steps past the block's last rating
  // only change values nothing reads.
#pragma unroll
  for (int t = 0; t < kHB; ++t) {
    const float g = G[lane * kGStride + t];  // independent of the chain: loaded ahead
    const float kt = __shfl_sync(kFull, k, t);
    my_e = lane == t ? fmaf(cp, beta, -v) : my_e;  // e_t, from beta before its own update
    beta = fmaf(kt, g, beta);
    k = fmaf(beta, a, bj);
  }
  nesh[lane] = lane < nr ? -step * my_e : 0.f;
  ksh[lane] = lane < nr ? -step * my_e * cinv[lane] : 0.f;
  return lane < nr ? my_e * my_e : 0.f;
}

// Rows [t0, t1) of a block (one warp): form h at row t0 from the rows before it, then
// update each row and h.  The last warp also leaves h after the block in h_out, or, after
// the visit's final block, writes it to the column's row `hrow` in HBM.
template <typename Store, int NV>
__device__ __forceinline__ void cta_rows(const char* X, int sw, const int2* rvb, const float* nesh, const float* ksh,
                                         const float* cpow,
                                         const float* h_in, float* h_out, int nr, int t0, int t1, bool last, float c,
                                         void* W, const Shape& s, uint32_t colkey, Store* hrow, uint32_t hkey,
                                         int lane) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  // h_{t0} = c^{t0} (h_0 + sum_{s < t0} k_s w_s), two partial sums
  const int pre = min(t0, nr);
  float h[NV][E], h2[NV][E];
  {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int v = lane + 32 * q;
      const float4 x = v < s.nvec ? reinterpret_cast<const float4*>(h_in)[v] : make_float4(0.f, 0.f, 0.f, 0.f);
      h[q][0] = x.x; h[q][1] = x.y; h[q][2] = x.z; h[q][3] = x.w;
#pragma unroll
      for (int e = 0; e < E; ++e) h2[q][e] = 0.f;
    }
  }
#pragma unroll 4
  for (int t = 0; t < pre; ++t) {
    const float coef = ksh[t];
    const Raw* row = reinterpret_cast<const Raw*>(X + static_cast<size_t>(t) * sw * 4);
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int v = lane + 32 * q;
      float wo[E];
      nd::unpack(v < s.nvec ? row[v] : nd::zero_raw<Raw>(), wo);
      if (t & 1) {
#pragma unroll
        for (int e = 0; e < E; ++e) h2[q][e] = fmaf(coef, wo[e], h2[q][e]);
      } else {
#pragma unroll
        for (int e = 0; e < E; ++e) h[q][e] = fmaf(coef, wo[e], h[q][e]);
      }
    }
  }
  {
    const float cp = cpow[pre];
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
      for (int e = 0; e < E; ++e) h[q][e] = cp * (h[q][e] + h2[q][e]);
  }
  const int end = min(t1, nr);
  for (int t = t0; t < end; ++t) {
    const float ne = nesh[t];
    const Raw* row = reinterpret_cast<const Raw*>(X + static_cast<size_t>(t) * sw * 4);
    float wn[NV][E];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int v = lane + 32 * q;
      float wo[E];
      nd::unpack(v < s.nvec ? row[v] : nd::zero_raw<Raw>(), wo);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        wn[q][e] = fmaf(ne, h[q][e], c * wo[e]);
        h[q][e] = fmaf(ne, wo[e], c * h[q][e]);
      }
    }
    const int r = rvb[t].x;
    store_row<Store, NV>(W, r, s, lane, wn, nd::row_key(r, colkey));
  }
  if (last) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int v = lane + 32 * q;
      if (v >= s.nvec) continue;
      if (hrow)
        nd::store_vec<Store, true>(hrow, v, h[q], hkey + 4u * static_cast<uint32_t>(v));
      else
        reinterpret_cast<float4*>(h_out)[v] = make_float4(h[q][0], h[q][1], h[q][2], h[q][3]);
    }
  }
}

// Join of the block's live warps before a block visit: all of them enter the visit or
// none does.  A warp whose wait runs out blocks the join's current phase with a pending
// transaction byte (mbarrier.expect_tx), so a warp arriving later cannot complete it;
// if the phase had completed just before (the block then lands on the next phase), every
// warp is in, so the warp undoes the byte (complete_tx) and enters too.  Both operations
// are atomic on the barrier, so exactly one of the two outcomes holds for every warp.
__device__ __forceinline__ bool cta_join(uint32_t bar, uint32_t& phase, const nomad::AsyncArgs& a, int lane) {
  int ok = 1;
  if (lane == 0) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
    if (!mbar_wait_bounded(bar, phase, a)) {
      asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
      if (mbar_test_wait(bar, phase)) {
        asm volatile("mbarrier.complete_tx.relaxed.cta.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
      } else {
        atomicCAS(&a.ctrl[1], 0, nd::kDevErrTimeout);
        ok = 0;
      }
    }
  }
  phase ^= 1u;
  return __shfl_sync(kFull, ok, 0) != 0;
}

struct CtaVisitOut {
  float e2;
  int len;
};

// Rows of block b of the visit into its shared-memory slot (warp wib of nw warps copies
// rows wib, wib + nw, ...).
__device__ __forceinline__ void cta_stage_rows(const CtaRegion& C, int b, int len, const void* W, int row_bytes,
                                               int nw, int wib, int lane) {
  const int2* rvb = C.rv + (b % kHRv) * kHB;
  const int nrb = min(kHB, len - b * kHB);
  char* dst = C.rows + static_cast<size_t>(b % kHStages) * kHB * C.sw * 4;
  const int cpr = row_bytes / 16;
  for (int r = wib; r < nrb; r += nw) {
    const char* src = static_cast<const char*>(W) + static_cast<int64_t>(rvb[r].x) * row_bytes;
    const uint32_t d = smem_u32(dst + static_cast<size_t>(r) * C.sw * 4);
    for (int k = lane; k < cpr; k += 32) cp16(d + 16 * k, src + 16 * k);
  }
}
// Rating indices of block b (missing entries zero).
__device__ __forceinline__ void cta_stage_rv(const CtaRegion& C, int b, int64_t start, int len, const int2* ratings,
                                             int tid, int nthr) {
  int2* dst = C.rv + (b % kHRv) * kHB;
  for (int t = tid; t < kHB; t += nthr) {
    const int o = b * kHB + t;
    if (o < len) cp8(smem_u32(dst + t), ratings + start + o);
    else dst[t] = make_int2(0, 0);
  }
}

// fp32 rows: the tf32 high and low parts of block b's rows for the Gram tiles, split by
// the threads that staged them -- each thread its own chunks (rows wib, wib + nw, ... and
// 16-byte chunks lane, lane + 32, ... of each, as cta_stage_rows copies them), once its
// copies have landed, so no other thread's copies need to be waited for.
template <typename Store>
__device__ __forceinline__ void cta_split_rows(const CtaRegion& C, int b, int len, int row_bytes, int nw, int wib,
                                               int lane) {
  if (sizeof(Store) != 4) return;
  const int nrb = min(kHB, len - b * kHB);
  const float* X = reinterpret_cast<const float*>(C.rows + static_cast<size_t>(b % kHStages) * kHB * C.sw * 4);
  const int cpr = row_bytes / 16;
  for (int r = wib; r < nrb; r += nw)
    for (int k = lane; k < cpr; k += 32) {
      const float4 x = reinterpret_cast<const float4*>(X + r * C.sw)[k];
      uint4 h, l;
      split_tf32(x.x, h.x, l.x);
      split_tf32(x.y, h.y, l.y);
      split_tf32(x.z, h.z, l.z);
      split_tf32(x.w, h.w, l.w);
      reinterpret_cast<uint4*>(C.xhi + r * C.sw)[k] = h;
      reinterpret_cast<uint4*>(C.xlo + r * C.sw)[k] = l;
    }
}

// One visit of priority token `tok` by the block's nw live warps (all of them call it).
// The last warp writes the column back; warp 0 returns the squared errors.  The shared
// region is free again when this returns (the warps' long-visit rings alias it).
template <typename Store, int NV>
__device__ __forceinline__ void cta_visit(int tok, const nomad::AsyncArgs& a, const Shape& s, const CtaRegion& C, int nw, int wib,
                          int lane, CtaVisitOut& out) {
  const int tid = wib * 32 + lane;
  const int nthr = nw * 32;
  const int kpad = s.row_bytes / static_cast<int>(sizeof(Store));
  const int4 ma = __ldcg(a.mailbox + 4 * static_cast<int64_t>(tok));
  const int4 mb = __ldcg(a.mailbox + 4 * static_cast<int64_t>(tok) + 1);
  const int64_t start = lo_hi(ma.x, ma.y);
  const int len = ma.z, pos = ma.w, ep = mb.x;
  const int nblk = (len + kHB - 1) / kHB;
  const float step = __ldg(&a.steps[min(ep, a.n_steps - 1)]);
  const float c = 1.f - step * a.lambda;
  const uint32_t colkey =
      nd::hash32(a.seed32 ^ static_cast<uint32_t>(tok) * 0x85EBCA77u ^ static_cast<uint32_t>(ep) * 0xC2B2AE3Du);
  void* W = a.f.W;
  Store* hrow = reinterpret_cast<Store*>(static_cast<char*>(a.f.H) + static_cast<int64_t>(tok) * s.row_bytes);
  const uint32_t hkey = nd::hash32(colkey ^ static_cast<uint32_t>(pos) * 0x27D4EB2Fu);
  // rating indices of the first blocks, then the held column (fp32, h buffer 0) while
  // they are in flight
  for (int b = 0; b < 4 && b < nblk; ++b) cta_stage_rv(C, b, start, len, a.ratings, tid, nthr);
  cp_async_commit();
  for (int v = tid; v < s.nvec; v += nthr) {
    float x[4];
    nd::load_vec_cg<Store>(hrow, v, x);
    reinterpret_cast<float4*>(C.h)[v] = make_float4(x[0], x[1], x[2], x[3]);
  }
  // zero the columns past an fp32 row that the last k8 tile reads (staged rows and the
  // tf32 parts, which follow them)
  if (sizeof(Store) == 4 && (kpad & 7) != 0)
    for (int r = tid; r < (kHStages + 2) * kHB; r += nthr)
      *reinterpret_cast<float4*>(C.rows + static_cast<size_t>(r) * C.sw * 4 + kpad * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid == 0) {  // c^k and c^-(k+1)
    float x = 1.f, y = 1.f / c, yi = y;
    for (int i = 0; i <= kHB; ++i) {
      C.cpow[i] = x;
      x *= c;
      if (i < kHB) {
        C.cinv[i] = yi;
        yi *= y;
      }
    }
  }
  cp_async_wait<0>();
  bar_sync_named(nthr);
  cta_stage_rows(C, 0, len, W, s.row_bytes, nw, wib, lane);
  cp_async_commit();
  if (nblk > 1) cta_stage_rows(C, 1, len, W, s.row_bytes, nw, wib, lane);
  cp_async_commit();
  cp_async_wait<1>();  // this thread's copies of block 0's rows have landed
  cta_split_rows<Store>(C, 0, len, s.row_bytes, nw, wib, lane);
  float e2 = 0.f;
  const int rpg = (kHB + nw - 1) / nw;
  for (int i = 0; i < nblk; ++i) {
    cp_async_wait<1>();  // rows of block i and indices of block i + 2 have landed
    bar_sync_named(nthr);
    const float* hcur = C.h + (i & 1) * kpad;
    float* hnext = C.h + ((i + 1) & 1) * kpad;
    const char* X = C.rows + static_cast<size_t>(i % kHStages) * kHB * C.sw * 4;
    const int2* rvb = C.rv + (i % kHRv) * kHB;
    const int nr = min(kHB, len - i * kHB);
    // Gram tiles (lower triangle of 16x8 tiles) and the dots with h (four quarters)
    for (int it = wib; it < 10; it += nw) {
      if (it < 6) {
        const int r0 = it < 2 ? 0 : 16;
        const int n0 = it < 2 ? 8 * it : 8 * (it - 2);
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        block_gram_tile(C, X, static_cast<const Store*>(nullptr), kpad, r0, n0, d, lane);
        const int g = lane >> 2, t = lane & 3;
        C.G[(r0 + g) * kGStride + n0 + 2 * t] = d[0];
        C.G[(r0 + g) * kGStride + n0 + 2 * t + 1] = d[1];
        C.G[(r0 + g + 8) * kGStride + n0 + 2 * t] = d[2];
        C.G[(r0 + g + 8) * kGStride + n0 + 2 * t + 1] = d[3];
      } else {
        const int r0 = 8 * (it - 6);
        const float bv = cta_dots8<Store, NV>(X + static_cast<size_t>(r0) * C.sw * 4, C.sw, hcur, s, lane);
        if (lane < 8) C.bsh[r0 + lane] = bv;
      }
    }
    bar_sync_named(nthr);
    // While warp 0 runs the chain, the other warps issue the copies of block i + 2's rows
    // and block i + 4's indices (issuing them took 900-2,000 cycles per warp, which at
    // the start of the block delayed the Gram tiles); with one warp, warp 0 issues them
    // after the chain.  Each thread commits one copy group per block either way.
    if (wib == 0) e2 += cta_chain(C.G, C.bsh, rvb, C.nesh, C.ksh, C.cpow, C.cinv, nr, step, c, lane);
    // fp32 rows: the tf32 parts of block i + 1, split by the threads that staged it (every
    // warp for block 1, the copying warps after it; warp 0 after its chain)
    if (sizeof(Store) == 4 && i + 1 < nblk) {
      const bool all = i == 0;
      if (all || wib != 0 || nw == 1) {
        cp_async_wait<0>();
        cta_split_rows<Store>(C, i + 1, len, s.row_bytes, all ? nw : (nw > 1 ? nw - 1 : 1),
                              all ? wib : (nw > 1 ? wib - 1 : 0), lane);
      }
    }
    if (wib != 0 || nw == 1) {
      const int sw_ = nw > 1 ? wib - 1 : 0, snw = nw > 1 ? nw - 1 : 1;
      if (i + 2 < nblk) cta_stage_rows(C, i + 2, len, W, s.row_bytes, snw, sw_, lane);
      if (i + 4 < nblk) cta_stage_rv(C, i + 4, start, len, a.ratings, sw_ * 32 + lane, snw * 32);
    }
    cp_async_commit();
    bar_sync_named(nthr);
    cta_rows<Store, NV>(X, C.sw, rvb, C.nesh, C.ksh, C.cpow, hcur, hnext, nr, wib * rpg, (wib + 1) * rpg, wib == nw - 1, c,
                        W, s, colkey, i + 1 == nblk ? hrow : nullptr, hkey, lane);
  }
  cp_async_wait<0>();
  bar_sync_named(nthr);  // rows and column written; the region is free
  if (wib == 0) {
    out.e2 = nd::warp_allreduce(e2, 32);
    out.len = len;
  }
}

// ---- stages of the token pipeline -------------------------------------------------------
// D (issued by the pop warp): the mailbox and the held column, into an inbox slot.
// R (compute warp): needs the mailbox -- the visit's rating indices when it holds more
// ratings than the mailbox carries, and the route's next visit with its first ratings
// (they go into the next hop's mailbox).
__device__ __forceinline__ void stage_r(char* slot, const nomad::AsyncArgs& a, int heavy_min, int lane) {
  const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slot);
  const int4 ma = hd->a, mb = hd->b;
  const int64_t start = lo_hi(ma.x, ma.y);
  const uint32_t d = smem_u32(slot);
  const int nidx = ma.z > kPF || ma.z >= heavy_min ? min(ma.z, kChunk) : 0;
  if (lane < nidx) cp8(d + static_cast<uint32_t>(offsetof(SlotHdr, rv)) + 8 * lane, a.ratings + start + lane);
  if (lane >= 29) {
    const int nseg = mb.y & 0x7fffffff;
    const int npos = ma.w + 1 < nseg ? ma.w + 1 : 0;
    const int k = lane - 29;
    cp16(d + static_cast<uint32_t>(offsetof(SlotHdr, nxt)) + 16 * k, a.segx + 3 * (lo_hi(mb.z, mb.w) + npos) + k);
  }
}

__device__ __forceinline__ bool entry_valid(unsigned long long e, unsigned head) {
  return static_cast<unsigned>(e >> 32) == head && (e & 0x80000000ull) == 0;
}

// ---- hand-off between the warps of a block ---------------------------------------------
// Compute warps touch no global queue: the pop warp moves tokens from each compute warp's
// ring into its inbox -- an entry plus a slot that a bulk copy fills with the token's
// mailbox and held column -- and the push warp moves processed tokens from the outboxes
// into the rings, one gpu-scope release fence per batch.  Entries carry the producer's
// count in their high word, so a slot holds a new entry when that count is the one
// expected.  A compute warp frees an inbox slot when its token's visit is done.
constexpr int kInbox = 8;
constexpr int kOutbox = 8;

struct WarpBox {
  unsigned long long inbox[kInbox];       // (count << 32) | token, written by the pop warp
  unsigned long long outbox[kOutbox][2];  // (count << 32) | token, then (queue << 1) | retire
  unsigned long long bars[kInbox];        // mbarrier of each inbox slot's copy
  unsigned in_head;                       // inbox slots the compute warp has freed
  unsigned out_head;                      // outbox entries the push warp has published
  unsigned pad[2];
};
static_assert(sizeof(WarpBox) == 272, "box layout");
constexpr int kBoxWords = sizeof(WarpBox) / 8;
constexpr int kBoxBarWord = offsetof(WarpBox, bars) / 8;       // initialised as mbarriers
constexpr int kBoxCountWord = offsetof(WarpBox, in_head) / 8;  // counters start at zero

__device__ __forceinline__ unsigned long long ld_acquire_cta_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.cta.shared::cta.b64 %0, [%1];" : "=l"(v) : "r"(smem_u32(p)) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(p)), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_cta_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}

// A processed token into the warp's outbox (lane 0): qr = (queue << 1) | retire.  Waits
// (bounded) for room; false when the launch is stopping or the wait ran out.
__device__ __forceinline__ bool outbox_put(WarpBox& B, unsigned& out_tail, int tok, unsigned qr, const CtaHdr* hdr,
                                           const nomad::AsyncArgs& a) {
  if (out_tail - ld_acquire_cta_u32(&B.out_head) >= static_cast<unsigned>(kOutbox)) {
    const uint64_t t0 = nd::globaltimer();
    while (out_tail - ld_acquire_cta_u32(&B.out_head) >= static_cast<unsigned>(kOutbox)) {
      __nanosleep(64);
      if (ld_volatile_shared(&hdr->stop)) return false;
      if (static_cast<int64_t>(nd::globaltimer() - t0) > a.budget_ns) {
        atomicCAS(&a.ctrl[1], 0, nd::kDevErrTimeout);
        return false;
      }
    }
  }
  unsigned long long* e = B.outbox[out_tail % kOutbox];
  e[1] = qr;
  st_release_cta_u64(&e[0], (static_cast<unsigned long long>(out_tail) << 32) | static_cast<unsigned>(tok));
  ++out_tail;
  return true;
}

// The pop warp: lane i < nc fills compute warp i's inbox from its ring (two probes per
// round); lane 31 takes the block's priority tokens.  Lane 0 also watches for the end of
// the launch (every token retired, an error, or no progress within the budget) and raises
// the block's stop flag.
__device__ void pop_warp(const nomad::AsyncArgs& a, CtaHdr* hdr, WarpBox* boxes, char* slots_all, int slot_bytes,
                         int row_bytes, int ncw, int nc_live, int lane) {
  const int P = a.P;
  const int w0 = static_cast<int>(blockIdx.x) * ncw;
  const bool mine = lane < nc_live;
  const bool heavy_lane = a.cta_heavy && lane == 31;
  unsigned long long* ring = nullptr;
  unsigned mask = 0, head = 0;
  if (mine) {
    ring = a.ring_lo + static_cast<int64_t>(w0 + lane) * (a.mask_lo + 1);
    mask = a.mask_lo;
    head = a.heads[w0 + lane];
  } else if (heavy_lane) {
    ring = a.ring_hi + static_cast<int64_t>(blockIdx.x) * (a.mask_hi + 1);
    mask = a.mask_hi;
    head = a.heads[P + blockIdx.x];
  }
  unsigned in_tail = 0;  // inboxes start empty every launch
  unsigned long long seen = ~0ull;
  uint64_t idle_since = nd::globaltimer();
  unsigned backoff = 32, rounds = 0;
  while (true) {
    unsigned long long p0 = ~0ull, p1 = ~0ull;
    if (ring) {
      p0 = ld_acquire_u64(ring + (head & mask));
      if (mine) p1 = ld_acquire_u64(ring + ((head + 1) & mask));
    }
    int took = 0;
    if (mine) {
      WarpBox& B = boxes[lane];
      const unsigned used = in_tail - ld_acquire_cta_u32(&B.in_head);  // freed slots: their reads are done
      if (used < static_cast<unsigned>(kInbox) && entry_valid(p0, head)) {
        fence_proxy_async_global();  // the acquired mailbox and column, for the bulk copies
        fence_proxy_async_shared();  // the slot's earlier generic reads precede the copy's writes
        const int ntake = used + 1 < static_cast<unsigned>(kInbox) && entry_valid(p1, head + 1) ? 2 : 1;
        for (int i = 0; i < ntake; ++i) {
          const unsigned tok = static_cast<unsigned>((i ? p1 : p0) & 0x7fffffffull);
          const int sl = static_cast<int>(in_tail % kInbox);
          char* slot = slots_all + (static_cast<size_t>(lane) * kInbox + sl) * slot_bytes;
          const uint32_t bar = smem_u32(&B.bars[sl]);
          mbar_expect_tx(bar, static_cast<uint32_t>(64 + row_bytes));
          tma_row(smem_u32(slot), a.mailbox + 4 * static_cast<int64_t>(tok), 64u, bar);
          tma_row(smem_u32(slot + sizeof(SlotHdr)), static_cast<const char*>(a.f.H) + static_cast<int64_t>(tok) * row_bytes,
                  static_cast<uint32_t>(row_bytes), bar);
          st_release_cta_u64(&B.inbox[sl], (static_cast<unsigned long long>(in_tail) << 32) | tok);
          ++in_tail;
          ++head;
        }
        took = ntake;
      }
    } else if (heavy_lane) {
      if (ld_acquire_cta_u32(reinterpret_cast<const unsigned*>(&hdr->hv_tok)) == 0xffffffffu && entry_valid(p0, head)) {
        st_release_cta_u32(reinterpret_cast<unsigned*>(&hdr->hv_tok), static_cast<unsigned>(p0 & 0x7fffffffull));
        ++head;
        took = 1;
      }
    }
    const bool any = __any_sync(kFull, took != 0);
    int stop = 0;
    if (lane == 0 && (!any || (++rounds & 15) == 0)) {
      if (nd::ld_acquire(&a.ctrl[1]) != 0 || nd::ld_acquire(&a.ctrl[0]) >= a.n_active) {
        stop = 1;
      } else {
        const unsigned long long pr = nd::ld_relaxed_u64(a.progress);
        const uint64_t now = nd::globaltimer();
        if (pr != seen) {
          seen = pr;
          idle_since = now;
        } else if (static_cast<int64_t>(now - idle_since) > a.budget_ns) {
          atomicCAS(&a.ctrl[1], 0, nd::kDevErrTimeout);
          stop = 1;
        }
      }
      if (stop) st_volatile_shared(&hdr->stop, 1);
    }
    if (__shfl_sync(kFull, stop, 0)) break;
    if (any) {
      backoff = 32;
    } else {
      __nanosleep(backoff);
      backoff = min(backoff * 2, 256u);
    }
  }
  if (mine) {
    a.heads[w0 + lane] = head;
    // copies still in flight land before the block's shared memory goes away (bounded)
    WarpBox& B = boxes[lane];
    for (unsigned c = in_tail > kInbox ? in_tail - kInbox : 0u; c < in_tail; ++c)
      for (int it = 0; it < (1 << 16) && !mbar_try_wait(smem_u32(&B.bars[c % kInbox]), (c / kInbox) & 1u); ++it) {
      }
  } else if (heavy_lane) {
    a.heads[P + blockIdx.x] = head;
  }
}

// The push warp: lane i < nc publishes up to four entries of compute warp i's outbox per
// round, after one release fence of the whole warp (cumulative over the compute warps'
// stores, which the outbox acquire ordered before it).
__device__ void push_warp(const nomad::AsyncArgs& a, const CtaHdr* hdr, WarpBox* boxes, int nc_live, int lane) {
  const int P = a.P;
  const bool mine = lane < nc_live;
  unsigned out_head = 0;
  unsigned pend = 0;  // published hops not yet added to the progress counter
  unsigned backoff = 32;
  while (true) {
    int n = 0;
    unsigned tok[4], qr[4];
    if (mine) {
      WarpBox& B = boxes[lane];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        tok[k] = 0;
        qr[k] = 0;
        if (n == k) {
          const unsigned long long* e = B.outbox[(out_head + k) % kOutbox];
          const unsigned long long e0 = ld_acquire_cta_u64(&e[0]);
          if (static_cast<unsigned>(e0 >> 32) == out_head + k) {
            tok[k] = static_cast<unsigned>(e0) & 0x7fffffffu;
            qr[k] = static_cast<unsigned>(e[1]);
            n = k + 1;
          }
        }
      }
    }
    if (__any_sync(kFull, n > 0)) {
      fence_acq_rel_gpu();
      unsigned seq[4] = {0u, 0u, 0u, 0u};
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < n && !(qr[k] & 1u)) seq[k] = atomicAdd(&a.tails[qr[k] >> 1], 1u);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (k >= n) continue;
        if (qr[k] & 1u) {
          if (a.finish_ns) a.finish_ns[tok[k]] = nd::globaltimer();
          atomicAdd(&a.ctrl[0], 1);
        } else {
          const int q = static_cast<int>(qr[k] >> 1);
          unsigned long long* rq = q >= P ? a.ring_hi + static_cast<int64_t>(q - P) * (a.mask_hi + 1) + (seq[k] & a.mask_hi)
                                          : a.ring_lo + static_cast<int64_t>(q) * (a.mask_lo + 1) + (seq[k] & a.mask_lo);
          st_relaxed_u64(rq, (static_cast<unsigned long long>(seq[k]) << 32) | tok[k]);
        }
      }
      if (n > 0) {
        out_head += static_cast<unsigned>(n);
        st_release_cta_u32(&boxes[lane].out_head, out_head);
        pend += static_cast<unsigned>(n);
        if (pend >= 64) {
          atomicAdd(a.progress, static_cast<unsigned long long>(pend));
          pend = 0;
        }
      }
      backoff = 32;
    } else {
      if (ld_volatile_shared(&hdr->stop)) break;
      __nanosleep(backoff);
      backoff = min(backoff * 2, 256u);
    }
  }
  if (pend) atomicAdd(a.progress, static_cast<unsigned long long>(pend));
}

// Threads per block of the pipelined kernel: compute warps plus the pop and push warps.
// Fewer compute warps leave more registers to each thread (65,536 per SM over the block);
// measured on the 480,189 x 17,770 workload (ms per epoch, fp32 / bf16): 14 compute warps
// (128 registers) 86.1 / 88.2, 12 (128) 83.7 / 86.2, 11 (128) 85.2 / 86.1, 10 (168)
// 81.5 / 87.3, 8 (168) 85.6 / 96.2.
template <typename Store>
struct Async2Block {
  static constexpr int kThreads = sizeof(Store) == 4 ? 12 * 32 : 14 * 32;
};

template <typename Store, int NV>
__global__ void __launch_bounds__(Async2Block<Store>::kThreads, 1) nomad_async2_kernel(nomad::AsyncArgs a) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  extern __shared__ __align__(128) char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int ncw = static_cast<int>(blockDim.x >> 5) - 2;  // compute warps (workers) per block
  const int P = a.P;
  const int nc_live = min(ncw, P - static_cast<int>(blockIdx.x) * ncw);
  Shape s;
  s.nvec = a.f.nvec;
  s.red_width = a.f.red_width;
  s.row_bytes = a.f.kpad * static_cast<int>(sizeof(Store));
  s.heavy_min = min(max(a.heavy_min, 1), kChunk + 1);  // longer visits always take the blocked path
  s.slot_bytes = static_cast<int>(sizeof(SlotHdr)) + s.row_bytes;
  // shared memory: block header | boxes | inbox slots | long-visit rings (the block visit
  // region aliases them) | mbarriers | gather buffers; per compute warp where repeated
  const size_t ring_bytes = static_cast<size_t>(kRing) * kBlk * s.row_bytes;
  size_t region_bytes = static_cast<size_t>(ncw) * ring_bytes;
  if (a.cta_heavy) region_bytes = max(region_bytes, cta_region_bytes(a.f.kpad, static_cast<int>(sizeof(Store))));
  CtaHdr* hdr = reinterpret_cast<CtaHdr*>(smem);
  WarpBox* boxes = reinterpret_cast<WarpBox*>(smem + kCtaHdrBytes);
  char* slots_all = reinterpret_cast<char*>(boxes + ncw);
  char* region = slots_all + static_cast<size_t>(ncw) * kInbox * s.slot_bytes;
  char* bars = region + region_bytes;
  char* gathers = bars + static_cast<size_t>(ncw) * kBarBytes;
  for (int i = threadIdx.x; i < ncw * kBoxWords; i += blockDim.x) {
    const int wd = i % kBoxWords;
    if (wd >= kBoxCountWord) reinterpret_cast<unsigned long long*>(boxes)[i] = 0ull;
    else if (wd >= kBoxBarWord) mbar_init(smem_u32(reinterpret_cast<unsigned long long*>(boxes) + i), 1);
    else reinterpret_cast<unsigned long long*>(boxes)[i] = ~0ull;
  }
  const uint32_t join_bar = smem_u32(&hdr->join);
  if (threadIdx.x == 0) {
    hdr->hv_tok = -1;
    hdr->stop = 0;
    mbar_init(join_bar, static_cast<uint32_t>(max(nc_live, 1)));
  }
  Ring R;
  R.rows = region + static_cast<size_t>(min(wib, ncw - 1)) * ring_bytes;
  R.bars = smem_u32(bars + static_cast<size_t>(min(wib, ncw - 1)) * kBarBytes);
  R.gather = reinterpret_cast<float*>(gathers + static_cast<size_t>(min(wib, ncw - 1)) * 128);
  R.phase = 0;
  if (lane == 0 && NOMAD_STAGE_TMA && wib < ncw)
    for (int i = 0; i < kRing; ++i) mbar_init(R.bars + 8u * i, 1);
  fence_mbar_init();
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0 && a.finish_ns) a.finish_ns[a.f.n] = nd::globaltimer();
  if (wib == ncw) {
    pop_warp(a, hdr, boxes, slots_all, s.slot_bytes, s.row_bytes, ncw, nc_live, lane);
    return;
  }
  if (wib == ncw + 1) {
    push_warp(a, hdr, boxes, nc_live, lane);
    return;
  }
  if (wib >= nc_live) return;
  // ---- a compute warp ----------------------------------------------------------------
  void* W = a.f.W;
  WarpBox& B = boxes[wib];
  char* slots = slots_all + static_cast<size_t>(wib) * kInbox * s.slot_bytes;
  const bool leader = wib == 0 && a.cta_heavy;  // finishes the block's priority visits
  CtaRegion C = cta_region(region, a.f.kpad, static_cast<int>(sizeof(Store)));
  uint32_t join_phase = 0;
  unsigned in_take = 0, in_done = 0, out_tail = 0;
  // test hook (debug bit 1): the block's last compute warp never joins a block visit,
  // so the others' join runs out of budget
  const bool skip_joins = (a.debug_flags & 2) != 0 && wib == nc_live - 1;
  unsigned long long n_upd = 0, n_hops = 0, n_fail = 0;
  double esum = 0.0;
  unsigned backoff = 32;
  bool failed = false;
  // tk0: processed this iteration, in inbox slot in_done % kInbox; the token taken ahead
  // of it (its first rows prefetched, its indices copied) is processed next iteration
  int tk0 = -1;

  while (true) {
    {
      int stop = 0;
      if (lane == 0) stop = ld_volatile_shared(&hdr->stop);
      if (__shfl_sync(kFull, stop, 0)) break;
    }
    // ---- a priority token at this block: every live compute warp joins the visit -------
    if (a.cta_heavy) {
      int hv = -1;
      if (lane == 0) {
        hv = ld_volatile_shared(&hdr->hv_tok);
        if (hv >= 0) hv = static_cast<int>(ld_acquire_cta_u32(reinterpret_cast<const unsigned*>(&hdr->hv_tok)));
      }
      hv = __shfl_sync(kFull, hv, 0);
      if (hv >= 0 && !skip_joins) {
        cp_async_wait<0>();  // tk0's indices land before the region is reused
        __syncwarp();
        if (!cta_join(join_bar, join_phase, a, lane)) break;
        if (leader && lane == 0) st_release_cta_u32(reinterpret_cast<unsigned*>(&hdr->hv_tok), 0xffffffffu);
        CtaVisitOut vo{0.f, 0};
        cta_visit<Store, NV>(hv, a, s, C, nc_live, wib, lane, vo);
        if (leader) {
          const int4 ma = __ldcg(a.mailbox + 4 * static_cast<int64_t>(hv));
          const int4 mb = __ldcg(a.mailbox + 4 * static_cast<int64_t>(hv) + 1);
          int npos = ma.w + 1, nep = mb.x;
          if (npos == (mb.y & 0x7fffffff)) {
            npos = 0;
            nep = mb.x + 1;
          }
          const bool retire = nep >= a.target_epoch;
          n_upd += static_cast<unsigned long long>(vo.len);
          ++n_hops;
          int ok = 1;
          if (lane == 0) {
            unsigned qr = 1u;
            if (!retire) {
              const int4 nx = __ldg(a.segs + lo_hi(mb.z, mb.w) + npos);
              int4* mbox = a.mailbox + 4 * static_cast<int64_t>(hv);
              __stcg(mbox, make_int4(nx.x, nx.y, nx.z, npos));
              __stcg(mbox + 1, make_int4(nep, mb.y, mb.z, mb.w));
              qr = static_cast<unsigned>(P + nx.w) << 1;
            }
            esum += static_cast<double>(vo.e2);
            // the column (stored by the last warp before the visit's exit barrier) and the
            // mailbox precede the outbox entry
            ok = outbox_put(B, out_tail, hv, qr, hdr, a);
          }
          if (!__shfl_sync(kFull, ok, 0)) break;
        }
      }
    }
    // ---- take the next token ahead of processing tk0: its mailbox and column have
    //      (usually) landed; prefetch its first rows into L1 and copy its indices -------
    int newtok = -1;
    if (lane == 0) {
      const unsigned long long e = ld_acquire_cta_u64(&B.inbox[in_take % kInbox]);
      if (static_cast<unsigned>(e >> 32) == in_take) {
        const uint32_t bar = smem_u32(&B.bars[in_take % kInbox]);
        const uint32_t par = (in_take / kInbox) & 1u;
        uint64_t t0 = 0;
        bool ok = true;
        for (uint32_t it = 0; !mbar_try_wait(bar, par); ++it) {
          if ((it & 63u) == 0) {
            const uint64_t now = nd::globaltimer();
            if (it == 0) {
              t0 = now;
            } else if (static_cast<int64_t>(now - t0) > a.budget_ns) {
              atomicCAS(&a.ctrl[1], 0, nd::kDevErrTimeout);
              ok = false;
              break;
            }
          }
        }
        newtok = ok ? static_cast<int>(e & 0x7fffffffull) : -2;
        if (ok) ++in_take;
      }
    }
    newtok = __shfl_sync(kFull, newtok, 0);
    if (newtok == -2) {
      failed = true;
      break;
    }
    __syncwarp();
    const bool took = newtok >= 0;
    if (took) {
      char* slot = slots + static_cast<size_t>((in_done + (tk0 >= 0 ? 1u : 0u)) % kInbox) * s.slot_bytes;
      const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slot);
      const int len = hd->a.z;
      if (len < s.heavy_min && lane < 5 * min(len, kPF)) {  // 5 lines cover a row of <= 512 bytes
        const int line = lane % 5;
        if (line * 128 < s.row_bytes)
          prefetch_l1(static_cast<const char*>(W) + static_cast<int64_t>(first_rating(hd, lane / 5).x) * s.row_bytes +
                      line * 128);
      }
      stage_r(slot, a, s.heavy_min, lane);
      cp_async_commit();
    }
    // ---- process tk0 ----------------------------------------------------------------
    if (tk0 >= 0) {
      char* slot = slots + static_cast<size_t>(in_done % kInbox) * s.slot_bytes;
      const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slot);
      const int4 ma = hd->a, mb = hd->b;
      const int len = ma.z, pos = ma.w, ep = mb.x;
      const int nseg = mb.y & 0x7fffffff;
      const float step = __ldg(&a.steps[min(ep, a.n_steps - 1)]);
      const uint32_t colkey = nd::hash32(a.seed32 ^ static_cast<uint32_t>(tk0) * 0x85EBCA77u ^
                                         static_cast<uint32_t>(ep) * 0xC2B2AE3Du);
      float h[NV][E];
      const Raw* hs = reinterpret_cast<const Raw*>(slot + sizeof(SlotHdr));
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const int v = lane + 32 * q;
        nd::unpack(v < s.nvec ? hs[v] : nd::zero_raw<Raw>(), h[q]);
      }
      // tk0's copies (indices, next visit) are the older group when a token was just taken
      if (took) cp_async_wait<1>(); else cp_async_wait<0>();
      __syncwarp();
      float e2;
      if (len >= s.heavy_min)
        e2 = visit_long<Store, NV>(hd, lo_hi(ma.x, ma.y), len, h, W, s, R, a.ratings, step, a.lambda, colkey, lane,
                                   a.ctrl, a.budget_ns, failed);
      else
        e2 = visit_short<Store, NV>(hd, len, h, W, s, step, a.lambda, colkey, lane);
      if (failed) break;
      // the column goes back to HBM; the mailbox gets the route's next visit, and a longer
      // visit's indices are prefetched into L2 for its worker.  (Prefetching the next
      // visit's first rows here as well cost more in this tail than it saved: 86 vs 88 ms
      // per epoch on the 480,189 x 17,770 workload, 1.20 vs 1.26 s on 1,000,990 x 624,961.)
      Store* hrow = reinterpret_cast<Store*>(static_cast<char*>(a.f.H) + static_cast<int64_t>(tk0) * s.row_bytes);
      const uint32_t hkey = nd::hash32(colkey ^ static_cast<uint32_t>(pos) * 0x27D4EB2Fu);
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const int v = lane + 32 * q;
        if (v < s.nvec) nd::store_vec<Store, true>(hrow, v, h[q], hkey + 4u * static_cast<uint32_t>(v));
      }
      int npos = pos + 1, nep = ep;
      if (npos == nseg) {
        npos = 0;
        nep = ep + 1;
      }
      const bool retire = nep >= a.target_epoch;
      const int4 nx = hd->nxt[0];
      n_upd += static_cast<unsigned long long>(len);
      ++n_hops;
      if (!retire) {
        if (lane < 4) {
          int4 m;
          if (lane == 0) m = make_int4(nx.x, nx.y, nx.z, npos);
          else if (lane == 1) m = make_int4(nep, mb.y, mb.z, mb.w);
          else m = hd->nxt[lane - 1];
          __stcg(a.mailbox + 4 * static_cast<int64_t>(tk0) + lane, m);
        } else if (lane == 8 && nx.z > kPF) {
          const int64_t st0 = lo_hi(nx.x, nx.y) & ~static_cast<int64_t>(1);  // 16-byte aligned start
          const int64_t end = lo_hi(nx.x, nx.y) + min(nx.z, kChunk);
          prefetch_l2(a.ratings + st0, static_cast<uint32_t>(((end - st0) * 8 + 15) & ~15ll));
        }
      }
      if (lane == 0) esum += static_cast<double>(e2);
      __syncwarp();  // every lane's stores and slot reads precede lane 0's releases
      int ok = 1;
      if (lane == 0) {
        ok = outbox_put(B, out_tail, tk0, retire ? 1u : static_cast<unsigned>(nx.w) << 1, hdr, a);
        st_release_cta_u32(&B.in_head, in_done + 1);  // the slot goes back to the pop warp
      }
      ++in_done;  // warp-uniform: every lane locates slots by it
      if (!__shfl_sync(kFull, ok, 0)) break;
    }
    tk0 = newtok;
    if (tk0 < 0) {
      ++n_fail;
      __nanosleep(backoff);
      backoff = min(backoff * 2, 256u);
    } else {
      backoff = 32;
    }
  }
  cp_async_wait<0>();
  if (failed && NOMAD_STAGE_TMA) {
    for (int sl = 0; sl < kRing; ++sl) {
      const uint32_t bar = R.bars + 8u * sl;
      for (int it = 0; it < 4096 && !mbar_try_wait(bar, (R.phase >> sl) & 1u); ++it) {
      }
    }
  }
  if (failed && lane == 0) st_volatile_shared(&hdr->stop, 1);
  if (lane == 0) {
    atomicAdd(&a.stats[0], n_upd);
    atomicAdd(&a.stats[1], n_hops);
    atomicAdd(&a.stats[2], n_fail);
    atomicAdd(a.err_sum, esum);
  }
}

// Per launch: every active token's mailbox gets its first visit (pass count `ep`) with the
// visit's first ratings, and the token enters its first queue at sequence tails[q] + rank
// (column order in a queue).
__global__ void seed_queues_kernel(nomad::AsyncArgs a, const int4* __restrict__ first_mail,
                                   const int2* __restrict__ first_q, int n, int ep) {
  const int P = a.P;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int2 fq = first_q[j];  // {queue, rank}; queue < 0: the column has no training rating
    if (fq.x < 0) continue;
    int4 m1 = first_mail[2 * j + 1];
    m1.x = ep;
    const int64_t vb = lo_hi(m1.z, m1.w);
    int4* mb = a.mailbox + 4 * static_cast<int64_t>(j);
    mb[0] = first_mail[2 * j];
    mb[1] = m1;
    mb[2] = a.segx[3 * vb + 1];
    mb[3] = a.segx[3 * vb + 2];
    const unsigned seq = a.tails[fq.x] + static_cast<unsigned>(fq.y);
    unsigned long long* rq = fq.x >= P ? a.ring_hi + static_cast<int64_t>(fq.x - P) * (a.mask_hi + 1) + (seq & a.mask_hi)
                                       : a.ring_lo + static_cast<int64_t>(fq.x) * (a.mask_lo + 1) + (seq & a.mask_lo);
    *rq = (static_cast<unsigned long long>(seq) << 32) | static_cast<unsigned>(j);
  }
}
__global__ void advance_tails_kernel(unsigned* tails, const int* __restrict__ counts, int nq) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
    tails[q] += static_cast<unsigned>(counts[q]);
}
// After a failed launch: drop whatever the queues still hold.
__global__ void drain_queues_kernel(unsigned* heads, const unsigned* tails, int nq) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) heads[q] = tails[q];
}
// Extended visit table: each visit {start, len, worker} followed by its first four ratings.
__global__ void build_segx_kernel(const int4* __restrict__ segs, const int2* __restrict__ ratings, int64_t nseg,
                                  int4* __restrict__ segx) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nseg;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int4 sg = segs[i];
    const int64_t start = lo_hi(sg.x, sg.y);
    int2 r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) r[k] = k < sg.z ? ratings[start + k] : make_int2(0, 0);
    segx[3 * i] = sg;
    segx[3 * i + 1] = make_int4(r[0].x, r[0].y, r[1].x, r[1].y);
    segx[3 * i + 2] = make_int4(r[2].x, r[2].y, r[3].x, r[3].y);
  }
}

template <typename Store, int NV>
size_t smem_per_block(int ncw, int kpad, int cta_heavy) {
  const size_t row_bytes = static_cast<size_t>(kpad) * sizeof(Store);
  const size_t slot = sizeof(SlotHdr) + row_bytes;
  size_t region = static_cast<size_t>(ncw) * kRing * kBlk * row_bytes;
  if (cta_heavy) region = std::max(region, cta_region_bytes(kpad, static_cast<int>(sizeof(Store))));
  static_assert(sizeof(SlotHdr) % 16 == 0 && kBarBytes % 16 == 0, "16-byte alignment of the per-warp layout");
  // every term is a multiple of 16 (row_bytes is)
  return kCtaHdrBytes + static_cast<size_t>(ncw) * (sizeof(WarpBox) + kInbox * slot + kBarBytes + 128) + region;
}

template <typename Store, int NV>
cudaError_t launch2_t(const nomad::AsyncArgs& a, cudaStream_t st) {
  const size_t smem = smem_per_block<Store, NV>(a.warps_per_block, a.f.kpad, a.cta_heavy);
  cudaError_t e = cudaFuncSetAttribute(&nomad_async2_kernel<Store, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<nomad::AsyncArgs*>(&a)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<void*>(&nomad_async2_kernel<Store, NV>), dim3(a.grid),
                                     dim3((a.warps_per_block + 2) * 32), args, smem, st);
}

template <typename Store, int NV>
cudaError_t occ2_t(int ncw, int kpad, int cta_heavy, int* bps) {
  if ((ncw + 2) * 32 > Async2Block<Store>::kThreads) {  // more warps than the kernel was compiled for
    *bps = 0;
    return cudaSuccess;
  }
  const size_t smem = smem_per_block<Store, NV>(ncw, kpad, cta_heavy);
  int dev = 0, max_smem = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if (smem > static_cast<size_t>(max_smem)) {  // does not fit: no block per SM
    *bps = 0;
    return cudaSuccess;
  }
  e = cudaFuncSetAttribute(&nomad_async2_kernel<Store, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, &nomad_async2_kernel<Store, NV>, (ncw + 2) * 32, smem);
}

}  // namespace

namespace nomad {

cudaError_t launch_async2(const AsyncArgs& a, cudaStream_t s) {
  const int nv = a.f.nvec <= 32 ? 1 : (a.f.nvec <= 64 ? 2 : 4);
  if (a.f.bf16) {
    switch (nv) {
      case 1: return launch2_t<__nv_bfloat16, 1>(a, s);
      case 2: return launch2_t<__nv_bfloat16, 2>(a, s);
      default: return launch2_t<__nv_bfloat16, 4>(a, s);
    }
  }
  switch (nv) {
    case 1: return launch2_t<float, 1>(a, s);
    case 2: return launch2_t<float, 2>(a, s);
    default: return launch2_t<float, 4>(a, s);
  }
}

cudaError_t async2_occupancy(int bf16, int nv, int ncw, int kpad, int cta_heavy, int* bps) {
  if (bf16) {
    switch (nv) {
      case 1: return occ2_t<__nv_bfloat16, 1>(ncw, kpad, cta_heavy, bps);
      case 2: return occ2_t<__nv_bfloat16, 2>(ncw, kpad, cta_heavy, bps);
      default: return occ2_t<__nv_bfloat16, 4>(ncw, kpad, cta_heavy, bps);
    }
  }
  switch (nv) {
    case 1: return occ2_t<float, 1>(ncw, kpad, cta_heavy, bps);
    case 2: return occ2_t<float, 2>(ncw, kpad, cta_heavy, bps);
    default: return occ2_t<float, 4>(ncw, kpad, cta_heavy, bps);
  }
}

cudaError_t launch_seed_queues(const AsyncArgs& a, const int4* first_mail, const int2* first_q, const int* counts,
                               int n, int ep, cudaStream_t s) {
  const int threads = 256;
  const cudaError_t stale = cudaGetLastError();  // an earlier, unconsumed error would be misattributed
  if (stale != cudaSuccess) return stale;
  if (n > 0) {
    seed_queues_kernel<<<(n + threads - 1) / threads, threads, 0, s>>>(a, first_mail, first_q, n, ep);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  advance_tails_kernel<<<(2 * a.P + threads - 1) / threads, threads, 0, s>>>(a.tails, counts, 2 * a.P);
  return cudaGetLastError();
}

cudaError_t launch_drain_queues(const AsyncArgs& a, cudaStream_t s) {
  drain_queues_kernel<<<(2 * a.P + 255) / 256, 256, 0, s>>>(a.heads, a.tails, 2 * a.P);
  return cudaGetLastError();
}

cudaError_t launch_build_segx(const int4* segs, const int2* ratings, int64_t nseg, int4* segx, cudaStream_t s) {
  if (nseg <= 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((nseg + 255) / 256, 1 << 16);
  build_segx_kernel<<<static_cast<int>(blocks), 256, 0, s>>>(segs, ratings, nseg, segx);
  return cudaGetLastError();
}

}  // namespace nomad
