// kernels_async.cu -- the pipelined asynchronous NOMAD kernel for sm_103a.
//
// Same algorithm as Code/nomad/nb_main.cpp:480-572: persistent worker warps own row
// blocks, column tokens move between workers through per-worker queues, each visit runs
// SGD over the (worker rows x column) ratings, and the step size of a visit follows the
// token's pass count.  What makes a hop cheap on this GPU:
//
//  1. Ring queues with sequence-tagged 64-bit entries.  A producer takes a slot with one
//     atomic add and writes (sequence << 32 | token); a consumer owns its head counter and
//     takes a token with one acquire load of the slot it expects.  Heads and tails never
//     reset, so an entry left from an earlier pass can never match.  Each worker has a
//     normal ring and a priority ring for long columns, whose serial chains set the epoch
//     time; the worker drains the priority ring first.
//  2. A per-token mailbox: the producer of a hop writes the next visit's descriptor (rating
//     run, route position, pass count, route) next to the token, so the consumer needs no
//     route lookups of its own.
//  3. A four-stage token pipeline per warp.  A popped token's mailbox and held column are
//     copied into a shared-memory slot by cp.async (stage D), then its rating indices
//     (stage R), then its first rows are loaded (stage W), then it is processed.  Each
//     stage's copies are issued one iteration before they are used.  The release fence of
//     a hop comes right after the visit's stores and before the next copies are issued, so
//     it waits only for those stores.
//  4. Long visits run in blocks of 7 ratings with the chain rewritten exactly: with
//     c = 1 - eta*lambda and b_j = <h_t, w_j> for the block's (distinct, old) rows,
//        e_t = b_t - v_t,   b_j <- c b_j - eta e_t <w_t, w_j>   (j > t),
//     so one reduce-scatter of the 7 <h, w_t> and 21 <w_s, w_t> replaces 7 dependent warp
//     reductions; then w_t' = c w_t - eta e_t h_t and h_{t+1} = c h_t - eta e_t w_t are
//     lane-local.  Rows are staged kRing-1 blocks ahead in shared memory by cp.async (a TMA
//     bulk-copy variant is kept behind NOMAD_STAGE_TMA).
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
constexpr int kStages = 4;   // token pipeline slots (D, R, W, process)
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
// Mailbox (32 bytes, written by the producer of the hop):
//   a = {start lo, start hi, len, pos}        the visit's rating run and route position
//   b = {ep, nseg | priority bit, vb lo, vb hi}  pass count, route length, route start
struct SlotHdr {
  int4 a;
  int4 b;
  int4 nxt;            // the route's next visit {start lo, start hi, len, worker}
  int4 pad;
  int2 rv[kChunk];     // the visit's first rating indices {row, value bits}
};
static_assert(sizeof(SlotHdr) == 64 + 8 * kChunk, "slot header layout");

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

// ---- short visit: one warp reduction per rating, rows kPF ahead in registers ----------
template <typename Store, int NV>
__device__ __forceinline__ float visit_short(const SlotHdr* hd, int len, typename Vec<Store>::Raw (&wb)[kPF][NV],
                                             float (&h)[NV][Vec<Store>::E], void* W, const Shape& s, float step,
                                             float lambda, uint32_t colkey, int lane) {
  constexpr int E = Vec<Store>::E;
  float err2 = 0.f;
  for (int t0 = 0; t0 < len; t0 += kPF) {
#pragma unroll
    for (int i = 0; i < kPF; ++i) {
      const int t = t0 + i;
      if (t < len) {
        const int2 rt = hd->rv[t];
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
        store_row<Store, NV>(W, rt.x, s, lane, w, nd::hash32(static_cast<uint32_t>(rt.x) * 0x9E3779B1u ^ colkey));
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
        store_row<Store, NV>(W, rr[t], s, lane, wn, nd::hash32(static_cast<uint32_t>(rr[t]) * 0x9E3779B1u ^ colkey));
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
//       rows, exact bf16 products for bf16 rows; b = X h -- one warp;
//   e_t = b_t - v_t,  b_j <- c b_j - eta e_t G_jt (j > t) -- one warp, lane j holds b_j;
//   w_t' = c w_t - eta e_t h_t,  h_{t+1} = c h_t - eta e_t w_t -- each warp for its rows,
//       after replaying the h recurrence over the rows before them.
constexpr int kHB = 32;          // ratings per block
constexpr int kHStages = 3;      // row blocks in shared memory (one in use, two in flight)
constexpr int kHRv = 8;          // rating-index blocks in shared memory (ring)
constexpr int kGStride = kHB + 1;
constexpr int kCtaHdrBytes = 16;

struct CtaHdr {
  int hv_tok;                // priority token the block processes next (-1: none)
  int pad;
  unsigned long long join;   // mbarrier, one arrival per live warp
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
  const size_t rows = static_cast<size_t>(kHStages) * kHB * cta_row_words(kpad, esz) * 4;
  const size_t gram = static_cast<size_t>(kHB) * kGStride * 4;
  const size_t h = (static_cast<size_t>(2) * kpad * 4 + 15) / 16 * 16;
  return rows + gram + h + 2 * kHB * 4 + static_cast<size_t>(kHRv) * kHB * 8 + 48 * 4;
}

struct CtaRegion {
  char* rows;   // kHStages x kHB rows of sw words
  float* G;     // kHB x kGStride
  float* h;     // 2 x kpad, the held column (fp32) before and after a block
  float* bsh;   // kHB
  float* nesh;  // kHB: -eta e_t
  int2* rv;     // kHRv x kHB rating indices
  float* cpow;  // kHB + 1: c^k
  int sw;
};

__device__ __forceinline__ CtaRegion cta_region(char* base, int kpad, int esz) {
  CtaRegion C;
  C.sw = cta_row_words(kpad, esz);
  C.rows = base;
  char* p = base + static_cast<size_t>(kHStages) * kHB * C.sw * 4;
  C.G = reinterpret_cast<float*>(p);
  p += static_cast<size_t>(kHB) * kGStride * 4;
  C.h = reinterpret_cast<float*>(p);
  p += (static_cast<size_t>(2) * kpad * 4 + 15) / 16 * 16;
  C.bsh = reinterpret_cast<float*>(p);
  C.nesh = C.bsh + kHB;
  C.rv = reinterpret_cast<int2*>(C.nesh + kHB);
  C.cpow = reinterpret_cast<float*>(C.rv + kHRv * kHB);
  return C;
}

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

// One 16x8 tile of G = X X^T: rows r0.., columns n0.. (fragment layouts of mma.m16n8k8 /
// m16n8k16: g = lane / 4 selects the row, t = lane % 4 the k pair or k element).  G only
// enters the chain multiplied by eta e_t, so TF32 operands (10-bit mantissa) move e_t by
// ~1e-3 * eta |e| |G| per step -- far below fp32 noise in w; b = X h stays in fp32.
__device__ __forceinline__ void gram_tile(const float* X, int sw, int kpad, int r0, int n0, float (&d)[4], int lane) {
  const int g = lane >> 2, t = lane & 3;
  const float* A0 = X + (r0 + g) * sw;
  const float* A1 = A0 + 8 * sw;
  const float* B = X + (n0 + g) * sw;
  float d2[4] = {0.f, 0.f, 0.f, 0.f};  // second accumulator: two independent mma chains
  const int kmma = (kpad + 7) / 8 * 8;  // the row padded with zeros to whole k8 steps
  int k0 = 0;
#pragma unroll 2
  for (; k0 + 16 <= kmma; k0 += 16) {
    const uint32_t a[4] = {tf32_bits(A0[k0 + t]), tf32_bits(A1[k0 + t]), tf32_bits(A0[k0 + t + 4]),
                           tf32_bits(A1[k0 + t + 4])};
    const uint32_t b[2] = {tf32_bits(B[k0 + t]), tf32_bits(B[k0 + t + 4])};
    const uint32_t a2[4] = {tf32_bits(A0[k0 + 8 + t]), tf32_bits(A1[k0 + 8 + t]), tf32_bits(A0[k0 + 12 + t]),
                            tf32_bits(A1[k0 + 12 + t])};
    const uint32_t b2[2] = {tf32_bits(B[k0 + 8 + t]), tf32_bits(B[k0 + 12 + t])};
    mma_tf32(d, a, b);
    mma_tf32(d2, a2, b2);
  }
  if (k0 < kpad) {
    const uint32_t a[4] = {tf32_bits(A0[k0 + t]), tf32_bits(A1[k0 + t]), tf32_bits(A0[k0 + t + 4]),
                           tf32_bits(A1[k0 + t + 4])};
    const uint32_t b[2] = {tf32_bits(B[k0 + t]), tf32_bits(B[k0 + t + 4])};
    mma_tf32(d, a, b);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] += d2[i];
}
__device__ __forceinline__ void gram_tile(const __nv_bfloat16* X, int sw, int kpad, int r0, int n0, float (&d)[4],
                                          int lane) {
  const int g = lane >> 2, t = lane & 3;
  const uint32_t* A0 = reinterpret_cast<const uint32_t*>(X) + (r0 + g) * sw;
  const uint32_t* A1 = A0 + 8 * sw;
  const uint32_t* B = reinterpret_cast<const uint32_t*>(X) + (n0 + g) * sw;
  const int kw = kpad / 2;  // words per row; a multiple of 4
  float d2[4] = {0.f, 0.f, 0.f, 0.f};
  int k = 0;
#pragma unroll 2
  for (; k + 16 <= kw; k += 16) {
    const uint32_t a[4] = {A0[k + t], A1[k + t], A0[k + 4 + t], A1[k + 4 + t]};
    const uint32_t b[2] = {B[k + t], B[k + 4 + t]};
    const uint32_t a2[4] = {A0[k + 8 + t], A1[k + 8 + t], A0[k + 12 + t], A1[k + 12 + t]};
    const uint32_t b2[2] = {B[k + 8 + t], B[k + 12 + t]};
    mma_bf16_k16(d, a, b);
    mma_bf16_k16(d2, a2, b2);
  }
  if (k + 8 <= kw) {
    const uint32_t a[4] = {A0[k + t], A1[k + t], A0[k + 4 + t], A1[k + 4 + t]};
    const uint32_t b[2] = {B[k + t], B[k + 4 + t]};
    mma_bf16_k16(d, a, b);
    k += 8;
  }
  if (k < kw) mma_bf16_k8(d2, A0[k + t], A1[k + t], B[k + t]);
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] += d2[i];
}

// Reduce-scatter of 16 per-lane partials: lane l ends with the warp total of index l % 16.
__device__ __forceinline__ float reduce_scatter16(float (&v)[16], int lane) {
#pragma unroll
  for (int lvl = 0; lvl < 4; ++lvl) {
    const int half = 8 >> lvl;
    const bool up = (lane & half) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = up ? v[i] : v[i + half];
      const float keep = up ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, half);
    }
  }
  return v[0] + __shfl_xor_sync(kFull, v[0], 16);
}

// b_j = <h, x_j> for 16 rows x_j of a block, one warp; lane j ends with b_{j % 16}.
template <typename Store, int NV>
__device__ __forceinline__ float cta_dots16(const char* X, int sw, const float* h, const Shape& s, int lane) {
  using Raw = typename Vec<Store>::Raw;
  float p[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) p[j] = 0.f;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    if (v < s.nvec) {
      const float4 hv = reinterpret_cast<const float4*>(h)[v];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float w[4];
        nd::unpack(reinterpret_cast<const Raw*>(X + static_cast<size_t>(j) * sw * 4)[v], w);
        p[j] = fmaf(hv.x, w[0], p[j]);
        p[j] = fmaf(hv.y, w[1], p[j]);
        p[j] = fmaf(hv.z, w[2], p[j]);
        p[j] = fmaf(hv.w, w[3], p[j]);
      }
    }
  }
  return reduce_scatter16(p, lane);
}

// The serial part of a block: lane j holds b_j; returns this lane's share of the squared
// errors and leaves -eta e_t in nesh[t].
__device__ __forceinline__ float cta_chain(const float* G, const float* bsh, const int2* rvb, float* nesh, int nr,
                                           float step, float c, int lane) {
  float bj = bsh[lane];
  float my_e = 0.f, my_ne = 0.f;
#pragma unroll
  for (int t = 0; t < kHB; ++t) {
    if (t >= nr) break;
    const float g = G[lane * kGStride + t];  // independent of the chain: loaded ahead
    const float bt = __shfl_sync(kFull, bj, t);
    const float e = bt - __int_as_float(rvb[t].y);
    const float ne = -step * e;
    my_e = lane == t ? e : my_e;
    my_ne = lane == t ? ne : my_ne;
    const float upd = fmaf(ne, g, c * bj);
    bj = lane > t ? upd : bj;
  }
  nesh[lane] = my_ne;  // 0 past the block's last rating
  return my_e * my_e;
}

// Rows [t0, t1) of a block (one warp): replay h over the rows before t0, then update
// each row and h.  The last warp also leaves h after the block in h_out, or, after the
// visit's final block, writes it to the column's row `hrow` in HBM.
template <typename Store, int NV>
__device__ __forceinline__ void cta_rows(const char* X, int sw, const int2* rvb, const float* nesh, const float* cpow,
                                         const float* h_in, float* h_out, int nr, int t0, int t1, bool last, float c,
                                         void* W, const Shape& s, uint32_t colkey, Store* hrow, uint32_t hkey,
                                         int lane) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  // h_{t0} = c^{t0} h_0 + sum_{s < t0} c^{t0-1-s} (-eta e_s) w_s, two partial sums
  const int pre = min(t0, nr);
  float h[NV][E], h2[NV][E];
  {
    const float cp = cpow[pre];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int v = lane + 32 * q;
      const float4 x = v < s.nvec ? reinterpret_cast<const float4*>(h_in)[v] : make_float4(0.f, 0.f, 0.f, 0.f);
      h[q][0] = cp * x.x; h[q][1] = cp * x.y; h[q][2] = cp * x.z; h[q][3] = cp * x.w;
#pragma unroll
      for (int e = 0; e < E; ++e) h2[q][e] = 0.f;
    }
  }
#pragma unroll 4
  for (int t = 0; t < pre; ++t) {
    const float coef = cpow[pre - 1 - t] * nesh[t];
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
#pragma unroll
  for (int q = 0; q < NV; ++q)
#pragma unroll
    for (int e = 0; e < E; ++e) h[q][e] += h2[q][e];
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
    store_row<Store, NV>(W, r, s, lane, wn, nd::hash32(static_cast<uint32_t>(r) * 0x9E3779B1u ^ colkey));
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

// Join of the block's live warps before a block visit; false (and the timeout status)
// when some warp did not arrive within the budget.
__device__ __forceinline__ bool cta_join(uint32_t bar, uint32_t& phase, const nomad::AsyncArgs& a, int lane) {
  int ok = 1;
  if (lane == 0) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
    uint64_t t0 = 0;
    for (uint32_t it = 0;; ++it) {
      if (mbar_try_wait(bar, phase)) break;
      if ((it & 63u) == 0) {
        const uint64_t now = nd::globaltimer();
        if (it == 0) {
          t0 = now;
        } else if (static_cast<int64_t>(now - t0) > a.budget_ns) {
          atomicCAS(&a.ctrl[1], 0, nd::kDevErrTimeout);
          ok = 0;
          break;
        }
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

// Rows of block b of the visit into its shared-memory slot (each warp some rows).
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

// One visit of priority token `tok` by the block's nw live warps (all of them call it).
// The last warp writes the column back; warp 0 returns the squared errors.  The shared
// region is free again when this returns (the warps' long-visit rings alias it).
template <typename Store, int NV>
__device__ __forceinline__ void cta_visit(int tok, const nomad::AsyncArgs& a, const Shape& s, const CtaRegion& C, int nw, int wib,
                          int lane, CtaVisitOut& out) {
  const int tid = wib * 32 + lane;
  const int nthr = nw * 32;
  const int kpad = s.row_bytes / static_cast<int>(sizeof(Store));
  const int4 ma = __ldcg(a.mailbox + 2 * static_cast<int64_t>(tok));
  const int4 mb = __ldcg(a.mailbox + 2 * static_cast<int64_t>(tok) + 1);
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
  // zero the columns past an fp32 row that the last k8 tile reads
  if (sizeof(Store) == 4 && (kpad & 7) != 0)
    for (int r = tid; r < kHStages * kHB; r += nthr)
      *reinterpret_cast<float4*>(C.rows + static_cast<size_t>(r) * C.sw * 4 + kpad * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid == 0) {  // c^k
    float x = 1.f;
    for (int i = 0; i <= kHB; ++i) {
      C.cpow[i] = x;
      x *= c;
    }
  }
  cp_async_wait<0>();
  bar_sync_named(nthr);
  cta_stage_rows(C, 0, len, W, s.row_bytes, nw, wib, lane);
  cp_async_commit();
  if (nblk > 1) cta_stage_rows(C, 1, len, W, s.row_bytes, nw, wib, lane);
  cp_async_commit();
  float e2 = 0.f;
  const int rpg = (kHB + nw - 1) / nw;
  for (int i = 0; i < nblk; ++i) {
    cp_async_wait<1>();  // rows of block i and indices of block i + 2 have landed
    bar_sync_named(nthr);
    const float* hcur = C.h + (i & 1) * kpad;
    float* hnext = C.h + ((i + 1) & 1) * kpad;
    if (i + 2 < nblk) cta_stage_rows(C, i + 2, len, W, s.row_bytes, nw, wib, lane);
    if (i + 4 < nblk) cta_stage_rv(C, i + 4, start, len, a.ratings, tid, nthr);
    cp_async_commit();
    const char* X = C.rows + static_cast<size_t>(i % kHStages) * kHB * C.sw * 4;
    const int2* rvb = C.rv + (i % kHRv) * kHB;
    const int nr = min(kHB, len - i * kHB);
    // Gram tiles (lower triangle of 16x8 tiles) and the dots with h (two halves)
    for (int it = wib; it < 8; it += nw) {
      if (it < 6) {
        const int r0 = it < 2 ? 0 : 16;
        const int n0 = it < 2 ? 8 * it : 8 * (it - 2);
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        gram_tile(reinterpret_cast<const Store*>(X), C.sw, kpad, r0, n0, d, lane);
        const int g = lane >> 2, t = lane & 3;
        C.G[(r0 + g) * kGStride + n0 + 2 * t] = d[0];
        C.G[(r0 + g) * kGStride + n0 + 2 * t + 1] = d[1];
        C.G[(r0 + g + 8) * kGStride + n0 + 2 * t] = d[2];
        C.G[(r0 + g + 8) * kGStride + n0 + 2 * t + 1] = d[3];
      } else {
        const int r0 = 16 * (it - 6);
        const float bv = cta_dots16<Store, NV>(X + static_cast<size_t>(r0) * C.sw * 4, C.sw, hcur, s, lane);
        if (lane < 16) C.bsh[r0 + lane] = bv;
      }
    }
    bar_sync_named(nthr);
    if (wib == 0) e2 += cta_chain(C.G, C.bsh, rvb, C.nesh, nr, step, c, lane);
    bar_sync_named(nthr);
    cta_rows<Store, NV>(X, C.sw, rvb, C.nesh, C.cpow, hcur, hnext, nr, wib * rpg, (wib + 1) * rpg, wib == nw - 1, c,
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
// D: the mailbox and the held column, into the token's slot.
__device__ __forceinline__ void stage_d(char* slot, int tok, const nomad::AsyncArgs& a, int row_bytes, int lane) {
  const uint32_t d = smem_u32(slot);
  if (lane < 2) cp16(d + 16 * lane, reinterpret_cast<const char*>(a.mailbox + 2 * static_cast<int64_t>(tok) + lane));
  const char* hrow = static_cast<const char*>(a.f.H) + static_cast<int64_t>(tok) * row_bytes;
  const uint32_t hd = d + static_cast<uint32_t>(sizeof(SlotHdr));
  for (int v = lane; v * 16 < row_bytes; v += 32) cp16(hd + 16 * v, hrow + 16 * v);
}
// R: needs the mailbox -- the visit's rating indices and the route's next visit.
__device__ __forceinline__ void stage_r(char* slot, const nomad::AsyncArgs& a, int lane) {
  const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slot);
  const int4 ma = hd->a, mb = hd->b;
  const int64_t start = lo_hi(ma.x, ma.y);
  const uint32_t d = smem_u32(slot);
  if (lane < min(ma.z, kChunk)) cp8(d + static_cast<uint32_t>(offsetof(SlotHdr, rv)) + 8 * lane, a.ratings + start + lane);
  if (lane == 0) {
    const int nseg = mb.y & 0x7fffffff;
    const int npos = ma.w + 1 < nseg ? ma.w + 1 : 0;
    cp16(d + static_cast<uint32_t>(offsetof(SlotHdr, nxt)), a.segs + lo_hi(mb.z, mb.w) + npos);
  }
}

__device__ __forceinline__ bool entry_valid(unsigned long long e, unsigned head) {
  return static_cast<unsigned>(e >> 32) == head && (e & 0x80000000ull) == 0;
}

template <typename Store, int NV>
__global__ void __launch_bounds__(256, 2) nomad_async2_kernel(nomad::AsyncArgs a) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  extern __shared__ __align__(128) char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int w = blockIdx.x * (blockDim.x >> 5) + wib;
  const int P = a.P;
  Shape s;
  s.nvec = a.f.nvec;
  s.red_width = a.f.red_width;
  s.row_bytes = a.f.kpad * static_cast<int>(sizeof(Store));
  s.heavy_min = min(max(a.heavy_min, 1), kChunk + 1);  // longer visits always take the blocked path
  s.slot_bytes = static_cast<int>(sizeof(SlotHdr)) + s.row_bytes;
  // shared memory: block header | every warp's token slots | long-visit rings (the block
  // visit region aliases them) | mbarriers | gather buffers
  const int nwarps = blockDim.x >> 5;
  const int nw_live = min(nwarps, P - static_cast<int>(blockIdx.x) * nwarps);
  const size_t ring_bytes = static_cast<size_t>(kRing) * kBlk * s.row_bytes;
  size_t region_bytes = static_cast<size_t>(nwarps) * ring_bytes;
  if (a.cta_heavy) region_bytes = max(region_bytes, cta_region_bytes(a.f.kpad, static_cast<int>(sizeof(Store))));
  CtaHdr* hdr = reinterpret_cast<CtaHdr*>(smem);
  char* region = smem + kCtaHdrBytes + static_cast<size_t>(nwarps) * kStages * s.slot_bytes;
  char* bars = region + region_bytes;
  char* slots = smem + kCtaHdrBytes + static_cast<size_t>(wib) * kStages * s.slot_bytes;
  Ring R;
  R.rows = region + static_cast<size_t>(wib) * ring_bytes;
  R.bars = smem_u32(bars + static_cast<size_t>(wib) * kBarBytes);
  R.gather = reinterpret_cast<float*>(bars + static_cast<size_t>(nwarps) * kBarBytes + static_cast<size_t>(wib) * 128);
  R.phase = 0;
  if (lane == 0 && NOMAD_STAGE_TMA)
    for (int i = 0; i < kRing; ++i) mbar_init(R.bars + 8u * i, 1);
  const uint32_t join_bar = smem_u32(&hdr->join);
  if (threadIdx.x == 0) {
    hdr->hv_tok = -1;
    if (nw_live > 0) mbar_init(join_bar, static_cast<uint32_t>(nw_live));
  }
  fence_mbar_init();
  __syncthreads();
  if (w >= P) return;
  if (w == 0 && lane == 0 && a.finish_ns) a.finish_ns[a.f.n] = nd::globaltimer();
  void* W = a.f.W;
  const bool leader = wib == 0 && a.cta_heavy;  // polls the block's ring of priority tokens
  CtaRegion C = cta_region(region, a.f.kpad, static_cast<int>(sizeof(Store)));
  uint32_t join_phase = 0;
  bool hv_held = false;
  unsigned long long* my_lo = a.ring_lo + static_cast<int64_t>(w) * (a.mask_lo + 1);
  unsigned long long* my_hi = a.ring_hi + static_cast<int64_t>(blockIdx.x) * (a.mask_hi + 1);
  unsigned head_lo = 0, head_hi = 0;  // consumer counters (lane 0)
  unsigned long long probe_lo = ~0ull, probe_hi = ~0ull;
  if (lane == 0) {
    head_lo = a.heads[w];
    probe_lo = ld_acquire_u64(my_lo + (head_lo & a.mask_lo));
    if (leader) {
      head_hi = a.heads[P + blockIdx.x];
      probe_hi = ld_acquire_u64(my_hi + (head_hi & a.mask_hi));
    }
  }
  unsigned long long n_upd = 0, n_hops = 0, n_fail = 0, pending = 0, seen = ~0ull;
  uint64_t idle_since = 0;
  double esum = 0.0;
  unsigned backoff = 32;
  bool failed = false;
  // tk0: processed this iteration (rows in wb), tk1: its W stage is due, tk2: its R stage
  // is due.  sl*: their slots; slf: the free slot the next popped token takes.
  int tk0 = -1, tk1 = -1, tk2 = -1;
  int sl0 = 0, sl1 = 1, sl2 = 2, slf = 3;
  Raw wb[kPF][NV];
#pragma unroll
  for (int i = 0; i < kPF; ++i)
#pragma unroll
    for (int q = 0; q < NV; ++q) wb[i][q] = nd::zero_raw<Raw>();

  while (true) {
    cp_async_wait<0>();  // the previous iteration's copies ...
    __syncwarp();        // ... visible to every lane
    // ---- a priority token at this block: every live warp joins the visit -------------
    if (a.cta_heavy) {
      int hv = -1;
      if (lane == 0) hv = ld_volatile_shared(&hdr->hv_tok);
      hv = __shfl_sync(kFull, hv, 0);
      if (hv >= 0) {
        if (!cta_join(join_bar, join_phase, a, lane)) break;
        if (leader && lane == 0) st_volatile_shared(&hdr->hv_tok, -1);  // every warp has read it
        CtaVisitOut vo{0.f, 0};
        cta_visit<Store, NV>(hv, a, s, C, nw_live, wib, lane, vo);
        if (leader) {
          hv_held = false;
          const int4 ma = __ldcg(a.mailbox + 2 * static_cast<int64_t>(hv));
          const int4 mb = __ldcg(a.mailbox + 2 * static_cast<int64_t>(hv) + 1);
          int npos = ma.w + 1, nep = mb.x;
          if (npos == (mb.y & 0x7fffffff)) {
            npos = 0;
            nep = mb.x + 1;
          }
          const bool retire = nep >= a.target_epoch;
          n_upd += static_cast<unsigned long long>(vo.len);
          ++n_hops;
          if (lane == 0) {
            int4 nx = make_int4(0, 0, 0, 0);
            if (!retire) {
              nx = __ldg(a.segs + lo_hi(mb.z, mb.w) + npos);
              int4* mbox = a.mailbox + 2 * static_cast<int64_t>(hv);
              __stcg(mbox, make_int4(nx.x, nx.y, nx.z, npos));
              __stcg(mbox + 1, make_int4(nep, mb.y, mb.z, mb.w));
            }
            esum += static_cast<double>(vo.e2);
            ++pending;
            fence_acq_rel_gpu();  // the column (stored by the last warp before the exit barrier) and mailbox
            if (retire) {
              if (a.finish_ns) a.finish_ns[hv] = nd::globaltimer();
              atomicAdd(&a.ctrl[0], 1);
            } else {
              const int q = P + nx.w;
              const unsigned seq = atomicAdd(&a.tails[q], 1u);
              st_relaxed_u64(a.ring_hi + static_cast<int64_t>(nx.w) * (a.mask_hi + 1) + (seq & a.mask_hi),
                             (static_cast<unsigned long long>(seq) << 32) | static_cast<unsigned>(hv));
            }
          }
          __syncwarp();
        }
        // the visit may have changed rows that tk0's prefetched registers hold
        if (tk0 >= 0) {
          const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slots + static_cast<size_t>(sl0) * s.slot_bytes);
          const int len = hd->a.z;
          if (len < s.heavy_min) {
#pragma unroll
            for (int i = 0; i < kPF; ++i)
              if (i < len) load_row_regs<Store, NV>(W, hd->rv[i].x, s, lane, wb[i]);
          }
        }
      }
    }
    // ---- process tk0 ----------------------------------------------------------------
    int push_q = -1;
    unsigned push_seq = 0;
    if (tk0 >= 0) {
      char* slot = slots + static_cast<size_t>(sl0) * s.slot_bytes;
      const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slot);
      const int4 ma = hd->a, mb = hd->b, nx = hd->nxt;
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
      float e2;
      if (len >= s.heavy_min)
        e2 = visit_long<Store, NV>(hd, lo_hi(ma.x, ma.y), len, h, W, s, R, a.ratings, step, a.lambda, colkey, lane,
                                   a.ctrl, a.budget_ns, failed);
      else
        e2 = visit_short<Store, NV>(hd, len, wb, h, W, s, step, a.lambda, colkey, lane);
      if (failed) break;
      // the column goes back to HBM; the mailbox gets the route's next visit
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
      n_upd += static_cast<unsigned long long>(len);
      ++n_hops;
      if (lane == 0) {
        if (!retire) {
          int4* mbox = a.mailbox + 2 * static_cast<int64_t>(tk0);
          __stcg(mbox, make_int4(nx.x, nx.y, nx.z, npos));
          __stcg(mbox + 1, make_int4(nep, mb.y, mb.z, mb.w));
        }
        esum += static_cast<double>(e2);
        ++pending;
      }
      __syncwarp();  // every lane's stores precede lane 0's release fence
      if (lane == 0) {
        fence_acq_rel_gpu();
        if (retire) {
          if (a.finish_ns) a.finish_ns[tk0] = nd::globaltimer();
          atomicAdd(&a.ctrl[0], 1);
        } else {
          push_q = nx.w;
          push_seq = atomicAdd(&a.tails[push_q], 1u);  // the entry store follows the copies below
        }
        if (pending >= 64) {
          atomicAdd(a.progress, pending);
          pending = 0;
        }
      }
    }
    // ---- W stage for tk1: its first rows (after this visit's row stores) ---------------
    if (tk1 >= 0) {
      const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slots + static_cast<size_t>(sl1) * s.slot_bytes);
      const int len = hd->a.z;
      if (len < s.heavy_min) {
#pragma unroll
        for (int i = 0; i < kPF; ++i)
          if (i < len) load_row_regs<Store, NV>(W, hd->rv[i].x, s, lane, wb[i]);
      }
    }
    // ---- R stage for tk2 ---------------------------------------------------------------
    if (tk2 >= 0) stage_r(slots + static_cast<size_t>(sl2) * s.slot_bytes, a, lane);
    // ---- D stage for a newly taken token (priority ring first) ---------------------------
    int newtok = -1;
    if (lane == 0) {
      if (leader && !hv_held && entry_valid(probe_hi, head_hi)) {  // every warp sees it next iteration
        st_volatile_shared(&hdr->hv_tok, static_cast<int>(probe_hi & 0x7fffffffull));
        hv_held = true;
        ++head_hi;
      }
      if (entry_valid(probe_lo, head_lo)) {
        newtok = static_cast<int>(probe_lo & 0x7fffffffull);
        ++head_lo;
      }
    }
    newtok = __shfl_sync(kFull, newtok, 0);
    if (newtok >= 0) stage_d(slots + static_cast<size_t>(slf) * s.slot_bytes, newtok, a, s.row_bytes, lane);
    cp_async_commit();
    if (lane == 0) {
      if (leader) probe_hi = ld_acquire_u64(my_hi + (head_hi & a.mask_hi));  // for the next iteration
      probe_lo = ld_acquire_u64(my_lo + (head_lo & a.mask_lo));
      if (push_q >= 0)  // publish the processed token
        st_relaxed_u64(a.ring_lo + static_cast<int64_t>(push_q) * (a.mask_lo + 1) + (push_seq & a.mask_lo),
                       (static_cast<unsigned long long>(push_seq) << 32) | static_cast<unsigned>(tk0));
    }
    // ---- shift the pipeline; the processed token's slot becomes the free one -----------
    const int freed = sl0;
    tk0 = tk1;
    sl0 = sl1;
    tk1 = tk2;
    sl1 = sl2;
    tk2 = newtok;
    sl2 = slf;
    slf = freed;
    if (tk0 < 0 && tk1 < 0 && tk2 < 0) {
      // nothing in the pipeline: idle poll
      int stop = 0;
      if (lane == 0 && (++n_fail & 7) == 1) {
        if (pending) {
          atomicAdd(a.progress, pending);
          pending = 0;
        }
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
      }
      if (__shfl_sync(kFull, stop, 0)) break;
      __nanosleep(backoff);
      backoff = min(backoff * 2, 256u);
    } else {
      backoff = 32;
      if ((n_hops & 15) == 0) {
        int stop = 0;
        if (lane == 0) stop = nd::ld_acquire(&a.ctrl[1]) != 0;
        if (__shfl_sync(kFull, stop, 0)) break;
      }
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
  if (lane == 0) {
    a.heads[w] = head_lo;
    if (leader) a.heads[P + blockIdx.x] = head_hi;
    if (pending) atomicAdd(a.progress, pending);
    atomicAdd(&a.stats[0], n_upd);
    atomicAdd(&a.stats[1], n_hops);
    atomicAdd(&a.stats[2], n_fail);
    atomicAdd(a.err_sum, esum);
  }
}

// Per launch: every active token's mailbox gets its first visit (pass count `ep`), and
// the token enters its first queue at sequence tails[q] + rank (column order in a queue).
__global__ void seed_queues_kernel(nomad::AsyncArgs a, const int4* __restrict__ first_mail,
                                   const int2* __restrict__ first_q, int n, int ep) {
  const int P = a.P;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int2 fq = first_q[j];  // {queue, rank}; queue < 0: the column has no training rating
    if (fq.x < 0) continue;
    int4 m1 = first_mail[2 * j + 1];
    m1.x = ep;
    a.mailbox[2 * static_cast<int64_t>(j)] = first_mail[2 * j];
    a.mailbox[2 * static_cast<int64_t>(j) + 1] = m1;
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

template <typename Store, int NV>
size_t smem_per_block(int warps, int kpad, int cta_heavy) {
  const size_t row_bytes = static_cast<size_t>(kpad) * sizeof(Store);
  const size_t slot = sizeof(SlotHdr) + row_bytes;
  size_t region = static_cast<size_t>(warps) * kRing * kBlk * row_bytes;
  if (cta_heavy) region = std::max(region, cta_region_bytes(kpad, static_cast<int>(sizeof(Store))));
  static_assert(sizeof(SlotHdr) % 16 == 0 && kBarBytes % 16 == 0, "16-byte alignment of the per-warp layout");
  // every term is a multiple of 16 (row_bytes is)
  return kCtaHdrBytes + static_cast<size_t>(warps) * (kStages * slot + kBarBytes + 128) + region;
}

template <typename Store, int NV>
cudaError_t launch2_t(const nomad::AsyncArgs& a, cudaStream_t st) {
  const size_t smem = smem_per_block<Store, NV>(a.warps_per_block, a.f.kpad, a.cta_heavy);
  cudaError_t e = cudaFuncSetAttribute(&nomad_async2_kernel<Store, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<nomad::AsyncArgs*>(&a)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<void*>(&nomad_async2_kernel<Store, NV>), dim3(a.grid),
                                     dim3(a.warps_per_block * 32), args, smem, st);
}

template <typename Store, int NV>
cudaError_t occ2_t(int warps, int kpad, int cta_heavy, int* bps) {
  const size_t smem = smem_per_block<Store, NV>(warps, kpad, cta_heavy);
  cudaError_t e = cudaFuncSetAttribute(&nomad_async2_kernel<Store, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, &nomad_async2_kernel<Store, NV>, warps * 32, smem);
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

cudaError_t async2_occupancy(int bf16, int nv, int warps, int kpad, int cta_heavy, int* bps) {
  if (bf16) {
    switch (nv) {
      case 1: return occ2_t<__nv_bfloat16, 1>(warps, kpad, cta_heavy, bps);
      case 2: return occ2_t<__nv_bfloat16, 2>(warps, kpad, cta_heavy, bps);
      default: return occ2_t<__nv_bfloat16, 4>(warps, kpad, cta_heavy, bps);
    }
  }
  switch (nv) {
    case 1: return occ2_t<float, 1>(warps, kpad, cta_heavy, bps);
    case 2: return occ2_t<float, 2>(warps, kpad, cta_heavy, bps);
    default: return occ2_t<float, 4>(warps, kpad, cta_heavy, bps);
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

}  // namespace nomad
