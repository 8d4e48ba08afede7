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
constexpr unsigned kHeavyBit = 0x80000000u;
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
//   b = {ep, nseg | heavy bit, vb lo, vb hi}  pass count, route length, route start
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
  const size_t ring_bytes = static_cast<size_t>(kRing) * kBlk * s.row_bytes;
  const size_t per_warp = static_cast<size_t>(kStages) * s.slot_bytes + ring_bytes + kBarBytes + 32 * sizeof(float);
  char* base = smem + static_cast<size_t>(wib) * per_warp;
  char* slots = base;
  Ring R;
  R.rows = base + static_cast<size_t>(kStages) * s.slot_bytes;
  R.bars = smem_u32(R.rows + ring_bytes);
  R.gather = reinterpret_cast<float*>(R.rows + ring_bytes + kBarBytes);
  R.phase = 0;
  if (lane == 0 && NOMAD_STAGE_TMA)
    for (int i = 0; i < kRing; ++i) mbar_init(R.bars + 8u * i, 1);
  fence_mbar_init();
  __syncwarp();
  if (w >= P) return;
  if (w == 0 && lane == 0 && a.finish_ns) a.finish_ns[a.f.n] = nd::globaltimer();
  void* W = a.f.W;
  unsigned long long* my_lo = a.ring_lo + static_cast<int64_t>(w) * (a.mask_lo + 1);
  unsigned long long* my_hi = a.ring_hi + static_cast<int64_t>(w) * (a.mask_hi + 1);
  unsigned head_lo = 0, head_hi = 0;  // this worker's consumer counters (lane 0)
  unsigned long long probe_lo = ~0ull, probe_hi = ~0ull;
  if (lane == 0) {
    head_lo = a.heads[w];
    head_hi = a.heads[P + w];
    probe_hi = ld_acquire_u64(my_hi + (head_hi & a.mask_hi));
    probe_lo = ld_acquire_u64(my_lo + (head_lo & a.mask_lo));
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
    // ---- process tk0 ----------------------------------------------------------------
    int push_q = -1;
    unsigned push_seq = 0;
    if (tk0 >= 0) {
      char* slot = slots + static_cast<size_t>(sl0) * s.slot_bytes;
      const SlotHdr* hd = reinterpret_cast<const SlotHdr*>(slot);
      const int4 ma = hd->a, mb = hd->b, nx = hd->nxt;
      const int len = ma.z, pos = ma.w, ep = mb.x;
      const int nseg = mb.y & 0x7fffffff;
      const bool heavy = (static_cast<unsigned>(mb.y) & kHeavyBit) != 0;
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
          push_q = heavy ? P + nx.w : nx.w;
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
      if (entry_valid(probe_hi, head_hi)) {
        newtok = static_cast<int>(probe_hi & 0x7fffffffull);
        ++head_hi;
      } else if (entry_valid(probe_lo, head_lo)) {
        newtok = static_cast<int>(probe_lo & 0x7fffffffull);
        ++head_lo;
      }
    }
    newtok = __shfl_sync(kFull, newtok, 0);
    if (newtok >= 0) stage_d(slots + static_cast<size_t>(slf) * s.slot_bytes, newtok, a, s.row_bytes, lane);
    cp_async_commit();
    if (lane == 0) {
      probe_hi = ld_acquire_u64(my_hi + (head_hi & a.mask_hi));  // for the next iteration
      probe_lo = ld_acquire_u64(my_lo + (head_lo & a.mask_lo));
      if (push_q >= 0) {  // publish the processed token
        unsigned long long* rq =
            push_q >= P ? a.ring_hi + static_cast<int64_t>(push_q - P) * (a.mask_hi + 1) + (push_seq & a.mask_hi)
                        : a.ring_lo + static_cast<int64_t>(push_q) * (a.mask_lo + 1) + (push_seq & a.mask_lo);
        st_relaxed_u64(rq, (static_cast<unsigned long long>(push_seq) << 32) | static_cast<unsigned>(tk0));
      }
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
    a.heads[P + w] = head_hi;
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
size_t smem_per_block(int warps, int kpad) {
  const size_t row_bytes = static_cast<size_t>(kpad) * sizeof(Store);
  const size_t slot = sizeof(SlotHdr) + row_bytes;
  const size_t per_warp = kStages * slot + kRing * kBlk * row_bytes + kBarBytes + 32 * sizeof(float);
  static_assert(sizeof(SlotHdr) % 16 == 0 && kBarBytes % 16 == 0, "16-byte alignment of the per-warp layout");
  return static_cast<size_t>(warps) * per_warp;  // every term is a multiple of 16 (row_bytes is)
}

template <typename Store, int NV>
cudaError_t launch2_t(const nomad::AsyncArgs& a, cudaStream_t st) {
  const size_t smem = smem_per_block<Store, NV>(a.warps_per_block, a.f.kpad);
  cudaError_t e = cudaFuncSetAttribute(&nomad_async2_kernel<Store, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<nomad::AsyncArgs*>(&a)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<void*>(&nomad_async2_kernel<Store, NV>), dim3(a.grid),
                                     dim3(a.warps_per_block * 32), args, smem, st);
}

template <typename Store, int NV>
cudaError_t occ2_t(int warps, int kpad, int* bps) {
  const size_t smem = smem_per_block<Store, NV>(warps, kpad);
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

cudaError_t async2_occupancy(int bf16, int nv, int warps, int kpad, int* bps) {
  if (bf16) {
    switch (nv) {
      case 1: return occ2_t<__nv_bfloat16, 1>(warps, kpad, bps);
      case 2: return occ2_t<__nv_bfloat16, 2>(warps, kpad, bps);
      default: return occ2_t<__nv_bfloat16, 4>(warps, kpad, bps);
    }
  }
  switch (nv) {
    case 1: return occ2_t<float, 1>(warps, kpad, bps);
    case 2: return occ2_t<float, 2>(warps, kpad, bps);
    default: return occ2_t<float, 4>(warps, kpad, bps);
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
