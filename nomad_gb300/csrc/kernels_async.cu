// kernels_async.cu -- the pipelined asynchronous NOMAD kernel for sm_103a.
//
// Same algorithm as Code/nomad/nb_main.cpp:480-572: persistent worker warps own row
// blocks, column tokens move between workers through per-worker lock-free queues,
// each visit runs SGD over the (worker rows x column) ratings, the step size of a
// visit follows the token's pass count.  Three things make a hop cheap:
//
//  1. Cross-token pipelining.  A worker pops its next token B before it works on the
//     current token A, and B's visit descriptor, held column h_B, rating indices and
//     first factor rows are in flight while A computes.  The producer of a hop writes
//     the descriptor of the token's next visit into a per-token mailbox, so a
//     consumer needs one round trip after the pop, not three.  B's factor rows are
//     requested only after A's row stores are issued: the same lane stores and later
//     loads each 16-byte piece of a row, so program order makes A's updates visible.
//  2. Two queues per worker.  Tokens of long columns (whose serial update chain sets
//     the epoch time) use a priority queue that the worker drains first.
//  3. Long visits run in blocks of 7 ratings with the chain rewritten exactly:
//     with c = 1 - eta*lambda, h_{t+1} = c h_t - eta e_t w_t, so for the block's rows
//     w_0..w_6 (distinct rows, old values) and b_j = <h_t, w_j>:
//        e_t = b_t - v_t,   b_j <- c b_j - eta e_t <w_t, w_j>   (j > t)
//     One batched reduction of the 7 <h, w_t> and 21 <w_s, w_t> products replaces 7
//     dependent warp reductions; the 7 errors then follow from a scalar recurrence and
//     the row / column updates w_t' = c w_t - eta e_t h_t, h_{t+1} = c h_t - eta e_t w_t
//     are lane-local.  The rows of the next blocks are staged into shared memory by
//     TMA bulk copies (cp.async.bulk, mbarrier completion, bounded waits).
#include <cuda_bf16.h>

#include "device_common.cuh"
#include "launch.h"

namespace {

using nd::kFull;
using nd::Vec;

constexpr int kPF = 4;       // rows prefetched in registers on the short-visit path
constexpr int kBlk = 7;      // ratings per block on the long-visit path
constexpr int kChunk = 28;   // ratings indexed per register chunk (4 blocks)
constexpr int kRing = 4;     // staged blocks per warp (current + 3 ahead)
constexpr unsigned kHeavyBit = 0x80000000u;

// ---- small PTX helpers -----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
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
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Per-lane asynchronous global -> shared copies (cp.async, completion by commit groups).
template <int BYTES>
__device__ __forceinline__ void cp_async(uint32_t dst, const void* src) {
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

#ifndef NOMAD_STAGE_TMA
#define NOMAD_STAGE_TMA 0
#endif

// ---- one token context (the state a hop carries) ---------------------------------
template <typename Store, int NV>
struct Tok {
  using Raw = typename Vec<Store>::Raw;
  int tok;       // -1: none
  int4 desc;     // {start lo, start hi, len, pos | heavy bit}
  int ep;        // pass count
  int64_t vb;    // visit list start
  int nseg;      // visit list length
  Raw h[NV];     // held column, packed
  int2 rv;       // lane t < min(len, 28): rating t of the visit
  Raw w[kPF][NV];  // first rows of a short visit, packed
  int4 nseg4;    // the visit that follows this one (routing)
};

struct Shape {
  int kpad, nvec, red_width, dim, row_bytes, heavy_min;
};

__device__ __forceinline__ int64_t desc_start(const int4& d) {
  return static_cast<int64_t>(static_cast<uint32_t>(d.x)) | (static_cast<int64_t>(d.y) << 32);
}

// stage 1: after the pop -- descriptor, pass count, route bounds, held column
template <typename Store, int NV>
__device__ __forceinline__ void stage1(Tok<Store, NV>& T, const nomad::AsyncArgs& a, const Shape& s, int lane) {
  using Raw = typename Vec<Store>::Raw;
  T.desc = __ldcg(&a.tok_desc[T.tok]);
  T.ep = __ldcg(&a.tok_epoch[T.tok]);
  T.vb = __ldg(&a.vl_ptr[T.tok]);
  T.nseg = static_cast<int>(__ldg(&a.vl_ptr[T.tok + 1]) - T.vb);
  const Raw* hr = reinterpret_cast<const Raw*>(static_cast<const char*>(a.f.H) +
                                               static_cast<int64_t>(T.tok) * s.row_bytes);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    T.h[q] = v < s.nvec ? __ldcg(hr + v) : nd::zero_raw<Raw>();
  }
}
// stage 2: needs the descriptor -- rating indices and the next visit of the route
template <typename Store, int NV>
__device__ __forceinline__ void stage2(Tok<Store, NV>& T, const nomad::AsyncArgs& a, int lane) {
  const int len = T.desc.z;
  const int64_t start = desc_start(T.desc);
  T.rv = lane < min(len, kChunk) ? __ldg(&a.ratings[start + lane]) : make_int2(0, 0);
  const int pos = T.desc.w & 0x7fffffff;
  const int npos = pos + 1 < T.nseg ? pos + 1 : 0;
  T.nseg4 = __ldg(&a.segs[T.vb + npos]);
}
// stage 3: needs the rating indices -- first rows of a short visit
template <typename Store, int NV>
__device__ __forceinline__ void stage3(Tok<Store, NV>& T, const void* W, const Shape& s, int lane) {
  using Raw = typename Vec<Store>::Raw;
  const int len = T.desc.z;
  if (len >= s.heavy_min) return;
#pragma unroll
  for (int i = 0; i < kPF; ++i) {
    const int r = __shfl_sync(kFull, T.rv.x, i);
    if (i < len) {
      const Raw* row = reinterpret_cast<const Raw*>(static_cast<const char*>(W) +
                                                    static_cast<int64_t>(r) * s.row_bytes);
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const int v = lane + 32 * q;
        T.w[i][q] = v < s.nvec ? row[v] : nd::zero_raw<Raw>();
      }
    }
  }
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

// ---- short visit: one warp reduction per rating, rows PF ahead in registers --------
template <typename Store, int NV>
__device__ __forceinline__ float visit_short(Tok<Store, NV>& T, float (&h)[NV][Vec<Store>::E], void* W,
                                             const Shape& s, float step, float lambda,
                                             uint32_t colkey, int lane) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  const int len = T.desc.z;
  float err2 = 0.f;
  for (int t0 = 0; t0 < len; t0 += kPF) {
#pragma unroll
    for (int i = 0; i < kPF; ++i) {
      const int t = t0 + i;
      if (t < len) {
        const int r = __shfl_sync(kFull, T.rv.x, t);
        const float v = __int_as_float(__shfl_sync(kFull, T.rv.y, t));
        float w[NV][E];
#pragma unroll
        for (int q = 0; q < NV; ++q) nd::unpack(T.w[i][q], w[q]);
        float part = 0.f;
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
          for (int e = 0; e < E; ++e) part = fmaf(h[q][e], w[q][e], part);
        const float err = nd::warp_allreduce(part, s.red_width) - v;
        err2 += err * err;
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const float wo = w[q][e], ho = h[q][e];
            w[q][e] = fmaf(-step, fmaf(err, ho, lambda * wo), wo);
            h[q][e] = fmaf(-step, fmaf(err, wo, lambda * ho), ho);
          }
        store_row<Store, NV>(W, r, s, lane, w, nd::hash32(static_cast<uint32_t>(r) * 0x9E3779B1u ^ colkey));
        const int tn = t + kPF;
        const int rn = __shfl_sync(kFull, T.rv.x, tn & 31);
        if (tn < len) {
          const Raw* row = reinterpret_cast<const Raw*>(static_cast<const char*>(W) +
                                                        static_cast<int64_t>(rn) * s.row_bytes);
#pragma unroll
          for (int q = 0; q < NV; ++q) {
            const int v2 = lane + 32 * q;
            T.w[i][q] = v2 < s.nvec ? row[v2] : nd::zero_raw<Raw>();
          }
        }
      }
    }
  }
  return err2;
}

// ---- long visit: blocks of 7 ratings, rows staged by TMA ------------------------------
struct Ring {
  char* rows;         // kRing slots x kBlk rows x row_bytes
  uint32_t bars;      // shared address of kRing mbarriers (8 bytes each)
  float* gather;      // 32 floats
  uint32_t phase;     // parity bit per slot
};

// Issue the copies of block `b` of the visit (rows from the chunk registers).
// VB = bytes per lane vector (16 fp32, 8 bf16).
template <int VB>
__device__ __forceinline__ void issue_block(const Ring& R, int b, int len, int chunk_base,
                                            int2 rv_cur, int2 rv_nxt, const void* W, int row_bytes,
                                            int lane) {
  const int first = b * kBlk;
  const int nr = min(kBlk, len - first);
  const int slot = b % kRing;
  // the rows of this block live in the current or the next rating chunk
  int r = 0;
  if (lane < nr) {
    const int idx = first + lane - chunk_base;  // 0..55
    r = idx;
  }
  const int src_cur = min(max(r, 0), 31);
  const int src_nxt = min(max(r - kChunk, 0), 31);
  const int a_row = __shfl_sync(kFull, rv_cur.x, src_cur);
  const int b_row = __shfl_sync(kFull, rv_nxt.x, src_nxt);
  const int row = r < kChunk ? a_row : b_row;
#if NOMAD_STAGE_TMA
  if (lane == 0) {
    fence_proxy_async_shared();  // earlier generic reads of this slot precede the copy
    mbar_expect_tx(R.bars + 8u * slot, static_cast<uint32_t>(nr * row_bytes));
  }
  __syncwarp();
  if (lane < nr) {
    const uint32_t dst = smem_u32(R.rows + (static_cast<size_t>(slot) * kBlk + lane) * row_bytes);
    tma_row(dst, static_cast<const char*>(W) + static_cast<int64_t>(row) * row_bytes,
            static_cast<uint32_t>(row_bytes), R.bars + 8u * slot);
  }
#else
  // every lane stages (and later reads) only its own slice of each row, so the data
  // needs no cross-lane synchronisation: the lane's own wait_group makes it visible
  for (int t = 0; t < kBlk; ++t) {
    const int rt = __shfl_sync(kFull, row, t);
    if (t < nr) {
      const char* src = static_cast<const char*>(W) + static_cast<int64_t>(rt) * row_bytes;
      const uint32_t dst = smem_u32(R.rows + (static_cast<size_t>(slot) * kBlk + t) * row_bytes);
      for (int v = lane; v * VB < row_bytes; v += 32) cp_async<VB>(dst + v * VB, src + v * VB);
    }
  }
#endif
}

// Bounded wait for a staged block; false = gave up (status already recorded).
__device__ __forceinline__ bool wait_block(Ring& R, int slot, int* ctrl, int64_t budget_ns) {
#if !NOMAD_STAGE_TMA
  // one commit group per block, kRing - 1 younger groups may stay in flight
  cp_async_wait<kRing - 1>();
  return true;
#endif
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
}

// Reduce-scatter of 32 per-lane partials: lane l ends with the warp total of index l.
__device__ __forceinline__ float reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
  for (int lvl = 0; lvl < 5; ++lvl) {
    const int o = 16 >> lvl;
    const int half = o;  // current size 2*o -> o
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = up ? v[i] : v[i + half];
      const float keep = up ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
  return v[0];
}

template <typename Store, int NV>
__device__ __forceinline__ float visit_long(Tok<Store, NV>& T, float (&h)[NV][Vec<Store>::E], void* W,
                                            const Shape& s, Ring& R, const int2* __restrict__ ratings,
                                            float step, float lambda, uint32_t colkey, int lane,
                                            int* ctrl, int64_t budget_ns, bool& failed) {
  constexpr int E = Vec<Store>::E;
  using Raw = typename Vec<Store>::Raw;
  const int len = T.desc.z;
  const int64_t start = desc_start(T.desc);
  const int nblocks = (len + kBlk - 1) / kBlk;
  const float c = 1.f - step * lambda;
  float err2 = 0.f;
#if NOMAD_STAGE_TMA
  // rows written by earlier generic stores must be visible to the TMA engine
  fence_proxy_async_global();
  __syncwarp();
#endif
  int2 rv_cur = T.rv;
  int2 rv_nxt = lane + kChunk < len && lane < kChunk ? __ldg(&ratings[start + kChunk + lane]) : make_int2(0, 0);
  int chunk_base = 0;  // rating index of rv_cur's lane 0
  constexpr int VB = static_cast<int>(sizeof(Raw));
  for (int b = 0; b < kRing - 1; ++b) {
    if (b < nblocks) issue_block<VB>(R, b, len, chunk_base, rv_cur, rv_nxt, W, s.row_bytes, lane);
    if (!NOMAD_STAGE_TMA) cp_async_commit();
  }
  for (int b = 0; b < nblocks; ++b) {
    if (b + kRing - 1 < nblocks)
      issue_block<VB>(R, b + kRing - 1, len, chunk_base, rv_cur, rv_nxt, W, s.row_bytes, lane);
    if (!NOMAD_STAGE_TMA) cp_async_commit();
    const int slot = b % kRing;
    if (!wait_block(R, slot, ctrl, budget_ns)) {
      failed = true;
      return err2;
    }
    const int first = b * kBlk;
    const int nr = min(kBlk, len - first);
    const char* srow = R.rows + static_cast<size_t>(slot) * kBlk * s.row_bytes;
    // the block's ratings
    int rr[kBlk];
    float vv[kBlk];
#pragma unroll
    for (int t = 0; t < kBlk; ++t) {
      const int idx = first + t - chunk_base;
      const int srcl = min(max(idx, 0), 31);
      const int x1 = __shfl_sync(kFull, rv_cur.x, srcl), y1 = __shfl_sync(kFull, rv_cur.y, srcl);
      const int srcn = min(max(idx - kChunk, 0), 31);
      const int x2 = __shfl_sync(kFull, rv_nxt.x, srcn), y2 = __shfl_sync(kFull, rv_nxt.y, srcn);
      rr[t] = idx < kChunk ? x1 : x2;
      vv[t] = t < nr ? __int_as_float(idx < kChunk ? y1 : y2) : 0.f;
    }
    // partial dot products: p[t] = <h, w_t>, p[7 + t(t-1)/2 + s] = <w_s, w_t>
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
            for (int e = 0; e < E; ++e) p[kBlk + t * (t - 1) / 2 + u] = fmaf(w[u][e], w[t][e], p[kBlk + t * (t - 1) / 2 + u]);
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
    // scalar recurrence for the block's errors
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
    // lane-local row and column updates, row stores
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
    // advance the rating chunk after its fourth block
    if ((b & 3) == 3) {
      rv_cur = rv_nxt;
      chunk_base += kChunk;
      const int nx = chunk_base + kChunk + lane;
      rv_nxt = lane < kChunk && nx < len ? __ldg(&ratings[start + nx]) : make_int2(0, 0);
    }
  }
  return err2;
}

__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// The consumer side of queue q (tail qtail[q], stub node n + q), given `next` =
// qnext[head] already read.  Same steps as nd::mpsc_pop with relaxed loads; the caller
// fences once when it takes a token.
__device__ __forceinline__ int pop_one(int* qnext, int* qtail, int q, int stub, int& head, int next) {
  int h = head;
  if (h == stub) {
    if (next < 0) return -1;
    head = next;
    h = next;
    next = ld_relaxed(&qnext[h]);
  }
  if (next >= 0) {
    head = next;
    return h;
  }
  if (ld_relaxed(&qtail[q]) != h) return -1;
  nd::mpsc_push(qnext, qtail, q, stub);
  next = ld_relaxed(&qnext[h]);
  if (next >= 0) {
    head = next;
    return h;
  }
  return -1;
}

// Producer side of a hop: the caller's stores (every lane's, ordered by the preceding
// __syncwarp) are released by one fence; the tail exchange takes acquire semantics so
// the link store stays after it (Vyukov's push order: next = null, exchange, link).
__device__ __forceinline__ void push_token(int* qnext, int* qtail, int q, int node) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(qnext + node), "r"(-1) : "memory");
  fence_acq_rel_gpu();
  int prev;
  asm volatile("atom.acquire.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(prev) : "l"(qtail + q), "r"(node) : "memory");
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(qnext + prev), "r"(node) : "memory");
}

// Priority queue first; both heads are probed in one round trip.
__device__ __forceinline__ int pop_pref(int* qnext, int* qtail, int w, int P, int n, int& head_lo,
                                        int& head_hi) {
  const int nh = ld_relaxed(&qnext[head_hi]);
  const int nl = ld_relaxed(&qnext[head_lo]);
  int t = pop_one(qnext, qtail, P + w, n + P + w, head_hi, nh);
  if (t < 0) t = pop_one(qnext, qtail, w, n + w, head_lo, nl);
  if (t >= 0) fence_acq_rel_gpu();  // acquire: the token's column and descriptor
  return t;
}

template <typename Store, int NV>
__global__ void __launch_bounds__(256, 2) nomad_async2_kernel(nomad::AsyncArgs a) {
  constexpr int E = Vec<Store>::E;
  extern __shared__ __align__(128) char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int w = blockIdx.x * (blockDim.x >> 5) + wib;
  const int P = a.P, n = a.f.n;
  Shape s;
  s.kpad = a.f.kpad;
  s.nvec = a.f.nvec;
  s.red_width = a.f.red_width;
  s.dim = a.f.dim;
  s.row_bytes = a.f.kpad * static_cast<int>(sizeof(Store));
  s.heavy_min = min(max(a.heavy_min, 1), kChunk + 1);  // longer visits always take the blocked path
  // per-warp shared memory: ring rows | mbarriers | gather
  const size_t ring_bytes = static_cast<size_t>(kRing) * kBlk * s.row_bytes;
  const size_t per_warp = ring_bytes + 8 * kRing + 32 * sizeof(float);
  char* base = smem + static_cast<size_t>(wib) * per_warp;
  Ring R;
  R.rows = base;
  R.bars = smem_u32(base + ring_bytes);
  R.gather = reinterpret_cast<float*>(base + ring_bytes + 8 * kRing);
  R.phase = 0;
  if (lane == 0)
    for (int i = 0; i < kRing; ++i) mbar_init(R.bars + 8u * i, 1);
  fence_mbar_init();
  __syncwarp();
  if (w >= P) return;
  if (w == 0 && lane == 0 && a.finish_ns) a.finish_ns[n] = nd::globaltimer();
  void* W = a.f.W;
  void* H = a.f.H;
  int head_lo = n + w, head_hi = n + P + w;  // lane 0's consumer cursors
  unsigned long long n_upd = 0, n_hops = 0, n_fail = 0, pending = 0, seen = ~0ull;
  uint64_t idle_since = 0;
  double esum = 0.0;
  unsigned backoff = 32;
  bool failed = false;
  Tok<Store, NV> A, B;
  A.tok = -1;
  while (!failed) {
    if (A.tok < 0) {
      int tok = -1;
      if (lane == 0) tok = pop_pref(a.qnext, a.qtail, w, P, n, head_lo, head_hi);
      tok = __shfl_sync(kFull, tok, 0);
      if (tok < 0) {
        int stop = 0;
        if (lane == 0 && (++n_fail & 7) == 1) {  // status checks on every 8th empty poll
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
        continue;
      }
      backoff = 32;
      __syncwarp();
      A.tok = tok;
      stage1<Store, NV>(A, a, s, lane);
      stage2<Store, NV>(A, a, lane);
      stage3<Store, NV>(A, W, s, lane);
    }
    // the next token: pop now, fetch its descriptor and column while A computes
    {
      int tok = -1;
      if (lane == 0) tok = pop_pref(a.qnext, a.qtail, w, P, n, head_lo, head_hi);
      B.tok = __shfl_sync(kFull, tok, 0);
      __syncwarp();
      if (B.tok >= 0) stage1<Store, NV>(B, a, s, lane);
    }
    // ---- process A ------------------------------------------------------------------
    const int len = A.desc.z;
    const int pos = A.desc.w & 0x7fffffff;
    const bool heavy = (static_cast<unsigned>(A.desc.w) & kHeavyBit) != 0;
    const float step = __ldg(&a.steps[min(A.ep, a.n_steps - 1)]);
    const uint32_t colkey = nd::hash32(a.seed32 ^ static_cast<uint32_t>(A.tok) * 0x85EBCA77u ^
                                       static_cast<uint32_t>(A.ep) * 0xC2B2AE3Du);
    float h[NV][E];
#pragma unroll
    for (int q = 0; q < NV; ++q) nd::unpack(A.h[q], h[q]);
    float e2;
    if (len >= s.heavy_min)
      e2 = visit_long<Store, NV>(A, h, W, s, R, a.ratings, step, a.lambda, colkey, lane, a.ctrl,
                                 a.budget_ns, failed);
    else
      e2 = visit_short<Store, NV>(A, h, W, s, step, a.lambda, colkey, lane);
    if (failed) break;
    if (B.tok >= 0) stage2<Store, NV>(B, a, lane);
    // ---- hand A to the next worker of its route (nb_main.cpp:551-565) ------------------
    {
      Store* hrow = reinterpret_cast<Store*>(static_cast<char*>(H) + static_cast<int64_t>(A.tok) * s.row_bytes);
      const uint32_t hkey = nd::hash32(colkey ^ static_cast<uint32_t>(pos) * 0x27D4EB2Fu);
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const int v = lane + 32 * q;
        if (v < s.nvec) nd::store_vec<Store, true>(hrow, v, h[q], hkey + 4u * static_cast<uint32_t>(v));
      }
    }
    int npos = pos + 1, nep = A.ep;
    if (npos == A.nseg) {
      npos = 0;
      nep = A.ep + 1;
    }
    const bool retire = nep >= a.target_epoch;
    n_upd += static_cast<unsigned long long>(len);
    ++n_hops;
    if (lane == 0) {
      if (!retire)
        __stcg(&a.tok_desc[A.tok], make_int4(A.nseg4.x, A.nseg4.y, A.nseg4.z,
                                             npos | (heavy ? static_cast<int>(kHeavyBit) : 0)));
      __stcg(&a.tok_epoch[A.tok], nep);
      esum += static_cast<double>(e2);
      ++pending;
    }
    if (B.tok >= 0) stage3<Store, NV>(B, W, s, lane);  // after A's row stores
    __syncwarp();
    if (lane == 0) {
      if (retire) {
        if (a.finish_ns) a.finish_ns[A.tok] = nd::globaltimer();
        fence_acq_rel_gpu();
        atomicAdd(&a.ctrl[0], 1);
      } else {
        push_token(a.qnext, a.qtail, (heavy ? P : 0) + A.nseg4.w, A.tok);
      }
      if (pending >= 64) {
        atomicAdd(a.progress, pending);
        pending = 0;
      }
    }
    A = B;
    if ((n_hops & 15) == 0) {
      int stop = 0;
      if (lane == 0) stop = nd::ld_acquire(&a.ctrl[1]) != 0;
      if (__shfl_sync(kFull, stop, 0)) break;
    }
  }
  // wait (bounded) for any staged block still in flight before leaving
  if (!NOMAD_STAGE_TMA) cp_async_wait<0>();
  if (failed) {
    for (int slot = 0; slot < kRing; ++slot) {
      const uint32_t bar = R.bars + 8u * slot;
      for (int it = 0; it < 4096 && !mbar_try_wait(bar, (R.phase >> slot) & 1u); ++it) {
      }
    }
  }
  if (lane == 0) {
    if (pending) atomicAdd(a.progress, pending);
    atomicAdd(&a.stats[0], n_upd);
    atomicAdd(&a.stats[1], n_hops);
    atomicAdd(&a.stats[2], n_fail);
    atomicAdd(a.err_sum, esum);
  }
}

template <typename Store, int NV>
size_t smem_per_block(int warps, int kpad) {
  const size_t row_bytes = static_cast<size_t>(kpad) * sizeof(Store);
  return static_cast<size_t>(warps) * (kRing * kBlk * row_bytes + 8 * kRing + 32 * sizeof(float));
}

template <typename Store, int NV>
cudaError_t launch2_t(const nomad::AsyncArgs& a, cudaStream_t st) {
  const size_t smem = smem_per_block<Store, NV>(a.warps_per_block, a.f.kpad);
  cudaError_t e = cudaFuncSetAttribute(&nomad_async2_kernel<Store, NV>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<nomad::AsyncArgs*>(&a)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<void*>(&nomad_async2_kernel<Store, NV>),
                                     dim3(a.grid), dim3(a.warps_per_block * 32), args, smem, st);
}

template <typename Store, int NV>
cudaError_t occ2_t(int warps, int kpad, int* bps) {
  const size_t smem = smem_per_block<Store, NV>(warps, kpad);
  cudaError_t e = cudaFuncSetAttribute(&nomad_async2_kernel<Store, NV>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
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

}  // namespace nomad
