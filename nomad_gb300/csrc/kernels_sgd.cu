// kernels_sgd.cu -- NOMAD SGD kernels for sm_103a: the asynchronous token-passing
// persistent kernel, the deterministic replay kernel and the DSGD stratum kernel.
//
// Per rating (row i, column j, value v), as Code/nomad/nb_main.cpp:520-542 defines it:
//   e   = <h_j, w_i> - v
//   w_i = w_i - step * (e * h_j + lambda * w_i)
//   h_j = h_j - step * (e * w_i_old + lambda * h_j)
// One warp runs one rating at a time: each lane holds one 16-byte vector of the row
// (4 fp32 or 8 bf16), the dot product is a warp-shuffle reduction, and the held
// column h_j lives in fp32 registers for the whole visit.
#include <cuda_bf16.h>

#include "device_common.cuh"
#include "launch.h"

namespace {

using nd::kFull;
using nd::Vec;

// Raw vectors of a row (fp32 x4 = 16 bytes, bf16 x4 = 8 bytes): kept packed while in
// flight, unpacked to fp32 when used.
template <typename Store, int NV>
__device__ __forceinline__ void load_row_raw(const Store* __restrict__ W, int r, int kpad, int nvec,
                                             int lane, typename Vec<Store>::Raw (&x)[NV]) {
  using Raw = typename Vec<Store>::Raw;
  const Raw* row = reinterpret_cast<const Raw*>(W + static_cast<int64_t>(r) * kpad);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    x[q] = v < nvec ? row[v] : nd::zero_raw<Raw>();
  }
}

template <typename Store, int NV>
__device__ __forceinline__ void load_row(const Store* __restrict__ W, int r, int kpad,
                                         int nvec, int lane,
                                         float (&x)[NV][Vec<Store>::E]) {
  typename Vec<Store>::Raw raw[NV];
  load_row_raw<Store, NV>(W, r, kpad, nvec, lane, raw);
#pragma unroll
  for (int q = 0; q < NV; ++q) nd::unpack(raw[q], x[q]);
}

template <typename Store, int NV>
__device__ __forceinline__ void store_row(Store* __restrict__ W, int r, int kpad, int nvec,
                                          int lane, const float (&x)[NV][Vec<Store>::E],
                                          uint32_t key) {
  Store* row = W + static_cast<int64_t>(r) * kpad;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    if (v < nvec) nd::store_vec<Store, false>(row, v, x[q], key + 4u * static_cast<uint32_t>(v));
  }
}

// Error of one rating.  Fast form: lane-local FMAs, then a butterfly reduction.
// Exact form: the reference's order -- -v + h0*w0 + h1*w1 + ... each product and sum
// rounded separately (std::inner_product seeded with -v) -- by lane 0 over the
// products staged in shared memory.
template <typename Store, int NV, bool EXACT>
__device__ __forceinline__ float rating_error(const float (&h)[NV][Vec<Store>::E],
                                              const float (&w)[NV][Vec<Store>::E], float v,
                                              int nvec, int red_width, int dim, int lane,
                                              float* xbuf) {
  constexpr int E = Vec<Store>::E;
  if (!EXACT) {
    float part = 0.f;
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
      for (int e = 0; e < E; ++e) part = fmaf(h[q][e], w[q][e], part);
    return nd::warp_allreduce(part, red_width) - v;
  } else {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int vv = lane + 32 * q;
      if (vv < nvec)
#pragma unroll
        for (int e = 0; e < E; ++e) xbuf[vv * E + e] = __fmul_rn(h[q][e], w[q][e]);
    }
    __syncwarp();
    float acc = -v;
    if (lane == 0)
      for (int i = 0; i < dim; ++i) acc = __fadd_rn(acc, xbuf[i]);
    __syncwarp();
    return __shfl_sync(kFull, acc, 0);
  }
}

template <typename Store, int NV, bool EXACT>
__device__ __forceinline__ void apply_update(float (&h)[NV][Vec<Store>::E],
                                             float (&w)[NV][Vec<Store>::E], float err,
                                             float step, float lambda) {
  constexpr int E = Vec<Store>::E;
#pragma unroll
  for (int q = 0; q < NV; ++q)
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const float wo = w[q][e];
      const float ho = h[q][e];
      if (EXACT) {
        w[q][e] = __fsub_rn(wo, __fmul_rn(step, __fadd_rn(__fmul_rn(err, ho), __fmul_rn(lambda, wo))));
        h[q][e] = __fsub_rn(ho, __fmul_rn(step, __fadd_rn(__fmul_rn(err, wo), __fmul_rn(lambda, ho))));
      } else {
        w[q][e] = fmaf(-step, fmaf(err, ho, lambda * wo), wo);
        h[q][e] = fmaf(-step, fmaf(err, wo, lambda * ho), ho);
      }
    }
}

// One visit of a held column over a run of ratings [start, start+len) whose rows are
// distinct (a column segment), so the rows can be prefetched PF ratings ahead.
template <typename Store, int NV, bool EXACT, int PF>
__device__ __forceinline__ float visit_segment(Store* __restrict__ W, const nomad::DevFactors& f,
                                               float (&h)[NV][Vec<Store>::E],
                                               const int2* __restrict__ ratings,
                                               int64_t start, int len, float step,
                                               float lambda, uint32_t colkey, int lane,
                                               float* xbuf) {
  float seg_err = 0.f;
  for (int base = 0; base < len; base += 32) {
    const int cnt = min(32, len - base);
    int2 rv = make_int2(0, 0);
    if (lane < cnt) rv = __ldg(&ratings[start + base + lane]);
    typename Vec<Store>::Raw wbuf[PF][NV];
#pragma unroll
    for (int i = 0; i < PF; ++i) {
      const int r = __shfl_sync(kFull, rv.x, i);
      if (i < cnt) load_row_raw<Store, NV>(W, r, f.kpad, f.nvec, lane, wbuf[i]);
    }
    for (int t0 = 0; t0 < cnt; t0 += PF) {
#pragma unroll
      for (int i = 0; i < PF; ++i) {
        const int t = t0 + i;
        if (t < cnt) {
          const int r = __shfl_sync(kFull, rv.x, t);
          const float v = __int_as_float(__shfl_sync(kFull, rv.y, t));
          float w[NV][Vec<Store>::E];
#pragma unroll
          for (int q = 0; q < NV; ++q) nd::unpack(wbuf[i][q], w[q]);
          const float err = rating_error<Store, NV, EXACT>(h, w, v, f.nvec, f.red_width, f.dim, lane, xbuf);
          seg_err += err * err;
          apply_update<Store, NV, EXACT>(h, w, err, step, lambda);
          store_row<Store, NV>(W, r, f.kpad, f.nvec, lane, w,
                               nd::row_key(r, colkey));
          const int tn = t + PF;
          const int rn = __shfl_sync(kFull, rv.x, tn & 31);
          if (tn < cnt) load_row_raw<Store, NV>(W, rn, f.kpad, f.nvec, lane, wbuf[i]);
        }
      }
    }
  }
  return seg_err;
}

template <typename Store, int NV>
__device__ __forceinline__ void load_col(const Store* __restrict__ H, int j, const nomad::DevFactors& f,
                                         int lane, float (&h)[NV][Vec<Store>::E]) {
  const Store* row = H + static_cast<int64_t>(j) * f.kpad;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    if (v < f.nvec) {
      nd::load_vec_cg<Store>(row, v, h[q]);
    } else {
#pragma unroll
      for (int e = 0; e < Vec<Store>::E; ++e) h[q][e] = 0.f;
    }
  }
}

template <typename Store, int NV>
__device__ __forceinline__ void store_col(Store* __restrict__ H, int j, const nomad::DevFactors& f,
                                          int lane, const float (&h)[NV][Vec<Store>::E],
                                          uint32_t key) {
  Store* row = H + static_cast<int64_t>(j) * f.kpad;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int v = lane + 32 * q;
    if (v < f.nvec) nd::store_vec<Store, true>(row, v, h[q], key + 4u * static_cast<uint32_t>(v));
  }
}

// ---------------------------------------------------------------------------------
// Asynchronous NOMAD: one persistent warp per worker (NomadBody::updater_func,
// nb_main.cpp:480-572).  A worker owns a contiguous block of rows; column tokens move
// between workers through the per-worker MPSC queues.  A token's visit list holds only
// the workers that own ratings of the column, in a seeded random order (the
// reference's per-token permutation, pool.cpp:32-38, restricted to non-empty visits);
// after its last visit the pass count goes up, which drives the step size exactly
// as col_update_counts does (nb_main.cpp:514-515, 544).  The kernel returns when
// every token has completed target_epoch passes.
// ---------------------------------------------------------------------------------
template <typename Store, int NV, bool EXACT, int PF>
__global__ void __launch_bounds__(256) nomad_async_kernel(nomad::AsyncArgs a) {
  constexpr int E = Vec<Store>::E;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int w = blockIdx.x * (blockDim.x >> 5) + wib;
  if (w >= a.P) return;
  float* xbuf = smem + wib * a.f.kpad;
  Store* __restrict__ W = static_cast<Store*>(a.f.W);
  Store* __restrict__ H = static_cast<Store*>(a.f.H);
  const int n = a.f.n;
  const int stub = n + w;
  int head = stub;  // consumer cursor, used by lane 0 only
  unsigned long long n_upd = 0, n_hops = 0, n_fail = 0, pending = 0, seen = ~0ull;
  uint64_t idle_since = 0;
  double esum = 0.0;
  unsigned backoff = 64;

  while (true) {
    int tok = -1;
    if (lane == 0) tok = nd::mpsc_pop(a.qnext, a.qtail, w, stub, head);
    tok = __shfl_sync(kFull, tok, 0);
    if (tok < 0) {
      int stop = 0;
      if (lane == 0) {
        ++n_fail;
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
      backoff = min(backoff * 2, 2048u);
      continue;
    }
    backoff = 64;
    __syncwarp();  // lane 0 acquired the token; order the other lanes after it

    const int pos = __ldcg(&a.tok_pos[tok]);
    const int ep = __ldcg(&a.tok_epoch[tok]);
    const int64_t vb = __ldg(&a.vl_ptr[tok]);
    const int64_t ve = __ldg(&a.vl_ptr[tok + 1]);
    const int4 sg = __ldg(&a.segs[vb + pos]);
    const int64_t s_start = static_cast<int64_t>(static_cast<uint32_t>(sg.x)) |
                            (static_cast<int64_t>(sg.y) << 32);
    const int len = sg.z;
    const float step = __ldg(&a.steps[min(ep, a.n_steps - 1)]);
    const uint32_t colkey = nd::hash32(a.seed32 ^ static_cast<uint32_t>(tok) * 0x85EBCA77u ^
                                       static_cast<uint32_t>(ep) * 0xC2B2AE3Du);

    float h[NV][E];
    load_col<Store, NV>(H, tok, a.f, lane, h);
    const float e2 = visit_segment<Store, NV, EXACT, PF>(W, a.f, h, a.ratings, s_start, len, step,
                                                         a.lambda, colkey, lane, xbuf);
    store_col<Store, NV>(H, tok, a.f, lane, h, nd::hash32(colkey ^ static_cast<uint32_t>(pos) * 0x27D4EB2Fu));

    // routing (nb_main.cpp:551-565): next worker of the visit list, or the next pass
    int npos = pos + 1, nep = ep;
    if (vb + npos == ve) {
      npos = 0;
      nep = ep + 1;
    }
    const bool retire = nep >= a.target_epoch;
    int next_w = 0;
    if (!retire) next_w = __ldg(&a.segs[vb + npos]).w;
    n_upd += static_cast<unsigned long long>(len);  // warp-uniform counters
    ++n_hops;
    if (lane == 0) {
      __stcg(&a.tok_pos[tok], npos);
      __stcg(&a.tok_epoch[tok], nep);
      esum += static_cast<double>(e2);
      ++pending;
    }
    __syncwarp();  // every lane's H stores precede lane 0's fence and publication
    if (lane == 0) {
      __threadfence();
      if (retire)
        atomicAdd(&a.ctrl[0], 1);
      else
        nd::mpsc_push(a.qnext, a.qtail, next_w, tok);
      if (pending >= 64) {
        atomicAdd(a.progress, pending);
        pending = 0;
      }
    }
    if ((n_hops & 15) == 0) {
      int stop = 0;
      if (lane == 0) stop = nd::ld_acquire(&a.ctrl[1]) != 0;
      if (__shfl_sync(kFull, stop, 0)) break;
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

// ---------------------------------------------------------------------------------
// Deterministic replay: one warp, columns 0..n-1 per epoch in index order, exact
// arithmetic.  This is the reference's schedule with one worker and one rank
// (FIFO queue starting in column order, nb_main.cpp:82-97, 554-558).
// ---------------------------------------------------------------------------------
template <typename Store, int NV>
__global__ void __launch_bounds__(32) nomad_replay_kernel(nomad::ReplayArgs a) {
  constexpr int E = Vec<Store>::E;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31;
  Store* __restrict__ W = static_cast<Store*>(a.f.W);
  Store* __restrict__ H = static_cast<Store*>(a.f.H);
  double esum = 0.0;
  for (int ep = a.first_epoch; ep < a.first_epoch + a.n_epochs; ++ep) {
    const float step = a.steps[ep];
    for (int j = 0; j < a.f.n; ++j) {
      const int64_t b = a.col_ptr[j], e = a.col_ptr[j + 1];
      if (b == e) continue;
      const uint32_t colkey = nd::hash32(a.seed32 ^ static_cast<uint32_t>(j) * 0x85EBCA77u ^
                                         static_cast<uint32_t>(ep) * 0xC2B2AE3Du);
      float h[NV][E];
      load_col<Store, NV>(H, j, a.f, lane, h);
      esum += visit_segment<Store, NV, true, 2>(W, a.f, h, a.ratings, b, static_cast<int>(e - b),
                                                step, a.lambda, colkey, lane, smem);
      store_col<Store, NV>(H, j, a.f, lane, h, nd::hash32(colkey));
      __syncwarp();
    }
  }
  if (lane == 0 && a.err_sum) *a.err_sum += esum;
}

// ---------------------------------------------------------------------------------
// DSGD stratum (Code/competitor/sgd-mpi-omp.cpp:354-365; DSGD++ dsgdpp.cpp:403-415,
// 444-456): warp bi runs block (bi, sched[stratum][bi]) of the innerB x col_blocks
// grid; the blocks of a stratum share no row and no column.  Inside a block, ratings run in the reference's order
// (sgd() walks each block from its last entry to its first; the host stores blocks
// already reversed).  Exact form: err = (sum from index k-1 down to 0 of w*h) - v.
// The next rating's rows are fetched ahead unless it shares the row or the column.
// ---------------------------------------------------------------------------------
template <typename Store, int NV, bool EXACT>
__global__ void __launch_bounds__(128) nomad_dsgd_kernel(nomad::DsgdArgs a, int stratum) {
  constexpr int E = Vec<Store>::E;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int bi = blockIdx.x * (blockDim.x >> 5) + wib;
  if (bi >= a.innerB) return;
  float* xbuf = smem + wib * a.f.kpad;
  Store* __restrict__ W = static_cast<Store*>(a.f.W);
  Store* __restrict__ H = static_cast<Store*>(a.f.H);
  const int bj = a.sched[static_cast<int64_t>(stratum) * a.innerB + bi];
  const int64_t bid = static_cast<int64_t>(bi) * a.col_blocks + bj;
  const int64_t b = a.blk_ptr[bid], e = a.blk_ptr[bid + 1];
  if (b == e) return;
  const nomad::DevFactors& f = a.f;
  int4 cur = __ldg(&a.rates[b]);
  float w[NV][E], h[NV][E];
  load_row<Store, NV>(W, cur.x, f.kpad, f.nvec, lane, w);
  load_row<Store, NV>(H, cur.y, f.kpad, f.nvec, lane, h);
  for (int64_t o = b; o < e; ++o) {
    const bool has_next = o + 1 < e;
    int4 nxt = has_next ? __ldg(&a.rates[o + 1]) : make_int4(-1, -1, 0, 0);
    float wn[NV][E], hn[NV][E];
    const bool pre_w = has_next && nxt.x != cur.x;
    const bool pre_h = has_next && nxt.y != cur.y;
    if (pre_w) load_row<Store, NV>(W, nxt.x, f.kpad, f.nvec, lane, wn);
    if (pre_h) load_row<Store, NV>(H, nxt.y, f.kpad, f.nvec, lane, hn);
    const float v = __int_as_float(cur.z);
    float err;
    if (!EXACT) {
      float part = 0.f;
#pragma unroll
      for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int k = 0; k < E; ++k) part = fmaf(w[q][k], h[q][k], part);
      err = nd::warp_allreduce(part, f.red_width) - v;
    } else {
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const int vv = lane + 32 * q;
        if (vv < f.nvec)
#pragma unroll
          for (int k = 0; k < E; ++k) xbuf[vv * E + k] = __fmul_rn(w[q][k], h[q][k]);
      }
      __syncwarp();
      float acc = 0.f;
      if (lane == 0)
        for (int i = f.dim - 1; i >= 0; --i) acc = __fadd_rn(acc, xbuf[i]);
      __syncwarp();
      err = __fsub_rn(__shfl_sync(kFull, acc, 0), v);
    }
    apply_update<Store, NV, EXACT>(h, w, err, a.step, a.lambda);
    const uint32_t key = nd::hash32(a.seed32 ^ static_cast<uint32_t>(o) * 0x9E3779B1u ^
                                    static_cast<uint32_t>(a.iter) * 0xC2B2AE3Du);
    store_row<Store, NV>(W, cur.x, f.kpad, f.nvec, lane, w, key);
    store_row<Store, NV>(H, cur.y, f.kpad, f.nvec, lane, h, nd::hash32(key));
    if (has_next) {
      if (pre_w) {
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
          for (int k = 0; k < E; ++k) w[q][k] = wn[q][k];
      } else if (sizeof(Store) == 2) {
        // bf16: continue from the stored (rounded) value, as a reload would see it
        load_row<Store, NV>(W, cur.x, f.kpad, f.nvec, lane, w);
      }
      if (pre_h) {
#pragma unroll
        for (int q = 0; q < NV; ++q)
#pragma unroll
          for (int k = 0; k < E; ++k) h[q][k] = hn[q][k];
      } else if (sizeof(Store) == 2) {
        load_row<Store, NV>(H, cur.y, f.kpad, f.nvec, lane, h);
      }
    }
    cur = nxt;
  }
}

template <typename Store, int NV, bool EXACT, int PF>
cudaError_t launch_async_t(const nomad::AsyncArgs& a, cudaStream_t s) {
  const int threads = a.warps_per_block * 32;
  const size_t smem = EXACT ? static_cast<size_t>(a.warps_per_block) * a.f.kpad * sizeof(float) : 0;
  void* args[] = {const_cast<nomad::AsyncArgs*>(&a)};
  return cudaLaunchCooperativeKernel(reinterpret_cast<void*>(&nomad_async_kernel<Store, NV, EXACT, PF>),
                                     dim3(a.grid), dim3(threads), args, smem, s);
}

template <typename Store, int NV, bool EXACT, int PF>
cudaError_t occ_t(int warps_per_block, int kpad, int* bps) {
  const size_t smem = EXACT ? static_cast<size_t>(warps_per_block) * kpad * sizeof(float) : 0;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      bps, &nomad_async_kernel<Store, NV, EXACT, PF>, warps_per_block * 32, smem);
}

constexpr int kPF = 4;


// ---------------------------------------------------------------------------------
// Batched problems: independent completion problems taken one at a time by a warp from
// a device work queue (problems by decreasing rating count).  Each problem runs the
// reference's one-worker schedule -- columns in index order, every column's ratings in
// row order (nb_main.cpp:82-97, 554-558 with one thread and one rank) -- so the exact
// form reproduces the one-worker replay of every problem bit for bit.  k <= 128 (one
// vector of 4 values per lane); lanes past k/4 idle, reductions span the k/4 lanes.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ nomad::DevFactors batch_factors(const nomad::BatchArgs& a, const nomad::BatchProblem& pb,
                                                           int esz) {
  nomad::DevFactors f;
  f.W = static_cast<char*>(a.W) + pb.w_off * esz;
  f.H = static_cast<char*>(a.H) + pb.h_off * esz;
  f.m = pb.m;
  f.n = pb.n;
  f.dim = pb.dim;
  f.kpad = pb.kpad;
  f.nvec = pb.nvec;
  f.red_width = pb.red_width;
  f.bf16 = esz == 2;
  return f;
}

template <typename Store, bool EXACT>
__global__ void __launch_bounds__(nomad::kBatchThreads) nomad_batch_kernel(nomad::BatchArgs a) {
  constexpr int NV = 1;
  constexpr int E = Vec<Store>::E;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31;
  float* xbuf = smem + (threadIdx.x >> 5) * 128;  // exact form: one row of products
  const int ep = *a.epoch;
  const float step = a.steps[min(ep, a.n_steps - 1)];
  double esum = 0.0;
  unsigned long long n_upd = 0;
  while (true) {
    int p = 0;
    if (lane == 0) p = atomicAdd(a.next, 1);
    p = __shfl_sync(kFull, p, 0);
    if (p >= a.count) break;
    const int prob = a.order[p];
    const nomad::BatchProblem pb = a.problems[prob];
    const nomad::DevFactors f = batch_factors(a, pb, static_cast<int>(sizeof(Store)));
    Store* __restrict__ W = static_cast<Store*>(f.W);
    Store* __restrict__ H = static_cast<Store*>(f.H);
    const int64_t* cp = a.col_ptr + pb.col_off;
    const uint32_t pkey = nd::hash32(a.seed32 ^ static_cast<uint32_t>(prob) * 0x27D4EB2Fu);
    for (int j = 0; j < pb.n; ++j) {
      const int64_t b = cp[j], e = cp[j + 1];
      if (b == e) continue;
      const uint32_t colkey = nd::hash32(pkey ^ static_cast<uint32_t>(j) * 0x85EBCA77u ^
                                         static_cast<uint32_t>(ep) * 0xC2B2AE3Du);
      float h[NV][E];
      load_col<Store, NV>(H, j, f, lane, h);
      esum += visit_segment<Store, NV, EXACT, 2>(W, f, h, a.ratings, b, static_cast<int>(e - b), step, a.lambda,
                                                 colkey, lane, xbuf);
      store_col<Store, NV>(H, j, f, lane, h, nd::hash32(colkey));
      n_upd += static_cast<unsigned long long>(e - b);
      __syncwarp();
    }
  }
  if (lane == 0) {
    atomicAdd(&a.stats[0], n_upd);
    atomicAdd(a.err_sum, esum);
  }
}

// After an epoch launch: the next pass count, and the work queue back at its head.
__global__ void batch_advance_kernel(int32_t* epoch, int32_t* next) {
  *epoch += 1;
  *next = 0;
}

// FP64 squared errors of the evaluation's parts, a warp per part: the part's first column
// by a binary search of its problem's column offsets, then rating by rating, the column
// reloaded as it changes.  (A warp per whole problem left the largest problems' millions
// of ratings on one warp each.)  The host adds the parts of a problem in order.
template <typename Store>
__global__ void __launch_bounds__(nomad::kBatchThreads) batch_sse_kernel(nomad::BatchArgs a) {
  constexpr int NV = 1;
  constexpr int E = Vec<Store>::E;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int part = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); part < a.n_parts; part += warps) {
    const nomad::SsePart pt = a.parts[part];
    const nomad::BatchProblem pb = a.problems[pt.prob];
    const nomad::DevFactors f = batch_factors(a, pb, static_cast<int>(sizeof(Store)));
    const Store* __restrict__ W = static_cast<const Store*>(f.W);
    const Store* __restrict__ H = static_cast<const Store*>(f.H);
    const int2* rt = pt.set ? a.test : a.ratings;
    const int64_t* cp = pt.set ? a.test_col_ptr + pb.test_col_off : a.col_ptr + pb.col_off;
    int lo = 0, hi = pb.n;  // the last column j with cp[j] <= start (cp[0] <= start < cp[n])
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (cp[mid] <= pt.start) lo = mid;
      else hi = mid;
    }
    int j = lo;
    float h[NV][E];
    load_col<Store, NV>(H, j, f, lane, h);
    double acc = 0.0;
    // kU ratings at a time: their rows are loaded together, then the errors are summed in
    // rating order (the same FP64 sum as one at a time)
    constexpr int kU = 4;
    for (int64_t o0 = pt.start; o0 < pt.end; o0 += kU) {
      int2 r[kU];
      typename Vec<Store>::Raw wr[kU][NV];
#pragma unroll
      for (int u = 0; u < kU; ++u) r[u] = o0 + u < pt.end ? __ldg(&rt[o0 + u]) : make_int2(0, 0);
#pragma unroll
      for (int u = 0; u < kU; ++u)
        if (o0 + u < pt.end) load_row_raw<Store, NV>(W, r[u].x, f.kpad, f.nvec, lane, wr[u]);
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int64_t o = o0 + u;
        if (o < pt.end) {
          if (cp[j + 1] <= o) {
            do ++j;
            while (cp[j + 1] <= o);
            load_col<Store, NV>(H, j, f, lane, h);
          }
          float w[NV][E];
#pragma unroll
          for (int q = 0; q < NV; ++q) nd::unpack(wr[u][q], w[q]);
          const float err = rating_error<Store, NV, false>(h, w, __int_as_float(r[u].y), f.nvec, f.red_width,
                                                           f.dim, lane, nullptr);
          acc += static_cast<double>(err) * err;
        }
      }
    }
    if (lane == 0) a.part_sse[part] = acc;
  }
}

// ---------------------------------------------------------------------------------
// FMA form of the batch: a problem with more ratings than a warp's fair share runs on all
// kBatchWorkers warps of one block as NOMAD workers.  Warp r owns rows
// [row_start[r], row_start[r+1]); a column token visits the row blocks (j + i) mod R,
// i = 0..R-1, once per epoch (the reference's routing on one rank, with a rotation in
// place of the shuffled permutation, nb_main.cpp:551-565).  Tokens move through per-warp
// rings of sequence-tagged entries in global memory; every producer and consumer is in
// the block, so block-scope release/acquire orders them and the tail counters are
// shared-memory atomics.  The ring counters persist across problems and launches, so an
// old entry never matches.  Other problems run the one-worker schedule on one warp.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ld_acquire_cta_g64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.cta.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta_g64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.cta.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// A large problem's epoch on the block's R warps (all call it; it ends with a barrier).
template <typename Store>
__device__ __forceinline__ void batch_large_problem(const nomad::BatchArgs& a, int prob, int ep, float step,
                                                    double& esum, unsigned long long& n_upd, unsigned* s_tail,
                                                    int* s_done, int lane, int wib) {
  constexpr int NV = 1;
  constexpr int E = Vec<Store>::E;
  constexpr int R = nomad::kBatchWorkers;
  constexpr unsigned kMask = nomad::kBatchRing - 1;
  const nomad::BatchProblem pb = a.problems[prob];
  const nomad::DevFactors f = batch_factors(a, pb, static_cast<int>(sizeof(Store)));
  Store* __restrict__ W = static_cast<Store*>(f.W);
  Store* __restrict__ H = static_cast<Store*>(f.H);
  const int64_t* seg = a.seg + pb.seg_off;
  const int64_t* cp = a.col_ptr + pb.col_off;
  unsigned long long* rings = a.rings + static_cast<int64_t>(blockIdx.x) * R * nomad::kBatchRing;
  unsigned long long* ring = rings + static_cast<int64_t>(wib) * nomad::kBatchRing;
  unsigned* ctr = a.ring_ctr + static_cast<int64_t>(blockIdx.x) * R;
  const uint32_t pkey = nd::hash32(a.seed32 ^ static_cast<uint32_t>(prob) * 0x27D4EB2Fu);
  // seed this warp's ring: the columns j = wib (mod R) with ratings, in index order
  const unsigned base = ctr[wib];
  unsigned k = 0;
  for (int j0 = wib; j0 < pb.n; j0 += 32 * R) {
    const int j = j0 + lane * R;
    const bool has = j < pb.n && cp[j + 1] > cp[j];
    const unsigned bal = __ballot_sync(kFull, has);
    if (has) {
      const unsigned seq = base + k + __popc(bal & ((1u << lane) - 1u));
      ring[seq & kMask] = (static_cast<unsigned long long>(seq) << 32) | static_cast<unsigned>(j);
    }
    k += __popc(bal);
  }
  if (lane == 0) s_tail[wib] = base + k;
  __syncthreads();  // every ring seeded; s_done was cleared before the caller's barrier
  unsigned head = base, backoff = 32;
  uint64_t idle_since = 0;
  while (true) {
    unsigned long long e = 0;
    if (lane == 0) e = ld_acquire_cta_g64(ring + (head & kMask));
    const unsigned hi = __shfl_sync(kFull, static_cast<unsigned>(e >> 32), 0);
    const unsigned lo = __shfl_sync(kFull, static_cast<unsigned>(e), 0);
    if (hi == head && !(lo & 0x80000000u)) {
      __syncwarp();
      ++head;
      const int j = static_cast<int>(lo & 0xffffu), pos = static_cast<int>(lo >> 16);
      const int64_t b = seg[static_cast<int64_t>(j) * (R + 1) + wib];
      const int64_t en = seg[static_cast<int64_t>(j) * (R + 1) + wib + 1];
      if (en > b) {
        const uint32_t colkey = nd::hash32(pkey ^ static_cast<uint32_t>(j) * 0x85EBCA77u ^
                                           static_cast<uint32_t>(ep) * 0xC2B2AE3Du);
        float h[NV][E];
        const Store* hrow = H + static_cast<int64_t>(j) * f.kpad;  // last written by a warp of this block
        if (lane < f.nvec) nd::load_vec<Store>(hrow, lane, h[0]);
        else
#pragma unroll
          for (int i = 0; i < E; ++i) h[0][i] = 0.f;
        esum += visit_segment<Store, NV, false, 2>(W, f, h, a.ratings, b, static_cast<int>(en - b), step, a.lambda,
                                                   colkey, lane, nullptr);
        store_col<Store, NV>(H, j, f, lane, h, nd::hash32(colkey));
        n_upd += static_cast<unsigned long long>(en - b);
      }
      __syncwarp();  // the column's stores precede lane 0's release
      if (lane == 0) {
        if (pos + 1 < R) {
          const int nr = (j + pos + 1) % R;
          const unsigned seq = atomicAdd(&s_tail[nr], 1u);
          st_release_cta_g64(rings + static_cast<int64_t>(nr) * nomad::kBatchRing + (seq & kMask),
                             (static_cast<unsigned long long>(seq) << 32) |
                                 static_cast<unsigned>(j | ((pos + 1) << 16)));
        } else {
          atomicAdd(s_done, 1);
        }
      }
      backoff = 32;
      idle_since = 0;
    } else {
      int fin = 0;
      if (lane == 0) {
        fin = *reinterpret_cast<volatile int*>(s_done) >= pb.n_active;
        const uint64_t now = nd::globaltimer();
        if (!fin) {
          if (idle_since == 0) {
            idle_since = now;
          } else if (static_cast<int64_t>(now - idle_since) > a.budget_ns) {
            atomicCAS(&a.ctrl[1], 0, nd::kDevErrTimeout);
            fin = 1;
          }
        }
      }
      if (__shfl_sync(kFull, fin, 0)) break;
      __nanosleep(backoff);
      backoff = min(backoff * 2, 256u);
    }
  }
  if (lane == 0) ctr[wib] = head;
  __syncthreads();
}

// Built for one block per SM (74 / 86 registers) and for four (64 warps, the SM's limit;
// 32 registers, a few spilled): a warp's visit waits on its row loads, so four blocks
// carry more work at once, while one leaves the SM to a single large problem's workers.
template <typename Store, int MB>
__global__ void __launch_bounds__(nomad::kBatchWorkers * 32, MB) nomad_batch2_kernel(nomad::BatchArgs a) {
  constexpr int NV = 1;
  constexpr int E = Vec<Store>::E;
  __shared__ unsigned s_tail[nomad::kBatchWorkers];
  __shared__ int s_done, s_big;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int ep = *a.epoch;
  const float step = a.steps[min(ep, a.n_steps - 1)];
  double esum = 0.0;
  unsigned long long n_upd = 0;
  // large problems, a block each
  while (true) {
    if (threadIdx.x == 0) {  // one thread decides for the block, so every thread leaves together
      s_big = nd::ld_acquire(&a.ctrl[1]) != 0 ? a.n_big : atomicAdd(a.next_big, 1);
      s_done = 0;
    }
    __syncthreads();
    const int q = s_big;
    if (q >= a.n_big) break;
    batch_large_problem<Store>(a, a.order[q], ep, step, esum, n_upd, s_tail, &s_done, lane, wib);
  }
  // the rest, a warp each: the one-worker schedule in FMA arithmetic
  while (true) {
    int p = 0;
    if (lane == 0) p = atomicAdd(a.next, 1);
    p = __shfl_sync(kFull, p, 0);
    if (p >= a.count) break;
    const int prob = a.order[p];
    const nomad::BatchProblem pb = a.problems[prob];
    const nomad::DevFactors f = batch_factors(a, pb, static_cast<int>(sizeof(Store)));
    Store* __restrict__ W = static_cast<Store*>(f.W);
    Store* __restrict__ H = static_cast<Store*>(f.H);
    const int64_t* cp = a.col_ptr + pb.col_off;
    const uint32_t pkey = nd::hash32(a.seed32 ^ static_cast<uint32_t>(prob) * 0x27D4EB2Fu);
    for (int j = 0; j < pb.n; ++j) {
      const int64_t b = cp[j], e = cp[j + 1];
      if (b == e) continue;
      const uint32_t colkey = nd::hash32(pkey ^ static_cast<uint32_t>(j) * 0x85EBCA77u ^
                                         static_cast<uint32_t>(ep) * 0xC2B2AE3Du);
      float h[NV][E];
      load_col<Store, NV>(H, j, f, lane, h);
      esum += visit_segment<Store, NV, false, 2>(W, f, h, a.ratings, b, static_cast<int>(e - b), step, a.lambda,
                                                 colkey, lane, nullptr);
      store_col<Store, NV>(H, j, f, lane, h, nd::hash32(colkey));
      n_upd += static_cast<unsigned long long>(e - b);
      __syncwarp();
    }
  }
  if (lane == 0) {
    atomicAdd(&a.stats[0], n_upd);
    atomicAdd(a.err_sum, esum);
  }
}

__global__ void batch2_advance_kernel(int32_t* epoch, int32_t* next, int32_t* next_big, int32_t n_big) {
  *epoch += 1;
  *next = n_big;
  *next_big = 0;
}
}  // namespace

namespace nomad {

#define NOMAD_DISPATCH_NV(NVVAL, ...)                  \
  switch (NVVAL) {                                     \
    case 1: { constexpr int NV = 1; __VA_ARGS__; }     \
    case 2: { constexpr int NV = 2; __VA_ARGS__; }     \
    case 4: { constexpr int NV = 4; __VA_ARGS__; }     \
    default: return cudaErrorInvalidValue;             \
  }

static int nv_of(const DevFactors& f) { return f.nvec <= 32 ? 1 : (f.nvec <= 64 ? 2 : 4); }

cudaError_t launch_async(const AsyncArgs& a, cudaStream_t s) {
  const int nv = nv_of(a.f);
  if (a.f.bf16) {
    if (a.exact) { NOMAD_DISPATCH_NV(nv, return (launch_async_t<__nv_bfloat16, NV, true, kPF>(a, s))); }
    NOMAD_DISPATCH_NV(nv, return (launch_async_t<__nv_bfloat16, NV, false, kPF>(a, s)));
  }
  if (a.exact) { NOMAD_DISPATCH_NV(nv, return (launch_async_t<float, NV, true, kPF>(a, s))); }
  NOMAD_DISPATCH_NV(nv, return (launch_async_t<float, NV, false, kPF>(a, s)));
}

cudaError_t async_occupancy(int bf16, int nv, int exact, int warps_per_block, int kpad,
                            int* bps) {
  if (bf16) {
    if (exact) { NOMAD_DISPATCH_NV(nv, return (occ_t<__nv_bfloat16, NV, true, kPF>(warps_per_block, kpad, bps))); }
    NOMAD_DISPATCH_NV(nv, return (occ_t<__nv_bfloat16, NV, false, kPF>(warps_per_block, kpad, bps)));
  }
  if (exact) { NOMAD_DISPATCH_NV(nv, return (occ_t<float, NV, true, kPF>(warps_per_block, kpad, bps))); }
  NOMAD_DISPATCH_NV(nv, return (occ_t<float, NV, false, kPF>(warps_per_block, kpad, bps)));
}

cudaError_t launch_replay(const ReplayArgs& a, cudaStream_t s) {
  const int nv = nv_of(a.f);
  const size_t smem = static_cast<size_t>(a.f.kpad) * sizeof(float);
  if (a.f.bf16) {
    NOMAD_DISPATCH_NV(nv, nomad_replay_kernel<__nv_bfloat16, NV><<<1, 32, smem, s>>>(a); return cudaGetLastError());
  }
  NOMAD_DISPATCH_NV(nv, nomad_replay_kernel<float, NV><<<1, 32, smem, s>>>(a); return cudaGetLastError());
}

cudaError_t launch_dsgd_stratum(const DsgdArgs& a, int stratum, cudaStream_t s) {
  const int nv = nv_of(a.f);
  const int wpb = 4;
  const int grid = (a.innerB + wpb - 1) / wpb;
  const size_t smem = a.exact ? static_cast<size_t>(wpb) * a.f.kpad * sizeof(float) : 0;
  if (a.f.bf16) {
    if (a.exact) { NOMAD_DISPATCH_NV(nv, nomad_dsgd_kernel<__nv_bfloat16, NV, true><<<grid, wpb * 32, smem, s>>>(a, stratum); return cudaGetLastError()); }
    NOMAD_DISPATCH_NV(nv, nomad_dsgd_kernel<__nv_bfloat16, NV, false><<<grid, wpb * 32, smem, s>>>(a, stratum); return cudaGetLastError());
  }
  if (a.exact) { NOMAD_DISPATCH_NV(nv, nomad_dsgd_kernel<float, NV, true><<<grid, wpb * 32, smem, s>>>(a, stratum); return cudaGetLastError()); }
  NOMAD_DISPATCH_NV(nv, nomad_dsgd_kernel<float, NV, false><<<grid, wpb * 32, smem, s>>>(a, stratum); return cudaGetLastError());
}


template <typename Store, bool EXACT>
static cudaError_t batch_epoch_t(const BatchArgs& a, int grid, cudaStream_t s) {
  const size_t smem = EXACT ? static_cast<size_t>(kBatchThreads / 32) * 128 * sizeof(float) : 0;
  nomad_batch_kernel<Store, EXACT><<<grid, kBatchThreads, smem, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  batch_advance_kernel<<<1, 1, 0, s>>>(a.epoch, a.next);
  return cudaGetLastError();
}

cudaError_t launch_batch_epoch(const BatchArgs& a, int grid, cudaStream_t s) {
  if (a.bf16) return a.exact ? batch_epoch_t<__nv_bfloat16, true>(a, grid, s) : batch_epoch_t<__nv_bfloat16, false>(a, grid, s);
  return a.exact ? batch_epoch_t<float, true>(a, grid, s) : batch_epoch_t<float, false>(a, grid, s);
}

cudaError_t batch_occupancy(int bf16, int exact, int* bps) {
  const size_t smem = exact ? static_cast<size_t>(kBatchThreads / 32) * 128 * sizeof(float) : 0;
  if (bf16)
    return exact ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch_kernel<__nv_bfloat16, true>, kBatchThreads, smem)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch_kernel<__nv_bfloat16, false>, kBatchThreads, smem);
  return exact ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch_kernel<float, true>, kBatchThreads, smem)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch_kernel<float, false>, kBatchThreads, smem);
}

cudaError_t launch_batch_sse(const BatchArgs& a, int grid, cudaStream_t s) {
  if (a.bf16)
    batch_sse_kernel<__nv_bfloat16><<<grid, kBatchThreads, 0, s>>>(a);
  else
    batch_sse_kernel<float><<<grid, kBatchThreads, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename Store>
static cudaError_t batch_epoch2_t(const BatchArgs& a, int grid, cudaStream_t s) {
  if (a.blocks_per_sm == 4)
    nomad_batch2_kernel<Store, 4><<<grid, kBatchWorkers * 32, 0, s>>>(a);
  else
    nomad_batch2_kernel<Store, 1><<<grid, kBatchWorkers * 32, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  batch2_advance_kernel<<<1, 1, 0, s>>>(a.epoch, a.next, a.next_big, a.n_big);
  return cudaGetLastError();
}

cudaError_t launch_batch_epoch2(const BatchArgs& a, int grid, cudaStream_t s) {
  return a.bf16 ? batch_epoch2_t<__nv_bfloat16>(a, grid, s) : batch_epoch2_t<float>(a, grid, s);
}

cudaError_t batch2_occupancy(int bf16, int blocks_per_sm, int* bps) {
  constexpr int T = kBatchWorkers * 32;
  if (blocks_per_sm == 4)
    return bf16 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch2_kernel<__nv_bfloat16, 4>, T, 0)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch2_kernel<float, 4>, T, 0);
  return bf16 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch2_kernel<__nv_bfloat16, 1>, T, 0)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, nomad_batch2_kernel<float, 1>, T, 0);
}
}  // namespace nomad
