// layout_device.cu -- the visit lists of the asynchronous modes built on the device from
// the device CSC, for context set-up: the same segments and the same seeded routes as the
// host build (host_layout.cpp: build_async_layout), so the layout is equal bit for bit.
//   count:  the worker of every row; a flag on each rating that starts a visit (the first
//           of its column, or the first whose row leaves the previous owner's rows); the
//           visit index of every rating by an exclusive scan of the flags;
//   fill:   every visit {start, len, owner} in column order; each column's visit offset;
//           then one warp per column puts its visits in route order.
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <climits>

#include "launch.h"
#include "trace.h"

namespace {

// SplitMix64 and stream_key of the host build (common.h), in device code.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t stream_key64(uint64_t seed, uint64_t tag, uint64_t id) {
  return mix64(seed ^ mix64(tag * 0x632BE59BD9B4E019ULL + id));
}

__global__ void row_worker_kernel(const int32_t* row_start, int32_t P, int32_t m, int32_t* row_worker) {
  const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= m) return;
  // the last worker w with row_start[w] <= r
  int32_t lo = 0, hi = P;  // row_start[0] = 0 <= r < row_start[P] = m
  while (hi - lo > 1) {
    const int32_t mid = (lo + hi) >> 1;
    if (row_start[mid] <= r) lo = mid;
    else hi = mid;
  }
  row_worker[r] = lo;
}

__device__ __forceinline__ bool is_priority(const int64_t* col_ptr, int64_t j, int64_t priority_min) {
  return priority_min > 0 && col_ptr[j + 1] - col_ptr[j] >= priority_min;
}

// One block per column: flag[o] = 1 where rating o starts a visit.
__global__ void visit_flags_kernel(const int2* ratings, const int64_t* col_ptr, const int32_t* row_worker,
                                   int32_t group, int64_t priority_min, int32_t* flags) {
  const int64_t j = blockIdx.x;
  const int64_t b = col_ptr[j], e = col_ptr[j + 1];
  const int32_t div = is_priority(col_ptr, j, priority_min) ? group : 1;
  for (int64_t o = b + threadIdx.x; o < e; o += blockDim.x) {
    const int32_t own = row_worker[ratings[o].x] / div;
    flags[o] = (o == b || row_worker[ratings[o - 1].x] / div != own) ? 1 : 0;
  }
}

// One block per column: the visits in column order, {start lo, start hi, 0, owner}.
__global__ void visit_starts_kernel(const int2* ratings, const int64_t* col_ptr, const int32_t* row_worker,
                                    const int32_t* seg_id, int32_t group, int64_t priority_min, int4* segs) {
  const int64_t j = blockIdx.x;
  const int64_t b = col_ptr[j], e = col_ptr[j + 1];
  const int32_t div = is_priority(col_ptr, j, priority_min) ? group : 1;
  for (int64_t o = b + threadIdx.x; o < e; o += blockDim.x) {
    const int32_t own = row_worker[ratings[o].x] / div;
    if (o == b || row_worker[ratings[o - 1].x] / div != own)
      segs[seg_id[o]] = make_int4(static_cast<int32_t>(static_cast<uint64_t>(o) & 0xffffffffu),
                                  static_cast<int32_t>(o >> 32), 0, own);
  }
}

// A visit ends where the next begins (the next non-empty column starts where this one
// ends); the longest visit.
__global__ void visit_lens_kernel(int4* segs, int64_t nseg, int64_t nnz, int* max_len) {
  const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  auto start = [&](int64_t i) {
    return static_cast<int64_t>(static_cast<uint32_t>(segs[i].x)) | (static_cast<int64_t>(segs[i].y) << 32);
  };
  const int64_t end = s + 1 < nseg ? start(s + 1) : nnz;
  const int len = static_cast<int>(end - start(s));
  segs[s].z = len;
  atomicMax(max_len, len);
}

// Each column's first visit in route order (zeros for an empty column).
__global__ void firsts_kernel(const int4* segs, const int64_t* vl_ptr, int32_t n, int4* firsts) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j < n) firsts[j] = vl_ptr[j + 1] > vl_ptr[j] ? segs[vl_ptr[j]] : make_int4(0, 0, 0, 0);
}

__global__ void vl_ptr_kernel(const int64_t* col_ptr, const int32_t* seg_id, int32_t n, int64_t* vl_ptr) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j <= n) vl_ptr[j] = seg_id[col_ptr[j]];
}

// A column's visits (in column order in `s`) into route order in `d`, as the host build
// orders them.  Hierarchical routes: runs of one group's visits ordered by the group key,
// inside a run by the worker key, both as (key, index) pairs.  Otherwise a Fisher-Yates
// shuffle by the column's stream.
constexpr int kMaxGroup = 32;

// The runs sorted by insertion in `key`/`idx` (scratch at the column's visit offset), a
// run's visits in registers (at most kMaxGroup): one thread.
__device__ void group_route_serial(const int4* s, int4* d, int64_t k, int32_t group, uint64_t kb, uint64_t kw,
                                   uint64_t* key, int32_t* idx) {
  int64_t nr = 0;
  for (int64_t i = 0; i < k; ++i)
    if (i == 0 || s[i].w / group != s[i - 1].w / group) {
      // insertion into the sorted runs
      const uint64_t kk = mix64(kb ^ static_cast<uint64_t>(s[i].w / group));
      int64_t p = nr++;
      while (p > 0 && (key[p - 1] > kk || (key[p - 1] == kk && idx[p - 1] > i))) {
        key[p] = key[p - 1];
        idx[p] = idx[p - 1];
        --p;
      }
      key[p] = kk;
      idx[p] = static_cast<int32_t>(i);
    }
  int64_t o = 0;
  for (int64_t r = 0; r < nr; ++r) {
    const int64_t b = idx[r];
    int64_t e = b + 1;
    while (e < k && s[e].w / group == s[b].w / group) ++e;
    uint64_t ik[kMaxGroup];
    int32_t ii[kMaxGroup];
    int c = 0;
    for (int64_t i = b; i < e; ++i) {
      const uint64_t kk = mix64(kw ^ static_cast<uint64_t>(s[i].w));
      int p = c++;
      while (p > 0 && (ik[p - 1] > kk || (ik[p - 1] == kk && ii[p - 1] > i))) {
        ik[p] = ik[p - 1];
        ii[p] = ii[p - 1];
        --p;
      }
      ik[p] = kk;
      ii[p] = static_cast<int32_t>(i);
    }
    for (int x = 0; x < c; ++x) d[o++] = s[ii[x]];
  }
}

// One warp per column.  Hierarchical routes with at most kRunCap runs are ordered by the
// whole warp: run starts found by ballot; each run's rank by (group key, start) counted
// against every other run; the runs' output offsets by an exclusive sum of their lengths
// in rank order; each run's visits sorted by (worker key, index) on one lane.  The same
// order as group_route_serial, which lane 0 runs for columns with more runs, as it runs
// the Fisher-Yates shuffle.
constexpr int kRouteWarps = 4;
constexpr int kRunCap = 256;

__global__ void __launch_bounds__(kRouteWarps * 32)
    visit_routes_kernel(const int4* in, const int64_t* vl_ptr, const int64_t* col_ptr, int32_t n, int32_t group,
                        bool group_routes, int64_t priority_min, uint64_t seed, uint64_t* rkey, int32_t* ridx,
                        int4* out) {
  __shared__ uint64_t s_key[kRouteWarps][kRunCap];
  __shared__ int32_t s_start[kRouteWarps][kRunCap];
  __shared__ int32_t s_off[kRouteWarps][kRunCap + 1];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int64_t j = static_cast<int64_t>(blockIdx.x) * kRouteWarps + wib;
  if (j >= n) return;  // the whole warp
  const int64_t v0 = vl_ptr[j];
  const int64_t k = vl_ptr[j + 1] - v0;
  if (k == 0) return;
  const int4* s = in + v0;
  int4* d = out + v0;
  const bool pri = is_priority(col_ptr, j, priority_min);
  if (!(group_routes && !pri && group > 1 && k > 1)) {
    if (lane == 0) {
      for (int64_t i = 0; i < k; ++i) d[i] = s[i];
      uint64_t st = stream_key64(seed, 137, static_cast<uint64_t>(j));
      for (int64_t i = k - 1; i > 0; --i) {
        st += 0x9E3779B97F4A7C15ULL;
        const uint64_t t = __umul64hi(mix64(st), static_cast<uint64_t>(i + 1));
        const int4 a = d[i];
        d[i] = d[t];
        d[t] = a;
      }
    }
    return;
  }
  const uint64_t kb = stream_key64(seed, 149, static_cast<uint64_t>(j));
  const uint64_t kw = stream_key64(seed, 151, static_cast<uint64_t>(j));
  uint64_t* skey = s_key[wib];
  int32_t* sstart = s_start[wib];
  int32_t* soff = s_off[wib];
  // run starts, in index order
  int nr = 0;
  for (int64_t i0 = 0; i0 < k; i0 += 32) {
    const int64_t i = i0 + lane;
    bool st = false;
    int32_t g = 0;
    if (i < k) {
      g = s[i].w / group;
      st = i == 0 || s[i - 1].w / group != g;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, st);
    const int pos = nr + __popc(bal & ((1u << lane) - 1u));
    if (st && pos < kRunCap) {
      skey[pos] = mix64(kb ^ static_cast<uint64_t>(g));
      sstart[pos] = static_cast<int32_t>(i);
    }
    nr += __popc(bal);
  }
  __syncwarp();
  if (nr > kRunCap) {
    if (lane == 0) group_route_serial(s, d, k, group, kb, kw, rkey + v0, ridx + v0);
    return;
  }
  constexpr int kPer = kRunCap / 32;
  int rk[kPer];
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int r = lane + 32 * t;
    rk[t] = 0;
    if (r < nr) {
      const uint64_t kr = skey[r];
      const int32_t br = sstart[r];
      int rank = 0;
      for (int q = 0; q < nr; ++q) {
        const uint64_t kq = skey[q];
        rank += (kq < kr || (kq == kr && sstart[q] < br)) ? 1 : 0;
      }
      rk[t] = rank;
      soff[rank + 1] = (r + 1 < nr ? sstart[r + 1] : static_cast<int32_t>(k)) - br;  // the run's length
    }
  }
  __syncwarp();
  if (lane == 0) {  // offsets in rank order: exclusive sum of the lengths
    soff[0] = 0;
    for (int q = 1; q <= nr; ++q) soff[q] += soff[q - 1];
  }
  __syncwarp();
#pragma unroll
  for (int t = 0; t < kPer; ++t) {
    const int r = lane + 32 * t;
    if (r < nr) {
      const int64_t b = sstart[r];
      const int64_t e = r + 1 < nr ? sstart[r + 1] : k;
      uint64_t ik[kMaxGroup];
      int32_t ii[kMaxGroup];
      int c = 0;
      for (int64_t i = b; i < e && c < kMaxGroup; ++i) {
        const uint64_t kk = mix64(kw ^ static_cast<uint64_t>(s[i].w));
        int p = c++;
        while (p > 0 && (ik[p - 1] > kk || (ik[p - 1] == kk && ii[p - 1] > i))) {
          ik[p] = ik[p - 1];
          ii[p] = ii[p - 1];
          --p;
        }
        ik[p] = kk;
        ii[p] = static_cast<int32_t>(i);
      }
      int4* o = d + soff[rk[t]];
      for (int x = 0; x < c; ++x) o[x] = s[ii[x]];
    }
  }
}

}  // namespace

namespace nomad {

cudaError_t device_layout_count(const int2* ratings, const int64_t* col_ptr, int64_t nnz, int32_t m, int32_t n,
                                const int32_t* row_start, int32_t P, int32_t group, int64_t priority_min,
                                DeviceLayout* t, cudaStream_t s) {
  *t = DeviceLayout{};
  if (nnz <= 0 || nnz > INT_MAX || m <= 0 || n <= 0 || P <= 0 || group <= 0 || group > kMaxGroup)
    return cudaErrorInvalidValue;
  InitTrace trace;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMallocAsync(p, std::max<size_t>(bytes, 16), s);
  };
  alloc(reinterpret_cast<void**>(&t->row_start), (static_cast<size_t>(P) + 1) * 4);
  alloc(reinterpret_cast<void**>(&t->row_worker), static_cast<size_t>(m) * 4);
  alloc(reinterpret_cast<void**>(&t->flags), (static_cast<size_t>(nnz) + 1) * 4);
  alloc(reinterpret_cast<void**>(&t->seg_id), (static_cast<size_t>(nnz) + 1) * 4);
  size_t tmp_bytes = 0;
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, t->flags, t->seg_id, static_cast<int>(nnz + 1), s);
  alloc(&t->tmp, tmp_bytes);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(t->row_start, row_start, (static_cast<size_t>(P) + 1) * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->flags + nnz, 0, 4, s);
  if (trace.on && e == cudaSuccess) trace.mark("  layout: allocations", s);
  if (e == cudaSuccess) {
    row_worker_kernel<<<static_cast<unsigned>((m + 255) / 256), 256, 0, s>>>(t->row_start, P, m, t->row_worker);
    visit_flags_kernel<<<static_cast<unsigned>(n), 256, 0, s>>>(ratings, col_ptr, t->row_worker, group, priority_min,
                                                               t->flags);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(t->tmp, tmp_bytes, t->flags, t->seg_id, static_cast<int>(nnz + 1), s);
  int32_t total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, t->seg_id + nnz, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (trace.on && e == cudaSuccess) trace.mark("  layout: visit flags and scan", s);
  t->nseg = total;
  if (e != cudaSuccess) device_layout_release(t, s);
  return e;
}

cudaError_t device_layout_fill(const int2* ratings, const int64_t* col_ptr, int64_t nnz, int32_t n, int32_t group,
                               bool group_routes, int64_t priority_min, uint64_t seed, DeviceLayout* t, int4* segs,
                               int64_t* vl_ptr, int64_t* vl_ptr_host, int4* firsts_host, int32_t* max_seg,
                               cudaStream_t s) {
  InitTrace trace;
  cudaError_t e = cudaSuccess;
  int4 *in = nullptr, *firsts = nullptr;
  uint64_t* rkey = nullptr;
  int32_t* ridx = nullptr;
  int* mx = nullptr;
  const size_t ns = static_cast<size_t>(std::max<int64_t>(t->nseg, 1));
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMallocAsync(p, std::max<size_t>(bytes, 16), s);
  };
  alloc(reinterpret_cast<void**>(&in), ns * 16);
  alloc(reinterpret_cast<void**>(&rkey), ns * 8);
  alloc(reinterpret_cast<void**>(&ridx), ns * 4);
  alloc(reinterpret_cast<void**>(&mx), 4);
  alloc(reinterpret_cast<void**>(&firsts), static_cast<size_t>(n) * 16);
  if (e == cudaSuccess) e = cudaMemsetAsync(mx, 0, 4, s);
  if (e == cudaSuccess) {
    visit_starts_kernel<<<static_cast<unsigned>(n), 256, 0, s>>>(ratings, col_ptr, t->row_worker, t->seg_id, group,
                                                                priority_min, in);
    visit_lens_kernel<<<static_cast<unsigned>((t->nseg + 255) / 256), 256, 0, s>>>(in, t->nseg, nnz, mx);
    vl_ptr_kernel<<<static_cast<unsigned>((n + 1 + 255) / 256), 256, 0, s>>>(col_ptr, t->seg_id, n, vl_ptr);
    if (trace.on) trace.mark("  layout: allocations, visit starts and lengths", s);
    visit_routes_kernel<<<static_cast<unsigned>((n + kRouteWarps - 1) / kRouteWarps), kRouteWarps * 32, 0, s>>>(
        in, vl_ptr, col_ptr, n, group, group_routes, priority_min, seed, rkey, ridx, segs);
    e = cudaGetLastError();
  }
  if (trace.on && e == cudaSuccess) trace.mark("  layout: routes", s);
  // the visit offsets and each column's first visit in route order, for the host's
  // initial queues
  if (e == cudaSuccess) {
    firsts_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(segs, vl_ptr, n, firsts);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(vl_ptr_host, vl_ptr, (static_cast<size_t>(n) + 1) * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(firsts_host, firsts, static_cast<size_t>(n) * 16, cudaMemcpyDeviceToHost, s);
  int mxh = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&mxh, mx, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (trace.on && e == cudaSuccess) trace.mark("  layout: first visits, copies out", s);
  *max_seg = mxh;
  for (void* p : {static_cast<void*>(in), static_cast<void*>(rkey), static_cast<void*>(ridx), static_cast<void*>(mx),
                  static_cast<void*>(firsts)})
    if (p) cudaFreeAsync(p, s);
  device_layout_release(t, s);
  if (trace.on && e == cudaSuccess) trace.mark("  layout: frees", s);
  return e;
}

void device_layout_release(DeviceLayout* t, cudaStream_t s) {
  for (void* p : {static_cast<void*>(t->row_start), static_cast<void*>(t->row_worker), static_cast<void*>(t->flags),
                  static_cast<void*>(t->seg_id), t->tmp})
    if (p) cudaFreeAsync(p, s);
  *t = DeviceLayout{};
}

}  // namespace nomad
