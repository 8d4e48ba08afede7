// csc_device.cu -- the CSC of a row-major rating set built on the device, for context
// set-up: the entries are copied in as they are (row counts, column indices, values),
// sorted by column with a stable radix sort -- rows stay ascending inside a column, as
// the host build (host_layout.cpp: build_csc) and the reference's read_data leave them
// (Code/nomad/nb_data.cpp:131-169) -- and left in place for the kernels.  A batch of
// problems is sorted in one pass, keyed by (problem, column).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <climits>
#include <vector>

#include "common.h"
#include "launch.h"
#include "trace.h"

namespace {

// Row counts as int64, with a zero after the last row (its exclusive sum is row_ptr).
__global__ void counts64_kernel(const int32_t* rc, int64_t m, int64_t* out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i <= m) out[i] = i < m ? rc[i] : 0;
}

// The first entry whose column lies outside [0, n).
__global__ void check_cols_kernel(const uint32_t* cols, int64_t nnz, int32_t n, unsigned long long* bad) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < nnz && cols[i] >= static_cast<uint32_t>(n)) atomicMin(bad, static_cast<unsigned long long>(i));
}

// One warp per row: every entry of row r becomes {r, value bits}.
__global__ void expand_rows_kernel(const int64_t* row_ptr, int32_t m, const float* vals, int2* pairs) {
  const int64_t r = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= m) return;
  const int64_t b = row_ptr[r], e = row_ptr[r + 1];
  for (int64_t i = b + lane; i < e; i += 32) pairs[i] = make_int2(static_cast<int32_t>(r), __float_as_int(vals[i]));
}

// col_ptr from the sorted column keys (each column's first entry, empty columns included)
// and the smallest column holding a repeated (row, column) cell.
__global__ void col_ptr_kernel(const uint32_t* keys, const int2* pairs, int64_t nnz, int32_t n, int64_t* col_ptr,
                               int32_t* dup) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nnz) return;
  const int64_t k = keys[i];
  const int64_t kp = i > 0 ? static_cast<int64_t>(keys[i - 1]) : -1;
  for (int64_t c = kp + 1; c <= k; ++c) col_ptr[c] = i;
  if (i == nnz - 1)
    for (int64_t c = k + 1; c <= n; ++c) col_ptr[c] = nnz;
  if (i > 0 && k == kp && pairs[i].x == pairs[i - 1].x) atomicMin(dup, static_cast<int32_t>(k));
}

// The row of every rating.
__global__ void rows_kernel(const int2* ratings, int64_t nnz, int32_t* rows) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < nnz) rows[i] = ratings[i].x;
}

// The last p with at[p] <= x, for at[0] = 0 <= x < at[count] and at increasing.
__device__ __forceinline__ int32_t owner_of(const int64_t* at, int32_t count, int64_t x) {
  int32_t lo = 0, hi = count;
  while (hi - lo > 1) {
    const int32_t mid = (lo + hi) >> 1;
    if (at[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Batched sets, one warp per row of the concatenated row-major entries: row r of problem
// p gives each of its entries the key colbase[p] + column and the pair {local row, value
// bits}; the first entry with a column outside [0, n_p) goes to *bad.
__global__ void batch_expand_kernel(const int64_t* row_ptr, int64_t rows, const int64_t* row_at,
                                    const int64_t* colbase, int32_t count, const uint32_t* cols, const float* vals,
                                    uint32_t* keys, int2* pairs, unsigned long long* bad) {
  const int64_t r = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  const int32_t p = owner_of(row_at, count, r);
  const int64_t base = colbase[p];
  const uint32_t n = static_cast<uint32_t>(colbase[p + 1] - base);
  const int32_t local = static_cast<int32_t>(r - row_at[p]);
  const int64_t b = row_ptr[r], e = row_ptr[r + 1];
  for (int64_t i = b + lane; i < e; i += 32) {
    const uint32_t c = cols[i];
    if (c >= n) atomicMin(bad, static_cast<unsigned long long>(i));
    keys[i] = c < n ? static_cast<uint32_t>(base + c) : 0u;
    pairs[i] = make_int2(local, __float_as_int(vals[i]));
  }
}

// Each problem's n + 1 column pointers out of the global ones (col_ptr over all problems'
// columns): entry t of the output is column t - cpo[p] of the problem p it falls in.
__global__ void batch_col_ptr_kernel(const int64_t* gptr, const int64_t* cpo, const int64_t* colbase, int32_t count,
                                     int64_t total, int64_t* col_ptr) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int32_t p = owner_of(cpo, count, t);
  col_ptr[t] = gptr[colbase[p] + (t - cpo[p])];
}

// One block per problem: its columns with at least one rating.
__global__ void batch_active_kernel(const int64_t* gptr, const int64_t* colbase, int32_t* act) {
  const int64_t b = colbase[blockIdx.x], e = colbase[blockIdx.x + 1];
  int c = 0;
  for (int64_t j0 = b; j0 < e; j0 += blockDim.x) {
    const int64_t j = j0 + threadIdx.x;
    c += __syncthreads_count(j < e && gptr[j + 1] > gptr[j]);
  }
  if (threadIdx.x == 0) act[blockIdx.x] = c;
}

// One block per large problem, a thread per column: the R + 1 visit bounds of the column
// (rows ascend inside it, so each bound is a lower bound from the previous one).
__global__ void batch_segs_kernel(const int2* ratings, const int64_t* col_ptr, const nomad::BatchSegIn* big,
                                  const int32_t* rs, int32_t R, int64_t* seg) {
  const nomad::BatchSegIn g = big[blockIdx.x];
  for (int32_t j = threadIdx.x; j < g.n; j += blockDim.x) {
    int64_t o = col_ptr[g.col_off + j];
    const int64_t e = col_ptr[g.col_off + j + 1];
    int64_t* out = seg + g.seg_off + static_cast<int64_t>(j) * (R + 1);
    for (int32_t w = 0; w <= R; ++w) {
      const int32_t bound = rs[g.rs_off + w];
      int64_t hi = e;
      while (o < hi) {
        const int64_t mid = o + ((hi - o) >> 1);
        if (ratings[mid].x < bound) o = mid + 1;
        else hi = mid;
      }
      out[w] = o;
    }
  }
}

}  // namespace

namespace nomad {

cudaError_t device_csc_rows(const int2* ratings, int64_t nnz, int32_t* host_rows, cudaStream_t s) {
  if (nnz <= 0 || nnz > INT_MAX) return cudaErrorInvalidValue;
  int32_t* rows = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&rows), static_cast<size_t>(nnz) * 4, s);
  if (e == cudaSuccess) {
    rows_kernel<<<static_cast<unsigned>((nnz + 255) / 256), 256, 0, s>>>(ratings, nnz, rows);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(host_rows, rows, static_cast<size_t>(nnz) * 4, cudaMemcpyDeviceToHost, s);
  if (rows) cudaFreeAsync(rows, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}


cudaError_t device_csc(int64_t nnz, int32_t m, int32_t n, const int32_t* row_counts, const int32_t* cols,
                       const double* v64, const float* v32, int2* ratings, int64_t* col_ptr, int64_t* bad_col,
                       int32_t* dup_col, int64_t* h2d_bytes, cudaStream_t s) {
  *dup_col = -1;
  *bad_col = -1;
  InitTrace trace;
  if (nnz <= 0 || nnz > INT_MAX || m <= 0 || n <= 0) return cudaErrorInvalidValue;
  const int items = static_cast<int>(nnz);
  int end_bit = 1;
  while (end_bit < 32 && (static_cast<uint32_t>(n - 1) >> end_bit) != 0) ++end_bit;
  uint32_t *keys_in = nullptr, *keys_out = nullptr;
  int2* pairs_in = nullptr;
  int32_t* rc = nullptr;
  int32_t* dup = nullptr;
  unsigned long long* bad = nullptr;
  int64_t *cnt = nullptr, *row_ptr = nullptr;
  void* vals = nullptr;
  void* tmp = nullptr;
  const size_t vbytes = static_cast<size_t>(nnz) * sizeof(float);  // fp64 values narrowed as they are staged
  size_t tmp_scan = 0, tmp_sort = 0;
  cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, tmp_scan, cnt, row_ptr, m + 1, s);
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, keys_in, keys_out, pairs_in, ratings, items, 0, end_bit, s);
  const size_t tmp_bytes = std::max(tmp_scan, tmp_sort);
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMallocAsync(p, std::max<size_t>(bytes, 16), s);
  };
  alloc(reinterpret_cast<void**>(&keys_in), static_cast<size_t>(nnz) * 4);
  alloc(reinterpret_cast<void**>(&keys_out), static_cast<size_t>(nnz) * 4);
  alloc(reinterpret_cast<void**>(&pairs_in), static_cast<size_t>(nnz) * 8);
  alloc(reinterpret_cast<void**>(&rc), static_cast<size_t>(m) * 4);
  alloc(reinterpret_cast<void**>(&cnt), (static_cast<size_t>(m) + 1) * 8);
  alloc(reinterpret_cast<void**>(&row_ptr), (static_cast<size_t>(m) + 1) * 8);
  alloc(reinterpret_cast<void**>(&dup), 4);
  alloc(reinterpret_cast<void**>(&bad), 8);
  alloc(&vals, vbytes);
  alloc(&tmp, tmp_bytes);
  if (trace.on && e == cudaSuccess) trace.mark("  csc: allocations", s);
  // the caller's arrays are pageable memory of any mapping: staged through pinned buffers
  if (e == cudaSuccess) e = upload_staged(keys_in, cols, static_cast<size_t>(nnz) * 4, s);
  if (e == cudaSuccess) e = upload_staged(rc, row_counts, static_cast<size_t>(m) * 4, s);
  if (e == cudaSuccess) {
    const size_t n_vals = static_cast<size_t>(nnz);
    e = v64 ? upload_staged_narrow(static_cast<float*>(vals), &v64, &n_vals, 1, s) : upload_staged(vals, v32, vbytes, s);
  }
  if (e == cudaSuccess) {
    *h2d_bytes += static_cast<int64_t>(nnz) * 4 + static_cast<int64_t>(m) * 4 + static_cast<int64_t>(vbytes);
    const int dup_none = INT_MAX;
    e = cudaMemcpyAsync(dup, &dup_none, 4, cudaMemcpyHostToDevice, s);
  }
  // columns in range before anything is indexed by them
  unsigned long long b = ~0ull;
  if (e == cudaSuccess) e = cudaMemcpyAsync(bad, &b, 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    check_cols_kernel<<<static_cast<unsigned>((nnz + 255) / 256), 256, 0, s>>>(keys_in, nnz, n, bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&b, bad, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && b != ~0ull) {
    *bad_col = static_cast<int64_t>(b);
    e = cudaErrorInvalidValue;
  }
  if (trace.on && e == cudaSuccess) trace.mark("  csc: copies in", s);
  if (e == cudaSuccess) {
    counts64_kernel<<<static_cast<unsigned>((m + 256) / 256), 256, 0, s>>>(rc, m, cnt);
    e = cub::DeviceScan::ExclusiveSum(tmp, tmp_scan, cnt, row_ptr, m + 1, s);
  }
  if (e == cudaSuccess) {
    const int64_t threads = static_cast<int64_t>(m) * 32;
    expand_rows_kernel<<<static_cast<unsigned>((threads + 255) / 256), 256, 0, s>>>(
        row_ptr, m, static_cast<const float*>(vals), pairs_in);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(tmp, tmp_sort, keys_in, keys_out, pairs_in, ratings, items, 0, end_bit, s);
  if (e == cudaSuccess) {
    col_ptr_kernel<<<static_cast<unsigned>((nnz + 255) / 256), 256, 0, s>>>(keys_out, ratings, nnz, n, col_ptr, dup);
    e = cudaGetLastError();
  }
  int32_t d = INT_MAX;
  if (trace.on && e == cudaSuccess) trace.mark("  csc: sort and offsets", s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&d, dup, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && d != INT_MAX) *dup_col = d;
  for (void* p : {static_cast<void*>(keys_in), static_cast<void*>(keys_out), static_cast<void*>(pairs_in),
                  static_cast<void*>(rc), static_cast<void*>(cnt), static_cast<void*>(row_ptr),
                  static_cast<void*>(dup), static_cast<void*>(bad), vals, tmp})
    if (p) cudaFreeAsync(p, s);
  if (trace.on && e == cudaSuccess) trace.mark("  csc: frees", s);
  return e;
}

cudaError_t device_batch_csc(const BatchSetIn* sets, int32_t count, bool f64, int2* ratings, int64_t* col_ptr,
                             int32_t* n_active_host, bool* faulty, int64_t* h2d_bytes, cudaStream_t s) {
  *faulty = false;
  if (count <= 0) return cudaErrorInvalidValue;
  InitTrace trace;
  // problem p's rows, columns and column pointers start at row_at[p], colbase[p], cpo[p]
  std::vector<int64_t> meta(3 * (static_cast<size_t>(count) + 1), 0);
  int64_t* row_at = meta.data();
  int64_t* colbase = row_at + count + 1;
  int64_t* cpo = colbase + count + 1;
  int64_t nnz = 0;
  int32_t max_m = 0;
  for (int32_t p = 0; p < count; ++p) {
    const BatchSetIn& q = sets[p];
    if (q.m <= 0 || q.n <= 0 || q.nnz < 0) return cudaErrorInvalidValue;
    nnz += q.nnz;
    max_m = std::max(max_m, q.m);
    row_at[p + 1] = row_at[p] + q.m;
    colbase[p + 1] = colbase[p] + q.n;
    cpo[p + 1] = cpo[p] + q.n + 1;
  }
  const int64_t rows = row_at[count], cols_total = colbase[count], ptrs = cpo[count];
  if (nnz > INT_MAX || cols_total > INT_MAX || rows >= INT_MAX) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  if (nnz == 0) {  // no ratings: every column pointer 0
    e = cudaMemsetAsync(col_ptr, 0, static_cast<size_t>(ptrs) * sizeof(int64_t), s);
    if (n_active_host) std::fill(n_active_host, n_active_host + count, 0);
    return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
  }
  const int items = static_cast<int>(nnz);
  const int32_t n_keys = static_cast<int32_t>(cols_total);
  int end_bit = 1;
  while (end_bit < 32 && (static_cast<uint32_t>(n_keys - 1) >> end_bit) != 0) ++end_bit;
  uint32_t *keys_in = nullptr, *keys_out = nullptr;
  int2* pairs_in = nullptr;
  int32_t *rc = nullptr, *dup = nullptr, *act = nullptr;
  unsigned long long* bad = nullptr;
  int64_t *cnt = nullptr, *row_ptr = nullptr, *gptr = nullptr, *meta_d = nullptr;
  void* vals = nullptr;
  void* tmp = nullptr;
  const size_t vsize = sizeof(float);  // fp64 values narrowed as they are staged
  size_t tmp_scan = 0, tmp_sort = 0;
  e = cub::DeviceScan::ExclusiveSum(nullptr, tmp_scan, cnt, row_ptr, static_cast<int>(rows + 1), s);
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, keys_in, keys_out, pairs_in, ratings, items, 0, end_bit, s);
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMallocAsync(p, std::max<size_t>(bytes, 16), s);
  };
  alloc(reinterpret_cast<void**>(&keys_in), static_cast<size_t>(nnz) * 4);
  alloc(reinterpret_cast<void**>(&keys_out), static_cast<size_t>(nnz) * 4);
  alloc(reinterpret_cast<void**>(&pairs_in), static_cast<size_t>(nnz) * 8);
  alloc(reinterpret_cast<void**>(&rc), static_cast<size_t>(rows) * 4);
  alloc(reinterpret_cast<void**>(&cnt), (static_cast<size_t>(rows) + 1) * 8);
  alloc(reinterpret_cast<void**>(&row_ptr), (static_cast<size_t>(rows) + 1) * 8);
  alloc(reinterpret_cast<void**>(&gptr), (static_cast<size_t>(cols_total) + 1) * 8);
  alloc(reinterpret_cast<void**>(&meta_d), meta.size() * 8);
  alloc(reinterpret_cast<void**>(&act), static_cast<size_t>(count) * 4);
  alloc(reinterpret_cast<void**>(&dup), 4);
  alloc(reinterpret_cast<void**>(&bad), 8);
  alloc(&vals, static_cast<size_t>(nnz) * vsize);
  alloc(&tmp, std::max(tmp_scan, tmp_sort));
  if (trace.on && e == cudaSuccess) trace.mark("  batch csc: allocations", s);
  // every problem's arrays, concatenated (a set without ratings may come without arrays:
  // its row counts are zeros)
  std::vector<int32_t> zeros;
  std::vector<const void*> src_c(count), src_r(count), src_v(count);
  std::vector<size_t> len_c(count), len_r(count), len_v(count);
  for (int32_t p = 0; p < count; ++p) {
    const BatchSetIn& q = sets[p];
    if (!q.row_counts && zeros.empty()) zeros.assign(static_cast<size_t>(max_m), 0);
    src_c[p] = q.cols;
    src_r[p] = q.row_counts ? static_cast<const void*>(q.row_counts) : static_cast<const void*>(zeros.data());
    src_v[p] = q.vals;
    len_c[p] = static_cast<size_t>(q.nnz) * 4;
    len_r[p] = static_cast<size_t>(q.m) * 4;
    len_v[p] = static_cast<size_t>(q.nnz) * (f64 ? 1 : vsize);  // values (fp64) or bytes (fp32)
  }
  if (e == cudaSuccess) e = upload_staged_many(keys_in, src_c.data(), len_c.data(), count, s);
  if (e == cudaSuccess) e = upload_staged_many(rc, src_r.data(), len_r.data(), count, s);
  if (e == cudaSuccess)
    e = f64 ? upload_staged_narrow(static_cast<float*>(vals), reinterpret_cast<const double* const*>(src_v.data()),
                                   len_v.data(), count, s)
            : upload_staged_many(vals, src_v.data(), len_v.data(), count, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(meta_d, meta.data(), meta.size() * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    *h2d_bytes += static_cast<int64_t>(nnz) * (4 + static_cast<int64_t>(vsize)) + rows * 4 +
                  static_cast<int64_t>(meta.size()) * 8;
    const int dup_none = INT_MAX;
    e = cudaMemcpyAsync(dup, &dup_none, 4, cudaMemcpyHostToDevice, s);
  }
  unsigned long long b = ~0ull;
  if (e == cudaSuccess) e = cudaMemcpyAsync(bad, &b, 8, cudaMemcpyHostToDevice, s);
  if (trace.on && e == cudaSuccess) trace.mark("  batch csc: copies in", s);
  const int64_t* row_at_d = meta_d;
  const int64_t* colbase_d = meta_d + count + 1;
  const int64_t* cpo_d = colbase_d + count + 1;
  if (e == cudaSuccess) {
    counts64_kernel<<<static_cast<unsigned>((rows + 256) / 256), 256, 0, s>>>(rc, rows, cnt);
    e = cub::DeviceScan::ExclusiveSum(tmp, tmp_scan, cnt, row_ptr, static_cast<int>(rows + 1), s);
  }
  if (e == cudaSuccess) {
    batch_expand_kernel<<<static_cast<unsigned>((rows * 32 + 255) / 256), 256, 0, s>>>(
        row_ptr, rows, row_at_d, colbase_d, count, keys_in, static_cast<const float*>(vals), keys_in, pairs_in, bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&b, bad, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && b != ~0ull) *faulty = true;  // a column out of range: nothing is sorted
  if (e == cudaSuccess && !*faulty)
    e = cub::DeviceRadixSort::SortPairs(tmp, tmp_sort, keys_in, keys_out, pairs_in, ratings, items, 0, end_bit, s);
  if (e == cudaSuccess && !*faulty) {
    col_ptr_kernel<<<static_cast<unsigned>((nnz + 255) / 256), 256, 0, s>>>(keys_out, ratings, nnz, n_keys, gptr,
                                                                            dup);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && !*faulty) {
    batch_col_ptr_kernel<<<static_cast<unsigned>((ptrs + 255) / 256), 256, 0, s>>>(gptr, cpo_d, colbase_d, count,
                                                                                   ptrs, col_ptr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && !*faulty && n_active_host) {
    batch_active_kernel<<<static_cast<unsigned>(count), 256, 0, s>>>(gptr, colbase_d, act);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(n_active_host, act, static_cast<size_t>(count) * 4, cudaMemcpyDeviceToHost, s);
  }
  int32_t d = INT_MAX;
  if (e == cudaSuccess && !*faulty) e = cudaMemcpyAsync(&d, dup, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && d != INT_MAX) *faulty = true;
  if (trace.on && e == cudaSuccess) trace.mark("  batch csc: sort and offsets", s);
  for (void* p : {static_cast<void*>(keys_in), static_cast<void*>(keys_out), static_cast<void*>(pairs_in),
                  static_cast<void*>(rc), static_cast<void*>(cnt), static_cast<void*>(row_ptr),
                  static_cast<void*>(gptr), static_cast<void*>(meta_d), static_cast<void*>(act),
                  static_cast<void*>(dup), static_cast<void*>(bad), vals, tmp})
    if (p) cudaFreeAsync(p, s);
  return e;
}

cudaError_t device_batch_segs(const int2* ratings, const int64_t* col_ptr, const BatchSegIn* big_host, int32_t n_big,
                              const int32_t* rs, int32_t R, int64_t* seg, cudaStream_t s) {
  if (n_big <= 0) return cudaSuccess;
  BatchSegIn* big = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&big), static_cast<size_t>(n_big) * sizeof(BatchSegIn), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(big, big_host, static_cast<size_t>(n_big) * sizeof(BatchSegIn), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    batch_segs_kernel<<<static_cast<unsigned>(n_big), 256, 0, s>>>(ratings, col_ptr, big, rs, R, seg);
    e = cudaGetLastError();
  }
  if (big) cudaFreeAsync(big, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace nomad
