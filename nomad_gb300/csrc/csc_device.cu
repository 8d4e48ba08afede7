// csc_device.cu -- the CSC of a row-major rating set built on the device, for context
// set-up: the entries are copied in as they are (row counts, column indices, values),
// sorted by column with a stable radix sort -- rows stay ascending inside a column, as
// the host build (host_layout.cpp: build_csc) and the reference's read_data leave them
// (Code/nomad/nb_data.cpp:131-169) -- and left in place for the kernels.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>

#include "common.h"
#include "launch.h"
#include "trace.h"

namespace {

// Row counts as int64, with a zero after the last row (its exclusive sum is row_ptr).
__global__ void counts64_kernel(const int32_t* rc, int32_t m, int64_t* out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i <= m) out[i] = i < m ? rc[i] : 0;
}

// The first entry whose column lies outside [0, n).
__global__ void check_cols_kernel(const uint32_t* cols, int64_t nnz, int32_t n, unsigned long long* bad) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < nnz && cols[i] >= static_cast<uint32_t>(n)) atomicMin(bad, static_cast<unsigned long long>(i));
}

// One warp per row: every entry of row r becomes {r, value as fp32}.
__global__ void expand_rows_kernel(const int64_t* row_ptr, int32_t m, const double* v64, const float* v32,
                                   int2* pairs) {
  const int64_t r = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= m) return;
  const int64_t b = row_ptr[r], e = row_ptr[r + 1];
  for (int64_t i = b + lane; i < e; i += 32) {
    const float v = v64 ? static_cast<float>(v64[i]) : v32[i];
    pairs[i] = make_int2(static_cast<int32_t>(r), __float_as_int(v));
  }
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

// Two pinned staging buffers for uploads from pageable memory, kept for the life of the
// process and used under a lock.
constexpr size_t kStageBytes = size_t{32} << 20;
std::mutex g_stage_mu;
char* g_stage[2] = {nullptr, nullptr};

}  // namespace

namespace nomad {

cudaError_t upload_staged(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return cudaSuccess;
  std::lock_guard<std::mutex> lock(g_stage_mu);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; ++i)
    if (!g_stage[i]) e = cudaHostAlloc(reinterpret_cast<void**>(&g_stage[i]), kStageBytes, cudaHostAllocPortable);
  cudaEvent_t done[2] = {nullptr, nullptr};
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
  const int threads = host_threads();
  bool used[2] = {false, false};
  for (size_t off = 0, k = 0; off < bytes && e == cudaSuccess; off += kStageBytes, k ^= 1) {
    const size_t n = std::min(kStageBytes, bytes - off);
    if (used[k]) e = cudaEventSynchronize(done[k]);  // the copy out of this buffer is done
    if (e != cudaSuccess) break;
    const char* from = static_cast<const char*>(src) + off;
    char* to = g_stage[k];
    const int64_t pieces = static_cast<int64_t>((n + (size_t{1} << 20) - 1) >> 20);
    parallel_chunks(pieces, threads, [&](int, int64_t lo, int64_t hi) {
      const size_t a = static_cast<size_t>(lo) << 20, b = std::min(n, static_cast<size_t>(hi) << 20);
      std::memcpy(to + a, from + a, b - a);
    });
    e = cudaMemcpyAsync(static_cast<char*>(dst) + off, to, n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(done[k], s);
    used[k] = true;
  }
  // the buffers are reused by the next upload: its copies into them wait for these
  for (int i = 0; i < 2; ++i)
    if (done[i]) {
      if (used[i] && e == cudaSuccess) e = cudaEventSynchronize(done[i]);
      cudaEventDestroy(done[i]);
    }
  return e;
}

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
  const size_t vbytes = static_cast<size_t>(nnz) * (v64 ? sizeof(double) : sizeof(float));
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
  if (e == cudaSuccess)
    e = upload_staged(vals, v64 ? static_cast<const void*>(v64) : static_cast<const void*>(v32), vbytes, s);
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
        row_ptr, m, v64 ? static_cast<const double*>(vals) : nullptr, v64 ? nullptr : static_cast<const float*>(vals),
        pairs_in);
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

}  // namespace nomad
