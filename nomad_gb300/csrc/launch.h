// launch.h -- host-side launch wrappers of the sm_103a kernels (kernels_*.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "stage.h"

namespace nomad {

// Factor storage on the device: rows padded to `kpad` elements (a multiple of the
// 16-byte vector: 4 fp32 or 8 bf16), padding kept at zero.
struct DevFactors {
  void* W = nullptr;  // [m * kpad]
  void* H = nullptr;  // [n * kpad]
  int32_t m = 0, n = 0, dim = 0, kpad = 0;
  int32_t nvec = 0;       // kpad / elements-per-vector = lanes that hold a row
  int32_t red_width = 0;  // power of two >= min(nvec, 32): shuffle-reduction width
  int32_t bf16 = 0;       // storage: 0 fp32, 1 bf16
};

struct AsyncArgs {
  DevFactors f;
  const int2* ratings = nullptr;    // CSC-by-column {row, float bits}
  const int4* segs = nullptr;       // {start lo, start hi, len, worker}
  const int64_t* vl_ptr = nullptr;  // [n+1] visit list of each token
  int32_t* tok_pos = nullptr;       // [n]
  int32_t* tok_epoch = nullptr;     // [n]
  int4* tok_desc = nullptr;         // [n] next visit {start lo, start hi, len, pos | heavy bit}
  const float* steps = nullptr;     // [n_steps] step size per pass count
  int32_t n_steps = 0;
  int32_t* qnext = nullptr;         // [n + P]
  int32_t* qtail = nullptr;         // [P]
  int32_t* ctrl = nullptr;          // [0] retired tokens, [1] device status
  unsigned long long* progress = nullptr;  // [1] hop counter (batched)
  unsigned long long* stats = nullptr;     // [0] updates [1] hops [2] empty polls
  double* err_sum = nullptr;               // [1] online squared error
  int32_t P = 0, n_active = 0, target_epoch = 0;
  float lambda = 0.f;
  uint32_t seed32 = 0;
  int64_t budget_ns = 0;
  int32_t exact = 0;
  int32_t warps_per_block = 0, grid = 0;  // pipelined kernel: compute warps (workers) per block
  int32_t heavy_min = 14;  // visits with at least this many ratings take the blocked path
  unsigned long long* finish_ns = nullptr;  // [n] globaltimer when each token retired
  // ring queues of the pipelined kernel: worker w's ring is ring_lo[w*(mask_lo+1)..];
  // thread block b's ring of priority tokens is ring_hi[b*(mask_hi+1)..]; queue ids
  // 0..P-1 are worker rings, P+b block rings
  unsigned long long* ring_lo = nullptr;
  unsigned long long* ring_hi = nullptr;
  unsigned mask_lo = 0, mask_hi = 0;
  unsigned* tails = nullptr;  // [2P] producer counters
  unsigned* heads = nullptr;  // [2P] consumer counters
  int4* mailbox = nullptr;    // [4n] next visit of each token (four int4)
  const int4* segx = nullptr; // [3 * segments] each visit followed by its first four ratings
  int32_t cta_heavy = 0;      // priority tokens visit thread blocks, whose warps process them together
  int32_t debug_flags = 0;    // test hooks (nomad_gpu_params.debug_flags)
};

struct ReplayArgs {
  DevFactors f;
  const int2* ratings = nullptr;
  const int64_t* col_ptr = nullptr;
  const float* steps = nullptr;
  int32_t first_epoch = 0, n_epochs = 0;
  float lambda = 0.f;
  uint32_t seed32 = 0;
  double* err_sum = nullptr;
};

struct DsgdArgs {
  DevFactors f;
  const int4* rates = nullptr;       // {row, col, float bits, 0} grouped by block
  const int64_t* blk_ptr = nullptr;  // [innerB * col_blocks + 1]
  const int32_t* sched = nullptr;    // [strata * innerB]: bj of row block bi in stratum i
  int32_t innerB = 0;
  int32_t col_blocks = 0;            // innerB (DSGD) or 2 * innerB (DSGD++)
  float step = 0.f, lambda = 0.f;
  int32_t iter = 0;
  uint32_t seed32 = 0;
  int32_t exact = 0;
};

// Batched problems: one entry per problem of the concatenated storage.
struct BatchProblem {
  int64_t w_off, h_off;           // element offsets of the problem's W and H rows
  int64_t col_off, test_col_off;  // offsets of its n + 1 column pointers (train, test)
  int32_t m, n, dim, kpad;
  int32_t nvec, red_width;
  int32_t rs_off;                 // large problems: offset of the warps' row-block bounds
  int32_t n_active;               // columns with training ratings
  int64_t seg_off;                // large problems: offset of the n x (R + 1) visit bounds
  int64_t pad;
};
static_assert(sizeof(BatchProblem) == 80, "batch problem entry");

// Large batched problems run on every warp of a block as NOMAD workers; the row blocks
// and the column visit bounds are laid out for this many warps.
constexpr int kBatchWorkers = 16;
constexpr int kBatchRing = 8192;  // ring capacity: a large problem has at most 5,000 + columns

// A part of one problem's train (set 0) or test (set 1) ratings for the evaluation:
// absolute offsets [start, end) into that set's concatenated ratings.
struct SsePart {
  int64_t start, end;
  int32_t prob, set;
};

struct BatchArgs {
  void* W = nullptr;  // every problem's rows, concatenated
  void* H = nullptr;
  const BatchProblem* problems = nullptr;
  const int32_t* order = nullptr;  // problems by decreasing rating count (the work queue)
  int32_t count = 0;
  const int2* ratings = nullptr;    // train ratings, CSC per problem, concatenated
  const int64_t* col_ptr = nullptr; // absolute offsets into `ratings`
  const int2* test = nullptr;
  const int64_t* test_col_ptr = nullptr;
  const float* steps = nullptr;     // [n_steps] step size per pass count
  int32_t n_steps = 0;
  int32_t* next = nullptr;          // [1] work-queue head
  int32_t* epoch = nullptr;         // [1] pass count of the next launch
  float lambda = 0.f;
  uint32_t seed32 = 0;
  int32_t bf16 = 0, exact = 0;
  unsigned long long* stats = nullptr;  // [0] updates
  double* err_sum = nullptr;            // [1] online squared error
  const SsePart* parts = nullptr;       // the evaluation's parts, problems and sets in order
  int32_t n_parts = 0;
  double* part_sse = nullptr;           // [n_parts] FP64 squared-error sum of each part
  // large problems: the first n_big entries of `order`, taken a block at a time
  int32_t n_big = 0;
  int32_t* next_big = nullptr;          // [1] large-problem queue head
  const int32_t* row_start = nullptr;   // per large problem: kBatchWorkers + 1 row bounds
  const int64_t* seg = nullptr;         // per large problem: n x (kBatchWorkers + 1) rating offsets
  unsigned long long* rings = nullptr;  // [grid x kBatchWorkers x kBatchRing] token rings
  unsigned* ring_ctr = nullptr;         // [grid x kBatchWorkers] ring counters (persist)
  int32_t* ctrl = nullptr;              // [2]: [1] device status (a large problem's wait ran out)
  int64_t budget_ns = 0;                // bound of a worker's idle wait inside a large problem
  int32_t blocks_per_sm = 1;            // FMA form: the kernel's build, 1 or 4 blocks per SM
};

struct SseArgs {
  DevFactors f;
  const int2* ratings = nullptr;
  const int64_t* col_ptr = nullptr;
  int64_t nnz = 0;
  double* partials = nullptr;  // [grid] scratch
  double* out = nullptr;       // [1]
  int32_t grid = 0;
};

// Returns cudaError_t of the launch (cudaSuccess when nothing was launched).
cudaError_t launch_async(const AsyncArgs& a, cudaStream_t s);
cudaError_t async_occupancy(int bf16, int nv, int exact, int warps_per_block, int kpad,
                            int* blocks_per_sm);
cudaError_t launch_async2(const AsyncArgs& a, cudaStream_t s);
cudaError_t launch_seed_queues(const AsyncArgs& a, const int4* first_mail, const int2* first_q,
                               const int* counts, int n, int ep, cudaStream_t s);
cudaError_t launch_drain_queues(const AsyncArgs& a, cudaStream_t s);
// The CSC of a row-major rating set (row counts, column indices, fp64 or fp32 values, all
// host arrays; the row counts already checked to add up to nnz) built on the device by a
// stable radix sort of the entries by column, so rows stay ascending inside a column:
// ratings {row, value bits} (nnz entries) and col_ptr (n + 1), both caller-allocated.
// A column index outside [0, n) stops it before the sort with cudaErrorInvalidValue and
// its entry in *bad_col (else -1); *dup_col is the first column with a repeated (row,
// column) cell, else -1; *h2d_bytes grows by the bytes copied in.  1 <= nnz <= INT_MAX.
cudaError_t device_csc(int64_t nnz, int32_t m, int32_t n, const int32_t* row_counts, const int32_t* cols,
                       const double* v64, const float* v32, int2* ratings, int64_t* col_ptr, int64_t* bad_col,
                       int32_t* dup_col, int64_t* h2d_bytes, cudaStream_t s);
// The visit lists of the asynchronous modes built on the device (layout_device.cu) from a
// device CSC, equal to the host's build_async_layout: count() takes the worker row blocks
// (host row_start[P + 1]) and leaves the number of visits in t->nseg; fill() writes the
// visits in route order (segs[nseg], {start lo, start hi, len, owner}) and the visit
// offsets (vl_ptr[n + 1]) on the device, copies the offsets and each column's first
// visit (firsts[n]) to the host, the longest visit to *max_seg, and frees t.  1 <= nnz <=
// INT_MAX, 1 <= group <= 32.
struct DeviceLayout {
  int32_t* row_start = nullptr;
  int32_t* row_worker = nullptr;
  int32_t* flags = nullptr;
  int32_t* seg_id = nullptr;
  void* tmp = nullptr;
  int64_t nseg = 0;
};
cudaError_t device_layout_count(const int2* ratings, const int64_t* col_ptr, int64_t nnz, int32_t m, int32_t n,
                                const int32_t* row_start, int32_t P, int32_t group, int64_t priority_min,
                                DeviceLayout* t, cudaStream_t s);
cudaError_t device_layout_fill(const int2* ratings, const int64_t* col_ptr, int64_t nnz, int32_t n, int32_t group,
                               bool group_routes, int64_t priority_min, uint64_t seed, DeviceLayout* t, int4* segs,
                               int64_t* vl_ptr, int64_t* vl_ptr_host, int4* firsts_host, int32_t* max_seg,
                               cudaStream_t s);
void device_layout_release(DeviceLayout* t, cudaStream_t s);
// The rows of a device CSC's ratings (nnz entries) copied to host memory.
cudaError_t device_csc_rows(const int2* ratings, int64_t nnz, int32_t* host_rows, cudaStream_t s);
// One rating set of one problem of a batch, row-major as for device_csc (row counts
// already checked to add up to nnz); the arrays may be NULL when nnz is 0.
struct BatchSetIn {
  int64_t nnz;
  int32_t m, n;
  const int32_t* row_counts;
  const int32_t* cols;
  const void* vals;  // double or float, the same for every problem
};
// The CSCs of `count` problems' sets built together on the device: one stable radix sort
// of all entries by (problem, column), so ratings hold problem after problem, each in
// column order with rows ascending inside a column ({row, value bits}, sum of nnz
// entries), and col_ptr problem after problem n + 1 offsets into ratings (sum of n + 1
// entries); both caller-allocated.  n_active_host (or NULL) receives each problem's
// columns with ratings.  *faulty is set, with nothing else guaranteed, when a column index
// is out of range or a (row, column) cell repeats.  The sum of nnz is at most INT_MAX,
// the sum of n below 2^32.
cudaError_t device_batch_csc(const BatchSetIn* sets, int32_t count, bool f64, int2* ratings, int64_t* col_ptr,
                             int32_t* n_active_host, bool* faulty, int64_t* h2d_bytes, cudaStream_t s);
// A large batched problem's visit bounds: for each of its n columns, R + 1 offsets into
// ratings, the first rating of the column whose row is at least rs[w] (w = 0..R).
struct BatchSegIn {
  int64_t col_off, seg_off;  // the problem's column pointers in col_ptr; its bounds in seg
  int32_t n, rs_off;         // columns; its R + 1 row-block starts in rs
};
cudaError_t device_batch_segs(const int2* ratings, const int64_t* col_ptr, const BatchSegIn* big_host, int32_t n_big,
                              const int32_t* rs, int32_t R, int64_t* seg, cudaStream_t s);
cudaError_t launch_build_segx(const int4* segs, const int2* ratings, int64_t nseg, int4* segx, cudaStream_t s);
cudaError_t async2_occupancy(int bf16, int nv, int warps, int kpad, int cta_heavy, int* blocks_per_sm);
cudaError_t launch_replay(const ReplayArgs& a, cudaStream_t s);
// One epoch of every batched problem (the work-queue kernel, then the pass-count advance);
// `grid` blocks of kBatchThreads threads.
constexpr int kBatchThreads = 128;
cudaError_t launch_batch_epoch(const BatchArgs& a, int grid, cudaStream_t s);
cudaError_t batch_occupancy(int bf16, int exact, int* blocks_per_sm);
// FMA form: blocks of kBatchWorkers warps; large problems first (a block each), then the
// rest a warp each.
cudaError_t launch_batch_epoch2(const BatchArgs& a, int grid, cudaStream_t s);
// blocks_per_sm selects the FMA kernel's build (1 or 4 resident blocks per SM); *bps is
// how many of its blocks fit on an SM.
cudaError_t batch2_occupancy(int bf16, int blocks_per_sm, int* bps);
cudaError_t launch_batch_sse(const BatchArgs& a, int grid, cudaStream_t s);
cudaError_t launch_dsgd_stratum(const DsgdArgs& a, int stratum, cudaStream_t s);
cudaError_t launch_sse(const SseArgs& a, cudaStream_t s);
cudaError_t launch_init_hash(const DevFactors& f, uint64_t seed, cudaStream_t s);
// Ratings per row of a CSC rating set (counts[m], zeroed first).
cudaError_t launch_count_rows(const int2* ratings, int64_t nnz, int32_t* counts, int32_t m, cudaStream_t s);
// *out = sum over rows r of W (rows_of_w) or H of count(r) * |x_r|^2, count from
// counts[r] or ptr[r+1] - ptr[r]; FP64, deterministic (partials[grid] scratch).
cudaError_t launch_weighted_norm(const DevFactors& f, bool rows_of_w, const int32_t* counts,
                                 const int64_t* ptr, double* partials, int32_t grid, double* out,
                                 cudaStream_t s);
cudaError_t launch_f32_to_store(const float* src, void* dst, int64_t rows, int32_t dim,
                                int32_t kpad, int bf16, cudaStream_t s);
cudaError_t launch_store_to_f32(const void* src, float* dst, int64_t rows, int32_t dim,
                                int32_t kpad, int bf16, cudaStream_t s);
// The reference init of batched problems' rows on the device.  Every problem draws from
// the same streams (W's row block t from one stream, H from another), so the streams'
// canonical values are drawn once on the host as far as the longest problem needs and
// uploaded; value k of row r of W is float(c[t][(r - t rpp) dim + k] b + 0.0), t = r /
// rpp, and of H float(ch[r dim + k] b + 0.0), padding columns 0, stored as fp32 or bf16
// (round to nearest) at the problem's offsets.  Problems whose `side` flag is 0 are
// left alone.  off[p] are the problems' element offsets in the side's concatenation
// (count + 1 entries, increasing).
struct BatchInitIn {
  int32_t rows, dim, kpad, rpp;  // rows of the side; rpp: rows per row block (W), else rows
  int32_t init, pad;             // 1: draw this side's rows
  double b;                      // 1 / sqrt(dim)
};
cudaError_t launch_batch_ref_init(const BatchInitIn* probs, const int64_t* off, int32_t count, int64_t total,
                                  const double* c, const int64_t* c_off, void* dst, int bf16, cudaStream_t s);
cudaError_t launch_empty_queues(int32_t* qnext, int32_t* qtail, int32_t n, int32_t P,
                                cudaStream_t s);

}  // namespace nomad
