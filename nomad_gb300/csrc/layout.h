// layout.h -- host-side construction of the device data layout.
#pragma once

#include <sys/mman.h>

#include <cstdint>
#include <cstdlib>
#include <memory>
#include <new>
#include <type_traits>
#include <utility>
#include <vector>

#include "common.h"

namespace nomad {

// One rating in CSC-by-column order: row index and the value's float bits.
struct Rating {
  int32_t row;
  float val;
};

// Allocator whose value construction leaves trivial elements uninitialised, so that
// resize() of a large buffer that is filled next writes no zeros first (the first touch
// of its pages then happens in the parallel fill).  Buffers of 32 MB and more are
// 2 MB-aligned and advised for transparent huge pages: fewer page faults on first touch.
template <typename T>
struct NoInitAllocator : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = NoInitAllocator<U>;
  };
  static constexpr size_t kHugeBytes = size_t{32} << 20;
  NoInitAllocator() = default;
  template <typename U>
  NoInitAllocator(const NoInitAllocator<U>&) noexcept {}
  T* allocate(size_t count) {
    const size_t bytes = count * sizeof(T);
    if (bytes < kHugeBytes) return std::allocator<T>::allocate(count);
    void* p = nullptr;
    if (posix_memalign(&p, size_t{2} << 20, bytes) != 0) throw std::bad_alloc();
    madvise(p, bytes, MADV_HUGEPAGE);  // advice only: ignored where huge pages are off
    return static_cast<T*>(p);
  }
  void deallocate(T* p, size_t count) noexcept {
    if (count * sizeof(T) < kHugeBytes) {
      std::allocator<T>::deallocate(p, count);
      return;
    }
    std::free(p);
  }
  template <typename U>
  void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new (static_cast<void*>(p)) U;
  }
  template <typename U, typename... Args>
  void construct(U* p, Args&&... args) {
    ::new (static_cast<void*>(p)) U(std::forward<Args>(args)...);
  }
};

// Ratings grouped by column, rows ascending inside a column (what read_data builds
// for one part, Code/nomad/nb_data.cpp:131-169).
struct Csc {
  int32_t m = 0, n = 0;
  std::vector<int64_t> col_ptr;  // [n+1]
  std::vector<Rating, NoInitAllocator<Rating>> ratings;  // [nnz]
  std::vector<int32_t> row_nnz;  // [m] ratings per row (from the row-major input)
  // [nnz] the rows alone, in place of `ratings`, for a CSC kept on the device whose host
  // copy only feeds the layout builds
  std::vector<int32_t, NoInitAllocator<int32_t>> rows;
  int64_t nnz() const { return col_ptr.empty() ? 0 : col_ptr.back(); }
  int32_t row(int64_t o) const { return rows.empty() ? ratings[o].row : rows[o]; }
};

// A token visit: the ratings of one column owned by one worker.  16 bytes, read by
// the device as an int4 {start lo, start hi, len, worker}.
struct Segment {
  int64_t start;
  int32_t len;
  int32_t worker;
};
static_assert(sizeof(Segment) == 16, "segment must be 16 bytes");

struct AsyncLayout {
  int32_t P = 0;
  std::vector<int32_t> row_start;  // [P+1] first row of each worker's block
  std::vector<int64_t> vl_ptr;     // [n+1] visit list of each column
  std::vector<Segment, NoInitAllocator<Segment>> segs;  // visits, each column's list in its route order
  std::vector<int32_t> qnext0;     // [n+2P] initial queues (tokens in column order)
  std::vector<int32_t> qtail0;     // [2P]: queue w = worker w's queue, P+w its priority queue
  std::vector<int32_t> desc0;      // [4n] first visit of each token {start lo, hi, len, 0|heavy}
  int32_t n_priority = 0;          // tokens that use the priority queues
  // pipelined kernel: first mailbox of each token (8 ints: start lo/hi, len, pos = 0;
  // ep, nseg | heavy bit, vb lo/hi), its first queue and rank there, tokens per queue
  std::vector<int32_t> first_mail;  // [8n]
  std::vector<int32_t> first_q;     // [2n] {queue, rank}, queue -1 for an empty column
  std::vector<int32_t> q_count;     // [2P]
  int32_t n_active = 0;
  int64_t max_column = 0;
  int64_t max_segment = 0;
};

// DSGD blocks of one process (Code/competitor/sgd-mpi-omp.cpp:39-60, 539-588):
// innerB x innerB blocks; entries of a block in reversed file order, so the device
// walks forward through what sgd() walks backward.
struct DsgdLayout {
  int32_t innerB = 0, col_blocks = 0, innerBm = 0, innerBn = 0;
  std::vector<int64_t> blk_ptr;  // [innerB * col_blocks + 1]
  std::vector<int32_t> rates;    // 4 ints per entry: row, col, float bits, 0
};

// The argument checks of build_csc that need no sort (array presence, row counts adding
// up to nnz, with check_cols column indices in range), for a CSC built elsewhere
// (csc_device.cu).
int check_rating_set(const nomad_gpu_matrix& A, int32_t m, int32_t n, int threads, bool check_cols);

// Build the CSC of a rating set given in the row-major file layout or as COO.
// Fails on out-of-range indices and on repeated (row, column) cells.
int build_csc(const nomad_gpu_matrix& A, int32_t m, int32_t n, Csc& out, int threads);

// Row blocks, visit lists (shuffled with `seed`) and the initial queues.
// priority_min: columns with at least this many ratings use the priority queues
// (<= 0: none).  group: a priority column visits groups of `group` consecutive workers
// (the warps of one thread block, which process the visit together); its segments name
// the group, and its queue is P + group index.  group_routes: the other columns' routes
// keep the visits to one group's workers consecutive.
int build_async_layout(const Csc& csc, int32_t P, int balance, uint64_t seed,
                       int64_t priority_min, int32_t group, bool group_routes, AsyncLayout& out,
                       int threads);

// The two host parts of build_async_layout that a visit list built elsewhere
// (layout_device.cu) still needs: the worker row blocks (L.P, L.row_start), and, from
// each column's visit count (L.vl_ptr) and first visit in route order (firsts[n], read
// only for active columns), the initial queues, first mailboxes and token counts.
int async_layout_rows(const Csc& csc, int32_t P, int balance, AsyncLayout& L, int threads);
void async_layout_queues(const Csc& csc, int64_t priority_min, const Segment* firsts, AsyncLayout& L);

// innerB row blocks x col_blocks column blocks (innerB for DSGD, 2*innerB for
// DSGD++: dsgdpp.cpp:42-52, 64-69); block (bi, bj) has id bi*col_blocks + bj.
int build_dsgd_layout(const nomad_gpu_matrix& A, int32_t m, int32_t n, int32_t innerB,
                      int32_t col_blocks, DsgdLayout& out);

// DSGD inner-stratum schedule of iteration `iter` (1-based): bj of row block bi in
// stratum i at [i*innerB + bi] (sgd-mpi-omp.cpp:268-365 with B = 1).
void dsgd_schedule(int32_t innerB, int32_t iter, int32_t strategy, std::vector<int32_t>& out);

// DSGD++ schedule of iteration `iter`: 2*innerB strata, phase 0 (column blocks
// 0..innerB-1) then phase 1 (innerB..2*innerB-1); column block of row block bi in
// stratum s at [s*innerB + bi] (dsgdpp.cpp:347-355, 393-401, 434-441 with B = 1).
void dsgdpp_schedule(int32_t innerB, int32_t iter, int32_t strategy, std::vector<int32_t>& out);

// Step size of pass `cnt` in float semantics (nomad_body.hpp:326-327).
float step_size_f32(double lrate, double drate, int32_t cnt);

}  // namespace nomad
