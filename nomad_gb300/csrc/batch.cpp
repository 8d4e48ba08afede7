// batch.cpp -- the batched-problem C-ABI (include/nomad_gpu.h, nomad_gpu_batch_*): many
// independent completion problems in one context, trained by one persistent launch per
// epoch that is captured once as a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#include "common.h"
#include "launch.h"
#include "layout.h"
#include "trace.h"
#include "tune.h"

struct nomad_gpu_batch {
  nomad_gpu_params prm{};
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<void*> allocs;
  std::vector<nomad::BatchProblem> probs;
  nomad::BatchArgs a;
  int esz = 4;
  int grid = 0, sse_grid = 0;
  std::vector<int32_t> part_of;   // per evaluation part: 2 * problem + set
  std::vector<int64_t> set_count; // [2 * count] train and test ratings of each problem
  int32_t n_steps = 0, epochs_done = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int32_t n_big = 0;  // problems on whole thread blocks
};

namespace {

int cuda_fail(cudaError_t e, const char* what) {
  nomad::set_last_error("%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? NOMAD_ERR_OOM : NOMAD_ERR_CUDA;
}

#define CK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

#define RC(call)         \
  do {                   \
    int rc_ = (call);    \
    if (rc_) return rc_; \
  } while (0)

template <typename T>
int dalloc(nomad_gpu_batch* b, T** p, size_t count) {
  *p = nullptr;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    NOMAD_FAIL(NOMAD_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", std::max<size_t>(count, 1) * sizeof(T),
               cudaGetErrorString(e));
  }
  b->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return NOMAD_OK;
}

template <typename T>
int upload(nomad_gpu_batch* b, T** p, const T* src, size_t count) {
  RC(dalloc(b, p, count));
  if (count) CK(cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, b->stream));
  return NOMAD_OK;
}

// Step sizes for every pass count below `needed`.  The captured graph holds the table's
// address, so a new table means a new graph.
int ensure_steps(nomad_gpu_batch* b, int32_t needed) {
  if (needed <= b->n_steps) return NOMAD_OK;
  int32_t cap = std::max<int32_t>(256, b->n_steps);
  while (cap < needed) cap *= 2;
  std::vector<float> h(cap);
  for (int32_t e = 0; e < cap; ++e) h[e] = nomad::step_size_f32(b->prm.lrate, b->prm.drate, e);
  float* d = nullptr;
  RC(upload(b, &d, h.data(), h.size()));
  CK(cudaStreamSynchronize(b->stream));
  b->a.steps = d;
  b->a.n_steps = cap;
  b->n_steps = cap;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  return NOMAD_OK;
}

// The epoch launch (work-queue kernel + pass-count advance) as a graph.
int ensure_graph(nomad_gpu_batch* b) {
  if (b->exec) return NOMAD_OK;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const cudaError_t le = b->a.exact ? nomad::launch_batch_epoch(b->a, b->grid, b->stream)
                                    : nomad::launch_batch_epoch2(b->a, b->grid, b->stream);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
  if (le != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(le, "nomad::launch_batch_epoch (capture)");
  }
  CK(ce);
  b->graph = g;
  CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return NOMAD_OK;
}

// A temporary device buffer, freed when it goes out of scope.
struct DevTemp {
  void* p = nullptr;
  cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, std::max<size_t>(bytes, 16)); }
  ~DevTemp() {
    if (p) cudaFree(p);
  }
};

// Whether the device build takes every problem's sets: each row-major or empty, one value
// type throughout (*f64), the totals within its limits.
bool device_batch_ok(const nomad_gpu_batch_problem* P, int32_t count, bool* f64) {
  int kind = 0;  // 1: fp64 values, 2: fp32
  int64_t tr = 0, te = 0, rows = 0, cols = 0;
  for (int32_t i = 0; i < count; ++i) {
    for (const nomad_gpu_matrix* A : {&P[i].train, &P[i].test}) {
      if (A->nnz == 0) continue;
      if (A->nnz < 0 || !A->row_counts || !A->cols || (A->vals_f64 != nullptr) == (A->vals_f32 != nullptr))
        return false;
      const int k = A->vals_f64 ? 1 : 2;
      if (kind && k != kind) return false;
      kind = k;
    }
    tr += std::max<int64_t>(P[i].train.nnz, 0);
    te += std::max<int64_t>(P[i].test.nnz, 0);
    rows += P[i].m;
    cols += P[i].n;
  }
  *f64 = kind == 1;
  return kind != 0 && tr <= INT_MAX && te <= INT_MAX && rows < INT_MAX && cols <= INT_MAX;
}

// Compares `bytes` of device memory with a host copy; the first difference names *differs.
int same_as_device(nomad_gpu_batch* b, const void* dev, const void* host, size_t bytes, const char* what,
                   const char** differs) {
  if (*differs || bytes == 0) return NOMAD_OK;
  std::vector<char> got(bytes);
  CK(cudaMemcpyAsync(got.data(), dev, bytes, cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (std::memcmp(got.data(), host, bytes) != 0) *differs = what;
  return NOMAD_OK;
}

int init_impl(nomad_gpu_batch* b, const nomad_gpu_batch_problem* P, int32_t count) {
  const nomad_gpu_params& p = b->prm;
  const int threads = nomad::host_threads();
  nomad::InitTrace trace;
  CK(cudaSetDevice(b->device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, b->device));
  if (prop.major * 10 + prop.minor != 103)
    NOMAD_FAIL(NOMAD_ERR_NO_DEVICE, "device %d is sm_%d%d; the library is compiled for sm_103a", b->device, prop.major,
               prop.minor);
  b->num_sms = prop.multiProcessorCount;
  CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&b->ev0));
  CK(cudaEventCreate(&b->ev1));
  const bool bf16 = p.precision == NOMAD_PREC_BF16_SR;
  b->esz = bf16 ? 2 : 4;

  // ---- per-problem layout, concatenated ------------------------------------------------
  // The sets are built into CSC on the device in one sort of every problem's entries
  // (csc_device.cu) when every set is row-major; else, and to name a fault the device
  // build found, each problem's CSC is built on one host thread and the results are
  // concatenated.
  b->probs.resize(count);
  for (int32_t i = 0; i < count; ++i) {
    const nomad_gpu_batch_problem& q = P[i];
    if (q.m <= 0 || q.n <= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "problem %d: m and n must be positive", i);
    if (q.dim <= 0 || q.dim > 128) NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "problem %d: dim %d outside [1, 128]", i, q.dim);
  }
  std::vector<int64_t> nnz(count), nnz_te(count);
  int64_t w_off = 0, h_off = 0, tr_len = 0, te_len = 0, cp_len = 0, tcp_len = 0;
  std::vector<int64_t> tr_at(count), te_at(count);
  for (int32_t i = 0; i < count; ++i) {
    const nomad_gpu_batch_problem& q = P[i];
    nomad::BatchProblem& pb = b->probs[i];
    std::memset(&pb, 0, sizeof(pb));
    pb.m = q.m;
    pb.n = q.n;
    pb.dim = q.dim;
    pb.kpad = bf16 ? (q.dim + 7) / 8 * 8 : (q.dim + 3) / 4 * 4;
    pb.nvec = pb.kpad / 4;
    pb.red_width = 1;
    while (pb.red_width < std::min(pb.nvec, 32)) pb.red_width <<= 1;
    pb.w_off = w_off;
    pb.h_off = h_off;
    w_off += static_cast<int64_t>(q.m) * pb.kpad;
    h_off += static_cast<int64_t>(q.n) * pb.kpad;
    pb.col_off = cp_len;
    pb.test_col_off = tcp_len;
    cp_len += q.n + 1;
    tcp_len += q.n + 1;
    tr_at[i] = tr_len;
    te_at[i] = te_len;
    nnz[i] = std::max<int64_t>(q.train.nnz, 0);  // a negative count fails the checks below
    nnz_te[i] = std::max<int64_t>(q.test.nnz, 0);
    tr_len += nnz[i];
    te_len += nnz_te[i];
  }
  bool f64 = false;
  bool on_device = device_batch_ok(P, count, &f64);
  if (on_device) {  // the checks of the host build that need no sort
    std::atomic<bool> ok{true};
    nomad::parallel_dynamic(count, 16, threads, [&](int, int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi && ok.load(std::memory_order_relaxed); ++i)
        if (nomad::check_rating_set(P[i].train, P[i].m, P[i].n, 1, false) ||
            nomad::check_rating_set(P[i].test, P[i].m, P[i].n, 1, false))
          ok = false;
    });
    on_device = ok;
  }
  int2 *tr = nullptr, *te = nullptr;
  int64_t *cp = nullptr, *tcp = nullptr;
  RC(dalloc(b, &tr, static_cast<size_t>(tr_len)));
  RC(dalloc(b, &te, static_cast<size_t>(te_len)));
  RC(dalloc(b, &cp, static_cast<size_t>(cp_len)));
  RC(dalloc(b, &tcp, static_cast<size_t>(tcp_len)));
  std::vector<int32_t> active(count, 0);
  bool built = false;
  if (on_device) {
    std::vector<nomad::BatchSetIn> in(count);
    auto sets = [&](int test) {
      for (int32_t i = 0; i < count; ++i) {
        const nomad_gpu_matrix& A = test ? P[i].test : P[i].train;
        in[i] = nomad::BatchSetIn{A.nnz, P[i].m, P[i].n, A.row_counts, A.cols,
                                  f64 ? static_cast<const void*>(A.vals_f64) : static_cast<const void*>(A.vals_f32)};
      }
      return in.data();
    };
    bool faulty = false;
    int64_t h2d = 0;
    CK(nomad::device_batch_csc(sets(0), count, f64, tr, cp, active.data(), &faulty, &h2d, b->stream));
    if (!faulty) CK(nomad::device_batch_csc(sets(1), count, f64, te, tcp, nullptr, &faulty, &h2d, b->stream));
    built = !faulty;
    trace.mark("CSC builds (device)");
  }
  std::vector<nomad::Csc> csc_tr;  // the host builds, when made
  if (!built || (p.debug_flags & 4)) {
    std::vector<nomad::Csc> csc_te(count);
    csc_tr.resize(count);
    std::vector<int> status(count, NOMAD_OK);
    std::vector<std::string> errors(count);
    nomad::parallel_dynamic(count, 4, threads, [&](int, int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi; ++i) {
        const nomad_gpu_batch_problem& q = P[i];
        int rc = nomad::build_csc(q.train, q.m, q.n, csc_tr[i], 1);
        if (!rc) rc = nomad::build_csc(q.test, q.m, q.n, csc_te[i], 1);
        if (rc) {
          status[i] = rc;
          errors[i] = nomad::last_error();
        }
      }
    });
    for (int32_t i = 0; i < count; ++i)
      if (status[i]) NOMAD_FAIL(status[i], "problem %d: %s", i, errors[i].c_str());
    if (built) trace.mark("CSC builds (host, for the check)");
    else trace.mark("CSC builds (host)");
    std::vector<nomad::Rating, nomad::NoInitAllocator<nomad::Rating>> tr_all(tr_len), te_all(te_len);
    std::vector<int64_t> cp_all(cp_len), tcp_all(tcp_len);
    std::vector<int32_t> act(count, 0);
    nomad::parallel_dynamic(count, 4, threads, [&](int, int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi; ++i) {
        const nomad::BatchProblem& pb = b->probs[i];
        const nomad::Csc& c = csc_tr[i];
        const nomad::Csc& t = csc_te[i];
        for (int32_t j = 0; j <= pb.n; ++j) {
          cp_all[pb.col_off + j] = tr_at[i] + c.col_ptr[j];
          tcp_all[pb.test_col_off + j] = te_at[i] + t.col_ptr[j];
        }
        std::copy(c.ratings.begin(), c.ratings.end(), tr_all.begin() + tr_at[i]);
        std::copy(t.ratings.begin(), t.ratings.end(), te_all.begin() + te_at[i]);
        for (int32_t j = 0; j < pb.n; ++j) act[i] += c.col_ptr[j + 1] > c.col_ptr[j] ? 1 : 0;
      }
    });
    static_assert(sizeof(nomad::Rating) == sizeof(int2), "rating layout");
    if (!built) {
      CK(nomad::upload_staged(tr, tr_all.data(), tr_all.size() * sizeof(int2), b->stream));
      CK(nomad::upload_staged(te, te_all.data(), te_all.size() * sizeof(int2), b->stream));
      CK(nomad::upload_staged(cp, cp_all.data(), cp_all.size() * sizeof(int64_t), b->stream));
      CK(nomad::upload_staged(tcp, tcp_all.data(), tcp_all.size() * sizeof(int64_t), b->stream));
      active = act;
    } else {  // debug bit 2: the device build must equal the host's, entry for entry
      const char* differs = nullptr;
      RC(same_as_device(b, tr, tr_all.data(), tr_all.size() * sizeof(int2), "train ratings", &differs));
      RC(same_as_device(b, te, te_all.data(), te_all.size() * sizeof(int2), "test ratings", &differs));
      RC(same_as_device(b, cp, cp_all.data(), cp_all.size() * sizeof(int64_t), "train column pointers", &differs));
      RC(same_as_device(b, tcp, tcp_all.data(), tcp_all.size() * sizeof(int64_t), "test column pointers", &differs));
      if (!differs && act != active) differs = "columns with ratings";
      if (differs) NOMAD_FAIL(NOMAD_ERR_BOUNDS, "device batch CSC differs from the host build: %s", differs);
    }
    trace.mark("concatenation", b->stream);
  }
  for (int32_t i = 0; i < count; ++i) b->probs[i].n_active = active[i];
  // the evaluation's parts: each problem's train and test ratings in runs of at most
  // kSsePart, problems and sets in order
  constexpr int64_t kSsePart = 32768;
  std::vector<nomad::SsePart> parts;
  b->set_count.assign(2 * static_cast<size_t>(count), 0);
  for (int32_t i = 0; i < count; ++i)
    for (int32_t set = 0; set < 2; ++set) {
      const int64_t b0 = set ? te_at[i] : tr_at[i], e0 = b0 + (set ? nnz_te[i] : nnz[i]);
      b->set_count[2 * static_cast<size_t>(i) + set] = e0 - b0;
      for (int64_t s0 = b0; s0 < e0; s0 += kSsePart) {
        parts.push_back(nomad::SsePart{s0, std::min(e0, s0 + kSsePart), i, set});
        b->part_of.push_back(2 * i + set);
      }
    }
  // work queue: the largest problems first, so the longest epochs start first
  std::vector<int32_t> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return nnz[x] > nnz[y]; });
  // FMA form: problems with more than `batch_share` (default 1) warps' fair share of the
  // ratings run on a whole block as NOMAD workers (rows split into kBatchWorkers blocks of
  // equal rating counts)
  // FMA form at one or four blocks per SM (the kernel is built for each).  Four carry more
  // work at once; one leaves the SM to a large problem's workers, whose epoch bounds the
  // batch's when that problem is a large part of it (4,096-problem batch, largest problem
  // 0.76% of the ratings: 149 against 166 ms per fp32 epoch with four; 512 problems,
  // largest 4.1%: 45 against 57 ms with one).  params.blocks_per_sm = 1 or > 1 forces one
  // or four.
  const int64_t total = std::accumulate(nnz.begin(), nnz.end(), int64_t(0));
  const int64_t largest = nnz[order[0]];
  const int mb = p.blocks_per_sm == 1 ? 1 : p.blocks_per_sm > 1 ? 4 : (largest * 50 <= total ? 4 : 1);
  int bps = 0;
  if (p.exact)
    CK(nomad::batch_occupancy(bf16, 1, &bps));
  else
    CK(nomad::batch2_occupancy(bf16, mb, &bps));
  if (bps <= 0) NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "batched kernel does not fit on an SM");
  b->grid = bps * b->num_sms;
  b->a.blocks_per_sm = mb;
  const int64_t warps = static_cast<int64_t>(b->grid) * (p.exact ? nomad::kBatchThreads / 32 : nomad::kBatchWorkers);
  const int64_t share = p.batch_share == 0 ? 1 : p.batch_share;
  const int64_t big_min = share < 0 ? std::numeric_limits<int64_t>::max()
                                    : std::max<int64_t>(8192, share * total / std::max<int64_t>(warps, 1));
  int32_t n_big = 0;
  constexpr int R = nomad::kBatchWorkers;
  int32_t* rs_d = nullptr;
  int64_t* seg_d = nullptr;
  if (!p.exact) {
    while (n_big < count && nnz[order[n_big]] >= big_min && P[order[n_big]].n < nomad::kBatchRing &&
           P[order[n_big]].n < 65536)
      ++n_big;
  }
  if (n_big > 0) {
    // slices: R + 1 row starts per large problem from its row counts (equal rating counts
    // per warp), and n (R + 1) visit bounds, found on the device
    std::vector<nomad::BatchSegIn> big(n_big);
    int64_t seg_len = 0;
    for (int32_t t = 0; t < n_big; ++t) {
      nomad::BatchProblem& pb = b->probs[order[t]];
      pb.rs_off = t * (R + 1);
      pb.seg_off = seg_len;
      big[t] = nomad::BatchSegIn{pb.col_off, pb.seg_off, pb.n, pb.rs_off};
      seg_len += static_cast<int64_t>(pb.n) * (R + 1);
    }
    std::vector<int32_t> rs_all(static_cast<size_t>(n_big) * (R + 1), 0);
    nomad::parallel_dynamic(n_big, 1, threads, [&](int, int64_t lo, int64_t hi) {
      for (int64_t t = lo; t < hi; ++t) {
        const int32_t i = order[t];
        const nomad::BatchProblem& pb = b->probs[i];
        const int32_t* row_nnz = built ? P[i].train.row_counts : csc_tr[i].row_nnz.data();
        int32_t* rs = rs_all.data() + pb.rs_off;
        const int64_t nz = nnz[i];
        int64_t acc = 0;
        int32_t r = 1;
        rs[0] = 0;
        for (int32_t row = 0; row < pb.m && r < R; ++row) {
          acc += row_nnz[row];
          while (r < R && acc >= (nz * r + R - 1) / R) rs[r++] = row + 1;
        }
        for (; r <= R; ++r) rs[r] = pb.m;
      }
    });
    RC(upload(b, &rs_d, rs_all.data(), rs_all.size()));
    RC(dalloc(b, &seg_d, static_cast<size_t>(seg_len)));
    CK(nomad::device_batch_segs(tr, cp, big.data(), n_big, rs_d, R, seg_d, b->stream));
    if (!csc_tr.empty() && built) {  // debug bit 2: the bounds as the host finds them
      std::vector<int64_t> seg_all(static_cast<size_t>(seg_len));
      nomad::parallel_dynamic(n_big, 1, threads, [&](int, int64_t lo, int64_t hi) {
        for (int64_t t = lo; t < hi; ++t) {
          const nomad::BatchProblem& pb = b->probs[order[t]];
          const nomad::Csc& c = csc_tr[order[t]];
          const int32_t* rs = rs_all.data() + pb.rs_off;
          int64_t* sg = seg_all.data() + pb.seg_off;
          for (int32_t j = 0; j < pb.n; ++j) {
            int64_t o = c.col_ptr[j];
            for (int32_t w = 0; w <= R; ++w) {
              while (o < c.col_ptr[j + 1] && c.ratings[o].row < rs[w]) ++o;
              *sg++ = tr_at[order[t]] + o;
            }
          }
        }
      });
      const char* differs = nullptr;
      RC(same_as_device(b, seg_d, seg_all.data(), seg_all.size() * sizeof(int64_t), "visit bounds", &differs));
      if (differs) NOMAD_FAIL(NOMAD_ERR_BOUNDS, "device batch CSC differs from the host build: %s", differs);
    }
  }
  csc_tr.clear();
  trace.mark("large-problem layout", b->stream);

  nomad::BatchArgs& a = b->a;
  a.count = count;
  a.bf16 = bf16;
  a.exact = p.exact;
  a.lambda = static_cast<float>(p.reg);
  a.seed32 = static_cast<uint32_t>(p.seed ^ (p.seed >> 32));
  char *W = nullptr, *H = nullptr;
  RC(dalloc(b, &W, static_cast<size_t>(w_off) * b->esz));
  RC(dalloc(b, &H, static_cast<size_t>(h_off) * b->esz));
  a.W = W;
  a.H = H;
  nomad::BatchProblem* dp = nullptr;
  int32_t* dord = nullptr;
  RC(upload(b, &dp, b->probs.data(), b->probs.size()));
  RC(upload(b, &dord, order.data(), order.size()));
  a.ratings = tr;
  a.test = te;
  a.col_ptr = cp;
  a.test_col_ptr = tcp;
  a.problems = dp;
  a.order = dord;
  RC(dalloc(b, &a.next, 1));
  RC(dalloc(b, &a.epoch, 1));
  RC(dalloc(b, &a.stats, 4));
  RC(dalloc(b, &a.err_sum, 1));
  nomad::SsePart* dparts = nullptr;
  RC(upload(b, &dparts, parts.data(), parts.size()));
  a.parts = dparts;
  a.n_parts = static_cast<int32_t>(parts.size());
  RC(dalloc(b, &a.part_sse, std::max<size_t>(parts.size(), 1)));
  CK(cudaMemsetAsync(a.epoch, 0, sizeof(int32_t), b->stream));
  a.n_big = n_big;
  b->n_big = n_big;
  RC(dalloc(b, &a.next_big, 1));
  RC(dalloc(b, &a.ctrl, 2));
  CK(cudaMemsetAsync(a.next_big, 0, sizeof(int32_t), b->stream));
  CK(cudaMemsetAsync(a.ctrl, 0, 2 * sizeof(int32_t), b->stream));
  CK(cudaMemcpyAsync(a.next, &a.n_big, sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));  // small ones after
  a.budget_ns = static_cast<int64_t>(std::max(p.spin_budget_ms, 1)) * 1000000LL;
  if (n_big > 0) {
    a.row_start = rs_d;
    a.seg = seg_d;
    RC(dalloc(b, &a.rings, static_cast<size_t>(b->grid) * R * nomad::kBatchRing));
    RC(dalloc(b, &a.ring_ctr, static_cast<size_t>(b->grid) * R));
    CK(cudaMemsetAsync(a.rings, 0xff, static_cast<size_t>(b->grid) * R * nomad::kBatchRing * 8, b->stream));
    CK(cudaMemsetAsync(a.ring_ctr, 0, static_cast<size_t>(b->grid) * R * sizeof(unsigned), b->stream));
  }

  trace.mark("uploads", b->stream);
  // ---- factors.  Rows not given take the reference init (nomad_reference_init): every
  // such problem draws from the same streams -- W's row block t from seed + t + 1, H from
  // seed + 139 -- so each stream is drawn here once, as far as the longest problem needs,
  // and a kernel scales and stores every problem's rows.  Given rows are copied in
  // through the pinned staging buffers in groups of at most kStage floats and converted
  // to the padded storage on the device.
  {
    const int32_t parts = std::max(p.init_parts, 1);
    std::vector<int64_t> lw(parts, 0), c_off(static_cast<size_t>(parts) + 1, 0);
    int64_t lh = 0;
    std::vector<nomad::BatchInitIn> init_in(2 * static_cast<size_t>(count));  // W sides, then H sides
    std::vector<int64_t> offs(2 * (static_cast<size_t>(count) + 1));          // element offsets, likewise
    bool any = false;
    for (int32_t i = 0; i < count; ++i) {
      const nomad_gpu_batch_problem& q = P[i];
      const nomad::BatchProblem& pb = b->probs[i];
      const int32_t rpp = q.m / parts + (q.m % parts > 0 ? 1 : 0);
      const double bound = 1.0 / std::sqrt(q.dim);
      init_in[i] = nomad::BatchInitIn{q.m, q.dim, pb.kpad, rpp, q.W0 ? 0 : 1, 0, bound};
      init_in[count + i] = nomad::BatchInitIn{q.n, q.dim, pb.kpad, q.n, q.H0 ? 0 : 1, 0, bound};
      offs[i] = pb.w_off;
      offs[count + 1 + i] = pb.h_off;
      if (!q.W0)
        for (int32_t t = 0; t < parts; ++t) {
          const int64_t lo = std::min<int64_t>(int64_t(rpp) * t, q.m), hi = std::min<int64_t>(int64_t(rpp) * (t + 1), q.m);
          lw[t] = std::max(lw[t], (hi - lo) * q.dim);
        }
      if (!q.H0) lh = std::max<int64_t>(lh, int64_t(q.n) * q.dim);
      any = any || !q.W0 || !q.H0;
    }
    offs[count] = w_off;
    offs[2 * static_cast<size_t>(count) + 1] = h_off;
    if (any) {
      for (int32_t t = 0; t < parts; ++t) c_off[t + 1] = c_off[t] + lw[t];
      // the canonical values: W's row-block streams, then H's stream at c_off[parts]
      std::vector<double> c(static_cast<size_t>(c_off[parts] + lh));
      nomad::parallel_dynamic(parts + 1, 1, threads, [&](int, int64_t lo, int64_t hi) {
        for (int64_t t = lo; t < hi; ++t) {
          if (t < parts) nomad::reference_canonical(p.seed + static_cast<uint64_t>(t) + 1, lw[t], c.data() + c_off[t]);
          else nomad::reference_canonical(p.seed + 139, lh, c.data() + c_off[parts]);
        }
      });
      DevTemp c_d, coff_d, in_d, offs_d;
      CK(c_d.alloc(c.size() * sizeof(double)));
      CK(coff_d.alloc(c_off.size() * sizeof(int64_t)));
      CK(in_d.alloc(init_in.size() * sizeof(nomad::BatchInitIn)));
      CK(offs_d.alloc(offs.size() * sizeof(int64_t)));
      CK(nomad::upload_staged(c_d.p, c.data(), c.size() * sizeof(double), b->stream));
      CK(cudaMemcpyAsync(coff_d.p, c_off.data(), c_off.size() * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
      CK(cudaMemcpyAsync(in_d.p, init_in.data(), init_in.size() * sizeof(nomad::BatchInitIn), cudaMemcpyHostToDevice,
                         b->stream));
      CK(cudaMemcpyAsync(offs_d.p, offs.data(), offs.size() * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
      const auto* in = static_cast<const nomad::BatchInitIn*>(in_d.p);
      const auto* of = static_cast<const int64_t*>(offs_d.p);
      const auto* cd = static_cast<const double*>(c_d.p);
      const auto* co = static_cast<const int64_t*>(coff_d.p);
      CK(nomad::launch_batch_ref_init(in, of, count, w_off, cd, co, W, bf16, b->stream));
      CK(nomad::launch_batch_ref_init(in + count, of + count + 1, count, h_off, cd, co + parts, H, bf16, b->stream));
      CK(cudaStreamSynchronize(b->stream));
    }
    trace.mark("factors: reference init");
    constexpr int64_t kStage = int64_t(1) << 26;  // 256 MB of fp32
    std::vector<int32_t> given;
    int64_t stage_len = 0, all = 0;
    auto need = [&](int32_t i) {
      return (P[i].W0 ? int64_t(P[i].m) * P[i].dim : 0) + (P[i].H0 ? int64_t(P[i].n) * P[i].dim : 0);
    };
    for (int32_t i = 0; i < count; ++i)
      if (P[i].W0 || P[i].H0) {
        given.push_back(i);
        stage_len = std::max(stage_len, need(i));
        all += need(i);
      }
    if (!given.empty()) {
      stage_len = std::max(stage_len, std::min(kStage, all));
      DevTemp stage_d;
      CK(stage_d.alloc(static_cast<size_t>(stage_len) * sizeof(float)));
      float* stage = static_cast<float*>(stage_d.p);
      for (size_t g0 = 0; g0 < given.size();) {
        // the group [g0, g1): consecutive problems whose given rows fit the staging buffer
        std::vector<const void*> srcs;
        std::vector<size_t> lens;
        std::vector<int64_t> at;
        int64_t used = 0;
        size_t g1 = g0;
        while (g1 < given.size()) {
          const nomad_gpu_batch_problem& q = P[given[g1]];
          if (g1 > g0 && used + need(given[g1]) > stage_len) break;
          at.push_back(used);
          if (q.W0) {
            srcs.push_back(q.W0);
            lens.push_back(static_cast<size_t>(q.m) * q.dim * sizeof(float));
          }
          if (q.H0) {
            srcs.push_back(q.H0);
            lens.push_back(static_cast<size_t>(q.n) * q.dim * sizeof(float));
          }
          used += need(given[g1]);
          ++g1;
        }
        // conversions of the previous group are ahead of this copy on the stream
        CK(nomad::upload_staged_many(stage, srcs.data(), lens.data(), srcs.size(), b->stream));
        for (size_t g = g0; g < g1; ++g) {
          const nomad_gpu_batch_problem& q = P[given[g]];
          const nomad::BatchProblem& pb = b->probs[given[g]];
          const float* src = stage + at[g - g0];
          if (q.W0) {
            CK(nomad::launch_f32_to_store(src, W + pb.w_off * b->esz, q.m, q.dim, pb.kpad, bf16, b->stream));
            src += static_cast<int64_t>(q.m) * q.dim;
          }
          if (q.H0)
            CK(nomad::launch_f32_to_store(src, H + pb.h_off * b->esz, q.n, q.dim, pb.kpad, bf16, b->stream));
        }
        g0 = g1;
      }
      CK(cudaStreamSynchronize(b->stream));
    }
  }

  trace.mark("factors");
  b->sse_grid = std::max(1, std::min((b->a.n_parts + 3) / 4, 16 * b->num_sms));  // 4 warps a block
  RC(ensure_steps(b, 64));
  CK(cudaStreamSynchronize(b->stream));
  return NOMAD_OK;
}

void release(nomad_gpu_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (void* q : b->allocs) cudaFree(q);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // namespace

extern "C" {

int nomad_gpu_batch_init(nomad_gpu_batch** out, const nomad_gpu_batch_problem* problems, int32_t count,
                         const nomad_gpu_params* params) {
  nomad::clear_last_error();
  if (!out || !problems || !params || count <= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid batch arguments");
  if (params->struct_size != static_cast<int32_t>(sizeof(nomad_gpu_params)))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "params.struct_size mismatch");
  if (params->precision != NOMAD_PREC_FP32 && params->precision != NOMAD_PREC_BF16_SR)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "unknown precision %d", params->precision);
  *out = nullptr;
  nomad_gpu_batch* b = new nomad_gpu_batch();
  b->prm = *params;
  b->device = params->device;
  const int rc = init_impl(b, problems, count);
  if (rc) {
    release(b);
    return rc;
  }
  *out = b;
  return NOMAD_OK;
}

int nomad_gpu_batch_epoch(nomad_gpu_batch* b, int32_t n_epochs, nomad_gpu_epoch_stats* st) {
  nomad::clear_last_error();
  if (!b || n_epochs < 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments");
  const auto t0 = std::chrono::steady_clock::now();
  CK(cudaSetDevice(b->device));
  RC(ensure_steps(b, b->epochs_done + n_epochs + 1));
  RC(ensure_graph(b));
  CK(cudaMemsetAsync(b->a.stats, 0, 4 * sizeof(unsigned long long), b->stream));
  CK(cudaMemsetAsync(b->a.err_sum, 0, sizeof(double), b->stream));
  CK(cudaEventRecord(b->ev0, b->stream));
  for (int32_t e = 0; e < n_epochs; ++e) CK(cudaGraphLaunch(b->exec, b->stream));
  CK(cudaEventRecord(b->ev1, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  unsigned long long stats[4];
  double esum = 0.0;
  int32_t ctrl[2] = {0, 0};
  CK(cudaMemcpy(ctrl, b->a.ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost));
  if (ctrl[1] != 0) NOMAD_FAIL(NOMAD_ERR_TIMEOUT, "a large problem's worker waited past the budget");
  CK(cudaMemcpy(stats, b->a.stats, sizeof(stats), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&esum, b->a.err_sum, sizeof(double), cudaMemcpyDeviceToHost));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  b->epochs_done += n_epochs;
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->updates = static_cast<int64_t>(stats[0]);
    st->hops = 0;
    st->epochs_done = b->epochs_done;
    st->device_ms = ms;
    st->online_sse = esum;
    st->host_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return NOMAD_OK;
}

int nomad_gpu_batch_rmse(nomad_gpu_batch* b, double* train_rmse, double* test_rmse) {
  nomad::clear_last_error();
  if (!b) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null batch");
  CK(cudaSetDevice(b->device));
  const size_t np = b->part_of.size();
  std::vector<double> part(np), sse(2 * static_cast<size_t>(b->a.count), 0.0);
  if (np) {
    CK(nomad::launch_batch_sse(b->a, b->sse_grid, b->stream));
    CK(cudaMemcpyAsync(part.data(), b->a.part_sse, np * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
  }
  for (size_t k = 0; k < np; ++k) sse[b->part_of[k]] += part[k];  // a problem's parts in order
  for (int32_t i = 0; i < b->a.count; ++i) {
    const int64_t ntr = b->set_count[2 * static_cast<size_t>(i)], nte = b->set_count[2 * static_cast<size_t>(i) + 1];
    if (train_rmse) train_rmse[i] = ntr > 0 ? std::sqrt(sse[2 * i] / static_cast<double>(ntr)) : 0.0;
    if (test_rmse) test_rmse[i] = nte > 0 ? std::sqrt(sse[2 * i + 1] / static_cast<double>(nte)) : 0.0;
  }
  return NOMAD_OK;
}

int nomad_gpu_batch_get_factors(nomad_gpu_batch* b, int32_t problem, float* W, float* H) {
  nomad::clear_last_error();
  if (!b || problem < 0 || problem >= b->a.count) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid problem index");
  CK(cudaSetDevice(b->device));
  const nomad::BatchProblem& pb = b->probs[problem];
  for (int side = 0; side < 2; ++side) {
    float* dst = side ? H : W;
    if (!dst) continue;
    const int64_t rows = side ? pb.n : pb.m;
    float* stage = nullptr;
    CK(cudaMalloc(&stage, std::max<int64_t>(rows, 1) * pb.dim * sizeof(float)));
    const char* src = static_cast<const char*>(side ? b->a.H : b->a.W) + (side ? pb.h_off : pb.w_off) * b->esz;
    cudaError_t e = nomad::launch_store_to_f32(src, stage, rows, pb.dim, pb.kpad, b->a.bf16, b->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dst, stage, static_cast<size_t>(rows) * pb.dim * sizeof(float), cudaMemcpyDeviceToHost,
                          b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(stage);
    if (e != cudaSuccess) return cuda_fail(e, "batch factor download");
  }
  return NOMAD_OK;
}

void nomad_gpu_batch_destroy(nomad_gpu_batch* b) {
  if (b) cudaSetDevice(b->device);
  release(b);
}

int nomad_gpu_batch_autotune(const nomad_gpu_batch_problem* problems, int32_t count, nomad_gpu_params* params,
                             int32_t epochs, nomad_gpu_batch_tune_trial* trials, int32_t max_trials,
                             int32_t* n_trials) {
  nomad::clear_last_error();
  if (!problems || count <= 0 || !params || epochs < 1 || max_trials < 0 || (max_trials > 0 && !trials))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_gpu_batch_autotune");
  if (params->exact) NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "exact = 1 runs every problem on one warp: nothing to tune");
  if (n_trials) *n_trials = 0;
  std::vector<nomad_gpu_batch_tune_trial> done;
  // one trial: a fresh batch, an untimed epoch, `epochs` timed ones
  auto measure = [&](nomad_gpu_batch_tune_trial& t) {
    nomad_gpu_params q = *params;
    q.batch_share = t.batch_share;
    nomad_gpu_batch* b = nullptr;
    t.status = nomad_gpu_batch_init(&b, problems, count, &q);
    if (t.status == NOMAD_OK) {
      nomad_gpu_epoch_stats st;
      t.status = nomad_gpu_batch_epoch(b, 1, &st);
      if (t.status == NOMAD_OK) t.status = nomad_gpu_batch_epoch(b, epochs, &st);
      if (t.status == NOMAD_OK) {
        t.device_ms = st.device_ms / epochs;
        t.large_problems = b->n_big;
      }
    }
    nomad_gpu_batch_destroy(b);
  };
  int32_t share = 0;
  const bool ok = nomad::batch_share_search(params->batch_share, measure, done, &share);
  const int32_t stored = std::min<int32_t>(max_trials, static_cast<int32_t>(done.size()));
  for (int32_t i = 0; i < stored; ++i) trials[i] = done[i];
  if (n_trials) *n_trials = stored;
  if (!ok) NOMAD_FAIL(done.front().status, "no large-problem threshold completed an epoch");
  params->batch_share = share;
  nomad::clear_last_error();  // a trial that failed left its detail behind
  return NOMAD_OK;
}

}  // extern "C"
