// ctx.cpp -- the C-ABI of libnomad_gpu (include/nomad_gpu.h): context lifetime, device
// memory, layout upload and the launch sequence of each call.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "common.h"
#include "launch.h"
#include "trace.h"
#include "tune.h"
#include "layout.h"

using nomad::DevFactors;

struct nomad_gpu_ctx {
  nomad_gpu_params prm{};
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  DevFactors f;
  std::vector<void*> allocs;
  int64_t device_bytes = 0;
  // rating sets (CSC by column)
  int2* train = nullptr;
  int64_t* train_ptr = nullptr;
  int64_t nnz_train = 0;
  int2* test = nullptr;
  int64_t* test_ptr = nullptr;
  int64_t nnz_test = 0;
  int64_t max_column = 0;
  // async NOMAD
  int4* segs = nullptr;
  int64_t* vl_ptr = nullptr;
  int32_t *tok_pos = nullptr, *tok_epoch = nullptr;
  int32_t *qnext = nullptr, *qtail = nullptr, *qnext0 = nullptr, *qtail0 = nullptr;
  int4 *tok_desc = nullptr, *tok_desc0 = nullptr;
  // pipelined kernel state
  unsigned long long *ring_lo = nullptr, *ring_hi = nullptr;
  unsigned mask_lo = 0, mask_hi = 0;
  unsigned *tails = nullptr, *heads = nullptr;
  int4 *mailbox = nullptr, *first_mail = nullptr;
  int4* segx = nullptr;
  int2* first_q = nullptr;
  int32_t* q_count = nullptr;
  unsigned long long* finish_ns = nullptr;  // [n+1]: per-token retire time, [n] = launch start
  int32_t n_priority = 0, long_visit = 14;
  int32_t cta_heavy = 0;  // priority tokens visit thread blocks (pipelined kernel)
  int32_t* ctrl = nullptr;
  unsigned long long *progress = nullptr, *stats = nullptr;
  double* err_sum = nullptr;
  int32_t P = 0, n_active = 0, grid = 0, wpb = 0;
  int64_t n_segments = 0;
  // DSGD
  int4* rates = nullptr;
  int64_t* blk_ptr = nullptr;
  int32_t* sched = nullptr;
  int32_t innerB = 0, col_blocks = 0;
  // bold driver (DSGD, DSGD++): learning rate of the next pass, objective after the
  // last one (< 0: not computed yet)
  double cur_lr = 0, last_obj = -1;
  int32_t* row_nnz = nullptr;  // ratings per row, for the objective (lazily counted)
  // step sizes per pass count
  float* steps = nullptr;
  int32_t n_steps = 0;
  // evaluation scratch
  double* partials = nullptr;
  double* sse_out = nullptr;
  int32_t sse_grid = 0;
  int32_t epochs_done = 0;
  int64_t h2d_bytes = 0, d2h_bytes = 0;
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

template <typename T>
int dalloc(nomad_gpu_ctx* c, T** p, size_t count) {
  *p = nullptr;
  const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    nomad::set_last_error("cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    cudaGetLastError();
    return NOMAD_ERR_OOM;
  }
  c->allocs.push_back(q);
  c->device_bytes += static_cast<int64_t>(bytes);
  *p = static_cast<T*>(q);
  return NOMAD_OK;
}

template <typename T>
int upload(nomad_gpu_ctx* c, T** p, const T* src, size_t count) {
  int rc = dalloc(c, p, count);
  if (rc) return rc;
  if (count) CK(cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  c->h2d_bytes += static_cast<int64_t>(count * sizeof(T));
  return NOMAD_OK;
}

#define RC(call)               \
  do {                         \
    int rc_ = (call);          \
    if (rc_) return rc_;       \
  } while (0)

int ensure_steps(nomad_gpu_ctx* c, int32_t needed) {
  if (needed <= c->n_steps) return NOMAD_OK;
  int32_t cap = std::max<int32_t>(64, c->n_steps);
  while (cap < needed) cap *= 2;
  std::vector<float> h(cap);
  for (int32_t e = 0; e < cap; ++e) h[e] = nomad::step_size_f32(c->prm.lrate, c->prm.drate, e);
  float* d = nullptr;
  RC(dalloc(c, &d, cap));
  CK(cudaMemcpyAsync(d, h.data(), cap * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->h2d_bytes += static_cast<int64_t>(cap * sizeof(float));
  c->steps = d;  // the previous table stays allocated until destroy (small)
  c->n_steps = cap;
  return NOMAD_OK;
}

// Upload a dense fp32 [rows x dim] host array into padded storage, in chunks through
// a bounded staging buffer.
int put_factor(nomad_gpu_ctx* c, void* dst, const float* src, int64_t rows) {
  const DevFactors& f = c->f;
  const int64_t chunk_rows = std::max<int64_t>(1, (int64_t(16) << 20) / std::max(f.dim, 1));
  float* stage = nullptr;
  CK(cudaMalloc(&stage, std::max<int64_t>(1, std::min(rows, chunk_rows)) * f.dim * sizeof(float)));
  const size_t esz = f.bf16 ? 2 : 4;
  int rc = NOMAD_OK;
  for (int64_t r0 = 0; r0 < rows && rc == NOMAD_OK; r0 += chunk_rows) {
    const int64_t nr = std::min(chunk_rows, rows - r0);
    cudaError_t e = cudaMemcpyAsync(stage, src + r0 * f.dim, nr * f.dim * sizeof(float),
                                    cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = nomad::launch_f32_to_store(stage, static_cast<char*>(dst) + r0 * f.kpad * esz, nr, f.dim,
                                     f.kpad, f.bf16, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "factor upload");
    c->h2d_bytes += nr * f.dim * static_cast<int64_t>(sizeof(float));
  }
  cudaFree(stage);
  return rc;
}

int get_factor(nomad_gpu_ctx* c, const void* src, float* dst, int64_t rows) {
  const DevFactors& f = c->f;
  const int64_t chunk_rows = std::max<int64_t>(1, (int64_t(16) << 20) / std::max(f.dim, 1));
  float* stage = nullptr;
  CK(cudaMalloc(&stage, std::max<int64_t>(1, std::min(rows, chunk_rows)) * f.dim * sizeof(float)));
  {  // pageable host memory only: touch its pages ahead of the copies
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, dst) == cudaSuccess && pa.type == cudaMemoryTypeUnregistered)
      nomad::prefault(dst, static_cast<size_t>(rows) * f.dim * sizeof(float), nomad::host_threads());
    cudaGetLastError();
  }
  const size_t esz = f.bf16 ? 2 : 4;
  int rc = NOMAD_OK;
  for (int64_t r0 = 0; r0 < rows && rc == NOMAD_OK; r0 += chunk_rows) {
    const int64_t nr = std::min(chunk_rows, rows - r0);
    cudaError_t e = nomad::launch_store_to_f32(static_cast<const char*>(src) + r0 * f.kpad * esz,
                                               stage, nr, f.dim, f.kpad, f.bf16, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dst + r0 * f.dim, stage, nr * f.dim * sizeof(float),
                          cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "factor download");
    c->d2h_bytes += nr * f.dim * static_cast<int64_t>(sizeof(float));
  }
  cudaFree(stage);
  return rc;
}

int upload_csc(nomad_gpu_ctx* c, const nomad::Csc& csc, int2** ratings, int64_t** ptr) {
  RC(upload(c, ptr, csc.col_ptr.data(), csc.col_ptr.size()));
  // two spare entries: 16-byte-rounded prefetches of a run may reach 8 bytes past its end
  const size_t n = csc.ratings.size();
  RC(dalloc(c, ratings, n + 2));
  CK(cudaMemsetAsync(*ratings + n, 0, 2 * sizeof(int2), c->stream));
  if (n) CK(cudaMemcpyAsync(*ratings, csc.ratings.data(), n * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
  c->h2d_bytes += static_cast<int64_t>(n * sizeof(int2));
  return NOMAD_OK;
}

// A rating set whose CSC is built on the device: row-major (the order the sort keeps),
// and few enough ratings for 32-bit sort indices.
bool device_csc_ok(const nomad_gpu_matrix& A) {
  return A.row_counts && A.nnz > 0 && A.nnz <= INT_MAX && A.cols && (A.vals_f64 || A.vals_f32);
}

// The CSC of a checked row-major set built on the device (csc_device.cu) into the context's
// buffers; its col_ptr (and with `with_ratings` the row of every rating, for the layout
// builds) copied to `host` when that is given.
int device_csc_set(nomad_gpu_ctx* c, const nomad_gpu_matrix& A, int32_t m, int32_t n, int2** ratings, int64_t** ptr,
                   nomad::Csc* host, bool with_ratings) {
  const size_t nnz = static_cast<size_t>(A.nnz);
  // two spare entries: 16-byte-rounded prefetches of a run may reach 8 bytes past its end
  RC(dalloc(c, ratings, nnz + 2));
  RC(dalloc(c, ptr, static_cast<size_t>(n) + 1));
  CK(cudaMemsetAsync(*ratings + nnz, 0, 2 * sizeof(int2), c->stream));
  int32_t dup = -1;
  int64_t bad = -1;
  const cudaError_t e = nomad::device_csc(A.nnz, m, n, A.row_counts, A.cols, A.vals_f64, A.vals_f32, *ratings, *ptr,
                                          &bad, &dup, &c->h2d_bytes, c->stream);
  if (bad >= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "column index %d out of range [0, %d)", A.cols[bad], n);
  CK(e);
  if (dup >= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "repeated (row, column) cell in column %d", dup);
  nomad::InitTrace trace;
  if (host) {
    host->m = m;
    host->n = n;
    host->col_ptr.resize(static_cast<size_t>(n) + 1);
    host->row_nnz.assign(A.row_counts, A.row_counts + m);
    CK(cudaMemcpyAsync(host->col_ptr.data(), *ptr, (static_cast<size_t>(n) + 1) * sizeof(int64_t),
                       cudaMemcpyDeviceToHost, c->stream));
    c->d2h_bytes += static_cast<int64_t>((static_cast<size_t>(n) + 1) * sizeof(int64_t));
    CK(cudaStreamSynchronize(c->stream));
    if (with_ratings) {  // the rows alone: all the layout builds read
      host->rows.resize(nnz);
      nomad::prefault(host->rows.data(), nnz * sizeof(int32_t), nomad::host_threads());
      CK(nomad::device_csc_rows(*ratings, A.nnz, host->rows.data(), c->stream));
      c->d2h_bytes += static_cast<int64_t>(nnz * sizeof(int32_t));
    }
    trace.mark("  csc: copies out");
  }
  return NOMAD_OK;
}

int reset_tokens(nomad_gpu_ctx* c) {
  const int32_t n = c->f.n;
  std::vector<int32_t> ep(static_cast<size_t>(std::max(n, 1)), c->epochs_done);
  CK(cudaMemsetAsync(c->tok_pos, 0, sizeof(int32_t) * std::max(n, 1), c->stream));
  CK(cudaMemcpyAsync(c->tok_epoch, ep.data(), sizeof(int32_t) * std::max(n, 1),
                     cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return NOMAD_OK;
}

// Test hook (debug bit 2): the host build of the same layout, compared with the device
// build field by field; NOMAD_ERR_BOUNDS names the first field that differs.
int check_device_layout(nomad_gpu_ctx* c, const nomad::Csc& train, const nomad_gpu_params& p, int64_t pri_min,
                        int32_t group, const nomad::AsyncLayout& L, int threads) {
  nomad::AsyncLayout H;
  RC(nomad::build_async_layout(train, c->P, p.balance, p.seed, pri_min, group, !p.exact, H, threads));
  std::vector<nomad::Segment> segs(static_cast<size_t>(c->n_segments));
  CK(cudaMemcpy(segs.data(), c->segs, segs.size() * sizeof(nomad::Segment), cudaMemcpyDeviceToHost));
  auto same_segs = [&] {
    if (segs.size() != H.segs.size()) return false;
    for (size_t i = 0; i < segs.size(); ++i)
      if (segs[i].start != H.segs[i].start || segs[i].len != H.segs[i].len || segs[i].worker != H.segs[i].worker)
        return false;
    return true;
  };
  const char* bad = nullptr;
  if (L.row_start != H.row_start) bad = "row blocks";
  else if (!same_segs()) bad = "visits";
  else if (L.vl_ptr != H.vl_ptr) bad = "visit offsets";
  else if (L.desc0 != H.desc0 || L.first_mail != H.first_mail) bad = "first visits";
  else if (L.first_q != H.first_q || L.q_count != H.q_count || L.qnext0 != H.qnext0 || L.qtail0 != H.qtail0)
    bad = "initial queues";
  else if (L.n_active != H.n_active || L.n_priority != H.n_priority || L.max_segment != H.max_segment ||
           L.max_column != H.max_column)
    bad = "counts";
  if (bad) NOMAD_FAIL(NOMAD_ERR_BOUNDS, "device layout differs from the host layout: %s", bad);
  return NOMAD_OK;
}

int init_impl(nomad_gpu_ctx* c, const nomad_gpu_problem* prob) {
  const nomad_gpu_params& p = c->prm;
  const int threads = nomad::host_threads();
  nomad::InitTrace trace;
  CK(cudaSetDevice(c->device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, c->device));
  if (prop.major * 10 + prop.minor != 103)
    NOMAD_FAIL(NOMAD_ERR_NO_DEVICE, "device %d is sm_%d%d; the library is compiled for sm_103a", c->device,
               prop.major, prop.minor);
  if (!prop.cooperativeLaunch) NOMAD_FAIL(NOMAD_ERR_NO_DEVICE, "device lacks cooperative launch");
  c->num_sms = prop.multiProcessorCount;
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&c->ev0));
  CK(cudaEventCreate(&c->ev1));
  trace.mark("device and stream");

  // ---- factors -----------------------------------------------------------------
  DevFactors& f = c->f;
  f.m = prob->m;
  f.n = prob->n;
  f.dim = p.dim;
  f.bf16 = p.precision == NOMAD_PREC_BF16_SR;
  // rows are whole 16-byte units (TMA bulk copies need it); a lane holds 4 values
  const int align = f.bf16 ? 8 : 4;
  f.kpad = (p.dim + align - 1) / align * align;
  f.nvec = f.kpad / 4;
  if (f.nvec > 128) NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "dim %d exceeds the supported maximum", p.dim);
  f.red_width = 1;
  while (f.red_width < std::min(f.nvec, 32)) f.red_width <<= 1;
  const size_t esz = f.bf16 ? 2 : 4;
  char* Wd = nullptr;
  char* Hd = nullptr;
  RC(dalloc(c, &Wd, static_cast<size_t>(f.m) * f.kpad * esz));
  RC(dalloc(c, &Hd, static_cast<size_t>(f.n) * f.kpad * esz));
  f.W = Wd;
  f.H = Hd;
  if (p.init == NOMAD_INIT_HASH && !(prob->W0 && prob->H0)) {
    CK(nomad::launch_init_hash(f, p.seed, c->stream));
  }
  // The reference init of W (parallel over its row parts) and of H (one sequential stream)
  // runs on two threads beside the CSC builds; the uploads follow.
  const bool host_w = !prob->W0 && p.init != NOMAD_INIT_HASH;
  const bool host_h = !prob->H0 && p.init != NOMAD_INIT_HASH;
  std::vector<float, nomad::NoInitAllocator<float>> Wh(host_w ? static_cast<size_t>(f.m) * f.dim : 0);
  std::vector<float, nomad::NoInitAllocator<float>> Hh(host_h ? static_cast<size_t>(f.n) * f.dim : 0);
  int rc_w = NOMAD_OK, rc_h = NOMAD_OK;
  std::thread tw, th;
  struct Join {  // no early return leaves a running thread behind
    std::thread& a;
    std::thread& b;
    ~Join() {
      if (a.joinable()) a.join();
      if (b.joinable()) b.join();
    }
  } join{tw, th};
  if (host_w) tw = std::thread([&] { rc_w = nomad_reference_init(f.m, 0, f.dim, p.seed, p.init_parts, Wh.data(), nullptr); });
  if (host_h) th = std::thread([&] { rc_h = nomad_reference_init(0, f.n, f.dim, p.seed, p.init_parts, nullptr, Hh.data()); });
  // ---- rating sets ---------------------------------------------------------------
  // Row-major sets are sorted into CSC order on the device (their row counts are checked
  // here first, their column indices on the device before the sort); COO input and sets
  // past INT_MAX ratings are sorted on the host.
  nomad::Csc train, test;
  const bool dev_train = device_csc_ok(prob->train), dev_test = device_csc_ok(prob->test);
  // the asynchronous modes' visit lists follow the training CSC onto the device
  const bool dev_layout = dev_train && p.mode == NOMAD_MODE_ASYNC;
  if (dev_train) RC(nomad::check_rating_set(prob->train, f.m, f.n, threads, false));
  else RC(nomad::build_csc(prob->train, f.m, f.n, train, threads));
  if (dev_test) RC(nomad::check_rating_set(prob->test, f.m, f.n, threads, false));
  else RC(nomad::build_csc(prob->test, f.m, f.n, test, threads));
  trace.mark("CSC checks / host builds (factor init beside it)");
  if (tw.joinable()) tw.join();
  if (th.joinable()) th.join();
  if (rc_w != NOMAD_OK || rc_h != NOMAD_OK) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "reference init of the factors failed");
  if (prob->W0) {
    RC(put_factor(c, f.W, prob->W0, f.m));
  } else if (host_w) {
    RC(put_factor(c, f.W, Wh.data(), f.m));
  }
  if (prob->H0) {
    RC(put_factor(c, f.H, prob->H0, f.n));
  } else if (host_h) {
    RC(put_factor(c, f.H, Hh.data(), f.n));
  }
  trace.mark("factors (init wait + upload)", c->stream);
  c->nnz_train = prob->train.nnz;
  c->nnz_test = prob->test.nnz;
  // a host layout build of the asynchronous modes reads the training CSC's rows, so then
  // they come back from the device (else only its column offsets)
  if (dev_train)
    RC(device_csc_set(c, prob->train, f.m, f.n, &c->train, &c->train_ptr, &train,
                      p.mode == NOMAD_MODE_ASYNC && (!dev_layout || (p.debug_flags & 4))));
  else RC(upload_csc(c, train, &c->train, &c->train_ptr));
  if (dev_test) RC(device_csc_set(c, prob->test, f.m, f.n, &c->test, &c->test_ptr, nullptr, false));
  else RC(upload_csc(c, test, &c->test, &c->test_ptr));
  for (int32_t j = 0; j < f.n; ++j)
    c->max_column = std::max<int64_t>(c->max_column, train.col_ptr[j + 1] - train.col_ptr[j]);
  trace.mark("CSC on the device", c->stream);

  // ---- mode-specific layout --------------------------------------------------------
  if (p.mode == NOMAD_MODE_ASYNC) {
    // exact kernel: up to 8 worker warps per block; pipelined kernel: up to 14 compute
    // warps (workers) plus the pop and push warps, fewer where the kernel was compiled
    // for smaller blocks (10 for fp32 rows, 12 for bf16: the occupancy query says so)
    if (p.exact)
      c->wpb = p.warps_per_block > 0 ? std::min(p.warps_per_block, 8) : 8;
    else
      c->wpb = p.warps_per_block > 0 ? std::min(p.warps_per_block, 14) : 14;
    const int nv = f.nvec <= 32 ? 1 : (f.nvec <= 64 ? 2 : 4);
    // pipelined kernel: long columns visit whole thread blocks (unless priority is off)
    int cta_heavy = !p.exact && p.priority_permille >= 0 ? 1 : 0;
    int bps = 0;
    if (p.exact) {
      CK(nomad::async_occupancy(f.bf16, nv, 1, c->wpb, f.kpad, &bps));
    } else {
      // fewer compute warps per block when long rows do not fit the shared memory, and
      // no block visits when their staged rows do not fit even beside one warp
      const int wpb0 = c->wpb;
      while (true) {
        CK(nomad::async2_occupancy(f.bf16, nv, c->wpb, f.kpad, cta_heavy, &bps));
        if (bps > 0) break;
        if (c->wpb > 1) {
          --c->wpb;
        } else if (cta_heavy) {
          cta_heavy = 0;
          c->wpb = wpb0;
        } else {
          break;
        }
      }
    }
    if (bps <= 0) NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "async kernel does not fit on an SM");
    if (p.blocks_per_sm > 0) bps = std::min(bps, p.blocks_per_sm);
    const int64_t capacity = static_cast<int64_t>(bps) * c->num_sms * c->wpb;
    c->P = static_cast<int32_t>(p.workers > 0 ? std::min<int64_t>(p.workers, capacity) : capacity);
    c->grid = (c->P + c->wpb - 1) / c->wpb;
    // blocked-path threshold: 14 for fp32 rows, 17 for bf16 (measured on the 480,189 x
    // 17,770 workload: bf16 epochs 0.9% shorter at 17-32 than at 14, fp32 no better)
    c->long_visit = p.long_visit > 0 ? p.long_visit : nomad::default_long_visit(f.bf16);
    // columns whose serial chain is long enough to set the epoch time skip the queue
    int64_t pri_min = 0;
    if (cta_heavy) {
      const int permille = p.priority_permille > 0 ? p.priority_permille : 50;
      pri_min = std::max<int64_t>(1, c->max_column * permille / 1000);
    }
    nomad::AsyncLayout L;
    const int32_t group = p.exact ? 1 : c->wpb;
    if (dev_layout) {
      // visit lists on the device from the device CSC; the host keeps the row blocks and
      // builds the initial queues from each column's first visit
      RC(nomad::async_layout_rows(train, c->P, p.balance, L, threads));
      trace.mark("  layout: row blocks (host)");
      nomad::DeviceLayout t;
      CK(nomad::device_layout_count(c->train, c->train_ptr, c->nnz_train, f.m, f.n, L.row_start.data(), c->P, group,
                                    pri_min, &t, c->stream));
      c->n_segments = t.nseg;
      RC(dalloc(c, &c->segs, static_cast<size_t>(t.nseg)));
      RC(dalloc(c, &c->vl_ptr, static_cast<size_t>(f.n) + 1));
      trace.mark("  layout: visit allocations");
      L.vl_ptr.resize(static_cast<size_t>(f.n) + 1);
      std::vector<nomad::Segment> firsts(static_cast<size_t>(f.n));
      static_assert(sizeof(nomad::Segment) == sizeof(int4), "a visit is {start lo, start hi, len, owner}");
      int32_t max_seg = 0;
      CK(nomad::device_layout_fill(c->train, c->train_ptr, c->nnz_train, f.n, group, !p.exact, pri_min, p.seed, &t,
                                   c->segs, c->vl_ptr, L.vl_ptr.data(), reinterpret_cast<int4*>(firsts.data()),
                                   &max_seg, c->stream));
      L.max_segment = max_seg;
      nomad::async_layout_queues(train, pri_min, firsts.data(), L);
      trace.mark("  layout: initial queues (host)");
      c->d2h_bytes += static_cast<int64_t>((static_cast<size_t>(f.n) + 1) * 8 + static_cast<size_t>(f.n) * 16);
      if (p.debug_flags & 4) RC(check_device_layout(c, train, p, pri_min, group, L, threads));
    } else {
      RC(nomad::build_async_layout(train, c->P, p.balance, p.seed, pri_min, group, !p.exact, L, threads));
      c->n_segments = static_cast<int64_t>(L.segs.size());
    }
    trace.mark("async layout build");
    c->cta_heavy = cta_heavy && pri_min > 0;
    c->n_active = L.n_active;
    c->n_priority = L.n_priority;
    RC(upload(c, &c->tok_desc0, reinterpret_cast<const int4*>(L.desc0.data()), L.desc0.size() / 4));
    RC(dalloc(c, &c->tok_desc, std::max<size_t>(L.desc0.size() / 4, 1)));
    if (!p.exact) {
      // rings hold at most every token of their class at once
      auto pow2 = [](int64_t x) { unsigned v = 2; while (v < x) v <<= 1; return v; };
      c->mask_lo = pow2(static_cast<int64_t>(c->n_active) + 1) - 1;
      c->mask_hi = pow2(static_cast<int64_t>(c->n_priority) + 1) - 1;
      RC(dalloc(c, &c->ring_lo, static_cast<size_t>(c->P) * (c->mask_lo + 1)));
      RC(dalloc(c, &c->ring_hi, static_cast<size_t>(c->grid) * (c->mask_hi + 1)));  // one per block
      // all-ones entries never match a head (their token field has bit 31 set)
      CK(cudaMemsetAsync(c->ring_lo, 0xff, static_cast<size_t>(c->P) * (c->mask_lo + 1) * 8, c->stream));
      CK(cudaMemsetAsync(c->ring_hi, 0xff, static_cast<size_t>(c->grid) * (c->mask_hi + 1) * 8, c->stream));
      RC(dalloc(c, &c->tails, 2 * static_cast<size_t>(c->P)));
      RC(dalloc(c, &c->heads, 2 * static_cast<size_t>(c->P)));
      CK(cudaMemsetAsync(c->tails, 0, 2 * static_cast<size_t>(c->P) * sizeof(unsigned), c->stream));
      CK(cudaMemsetAsync(c->heads, 0, 2 * static_cast<size_t>(c->P) * sizeof(unsigned), c->stream));
      RC(dalloc(c, &c->mailbox, 4 * static_cast<size_t>(std::max(f.n, 1))));
      RC(upload(c, &c->first_mail, reinterpret_cast<const int4*>(L.first_mail.data()), L.first_mail.size() / 4));
      RC(upload(c, &c->first_q, reinterpret_cast<const int2*>(L.first_q.data()), L.first_q.size() / 2));
      RC(upload(c, &c->q_count, L.q_count.data(), L.q_count.size()));
    }
    RC(dalloc(c, &c->finish_ns, static_cast<size_t>(f.n) + 1));
    if (!dev_layout) {
      RC(upload(c, &c->segs, reinterpret_cast<const int4*>(L.segs.data()), L.segs.size()));
      RC(upload(c, &c->vl_ptr, L.vl_ptr.data(), L.vl_ptr.size()));
    }
    if (!p.exact) {
      RC(dalloc(c, &c->segx, 3 * std::max<size_t>(static_cast<size_t>(c->n_segments), 1)));
      CK(nomad::launch_build_segx(c->segs, c->train, c->n_segments, c->segx, c->stream));
    }
    RC(upload(c, &c->qnext0, L.qnext0.data(), L.qnext0.size()));
    RC(upload(c, &c->qtail0, L.qtail0.data(), L.qtail0.size()));
    RC(dalloc(c, &c->qnext, L.qnext0.size()));
    RC(dalloc(c, &c->qtail, L.qtail0.size()));
    RC(dalloc(c, &c->tok_pos, f.n));
    RC(dalloc(c, &c->tok_epoch, f.n));
    RC(dalloc(c, &c->ctrl, 4));
    RC(dalloc(c, &c->progress, 1));
    RC(dalloc(c, &c->stats, 4));
    RC(dalloc(c, &c->err_sum, 1));
    RC(reset_tokens(c));
  } else if (p.mode == NOMAD_MODE_DSGD || p.mode == NOMAD_MODE_DSGDPP) {
    c->innerB = p.dsgd_inner_blocks > 0 ? p.dsgd_inner_blocks : 2 * c->num_sms * 4;
    c->col_blocks = p.mode == NOMAD_MODE_DSGDPP ? 2 * c->innerB : c->innerB;
    nomad::DsgdLayout D;
    RC(nomad::build_dsgd_layout(prob->train, f.m, f.n, c->innerB, c->col_blocks, D));
    RC(upload(c, &c->blk_ptr, D.blk_ptr.data(), D.blk_ptr.size()));
    RC(upload(c, &c->rates, reinterpret_cast<const int4*>(D.rates.data()), D.rates.size() / 4));
    RC(dalloc(c, &c->sched, static_cast<size_t>(c->col_blocks) * c->innerB));
  } else if (p.mode == NOMAD_MODE_REPLAY) {
    c->P = 1;
  } else {
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "unknown mode %d", p.mode);
  }
  trace.mark("mode layout upload", c->stream);
  if (!c->err_sum) RC(dalloc(c, &c->err_sum, 1));
  c->sse_grid = c->num_sms * 8;
  RC(dalloc(c, &c->partials, c->sse_grid));
  RC(dalloc(c, &c->sse_out, 5));  // train, test, objective: SSE, |W|, |H| terms
  c->cur_lr = p.lrate;
  RC(ensure_steps(c, 64));
  CK(cudaStreamSynchronize(c->stream));
  trace.mark("scratch");
  return NOMAD_OK;
}

int epoch_async(nomad_gpu_ctx* c, int32_t E, nomad_gpu_epoch_stats* st) {
  const int32_t n = c->f.n;
  const size_t qn = static_cast<size_t>(n) + 2 * static_cast<size_t>(c->P);
  const bool pipelined = !c->prm.exact;
  if (!pipelined) {
    if (c->prm.debug_flags & 1) {
      CK(nomad::launch_empty_queues(c->qnext, c->qtail, n, 2 * c->P, c->stream));
    } else {
      CK(cudaMemcpyAsync(c->qnext, c->qnext0, qn * sizeof(int32_t), cudaMemcpyDeviceToDevice, c->stream));
      CK(cudaMemcpyAsync(c->qtail, c->qtail0, 2 * static_cast<size_t>(c->P) * sizeof(int32_t),
                         cudaMemcpyDeviceToDevice, c->stream));
    }
  }
  CK(cudaMemsetAsync(c->ctrl, 0, 4 * sizeof(int32_t), c->stream));
  CK(cudaMemsetAsync(c->progress, 0, sizeof(unsigned long long), c->stream));
  CK(cudaMemsetAsync(c->stats, 0, 4 * sizeof(unsigned long long), c->stream));
  CK(cudaMemsetAsync(c->err_sum, 0, sizeof(double), c->stream));
  CK(cudaMemsetAsync(c->finish_ns, 0, (static_cast<size_t>(n) + 1) * sizeof(unsigned long long), c->stream));
  nomad::AsyncArgs a;
  a.f = c->f;
  a.ratings = c->train;
  a.segs = c->segs;
  a.vl_ptr = c->vl_ptr;
  a.tok_pos = c->tok_pos;
  a.tok_epoch = c->tok_epoch;
  a.tok_desc = c->tok_desc;
  a.heavy_min = c->long_visit;
  a.finish_ns = c->finish_ns;
  a.ring_lo = c->ring_lo;
  a.ring_hi = c->ring_hi;
  a.mask_lo = c->mask_lo;
  a.mask_hi = c->mask_hi;
  a.tails = c->tails;
  a.heads = c->heads;
  a.mailbox = c->mailbox;
  a.segx = c->segx;
  a.cta_heavy = c->cta_heavy;
  a.steps = c->steps;
  a.n_steps = c->n_steps;
  a.qnext = c->qnext;
  a.qtail = c->qtail;
  a.ctrl = c->ctrl;
  a.progress = c->progress;
  a.stats = c->stats;
  a.err_sum = c->err_sum;
  a.P = c->P;
  a.n_active = c->n_active;
  a.target_epoch = c->epochs_done + E;
  a.lambda = static_cast<float>(c->prm.reg);
  a.seed32 = static_cast<uint32_t>(c->prm.seed ^ (c->prm.seed >> 32));
  a.budget_ns = static_cast<int64_t>(std::max(c->prm.spin_budget_ms, 1)) * 1000000LL;
  a.exact = c->prm.exact;
  a.warps_per_block = c->wpb;
  a.grid = c->grid;
  a.debug_flags = c->prm.debug_flags;
  // Seeding reads the ring geometry (a.P) and must follow every assignment above; it is
  // part of the timed epoch.
  CK(cudaEventRecord(c->ev0, c->stream));
  if (pipelined && !(c->prm.debug_flags & 1))
    CK(nomad::launch_seed_queues(a, c->first_mail, c->first_q, c->q_count, n, c->epochs_done, c->stream));
  if (c->n_active > 0) {
    if (c->prm.exact)
      CK(nomad::launch_async(a, c->stream));
    else
      CK(nomad::launch_async2(a, c->stream));
  }
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  int32_t ctrl[4];
  unsigned long long stats[4];
  double esum = 0;
  CK(cudaMemcpy(ctrl, c->ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(stats, c->stats, sizeof(stats), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&esum, c->err_sum, sizeof(double), cudaMemcpyDeviceToHost));
  c->d2h_bytes += static_cast<int64_t>(sizeof(ctrl) + sizeof(stats) + sizeof(double));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (st) {
    st->updates = static_cast<int64_t>(stats[0]);
    st->hops = static_cast<int64_t>(stats[1]);
    st->failures = static_cast<int64_t>(stats[2]);
    st->device_ms = ms;
    st->online_sse = esum;
  }
  if (ctrl[1] != 0 || (c->n_active > 0 && ctrl[0] != c->n_active)) {
    RC(reset_tokens(c));
    if (pipelined) {
      CK(nomad::launch_drain_queues(a, c->stream));
      CK(cudaStreamSynchronize(c->stream));
    }
    if (ctrl[1] == 2) NOMAD_FAIL(NOMAD_ERR_BOUNDS, "device bounds check failed");
    NOMAD_FAIL(NOMAD_ERR_TIMEOUT,
               "async epoch stopped: %d of %d tokens finished, no progress for %d ms",
               ctrl[0], c->n_active, c->prm.spin_budget_ms);
  }
  return NOMAD_OK;
}

int epoch_replay(nomad_gpu_ctx* c, int32_t E, nomad_gpu_epoch_stats* st) {
  CK(cudaMemsetAsync(c->err_sum, 0, sizeof(double), c->stream));
  nomad::ReplayArgs a;
  a.f = c->f;
  a.ratings = c->train;
  a.col_ptr = c->train_ptr;
  a.steps = c->steps;
  a.first_epoch = c->epochs_done;
  a.n_epochs = E;
  a.lambda = static_cast<float>(c->prm.reg);
  a.seed32 = static_cast<uint32_t>(c->prm.seed ^ (c->prm.seed >> 32));
  a.err_sum = c->err_sum;
  CK(cudaEventRecord(c->ev0, c->stream));
  CK(nomad::launch_replay(a, c->stream));
  CK(cudaEventRecord(c->ev1, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  double esum = 0;
  CK(cudaMemcpy(&esum, c->err_sum, sizeof(double), cudaMemcpyDeviceToHost));
  if (st) {
    st->updates = c->nnz_train * E;
    st->hops = static_cast<int64_t>(c->f.n) * E;
    st->device_ms = ms;
    st->online_sse = esum;
  }
  return NOMAD_OK;
}

// The DSGD objective (calobj_mpi, sgd-mpi-omp.cpp:122-160): training SSE plus
// reg * (sum_i nnz_row(i) |w_i|^2 + sum_j nnz_col(j) |h_j|^2), all sums in FP64.
int objective(nomad_gpu_ctx* c, double* obj) {
  if (!c->row_nnz) {
    RC(dalloc(c, &c->row_nnz, c->f.m));
    CK(nomad::launch_count_rows(c->train, c->nnz_train, c->row_nnz, c->f.m, c->stream));
  }
  nomad::SseArgs a;
  a.f = c->f;
  a.partials = c->partials;
  a.grid = c->sse_grid;
  a.ratings = c->train;
  a.col_ptr = c->train_ptr;
  a.nnz = c->nnz_train;
  a.out = c->sse_out + 2;
  CK(nomad::launch_sse(a, c->stream));
  // the kernels share the partials scratch; stream order keeps them apart
  CK(nomad::launch_weighted_norm(c->f, true, c->row_nnz, nullptr, c->partials, c->sse_grid, c->sse_out + 3,
                                 c->stream));
  CK(nomad::launch_weighted_norm(c->f, false, nullptr, c->train_ptr, c->partials, c->sse_grid, c->sse_out + 4,
                                 c->stream));
  double h[3];
  CK(cudaMemcpyAsync(h, c->sse_out + 2, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->d2h_bytes += static_cast<int64_t>(sizeof(h));
  *obj = h[0] + c->prm.reg * (h[1] + h[2]);
  return NOMAD_OK;
}

// DSGD (sgd-mpi-omp.cpp:220-424) and DSGD++ (dsgdpp.cpp:300-540), one process:
// every pass runs its strata one launch after another (innerB strata for DSGD;
// 2*innerB for DSGD++, the first innerB over the left column half, the rest over the
// right half).  FIXED: step = 1.5*lrate/(1 + drate*iter^1.5) (sgd-mpi-omp.cpp:308-309,
// dsgdpp.cpp:358-359).  BOLD_DRIVER: the step is the running learning rate; after the
// pass the objective is recomputed and the rate multiplied by drate if the objective
// rose, else by 1.05 (sgd-mpi-omp.cpp:384-394, dsgdpp.cpp:512-521); the objective of
// the starting factors is computed once, before the first pass.
int epoch_dsgd(nomad_gpu_ctx* c, int32_t E, nomad_gpu_epoch_stats* st) {
  const bool pp = c->prm.mode == NOMAD_MODE_DSGDPP;
  const bool bold = c->prm.lr_strategy == NOMAD_LR_BOLD_DRIVER;
  nomad::DsgdArgs a;
  a.f = c->f;
  a.rates = c->rates;
  a.blk_ptr = c->blk_ptr;
  a.sched = c->sched;
  a.innerB = c->innerB;
  a.col_blocks = c->col_blocks;
  a.lambda = static_cast<float>(c->prm.reg);
  a.seed32 = static_cast<uint32_t>(c->prm.seed ^ (c->prm.seed >> 32));
  a.exact = c->prm.exact;
  const int32_t strata = pp ? 2 * c->innerB : c->innerB;
  std::vector<int32_t> sched;
  float total_ms = 0;
  if (bold && c->last_obj < 0) RC(objective(c, &c->last_obj));
  for (int32_t k = 0; k < E; ++k) {
    const int32_t iter = c->epochs_done + k + 1;
    if (pp)
      nomad::dsgdpp_schedule(c->innerB, iter, c->prm.dsgd_strategy, sched);
    else
      nomad::dsgd_schedule(c->innerB, iter, c->prm.dsgd_strategy, sched);
    CK(cudaMemcpyAsync(c->sched, sched.data(), sched.size() * sizeof(int32_t),
                       cudaMemcpyHostToDevice, c->stream));
    a.step = bold ? static_cast<float>(c->cur_lr)
                  : static_cast<float>(1.5 * c->prm.lrate / (1.0 + c->prm.drate * std::pow(iter, 1.5)));
    a.iter = iter;
    CK(cudaEventRecord(c->ev0, c->stream));
    for (int32_t s = 0; s < strata; ++s) CK(nomad::launch_dsgd_stratum(a, s, c->stream));
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    total_ms += ms;
    if (bold) {
      double obj = 0;
      RC(objective(c, &obj));
      c->cur_lr *= obj > c->last_obj ? c->prm.drate : 1.05;
      c->last_obj = obj;
    }
  }
  if (st) {
    st->updates = c->nnz_train * E;
    st->device_ms = total_ms;
    if (bold) {
      st->objective = c->last_obj;
      st->lrate = c->cur_lr;
    }
  }
  return NOMAD_OK;
}

}  // namespace

extern "C" {

int nomad_gpu_params_default(nomad_gpu_params* p) {
  if (!p) return NOMAD_ERR_INVALID_ARG;
  std::memset(p, 0, sizeof(*p));
  p->struct_size = sizeof(*p);
  // NomadOption defaults (Code/nomad/nomad_option.cpp:18-47)
  p->dim = 100;
  p->lrate = 0.001;
  p->drate = 0.1;
  p->reg = 1.0;
  p->seed = 12345;
  p->mode = NOMAD_MODE_ASYNC;
  p->precision = NOMAD_PREC_FP32;
  p->init = NOMAD_INIT_REFERENCE;
  p->init_parts = 1;
  p->balance = 1;
  p->spin_budget_ms = 2000;
  return NOMAD_OK;
}

int nomad_gpu_init(nomad_gpu_ctx** out, const nomad_gpu_problem* prob,
                   const nomad_gpu_params* params) {
  nomad::clear_last_error();
  if (!out || !prob || !params) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (params->struct_size != static_cast<int32_t>(sizeof(nomad_gpu_params)))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "params.struct_size %d != %zu (ABI mismatch)",
               params->struct_size, sizeof(nomad_gpu_params));
  if (prob->m < 0 || prob->n < 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "negative matrix size");
  if (params->dim <= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "dim must be positive");
  if (params->init_parts <= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "init_parts must be positive");
  if (params->precision != NOMAD_PREC_FP32 && params->precision != NOMAD_PREC_BF16_SR)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "unknown precision %d", params->precision);
  if (!(params->lrate >= 0) || !(params->drate >= 0) || !(params->reg >= 0))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "lrate, drate and reg must be non-negative");
  if (params->lr_strategy != NOMAD_LR_FIXED && params->lr_strategy != NOMAD_LR_BOLD_DRIVER)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "unknown lr_strategy %d", params->lr_strategy);
  if (params->lr_strategy == NOMAD_LR_BOLD_DRIVER && params->mode != NOMAD_MODE_DSGD &&
      params->mode != NOMAD_MODE_DSGDPP)
    NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "the bold driver is a DSGD / DSGD++ learning-rate strategy");
  std::unique_ptr<nomad_gpu_ctx> c(new nomad_gpu_ctx());
  c->prm = *params;
  if (c->prm.mode == NOMAD_MODE_REPLAY) c->prm.exact = 1;
  c->device = params->device;
  int rc = init_impl(c.get(), prob);
  if (rc) {
    std::string msg = nomad::last_error();
    nomad_gpu_destroy(c.release());
    nomad::set_last_error("%s", msg.c_str());
    return rc;
  }
  *out = c.release();
  return NOMAD_OK;
}

int nomad_gpu_epoch(nomad_gpu_ctx* c, int32_t n_epochs, nomad_gpu_epoch_stats* st) {
  nomad::clear_last_error();
  if (!c || n_epochs < 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments");
  if (st) std::memset(st, 0, sizeof(*st));
  const auto t0 = std::chrono::steady_clock::now();
  CK(cudaSetDevice(c->device));
  int rc = NOMAD_OK;
  if (n_epochs > 0) {
    RC(ensure_steps(c, c->epochs_done + n_epochs + 1));
    if (c->prm.mode == NOMAD_MODE_ASYNC)
      rc = epoch_async(c, n_epochs, st);
    else if (c->prm.mode == NOMAD_MODE_REPLAY)
      rc = epoch_replay(c, n_epochs, st);
    else
      rc = epoch_dsgd(c, n_epochs, st);
    if (rc == NOMAD_OK) c->epochs_done += n_epochs;
  }
  if (st) {
    st->epochs_done = c->epochs_done;
    st->host_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return rc;
}

int nomad_gpu_sse(nomad_gpu_ctx* c, double* train_sse, int64_t* train_count, double* test_sse,
                  int64_t* test_count) {
  nomad::clear_last_error();
  if (!c) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null context");
  CK(cudaSetDevice(c->device));
  nomad::SseArgs a;
  a.f = c->f;
  a.partials = c->partials;
  a.grid = c->sse_grid;
  // a set whose two outputs are both NULL is not evaluated
  const bool want_train = train_sse || train_count, want_test = test_sse || test_count;
  a.ratings = c->train;
  a.col_ptr = c->train_ptr;
  a.nnz = want_train ? c->nnz_train : 0;
  a.out = c->sse_out;
  CK(nomad::launch_sse(a, c->stream));
  a.ratings = c->test;
  a.col_ptr = c->test_ptr;
  a.nnz = want_test ? c->nnz_test : 0;
  a.out = c->sse_out + 1;
  CK(nomad::launch_sse(a, c->stream));
  double h[2];
  CK(cudaMemcpyAsync(h, c->sse_out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->d2h_bytes += static_cast<int64_t>(sizeof(h));
  if (train_sse) *train_sse = h[0];
  if (test_sse) *test_sse = h[1];
  if (train_count) *train_count = c->nnz_train;
  if (test_count) *test_count = c->nnz_test;
  return NOMAD_OK;
}

int nomad_gpu_rmse(nomad_gpu_ctx* c, double* train_rmse, double* test_rmse) {
  double s0 = 0, s1 = 0;
  int64_t c0 = 0, c1 = 0;
  int rc = nomad_gpu_sse(c, train_rmse ? &s0 : nullptr, train_rmse ? &c0 : nullptr, test_rmse ? &s1 : nullptr,
                         test_rmse ? &c1 : nullptr);
  if (rc) return rc;
  if (train_rmse) *train_rmse = c0 ? std::sqrt(s0 / c0) : NAN;
  if (test_rmse) *test_rmse = c1 ? std::sqrt(s1 / c1) : NAN;
  return NOMAD_OK;
}

int nomad_gpu_get_factors(nomad_gpu_ctx* c, float* W, float* H) {
  nomad::clear_last_error();
  if (!c) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null context");
  CK(cudaSetDevice(c->device));
  if (W) RC(get_factor(c, c->f.W, W, c->f.m));
  if (H) RC(get_factor(c, c->f.H, H, c->f.n));
  return NOMAD_OK;
}

int nomad_gpu_set_factors(nomad_gpu_ctx* c, const float* W, const float* H) {
  nomad::clear_last_error();
  if (!c) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null context");
  CK(cudaSetDevice(c->device));
  if (W) RC(put_factor(c, c->f.W, W, c->f.m));
  if (H) RC(put_factor(c, c->f.H, H, c->f.n));
  return NOMAD_OK;
}

int nomad_gpu_set_epochs_done(nomad_gpu_ctx* c, int32_t epochs_done) {
  nomad::clear_last_error();
  if (!c || epochs_done < 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments");
  CK(cudaSetDevice(c->device));
  c->epochs_done = epochs_done;
  // the exact kernel keeps each token's pass count on the device between calls
  if (c->tok_epoch) RC(reset_tokens(c));
  return NOMAD_OK;
}

int nomad_gpu_objective(nomad_gpu_ctx* c, double* obj) {
  nomad::clear_last_error();
  if (!c || !obj) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments");
  CK(cudaSetDevice(c->device));
  return objective(c, obj);
}

int nomad_gpu_save_checkpoint(nomad_gpu_ctx* c, const char* path) {
  nomad::clear_last_error();
  if (!c || !path) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments");
  std::vector<float> W(static_cast<size_t>(c->f.m) * c->f.dim), H(static_cast<size_t>(c->f.n) * c->f.dim);
  RC(nomad_gpu_get_factors(c, W.data(), H.data()));
  nomad_io_checkpoint_info info{c->f.m, c->f.n, c->f.dim, c->epochs_done, 0.0, -1.0};
  if (c->prm.lr_strategy == NOMAD_LR_BOLD_DRIVER) {
    info.lrate = c->cur_lr;
    info.objective = c->last_obj;
  }
  return nomad_io_write_checkpoint(path, &info, W.data(), H.data());
}

int nomad_gpu_load_checkpoint(nomad_gpu_ctx* c, const char* path) {
  nomad::clear_last_error();
  if (!c || !path) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments");
  std::vector<float> W(static_cast<size_t>(c->f.m) * c->f.dim), H(static_cast<size_t>(c->f.n) * c->f.dim);
  nomad_io_checkpoint_info info;
  RC(nomad_io_read_checkpoint(path, c->f.m, c->f.n, c->f.dim, W.data(), H.data(), &info));
  if (c->prm.lr_strategy == NOMAD_LR_BOLD_DRIVER && info.lrate <= 0)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "checkpoint %s holds no bold-driver learning rate", path);
  RC(nomad_gpu_set_factors(c, W.data(), H.data()));
  if (c->prm.lr_strategy == NOMAD_LR_BOLD_DRIVER) {
    c->cur_lr = info.lrate;
    c->last_obj = info.objective;
  }
  return nomad_gpu_set_epochs_done(c, info.epochs_done);
}

int nomad_gpu_get_info(nomad_gpu_ctx* c, nomad_gpu_info* info) {
  if (!c || !info) return NOMAD_ERR_INVALID_ARG;
  std::memset(info, 0, sizeof(*info));
  info->m = c->f.m;
  info->n = c->f.n;
  info->dim = c->f.dim;
  info->dim_padded = c->f.kpad;
  info->nnz_train = c->nnz_train;
  info->nnz_test = c->nnz_test;
  info->workers = c->P;
  info->active_tokens = c->n_active;
  info->segments = c->n_segments;
  info->max_column = c->max_column;
  info->grid_blocks = c->grid;
  info->block_threads = (c->prm.mode == NOMAD_MODE_ASYNC && !c->prm.exact ? c->wpb + 2 : c->wpb) * 32;
  info->num_sms = c->num_sms;
  info->inner_blocks = c->innerB;
  info->device_bytes = c->device_bytes;
  info->mode = c->prm.mode;
  info->precision = c->prm.precision;
  info->h2d_bytes = c->h2d_bytes;
  info->d2h_bytes = c->d2h_bytes;
  info->priority_tokens = c->cta_heavy ? c->n_priority : 0;
  info->reserved0 = 0;
  return NOMAD_OK;
}

void nomad_gpu_destroy(nomad_gpu_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void* p : c->allocs) cudaFree(p);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* nomad_gpu_strerror(int status) {
  switch (status) {
    case NOMAD_OK: return "ok";
    case NOMAD_ERR_INVALID_ARG: return "invalid argument";
    case NOMAD_ERR_CUDA: return "CUDA runtime error";
    case NOMAD_ERR_OOM: return "out of memory";
    case NOMAD_ERR_TIMEOUT: return "device wait timed out";
    case NOMAD_ERR_BOUNDS: return "device bounds check failed";
    case NOMAD_ERR_IO: return "I/O error";
    case NOMAD_ERR_FORMAT: return "not a train.dat/test.dat binary matrix";
    case NOMAD_ERR_NO_DEVICE: return "no usable sm_103 device";
    case NOMAD_ERR_UNSUPPORTED: return "unsupported option combination";
    default: return "unknown status";
  }
}

const char* nomad_gpu_last_error(void) { return nomad::last_error(); }

int nomad_gpu_autotune(const nomad_gpu_problem* prob, nomad_gpu_params* params, int32_t epochs,
                       nomad_gpu_tune_trial* trials, int32_t max_trials, int32_t* n_trials) {
  nomad::clear_last_error();
  if (!prob || !params || epochs < 1 || max_trials < 0 || (max_trials > 0 && !trials))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_gpu_autotune");
  if (params->mode != NOMAD_MODE_ASYNC || params->exact)
    NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "autotuning covers the ASYNC kernel (exact = 0)");
  if (n_trials) *n_trials = 0;
  std::vector<nomad_gpu_tune_trial> done;
  // one trial: a fresh context, an untimed epoch, `epochs` timed ones
  auto measure = [&](nomad_gpu_tune_trial& t) {
    nomad_gpu_params q = *params;
    q.warps_per_block = t.warps_per_block;
    q.priority_permille = t.priority_permille;
    q.long_visit = t.long_visit;
    nomad_gpu_ctx* c = nullptr;
    t.status = nomad_gpu_init(&c, prob, &q);
    if (t.status == NOMAD_OK) {
      nomad_gpu_epoch_stats st;
      t.status = nomad_gpu_epoch(c, 1, &st);
      double ms = 0;
      for (int32_t e = 0; e < epochs && t.status == NOMAD_OK; ++e) {
        t.status = nomad_gpu_epoch(c, 1, &st);
        ms += st.device_ms;
      }
      if (t.status == NOMAD_OK) {
        nomad_gpu_info info;
        nomad_gpu_get_info(c, &info);
        t.warps_per_block = info.block_threads / 32 - 2;  // what the kernel ran with
        t.device_ms = ms / epochs;
      }
    }
    nomad_gpu_destroy(c);
  };
  int32_t wpb = 0, pri = 0, lv = 0;
  const bool ok = nomad::tune_descent(params->priority_permille, params->long_visit, measure, done, &wpb, &pri, &lv,
                                      nomad::default_long_visit(params->precision == NOMAD_PREC_BF16_SR));
  const int32_t stored = std::min<int32_t>(max_trials, static_cast<int32_t>(done.size()));
  for (int32_t i = 0; i < stored; ++i) trials[i] = done[i];
  if (n_trials) *n_trials = stored;
  if (!ok) NOMAD_FAIL(done.front().status, "no configuration completed an epoch");
  params->warps_per_block = wpb;
  params->priority_permille = pri;
  params->long_visit = lv;
  nomad::clear_last_error();  // a trial that failed left its detail behind
  return NOMAD_OK;
}

int nomad_gpu_token_finish_times(nomad_gpu_ctx* c, double* seconds) {
  nomad::clear_last_error();
  if (!c || !seconds) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null argument");
  if (c->prm.mode != NOMAD_MODE_ASYNC || !c->finish_ns)
    NOMAD_FAIL(NOMAD_ERR_UNSUPPORTED, "token finish times exist in ASYNC mode only");
  CK(cudaSetDevice(c->device));
  const int32_t n = c->f.n;
  std::vector<unsigned long long> t(static_cast<size_t>(n) + 1);
  CK(cudaMemcpy(t.data(), c->finish_ns, t.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  c->d2h_bytes += static_cast<int64_t>(t.size() * sizeof(unsigned long long));
  const unsigned long long t0 = t[n];
  for (int32_t j = 0; j < n; ++j)
    seconds[j] = (t[j] && t0 && t[j] >= t0) ? static_cast<double>(t[j] - t0) * 1e-9 : 0.0;
  return NOMAD_OK;
}

int nomad_gpu_device_ok(int32_t device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return 0;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return 0;
  return prop.major * 10 + prop.minor == 103 ? 1 : 0;
}

}  // extern "C"
