// nomad_oracle.cpp -- CPU restatement of NOMAD's hot path (TEST INFRASTRUCTURE ONLY).
//
// This file is the checker for the GPU library.  It is loaded by tests/, by
// __graft_entry__.smoke() and by bench.py's cpu_baseline / reference leg, never by the
// product.  Every function cites the reference lines it restates; the arithmetic is
// written so that, compiled with -ffp-contract=off, each scalar operation rounds the
// way the reference's own scalar loops do.
#include "nomad_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <fstream>
#include <mutex>
#include <numeric>
#include <queue>
#include <random>
#include <thread>
#include <vector>

namespace {

constexpr int32_t kMatFileClassId = 1211216;  // nb_data.cpp:14
constexpr int32_t kLongFileClassId = 1015;    // nb_data.cpp:15

// nb_main.cpp:514-515 (fork, S = double) and nomad_body.hpp:326-327 (S = float):
// lrate and drate are held in S, the expression is evaluated in double and the
// result converted to S.
template <typename S>
S step_size(double lrate, double drate, int32_t cnt) {
  const S learn_rate = static_cast<S>(lrate);
  const S decay_rate = static_cast<S>(drate);
  return static_cast<S>(learn_rate * 1.5 /
                        (1.0 + decay_rate * std::pow(cnt + 1, 1.5)));
}

// One column visit over the ratings [b, e) of a CSC: nb_main.cpp:520-542.
//   cur = inner_product(col, col+dim, row, -v)   -> -v + c0*r0 + c1*r1 + ...
//   err += cur*cur
//   row[i] -= step*(cur*col[i] + lambda*tmp);  col[i] -= step*(cur*tmp + lambda*col[i])
template <typename S>
int64_t visit_column(S* col, S* W, int32_t dim, const int32_t* rows,
                     const S* vals, int64_t b, int64_t e, S step, S lambda,
                     double* err) {
  for (int64_t o = b; o < e; ++o) {
    S* row = W + static_cast<int64_t>(dim) * rows[o];
    S cur = -vals[o];
    for (int32_t i = 0; i < dim; ++i) cur = cur + col[i] * row[i];
    if (err) *err += cur * cur;
    for (int32_t i = 0; i < dim; ++i) {
      S tmp = row[i];
      row[i] -= step * (cur * col[i] + lambda * tmp);
      col[i] -= step * (cur * tmp + lambda * col[i]);
    }
  }
  return e - b;
}

template <typename S>
std::vector<S> cast_vals(const double* vals, int64_t nnz) {
  // realdata_body.hpp:172 casts every value to the scalar type on load.
  std::vector<S> out(static_cast<size_t>(nnz));
  for (int64_t i = 0; i < nnz; ++i) out[i] = static_cast<S>(vals[i]);
  return out;
}

template <typename S>
int replay(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
           const int32_t* row_idx, const double* vals, S* W, S* H,
           int32_t first_epoch, int32_t n_epochs, double lrate, double drate,
           double reg, double* epoch_err) {
  if (m < 0 || n < 0 || dim <= 0 || n_epochs < 0 || first_epoch < 0) return -1;
  const int64_t nnz = col_ptr[n];
  std::vector<S> v = cast_vals<S>(vals, nnz);
  const S lambda = static_cast<S>(reg);
  // One worker: set_perm gives perm = {0}; after each visit pos_ >= 1 so the token
  // goes back to queue 0 (nb_main.cpp:554-558).  The queue is FIFO and starts in
  // column order (nb_main.cpp:82-97), so visits run 0..n-1, 0..n-1, ...; the visit
  // counter of every column equals the epoch number.
  for (int32_t ep = 0; ep < n_epochs; ++ep) {
    const int32_t cnt = first_epoch + ep;
    const S step = step_size<S>(lrate, drate, cnt);
    double err = 0.0;
    for (int32_t j = 0; j < n; ++j) {
      visit_column<S>(H + static_cast<int64_t>(dim) * j, W, dim, row_idx, v.data(),
                      col_ptr[j], col_ptr[j + 1], step, lambda, &err);
    }
    if (epoch_err) epoch_err[ep] = err;
  }
  return 0;
}

// nb_main.cpp:617-653 (fork) / nomad_body.hpp:427-456 (legacy float).
template <typename S>
int sse(int32_t n, int32_t dim, const int64_t* col_ptr, const int32_t* row_idx,
        const double* vals, const S* W, const S* H, double* out_sse,
        int64_t* out_count) {
  double s = 0.0;
  int64_t c = 0;
  for (int32_t j = 0; j < n; ++j) {
    const S* col = H + static_cast<int64_t>(dim) * j;
    for (int64_t o = col_ptr[j]; o < col_ptr[j + 1]; ++o) {
      const S* row = W + static_cast<int64_t>(dim) * row_idx[o];
      S cur = -static_cast<S>(vals[o]);
      for (int32_t i = 0; i < dim; ++i) cur += col[i] * row[i];
      s += cur * cur;
      ++c;
    }
  }
  *out_sse = s;
  *out_count = c;
  return 0;
}

// ---------------------------------------------------------------------------------
// Asynchronous NOMAD on host threads (nb_main.cpp:415-572, single rank).
// ---------------------------------------------------------------------------------
template <typename S>
struct Token {  // ColumnData, pool.h:11-37
  int32_t col_index;
  int32_t pos;
  int32_t epoch;  // completed passes over the permutation (epoch mode only)
  double error;
  std::vector<int32_t> perm;
  S* values;  // points into H
};

template <typename S>
struct WorkerQueue {  // tbb::concurrent_queue stand-in (nomad_body.h:31)
  std::mutex mu;
  std::deque<Token<S>*> q;
  void push(Token<S>* t) {
    std::lock_guard<std::mutex> g(mu);
    q.push_back(t);
  }
  bool try_pop(Token<S>*& t) {
    std::lock_guard<std::mutex> g(mu);
    if (q.empty()) return false;
    t = q.front();
    q.pop_front();
    return true;
  }
};

template <typename S>
int async_run(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
              const int32_t* row_idx, const double* vals, S* W, S* H,
              int32_t nthreads, int32_t n_epochs, double timeout_sec,
              double lrate, double drate, double reg, uint64_t seed,
              int64_t* updates, int64_t* failures, double* train_seconds) {
  if (nthreads <= 0 || dim <= 0 || m < 0 || n < 0) return -1;
  if (n_epochs <= 0 && !(timeout_sec > 0)) return -1;
  const int32_t P = nthreads;
  // Row partition of read_data (nb_data.cpp:83-89): ceil(m/P) rows per part.
  const int32_t rows_per_part = m / P + ((m % P > 0) ? 1 : 0);
  struct LocalCsc {
    int32_t min_row = 0;
    std::vector<int64_t> col_offset;
    std::vector<int32_t> row_idx;
    std::vector<S> row_val;
  };
  std::vector<LocalCsc> local(P);
  for (int32_t p = 0; p < P; ++p) {
    const int32_t lo = std::min<int64_t>(static_cast<int64_t>(rows_per_part) * p, m);
    const int32_t hi = std::min<int64_t>(static_cast<int64_t>(rows_per_part) * (p + 1), m);
    LocalCsc& L = local[p];
    L.min_row = lo;
    L.col_offset.assign(n + 1, 0);
    for (int32_t j = 0; j < n; ++j) {
      // rows ascending inside a column: the part's entries are one contiguous run
      const int32_t* b = row_idx + col_ptr[j];
      const int32_t* e = row_idx + col_ptr[j + 1];
      const int32_t* lb = std::lower_bound(b, e, lo);
      const int32_t* ub = std::lower_bound(lb, e, hi);
      for (const int32_t* it = lb; it != ub; ++it) {
        L.row_idx.push_back(*it - lo);  // relative row index (nb_data.cpp:137)
        L.row_val.push_back(static_cast<S>(vals[it - row_idx]));
      }
      L.col_offset[j + 1] = static_cast<int64_t>(L.row_idx.size());
    }
  }

  std::vector<WorkerQueue<S>> queues(P);
  std::vector<Token<S>> tokens(n);
  // nb_main.cpp:79-96: one rng_temp(seed + rank + 137) draws every column's
  // permutation in column order; set_perm = identity then std::shuffle (pool.cpp:32-38).
  std::mt19937_64 rng_temp(seed + 0 + 137);
  for (int32_t j = 0; j < n; ++j) {
    Token<S>& t = tokens[j];
    t.col_index = j;
    t.pos = 0;
    t.epoch = 0;
    t.error = 0.0;
    t.perm.resize(P);
    for (int32_t i = 0; i < P; ++i) t.perm[i] = i;
    std::shuffle(t.perm.begin(), t.perm.end(), rng_temp);
    t.values = H + static_cast<int64_t>(dim) * j;
    queues[t.perm[t.pos]].push(&t);
  }

  std::atomic<bool> stop{false};
  std::atomic<int32_t> retired{0};
  std::vector<int64_t> num_updates(P, 0), num_failures(P, 0);
  const S lambda = static_cast<S>(reg);
  const int32_t num_reuse = 1;

  auto updater = [&](int32_t p) {
    LocalCsc& L = local[p];
    S* latent_rows = W + static_cast<int64_t>(dim) * L.min_row;
    std::vector<int32_t> col_update_counts(n, 0);  // nb_main.cpp:458-459
    int64_t u = 0, f = 0;
    while (!stop.load(std::memory_order_relaxed)) {
      Token<S>* t = nullptr;
      if (queues[p].try_pop(t)) {
        const int32_t c = t->col_index;
        const S step = step_size<S>(lrate, drate, col_update_counts[c]);
        u += visit_column<S>(t->values, latent_rows, dim, L.row_idx.data(),
                             L.row_val.data(), L.col_offset[c], L.col_offset[c + 1],
                             step, lambda, &t->error);
        col_update_counts[c]++;
        // routing, nb_main.cpp:551-565 (mpi_size == 1 branch)
        t->pos++;
        if (t->pos >= P * num_reuse) {
          t->pos = 0;
          if (n_epochs > 0 && ++t->epoch >= n_epochs) {
            if (retired.fetch_add(1) + 1 == n) stop.store(true);
            continue;
          }
        }
        queues[t->perm[t->pos % P]].push(t);
      } else {
        ++f;
        std::this_thread::yield();
      }
    }
    num_updates[p] = u;
    num_failures[p] = f;
  };

  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> threads;
  if (n == 0) stop.store(true);
  for (int32_t p = 0; p < P; ++p) threads.emplace_back(updater, p);
  if (n_epochs <= 0) {
    std::this_thread::sleep_for(std::chrono::duration<double>(timeout_sec));
    stop.store(true);
  }
  for (auto& th : threads) th.join();
  auto t1 = std::chrono::steady_clock::now();
  if (updates) *updates = std::accumulate(num_updates.begin(), num_updates.end(), int64_t(0));
  if (failures) *failures = std::accumulate(num_failures.begin(), num_failures.end(), int64_t(0));
  if (train_seconds) *train_seconds = std::chrono::duration<double>(t1 - t0).count();
  return 0;
}

// ---------------------------------------------------------------------------------
// Asynchronous NOMAD with P workers under a deterministic timing model.
//
// The reference with --nthreads P (one rank) is nondeterministic: which token a worker
// pops depends on thread timing.  This restatement runs the same algorithm on one host
// thread as a discrete-event simulation, so that a P-worker trajectory can be computed
// exactly and repeatably:
//  * rows: P contiguous parts, either ceil(m/P) rows each (read_data,
//    nb_data.cpp:83-89) or parts of about nnz/P ratings each;
//  * routes: each column's permutation of the P workers drawn as nb_main.cpp:79-96 does
//    (one mt19937_64(seed + 137), set_perm = identity + std::shuffle, pool.cpp:32-38, in
//    column order); a visit to a worker without ratings of the column changes nothing
//    (nb_main.cpp:520 runs zero iterations), so the route keeps only the other workers;
//  * step: every worker sees a column once per pass, so its per-worker count
//    col_update_counts (nb_main.cpp:458-459, 544) equals the pass number;
//  * time: a visit of len ratings occupies its worker for visit_cost + rating_cost*len,
//    a token reaches its next worker hop_cost after the visit ends, a worker takes its
//    queue in FIFO order (tbb::concurrent_queue) and ties are broken by event order.
// Each epoch every token starts at its route's first worker, queues filled in column
// order.  The per-visit arithmetic is visit_column (nb_main.cpp:520-542) over the
// worker's run of the column (rows ascending, a contiguous run of the CSC).
// ---------------------------------------------------------------------------------
template <typename S>
int async_sim(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr, const int32_t* row_idx,
              const double* vals, S* W, S* H, int32_t P, int32_t partition, int32_t first_epoch,
              int32_t n_epochs, double lrate, double drate, double reg, uint64_t seed, double visit_cost,
              double rating_cost, double hop_cost, double* epoch_err) {
  if (P <= 0 || dim <= 0 || m < 0 || n < 0 || n_epochs < 0 || first_epoch < 0) return -1;
  const int64_t nnz = n > 0 ? col_ptr[n] : 0;
  // row parts: part_lo[p] .. part_lo[p + 1]
  std::vector<int32_t> part_lo(P + 1, m);
  if (partition == 0) {
    const int64_t rpp = m / P + ((m % P > 0) ? 1 : 0);
    for (int32_t p = 0; p <= P; ++p) part_lo[p] = static_cast<int32_t>(std::min<int64_t>(rpp * p, m));
  } else {
    std::vector<int64_t> cnt(static_cast<size_t>(m) + 1, 0);
    for (int64_t o = 0; o < nnz; ++o) cnt[row_idx[o] + 1]++;
    for (int32_t r = 0; r < m; ++r) cnt[r + 1] += cnt[r];
    int32_t r = 0;
    for (int32_t p = 0; p < P; ++p) {
      const int64_t goal = (nnz * p + P - 1) / P;
      while (r < m && cnt[r] < goal) ++r;
      part_lo[p] = r;
    }
    part_lo[P] = m;
  }
  std::vector<int32_t> row_part(m);
  for (int32_t p = 0; p < P; ++p)
    for (int32_t r = part_lo[p]; r < part_lo[p + 1]; ++r) row_part[r] = p;
  // each column's visits {worker, start, len} in permutation order
  struct Visit {
    int32_t worker;
    int32_t len;
    int64_t start;
  };
  std::vector<int64_t> vptr(static_cast<size_t>(n) + 1, 0);
  std::vector<Visit> visits;
  std::vector<int32_t> perm(P), inv(P);
  std::mt19937_64 rng_temp(seed + 0 + 137);
  for (int32_t j = 0; j < n; ++j) {
    for (int32_t i = 0; i < P; ++i) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), rng_temp);
    for (int32_t i = 0; i < P; ++i) inv[perm[i]] = i;
    const size_t first = visits.size();
    for (int64_t o = col_ptr[j]; o < col_ptr[j + 1];) {
      const int32_t w = row_part[row_idx[o]];
      int64_t e = o + 1;
      while (e < col_ptr[j + 1] && row_part[row_idx[e]] == w) ++e;
      visits.push_back({w, static_cast<int32_t>(e - o), o});
      o = e;
    }
    std::sort(visits.begin() + first, visits.end(),
              [&](const Visit& a, const Visit& b) { return inv[a.worker] < inv[b.worker]; });
    vptr[j + 1] = static_cast<int64_t>(visits.size());
  }
  std::vector<S> sv;
  const S* v = nullptr;
  if (sizeof(S) == sizeof(double)) {
    v = reinterpret_cast<const S*>(vals);
  } else {
    sv = cast_vals<S>(vals, nnz);
    v = sv.data();
  }
  const S lambda = static_cast<S>(reg);
  struct Event {
    double t;
    int64_t seq;
    int32_t kind;  // 0: a worker's visit ends, 1: a token arrives
    int32_t a;     // worker (kind 0) or token (kind 1)
    int32_t b;     // target worker (kind 1)
    bool operator>(const Event& o) const { return t != o.t ? t > o.t : seq > o.seq; }
  };
  for (int32_t ep = first_epoch; ep < first_epoch + n_epochs; ++ep) {
    const S step = step_size<S>(lrate, drate, ep);
    std::vector<std::deque<int32_t>> q(P);
    std::vector<int32_t> cur(P, -1), pos(n, 0);
    std::priority_queue<Event, std::vector<Event>, std::greater<Event>> heap;
    int64_t seq = 0;
    double err = 0.0;
    auto start = [&](int32_t w, double t) {
      const int32_t j = q[w].front();
      q[w].pop_front();
      cur[w] = j;
      const Visit& vi = visits[vptr[j] + pos[j]];
      visit_column<S>(H + static_cast<int64_t>(dim) * j, W, dim, row_idx, v, vi.start, vi.start + vi.len, step,
                      lambda, &err);
      heap.push({t + visit_cost + rating_cost * vi.len, seq++, 0, w, 0});
    };
    for (int32_t j = 0; j < n; ++j)
      if (vptr[j + 1] > vptr[j]) q[visits[vptr[j]].worker].push_back(j);
    for (int32_t w = 0; w < P; ++w)
      if (!q[w].empty()) start(w, 0.0);
    while (!heap.empty()) {
      const Event e = heap.top();
      heap.pop();
      if (e.kind == 0) {
        const int32_t w = e.a, j = cur[w];
        cur[w] = -1;
        if (++pos[j] < vptr[j + 1] - vptr[j]) heap.push({e.t + hop_cost, seq++, 1, j, visits[vptr[j] + pos[j]].worker});
        if (!q[w].empty()) start(w, e.t);
      } else {
        q[e.b].push_back(e.a);
        if (cur[e.b] < 0) start(e.b, e.t);
      }
    }
    if (epoch_err) epoch_err[ep - first_epoch] = err;
  }
  return 0;
}

// ---------------------------------------------------------------------------------
// DSGD (Code/competitor/sgd-mpi-omp.cpp), one process.
// ---------------------------------------------------------------------------------

// glibc rand() stream without touching the process-global state: srand(s) seeds the
// TYPE_3 additive generator exactly as initstate_r with a 128-byte buffer does.
struct GlibcRand {
  struct random_data data {};
  char state[128];
  explicit GlibcRand(unsigned seed) {
    data.state = nullptr;
    initstate_r(seed, state, sizeof(state), &data);
  }
  int next() {
    int32_t r;
    random_r(&data, &r);
    return r;
  }
};

// std::random_shuffle(first, last) as libstdc++ defines it: for i = 1..N-1 swap a[i]
// with a[rand() % (i+1)].
void rand_shuffle(std::vector<int32_t>& a, GlibcRand& rng) {
  for (size_t i = 1; i < a.size(); ++i) {
    size_t j = static_cast<size_t>(rng.next()) % (i + 1);
    if (i != j) std::swap(a[i], a[j]);
  }
}

// Inner-stratum schedule of dsgd_mpi (sgd-mpi-omp.cpp:268-365) for iterations
// 1..iter; inner_perm / inner_offset persist across iterations.
void dsgd_schedule(int32_t innerB, int32_t iter, int32_t strategy,
                   std::vector<int32_t>& bj_out) {
  std::vector<int32_t> inner_perm(innerB), inner_offset(innerB), cur(innerB);
  for (int32_t i = 0; i < innerB; ++i) inner_perm[i] = inner_offset[i] = cur[i] = i;
  const unsigned seed = 34586;
  for (int32_t it = 1; it <= iter; ++it) {
    GlibcRand rng(seed + it);
    // B = 1: random_shuffle of perm_matrix and of indices draw nothing.
    if (strategy == 2) {  // WOR_STRATUM
      rand_shuffle(inner_perm, rng);
      rand_shuffle(inner_offset, rng);
    }
  }
  bj_out.assign(static_cast<size_t>(innerB) * innerB, 0);
  for (int32_t i = 0; i < innerB; ++i) {
    for (int32_t ii = 0; ii < innerB; ++ii) cur[inner_perm[ii]] = (ii + inner_offset[i]) % innerB;
    for (int32_t bi = 0; bi < innerB; ++bi) bj_out[static_cast<size_t>(i) * innerB + bi] = cur[bi];
  }
}

// Schedule of dsgd_mpi in dsgdpp.cpp for iteration `iter`: inner_perm / inner_offset
// restart from the identity every iteration (dsgdpp.cpp:349-350); under WOR_STRATUM
// phase 0 shuffles them after srand(34586 + iter) (dsgdpp.cpp:351-356, 397-400; the
// B = 1 outer shuffles draw nothing) and phase 1 reuses them (dsgdpp.cpp:434-441).
// bj_out[(phase*innerB + i)*innerB + bi] = phase*innerB + inner column block.
void dsgdpp_schedule(int32_t innerB, int32_t iter, int32_t strategy,
                     std::vector<int32_t>& bj_out) {
  std::vector<int32_t> inner_perm(innerB), inner_offset(innerB), cur(innerB);
  for (int32_t i = 0; i < innerB; ++i) inner_perm[i] = inner_offset[i] = cur[i] = i;
  GlibcRand rng(34586u + static_cast<unsigned>(iter));
  if (strategy == 2) {  // WOR_STRATUM
    rand_shuffle(inner_perm, rng);
    rand_shuffle(inner_offset, rng);
  }
  bj_out.assign(static_cast<size_t>(2) * innerB * innerB, 0);
  for (int32_t phase = 0; phase < 2; ++phase)
    for (int32_t i = 0; i < innerB; ++i) {
      for (int32_t ii = 0; ii < innerB; ++ii) cur[inner_perm[ii]] = (ii + inner_offset[i]) % innerB;
      for (int32_t bi = 0; bi < innerB; ++bi)
        bj_out[(static_cast<size_t>(phase) * innerB + i) * innerB + bi] = phase * innerB + cur[bi];
    }
}

// calobj_mpi (sgd-mpi-omp.cpp:122-160, the same in dsgdpp.cpp), one process: the sum
// over training ratings of (dot(W_i, H_j) - v)^2 in double, dot summed from index
// k-1 down to 0 (util.cpp:75-80), plus lambda * (sum_r nnz_row(r) * norm(W_r) +
// sum_c nnz_col(c) * norm(H_c)), norm = sum of squares from index k-1 down to 0
// (util.cpp:95-100).  Factors are read as stored.
template <typename S>
double objective(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                 const int32_t* cols, const double* vals, const S* W, const S* H, double reg) {
  double loss = 0;
  std::vector<int64_t> col_cnt(static_cast<size_t>(n), 0);
  int64_t idx = 0;
  for (int32_t r = 0; r < m; ++r)
    for (int32_t t = 0; t < row_counts[r]; ++t, ++idx) {
      const S* Wi = W + static_cast<int64_t>(dim) * r;
      const S* Hj = H + static_cast<int64_t>(dim) * cols[idx];
      double diff = -vals[idx];
      double dot = 0;
      for (int32_t kk = dim - 1; kk >= 0; --kk) dot += static_cast<double>(Wi[kk]) * static_cast<double>(Hj[kk]);
      diff += dot;
      loss += diff * diff;
      col_cnt[cols[idx]]++;
    }
  (void)nnz;
  auto norm = [&](const S* x) {
    double ret = 0;
    for (int32_t kk = dim - 1; kk >= 0; --kk) ret += static_cast<double>(x[kk]) * static_cast<double>(x[kk]);
    return ret;
  };
  double regsum = 0;
  for (int32_t r = 0; r < m; ++r) regsum += row_counts[r] * norm(W + static_cast<int64_t>(dim) * r);
  for (int32_t c = 0; c < n; ++c) regsum += col_cnt[c] * norm(H + static_cast<int64_t>(dim) * c);
  return loss + reg * regsum;
}

// variant 0: DSGD (sgd-mpi-omp.cpp), innerB x innerB blocks, innerB strata per pass.
// variant 1: DSGD++ (dsgdpp.cpp), innerB x 2*innerB blocks (mpi_blocks_t,
// dsgdpp.cpp:42-69), 2*innerB strata per pass.  lr_strategy 1 (BOLDDRIVER):
// lr_state = {current learning rate, objective after the previous pass (< 0: not yet
// computed)}, updated in place (sgd-mpi-omp.cpp:278-283, 384-394; dsgdpp.cpp:330-336,
// 512-521).
template <typename S>
int dsgd(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
         const int32_t* cols, const double* vals, S* W, S* H, int32_t nthreads,
         int32_t first_iter, int32_t n_iters, double lrate, double decay,
         double reg, int32_t strategy, int32_t variant = 0, int32_t lr_strategy = 0,
         double* lr_state = nullptr) {
  if (nthreads <= 0 || dim <= 0 || first_iter < 1 || n_iters < 0) return -1;
  if (lr_strategy == 1 && !lr_state) return -1;
  const int32_t innerB = 2 * nthreads;  // sgd-mpi-omp.cpp:747, dsgdpp.cpp:760
  const int32_t col_blocks = variant == 1 ? 2 * innerB : innerB;
  // mpi_blocks_t::set_parameters with B = 1 (sgd-mpi-omp.cpp:39-50, dsgdpp.cpp:42-52)
  const int32_t Bm = m, Bn = n;
  const int32_t innerBm = Bm / innerB + ((Bm % innerB) ? 1 : 0);
  const int32_t innerBn = Bn / col_blocks + ((Bn % col_blocks) ? 1 : 0);
  const int32_t nblocks = innerB * col_blocks;
  struct Rate {
    int32_t i, j;
    S v;
  };
  // PETSc_reader::receive_blocks (sgd-mpi-omp.cpp:539-588): stable counting sort of
  // the row-major entries by block id.
  std::vector<int64_t> block_ptr(nblocks + 1, 0);
  auto bid_of = [&](int32_t r, int32_t c) {
    return (r / innerBm) * col_blocks + (c / innerBn);
  };
  {
    int64_t idx = 0;
    for (int32_t r = 0; r < m; ++r)
      for (int32_t t = 0; t < row_counts[r]; ++t, ++idx) block_ptr[bid_of(r, cols[idx]) + 1]++;
    if (idx != nnz) return -1;
  }
  for (int32_t b = 0; b < nblocks; ++b) block_ptr[b + 1] += block_ptr[b];
  std::vector<Rate> rates(static_cast<size_t>(nnz));
  {
    std::vector<int64_t> fill(block_ptr.begin(), block_ptr.end() - 1);
    int64_t idx = 0;
    for (int32_t r = 0; r < m; ++r)
      for (int32_t t = 0; t < row_counts[r]; ++t, ++idx)
        rates[fill[bid_of(r, cols[idx])]++] = Rate{r, cols[idx], static_cast<S>(vals[idx])};
  }
  const S lambda = static_cast<S>(reg);
  std::vector<int32_t> sched;
  const int32_t strata = variant == 1 ? 2 * innerB : innerB;
  if (lr_strategy == 1 && lr_state[1] < 0)
    lr_state[1] = objective<S>(m, n, dim, nnz, row_counts, cols, vals, W, H, reg);
  for (int32_t it = first_iter; it < first_iter + n_iters; ++it) {
    // FIXED strategy (sgd-mpi-omp.cpp:308-309); lrate/decay are doubles there.
    const S cur_lrate = lr_strategy == 1 ? static_cast<S>(lr_state[0])
                                         : static_cast<S>(1.5 * lrate / (1.0 + decay * std::pow(it, 1.5)));
    if (variant == 1)
      dsgdpp_schedule(innerB, it, strategy, sched);
    else
      dsgd_schedule(innerB, it, strategy, sched);
    for (int32_t i = 0; i < strata; ++i) {
      for (int32_t bi = 0; bi < innerB; ++bi) {
        const int32_t bid = bi * col_blocks + sched[static_cast<size_t>(i) * innerB + bi];
        const int64_t b = block_ptr[bid], e = block_ptr[bid + 1];
        // sgd() (sgd-mpi-omp.cpp:186-210): walks the block from its last entry to its
        // first; err = dot(Wi, Hj) - v with dot summed from index k-1 down to 0.
        for (int64_t idx = e - 1; idx >= b; --idx) {
          const Rate& R = rates[idx];
          S* Wi = W + static_cast<int64_t>(dim) * R.i;
          S* Hj = H + static_cast<int64_t>(dim) * R.j;
          S dot = 0;
          for (int32_t kk = dim - 1; kk >= 0; --kk) dot += Wi[kk] * Hj[kk];
          const S err = dot - R.v;
          for (int32_t kk = 0; kk < dim; ++kk) {
            S tmp = Wi[kk];
            Wi[kk] -= cur_lrate * (err * Hj[kk] + lambda * Wi[kk]);
            Hj[kk] -= cur_lrate * (err * tmp + lambda * Hj[kk]);
          }
        }
      }
    }
    if (lr_strategy == 1) {
      const double obj = objective<S>(m, n, dim, nnz, row_counts, cols, vals, W, H, reg);
      lr_state[0] *= obj > lr_state[1] ? decay : 1.05;
      lr_state[1] = obj;
    }
  }
  return 0;
}

}  // namespace

extern "C" {

void oracle_init_factors(int32_t m, int32_t n, int32_t dim, uint64_t seed,
                         int32_t nthreads, double* W, double* H) {
  const int32_t rank = 0;
  std::uniform_real_distribution<double> init_dist(0, 1.0 / std::sqrt(dim));
  if (W) {
    const int32_t P = nthreads;
    const int32_t rows_per_part = m / P + ((m % P > 0) ? 1 : 0);
    for (int32_t t = 0; t < P; ++t) {
      const int64_t lo = std::min<int64_t>(static_cast<int64_t>(rows_per_part) * t, m);
      const int64_t hi = std::min<int64_t>(static_cast<int64_t>(rows_per_part) * (t + 1), m);
      std::mt19937_64 rng(seed + rank * 131 + t + 1);  // nb_main.cpp:451
      for (int64_t i = lo * dim; i < hi * dim; ++i) W[i] = init_dist(rng);
    }
  }
  if (H) {
    std::mt19937_64 rng(seed + rank * 131 + 139);  // nb_main.cpp:71
    for (int64_t i = 0; i < static_cast<int64_t>(n) * dim; ++i) H[i] = init_dist(rng);
  }
}

int oracle_row_major_to_csc(int32_t m, int32_t n, int64_t nnz,
                            const int32_t* row_counts, const int32_t* cols,
                            const double* vals, int64_t* col_ptr,
                            int32_t* row_idx, double* csc_vals) {
  std::fill(col_ptr, col_ptr + n + 1, 0);
  int64_t idx = 0;
  for (int32_t r = 0; r < m; ++r) {
    for (int32_t t = 0; t < row_counts[r]; ++t, ++idx) {
      if (idx >= nnz || cols[idx] < 0 || cols[idx] >= n) return -1;
      col_ptr[cols[idx] + 1]++;
    }
  }
  if (idx != nnz) return -1;
  for (int32_t j = 0; j < n; ++j) col_ptr[j + 1] += col_ptr[j];
  std::vector<int64_t> fill(col_ptr, col_ptr + n);
  idx = 0;
  for (int32_t r = 0; r < m; ++r) {
    for (int32_t t = 0; t < row_counts[r]; ++t, ++idx) {
      const int64_t o = fill[cols[idx]]++;
      row_idx[o] = r;
      csc_vals[o] = vals[idx];
    }
  }
  return 0;
}

float oracle_step_f32(double lrate, double drate, int32_t cnt) {
  return step_size<float>(lrate, drate, cnt);
}
double oracle_step_f64(double lrate, double drate, int32_t cnt) {
  return step_size<double>(lrate, drate, cnt);
}

int oracle_replay_f32(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                      const int32_t* row_idx, const double* vals, float* W,
                      float* H, int32_t first_epoch, int32_t n_epochs,
                      double lrate, double drate, double reg, double* epoch_err) {
  return replay<float>(m, n, dim, col_ptr, row_idx, vals, W, H, first_epoch,
                       n_epochs, lrate, drate, reg, epoch_err);
}
int oracle_replay_f64(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                      const int32_t* row_idx, const double* vals, double* W,
                      double* H, int32_t first_epoch, int32_t n_epochs,
                      double lrate, double drate, double reg, double* epoch_err) {
  return replay<double>(m, n, dim, col_ptr, row_idx, vals, W, H, first_epoch,
                        n_epochs, lrate, drate, reg, epoch_err);
}

int oracle_sse_f32(int32_t, int32_t n, int32_t dim, const int64_t* col_ptr,
                   const int32_t* row_idx, const double* vals, const float* W,
                   const float* H, double* s, int64_t* c) {
  return sse<float>(n, dim, col_ptr, row_idx, vals, W, H, s, c);
}
int oracle_sse_f64(int32_t, int32_t n, int32_t dim, const int64_t* col_ptr,
                   const int32_t* row_idx, const double* vals, const double* W,
                   const double* H, double* s, int64_t* c) {
  return sse<double>(n, dim, col_ptr, row_idx, vals, W, H, s, c);
}

int oracle_async_f32(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                     const int32_t* row_idx, const double* vals, float* W,
                     float* H, int32_t nthreads, int32_t n_epochs,
                     double timeout_sec, double lrate, double drate, double reg,
                     uint64_t seed, int64_t* updates, int64_t* failures,
                     double* train_seconds) {
  return async_run<float>(m, n, dim, col_ptr, row_idx, vals, W, H, nthreads,
                          n_epochs, timeout_sec, lrate, drate, reg, seed, updates,
                          failures, train_seconds);
}
int oracle_async_f64(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                     const int32_t* row_idx, const double* vals, double* W,
                     double* H, int32_t nthreads, int32_t n_epochs,
                     double timeout_sec, double lrate, double drate, double reg,
                     uint64_t seed, int64_t* updates, int64_t* failures,
                     double* train_seconds) {
  return async_run<double>(m, n, dim, col_ptr, row_idx, vals, W, H, nthreads,
                           n_epochs, timeout_sec, lrate, drate, reg, seed, updates,
                           failures, train_seconds);
}

int oracle_async_sim_f32(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr, const int32_t* row_idx,
                         const double* vals, float* W, float* H, int32_t P, int32_t partition, int32_t first_epoch,
                         int32_t n_epochs, double lrate, double drate, double reg, uint64_t seed,
                         double visit_cost, double rating_cost, double hop_cost, double* epoch_err) {
  return async_sim<float>(m, n, dim, col_ptr, row_idx, vals, W, H, P, partition, first_epoch, n_epochs, lrate,
                          drate, reg, seed, visit_cost, rating_cost, hop_cost, epoch_err);
}
int oracle_async_sim_f64(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr, const int32_t* row_idx,
                         const double* vals, double* W, double* H, int32_t P, int32_t partition, int32_t first_epoch,
                         int32_t n_epochs, double lrate, double drate, double reg, uint64_t seed,
                         double visit_cost, double rating_cost, double hop_cost, double* epoch_err) {
  return async_sim<double>(m, n, dim, col_ptr, row_idx, vals, W, H, P, partition, first_epoch, n_epochs, lrate,
                           drate, reg, seed, visit_cost, rating_cost, hop_cost, epoch_err);
}

int oracle_dsgd_f32(int32_t m, int32_t n, int32_t dim, int64_t nnz,
                    const int32_t* row_counts, const int32_t* cols,
                    const double* vals, float* W, float* H, int32_t nthreads,
                    int32_t first_iter, int32_t n_iters, double lrate,
                    double decay, double reg, int32_t stratum_strategy) {
  return dsgd<float>(m, n, dim, nnz, row_counts, cols, vals, W, H, nthreads,
                     first_iter, n_iters, lrate, decay, reg, stratum_strategy);
}
int oracle_dsgd_f64(int32_t m, int32_t n, int32_t dim, int64_t nnz,
                    const int32_t* row_counts, const int32_t* cols,
                    const double* vals, double* W, double* H, int32_t nthreads,
                    int32_t first_iter, int32_t n_iters, double lrate,
                    double decay, double reg, int32_t stratum_strategy) {
  return dsgd<double>(m, n, dim, nnz, row_counts, cols, vals, W, H, nthreads,
                      first_iter, n_iters, lrate, decay, reg, stratum_strategy);
}

int oracle_dsgd2_f32(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                     const int32_t* cols, const double* vals, float* W, float* H, int32_t nthreads,
                     int32_t first_iter, int32_t n_iters, double lrate, double decay, double reg,
                     int32_t stratum_strategy, int32_t variant, int32_t lr_strategy, double* lr_state) {
  return dsgd<float>(m, n, dim, nnz, row_counts, cols, vals, W, H, nthreads, first_iter, n_iters,
                     lrate, decay, reg, stratum_strategy, variant, lr_strategy, lr_state);
}
int oracle_dsgd2_f64(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                     const int32_t* cols, const double* vals, double* W, double* H, int32_t nthreads,
                     int32_t first_iter, int32_t n_iters, double lrate, double decay, double reg,
                     int32_t stratum_strategy, int32_t variant, int32_t lr_strategy, double* lr_state) {
  return dsgd<double>(m, n, dim, nnz, row_counts, cols, vals, W, H, nthreads, first_iter, n_iters,
                      lrate, decay, reg, stratum_strategy, variant, lr_strategy, lr_state);
}

int oracle_objective_f32(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                         const int32_t* cols, const double* vals, const float* W, const float* H,
                         double reg, double* out) {
  if (dim <= 0 || !out) return -1;
  *out = objective<float>(m, n, dim, nnz, row_counts, cols, vals, W, H, reg);
  return 0;
}
int oracle_objective_f64(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                         const int32_t* cols, const double* vals, const double* W, const double* H,
                         double reg, double* out) {
  if (dim <= 0 || !out) return -1;
  *out = objective<double>(m, n, dim, nnz, row_counts, cols, vals, W, H, reg);
  return 0;
}

int oracle_dsgdpp_schedule(int32_t innerB, int32_t iter, int32_t stratum_strategy, int32_t* bj) {
  if (innerB <= 0 || iter < 1) return -1;
  std::vector<int32_t> s;
  dsgdpp_schedule(innerB, iter, stratum_strategy, s);
  std::copy(s.begin(), s.end(), bj);
  return 0;
}

int oracle_dsgd_schedule(int32_t innerB, int32_t iter, int32_t stratum_strategy,
                         int32_t* bj) {
  if (innerB <= 0 || iter < 1) return -1;
  std::vector<int32_t> s;
  dsgd_schedule(innerB, iter, stratum_strategy, s);
  std::copy(s.begin(), s.end(), bj);
  return 0;
}

// nb_data.cpp:19-78: header of either file id.
int oracle_read_header(const char* path, int32_t* file_id, int32_t* m, int32_t* n,
                       int64_t* nnz) {
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) return -1;
  int32_t id = 0;
  if (!f.read(reinterpret_cast<char*>(&id), sizeof(id))) return -2;
  if (id == kMatFileClassId) {
    int32_t h[3];
    if (!f.read(reinterpret_cast<char*>(h), sizeof(h))) return -2;
    *m = h[0];
    *n = h[1];
    *nnz = h[2];
  } else if (id == kLongFileClassId) {
    int32_t h[2];
    if (!f.read(reinterpret_cast<char*>(h), sizeof(h))) return -2;
    *m = h[0];
    *n = h[1];
    long long t = 0;
    if (!f.read(reinterpret_cast<char*>(&t), sizeof(t))) return -2;
    *nnz = t;
  } else {
    return -3;
  }
  *file_id = id;
  return 0;
}

int oracle_read_matrix(const char* path, int32_t* row_counts, int32_t* cols,
                       double* vals) {
  int32_t id, m, n;
  int64_t nnz;
  int rc = oracle_read_header(path, &id, &m, &n, &nnz);
  if (rc) return rc;
  std::ifstream f(path, std::ios::in | std::ios::binary);
  f.seekg(id == kMatFileClassId ? 16 : 20, std::ios::beg);
  if (!f.read(reinterpret_cast<char*>(row_counts), static_cast<std::streamsize>(m) * 4)) return -2;
  if (!f.read(reinterpret_cast<char*>(cols), static_cast<std::streamsize>(nnz) * 4)) return -2;
  if (!f.read(reinterpret_cast<char*>(vals), static_cast<std::streamsize>(nnz) * 8)) return -2;
  return 0;
}

uint64_t oracle_mt19937_64_10000th(void) {
  std::mt19937_64 g;
  g.discard(9999);
  return g();
}

}  // extern "C"
