// host_layout.cpp -- host-side construction of the device data layout: CSC by column,
// worker row blocks, token visit lists, initial queues, DSGD blocks and schedules.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <tuple>

#include "layout.h"

namespace nomad {

namespace {

// Row-major view of a rating set: entries listed row by row.
struct RowMajor {
  std::vector<int64_t> row_ptr;  // [m+1]
  const int32_t* cols = nullptr;
  const double* v64 = nullptr;
  const float* v32 = nullptr;
  // storage when the input was COO and had to be reordered
  std::vector<int32_t> own_cols;
  std::vector<float> own_vals;
  float val(int64_t i) const { return v64 ? static_cast<float>(v64[i]) : v32[i]; }
};

int to_row_major(const nomad_gpu_matrix& A, int32_t m, int32_t n, RowMajor& R, int threads,
                 bool check_cols = true) {
  if (A.nnz < 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "negative nnz");
  if (A.nnz > 0 && (!A.cols || (!A.vals_f64 && !A.vals_f32)))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "rating set has nnz > 0 but null arrays");
  if (A.vals_f64 && A.vals_f32) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "give vals_f64 or vals_f32, not both");
  R.row_ptr.assign(static_cast<size_t>(m) + 1, 0);
  if (A.row_counts) {
    for (int32_t i = 0; i < m; ++i) {
      if (A.row_counts[i] < 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "negative row count at row %d", i);
      R.row_ptr[i + 1] = R.row_ptr[i] + A.row_counts[i];
    }
    if (R.row_ptr[m] != A.nnz)
      NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "row counts add up to %lld, nnz is %lld",
                 (long long)R.row_ptr[m], (long long)A.nnz);
    R.cols = A.cols;
    R.v64 = A.vals_f64;
    R.v32 = A.vals_f32;
  } else if (A.nnz > 0) {
    if (!A.rows) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "rating set needs row_counts or rows");
    for (int64_t i = 0; i < A.nnz; ++i) {
      const int32_t r = A.rows[i];
      if (r < 0 || r >= m) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "row index %d out of range [0, %d)", r, m);
      R.row_ptr[r + 1]++;
    }
    for (int32_t i = 0; i < m; ++i) R.row_ptr[i + 1] += R.row_ptr[i];
    std::vector<int64_t> fill(R.row_ptr.begin(), R.row_ptr.end() - 1);
    R.own_cols.resize(A.nnz);
    R.own_vals.resize(A.nnz);
    for (int64_t i = 0; i < A.nnz; ++i) {
      const int64_t o = fill[A.rows[i]]++;
      R.own_cols[o] = A.cols[i];
      R.own_vals[o] = A.vals_f64 ? static_cast<float>(A.vals_f64[i]) : A.vals_f32[i];
    }
    R.cols = R.own_cols.data();
    R.v32 = R.own_vals.data();
  }
  if (!check_cols) return NOMAD_OK;  // the caller checks them in its own pass
  // first out-of-range column index, checked in parallel
  std::atomic<int64_t> bad{A.nnz};
  const int32_t* cols = R.cols;
  parallel_chunks(A.nnz, threads, [&](int, int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i)
      if (cols[i] < 0 || cols[i] >= n) {
        int64_t cur = bad.load();
        while (i < cur && !bad.compare_exchange_weak(cur, i)) {
        }
        break;
      }
  });
  if (bad.load() < A.nnz)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "column index %d out of range [0, %d)", cols[bad.load()], n);
  return NOMAD_OK;
}

// glibc's rand() stream (srand seeds the TYPE_3 additive generator; initstate_r with a
// 128-byte state does the same) kept private so the process-global state is untouched.
struct GlibcRand {
  struct random_data data {};
  char state[128];
  explicit GlibcRand(unsigned seed) {
    std::memset(state, 0, sizeof(state));
    data.state = nullptr;
    initstate_r(seed, state, sizeof(state), &data);
  }
  int next() {
    int32_t r;
    random_r(&data, &r);
    return r;
  }
};

}  // namespace

float step_size_f32(double lrate, double drate, int32_t cnt) {
  const float learn_rate = static_cast<float>(lrate);
  const float decay_rate = static_cast<float>(drate);
  return static_cast<float>(learn_rate * 1.5 / (1.0 + decay_rate * std::pow(cnt + 1, 1.5)));
}

int check_rating_set(const nomad_gpu_matrix& A, int32_t m, int32_t n, int threads, bool check_cols) {
  RowMajor R;
  return to_row_major(A, m, n, R, threads, check_cols);
}

int build_csc(const nomad_gpu_matrix& A, int32_t m, int32_t n, Csc& out, int threads) {
  RowMajor R;
  int rc = to_row_major(A, m, n, R, threads, false);
  if (rc) return rc;
  const int64_t nnz = A.nnz;
  out.m = m;
  out.n = n;
  out.col_ptr.assign(static_cast<size_t>(n) + 1, 0);
  out.ratings.resize(static_cast<size_t>(nnz));
  out.row_nnz.resize(static_cast<size_t>(m));
  parallel_chunks(m, threads, [&](int, int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) out.row_nnz[i] = static_cast<int32_t>(R.row_ptr[i + 1] - R.row_ptr[i]);
  });
  if (nnz == 0) return NOMAD_OK;
  // Stable counting sort by column: contiguous chunks of the row-major entries, one
  // column histogram per chunk, then each chunk scatters in order.
  const int T = std::max<int>(1, std::min<int64_t>(threads, std::max<int64_t>(1, nnz / 65536)));
  std::vector<std::vector<int64_t>> hist(T, std::vector<int64_t>(n, 0));
  std::vector<int64_t> first_bad(T, nnz);  // the column indices are checked in the same pass
  parallel_chunks(nnz, T, [&](int t, int64_t lo, int64_t hi) {
    std::vector<int64_t>& h = hist[t];
    for (int64_t i = lo; i < hi; ++i) {
      const int32_t c = R.cols[i];
      if (static_cast<uint32_t>(c) >= static_cast<uint32_t>(n)) {
        first_bad[t] = i;
        break;
      }
      h[c]++;
    }
  });
  const int64_t bad = *std::min_element(first_bad.begin(), first_bad.end());
  if (bad < nnz) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "column index %d out of range [0, %d)", R.cols[bad], n);
  for (int32_t j = 0; j < n; ++j) {
    int64_t s = 0;
    for (int t = 0; t < T; ++t) s += hist[t][j];
    out.col_ptr[j + 1] = out.col_ptr[j] + s;
  }
  for (int32_t j = 0; j < n; ++j) {  // hist[t][j] becomes chunk t's write cursor
    int64_t pos = out.col_ptr[j];
    for (int t = 0; t < T; ++t) {
      const int64_t c = hist[t][j];
      hist[t][j] = pos;
      pos += c;
    }
  }
  parallel_chunks(nnz, T, [&](int t, int64_t lo, int64_t hi) {
    std::vector<int64_t>& cur = hist[t];
    int32_t r = static_cast<int32_t>(std::upper_bound(R.row_ptr.begin(), R.row_ptr.end(), lo) -
                                     R.row_ptr.begin()) - 1;
    for (int64_t i = lo; i < hi; ++i) {
      while (R.row_ptr[r + 1] <= i) ++r;
      out.ratings[cur[R.cols[i]]++] = Rating{r, R.val(i)};
    }
  });
  // repeated cells would break the distinct-rows property a column visit relies on
  std::atomic<int64_t> dup{-1};
  parallel_dynamic(n, 64, threads, [&](int, int64_t lo, int64_t hi) {
    for (int64_t j = lo; j < hi && dup.load(std::memory_order_relaxed) < 0; ++j)
      for (int64_t o = out.col_ptr[j] + 1; o < out.col_ptr[j + 1]; ++o)
        if (out.ratings[o].row == out.ratings[o - 1].row) {
          dup.store(j);
          break;
        }
  });
  if (dup.load() >= 0)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "repeated (row, column) cell in column %lld", (long long)dup.load());
  return NOMAD_OK;
}

int async_layout_rows(const Csc& csc, int32_t P, int balance, AsyncLayout& L, int threads) {
  const int32_t m = csc.m;
  const int64_t nnz = csc.nnz();
  if (P <= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "worker count must be positive");
  L.P = P;
  L.row_start.assign(static_cast<size_t>(P) + 1, m);
  if (balance == 0 || nnz == 0) {
    // read_data's split: ceil(m/P) rows per worker (nb_data.cpp:83-89)
    const int64_t per = m / P + ((m % P > 0) ? 1 : 0);
    for (int32_t w = 0; w <= P; ++w) L.row_start[w] = static_cast<int32_t>(std::min<int64_t>(per * w, m));
  } else {
    // contiguous blocks holding ~nnz/P ratings each; ratings per row as build_csc
    // counted them, else from per-thread histograms (no shared counters)
    std::vector<int32_t> counted;
    if (csc.row_nnz.size() != static_cast<size_t>(m)) {
      const int nt = std::max(1, std::min<int>(threads, 64));
      std::vector<std::vector<int32_t>> part(static_cast<size_t>(nt));
      parallel_chunks(nnz, nt, [&](int t, int64_t lo, int64_t hi) {
        std::vector<int32_t>& h = part[static_cast<size_t>(t)];
        h.assign(static_cast<size_t>(m), 0);
        for (int64_t o = lo; o < hi; ++o) ++h[csc.row(o)];
      });
      counted.assign(static_cast<size_t>(m), 0);
      parallel_chunks(m, nt, [&](int, int64_t lo, int64_t hi) {
        for (const auto& h : part)
          if (!h.empty())
            for (int64_t i = lo; i < hi; ++i) counted[i] += h[i];
      });
    }
    const std::vector<int32_t>& row_nnz = counted.empty() ? csc.row_nnz : counted;
    int64_t acc = 0;
    int32_t w = 1;
    L.row_start[0] = 0;
    for (int32_t i = 0; i < m && w < P; ++i) {
      acc += row_nnz[i];
      while (w < P && acc >= (nnz * w + P - 1) / P) L.row_start[w++] = i + 1;
    }
    for (; w <= P; ++w) L.row_start[w] = m;
  }
  return NOMAD_OK;
}

int build_async_layout(const Csc& csc, int32_t P, int balance, uint64_t seed,
                       int64_t priority_min, int32_t group, bool group_routes, AsyncLayout& L,
                       int threads) {
  const int32_t m = csc.m, n = csc.n;
  if (group <= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "worker group size must be positive");
  int rc = async_layout_rows(csc, P, balance, L, threads);
  if (rc) return rc;
  // visit lists: the rows of a column are ascending, so each worker's share is a run;
  // a priority column's visits are the runs of whole worker groups
  L.vl_ptr.assign(static_cast<size_t>(n) + 1, 0);
  std::vector<int32_t> row_worker(static_cast<size_t>(std::max(m, 1)));
  parallel_chunks(P, threads, [&](int, int64_t lo, int64_t hi) {
    for (int64_t w = lo; w < hi; ++w)
      for (int32_t r = L.row_start[w]; r < L.row_start[w + 1]; ++r) row_worker[r] = static_cast<int32_t>(w);
  });
  auto worker_of = [&](int32_t row) { return row_worker[row]; };
  auto is_priority = [&](int64_t j) {
    return priority_min > 0 && csc.col_ptr[j + 1] - csc.col_ptr[j] >= priority_min;
  };
  // owner of `row` for column j: {worker or group index, first row past its block}
  auto owner_of = [&](int32_t row, bool pri) {
    const int32_t w = worker_of(row);
    if (!pri) return std::make_pair(w, L.row_start[w + 1]);
    const int32_t g = w / group;
    return std::make_pair(g, L.row_start[std::min<int64_t>(static_cast<int64_t>(g + 1) * group, P)]);
  };
  // End of the run that starts at rating o of a column ending at e: the first rating past
  // o whose row is at least wend.  Rows ascend inside a column: a short scan covers the
  // common short run, then a galloping search takes a long one in O(log len).
  auto run_end = [&](int64_t o, int64_t e, int32_t wend) {
    int64_t lo = o + 1;
    for (int i = 0; i < 8; ++i, ++lo)
      if (lo >= e || csc.row(lo) >= wend) return lo;
    int64_t step = 1;
    while (lo < e && csc.row(lo) < wend) {
      const int64_t hi = std::min(e, lo + step);
      if (hi < e && csc.row(hi) < wend) {
        lo = hi + 1;
        step <<= 1;
        continue;
      }
      int64_t a = lo, b = hi;  // first index in [a, b) with row >= wend (b if none)
      while (a < b) {
        const int64_t mid = a + (b - a) / 2;
        if (csc.row(mid) < wend) a = mid + 1;
        else b = mid;
      }
      return a;
    }
    return lo;
  };
  // columns are uneven (a Zipf column holds ~5% of all ratings): hand them out in small
  // chunks on demand
  std::vector<int64_t> nseg(n, 0);
  parallel_dynamic(n, 16, threads, [&](int, int64_t lo, int64_t hi) {
    for (int64_t j = lo; j < hi; ++j) {
      const bool pri = is_priority(j);
      int64_t c = 0;
      const int64_t e = csc.col_ptr[j + 1];
      for (int64_t o = csc.col_ptr[j]; o < e; ++c) o = run_end(o, e, owner_of(csc.row(o), pri).second);
      nseg[j] = c;
    }
  });
  for (int32_t j = 0; j < n; ++j) L.vl_ptr[j + 1] = L.vl_ptr[j] + nseg[j];
  L.segs.resize(static_cast<size_t>(L.vl_ptr[n]));
  std::vector<int64_t> maxseg(std::max(threads, 1), 0);
  parallel_dynamic(n, 16, threads, [&](int t, int64_t lo, int64_t hi) {
    std::vector<std::pair<uint64_t, int64_t>> runs, inner;
    std::vector<Segment> tmp;
    for (int64_t j = lo; j < hi; ++j) {
      Segment* s = L.segs.data() + L.vl_ptr[j];
      const bool pri = is_priority(j);
      const int64_t e = csc.col_ptr[j + 1];
      int64_t c = 0;
      for (int64_t o = csc.col_ptr[j]; o < e; ++c) {
        const auto own = owner_of(csc.row(o), pri);
        const int64_t next = run_end(o, e, own.second);
        s[c] = Segment{o, static_cast<int32_t>(next - o), own.first};
        o = next;
      }
      const int64_t k = nseg[j];
      for (int64_t i = 0; i < k; ++i) maxseg[t] = std::max<int64_t>(maxseg[t], s[i].len);
      // the token's route: a seeded random order of its visits (pool.cpp:32-38 draws
      // a random permutation of the workers; empty visits are skipped here)
      if (group_routes && !pri && group > 1 && k > 1) {
        // hierarchical route: the visits to one group's workers (a thread block) stay
        // consecutive, like the reference's token that makes its round of one machine's
        // threads before it leaves for another machine (nb_main.cpp:551-565); groups and
        // workers in a group in seeded random order: visits ordered by (key of the
        // group, key of the worker).  The visits arrive in worker order, so each group's
        // visits are one run: order the runs by group key, then each run by worker key
        // (keys are distinct, so they alone fix the order).
        const uint64_t kb = stream_key(seed, 149, static_cast<uint64_t>(j));
        const uint64_t kw = stream_key(seed, 151, static_cast<uint64_t>(j));
        runs.clear();
        for (int64_t i = 0; i < k; ++i)
          if (i == 0 || s[i].worker / group != s[i - 1].worker / group)
            runs.push_back({SplitMix64::mix(kb ^ static_cast<uint64_t>(s[i].worker / group)), i});
        std::sort(runs.begin(), runs.end());
        tmp.assign(s, s + k);
        int64_t o = 0;
        for (const auto& rn : runs) {
          const int64_t b = rn.second;
          int64_t e = b + 1;
          while (e < k && tmp[e].worker / group == tmp[b].worker / group) ++e;
          inner.clear();
          for (int64_t i = b; i < e; ++i) inner.push_back({SplitMix64::mix(kw ^ static_cast<uint64_t>(tmp[i].worker)), i});
          std::sort(inner.begin(), inner.end());
          for (const auto& x : inner) s[o++] = tmp[x.second];
        }
      } else {
        SplitMix64 rng(stream_key(seed, 137, static_cast<uint64_t>(j)));
        for (int64_t i = k - 1; i > 0; --i) std::swap(s[i], s[rng.below(i + 1)]);
      }
    }
  });
  L.max_segment = *std::max_element(maxseg.begin(), maxseg.end());
  std::vector<Segment> firsts(static_cast<size_t>(n));
  for (int32_t j = 0; j < n; ++j)
    if (L.vl_ptr[j + 1] > L.vl_ptr[j]) firsts[j] = L.segs[L.vl_ptr[j]];
  async_layout_queues(csc, priority_min, firsts.data(), L);
  return NOMAD_OK;
}

void async_layout_queues(const Csc& csc, int64_t priority_min, const Segment* firsts, AsyncLayout& L) {
  const int32_t n = csc.n, P = L.P;
  auto is_priority = [&](int64_t j) {
    return priority_min > 0 && csc.col_ptr[j + 1] - csc.col_ptr[j] >= priority_min;
  };
  auto nseg = [&](int32_t j) { return L.vl_ptr[j + 1] - L.vl_ptr[j]; };
  L.max_column = 0;
  L.n_active = 0;
  for (int32_t j = 0; j < n; ++j) {
    L.max_column = std::max<int64_t>(L.max_column, csc.col_ptr[j + 1] - csc.col_ptr[j]);
    if (nseg(j) > 0) ++L.n_active;
  }
  // initial queues: every active token at its first worker, in column order
  // (nb_main.cpp:82-97 pushes the tokens in index order); long columns go to the
  // worker's priority queue (queue P + w)
  L.qnext0.assign(static_cast<size_t>(n) + 2 * static_cast<size_t>(P), -1);
  L.qtail0.resize(2 * static_cast<size_t>(P));
  for (int32_t q = 0; q < 2 * P; ++q) L.qtail0[q] = n + q;
  L.desc0.assign(4 * static_cast<size_t>(n), 0);
  L.first_mail.assign(8 * static_cast<size_t>(n), 0);
  L.first_q.assign(2 * static_cast<size_t>(n), -1);
  L.q_count.assign(2 * static_cast<size_t>(P), 0);
  L.n_priority = 0;
  for (int32_t j = 0; j < n; ++j) {
    if (nseg(j) == 0) continue;
    const Segment& s0 = firsts[j];
    const bool pri = is_priority(j);
    L.n_priority += pri ? 1 : 0;
    const int32_t q = (pri ? P : 0) + s0.worker;
    L.qnext0[L.qtail0[q]] = j;
    L.qtail0[q] = j;
    L.desc0[4 * static_cast<size_t>(j) + 0] = static_cast<int32_t>(static_cast<uint64_t>(s0.start) & 0xffffffffu);
    L.desc0[4 * static_cast<size_t>(j) + 1] = static_cast<int32_t>(s0.start >> 32);
    L.desc0[4 * static_cast<size_t>(j) + 2] = s0.len;
    L.desc0[4 * static_cast<size_t>(j) + 3] = pri ? static_cast<int32_t>(0x80000000u) : 0;
    int32_t* fm = L.first_mail.data() + 8 * static_cast<size_t>(j);
    fm[0] = static_cast<int32_t>(static_cast<uint64_t>(s0.start) & 0xffffffffu);
    fm[1] = static_cast<int32_t>(s0.start >> 32);
    fm[2] = s0.len;
    fm[3] = 0;
    fm[4] = 0;  // pass count, set per launch
    fm[5] = static_cast<int32_t>(static_cast<uint32_t>(nseg(j)) | (pri ? 0x80000000u : 0u));
    fm[6] = static_cast<int32_t>(static_cast<uint64_t>(L.vl_ptr[j]) & 0xffffffffu);
    fm[7] = static_cast<int32_t>(L.vl_ptr[j] >> 32);
    L.first_q[2 * static_cast<size_t>(j)] = q;
    L.first_q[2 * static_cast<size_t>(j) + 1] = L.q_count[q]++;
  }
}

int build_dsgd_layout(const nomad_gpu_matrix& A, int32_t m, int32_t n, int32_t innerB,
                      int32_t col_blocks, DsgdLayout& D) {
  RowMajor R;
  int rc = to_row_major(A, m, n, R, host_threads());
  if (rc) return rc;
  if (innerB <= 0 || col_blocks <= 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "DSGD needs innerB > 0");
  D.innerB = innerB;
  D.col_blocks = col_blocks;
  D.innerBm = m / innerB + ((m % innerB) ? 1 : 0);
  D.innerBn = n / col_blocks + ((n % col_blocks) ? 1 : 0);
  if (D.innerBm == 0) D.innerBm = 1;
  if (D.innerBn == 0) D.innerBn = 1;
  const int64_t nb = static_cast<int64_t>(innerB) * col_blocks;
  const int64_t nnz = A.nnz;
  D.blk_ptr.assign(static_cast<size_t>(nb) + 1, 0);
  auto bid_of = [&](int32_t r, int32_t c) {
    return static_cast<int64_t>(r / D.innerBm) * col_blocks + c / D.innerBn;
  };
  for (int32_t r = 0; r < m; ++r)
    for (int64_t i = R.row_ptr[r]; i < R.row_ptr[r + 1]; ++i) D.blk_ptr[bid_of(r, R.cols[i]) + 1]++;
  for (int64_t b = 0; b < nb; ++b) D.blk_ptr[b + 1] += D.blk_ptr[b];
  D.rates.resize(static_cast<size_t>(nnz) * 4);
  std::vector<int64_t> fill(D.blk_ptr.begin() + 1, D.blk_ptr.end());  // fill backwards
  for (int32_t r = 0; r < m; ++r)
    for (int64_t i = R.row_ptr[r]; i < R.row_ptr[r + 1]; ++i) {
      const int64_t o = --fill[bid_of(r, R.cols[i])];
      const float v = R.val(i);
      int32_t bits;
      std::memcpy(&bits, &v, 4);
      D.rates[o * 4 + 0] = r;
      D.rates[o * 4 + 1] = R.cols[i];
      D.rates[o * 4 + 2] = bits;
      D.rates[o * 4 + 3] = 0;
    }
  return NOMAD_OK;
}

void dsgd_schedule(int32_t innerB, int32_t iter, int32_t strategy, std::vector<int32_t>& out) {
  // inner_perm / inner_offset persist across iterations and are reshuffled under
  // WOR_STRATUM after srand(34586 + iter) (sgd-mpi-omp.cpp:290-352); with B = 1 the
  // outer shuffles draw nothing.  Shuffle = libstdc++ random_shuffle: for i = 1..N-1
  // swap a[i] with a[rand() % (i+1)].
  std::vector<int32_t> perm(innerB), offset(innerB), cur(innerB);
  std::iota(perm.begin(), perm.end(), 0);
  std::iota(offset.begin(), offset.end(), 0);
  auto shuffle = [](std::vector<int32_t>& a, GlibcRand& g) {
    for (size_t i = 1; i < a.size(); ++i) {
      const size_t j = static_cast<size_t>(g.next()) % (i + 1);
      if (i != j) std::swap(a[i], a[j]);
    }
  };
  for (int32_t it = 1; it <= iter; ++it) {
    GlibcRand g(34586u + static_cast<unsigned>(it));
    if (strategy == 2) {
      shuffle(perm, g);
      shuffle(offset, g);
    }
  }
  out.assign(static_cast<size_t>(innerB) * innerB, 0);
  for (int32_t i = 0; i < innerB; ++i) {
    for (int32_t ii = 0; ii < innerB; ++ii) cur[perm[ii]] = (ii + offset[i]) % innerB;
    for (int32_t bi = 0; bi < innerB; ++bi) out[static_cast<size_t>(i) * innerB + bi] = cur[bi];
  }
}

void dsgdpp_schedule(int32_t innerB, int32_t iter, int32_t strategy, std::vector<int32_t>& out) {
  // dsgd_mpi of dsgdpp.cpp resets inner_perm / inner_offset to the identity every
  // iteration; under WOR_STRATUM they are shuffled once, in phase 0, after
  // srand(34586 + iter) (the outer B = 1 shuffles draw nothing), and phase 1 reuses
  // them.
  std::vector<int32_t> perm(innerB), offset(innerB), cur(innerB);
  std::iota(perm.begin(), perm.end(), 0);
  std::iota(offset.begin(), offset.end(), 0);
  if (strategy == 2) {
    GlibcRand g(34586u + static_cast<unsigned>(iter));
    for (auto* a : {&perm, &offset})
      for (size_t i = 1; i < a->size(); ++i) {
        const size_t j = static_cast<size_t>(g.next()) % (i + 1);
        if (i != j) std::swap((*a)[i], (*a)[j]);
      }
  }
  out.assign(static_cast<size_t>(2) * innerB * innerB, 0);
  for (int32_t p = 0; p < 2; ++p)
    for (int32_t i = 0; i < innerB; ++i) {
      for (int32_t ii = 0; ii < innerB; ++ii) cur[perm[ii]] = (ii + offset[i]) % innerB;
      for (int32_t bi = 0; bi < innerB; ++bi)
        out[(static_cast<size_t>(p) * innerB + i) * innerB + bi] = p * innerB + cur[bi];
    }
}

}  // namespace nomad
