// Invariants of the host-side layouts (nomad_gb300/csrc/host_layout.cpp) on seeded
// random matrices, on the CPU: the CSC holds every rating once, columns ascending by
// row, with the row counts of the input; the worker row blocks are contiguous and cover
// every row; a column's visits cover its ratings exactly once, each visit a run of rows
// owned by one worker (or one group of `group` workers for a priority column); routes
// that keep a group's visits consecutive do so; every active token starts in exactly one
// queue, at a rank below that queue's count; the DSGD blocks hold every rating exactly
// once, in the block of its cell.  Prints "layout ok" and exits 0 when all cases hold.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <set>
#include <tuple>
#include <vector>

#include "layout.h"

namespace {

int g_fail = 0;
#define CHECK(c)                                                             \
  do {                                                                       \
    if (!(c)) {                                                              \
      std::printf("FAIL line %d: %s\n", __LINE__, #c);                       \
      if (++g_fail > 20) return;                                             \
    }                                                                        \
  } while (0)

uint64_t g_s = 0x243F6A8885A308D3ull;
uint32_t next_u32() {
  g_s ^= g_s << 13;
  g_s ^= g_s >> 7;
  g_s ^= g_s << 17;
  return static_cast<uint32_t>(g_s >> 11);
}

// m x n with about `per_row` distinct columns per row, skewed towards low column ids.
void run_case(int32_t m, int32_t n, int per_row, int32_t P, int balance, int64_t pri_min, int32_t group,
              bool group_routes, int threads) {
  std::vector<int32_t> rc(m), cols;
  std::vector<float> vals;
  for (int32_t i = 0; i < m; ++i) {
    std::set<int32_t> cs;
    const int k = static_cast<int>(next_u32() % (2 * per_row + 1));
    while (static_cast<int>(cs.size()) < std::min(k, n)) {
      const uint32_t a = next_u32() % n, b = next_u32() % n;
      cs.insert(static_cast<int32_t>(std::min(a, b)));  // skew: more ratings in low columns
    }
    rc[i] = static_cast<int32_t>(cs.size());
    for (int32_t c : cs) {
      cols.push_back(c);
      vals.push_back(static_cast<float>(1 + next_u32() % 5));
    }
  }
  const int64_t nnz = static_cast<int64_t>(cols.size());
  nomad_gpu_matrix A{nnz, rc.data(), nullptr, cols.data(), nullptr, vals.data()};
  nomad::Csc csc;
  CHECK(nomad::build_csc(A, m, n, csc, threads) == 0);
  CHECK(csc.nnz() == nnz);
  CHECK(csc.row_nnz.size() == static_cast<size_t>(m));
  for (int32_t i = 0; i < m && i < static_cast<int32_t>(csc.row_nnz.size()); ++i) CHECK(csc.row_nnz[i] == rc[i]);
  std::vector<int32_t> seen_per_row(m, 0);
  for (int32_t j = 0; j < n; ++j)
    for (int64_t o = csc.col_ptr[j]; o < csc.col_ptr[j + 1]; ++o) {
      if (o > csc.col_ptr[j]) CHECK(csc.ratings[o].row > csc.ratings[o - 1].row);
      ++seen_per_row[csc.ratings[o].row];
    }
  CHECK(seen_per_row == rc);

  for (int with_counts = 0; with_counts < 2; ++with_counts) {
    nomad::Csc c2;
    const nomad::Csc* cp = &csc;
    if (!with_counts) {  // the same layout without the row counts (per-thread histograms)
      c2.m = csc.m;
      c2.n = csc.n;
      c2.col_ptr = csc.col_ptr;
      c2.ratings = csc.ratings;
      cp = &c2;
    }
    nomad::AsyncLayout L;
    CHECK(nomad::build_async_layout(*cp, P, balance, 12345, pri_min, group, group_routes, L, threads) == 0);
    CHECK(L.row_start.size() == static_cast<size_t>(P) + 1);
    CHECK(L.row_start[0] == 0 && L.row_start[P] == m);
    for (int32_t w = 0; w < P; ++w) CHECK(L.row_start[w] <= L.row_start[w + 1]);
    std::vector<int32_t> owner(m);
    for (int32_t w = 0; w < P; ++w)
      for (int32_t r = L.row_start[w]; r < L.row_start[w + 1]; ++r) owner[r] = w;
    int64_t covered = 0, n_pri = 0, n_active = 0;
    std::vector<int32_t> qcount(2 * static_cast<size_t>(P), 0);
    for (int32_t j = 0; j < n; ++j) {
      const int64_t len = csc.col_ptr[j + 1] - csc.col_ptr[j];
      const bool pri = pri_min > 0 && len >= pri_min;
      n_pri += pri && len > 0;
      std::vector<int64_t> starts;
      std::set<int32_t> targets;
      int32_t prev_group = -1;
      std::set<int32_t> closed_groups;
      for (int64_t v = L.vl_ptr[j]; v < L.vl_ptr[j + 1]; ++v) {
        const nomad::Segment& sg = L.segs[v];
        CHECK(sg.len > 0);
        CHECK(sg.start >= csc.col_ptr[j] && sg.start + sg.len <= csc.col_ptr[j + 1]);
        starts.push_back(sg.start);
        covered += sg.len;
        for (int64_t o = sg.start; o < sg.start + sg.len; ++o) {
          const int32_t w = owner[csc.ratings[o].row];
          CHECK((pri ? w / group : w) == sg.worker);
        }
        CHECK(targets.insert(sg.worker).second);  // one visit per owner
        if (group_routes && !pri && group > 1) {  // a group's visits stay consecutive
          const int32_t g = sg.worker / group;
          if (g != prev_group) {
            CHECK(closed_groups.count(g) == 0);
            if (prev_group >= 0) closed_groups.insert(prev_group);
            prev_group = g;
          }
        }
      }
      std::sort(starts.begin(), starts.end());  // the visits tile the column
      int64_t pos = csc.col_ptr[j];
      for (int64_t st : starts) {
        CHECK(st == pos);
        int64_t l = 0;
        for (int64_t v = L.vl_ptr[j]; v < L.vl_ptr[j + 1]; ++v)
          if (L.segs[v].start == st) l = L.segs[v].len;
        pos += l;
      }
      CHECK(pos == csc.col_ptr[j + 1]);
      const int32_t q = L.first_q[2 * static_cast<size_t>(j)], rank = L.first_q[2 * static_cast<size_t>(j) + 1];
      if (len == 0) {
        CHECK(q == -1);
        continue;
      }
      ++n_active;
      const nomad::Segment& s0 = L.segs[L.vl_ptr[j]];
      CHECK(q == (pri ? P : 0) + s0.worker);
      CHECK(rank == qcount[q]++);
    }
    CHECK(covered == nnz);
    CHECK(L.n_active == n_active);
    CHECK(L.n_priority == n_pri);
    for (size_t q = 0; q < qcount.size(); ++q) CHECK(L.q_count[q] == qcount[q]);
  }
}

// DSGD blocks: innerB row blocks x col_blocks column blocks of ceil(m / innerB) rows and
// ceil(n / col_blocks) columns; every rating exactly once, in the block of its cell
// (the order inside a block is the fill's; only membership is checked).
void run_dsgd_case(int32_t m, int32_t n, int per_row, int32_t innerB, int32_t col_blocks) {
  std::vector<int32_t> rc(m), cols;
  std::vector<float> vals;
  for (int32_t i = 0; i < m; ++i) {
    std::set<int32_t> cs;
    const int k = static_cast<int>(next_u32() % (2 * per_row + 1));
    while (static_cast<int>(cs.size()) < std::min(k, n)) cs.insert(static_cast<int32_t>(next_u32() % n));
    rc[i] = static_cast<int32_t>(cs.size());
    for (int32_t c : cs) {
      cols.push_back(c);
      vals.push_back(static_cast<float>(next_u32() % 1000) / 7.f);
    }
  }
  const int64_t nnz = static_cast<int64_t>(cols.size());
  nomad_gpu_matrix A{nnz, rc.data(), nullptr, cols.data(), nullptr, vals.data()};
  nomad::DsgdLayout D;
  CHECK(nomad::build_dsgd_layout(A, m, n, innerB, col_blocks, D) == 0);
  CHECK(D.innerBm == std::max(1, m / innerB + (m % innerB ? 1 : 0)));
  CHECK(D.innerBn == std::max(1, n / col_blocks + (n % col_blocks ? 1 : 0)));
  const int64_t nb = static_cast<int64_t>(innerB) * col_blocks;
  CHECK(D.blk_ptr.size() == static_cast<size_t>(nb) + 1 && D.blk_ptr[0] == 0 && D.blk_ptr[nb] == nnz);
  std::multiset<std::tuple<int32_t, int32_t, float>> want, got;
  int64_t o = 0;
  for (int32_t i = 0; i < m; ++i)
    for (int32_t q = 0; q < rc[i]; ++q, ++o) want.insert({i, cols[o], vals[o]});
  for (int64_t b = 0; b < nb; ++b) {
    CHECK(D.blk_ptr[b] <= D.blk_ptr[b + 1]);
    for (int64_t e = D.blk_ptr[b]; e < D.blk_ptr[b + 1]; ++e) {
      const int32_t r = D.rates[4 * e], c = D.rates[4 * e + 1];
      float v;
      std::memcpy(&v, &D.rates[4 * e + 2], 4);
      CHECK(D.rates[4 * e + 3] == 0);
      CHECK(static_cast<int64_t>(r / D.innerBm) * col_blocks + c / D.innerBn == b);
      got.insert({r, c, v});
    }
  }
  CHECK(got == want);
}

// Out-of-range column indices anywhere in the input (first, middle, last entry; too large
// or negative) are an invalid argument, for one and several threads.
void run_bad_column_cases() {
  const int32_t m = 3000, n = 40;
  for (int threads : {1, 4})
    for (int64_t where : {int64_t(0), int64_t(60000), int64_t(m) * n - 1})
      for (int32_t badc : {n, -1}) {
        std::vector<int32_t> rc(m, n), cols;
        for (int32_t i = 0; i < m; ++i)
          for (int32_t j = 0; j < n; ++j) cols.push_back(j);
        cols[static_cast<size_t>(where)] = badc;
        std::vector<float> vals(cols.size(), 1.f);
        nomad_gpu_matrix A{static_cast<int64_t>(cols.size()), rc.data(), nullptr, cols.data(), nullptr, vals.data()};
        nomad::Csc csc;
        CHECK(nomad::build_csc(A, m, n, csc, threads) == NOMAD_ERR_INVALID_ARG);
      }
}

}  // namespace

int main() {
  // m, n, ratings per row, workers, balance, priority threshold, group, group routes, threads
  run_case(3000, 200, 12, 64, 1, 0, 1, false, 4);
  run_case(3000, 200, 12, 64, 0, 0, 1, false, 3);
  run_case(5000, 300, 20, 60, 1, 150, 12, true, 8);
  run_case(5000, 300, 20, 40, 1, 100, 10, true, 1);
  run_case(400, 50, 5, 7, 1, 30, 3, true, 2);
  run_case(17, 9, 3, 30, 1, 0, 1, false, 4);  // more workers than rows
  run_bad_column_cases();
  run_dsgd_case(500, 80, 6, 4, 4);
  run_dsgd_case(501, 83, 6, 7, 14);  // DSGD++'s innerB x 2 innerB grid, ragged edges
  run_dsgd_case(3, 2, 1, 8, 8);      // more blocks than rows and columns
  std::printf("%s\n", g_fail ? "layout FAILED" : "layout ok");
  return g_fail ? 1 : 0;
}
