// host_synth.cpp -- seeded synthetic rating matrices with planted low-rank factors.
//
// The approach follows the one Code/nomad/synthgen.cpp:231-262 takes (draw a degree
// per row, draw that many distinct columns from a weighted column law, value =
// <w*_i, h*_j> + noise) but is a new generator: per-row counter-based streams make
// the output independent of the thread count, the totals are exact, dense rows are
// sampled by exponential keys instead of rejection, and the split is exact.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <unordered_set>

#include "common.h"

namespace {

using nomad::SplitMix64;
using nomad::stream_key;

enum : uint64_t {
  kTagRowPerm = 1, kTagColPerm, kTagRowDeg, kTagRow, kTagRowFactor, kTagColFactor,
  kTagSplit, kTagCells, kTagFix
};

// Walker/Vose alias table for O(1) weighted draws.
struct Alias {
  std::vector<double> prob;
  std::vector<int32_t> alias;
  explicit Alias(const std::vector<double>& w) {
    const int32_t n = static_cast<int32_t>(w.size());
    prob.assign(n, 0.0);
    alias.assign(n, 0);
    const double total = std::accumulate(w.begin(), w.end(), 0.0);
    std::vector<double> p(n);
    std::vector<int32_t> small, large;
    for (int32_t i = 0; i < n; ++i) {
      p[i] = w[i] * n / total;
      (p[i] < 1.0 ? small : large).push_back(i);
    }
    while (!small.empty() && !large.empty()) {
      const int32_t s = small.back(), l = large.back();
      small.pop_back();
      prob[s] = p[s];
      alias[s] = l;
      p[l] = (p[l] + p[s]) - 1.0;
      if (p[l] < 1.0) {
        large.pop_back();
        small.push_back(l);
      }
    }
    for (int32_t i : large) prob[i] = 1.0;
    for (int32_t i : small) prob[i] = 1.0;
  }
  int32_t draw(SplitMix64& r) const {
    const int32_t i = static_cast<int32_t>(r.below(prob.size()));
    return r.uniform() < prob[i] ? i : alias[i];
  }
};

// Weights of a law over `count` indices; ZIPF ranks are a seeded permutation so the
// heavy indices are scattered (as convert.py's shuffled ids scatter real ones).
std::vector<double> law_weights(int32_t law, double param, int32_t count,
                                uint64_t seed, uint64_t tag) {
  std::vector<double> w(count, 1.0);
  if (law == NOMAD_LAW_ZIPF) {
    std::vector<int32_t> rank(count);
    std::iota(rank.begin(), rank.end(), 0);
    SplitMix64 r(stream_key(seed, tag, 0));
    for (int32_t i = count - 1; i > 0; --i) std::swap(rank[i], rank[r.below(i + 1)]);
    for (int32_t i = 0; i < count; ++i) w[i] = std::pow(static_cast<double>(rank[i]) + 1.0, -param);
  } else if (law == NOMAD_LAW_GEOMETRIC) {
    const double p = 1.0 / std::max(param, 1.0);
    const double lq = std::log1p(-std::min(p, 1.0 - 1e-12));
    for (int32_t i = 0; i < count; ++i) {
      SplitMix64 r(stream_key(seed, tag, static_cast<uint64_t>(i)));
      const double u = 1.0 - r.uniform();
      w[i] = p >= 1.0 ? 1.0 : 1.0 + std::floor(std::log(u) / lq);
    }
  }
  return w;
}

// Integer degrees proportional to w, capped at `cap`, summing exactly to `total`
// (water-filling on the scale c, then largest remainders).
bool exact_degrees(const std::vector<double>& w, int64_t cap, int64_t total,
                   std::vector<int64_t>& d) {
  const size_t n = w.size();
  d.assign(n, 0);
  if (total == 0) return true;
  if (static_cast<double>(cap) * n < static_cast<double>(total)) return false;
  auto mass = [&](double c) {
    double s = 0;
    for (size_t i = 0; i < n; ++i) s += std::min(c * w[i], static_cast<double>(cap));
    return s;
  };
  double lo = 0, hi = 1;
  while (mass(hi) < total) hi *= 2;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    (mass(mid) < total ? lo : hi) = mid;
  }
  int64_t sum = 0;
  std::vector<std::pair<double, size_t>> frac;
  frac.reserve(n);
  for (size_t i = 0; i < n; ++i) {
    const double x = std::min(hi * w[i], static_cast<double>(cap));
    d[i] = static_cast<int64_t>(std::floor(x));
    sum += d[i];
    if (d[i] < cap) frac.emplace_back(x - std::floor(x), i);
  }
  // total - sum is small (< n); hand out the remainder to the largest fractions,
  // then (if the floor overshoots after capping) take it back from the smallest.
  std::sort(frac.begin(), frac.end(), [](const auto& a, const auto& b) {
    return a.first != b.first ? a.first > b.first : a.second < b.second;
  });
  size_t k = 0;
  while (sum < total && !frac.empty()) {
    const size_t i = frac[k % frac.size()].second;
    if (d[i] < cap) {
      d[i]++;
      sum++;
    }
    ++k;
    if (k > 4 * n + 16) return false;
  }
  for (size_t i = 0; sum > total && i < n; ++i) {
    const int64_t take = std::min<int64_t>(d[i], sum - total);
    d[i] -= take;
    sum -= take;
  }
  return sum == total;
}

void fill_factor(std::vector<float>& f, int32_t count, int32_t rank, double sd,
                 uint64_t seed, uint64_t tag, int threads) {
  f.assign(static_cast<size_t>(count) * rank, 0.0f);
  nomad::parallel_chunks(count, threads, [&](int, int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      SplitMix64 r(stream_key(seed, tag, static_cast<uint64_t>(i)));
      for (int32_t t = 0; t < rank; ++t) f[i * rank + t] = static_cast<float>(sd * r.normal());
    }
  });
}

int alloc_matrix(nomad_io_matrix* mat, int32_t m, int32_t n, int64_t nnz) {
  std::memset(mat, 0, sizeof(*mat));
  mat->file_id = nnz < (int64_t(1) << 31) ? NOMAD_FILE_ID_INT : NOMAD_FILE_ID_LONG;
  mat->m = m;
  mat->n = n;
  mat->nnz = nnz;
  mat->row_counts = static_cast<int32_t*>(std::calloc(std::max<int64_t>(m, 1), 4));
  mat->cols = static_cast<int32_t*>(std::malloc(std::max<int64_t>(nnz, 1) * 4));
  mat->vals = static_cast<double*>(std::malloc(std::max<int64_t>(nnz, 1) * 8));
  if (!mat->row_counts || !mat->cols || !mat->vals) {
    nomad_io_free(mat);
    return NOMAD_ERR_OOM;
  }
  return NOMAD_OK;
}

}  // namespace

extern "C" {

int nomad_synth_preset(int32_t workload, nomad_synth_spec* s) {
  nomad::clear_last_error();
  if (!s) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null spec");
  std::memset(s, 0, sizeof(*s));
  s->struct_size = sizeof(*s);
  s->seed = 12345;
  s->scale = 1.0;
  switch (workload) {
    case 1:  // 10,000 x 2,000 planted rank 10
      s->m = 10000; s->n = 2000; s->positions = NOMAD_SYNTH_UNIFORM;
      s->nnz_train = 360000; s->nnz_test = 40000;
      s->rank = 10; s->factor_std = 1.0 / std::sqrt(10.0); s->noise_std = 0.1;
      break;
    case 2:  // 480,189 x 17,770 (the Netflix prize shape)
      s->m = 480189; s->n = 17770; s->positions = NOMAD_SYNTH_DEGREES;
      s->nnz_train = 100480507; s->nnz_test = 1408395;
      s->row_law = NOMAD_LAW_ZIPF; s->row_param = 0.8;
      s->col_law = NOMAD_LAW_ZIPF; s->col_param = 1.1;
      s->rank = 20; s->noise_std = 0.3; s->offset = 3.0;
      s->integer_values = 1; s->clip_lo = 1; s->clip_hi = 5;
      break;
    case 3:  // 1,000,990 x 624,961 (the Yahoo! Music shape)
      s->m = 1000990; s->n = 624961; s->positions = NOMAD_SYNTH_DEGREES;
      s->nnz_train = 252800275; s->nnz_test = 4003960;
      s->row_law = NOMAD_LAW_ZIPF; s->row_param = 0.9;
      s->col_law = NOMAD_LAW_ZIPF; s->col_param = 0.9;
      s->rank = 30; s->noise_std = 8.0; s->offset = 50.0; s->scale = 20.0;
      s->integer_values = 1; s->clip_lo = 0; s->clip_hi = 100;
      break;
    case 4:  // 50,082,603 x 39,780 (the Hugewiki shape)
      s->m = 50082603; s->n = 39780; s->positions = NOMAD_SYNTH_DEGREES;
      s->nnz_train = 2740000000LL; s->nnz_test = 30000000LL;
      s->row_law = NOMAD_LAW_GEOMETRIC; s->row_param = 55.0;
      s->col_law = NOMAD_LAW_ZIPF; s->col_param = 1.0;
      s->rank = 50; s->noise_std = 0.2;
      break;
    default:
      NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "unknown workload %d", workload);
  }
  return NOMAD_OK;
}

int nomad_synth_batch_problem(uint64_t seed, int32_t index, nomad_synth_spec* s, int32_t* dim) {
  nomad::clear_last_error();
  if (!s || !dim || index < 0) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid batch problem request");
  std::memset(s, 0, sizeof(*s));
  s->struct_size = sizeof(*s);
  s->scale = 1.0;
  nomad::SplitMix64 rng(nomad::stream_key(seed, 211, static_cast<uint64_t>(index)));
  auto log_uniform = [&](double lo, double hi) { return lo * std::exp(rng.uniform() * std::log(hi / lo)); };
  const int32_t m = static_cast<int32_t>(std::lround(log_uniform(200.0, 20000.0)));
  const int32_t n = static_cast<int32_t>(std::lround(log_uniform(100.0, 5000.0)));
  const double density = log_uniform(0.005, 0.05);
  static const int32_t kRanks[3] = {16, 32, 64};
  const int32_t k = kRanks[rng.below(3)];
  const int64_t cells = std::max<int64_t>(2, std::llround(density * static_cast<double>(m) * n));
  s->m = m;
  s->n = n;
  s->positions = NOMAD_SYNTH_UNIFORM;
  s->nnz_test = std::max<int64_t>(1, cells / 10);
  s->nnz_train = cells - s->nnz_test;
  s->rank = k / 4;
  s->factor_std = 1.0 / std::sqrt(static_cast<double>(k / 4));
  s->noise_std = 0.1;
  s->seed = nomad::stream_key(seed, 223, static_cast<uint64_t>(index));
  *dim = k;
  return NOMAD_OK;
}

int nomad_synth_generate(const nomad_synth_spec* spec, nomad_io_matrix* train,
                         nomad_io_matrix* test) {
  nomad::clear_last_error();
  if (!spec || !train || !test || spec->struct_size != static_cast<int32_t>(sizeof(nomad_synth_spec)))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid spec");
  const nomad_synth_spec& s = *spec;
  const int32_t m = s.m, n = s.n;
  const int64_t T = s.nnz_train + s.nnz_test;
  if (m <= 0 || n <= 0 || s.nnz_train < 0 || s.nnz_test < 0 || s.rank <= 0 ||
      static_cast<double>(T) > static_cast<double>(m) * n)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid synthetic sizes");
  const int threads = nomad::host_threads(s.threads);
  const uint64_t seed = s.seed;

  // ---- positions: per-row sorted column lists in one flat array ------------------
  std::vector<int64_t> row_ptr(static_cast<size_t>(m) + 1, 0);
  std::vector<int32_t> cells_col(static_cast<size_t>(T));
  if (s.positions == NOMAD_SYNTH_UNIFORM) {
    // Floyd's sampling of T distinct cells of the m*n grid, then row-major order.
    const uint64_t N = static_cast<uint64_t>(m) * n;
    std::unordered_set<uint64_t> chosen;
    chosen.reserve(static_cast<size_t>(T) * 2);
    SplitMix64 r(stream_key(seed, kTagCells, 0));
    for (uint64_t j = N - T; j < N; ++j) {
      const uint64_t t = r.below(j + 1);
      if (!chosen.insert(t).second) chosen.insert(j);
    }
    std::vector<uint64_t> ids(chosen.begin(), chosen.end());
    std::sort(ids.begin(), ids.end());
    for (int64_t k = 0; k < T; ++k) {
      row_ptr[ids[k] / n + 1]++;
      cells_col[k] = static_cast<int32_t>(ids[k] % n);
    }
    for (int32_t i = 0; i < m; ++i) row_ptr[i + 1] += row_ptr[i];
  } else if (s.positions == NOMAD_SYNTH_DEGREES) {
    std::vector<int64_t> deg;
    if (!exact_degrees(law_weights(s.row_law, s.row_param, m, seed, kTagRowDeg), n, T, deg))
      NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "cannot place %lld ratings on %d x %d", (long long)T, m, n);
    for (int32_t i = 0; i < m; ++i) row_ptr[i + 1] = row_ptr[i] + deg[i];
    const std::vector<double> cw = law_weights(s.col_law, s.col_param, n, seed, kTagColPerm);
    const Alias alias(cw);
    // Rows are handed out in interleaved blocks so heavy rows spread over threads.
    const int64_t blk = 256;
    const int64_t nblk = (m + blk - 1) / blk;
    nomad::parallel_chunks(threads, threads, [&](int t, int64_t, int64_t) {
      std::vector<uint32_t> stamp(n, 0);
      uint32_t gen = 0;
      std::vector<std::pair<double, int32_t>> keys;
      for (int64_t b = t; b < nblk; b += threads) {
        for (int64_t i = b * blk; i < std::min<int64_t>((b + 1) * blk, m); ++i) {
          const int64_t d = row_ptr[i + 1] - row_ptr[i];
          int32_t* out = cells_col.data() + row_ptr[i];
          SplitMix64 r(stream_key(seed, kTagRow, static_cast<uint64_t>(i)));
          if (d == 0) continue;
          if (d * 16 <= n) {
            // rejection sampling with a generation-stamped membership array
            if (++gen == 0) {
              std::fill(stamp.begin(), stamp.end(), 0);
              gen = 1;
            }
            for (int64_t k = 0; k < d;) {
              const int32_t c = alias.draw(r);
              if (stamp[c] != gen) {
                stamp[c] = gen;
                out[k++] = c;
              }
            }
          } else {
            // Efraimidis-Spirakis: the d largest keys log(u)/w are a weighted
            // sample without replacement.
            keys.resize(n);
            for (int32_t c = 0; c < n; ++c) keys[c] = {std::log(1.0 - r.uniform()) / cw[c], c};
            std::nth_element(keys.begin(), keys.begin() + (d - 1), keys.end(),
                             [](const auto& a, const auto& b) { return a.first > b.first; });
            for (int64_t k = 0; k < d; ++k) out[k] = keys[k].second;
          }
          std::sort(out, out + d);
        }
      }
    });
  } else {
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "unknown positions mode %d", s.positions);
  }

  // ---- exact split: randomized rounding per row, then a seeded fix-up -------------
  std::vector<int64_t> tcount(m, 0);
  {
    const double q = T ? static_cast<double>(s.nnz_test) / static_cast<double>(T) : 0.0;
    int64_t sum = 0;
    for (int32_t i = 0; i < m; ++i) {
      const int64_t d = row_ptr[i + 1] - row_ptr[i];
      SplitMix64 r(stream_key(seed, kTagSplit, static_cast<uint64_t>(i)));
      tcount[i] = std::min<int64_t>(d, static_cast<int64_t>(std::floor(d * q + r.uniform())));
      sum += tcount[i];
    }
    SplitMix64 r(stream_key(seed, kTagFix, 0));
    int64_t guard = 0;
    while (sum != s.nnz_test && guard++ < int64_t(1) << 40) {
      const int32_t i = static_cast<int32_t>(r.below(m));
      const int64_t d = row_ptr[i + 1] - row_ptr[i];
      if (sum < s.nnz_test && tcount[i] < d) {
        tcount[i]++;
        sum++;
      } else if (sum > s.nnz_test && tcount[i] > 0) {
        tcount[i]--;
        sum--;
      }
    }
  }

  int rc = alloc_matrix(train, m, n, s.nnz_train);
  if (rc) NOMAD_FAIL(rc, "host allocation failed");
  rc = alloc_matrix(test, m, n, s.nnz_test);
  if (rc) {
    nomad_io_free(train);
    NOMAD_FAIL(rc, "host allocation failed");
  }
  std::vector<int64_t> tr_ptr(static_cast<size_t>(m) + 1, 0), te_ptr(static_cast<size_t>(m) + 1, 0);
  for (int32_t i = 0; i < m; ++i) {
    const int64_t d = row_ptr[i + 1] - row_ptr[i];
    train->row_counts[i] = static_cast<int32_t>(d - tcount[i]);
    test->row_counts[i] = static_cast<int32_t>(tcount[i]);
    tr_ptr[i + 1] = tr_ptr[i] + (d - tcount[i]);
    te_ptr[i + 1] = te_ptr[i] + tcount[i];
  }

  // ---- planted values -------------------------------------------------------------
  const double fsd = s.factor_std > 0 ? s.factor_std : std::pow(static_cast<double>(s.rank), -0.25);
  std::vector<float> U, V;
  fill_factor(U, m, s.rank, fsd, seed, kTagRowFactor, threads);
  fill_factor(V, n, s.rank, fsd, seed, kTagColFactor, threads);
  nomad::parallel_chunks(m, threads, [&](int, int64_t lo, int64_t hi) {
    std::vector<uint8_t> is_test;
    for (int64_t i = lo; i < hi; ++i) {
      const int64_t d = row_ptr[i + 1] - row_ptr[i];
      const int32_t* c = cells_col.data() + row_ptr[i];
      SplitMix64 r(stream_key(seed, kTagSplit ^ 0x55, static_cast<uint64_t>(i)));
      // choose which tcount[i] of the row's d cells are test cells (partial shuffle)
      is_test.assign(d, 0);
      std::vector<int32_t> idx(d);
      std::iota(idx.begin(), idx.end(), 0);
      for (int64_t k = 0; k < tcount[i]; ++k) {
        const int64_t pick = k + static_cast<int64_t>(r.below(d - k));
        std::swap(idx[k], idx[pick]);
        is_test[idx[k]] = 1;
      }
      int64_t a = tr_ptr[i], b = te_ptr[i];
      const float* u = U.data() + i * s.rank;
      for (int64_t k = 0; k < d; ++k) {
        const float* v = V.data() + static_cast<int64_t>(c[k]) * s.rank;
        double dot = 0;
        for (int32_t t = 0; t < s.rank; ++t) dot += static_cast<double>(u[t]) * v[t];
        double val = s.offset + s.scale * dot + s.noise_std * r.normal();
        if (s.integer_values) val = std::min(s.clip_hi, std::max(s.clip_lo, std::nearbyint(val)));
        if (is_test[k]) {
          test->cols[b] = c[k];
          test->vals[b++] = val;
        } else {
          train->cols[a] = c[k];
          train->vals[a++] = val;
        }
      }
    }
  });
  return NOMAD_OK;
}

}  // extern "C"
