// tune.h -- the search of nomad_gpu_autotune, apart from the measurement.
#pragma once

#include <cstdint>
#include <vector>

#include "nomad_gpu.h"

namespace nomad {

// The ASYNC kernel's default long-visit length for the row type.
inline int32_t default_long_visit(bool bf16) { return bf16 ? 17 : 14; }

// Coordinate descent over the ASYNC kernel's runtime knobs: warps per block (the compiled
// maximum -- what 0 asks for -- then two and four fewer), then the priority threshold
// (25, 50, 100 permille, off), then the long-visit length (10, 14, 20), each stage
// starting from the best so far.  measure(trial) runs trial.{warps_per_block,
// priority_permille, long_visit} and fills trial.status, trial.device_ms and
// trial.warps_per_block (the count the kernel ran with).  A configuration is measured
// once; failed trials (status != NOMAD_OK) never win.  Every trial is appended to `done`.
// lv0 = 0 starts from lv_default (the context's default for the row type).  Returns false
// when no trial succeeded; else the winner in *wpb, *pri, *lv.
template <typename Measure>
bool tune_descent(int32_t pri0, int32_t lv0, Measure&& measure, std::vector<nomad_gpu_tune_trial>& done,
                  int32_t* wpb, int32_t* pri, int32_t* lv, int32_t lv_default = 14) {
  auto run = [&](int32_t w, int32_t p, int32_t l) -> double {
    for (const auto& t : done)
      if (t.warps_per_block == w && t.priority_permille == p && t.long_visit == l)
        return t.status == NOMAD_OK ? t.device_ms : -1.0;
    nomad_gpu_tune_trial t{w, p, l, NOMAD_OK, -1.0};
    measure(t);
    t.priority_permille = p;
    t.long_visit = l;
    done.push_back(t);
    return t.status == NOMAD_OK ? t.device_ms : -1.0;
  };
  auto better = [](double a, double b) { return a >= 0 && (b < 0 || a < b); };
  *pri = pri0 == 0 ? 50 : pri0;  // the defaults, spelt out
  *lv = lv0 > 0 ? lv0 : lv_default;
  double best = run(0, *pri, *lv);
  const int32_t cap = done.back().status == NOMAD_OK ? done.back().warps_per_block : 0;
  *wpb = cap;
  for (int32_t w : {cap - 2, cap - 4}) {
    if (w < 1) continue;
    const double ms = run(w, *pri, *lv);
    if (better(ms, best)) {
      best = ms;
      *wpb = w;
    }
  }
  for (int32_t p : {25, 50, 100, -1}) {
    const double ms = run(*wpb, p, *lv);
    if (better(ms, best)) {
      best = ms;
      *pri = p;
    }
  }
  for (int32_t l : {10, 14, 20}) {
    const double ms = run(*wpb, *pri, l);
    if (better(ms, best)) {
      best = ms;
      *lv = l;
    }
  }
  return best >= 0;
}

// The batched form's large-problem threshold (params.batch_share): the starting share
// (0 means the default 1) first, then every other share of {1, 2, 4, 8, 16, never (-1)},
// each measured once.  measure(trial) runs trial.batch_share and fills trial.status,
// trial.device_ms and trial.large_problems; failed trials never win.  Every trial is
// appended to `done`.  Returns false when no trial succeeded; else the winner in *share.
template <typename Measure>
bool batch_share_search(int32_t share0, Measure&& measure, std::vector<nomad_gpu_batch_tune_trial>& done,
                        int32_t* share) {
  const int32_t first = share0 == 0 ? 1 : share0;
  std::vector<int32_t> order{first};
  for (int32_t v : {1, 2, 4, 8, 16, -1})
    if (v != first) order.push_back(v);
  double best = -1.0;
  for (int32_t v : order) {
    nomad_gpu_batch_tune_trial t{v, NOMAD_OK, -1.0, 0, 0};
    measure(t);
    t.batch_share = v;
    done.push_back(t);
    if (t.status == NOMAD_OK && t.device_ms >= 0 && (best < 0 || t.device_ms < best)) {
      best = t.device_ms;
      *share = v;
    }
  }
  return best >= 0;
}

}  // namespace nomad
