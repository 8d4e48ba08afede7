// The search of nomad_gpu_autotune (nomad_gb300/csrc/tune.h) against synthetic cost
// functions, on the CPU: the configuration it returns, which trials it measures (each
// once), and how it treats failed trials and small warp counts.  Prints "tune ok" and
// exits 0 when every case holds.
#include <cstdio>
#include <vector>

#include "tune.h"

namespace {

int g_fail = 0;
#define CHECK(c)                                               \
  do {                                                         \
    if (!(c)) {                                                \
      std::printf("FAIL line %d: %s\n", __LINE__, #c);         \
      ++g_fail;                                                \
    }                                                          \
  } while (0)

// A kernel compiled for `cap` warps per block whose epoch time is the sum of one
// penalty per knob; configurations in `fail` end with an error.
struct Model {
  int cap;
  int best_w, best_p, best_l;
  std::vector<std::vector<int>> fail;
  int calls = 0;
  void operator()(nomad_gpu_tune_trial& t) {
    ++calls;
    const int w = t.warps_per_block == 0 ? cap : t.warps_per_block;
    for (const auto& f : fail)
      if (f[0] == t.warps_per_block && f[1] == t.priority_permille && f[2] == t.long_visit) {
        t.status = NOMAD_ERR_CUDA;
        return;
      }
    t.warps_per_block = w;
    t.device_ms = 50.0 + (w == best_w ? 0 : 3) + (t.priority_permille == best_p ? 0 : 2) +
                  (t.long_visit == best_l ? 0 : 1) + 0.01 * w;
  }
};

void case_descent() {
  Model m{10, 8, 100, 10, {}};
  std::vector<nomad_gpu_tune_trial> done;
  int32_t w = 0, p = 0, l = 0;
  CHECK(nomad::tune_descent(0, 0, m, done, &w, &p, &l));
  CHECK(w == 8 && p == 100 && l == 10);
  CHECK(done.size() == 8 && m.calls == 8);  // 3 + 3 + 2: repeated configurations are not re-run
  CHECK(done[0].warps_per_block == 10 && done[0].priority_permille == 50 && done[0].long_visit == 14);
  for (size_t i = 0; i < done.size(); ++i)
    for (size_t j = i + 1; j < done.size(); ++j)
      CHECK(!(done[i].warps_per_block == done[j].warps_per_block &&
              done[i].priority_permille == done[j].priority_permille && done[i].long_visit == done[j].long_visit));
}

void case_defaults_kept() {  // the starting point already the best: nothing changes
  Model m{12, 12, -1, 20, {}};
  std::vector<nomad_gpu_tune_trial> done;
  int32_t w = 0, p = 0, l = 0;
  CHECK(nomad::tune_descent(-1, 20, m, done, &w, &p, &l));
  CHECK(w == 12 && p == -1 && l == 20);
  CHECK(done[0].priority_permille == -1 && done[0].long_visit == 20);
}

void case_failures() {
  std::vector<nomad_gpu_tune_trial> done;
  int32_t w = 0, p = 0, l = 0;
  // the otherwise best configuration fails: the next best wins
  Model m{10, 8, 100, 10, {{8, 100, 14}, {8, 100, 10}}};
  CHECK(nomad::tune_descent(0, 0, m, done, &w, &p, &l));
  CHECK(w == 8 && p != 100);
  for (const auto& t : done)
    if (t.status != NOMAD_OK) CHECK(t.device_ms < 0);
  // nothing completes
  struct Never {
    void operator()(nomad_gpu_tune_trial& t) { t.status = NOMAD_ERR_TIMEOUT; }
  } never;
  done.clear();
  CHECK(!nomad::tune_descent(0, 0, never, done, &w, &p, &l));
  CHECK(!done.empty() && done.front().status == NOMAD_ERR_TIMEOUT);
}

void case_small_blocks() {  // two warps per block: no trial below one warp
  Model m{2, 2, 50, 14, {}};
  std::vector<nomad_gpu_tune_trial> done;
  int32_t w = 0, p = 0, l = 0;
  CHECK(nomad::tune_descent(0, 0, m, done, &w, &p, &l));
  CHECK(w == 2);
  for (const auto& t : done) CHECK(t.warps_per_block >= 1);
}

// The batched threshold search against a synthetic cost with its minimum at `best`.
struct BatchModel {
  int best;
  int fail_share = 999;
  int calls = 0;
  void operator()(nomad_gpu_batch_tune_trial& t) {
    ++calls;
    if (t.batch_share == fail_share) {
      t.status = NOMAD_ERR_OOM;
      return;
    }
    const int s = t.batch_share < 0 ? 64 : t.batch_share;
    const int b = best < 0 ? 64 : best;
    t.device_ms = 10.0 + (s > b ? s - b : b - s);
    t.large_problems = t.batch_share < 0 ? 0 : 100 / s;
  }
};

void case_batch_share() {
  std::vector<nomad_gpu_batch_tune_trial> done;
  int32_t share = 0;
  BatchModel m{8};
  CHECK(nomad::batch_share_search(0, m, done, &share));
  CHECK(share == 8 && m.calls == 6 && done.size() == 6);
  CHECK(done[0].batch_share == 1);  // the default first
  for (size_t i = 0; i < done.size(); ++i)
    for (size_t j = i + 1; j < done.size(); ++j) CHECK(done[i].batch_share != done[j].batch_share);
  done.clear();
  BatchModel never_big{-1};
  CHECK(nomad::batch_share_search(0, never_big, done, &share));
  CHECK(share == -1 && done.back().large_problems == 0);
  done.clear();
  BatchModel odd{3};  // a starting share outside the list is measured too
  CHECK(nomad::batch_share_search(3, odd, done, &share));
  CHECK(share == 3 && done.size() == 7 && done[0].batch_share == 3);
  done.clear();
  BatchModel failing{2};
  failing.fail_share = 2;  // the best share fails: the next best wins
  CHECK(nomad::batch_share_search(0, failing, done, &share));
  CHECK(share == 1);  // |1 - 2| = 1 beats |4 - 2| = 2
  struct Never {
    void operator()(nomad_gpu_batch_tune_trial& t) { t.status = NOMAD_ERR_TIMEOUT; }
  } never;
  done.clear();
  CHECK(!nomad::batch_share_search(0, never, done, &share));
}

}  // namespace

int main() {
  case_batch_share();
  case_descent();
  case_defaults_kept();
  case_failures();
  case_small_blocks();
  std::printf("%s\n", g_fail ? "tune FAILED" : "tune ok");
  return g_fail ? 1 : 0;
}
