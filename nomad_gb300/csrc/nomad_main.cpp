// nomad_main.cpp -- `nomad_gpu`, the command-line driver.  It keeps the reference's
// command-line surface (NomadOption, Code/nomad/nomad_option.cpp:16-77, plus the legacy
// --path of realdata_body.hpp:223), reads train.dat / test.dat from the data directory
// (nb_data.cpp:180-226), trains through the C-ABI and prints the reference's statistics
// block after every --timeout point (nb_main.cpp:264-300).
//
// The timeout list is cumulative wall-clock seconds of training, as in the reference
// (nb_main.cpp:109-113); training advances in whole epochs and the budget is checked
// between epochs.  --epochs N trains exactly N epochs per timeout point instead.
//
// Online termination follows NomadBody::master_termcheck (nb_master.cpp:16-46): every
// --tm_interval seconds of training the online RMSE, sqrt(sum of the squared errors the
// column tokens saw on their latest pass / training nnz), is compared with the previous
// check; training stops for good once it changed by at most --tm_error, or once it is
// at most --tm_value after 8 passes of every column (the reference's 8 * machines *
// columns column sends: one send per machine per pass).
//
// Checkpoints (--cptype, --cpinterval, --cppath) are taken between epochs, every
// --cpinterval seconds of training, as <cppath>/cp-t<jobid>-e<k>.ckpt; --recover k
// resumes from one (nb_master.cpp:69-104, nb_checkpoint.cpp:37-42, nb_main.cpp:446-449).
// Between epochs no column token is in flight, so the reference's sync, async and vs
// protocols, which differ in how they capture messages in flight, all save the same
// state here: the factors and the pass count.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "nomad_gpu.h"
#include "nomad_io.h"

namespace {

struct Options {
  int nthreads = 4;
  double lrate = 0.001, drate = 0.1, reg = 1.0;
  unsigned long long seed = 12345;
  int cpm = 100;
  double tpm = 0.5;
  std::vector<double> timeouts{10.0};
  double tm_value = 1, tm_error = 1e-6, tm_interval = 1, tm_portion = 0.01;
  int dim = 100, reuse = 1;
  bool pause = true, random_send = true;
  double r0delay = 0;
  std::string path, output;
  int recover = -1, jobid = 1;
  std::string cptype = "none";
  double cpinterval = 0;
  std::string cppath;
  double net_delay = 0;
  std::string net_ratio = "inf";
  int verbose = 0;
  // GPU options
  std::string mode = "async", precision = "fp32", lr_strategy = "fixed";
  int epochs = 0, workers = 0, device = 0, exact = 0, dsgd_blocks = 0, autotune = 0;
  std::string init = "reference";
};

const char* kUsage =
    "nomad options:\n"
    "  -h [ --help ]                produce help message\n"
    "  -n [ --nthreads ] arg (=4)   reference threads (row blocks of the initial W)\n"
    "  -l [ --lrate ] arg (=0.001)  learning rate\n"
    "  -d [ --drate ] arg (=0.1)    decay rate\n"
    "  -r [ --reg ] arg (=1)        regularization parameter lambda\n"
    "  -s [ --seed ] arg (=12345)   seed value of random number generator\n"
    "  --cpm arg (=100)             accepted for compatibility (single GPU: no messages)\n"
    "  --tpm arg (=0.5)             accepted for compatibility\n"
    "  -t [ --timeout ] arg (=10.0) timeout seconds until completion (cumulative list)\n"
    "  -u [ --tm_value ] arg (=1)   stop when the online RMSE is at most this (after 8\n"
    "                               passes of every column)\n"
    "  -e [ --tm_error ] arg (=1e-6) stop when the online RMSE changes by at most this\n"
    "                               between two checks\n"
    "  --tm_interval arg (=1)       seconds of training between termination checks\n"
    "  --tm_portion arg (=0.01)     accepted for compatibility (checks see whole passes)\n"
    "  --dim arg (=100)             dimension of latent space\n"
    "  --reuse arg (=1)             number of column reuse (only 1 is supported)\n"
    "  --pause arg (=1)             pause 3 s after each timeout point\n"
    "  --random_send arg (=1)       accepted for compatibility\n"
    "  --r0delay arg (=0)           accepted for compatibility\n"
    "  -i [ --input ] arg           path of data (train.dat, test.dat)\n"
    "  --path arg                   path of data (legacy name of --input)\n"
    "  -o [ --output ] arg          prefix of the factor dump (<output>0)\n"
    "  --recover arg (=-1)          resume from checkpoint arg (-1 means do not recover)\n"
    "  -j [ --jobid ] arg (=1)      job id in checkpoint file names\n"
    "  -c [ --cptype ] arg (=none)  type of checkpoint (none, sync, async, vs); all are\n"
    "                               taken between epochs\n"
    "  -k [ --cpinterval ] arg (=0) seconds of training between checkpoints\n"
    "  -p [ --cppath ] arg          directory of checkpoint files\n"
    "  --net_delay arg (=0)         accepted for compatibility\n"
    "  --net_ratio arg (=inf)       accepted for compatibility\n"
    "  -v [ --verbose ] arg (=0)    verbose level\n"
    "GPU options:\n"
    "  --mode arg (=async)          async | dsgd | dsgdpp | replay\n"
    "  --lr_strategy arg (=fixed)   fixed | bold (bold driver; dsgd and dsgdpp)\n"
    "  --precision arg (=fp32)      fp32 | bf16 (bf16 storage, stochastic rounding)\n"
    "  --epochs arg (=0)            train this many epochs per timeout point\n"
    "  --workers arg (=0)           async worker warps (0 = all resident)\n"
    "  --dsgd_blocks arg (=0)       DSGD blocks per side (0 = auto)\n"
    "  --exact arg (=0)             reference operation order\n"
    "  --autotune arg (=0)          async: first measure configurations, this many timed\n"
    "                               epochs each, and train with the fastest\n"
    "  --init arg (=reference)      reference | hash\n"
    "  --device arg (=0)            CUDA device\n";

bool parse_bool(const std::string& s, bool& out) {
  if (s == "1" || s == "true" || s == "yes" || s == "on") return out = true, true;
  if (s == "0" || s == "false" || s == "no" || s == "off") return out = false, true;
  return false;
}

// boost::program_options-style parsing: --name value, --name=value, -x value, -xvalue;
// --timeout takes every following token up to the next option.
bool parse(int argc, char** argv, Options& o, bool& help) {
  std::vector<std::string> a(argv + 1, argv + argc);
  const std::pair<const char*, const char*> shorts[] = {
      {"h", "help"}, {"n", "nthreads"}, {"l", "lrate"}, {"d", "drate"}, {"r", "reg"},
      {"s", "seed"}, {"t", "timeout"}, {"u", "tm_value"}, {"e", "tm_error"}, {"i", "input"},
      {"o", "output"}, {"j", "jobid"}, {"c", "cptype"}, {"k", "cpinterval"}, {"p", "cppath"},
      {"v", "verbose"}};
  for (size_t i = 0; i < a.size(); ++i) {
    std::string name, val;
    bool has_val = false;
    if (a[i].rfind("--", 0) == 0) {
      name = a[i].substr(2);
      const size_t eq = name.find('=');
      if (eq != std::string::npos) {
        val = name.substr(eq + 1);
        name = name.substr(0, eq);
        has_val = true;
      }
    } else if (a[i].size() >= 2 && a[i][0] == '-') {
      const std::string s = a[i].substr(1, 1);
      bool found = false;
      for (auto& p : shorts)
        if (s == p.first) {
          name = p.second;
          found = true;
        }
      if (!found) {
        std::cerr << "error: unrecognised option '" << a[i] << "'\n";
        return false;
      }
      if (a[i].size() > 2) {
        val = a[i].substr(2);
        has_val = true;
      }
    } else {
      std::cerr << "error: unexpected token '" << a[i] << "'\n";
      return false;
    }
    if (name == "help") {
      help = true;
      continue;
    }
    auto next = [&](std::string& v) {
      if (has_val) return (v = val), true;
      if (i + 1 >= a.size()) return false;
      v = a[++i];
      return true;
    };
    std::string v;
    try {
      if (name == "timeout") {
        o.timeouts.clear();
        if (has_val) o.timeouts.push_back(std::stod(val));
        while (i + 1 < a.size() && !(a[i + 1].size() > 1 && a[i + 1][0] == '-' &&
                                     !std::isdigit(static_cast<unsigned char>(a[i + 1][1])) &&
                                     a[i + 1][1] != '.'))
          o.timeouts.push_back(std::stod(a[++i]));
        if (o.timeouts.empty()) throw std::invalid_argument("timeout needs a value");
        continue;
      }
      if (!next(v)) {
        std::cerr << "error: the required argument for option '--" << name << "' is missing\n";
        return false;
      }
      if (name == "nthreads") o.nthreads = std::stoi(v);
      else if (name == "lrate") o.lrate = std::stod(v);
      else if (name == "drate") o.drate = std::stod(v);
      else if (name == "reg") o.reg = std::stod(v);
      else if (name == "seed") o.seed = std::stoull(v);
      else if (name == "cpm") o.cpm = std::stoi(v);
      else if (name == "tpm") o.tpm = std::stod(v);
      else if (name == "tm_value") o.tm_value = std::stod(v);
      else if (name == "tm_error") o.tm_error = std::stod(v);
      else if (name == "tm_interval") o.tm_interval = std::stod(v);
      else if (name == "tm_portion") o.tm_portion = std::stod(v);
      else if (name == "dim") o.dim = std::stoi(v);
      else if (name == "reuse") o.reuse = std::stoi(v);
      else if (name == "pause") { if (!parse_bool(v, o.pause)) throw std::invalid_argument(v); }
      else if (name == "random_send") { if (!parse_bool(v, o.random_send)) throw std::invalid_argument(v); }
      else if (name == "r0delay") o.r0delay = std::stod(v);
      else if (name == "input" || name == "path") o.path = v;
      else if (name == "output") o.output = v;
      else if (name == "recover") o.recover = std::stoi(v);
      else if (name == "jobid") o.jobid = std::stoi(v);
      else if (name == "cptype") o.cptype = v;
      else if (name == "cpinterval") o.cpinterval = std::stod(v);
      else if (name == "cppath") o.cppath = v;
      else if (name == "net_delay") o.net_delay = std::stod(v);
      else if (name == "net_ratio") o.net_ratio = v;
      else if (name == "verbose") o.verbose = std::stoi(v);
      else if (name == "mode") o.mode = v;
      else if (name == "lr_strategy") o.lr_strategy = v;
      else if (name == "precision") o.precision = v;
      else if (name == "epochs") o.epochs = std::stoi(v);
      else if (name == "workers") o.workers = std::stoi(v);
      else if (name == "device") o.device = std::stoi(v);
      else if (name == "exact") o.exact = std::stoi(v);
      else if (name == "dsgd_blocks") o.dsgd_blocks = std::stoi(v);
      else if (name == "autotune") o.autotune = std::stoi(v);
      else if (name == "init") o.init = v;
      else {
        std::cerr << "error: unrecognised option '--" << name << "'\n";
        return false;
      }
    } catch (const std::exception&) {
      std::cerr << "error: the argument ('" << v << "') for option '--" << name << "' is invalid\n";
      return false;
    }
  }
  // validation as NomadOption::parse_command (nomad_option.cpp:89-111)
  bool ok = true;
  for (auto& ch : o.cptype) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  if (o.path.empty()) { std::cerr << "input path has to be specified.\n"; ok = false; }
  if (o.cptype != "none" && o.cptype != "sync" && o.cptype != "async" && o.cptype != "vs") {
    std::cerr << "checkpoint type is inalid.\n"; ok = false;
  }
  if (o.cptype != "none" && o.cpinterval <= 0) { std::cerr << "checkpoint interval is invalid.\n"; ok = false; }
  if (o.cptype != "none" && o.cppath.empty()) { std::cerr << "checkpoint path is not given.\n"; ok = false; }
  if (o.reuse != 1) { std::cerr << "only --reuse 1 is supported.\n"; ok = false; }
  if (o.mode != "async" && o.mode != "dsgd" && o.mode != "dsgdpp" && o.mode != "replay") {
    std::cerr << "unknown --mode.\n";
    ok = false;
  }
  if (o.lr_strategy != "fixed" && o.lr_strategy != "bold") { std::cerr << "unknown --lr_strategy.\n"; ok = false; }
  if (o.lr_strategy == "bold" && o.mode != "dsgd" && o.mode != "dsgdpp") {
    std::cerr << "--lr_strategy bold needs --mode dsgd or dsgdpp.\n";
    ok = false;
  }
  if (o.precision != "fp32" && o.precision != "bf16") { std::cerr << "unknown --precision.\n"; ok = false; }
  if (o.nthreads <= 0) { std::cerr << "--nthreads must be positive.\n"; ok = false; }
  return ok;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  bool help = false;
  if (!parse(argc, argv, o, help) || help) {
    std::cerr << kUsage << std::endl;
    return 1;
  }
  nomad_io_matrix train{}, test{};
  int rc = nomad_io_read((o.path + "/train.dat").c_str(), &train);
  if (rc) {
    std::cerr << "error in reading training file: " << nomad_gpu_last_error() << "\n";
    return 11;
  }
  rc = nomad_io_read((o.path + "/test.dat").c_str(), &test);
  if (rc) {
    std::cerr << "error in reading test file: " << nomad_gpu_last_error() << "\n";
    nomad_io_free(&train);
    return 11;
  }
  nomad_gpu_params prm;
  nomad_gpu_params_default(&prm);
  prm.dim = o.dim;
  prm.lrate = o.lrate;
  prm.drate = o.drate;
  prm.reg = o.reg;
  prm.seed = o.seed;
  prm.mode = o.mode == "dsgd"     ? NOMAD_MODE_DSGD
             : o.mode == "dsgdpp" ? NOMAD_MODE_DSGDPP
             : o.mode == "replay" ? NOMAD_MODE_REPLAY
                                  : NOMAD_MODE_ASYNC;
  prm.lr_strategy = o.lr_strategy == "bold" ? NOMAD_LR_BOLD_DRIVER : NOMAD_LR_FIXED;
  prm.precision = o.precision == "bf16" ? NOMAD_PREC_BF16_SR : NOMAD_PREC_FP32;
  prm.init = o.init == "hash" ? NOMAD_INIT_HASH : NOMAD_INIT_REFERENCE;
  prm.init_parts = o.nthreads;
  prm.workers = o.workers;
  prm.device = o.device;
  prm.exact = o.exact;
  prm.dsgd_inner_blocks = o.dsgd_blocks;
  nomad_gpu_problem prob{};
  prob.m = train.m;
  prob.n = train.n;
  prob.train = nomad_gpu_matrix{train.nnz, train.row_counts, nullptr, train.cols, train.vals, nullptr};
  prob.test = nomad_gpu_matrix{test.nnz, test.row_counts, nullptr, test.cols, test.vals, nullptr};
  if (o.autotune > 0 && prm.mode == NOMAD_MODE_ASYNC && !prm.exact) {
    nomad_gpu_tune_trial trials[32];
    int32_t nt = 0;
    rc = nomad_gpu_autotune(&prob, &prm, o.autotune, trials, 32, &nt);
    if (rc) {
      std::cerr << "nomad_gpu_autotune: " << nomad_gpu_strerror(rc) << ": " << nomad_gpu_last_error() << "\n";
      return 1;
    }
    double best = -1;
    for (int32_t i = 0; i < nt; ++i) {
      std::cerr << "M: autotune trial: warps per block " << trials[i].warps_per_block << ", priority "
                << trials[i].priority_permille << " permille, long visit " << trials[i].long_visit << ": "
                << trials[i].device_ms << " ms per epoch\n";
      if (trials[i].status == NOMAD_OK && trials[i].warps_per_block == prm.warps_per_block &&
          trials[i].priority_permille == prm.priority_permille && trials[i].long_visit == prm.long_visit)
        best = trials[i].device_ms;
    }
    std::cerr << "M: autotune: warps per block " << prm.warps_per_block << ", priority "
              << prm.priority_permille << " permille, long visit " << prm.long_visit << " (" << best
              << " ms per epoch)\n";
  }
  nomad_gpu_ctx* ctx = nullptr;
  rc = nomad_gpu_init(&ctx, &prob, &prm);
  if (rc) {
    std::cerr << "nomad_gpu_init: " << nomad_gpu_strerror(rc) << ": " << nomad_gpu_last_error() << "\n";
    nomad_io_free(&train);
    nomad_io_free(&test);
    return 1;
  }
  std::string cp_dir = o.cppath.empty() ? "" : o.cppath + "/";
  auto cp_file = [&](int k) { return cp_dir + "cp-t" + std::to_string(o.jobid) + "-e" + std::to_string(k) + ".ckpt"; };
  int cp_epoch = 0;  // number of the next checkpoint
  if (o.recover >= 0) {
    const std::string f = cp_file(o.recover);
    rc = nomad_gpu_load_checkpoint(ctx, f.c_str());
    if (rc) {
      std::cerr << "error in restoring checkpoint " << f << ": " << nomad_gpu_last_error() << "\n";
      nomad_gpu_destroy(ctx);
      nomad_io_free(&train);
      nomad_io_free(&test);
      return 1;
    }
    cp_epoch = o.recover + 1;
  }
  for (double t : o.timeouts) std::cerr << "timeout: " << t << "\n";
  double train_time = 0, test_time = 0;
  long long updates = 0, failures = 0, sends = 0;
  // online termination state (nb_master.cpp:18-20)
  const long long mini_stop_passes = 8LL * train.n;
  long long passes = 0;
  double global_error = std::numeric_limits<double>::infinity(), last_check = 0;
  bool finished = false;
  // checkpoint state
  const bool checkpointing = o.cptype != "none";
  double last_cp = 0, cp_time = 0;
  int cp_count = 0;
  for (size_t it = 0; it < o.timeouts.size() && rc == NOMAD_OK && !finished; ++it) {
    // train until the cumulative training time reaches this timeout point
    const auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&] { return train_time + std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    int done_here = 0;
    while (rc == NOMAD_OK) {
      if (o.epochs > 0 ? done_here >= o.epochs : elapsed() >= o.timeouts[it]) break;
      nomad_gpu_epoch_stats st;
      rc = nomad_gpu_epoch(ctx, 1, &st);
      if (rc) break;
      updates += st.updates;
      failures += st.failures;
      sends += st.hops;
      passes += train.n;  // one pass of every column token
      ++done_here;
      const double now = elapsed();
      if (now - last_check >= o.tm_interval) {
        // NomadBody::master_termcheck: one check (nb_master.cpp:35-44)
        last_check = now;
        const double rmse = std::sqrt(st.online_sse / static_cast<double>(std::max<int64_t>(train.nnz, 1)));
        const double diff = std::fabs(rmse - global_error);
        std::cerr << "M: termination check at " << std::fixed << std::setprecision(2) << now
                  << ": RMSE: " << std::setprecision(12) << rmse << ", difference: " << std::defaultfloat
                  << diff << ", update: " << passes << "\n";
        global_error = rmse;
        if (diff <= o.tm_error || (passes >= mini_stop_passes && rmse <= o.tm_value)) {
          std::cerr << "M: send terimination signal\n";
          finished = true;
          break;
        }
      }
      if (checkpointing && now - last_cp >= o.cpinterval) {
        const auto c0 = std::chrono::steady_clock::now();
        const std::string f = cp_file(cp_epoch);
        rc = nomad_gpu_save_checkpoint(ctx, f.c_str());
        if (rc) {
          std::cerr << "error in writing checkpoint " << f << ": " << nomad_gpu_last_error() << "\n";
          break;
        }
        cp_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count();
        last_cp = elapsed();
        ++cp_epoch;
        ++cp_count;
      }
    }
    const auto t1 = std::chrono::steady_clock::now();
    train_time += std::chrono::duration<double>(t1 - t0).count();
    if (rc) break;
    double s_tr = 0, s_te = 0;
    int64_t c_tr = 0, c_te = 0;
    rc = nomad_gpu_sse(ctx, &s_tr, &c_tr, &s_te, &c_te);
    test_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    if (rc) break;
    // NomadBody::run statistics block (nb_main.cpp:267-299)
    std::ostringstream buf;
    buf << "Statistics:\n"
        << "=====================================================\n";
    buf << "elapsed time: " << (finished ? train_time : o.timeouts[it]) << " total training time: " << train_time
        << " total testing time: " << test_time;
    buf << " current training RMSE: " << std::fixed << std::setprecision(10) << std::sqrt(s_tr / c_tr) << "\n";
    buf << "current test RMSE: " << std::fixed << std::setprecision(10) << std::sqrt(s_te / c_te) << "\n";
    buf << std::fixed << std::setprecision(4) << "detail: "
        << "train: s=" << s_tr << ", c=" << c_tr << "; test: s=" << s_te << ", c=" << c_te
        << "; u=" << updates << ", f=" << failures << ", s=" << sends << "\n";
    if (checkpointing) {
      // one writer: the master's and the workers' times are the same figure; no column
      // message is in flight between epochs, so none is archived
      const double each = cp_count ? cp_time / cp_count : 0.0;
      buf << std::defaultfloat << "Number of checkpoints: " << cp_count << " Total time by master: " << cp_time
          << " by worker: " << cp_time << " each one: " << each << "\n";
      buf << "Total checkpoint writing time: " << cp_time << " each one: " << each
          << " average on worker: " << each << "\n";
      buf << "Number of archived message in each checkpoint:";
      for (int i = 0; i < cp_count; ++i) buf << " 0";
      buf << "\n";
    }
    buf << "=====================================================";
    std::cout << buf.str() << std::endl;
    if (o.pause) std::this_thread::sleep_for(std::chrono::duration<double>(3.0));
  }
  if (rc) {
    std::cerr << "training failed: " << nomad_gpu_strerror(rc) << ": " << nomad_gpu_last_error() << "\n";
  } else if (!o.output.empty()) {
    std::vector<float> W(static_cast<size_t>(train.m) * o.dim), H(static_cast<size_t>(train.n) * o.dim);
    rc = nomad_gpu_get_factors(ctx, W.data(), H.data());
    if (!rc) rc = nomad_io_write_factors((o.output + "0").c_str(), train.m, train.n, o.dim, W.data(), H.data());
    if (rc) std::cerr << "output failed: " << nomad_gpu_last_error() << "\n";
  }
  nomad_gpu_destroy(ctx);
  nomad_io_free(&train);
  nomad_io_free(&test);
  return rc ? 1 : 0;
}
