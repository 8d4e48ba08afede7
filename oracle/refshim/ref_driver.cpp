// ref_driver.cpp -- runs the reference's own updater thread (Code/nomad/nb_main.cpp,
// NomadBody::updater_func, compiled unmodified from the reference tree) on one rank with
// one worker thread, so that the oracle can be compared with the reference itself.
//
// TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ by oracle/Makefile.ref against the
// stand-in headers under oracle/refshim/include (TBB, glog, boost::format, MPI) and
// loaded only by tests/.
//
// What runs is the reference's code: read_data / load_train / load_test
// (nb_data.cpp:19-226) build the per-worker CSC from a train.dat/test.dat pair; the
// updater thread initialises its rows (nb_main.cpp:441-455), trains on the column
// tokens (nb_main.cpp:480-572), then evaluates the training and test squared errors
// (nb_main.cpp:577-676) and, with an output prefix, writes its rows
// (nb_main.cpp:683-705).  This driver does what NomadBody::run and the MPI/send threads
// would do around it on one rank: it creates the column tokens the way
// nb_main.cpp:70-98 does (Pool, ColumnData::set_perm from pool.cpp), flips the
// training/testing flags, and stops training after exactly `epochs` passes of every
// column: the stand-in queue refuses pops after epochs*n visits, and the driver raises
// flag_train_stop once the updater has come back for one more (so the last visit's
// column is back in the queue).  With one thread and one rank the token order is the
// FIFO round robin over columns 0..n-1, so the result is deterministic.
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <functional>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "tbb/tbb.h"

// The driver sets the updater's private state directly (one translation unit only;
// the class layout does not depend on access specifiers).
#define private public
#define protected public
#include "nomad_body.h"
#undef private
#undef protected

namespace {
[[noreturn]] void not_in_one_rank_run(const char* what) {
  std::fprintf(stderr, "reference driver: %s is not used by a one-rank, one-thread run\n", what);
  std::abort();
}
void wait_until(const std::function<bool()>& cond) {
  while (!cond()) std::this_thread::sleep_for(std::chrono::microseconds(200));
}
}  // namespace

// Members that NomadBody::run and updater_func name but that live in translation units
// this build does not compile (MPI set-up, the send/receive and master threads,
// checkpointing).  The one-rank run below never reaches them.
bool NomadBody::initial(NomadOption*) { not_in_one_rank_run("initial"); }
void NomadBody::master_checkpoint() { not_in_one_rank_run("master_checkpoint"); }
void NomadBody::master_termcheck() { not_in_one_rank_run("master_termcheck"); }
void NomadBody::train_send_func(const double) { not_in_one_rank_run("train_send_func"); }
void NomadBody::train_recv_func() { not_in_one_rank_run("train_recv_func"); }
void NomadBody::test_send_func() { not_in_one_rank_run("test_send_func"); }
void NomadBody::test_recv_func() { not_in_one_rank_run("test_recv_func"); }
void NomadBody::restore(int, int, double*, int&, int&) { not_in_one_rank_run("restore"); }
void NomadBody::archive_msg(int, ColumnData*) { not_in_one_rank_run("archive_msg"); }
void NomadBody::cp_update_func_action(int, int, double*, int) { not_in_one_rank_run("cp_update_func_action"); }
void NomadBody::cp_sht_start(int, int, int, double*, int) { not_in_one_rank_run("cp_sht_start"); }
void NomadBody::cp_sht_clear(int, int, int, double*, int) { not_in_one_rank_run("cp_sht_clear"); }
void NomadBody::cp_sht_resume(int, int, int) { not_in_one_rank_run("cp_sht_resume"); }

extern "C" {

// Trains the reference updater for `epochs` passes from the reference init with
// `seed`, then evaluates.  Outputs: H[n*dim] (every column's values), col_err[n] (each
// token's accumulated online error, p_col->error), the training and test squared-error
// sums and counts of the final evaluation, the updater's update count.  With a
// non-empty rows_prefix the updater writes its rows to <rows_prefix>0.
// Returns 0, or -1 when a data file cannot be read.
int ref_replay_f64(const char* data_dir, int32_t dim, double lrate, double drate, double reg, uint64_t seed,
                   int32_t epochs, const char* rows_prefix, double* H, double* col_err, double* train_sse,
                   int64_t* train_count, double* test_sse, int64_t* test_count, int64_t* updates) {
  NomadOption opt{};
  opt.num_threads_ = 1;
  opt.learn_rate_ = lrate;
  opt.decay_rate_ = drate;
  opt.par_lambda_ = reg;
  opt.seed_ = seed;
  opt.latent_dimension_ = dim;
  opt.timeouts_ = {1.0};
  opt.num_reuse_ = 1;
  opt.path_ = data_dir;
  opt.output_path_ = rows_prefix ? rows_prefix : "";
  opt.recover_epoch = -1;
  opt.cp_type_ = "none";

  NomadBody* nb = new NomadBody();
  nb->option = &opt;
  nb->mpi_size = 1;
  nb->mpi_rank = 0;
  nb->num_parts = 1;
  nb->dstrain.resize(1);
  nb->dstest.resize(1);
  if (!nb->load_train(opt.path_, 0, 1, nb->dstrain[0]) || !nb->load_test(opt.path_, 0, 1, nb->dstest[0])) {
    delete nb;
    return -1;
  }
  const int n = nb->dstrain[0].num_cols;
  nb->global_num_cols = n;
  nb->job_queues = new colque[1];
  nb->column_pool = new Pool(dim, 1);
  nb->count_setup_threads = 0;
  nb->flag_train_ready = false;
  nb->flag_train_stop = false;
  nb->flag_test_ready = false;
  nb->flag_test_stop = false;
  nb->finished = false;
  nb->checkpointing = false;
  nb->allow_processing = true;
  nb->allow_sending = true;
  nb->allow_processing_thread = new std::atomic<bool>[1];
  nb->allow_processing_thread[0] = true;
  nb->cp_action_ready = new std::atomic<bool>[1];
  nb->cp_action_ready[0] = false;
  nb->cp_need_archive_msg_from.assign(1, nullptr);
  nb->cp_need_archive_msg_from[0] = new std::atomic<bool>[1];
  nb->cp_need_archive_msg_from[0][0] = false;
  nb->num_updates = new std::atomic<long long>[1];
  nb->num_failures = new std::atomic<long long>[1];
  nb->num_updates[0] = 0;
  nb->num_failures[0] = 0;
  nb->train_count_errors = new int[1]();
  nb->train_sum_errors = new double[1]();
  nb->test_count_errors = new int[1]();
  nb->test_sum_errors = new double[1]();
  nb->wait_number = 0;

  std::thread updater(&NomadBody::updater_func, nb, 0);
  wait_until([&] { return nb->count_setup_threads.load() >= 1; });  // rows initialised

  // the column tokens, as nb_main.cpp:70-98 creates them on rank 0 of one
  std::mt19937_64 rng(seed + 139);
  std::uniform_real_distribution<double> init_dist(0, 1.0 / std::sqrt(static_cast<double>(dim)));
  std::mt19937_64 rng_temp(seed + 137);
  for (int i = 0; i < n; ++i) {
    ColumnData* p_col = nb->column_pool->pop();
    p_col->col_index_ = i;
    p_col->flag_ = 0;
    p_col->source_ = 0;
    p_col->set_perm(1, rng_temp);
    for (int j = 0; j < dim; ++j) p_col->values_[j] = init_dist(rng);
    nb->job_queues[p_col->perm_[p_col->pos_]].push(p_col);
  }

  nb->job_queues[0].shim_set_pop_budget(static_cast<long long>(epochs) * n);
  nb->flag_train_ready = true;
  wait_until([&] { return nb->job_queues[0].shim_refused(); });  // every pass done, last column queued
  nb->flag_train_stop = true;
  nb->job_queues[0].shim_set_pop_budget(-1);
  nb->flag_test_ready = true;
  wait_until([&] { return nb->count_setup_threads.load() >= 2; });  // evaluation done
  updater.join();

  std::vector<ColumnData*> cols;
  ColumnData* p_col = nullptr;
  while (nb->send_queue.try_pop(p_col)) cols.push_back(p_col);
  for (ColumnData* c : cols) {
    if (c->col_index_ >= 0 && c->col_index_ < n) {
      if (H)
        for (int j = 0; j < dim; ++j) H[static_cast<int64_t>(c->col_index_) * dim + j] = c->values_[j];
      if (col_err) col_err[c->col_index_] = c->error;
    }
    nb->column_pool->push(c);
  }
  if (train_sse) *train_sse = nb->train_sum_errors[0];
  if (train_count) *train_count = nb->train_count_errors[0];
  if (test_sse) *test_sse = nb->test_sum_errors[0];
  if (test_count) *test_count = nb->test_count_errors[0];
  if (updates) *updates = nb->num_updates[0];
  const int ncols = static_cast<int>(cols.size());

  delete nb->column_pool;
  delete[] nb->job_queues;
  delete[] nb->allow_processing_thread;
  delete[] nb->cp_action_ready;
  delete[] nb->cp_need_archive_msg_from[0];
  delete[] nb->num_updates;
  delete[] nb->num_failures;
  delete[] nb->train_count_errors;
  delete[] nb->train_sum_errors;
  delete[] nb->test_count_errors;
  delete[] nb->test_sum_errors;
  delete nb;
  return ncols == n ? 0 : -2;
}

}  // extern "C"
