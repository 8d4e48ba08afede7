/*
 * nomad_oracle.h -- CPU restatement of NOMAD's SGD matrix-completion hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU library
 * (nomad_gb300); only tests/, __graft_entry__.smoke() and the cpu_baseline leg of
 * bench.py may load it.  Nothing in the product links or calls it.
 *
 * It restates, in plain C++ (built with -ffp-contract=off so every float/double
 * operation rounds exactly as the reference's scalar code does on x86_64/aarch64):
 *
 *   - factor init            Code/nomad/nb_main.cpp:450-455 (rows), :70-98 (columns)
 *   - per-rating SGD update   Code/nomad/nb_main.cpp:513-542 (double, fork)
 *                             Code/nomad/nomad_body.hpp:324-357 (scalar=float, legacy)
 *   - token routing           Code/nomad/nb_main.cpp:551-565, pool.cpp:32-38 (set_perm)
 *   - evaluation (SSE)        Code/nomad/nb_main.cpp:601-667, nomad_body.hpp:420-470
 *   - file reader             Code/nomad/nb_data.cpp:19-176 (train.dat / test.dat)
 *   - DSGD                    Code/competitor/sgd-mpi-omp.cpp:186-210 (sgd), :220-424
 *                             (dsgd_mpi, single process), :35-101 (block layout)
 *   - DSGD++, bold driver     Code/competitor/dsgdpp.cpp:300-540, :42-69 (blocks);
 *                             sgd-mpi-omp.cpp:122-160 (calobj_mpi), :384-394
 *
 * Parity status: pinned to the reference itself.  The reference ships no tests or
 * golden vectors, but its updater (Code/nomad/nb_main.cpp, nb_data.cpp, pool.cpp)
 * compiles unmodified against single-process stand-ins for TBB, glog, boost::format
 * and MPI (oracle/Makefile.ref, oracle/refshim/), and run on one rank with one thread
 * it gives the same columns and evaluation sums as oracle_replay_f64 / oracle_sse_f64
 * bit for bit (tests/test_reference_pin.py, golden outputs in
 * tests/golden/reference_replay.npz).  The float forms follow the legacy float body,
 * which cannot be built (it includes a header missing from the reference tree); they
 * are pinned by the pure-Python restatements of tests/golden/make_golden.py.
 *
 * Data layout conventions used by every entry point:
 *   CSC-by-column: col_ptr[n+1] (int64), row_idx[nnz] (int32, ascending inside a
 *   column, as nb_data.cpp:131-169 produces from a row-major file), vals[nnz] (double,
 *   cast to the scalar type on entry exactly as realdata_body.hpp:172 does).
 *   Factors: row-major, W[m*dim], H[n*dim].
 */
#ifndef NOMAD_ORACLE_H_
#define NOMAD_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference init: W rows from mt19937_64(seed + rank*131 + thread + 1) over each
 * thread's row block (ceil(m/nthreads) rows per block), H from
 * mt19937_64(seed + rank*131 + 139) over all columns in index order, both
 * uniform_real_distribution<double>(0, 1/sqrt(dim)).  Single rank (rank 0). */
void oracle_init_factors(int32_t m, int32_t n, int32_t dim, uint64_t seed,
                         int32_t nthreads, double* W, double* H);

/* Row-major file layout (row counts, column index per entry, value per entry) to
 * CSC-by-column with rows ascending (nb_data.cpp:131-169 with one part). */
int oracle_row_major_to_csc(int32_t m, int32_t n, int64_t nnz,
                            const int32_t* row_counts, const int32_t* cols,
                            const double* vals, int64_t* col_ptr,
                            int32_t* row_idx, double* csc_vals);

/* Step size of one column visit: lrate*1.5/(1+drate*(cnt+1)^1.5) computed in double
 * from scalar-typed lrate/drate, then cast to the scalar (nb_main.cpp:514-515). */
float  oracle_step_f32(double lrate, double drate, int32_t cnt);
double oracle_step_f64(double lrate, double drate, int32_t cnt);

/* Deterministic replay: one worker, one rank -- tokens circulate round-robin over
 * columns 0..n-1 in FIFO order, so one sweep is one epoch and every visit of epoch e
 * uses cnt = e.  Runs epochs [first_epoch, first_epoch + n_epochs).  If epoch_err is
 * non-null it receives the online squared-error sum per epoch (p_col->error). */
int oracle_replay_f32(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                      const int32_t* row_idx, const double* vals, float* W,
                      float* H, int32_t first_epoch, int32_t n_epochs,
                      double lrate, double drate, double reg, double* epoch_err);
int oracle_replay_f64(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                      const int32_t* row_idx, const double* vals, double* W,
                      double* H, int32_t first_epoch, int32_t n_epochs,
                      double lrate, double drate, double reg, double* epoch_err);

/* Evaluation: squared-error sum and count over a CSC set (nb_main.cpp:617-653).
 * f32 follows the legacy float body: error in float, squared in float, summed in
 * double.  f64 follows the fork: everything in double. */
int oracle_sse_f32(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                   const int32_t* row_idx, const double* vals, const float* W,
                   const float* H, double* sse, int64_t* count);
int oracle_sse_f64(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                   const int32_t* row_idx, const double* vals, const double* W,
                   const double* H, double* sse, int64_t* count);

/* Asynchronous NOMAD on host threads: nthreads workers own ceil(m/nthreads)-row
 * blocks, column tokens circulate through per-worker queues following a per-token
 * permutation drawn with mt19937_64(seed + 137) (nb_main.cpp:79-96).
 * n_epochs > 0: each token makes exactly n_epochs passes over its permutation, then
 *               retires; the call returns when every token has retired.
 * n_epochs = 0: run for timeout_sec of wall clock (the reference's --timeout).
 * Counters: updates (u=), failures (f= empty pops), train_seconds. */
int oracle_async_f32(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                     const int32_t* row_idx, const double* vals, float* W,
                     float* H, int32_t nthreads, int32_t n_epochs,
                     double timeout_sec, double lrate, double drate, double reg,
                     uint64_t seed, int64_t* updates, int64_t* failures,
                     double* train_seconds);
int oracle_async_f64(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                     const int32_t* row_idx, const double* vals, double* W,
                     double* H, int32_t nthreads, int32_t n_epochs,
                     double timeout_sec, double lrate, double drate, double reg,
                     uint64_t seed, int64_t* updates, int64_t* failures,
                     double* train_seconds);

/* Asynchronous NOMAD with P workers as a deterministic discrete-event simulation on one
 * host thread (the reference with --nthreads P, nb_main.cpp:415-572, whose schedule
 * depends on thread timing).  Rows in P contiguous parts (partition 0: ceil(m/P) rows,
 * nb_data.cpp:83-89; partition 1: about nnz/P ratings each); each column's route is its
 * permutation of the workers drawn with mt19937_64(seed + 137) in column order
 * (nb_main.cpp:79-96, pool.cpp:32-38) without the workers that hold none of its
 * ratings; step of pass e = step(cnt = e).  A visit of len ratings takes
 * visit_cost + rating_cost*len time units, a hop hop_cost; queues are FIFO.  Runs
 * passes [first_epoch, first_epoch + n_epochs), every token starting each pass at its
 * route's first worker; epoch_err[i] = the pass's online squared-error sum. */
int oracle_async_sim_f32(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                         const int32_t* row_idx, const double* vals, float* W, float* H,
                         int32_t P, int32_t partition, int32_t first_epoch, int32_t n_epochs,
                         double lrate, double drate, double reg, uint64_t seed,
                         double visit_cost, double rating_cost, double hop_cost,
                         double* epoch_err);
int oracle_async_sim_f64(int32_t m, int32_t n, int32_t dim, const int64_t* col_ptr,
                         const int32_t* row_idx, const double* vals, double* W, double* H,
                         int32_t P, int32_t partition, int32_t first_epoch, int32_t n_epochs,
                         double lrate, double drate, double reg, uint64_t seed,
                         double visit_cost, double rating_cost, double hop_cost,
                         double* epoch_err);

/* DSGD, single process (numprocs = 1 => B = 1, innerB = 2*nthreads), FIXED learning
 * rate schedule lr = 1.5*lrate/(1+decay*iter^1.5).  Input is the row-major file
 * layout (row_counts, cols, vals) because block order follows file order.  Blocks in
 * one inner stratum are disjoint, so running them one after another gives the same
 * bits as the reference's OpenMP loop.  stratum_strategy: 0 semi-WOR, 2 WOR (inner
 * permutations reshuffled with srand(34586+iter)/random_shuffle). */
int oracle_dsgd_f32(int32_t m, int32_t n, int32_t dim, int64_t nnz,
                    const int32_t* row_counts, const int32_t* cols,
                    const double* vals, float* W, float* H, int32_t nthreads,
                    int32_t first_iter, int32_t n_iters, double lrate,
                    double decay, double reg, int32_t stratum_strategy);
int oracle_dsgd_f64(int32_t m, int32_t n, int32_t dim, int64_t nnz,
                    const int32_t* row_counts, const int32_t* cols,
                    const double* vals, double* W, double* H, int32_t nthreads,
                    int32_t first_iter, int32_t n_iters, double lrate,
                    double decay, double reg, int32_t stratum_strategy);

/* DSGD (variant 0) or DSGD++ (variant 1, Code/competitor/dsgdpp.cpp:300-540: innerB x
 * 2*innerB blocks, phase 0 over the left column half then phase 1 over the right
 * half) with the FIXED (lr_strategy 0) or BOLDDRIVER (1) learning rate.  Bold driver:
 * lr_state = {learning rate of the next pass, objective after the previous pass or
 * < 0 when not yet computed}, updated in place: after each pass the objective is
 * recomputed and the rate multiplied by decay if it rose, else by 1.05. */
int oracle_dsgd2_f32(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                     const int32_t* cols, const double* vals, float* W, float* H, int32_t nthreads,
                     int32_t first_iter, int32_t n_iters, double lrate, double decay, double reg,
                     int32_t stratum_strategy, int32_t variant, int32_t lr_strategy, double* lr_state);
int oracle_dsgd2_f64(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                     const int32_t* cols, const double* vals, double* W, double* H, int32_t nthreads,
                     int32_t first_iter, int32_t n_iters, double lrate, double decay, double reg,
                     int32_t stratum_strategy, int32_t variant, int32_t lr_strategy, double* lr_state);

/* The DSGD objective calobj_mpi (sgd-mpi-omp.cpp:122-160) of factors W, H: sum of
 * squared errors in double plus reg * (sum_r nnz_row(r) |W_r|^2 + sum_c nnz_col(c)
 * |H_c|^2).  Row-major rating input as oracle_dsgd_f32. */
int oracle_objective_f32(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                         const int32_t* cols, const double* vals, const float* W, const float* H,
                         double reg, double* out);
int oracle_objective_f64(int32_t m, int32_t n, int32_t dim, int64_t nnz, const int32_t* row_counts,
                         const int32_t* cols, const double* vals, const double* W, const double* H,
                         double reg, double* out);

/* DSGD++ schedule for one iteration: bj[(phase*innerB + i)*innerB + bi] is the column
 * block (of 2*innerB) that row block bi processes in stratum i of the phase. */
int oracle_dsgdpp_schedule(int32_t innerB, int32_t iter, int32_t stratum_strategy, int32_t* bj);

/* DSGD inner-stratum schedule for one iteration: bj[i*innerB + bi] is the column
 * block that row block bi processes in inner stratum i (sgd-mpi-omp.cpp:293-365). */
int oracle_dsgd_schedule(int32_t innerB, int32_t iter, int32_t stratum_strategy,
                         int32_t* bj);

/* File reader restating nb_data.cpp:19-176 for one part: fills m, n, nnz.  With
 * null output arrays only the header is read. */
int oracle_read_header(const char* path, int32_t* file_id, int32_t* m, int32_t* n,
                       int64_t* nnz);
int oracle_read_matrix(const char* path, int32_t* row_counts, int32_t* cols,
                       double* vals);

/* Known answer for the RNG the init relies on: the 10000th output of a
 * default-seeded std::mt19937_64 (C++ standard [rand.predef]: 9981545732273789042). */
uint64_t oracle_mt19937_64_10000th(void);

#ifdef __cplusplus
}
#endif

#endif
