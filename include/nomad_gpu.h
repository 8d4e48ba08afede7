/*
 * nomad_gpu.h -- C-ABI of the GB300 NOMAD matrix-completion library.
 *
 * Single-GPU, sm_103a.  The library owns all device memory of a context; every
 * argument is a plain pointer or scalar.  No C++ types and no exceptions cross
 * this boundary; every call returns a status (0 = OK, < 0 = error).
 *
 * Reference entry points each call replaces (yxtj/nomad, paths inside the project):
 *   nomad_gpu_init         NomadBody::initial (Code/nomad/nb_init.cpp:189-235), the
 *                          per-worker CSC build of read_data (nb_data.cpp:131-169),
 *                          row init (nb_main.cpp:443-456) and column-token init
 *                          (nb_main.cpp:67-98)
 *   nomad_gpu_epoch        one training interval of NomadBody::run
 *                          (nb_main.cpp:109-135) running NomadBody::updater_func's
 *                          training loop (nb_main.cpp:480-572) on every worker
 *   nomad_gpu_sse /        the evaluation pass (nb_main.cpp:577-676) and the
 *   nomad_gpu_rmse         statistics block (nb_main.cpp:215-285)
 *   nomad_gpu_get_factors  the --output dump of rows and columns
 *                          (nb_main.cpp:349-366, 683-705)
 *   nomad_gpu_destroy      teardown (nb_main.cpp:368-408)
 *   nomad_gpu_save_checkpoint / nomad_gpu_load_checkpoint
 *                          a checkpoint taken at an epoch boundary
 *                          (NomadBody::archive_local, nb_checkpoint.cpp:47-59) and
 *                          the --recover path (NomadBody::restore,
 *                          nb_checkpoint.cpp:135-143; nb_main.cpp:446-449)
 */
#ifndef NOMAD_GPU_H_
#define NOMAD_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NOMAD_GPU_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------------- */
enum nomad_gpu_status {
  NOMAD_OK = 0,
  NOMAD_ERR_INVALID_ARG = -1, /* bad sizes, indices out of range, null pointers   */
  NOMAD_ERR_CUDA = -2,        /* a CUDA runtime call failed                       */
  NOMAD_ERR_OOM = -3,         /* device or host allocation failed                 */
  NOMAD_ERR_TIMEOUT = -4,     /* a bounded device wait ran out (no global progress) */
  NOMAD_ERR_BOUNDS = -5,      /* a device-side bounds check failed                */
  NOMAD_ERR_IO = -6,          /* file could not be opened / read / written        */
  NOMAD_ERR_FORMAT = -7,      /* file is not a train.dat/test.dat binary matrix   */
  NOMAD_ERR_NO_DEVICE = -8,   /* no CUDA device, or not an sm_103 device          */
  NOMAD_ERR_UNSUPPORTED = -9  /* combination of options not supported             */
};

/* ---- options ------------------------------------------------------------------ */
enum nomad_gpu_mode {
  NOMAD_MODE_ASYNC = 0,  /* NOMAD: worker warps pass column tokens through queues */
  NOMAD_MODE_DSGD = 1,   /* DSGD stratum sweep (Code/competitor/sgd-mpi-omp.cpp)  */
  NOMAD_MODE_REPLAY = 2, /* one worker, columns round-robin: deterministic order  */
  NOMAD_MODE_DSGDPP = 3  /* DSGD++ (Code/competitor/dsgdpp.cpp): innerB row blocks x
                            2*innerB column blocks, two column halves per pass     */
};
enum nomad_gpu_lr_strategy {
  NOMAD_LR_FIXED = 0,      /* step = lrate*1.5/(1 + drate*pass^1.5)                 */
  NOMAD_LR_BOLD_DRIVER = 1 /* DSGD / DSGD++: after each pass the objective is
                              recomputed; lr *= drate if it rose, else lr *= 1.05
                              (sgd-mpi-omp.cpp:384-394, dsgdpp.cpp:512-521)         */
};
enum nomad_gpu_precision {
  NOMAD_PREC_FP32 = 0,   /* W, H stored in fp32                                   */
  NOMAD_PREC_BF16_SR = 1 /* W, H stored in bf16, fp32 arithmetic, stochastic-
                            rounding write-back                                   */
};
enum nomad_gpu_init_kind {
  NOMAD_INIT_REFERENCE = 0, /* the reference's mt19937_64 streams (bit-identical) */
  NOMAD_INIT_HASH = 1       /* U(0, 1/sqrt(dim)) from a counter hash, on device   */
};

typedef struct nomad_gpu_params {
  int32_t struct_size; /* = sizeof(nomad_gpu_params); set by nomad_gpu_params_default */
  int32_t dim;         /* --dim (latent dimension k)                   default 100   */
  double lrate;        /* --lrate                                      default 0.001 */
  double drate;        /* --drate                                      default 0.1   */
  double reg;          /* --reg (lambda)                               default 1.0   */
  uint64_t seed;       /* --seed                                       default 12345 */
  int32_t mode;        /* nomad_gpu_mode                               default ASYNC */
  int32_t precision;   /* nomad_gpu_precision                          default FP32  */
  int32_t init;        /* nomad_gpu_init_kind (ignored when W0/H0 given) REFERENCE   */
  int32_t init_parts;  /* row blocks of the reference init = ranks x --nthreads (1)  */
  int32_t device;      /* CUDA device ordinal                          default 0     */
  int32_t workers;     /* ASYNC: worker warps, 0 = every resident warp slot          */
  int32_t warps_per_block; /* 0 = auto                                               */
  int32_t blocks_per_sm;   /* 0 = as many as fit; batched form: 1 or > 1 (four) blocks
                              of its kernel per SM, 0 = four when no problem holds more
                              than 2% of the batch's ratings, else one               */
  int32_t balance;     /* row blocks: 0 = equal rows (reference), 1 = equal ratings  */
  int32_t dsgd_inner_blocks; /* DSGD innerB (blocks per side), 0 = auto              */
  int32_t dsgd_strategy;     /* DSGD stratum strategy: 0 semi-WOR, 2 WOR             */
  int32_t exact;       /* 1: reference operation order (sequential dot, no FMA);
                          REPLAY always uses it                                      */
  int32_t spin_budget_ms; /* device waits give up after this long without global
                             progress and the call returns NOMAD_ERR_TIMEOUT (2000)  */
  int32_t debug_flags; /* test hooks; bit 0 = enqueue no tokens (forces a timeout);   *
                        * bit 1 = one worker per thread block never joins a block     *
                        * visit (the others' join wait runs out: a timeout);          *
                        * bit 2 = ASYNC: build the visit lists on the host as well as *
                        * on the device and refuse with NOMAD_ERR_BOUNDS if they      *
                        * differ; batched form: the same for the CSCs and the large   *
                        * problems' visit bounds                                      */
  int32_t long_visit;  /* ASYNC: visits with at least this many ratings run the blocked
                          (7-rating) path with TMA-staged rows; 0 = default 14 for
                          FP32 rows, 17 for BF16_SR rows                             */
  int32_t priority_permille; /* ASYNC: columns with at least this many permille of the
                          largest column's ratings use the workers' priority queues;
                          0 = default 50, negative = no priority queue                */
  int32_t lr_strategy; /* nomad_gpu_lr_strategy (BOLD_DRIVER: DSGD and DSGDPP)  FIXED */
  int32_t batch_share; /* batched form (exact = 0): a problem with at least this many
                          times one warp's fair share of the batch's ratings (and at
                          least 8,192) runs on a whole thread block of NOMAD workers;
                          0 = default 1, negative = every problem on one warp        */
  int32_t reserved[4];
} nomad_gpu_params;

/* One rating set in either the reference's row-major file layout (row_counts !=
 * NULL: entries listed row by row, as train.dat stores them, nb_data.cpp:40-64) or
 * COO (rows != NULL).  Exactly one of vals_f64 / vals_f32 is non-NULL. */
typedef struct nomad_gpu_matrix {
  int64_t nnz;
  const int32_t* row_counts; /* [m]   or NULL                                      */
  const int32_t* rows;       /* [nnz] or NULL                                      */
  const int32_t* cols;       /* [nnz]                                              */
  const double* vals_f64;    /* [nnz] or NULL                                      */
  const float* vals_f32;     /* [nnz] or NULL                                      */
} nomad_gpu_matrix;

typedef struct nomad_gpu_problem {
  int32_t m;              /* rows (users)                                          */
  int32_t n;              /* columns (items): one token each                      */
  nomad_gpu_matrix train;
  nomad_gpu_matrix test;  /* nnz may be 0                                          */
  const float* W0;        /* optional initial rows    [m * dim], row-major         */
  const float* H0;        /* optional initial columns [n * dim], row-major         */
} nomad_gpu_problem;

typedef struct nomad_gpu_epoch_stats {
  int64_t updates;     /* ratings visited (the reference's u=)                     */
  int64_t hops;        /* token hand-offs between workers                          */
  int64_t failures;    /* empty queue polls (the reference's f=)                   */
  int32_t epochs_done; /* cumulative epochs after this call                        */
  int32_t reserved0;
  double device_ms;    /* CUDA-event time of the call's device work on its stream  */
  double host_seconds; /* wall time of the call                                    */
  double online_sse;   /* sum of e^2 seen while training (ColumnData::error)       */
  double objective;    /* BOLD_DRIVER: objective after the call (calobj_mpi), else 0 */
  double lrate;        /* BOLD_DRIVER: learning rate of the next pass, else 0      */
} nomad_gpu_epoch_stats;

typedef struct nomad_gpu_info {
  int32_t m, n, dim, dim_padded;
  int64_t nnz_train, nnz_test;
  int32_t workers;          /* ASYNC worker warps (REPLAY: 1)                      */
  int32_t active_tokens;    /* columns with at least one training rating          */
  int64_t segments;         /* visits per epoch: non-empty (worker, column) pairs, and
                               (thread block, column) pairs of priority columns    */
  int64_t max_column;       /* largest column (ratings)                            */
  int32_t grid_blocks, block_threads, num_sms, inner_blocks;
  int64_t device_bytes;     /* device memory held by the context                   */
  int32_t mode, precision;
  int64_t h2d_bytes;        /* host-to-device bytes copied since init (cumulative) */
  int64_t d2h_bytes;        /* device-to-host bytes copied since init (cumulative) */
  int32_t priority_tokens;  /* columns whose visits run on all warps of a block    */
  int32_t reserved0;
} nomad_gpu_info;

typedef struct nomad_gpu_ctx nomad_gpu_ctx; /* opaque */

/* ---- API ------------------------------------------------------------------------ */

/* Fill *p with the reference's defaults (nomad_option.cpp:16-77). */
int nomad_gpu_params_default(nomad_gpu_params* p);

/* Copy the problem to the device, build the layout and initialise W and H.  Host
 * buffers stay owned by the caller and are not referenced after the call.  Row-major
 * rating sets (row_counts given, up to INT_MAX ratings) are sorted into column order on
 * the device, and in ASYNC mode the visit lists are built there too; their arrays are
 * copied in through two 32 MB pinned host buffers that the library allocates on first use
 * and keeps for the life of the process.  Row counts are checked before any device work;
 * column indices out of range and repeated (row, column) cells are refused
 * (NOMAD_ERR_INVALID_ARG) before training starts. */
int nomad_gpu_init(nomad_gpu_ctx** out, const nomad_gpu_problem* prob,
                   const nomad_gpu_params* params);

/* Run n_epochs epochs.  One epoch = every training rating is visited once: in ASYNC
 * every column token makes one full pass over the workers that hold its ratings; the
 * step size of a visit uses the token's pass count (nb_main.cpp:514-515).  Blocks
 * until the device work is done; st may be NULL. */
int nomad_gpu_epoch(nomad_gpu_ctx* ctx, int32_t n_epochs, nomad_gpu_epoch_stats* st);

/* Squared-error sums and counts over the training and test sets (nb_main.cpp:617-653);
 * FP64 accumulation on the device. Any pointer may be NULL; a set whose sum and count
 * pointers are both NULL is not evaluated (the training set is ~70x the test set). */
int nomad_gpu_sse(nomad_gpu_ctx* ctx, double* train_sse, int64_t* train_count,
                  double* test_sse, int64_t* test_count);

/* RMSE = sqrt(sse / count) for both sets (nb_main.cpp:272-275); a NULL output skips
 * that set's evaluation. */
int nomad_gpu_rmse(nomad_gpu_ctx* ctx, double* train_rmse, double* test_rmse);

/* Copy the factors to host float arrays W[m*dim], H[n*dim] (either may be NULL). */
int nomad_gpu_get_factors(nomad_gpu_ctx* ctx, float* W, float* H);

/* Overwrite the factors from host float arrays (either may be NULL). */
int nomad_gpu_set_factors(nomad_gpu_ctx* ctx, const float* W, const float* H);

/* Set the cumulative pass count, the quantity the step size of the next epoch is
 * computed from (nb_main.cpp:514-515): the next nomad_gpu_epoch runs pass
 * epochs_done + 1.  Used when training resumes from saved factors.  Under the bold
 * driver the learning rate and the last objective are the rest of the state; a
 * checkpoint carries them. */
int nomad_gpu_set_epochs_done(nomad_gpu_ctx* ctx, int32_t epochs_done);

/* Write the context's factors, pass count and bold-driver state to a checkpoint file
 * (the format of nomad_io_write_checkpoint).  Between nomad_gpu_epoch calls every
 * column token has finished its pass, so this is the whole training state.  BF16
 * factors are widened to fp32 exactly. */
int nomad_gpu_save_checkpoint(nomad_gpu_ctx* ctx, const char* path);

/* Restore factors, pass count and bold-driver state from a checkpoint file written
 * for a problem of the same m, n and dim (NOMAD_ERR_INVALID_ARG otherwise).  A
 * REPLAY, DSGD or DSGDPP context restored from the checkpoint of epoch k and run for
 * e epochs ends with the same factors, bit for bit, as one that ran k + e epochs
 * without stopping. */
int nomad_gpu_load_checkpoint(nomad_gpu_ctx* ctx, const char* path);

/* The DSGD objective of the current factors (calobj_mpi, sgd-mpi-omp.cpp:122-160):
 * sum over training ratings of e^2 + reg * (sum_i nnz_row(i) |w_i|^2 +
 * sum_j nnz_col(j) |h_j|^2), e in fp32 as in nomad_gpu_sse, everything summed in
 * FP64.  Any mode.  The first call counts the ratings of every row on the device. */
int nomad_gpu_objective(nomad_gpu_ctx* ctx, double* objective);

/* Describe the context (sizes, workers, segments, memory). */
int nomad_gpu_get_info(nomad_gpu_ctx* ctx, nomad_gpu_info* info);

/* Free every device and host resource of the context.  NULL is a no-op. */
void nomad_gpu_destroy(nomad_gpu_ctx* ctx);

/* Static description of a status code. */
const char* nomad_gpu_strerror(int status);

/* Detail of the most recent failing call made by this thread ("" if none). */
const char* nomad_gpu_last_error(void);

/* 1 when a usable sm_103 device is present, else 0. */
int nomad_gpu_device_ok(int32_t device);

/* Tracing: for every column token, the seconds from the start of the most recent ASYNC
 * nomad_gpu_epoch launch to the moment the token finished its last pass (0 for a
 * column without training ratings).  `seconds` has n entries.  Shows which serial
 * column chains set the epoch time.  NOMAD_ERR_UNSUPPORTED in other modes. */
int nomad_gpu_token_finish_times(nomad_gpu_ctx* ctx, double* seconds);

/* ---- autotuning of the ASYNC kernel ------------------------------------------------
 * One configuration tried by nomad_gpu_autotune and its mean device time per epoch. */
typedef struct nomad_gpu_tune_trial {
  int32_t warps_per_block;   /* compute warps per thread block                          */
  int32_t priority_permille; /* priority threshold (negative: no priority queues)       */
  int32_t long_visit;        /* visits this long or longer take the blocked path        */
  int32_t status;            /* NOMAD_OK, or the status the trial ended with            */
  double device_ms;          /* mean device time of the timed epochs                    */
} nomad_gpu_tune_trial;

/* Chooses the runtime configuration of the ASYNC (non-exact) kernel for this problem by
 * measurement: coordinate descent over warps per block (the compiled maximum and two
 * and four fewer), then the priority threshold (25, 50, 100 permille, off), then the
 * long-visit length (10, 14, 20).  Each trial is a fresh context from params (the same
 * initial factors every time), one untimed epoch and `epochs` timed ones; the factors it
 * trains are discarded.  On success *params holds the fastest configuration (the other
 * fields unchanged) and trials[0 .. *n_trials) the measurements (at most max_trials are
 * stored; trials may be NULL when max_trials is 0).  NOMAD_ERR_UNSUPPORTED for other
 * modes and for exact = 1. */
int nomad_gpu_autotune(const nomad_gpu_problem* prob, nomad_gpu_params* params, int32_t epochs,
                       nomad_gpu_tune_trial* trials, int32_t max_trials, int32_t* n_trials);

/* ---- evaluation without device allocation ---------------------------------------
 * No counterpart in the reference: it is an extra entry point for callers that
 * cannot obtain device memory from the CUDA allocator -- a host runtime that hands
 * out device memory only from its own pool, or a latency-sensitive loop that must
 * not call cudaMalloc/cudaFree because cudaFree waits for the whole device.  Such a
 * caller owns every buffer (inputs and the output) and this call allocates nothing:
 * the evaluation kernel's per-block FP64 partial sums live in one fixed array
 * compiled into the library (NOMAD_NOALLOC_MAX_BLOCKS doubles, 16 KiB on every GPU
 * that loads the library, held until the process exits).
 *
 * Computes, asynchronously on `stream` (a cudaStream_t, NULL = default stream), the
 * squared-error sum  sum (<h_j, w_i> - v)^2  of one CSC rating set and writes it to
 * the device double *sse_out.  Layout (as nomad_gpu_init builds it):
 *   W        [m x kpad] factor rows, H [n x kpad] factor columns, row-major, in fp32
 *            (precision NOMAD_PREC_FP32, kpad = dim rounded up to 4) or bf16
 *            (NOMAD_PREC_BF16_SR, kpad = dim rounded up to 8); padding zero;
 *   ratings  nnz pairs {int32 row, float value}, grouped by column;
 *   col_ptr  n + 1 int64 offsets of the columns in `ratings`: col_ptr[0] == 0,
 *            non-decreasing, col_ptr[n] == nnz (not checked: the host cannot read
 *            them; an offset table that breaks this reads past `ratings`).
 * W and H must be 16-byte aligned, ratings, col_ptr and sse_out 8-byte aligned (a
 * sub-view at an odd offset is refused with NOMAD_ERR_INVALID_ARG before any device
 * work), and nnz > 0 needs n > 0.  nnz = 0 writes 0 to *sse_out.
 * blocks = 0 picks 8 per SM (at most NOMAD_NOALLOC_MAX_BLOCKS); larger values are
 * rejected with NOMAD_ERR_INVALID_ARG.  The first call on a device looks up the
 * array's device address with that device made current (it is restored afterwards)
 * and keeps it for the life of the process, so a device reset (cudaDeviceReset, or
 * re-creating the primary context) after that first call is not supported; make that
 * first call before capturing any stream.  Every call uses the same array, so calls
 * that overlap on the GPU (different streams, no ordering) race and give wrong sums;
 * each call rewrites every partial it reads, so nothing needs clearing.  Work is
 * ordered on `stream` only: inputs produced by earlier work on the same stream are
 * read after it. */
#define NOMAD_NOALLOC_MAX_BLOCKS 2048
int nomad_gpu_sse_noalloc(int32_t device, int32_t precision, int32_t n, int32_t dim,
                          const void* W, const void* H, const void* ratings,
                          const int64_t* col_ptr, int64_t nnz, int32_t blocks,
                          double* sse_out, void* stream);

/* ---- batched problems ------------------------------------------------------------ */
/* Many independent completion problems of uneven m, n, nnz and rank trained together:
 * one persistent launch per epoch (captured once as a CUDA graph and replayed), fed by a
 * device work queue of problems sorted by size (largest first); a warp takes a problem
 * and runs its epoch with the reference's one-worker schedule -- columns in index order,
 * each column's ratings in row order (nb_main.cpp:82-97, 554-558 with one thread and one
 * rank).  With params.exact = 1 and FP32 storage every problem's factors equal the
 * one-worker replay bit for bit; otherwise FMA arithmetic, FP32 or BF16_SR storage.
 * Uses params.precision, exact, lrate, drate, reg, seed, init_parts, device; dim comes
 * per problem (at most 128).  No counterpart in the reference (it trains one problem
 * per run).  When every set is row-major with one value type, the CSCs of all
 * problems are built on the device in one sort (else on the host, problem by problem);
 * a column out of range or a repeated cell is refused either way, naming the problem. */
typedef struct nomad_gpu_batch_problem {
  int32_t m, n, dim, reserved;
  nomad_gpu_matrix train, test; /* as in nomad_gpu_problem                             */
  const float* W0;              /* optional [m x dim]; NULL: reference init            */
  const float* H0;              /* optional [n x dim]                                  */
} nomad_gpu_batch_problem;

typedef struct nomad_gpu_batch nomad_gpu_batch; /* opaque */

int nomad_gpu_batch_init(nomad_gpu_batch** out, const nomad_gpu_batch_problem* problems,
                         int32_t count, const nomad_gpu_params* params);
/* n_epochs epochs of every problem; st->updates sums over problems, device_ms times the
 * graph launches (CUDA events). */
int nomad_gpu_batch_epoch(nomad_gpu_batch* b, int32_t n_epochs, nomad_gpu_epoch_stats* st);
/* One configuration tried by nomad_gpu_batch_autotune and its mean device time per epoch. */
typedef struct nomad_gpu_batch_tune_trial {
  int32_t batch_share;  /* large-problem threshold (params.batch_share)            */
  int32_t status;       /* NOMAD_OK, or the status the trial ended with             */
  double device_ms;     /* mean device time of the timed epochs                     */
  int32_t large_problems; /* problems that ran on whole thread blocks               */
  int32_t reserved;
} nomad_gpu_batch_tune_trial;

/* Chooses the batched form's large-problem threshold (params.batch_share) for these
 * problems by measurement: shares 2, 4, 8, 16 and "never", each a fresh batch from
 * params, one untimed epoch and `epochs` timed ones (the factors are discarded).  On
 * success params->batch_share holds the fastest share and trials[0 .. *n_trials) the
 * measurements.  NOMAD_ERR_UNSUPPORTED for exact = 1 (one warp per problem).  No
 * counterpart in the reference (it trains one problem per run). */
int nomad_gpu_batch_autotune(const nomad_gpu_batch_problem* problems, int32_t count, nomad_gpu_params* params,
                             int32_t epochs, nomad_gpu_batch_tune_trial* trials, int32_t max_trials,
                             int32_t* n_trials);

/* Per-problem RMSE (FP64 sums), arrays of `count` doubles; a problem without ratings in a
 * set gets 0. */
int nomad_gpu_batch_rmse(nomad_gpu_batch* b, double* train_rmse, double* test_rmse);
int nomad_gpu_batch_get_factors(nomad_gpu_batch* b, int32_t problem, float* W, float* H);
void nomad_gpu_batch_destroy(nomad_gpu_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* NOMAD_GPU_H_ */
