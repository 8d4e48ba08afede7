/*
 * nomad_io.h -- host-side C-ABI of the GB300 NOMAD library: the reference's
 * train.dat / test.dat binary format, its --output factor dump, the reference's
 * factor initialisation, and seeded synthetic workloads.  These calls need no GPU.
 *
 * Reference interfaces each call replaces (yxtj/nomad, paths inside the project):
 *   nomad_io_read_header   NomadBody::get_num_cols (Code/nomad/nb_data.cpp:180-202)
 *                          and the header branch of read_data (nb_data.cpp:32-78)
 *   nomad_io_read          read_data for one part covering every row
 *                          (nb_data.cpp:19-130)
 *   nomad_io_write         the writers of Scripts/convert.py:99-105 (id 1211216) and
 *                          Code/nomad/synthgen.cpp:298-311 (id 1015)
 *   nomad_io_write_factors the --output dump (nb_main.cpp:349-366, 683-705)
 *   nomad_reference_init   row init nb_main.cpp:450-455 and column init
 *                          nb_main.cpp:70-92 (values only)
 *   nomad_synth_generate   Code/nomad/synthgen.cpp:180-327 (planted-factor ratings
 *                          from degree laws); a new generator, not a port
 *   nomad_io_write_checkpoint / nomad_io_read_checkpoint(_header)
 *                          NomadBody::archive_local / restore_local
 *                          (nb_checkpoint.cpp:47-59, 114-120), one file per
 *                          checkpoint instead of one per worker thread
 */
#ifndef NOMAD_IO_H_
#define NOMAD_IO_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NOMAD_FILE_ID_INT 1211216 /* header: id, m, n, int32 nnz (PETSc MAT_FILE_CLASSID) */
#define NOMAD_FILE_ID_LONG 1015   /* header: id, m, n, int64 nnz                         */

/* A rating matrix in the file's row-major layout.  Arrays returned by
 * nomad_io_read / nomad_synth_generate are owned by the library: release them
 * with nomad_io_free. */
typedef struct nomad_io_matrix {
  int32_t file_id;
  int32_t m;
  int32_t n;
  int32_t reserved;
  int64_t nnz;
  int32_t* row_counts; /* [m]   ratings per row                                   */
  int32_t* cols;       /* [nnz] column index, rows in order                        */
  double* vals;        /* [nnz] value                                              */
} nomad_io_matrix;

/* Header only.  Returns NOMAD_ERR_FORMAT for an unknown id (the reference exits(1)
 * there, nb_data.cpp:76-78; here it is a status). */
int nomad_io_read_header(const char* path, int32_t* file_id, int32_t* m, int32_t* n,
                         int64_t* nnz);

/* Whole file.  Checks the row counts add up to nnz and every column is in [0, n). */
int nomad_io_read(const char* path, nomad_io_matrix* out);

/* Write a matrix.  file_id 0 picks 1211216 when nnz < 2^31 and 1015 otherwise. */
int nomad_io_write(const char* path, int32_t m, int32_t n, int64_t nnz,
                   const int32_t* row_counts, const int32_t* cols, const double* vals,
                   int32_t file_id);

/* Release arrays owned by the library and zero the struct. */
void nomad_io_free(nomad_io_matrix* mat);

/* Text dump "row,<index>,v0,...,v(dim-1)" for every row followed by
 * "column,<index>,..." for every column, values in C++ ostream default format
 * (6 significant digits), as the reference's --output writes them. */
int nomad_io_write_factors(const char* path, int32_t m, int32_t n, int32_t dim,
                           const float* W, const float* H);

/* Checkpoint file: the whole training state at an epoch boundary, where every column
 * token has finished its pass, so no token is in flight and the factors, the pass
 * count and (bold driver) the learning rate and last objective are all there is to
 * keep (the reference also archives the column messages queued at the cut,
 * nb_checkpoint.cpp:61-102; at an epoch boundary there are none).
 * Layout, little-endian:
 *   char     magic[8] = "NOMADCP1"
 *   int32    m, n, dim, epochs_done
 *   float64  lrate, objective      (0 and -1 when no bold-driver state is kept)
 *   uint64   FNV-1a 64 hash of the 32 bytes of sizes, pass count, lrate and
 *            objective above, continued over the W and H bytes that follow
 *   float32  W[m * dim], H[n * dim]   (row-major)
 * The file is written under path + ".tmp" and renamed over path, so a crash while
 * writing leaves an existing checkpoint at path intact. */
typedef struct nomad_io_checkpoint_info {
  int32_t m, n, dim, epochs_done;
  double lrate;      /* bold driver: learning rate of the next pass; 0: none       */
  double objective;  /* bold driver: objective after the last pass; < 0: none      */
} nomad_io_checkpoint_info;

int nomad_io_write_checkpoint(const char* path, const nomad_io_checkpoint_info* info,
                              const float* W, const float* H);

/* Header of a checkpoint file.  NOMAD_ERR_FORMAT when the magic or the sizes are
 * wrong. */
int nomad_io_read_checkpoint_header(const char* path, nomad_io_checkpoint_info* info);

/* Read a checkpoint whose sizes must equal m, n, dim (else NOMAD_ERR_INVALID_ARG).
 * NOMAD_ERR_FORMAT when the file is short, longer than its sizes say, or its hash
 * does not match.  W or H may be NULL to skip it (the hash is still checked); info
 * may be NULL. */
int nomad_io_read_checkpoint(const char* path, int32_t m, int32_t n, int32_t dim,
                             float* W, float* H, nomad_io_checkpoint_info* info);

/* The reference's initial factors, single rank: rows in init_parts blocks of
 * ceil(m/init_parts), block t drawn from mt19937_64(seed + t + 1); columns from
 * mt19937_64(seed + 139) in index order; values uniform_real_distribution<double>
 * (0, 1/sqrt(dim)) rounded to float.  Either output may be NULL. */
int nomad_reference_init(int32_t m, int32_t n, int32_t dim, uint64_t seed,
                         int32_t init_parts, float* W, float* H);

/* ---- synthetic workloads -------------------------------------------------------- */
enum nomad_synth_positions {
  NOMAD_SYNTH_UNIFORM = 0, /* nnz distinct cells uniformly from the m x n grid      */
  NOMAD_SYNTH_DEGREES = 1  /* per-row degree law, columns drawn by a column law
                              without replacement                                  */
};
enum nomad_synth_law {
  NOMAD_LAW_UNIFORM = 0,   /* equal weights                                         */
  NOMAD_LAW_ZIPF = 1,      /* weight of the r-th ranked index = r^-param            */
  NOMAD_LAW_GEOMETRIC = 2  /* i.i.d. geometric degrees with mean param (rows only)  */
};

typedef struct nomad_synth_spec {
  int32_t struct_size; /* = sizeof(nomad_synth_spec)                                */
  int32_t m, n;
  int32_t positions;   /* nomad_synth_positions                                     */
  int64_t nnz_train, nnz_test;
  int32_t row_law, col_law;     /* nomad_synth_law                                  */
  double row_param, col_param;
  int32_t rank;        /* planted rank                                              */
  int32_t integer_values; /* 1: round to integers and clip to [clip_lo, clip_hi]    */
  double factor_std;   /* std of planted factor entries; 0 = rank^-1/4 (unit-variance
                          inner products)                                           */
  double noise_std;
  double offset, scale; /* value = offset + scale*<w*,h*> + noise                   */
  double clip_lo, clip_hi;
  uint64_t seed;
  int32_t threads;     /* host threads, 0 = all                                      */
  int32_t reserved[7];
} nomad_synth_spec;

/* Fill spec with a named workload:
 *   1  10,000 x 2,000, 360,000 / 40,000 uniform cells, rank 10, N(0, 0.1^2) noise
 *   2  480,189 x 17,770, 100,480,507 / 1,408,395, Zipf(0.8) rows, Zipf(1.1) columns,
 *      integers 1-5 from 3 + <w*,h*>_rank20 + N(0, 0.3^2)
 *   3  1,000,990 x 624,961, 252,800,275 / 4,003,960, Zipf(0.9) both sides,
 *      integers 0-100 from 50 + 20<w*,h*>_rank30 + N(0, 8^2)
 *   4  50,082,603 x 39,780, 2.74e9 / 3.0e7, geometric(mean 55) rows, Zipf(1.0)
 *      columns, real values <w*,h*>_rank50 + N(0, 0.2^2)
 * Returns NOMAD_ERR_INVALID_ARG for other numbers. */
int nomad_synth_preset(int32_t workload, nomad_synth_spec* spec);

/* Problem `index` of the batched workload (4,096 independent problems of uneven shape and rank), drawn from `seed`:
 * m log-uniform in [200, 20,000], n log-uniform in [100, 5,000], density log-uniform in
 * [0.5%, 5%] (90% train / 10% test cells, uniform without replacement), rank k drawn from
 * {16, 32, 64}, planted rank k/4 with N(0, (k/4)^-1/2) factors, values <w*,h*> + N(0, 0.1^2).
 * Fills spec (for nomad_synth_generate) and *dim = k. */
int nomad_synth_batch_problem(uint64_t seed, int32_t index, nomad_synth_spec* spec, int32_t* dim);

/* Generate the train and test matrices of a spec (row-major, columns ascending in
 * each row).  Deterministic for a given spec, whatever the thread count. */
int nomad_synth_generate(const nomad_synth_spec* spec, nomad_io_matrix* train,
                         nomad_io_matrix* test);

#ifdef __cplusplus
}
#endif

#endif /* NOMAD_IO_H_ */
