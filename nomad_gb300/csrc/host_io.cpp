// host_io.cpp -- train.dat/test.dat I/O, the --output factor dump, the reference's
// factor initialisation, and the library's host-side helpers.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <random>

#include <unistd.h>

#include "common.h"

namespace nomad {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}
void clear_last_error() { g_last_error.clear(); }
const char* last_error() { return g_last_error.c_str(); }

int host_threads(int requested) {
  if (requested > 0) return requested;
  unsigned hw = std::thread::hardware_concurrency();
  return hw ? static_cast<int>(hw) : 1;
}

void parallel_dynamic(int64_t count, int64_t grain, int threads,
                      const std::function<void(int, int64_t, int64_t)>& fn) {
  if (count <= 0) return;
  grain = std::max<int64_t>(grain, 1);
  const int64_t nchunks = (count + grain - 1) / grain;
  threads = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(threads, nchunks)));
  std::atomic<int64_t> next{0};
  auto run = [&](int t) {
    for (int64_t c = next.fetch_add(1); c < nchunks; c = next.fetch_add(1))
      fn(t, c * grain, std::min(count, (c + 1) * grain));
  };
  if (threads == 1) {
    run(0);
    return;
  }
  std::vector<std::thread> pool;
  pool.reserve(threads);
  for (int t = 0; t < threads; ++t) pool.emplace_back(run, t);
  for (auto& th : pool) th.join();
}

void prefault(void* p, size_t bytes, int threads) {
  if (!p || bytes == 0) return;
  const long ps = sysconf(_SC_PAGESIZE);
  const size_t page = ps > 0 ? static_cast<size_t>(ps) : 4096;
  char* b = static_cast<char*>(p);
  const int64_t pages = static_cast<int64_t>((bytes + page - 1) / page);
  const int t = static_cast<int>(std::min<int64_t>(threads, std::max<int64_t>(1, pages / 64)));
  parallel_chunks(pages, t, [&](int, int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      const size_t at = std::min(static_cast<size_t>(i) * page, bytes - 1);
      reinterpret_cast<volatile char*>(b)[at] = 0;
    }
  });
}

void parallel_chunks(int64_t count, int threads,
                     const std::function<void(int, int64_t, int64_t)>& fn) {
  if (count <= 0) return;
  threads = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(threads, count)));
  if (threads == 1) {
    fn(0, 0, count);
    return;
  }
  std::vector<std::thread> pool;
  pool.reserve(threads);
  for (int t = 0; t < threads; ++t) {
    const int64_t lo = count * t / threads, hi = count * (t + 1) / threads;
    pool.emplace_back([&fn, t, lo, hi] { fn(t, lo, hi); });
  }
  for (auto& th : pool) th.join();
}

double SplitMix64::normal() {
  // Box-Muller on two uniforms; u1 in (0, 1] so the log is finite.
  const double u1 = 1.0 - uniform();
  const double u2 = uniform();
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

}  // namespace nomad

using nomad::set_last_error;

extern "C" {

// nb_data.cpp:32-78 -- header of the PETSc-style binary matrix, either id.
int nomad_io_read_header(const char* path, int32_t* file_id, int32_t* m, int32_t* n,
                         int64_t* nnz) {
  nomad::clear_last_error();
  if (!path) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null path");
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) NOMAD_FAIL(NOMAD_ERR_IO, "cannot open file: %s", path);
  int32_t id = 0;
  if (!f.read(reinterpret_cast<char*>(&id), 4)) NOMAD_FAIL(NOMAD_ERR_FORMAT, "error in reading ID from %s", path);
  int32_t mm = 0, nn = 0;
  int64_t z = 0;
  if (id == NOMAD_FILE_ID_INT) {
    int32_t h[3];
    if (!f.read(reinterpret_cast<char*>(h), sizeof(h))) NOMAD_FAIL(NOMAD_ERR_FORMAT, "error in reading header from %s", path);
    mm = h[0];
    nn = h[1];
    z = h[2];
  } else if (id == NOMAD_FILE_ID_LONG) {
    int32_t h[2];
    if (!f.read(reinterpret_cast<char*>(h), sizeof(h))) NOMAD_FAIL(NOMAD_ERR_FORMAT, "error in reading header from %s", path);
    mm = h[0];
    nn = h[1];
    if (!f.read(reinterpret_cast<char*>(&z), sizeof(z))) NOMAD_FAIL(NOMAD_ERR_FORMAT, "error in reading nnz from %s", path);
  } else {
    NOMAD_FAIL(NOMAD_ERR_FORMAT, "%d does not identify a valid binary matrix file (%s)", id, path);
  }
  if (mm < 0 || nn < 0 || z < 0) NOMAD_FAIL(NOMAD_ERR_FORMAT, "negative sizes in header of %s", path);
  if (file_id) *file_id = id;
  if (m) *m = mm;
  if (n) *n = nn;
  if (nnz) *nnz = z;
  return NOMAD_OK;
}

// nb_data.cpp:83-130 with one part: row counts, then every column index, then every
// value.  Unlike the reference (which trusts the file) the counts and indices are
// validated, and a short file is a NOMAD_ERR_FORMAT status rather than exit(1).
int nomad_io_read(const char* path, nomad_io_matrix* out) {
  if (!out) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "null output");
  std::memset(out, 0, sizeof(*out));
  int32_t id, m, n;
  int64_t nnz;
  int rc = nomad_io_read_header(path, &id, &m, &n, &nnz);
  if (rc) return rc;
  std::ifstream f(path, std::ios::in | std::ios::binary);
  f.seekg(id == NOMAD_FILE_ID_INT ? 16 : 20, std::ios::beg);
  int32_t* rcnt = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max<int64_t>(m, 1)));
  int32_t* cols = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
  double* vals = static_cast<double*>(std::malloc(sizeof(double) * std::max<int64_t>(nnz, 1)));
  auto fail = [&](int code, const char* what) {
    std::free(rcnt);
    std::free(cols);
    std::free(vals);
    set_last_error("%s (%s)", what, path);
    return code;
  };
  if (!rcnt || !cols || !vals) return fail(NOMAD_ERR_OOM, "host allocation failed");
  if (!f.read(reinterpret_cast<char*>(rcnt), static_cast<std::streamsize>(m) * 4))
    return fail(NOMAD_ERR_FORMAT, "error in reading nnz values from file");
  int64_t total = 0;
  for (int32_t i = 0; i < m; ++i) {
    if (rcnt[i] < 0) return fail(NOMAD_ERR_FORMAT, "negative row count");
    total += rcnt[i];
  }
  if (total != nnz) return fail(NOMAD_ERR_FORMAT, "row counts do not add up to nnz");
  if (!f.read(reinterpret_cast<char*>(cols), static_cast<std::streamsize>(nnz) * 4))
    return fail(NOMAD_ERR_FORMAT, "error in reading column indices from file");
  if (!f.read(reinterpret_cast<char*>(vals), static_cast<std::streamsize>(nnz) * 8))
    return fail(NOMAD_ERR_FORMAT, "error in reading matrix values from file");
  for (int64_t i = 0; i < nnz; ++i)
    if (cols[i] < 0 || cols[i] >= n) return fail(NOMAD_ERR_FORMAT, "column index out of range");
  out->file_id = id;
  out->m = m;
  out->n = n;
  out->nnz = nnz;
  out->row_counts = rcnt;
  out->cols = cols;
  out->vals = vals;
  return NOMAD_OK;
}

// convert.py:99-105 ("=iiii" header, then "=%si" row sizes, "=%si" indices,
// "=%sd" values) and synthgen.cpp:298-311 (id 1015 with a long long nnz).
int nomad_io_write(const char* path, int32_t m, int32_t n, int64_t nnz,
                   const int32_t* row_counts, const int32_t* cols, const double* vals,
                   int32_t file_id) {
  nomad::clear_last_error();
  if (!path || m < 0 || n < 0 || nnz < 0 || (m > 0 && !row_counts) ||
      (nnz > 0 && (!cols || !vals)))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_io_write");
  if (file_id == 0) file_id = nnz < (int64_t(1) << 31) ? NOMAD_FILE_ID_INT : NOMAD_FILE_ID_LONG;
  if (file_id != NOMAD_FILE_ID_INT && file_id != NOMAD_FILE_ID_LONG)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "unknown file id %d", file_id);
  if (file_id == NOMAD_FILE_ID_INT && nnz >= (int64_t(1) << 31))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "nnz %lld does not fit the 1211216 header", (long long)nnz);
  std::ofstream f(path, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!f) NOMAD_FAIL(NOMAD_ERR_IO, "cannot open %s for writing", path);
  f.write(reinterpret_cast<const char*>(&file_id), 4);
  f.write(reinterpret_cast<const char*>(&m), 4);
  f.write(reinterpret_cast<const char*>(&n), 4);
  if (file_id == NOMAD_FILE_ID_INT) {
    const int32_t z = static_cast<int32_t>(nnz);
    f.write(reinterpret_cast<const char*>(&z), 4);
  } else {
    const long long z = nnz;
    f.write(reinterpret_cast<const char*>(&z), 8);
  }
  f.write(reinterpret_cast<const char*>(row_counts), static_cast<std::streamsize>(m) * 4);
  f.write(reinterpret_cast<const char*>(cols), static_cast<std::streamsize>(nnz) * 4);
  f.write(reinterpret_cast<const char*>(vals), static_cast<std::streamsize>(nnz) * 8);
  if (!f) NOMAD_FAIL(NOMAD_ERR_IO, "short write to %s", path);
  return NOMAD_OK;
}

void nomad_io_free(nomad_io_matrix* mat) {
  if (!mat) return;
  std::free(mat->row_counts);
  std::free(mat->cols);
  std::free(mat->vals);
  std::memset(mat, 0, sizeof(*mat));
}

// nb_main.cpp:683-705 (rows) then :349-366 (columns); `ofs << "," << v` uses the
// stream's default floatfield, i.e. %g with 6 significant digits.
int nomad_io_write_factors(const char* path, int32_t m, int32_t n, int32_t dim,
                           const float* W, const float* H) {
  nomad::clear_last_error();
  if (!path || dim <= 0 || (m > 0 && !W) || (n > 0 && !H))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_io_write_factors");
  std::ofstream ofs(path, std::ios::out | std::ios::trunc);
  if (!ofs) NOMAD_FAIL(NOMAD_ERR_IO, "cannot open %s for writing", path);
  for (int32_t i = 0; i < m; ++i) {
    ofs << "row," << i;
    for (int32_t t = 0; t < dim; ++t) ofs << "," << static_cast<double>(W[int64_t(i) * dim + t]);
    ofs << "\n";
  }
  for (int32_t j = 0; j < n; ++j) {
    ofs << "column," << j;
    for (int32_t t = 0; t < dim; ++t) ofs << "," << static_cast<double>(H[int64_t(j) * dim + t]);
    ofs << "\n";
  }
  if (!ofs) NOMAD_FAIL(NOMAD_ERR_IO, "short write to %s", path);
  return NOMAD_OK;
}

namespace {

// The 64-bit Mersenne Twister with std::mt19937_64's parameters (Matsumoto and
// Nishimura's MT19937-64), producing 312 tempered outputs per twist, and the values of
// std::uniform_real_distribution<double>(0, b) drawn from it as C++ specifies them
// (generate_canonical: one 64-bit draw x gives x / 2^64, or the largest double below 1
// when that rounds to 1; then times b), narrowed to float.  Identical to drawing through
// the standard library one value at a time, and faster.
class Mt64Uniform {
 public:
  explicit Mt64Uniform(uint64_t seed) {
    mt_[0] = seed;
    for (int i = 1; i < kN; ++i) mt_[i] = 6364136223846793005ULL * (mt_[i - 1] ^ (mt_[i - 1] >> 62)) + static_cast<uint64_t>(i);
  }
  // the canonical values x / 2^64 (below 1) themselves
  void fill_canonical(double* dst, int64_t count) {
    const double below_one = std::nextafter(1.0, 0.0);
    while (count > 0) {
      if (pos_ == kN) twist();
      const int take = static_cast<int>(std::min<int64_t>(count, kN - pos_));
      for (int k = 0; k < take; ++k) {
        const double c = static_cast<double>(out_[pos_ + k]) * 0x1p-64;
        dst[k] = c >= 1.0 ? below_one : c;
      }
      pos_ += take;
      dst += take;
      count -= take;
    }
  }
  void fill(float* dst, int64_t count, double b) {
    const double below_one = std::nextafter(1.0, 0.0);
    while (count > 0) {
      if (pos_ == kN) twist();
      const int take = static_cast<int>(std::min<int64_t>(count, kN - pos_));
      for (int k = 0; k < take; ++k) {
        double c = static_cast<double>(out_[pos_ + k]) * 0x1p-64;
        if (c >= 1.0) c = below_one;
        dst[k] = static_cast<float>(c * b + 0.0);
      }
      pos_ += take;
      dst += take;
      count -= take;
    }
  }

 private:
  static constexpr int kN = 312, kM = 156;
  void twist() {
    constexpr uint64_t kUpper = 0xFFFFFFFF80000000ULL, kLower = 0x7FFFFFFFULL, kA = 0xB5026F5AA96619E9ULL;
    auto step = [&](int i, int next, int far) {
      const uint64_t x = (mt_[i] & kUpper) | (mt_[next] & kLower);
      mt_[i] = mt_[far] ^ (x >> 1) ^ ((x & 1) ? kA : 0);
    };
    int i = 0;
    for (; i < kN - kM; ++i) step(i, i + 1, i + kM);
    for (; i < kN - 1; ++i) step(i, i + 1, i + kM - kN);
    step(kN - 1, 0, kM - 1);
    for (int k = 0; k < kN; ++k) {
      uint64_t y = mt_[k];
      y ^= (y >> 29) & 0x5555555555555555ULL;
      y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
      y ^= (y << 37) & 0xFFF7EEE000000000ULL;
      y ^= y >> 43;
      out_[k] = y;
    }
    pos_ = 0;
  }
  uint64_t mt_[kN];
  uint64_t out_[kN];
  int pos_ = kN;
};

}  // namespace

extern "C++" {
namespace nomad {
void reference_canonical(uint64_t stream_seed, int64_t count, double* dst) {
  Mt64Uniform(stream_seed).fill_canonical(dst, count);
}
}  // namespace nomad
}

// nb_main.cpp:450-455 (rows of part t from mt19937_64(seed + rank*131 + t + 1)) and
// nb_main.cpp:71-92 (every column's values from mt19937_64(seed + rank*131 + 139)),
// single rank, each value uniform_real_distribution<double>(0, 1/sqrt(dim)) narrowed to
// float.  Row blocks follow read_data's ceil(m / parts) split (nb_data.cpp:83-89).
int nomad_reference_init(int32_t m, int32_t n, int32_t dim, uint64_t seed,
                         int32_t init_parts, float* W, float* H) {
  nomad::clear_last_error();
  if (m < 0 || n < 0 || dim <= 0 || init_parts <= 0)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_reference_init");
  const double b = 1.0 / std::sqrt(dim);
  const int32_t P = init_parts;
  const int32_t rows_per_part = m / P + ((m % P > 0) ? 1 : 0);
  if (W) {
    nomad::parallel_chunks(P, nomad::host_threads(), [&](int, int64_t lo_t, int64_t hi_t) {
      for (int64_t t = lo_t; t < hi_t; ++t) {
        const int64_t lo = std::min<int64_t>(int64_t(rows_per_part) * t, m);
        const int64_t hi = std::min<int64_t>(int64_t(rows_per_part) * (t + 1), m);
        Mt64Uniform(seed + 0 * 131 + t + 1).fill(W + lo * dim, (hi - lo) * dim, b);
      }
    });
  }
  if (H) Mt64Uniform(seed + 0 * 131 + 139).fill(H, int64_t(n) * dim, b);
  return NOMAD_OK;
}

// Checkpoint file (own format): factors, pass count and bold-driver state at an
// epoch boundary.  Plays the part of NomadBody::archive_local / restore_local
// (nb_checkpoint.cpp:47-59, 114-120), which keep each worker thread's rows as
// doubles in a ".state" file.
namespace {
constexpr char kCkptMagic[8] = {'N', 'O', 'M', 'A', 'D', 'C', 'P', '1'};

uint64_t fnv1a64(uint64_t h, const void* data, size_t bytes) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < bytes; ++i) {
    h ^= p[i];
    h *= 1099511628211ULL;
  }
  return h;
}
constexpr uint64_t kFnvBasis = 14695981039346656037ULL;

// header after the magic: int32 m, n, dim, epochs_done; float64 lrate, objective.
// *fields_hash = FNV-1a 64 of those 32 bytes, the start of the file's hash.
int ckpt_header(std::ifstream& f, const char* path, nomad_io_checkpoint_info* info, uint64_t* hash,
                uint64_t* fields_hash) {
  char magic[8];
  if (!f.read(magic, 8) || std::memcmp(magic, kCkptMagic, 8) != 0)
    NOMAD_FAIL(NOMAD_ERR_FORMAT, "%s is not a checkpoint file", path);
  int32_t h[4];
  double d[2];
  if (!f.read(reinterpret_cast<char*>(h), 16) || !f.read(reinterpret_cast<char*>(d), 16) ||
      !f.read(reinterpret_cast<char*>(hash), 8))
    NOMAD_FAIL(NOMAD_ERR_FORMAT, "short checkpoint header in %s", path);
  if (h[0] < 0 || h[1] < 0 || h[2] <= 0 || h[3] < 0)
    NOMAD_FAIL(NOMAD_ERR_FORMAT, "invalid sizes in checkpoint header of %s", path);
  info->m = h[0];
  info->n = h[1];
  info->dim = h[2];
  info->epochs_done = h[3];
  info->lrate = d[0];
  info->objective = d[1];
  *fields_hash = fnv1a64(fnv1a64(kFnvBasis, h, sizeof(h)), d, sizeof(d));
  return NOMAD_OK;
}
}  // namespace

int nomad_io_write_checkpoint(const char* path, const nomad_io_checkpoint_info* info, const float* W,
                              const float* H) {
  nomad::clear_last_error();
  if (!path || !info) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_io_write_checkpoint");
  const int32_t m = info->m, n = info->n, dim = info->dim;
  if (m < 0 || n < 0 || dim <= 0 || info->epochs_done < 0 || (m > 0 && !W) || (n > 0 && !H))
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_io_write_checkpoint");
  const size_t wb = static_cast<size_t>(m) * dim * sizeof(float);
  const size_t hb = static_cast<size_t>(n) * dim * sizeof(float);
  const int32_t h[4] = {m, n, dim, info->epochs_done};
  const double d[2] = {info->lrate, info->objective};
  uint64_t hash = fnv1a64(fnv1a64(kFnvBasis, h, sizeof(h)), d, sizeof(d));
  hash = fnv1a64(fnv1a64(hash, W, m ? wb : 0), H, n ? hb : 0);
  const std::string tmp = std::string(path) + ".tmp";
  {
    std::ofstream f(tmp, std::ios::out | std::ios::binary | std::ios::trunc);
    if (!f) NOMAD_FAIL(NOMAD_ERR_IO, "cannot open %s for writing", tmp.c_str());
    f.write(kCkptMagic, 8);
    f.write(reinterpret_cast<const char*>(h), sizeof(h));
    f.write(reinterpret_cast<const char*>(d), sizeof(d));
    f.write(reinterpret_cast<const char*>(&hash), sizeof(hash));
    if (m) f.write(reinterpret_cast<const char*>(W), static_cast<std::streamsize>(wb));
    if (n) f.write(reinterpret_cast<const char*>(H), static_cast<std::streamsize>(hb));
    f.flush();
    if (!f) {
      std::remove(tmp.c_str());
      NOMAD_FAIL(NOMAD_ERR_IO, "short write to %s", tmp.c_str());
    }
  }
  if (std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    NOMAD_FAIL(NOMAD_ERR_IO, "cannot rename %s to %s", tmp.c_str(), path);
  }
  return NOMAD_OK;
}

int nomad_io_read_checkpoint_header(const char* path, nomad_io_checkpoint_info* info) {
  nomad::clear_last_error();
  if (!path || !info) NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments");
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) NOMAD_FAIL(NOMAD_ERR_IO, "cannot open file: %s", path);
  uint64_t hash = 0, fields = 0;
  return ckpt_header(f, path, info, &hash, &fields);
}

int nomad_io_read_checkpoint(const char* path, int32_t m, int32_t n, int32_t dim, float* W, float* H,
                             nomad_io_checkpoint_info* info) {
  nomad::clear_last_error();
  if (!path || m < 0 || n < 0 || dim <= 0)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "invalid arguments to nomad_io_read_checkpoint");
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) NOMAD_FAIL(NOMAD_ERR_IO, "cannot open file: %s", path);
  nomad_io_checkpoint_info hdr;
  uint64_t want = 0, hash = 0;
  const int rc = ckpt_header(f, path, &hdr, &want, &hash);
  if (rc) return rc;
  if (hdr.m != m || hdr.n != n || hdr.dim != dim)
    NOMAD_FAIL(NOMAD_ERR_INVALID_ARG, "checkpoint %s holds m=%d n=%d dim=%d, expected m=%d n=%d dim=%d", path,
               hdr.m, hdr.n, hdr.dim, m, n, dim);
  // Read in bounded chunks so that a NULL output still has its bytes hashed.
  std::vector<char> buf;
  auto part = [&](float* out, int64_t count) -> bool {
    int64_t left = count * static_cast<int64_t>(sizeof(float));
    char* dst = reinterpret_cast<char*>(out);
    if (!out) buf.resize(static_cast<size_t>(std::min<int64_t>(left, 1 << 22)));
    while (left > 0) {
      const int64_t k = out ? left : std::min<int64_t>(left, static_cast<int64_t>(buf.size()));
      char* p = out ? dst : buf.data();
      if (!f.read(p, static_cast<std::streamsize>(k))) return false;
      hash = fnv1a64(hash, p, static_cast<size_t>(k));
      if (out) dst += k;
      left -= k;
    }
    return true;
  };
  if (!part(W, static_cast<int64_t>(m) * dim) || !part(H, static_cast<int64_t>(n) * dim))
    NOMAD_FAIL(NOMAD_ERR_FORMAT, "checkpoint %s is shorter than its header says", path);
  if (f.peek() != std::char_traits<char>::eof())
    NOMAD_FAIL(NOMAD_ERR_FORMAT, "checkpoint %s is longer than its header says", path);
  if (hash != want) NOMAD_FAIL(NOMAD_ERR_FORMAT, "checkpoint %s fails its hash check", path);
  if (info) *info = hdr;
  return NOMAD_OK;
}

}  // extern "C"
