// common.h -- internal helpers shared by the host sources of libnomad_gpu.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "nomad_gpu.h"
#include "nomad_io.h"

namespace nomad {

// Thread-local detail string behind nomad_gpu_last_error().
void set_last_error(const char* fmt, ...);
void clear_last_error();
const char* last_error();

// Host threads to use (all hardware threads unless a positive request is given).
int host_threads(int requested = 0);

// Run fn(t, lo, hi) on `threads` contiguous chunks of [0, count).
void parallel_chunks(int64_t count, int threads,
                     const std::function<void(int, int64_t, int64_t)>& fn);
// Writes a zero into every page of an output buffer that is about to be filled by a
// device-to-host copy, on `threads` threads: a copy into pages that are not yet mapped
// takes its page faults one after another inside the copy (~0.3 GB/s on the GB300's host),
// touched pages take the copy at full speed.
void prefault(void* p, size_t bytes, int threads);
// Chunks of `grain` items handed to `threads` threads on demand (for uneven items);
// fn(thread, lo, hi) as for parallel_chunks.
void parallel_dynamic(int64_t count, int64_t grain, int threads,
                      const std::function<void(int, int64_t, int64_t)>& fn);

// SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014): a counter-based 64-bit generator, used for every seeded draw the
// library makes on the host so that results do not depend on the thread count.
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  uint64_t next() { return mix(s += 0x9E3779B97F4A7C15ULL); }
  // uniform double in [0, 1) with 53 random bits
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
  // uniform integer in [0, bound) (bound > 0), Lemire's multiply-shift reduction
  uint64_t below(uint64_t bound) {
    return static_cast<uint64_t>((static_cast<unsigned __int128>(next()) * bound) >> 64);
  }
  double normal();  // Box-Muller
};

// The first `count` draws of mt19937_64(stream_seed) as generate_canonical<double>
// values in [0, 1): the reference init's value i of that stream is float(c[i] * b + 0.0)
// for b = 1/sqrt(dim) (nomad_reference_init draws the same values).
void reference_canonical(uint64_t stream_seed, int64_t count, double* dst);

// Stream key for entity `id` of purpose `tag` under `seed`.
inline uint64_t stream_key(uint64_t seed, uint64_t tag, uint64_t id) {
  return SplitMix64::mix(seed ^ SplitMix64::mix(tag * 0x632BE59BD9B4E019ULL + id));
}

}  // namespace nomad

#define NOMAD_FAIL(code, ...)                 \
  do {                                        \
    ::nomad::set_last_error(__VA_ARGS__);     \
    return (code);                            \
  } while (0)
