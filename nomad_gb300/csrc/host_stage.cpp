// host_stage.cpp -- staged uploads (stage.h): the caller's pageable arrays are copied by
// host threads into two pinned buffers, window by window, while the copy engine moves the
// previous window to the device.
#include "stage.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.h"

namespace {

// Two pinned staging buffers for uploads from pageable memory, kept for the life of the
// process and used under a lock.
constexpr size_t kStageBytes = size_t{32} << 20;
std::mutex g_stage_mu;
char* g_stage[2] = {nullptr, nullptr};

// The staged copy of `count` host arrays, one after another, into dst: bytes[i] bytes of
// destination each, copied as they are or (narrow) narrowed from twice as many bytes of
// doubles to floats, round to nearest.
cudaError_t staged(void* dst, const void* const* srcs, const size_t* bytes, size_t count, bool narrow,
                   cudaStream_t s) {
  // pieces of at most 1 MB of destination, none across a staging window
  struct Piece {
    const char* src;
    size_t at, len;
  };
  std::vector<Piece> pieces;
  size_t total = 0;
  for (size_t i = 0; i < count; ++i) {
    const char* p = static_cast<const char*>(srcs[i]);
    for (size_t left = bytes[i]; left > 0;) {
      const size_t len = std::min({left, kStageBytes - total % kStageBytes, size_t{1} << 20});
      pieces.push_back(Piece{p, total, len});
      p += narrow ? 2 * len : len;
      total += len;
      left -= len;
    }
  }
  if (total == 0) return cudaSuccess;
  // window w: bytes [w S, (w + 1) S) of the concatenation (S = kStageBytes), pieces
  // [wfirst[w], wfirst[w + 1]), staged in buffer w % 2
  const size_t nwin = (total + kStageBytes - 1) / kStageBytes;
  std::vector<size_t> wfirst(nwin + 1, pieces.size());
  for (size_t q = pieces.size(); q-- > 0;) wfirst[pieces[q].at / kStageBytes] = q;
  std::lock_guard<std::mutex> lock(g_stage_mu);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; ++i)
    if (!g_stage[i]) e = cudaHostAlloc(reinterpret_cast<void**>(&g_stage[i]), kStageBytes, cudaHostAllocPortable);
  cudaEvent_t done[2] = {nullptr, nullptr};
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
  if (e == cudaSuccess) {
    // T host threads, started once, fill window w when its buffer is free (w <= ready);
    // this thread queues each window's copy once every filler is through it (filled[w] =
    // T), then waits for the previous window's copy, which frees that buffer for w + 1.
    const int T =
        static_cast<int>(std::min<size_t>(static_cast<size_t>(std::max(1, nomad::host_threads() - 1)), pieces.size()));
    std::unique_ptr<std::atomic<int>[]> filled(new std::atomic<int>[nwin]);
    for (size_t w = 0; w < nwin; ++w) filled[w].store(0);
    std::atomic<int64_t> ready{1};
    std::atomic<bool> stop{false};
    auto fill = [&](int t) {
      for (size_t w = 0; w < nwin; ++w) {
        while (ready.load(std::memory_order_acquire) < static_cast<int64_t>(w) && !stop.load())
          std::this_thread::yield();
        if (!stop.load()) {
          char* to = g_stage[w & 1];
          for (size_t q = wfirst[w] + static_cast<size_t>(t); q < wfirst[w + 1]; q += static_cast<size_t>(T)) {
            char* at = to + (pieces[q].at - w * kStageBytes);
            if (!narrow) {
              std::memcpy(at, pieces[q].src, pieces[q].len);
              continue;
            }
            const double* from = reinterpret_cast<const double*>(pieces[q].src);
            float* out = reinterpret_cast<float*>(at);
            for (size_t k = 0; k < pieces[q].len / sizeof(float); ++k) out[k] = static_cast<float>(from[k]);
          }
        }
        filled[w].fetch_add(1, std::memory_order_release);
      }
    };
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(T));
    for (int t = 0; t < T; ++t) pool.emplace_back(fill, t);
    for (size_t w = 0; w < nwin && e == cudaSuccess; ++w) {
      while (filled[w].load(std::memory_order_acquire) < T) std::this_thread::yield();
      const size_t n = std::min(kStageBytes, total - w * kStageBytes);
      e = cudaMemcpyAsync(static_cast<char*>(dst) + w * kStageBytes, g_stage[w & 1], n, cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaEventRecord(done[w & 1], s);
      if (e == cudaSuccess && w >= 1) e = cudaEventSynchronize(done[(w - 1) & 1]);
      ready.store(static_cast<int64_t>(w) + 1, std::memory_order_release);
    }
    if (e != cudaSuccess) stop.store(true);
    for (auto& th : pool) th.join();
  }
  // the buffers are reused by the next upload: its copies into them wait for these
  for (int i = 0; i < 2; ++i)
    if (done[i]) {
      if (e == cudaSuccess) e = cudaEventSynchronize(done[i]);
      cudaEventDestroy(done[i]);
    }
  return e;
}

}  // namespace

namespace nomad {

cudaError_t upload_staged(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  return staged(dst, &src, &bytes, 1, false, s);
}

cudaError_t upload_staged_many(void* dst, const void* const* srcs, const size_t* bytes, size_t count,
                               cudaStream_t s) {
  return staged(dst, srcs, bytes, count, false, s);
}

cudaError_t upload_staged_narrow(float* dst, const double* const* srcs, const size_t* counts, size_t count,
                                 cudaStream_t s) {
  std::vector<size_t> bytes(count);
  for (size_t i = 0; i < count; ++i) bytes[i] = counts[i] * sizeof(float);
  return staged(dst, reinterpret_cast<const void* const*>(srcs), bytes.data(), count, true, s);
}

}  // namespace nomad
