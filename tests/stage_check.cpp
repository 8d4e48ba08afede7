// The staged uploads of nomad_gb300/csrc/host_stage.cpp on the CPU, against the stand-in
// runtime of tests/stub/cuda_runtime.h whose copies complete late, on a thread of their
// own, in queue order.  For random sets of source arrays (empty ones, ones far larger than
// a 32 MB staging window, many small ones) the destination must hold their concatenation
// exactly, narrowed uploads the static_cast of every double, and no byte past the end may
// be written -- a staging buffer refilled before its copy had finished would show up as
// wrong bytes.  Prints "stage ok" and exits 0 when every case holds.
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

#include "stage.h"

namespace nomad {
int host_threads(int) { return 8; }
}  // namespace nomad

namespace {

struct Copy {
  void* dst;
  const void* src;
  size_t bytes;
};
std::mutex g_mu;
std::condition_variable g_cv;
std::deque<Copy> g_queue;
long g_queued = 0, g_done = 0;
bool g_quit = false;

void copy_engine() {
  std::mt19937 rng(7);
  for (;;) {
    Copy c;
    {
      std::unique_lock<std::mutex> l(g_mu);
      g_cv.wait(l, [] { return g_quit || !g_queue.empty(); });
      if (g_queue.empty()) return;
      c = g_queue.front();
    }
    std::this_thread::sleep_for(std::chrono::microseconds(200 + rng() % 800));  // a slow engine
    std::memcpy(c.dst, c.src, c.bytes);
    {
      std::lock_guard<std::mutex> l(g_mu);
      g_queue.pop_front();
      ++g_done;
    }
    g_cv.notify_all();
  }
}

}  // namespace

struct StubEvent {
  long after = 0;  // copies queued when the event was recorded
};

cudaError_t cudaHostAlloc(void** p, size_t bytes, unsigned) {
  *p = std::malloc(bytes);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned) {
  *e = new StubEvent;
  return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t) {
  std::lock_guard<std::mutex> l(g_mu);
  e->after = g_queued;
  return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t e) {
  std::unique_lock<std::mutex> l(g_mu);
  g_cv.wait(l, [&] { return g_done >= e->after; });
  return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e) {
  delete e;
  return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, cudaMemcpyKind, cudaStream_t) {
  {
    std::lock_guard<std::mutex> l(g_mu);
    g_queue.push_back(Copy{dst, src, bytes});
    ++g_queued;
  }
  g_cv.notify_all();
  return cudaSuccess;
}

int main() {
  std::thread engine(copy_engine);
  std::mt19937_64 rng(5);
  int fails = 0;
  for (int trial = 0; trial < 12 && !fails; ++trial) {
    const int count = 1 + static_cast<int>(rng() % 200);
    std::vector<std::vector<char>> src(count);
    std::vector<const void*> ptrs(count);
    std::vector<size_t> bytes(count), counts(count);
    std::vector<const double*> dptrs(count);
    size_t total = 0, total_d = 0;
    for (int i = 0; i < count; ++i) {
      const uint64_t kind = rng() % 8;
      size_t n = kind == 0 ? 0 : kind == 1 ? rng() % (72u << 20) : rng() % (600u << 10);
      n &= ~size_t{7};  // whole doubles, for the narrowed uploads
      src[i].resize(n);
      for (size_t j = 0; j < n; j += 8) {  // finite doubles (NaN payloads need not survive a cast)
        const double v = static_cast<double>(static_cast<int64_t>(rng() % 2000001) - 1000000) / 997.0;
        std::memcpy(&src[i][j], &v, 8);
      }
      ptrs[i] = n ? src[i].data() : nullptr;
      bytes[i] = n;
      counts[i] = n / 8;
      dptrs[i] = reinterpret_cast<const double*>(ptrs[i]);
      total += n;
      total_d += n / 8;
    }
    std::vector<char> want;
    want.reserve(total);
    for (const auto& v : src) want.insert(want.end(), v.begin(), v.end());
    std::vector<char> dst(total + 16, 0x5a);
    if (nomad::upload_staged_many(dst.data(), ptrs.data(), bytes.data(), count, nullptr) != cudaSuccess ||
        std::memcmp(dst.data(), want.data(), total) != 0 || dst[total] != 0x5a) {
      std::printf("FAIL: concatenation, trial %d (%d arrays, %zu bytes)\n", trial, count, total);
      ++fails;
    }
    std::vector<float> nwant;
    nwant.reserve(total_d);
    for (int i = 0; i < count; ++i)
      for (size_t k = 0; k < counts[i]; ++k) nwant.push_back(static_cast<float>(dptrs[i][k]));
    std::vector<float> nd(total_d + 4, 7.f);
    if (nomad::upload_staged_narrow(nd.data(), dptrs.data(), counts.data(), count, nullptr) != cudaSuccess ||
        std::memcmp(nd.data(), nwant.data(), total_d * sizeof(float)) != 0 || nd[total_d] != 7.f) {
      std::printf("FAIL: narrowed, trial %d (%d arrays, %zu values)\n", trial, count, total_d);
      ++fails;
    }
    if (count == 1 || trial == 0) {  // the single-array form
      std::vector<char> one(bytes[0] + 16, 0x33);
      if (nomad::upload_staged(one.data(), ptrs[0], bytes[0], nullptr) != cudaSuccess ||
          (bytes[0] && std::memcmp(one.data(), src[0].data(), bytes[0]) != 0) || one[bytes[0]] != 0x33) {
        std::printf("FAIL: single array, trial %d\n", trial);
        ++fails;
      }
    }
  }
  {
    std::lock_guard<std::mutex> l(g_mu);
    g_quit = true;
  }
  g_cv.notify_all();
  engine.join();
  std::printf("%s\n", fails ? "stage FAILED" : "stage ok");
  return fails ? 1 : 0;
}
