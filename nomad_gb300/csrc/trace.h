// trace.h -- opt-in wall-time tracing of context set-up phases.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>

namespace nomad {

// Wall time of each phase of a context's set-up, printed to stderr when the environment
// variable NOMAD_TRACE_INIT is set (the set-up is part of a job's end-to-end time).  A mark
// given a stream waits for it first, unless NOMAD_TRACE_INIT is "2" (phases then show
// where the host waits, without the marks changing the order of the work).
struct InitTrace {
  const char* env = std::getenv("NOMAD_TRACE_INIT");
  bool on = env != nullptr;
  bool sync = !(env && env[0] == '2');
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char* phase, cudaStream_t s = nullptr) {
    if (!on) return;
    if (s && sync) cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[nomad init] %-24s %8.1f ms\n", phase,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

}  // namespace nomad
