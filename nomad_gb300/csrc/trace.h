// trace.h -- opt-in wall-time tracing of context set-up phases.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>

namespace nomad {

// Wall time of each phase of a context's set-up, printed to stderr when the environment
// variable NOMAD_TRACE_INIT is set (the set-up is part of a job's end-to-end time).
struct InitTrace {
  bool on = std::getenv("NOMAD_TRACE_INIT") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char* phase, cudaStream_t s = nullptr) {
    if (!on) return;
    if (s) cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[nomad init] %-24s %8.1f ms\n", phase,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

}  // namespace nomad
