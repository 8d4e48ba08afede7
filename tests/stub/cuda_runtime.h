// Stand-in for the CUDA runtime calls that nomad_gb300/csrc/host_stage.cpp makes, so that
// tests/stage_check.cpp can run the staged uploads on a machine without a GPU: the copies
// are carried out later by a thread of the test ("copy engine"), events record how many
// copies were queued before them.
#pragma once

#include <cstddef>

typedef int cudaError_t;
typedef struct StubStream* cudaStream_t;
typedef struct StubEvent* cudaEvent_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum { cudaHostAllocPortable = 1, cudaEventDisableTiming = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1 };

cudaError_t cudaHostAlloc(void** p, size_t bytes, unsigned flags);
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned flags);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventDestroy(cudaEvent_t e);
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s);
