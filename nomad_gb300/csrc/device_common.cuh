// device_common.cuh -- device helpers shared by the sm_103a kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace nd {

constexpr unsigned kFull = 0xffffffffu;

// Device status words (ctrl[1]); mapped to nomad_gpu_status by the host.
constexpr int kDevErrTimeout = 1;
constexpr int kDevErrBounds = 2;

// ---- memory-ordering primitives (PTX memory model, gpu scope) -----------------
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(int* p, int v) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int atom_exch_acq_rel(int* p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(p), "r"(v)
               : "memory");
  return old;
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- token queues ---------------------------------------------------------------
// One intrusive multi-producer / single-consumer queue per worker (the lock-free
// design of D. Vyukov's "intrusive MPSC node-based queue"), index based: nodes
// 0..n-1 are column tokens, node n+w is worker w's stub.  qnext[node] = next node
// or -1; qtail[w] = last node.  The consumer cursor `head` lives in a register of
// the worker's lane 0.  A token is in at most one queue, so n + P words suffice
// whatever the routing -- no capacity can overflow.
__device__ __forceinline__ void mpsc_push(int* qnext, int* qtail, int w, int node) {
  st_relaxed(&qnext[node], -1);
  const int prev = atom_exch_acq_rel(&qtail[w], node);
  st_release(&qnext[prev], node);  // publishes the node (and the token's state)
}

// Returns a node or -1 (empty, or a producer is between its exchange and its link;
// the caller simply polls again later).
__device__ __forceinline__ int mpsc_pop(int* qnext, int* qtail, int w, int stub, int& head) {
  int h = head;
  int next = ld_acquire(&qnext[h]);
  if (h == stub) {
    if (next < 0) return -1;
    head = next;
    h = next;
    next = ld_acquire(&qnext[h]);
  }
  if (next >= 0) {
    head = next;
    return h;
  }
  if (ld_acquire(&qtail[w]) != h) return -1;
  mpsc_push(qnext, qtail, w, stub);
  next = ld_acquire(&qnext[h]);
  if (next >= 0) {
    head = next;
    return h;
  }
  return -1;
}

// ---- counter-based hashing for stochastic rounding --------------------------------
// "lowbias32" integer hash (C. Wellons, hash-prospector, public domain).
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// fp32 -> bf16 with stochastic rounding: add 16 uniform random bits below the bf16
// mantissa and truncate, so the value rounds up with probability equal to the
// discarded fraction (unbiased).  Inf/NaN are truncated (NaN kept quiet).
__device__ __forceinline__ uint32_t f32_to_bf16_sr_bits(float f, uint32_t r16) {
  uint32_t u = __float_as_uint(f);
  if ((u & 0x7f800000u) == 0x7f800000u) return (u >> 16) | ((u & 0x007fffffu) ? 0x40u : 0u);
  return (u + (r16 & 0xffffu)) >> 16;
}
__device__ __forceinline__ float bf16_bits_to_f32(uint32_t b) { return __uint_as_float(b << 16); }

// ---- storage traits ---------------------------------------------------------------
// A lane moves one 16-byte vector of a factor row: 4 fp32 or 8 bf16 values.
template <typename Store>
struct Vec;
template <>
struct Vec<float> {
  static constexpr int E = 4;
};
template <>
struct Vec<__nv_bfloat16> {
  static constexpr int E = 8;
};

template <typename Store>
__device__ __forceinline__ void load_vec(const Store* row, int v, float (&x)[Vec<Store>::E]);
template <>
__device__ __forceinline__ void load_vec<float>(const float* row, int v, float (&x)[4]) {
  const float4 q = reinterpret_cast<const float4*>(row)[v];
  x[0] = q.x; x[1] = q.y; x[2] = q.z; x[3] = q.w;
}
template <>
__device__ __forceinline__ void load_vec<__nv_bfloat16>(const __nv_bfloat16* row, int v, float (&x)[8]) {
  const uint4 q = reinterpret_cast<const uint4*>(row)[v];
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    x[2 * i] = __uint_as_float(w[i] << 16);
    x[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}
// L2-only (coherent) variants for data that other workers hand over (H rows).
template <typename Store>
__device__ __forceinline__ void load_vec_cg(const Store* row, int v, float (&x)[Vec<Store>::E]);
template <>
__device__ __forceinline__ void load_vec_cg<float>(const float* row, int v, float (&x)[4]) {
  const float4 q = __ldcg(reinterpret_cast<const float4*>(row) + v);
  x[0] = q.x; x[1] = q.y; x[2] = q.z; x[3] = q.w;
}
template <>
__device__ __forceinline__ void load_vec_cg<__nv_bfloat16>(const __nv_bfloat16* row, int v, float (&x)[8]) {
  const uint4 q = __ldcg(reinterpret_cast<const uint4*>(row) + v);
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    x[2 * i] = __uint_as_float(w[i] << 16);
    x[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}

// Store a vector; bf16 uses stochastic rounding keyed by `key` (lane-distinct).
template <typename Store, bool CG>
__device__ __forceinline__ void store_vec(Store* row, int v, const float (&x)[Vec<Store>::E], uint32_t key);
template <>
__device__ __forceinline__ void store_vec<float, false>(float* row, int v, const float (&x)[4], uint32_t) {
  reinterpret_cast<float4*>(row)[v] = make_float4(x[0], x[1], x[2], x[3]);
}
template <>
__device__ __forceinline__ void store_vec<float, true>(float* row, int v, const float (&x)[4], uint32_t) {
  __stcg(reinterpret_cast<float4*>(row) + v, make_float4(x[0], x[1], x[2], x[3]));
}
__device__ __forceinline__ uint4 pack_bf16_sr(const float (&x)[8], uint32_t key) {
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t r = hash32(key + static_cast<uint32_t>(i));
    const uint32_t lo = f32_to_bf16_sr_bits(x[2 * i], r);
    const uint32_t hi = f32_to_bf16_sr_bits(x[2 * i + 1], r >> 16);
    w[i] = (lo & 0xffffu) | (hi << 16);
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}
template <>
__device__ __forceinline__ void store_vec<__nv_bfloat16, false>(__nv_bfloat16* row, int v, const float (&x)[8], uint32_t key) {
  reinterpret_cast<uint4*>(row)[v] = pack_bf16_sr(x, key);
}
template <>
__device__ __forceinline__ void store_vec<__nv_bfloat16, true>(__nv_bfloat16* row, int v, const float (&x)[8], uint32_t key) {
  __stcg(reinterpret_cast<uint4*>(row) + v, pack_bf16_sr(x, key));
}

__device__ __forceinline__ float warp_allreduce(float v, int width) {
  for (int s = width >> 1; s >= 1; s >>= 1) v += __shfl_xor_sync(kFull, v, s);
  return v;
}

}  // namespace nd
