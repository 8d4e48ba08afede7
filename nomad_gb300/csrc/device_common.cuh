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
// A lane moves one vector of 4 values of a factor row: 16 bytes of fp32 or 8 bytes of
// bf16 ("Raw" is the packed form kept in registers while a row is in flight).
template <typename Store>
struct Vec;
template <>
struct Vec<float> {
  static constexpr int E = 4;
  using Raw = uint4;
};
template <>
struct Vec<__nv_bfloat16> {
  static constexpr int E = 4;
  using Raw = uint2;
};

__device__ __forceinline__ void unpack(const uint4& q, float (&x)[4]) {
  x[0] = __uint_as_float(q.x); x[1] = __uint_as_float(q.y);
  x[2] = __uint_as_float(q.z); x[3] = __uint_as_float(q.w);
}
__device__ __forceinline__ void unpack(const uint2& q, float (&x)[4]) {
  x[0] = __uint_as_float(q.x << 16); x[1] = __uint_as_float(q.x & 0xffff0000u);
  x[2] = __uint_as_float(q.y << 16); x[3] = __uint_as_float(q.y & 0xffff0000u);
}
template <typename Raw>
__device__ __forceinline__ Raw zero_raw();
template <>
__device__ __forceinline__ uint4 zero_raw<uint4>() { return make_uint4(0u, 0u, 0u, 0u); }
template <>
__device__ __forceinline__ uint2 zero_raw<uint2>() { return make_uint2(0u, 0u); }

// Stochastic-rounding key of a factor row written during one visit: distinct rows and
// visits give distinct keys; the hash of key + vector index supplies the random bits.
__device__ __forceinline__ uint32_t row_key(int row, uint32_t colkey) {
  return static_cast<uint32_t>(row) * 0x9E3779B1u ^ colkey;
}

// fp32 values to the stored form; bf16 uses stochastic rounding keyed by `key`
// (the caller makes keys distinct per row, update and vector).  One hash per vector: its
// two halves round the first two values, and the high halves of its products with two
// odd constants (bijections of the hash, so again uniform) round the other two.  The
// bits of one vector are correlated, which leaves each value's rounding unbiased.
__device__ __forceinline__ uint4 pack_raw(const float (&x)[4], uint32_t, uint4*) {
  return make_uint4(__float_as_uint(x[0]), __float_as_uint(x[1]), __float_as_uint(x[2]),
                    __float_as_uint(x[3]));
}
// Two bf16 values with stochastic rounding in one instruction: cvt.rs rounds the upper
// element with rbits[31:16] and the lower with rbits[15:0], each as (bits(x) + r16) >> 16
// -- the rule of f32_to_bf16_sr_bits for finite x (tests/test_sr_convert.py checks the
// two on 2^20 random pairs); non-finite inputs saturate to the largest finite value.
__device__ __forceinline__ uint32_t bf16x2_sr(float lo, float hi, uint32_t rbits) {
  uint32_t d;
  asm("cvt.rs.satfinite.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
  return d;
}
// Random bits per vector: one hash; value 0 takes r0[15:0], value 1 r0[31:16], value 2
// r1[31:16] and value 3 r2[31:16] (r1, r2 odd multiples of r0).
__device__ __forceinline__ uint2 pack_raw(const float (&x)[4], uint32_t key, uint2*) {
  const uint32_t r0 = hash32(key);
  const uint32_t r1 = r0 * 0x9E3779B1u, r2 = r0 * 0x85EBCA77u;
  return make_uint2(bf16x2_sr(x[0], x[1], r0), bf16x2_sr(x[2], x[3], __byte_perm(r1, r2, 0x7632)));
}

template <typename Store>
__device__ __forceinline__ void load_vec(const Store* row, int v, float (&x)[4]) {
  using Raw = typename Vec<Store>::Raw;
  unpack(reinterpret_cast<const Raw*>(row)[v], x);
}
// L2-only (coherent) load for data other workers hand over (H rows).
template <typename Store>
__device__ __forceinline__ void load_vec_cg(const Store* row, int v, float (&x)[4]) {
  using Raw = typename Vec<Store>::Raw;
  unpack(__ldcg(reinterpret_cast<const Raw*>(row) + v), x);
}
template <typename Store, bool CG>
__device__ __forceinline__ void store_vec(Store* row, int v, const float (&x)[4], uint32_t key) {
  using Raw = typename Vec<Store>::Raw;
  const Raw q = pack_raw(x, key, static_cast<Raw*>(nullptr));
  if (CG)
    __stcg(reinterpret_cast<Raw*>(row) + v, q);
  else
    reinterpret_cast<Raw*>(row)[v] = q;
}

__device__ __forceinline__ float warp_allreduce(float v, int width) {
  for (int s = width >> 1; s >= 1; s >>= 1) v += __shfl_xor_sync(kFull, v, s);
  return v;
}

}  // namespace nd
