// Checks the hardware stochastic-rounding convert used for bf16 write-back
// (cvt.rs.satfinite.bf16x2.f32, as in nomad_gb300/csrc/device_common.cuh: bf16x2_sr)
// against the software rule it replaces: bf16 bits = (bits(x) + r16) >> 16 for finite x,
// the upper element taking rbits[31:16] and the lower rbits[15:0].  Prints the number of
// mismatching pairs; exit status 0 when there are none.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <cuda_runtime.h>

__global__ void convert(const float* x, const uint32_t* r, uint32_t* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t d;
  asm("cvt.rs.satfinite.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(x[2 * i + 1]), "f"(x[2 * i]), "r"(r[i]));
  out[i] = d;
}

static uint32_t sr(float f, uint32_t r16) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (u + (r16 & 0xffffu)) >> 16;
}

int main() {
  const int n = 1 << 20;
  uint64_t s = 0x9E3779B97F4A7C15ull;
  auto next = [&]() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return static_cast<uint32_t>(s >> 11);
  };
  float* hx = new float[2 * n];
  uint32_t* hr = new uint32_t[n];
  uint32_t* ho = new uint32_t[n];
  for (int i = 0; i < 2 * n; ++i) {
    const float m = static_cast<float>(static_cast<int>(next() % 2000001u) - 1000000) * 1e-6f;
    hx[i] = std::ldexp(m, static_cast<int>(next() % 60u) - 40);  // both signs, 2^-40 .. 2^20
  }
  for (int i = 0; i < n; ++i) hr[i] = next() ^ (next() << 16);
  float* dx = nullptr;
  uint32_t *dr = nullptr, *dout = nullptr;
  if (cudaMalloc(&dx, 8ull * n) || cudaMalloc(&dr, 4ull * n) || cudaMalloc(&dout, 4ull * n)) return 2;
  cudaMemcpy(dx, hx, 8ull * n, cudaMemcpyHostToDevice);
  cudaMemcpy(dr, hr, 4ull * n, cudaMemcpyHostToDevice);
  convert<<<(n + 255) / 256, 256>>>(dx, dr, dout, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 2;
  cudaMemcpy(ho, dout, 4ull * n, cudaMemcpyDeviceToHost);
  long bad = 0;
  for (int i = 0; i < n; ++i) {
    const uint32_t want = sr(hx[2 * i], hr[i]) | (sr(hx[2 * i + 1], hr[i] >> 16) << 16);
    bad += ho[i] != want;
  }
  std::printf("mismatches %ld of %d\n", bad, n);
  return bad == 0 ? 0 : 1;
}
