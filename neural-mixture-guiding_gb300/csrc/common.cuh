// common.cuh -- small device/host helpers shared by every kernel file.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#define NMG_PI 3.14159265358979323846f
#define NMG_TWO_PI 6.28318530717958647693f
#define NMG_INV_PI 0.318309886183790671538f
#define NMG_INV_2PI 0.15915494309189533577f
#define NMG_INV_4PI 0.07957747154594766788f
#define NMG_EPS 1e-5f

#define NMG_HD __host__ __device__ __forceinline__
#define NMG_D __device__ __forceinline__

namespace nmg {

struct f3 {
  float x, y, z;
};
NMG_HD f3 mk(float x, float y, float z) { return f3{x, y, z}; }
NMG_HD float dot3(f3 a, f3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
NMG_HD f3 cross3(f3 a, f3 b) { return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
NMG_HD f3 scale3(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
NMG_HD f3 add3(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
NMG_D f3 normalize3(f3 a) {
  float n2 = dot3(a, a);
  if (n2 > 0.f) {
    float n = sqrtf(n2);
    return f3{a.x / n, a.y / n, a.z / n};
  }
  return a;
}

NMG_D f3 load3(const float* p, long i) { return f3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
NMG_D void store3(float* p, long i, f3 v) {
  p[3 * i] = v.x;
  p[3 * i + 1] = v.y;
  p[3 * i + 2] = v.z;
}

// store3 by a warp whose lane i holds row q0 + i (q0 a multiple of 32).
// When all 32 lanes arrive together with valid rows and p is 16-byte
// aligned, the warp's 96 floats go out as 24 float4, each gathered from its
// owning lanes by shuffles, instead of three 4-byte stores per lane at a
// 12-byte stride: every 32-byte sector is written whole, with a third of
// the L2 write requests, and as whole sectors across the host link when p
// is mapped host memory. Otherwise (a partial last tile, lanes that left
// after a failed wait) each valid lane stores its own row.
NMG_D void store3_warp(float* p, long q, f3 v, bool valid) {
  const unsigned act = __activemask();
  const unsigned all = __ballot_sync(act, valid);
  const int lane = threadIdx.x & 31;
  if (act != 0xffffffffu || all != 0xffffffffu || (reinterpret_cast<uintptr_t>(p) & 15u) != 0u) {
    if (valid) store3(p, q, v);
    return;
  }
  float o[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int e = 4 * lane + j;      // float e of the warp's 96 (lanes 24..31 gather nothing they store)
    const int src = (e / 3) & 31, c = e % 3;
    const float x = __shfl_sync(0xffffffffu, v.x, src);
    const float y = __shfl_sync(0xffffffffu, v.y, src);
    const float z = __shfl_sync(0xffffffffu, v.z, src);
    o[j] = c == 0 ? x : (c == 1 ? y : z);
  }
  if (lane < 24) reinterpret_cast<float4*>(p + 3 * (q - lane))[lane] = make_float4(o[0], o[1], o[2], o[3]);
}

NMG_HD int ceil_div(long a, long b) { return int((a + b - 1) / b); }

}  // namespace nmg
