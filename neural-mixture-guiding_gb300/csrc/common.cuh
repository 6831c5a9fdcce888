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

NMG_HD int ceil_div(long a, long b) { return int((a + b - 1) / b); }

}  // namespace nmg
