// encoding.cuh -- device code of the input featurisation and the composite
// encoding (multiresolution grid + spherical harmonics + one-blob).
//
// Semantics follow tiny-cuda-nn 1.7 as vendored by the reference
// (src/ext/tcnn/include/tiny-cuda-nn/encodings/grid.h:171-510,
// spherical_harmonics.h:46-153, oneblob.h:99-125, common_device.h:429-547)
// and the reference's featurisation (src/render/guided/train.cu:174-191).
// Per-level scales, resolutions and table offsets are computed once on the
// host (with the same expression as grid.h:195-204) and passed in
// EncodingParams, so every device evaluates the identical grid geometry.
#pragma once
#include "common.cuh"

namespace nmg {

constexpr int kMaxLevels = 24;

struct EncodingParams {
  int input_mode;     // 0: reference inputs (9 dims), 1: SH-of-normal inputs (10 dims)
  int n_input;        // 9 or 10
  int grid_hash;      // 0 dense, 1 hash
  int levels, feats;  // grid levels, features per level
  int smoothstep;     // interpolation: 0 linear, 1 smoothstep
  int sh_degree;      // 1..4 (d^2 outputs)
  int oneblob_bins;   // bins per one-blob dimension
  int n_enc;          // encoded width before padding
  int n_enc_pad;      // padded to a multiple of 16 with 1.0 (oneblob.h:206-209)
  float scale[kMaxLevels];
  uint32_t res[kMaxLevels];
  uint32_t offset[kMaxLevels + 1];  // level start, in table entries
  float aabb[6];
  float center[3];  // centre of the inflated box
  float inv_size[3];  // 1 / size of the inflated box
};

// grid.h:171-187 with the coherent-prime hash (grid.h:132-135).
NMG_D uint32_t grid_index(int hash, uint32_t T, uint32_t res, uint32_t x, uint32_t y, uint32_t z) {
  uint32_t stride = 1, index = 0;
  const uint32_t p[3] = {x, y, z};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (stride <= T) {
      index += p[d] * stride;
      stride *= res;
    }
  }
  if (hash && T < stride) index = (x * 1u) ^ (y * 2654435761u) ^ (z * 805459861u);
  return index % T;
}

// common_device.h:484-495 (pos_fract) without FMA contraction so the cell
// index matches the host computation bit for bit.
NMG_D f3 unit3f(f3 a) {
  const float n2 = dot3(a, a);
  if (!(n2 > 0.f)) return a;
  const float r = rsqrtf(n2);
  return f3{a.x * r, a.y * r, a.z * r};
}

NMG_D void pos_fract(float x, float scale, int smooth, float* w, uint32_t* g) {
  float p = __fadd_rn(__fmul_rn(x, scale), 0.5f);
  float fl = floorf(p);
  *g = uint32_t(int(fl));
  float f = p - fl;
  *w = smooth ? f * f * (3.f - 2.f * f) : f;
}

// Corner c of the level's cell around `pos`: entry index into the table and
// trilinear weight.
struct Corners {
  uint32_t g[3];
  float w[3];
};

NMG_D void level_cell(const EncodingParams& e, int l, const float* pos, Corners& c) {
#pragma unroll
  for (int d = 0; d < 3; ++d) pos_fract(pos[d], e.scale[l], e.smoothstep, &c.w[d], &c.g[d]);
}

NMG_D void corner(const EncodingParams& e, int l, const Corners& c, int k, uint32_t* entry, float* weight) {
  float wt = 1.f;
  uint32_t p[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if ((k & (1 << d)) == 0) {
      wt *= 1.f - c.w[d];
      p[d] = c.g[d];
    } else {
      wt *= c.w[d];
      p[d] = c.g[d] + 1;
    }
  }
  const uint32_t T = e.offset[l + 1] - e.offset[l];
  *entry = e.offset[l] + grid_index(e.grid_hash, T, e.res[l], p[0], p[1], p[2]);
  *weight = wt;
}

// spherical_harmonics.h:46-85: real SH basis of (x, y, z) up to degree 4.
NMG_D void sh_basis(int degree, float x, float y, float z, float* o) {
  float xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
  o[0] = 0.28209479177387814f;
  if (degree <= 1) return;
  o[1] = -0.48860251190291987f * y;
  o[2] = 0.48860251190291987f * z;
  o[3] = -0.48860251190291987f * x;
  if (degree <= 2) return;
  o[4] = 1.0925484305920792f * xy;
  o[5] = -1.0925484305920792f * yz;
  o[6] = 0.94617469575755997f * z2 - 0.31539156525251999f;
  o[7] = -1.0925484305920792f * xz;
  o[8] = 0.54627421529603959f * x2 - 0.54627421529603959f * y2;
  if (degree <= 3) return;
  o[9] = 0.59004358992664352f * y * (-3.0f * x2 + y2);
  o[10] = 2.8906114426405538f * xy * z;
  o[11] = 0.45704579946446572f * y * (1.0f - 5.0f * z2);
  o[12] = 0.3731763325901154f * z * (5.0f * z2 - 3.0f);
  o[13] = 0.45704579946446572f * x * (1.0f - 5.0f * z2);
  o[14] = 1.4453057213202769f * z * (x2 - y2);
  o[15] = 0.59004358992664352f * x * (-x2 + 3.0f * y2);
}

// common_device.h:543-547 and oneblob.h:99-125: one-blob of x into n bins
// with the quartic kernel wrapped around +-1.
NMG_D float quartic_cdf(float x, float inv_r) {
  float u = x * inv_r, u2 = u * u, u4 = u2 * u2;
  return fmaxf(0.f, fminf(1.f, (15.f / 16.f) * u * (1.f - (2.f / 3.f) * u2 + (1.f / 5.f) * u4) + 0.5f));
}
NMG_D void oneblob(int n_bins, float x, float* o) {
  const float nb = float(n_bins);
  float left = quartic_cdf(-x, nb) + quartic_cdf(-x - 1.f, nb) + quartic_cdf(-x + 1.f, nb);
  for (int k = 0; k < n_bins; ++k) {
    float rb = float(k + 1) / nb;
    float right = quartic_cdf(rb - x, nb) + quartic_cdf(rb - x - 1.f, nb) + quartic_cdf(rb - x + 1.f, nb);
    o[k] = right - left;
    left = right;
  }
}

// Non-grid part of the composite encoding of one input row, written to
// out[0 .. n_enc_pad - L*F): SH(wo) | OneBlob(x6..x8) or SH(wo) | SH(n) |
// OneBlob(x9), then 1.0 padding.
NMG_D void encode_directional(const EncodingParams& e, const float* x, float* out) {
  const int d2 = e.sh_degree * e.sh_degree;
  int o = 0;
  sh_basis(e.sh_degree, x[3] * 2.f - 1.f, x[4] * 2.f - 1.f, x[5] * 2.f - 1.f, out + o);
  o += d2;
  if (e.input_mode == 0) {
    for (int d = 6; d < 9; ++d) {
      oneblob(e.oneblob_bins, x[d], out + o);
      o += e.oneblob_bins;
    }
  } else {
    sh_basis(e.sh_degree, x[6] * 2.f - 1.f, x[7] * 2.f - 1.f, x[8] * 2.f - 1.f, out + o);
    o += d2;
    oneblob(e.oneblob_bins, x[9], out + o);
    o += e.oneblob_bins;
  }
  for (int k = e.levels * e.feats + o; k < e.n_enc_pad; ++k) out[o++] = 1.f;
}

// normalizeSpatialCoord (train.h:173-177) one IEEE operation at a time in the
// reference's order, without contraction into fused multiply-adds, so that the
// result equals the reference's FP32 value bit for bit: the box is inflated by
// 0.005 x its diagonal's length (Eigen sums the squares as x^2 + (y^2 + z^2)),
// then 0.5 + (p - centre) / diagonal per axis.
NMG_D float aabb_inflation(const float* aabb) {
  const float dx = __fsub_rn(aabb[3], aabb[0]), dy = __fsub_rn(aabb[4], aabb[1]), dz = __fsub_rn(aabb[5], aabb[2]);
  const float n2 = __fadd_rn(__fmul_rn(dx, dx), __fadd_rn(__fmul_rn(dy, dy), __fmul_rn(dz, dz)));
  return __fmul_rn(__fsqrt_rn(n2), 0.005f);
}
NMG_D float normalize_coord(const float* aabb, float infl, int k, float p) {
  const float lo = __fsub_rn(aabb[k], infl), hi = __fadd_rn(aabb[k + 3], infl);
  const float ctr = __fdiv_rn(__fadd_rn(lo, hi), 2.f);
  return __fadd_rn(0.5f, __fdiv_rn(__fsub_rn(p, ctr), __fsub_rn(hi, lo)));
}

// train.cu:174-191 (mode 0) / SH-of-normal variant (mode 1): shading data ->
// network input row x[n_input]. The box is inflated by 0.5% of its diagonal
// (train.h:173-177).
// FAST = true uses the box centre / inverse size precomputed on the host
// and rsqrt normalisation (the fused path); FAST = false evaluates the
// reference's expressions literally (the FP32 path).
template <bool FAST = false>
NMG_D void featurize(const EncodingParams& e, f3 pos, f3 wo, f3 n, float rough, float* x) {
  const float p[3] = {pos.x, pos.y, pos.z};
  if (FAST) {
#pragma unroll
    for (int d = 0; d < 3; ++d) x[d] = 0.5f + (p[d] - e.center[d]) * e.inv_size[d];
  } else {
    const float infl = aabb_inflation(e.aabb);
#pragma unroll
    for (int d = 0; d < 3; ++d) x[d] = normalize_coord(e.aabb, infl, d, p[d]);
  }
  f3 w = FAST ? unit3f(wo) : normalize3(wo);
  x[3] = (w.x + 1.f) * 0.5f;
  x[4] = (w.y + 1.f) * 0.5f;
  x[5] = (w.z + 1.f) * 0.5f;
  f3 nn = FAST ? unit3f(n) : normalize3(n);
  if (e.input_mode == 0) {
    float th = acosf(fminf(1.f, fmaxf(-1.f, nn.z)));
    float ph = atan2f(nn.y, nn.x);
    if (ph < 0.f) ph += NMG_TWO_PI;
    x[6] = float(double(th) / 3.14159265358979323846);
    x[7] = ph / NMG_TWO_PI;
    x[8] = 1.f - expf(-rough);
  } else {
    x[6] = (nn.x + 1.f) * 0.5f;
    x[7] = (nn.y + 1.f) * 0.5f;
    x[8] = (nn.z + 1.f) * 0.5f;
    x[9] = 1.f - expf(-rough);
  }
}

}  // namespace nmg
