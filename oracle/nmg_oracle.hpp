// nmg_oracle.hpp -- CPU oracle for the neural parametric mixture guiding step.
//
// TEST INFRASTRUCTURE ONLY. This file restates, on the host, the arithmetic of
// the reference's guiding step so that the GPU kernels can be checked against
// it. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
// load it; the product path never does.
//
// Every function is templated on the scalar type S:
//   * S = float  follows the reference's FP32 operation order (same sequential
//     sums, same clamps, same constants written as float literals) so that it
//     can be compared bit-for-bit with the reference's own host build
//     (oracle/ref_shim.cu, built by oracle/build_ref.sh);
//   * S = double is the FP64 oracle used for tolerance checks of the GPU path.
// Two switches select between the reference's formula and the exact one where
// they differ: Opts::kappa_poly (the kappa<1 polynomial of
// distribution.h:165-166 vs the exact 1/k - coth k) and Opts::expm1_norm (the
// 1-exp(-2k) normaliser of vmf.h:25-26 vs -expm1(-2k)).
//
// Reference files are cited relative to the reference project's root;
// "tcnn/" abbreviates src/ext/tcnn/ (tiny-cuda-nn 1.7, vendored).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>

namespace nmgo {

// ---------------------------------------------------------------- constants
// krrmath/constants.h:16-25 (float literals in the reference).
template <class S> struct C;
template <> struct C<float> {
  static constexpr float PI = 3.14159265358979323846f;
  static constexpr float TWO_PI = 6.28318530717958647693f;
  static constexpr float INV_PI = 0.318309886183790671538f;
  static constexpr float INV_2PI = 0.15915494309189533577f;
  static constexpr float INV_4PI = 0.07957747154594766788f;
  static constexpr float EPS = 1e-5f;  // M_EPSILON
};
template <> struct C<double> {
  static constexpr double PI = 3.14159265358979323846;
  static constexpr double TWO_PI = 6.28318530717958647693;
  static constexpr double INV_PI = 0.318309886183790671538;
  static constexpr double INV_2PI = 0.15915494309189533577;
  static constexpr double INV_4PI = 0.07957747154594766788;
  static constexpr double EPS = 1e-5;
};

// Math functions: float uses the C library's single-precision entry points,
// which is what the reference's host build calls (std::sin(float) -> sinf ...).
inline float xexp(float x) { return expf(x); }
inline double xexp(double x) { return std::exp(x); }
inline float xlog(float x) { return logf(x); }
inline double xlog(double x) { return std::log(x); }
inline float xlog1p(float x) { return log1pf(x); }
inline double xlog1p(double x) { return std::log1p(x); }
inline float xexpm1(float x) { return expm1f(x); }
inline double xexpm1(double x) { return std::expm1(x); }
inline float xsin(float x) { return sinf(x); }
inline double xsin(double x) { return std::sin(x); }
inline float xcos(float x) { return cosf(x); }
inline double xcos(double x) { return std::cos(x); }
inline float xacos(float x) { return acosf(x); }
inline double xacos(double x) { return std::acos(x); }
inline float xatan2(float y, float x) { return atan2f(y, x); }
inline double xatan2(double y, double x) { return std::atan2(y, x); }
inline float xsqrt(float x) { return sqrtf(x); }
inline double xsqrt(double x) { return std::sqrt(x); }

template <class S> struct V3 {
  S x, y, z;
  S operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

// Eigen's fixed-size-3 reductions unroll as v0 + (v1 + v2); krrmath's dot,
// squaredNorm and mean inherit that order (Eigen redux_novec_unroller).
template <class S> inline S dot(V3<S> a, V3<S> b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
template <class S> inline S norm(V3<S> a) { return xsqrt(dot(a, a)); }
template <class S> inline V3<S> normalized(V3<S> a) {
  S n2 = dot(a, a);
  if (n2 > S(0)) {
    S n = xsqrt(n2);
    return {a.x / n, a.y / n, a.z / n};
  }
  return a;
}
template <class S> inline V3<S> cross(V3<S> a, V3<S> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// util/math_utils.h:191-201
template <class S> inline V3<S> sph_to_cart(S theta, S phi) {
  S st = xsin(theta), ct = xcos(theta), sp = xsin(phi), cp = xcos(phi);
  return {st * cp, st * sp, ct};
}
// util/math_utils.h:176-183
template <class S> inline void cart_to_sph(V3<S> v, S* theta, S* phi) {
  V3<S> vn = normalized(v);
  *theta = xacos(vn.z);
  *phi = xatan2(vn.y, vn.x);
  if (*phi < S(0)) *phi += C<S>::TWO_PI;
}

// util/math_utils.h:141-151 (branchless axis pick) and core/raytracing.h:35-49
template <class S> inline V3<S> perpendicular(V3<S> u) {
  S ax = std::fabs(u.x), ay = std::fabs(u.y), az = std::fabs(u.z);
  uint32_t uyx = (ax - ay) < 0 ? 1u : 0u;
  uint32_t uzx = (ax - az) < 0 ? 1u : 0u;
  uint32_t uzy = (ay - az) < 0 ? 1u : 0u;
  uint32_t xm = uyx & uzx;
  uint32_t ym = (1u ^ xm) & uzy;
  uint32_t zm = 1u ^ (xm | ym);
  return normalized(cross(u, V3<S>{S(xm), S(ym), S(zm)}));
}
template <class S> inline V3<S> frame_to_world(V3<S> n, V3<S> v) {
  V3<S> t = perpendicular(n);
  V3<S> b = normalized(cross(n, t));
  return {t.x * v.x + b.x * v.y + n.x * v.z, t.y * v.x + b.y * v.y + n.y * v.z,
          t.z * v.x + b.z * v.y + n.z * v.z};
}

// render/sampling.h:32-37
template <class S> inline V3<S> uniform_sphere(S u0, S u1) {
  S z = S(1) - S(2) * u0;
  S r = xsqrt(std::max(S(0), S(1) - z * z));
  S phi = C<S>::TWO_PI * u1;
  return {r * xcos(phi), r * xsin(phi), z};
}

struct Opts {
  int kappa_poly = 1;   // 1: distribution.h:165-166 polynomial for kappa<1; 0: exact
  int expm1_norm = 0;   // 1: vMF normaliser via -expm1(-2k); 0: 1-exp(-2k) (vmf.h:25-26)
  int kappa_softplus = 0;  // 1: kappa = log(1+e^x) (train.h:398); 0: exp(clamp) (train.h:243-244)
  int half_grad = 0;    // 1: round the gradient to binary16 where the reference stores __half
};

// vmf.h:22-27 -- pdf of a vMF lobe at cos(angle to the mean).
template <class S> inline S vmf_eval(S kappa, S cos_t, const Opts& o) {
  if (kappa < C<S>::EPS) return C<S>::INV_4PI;
  S den = o.expm1_norm ? -xexpm1(S(-2) * kappa) : (S(1) - xexp(S(-2) * kappa));
  return xexp(kappa * std::min(S(0), cos_t - S(1))) * kappa / (C<S>::TWO_PI * den);
}

// vmf.h:48-57 -- sample around +z.
template <class S> inline V3<S> vmf_sample_local(S kappa, S u0, S u1) {
  if (kappa < C<S>::EPS) return uniform_sphere(u0, u1);
  S cos_t = S(1) + xlog1p(-u0 + xexp(S(-2) * kappa) * u0) / kappa;
  S sin_t = xsqrt(std::max(S(0), S(1) - cos_t * cos_t));
  S phi = C<S>::TWO_PI * u1;
  S sp = xsin(phi), cp = xcos(phi);
  return {cp * sin_t, sp * sin_t, cos_t};
}

// train.h:391-415 (tcnn/common_device.h:51 logistic).
template <class S> inline S logistic(S x) { return S(1) / (S(1) + xexp(-x)); }
template <class S> inline S act_exp(S x) { return xexp(std::min(std::max(x, S(-10)), S(15))); }
// FP32 follows train.h:398 literally (log(1+e^x)); FP64 uses the stable form.
inline float act_softplus(float x) { return logf(1.0f + expf(x)); }
inline double act_softplus(double x) { return std::max(x, 0.0) + std::log1p(std::exp(-std::fabs(x))); }
template <class S> inline S dact_softplus(S x) { S e = xexp(x); return e / (e + S(1)); }
template <class S> inline S dact_logistic(S x) { S f = logistic(x); return f * (S(1) - f); }

template <class S> struct Lobe { S lambda, kappa, theta, phi; };

// The K-lobe mixture: distribution.h:75-202.
template <class S> struct Mixture {
  int K = 0;
  Lobe<S> sg[32];
  S weight[32];
  S total = 0;

  // distribution.h:85-98 -- activation of the raw network outputs.
  void activate(const S* raw, int K_, const Opts& o) {
    K = K_;
    total = 0;
    for (int i = 0; i < K; ++i) {
      const S* r = raw + 4 * i;
      sg[i].lambda = act_exp(r[0]);
      sg[i].kappa = o.kappa_softplus ? act_softplus(r[1]) : act_exp(r[1]);
      sg[i].theta = C<S>::PI * logistic(r[2]);
      sg[i].phi = C<S>::TWO_PI * logistic(r[3]);
      total += sg[i].lambda;
    }
    for (int i = 0; i < K; ++i) weight[i] = sg[i].lambda / total;
  }

  S lobe_pdf(int i, V3<S> wi, const Opts& o) const {  // distribution.h:35-37
    return vmf_eval(sg[i].kappa, dot(wi, sph_to_cart(sg[i].theta, sg[i].phi)), o);
  }

  S pdf(V3<S> wi, const Opts& o) const {  // distribution.h:113-119
    S p = 0;
    for (int i = 0; i < K; ++i) p += weight[i] * lobe_pdf(i, wi, o);
    return p;
  }

  // distribution.h:132-140 -- sequential CDF subtraction, falling back to lobe 0.
  int select(S u) const {
    for (int i = 0; i < K; ++i) {
      if (u < weight[i]) return i;
      u -= weight[i];
    }
    return 0;
  }

  // vmf.h:67-71
  V3<S> sample_lobe(int i, S u0, S u1) const {
    V3<S> d = vmf_sample_local(sg[i].kappa, u0, u1);
    return frame_to_world(sph_to_cart(sg[i].theta, sg[i].phi), d);
  }

  V3<S> sample(S u_lobe, S u0, S u1, int* lobe) const {
    int i = select(u_lobe);
    if (lobe) *lobe = i;
    return sample_lobe(i, u0, u1);
  }

  // distribution.h:39-64 -- product of lobe i with another vMF lobe.
  static S prod_norm(S k) {
    return k < S(1e-3) ? C<S>::INV_4PI : k * C<S>::INV_2PI / (S(1) - xexp(S(-2) * k));
  }
  void product(int i, const Lobe<S>& other) {
    Lobe<S>& a = sg[i];
    V3<S> mu_a = sph_to_cart(a.theta, a.phi), mu_b = sph_to_cart(other.theta, other.phi);
    V3<S> nm = {mu_a.x * a.kappa + mu_b.x * other.kappa, mu_a.y * a.kappa + mu_b.y * other.kappa,
                mu_a.z * a.kappa + mu_b.z * other.kappa};
    S nk = norm(nm);
    if (nk >= S(1e-3)) {
      nm = {nm.x / nk, nm.y / nk, nm.z / nk};
    } else {
      nk = 0;
      nm = mu_a;
    }
    S th, ph;
    cart_to_sph(nm, &th, &ph);
    S e = xexp(a.kappa * (dot(nm, mu_a) - S(1)) + other.kappa * (dot(nm, mu_b) - S(1)));
    S s = prod_norm(a.kappa) * prod_norm(other.kappa) / prod_norm(nk) * e;
    a.lambda = s * a.lambda * other.lambda;
    a.kappa = nk;
    a.theta = th;
    a.phi = ph;
  }

  // distribution.h:184-195 -- multiply by the cosine lobe around `normal`.
  void apply_cosine_lobe(V3<S> normal) {
    S th, ph;
    cart_to_sph(normal, &th, &ph);
    Lobe<S> cl{S(1), S(2.18853f), th, ph};
    total = 0;
    for (int i = 0; i < K; ++i) {
      product(i, cl);
      total += sg[i].lambda;
    }
    total = std::max(total, C<S>::EPS);
    for (int i = 0; i < K; ++i) weight[i] = sg[i].lambda / total;
  }

  // distribution.h:144-181 -- mixture probability and its gradient with
  // respect to the activated parameters (lambda, kappa, theta, phi) per lobe.
  S gradients_probability(V3<S> wi, S* out, const Opts& o) const {
    S x = wi.x, y = wi.y, z = wi.z;
    S prob = 0;
    for (int s = 0; s < K; ++s) {
      S lambda = sg[s].lambda, kappa = sg[s].kappa, theta = sg[s].theta, phi = sg[s].phi;
      S vmf = lobe_pdf(s, wi, o);
      prob += weight[s] * vmf;
      S dl = vmf * (total - lambda) / (total * total);
      for (int k = 0; k < K; ++k)
        if (k != s) dl -= weight[k] / total * lobe_pdf(k, wi, o);
      S ik;
      if (o.kappa_poly && kappa < S(1)) {
        ik = S(0.000926f) + S(-0.344883f) * kappa + S(0.030147f) * (kappa * kappa);
      } else if (!o.kappa_poly && kappa < S(1e-4)) {
        ik = -kappa / S(3);  // series of 1/k - coth k near 0
      } else {
        ik = S(1) / kappa - (S(1) + xexp(S(-2) * kappa)) / (S(1) - xexp(S(-2) * kappa));
      }
      S st = xsin(theta), ct = xcos(theta), sp = xsin(phi), cp = xcos(phi);
      S dk = weight[s] * vmf * (x * st * cp + y * st * sp + z * ct + ik);
      S dt = weight[s] * vmf * kappa * (ct * (x * cp + y * sp) - z * st);
      S dp = weight[s] * vmf * kappa * (y * cp - x * sp) * st;
      out[4 * s + 0] = dl;
      out[4 * s + 1] = dk;
      out[4 * s + 2] = dt;
      out[4 * s + 3] = dp;
    }
    return prob;
  }
};

// binary16 round-trip (round to nearest even), used where the reference
// stores intermediate gradients as __half (train.cu:81-103, F8).
inline float to_half_and_back(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  uint32_t sign = x & 0x80000000u;
  float a = std::fabs(f);
  if (std::isnan(f)) return f;
  if (a >= 65520.0f) {  // overflows to inf
    uint32_t r = sign | 0x7f800000u;
    float out;
    std::memcpy(&out, &r, 4);
    return out;
  }
  if (a < 6.103515625e-05f) {  // subnormal half: quantum 2^-24
    float q = std::nearbyint(a * 16777216.0f) / 16777216.0f;
    return sign ? -q : q;
  }
  uint32_t ax = x & 0x7fffffffu;
  uint32_t lsb = (ax >> 13) & 1u;
  ax += 0xfffu + lsb;
  ax &= 0xffffe000u;
  uint32_t r = sign | ax;
  float out;
  std::memcpy(&out, &r, 4);
  return out;
}
// Direct double -> binary16 rounding (round to nearest even), as __half's
// constructor from double does.
inline double half_from_double(double d) {
  if (std::isnan(d)) return d;
  double a = std::fabs(d);
  if (a >= 65520.0) return d > 0 ? INFINITY : -INFINITY;
  int e;
  std::frexp(a, &e);                 // a = m * 2^e, m in [0.5, 1)
  int q = std::max(e - 11, -24);     // quantum exponent: 11 significant bits, subnormal floor 2^-24
  double r = std::nearbyint(std::ldexp(a, -q));
  r = std::ldexp(r, q);
  return d < 0 ? -r : r;
}
template <class S> inline S maybe_half(S v, const Opts& o) {
  if (!o.half_grad) return v;
  return S(to_half_and_back(float(v)));
}
inline double maybe_half_d(double v, const Opts& o) { return o.half_grad ? half_from_double(v) : v; }

// `a * M_PI * d` as the reference's Linux build evaluates it: krrmath only
// defines the float M_PI when the C library has not (constants.h:15-17), and
// glibc's M_PI is a double, so the product is formed in double and rounded
// once to the __half gradient slot (train.cu:102, :163).
inline float pi_product(float a, float d, const Opts& o) {
  double v = double(a) * 3.14159265358979323846 * double(d);
  return o.half_grad ? float(half_from_double(v)) : float(v);
}
inline double pi_product(double a, double d, const Opts& o) {
  return maybe_half_d(a * C<double>::PI * d, o);
}

// train.cu:69-124 -- KL divergence loss of one training sample and the
// gradient with respect to the raw network outputs.
//   raw[K*4]: raw outputs; theta_phi: sampled direction (spherical);
//   L[3]: radiance estimate; wi_pdf: pdf the direction was drawn with;
//   loss_scale_over_n: loss scale / batch size.
// Returns the per-sample loss; writes grad[K*4].
template <class S>
inline S kl_loss_grad(const S* raw, int K, S theta, S phi, const S* L, S wi_pdf, S loss_scale_over_n,
                      S* grad, const Opts& o) {
  Mixture<S> m;
  m.activate(raw, K, o);
  V3<S> wi = sph_to_cart(theta, phi);
  S Li = (L[0] + (L[1] + L[2])) / S(3);
  S wp = wi_pdf + C<S>::EPS;
  S g[128];
  S guide = m.gradients_probability(wi, g, o);
  for (int i = 0; i < 4 * K; ++i) g[i] = maybe_half(g[i], o);
  guide += C<S>::EPS;
  S prefix = -Li / wp / guide * loss_scale_over_n;
  S loss = -Li / wp * xlog(guide);
  for (int s = 0; s < K; ++s) {
    const S* r = raw + 4 * s;
    S dk = o.kappa_softplus ? dact_softplus(r[1]) : act_exp(r[1]);
    grad[4 * s + 0] = maybe_half(prefix * g[4 * s + 0] * act_exp(r[0]), o);
    grad[4 * s + 1] = maybe_half(prefix * g[4 * s + 1] * dk, o);
    grad[4 * s + 2] = pi_product(prefix * g[4 * s + 2], dact_logistic(r[2]), o);
    grad[4 * s + 3] = maybe_half(prefix * g[4 * s + 3] * C<S>::TWO_PI * dact_logistic(r[3]), o);
  }
  for (int i = 0; i < 4 * K; ++i) {
    if (std::isnan(grad[i]) || std::isinf(grad[i])) grad[i] = 0;
    grad[i] = std::min(S(150), grad[i]);
  }
  return loss;
}

// train.cu:126-172 -- the learned-selection variant: the extra output raw[4K]
// is the logit of the probability of sampling the mixture instead of the BSDF.
template <class S>
inline S kl_loss_grad_selection(const S* raw, int K, S theta, S phi, const S* L, S bsdf_pdf,
                                S loss_scale_over_n, S* grad, const Opts& o) {
  Mixture<S> m;
  m.activate(raw, K, o);
  V3<S> wi = sph_to_cart(theta, phi);
  S Li = (L[0] + (L[1] + L[2])) / S(3);
  S sel = logistic(raw[4 * K]);
  S g[132];
  S prob = m.gradients_probability(wi, g, o);
  for (int i = 0; i < 4 * K; ++i) g[i] = maybe_half(maybe_half(g[i], o) * sel, o);
  g[4 * K] = maybe_half(prob - bsdf_pdf, o);
  S guide = prob + C<S>::EPS;
  S wp = sel * guide + (S(1) - sel) * bsdf_pdf;
  S loss = -Li / wp * xlog(wp);
  S prefix = -Li / wp / wp * loss_scale_over_n;
  for (int s = 0; s < K; ++s) {
    const S* r = raw + 4 * s;
    S dk = o.kappa_softplus ? dact_softplus(r[1]) : act_exp(r[1]);
    grad[4 * s + 0] = maybe_half(prefix * g[4 * s + 0] * act_exp(r[0]), o);
    grad[4 * s + 1] = maybe_half(prefix * g[4 * s + 1] * dk, o);
    grad[4 * s + 2] = pi_product(prefix * g[4 * s + 2], dact_logistic(r[2]), o);
    grad[4 * s + 3] = maybe_half(prefix * g[4 * s + 3] * C<S>::TWO_PI * dact_logistic(r[3]), o);
  }
  grad[4 * K] = maybe_half(S(0.01f) * prefix * g[4 * K] * dact_logistic(raw[4 * K]), o);
  return loss;
}

// ------------------------------------------------------------------ encodings
// tcnn/include/tiny-cuda-nn/encodings/grid.h:195-204
inline float grid_scale(uint32_t level, float log2_scale, uint32_t base_res) {
  return exp2f(float(level) * log2_scale) * float(base_res) - 1.0f;
}
inline uint32_t grid_resolution(float scale) { return uint32_t(ceilf(scale)) + 1u; }

struct GridSpec {
  int hash = 1;            // 0 dense, 1 hash
  int levels = 16, feats = 2, log2_T = 19, base_res = 16;
  float per_level_scale = 1.447f;
  int smoothstep = 0;      // 0 linear, 1 smoothstep
  // derived
  uint32_t offset[33];     // entry offsets per level (in grid vertices)
  uint32_t n_entries = 0;  // total vertices; params = n_entries * feats
};

// grid.h:957-997 -- per-level sizes.
inline void grid_layout(GridSpec& g) {
  uint32_t off = 0;
  float l2s = std::log2(g.per_level_scale);
  for (int i = 0; i < g.levels; ++i) {
    uint32_t res = grid_resolution(grid_scale(uint32_t(i), l2s, uint32_t(g.base_res)));
    uint32_t maxp = 0xffffffffu / 2;
    uint32_t p = std::pow(float(res), 3.0f) > float(maxp) ? maxp : res * res * res;
    p = (p + 7u) / 8u * 8u;
    if (g.hash) p = std::min(p, 1u << g.log2_T);
    g.offset[i] = off;
    off += p;
  }
  g.offset[g.levels] = off;
  g.n_entries = off;
}

// grid.h:171-187 with the coherent-prime hash of grid.h:132-135.
inline uint32_t grid_index(int hash, uint32_t T, uint32_t res, const uint32_t p[3]) {
  uint32_t stride = 1, index = 0;
  for (int d = 0; d < 3 && stride <= T; ++d) {
    index += p[d] * stride;
    stride *= res;
  }
  if (hash && T < stride) index = (p[0] * 1u) ^ (p[1] * 2654435761u) ^ (p[2] * 805459861u);
  return index % T;
}

// grid.h:221-385 (forward) -- features of one position; out[levels*feats].
// S is the accumulation type; the table holds float master values.
template <class S>
inline void grid_encode(const GridSpec& g, const float* table, const float pos[3], S* out) {
  float l2s = std::log2(g.per_level_scale);
  for (int l = 0; l < g.levels; ++l) {
    float scale = grid_scale(uint32_t(l), l2s, uint32_t(g.base_res));
    uint32_t res = grid_resolution(scale);
    uint32_t T = g.offset[l + 1] - g.offset[l];
    S w[3];
    uint32_t pg[3];
    for (int d = 0; d < 3; ++d) {  // common_device.h:484-495 pos_fract
      float p = pos[d] * scale + 0.5f;
      float fl = floorf(p);
      pg[d] = uint32_t(int(fl));
      S f = S(p - fl);
      w[d] = g.smoothstep ? f * f * (S(3) - S(2) * f) : f;
    }
    for (int f = 0; f < g.feats; ++f) out[l * g.feats + f] = 0;
    for (int c = 0; c < 8; ++c) {
      S wt = 1;
      uint32_t lp[3];
      for (int d = 0; d < 3; ++d) {
        if ((c & (1 << d)) == 0) {
          wt *= S(1) - w[d];
          lp[d] = pg[d];
        } else {
          wt *= w[d];
          lp[d] = pg[d] + 1;
        }
      }
      uint32_t idx = (g.offset[l] + grid_index(g.hash, T, res, lp)) * uint32_t(g.feats);
      for (int f = 0; f < g.feats; ++f) out[l * g.feats + f] += wt * S(table[idx + f]);
    }
  }
}

// grid.h:387-510 (backward) -- scatter dL/dfeatures into the table gradient.
template <class S>
inline void grid_backward(const GridSpec& g, const float pos[3], const S* dfeat, S* grad_table) {
  float l2s = std::log2(g.per_level_scale);
  for (int l = 0; l < g.levels; ++l) {
    float scale = grid_scale(uint32_t(l), l2s, uint32_t(g.base_res));
    uint32_t res = grid_resolution(scale);
    uint32_t T = g.offset[l + 1] - g.offset[l];
    S w[3];
    uint32_t pg[3];
    for (int d = 0; d < 3; ++d) {
      float p = pos[d] * scale + 0.5f;
      float fl = floorf(p);
      pg[d] = uint32_t(int(fl));
      S f = S(p - fl);
      w[d] = g.smoothstep ? f * f * (S(3) - S(2) * f) : f;
    }
    for (int c = 0; c < 8; ++c) {
      S wt = 1;
      uint32_t lp[3];
      for (int d = 0; d < 3; ++d) {
        if ((c & (1 << d)) == 0) {
          wt *= S(1) - w[d];
          lp[d] = pg[d];
        } else {
          wt *= w[d];
          lp[d] = pg[d] + 1;
        }
      }
      uint32_t idx = (g.offset[l] + grid_index(g.hash, T, res, lp)) * uint32_t(g.feats);
      for (int f = 0; f < g.feats; ++f) grad_table[idx + f] += wt * dfeat[l * g.feats + f];
    }
  }
}

// tcnn/include/tiny-cuda-nn/encodings/spherical_harmonics.h:46-85 -- real SH
// basis up to degree 4 (16 coefficients) of the unit vector (x, y, z).
template <class S> inline void sh_encode(int degree, S x, S y, S z, S* o) {
  S xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
  S z4 = z2 * z2;
  o[0] = S(0.28209479177387814);
  if (degree <= 1) return;
  o[1] = S(-0.48860251190291987) * y;
  o[2] = S(0.48860251190291987) * z;
  o[3] = S(-0.48860251190291987) * x;
  if (degree <= 2) return;
  o[4] = S(1.0925484305920792) * xy;
  o[5] = S(-1.0925484305920792) * yz;
  o[6] = S(0.94617469575755997) * z2 - S(0.31539156525251999);
  o[7] = S(-1.0925484305920792) * xz;
  o[8] = S(0.54627421529603959) * x2 - S(0.54627421529603959) * y2;
  if (degree <= 3) return;
  o[9] = S(0.59004358992664352) * y * (S(-3) * x2 + y2);
  o[10] = S(2.8906114426405538) * xy * z;
  o[11] = S(0.45704579946446572) * y * (S(1) - S(5) * z2);
  o[12] = S(0.3731763325901154) * z * (S(5) * z2 - S(3));
  o[13] = S(0.45704579946446572) * x * (S(1) - S(5) * z2);
  o[14] = S(1.4453057213202769) * z * (x2 - y2);
  o[15] = S(0.59004358992664352) * x * (-x2 + S(3) * y2);
  (void)z4;
}

// tcnn/include/tiny-cuda-nn/common_device.h:543-547 quartic CDF and
// encodings/oneblob.h:99-125 -- one-blob encoding of x in [0,1] into n bins,
// with the kernel wrapped around +-1.
template <class S> inline S quartic_cdf(S x, S inv_radius) {
  S u = x * inv_radius, u2 = u * u, u4 = u2 * u2;
  return std::max(S(0), std::min(S(1), S(15) / S(16) * u * (S(1) - S(2) / S(3) * u2 + S(1) / S(5) * u4) + S(0.5)));
}
template <class S> inline void oneblob_encode(int n_bins, S x, S* o) {
  S nb = S(n_bins);
  S left = quartic_cdf(-x, nb) + quartic_cdf(-x - S(1), nb) + quartic_cdf(-x + S(1), nb);
  for (int k = 0; k < n_bins; ++k) {
    S rb = S(k + 1) / nb;
    S right = quartic_cdf(rb - x, nb) + quartic_cdf(rb - x - S(1), nb) + quartic_cdf(rb - x + S(1), nb);
    o[k] = right - left;
    left = right;
  }
}

}  // namespace nmgo
