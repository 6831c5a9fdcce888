// mixture.cuh -- FP32 device math of the K-lobe vMF mixture.
//
// Follows the reference's mixture (src/render/guided/distribution.h:13-202,
// src/backend/src/util/vmf.h:12-75) with one thread per query and the lobes
// held in registers. Mean directions are kept as unit vectors: the reference
// stores them as spherical angles and converts back with sin/cos at every
// evaluation (and through acos/atan2 after the cosine-lobe product,
// distribution.h:54); the Cartesian form skips those round trips and is
// closer to the exact value, not further from it.
//
// The FAST template flag selects hardware approximations (__expf, __sincosf,
// __fdividef) for the fused reduced-precision path; FAST = false uses CUDA's
// accurate expf/sincosf/log1pf for the FP32 path.
#pragma once
#include <string.h>

#include "common.cuh"

namespace nmg {

template <bool FAST> NMG_D float xexp(float x) { return FAST ? __expf(x) : expf(x); }
template <bool FAST> NMG_D void xsincos(float x, float* s, float* c) {
  if (FAST)
    __sincosf(x, s, c);
  else
    sincosf(x, s, c);
}
template <bool FAST> NMG_D float xdiv(float a, float b) { return FAST ? __fdividef(a, b) : a / b; }
// sin/cos of an angle x in [0, 2pi]. The hardware approximation is most
// accurate on [-pi, pi], so FAST evaluates it at x - pi and flips the signs.
template <bool FAST> NMG_D void xsincos_2pi(float x, float* s, float* c) {
  if (FAST) {
    float sn, cs;
    __sincosf(x - NMG_PI, &sn, &cs);
    *s = -sn;
    *c = -cs;
  } else {
    sincosf(x, s, c);
  }
}
// sin/cos of 2 pi t for t in [0, 1] (FAST: of pi (2t - 1), then the signs).
template <bool FAST> NMG_D void xsincos_turn(float t, float* s, float* c) {
  if (FAST) {
    float sn, cs;
    __sincosf(NMG_PI * (2.f * t - 1.f), &sn, &cs);
    *s = -sn;
    *c = -cs;
  } else {
    sincosf(NMG_TWO_PI * t, s, c);
  }
}

// sin(pi t) and cos(pi t) for t in [0, 2]: the argument is folded exactly
// (t - 1, 1 - t and 0.5 - t are exact where they are taken) onto [0, 1/4],
// where Taylor polynomials of degree 9 (sin) and 8 (cos) of x = pi t are
// accurate to 2e-9 and 3e-8; over [0, 2] the result is within 1e-7 of the
// exact value (tests/test_sincospi_host.py: at most 9.5e-8 against long
// double over 2e6 float arguments). TWO = false
// drops the fold of [1, 2] onto [0, 1] for arguments known to lie in [0, 1].
template <bool TWO = true>
NMG_HD void sincospi_poly(float t, float* s, float* c) {
  const bool hi = TWO && t >= 1.f;
  const float t1 = hi ? t - 1.f : t;
  const bool upper = t1 > 0.5f;
  const float a = upper ? 1.f - t1 : t1;
  const bool swap = a > 0.25f;
  const float b = swap ? 0.5f - a : a;
  const float x = b * NMG_PI, x2 = x * x;
  const float sp = x * (1.f + x2 * (-1.f / 6.f + x2 * (1.f / 120.f + x2 * (-1.f / 5040.f + x2 * (1.f / 362880.f)))));
  const float cp = 1.f + x2 * (-0.5f + x2 * (1.f / 24.f + x2 * (-1.f / 720.f + x2 * (1.f / 40320.f))));
  const float sa = swap ? cp : sp;  // sin(pi a)
  float ca = swap ? sp : cp;        // cos(pi a)
  if (upper) ca = -ca;              // sin(pi - y) = sin y, cos(pi - y) = -cos y
  *s = hi ? -sa : sa;               // sin(y + pi) = -sin y, cos(y + pi) = -cos y
  *c = hi ? -ca : ca;
}

// sin(pi k/32) and cos(pi k/32) for k = 0..127 (one period of t = k/32),
// each rounded once to FP32 from an 80-bit long-double evaluation (the
// multiples of 1/2 are exact).
#define NMG_SINCOSPI32_TABLE { \
  {0.000000000e+00f, 1.000000000e+00f}, /* k = 0 */ \
  {9.801714122e-02f, 9.951847196e-01f}, /* k = 1 */ \
  {1.950903237e-01f, 9.807852507e-01f}, /* k = 2 */ \
  {2.902846634e-01f, 9.569403529e-01f}, /* k = 3 */ \
  {3.826834261e-01f, 9.238795042e-01f}, /* k = 4 */ \
  {4.713967443e-01f, 8.819212914e-01f}, /* k = 5 */ \
  {5.555702448e-01f, 8.314695954e-01f}, /* k = 6 */ \
  {6.343932748e-01f, 7.730104327e-01f}, /* k = 7 */ \
  {7.071067691e-01f, 7.071067691e-01f}, /* k = 8 */ \
  {7.730104327e-01f, 6.343932748e-01f}, /* k = 9 */ \
  {8.314695954e-01f, 5.555702448e-01f}, /* k = 10 */ \
  {8.819212914e-01f, 4.713967443e-01f}, /* k = 11 */ \
  {9.238795042e-01f, 3.826834261e-01f}, /* k = 12 */ \
  {9.569403529e-01f, 2.902846634e-01f}, /* k = 13 */ \
  {9.807852507e-01f, 1.950903237e-01f}, /* k = 14 */ \
  {9.951847196e-01f, 9.801714122e-02f}, /* k = 15 */ \
  {1.000000000e+00f, 0.000000000e+00f}, /* k = 16 */ \
  {9.951847196e-01f, -9.801714122e-02f}, /* k = 17 */ \
  {9.807852507e-01f, -1.950903237e-01f}, /* k = 18 */ \
  {9.569403529e-01f, -2.902846634e-01f}, /* k = 19 */ \
  {9.238795042e-01f, -3.826834261e-01f}, /* k = 20 */ \
  {8.819212914e-01f, -4.713967443e-01f}, /* k = 21 */ \
  {8.314695954e-01f, -5.555702448e-01f}, /* k = 22 */ \
  {7.730104327e-01f, -6.343932748e-01f}, /* k = 23 */ \
  {7.071067691e-01f, -7.071067691e-01f}, /* k = 24 */ \
  {6.343932748e-01f, -7.730104327e-01f}, /* k = 25 */ \
  {5.555702448e-01f, -8.314695954e-01f}, /* k = 26 */ \
  {4.713967443e-01f, -8.819212914e-01f}, /* k = 27 */ \
  {3.826834261e-01f, -9.238795042e-01f}, /* k = 28 */ \
  {2.902846634e-01f, -9.569403529e-01f}, /* k = 29 */ \
  {1.950903237e-01f, -9.807852507e-01f}, /* k = 30 */ \
  {9.801714122e-02f, -9.951847196e-01f}, /* k = 31 */ \
  {0.000000000e+00f, -1.000000000e+00f}, /* k = 32 */ \
  {-9.801714122e-02f, -9.951847196e-01f}, /* k = 33 */ \
  {-1.950903237e-01f, -9.807852507e-01f}, /* k = 34 */ \
  {-2.902846634e-01f, -9.569403529e-01f}, /* k = 35 */ \
  {-3.826834261e-01f, -9.238795042e-01f}, /* k = 36 */ \
  {-4.713967443e-01f, -8.819212914e-01f}, /* k = 37 */ \
  {-5.555702448e-01f, -8.314695954e-01f}, /* k = 38 */ \
  {-6.343932748e-01f, -7.730104327e-01f}, /* k = 39 */ \
  {-7.071067691e-01f, -7.071067691e-01f}, /* k = 40 */ \
  {-7.730104327e-01f, -6.343932748e-01f}, /* k = 41 */ \
  {-8.314695954e-01f, -5.555702448e-01f}, /* k = 42 */ \
  {-8.819212914e-01f, -4.713967443e-01f}, /* k = 43 */ \
  {-9.238795042e-01f, -3.826834261e-01f}, /* k = 44 */ \
  {-9.569403529e-01f, -2.902846634e-01f}, /* k = 45 */ \
  {-9.807852507e-01f, -1.950903237e-01f}, /* k = 46 */ \
  {-9.951847196e-01f, -9.801714122e-02f}, /* k = 47 */ \
  {-1.000000000e+00f, 0.000000000e+00f}, /* k = 48 */ \
  {-9.951847196e-01f, 9.801714122e-02f}, /* k = 49 */ \
  {-9.807852507e-01f, 1.950903237e-01f}, /* k = 50 */ \
  {-9.569403529e-01f, 2.902846634e-01f}, /* k = 51 */ \
  {-9.238795042e-01f, 3.826834261e-01f}, /* k = 52 */ \
  {-8.819212914e-01f, 4.713967443e-01f}, /* k = 53 */ \
  {-8.314695954e-01f, 5.555702448e-01f}, /* k = 54 */ \
  {-7.730104327e-01f, 6.343932748e-01f}, /* k = 55 */ \
  {-7.071067691e-01f, 7.071067691e-01f}, /* k = 56 */ \
  {-6.343932748e-01f, 7.730104327e-01f}, /* k = 57 */ \
  {-5.555702448e-01f, 8.314695954e-01f}, /* k = 58 */ \
  {-4.713967443e-01f, 8.819212914e-01f}, /* k = 59 */ \
  {-3.826834261e-01f, 9.238795042e-01f}, /* k = 60 */ \
  {-2.902846634e-01f, 9.569403529e-01f}, /* k = 61 */ \
  {-1.950903237e-01f, 9.807852507e-01f}, /* k = 62 */ \
  {-9.801714122e-02f, 9.951847196e-01f}, /* k = 63 */ \
  {0.000000000e+00f, 1.000000000e+00f}, /* k = 64 */ \
  {9.801714122e-02f, 9.951847196e-01f}, /* k = 65 */ \
  {1.950903237e-01f, 9.807852507e-01f}, /* k = 66 */ \
  {2.902846634e-01f, 9.569403529e-01f}, /* k = 67 */ \
  {3.826834261e-01f, 9.238795042e-01f}, /* k = 68 */ \
  {4.713967443e-01f, 8.819212914e-01f}, /* k = 69 */ \
  {5.555702448e-01f, 8.314695954e-01f}, /* k = 70 */ \
  {6.343932748e-01f, 7.730104327e-01f}, /* k = 71 */ \
  {7.071067691e-01f, 7.071067691e-01f}, /* k = 72 */ \
  {7.730104327e-01f, 6.343932748e-01f}, /* k = 73 */ \
  {8.314695954e-01f, 5.555702448e-01f}, /* k = 74 */ \
  {8.819212914e-01f, 4.713967443e-01f}, /* k = 75 */ \
  {9.238795042e-01f, 3.826834261e-01f}, /* k = 76 */ \
  {9.569403529e-01f, 2.902846634e-01f}, /* k = 77 */ \
  {9.807852507e-01f, 1.950903237e-01f}, /* k = 78 */ \
  {9.951847196e-01f, 9.801714122e-02f}, /* k = 79 */ \
  {1.000000000e+00f, 0.000000000e+00f}, /* k = 80 */ \
  {9.951847196e-01f, -9.801714122e-02f}, /* k = 81 */ \
  {9.807852507e-01f, -1.950903237e-01f}, /* k = 82 */ \
  {9.569403529e-01f, -2.902846634e-01f}, /* k = 83 */ \
  {9.238795042e-01f, -3.826834261e-01f}, /* k = 84 */ \
  {8.819212914e-01f, -4.713967443e-01f}, /* k = 85 */ \
  {8.314695954e-01f, -5.555702448e-01f}, /* k = 86 */ \
  {7.730104327e-01f, -6.343932748e-01f}, /* k = 87 */ \
  {7.071067691e-01f, -7.071067691e-01f}, /* k = 88 */ \
  {6.343932748e-01f, -7.730104327e-01f}, /* k = 89 */ \
  {5.555702448e-01f, -8.314695954e-01f}, /* k = 90 */ \
  {4.713967443e-01f, -8.819212914e-01f}, /* k = 91 */ \
  {3.826834261e-01f, -9.238795042e-01f}, /* k = 92 */ \
  {2.902846634e-01f, -9.569403529e-01f}, /* k = 93 */ \
  {1.950903237e-01f, -9.807852507e-01f}, /* k = 94 */ \
  {9.801714122e-02f, -9.951847196e-01f}, /* k = 95 */ \
  {0.000000000e+00f, -1.000000000e+00f}, /* k = 96 */ \
  {-9.801714122e-02f, -9.951847196e-01f}, /* k = 97 */ \
  {-1.950903237e-01f, -9.807852507e-01f}, /* k = 98 */ \
  {-2.902846634e-01f, -9.569403529e-01f}, /* k = 99 */ \
  {-3.826834261e-01f, -9.238795042e-01f}, /* k = 100 */ \
  {-4.713967443e-01f, -8.819212914e-01f}, /* k = 101 */ \
  {-5.555702448e-01f, -8.314695954e-01f}, /* k = 102 */ \
  {-6.343932748e-01f, -7.730104327e-01f}, /* k = 103 */ \
  {-7.071067691e-01f, -7.071067691e-01f}, /* k = 104 */ \
  {-7.730104327e-01f, -6.343932748e-01f}, /* k = 105 */ \
  {-8.314695954e-01f, -5.555702448e-01f}, /* k = 106 */ \
  {-8.819212914e-01f, -4.713967443e-01f}, /* k = 107 */ \
  {-9.238795042e-01f, -3.826834261e-01f}, /* k = 108 */ \
  {-9.569403529e-01f, -2.902846634e-01f}, /* k = 109 */ \
  {-9.807852507e-01f, -1.950903237e-01f}, /* k = 110 */ \
  {-9.951847196e-01f, -9.801714122e-02f}, /* k = 111 */ \
  {-1.000000000e+00f, 0.000000000e+00f}, /* k = 112 */ \
  {-9.951847196e-01f, 9.801714122e-02f}, /* k = 113 */ \
  {-9.807852507e-01f, 1.950903237e-01f}, /* k = 114 */ \
  {-9.569403529e-01f, 2.902846634e-01f}, /* k = 115 */ \
  {-9.238795042e-01f, 3.826834261e-01f}, /* k = 116 */ \
  {-8.819212914e-01f, 4.713967443e-01f}, /* k = 117 */ \
  {-8.314695954e-01f, 5.555702448e-01f}, /* k = 118 */ \
  {-7.730104327e-01f, 6.343932748e-01f}, /* k = 119 */ \
  {-7.071067691e-01f, 7.071067691e-01f}, /* k = 120 */ \
  {-6.343932748e-01f, 7.730104327e-01f}, /* k = 121 */ \
  {-5.555702448e-01f, 8.314695954e-01f}, /* k = 122 */ \
  {-4.713967443e-01f, 8.819212914e-01f}, /* k = 123 */ \
  {-3.826834261e-01f, 9.238795042e-01f}, /* k = 124 */ \
  {-2.902846634e-01f, 9.569403529e-01f}, /* k = 125 */ \
  {-1.950903237e-01f, 9.807852507e-01f}, /* k = 126 */ \
  {-9.801714122e-02f, 9.951847196e-01f}, /* k = 127 */ \
}

// The bits of a float (bit cast, host and device).
NMG_HD int float_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_int(f);
#else
  int i;
  memcpy(&i, &f, sizeof(i));
  return i;
#endif
}

// sin(pi t) and cos(pi t) from that table: t = k/32 + r with k the integer
// nearest 32 t, where r = t - k/32 is exact and |r| <= 1/64; sin and cos of
// pi r by r (pi - (pi^3/6) r^2) and 1 + r^2 (-pi^2/2 + (pi^4/24) r^2)
// (truncation below 2.4e-9 and 2e-11), then the angle-sum formulas. The
// rounding to k adds 1.5 * 2^23 (so the sum's last mantissa bits hold k,
// ties to even like rint) and subtracts it again: no conversion
// instructions, and the table index is those bits modulo 128 -- in range
// for any t, exact for |t| < 2^17 (t of the mixture lies in [0, 2]). About
// 15 instructions and one 8-byte load against sincospi_poly's ~28, and
// within 1e-7 of the exact value over [0, 2] (tests/test_sincospi_host.py).
NMG_HD void sincospi_tab(const float2* tab, float t, float* s, float* c) {
  constexpr float kRound = 12582912.f;  // 1.5 * 2^23
  const float y = fmaf(t, 32.f, kRound);
  const float kf = y - kRound;
  const float r = fmaf(kf, -1.f / 32.f, t), r2 = r * r;
  const float sr = r * fmaf(r2, -5.16771278f, 3.14159265f);  // pi^3/6, pi
  const float cr = fmaf(r2, fmaf(r2, 4.05871213f, -4.93480220f), 1.f);  // pi^4/24, pi^2/2
  const float2 a = tab[float_bits(y) & 127];
  *s = fmaf(a.x, cr, a.y * sr);
  *c = fmaf(a.y, cr, -(a.x * sr));
}

// The table in constant memory and the per-block copy the kernels index (a
// warp's 32 different indices into constant memory would serialise).
// A kernel that evaluates angles with kAngTab calls sincospi_tab_fill() once
// at its start, before any thread can leave.
static __constant__ float2 c_sincospi32[128] = NMG_SINCOSPI32_TABLE;
static __shared__ float2 s_sincospi32[128];
NMG_D void sincospi_tab_fill() {
  for (int i = threadIdx.x; i < 128; i += blockDim.x) s_sincospi32[i] = c_sincospi32[i];
  __syncthreads();
}

// How lobe_angles evaluates sin/cos: the hardware approximation, the folded
// polynomial, or the shared-memory table.
enum : int { kAngHw = 0, kAngPoly = 1, kAngTab = 2 };

// sin/cos of the lobe angles theta = pi * st and phi = 2 pi * sp (st, sp the
// logistic outputs in (0, 1)). PRECISE (kAngPoly, kAngTab) evaluates them at
// pi * t without rounding pi * t first (sincospi_poly, or sincospi_tab from
// the block's shared table), keeping the mean direction to ~1e-7; the
// hardware approximation (kAngHw: FAST and not PRECISE) is off by up to
// ~4e-7, which a lobe of concentration kappa turns into a relative pdf
// error of ~4e-7 kappa.
// FOLD01 = false keeps the general fold for theta as well (shorter code is
// not always faster: it changes the register allocation of the caller).
template <bool FAST, int PRECISE, bool FOLD01 = true>
NMG_D void lobe_angles(float st, float sp, float* sth, float* cth, float* sph, float* cph) {
  if (PRECISE == kAngTab) {
    sincospi_tab(s_sincospi32, st, sth, cth);
    sincospi_tab(s_sincospi32, 2.f * sp, sph, cph);
  } else if (PRECISE) {
    sincospi_poly<!FOLD01>(st, sth, cth);
    sincospi_poly<true>(2.f * sp, sph, cph);
  } else {
    xsincos<FAST>(NMG_PI * st, sth, cth);
    xsincos_turn<FAST>(sp, sph, cph);
  }
}

// -expm1(-x) = 1 - e^{-x} for x >= 0 without cancellation: a degree-7 Taylor
// polynomial below x = 0.5 (relative error < 3e-8), 1 - e^{-x} above.
// (A branch-free select of both forms measured slower in the fused query
// kernel: the extra live values made its consumer warps spill.)
template <bool FAST> NMG_D float one_minus_exp_neg(float x) {
  if (!FAST) return -expm1f(-x);
  if (x >= 0.5f) return 1.f - __expf(-x);
  return x * (1.f - x * (1.f / 2.f) * (1.f - x * (1.f / 3.f) * (1.f - x * (1.f / 4.f) *
             (1.f - x * (1.f / 5.f) * (1.f - x * (1.f / 6.f) * (1.f - x * (1.f / 7.f)))))));
}
template <bool FAST> NMG_D f3 unit3(f3 a) {
  if (!FAST) return normalize3(a);
  const float n2 = dot3(a, a);
  if (!(n2 > 0.f)) return a;
  const float r = rsqrtf(n2);
  return f3{a.x * r, a.y * r, a.z * r};
}

// train.h:391-415 activations.
NMG_D float act_exp_clamp(float x) { return fminf(fmaxf(x, -10.f), 15.f); }
template <bool FAST> NMG_D float logistic(float x) { return xdiv<FAST>(1.f, 1.f + xexp<FAST>(-x)); }
// Softplus in the stable form max(x,0) + log1p(e^-|x|) (train.h:398 writes
// log(1+e^x), which loses all digits for x < -16).
template <bool FAST> NMG_D float softplus(float x) {
  return fmaxf(x, 0.f) + log1pf(xexp<FAST>(-fabsf(x)));
}

struct MixOpts {
  int kappa_softplus;  // 0: kappa = exp(clamp(x)) (train.h:244); 1: log(1+e^x)
  int kappa_poly;      // 1: distribution.h:165-166 polynomial for kappa < 1
  int cosine;          // multiply by the cosine lobe before sampling/pdf
};

template <int K> struct Mix {
  float lam[K];   // activated lambda (after any product)
  float kap[K];   // concentration
  f3 mu[K];       // unit mean direction
  float w[K];     // normalised weight lambda/total
  float nrm[K];   // vMF normaliser of each lobe (1/4pi for kappa < M_EPSILON)
  float total;
};

// vMF normaliser k / (2 pi (1 - e^{-2k})) (vmf.h:25-26); below M_EPSILON the
// lobe is uniform (1/4pi).
// The denominator uses -expm1(-2k) below k = 0.5, where 1 - e^{-2k} cancels.
template <bool FAST> NMG_D float vmf_norm(float k) {
  if (k < NMG_EPS) return NMG_INV_4PI;
  const float den = FAST ? one_minus_exp_neg<true>(2.f * k) : (k < 0.5f ? -expm1f(-2.f * k) : 1.f - expf(-2.f * k));
  return xdiv<FAST>(k, NMG_TWO_PI * den);
}

// distribution.h:85-98: activation of one query's raw outputs. `raw` points
// at 4K floats (lambda, kappa, theta, phi per lobe), 16-byte aligned.
template <int K, bool FAST, int PRECISE = !FAST>
NMG_D void mix_activate(Mix<K>& m, const float* raw, int kappa_softplus) {
  m.total = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float4 r = reinterpret_cast<const float4*>(raw)[i];
    m.lam[i] = xexp<FAST>(act_exp_clamp(r.x));
    m.kap[i] = kappa_softplus ? softplus<FAST>(r.y) : xexp<FAST>(act_exp_clamp(r.y));
    float st, ct, sp, cp;
    lobe_angles<FAST, PRECISE>(logistic<FAST>(r.z), logistic<FAST>(r.w), &st, &ct, &sp, &cp);
    m.mu[i] = f3{st * cp, st * sp, ct};
    m.total += m.lam[i];
  }
  const float inv = 1.f / m.total;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    m.w[i] = FAST ? m.lam[i] * inv : m.lam[i] / m.total;
    m.nrm[i] = vmf_norm<FAST>(m.kap[i]);
  }
}

// One lobe of mix_activate_regs from its raw (lambda, kappa, theta, phi).
template <bool FAST>
NMG_D void lobe_activate(float r0, float r1, float r2, float r3, int kappa_softplus, float& lam, float& kap,
                         f3& mu) {
  lam = xexp<FAST>(act_exp_clamp(r0));
  kap = kappa_softplus ? softplus<FAST>(r1) : xexp<FAST>(act_exp_clamp(r1));
  float st, ct, sp, cp;
  lobe_angles<FAST, !FAST>(logistic<FAST>(r2), logistic<FAST>(r3), &st, &ct, &sp, &cp);
  mu = f3{st * cp, st * sp, ct};
}

// Same activation from raw outputs held in registers (compile-time indices).
template <int K, bool FAST, int N>
NMG_D void mix_activate_regs(Mix<K>& m, const float (&raw)[N], int kappa_softplus) {
  static_assert(N >= 4 * K, "raw row too short");
  m.total = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    lobe_activate<FAST>(raw[4 * i], raw[4 * i + 1], raw[4 * i + 2], raw[4 * i + 3], kappa_softplus, m.lam[i],
                        m.kap[i], m.mu[i]);
    m.total += m.lam[i];
  }
  const float inv = 1.f / m.total;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    m.w[i] = FAST ? m.lam[i] * inv : m.lam[i] / m.total;
    m.nrm[i] = vmf_norm<FAST>(m.kap[i]);
  }
}

// Product normaliser k / (2 pi (1 - e^{-2k})) (distribution.h:40-42): 1/4pi
// below kappa = 1e-3.
template <bool FAST> NMG_D float prod_norm(float k) {
  return k < 1e-3f ? NMG_INV_4PI : xdiv<FAST>(k * NMG_INV_2PI, one_minus_exp_neg<FAST>(2.f * k));
}
constexpr float kCosineKappa = 2.18853f;  // distribution.h:184-195

// One lobe (lam, kap, mu, nrm = its vMF normaliser) times the cosine lobe of
// concentration kb = kCosineKappa around the unit mean mb (nb = its product
// normaliser): the lobe's new weight, concentration, mean and normaliser.
template <bool FAST>
NMG_D void lobe_cosine(f3 mb, float nb, float& lam, float& kap, f3& mu, float& nrm) {
  const float kb = kCosineKappa;
  const f3 ma = mu;
  const float ka = kap;
  f3 nm = add3(scale3(ma, ka), scale3(mb, kb));
  const float n2 = dot3(nm, nm);
  float nk;
  if (FAST) {
    const float rn = rsqrtf(n2);
    nk = n2 * rn;
    if (nk >= 1e-3f) {
      nm = scale3(nm, rn);
    } else {
      nk = 0.f;
      nm = ma;
    }
  } else {
    nk = sqrtf(n2);
    if (nk >= 1e-3f) {
      nm = f3{nm.x / nk, nm.y / nk, nm.z / nk};
    } else {
      nk = 0.f;
      nm = ma;
    }
  }
  const float e = xexp<FAST>(ka * (dot3(nm, ma) - 1.f) + kb * (dot3(nm, mb) - 1.f));
  const float pk = prod_norm<FAST>(nk);
  // prod_norm(ka) equals the lobe's cached vMF normaliser above kappa = 1e-3
  const float pa = FAST ? (ka < 1e-3f ? NMG_INV_4PI : nrm) : prod_norm<FAST>(ka);
  const float sc = xdiv<FAST>(pa * nb, pk) * e;
  lam = sc * lam;
  kap = nk;
  mu = nm;
  nrm = pk;  // equals vmf_norm(nk): nk is 0 or >= 1e-3 here
}

// distribution.h:39-64 + 184-195: product of every lobe with the cosine lobe
// (kappa 2.18853) around `n` (already face-forwarded, any length), then
// renormalisation with total clamped below at M_EPSILON.
template <int K, bool FAST>
NMG_D void mix_apply_cosine(Mix<K>& m, f3 n) {
  const f3 mb = unit3<FAST>(n);
  const float nb = prod_norm<FAST>(kCosineKappa);
  m.total = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    lobe_cosine<FAST>(mb, nb, m.lam[i], m.kap[i], m.mu[i], m.nrm[i]);
    m.total += m.lam[i];
  }
  m.total = fmaxf(m.total, NMG_EPS);
  const float inv = 1.f / m.total;
#pragma unroll
  for (int i = 0; i < K; ++i) m.w[i] = FAST ? m.lam[i] * inv : m.lam[i] / m.total;
}

// distribution.h:132-140: lobe selection by sequential CDF subtraction,
// falling back to lobe 0.
template <int K> NMG_D int mix_select(const Mix<K>& m, float u) {
  int sel = -1;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    if (sel < 0) {
      if (u < m.w[i])
        sel = i;
      else
        u -= m.w[i];
    }
  }
  return sel < 0 ? 0 : sel;
}

template <bool FAST> NMG_D f3 vmf_sample_dir(float k, f3 mu, float u0, float u1);
NMG_D f3 vmf_sample_lean(float k, f3 mu, float u0, float u1);

// raytracing.h:35-49 Frame(mu) applied to a direction in the lobe's local
// frame: T = normalize(mu x e), e the branchless axis pick
// (getPerpendicular, math_utils.h:141-151); B = normalize(mu x T).
template <bool FAST>
NMG_D f3 to_frame(f3 mu, f3 loc) {
  float ax = fabsf(mu.x), ay = fabsf(mu.y), az = fabsf(mu.z);
  unsigned xm = ((ax - ay) < 0.f) & ((ax - az) < 0.f);
  unsigned ym = (1u ^ xm) & ((ay - az) < 0.f);
  unsigned zm = 1u ^ (xm | ym);
  f3 t = unit3<FAST>(cross3(mu, f3{float(xm), float(ym), float(zm)}));
  f3 b = unit3<FAST>(cross3(mu, t));
  return f3{t.x * loc.x + b.x * loc.y + mu.x * loc.z, t.y * loc.x + b.y * loc.y + mu.y * loc.z,
            t.z * loc.x + b.z * loc.y + mu.z * loc.z};
}

// vmf.h:48-71: sample lobe `sel` with two uniforms, rotated by the frame of
// its mean (raytracing.h:35-49, getPerpendicular math_utils.h:141-151).
template <int K, bool FAST>
NMG_D f3 mix_sample_lobe(const Mix<K>& m, int sel, float u0, float u1) {
  float k = 0.f;
  f3 mu = m.mu[0];
#pragma unroll
  for (int i = 0; i < K; ++i)
    if (i == sel) {
      k = m.kap[i];
      mu = m.mu[i];
    }
  // FAST: the one-logarithm sampler (kappa below M_EPSILON is the uniform lobe, kappa 0 there)
  if constexpr (FAST) return vmf_sample_lean(k < NMG_EPS ? 0.f : k, mu, u0, u1);
  return vmf_sample_dir<FAST>(k, mu, u0, u1);
}

// vmf.h:48-71 for one lobe (concentration k, unit mean mu).
template <bool FAST>
NMG_D f3 vmf_sample_dir(float k, f3 mu, float u0, float u1) {
  f3 loc;
  float sp, cp;
  if (k < NMG_EPS) {  // render/sampling.h:32-37, then rotated like any lobe sample (vmf.h:67-71)
    float z = 1.f - 2.f * u0;
    float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    xsincos_turn<FAST>(u1, &sp, &cp);
    loc = f3{r * cp, r * sp, z};
  } else {
  // cos(theta) = 1 + log1p(-u0 + e^{-2k} u0) / k (vmf.h:51), evaluated as
  // 1 - cos = -log1p(u0 expm1(-2k)) / k and, on the far hemisphere,
  // 1 + cos = log1p((1 - u0) expm1(2k)) / k, so that sin^2 = (1-cos)(1+cos)
  // keeps its digits near both poles of the lobe (k < 8.3 there, so
  // expm1(2k) stays finite).
  const float omc = -log1pf(-u0 * one_minus_exp_neg<FAST>(2.f * k)) / k;
  float ct, s2;
  if (omc <= 1.f) {
    ct = 1.f - omc;
    s2 = omc * (2.f - omc);
  } else {
    const float opc = log1pf((1.f - u0) * expm1f(2.f * k)) / k;
    ct = opc - 1.f;
    s2 = opc * (2.f - opc);
  }
  float st = sqrtf(fmaxf(0.f, s2));
  xsincos_turn<FAST>(u1, &sp, &cp);
  loc = f3{cp * st, sp * st, ct};
  }
  return to_frame<FAST>(mu, loc);
}

// distribution.h:113-119 with vmf.h:22-27: mixture pdf at unit direction wi.
template <int K, bool FAST>
NMG_D float mix_pdf(const Mix<K>& m, f3 wi) {
  float p = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const float k = m.kap[i];
    const float c = dot3(wi, m.mu[i]);
    const float v = k < NMG_EPS ? NMG_INV_4PI : xexp<FAST>(k * fminf(0.f, c - 1.f)) * m.nrm[i];
    p += m.w[i] * v;
  }
  return p;
}

// ---------------------------------------------------------------------------
// The lean form (hardware exponentials and divides): only what selection,
// sampling and the pdf need, with the concentration-dependent branches of
// the general form evaluated branch-free. MixLean and its activation serve
// the mixture-only kernels (raw outputs in memory, no cosine lobe, table
// sin/cos of the lobe angles); the branch-free normaliser and the
// one-logarithm sampler also serve the network kernels' mixtures (the
// 16-lobe query, the sampler of the 8-lobe query, the training loss). The
// lobe selection is the general form's, operation for operation.

// B(x) = x / (1 - e^{-x}) for 0 <= x < 0.5 from its series
// 1 + x/2 + x^2/12 - x^4/720 + x^6/30240 (the Bernoulli numbers; the first
// omitted term, x^8/1209600, is below 3.3e-9 at x = 0.5).
NMG_HD float bernoulli_gen(float x) {
  const float x2 = x * x;
  return fmaf(x2, fmaf(x2, fmaf(x2, 1.f / 30240.f, -1.f / 720.f), 1.f / 12.f), fmaf(0.5f, x, 1.f));
}

// vMF normaliser k / (2 pi (1 - e^{-2k})) (vmf.h:25-26): (1/4pi) B(2k) below
// 2k = 0.5, where 1 - e^{-2k} cancels, k/(2pi) / (1 - e^{-2k}) above. Both
// are evaluated and one selected, so a warp whose lobes fall on both sides
// does not run two paths in turn. k = 0 gives 1/4pi exactly.
NMG_D float vmf_norm_sel(float k) {
  const float x = 2.f * k;
  const float lo = NMG_INV_4PI * bernoulli_gen(x);
  const float hi = __fdividef(k * NMG_INV_2PI, 1.f - __expf(-x));
  return x < 0.5f ? lo : hi;
}

// 32 bytes of global memory in one load (ld.global.v8.f32, sm_100 and
// later); p 32-byte aligned. The data must not change during the kernel.
NMG_D void ld_global_v8(const float* p, float4& a, float4& b) {
  asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

template <int K> struct MixLean {
  float lam[K];  // activated lambda
  float kap[K];  // concentration; 0 for a lobe below M_EPSILON (uniform, vmf.h:24)
  float ln[K];   // lambda times the lobe's vMF normaliser
  f3 mu[K];      // unit mean direction
  float total;   // sum of lambda
};

// distribution.h:85-98 for the mixture-only kernels (a kernel using it calls
// sincospi_tab_fill() first). A lobe below M_EPSILON gets kappa 0: its pdf
// term e^{0} times 1/4pi is the reference's uniform value exactly.
// WIDE: raw is 32-byte aligned in global memory and K is even, and the row
// comes in as K/2 32-byte loads (ld.global.v8.f32, sm_100 and later): half
// the load instructions, and half the L1 wavefronts when every lane of a warp
// reads a different row.
template <int K, bool WIDE = false>
NMG_D void mix_activate_lean(MixLean<K>& m, const float* raw, int kappa_softplus) {
  float4 row[WIDE ? K : 1];
  if constexpr (WIDE) {
    static_assert(K % 2 == 0, "32-byte loads take two lobes");
#pragma unroll
    for (int j = 0; j < K / 2; ++j) ld_global_v8(raw + 8 * j, row[2 * j], row[2 * j + 1]);
  }
  m.total = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const float4 r = WIDE ? row[WIDE ? i : 0] : reinterpret_cast<const float4*>(raw)[i];
    m.lam[i] = __expf(act_exp_clamp(r.x));
    float k = kappa_softplus ? softplus<true>(r.y) : __expf(act_exp_clamp(r.y));
    k = k < NMG_EPS ? 0.f : k;
    m.kap[i] = k;
    float st, ct, sp, cp;
    lobe_angles<true, kAngTab>(logistic<true>(r.z), logistic<true>(r.w), &st, &ct, &sp, &cp);
    m.mu[i] = f3{st * cp, st * sp, ct};
    m.ln[i] = m.lam[i] * vmf_norm_sel(k);
    m.total += m.lam[i];
  }
}

// distribution.h:132-140 (mix_select's arithmetic) that also picks the chosen
// lobe's concentration and mean; returns the lobe, and 1/total in *inv.
template <int K>
NMG_D int mix_select_lean(const MixLean<K>& m, float u, float* k, f3* mu, float* inv) {
  const float iv = 1.f / m.total;
  int sel = -1;
  *k = m.kap[0];
  *mu = m.mu[0];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const float w = m.lam[i] * iv;
    if (sel < 0) {
      if (u < w) {
        sel = i;
        *k = m.kap[i];
        *mu = m.mu[i];
      } else {
        u -= w;
      }
    }
  }
  *inv = iv;
  return sel < 0 ? 0 : sel;
}

// Sum over the lobes of lambda * vMF(wi) (distribution.h:113-119 times the
// total): the pdf is this over m.total.
template <int K>
NMG_D float mix_pdf_lean_sum(const MixLean<K>& m, f3 wi) {
  float p = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) p = fmaf(m.ln[i], __expf(m.kap[i] * fminf(0.f, dot3(wi, m.mu[i]) - 1.f)), p);
  return p;
}

// vmf.h:48-71 for one lobe (kappa k, 0 for uniform; unit mean mu) with one
// logarithm: 1 - cos(theta) <= 1 exactly when u0 <= 1 / (1 + e^{-k}), so
// the side is known before the logarithm. Near the mean,
// 1 - cos = -log1p(-u0 (1 - e^{-2k})) / k; on the far side,
// 1 + cos = log1p((1 - u0) (1 - e^{-2k}) / e^{-2k}) / k (= the expm1(2k)
// form of vmf_sample_dir); 1 - e^{-2k} is 2k / B(2k) below 2k = 0.5.
NMG_D f3 vmf_sample_lean(float k, f3 mu, float u0, float u1) {
  float sp, cp;
  xsincos_turn<true>(u1, &sp, &cp);
  f3 loc;
  if (k == 0.f) {  // render/sampling.h:32-37
    const float z = 1.f - 2.f * u0;
    const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    loc = f3{r * cp, r * sp, z};
  } else {
    const float em = __expf(-k), e2 = em * em;
    const float x = 2.f * k;
    const float den = x < 0.5f ? __fdividef(x, bernoulli_gen(x)) : 1.f - e2;
    const bool near = u0 * (1.f + em) <= 1.f;
    const float a = near ? -u0 * den : (1.f - u0) * __fdividef(den, e2);
    const float v = log1pf(a) / k;
    const float om = near ? -v : v;  // 1 - cos near the mean, 1 + cos on the far side
    const float ct = near ? 1.f - om : om - 1.f;
    const float st = sqrtf(fmaxf(0.f, om * (2.f - om)));
    loc = f3{cp * st, sp * st, ct};
  }
  return to_frame<true>(mu, loc);
}

// Raw outputs of lobe i, from memory (16-byte aligned) or from registers.
NMG_D float4 lobe4(const float* raw, int i) { return reinterpret_cast<const float4*>(raw)[i]; }
template <int N>
NMG_D float4 lobe4(const float (&raw)[N], int i) {
  return make_float4(raw[4 * i], raw[4 * i + 1], raw[4 * i + 2], raw[4 * i + 3]);
}
NMG_D float raw_at(const float* raw, int i) { return raw[i]; }
template <int N>
NMG_D float raw_at(const float (&raw)[N], int i) { return raw[i < N ? i : 0]; }

// Per-sample KL loss and gradient with respect to the raw outputs
// (train.cu:69-124, distribution.h:144-181), FP32.
//   raw: 4K raw outputs (16-byte aligned); rec: GuidedOutput {theta, phi,
//   L_r, L_g, L_b, wiPdf}; scale = loss_scale / batch size.
// dF/dlambda uses the O(K) form (vmf_s - q)/total, algebraically equal to
// the reference's O(K^2) sum. NaN/Inf gradients become 0 and gradients are
// clamped above at 150 (train.cu:109-123). Returns the per-sample loss.
template <int K, bool FAST, int PRECISE = !FAST, class RAW>
NMG_D float mix_kl_loss_grad(const RAW& raw, const float* rec, float scale, const MixOpts& o, float* grad) {
  float lam[K], kap[K], sth[K], cth[K], sph[K], cph[K], sgt[K], sgp[K], dkap[K];
  float total = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float4 r = lobe4(raw, i);
    lam[i] = xexp<FAST>(act_exp_clamp(r.x));
    if (o.kappa_softplus) {
      kap[i] = softplus<FAST>(r.y);
      dkap[i] = logistic<FAST>(r.y);
    } else {
      kap[i] = xexp<FAST>(act_exp_clamp(r.y));
      dkap[i] = kap[i];  // train.h:410: derivative ignores the clamp
    }
    sgt[i] = logistic<FAST>(r.z);
    sgp[i] = logistic<FAST>(r.w);
    lobe_angles<FAST, PRECISE, false>(sgt[i], sgp[i], &sth[i], &cth[i], &sph[i], &cph[i]);
    total += lam[i];
  }
  float swt, cwt, swp, cwp;
  xsincos<FAST && !PRECISE>(rec[0], &swt, &cwt);
  xsincos_2pi<FAST && !PRECISE>(rec[1], &swp, &cwp);
  const f3 wi{swt * cwp, swt * swp, cwt};
  float vmf[K];
  float q = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float k = kap[i];
    float c = wi.x * sth[i] * cph[i] + wi.y * sth[i] * sph[i] + wi.z * cth[i];
    vmf[i] = k < NMG_EPS ? NMG_INV_4PI : xexp<FAST>(k * fminf(0.f, c - 1.f)) * vmf_norm<FAST>(k);
    q += (lam[i] / total) * vmf[i];
  }
  const float Li = (rec[2] + (rec[3] + rec[4])) / 3.f;
  const float wp = rec[5] + NMG_EPS;
  const float guide = q + NMG_EPS;
  const float prefix = -Li / wp / guide * scale;
  const float loss = -Li / wp * logf(guide);
  const float inv_total = 1.f / total;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float k = kap[i];
    float wv = (lam[i] * inv_total) * vmf[i];
    float ik;
    if (o.kappa_poly && k < 1.f) {
      ik = 0.000926f + -0.344883f * k + 0.030147f * (k * k);
    } else if (!o.kappa_poly && k < 1e-2f) {
      ik = k * (-1.f / 3.f + k * k * (1.f / 45.f));
    } else {
      float e = xexp<FAST>(-2.f * k);
      ik = 1.f / k - (1.f + e) / (1.f - e);
    }
    float c = wi.x * sth[i] * cph[i] + wi.y * sth[i] * sph[i] + wi.z * cth[i];
    float dl = (vmf[i] - q) * inv_total;
    float dk = wv * (c + ik);
    float dt = wv * k * (cth[i] * (wi.x * cph[i] + wi.y * sph[i]) - wi.z * sth[i]);
    float dp = wv * k * (wi.y * cph[i] - wi.x * sph[i]) * sth[i];
    float g0 = prefix * dl * lam[i];
    float g1 = prefix * dk * dkap[i];
    float g2 = prefix * dt * NMG_PI * (sgt[i] * (1.f - sgt[i]));
    float g3 = prefix * dp * NMG_TWO_PI * (sgp[i] * (1.f - sgp[i]));
    g0 = isfinite(g0) ? fminf(g0, 150.f) : 0.f;
    g1 = isfinite(g1) ? fminf(g1, 150.f) : 0.f;
    g2 = isfinite(g2) ? fminf(g2, 150.f) : 0.f;
    g3 = isfinite(g3) ? fminf(g3, 150.f) : 0.f;
    grad[4 * i + 0] = g0;
    grad[4 * i + 1] = g1;
    grad[4 * i + 2] = g2;
    grad[4 * i + 3] = g3;
  }
  return loss;
}

// train.cu:126-172: the learned-selection variant. raw[4K] is the selection
// logit; rec[6] the BSDF pdf of the direction. No NaN/clamp post-pass
// (the reference has none for this variant). grad has 4K+1 entries.
template <int K, bool FAST, int PRECISE = !FAST, class RAW>
NMG_D float mix_kl_loss_grad_selection(const RAW& raw, const float* rec, float scale, const MixOpts& o,
                                       float* grad) {
  float lam[K], kap[K], sth[K], cth[K], sph[K], cph[K], sgt[K], sgp[K], dkap[K];
  float total = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float4 r = lobe4(raw, i);
    lam[i] = xexp<FAST>(act_exp_clamp(r.x));
    if (o.kappa_softplus) {
      kap[i] = softplus<FAST>(r.y);
      dkap[i] = logistic<FAST>(r.y);
    } else {
      kap[i] = xexp<FAST>(act_exp_clamp(r.y));
      dkap[i] = kap[i];
    }
    sgt[i] = logistic<FAST>(r.z);
    sgp[i] = logistic<FAST>(r.w);
    lobe_angles<FAST, PRECISE, false>(sgt[i], sgp[i], &sth[i], &cth[i], &sph[i], &cph[i]);
    total += lam[i];
  }
  const float xs = raw_at(raw, 4 * K);
  const float sel = logistic<FAST>(xs);
  float swt, cwt, swp, cwp;
  xsincos<FAST && !PRECISE>(rec[0], &swt, &cwt);
  xsincos_2pi<FAST && !PRECISE>(rec[1], &swp, &cwp);
  const f3 wi{swt * cwp, swt * swp, cwt};
  float vmf[K];
  float q = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float k = kap[i];
    float c = wi.x * sth[i] * cph[i] + wi.y * sth[i] * sph[i] + wi.z * cth[i];
    vmf[i] = k < NMG_EPS ? NMG_INV_4PI : xexp<FAST>(k * fminf(0.f, c - 1.f)) * vmf_norm<FAST>(k);
    q += (lam[i] / total) * vmf[i];
  }
  const float Li = (rec[2] + (rec[3] + rec[4])) / 3.f;
  const float bsdf = rec[6];
  const float guide = q + NMG_EPS;
  const float wp = sel * guide + (1.f - sel) * bsdf;
  const float loss = -Li / wp * logf(wp);
  const float prefix = -Li / wp / wp * scale;
  const float inv_total = 1.f / total;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    float k = kap[i];
    float wv = (lam[i] * inv_total) * vmf[i];
    float ik;
    if (o.kappa_poly && k < 1.f) {
      ik = 0.000926f + -0.344883f * k + 0.030147f * (k * k);
    } else if (!o.kappa_poly && k < 1e-2f) {
      ik = k * (-1.f / 3.f + k * k * (1.f / 45.f));
    } else {
      float e = xexp<FAST>(-2.f * k);
      ik = 1.f / k - (1.f + e) / (1.f - e);
    }
    float c = wi.x * sth[i] * cph[i] + wi.y * sth[i] * sph[i] + wi.z * cth[i];
    float dl = (vmf[i] - q) * inv_total * sel;
    float dk = wv * (c + ik) * sel;
    float dt = wv * k * (cth[i] * (wi.x * cph[i] + wi.y * sph[i]) - wi.z * sth[i]) * sel;
    float dp = wv * k * (wi.y * cph[i] - wi.x * sph[i]) * sth[i] * sel;
    grad[4 * i + 0] = prefix * dl * lam[i];
    grad[4 * i + 1] = prefix * dk * dkap[i];
    grad[4 * i + 2] = prefix * dt * NMG_PI * (sgt[i] * (1.f - sgt[i]));
    grad[4 * i + 3] = prefix * dp * NMG_TWO_PI * (sgp[i] * (1.f - sgp[i]));
  }
  grad[4 * K] = 0.01f * prefix * (q - bsdf) * (sel * (1.f - sel));
  return loss;
}

// The same loss (train.cu:69-172) with the lobes split over two threads
// that each hold KH of them. Part one (half_loss_lobes) computes the
// thread's lobes' activations and vMF values at the record's direction, the
// partial sums of the lobe weights and of the weighted vMF values, and
// folds each lobe's derivative factors into three numbers, so that only five
// values per lobe stay live while the caller adds the partner's partial
// sums; part two (half_loss_grad) forms q = sum(lam vmf) / sum(lam) and the
// thread's lobe gradients (and, SEL, the selection logit's). Lobe arithmetic
// and precision as mix_kl_loss_grad.
template <int KH> struct HalfLoss {
  float lam[KH], vmf[KH];
  float dk[KH];  // (cos + I(kappa)) dkappa/dx: the kappa gradient's factor
  float dt[KH];  // kappa dmu/dtheta . wi * pi sigma'(x_theta): the theta gradient's factor
  float dp[KH];  // kappa dmu/dphi . wi * 2 pi sigma'(x_phi): the phi gradient's factor
  float lt, nt;
};

template <int KH, bool FAST, int PRECISE = !FAST, class RAW>
NMG_D void half_loss_lobes(HalfLoss<KH>& s, const RAW& raw, const float* rec, const MixOpts& o) {
  float swt, cwt, swp, cwp;
  xsincos<FAST && !PRECISE>(rec[0], &swt, &cwt);
  xsincos_2pi<FAST && !PRECISE>(rec[1], &swp, &cwp);
  const f3 wi{swt * cwp, swt * swp, cwt};
  s.lt = 0.f;
  s.nt = 0.f;
#pragma unroll
  for (int i = 0; i < KH; ++i) {
    const float4 r = lobe4(raw, i);
    const float lam = xexp<FAST>(act_exp_clamp(r.x));
    float kap, dkap;
    if (o.kappa_softplus) {
      kap = softplus<FAST>(r.y);
      dkap = logistic<FAST>(r.y);
    } else {
      kap = xexp<FAST>(act_exp_clamp(r.y));
      dkap = kap;  // train.h:410: derivative ignores the clamp
    }
    const float sgt = logistic<FAST>(r.z), sgp = logistic<FAST>(r.w);
    float sth, cth, sph, cph;
    lobe_angles<FAST, PRECISE, false>(sgt, sgp, &sth, &cth, &sph, &cph);
    const float cc = wi.x * sth * cph + wi.y * sth * sph + wi.z * cth;
    const float k = kap;
    float vmf, ik;
    if (FAST) {
      // branch-free: kappa below M_EPSILON as 0 (e^{0} / 4pi, the uniform lobe), both forms of
      // the normaliser and of d log(normaliser) / d kappa evaluated and one selected
      const float kz = k < NMG_EPS ? 0.f : k;
      vmf = __expf(kz * fminf(0.f, cc - 1.f)) * vmf_norm_sel(kz);
      const float e = __expf(-2.f * k);
      const float ik_exact = 1.f / k - (1.f + e) / (1.f - e);
      const float ik_small = o.kappa_poly ? 0.000926f + -0.344883f * k + 0.030147f * (k * k)
                                          : k * (-1.f / 3.f + k * k * (1.f / 45.f));
      ik = k < (o.kappa_poly ? 1.f : 1e-2f) ? ik_small : ik_exact;
    } else {
      vmf = k < NMG_EPS ? NMG_INV_4PI : xexp<FAST>(k * fminf(0.f, cc - 1.f)) * vmf_norm<FAST>(k);
      if (o.kappa_poly && k < 1.f) {
        ik = 0.000926f + -0.344883f * k + 0.030147f * (k * k);
      } else if (!o.kappa_poly && k < 1e-2f) {
        ik = k * (-1.f / 3.f + k * k * (1.f / 45.f));
      } else {
        const float e = xexp<FAST>(-2.f * k);
        ik = 1.f / k - (1.f + e) / (1.f - e);
      }
    }
    s.lam[i] = lam;
    s.vmf[i] = vmf;
    s.dk[i] = (cc + ik) * dkap;
    s.dt[i] = k * (cth * (wi.x * cph + wi.y * sph) - wi.z * sth) * (NMG_PI * (sgt * (1.f - sgt)));
    s.dp[i] = k * ((wi.y * cph - wi.x * sph) * sth) * (NMG_TWO_PI * (sgp * (1.f - sgp)));
    s.lt += lam;
    s.nt += lam * vmf;
  }
}

// total / nt_total: both threads' sums; sel_logit: raw output 4K (SEL).
// Writes grad[4 KH] (and *gsel when SEL); returns the per-sample loss.
template <int KH, bool FAST, bool SEL>
NMG_D float half_loss_grad(const HalfLoss<KH>& s, float total, float nt_total, float sel_logit, const float* rec,
                           float scale, const MixOpts& o, float* grad, float* gsel) {
  const float inv_total = 1.f / total;
  const float q = nt_total * inv_total;
  const float Li = (rec[2] + (rec[3] + rec[4])) / 3.f;
  float prefix, loss, sel = 1.f;
  if (SEL) {
    sel = logistic<FAST>(sel_logit);
    const float wp = sel * (q + NMG_EPS) + (1.f - sel) * rec[6];
    loss = -Li / wp * logf(wp);
    prefix = -Li / wp / wp * scale;
    *gsel = 0.01f * prefix * (q - rec[6]) * (sel * (1.f - sel));
  } else {
    const float wp = rec[5] + NMG_EPS, guide = q + NMG_EPS;
    prefix = -Li / wp / guide * scale;
    loss = -Li / wp * logf(guide);
  }
#pragma unroll
  for (int i = 0; i < KH; ++i) {
    const float pw = prefix * ((s.lam[i] * inv_total) * s.vmf[i] * sel);  // prefix * wv * sel
    float g0 = prefix * ((s.vmf[i] - q) * inv_total * sel) * s.lam[i];
    float g1 = pw * s.dk[i];
    float g2 = pw * s.dt[i];
    float g3 = pw * s.dp[i];
    if (!SEL) {  // train.cu:109-123 (the selection variant has no such pass)
      g0 = isfinite(g0) ? fminf(g0, 150.f) : 0.f;
      g1 = isfinite(g1) ? fminf(g1, 150.f) : 0.f;
      g2 = isfinite(g2) ? fminf(g2, 150.f) : 0.f;
      g3 = isfinite(g3) ? fminf(g3, 150.f) : 0.f;
    }
    grad[4 * i + 0] = g0;
    grad[4 * i + 1] = g1;
    grad[4 * i + 2] = g2;
    grad[4 * i + 3] = g3;
  }
  return loss;
}

}  // namespace nmg
