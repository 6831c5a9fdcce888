// mixture_kernels.cu -- FP32 mixture kernels on raw network outputs and their
// C-ABI entry points (nmg_mixture_*).
//
// Sampling takes one thread per query, the pdf and the loss a lane pair per
// query (half the lobes each); lobes in registers; grid-stride loops over one
// wave of resident blocks. Each query reads its raw row directly: 32-byte
// loads (two lobes) where the rows are 32-byte aligned for sampling and the
// loss, else 16-byte loads (one lobe); its uniforms as one float4.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "api_common.cuh"
#include "mixture.cuh"

namespace nmg {

static thread_local char g_err[512] = "";

nmg_status set_error(nmg_status st, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return st;
}

constexpr int kThreads = 128;

// Hardware transcendental approximations (__expf, __fdividef, __sincosf for
// the sampled azimuth): the reference compiles all of its CUDA with
// --use_fast_math (src/backend/CMakeLists.txt:96), so its own GPU mixture
// code evaluates the same approximations. The lobe means and the record
// directions stay precise (sincospi / sincosf): their error is multiplied by
// kappa in exp(kappa (cos - 1)), up to kappa = 1000 in this workload. The
// vMF sampler keeps its accurate log1p.
constexpr bool kMixFast = true;

static int grid_for(long n) {
  long blocks = (n + kThreads - 1) / kThreads;
  long cap = 152L * 16;  // 16 resident 128-thread blocks per SM
  return int(blocks < cap ? (blocks > 0 ? blocks : 1) : cap);
}

// One wave of the blocks that fit on the device at once (the kernels loop
// over the queries with a grid stride), or fewer for small n.
template <class Kern>
static int resident_grid(Kern kernel, int smem, long n) {
  int dev = 0, sms = 152, per_sm = 1;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long blocks = (n + kThreads - 1) / kThreads, cap = long(sms) * per_sm;
  return int(blocks < cap ? (blocks > 0 ? blocks : 1) : cap);
}

// COS: with the cosine-lobe product (cosn given); without it the query takes
// the lean form (mix_activate_lean and its selection, sampler and pdf).
template <int K, bool FAST, bool COS, bool WIDE = false>
NMG_D void sample_one(const float* row, float4 u, const float* cosn, long q, int kappa_softplus, float* dir,
                      float* pdf, int* lobe) {
  if constexpr (FAST && !COS) {
    MixLean<K> m;
    mix_activate_lean<K, WIDE>(m, row, kappa_softplus);
    float k, inv;
    f3 mu;
    const int sel = mix_select_lean<K>(m, u.y, &k, &mu, &inv);
    const f3 d = vmf_sample_lean(k, mu, u.z, u.w);
    store3(dir, q, d);
    pdf[q] = mix_pdf_lean_sum<K>(m, d) * inv;
    if (lobe) lobe[q] = sel;
    return;
  }
  Mix<K> m;
  mix_activate<K, FAST, kAngTab>(m, row, kappa_softplus);
  if (cosn) mix_apply_cosine<K, FAST>(m, load3(cosn, q));
  int sel = mix_select<K>(m, u.y);
  f3 d = mix_sample_lobe<K, FAST>(m, sel, u.z, u.w);
  store3(dir, q, d);
  pdf[q] = mix_pdf<K, FAST>(m, d);
  if (lobe) lobe[q] = sel;
}

// Direct loads of each query's row and uniforms, one wave of resident blocks
// (a grid-stride loop). WIDE: 32-byte row loads (rows_32b). At K <= 8 the
// bound of 5 blocks per SM lets the lean form keep its lobes in 96 registers
// without spilling. 2,097,152 queries at K = 8: 90 us with 32-byte loads,
// 98 us with 16-byte loads (the L1 data pipe was then 73% busy with their
// wavefronts, one line per lane and load), 115 us with the rows staged in
// shared memory by per-thread cp.async copies (6 blocks per SM at 80
// registers), 108 us with 106 registers and 4 blocks.
template <int K, bool FAST, bool COS, bool WIDE = false>
__global__ void __launch_bounds__(kThreads, K <= 8 ? 5 : 1) k_mixture_sample(const float* __restrict__ raw,
                                                                             int stride,
                                                                             const float* __restrict__ u4,
                                                                             const float* __restrict__ cosn, int n,
                                                                             int kappa_softplus,
                                                                             float* __restrict__ dir,
                                                                             float* __restrict__ pdf,
                                                                             int* __restrict__ lobe) {
  sincospi_tab_fill();
  const long step = long(gridDim.x) * blockDim.x;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += step)
    sample_one<K, FAST, COS, WIDE>(raw + q * stride, reinterpret_cast<const float4*>(u4)[q], cosn, q,
                                   kappa_softplus, dir, pdf, lobe);
}

// Whether a row-major raw array can be read with 32-byte loads: rows of a
// multiple of 8 floats from a 32-byte aligned base.
static bool rows_32b(const float* raw, int stride) {
  return stride % 8 == 0 && (reinterpret_cast<uintptr_t>(raw) & 31u) == 0;
}

template <int K, bool FAST>
__global__ void __launch_bounds__(kThreads) k_mixture_pdf(const float* __restrict__ raw, int stride,
                                                          const float* __restrict__ wi,
                                                          const float* __restrict__ cosn, int n,
                                                          int kappa_softplus, float* __restrict__ pdf) {
  sincospi_tab_fill();
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    Mix<K> m;
    mix_activate<K, FAST, kAngTab>(m, raw + q * stride, kappa_softplus);
    if (cosn) mix_apply_cosine<K, FAST>(m, load3(cosn, q));
    pdf[q] = mix_pdf<K, FAST>(m, load3(wi, q));
  }
}

// Sums `v` over the block in a fixed order; the result is valid in thread 0.
__device__ __forceinline__ double block_sum_fixed(double v) {
  __shared__ double s[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) s[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < int(blockDim.x >> 5); ++w) r += s[w];
  __syncthreads();
  return r;
}

template <int K, bool SEL>
__global__ void __launch_bounds__(kThreads) k_mixture_loss_grad(const float* __restrict__ raw, int stride,
                                                                const float* __restrict__ rec, int rstride,
                                                                int n, float scale, MixOpts o,
                                                                float* __restrict__ grad,
                                                                float* __restrict__ loss,
                                                                double* __restrict__ partials) {
  sincospi_tab_fill();
  double acc = 0.0;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    float r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = j < rstride ? rec[q * rstride + j] : 0.f;
    float g[4 * K + 1];
    float l = SEL ? mix_kl_loss_grad_selection<K, kMixFast, kAngTab>(raw + q * stride, r, scale, o, g)
                  : mix_kl_loss_grad<K, kMixFast, kAngTab>(raw + q * stride, r, scale, o, g);
    float4* gr = reinterpret_cast<float4*>(grad + q * stride);
#pragma unroll
    for (int i = 0; i < K; ++i) gr[i] = make_float4(g[4 * i], g[4 * i + 1], g[4 * i + 2], g[4 * i + 3]);
    if (SEL) grad[q * stride + 4 * K] = g[4 * K];
    if (loss) loss[q] = l;
    acc += double(l);
  }
  double s = block_sum_fixed(acc);
  if (threadIdx.x == 0 && partials) partials[blockIdx.x] = s;
}

__global__ void k_sum_partials(const double* __restrict__ partials, int m, double* __restrict__ out) {
  double v = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) v += partials[i];
  double s = block_sum_fixed(v);
  if (threadIdx.x == 0) *out = s;
}

// ---------------------------------------------------------------------------
// Two threads per query (even K): lanes 2j and 2j+1 of a warp hold lobes
// [0, K/2) and [K/2, K) of query j and combine their partial sums with pair
// shuffles. Half the lobes per thread halves the registers that pin the
// occupancy of the one-thread-per-query kernels, and a warp's 128-bit loads
// cover 16 whole contiguous rows. Sums over all lobes (weights, pdf, loss)
// add the two halves' partial sums.
NMG_D unsigned pair_mask() { return 3u << ((threadIdx.x & 31) & ~1u); }
NMG_D float pair_sum(float v) { return v + __shfl_xor_sync(pair_mask(), v, 1); }

// Weights from the pair's total (after activation or the cosine product).
template <int KH, bool FAST>
NMG_D void pair_weights(Mix<KH>& m, float total) {
  m.total = total;
  const float inv = 1.f / total;
#pragma unroll
  for (int i = 0; i < KH; ++i) m.w[i] = FAST ? m.lam[i] * inv : m.lam[i] / total;
}

template <int K, bool FAST>
NMG_D void pair_mixture(Mix<K / 2>& m, const float* half_row, const float* cosn, long q, int kappa_softplus) {
  constexpr int KH = K / 2;
  mix_activate<KH, FAST, kAngTab>(m, half_row, kappa_softplus);
  float lt = 0.f;
#pragma unroll
  for (int i = 0; i < KH; ++i) lt += m.lam[i];
  pair_weights<KH, FAST>(m, pair_sum(lt));
  if (cosn) {
    mix_apply_cosine<KH, FAST>(m, load3(cosn, q));
    lt = 0.f;
#pragma unroll
    for (int i = 0; i < KH; ++i) lt += m.lam[i];
    pair_weights<KH, FAST>(m, fmaxf(pair_sum(lt), NMG_EPS));  // distribution.h:191
  }
}

// Direct loads, one wave of resident blocks. COS: with the cosine-lobe
// product; without it each lane sums lambda * vMF of its lobes in the lean
// form and the pdf is the pair's sum over the pair's total. 8 blocks per SM
// at K <= 8 (56 registers): 70 us for 2,097,152 queries at K = 8, against
// 80 us with the rows staged in shared memory by per-thread cp.async copies.
template <int K, bool FAST, bool COS>
__global__ void __launch_bounds__(kThreads, K <= 8 ? 8 : 1) k_mixture_pdf2(const float* __restrict__ raw, int stride,
                                                                         const float* __restrict__ wi,
                                                                         const float* __restrict__ cosn, int n,
                                                                         int kappa_softplus, float* __restrict__ pdf) {
  constexpr int KH = K / 2;
  const int h = threadIdx.x & 1;
  sincospi_tab_fill();
  const long step = long(gridDim.x) * blockDim.x;
  for (long t = long(blockIdx.x) * blockDim.x + threadIdx.x; (t >> 1) < n; t += step) {
    const long q = t >> 1;
    const float* half_row = raw + q * stride + h * KH * 4;
    const f3 w = load3(wi, q);
    float p;
    if constexpr (FAST && !COS) {
      MixLean<KH> m;
      mix_activate_lean<KH>(m, half_row, kappa_softplus);
      p = pair_sum(mix_pdf_lean_sum<KH>(m, w)) / pair_sum(m.total);
    } else {
      Mix<KH> m;
      pair_mixture<K, FAST>(m, half_row, cosn, q, kappa_softplus);
      p = pair_sum(mix_pdf<KH, FAST>(m, w));
    }
    if (h == 0) pdf[q] = p;
  }
}

// train.cu:69-172 with the lobes split over a lane pair: each lane computes
// its lobes' activations, vMF values and gradients; q and the total come
// from the pair's partial sums. Direct loads (WIDE: 32-byte loads of the
// half row, rows_32b); 8 blocks per SM at K <= 8 (64 registers). 2,097,152
// queries at K = 8: 152 us with 32-byte loads, 154 us with 16-byte loads,
// 178 us with the rows staged in shared memory by per-thread cp.async copies,
// 166 us at the 89 registers the compiler picks unbounded.
template <int K, bool SEL, bool WIDE = false>
__global__ void __launch_bounds__(kThreads, K <= 8 ? 8 : 1) k_mixture_loss_grad2(const float* __restrict__ raw,
                                                                               int stride,
                                                                               const float* __restrict__ rec,
                                                                               int rstride, int n, float scale,
                                                                               MixOpts o, float* __restrict__ grad,
                                                                               float* __restrict__ loss,
                                                                               double* __restrict__ partials) {
  constexpr int KH = K / 2;
  constexpr bool FAST = kMixFast;
  const int h = threadIdx.x & 1;
  sincospi_tab_fill();
  double acc = 0.0;
  const long step = long(gridDim.x) * blockDim.x;
  for (long t = long(blockIdx.x) * blockDim.x + threadIdx.x; (t >> 1) < n; t += step) {
    const long q = t >> 1;
    float r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = j < rstride ? rec[q * rstride + j] : 0.f;
    const float* row = raw + q * stride + h * KH * 4;
    float swt, cwt, swp, cwp;
    sincosf(r[0], &swt, &cwt);
    sincosf(r[1], &swp, &cwp);
    const f3 wi{swt * cwp, swt * swp, cwt};
    float lam[KH], kap[KH], dkap[KH], vmf[KH], cc[KH], dta[KH], dpa[KH], sgt[KH], sgp[KH];
    float lt = 0.f, nt = 0.f;
    float4 xw[WIDE ? KH : 1];  // WIDE: the half row in 32-byte loads (see mix_activate_lean)
    if constexpr (WIDE) {
#pragma unroll
      for (int j = 0; j < KH / 2; ++j) ld_global_v8(row + 8 * j, xw[2 * j], xw[2 * j + 1]);
    }
#pragma unroll
    for (int i = 0; i < KH; ++i) {
      const float4 x = WIDE ? xw[WIDE ? i : 0] : reinterpret_cast<const float4*>(row)[i];
      lam[i] = xexp<FAST>(act_exp_clamp(x.x));
      if (o.kappa_softplus) {
        kap[i] = softplus<FAST>(x.y);
        dkap[i] = logistic<FAST>(x.y);
      } else {
        kap[i] = xexp<FAST>(act_exp_clamp(x.y));
        dkap[i] = kap[i];  // train.h:410: the derivative ignores the clamp
      }
      sgt[i] = logistic<FAST>(x.z);
      sgp[i] = logistic<FAST>(x.w);
      float sth, cth, sph, cph;
      lobe_angles<FAST, kAngTab, false>(sgt[i], sgp[i], &sth, &cth, &sph, &cph);
      cc[i] = wi.x * sth * cph + wi.y * sth * sph + wi.z * cth;
      dta[i] = cth * (wi.x * cph + wi.y * sph) - wi.z * sth;
      dpa[i] = (wi.y * cph - wi.x * sph) * sth;
      // below M_EPSILON the lobe is uniform (vmf.h:24): kappa 0 gives e^{0} / 4pi without a branch
      const float kz = kap[i] < NMG_EPS ? 0.f : kap[i];
      vmf[i] = xexp<FAST>(kz * fminf(0.f, cc[i] - 1.f)) * vmf_norm_sel(kz);
      lt += lam[i];
      nt += lam[i] * vmf[i];
    }
    const float total = pair_sum(lt);
    const float inv_total = 1.f / total;
    const float qv = pair_sum(nt) * inv_total;
    const float Li = (r[2] + (r[3] + r[4])) / 3.f;
    float prefix, l, sel = 1.f;
    if (SEL) {
      sel = logistic<FAST>(raw[q * stride + 4 * K]);
      const float wp = sel * (qv + NMG_EPS) + (1.f - sel) * r[6];
      l = -Li / wp * logf(wp);
      prefix = -Li / wp / wp * scale;
    } else {
      const float wp = r[5] + NMG_EPS, guide = qv + NMG_EPS;
      prefix = -Li / wp / guide * scale;
      l = -Li / wp * logf(guide);
    }
    float4* gr = reinterpret_cast<float4*>(grad + q * stride) + h * KH;
#pragma unroll
    for (int i = 0; i < KH; ++i) {
      const float k = kap[i];
      const float wv = (lam[i] * inv_total) * vmf[i];
      // d log(vMF normaliser) / d kappa (distribution.h:160-172): the polynomial below kappa 1 or the
      // series below 1e-2, else 1/k - coth(k); both forms evaluated and one selected (no divergence)
      const float e = xexp<FAST>(-2.f * k);
      const float ik_exact = xdiv<FAST>(1.f, k) - xdiv<FAST>(1.f + e, 1.f - e);
      const float ik_small = o.kappa_poly ? 0.000926f + -0.344883f * k + 0.030147f * (k * k)
                                          : k * (-1.f / 3.f + k * k * (1.f / 45.f));
      const float ik = k < (o.kappa_poly ? 1.f : 1e-2f) ? ik_small : ik_exact;
      float g0 = prefix * ((vmf[i] - qv) * inv_total * sel) * lam[i];
      float g1 = prefix * (wv * (cc[i] + ik) * sel) * dkap[i];
      float g2 = prefix * (wv * k * dta[i] * sel) * NMG_PI * (sgt[i] * (1.f - sgt[i]));
      float g3 = prefix * (wv * k * dpa[i] * sel) * NMG_TWO_PI * (sgp[i] * (1.f - sgp[i]));
      if (!SEL) {  // train.cu:109-123 (the selection variant has no such pass)
        g0 = isfinite(g0) ? fminf(g0, 150.f) : 0.f;
        g1 = isfinite(g1) ? fminf(g1, 150.f) : 0.f;
        g2 = isfinite(g2) ? fminf(g2, 150.f) : 0.f;
        g3 = isfinite(g3) ? fminf(g3, 150.f) : 0.f;
      }
      gr[i] = make_float4(g0, g1, g2, g3);
    }
    if (h == 0) {
      if (SEL) grad[q * stride + 4 * K] = 0.01f * prefix * (qv - r[6]) * (sel * (1.f - sel));
      if (loss) loss[q] = l;
      acc += double(l);
    }
  }
  const double s = block_sum_fixed(acc);
  if (threadIdx.x == 0 && partials) partials[blockIdx.x] = s;
}

template <int K>
static nmg_status launch_sample(const nmg_mixture_opts* o, const float* raw, const float* u4, const float* cosn,
                                int n, float* dir, float* pdf, int* lobe, cudaStream_t st) {
  // one thread per query: splitting the lobes over a lane pair (as the loss does) measured slower here,
  // the selection and the sampling of the chosen lobe being per-query work both lanes would repeat
  if (cosn) {
    const int grid = resident_grid(k_mixture_sample<K, kMixFast, true>, 0, n);
    k_mixture_sample<K, kMixFast, true><<<grid, kThreads, 0, st>>>(raw, o->stride, u4, cosn, n, o->kappa_softplus,
                                                                   dir, pdf, lobe);
  } else if (K % 2 == 0 && rows_32b(raw, o->stride)) {
    const int grid = resident_grid(k_mixture_sample<K, kMixFast, false, K % 2 == 0>, 0, n);
    k_mixture_sample<K, kMixFast, false, K % 2 == 0><<<grid, kThreads, 0, st>>>(raw, o->stride, u4, nullptr, n,
                                                                                o->kappa_softplus, dir, pdf, lobe);
  } else {
    const int grid = resident_grid(k_mixture_sample<K, kMixFast, false>, 0, n);
    k_mixture_sample<K, kMixFast, false><<<grid, kThreads, 0, st>>>(raw, o->stride, u4, nullptr, n,
                                                                    o->kappa_softplus, dir, pdf, lobe);
  }
  return check_launch("nmg_mixture_sample");
}

template <int K>
static nmg_status launch_pdf(const nmg_mixture_opts* o, const float* raw, const float* wi, const float* cosn, int n,
                             float* pdf, cudaStream_t st) {
  if constexpr (K % 2 == 0) {
    if (cosn) {
      const int grid = resident_grid(k_mixture_pdf2<K, kMixFast, true>, 0, 2L * n);
      k_mixture_pdf2<K, kMixFast, true><<<grid, kThreads, 0, st>>>(raw, o->stride, wi, cosn, n, o->kappa_softplus,
                                                                   pdf);
    } else {
      // (the 32-byte row loads of the sampler and the loss measured 71.7 against 69.6 us here)
      const int grid = resident_grid(k_mixture_pdf2<K, kMixFast, false>, 0, 2L * n);
      k_mixture_pdf2<K, kMixFast, false><<<grid, kThreads, 0, st>>>(raw, o->stride, wi, nullptr, n,
                                                                    o->kappa_softplus, pdf);
    }
  }
  else
    k_mixture_pdf<K, kMixFast><<<grid_for(n), kThreads, 0, st>>>(raw, o->stride, wi, cosn, n, o->kappa_softplus, pdf);
  return check_launch("nmg_mixture_pdf");
}

template <int K>
static nmg_status launch_loss(const nmg_mixture_opts* o, const float* raw, const float* rec, int rstride, int n,
                              float loss_scale, float* grad, float* loss, double* loss_sum, double* partials,
                              cudaStream_t st) {
  MixOpts mo{o->kappa_softplus, o->kappa_poly, 0};
  int blocks = grid_for(n);  // the workspace holds one partial per block of this grid (at most)
  const float scale = loss_scale / float(n);
  if constexpr (K % 2 == 0) {
    if (o->selection) {
      blocks = std::min(blocks, resident_grid(k_mixture_loss_grad2<K, true>, 0, 2L * n));
      k_mixture_loss_grad2<K, true><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                 loss, loss_sum ? partials : nullptr);
    } else if ((K / 2) % 2 == 0 && rows_32b(raw, o->stride)) {
      constexpr bool W = (K / 2) % 2 == 0;
      blocks = std::min(blocks, resident_grid(k_mixture_loss_grad2<K, false, W>, 0, 2L * n));
      k_mixture_loss_grad2<K, false, W><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo,
                                                                     grad, loss, loss_sum ? partials : nullptr);
    } else {
      blocks = std::min(blocks, resident_grid(k_mixture_loss_grad2<K, false>, 0, 2L * n));
      k_mixture_loss_grad2<K, false><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                  loss, loss_sum ? partials : nullptr);
    }
  } else {
    if (o->selection)
      k_mixture_loss_grad<K, true><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                loss, loss_sum ? partials : nullptr);
    else
      k_mixture_loss_grad<K, false><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                 loss, loss_sum ? partials : nullptr);
  }
  nmg_status s = check_launch("nmg_mixture_loss_grad");
  if (s != NMG_OK || !loss_sum) return s;
  k_sum_partials<<<1, 256, 0, st>>>(partials, blocks, loss_sum);
  return check_launch("nmg_mixture_loss_grad (sum)");
}

static nmg_status check_opts(const nmg_mixture_opts* o) {
  NMG_REQUIRE(o != nullptr, "opts is NULL");
  NMG_REQUIRE(o->n_lobes == 4 || o->n_lobes == 7 || o->n_lobes == 8 || o->n_lobes == 16,
              "n_lobes=%d: compiled lobe counts are 4, 7, 8 and 16", o->n_lobes);
  NMG_REQUIRE(o->stride % 4 == 0, "stride=%d must be a multiple of 4", o->stride);
  NMG_REQUIRE(o->stride >= 4 * o->n_lobes + (o->selection ? 1 : 0), "stride=%d too small for %d lobes%s",
              o->stride, o->n_lobes, o->selection ? " + selection" : "");
  return NMG_OK;
}

}  // namespace nmg

using namespace nmg;

extern "C" {

const char* nmg_status_string(int s) {
  switch (s) {
    case NMG_OK: return "ok";
    case NMG_ERR_INVALID_ARG: return "invalid argument";
    case NMG_ERR_OOM: return "out of device memory";
    case NMG_ERR_CUDA: return "CUDA error";
    case NMG_ERR_NUMERIC: return "non-finite values";
    case NMG_ERR_TIMEOUT: return "device wait timed out";
    case NMG_ERR_UNSUPPORTED: return "unsupported configuration";
    case NMG_ERR_CAPACITY: return "size above reserved capacity";
    default: return "unknown status";
  }
}

const char* nmg_last_error(void) { return g_err; }

int nmg_version(void) { return 100; }

nmg_status nmg_mixture_sample(const nmg_mixture_opts* opts, const float* raw, const float* u4, const float* cos_normal,
                              int n, float* dir, float* pdf, int* lobe, nmg_stream stream) {
  nmg_status s = check_opts(opts);
  if (s != NMG_OK) return s;
  NMG_REQUIRE(n >= 0, "n=%d < 0", n);
  if (n == 0) return NMG_OK;
  NMG_REQUIRE(raw && u4 && dir && pdf, "raw, u4, dir and pdf must be non-NULL");
  NMG_REQUIRE(aligned16(raw) && aligned16(u4), "raw and u4 must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
#define CALL(K) launch_sample<K>(opts, raw, u4, cos_normal, n, dir, pdf, lobe, st)
  switch (opts->n_lobes) {
    case 4: return CALL(4);
    case 7: return CALL(7);
    case 8: return CALL(8);
    case 16: return CALL(16);
  }
#undef CALL
  return NMG_ERR_UNSUPPORTED;
}

nmg_status nmg_mixture_pdf(const nmg_mixture_opts* opts, const float* raw, const float* wi, const float* cos_normal,
                           int n, float* pdf, nmg_stream stream) {
  nmg_status s = check_opts(opts);
  if (s != NMG_OK) return s;
  NMG_REQUIRE(n >= 0, "n=%d < 0", n);
  if (n == 0) return NMG_OK;
  NMG_REQUIRE(raw && wi && pdf, "raw, wi and pdf must be non-NULL");
  NMG_REQUIRE(aligned16(raw), "raw must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
#define CALL(K) launch_pdf<K>(opts, raw, wi, cos_normal, n, pdf, st)
  switch (opts->n_lobes) {
    case 4: return CALL(4);
    case 7: return CALL(7);
    case 8: return CALL(8);
    case 16: return CALL(16);
  }
#undef CALL
  return NMG_ERR_UNSUPPORTED;
}

size_t nmg_mixture_loss_workspace_bytes(int n) { return sizeof(double) * size_t(grid_for(n < 1 ? 1 : n)); }

nmg_status nmg_mixture_loss_grad(const nmg_mixture_opts* opts, const float* raw, const float* record,
                                 int record_stride, int n, float loss_scale, float* grad, float* loss,
                                 double* loss_sum, void* workspace, size_t workspace_bytes, nmg_stream stream) {
  nmg_status s = check_opts(opts);
  if (s != NMG_OK) return s;
  NMG_REQUIRE(n >= 0, "n=%d < 0", n);
  NMG_REQUIRE(record_stride >= (opts->selection ? 7 : 6) && record_stride <= 8,
              "record_stride=%d: GuidedOutput rows have 6 floats (7 with selection), at most 8", record_stride);
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    if (loss_sum) NMG_CUDA_TRY(cudaMemsetAsync(loss_sum, 0, sizeof(double), st));
    return NMG_OK;
  }
  NMG_REQUIRE(raw && record && grad, "raw, record and grad must be non-NULL");
  NMG_REQUIRE(aligned16(raw) && aligned16(grad), "raw and grad must be 16-byte aligned");
  if (loss_sum) {
    NMG_REQUIRE(workspace != nullptr, "loss_sum needs a workspace");
    NMG_REQUIRE(workspace_bytes >= nmg_mixture_loss_workspace_bytes(n), "workspace_bytes=%zu < %zu", workspace_bytes,
                nmg_mixture_loss_workspace_bytes(n));
  }
#define CALL(K) launch_loss<K>(opts, raw, record, record_stride, n, loss_scale, grad, loss, loss_sum, \
                               (double*)workspace, st)
  switch (opts->n_lobes) {
    case 4: return CALL(4);
    case 7: return CALL(7);
    case 8: return CALL(8);
    case 16: return CALL(16);
  }
#undef CALL
  return NMG_ERR_UNSUPPORTED;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of nmg_mixture_loss_grad.
//
// Some callers of this library cannot hand it a scratch buffer: a renderer
// whose device memory is entirely carved into pools before the frame loop
// starts, a plugin that only ever receives raw pointers from its host and has
// no allocator of its own, or a real-time loop that cannot afford the
// device-wide synchronisation a cudaMalloc/cudaFree may cause in the middle
// of a frame. For them the FP64 loss reduction keeps its per-block partial
// sums in the fixed array below, which lives in this library's own device
// image: every GPU that loads the library holds these 64 KiB until the
// process exits. One slot per 128-sample block gives a limit of
// kNoAllocMaxSamples samples per call.
// ---------------------------------------------------------------------------
namespace nmg {
constexpr int kNoAllocSlots = 8192;                          // 64 KiB of FP64 partial sums
constexpr int kNoAllocMaxSamples = kNoAllocSlots * kThreads;  // 1,048,576 samples per call
static __device__ __align__(256) double g_noalloc_partials[kNoAllocSlots];

// Device address of g_noalloc_partials per device, looked up once per device
// (the symbol's host-side name is not a device address).
static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[128] = {};

static nmg_status noalloc_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(NMG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 128) return set_error(NMG_ERR_UNSUPPORTED, "device ordinal %d above 127", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess)
      return set_error(NMG_ERR_CUDA, "cudaGetSymbolAddress(loss scratch): %s", cudaGetErrorString(e));
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return NMG_OK;
}

template <int K>
static nmg_status launch_loss_noalloc(const nmg_mixture_opts* o, const float* raw, const float* rec, int rstride,
                                      int n, float loss_scale, float* grad, float* loss, double* loss_sum,
                                      double* partials, cudaStream_t st) {
  MixOpts mo{o->kappa_softplus, o->kappa_poly, 0};
  const int blocks = (n + kThreads - 1) / kThreads;  // one partial per block, every slot rewritten
  const float scale = loss_scale / float(n);
  // the kernels of nmg_mixture_loss_grad, so that both entry points give the same gradients
  if constexpr (K % 2 == 0) {
    if (o->selection)
      k_mixture_loss_grad2<K, true><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                 loss, loss_sum ? partials : nullptr);
    else
      k_mixture_loss_grad2<K, false><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                  loss, loss_sum ? partials : nullptr);
  } else {
    if (o->selection)
      k_mixture_loss_grad<K, true><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                loss, loss_sum ? partials : nullptr);
    else
      k_mixture_loss_grad<K, false><<<blocks, kThreads, 0, st>>>(raw, o->stride, rec, rstride, n, scale, mo, grad,
                                                                 loss, loss_sum ? partials : nullptr);
  }
  nmg_status s = check_launch("nmg_mixture_loss_grad_noalloc");
  if (s != NMG_OK || !loss_sum) return s;
  k_sum_partials<<<1, 256, 0, st>>>(partials, blocks, loss_sum);
  return check_launch("nmg_mixture_loss_grad_noalloc (sum)");
}
}  // namespace nmg

extern "C" nmg_status nmg_mixture_loss_grad_noalloc(const nmg_mixture_opts* opts, const float* raw,
                                                    const float* record, int record_stride, int n, float loss_scale,
                                                    float* grad, float* loss, double* loss_sum, nmg_stream stream) {
  nmg_status s = check_opts(opts);
  if (s != NMG_OK) return s;
  NMG_REQUIRE(n >= 0, "n=%d < 0", n);
  if (n > kNoAllocMaxSamples)
    return set_error(NMG_ERR_CAPACITY,
                     "n=%d above the %d-sample limit of nmg_mixture_loss_grad_noalloc (its fixed scratch holds "
                     "%d block sums); use nmg_mixture_loss_grad with a workspace",
                     n, kNoAllocMaxSamples, kNoAllocSlots);
  NMG_REQUIRE(record_stride >= (opts->selection ? 7 : 6) && record_stride <= 8,
              "record_stride=%d: GuidedOutput rows have 6 floats (7 with selection), at most 8", record_stride);
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    if (loss_sum) NMG_CUDA_TRY(cudaMemsetAsync(loss_sum, 0, sizeof(double), st));
    return NMG_OK;
  }
  NMG_REQUIRE(raw && record && grad, "raw, record and grad must be non-NULL");
  NMG_REQUIRE(aligned16(raw) && aligned16(grad), "raw and grad must be 16-byte aligned");
  double* partials = nullptr;
  if (loss_sum) {
    s = noalloc_scratch(&partials);
    if (s != NMG_OK) return s;
  }
  switch (opts->n_lobes) {
    case 4: return launch_loss_noalloc<4>(opts, raw, record, record_stride, n, loss_scale, grad, loss, loss_sum, partials, st);
    case 7: return launch_loss_noalloc<7>(opts, raw, record, record_stride, n, loss_scale, grad, loss, loss_sum, partials, st);
    case 8: return launch_loss_noalloc<8>(opts, raw, record, record_stride, n, loss_scale, grad, loss, loss_sum, partials, st);
    case 16: return launch_loss_noalloc<16>(opts, raw, record, record_stride, n, loss_scale, grad, loss, loss_sum, partials, st);
  }
  return NMG_ERR_UNSUPPORTED;
}
