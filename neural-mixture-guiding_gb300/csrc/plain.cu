// plain.cu -- the plain FP32 guiding step: one CUDA kernel per operation.
//
// This is the unfused baseline the fused tensor-core path is measured
// against. Every stage round-trips through HBM:
//   featurize -> encode -> linear x4 (SIMT FP32) -> mixture sample/pdf
//   train: ... -> KL loss/adjoint -> linear backward (data + weight) x4
//          -> grid scatter -> Adam+EMA
// Query counts are read from device memory (d_count, clamped to n_max), so
// every launch is shape-agnostic and capturable in a CUDA graph.
#include <math.h>
#include <stdio.h>

#include "api_common.cuh"
#include "ctx.cuh"

namespace nmg {

NMG_D int dev_count(const int* d_count, int n_max) {
  if (!d_count) return n_max;
  int n = *d_count;
  return n < 0 ? 0 : (n > n_max ? n_max : n);
}

static int blocks_for(long n, int threads, int cap_per_sm = 8) {
  long b = (n + threads - 1) / threads;
  long cap = 152L * cap_per_sm;
  return int(b < 1 ? 1 : (b > cap ? cap : b));
}

// ----------------------------------------------------------------- featurize
__global__ void k_featurize(EncodingParams e, const float* __restrict__ pos, const float* __restrict__ wo,
                            const float* __restrict__ nrm, const float* __restrict__ rough, const int* d_count,
                            int n_max, float* __restrict__ x) {
  const int n = dev_count(d_count, n_max);
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    float row[10];
    featurize(e, load3(pos, q), load3(wo, q), load3(nrm, q), rough[q], row);
    for (int d = 0; d < e.n_input; ++d) x[q * e.n_input + d] = row[d];
  }
}

// ------------------------------------------------------------------- encode
// One thread per input row: all grid levels (8 corner gathers each), SH and
// one-blob, written as one FP32 row of n_enc_pad.
__global__ void k_encode(EncodingParams e, const float* __restrict__ x, const float* __restrict__ table,
                         const int* d_count, int n_max, float* __restrict__ enc) {
  const int n = dev_count(d_count, n_max);
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    const float* xr = x + q * e.n_input;
    float* out = enc + q * e.n_enc_pad;
    const float pos[3] = {xr[0], xr[1], xr[2]};
    for (int l = 0; l < e.levels; ++l) {
      Corners c;
      level_cell(e, l, pos, c);
      float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int k = 0; k < 8; ++k) {
        uint32_t ent;
        float wt;
        corner(e, l, c, k, &ent, &wt);
        const float* t = table + size_t(ent) * e.feats;
        for (int f = 0; f < e.feats; ++f) acc[f] += wt * t[f];
      }
      for (int f = 0; f < e.feats; ++f) out[l * e.feats + f] = acc[f];
    }
    float rest[64];
    float xr10[10];
    for (int d = 0; d < e.n_input; ++d) xr10[d] = xr[d];
    encode_directional(e, xr10, rest);
    for (int k = e.levels * e.feats, j = 0; k < e.n_enc_pad; ++k, ++j) out[k] = rest[j];
  }
}

// ------------------------------------------------------------------ linear
// Y[r][j] = epi( sum_i X[r][i] * B(i, j) ) for r < count, j < nout, i < nin.
//   MODE 0 (forward):       B(i, j) = W[j][i]   (W row-major [nout][nin])
//   MODE 1 (backward data): B(i, j) = W[i][j]   (W row-major [nin][nout])
//   EPI 0: none; 1: ReLU; 2: multiply by (H[r][j] > 0)  (ReLU derivative)
// Block: 32 x (nout/8) threads, 128 rows; each thread owns 4 rows x 8 cols.
constexpr int kLinRows = 128;

template <int MODE, int EPI>
__global__ void k_linear(const float* __restrict__ X, int ldx, int nin, const float* __restrict__ W, int nout,
                         float* __restrict__ Y, int ldy, const float* __restrict__ H, int ldh, const int* d_count,
                         int n_max) {
  extern __shared__ float sm[];
  float* Bs = sm;                                   // [nin][nout]
  float* Xs = sm + nin * nout;                      // [kLinRows][nin + 1]
  const int n = dev_count(d_count, n_max);
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (int idx = tid; idx < nin * nout; idx += nthr) {
    int i = idx / nout, j = idx % nout;
    Bs[idx] = MODE == 0 ? W[j * nin + i] : W[i * nout + j];
  }
  const int cgroups = nout / 8;
  const int cg = tid % cgroups, rg = tid / cgroups;  // rg in [0, 32)
  for (long r0 = long(blockIdx.x) * kLinRows; r0 < n; r0 += long(gridDim.x) * kLinRows) {
    __syncthreads();
    for (int idx = tid; idx < kLinRows * nin; idx += nthr) {
      int r = idx / nin, i = idx % nin;
      long gr = r0 + r;
      Xs[r * (nin + 1) + i] = gr < n ? X[gr * ldx + i] : 0.f;
    }
    __syncthreads();
    float acc[4][8];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    for (int i = 0; i < nin; ++i) {
      float4 b0 = *reinterpret_cast<const float4*>(Bs + i * nout + cg * 8);
      float4 b1 = *reinterpret_cast<const float4*>(Bs + i * nout + cg * 8 + 4);
      const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        float xv = Xs[(rg + 32 * a) * (nin + 1) + i];
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(xv, bb[b], acc[a][b]);
      }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      long gr = r0 + rg + 32 * a;
      if (gr >= n) continue;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        int j = cg * 8 + b;
        float v = acc[a][b];
        if (EPI == 1) v = fmaxf(v, 0.f);
        if (EPI == 2) v = H[gr * ldh + j] > 0.f ? v : 0.f;
        Y[gr * ldy + j] = v;
      }
    }
  }
}

// dW[j][i] += sum_r D[r][j] * X[r][i] over the rows of this block's chunk,
// accumulated in registers (4x4 tile per thread) and added atomically.
constexpr int kWgRows = 32;
__global__ void k_linear_wgrad(const float* __restrict__ D, int ldd, int nout, const float* __restrict__ X, int ldx,
                               int nin, float* __restrict__ dW, const int* d_count, int n_max, int rows_per_block) {
  __shared__ float Ds[kWgRows][128 + 4];
  __shared__ float Xs[kWgRows][128 + 4];
  const int n = dev_count(d_count, n_max);
  const int jt = threadIdx.x % (nout / 4), it = threadIdx.x / (nout / 4);
  const bool active = it < nin / 4;
  float acc[4][4] = {};
  const long start = long(blockIdx.x) * rows_per_block;
  const long end = min(long(n), start + rows_per_block);
  for (long r0 = start; r0 < end; r0 += kWgRows) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < kWgRows * nout; idx += blockDim.x) {
      int r = idx / nout, j = idx % nout;
      Ds[r][j] = r0 + r < end ? D[(r0 + r) * ldd + j] : 0.f;
    }
    for (int idx = threadIdx.x; idx < kWgRows * nin; idx += blockDim.x) {
      int r = idx / nin, i = idx % nin;
      Xs[r][i] = r0 + r < end ? X[(r0 + r) * ldx + i] : 0.f;
    }
    __syncthreads();
    if (active) {
      for (int r = 0; r < kWgRows; ++r) {
        float dv[4], xv[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) dv[a] = Ds[r][jt * 4 + a];
#pragma unroll
        for (int b = 0; b < 4; ++b) xv[b] = Xs[r][it * 4 + b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(dv[a], xv[b], acc[a][b]);
      }
    }
  }
  if (active && start < end) {
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) atomicAdd(&dW[(jt * 4 + a) * nin + it * 4 + b], acc[a][b]);
  }
}

// ----------------------------------------------------------------- mixture
NMG_D f3 face_forward(f3 n, f3 v) { return dot3(n, v) > 0.f ? n : f3{-n.x, -n.y, -n.z}; }

template <int K>
__global__ void __launch_bounds__(128) k_query_mixture(const float* __restrict__ raw, int stride,
                                                       const float* __restrict__ nrm, const float* __restrict__ wo,
                                                       const float* __restrict__ u4, MixOpts o, const int* d_count,
                                                       int n_max, float* __restrict__ dir, float* __restrict__ pdf,
                                                       int* __restrict__ lobe, float* __restrict__ sel, int has_sel) {
  const int n = dev_count(d_count, n_max);
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    const float* r = raw + q * stride;
    Mix<K> m;
    mix_activate<K, false>(m, r, o.kappa_softplus);
    if (o.cosine) mix_apply_cosine<K, false>(m, face_forward(load3(nrm, q), load3(wo, q)));
    float4 u = reinterpret_cast<const float4*>(u4)[q];
    int s = mix_select<K>(m, u.y);
    f3 d = mix_sample_lobe<K, false>(m, s, u.z, u.w);
    store3(dir, q, d);
    pdf[q] = mix_pdf<K, false>(m, d);
    if (lobe) lobe[q] = s;
    if (sel && has_sel) sel[q] = logistic<false>(r[4 * K]);
  }
}

template <int K>
__global__ void __launch_bounds__(128) k_pdf_mixture(const float* __restrict__ raw, int stride,
                                                     const float* __restrict__ nrm, const float* __restrict__ wo,
                                                     const float* __restrict__ wi, MixOpts o, const int* d_count,
                                                     int n_max, float* __restrict__ pdf) {
  const int n = dev_count(d_count, n_max);
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    Mix<K> m;
    mix_activate<K, false>(m, raw + q * stride, o.kappa_softplus);
    if (o.cosine) mix_apply_cosine<K, false>(m, face_forward(load3(nrm, q), load3(wo, q)));
    pdf[q] = mix_pdf<K, false>(m, load3(wi, q));
  }
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < int(blockDim.x >> 5); ++w) r += s[w];
  return r;
}

template <int K, bool SEL>
__global__ void __launch_bounds__(128) k_train_loss(const float* __restrict__ raw, int stride,
                                                    const float* __restrict__ rec, int rstride, MixOpts o,
                                                    float loss_scale, const int* d_count, int n_max,
                                                    float* __restrict__ draw, double* __restrict__ partials) {
  const int n = dev_count(d_count, n_max);
  const float scale = n > 0 ? loss_scale / float(n) : 0.f;
  double acc = 0.0;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    float r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = j < rstride ? rec[q * rstride + j] : 0.f;
    float g[4 * K + 1];
    float l = SEL ? mix_kl_loss_grad_selection<K, false>(raw + q * stride, r, scale, o, g)
                  : mix_kl_loss_grad<K, false>(raw + q * stride, r, scale, o, g);
    float* gr = draw + q * stride;
    for (int j = 0; j < stride; ++j) gr[j] = j < 4 * K + (SEL ? 1 : 0) ? g[j] : 0.f;
    acc += double(l);
  }
  double s = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// ------------------------------------------------------------- grid backward
// grid.h:387-510: scatter dL/dfeature x interpolation weight into the table
// gradient (FP32 atomics). denc rows hold dL/d(encoded input).
__global__ void k_grid_backward(EncodingParams e, const float* __restrict__ x, const float* __restrict__ denc,
                                int ld, const int* d_count, int n_max, float* __restrict__ gtable) {
  const int n = dev_count(d_count, n_max);
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    const float* xr = x + q * e.n_input;
    const float pos[3] = {xr[0], xr[1], xr[2]};
    for (int l = 0; l < e.levels; ++l) {
      Corners c;
      level_cell(e, l, pos, c);
      float g[8];
      for (int f = 0; f < e.feats; ++f) g[f] = denc[q * ld + l * e.feats + f];
      for (int k = 0; k < 8; ++k) {
        uint32_t ent;
        float wt;
        corner(e, l, c, k, &ent, &wt);
        for (int f = 0; f < e.feats; ++f) atomicAdd(gtable + size_t(ent) * e.feats + f, wt * g[f]);
      }
    }
  }
}

// ---------------------------------------------------------------- optimiser
// A training step whose device count is zero takes no optimiser step (the
// reference's training loop stops before a batch below its minimum size,
// integrator.cpp:670-671): the step counter, Adam and the EMA leave the
// parameters and the optimiser state as they are.
__global__ void k_step_inc(uint32_t* step, const int* d_count) {
  if (d_count && *d_count <= 0) return;
  *step += 1;
}

// adam.h:47-119 + ema.h:62-75/102-145 in one pass over four parameters per
// thread (128-bit loads and stores); also writes the reduced-precision copies
// of the training and inference weights and FP64 partial sums of the squared
// unscaled gradient. Bias corrections beta^t use exp2(t log2 beta) with the
// logarithms computed once on the host (adam.h:103 evaluates powf per
// parameter). Requires n_params and n_matrix to be multiples of 4 (layer
// widths are multiples of 16).
struct AdamArgs {
  long n4;               // n_params / 4
  long n_matrix;         // parameters that get l2 and never skip
  float loss_scale, lr, beta1, beta2, eps, l2, ema_decay;
  float log2_beta1, log2_beta2, log2_decay;
  int use_ema, fp16;
};

NMG_D uint32_t pack16(float a, float b, int fp16) {
  if (fp16) return uint32_t(__half_as_ushort(__float2half_rn(a))) | (uint32_t(__half_as_ushort(__float2half_rn(b))) << 16);
  return uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(a))) |
         (uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(b))) << 16);
}

template <bool HALF16>
__global__ void __launch_bounds__(256) k_adam_ema(AdamArgs a, const float4* __restrict__ grad,
                                                  const uint32_t* __restrict__ d_step, float4* __restrict__ w,
                                                  float4* __restrict__ m, float4* __restrict__ v,
                                                  uint4* __restrict__ psteps, float4* __restrict__ w_inf,
                                                  uint2* __restrict__ w16, uint2* __restrict__ w16_inf,
                                                  double* __restrict__ partials, const int* __restrict__ d_count) {
  if (d_count && *d_count <= 0) return;  // an empty batch takes no step (see k_step_inc)
  const uint32_t step = *d_step;
  const float debias_old = 1.f - exp2f(float(step - 1) * a.log2_decay);
  const float debias_new = 1.f / (1.f - exp2f(float(step) * a.log2_decay));
  const bool separate_inf = w_inf != w;
  // squared-gradient sum: FP32 within each group of four (the FP64 pipe of
  // this GPU is narrow), FP64 across groups and threads
  double gn = 0.0;
  for (long j = long(blockIdx.x) * blockDim.x + threadIdx.x; j < a.n4; j += long(gridDim.x) * blockDim.x) {
    const bool matrix = 4 * j < a.n_matrix;
    const float4 g4 = grad[j];
    float gg[4] = {g4.x / a.loss_scale, g4.y / a.loss_scale, g4.z / a.loss_scale, g4.w / a.loss_scale};
    float4 w4 = w[j];
    float ww[4] = {w4.x, w4.y, w4.z, w4.w};
    bool any = matrix;
    float g2 = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      g2 = fmaf(gg[k], gg[k], g2);
      any |= gg[k] != 0.f;
    }
    gn += double(g2);
    if (any) {
      float4 m4 = m[j], v4 = v[j];
      uint4 t4 = psteps[j];
      float mm[4] = {m4.x, m4.y, m4.z, m4.w}, vv[4] = {v4.x, v4.y, v4.z, v4.w};
      uint32_t tt[4] = {t4.x, t4.y, t4.z, t4.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (!matrix && gg[k] == 0.f) continue;  // non-matrix parameters without gradient keep their state
        float g = gg[k];
        if (matrix) g += a.l2 * ww[k];
        mm[k] = a.beta1 * mm[k] + (1.f - a.beta1) * g;
        vv[k] = a.beta2 * vv[k] + (1.f - a.beta2) * (g * g);
        const uint32_t t = ++tt[k];
        // adam.h:102: the bias-correction quotient first, then the learning rate
        const float lr_t = a.lr * (sqrtf(1.f - exp2f(float(t) * a.log2_beta2)) / (1.f - exp2f(float(t) * a.log2_beta1)));
        ww[k] = ww[k] - lr_t / (sqrtf(vv[k]) + a.eps) * mm[k];
      }
      m[j] = make_float4(mm[0], mm[1], mm[2], mm[3]);
      v[j] = make_float4(vv[0], vv[1], vv[2], vv[3]);
      psteps[j] = make_uint4(tt[0], tt[1], tt[2], tt[3]);
      w[j] = make_float4(ww[0], ww[1], ww[2], ww[3]);
    }
    float wv[4] = {ww[0], ww[1], ww[2], ww[3]};
    if (a.use_ema) {
      const float4 e4 = w_inf[j];
      const float ee[4] = {e4.x, e4.y, e4.z, e4.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) wv[k] = (ee[k] * a.ema_decay * debias_old + ww[k] * (1.f - a.ema_decay)) * debias_new;
      w_inf[j] = make_float4(wv[0], wv[1], wv[2], wv[3]);
    } else if (separate_inf) {
      w_inf[j] = make_float4(ww[0], ww[1], ww[2], ww[3]);
    }
    if (HALF16) {
      w16[j] = make_uint2(pack16(ww[0], ww[1], a.fp16), pack16(ww[2], ww[3], a.fp16));
      w16_inf[j] = make_uint2(pack16(wv[0], wv[1], a.fp16), pack16(wv[2], wv[3], a.fp16));
    }
  }
  double s = block_sum(gn);
  if (threadIdx.x == 0 && partials) partials[blockIdx.x] = s;
}

// stats[0] = sum(loss partials) / n; stats[1] = sqrt(sum(grad-norm partials)).
// One block of kStatsThreads; the loads are unrolled so that each thread has
// its few partials in flight at once (a serial loop waited ~10 us on them).
constexpr int kStatsThreads = 1024;
__global__ void __launch_bounds__(kStatsThreads) k_finish_stats(const double* __restrict__ lp, int nl,
                                                                const double* __restrict__ gp, int ng,
                                                                const int* d_count, int n_max,
                                                                double* __restrict__ stats) {
  const int n = dev_count(d_count, n_max);
  double a = 0.0, b = 0.0;
#pragma unroll 4
  for (int i = threadIdx.x; i < nl; i += kStatsThreads) a += lp[i];
#pragma unroll 4
  for (int i = threadIdx.x; i < ng; i += kStatsThreads) b += gp[i];
  double sa = block_sum(a);
  double sb = block_sum(b);
  if (threadIdx.x == 0) {  // an empty batch ran no Adam pass: its gradient-norm partials are stale
    stats[0] = n > 0 ? sa / double(n) : 0.0;
    stats[1] = n > 0 ? sqrt(sb) : 0.0;
  }
}

// Counter-based uniform in [0,1) for parameter initialisation (splitmix64).
NMG_D float hash_uniform(uint64_t seed, uint64_t i) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + i * 0xBF58476D1CE4E5B9ull + 0x94D049BB133111EBull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return float(z >> 40) * (1.0f / 16777216.0f);
}

__global__ void k_init_params(Layout lay, uint32_t seed, float* __restrict__ w) {
  for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < lay.n_params; i += long(gridDim.x) * blockDim.x) {
    float u = hash_uniform(seed, uint64_t(i));
    float bound = 1e-4f;  // grid.h:1333-1336
    for (int l = 0; l < lay.n_layers; ++l)
      if (i >= lay.off[l] && i < lay.off[l + 1]) bound = sqrtf(6.f / float(lay.in[l] + lay.out[l]));
    w[i] = (2.f * u - 1.f) * bound;
  }
}

// ------------------------------------------------------------ host launchers
static nmg_status launch_linear(int mode, int epi, const float* X, int ldx, int nin, const float* W, int nout,
                                float* Y, int ldy, const float* H, int ldh, const int* d_count, int n_max,
                                cudaStream_t st) {
  if (nout % 8 != 0 || nout > 256) return set_error(NMG_ERR_UNSUPPORTED, "linear: nout=%d", nout);
  size_t smem = sizeof(float) * (size_t(nin) * nout + size_t(kLinRows) * (nin + 1));
  int threads = 32 * (nout / 8);
  int blocks = blocks_for(n_max, kLinRows, 4);
#define L(M, E)                                                                                           \
  do {                                                                                                    \
    auto kern = k_linear<M, E>;                                                                           \
    nmg_status s_ = ensure_smem(reinterpret_cast<const void*>(kern), smem);                              \
    if (s_ != NMG_OK) return s_;                                                                          \
    kern<<<blocks, threads, smem, st>>>(X, ldx, nin, W, nout, Y, ldy, H, ldh, d_count, n_max);            \
  } while (0)
  if (mode == 0 && epi == 0) L(0, 0);
  else if (mode == 0 && epi == 1) L(0, 1);
  else if (mode == 1 && epi == 0) L(1, 0);
  else L(1, 2);
#undef L
  return check_launch("k_linear");
}

static nmg_status launch_wgrad(const float* D, int ldd, int nout, const float* X, int ldx, int nin, float* dW,
                               const int* d_count, int n_max, cudaStream_t st) {
  if (nout % 4 || nin % 4 || nout > 128 || nin > 128 || (nout / 4) * (nin / 4) > 1024)
    return set_error(NMG_ERR_UNSUPPORTED, "wgrad: %d x %d", nout, nin);
  int rows_per_block = 2048;
  int blocks = (n_max + rows_per_block - 1) / rows_per_block;
  if (blocks < 1) blocks = 1;
  int threads = ((nout / 4) * (nin / 4) + 31) / 32 * 32;
  k_linear_wgrad<<<blocks, threads, 0, st>>>(D, ldd, nout, X, ldx, nin, dW, d_count, n_max, rows_per_block);
  return check_launch("k_linear_wgrad");
}

nmg_status plain_featurize(nmg_ctx* c, const nmg_shading* in, const int* d_count, int n_max, float* x,
                           cudaStream_t st) {
  k_featurize<<<blocks_for(n_max, 128, 16), 128, 0, st>>>(c->enc, in->pos, in->wo, in->normal, in->roughness,
                                                          d_count, n_max, x);
  return check_launch("k_featurize");
}

// Encode + MLP forward. With keep_hidden the per-layer activations stay in
// the workspace for the backward pass.
nmg_status plain_forward(nmg_ctx* c, const float* x, const int* d_count, int n_max, const float* weights,
                         bool keep_hidden, float* raw_out, cudaStream_t st) {
  const Layout& L = c->lay;
  Workspace& w = c->ws;
  k_encode<<<blocks_for(n_max, 128, 16), 128, 0, st>>>(c->enc, x, weights + L.n_mlp, d_count, n_max, w.enc);
  NMG_TRY(check_launch("k_encode"));
  const float* in = w.enc;
  int ldin = c->enc.n_enc_pad;
  for (int l = 0; l < L.n_layers; ++l) {
    const bool last = l == L.n_layers - 1;
    float* out = last ? raw_out : w.h[keep_hidden ? l : (l & 1)];
    int ldo = last ? L.n_out_pad : kWidth;
    NMG_TRY(launch_linear(0, last ? 0 : 1, in, ldin, L.in[l], weights + L.off[l], L.out[l], out, ldo, nullptr, 0,
                          d_count, n_max, st));
    in = out;
    ldin = ldo;
  }
  return NMG_OK;
}

template <int K>
static void launch_query_mix(nmg_ctx* c, const float* raw, const nmg_shading* in, const float* u4, const int* d_count,
                             int n_max, const nmg_query_out* out, cudaStream_t st) {
  k_query_mixture<K><<<blocks_for(n_max, 128, 16), 128, 0, st>>>(raw, c->lay.n_out_pad, in->normal, in->wo, u4, c->mix,
                                                                 d_count, n_max, out->dir, out->pdf, out->lobe,
                                                                 out->selection, c->cfg.selection);
}

nmg_status plain_query(nmg_ctx* c, const nmg_shading* in, const float* u4, const int* d_count, int n_max,
                       const nmg_query_out* out, cudaStream_t st) {
  Workspace& w = c->ws;
  NMG_TRY(plain_featurize(c, in, d_count, n_max, w.x, st));
  float* raw = out->raw ? out->raw : w.raw;
  NMG_TRY(plain_forward(c, w.x, d_count, n_max, c->w_inf, false, raw, st));
  switch (c->lay.K) {
    case 7: launch_query_mix<7>(c, raw, in, u4, d_count, n_max, out, st); break;
    case 8: launch_query_mix<8>(c, raw, in, u4, d_count, n_max, out, st); break;
    case 16: launch_query_mix<16>(c, raw, in, u4, d_count, n_max, out, st); break;
    default: return set_error(NMG_ERR_UNSUPPORTED, "K=%d", c->lay.K);
  }
  return check_launch("k_query_mixture");
}

nmg_status pdf_from_raw(nmg_ctx* c, const float* raw, const nmg_shading* in, const float* wi, const int* d_count,
                        int n_max, float* pdf, cudaStream_t st) {
  const int b = blocks_for(n_max, 128, 16);
  const int sd = c->lay.n_out_pad;
  switch (c->lay.K) {
    case 7: k_pdf_mixture<7><<<b, 128, 0, st>>>(raw, sd, in->normal, in->wo, wi, c->mix, d_count, n_max, pdf); break;
    case 8: k_pdf_mixture<8><<<b, 128, 0, st>>>(raw, sd, in->normal, in->wo, wi, c->mix, d_count, n_max, pdf); break;
    case 16: k_pdf_mixture<16><<<b, 128, 0, st>>>(raw, sd, in->normal, in->wo, wi, c->mix, d_count, n_max, pdf); break;
    default: return set_error(NMG_ERR_UNSUPPORTED, "K=%d", c->lay.K);
  }
  return check_launch("k_pdf_mixture");
}

nmg_status plain_pdf(nmg_ctx* c, const nmg_shading* in, const float* wi, const int* d_count, int n_max, float* pdf,
                     cudaStream_t st) {
  Workspace& w = c->ws;
  NMG_TRY(plain_featurize(c, in, d_count, n_max, w.x, st));
  NMG_TRY(plain_forward(c, w.x, d_count, n_max, c->w_inf, false, w.raw, st));
  return pdf_from_raw(c, w.raw, in, wi, d_count, n_max, pdf, st);
}

// Backward through the MLP and the grid from dL/draw held in w.draw; adds
// into dparams (layout of the parameters).
static nmg_status plain_backward(nmg_ctx* c, const float* x, const int* d_count, int n_max, const float* weights,
                                 float* dparams, cudaStream_t st) {
  const Layout& L = c->lay;
  Workspace& w = c->ws;
  const float* delta = w.draw;
  int ldd = L.n_out_pad;
  int ping = 0;
  for (int l = L.n_layers - 1; l >= 0; --l) {
    const float* in = l == 0 ? w.enc : w.h[l - 1];
    int ldin = l == 0 ? c->enc.n_enc_pad : kWidth;
    NMG_TRY(launch_wgrad(delta, ldd, L.out[l], in, ldin, L.in[l], dparams + L.off[l], d_count, n_max, st));
    // dL/d(input of layer l) = delta . W_l, masked by ReLU'(input) for hidden inputs
    float* dnext = w.dh[ping];
    NMG_TRY(launch_linear(1, l == 0 ? 0 : 2, delta, ldd, L.out[l], weights + L.off[l], L.in[l], dnext, L.in[l],
                          l == 0 ? nullptr : w.h[l - 1], kWidth, d_count, n_max, st));
    delta = dnext;
    ldd = L.in[l];
    ping ^= 1;
  }
  k_grid_backward<<<blocks_for(n_max, 128, 16), 128, 0, st>>>(c->enc, x, delta, c->enc.n_enc_pad, d_count, n_max,
                                                              dparams + L.n_mlp);
  return check_launch("k_grid_backward");
}

nmg_status optimizer_step(nmg_ctx* c, const int* d_count, int n_max, double* stats, cudaStream_t st) {
  const Layout& L = c->lay;
  const nmg_config& g = c->cfg;
  k_step_inc<<<1, 1, 0, st>>>(c->d_step, d_count);
  const int nb = 152 * 8;
  double* gp = c->ws.partials + c->ws.n_partials / 2;
  if (L.n_params % 4 || L.n_mlp % 4) return set_error(NMG_ERR_UNSUPPORTED, "parameter count not a multiple of 4");
  AdamArgs aa;
  aa.n4 = L.n_params / 4;
  aa.n_matrix = L.n_mlp;
  aa.loss_scale = g.loss_scale;
  aa.lr = g.learning_rate;
  aa.beta1 = g.beta1;
  aa.beta2 = g.beta2;
  aa.eps = g.epsilon;
  aa.l2 = g.l2_reg;
  aa.ema_decay = g.ema_decay;
  aa.log2_beta1 = log2f(g.beta1);
  aa.log2_beta2 = log2f(g.beta2);
  aa.log2_decay = log2f(g.ema_decay);
  aa.use_ema = g.use_ema;
  aa.fp16 = g.path == NMG_PATH_FP16;
  if (c->w16)
    k_adam_ema<true><<<nb, 256, 0, st>>>(aa, reinterpret_cast<const float4*>(c->grad), c->d_step,
                                         reinterpret_cast<float4*>(c->w), reinterpret_cast<float4*>(c->m),
                                         reinterpret_cast<float4*>(c->v), reinterpret_cast<uint4*>(c->psteps),
                                         reinterpret_cast<float4*>(c->w_inf), reinterpret_cast<uint2*>(c->w16),
                                         reinterpret_cast<uint2*>(c->w16_inf), gp, d_count);
  else
    k_adam_ema<false><<<nb, 256, 0, st>>>(aa, reinterpret_cast<const float4*>(c->grad), c->d_step,
                                          reinterpret_cast<float4*>(c->w), reinterpret_cast<float4*>(c->m),
                                          reinterpret_cast<float4*>(c->v), reinterpret_cast<uint4*>(c->psteps),
                                          reinterpret_cast<float4*>(c->w_inf), nullptr, nullptr, gp, d_count);
  NMG_TRY(check_launch("k_adam_ema"));
  if (stats) {
    k_finish_stats<<<1, kStatsThreads, 0, st>>>(c->ws.partials, c->ws.n_partials / 2, gp, nb, d_count, n_max,
                                                stats);
    NMG_TRY(check_launch("k_finish_stats"));
  }
  return NMG_OK;
}

nmg_status plain_train_step(nmg_ctx* c, const float* x, const float* rec, const int* d_count, int n_max,
                            double* stats, cudaStream_t st) {
  const Layout& L = c->lay;
  Workspace& w = c->ws;
  NMG_TRY(plain_forward(c, x, d_count, n_max, c->w, true, w.raw, st));
  const int lb = blocks_for(n_max, 128, 4);
  if (lb > w.n_partials / 2) return set_error(NMG_ERR_CAPACITY, "loss partials");
  cudaMemsetAsync(w.partials, 0, sizeof(double) * (w.n_partials / 2), st);
#define LOSS(KK)                                                                                                  \
  if (c->cfg.selection)                                                                                           \
    k_train_loss<KK, true><<<lb, 128, 0, st>>>(w.raw, L.n_out_pad, rec, L.record_floats, c->mix, c->cfg.loss_scale, \
                                               d_count, n_max, w.draw, w.partials);                              \
  else                                                                                                            \
    k_train_loss<KK, false><<<lb, 128, 0, st>>>(w.raw, L.n_out_pad, rec, L.record_floats, c->mix,                  \
                                                c->cfg.loss_scale, d_count, n_max, w.draw, w.partials);
  switch (L.K) {
    case 7: LOSS(7) break;
    case 8: LOSS(8) break;
    case 16: LOSS(16) break;
    default: return set_error(NMG_ERR_UNSUPPORTED, "K=%d", L.K);
  }
#undef LOSS
  NMG_TRY(check_launch("k_train_loss"));
  NMG_CUDA_TRY(cudaMemsetAsync(c->grad, 0, sizeof(float) * L.n_params, st));
  NMG_TRY(plain_backward(c, x, d_count, n_max, c->w, c->grad, st));
  return optimizer_step(c, d_count, n_max, stats, st);
}

// Network VJP at the training weights: draw given, accumulate unscaled
// dL/dparams.
nmg_status plain_vjp(nmg_ctx* c, const float* x, const float* draw, int n, float* raw, float* dparams,
                     cudaStream_t st) {
  const Layout& L = c->lay;
  Workspace& w = c->ws;
  NMG_TRY(plain_forward(c, x, nullptr, n, c->w, true, raw ? raw : w.raw, st));
  NMG_CUDA_TRY(cudaMemcpyAsync(w.draw, draw, sizeof(float) * size_t(n) * L.n_out_pad, cudaMemcpyDeviceToDevice, st));
  return plain_backward(c, x, nullptr, n, c->w, dparams, st);
}

nmg_status init_params(nmg_ctx* c, uint32_t seed, cudaStream_t st) {
  k_init_params<<<152 * 8, 256, 0, st>>>(c->lay, seed, c->w);
  return check_launch("k_init_params");
}

__global__ void k_sync_copies(long n, const float* __restrict__ w, const float* __restrict__ wi,
                              uint16_t* __restrict__ w16, uint16_t* __restrict__ w16i, int fp16) {
  for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    w16[i] = fp16 ? __half_as_ushort(__float2half_rn(w[i])) : __bfloat16_as_ushort(__float2bfloat16_rn(w[i]));
    w16i[i] = fp16 ? __half_as_ushort(__float2half_rn(wi[i])) : __bfloat16_as_ushort(__float2bfloat16_rn(wi[i]));
  }
}

// Refreshes the reduced-precision weight copies from the FP32 ones.
nmg_status sync_copies(nmg_ctx* c, cudaStream_t st) {
  if (!c->w16) return NMG_OK;
  k_sync_copies<<<152 * 8, 256, 0, st>>>(c->lay.n_params, c->w, c->w_inf, c->w16, c->w16_inf,
                                         c->cfg.path == NMG_PATH_FP16);
  NMG_TRY(check_launch("k_sync_copies"));
  return pack_images(c, st);
}

}  // namespace nmg
