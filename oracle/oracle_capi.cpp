// oracle_capi.cpp -- C entry points of the CPU oracle (test infrastructure).
//
// Built into oracle/_build/libnmg_oracle.so by oracle/build_oracle.py and
// loaded with ctypes by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline. Batched loops run OpenMP-parallel over queries/samples; every
// per-element body is the scalar restatement in nmg_oracle.hpp.
//
// The network half restates, in FP64:
//   * input featurisation  -- src/render/guided/train.cu:174-191, train.h:173-177
//   * composite encoding   -- tcnn encodings/composite.h:188-199 (concatenation,
//                             the last nested encoding pads with 1.0,
//                             oneblob.h:206-209)
//   * FullyFusedMLP        -- tcnn src/fully_fused_mlp.cu (ReLU hidden layers,
//                             no output activation, row-major [out][in]
//                             weights, layout fully_fused_mlp.cu:855-864)
//   * parameter layout     -- src/render/guided/network.h:85-100 (MLP first,
//                             then the encoding's grid table)
//   * Adam and EMA         -- tcnn optimizers/adam.h:47-119, ema.h:62-75,102-145
#include "nmg_oracle.hpp"

#include <cstdio>
#include <cstdlib>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace nmgo;

struct nmgo_opts {
  int kappa_poly, expm1_norm, kappa_softplus, half_grad;
};

static Opts to_opts(const nmgo_opts* o) {
  Opts r;
  if (o) {
    r.kappa_poly = o->kappa_poly;
    r.expm1_norm = o->expm1_norm;
    r.kappa_softplus = o->kappa_softplus;
    r.half_grad = o->half_grad;
  }
  return r;
}

extern "C" int nmgo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// ------------------------------------------------------------------ mixture
template <class S>
static void sample_one(const float* raw, int K, const float* u4, const float* cos_n, const Opts& o,
                       double* dir, double* pdf, int* lobe) {
  S r[132];
  for (int i = 0; i < 4 * K; ++i) r[i] = S(raw[i]);
  Mixture<S> m;
  m.activate(r, K, o);
  if (cos_n) m.apply_cosine_lobe(V3<S>{S(cos_n[0]), S(cos_n[1]), S(cos_n[2])});
  int l = 0;
  V3<S> d = m.sample(S(u4[1]), S(u4[2]), S(u4[3]), &l);
  if (dir) {
    dir[0] = double(d.x);
    dir[1] = double(d.y);
    dir[2] = double(d.z);
  }
  if (pdf) *pdf = double(m.pdf(d, o));
  if (lobe) *lobe = l;
}

// Sample one direction per query from the activated mixture (optionally
// multiplied by the cosine lobe around cos_normal[i]) with uniforms
// u4[i] = (u_guide, u_lobe, u_dir0, u_dir1), and evaluate its pdf.
extern "C" void nmgo_mixture_sample(int fp64, const float* raw, int stride, int K, long n, const float* u4,
                         const float* cos_normal, const nmgo_opts* opts, double* dir, double* pdf,
                         int* lobe) {
  Opts o = to_opts(opts);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    const float* cn = cos_normal ? cos_normal + 3 * i : nullptr;
    if (fp64)
      sample_one<double>(raw + i * stride, K, u4 + 4 * i, cn, o, dir ? dir + 3 * i : nullptr,
                         pdf ? pdf + i : nullptr, lobe ? lobe + i : nullptr);
    else
      sample_one<float>(raw + i * stride, K, u4 + 4 * i, cn, o, dir ? dir + 3 * i : nullptr,
                        pdf ? pdf + i : nullptr, lobe ? lobe + i : nullptr);
  }
}

// Lobe-selection CDF boundaries in FP64 (for excluding queries whose uniform
// sits within a rounding distance of a boundary): returns min |u - c_j|.
extern "C" void nmgo_mixture_boundary_distance(const float* raw, int stride, int K, long n, const float* u4,
                                    const float* cos_normal, const nmgo_opts* opts, double* dist) {
  Opts o = to_opts(opts);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    double r[132];
    for (int k = 0; k < 4 * K; ++k) r[k] = raw[i * stride + k];
    Mixture<double> m;
    m.activate(r, K, o);
    if (cos_normal)
      m.apply_cosine_lobe(V3<double>{cos_normal[3 * i], cos_normal[3 * i + 1], cos_normal[3 * i + 2]});
    double c = 0, best = 1e30, u = u4[4 * i + 1];
    for (int k = 0; k < K; ++k) {
      c += m.weight[k];
      best = std::min(best, std::fabs(u - c));
    }
    dist[i] = best;
  }
}

extern "C" void nmgo_mixture_pdf(int fp64, const float* raw, int stride, int K, long n, const float* wi,
                      const float* cos_normal, const nmgo_opts* opts, double* pdf) {
  Opts o = to_opts(opts);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    if (fp64) {
      double r[132];
      for (int k = 0; k < 4 * K; ++k) r[k] = raw[i * stride + k];
      Mixture<double> m;
      m.activate(r, K, o);
      if (cos_normal)
        m.apply_cosine_lobe(V3<double>{cos_normal[3 * i], cos_normal[3 * i + 1], cos_normal[3 * i + 2]});
      pdf[i] = m.pdf(V3<double>{wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]}, o);
    } else {
      float r[132];
      for (int k = 0; k < 4 * K; ++k) r[k] = raw[i * stride + k];
      Mixture<float> m;
      m.activate(r, K, o);
      if (cos_normal)
        m.apply_cosine_lobe(V3<float>{cos_normal[3 * i], cos_normal[3 * i + 1], cos_normal[3 * i + 2]});
      pdf[i] = m.pdf(V3<float>{wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]}, o);
    }
  }
}

// KL loss and gradient w.r.t. the raw outputs for a batch of training
// samples. sample[i*sstride ...] = {theta, phi, L_r, L_g, L_b, wi_pdf[, bsdf_pdf]}
// (the GuidedOutput record, src/render/guided/guideditem.h:54-61).
// loss_scale is divided by n as in train.cu:80. grad has row stride `stride`.
// Returns the FP64 sum of the per-sample losses.
extern "C" double nmgo_mixture_loss_grad(int fp64, int selection, const float* raw, int stride, int K, long n,
                              const float* sample, int sstride, float loss_scale,
                              const nmgo_opts* opts, double* grad, double* loss) {
  Opts o = to_opts(opts);
  double total = 0;
#pragma omp parallel for schedule(static) reduction(+ : total)
  for (long i = 0; i < n; ++i) {
    const float* s = sample + i * sstride;
    int nout = 4 * K + (selection ? 1 : 0);
    double l;
    if (fp64) {
      double r[133], g[133], L[3] = {s[2], s[3], s[4]};
      for (int k = 0; k < nout; ++k) r[k] = raw[i * stride + k];
      double scale = double(loss_scale) / double(n);
      l = selection ? kl_loss_grad_selection<double>(r, K, s[0], s[1], L, s[6], scale, g, o)
                    : kl_loss_grad<double>(r, K, s[0], s[1], L, s[5], scale, g, o);
      if (grad)
        for (int k = 0; k < nout; ++k) grad[i * stride + k] = g[k];
    } else {
      float r[133], g[133], L[3] = {s[2], s[3], s[4]};
      for (int k = 0; k < nout; ++k) r[k] = raw[i * stride + k];
      float scale = loss_scale / float(n);
      l = selection ? kl_loss_grad_selection<float>(r, K, s[0], s[1], L, s[6], scale, g, o)
                    : kl_loss_grad<float>(r, K, s[0], s[1], L, s[5], scale, g, o);
      if (grad)
        for (int k = 0; k < nout; ++k) grad[i * stride + k] = g[k];
    }
    if (loss) loss[i] = l;
    total += l;
  }
  return total;
}

// ------------------------------------------------------------------ network
// Network description. Must match the host-side layout of the product's
// configuration (filled from the same Python dict in the tests).
struct nmgo_net {
  int input_mode;      // 0: 9 dims (pos, (wo+1)/2, normal theta/pi phi/2pi, 1-e^-r) -> grid|SH|OneBlob(3 dims)
                       // 1: 10 dims (pos, (wo+1)/2, (n+1)/2, 1-e^-r) -> grid|SH(wo)|SH(n)|OneBlob(1 dim)
  int grid_hash, grid_levels, grid_feats, grid_log2_T, grid_base_res;
  float grid_scale;
  int grid_smoothstep;
  int sh_degree;       // SH degree (d^2 coefficients) for wo (and n in mode 1)
  int oneblob_bins;
  int width;           // 64
  int n_hidden;        // hidden layers (3 -> 4 weight matrices)
  int n_out;           // K*4 (+1 with learned selection)
  // derived (filled by nmgo_net_init)
  int n_input, n_enc, n_enc_padded, n_out_padded;
  long n_mlp_params, n_grid_params, n_params;
  long n_entries;
  uint32_t grid_offset[33];
};

static int round16(int x) { return (x + 15) / 16 * 16; }

extern "C" int nmgo_net_init(nmgo_net* net) {
  net->n_input = net->input_mode == 0 ? 9 : 10;
  int d2 = net->sh_degree * net->sh_degree;
  int grid = net->grid_levels * net->grid_feats;
  net->n_enc = net->input_mode == 0 ? grid + d2 + 3 * net->oneblob_bins : grid + 2 * d2 + net->oneblob_bins;
  net->n_enc_padded = round16(net->n_enc);
  net->n_out_padded = round16(net->n_out);
  net->n_mlp_params = (long)net->width * net->n_enc_padded +
                      (long)(net->n_hidden - 1) * net->width * net->width +
                      (long)net->n_out_padded * net->width;
  GridSpec g;
  g.hash = net->grid_hash;
  g.levels = net->grid_levels;
  g.feats = net->grid_feats;
  g.log2_T = net->grid_log2_T;
  g.base_res = net->grid_base_res;
  g.per_level_scale = net->grid_scale;
  g.smoothstep = net->grid_smoothstep;
  grid_layout(g);
  for (int i = 0; i <= g.levels; ++i) net->grid_offset[i] = g.offset[i];
  net->n_entries = g.n_entries;
  net->n_grid_params = (long)g.n_entries * g.feats;
  net->n_params = net->n_mlp_params + net->n_grid_params;
  return 0;
}

static GridSpec grid_of(const nmgo_net* net) {
  GridSpec g;
  g.hash = net->grid_hash;
  g.levels = net->grid_levels;
  g.feats = net->grid_feats;
  g.log2_T = net->grid_log2_T;
  g.base_res = net->grid_base_res;
  g.per_level_scale = net->grid_scale;
  g.smoothstep = net->grid_smoothstep;
  grid_layout(g);
  return g;
}

// train.cu:174-191 (mode 0) and its SH-of-normal variant (mode 1): shading
// data -> network input. aabb = {min xyz, max xyz} of the scene.
extern "C" void nmgo_featurize(const nmgo_net* net, long n, const float* pos, const float* wo, const float* nrm,
                    const float* rough, const float* aabb, float* out) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    float* o = out + i * net->n_input;
    // train.h:173-177: inflate by 0.5% of the diagonal length
    float mn[3] = {aabb[0], aabb[1], aabb[2]}, mx[3] = {aabb[3], aabb[4], aabb[5]};
    V3<float> dg{mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    float infl = norm(dg) * 0.005f;
    for (int d = 0; d < 3; ++d) {
      float lo = mn[d] - infl, hi = mx[d] + infl;
      float c = (lo + hi) / 2.0f, dd = hi - lo;
      o[d] = 0.5f + (pos[3 * i + d] - c) / dd;
    }
    V3<float> w = normalized(V3<float>{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]});
    o[3] = (w.x + 1.0f) * 0.5f;
    o[4] = (w.y + 1.0f) * 0.5f;
    o[5] = (w.z + 1.0f) * 0.5f;
    V3<float> nn{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
    if (net->input_mode == 0) {
      float th, ph;
      cart_to_sph(nn, &th, &ph);
      o[6] = float(double(th) / 3.14159265358979323846);  // double M_PI, see pi_product
      o[7] = float(ph / C<float>::TWO_PI);
      o[8] = 1.0f - expf(-rough[i]);
    } else {
      V3<float> nu = normalized(nn);
      o[6] = (nu.x + 1.0f) * 0.5f;
      o[7] = (nu.y + 1.0f) * 0.5f;
      o[8] = (nu.z + 1.0f) * 0.5f;
      o[9] = 1.0f - expf(-rough[i]);
    }
  }
}

// The network forward and backward are templated on the arithmetic type S:
// double is the FP64 parity oracle, float the FP32 restatement that the CPU
// baseline times (the reference has no CPU implementation of the network).

// Composite encoding of one input row into enc[n_enc_padded].
template <class S>
static void encode_row(const nmgo_net* net, const GridSpec& g, const float* table, const float* x, S* enc) {
  grid_encode<S>(g, table, x, enc);
  int o = net->grid_levels * net->grid_feats;
  int d2 = net->sh_degree * net->sh_degree;
  S sh[16];
  sh_encode<S>(net->sh_degree, S(x[3] * 2.0f - 1.0f), S(x[4] * 2.0f - 1.0f), S(x[5] * 2.0f - 1.0f), sh);
  for (int k = 0; k < d2; ++k) enc[o + k] = sh[k];
  o += d2;
  if (net->input_mode == 0) {
    for (int d = 6; d < 9; ++d) {
      oneblob_encode<S>(net->oneblob_bins, S(x[d]), enc + o);
      o += net->oneblob_bins;
    }
  } else {
    sh_encode<S>(net->sh_degree, S(x[6] * 2.0f - 1.0f), S(x[7] * 2.0f - 1.0f), S(x[8] * 2.0f - 1.0f), sh);
    for (int k = 0; k < d2; ++k) enc[o + k] = sh[k];
    o += d2;
    oneblob_encode<S>(net->oneblob_bins, S(x[9]), enc + o);
    o += net->oneblob_bins;
  }
  for (; o < net->n_enc_padded; ++o) enc[o] = S(1);
}

// y[rows] = W[rows x cols] * x[cols]
template <class S>
static void matvec(const float* W, int rows, int cols, const S* x, S* y) {
  for (int r = 0; r < rows; ++r) {
    S acc = 0;
    for (int c = 0; c < cols; ++c) acc += S(W[(long)r * cols + c]) * x[c];
    y[r] = acc;
  }
}

template <class S>
struct Fwd {
  S enc[256];
  S h[8][128];  // hidden activations after ReLU
  S y[256];
};

template <class S>
static void forward_row(const nmgo_net* net, const GridSpec& g, const float* params, const float* x, Fwd<S>& f) {
  const float* W = params;
  const float* table = params + net->n_mlp_params;
  encode_row<S>(net, g, table, x, f.enc);
  const S* in = f.enc;
  int in_w = net->n_enc_padded;
  for (int l = 0; l < net->n_hidden; ++l) {
    matvec<S>(W, net->width, in_w, in, f.h[l]);
    for (int k = 0; k < net->width; ++k) f.h[l][k] = std::max(S(0), f.h[l][k]);
    W += (long)net->width * in_w;
    in = f.h[l];
    in_w = net->width;
  }
  matvec<S>(W, net->n_out_padded, net->width, in, f.y);
}

// Network forward: inputs [n x n_input] -> raw outputs [n x n_out_padded]
// (optionally also the encoded inputs [n x n_enc_padded]).
template <class S>
static void network_forward(const nmgo_net* net, const float* params, long n, const float* inputs, S* raw,
                            S* enc_out) {
  GridSpec g = grid_of(net);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    Fwd<S> f;
    forward_row<S>(net, g, params, inputs + i * net->n_input, f);
    for (int k = 0; k < net->n_out_padded; ++k) raw[i * net->n_out_padded + k] = f.y[k];
    if (enc_out)
      for (int k = 0; k < net->n_enc_padded; ++k) enc_out[i * net->n_enc_padded + k] = f.enc[k];
  }
}
extern "C" void nmgo_network_forward(const nmgo_net* net, const float* params, long n, const float* inputs,
                                     double* raw, double* enc_out) {
  network_forward<double>(net, params, n, inputs, raw, enc_out);
}
extern "C" void nmgo_network_forward_f32(const nmgo_net* net, const float* params, long n, const float* inputs,
                                         float* raw) {
  network_forward<float>(net, params, n, inputs, raw, nullptr);
}

// grid_backward with OpenMP atomic accumulation (same weights as the forward).
template <class S>
static void grid_backward_atomic(const GridSpec& g, const float pos[3], const S* dfeat, S* grad) {
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
      for (int f = 0; f < g.feats; ++f) {
#pragma omp atomic
        grad[idx + f] += wt * dfeat[l * g.feats + f];
      }
    }
  }
}

// Network backward: dL/draw [n x n_out_padded] -> dL/dparams (accumulated,
// same layout as params) and optionally dL/dencoded [n x n_enc_padded].
template <class S>
static void network_backward(const nmgo_net* net, const float* params, long n, const float* inputs, const S* draw,
                             S* dparams, S* denc_out) {
  GridSpec g = grid_of(net);
  int nt = nmgo_num_threads();
  // MLP gradient: per-thread partials (small); grid gradient: atomic adds
  // straight into dparams (the table is large and sparsely touched).
  std::vector<std::vector<S>> part(nt, std::vector<S>(net->n_mlp_params, S(0)));
  S* dgrid = dparams + net->n_mlp_params;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
#ifdef _OPENMP
    std::vector<S>& acc = part[omp_get_thread_num()];
#else
    std::vector<S>& acc = part[0];
#endif
    Fwd<S> f;
    const float* x = inputs + i * net->n_input;
    forward_row<S>(net, g, params, x, f);
    // weight offsets
    long off[10];
    off[0] = 0;
    int in_w = net->n_enc_padded;
    for (int l = 0; l < net->n_hidden; ++l) {
      off[l + 1] = off[l] + (long)net->width * in_w;
      in_w = net->width;
    }
    S d[256], dn[256];
    for (int k = 0; k < net->n_out_padded; ++k) d[k] = draw[i * net->n_out_padded + k];
    // output layer
    int L = net->n_hidden;
    {
      const float* W = params + off[L];
      for (int r = 0; r < net->n_out_padded; ++r)
        for (int c = 0; c < net->width; ++c) acc[off[L] + (long)r * net->width + c] += d[r] * f.h[L - 1][c];
      for (int c = 0; c < net->width; ++c) {
        S s = 0;
        for (int r = 0; r < net->n_out_padded; ++r) s += S(W[(long)r * net->width + c]) * d[r];
        dn[c] = f.h[L - 1][c] > 0 ? s : S(0);
      }
    }
    for (int l = L - 1; l >= 0; --l) {
      for (int c = 0; c < net->width; ++c) d[c] = dn[c];
      const S* in = l == 0 ? f.enc : f.h[l - 1];
      int iw = l == 0 ? net->n_enc_padded : net->width;
      const float* W = params + off[l];
      for (int r = 0; r < net->width; ++r)
        for (int c = 0; c < iw; ++c) acc[off[l] + (long)r * iw + c] += d[r] * in[c];
      for (int c = 0; c < iw; ++c) {
        S s = 0;
        for (int r = 0; r < net->width; ++r) s += S(W[(long)r * iw + c]) * d[r];
        dn[c] = (l == 0) ? s : (f.h[l - 1][c] > 0 ? s : S(0));
      }
    }
    if (denc_out)
      for (int k = 0; k < net->n_enc_padded; ++k) denc_out[i * net->n_enc_padded + k] = dn[k];
    grid_backward_atomic<S>(g, x, dn, dgrid);
  }
  for (int t = 0; t < nt; ++t)
    for (long k = 0; k < net->n_mlp_params; ++k) dparams[k] += part[t][k];
}
extern "C" void nmgo_network_backward(const nmgo_net* net, const float* params, long n, const float* inputs,
                                      const double* draw, double* dparams, double* denc_out) {
  network_backward<double>(net, params, n, inputs, draw, dparams, denc_out);
}
extern "C" void nmgo_network_backward_f32(const nmgo_net* net, const float* params, long n, const float* inputs,
                                          const float* draw, float* dparams) {
  network_backward<float>(net, params, n, inputs, draw, dparams, nullptr);
}

// Adam (adam.h:47-119) followed by EMA (ema.h:62-75,102-145) over all params.
// grad holds loss-scaled gradients; step is the optimizer's step count after
// this call (1 for the first call). Only the first n_matrix params get l2.
extern "C" void nmgo_adam_ema(long n_params, long n_matrix, const float* grad, float loss_scale, float lr,
                   float beta1, float beta2, float eps, float l2, float ema_decay, uint32_t step,
                   float* w, float* m, float* v, uint32_t* psteps, float* ema) {
  float debias_old = 1.0f - (float)std::pow((double)ema_decay, (double)(step - 1));
  float debias_new = 1.0f / (1.0f - (float)std::pow((double)ema_decay, (double)step));
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n_params; ++i) {
    float g = grad[i] / loss_scale;
    bool skip = (i >= n_matrix) && g == 0.0f;
    if (!skip) {
      float wf = w[i];
      if (i < n_matrix) g += l2 * wf;
      float mm = m[i] = beta1 * m[i] + (1.0f - beta1) * g;
      float vv = v[i] = beta2 * v[i] + (1.0f - beta2) * (g * g);
      uint32_t t = ++psteps[i];
      // adam.h:102: learning_rate *= sqrtf(1 - beta2^t) / (1 - beta1^t), the quotient first
      float lr_t = lr * (sqrtf(1.0f - powf(beta2, (float)t)) / (1.0f - powf(beta1, (float)t)));
      float eff = lr_t / (sqrtf(vv) + eps);
      w[i] = wf - eff * mm;
    }
    if (ema) ema[i] = (ema[i] * ema_decay * debias_old + w[i] * (1.0f - ema_decay)) * debias_new;
  }
}

// Grid part of the backward only: dL/d(encoded input) rows denc[n x
// n_enc_padded] (FP64) -> table gradient (accumulated into dgrid).
extern "C" void nmgo_grid_backward(const nmgo_net* net, long n, const float* inputs, const double* denc, double* dgrid) {
  GridSpec g = grid_of(net);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i)
    grid_backward_atomic<double>(g, inputs + i * net->n_input, denc + i * net->n_enc_padded, dgrid);
}
