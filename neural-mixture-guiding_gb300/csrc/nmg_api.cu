// nmg_api.cu -- C ABI of the network-backed guiding field: configuration,
// device state, workspace reservation and dispatch to the plain FP32 or the
// fused tensor-core path.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "api_common.cuh"
#include "ctx.cuh"

namespace nmg {

static int round16(int x) { return (x + 15) / 16 * 16; }

// grid.h:195-204 and 957-997: per-level scale/resolution and table sizes,
// evaluated on the host once.
static void grid_geometry(const nmg_config& c, EncodingParams& e, long* n_entries) {
  const float l2s = log2f(c.grid_per_level_scale);
  uint32_t off = 0;
  for (int l = 0; l < c.grid_levels; ++l) {
    float scale = exp2f(float(l) * l2s) * float(c.grid_base_resolution) - 1.0f;
    uint32_t res = uint32_t(ceilf(scale)) + 1u;
    uint32_t maxp = 0xffffffffu / 2;
    uint32_t p = powf(float(res), 3.0f) > float(maxp) ? maxp : res * res * res;
    p = (p + 7u) / 8u * 8u;
    if (c.grid_hash) p = p < (1u << c.grid_log2_hashmap) ? p : (1u << c.grid_log2_hashmap);
    e.scale[l] = scale;
    e.res[l] = res;
    e.offset[l] = off;
    off += p;
  }
  e.offset[c.grid_levels] = off;
  *n_entries = off;
}

static nmg_status validate(const nmg_config& c) {
  NMG_REQUIRE(c.n_lobes == 7 || c.n_lobes == 8 || c.n_lobes == 16, "n_lobes=%d: compiled for 7, 8 and 16",
              c.n_lobes);
  NMG_REQUIRE(c.input_mode == 0 || c.input_mode == 1, "input_mode=%d", c.input_mode);
  NMG_REQUIRE(c.grid_levels >= 1 && c.grid_levels <= kMaxLevels, "grid_levels=%d (1..%d)", c.grid_levels,
              kMaxLevels);
  NMG_REQUIRE(c.grid_features == 1 || c.grid_features == 2 || c.grid_features == 4 || c.grid_features == 8,
              "grid_features=%d", c.grid_features);
  NMG_REQUIRE(c.grid_log2_hashmap >= 4 && c.grid_log2_hashmap <= 26, "grid_log2_hashmap=%d", c.grid_log2_hashmap);
  NMG_REQUIRE(c.grid_base_resolution >= 2, "grid_base_resolution=%d", c.grid_base_resolution);
  NMG_REQUIRE(c.grid_per_level_scale >= 1.0f && c.grid_per_level_scale <= 4.0f, "grid_per_level_scale");
  NMG_REQUIRE(c.sh_degree >= 1 && c.sh_degree <= 4, "sh_degree=%d (1..4)", c.sh_degree);
  NMG_REQUIRE(c.oneblob_bins >= 1 && c.oneblob_bins <= 16, "oneblob_bins=%d", c.oneblob_bins);
  NMG_REQUIRE(c.width == kWidth, "width=%d: only 64 is compiled", c.width);
  NMG_REQUIRE(c.hidden_layers >= 1 && c.hidden_layers <= kMaxLayers - 1, "hidden_layers=%d", c.hidden_layers);
  NMG_REQUIRE(c.path >= NMG_PATH_FP32 && c.path <= NMG_PATH_FP16, "path=%d", c.path);
  NMG_REQUIRE(c.aabb[3] > c.aabb[0] && c.aabb[4] > c.aabb[1] && c.aabb[5] > c.aabb[2], "empty aabb");
  NMG_REQUIRE(c.loss_scale > 0.f, "loss_scale must be positive");
  return NMG_OK;
}

static nmg_status derive(const nmg_config& c, EncodingParams& e, Layout& L) {
  nmg_status s = validate(c);
  if (s != NMG_OK) return s;
  memset(&e, 0, sizeof(e));
  e.input_mode = c.input_mode;
  e.n_input = c.input_mode == 0 ? 9 : 10;
  e.grid_hash = c.grid_hash;
  e.levels = c.grid_levels;
  e.feats = c.grid_features;
  e.smoothstep = c.grid_smoothstep;
  e.sh_degree = c.sh_degree;
  e.oneblob_bins = c.oneblob_bins;
  const int d2 = c.sh_degree * c.sh_degree;
  const int grid = c.grid_levels * c.grid_features;
  e.n_enc = c.input_mode == 0 ? grid + d2 + 3 * c.oneblob_bins : grid + 2 * d2 + c.oneblob_bins;
  e.n_enc_pad = round16(e.n_enc);
  NMG_REQUIRE(e.n_enc_pad <= 128, "encoded width %d above 128", e.n_enc_pad);
  NMG_REQUIRE(e.n_enc_pad - grid <= 64, "non-grid encoded width above 64");
  for (int i = 0; i < 6; ++i) e.aabb[i] = c.aabb[i];
  {  // inflated box (train.h:173-177), same float expressions as the device code
    const float dx = c.aabb[3] - c.aabb[0], dy = c.aabb[4] - c.aabb[1], dz = c.aabb[5] - c.aabb[2];
    const float infl = sqrtf(dx * dx + (dy * dy + dz * dz)) * 0.005f;
    for (int d = 0; d < 3; ++d) {
      const float lo = c.aabb[d] - infl, hi = c.aabb[d + 3] + infl;
      e.center[d] = (lo + hi) / 2.f;
      e.inv_size[d] = 1.f / (hi - lo);
    }
  }
  long n_entries = 0;
  grid_geometry(c, e, &n_entries);
  memset(&L, 0, sizeof(L));
  L.K = c.n_lobes;
  L.n_out = 4 * c.n_lobes + (c.selection ? 1 : 0);
  L.n_out_pad = round16(L.n_out);
  L.n_layers = c.hidden_layers + 1;
  long off = 0;
  for (int l = 0; l < L.n_layers; ++l) {
    L.in[l] = l == 0 ? e.n_enc_pad : kWidth;
    L.out[l] = l == L.n_layers - 1 ? L.n_out_pad : kWidth;
    L.off[l] = off;
    off += long(L.in[l]) * L.out[l];
  }
  L.off[L.n_layers] = off;
  L.n_mlp = off;
  L.n_entries = n_entries;
  L.n_grid = n_entries * c.grid_features;
  L.n_params = L.n_mlp + L.n_grid;
  L.record_floats = c.selection ? 7 : 6;
  return NMG_OK;
}

static void fill_info(const EncodingParams& e, const Layout& L, nmg_info* info) {
  info->n_input = e.n_input;
  info->n_encoded = e.n_enc;
  info->n_encoded_padded = e.n_enc_pad;
  info->n_output = L.n_out;
  info->n_output_padded = L.n_out_pad;
  info->n_mlp_params = L.n_mlp;
  info->n_grid_params = L.n_grid;
  info->n_params = L.n_params;
  info->grid_entries = L.n_entries;
  info->record_floats = L.record_floats;
}

template <class T>
static nmg_status dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return NMG_OK;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_error(e == cudaErrorMemoryAllocation ? NMG_ERR_OOM : NMG_ERR_CUDA, "cudaMalloc(%zu B): %s",
                     count * sizeof(T), cudaGetErrorString(e));
  }
  return NMG_OK;
}

static void free_workspace(nmg_ctx* c) {
  Workspace& w = c->ws;
  fused_release(c);
  cudaFree(w.fused_dev);
  cudaFree(w.x);
  cudaFree(w.enc);
  for (auto& h : w.h) cudaFree(h);
  cudaFree(w.raw);
  cudaFree(w.draw);
  cudaFree(w.dh[0]);
  cudaFree(w.dh[1]);
  cudaFree(w.partials);
  cudaFree(w.batch_counts);
  cudaFree(w.recs);
  w = Workspace();
}

static nmg_status reserve(nmg_ctx* c, int max_q, int max_b) {
  Workspace& w = c->ws;
  if (max_q <= w.cap_q && max_b <= w.cap_b && w.partials) return NMG_OK;
  max_q = max_q > w.cap_q ? max_q : w.cap_q;
  max_b = max_b > w.cap_b ? max_b : w.cap_b;
  cudaDeviceSynchronize();
  free_workspace(c);
  // The FP32 path stores every layer's activations of a batch for its
  // backward; the fused paths recompute them inside the training kernel and
  // keep only the query-side input rows and raw outputs (for nmg_pdf).
  const bool fp32 = c->cfg.path == NMG_PATH_FP32;
  const int cap = fp32 && max_b > max_q ? max_b : max_q;
  const Layout& L = c->lay;
  const size_t capz = size_t(cap > 1 ? cap : 1);
  nmg_status s;
#define A(p, n)                                       \
  do {                                                \
    if ((s = dalloc(&(p), (n))) != NMG_OK) return s; \
    w.bytes += size_t(n) * sizeof(*(p));              \
  } while (0)
  A(w.x, capz * c->enc.n_input);
  A(w.partials, 2 * 2048);
  A(w.batch_counts, kMaxFrameBatches);
  A(w.raw, capz * L.n_out_pad);
  w.n_partials = 2 * 2048;
  if (fp32) {
    A(w.enc, capz * c->enc.n_enc_pad);
    for (int l = 0; l < L.n_layers - 1; ++l)
      if (l < 2 || max_b > 0) A(w.h[l], capz * kWidth);
    if (max_b > 0) {
      const size_t wd = size_t(c->enc.n_enc_pad > kWidth ? c->enc.n_enc_pad : kWidth);
      A(w.draw, size_t(max_b) * L.n_out_pad);
      A(w.recs, size_t(max_b) * 8);
      A(w.dh[0], size_t(max_b) * wd);
      A(w.dh[1], size_t(max_b) * wd);
    }
  }
#undef A
  w.cap_q = max_q;
  w.cap_b = max_b;
  if (c->cfg.path != NMG_PATH_FP32) return fused_reserve(c);
  return NMG_OK;
}

static nmg_status need(nmg_ctx* c, int n_max, bool train) {
  NMG_REQUIRE(n_max >= 0, "n_max=%d < 0", n_max);
  if (train && n_max > c->ws.cap_b)
    return set_error(NMG_ERR_CAPACITY, "batch %d above reserved %d (call nmg_reserve)", n_max, c->ws.cap_b);
  if (!train && n_max > c->ws.cap_q)
    return set_error(NMG_ERR_CAPACITY, "%d queries above reserved %d (call nmg_reserve)", n_max, c->ws.cap_q);
  return NMG_OK;
}

}  // namespace nmg

using namespace nmg;

extern "C" {

nmg_status nmg_config_init(nmg_config* c, int preset) {
  NMG_REQUIRE(c != nullptr, "cfg is NULL");
  memset(c, 0, sizeof(*c));
  c->n_lobes = 8;
  c->kappa_poly = 1;
  c->cosine_aware = 1;
  c->aabb[3] = c->aabb[4] = c->aabb[5] = 1.f;
  c->width = 64;
  c->hidden_layers = 3;
  c->path = NMG_PATH_FP32;
  c->learning_rate = 1e-2f;
  c->beta1 = 0.9f;
  c->beta2 = 0.99f;
  c->epsilon = 1e-15f;
  c->l2_reg = 1e-6f;
  c->ema_decay = 0.95f;
  c->use_ema = 1;
  c->loss_scale = 128.f;
  c->seed = 7272;
  if (preset == NMG_PRESET_REFERENCE) {
    c->input_mode = 0;
    c->grid_hash = 0;
    c->grid_levels = 8;
    c->grid_features = 4;
    c->grid_log2_hashmap = 19;
    c->grid_base_resolution = 8;
    c->grid_per_level_scale = 1.405f;
    c->grid_smoothstep = 1;
    c->sh_degree = 2;
    c->oneblob_bins = 4;
    c->selection = 0;
  } else if (preset == NMG_PRESET_HASHGRID) {
    c->input_mode = 1;
    c->grid_hash = 1;
    c->grid_levels = 16;
    c->grid_features = 2;
    c->grid_log2_hashmap = 19;
    c->grid_base_resolution = 16;
    c->grid_per_level_scale = 1.447f;
    c->grid_smoothstep = 0;
    c->sh_degree = 4;
    c->oneblob_bins = 4;
    c->selection = 1;
  } else {
    return set_error(NMG_ERR_INVALID_ARG, "unknown preset %d", preset);
  }
  return NMG_OK;
}

nmg_status nmg_config_info(const nmg_config* cfg, nmg_info* info) {
  NMG_REQUIRE(cfg && info, "NULL argument");
  EncodingParams e;
  Layout L;
  nmg_status s = derive(*cfg, e, L);
  if (s != NMG_OK) return s;
  fill_info(e, L, info);
  return NMG_OK;
}

nmg_status nmg_create(const nmg_config* cfg, nmg_ctx** out) {
  NMG_REQUIRE(cfg && out, "NULL argument");
  *out = nullptr;
  nmg_ctx* c = new (std::nothrow) nmg_ctx();
  if (!c) return set_error(NMG_ERR_OOM, "host allocation failed");
  c->cfg = *cfg;
  nmg_status s = derive(*cfg, c->enc, c->lay);
  if (s != NMG_OK) {
    delete c;
    return s;
  }
  c->mix = MixOpts{cfg->kappa_softplus, cfg->kappa_poly, cfg->cosine_aware};
  cudaGetDevice(&c->device);
  const size_t n = size_t(c->lay.n_params);
#define A(p, k)                          \
  if ((s = dalloc(&(p), (k))) != NMG_OK) { \
    nmg_destroy(c);                      \
    return s;                            \
  }
  A(c->w, n);
  A(c->grad, n);
  A(c->m, n);
  A(c->v, n);
  A(c->psteps, n);
  A(c->d_step, 1);
  if (cfg->use_ema) {
    A(c->w_inf, n);
  } else {
    c->w_inf = c->w;
  }
  if (cfg->path != NMG_PATH_FP32) {
    A(c->w16, n);
    A(c->w16_inf, n);
  }
#undef A
  cudaMemset(c->grad, 0, n * sizeof(float));
  cudaMemset(c->m, 0, n * sizeof(float));
  cudaMemset(c->v, 0, n * sizeof(float));
  cudaMemset(c->psteps, 0, n * sizeof(uint32_t));
  cudaMemset(c->d_step, 0, sizeof(uint32_t));
  if ((s = init_params(c, cfg->seed, 0)) != NMG_OK || (s = reserve(c, 0, 0)) != NMG_OK) {
    nmg_destroy(c);
    return s;
  }
  if (c->w_inf != c->w) cudaMemcpy(c->w_inf, c->w, n * sizeof(float), cudaMemcpyDeviceToDevice);
  if ((s = sync_copies(c, 0)) != NMG_OK) {
    nmg_destroy(c);
    return s;
  }
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    nmg_destroy(c);
    return set_error(NMG_ERR_CUDA, "nmg_create: %s", cudaGetErrorString(e));
  }
  *out = c;
  return NMG_OK;
}

void nmg_destroy(nmg_ctx* c) {
  if (!c) return;
  cudaDeviceSynchronize();
  host_io_release(c);
  free_workspace(c);
  if (c->w_inf != c->w) cudaFree(c->w_inf);
  cudaFree(c->w);
  cudaFree(c->grad);
  cudaFree(c->m);
  cudaFree(c->v);
  cudaFree(c->psteps);
  cudaFree(c->d_step);
  cudaFree(c->w16);
  cudaFree(c->w16_inf);
  delete c;
}

nmg_status nmg_device_bytes(const nmg_ctx* c, uint64_t* bytes) {
  NMG_REQUIRE(c && bytes, "NULL argument");
  const size_t n = size_t(c->lay.n_params);
  size_t b = n * (sizeof(float) * 4 + sizeof(uint32_t)) + sizeof(uint32_t);  // w, grad, m, v, step counters
  if (c->w_inf != c->w) b += n * sizeof(float);
  if (c->w16) b += 2 * n * sizeof(uint16_t);
  *bytes = uint64_t(b + c->ws.bytes + c->ws.fused_bytes);
  return NMG_OK;
}

nmg_status nmg_get_info(const nmg_ctx* c, nmg_info* info) {
  NMG_REQUIRE(c && info, "NULL argument");
  fill_info(c->enc, c->lay, info);
  return NMG_OK;
}

nmg_status nmg_reserve(nmg_ctx* c, int max_queries, int max_batch) {
  NMG_REQUIRE(c != nullptr, "ctx is NULL");
  NMG_REQUIRE(max_queries >= 0 && max_batch >= 0, "negative capacity");
  return reserve(c, max_queries, max_batch);
}

nmg_status nmg_set_params(nmg_ctx* c, const float* params, nmg_stream stream) {
  NMG_REQUIRE(c && params, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = size_t(c->lay.n_params);
  NMG_CUDA_TRY(cudaMemcpyAsync(c->w, params, n * sizeof(float), cudaMemcpyDefault, st));
  if (c->w_inf != c->w) NMG_CUDA_TRY(cudaMemcpyAsync(c->w_inf, c->w, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
  NMG_CUDA_TRY(cudaMemsetAsync(c->m, 0, n * sizeof(float), st));
  NMG_CUDA_TRY(cudaMemsetAsync(c->v, 0, n * sizeof(float), st));
  NMG_CUDA_TRY(cudaMemsetAsync(c->psteps, 0, n * sizeof(uint32_t), st));
  NMG_CUDA_TRY(cudaMemsetAsync(c->d_step, 0, sizeof(uint32_t), st));
  return sync_copies(c, st);
}

nmg_status nmg_get_params(const nmg_ctx* c, int which, float* params, nmg_stream stream) {
  NMG_REQUIRE(c && params, "NULL argument");
  NMG_REQUIRE(which == 0 || which == 1, "which=%d", which);
  NMG_CUDA_TRY(cudaMemcpyAsync(params, which ? c->w_inf : c->w, size_t(c->lay.n_params) * sizeof(float),
                               cudaMemcpyDefault, (cudaStream_t)stream));
  return NMG_OK;
}

nmg_status nmg_get_gradients(const nmg_ctx* c, float* grads, nmg_stream stream) {
  NMG_REQUIRE(c && grads, "NULL argument");
  NMG_CUDA_TRY(cudaMemcpyAsync(grads, c->grad, size_t(c->lay.n_params) * sizeof(float), cudaMemcpyDefault,
                               (cudaStream_t)stream));
  return NMG_OK;
}

int nmg_get_step(const nmg_ctx* c) {
  if (!c) return -1;
  uint32_t s = 0;
  if (cudaMemcpy(&s, c->d_step, sizeof(s), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return int(s);
}

nmg_status nmg_featurize(nmg_ctx* c, const nmg_shading* in, int n, float* x, nmg_stream stream) {
  NMG_REQUIRE(c && in, "NULL argument");
  NMG_REQUIRE(n >= 0, "n < 0");
  if (n == 0) return NMG_OK;
  NMG_REQUIRE(in->pos && in->wo && in->normal && in->roughness && x, "NULL shading array or output");
  return plain_featurize(c, in, nullptr, n, x, (cudaStream_t)stream);
}

nmg_status nmg_infer_raw(nmg_ctx* c, const float* x, int n, int which, float* raw, nmg_stream stream) {
  NMG_REQUIRE(c && x && raw, "NULL argument");
  NMG_REQUIRE(which == 0 || which == 1, "which=%d", which);
  nmg_status s = need(c, n, false);
  if (s != NMG_OK || n == 0) return s;
  cudaStream_t st = (cudaStream_t)stream;
  if (c->cfg.path == NMG_PATH_FP32) return plain_forward(c, x, nullptr, n, which ? c->w_inf : c->w, false, raw, st);
  return fused_infer_raw(c, x, nullptr, n, which, raw, st);
}

nmg_status nmg_query(nmg_ctx* c, const nmg_shading* in, const float* u4, const int* d_count, int n_max,
                     const nmg_query_out* out, nmg_stream stream) {
  NMG_REQUIRE(c && in && out, "NULL argument");
  nmg_status s = need(c, n_max, false);
  if (s != NMG_OK || n_max == 0) return s;
  NMG_REQUIRE(in->pos && in->wo && in->normal && in->roughness && u4 && out->dir && out->pdf,
              "NULL shading array, uniforms or output");
  NMG_REQUIRE(aligned16(u4), "u4 must be 16-byte aligned");
  NMG_REQUIRE(!out->raw || aligned16(out->raw), "raw must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  if (c->cfg.path == NMG_PATH_FP32) return plain_query(c, in, u4, d_count, n_max, out, st);
  return fused_query(c, in, u4, d_count, n_max, out, st);
}

nmg_status nmg_pdf(nmg_ctx* c, const nmg_shading* in, const float* wi, const int* d_count, int n_max, float* pdf,
                   nmg_stream stream) {
  NMG_REQUIRE(c && in, "NULL argument");
  nmg_status s = need(c, n_max, false);
  if (s != NMG_OK || n_max == 0) return s;
  NMG_REQUIRE(in->pos && in->wo && in->normal && in->roughness && wi && pdf, "NULL input or output");
  cudaStream_t st = (cudaStream_t)stream;
  if (c->cfg.path == NMG_PATH_FP32) return plain_pdf(c, in, wi, d_count, n_max, pdf, st);
  return fused_pdf(c, in, wi, d_count, n_max, pdf, st);
}

nmg_status nmg_train_step(nmg_ctx* c, const float* x, const float* records, const int* d_count, int n_max,
                          double* stats, nmg_stream stream) {
  NMG_REQUIRE(c != nullptr, "ctx is NULL");
  nmg_status s = need(c, n_max, true);
  if (s != NMG_OK || n_max == 0) return s;
  NMG_REQUIRE(x && records, "NULL inputs");
  cudaStream_t st = (cudaStream_t)stream;
  if (c->cfg.path == NMG_PATH_FP32) return plain_train_step(c, x, records, d_count, n_max, stats, st);
  return fused_train_step(c, x, records, d_count, n_max, stats, st);
}

nmg_status nmg_network_vjp(nmg_ctx* c, const float* x, const float* draw, int n, float* raw, float* dparams,
                           nmg_stream stream) {
  NMG_REQUIRE(c && x && draw && dparams, "NULL argument");
  NMG_REQUIRE(c->cfg.path == NMG_PATH_FP32, "nmg_network_vjp runs on the FP32 path");
  nmg_status s = need(c, n, true);
  if (s != NMG_OK || n == 0) return s;
  return plain_vjp(c, x, draw, n, raw, dparams, (cudaStream_t)stream);
}

nmg_status nmg_set_query_tiling(nmg_ctx* c, int warpgroups_per_cta) {
  NMG_REQUIRE(c != nullptr, "ctx is NULL");
  NMG_REQUIRE(warpgroups_per_cta == 0 || (warpgroups_per_cta >= 4 && warpgroups_per_cta <= 12),
              "warpgroups_per_cta=%d (0 = default, 4..6, 7 = two threads per query, 8..12 = warp-specialised)",
              warpgroups_per_cta);
  NMG_REQUIRE(warpgroups_per_cta == 4 || warpgroups_per_cta == 7 || warpgroups_per_cta == 8 ||
                  warpgroups_per_cta == 0 || c->lay.n_out_pad <= 64,
              "tiling %d needs <= 64 outputs", warpgroups_per_cta);
  c->query_wg = warpgroups_per_cta;
  return NMG_OK;
}

int nmg_get_query_tiling(const nmg_ctx* c) {
  if (!c) return -1;
  if (c->query_wg > 0) return c->query_wg;
  return c->cfg.path == NMG_PATH_FP32 ? 0 : fused_default_tiling(c);
}

nmg_status nmg_autotune_query(nmg_ctx* c, const nmg_shading* in, const float* u4, int n, const nmg_query_out* out,
                              int use_cache, int* chosen, nmg_stream stream) {
  NMG_REQUIRE(c && in && out && u4, "NULL argument");
  nmg_status s = need(c, n, false);
  if (s != NMG_OK) return s;
  NMG_REQUIRE(n > 0, "n must be positive");
  if (c->cfg.path == NMG_PATH_FP32) {
    if (chosen) *chosen = 0;
    return NMG_OK;  // the plain path has no tunable tiling
  }
  return fused_autotune(c, in, u4, n, out, use_cache, chosen, (cudaStream_t)stream);
}

nmg_status nmg_check_errors(nmg_ctx* c) {
  NMG_REQUIRE(c != nullptr, "ctx is NULL");
  NMG_CUDA_TRY(cudaDeviceSynchronize());
  return fused_check_errors(c);
}

nmg_status nmg_selftest_wait_timeout(nmg_ctx* c, nmg_stream stream) {
  NMG_REQUIRE(c != nullptr, "ctx is NULL");
  return fused_selftest_wait_timeout(c, (cudaStream_t)stream);
}

static const uint32_t kMagic = 0x31474d4e;  // "NMG1"

nmg_status nmg_save(const nmg_ctx* c, const char* path) {
  NMG_REQUIRE(c && path, "NULL argument");
  const size_t n = size_t(c->lay.n_params);
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(NMG_ERR_INVALID_ARG, "cannot open %s", path);
  float* buf = (float*)malloc(n * sizeof(float));
  if (!buf) {
    fclose(f);
    return set_error(NMG_ERR_OOM, "host buffer");
  }
  uint32_t step = 0;
  cudaMemcpy(&step, c->d_step, sizeof(step), cudaMemcpyDeviceToHost);
  int64_t hdr[4] = {int64_t(kMagic), int64_t(n), int64_t(step), int64_t(c->lay.n_mlp)};
  bool ok = fwrite(hdr, sizeof(hdr), 1, f) == 1;
  const float* arrays[4] = {c->w, c->w_inf, c->m, c->v};
  for (int a = 0; a < 4 && ok; ++a) {
    ok = cudaMemcpy(buf, arrays[a], n * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess &&
         fwrite(buf, sizeof(float), n, f) == n;
  }
  if (ok) {
    ok = cudaMemcpy(buf, c->psteps, n * sizeof(uint32_t), cudaMemcpyDeviceToHost) == cudaSuccess &&
         fwrite(buf, sizeof(uint32_t), n, f) == n;
  }
  free(buf);
  fclose(f);
  return ok ? NMG_OK : set_error(NMG_ERR_CUDA, "checkpoint write failed");
}

nmg_status nmg_load(nmg_ctx* c, const char* path) {
  NMG_REQUIRE(c && path, "NULL argument");
  const size_t n = size_t(c->lay.n_params);
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(NMG_ERR_INVALID_ARG, "cannot open %s", path);
  int64_t hdr[4];
  if (fread(hdr, sizeof(hdr), 1, f) != 1 || hdr[0] != int64_t(kMagic) || hdr[1] != int64_t(n) ||
      hdr[3] != int64_t(c->lay.n_mlp)) {
    fclose(f);
    return set_error(NMG_ERR_INVALID_ARG, "%s: not a checkpoint of this configuration", path);
  }
  float* buf = (float*)malloc(n * sizeof(float));
  if (!buf) {
    fclose(f);
    return set_error(NMG_ERR_OOM, "host buffer");
  }
  float* arrays[4] = {c->w, c->w_inf, c->m, c->v};
  bool ok = true;
  for (int a = 0; a < 4 && ok; ++a) {
    ok = fread(buf, sizeof(float), n, f) == n;
    if (ok && (a != 1 || c->w_inf != c->w))
      ok = cudaMemcpy(arrays[a], buf, n * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  if (ok) {
    ok = fread(buf, sizeof(uint32_t), n, f) == n &&
         cudaMemcpy(c->psteps, buf, n * sizeof(uint32_t), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  uint32_t step = uint32_t(hdr[2]);
  if (ok) ok = cudaMemcpy(c->d_step, &step, sizeof(step), cudaMemcpyHostToDevice) == cudaSuccess;
  free(buf);
  fclose(f);
  if (!ok) return set_error(NMG_ERR_INVALID_ARG, "%s: truncated checkpoint", path);
  return sync_copies(c, 0);
}

}  // extern "C"
