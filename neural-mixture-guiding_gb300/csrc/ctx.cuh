// ctx.cuh -- the guiding field's device state and the internal interface
// between the C ABI (nmg_api.cu), the plain FP32 kernels (plain.cu) and the
// fused tensor-core kernels (fused_*.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "../../include/nmg.h"
#include "encoding.cuh"
#include "mixture.cuh"

namespace nmg {

constexpr int kWidth = 64;       // MLP width (the only one compiled)
constexpr int kMaxLayers = 8;    // weight matrices

struct Layout {
  int K, n_out, n_out_pad, n_layers;  // n_layers = hidden_layers + 1 weight matrices
  int in[kMaxLayers], out[kMaxLayers];
  long off[kMaxLayers + 1];           // element offset of each matrix; off[n_layers] = MLP size
  long n_mlp, n_grid, n_params, n_entries;
  int record_floats;
};

struct Workspace {
  int cap_q = 0, cap_b = 0;
  // plain path
  float* x = nullptr;      // [cap][n_input]
  float* enc = nullptr;    // [cap][n_enc_pad]
  float* h[kMaxLayers] = {};  // [cap][64] activations after ReLU
  float* raw = nullptr;    // [cap][n_out_pad]
  float* draw = nullptr;   // [cap_b][n_out_pad]
  float* dh[2] = {};       // [cap_b][max(64, n_enc_pad)] ping-pong deltas
  double* partials = nullptr;  // block partial sums (loss, grad norm)
  int n_partials = 0;
  int* batch_counts = nullptr; // [kMaxFrameBatches] record counts of nmg_train_frame's batches
  float* recs = nullptr;       // [cap_b][8] GuidedOutput rows of a batch (plain path of nmg_train_frame)
  // fused path: host-side state object and its device allocation
  void* fused = nullptr;
  void* fused_dev = nullptr;
  size_t fused_bytes = 0;
  size_t bytes = 0;  // device bytes of the buffers above except the fused allocation
};

}  // namespace nmg

struct nmg_ctx {
  nmg_config cfg;
  nmg::EncodingParams enc;
  nmg::MixOpts mix;
  nmg::Layout lay;
  int device = 0;
  // optimiser state (device)
  float* w = nullptr;        // master FP32 training weights [n_params]
  float* w_inf = nullptr;    // inference weights (EMA) [n_params]
  float* grad = nullptr;     // loss-scaled gradient [n_params]
  float* m = nullptr;
  float* v = nullptr;
  uint32_t* psteps = nullptr;
  uint32_t* d_step = nullptr;  // optimiser step counter (device, graph-safe)
  // reduced-precision copies for the fused path (bf16 or fp16 bits)
  uint16_t* w16 = nullptr;     // training weights
  uint16_t* w16_inf = nullptr; // inference weights
  int query_wg = 0;            // warpgroups per CTA of the fused query kernel (0: default)
  int host_chunks = 0;         // chunks of nmg_query_host (0: automatic)
  nmg::Workspace ws;
  void* host_io = nullptr;     // streams and staging of the host-buffer entry points (host_io.cu)
};

namespace nmg {

// plain.cu
nmg_status plain_featurize(nmg_ctx* c, const nmg_shading* in, const int* d_count, int n_max, float* x,
                           cudaStream_t st);
nmg_status plain_forward(nmg_ctx* c, const float* x, const int* d_count, int n_max, const float* weights,
                         bool keep_hidden, float* raw_out, cudaStream_t st);
nmg_status plain_query(nmg_ctx* c, const nmg_shading* in, const float* u4, const int* d_count, int n_max,
                       const nmg_query_out* out, cudaStream_t st);
nmg_status plain_pdf(nmg_ctx* c, const nmg_shading* in, const float* wi, const int* d_count, int n_max,
                     float* pdf, cudaStream_t st);
nmg_status pdf_from_raw(nmg_ctx* c, const float* raw, const nmg_shading* in, const float* wi, const int* d_count,
                        int n_max, float* pdf, cudaStream_t st);
nmg_status plain_train_step(nmg_ctx* c, const float* x, const float* rec, const int* d_count, int n_max,
                            double* stats, cudaStream_t st);
nmg_status plain_vjp(nmg_ctx* c, const float* x, const float* draw, int n, float* raw, float* dparams,
                     cudaStream_t st);
nmg_status optimizer_step(nmg_ctx* c, const int* d_count, int n_max, double* stats, cudaStream_t st);
nmg_status init_params(nmg_ctx* c, uint32_t seed, cudaStream_t st);
nmg_status sync_copies(nmg_ctx* c, cudaStream_t st);

// fused_query.cu / fused_train.cu
nmg_status fused_reserve(nmg_ctx* c);
nmg_status fused_query(nmg_ctx* c, const nmg_shading* in, const float* u4, const int* d_count, int n_max,
                       const nmg_query_out* out, cudaStream_t st);
nmg_status fused_infer_raw(nmg_ctx* c, const float* x, const int* d_count, int n_max, int which, float* raw,
                           cudaStream_t st);
nmg_status fused_pdf(nmg_ctx* c, const nmg_shading* in, const float* wi, const int* d_count, int n_max, float* pdf,
                     cudaStream_t st);
nmg_status pack_images(nmg_ctx* c, cudaStream_t st);
void fused_release(nmg_ctx* c);
nmg_status fused_check_errors(nmg_ctx* c);
nmg_status fused_selftest_wait_timeout(nmg_ctx* c, cudaStream_t st);
nmg_status fused_autotune(nmg_ctx* c, const nmg_shading* in, const float* u4, int n, const nmg_query_out* out,
                          int use_cache, int* chosen, cudaStream_t st);
nmg_status fused_train_step(nmg_ctx* c, const float* x, const float* rec, const int* d_count, int n_max,
                            double* stats, cudaStream_t st);
// A training batch read from the frame's radiance records: row q is the path
// vertex vid[id_base + q] (vertex id = depth * pixels + pixel).
struct TrainRecords {
  const uint32_t* vid;
  long id_base;
  uint32_t pixels;
  const nmg_radiance_records* rr;
};
constexpr int kMaxFrameBatches = 64;
nmg_status fused_train_step_src(nmg_ctx* c, const float* x, const float* rec, const TrainRecords* src,
                                const int* d_count, int n_max, double* stats, cudaStream_t st);
int fused_default_tiling(const nmg_ctx* c);

// host_io.cu
void host_io_release(nmg_ctx* c);

nmg_status set_error(nmg_status st, const char* fmt, ...);

}  // namespace nmg
