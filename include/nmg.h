/*
 * nmg.h -- C ABI of the GB300-native neural parametric mixture guiding step.
 *
 * One shared library (libnmg.so) built from hand-written sm_103a CUDA. All
 * entry points take plain pointers and sizes; no C++ or torch types cross the
 * boundary. Array arguments are DEVICE pointers unless a comment says
 * otherwise; every call is asynchronous on the given CUDA stream (NULL = the
 * legacy default stream) and never synchronises the host. Errors are
 * returned as nmg_status codes; no exception crosses the ABI.
 *
 * The reference reaches the guiding step through four internal call sites of
 * its wavefront integrator (src/render/guided/integrator.cpp):
 *   query      inferenceStep()            integrator.cpp:627-648
 *   sample     MixedSG(...).sample()      integrator.cpp:296-300
 *   pdf        MixedSG(...).pdf(wi)       integrator.cpp:201,260,315
 *   train-step trainStep() on TrainBuffer integrator.cpp:650-701
 * Each entry point below cites the reference interface it replaces.
 *
 * Layouts (row-major, one row per query / training sample):
 *   raw        float[n][stride]  per lobe i: (lambda, kappa, theta, phi) raw
 *              network outputs at 4i..4i+3 (distribution.h:85-98), followed
 *              by the selection logit at 4K when learned selection is on
 *              (distribution.h:205-241). stride % 4 == 0, 16-byte aligned.
 *   u4         float[n][4]       (u_guide, u_lobe, u_dir0, u_dir1) uniforms
 *              in [0,1): u_lobe picks the lobe (distribution.h:133), u_dir*
 *              sample the vMF (vmf.h:48-57); u_guide is the caller's
 *              guide-vs-BSDF decision (integrator.cpp:220) and is not read.
 *   record     float[n][rstride] GuidedOutput {theta, phi, L_r, L_g, L_b,
 *              wiPdf[, bsdfPdf]} (src/render/guided/guideditem.h:54-61).
 *   vectors    float[n][3].
 */
#ifndef NMG_H_
#define NMG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nmg_status {
  NMG_OK = 0,
  NMG_ERR_INVALID_ARG = 1, /* null/misaligned pointer, bad size or option */
  NMG_ERR_OOM = 2,         /* device allocation failed */
  NMG_ERR_CUDA = 3,        /* a CUDA call failed (see nmg_last_error) */
  NMG_ERR_NUMERIC = 4,     /* non-finite values detected by a checking call */
  NMG_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  NMG_ERR_UNSUPPORTED = 6, /* configuration not compiled in (e.g. K) */
  NMG_ERR_CAPACITY = 7     /* size above the reserved capacity */
} nmg_status;

/* cudaStream_t, kept opaque so this header needs no CUDA headers. */
typedef void* nmg_stream;

/* Human-readable text of a status code (static storage). */
const char* nmg_status_string(int status);
/* Last error message recorded by any call on this thread (static storage). */
const char* nmg_last_error(void);
/* Library version: major*10000 + minor*100 + patch. */
int nmg_version(void);

/* ------------------------------------------------------------------------
 * Mixture kernels on raw network outputs (no network).
 * ---------------------------------------------------------------------- */
typedef struct nmg_mixture_opts {
  int n_lobes;        /* K: 4, 7, 8 or 16 (the reference fixes 8, parameters.h:10) */
  int stride;         /* floats per raw row, multiple of 4, >= 4K (+1 with selection) */
  int kappa_softplus; /* 0: kappa = exp(clamp(x,-10,15)) as train.h:244; 1: log(1+e^x) */
  int kappa_poly;     /* 1: the kappa<1 polynomial of distribution.h:165-166 in the gradient; 0: exact */
  int selection;      /* 1: raw[4K] is the learned selection logit (GUIDED_LEARN_SELECTION) */
} nmg_mixture_opts;

/*
 * Samples one direction per query from the activated mixture and evaluates
 * the mixture pdf there. With cos_normal non-NULL the mixture is first
 * multiplied by the cosine lobe around cos_normal[i] (already face-forwarded;
 * MixedSG::applyCosineLobe, distribution.h:184-195).
 * Replaces: MixedSG(dist_data) [+ applyCosineLobe] + sample(sampler) +
 * pdf(wi) in hendleGuidedSampling (integrator.cpp:296-312).
 * Outputs: dir[n][3] (unit), pdf[n], lobe[n] (may be NULL).
 */
nmg_status nmg_mixture_sample(const nmg_mixture_opts* opts, const float* raw, const float* u4,
                              const float* cos_normal, int n, float* dir, float* pdf, int* lobe,
                              nmg_stream stream);

/*
 * Mixture pdf at given unit directions wi[n][3] (optionally times the cosine
 * lobe). Replaces: MixedSG::pdf in handleIntersections / handleBsdfSampling
 * (integrator.cpp:198-201, 257-260).
 */
nmg_status nmg_mixture_pdf(const nmg_mixture_opts* opts, const float* raw, const float* wi,
                           const float* cos_normal, int n, float* pdf, nmg_stream stream);

/*
 * KL-divergence loss per training sample and its gradient with respect to
 * the raw outputs, scaled by loss_scale / n (train.cu:69-124, or
 * train.cu:126-172 with opts->selection). grad has the raw layout (row stride
 * opts->stride; padding columns are left untouched). loss (may be NULL)
 * receives the per-sample loss; loss_sum (may be NULL) receives the FP64 sum
 * over the batch, reduced deterministically through `workspace`
 * (nmg_mixture_loss_workspace_bytes(n) bytes of device memory owned by the
 * caller).
 * Replaces: compute_dL_doutput_divergence + thrust::reduce of the loss
 * buffer (integrator.cpp:689-697).
 */
size_t nmg_mixture_loss_workspace_bytes(int n);
nmg_status nmg_mixture_loss_grad(const nmg_mixture_opts* opts, const float* raw, const float* record,
                                 int record_stride, int n, float loss_scale, float* grad, float* loss,
                                 double* loss_sum, void* workspace, size_t workspace_bytes,
                                 nmg_stream stream);


/*
 * nmg_mixture_loss_grad without a caller-provided workspace. This entry point
 * has no counterpart in the reference; it exists for callers that cannot
 * allocate device memory (all of it pooled before the frame loop, no
 * allocator handle of their own, or no tolerance for the synchronisation a
 * cudaMalloc/cudaFree may cause). It allocates nothing: the FP64 loss sum is
 * reduced through a fixed 64 KiB array inside libnmg.so that every GPU
 * loading the library keeps until the process exits, which limits n to
 * 1,048,576 samples (larger n returns NMG_ERR_CAPACITY). The first call on
 * each device looks up that array's device address; make that first call
 * before any stream capture. All calls share the array: calls that overlap
 * on the GPU (different streams, or different host threads) race on it and
 * must be ordered by the caller. Results equal nmg_mixture_loss_grad's
 * (loss_sum up to the order of the FP64 additions). The looked-up address is
 * kept per device for the life of the process: after a cudaDeviceReset of a
 * device this entry point must not be called on that device again.
 */
nmg_status nmg_mixture_loss_grad_noalloc(const nmg_mixture_opts* opts, const float* raw, const float* record,
                                         int record_stride, int n, float loss_scale, float* grad, float* loss,
                                         double* loss_sum, nmg_stream stream);

/* ------------------------------------------------------------------------
 * Network-backed guiding field (encoding -> MLP -> mixture).
 * ---------------------------------------------------------------------- */
typedef enum nmg_preset {
  /* src/render/guided + common/configs/nn/base.json: 9 inputs, DenseGrid
   * 8 levels x 4 features (base 8, scale 1.405, smoothstep), SH degree 2 of
   * wo, OneBlob 4 bins of (theta_n/pi, phi_n/2pi, 1-e^-r) = 48 features;
   * MLP 48-64-64-64-32; K = 8, exp kappa, no learned selection. */
  NMG_PRESET_REFERENCE = 0,
  /* Hash-grid configuration: 10 inputs, HashGrid 16 levels x 2 features
   * (2^19 entries per level, base 16, scale 1.447, linear), SH degree 4 of wo
   * and of the normal, OneBlob 4 bins of 1-e^-r = 68 features padded to 80;
   * MLP 80-64-64-64-48 (33 used: 8 lobes x 4 + selection logit). */
  NMG_PRESET_HASHGRID = 1
} nmg_preset;

typedef enum nmg_path {
  NMG_PATH_FP32 = 0, /* plain path: one FP32 CUDA kernel per op */
  NMG_PATH_BF16 = 1, /* fused path: BF16 features/weights/activations on tcgen05, FP32 accumulate */
  NMG_PATH_FP16 = 2  /* fused path with FP16 instead of BF16 */
} nmg_path;

typedef struct nmg_config {
  /* mixture head */
  int n_lobes;        /* K: 7, 8 or 16 */
  int selection;      /* 1: an extra output is the learned selection logit */
  int kappa_softplus; /* 0: exp(clamp) kappa (train.h:244); 1: softplus */
  int kappa_poly;     /* 1: reference kappa<1 polynomial in the gradient */
  int cosine_aware;   /* 1: query/pdf multiply by the cosine lobe around faceforward(n, wo) (integrator.cpp:198-200) */
  /* inputs and encoding */
  int input_mode;     /* 0: reference 9-dim inputs; 1: 10-dim inputs with SH of the normal */
  int grid_hash;      /* 0: dense grid; 1: hash grid */
  int grid_levels;    /* <= 24 */
  int grid_features;  /* 1, 2, 4 or 8 per level */
  int grid_log2_hashmap;
  int grid_base_resolution;
  float grid_per_level_scale;
  int grid_smoothstep;
  int sh_degree;      /* 1..4 */
  int oneblob_bins;
  float aabb[6];      /* scene box (min xyz, max xyz) for position normalisation */
  /* network */
  int width;          /* 64 (the only width compiled) */
  int hidden_layers;  /* 3 */
  int path;           /* nmg_path */
  /* optimiser (base.json:6-17): EMA(decay) around Adam */
  float learning_rate, beta1, beta2, epsilon, l2_reg;
  float ema_decay;    /* 0.95; inference uses the EMA weights when use_ema */
  int use_ema;
  float loss_scale;   /* 128 (parameters.h:24) */
  uint32_t seed;      /* 7272 */
} nmg_config;

/* Sizes derived from a configuration. */
typedef struct nmg_info {
  int n_input;        /* floats per network input row (9 or 10) */
  int n_encoded;      /* encoded width before padding */
  int n_encoded_padded;
  int n_output;       /* 4K (+1) */
  int n_output_padded;/* raw row stride */
  int64_t n_mlp_params, n_grid_params, n_params;
  int64_t grid_entries;
  int record_floats;  /* GuidedOutput floats per training record: 6 (7 with selection) */
} nmg_info;

typedef struct nmg_ctx nmg_ctx;

/* Per-query shading data (device pointers): pos[n][3] world position,
 * wo[n][3] outgoing direction, normal[n][3] shading normal, roughness[n]. */
typedef struct nmg_shading {
  const float* pos;
  const float* wo;
  const float* normal;
  const float* roughness;
} nmg_shading;

/* Query outputs (device pointers; any may be NULL except dir and pdf). */
typedef struct nmg_query_out {
  float* dir;       /* [n][3] sampled unit direction */
  float* pdf;       /* [n] guide pdf of dir */
  int* lobe;        /* [n] selected lobe */
  float* raw;       /* [n][n_output_padded] raw network outputs (FP32) */
  float* selection; /* [n] learned selection probability (selection configs) */
} nmg_query_out;

/* Fills *cfg with a preset (defaults of the reference's config). */
nmg_status nmg_config_init(nmg_config* cfg, int preset);
nmg_status nmg_config_info(const nmg_config* cfg, nmg_info* info);

/*
 * Creates a guiding field on the current CUDA device with parameters
 * initialised from cfg->seed (Xavier-uniform MLP weights, grid entries
 * U(-1e-4, 1e-4): fully_fused_mlp.cu:866-891, grid.h:1333-1336).
 * Replaces: GuidedPathTracer::resetNetwork (integrator.cpp:555-587).
 */
nmg_status nmg_create(const nmg_config* cfg, nmg_ctx** out);
void nmg_destroy(nmg_ctx* ctx);
nmg_status nmg_get_info(const nmg_ctx* ctx, nmg_info* info);

/* Allocates the workspaces for up to max_queries per query call and
 * max_batch per training step. After this, query/pdf/train calls with sizes
 * within capacity allocate nothing and may be captured in a CUDA graph. */
nmg_status nmg_reserve(nmg_ctx* ctx, int max_queries, int max_batch);

/* Device bytes the field holds: parameters, optimiser state, weight copies
 * and workspaces. The FP32 path stores each layer's activations of a
 * training batch (about 1.9 KB per record for the hash-grid network); the
 * BF16/FP16 paths recompute them inside the fused training kernel, so their
 * footprint does not grow with max_batch. No reference counterpart (tcnn
 * allocates every layer's forward activations per training call,
 * src/ext/tcnn/src/fully_fused_mlp.cu:711,839-853). */
nmg_status nmg_device_bytes(const nmg_ctx* ctx, uint64_t* bytes);

/* Parameters: [MLP weights, row-major [out][in] per layer | grid table]
 * (network.h:85-100, fully_fused_mlp.cu:855-864). which = 0: training
 * (master FP32) weights; 1: inference weights (the EMA when use_ema).
 * set_params sets both, resets Adam moments, step counters and the EMA. */
nmg_status nmg_set_params(nmg_ctx* ctx, const float* params, nmg_stream stream);
nmg_status nmg_get_params(const nmg_ctx* ctx, int which, float* params, nmg_stream stream);
/* Loss-scaled parameter gradient of the last training step (FP32). */
nmg_status nmg_get_gradients(const nmg_ctx* ctx, float* grads, nmg_stream stream);
/* Optimiser steps taken so far. */
int nmg_get_step(const nmg_ctx* ctx);

/*
 * Network input rows from shading data (train.cu:174-191).
 * Replaces: generate_inference_data (integrator.cpp:637).
 */
nmg_status nmg_featurize(nmg_ctx* ctx, const nmg_shading* in, int n, float* x, nmg_stream stream);

/*
 * Raw network outputs for input rows x[n][n_input] with the inference
 * (which = 1) or training (which = 0) weights.
 * Replaces: GuidingNetwork::inference (network.h:30-34, integrator.cpp:645).
 */
nmg_status nmg_infer_raw(nmg_ctx* ctx, const float* x, int n, int which, float* raw, nmg_stream stream);

/*
 * The guided query of one wavefront: featurise -> encode -> MLP ->
 * activate -> [cosine lobe] -> sample -> pdf. The number of queries is read
 * on the device from *d_count when d_count is non-NULL (clamped to
 * n_max), so a captured graph serves queues of any size up to n_max.
 * Replaces: inferenceStep + the MixedSG sample/pdf of hendleGuidedSampling
 * (integrator.cpp:283-340, 627-648).
 */
nmg_status nmg_query(nmg_ctx* ctx, const nmg_shading* in, const float* u4, const int* d_count, int n_max,
                     const nmg_query_out* out, nmg_stream stream);

/*
 * Guide pdf of given directions wi[n][3] (for MIS of BSDF- and light-sampled
 * directions). Replaces: MixedSG::pdf in handleIntersections and
 * handleBsdfSampling (integrator.cpp:198-201, 257-260).
 */
nmg_status nmg_pdf(nmg_ctx* ctx, const nmg_shading* in, const float* wi, const int* d_count, int n_max,
                   float* pdf, nmg_stream stream);

/*
 * One training step on a batch of records: x[n][n_input] network inputs
 * (GuidedInput) and records[n][record_floats] (GuidedOutput). Forward with
 * the training weights, KL loss and adjoint, backward through MLP and
 * encoding, Adam + EMA. stats (may be NULL) receives {mean loss, L2 norm of
 * the unscaled gradient} in FP64.
 * Replaces: the body of GuidedPathTracer::trainStep's batch loop
 * (integrator.cpp:666-700).
 */
nmg_status nmg_train_step(nmg_ctx* ctx, const float* x, const float* records, const int* d_count, int n_max,
                          double* stats, nmg_stream stream);

/*
 * nmg_query and nmg_train_step on HOST buffers (pinned memory gives the
 * overlap; pageable memory works but copies synchronously). Every input and
 * output array (all of in, u4, out->dir, out->pdf and, when non-NULL,
 * out->lobe and out->selection) is host memory; out->raw must be NULL.
 * nmg_query_host copies the inputs on a stream of its own into one of two
 * alternating device staging buffers; the copies wait only for the kernels
 * of the call before the previous one, so they overlap other work still
 * running on `stream` (the previous query and training step, for instance).
 * When `stream` is idle at the call, the wavefront is split into up to 4
 * chunks of at least 2^18 queries, so that chunk i+1's inputs are copied
 * while chunk i is computed (nmg_set_host_chunks fixes the count). When every
 * output given is pinned (page-locked) host memory, the query kernel writes
 * the results there itself through the host mapping; otherwise they are
 * staged on the device and copied back on a third stream.
 * nmg_train_step_host copies x and records to the device and runs the step;
 * stats (may be NULL) is HOST memory receiving the two FP64 statistics
 * (written by the kernel when pinned). The kernels of both calls run on
 * `stream` after the work already queued there, and `stream` waits for their
 * last copy: the host input arrays must be filled before the call, and all
 * host buffers stay valid until `stream` reaches the call's end. The first
 * call allocates device staging of the reserved capacity (not capturable);
 * later calls allocate nothing.
 * Replaces: the host side of the reference's inference/training calls, which
 * copy nothing themselves (integrator.cpp:627-701 operate on device queues);
 * no reference counterpart as an entry point.
 */
nmg_status nmg_query_host(nmg_ctx* ctx, const nmg_shading* in, const float* u4, int n, const nmg_query_out* out,
                          nmg_stream stream);
nmg_status nmg_train_step_host(nmg_ctx* ctx, const float* x, const float* records, int n, double* stats,
                               nmg_stream stream);

/*
 * Number of chunks nmg_query_host splits a wavefront into: 0 (the default)
 * chooses 1 when `stream` has work queued at the call and up to 4 when it is
 * idle; 1..8 fixes it (chunks stay at least 2^18 queries, so a small
 * wavefront may get fewer). nmg_get_host_chunks returns the fixed count, or
 * 4 when automatic. No reference counterpart (tuning).
 */
nmg_status nmg_set_host_chunks(nmg_ctx* ctx, int chunks);
int nmg_get_host_chunks(const nmg_ctx* ctx);

/*
 * Vector-Jacobian product of the network at the training weights:
 * given x[n][n_input] and dL/draw[n][n_output_padded], writes raw[n][..]
 * (may be NULL) and ACCUMULATES dL/dparams (FP32, unscaled) into dparams.
 * Used by the torch.autograd.Function binding and the gradient checks.
 */
nmg_status nmg_network_vjp(nmg_ctx* ctx, const float* x, const float* draw, int n, float* raw, float* dparams,
                           nmg_stream stream);

/*
 * Tiling of the fused query kernel: warpgroups (128-query tiles in flight)
 * per CTA, one CTA per SM; 5 and 6 are valid when the padded output width is
 * <= 64. 7: two tiles in flight, each on two warpgroups, two threads per
 * query splitting the lobes (queries that return raw outputs fall back to
 * 4). 8-12 select configurations of the warp-specialised kernel: encoder
 * warpgroups feed MLP + mixture warpgroups through a shared-memory ring
 * (8: 4 + 2 warpgroups, 4 slots; 9: 5 + 1, 5 slots; 10: 6 + 2, 6 slots;
 * 11: 4 + 2, 8 slots; 12: 4 + 2, 4 slots holding the hidden activations too).
 * 0 selects the default: 12 for the 8-lobe hash-grid network, 8 for the
 * reference network, 7 for 16-lobe networks. A tiling whose shared memory
 * exceeds the device's limit for this network's weight image makes the
 * query calls return NMG_ERR_UNSUPPORTED; the autotuner skips it.
 * nmg_get_query_tiling
 * reports the tiling in use (0 on the FP32 path). No counterpart in the
 * reference (its FullyFusedMLP launch shape is fixed,
 * fully_fused_mlp.cu:500-558).
 */
nmg_status nmg_set_query_tiling(nmg_ctx* ctx, int warpgroups_per_cta);
int nmg_get_query_tiling(const nmg_ctx* ctx);

/*
 * Training records of a frame from the per-pixel radiance records the
 * integrator keeps (the GuidedPixelStateBuffer SOA: for every path depth d a
 * RadianceRecordItem field array indexed by pixel, guideditem.soa /
 * workqueue.h:26-67). For every training pixel (offset + stride * (i, j) over
 * train_res, clipped to res) and every recorded non-delta vertex, appends one
 * network input row x[..][n_input] and one record[..][record_floats]
 * {theta, phi, L / thp * misWeight [* bsdfVal], wiPdf[, bsdfPdf]}. As in
 * train.cu:57-62, a vertex is dropped when its normalised position, its
 * direction, its warped outgoing direction, its pdf or L / thp * misWeight
 * (before the bsdfVal factor) has a NaN, or its pdf is zero.
 * *d_count (device) receives the number of records, which can be passed to
 * nmg_train_step as its device count; rows beyond `capacity` are counted but
 * not written. Record order is not deterministic (atomic append, as the
 * reference's TrainBuffer::push).
 * Replaces: generate_training_data (train.cu:14-67).
 */
#define NMG_MAX_TRAIN_DEPTH 8
typedef struct nmg_record_arrays {
  const float* L;           /* [pixels][3] accumulated radiance (Color) */
  const float* thp;         /* [pixels][3] path throughput at the vertex */
  const float* pos;         /* [pixels][3] vertex position */
  const float* dir;         /* [pixels][2] (theta, phi) of the scattered direction */
  const float* wi_pdf;      /* [pixels] */
  const float* bsdf_pdf;    /* [pixels] (may be NULL without learned selection) */
  const float* mis_weight;  /* [pixels] */
  const unsigned char* delta; /* [pixels] bool, may be NULL (no delta lobes) */
  const float* bsdf_val;    /* [pixels][3] (used with product sampling, may be NULL) */
  const float* wo;          /* [pixels][2] (theta, phi) of the outgoing direction */
  const float* normal;      /* [pixels][2] (theta, phi) of the shading normal */
  const float* roughness;   /* [pixels] */
} nmg_record_arrays;
typedef struct nmg_radiance_records {
  int max_depth;                              /* depths recorded (<= NMG_MAX_TRAIN_DEPTH) */
  int product;                                /* 1: multiply L by bsdfVal (GUIDED_PRODUCT_SAMPLING) */
  const unsigned* cur_depth;                  /* [pixels] vertices recorded per pixel */
  nmg_record_arrays depth[NMG_MAX_TRAIN_DEPTH];
} nmg_radiance_records;
typedef struct nmg_train_pixels {
  unsigned offset[2], stride[2], train_res[2], res[2];
} nmg_train_pixels;
nmg_status nmg_extract_records(nmg_ctx* ctx, const nmg_radiance_records* records, const nmg_train_pixels* pixels,
                               int capacity, float* x, float* out_records, int* d_count, nmg_stream stream);

/*
 * One frame's training on its radiance records, as the reference's trainStep
 * (integrator.cpp:650-701) does it: the records the rule of
 * nmg_extract_records keeps are compacted into vertex_ids[capacity] (one
 * 32-bit id per record, depth * image pixels + pixel; *d_count receives their
 * number N, records beyond capacity are counted but not stored), then up to
 * max_batches training steps run on consecutive batches of batch_size
 * records: batch i holds min(N - i * batch_size, batch_size) records rounded
 * down to a multiple of 128, and the batches stop at the first one below
 * min_batch (the reference's MIN_TRAIN_BATCH_SIZE; it also caps the batches
 * at batchPerFrame). N and the batch sizes are read on the device, so the call
 * needs no host synchronisation; a batch with no records takes no optimiser
 * step. On the fused paths the training kernel's load stage computes each
 * record's network input row and GuidedOutput from the radiance-record arrays
 * itself (the record rows never pass through HBM); the plain FP32 path
 * gathers each batch's rows first. batch_size must be a multiple of 128 and
 * at most the reserved batch. stats (may be NULL): [max_batches][2] FP64
 * {mean loss, gradient norm}, zeros for batches not run.
 * Replaces: GuidedPathTracer::trainStep (integrator.cpp:650-701):
 * generate_training_data, the host read of the buffer size and the loop of
 * network forward, compute_dL_doutput_divergence, backward and optimizer_step.
 */
nmg_status nmg_train_frame(nmg_ctx* ctx, const nmg_radiance_records* records, const nmg_train_pixels* pixels,
                           int capacity, uint32_t* vertex_ids, int* d_count, int batch_size, int max_batches,
                           int min_batch, double* stats, nmg_stream stream);

/*
 * One frame's bounce loop as a CUDA graph. Bounce i runs the guided query of
 * its queue (device SoA `in`, uniforms u4, queue length *d_count read on the
 * device, at most n_max; d_count NULL = n_max) and then, when train_x is
 * non-NULL, one training step on its batch (train_count / train_n_max as for
 * nmg_train_step; stats may be NULL). nmg_frame_capture records the whole
 * sequence once (the context must be reserved for every n_max and
 * train_n_max); nmg_frame_launch replays it on `stream` with one call. Queue
 * lengths and the optimiser step are read on the device, so one capture
 * serves every frame as long as the buffers stay where they were.
 * nmg_frame_run_eager issues the same sequence as individual launches.
 * Replaces: the per-bounce inferenceStep/trainStep calls of
 * GuidedPathTracer::render (integrator.cpp:431-438, 463, 627-701), which are
 * host-driven launches in the reference.
 */
typedef struct nmg_bounce {
  nmg_shading in;
  const float* u4;
  const int* d_count;
  int n_max;
  nmg_query_out out;
  const float* train_x;
  const float* train_records;
  const int* train_count;
  int train_n_max;
  double* stats;
} nmg_bounce;

typedef struct nmg_frame nmg_frame;
nmg_status nmg_frame_capture(nmg_ctx* ctx, const nmg_bounce* bounces, int n_bounces, nmg_frame** frame);
nmg_status nmg_frame_launch(nmg_frame* frame, nmg_stream stream);
/* Graph nodes (kernel launches and memsets) one replay executes. */
int nmg_frame_nodes(const nmg_frame* frame);
void nmg_frame_destroy(nmg_frame* frame);
nmg_status nmg_frame_run_eager(nmg_ctx* ctx, const nmg_bounce* bounces, int n_bounces, nmg_stream stream);

/*
 * Autotuner: times the fused query kernel on the caller's inputs for every
 * candidate tiling (outputs are overwritten), keeps the fastest for this
 * context and reports it in *chosen. With use_cache the choice is read from /
 * appended to a text cache ($NMG_TUNE_CACHE, default ~/.cache/nmg_tune.txt)
 * keyed by device, configuration and log2 of n. Synchronises the stream.
 */
nmg_status nmg_autotune_query(nmg_ctx* ctx, const nmg_shading* in, const float* u4, int n,
                              const nmg_query_out* out, int use_cache, int* chosen, nmg_stream stream);

/* Synchronises the device and reports an error recorded by a kernel of this
 * context since the last check (NMG_ERR_TIMEOUT when a bounded device wait
 * gave up). */
nmg_status nmg_check_errors(nmg_ctx* ctx);

/*
 * Failure-detection self-test (no counterpart in the reference, which exits
 * through Log(Fatal) instead of reporting device-side failures). Launches,
 * on `stream`, one thread that waits through the same bounded device wait
 * the fused kernels use on a barrier nothing arrives at: after about 2e9 SM
 * cycles (about one second at the maximum clock) the wait gives up, the
 * kernel records a timeout in the context's device error flag and returns.
 * The next nmg_check_errors then returns NMG_ERR_TIMEOUT and clears the
 * flag; the context stays usable. NMG_ERR_UNSUPPORTED for a context without
 * fused kernel state: the plain FP32 path (it has no device waits), or a
 * 16-bit configuration before its first nmg_reserve.
 */
nmg_status nmg_selftest_wait_timeout(nmg_ctx* ctx, nmg_stream stream);

/* Host-file checkpoint of {master params, inference params, Adam moments,
 * step counters, step}. */
nmg_status nmg_save(const nmg_ctx* ctx, const char* path);
nmg_status nmg_load(nmg_ctx* ctx, const char* path);

/* Parameters in tiny-cuda-nn's Trainer snapshot format: the MessagePack
 * encoding (nlohmann::json::to_msgpack) of the object Trainer::serialize
 * returns, {"n_params", "params_binary", "params_type"}
 * (src/ext/tcnn/include/tiny-cuda-nn/trainer.h:267-305). The parameter
 * vector is the network's [MLP | grid] in the reference's layout
 * (network.h:85-100), so weights trained by the reference load here and the
 * reverse. Export writes the inference (EMA) parameters as "__half"
 * (params_type 0, tcnn's network precision) or "float" (1); import accepts
 * either, ignores an "optimizer" entry and sets both parameter copies
 * (resetting Adam, as nmg_set_params). No reference call site: the
 * reference saves no networks. */
nmg_status nmg_export_tcnn(const nmg_ctx* ctx, const char* path, int params_type);
nmg_status nmg_import_tcnn(nmg_ctx* ctx, const char* path, nmg_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* NMG_H_ */
