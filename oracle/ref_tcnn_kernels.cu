// ref_tcnn_kernels.cu -- extern "C" wrapper that runs the reference's own
// tiny-cuda-nn 1.7 kernels on the host (TEST INFRASTRUCTURE ONLY).
//
// oracle/build_ref.sh compiles this file against host-callable copies of
// tcnn's kernel headers (oracle/tcnn_host_headers.py: each header cut before
// its class, device-function qualifiers widened to host + device, kernels
// turned into host functions; the arithmetic is untouched). Each entry point
// calls one kernel once per thread index of the launch shape the matching
// tcnn class uses, in index order:
//   grid encoding forward   kernel_grid           (grid.h:220-384)
//   grid encoding backward  kernel_grid_backward  (grid.h:386-510)
//   spherical harmonics     kernel_sh             (spherical_harmonics.h:126-153)
//   one-blob                kernel_one_blob_soa   (oneblob.h:98-127; the same
//                           wrapped encoding as the AoS kernel, without its
//                           warp shuffle)
//   Adam                    adam_step             (adam.h:47-119)
//   EMA                     ema_step_full_precision / ema_step_half_precision
//                           (ema.h:44-76)
// Positions, directions and scalars come in as rows (AoS); encoded features
// and gradients use the kernels' own SoA layout [feature][element].
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <limits>
#include <vector>

namespace tcnn_host_launch {
uint3 thread_idx, block_idx;
dim3 block_dim;
inline void set(uint32_t bx, uint32_t by, uint32_t bdx, uint32_t tx, uint32_t ty = 0, uint32_t bdy = 1) {
  block_idx = make_uint3(bx, by, 0);
  thread_idx = make_uint3(tx, ty, 0);
  block_dim = dim3(bdx, bdy, 1);
}
}  // namespace tcnn_host_launch

namespace tcnn {
// The kernels' float gradient accumulation, on the host (threads run one
// after the other, so a plain add is the atomic's effect).
inline float atomicAdd(float* a, float v) {
  const float old = *a;
  *a = old + v;
  return old;
}
// Only the AoS one-blob kernel shuffles, and it is never called here.
inline float __shfl_sync(unsigned, float, int, int) { abort(); }
}  // namespace tcnn

#define threadIdx ::tcnn_host_launch::thread_idx
#define blockIdx ::tcnn_host_launch::block_idx
#define blockDim ::tcnn_host_launch::block_dim
#include <tiny-cuda-nn/encodings/grid.h>
#include <tiny-cuda-nn/encodings/oneblob.h>
#include <tiny-cuda-nn/encodings/spherical_harmonics.h>
#include <tiny-cuda-nn/optimizers/adam.h>
#include <tiny-cuda-nn/optimizers/ema.h>
#undef threadIdx
#undef blockIdx
#undef blockDim

using namespace tcnn;

namespace {
GridOffsetTable offsets_of(const uint32_t* offsets, int levels) {
  GridOffsetTable t;
  for (int l = 0; l <= levels; ++l) t.data[l] = offsets[l];
  t.size = uint32_t(levels + 1);
  return t;
}
}  // namespace

extern "C" {

// Grid features enc[levels * F][n] (SoA) of positions pos[n][3] for a table
// of `offsets[levels]` entries x F float features. hash: 1 = GridType::Hash
// (coherent-prime hash, tcnn's default for HashGrid), 0 = Dense; smoothstep
// selects InterpolationType::Smoothstep instead of Linear.
int ref_tcnn_grid_forward(int F, int levels, const uint32_t* offsets, uint32_t base_res, float per_level_scale,
                          int hash, int smoothstep, const float* table, const float* pos, uint32_t n, float* enc) {
  const GridOffsetTable ot = offsets_of(offsets, levels);
  const MatrixView<const float> in(pos, 1, 3);
  const InterpolationType it = smoothstep ? InterpolationType::Smoothstep : InterpolationType::Linear;
  const GridType gt = hash ? GridType::Hash : GridType::Dense;
  constexpr uint32_t kThreads = 512;  // N_THREADS_HASHGRID of the forward launch (grid.h:1039-1040)
  for (uint32_t level = 0; level < uint32_t(levels); ++level)
    for (uint32_t i = 0; i < n; ++i) {
      tcnn_host_launch::set(i / kThreads, level, kThreads, i % kThreads);
      if (F == 2)
        kernel_grid<float, 3, 2, HashType::CoherentPrime>(n, levels * F, ot, base_res, std::log2(per_level_scale),
                                                          1000.f, nullptr, it, gt, table, in, enc, nullptr);
      else if (F == 4)
        kernel_grid<float, 3, 4, HashType::CoherentPrime>(n, levels * F, ot, base_res, std::log2(per_level_scale),
                                                          1000.f, nullptr, it, gt, table, in, enc, nullptr);
      else
        return -1;
    }
  return 0;
}

// Table gradient grad[offsets[levels] * F] (accumulated) of dL/d(features)
// dl_dy[levels * F][n] (SoA) at positions pos[n][3].
int ref_tcnn_grid_backward(int F, int levels, const uint32_t* offsets, uint32_t base_res, float per_level_scale,
                           int hash, int smoothstep, const float* pos, uint32_t n, const float* dl_dy, float* grad) {
  const GridOffsetTable ot = offsets_of(offsets, levels);
  const MatrixView<const float> in(pos, 1, 3);
  const InterpolationType it = smoothstep ? InterpolationType::Smoothstep : InterpolationType::Linear;
  const GridType gt = hash ? GridType::Hash : GridType::Dense;
  constexpr uint32_t kThreads = 256, kPerThread = 2;  // grid.h:1135-1138
  const uint32_t work = n * uint32_t(F) / kPerThread;
  for (uint32_t level = 0; level < uint32_t(levels); ++level)
    for (uint32_t w = 0; w < work; ++w) {
      tcnn_host_launch::set(w / kThreads, level, kThreads, w % kThreads);
      if (F == 2)
        kernel_grid_backward<float, float, 3, 2, 2, HashType::CoherentPrime>(
            n, levels * F, ot, base_res, std::log2(per_level_scale), 1000.f, nullptr, false, it, gt, grad, in, dl_dy);
      else if (F == 4)
        kernel_grid_backward<float, float, 3, 4, 2, HashType::CoherentPrime>(
            n, levels * F, ot, base_res, std::log2(per_level_scale), 1000.f, nullptr, false, it, gt, grad, in, dl_dy);
      else
        return -1;
    }
  return 0;
}

// Real spherical harmonics of degree `degree` of directions given as (d + 1) / 2
// rows in[n][3]: out[n][degree^2] (rows).
void ref_tcnn_sh(uint32_t degree, const float* in, uint32_t n, float* out) {
  const MatrixView<const float> vin(in, 1, 3);
  const MatrixView<float> vout(out, 1, degree * degree);
  for (uint32_t i = 0; i < n; ++i) {
    tcnn_host_launch::set(i / 128, 0, 128, i % 128);
    kernel_sh<float>(n, degree, 0, vin, vout);
  }
}

// One-blob encoding with 2^bins_log2 bins of dims values per row in[n][dims]:
// out[dims * bins][n] (SoA, dimension-major), the launch shape of
// OneBlobEncoding's SoA path (oneblob.h:211-222) with one element per block.
void ref_tcnn_oneblob(uint32_t bins_log2, const float* in, uint32_t n, uint32_t dims, float* out) {
  const MatrixView<const float> vin(in, 1, dims);
  for (uint32_t i = 0; i < n; ++i)
    for (uint32_t j = 0; j < dims; ++j) {
      tcnn_host_launch::set(i, 0, dims, j);
      kernel_one_blob_soa<float>(n, bins_log2, dims, vin, out);
    }
}

// One optimiser step of tcnn's EMA(Adam) on n parameters (the first n_matrix
// are matrix weights): adam_step with the given hyperparameters (no weight
// decay, clipping or learning-rate bounds: adam.h's defaults), then the EMA at
// `step` (the optimiser's step count after this call) in full precision
// (ema_tmp holds the FP32 average) or, with full_precision = 0, on the 16-bit
// weights. Weights and gradients are __half as in the reference's network
// (precision_t); they travel here as float and are rounded on the way in.
void ref_tcnn_adam_ema(uint32_t n, uint32_t n_matrix, float loss_scale, float lr, float beta1, float beta2,
                       float eps, float l2_reg, float ema_decay, uint32_t step, int full_precision,
                       float* w_full, float* w16, const float* grad16, float* m, float* v, uint32_t* psteps,
                       float* ema16, float* ema_tmp) {
  std::vector<__half> w(n), g(n), e(n);
  for (uint32_t i = 0; i < n; ++i) {
    w[i] = __float2half(w16[i]);
    g[i] = __float2half(grad16[i]);
    e[i] = __float2half(ema16[i]);
  }
  for (uint32_t i = 0; i < n; ++i) {
    tcnn_host_launch::set(i / 128, 0, 128, i % 128);
    adam_step<__half>(n, n_matrix, 0.f, 0.f, 0.f, loss_scale, lr, 1.f, true, true, beta1, beta2, eps, 0.f,
                      std::numeric_limits<float>::max(), l2_reg, w_full, w.data(), g.data(), m, v, psteps);
  }
  // EmaOptimizer::step (ema.h:107-108): std::pow of the float decay and the unsigned step
  const float debias_old = 1 - (float)std::pow(ema_decay, step - 1);
  const float debias_new = 1.0f / (1 - (float)std::pow(ema_decay, step));
  for (uint32_t i = 0; i < n; ++i) {
    tcnn_host_launch::set(i / 128, 0, 128, i % 128);
    if (full_precision)
      ema_step_full_precision<__half>(n, ema_decay, debias_old, debias_new, w.data(), e.data(), ema_tmp);
    else
      ema_step_half_precision<__half>(n, ema_decay, debias_old, debias_new, w.data(), e.data());
  }
  for (uint32_t i = 0; i < n; ++i) {
    w16[i] = __half2float(w[i]);
    ema16[i] = __half2float(e[i]);
  }
}

}  // extern "C"
