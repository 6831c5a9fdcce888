// fused_train.cu -- the fused reduced-precision training step on tcgen05.
//
// One persistent CTA per SM, one warpgroup (128 threads) walking tiles of
// 128 training records. For each tile, entirely on chip:
//   encode the input rows into a BF16/FP16 operand tile (A0)
//   forward:  h0 = relu(A0 W0^T), h1, h2 (kept in shared memory), raw = h2 W3^T
//   adjoint:  KL loss and dL/draw per record in registers (train.cu:69-124)
//   backward: for l = 3..0
//               weight gradient  dW_l += delta_l^T h_{l-1}   (M = 64, MN-major
//                                operand views, accumulated in TMEM across
//                                all tiles of the CTA)
//               data gradient    delta_{l-1} = (delta_l W_l) * relu'(h_{l-1})
//   grid:     dL/d(grid features) scattered into the table gradient with
//             float2 atomics (grid.h:387-510).
// Activations never reach HBM, so memory use does not grow with the batch
// (the recompute-instead-of-store mode of large batches is the only mode).
// After the last tile each CTA adds its TMEM weight gradients into the
// global gradient. Adam + EMA then run as one streaming kernel.
//
// TMEM (512 columns): [0,128) forward/data-gradient accumulator (M = 128);
// [128,208) dW0, [208,272) dW1, [272,336) dW2, [336,384) dW3^T (M = 64:
// rows live in lanes 0-15 of each 32-lane subpartition).
//
// Gradient scale: delta is the reference's loss_scale/n scaled gradient
// (train.cu:80) multiplied by S (n for BF16, min(n, 256) for FP16) to keep
// it in range of the 16-bit operand format; the global gradient is written
// with the 1/S factor back, so it carries the same loss_scale/n scaling as
// the reference's.
#include <stdio.h>
#include <string.h>

#include "api_common.cuh"
#include "fused_common.cuh"

namespace nmg {

constexpr uint32_t kColD = 0, kColW0 = 128, kColW1 = 208, kColW2 = 272, kColW3 = 336, kTrainCols = 512;

struct TrainArgs {
  FusedArgs f;          // encoding, weights image (training weights), table
  const float* x;       // [n][n_input]
  const float* rec;     // [n][rstride]
  int rstride;
  float loss_scale;
  float* grad;          // [n_params] FP32, zeroed by the caller
  long n_mlp;
  long layer_elem_off[kMaxLayers];  // element offset of each weight matrix in the parameter vector
  double* partials;     // [gridDim.x] loss partial sums
};

template <int K, int NOUTMAX>
NMG_D float tile_loss(const TrainArgs& a, const float (&r)[NOUTMAX], const float* rec, float scale, float* g) {
  if (a.f.selection) return mix_kl_loss_grad_selection<K, true>(r, rec, scale, a.f.mix, g);
  return mix_kl_loss_grad<K, true>(r, rec, scale, a.f.mix, g);
}

NMG_D void issue_mma_kmajor(uint32_t tmem, uint32_t a_addr, int a_chunks, uint32_t b_addr, uint32_t b_lbo,
                            uint32_t b_sbo, uint32_t b_step, int N, int ksteps, bool fp16, bool b_mn) {
  const uint32_t idesc = tc::idesc_f16(kRows, N, fp16, false, b_mn);
  for (int kk = 0; kk < ksteps; ++kk)
    tc::mma_f16(tmem, tc::smem_desc(a_addr + kk * 256u, 128u, uint32_t(a_chunks) * 128u),
                tc::smem_desc(b_addr + kk * b_step, b_lbo, b_sbo), idesc, kk > 0 ? 1u : 0u);
}

// dW (M = 64 rows of `a_tile` chunks, N = columns of `b_tile` chunks) +=
// a_tile^T b_tile over the 128 rows (K) of both tiles, MN-major views.
NMG_D void issue_wgrad(uint32_t tmem, uint32_t a_addr, int a_chunks, uint32_t b_addr, int b_chunks, int N,
                       bool fp16, bool accumulate) {
  const uint32_t idesc = tc::idesc_f16(64, N, fp16, true, true);
  for (int kk = 0; kk < kRows / 16; ++kk)
    tc::mma_f16(tmem, tc::smem_desc(a_addr + kk * 2u * a_chunks * 128u, uint32_t(a_chunks) * 128u, 128u),
                tc::smem_desc(b_addr + kk * 2u * b_chunks * 128u, uint32_t(b_chunks) * 128u, 128u), idesc,
                (accumulate || kk > 0) ? 1u : 0u);
}

// Reads 16-bit row `row` of a core-matrix tile (chunk c) as 8 floats.
NMG_D void load_chunk(const uint8_t* tile, int row, int chunk, int chunks, float* f, bool fp16) {
  const uint4 v = *reinterpret_cast<const uint4*>(tile + tc::cm_offset(row, chunk, chunks));
  float2 p;
  p = tc::unpack2(v.x, fp16);
  f[0] = p.x;
  f[1] = p.y;
  p = tc::unpack2(v.y, fp16);
  f[2] = p.x;
  f[3] = p.y;
  p = tc::unpack2(v.z, fp16);
  f[4] = p.x;
  f[5] = p.y;
  p = tc::unpack2(v.w, fp16);
  f[6] = p.x;
  f[7] = p.y;
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH>
__global__ void __launch_bounds__(kRows, 1) k_fused_train(const __grid_constant__ TrainArgs ta) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  constexpr uint32_t A_BYTES = kRows * NENC * 2;
  constexpr uint32_t H_BYTES = kRows * kWidth * 2;
  constexpr uint32_t D_BYTES = kRows * (NOUTMAX > kWidth ? NOUTMAX : kWidth) * 2;  // delta tile (output width)
  constexpr int NL = 4;  // three hidden layers
  static_assert(LEVELS * F <= 64, "grid features are read from the first 64 columns");
  extern __shared__ __align__(1024) uint8_t smem[];
  const FusedArgs& a = ta.f;

  const uint32_t w_region = (a.w_bytes + 1023u) & ~1023u;
  const int t = threadIdx.x, warp = t / 32, lane = t % 32;
  uint8_t* wsm = smem;
  uint8_t* A0 = smem + w_region;
  uint8_t* Hs = A0 + A_BYTES;              // three hidden tiles
  uint8_t* Dt = Hs + 3 * H_BYTES;          // delta tile
  uint64_t* bars = reinterpret_cast<uint64_t*>(Dt + D_BYTES);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 4);
  const bool fp16 = a.fp16 != 0;
  const int nout = a.n_out_pad;
  const int KC3 = nout / 8;

  if (t == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::fence_mbar_init();
  }
  if (t < 32) tc::tmem_alloc(tslot, kTrainCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (t == 0) {
    tc::mbar_arrive_expect_tx(&bars[0], a.w_bytes);
    for (uint32_t off = 0; off < a.w_bytes; off += 16384u) {
      const uint32_t nb = a.w_bytes - off < 16384u ? a.w_bytes - off : 16384u;
      tc::bulk_g2s(wsm + off, a.wimg + off, nb, &bars[0]);
    }
  }
  bool ok = tc::mbar_wait(&bars[0], 0);
  ok = __syncthreads_and(ok) != 0;

  const uint32_t tbase = *tslot;
  const uint32_t tD = tbase + kColD;
  const uint32_t lane_addr = tbase + (uint32_t(warp * 32) << 16);
  uint64_t* bar = &bars[1];
  uint32_t phase = 0;
  const int n = fused_count(a.d_count, a.n_max);
  const int ntiles = (n + kRows - 1) / kRows;
  const float scale = n > 0 ? ta.loss_scale / float(n) : 0.f;          // reference gradient scale
  const float S = fp16 ? fminf(float(n), 256.f) : float(n > 0 ? n : 1);  // operand range factor
  const float inv_S = 1.f / S;
  const uint32_t w_addr = tc::smem_u32(wsm);
  double loss_acc = 0.0;
  bool first = true;

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long q = long(tile) * kRows + t;
    const bool valid = q < n;
    float x[10];
#pragma unroll
    for (int d = 0; d < 10; ++d) x[d] = 0.f;
    if (valid) load_row(ta.x, q, a.enc.n_input, x);
    encode_row<F, LEVELS, MODE, SHDEG, BINS, SMOOTH>(a, x, A0, t);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    ok = bar_red_and(1, kRows, ok);
    if (!ok) break;

    // ------------------------------------------------------------ forward
    float r[NOUTMAX];
#pragma unroll
    for (int i = 0; i < NOUTMAX; ++i) r[i] = 0.f;
    for (int l = 0; l < NL; ++l) {
      const bool last = l == NL - 1;
      const int kin = l == 0 ? NENC : kWidth;
      if (t == 0) {
        tc::fence_after_sync();
        const uint32_t a_addr = tc::smem_u32(l == 0 ? A0 : Hs + (l - 1) * H_BYTES);
        const uint32_t sbo = uint32_t(kin / 8) * 128u;
        issue_mma_kmajor(tD, a_addr, kin / 8, w_addr + a.layer_off[l], 128u, sbo, 256u, last ? nout : kWidth,
                         kin / 16, fp16, false);
        tc::mma_commit(bar);
      }
      const bool done = tc::mbar_wait(bar, phase);
      phase ^= 1u;
      tc::fence_after_sync();
      if (!last) {
        float v[kWidth];
#pragma unroll
        for (int c = 0; c < kWidth / 16; ++c) tc::tmem_ld16(lane_addr + kColD + c * 16, v + 16 * c);
        tc::tmem_wait_ld();
        uint8_t* H = Hs + l * H_BYTES;
#pragma unroll
        for (int c = 0; c < kWidth / 8; ++c) {
          float fv[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) fv[i] = fmaxf(v[8 * c + i], 0.f);
          store_chunk(H, t, c, kWidth / 8, fv, fp16);
        }
      } else {
#pragma unroll
        for (int c = 0; c < NOUTMAX / 16; ++c)
          if (c * 16 < nout) tc::tmem_ld16(lane_addr + kColD + c * 16, r + 16 * c);
        tc::tmem_wait_ld();
      }
      tc::fence_proxy_async();
      tc::fence_before_sync();
      ok = bar_red_and(1, kRows, done);
      if (!ok) break;
    }
    if (!ok) break;

    // ------------------------------------------------- loss and adjoint
    {
      float g[NOUTMAX];
#pragma unroll
      for (int i = 0; i < NOUTMAX; ++i) g[i] = 0.f;
      if (valid) {
        float rr[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) rr[j] = j < ta.rstride ? ta.rec[q * ta.rstride + j] : 0.f;
        const float l = tile_loss<K, NOUTMAX>(ta, r, rr, scale, g);
        loss_acc += double(l);
      }
#pragma unroll
      for (int c = 0; c < NOUTMAX / 8; ++c) {
        if (c * 8 < nout) {
          float fv[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) fv[i] = g[8 * c + i] * S;
          store_chunk(Dt, t, c, KC3, fv, fp16);
        }
      }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    ok = bar_red_and(1, kRows, ok);
    if (!ok) break;

    // ------------------------------------------------------------ backward
    for (int l = NL - 1; l >= 0; --l) {
      const int dchunks = l == NL - 1 ? KC3 : kWidth / 8;   // chunks per row of delta_l
      const int dwidth = l == NL - 1 ? nout : kWidth;       // width of delta_l
      const int in_w = l == 0 ? NENC : kWidth;               // width of layer l's input
      const uint8_t* hin = l == 0 ? A0 : Hs + (l - 1) * H_BYTES;
      if (t == 0) {
        tc::fence_after_sync();
        // weight gradient of layer l
        if (l == NL - 1) {
          // dW3^T [in = 64][out] += h2^T delta3
          issue_wgrad(tbase + kColW3, tc::smem_u32(hin), kWidth / 8, tc::smem_u32(Dt), dchunks, dwidth, fp16, !first);
        } else {
          const uint32_t col = l == 0 ? kColW0 : (l == 1 ? kColW1 : kColW2);
          issue_wgrad(tbase + col, tc::smem_u32(Dt), dchunks, tc::smem_u32(hin), in_w / 8, in_w, fp16, !first);
        }
        // data gradient: delta_l [128 x dwidth] times W_l [dwidth x in_w]; W_l's image read as MN-major
        const uint32_t wk = uint32_t(in_w / 8) * 128u;  // image bytes per 8 rows of W_l (one K group)
        issue_mma_kmajor(tD, tc::smem_u32(Dt), dchunks, w_addr + a.layer_off[l], wk, 128u, 2u * wk, in_w, dwidth / 16,
                         fp16, true);
        tc::mma_commit(bar);
      }
      const bool done = tc::mbar_wait(bar, phase);
      phase ^= 1u;
      tc::fence_after_sync();
      if (l > 0) {
        float v[kWidth];
#pragma unroll
        for (int c = 0; c < kWidth / 16; ++c) tc::tmem_ld16(lane_addr + kColD + c * 16, v + 16 * c);
        tc::tmem_wait_ld();
        const uint8_t* H = Hs + (l - 1) * H_BYTES;
#pragma unroll
        for (int c = 0; c < kWidth / 8; ++c) {
          float hv[8], fv[8];
          load_chunk(H, t, c, kWidth / 8, hv, fp16);
#pragma unroll
          for (int i = 0; i < 8; ++i) fv[i] = hv[i] > 0.f ? v[8 * c + i] : 0.f;
          store_chunk(Dt, t, c, kWidth / 8, fv, fp16);
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        ok = bar_red_and(1, kRows, done);
        if (!ok) break;
      } else {
        // dL/d(encoded input): the grid columns feed the table gradient
        float dg[LEVELS * F];
#pragma unroll
        for (int c = 0; c < (LEVELS * F + 15) / 16; ++c) tc::tmem_ld16(lane_addr + kColD + c * 16, dg + 16 * c);
        tc::tmem_wait_ld();
        ok = done;
        if (valid && ok) {
          const float p3[3] = {x[0], x[1], x[2]};
          float* gt = ta.grad + ta.n_mlp;
#pragma unroll
          for (int lv = 0; lv < LEVELS; ++lv) {
            float w[3];
            uint32_t gc[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) pos_fract(p3[d], a.enc.scale[lv], a.enc.smoothstep, &w[d], &gc[d]);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
              const float wt = ((c & 1) ? w[0] : 1.f - w[0]) * ((c & 2) ? w[1] : 1.f - w[1]) *
                               ((c & 4) ? w[2] : 1.f - w[2]) * inv_S;
              const uint32_t e = a.enc.offset[lv] +
                                 level_index(a, lv, gc[0] + (c & 1), gc[1] + ((c >> 1) & 1), gc[2] + ((c >> 2) & 1));
              if (F == 2) {
                atomicAdd(reinterpret_cast<float2*>(gt) + e, make_float2(wt * dg[2 * lv], wt * dg[2 * lv + 1]));
              } else {
#pragma unroll
                for (int k = 0; k < F; k += 2)
                  atomicAdd(reinterpret_cast<float2*>(gt + size_t(e) * F + k),
                            make_float2(wt * dg[F * lv + k], wt * dg[F * lv + k + 1]));
              }
            }
          }
        }
      }
    }
    if (!ok) break;
    first = false;
  }

  // ---- flush this CTA's weight gradients (M = 64 accumulators) to global
  tc::fence_before_sync();
  ok = __syncthreads_and(ok) != 0;
  tc::fence_after_sync();
  if (ok && !first) {
    const int row = warp * 16 + lane;  // valid for lane < 16
    const uint32_t cols[4] = {kColW0, kColW1, kColW2, kColW3};
    const int widths[4] = {NENC, kWidth, kWidth, 64};  // dW3^T has out (<= 64 used) columns
    for (int m = 0; m < 4; ++m) {
      const int ncols = m == 3 ? nout : widths[m];
      for (int c0 = 0; c0 < ncols; c0 += 16) {
        float v[16];
        tc::tmem_ld16(lane_addr + cols[m] + c0, v);
        tc::tmem_wait_ld();
        if (lane < 16) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int col = c0 + i;
            if (col >= ncols) continue;
            long idx;
            if (m < 3)
              idx = ta.layer_elem_off[m] + long(row) * widths[m] + col;  // dW_m[out = row][in = col]
            else
              idx = ta.layer_elem_off[3] + long(col) * kWidth + row;     // W3[out = col][in = row]
            atomicAdd(ta.grad + idx, v[i] * inv_S);
          }
        }
      }
    }
  }
  if (!ok && t == 0) atomicExch(a.err, 3);
  // loss partial sum of this CTA
  {
    __shared__ double red[4];
    double v = loss_acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (t == 0) ta.partials[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
  }
  tc::fence_before_sync();
  __syncthreads();
  if (t < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tbase, kTrainCols);
  }
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH>
static nmg_status launch_train(const TrainArgs& a, int grid, cudaStream_t st) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  auto kern = k_fused_train<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH>;
  constexpr int DW = NOUTMAX > kWidth ? NOUTMAX : kWidth;
  const size_t smem = size_t((a.f.w_bytes + 1023u) & ~1023u) + size_t(kRows) * NENC * 2 +
                      3 * size_t(kRows) * kWidth * 2 + size_t(kRows) * DW * 2 + 128;
  nmg_status s = ensure_smem(reinterpret_cast<const void*>(kern), smem);
  if (s != NMG_OK) return s;
  kern<<<grid, kRows, smem, st>>>(a);
  return check_launch("k_fused_train");
}

nmg_status fused_train_step(nmg_ctx* c, const float* x, const float* rec, const int* d_count, int n_max,
                            double* stats, cudaStream_t st) {
  FusedState* s = fstate(c);
  if (!s) return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
  if (c->lay.n_layers != 4) return set_error(NMG_ERR_UNSUPPORTED, "fused training needs 3 hidden layers");
  TrainArgs a;
  memset(&a, 0, sizeof(a));
  a.f = fused_make_args(c, false);
  a.f.d_count = d_count;
  a.f.n_max = n_max;
  a.x = x;
  a.rec = rec;
  a.rstride = c->lay.record_floats;
  a.loss_scale = c->cfg.loss_scale;
  a.grad = c->grad;
  a.n_mlp = c->lay.n_mlp;
  for (int l = 0; l < c->lay.n_layers; ++l) a.layer_elem_off[l] = c->lay.off[l];
  a.partials = c->ws.partials;
  const int sms = sm_count();
  const int tiles = (n_max + kRows - 1) / kRows;
  int grid = tiles < sms ? tiles : sms;
  if (grid < 1) grid = 1;
  if (grid > c->ws.n_partials / 2) grid = c->ws.n_partials / 2;
  NMG_CUDA_TRY(cudaMemsetAsync(c->grad, 0, sizeof(float) * size_t(c->lay.n_params), st));
  NMG_CUDA_TRY(cudaMemsetAsync(c->ws.partials, 0, sizeof(double) * (c->ws.n_partials / 2), st));
  nmg_status r;
  switch (s->preset) {
    case 1: r = launch_train<2, 16, 1, 4, 4, 8, 48, false>(a, grid, st); break;
    case 2: r = launch_train<2, 16, 1, 4, 4, 16, 80, false>(a, grid, st); break;
    case 3: r = launch_train<4, 8, 0, 2, 4, 8, 48, true>(a, grid, st); break;
    default: return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
  }
  if (r != NMG_OK) return r;
  r = optimizer_step(c, d_count, n_max, stats, st);
  if (r != NMG_OK) return r;
  return pack_images(c, st);
}

}  // namespace nmg
