// fused.cu -- the fused reduced-precision guiding step on the sm_103a tensor
// cores: one persistent kernel per wavefront does
//   featurise -> encode (grid gathers + SH + one-blob, BF16/FP16 into a
//   shared-memory operand tile) -> MLP on tcgen05 (FP32 accumulators in TMEM,
//   ReLU epilogues back to shared memory) -> mixture activation, cosine lobe,
//   lobe selection, vMF sample and pdf (FP32, registers).
//
// CTA organisation (one CTA per SM, 512 threads): four independent
// warpgroups, each owning a 128-query tile at a time, its operand tiles in
// shared memory, a TMEM accumulator slice and an mbarrier. Thread t of a
// warpgroup owns row t of the tile: it encodes the row, reads the row back
// from TMEM lanes (warp w of the group reads lanes 32w..32w+31) and runs the
// mixture for that query. The weights of all layers (32 KB for the hash-grid
// network) are copied once per CTA into shared memory by a bulk copy
// (cp.async.bulk) from a pre-packed image in core-matrix order and stay
// resident. One elected thread per warpgroup issues that group's MMAs and
// commits them to the group's mbarrier.
//
// Matches the reference semantics of the plain path (encoding grid.h,
// spherical_harmonics.h, oneblob.h; MLP fully_fused_mlp.cu; mixture
// distribution.h / vmf.h) up to the BF16/FP16 rounding of features,
// weights and activations, and fast-math transcendental functions.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <string>

#include "api_common.cuh"
#include "ctx.cuh"
#include "tcgen05.cuh"
#include "fused_common.cuh"

namespace nmg {

// STREAM: the mixture epilogue reads the raw outputs from TMEM lobe group by
// lobe group (query_epilogue_streamed) instead of holding them in registers;
// used for 16-lobe queries that return no raw outputs.
template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH, int NWG,
          bool STREAM = false>
__global__ void __launch_bounds__(NWG * kRows, 1) k_fused_query(const __grid_constant__ FusedArgs a) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  // One operand tile per warpgroup: the encoded inputs, then (once the first
  // layer's MMA has read them) the hidden activations of every later layer.
  constexpr uint32_t TILE_BYTES = kRows * (NENC > kWidth ? NENC : kWidth) * 2;
  constexpr uint32_t COLS = NOUTMAX <= 64 ? 64 : 128;  // TMEM columns per warpgroup
  constexpr uint32_t TCOLS = COLS * NWG <= 256 ? (COLS * NWG <= 128 ? 128 : 256) : 512;
  static_assert(COLS * NWG <= 512, "TMEM holds 512 columns");
  extern __shared__ __align__(1024) uint8_t smem[];

  const uint32_t w_region = (a.w_bytes + 1023u) & ~1023u;
  const int wg = threadIdx.x / kRows, t = threadIdx.x % kRows, warp_in_wg = t / 32;
  uint8_t* wsm = smem;
  uint8_t* A = smem + w_region + wg * TILE_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + w_region + NWG * TILE_BYTES);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 8);

  if (threadIdx.x == 0) {
    tc::mbar_init(&bars[0], 1);
    for (int g = 0; g < NWG; ++g) tc::mbar_init(&bars[1 + g], 1);
    tc::fence_mbar_init();
  }
  if (threadIdx.x < 32) tc::tmem_alloc(tslot, TCOLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&bars[0], a.w_bytes);
    for (uint32_t off = 0; off < a.w_bytes; off += 16384u) {
      const uint32_t nb = a.w_bytes - off < 16384u ? a.w_bytes - off : 16384u;
      tc::bulk_g2s(wsm + off, a.wimg + off, nb, &bars[0]);
    }
  }
  bool ok = tc::mbar_wait(&bars[0], 0);
  ok = __syncthreads_and(ok) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(a.err, 1);

  const uint32_t tmem = *tslot + uint32_t(wg) * COLS;
  const uint32_t lane_addr = tmem + (uint32_t(warp_in_wg * 32) << 16);
  uint64_t* bar = &bars[1 + wg];
  uint32_t phase = 0;
  const int n = fused_count(a.d_count, a.n_max);
  const int ntiles = (n + kRows - 1) / kRows;
  const int nl = a.n_layers;
  const uint32_t a_addr = tc::smem_u32(A);
  constexpr bool streamed = STREAM;

  // Every early exit below follows a warpgroup-wide bar.red.and, so the 128
  // threads of a group always leave the loop together (no thread can be
  // left waiting at a named barrier).
  for (int tile = blockIdx.x * NWG + wg; tile < ntiles; tile += gridDim.x * NWG) {
    const long q = long(tile) * kRows + t;
    const bool valid = q < n;
    // ---- encode this thread's row into the tile
    float x[10];
#pragma unroll
    for (int d = 0; d < 10; ++d) x[d] = 0.f;
    if (valid) {
      if (a.raw_mode)
        load_row(a.x, q, a.enc.n_input, x);
      else
        featurize<true>(a.enc, load3(a.pos, q), load3(a.wo, q), load3(a.nrm, q), a.rough[q], x);
    }
    encode_row<F, LEVELS, MODE, SHDEG, BINS, SMOOTH, true, true>(a, x, A, t);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    ok = bar_red_and(1 + wg, kRows, ok);
    if (!ok) break;
    // ---- MLP: every layer reads the tile and writes TMEM; hidden layers write the tile back
    float r[NOUTMAX];
    bool last_ok = true;
    for (int l = 0; l < nl; ++l) {
      const bool last = l == nl - 1;
      const int kin = l == 0 ? NENC : kWidth;
      const int nout = last ? a.n_out_pad : kWidth;
      if (t == 0) {
        tc::fence_after_sync();
        issue_layer(a, l, tmem, a_addr, tc::smem_u32(wsm), kin, nout);
        tc::mma_commit(bar);
      }
      const bool done = tc::mbar_wait(bar, phase);
      phase ^= 1u;
      tc::fence_after_sync();
      if (!last) {
        float v[kWidth];
        tc::tmem_load<kWidth / 16>(lane_addr, v);
#pragma unroll
        for (int c = 0; c < kWidth / 8; ++c) store_chunk_relu(A, t, c, kWidth / 8, v + 8 * c, layer_fp16(a, l + 1));
        tc::fence_proxy_async();
        tc::fence_before_sync();
        ok = bar_red_and(1 + wg, kRows, done);
        if (!ok) break;
      } else {
        if constexpr (!streamed) {
          tc::tmem_load_n<NOUTMAX / 16>(lane_addr, r, (a.n_out_pad + 15) / 16);
        }
        last_ok = done;
      }
    }
    if (!ok) break;
    // ---- epilogue: raw outputs and/or mixture
    if constexpr (streamed) {
      // warp-collective TMEM reads: the group agrees on ok first; the accumulator stays
      // untouched until the next tile's layer 0, issued after the group's next barrier
      ok = bar_red_and(1 + wg, kRows, last_ok);
      if (!ok) break;
      query_epilogue_streamed<K>(a, q, valid, lane_addr);
    } else {
      ok = last_ok;  // reconciled across the group at the next tile's barrier
      if (valid && ok) query_epilogue<K, NOUTMAX>(a, q, r);
    }
  }
  if (!ok && t == 0) atomicExch(a.err, 2);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(*tslot, TCOLS);
  }
}

// Tiling 7: two pipelines per CTA, each two warpgroups on one 128-query tile
// (the layout of the training kernel): warps w and w + 4 read the same TMEM
// lane quadrant, so every query has two threads, which split the encoding's
// grid levels, each hidden epilogue's columns and the mixture's lobes. With
// K / 2 lobes per thread the lobes stay in registers from activation to pdf
// (one pass, where one thread holding all 16 re-derives them from TMEM);
// the lobe-weight total, the selection scan (continued by the second half
// where the first half's lobes ran out, the reference's sequential
// subtraction), the sampled lobe and the pdf's partial sums cross between
// the two through shared memory. Queries without raw outputs only.
template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH>
__global__ void __launch_bounds__(4 * kRows, 1) k_fused_query_pair(const __grid_constant__ FusedArgs a) {
  constexpr int NP = 2, KH = K / 2;
  static_assert(K % 8 == 0, "each half holds K / 2 lobes, whole 16-column TMEM groups");
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  constexpr uint32_t TILE_BYTES = kRows * (NENC > kWidth ? NENC : kWidth) * 2;
  constexpr uint32_t COLS = NOUTMAX <= kWidth ? kWidth : (NOUTMAX + 15) / 16 * 16;  // TMEM columns per pipeline
  constexpr uint32_t TCOLS = COLS * NP <= 128 ? 128 : 256;
  static_assert(COLS * NP <= 256, "two pipelines' accumulators within 256 columns");
  constexpr int XCH = 2 * kRows * 8;  // exchange floats per pipeline: [half][row][8]
  extern __shared__ __align__(1024) uint8_t smem[];

  const uint32_t w_region = (a.w_bytes + 1023u) & ~1023u;
  const int warp = threadIdx.x / 32;
  const int p = warp / 8, h = (warp / 4) & 1, t = threadIdx.x % kRows;
  const bool leader = h == 0 && t == 0;
  uint8_t* wsm = smem;
  uint8_t* A = smem + w_region + p * TILE_BYTES;
  float* xch = reinterpret_cast<float*>(smem + w_region + NP * TILE_BYTES) + p * XCH;
  float* mine = xch + (h * kRows + t) * 8;
  const float* other = xch + ((1 - h) * kRows + t) * 8;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + w_region + NP * TILE_BYTES + NP * XCH * 4);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1 + NP);

  if (threadIdx.x == 0) {
    tc::mbar_init(&bars[0], 1);
    for (int i = 0; i < NP; ++i) tc::mbar_init(&bars[1 + i], 1);
    tc::fence_mbar_init();
  }
  if (threadIdx.x < 32) tc::tmem_alloc(tslot, TCOLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&bars[0], a.w_bytes);
    for (uint32_t off = 0; off < a.w_bytes; off += 16384u) {
      const uint32_t nb = a.w_bytes - off < 16384u ? a.w_bytes - off : 16384u;
      tc::bulk_g2s(wsm + off, a.wimg + off, nb, &bars[0]);
    }
  }
  bool ok = tc::mbar_wait(&bars[0], 0);
  ok = __syncthreads_and(ok) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(a.err, 1);

  const uint32_t tmem = *tslot + uint32_t(p) * COLS;
  const uint32_t lane_addr = tmem + (uint32_t((warp & 3) * 32) << 16);
  uint64_t* bar = &bars[1 + p];
  uint32_t phase = 0;
  const int n = fused_count(a.d_count, a.n_max);
  const int ntiles = (n + kRows - 1) / kRows;
  const int nl = a.n_layers;
  const uint32_t a_addr = tc::smem_u32(A);
  const bool cosine = a.mix.cosine != 0;
  const float nb = prod_norm<true>(kCosineKappa);

  // Every named barrier is a bar.red.and over the pipeline's 256 threads, and
  // every early exit follows one, so the two warpgroups always leave together.
  for (int tile = blockIdx.x * NP + p; tile < ntiles; tile += gridDim.x * NP) {
    const long q = long(tile) * kRows + t;
    const bool valid = q < n;
    float x[10];
#pragma unroll
    for (int d = 0; d < 10; ++d) x[d] = 0.f;
    f3 wo3{0.f, 0.f, 1.f}, n3{0.f, 0.f, 1.f};
    if (valid) {
      wo3 = load3(a.wo, q);
      n3 = load3(a.nrm, q);
      featurize<true>(a.enc, load3(a.pos, q), wo3, n3, a.rough[q], x);
    }
    encode_row_half<F, LEVELS, MODE, SHDEG, BINS, SMOOTH, true>(a, x, A, t, h);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    ok = bar_red_and(1 + p, 2 * kRows, ok);
    if (!ok) break;
    // ---- MLP; this half's columns of each hidden layer, its lobes' raw outputs
    float rh[2 * K];
    float sel_logit = 0.f;
    bool last_ok = true;
    for (int l = 0; l < nl; ++l) {
      const bool last = l == nl - 1;
      const int kin = l == 0 ? NENC : kWidth;
      const int nout = last ? a.n_out_pad : kWidth;
      if (leader) {
        tc::fence_after_sync();
        issue_layer(a, l, tmem, a_addr, tc::smem_u32(wsm), kin, nout);
        tc::mma_commit(bar);
      }
      const bool done = tc::mbar_wait(bar, phase);
      phase ^= 1u;
      tc::fence_after_sync();
      if (!last) {
        float v[kWidth / 2];
        tc::tmem_load<kWidth / 32>(lane_addr + uint32_t(h * (kWidth / 2)), v);
#pragma unroll
        for (int c = 0; c < kWidth / 16; ++c)
          store_chunk_relu(A, t, h * (kWidth / 16) + c, kWidth / 8, v + 8 * c, layer_fp16(a, l + 1));
        tc::fence_proxy_async();
        tc::fence_before_sync();
        ok = bar_red_and(1 + p, 2 * kRows, done);
        if (!ok) break;
      } else {
        tc::tmem_load<K / 8>(lane_addr + uint32_t(h * 2 * K), rh);
        if (a.selection) {
          float v[16];
          tc::tmem_load<1>(lane_addr + uint32_t(4 * K), v);
          sel_logit = v[0];
        }
        last_ok = done;
      }
    }
    if (!ok) break;
    ok = bar_red_and(1 + p, 2 * kRows, last_ok);
    if (!ok) break;
    // ---- mixture: lobes [KH h, KH h + KH) (distribution.h:85-98, 184-195)
    f3 mb{0.f, 0.f, 1.f};
    if (cosine && valid) mb = unit3<true>(face_fwd(n3, wo3));
    float lam[KH], kap[KH], nrm[KH];
    f3 mu[KH];
    float part = 0.f;
#pragma unroll
    for (int i = 0; i < KH; ++i) {
      lobe_activate<true>(rh[4 * i], rh[4 * i + 1], rh[4 * i + 2], rh[4 * i + 3], a.mix.kappa_softplus, lam[i],
                          kap[i], mu[i]);
      // below M_EPSILON the lobe is uniform: kappa 0 (e^{0} and 1/4pi, no per-lobe branch in the pdf
      // or the sampler) and the branch-free normaliser
      const float kz = kap[i] < NMG_EPS ? 0.f : kap[i];
      nrm[i] = vmf_norm_sel(kz);
      if (cosine)
        lobe_cosine<true>(mb, nb, lam[i], kap[i], mu[i], nrm[i]);  // the product's kappa: 0 or >= 1e-3
      else
        kap[i] = kz;
      part += lam[i];
    }
    mine[0] = part;
    ok = bar_red_and(1 + p, 2 * kRows, ok);
    if (!ok) break;
    float total = h == 0 ? part + other[0] : other[0] + part;
    if (cosine) total = fmaxf(total, NMG_EPS);  // distribution.h:191
    const float inv = 1.f / total;
#pragma unroll
    for (int i = 0; i < KH; ++i) lam[i] *= inv;  // the lobe weights from here on
    f3 d{0.f, 0.f, 1.f};
    int sel = 0;
    if (a.wi) {
      if (valid) d = load3(a.wi, q);
    } else {
      // selection (distribution.h:132-140): half 0 scans its lobes with u and
      // hands the rest of u to half 1, which continues where lobe KH - 1 left off
      const float4 u = valid ? reinterpret_cast<const float4*>(a.u4)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
      float ks = kap[0];
      f3 ms = mu[0];
      if (h == 0) {
        float uu = u.y;
        int s0 = -1;
#pragma unroll
        for (int i = 0; i < KH; ++i) {
          if (s0 < 0) {
            if (uu < lam[i])
              s0 = i;
            else
              uu -= lam[i];
          }
        }
#pragma unroll
        for (int i = 1; i < KH; ++i)
          if (i == s0) {
            ks = kap[i];
            ms = mu[i];
          }
        mine[1] = __int_as_float(s0);
        mine[2] = uu;
        mine[3] = ks;  // lobe s0's, or lobe 0's when none of these was selected (the fallback)
        mine[4] = ms.x;
        mine[5] = ms.y;
        mine[6] = ms.z;
      }
      ok = bar_red_and(1 + p, 2 * kRows, ok);
      if (!ok) break;
      if (h == 1) {
        const int s0 = __float_as_int(other[1]);
        sel = s0;
        ks = other[3];
        ms = f3{other[4], other[5], other[6]};
        if (s0 < 0) {
          float uu = other[2];
          int s1 = -1;
#pragma unroll
          for (int i = 0; i < KH; ++i) {
            if (s1 < 0) {
              if (uu < lam[i])
                s1 = i;
              else
                uu -= lam[i];
            }
          }
          sel = 0;  // no lobe selected: lobe 0, whose parameters half 0 handed over
          if (s1 >= 0) {
            sel = KH + s1;
#pragma unroll
            for (int i = 0; i < KH; ++i)
              if (i == s1) {
                ks = kap[i];
                ms = mu[i];
              }
          }
        }
        mine[1] = __int_as_float(sel);
        mine[3] = ks;
        mine[4] = ms.x;
        mine[5] = ms.y;
        mine[6] = ms.z;
      }
      ok = bar_red_and(1 + p, 2 * kRows, ok);
      if (!ok) break;
      if (h == 0) {
        sel = __float_as_int(other[1]);
        ks = other[3];
        ms = f3{other[4], other[5], other[6]};
      }
      d = vmf_sample_lean(ks, ms, u.z, u.w);  // the same inputs in both halves
    }
    // pdf at d (distribution.h:113-119), this half's lobes
    float pd = 0.f;
#pragma unroll
    for (int i = 0; i < KH; ++i) {
      const float c = dot3(d, mu[i]);
      pd += lam[i] * (__expf(kap[i] * fminf(0.f, c - 1.f)) * nrm[i]);
    }
    mine[7] = pd;
    ok = bar_red_and(1 + p, 2 * kRows, ok);
    if (!ok) break;
    if (h == 0) {
      if (!a.wi) store3_warp(a.dir, q, d, valid);
      if (valid) {
        a.pdf[q] = pd + other[7];
        if (!a.wi && a.lobe) a.lobe[q] = sel;
        if (a.sel && a.selection) a.sel[q] = logistic<true>(sel_logit);
      }
    }
  }
  if (!ok && t == 0) atomicExch(a.err, 2);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(*tslot, TCOLS);
  }
}

// ------------------------------------------------------------ weight image
// Element (n, k) of layer l goes to byte layer_off[l] + cm_offset(n, k/8,
// in_l/8) + 2 (k % 8): each layer becomes a K-major operand of N = out_l rows,
// converted from the FP32 weights to the layer's operand format (PackArgs).
// W0's low parts, bf16(w - bf16(w)), go to the same place relative to
// w0_lo_off. blockIdx.y selects the image: 0 the training weights, 1 the
// inference ones.
__global__ void k_pack_weights(PackArgs p, const float* __restrict__ w_train, uint16_t* __restrict__ img_train,
                               const float* __restrict__ w_infer, uint16_t* __restrict__ img_infer) {
  const int which = blockIdx.y;
  const float* __restrict__ w = which ? w_infer : w_train;
  uint16_t* __restrict__ img = which ? img_infer : img_train;
  const uint32_t fp16_layers = p.fp16_layers[which], lo_off = p.w0_lo_off[which];
  const long total = p.off[p.n_layers];
  for (long i = long(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += long(gridDim.x) * blockDim.x) {
    int l = 0;
    while (l + 1 < p.n_layers && i >= p.off[l + 1]) ++l;
    const long j = i - p.off[l];
    const int in = p.in[l];
    const int nrow = int(j / in), k = int(j % in);
    const uint32_t b = tc::cm_offset(nrow, k >> 3, in >> 3) + uint32_t(k & 7) * 2u;
    const float v = w[i];
    if ((fp16_layers >> l) & 1u) {
      img[(p.layer_off[l] + b) >> 1] = __half_as_ushort(__float2half_rn(v));
    } else {
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      img[(p.layer_off[l] + b) >> 1] = __bfloat16_as_ushort(hi);
      if (l == 0 && lo_off)
        img[(lo_off + b) >> 1] = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(hi)));
    }
  }
}

// ------------------------------------------------------------------- host

static int preset_of(const nmg_ctx* c) {
  const nmg_config& g = c->cfg;
  const bool hash = g.input_mode == 1 && g.grid_features == 2 && g.grid_levels == 16 && g.sh_degree == 4 &&
                    g.oneblob_bins == 4;
  const bool ref = g.input_mode == 0 && g.grid_features == 4 && g.grid_levels == 8 && g.sh_degree == 2 &&
                   g.oneblob_bins == 4;
  if (hash && g.n_lobes == 8) return 1;
  if (hash && g.n_lobes == 16) return 2;
  if (ref && g.n_lobes == 8 && !g.selection) return 3;
  return 0;
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int NWG>
static size_t smem_bytes_for(uint32_t w_bytes) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  return size_t((w_bytes + 1023u) & ~1023u) + NWG * size_t(kRows) * (NENC > kWidth ? NENC : kWidth) * 2 + 128;
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH, int NWG>
static nmg_status launch_query_nwg(const FusedArgs& a, cudaStream_t st) {
  auto kern = k_fused_query<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, NWG>;
  if constexpr (K == 16)
    if (!a.raw && !a.raw_mode) kern = k_fused_query<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, NWG, true>;
  const size_t smem = smem_bytes_for<F, LEVELS, MODE, SHDEG, BINS, NWG>(a.w_bytes);
  nmg_status s = ensure_smem(reinterpret_cast<const void*>(kern), smem);
  if (s != NMG_OK) return s;
  const int sms = sm_count();
  const int tiles = (a.n_max + kRows - 1) / kRows;
  int grid = (tiles + NWG - 1) / NWG;
  if (grid > sms) grid = sms;
  if (grid < 1) grid = 1;
  kern<<<grid, NWG * kRows, smem, st>>>(a);
  return check_launch("k_fused_query");
}

// Warpgroups per CTA: 4 always fits (registers capped at 128 per thread);
// 5 and 6 trade registers for more resident warps (K = 8 only: TMEM holds
// 512 columns).
template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH>
static nmg_status launch_query(const FusedArgs& a, int nwg, cudaStream_t st) {
  if constexpr (NOUTMAX <= 64) {
    if (nwg == 5) return launch_query_nwg<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, 5>(a, st);
    if (nwg == 6) return launch_query_nwg<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, 6>(a, st);
  }
  return launch_query_nwg<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, 4>(a, st);
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH>
static nmg_status launch_query_pair(const FusedArgs& a, cudaStream_t st) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  auto kern = k_fused_query_pair<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH>;
  const size_t smem = size_t((a.w_bytes + 1023u) & ~1023u) +
                      2 * (size_t(kRows) * (NENC > kWidth ? NENC : kWidth) * 2 + 2 * size_t(kRows) * 8 * 4) + 128;
  nmg_status s = ensure_smem(reinterpret_cast<const void*>(kern), smem);
  if (s != NMG_OK) return s;
  const int sms = sm_count();
  const int tiles = (a.n_max + kRows - 1) / kRows;
  int grid = (tiles + 1) / 2;
  if (grid > sms) grid = sms;
  if (grid < 1) grid = 1;
  kern<<<grid, 4 * kRows, smem, st>>>(a);
  return check_launch("k_fused_query_pair");
}

// Default query tiling: the warp-specialised kernel (4 encoder + 2 consumer
// warpgroups) for the 8-lobe networks, measured 1.3x faster than one
// pipeline per warpgroup on a 2,073,600-query wavefront; for the hash-grid
// network its variant with the hidden activations kept in the ring slot
// (tiling 12: 32 KB more L1 for the table gathers) measured 630 us against
// 646 us. The 16-lobe network's consumer epilogue does not fit 128
// registers: it takes tiling 7, two threads per query with 8 lobes each in
// registers, 1.096 ms on a 2,073,600-query wavefront against 1.266 ms for one
// pipeline per warpgroup re-deriving the lobes from TMEM and 1.344 ms for the
// warp-specialised kernel (for 8 lobes tiling 7 measured 0.952 ms against
// 0.643 ms for tiling 12).
int fused_default_tiling(const nmg_ctx* c) {
  const FusedState* s = reinterpret_cast<const FusedState*>(c->ws.fused);
  if (!s) return 4;
  if (s->preset == 2) return kTilingPair;
  return s->preset == 1 ? kTilingWarpSpecialised + 4 : kTilingWarpSpecialised;
}

static nmg_status dispatch_query(nmg_ctx* c, const FusedArgs& a, cudaStream_t st) {
  const int nwg = c->query_wg > 0 ? c->query_wg : fused_default_tiling(c);
  if (nwg >= kTilingWarpSpecialised) return launch_query_ws(fstate(c)->preset, nwg, a, st);
  if (nwg == kTilingPair && !a.raw && !a.raw_mode) {
    switch (fstate(c)->preset) {
      case 1: return launch_query_pair<2, 16, 1, 4, 4, 8, 48, false>(a, st);
      case 2: return launch_query_pair<2, 16, 1, 4, 4, 16, 80, false>(a, st);
      case 3: return launch_query_pair<4, 8, 0, 2, 4, 8, 48, true>(a, st);
    }
  }
  switch (fstate(c)->preset) {
    case 1: return launch_query<2, 16, 1, 4, 4, 8, 48, false>(a, nwg, st);
    case 2: return launch_query<2, 16, 1, 4, 4, 16, 80, false>(a, nwg, st);
    case 3: return launch_query<4, 8, 0, 2, 4, 8, 48, true>(a, nwg, st);
  }
  return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
}

nmg_status pack_images(nmg_ctx* c, cudaStream_t st) {
  FusedState* s = fstate(c);
  if (!s) return NMG_OK;
  k_pack_weights<<<dim3(64, 2), 256, 0, st>>>(s->pack, c->w, reinterpret_cast<uint16_t*>(s->img_train), c->w_inf,
                                              reinterpret_cast<uint16_t*>(s->img_infer));
  return check_launch("k_pack_weights");
}

nmg_status fused_reserve(nmg_ctx* c) {
  const int preset = preset_of(c);
  if (!preset) return NMG_OK;  // fused calls will report UNSUPPORTED
  const Layout& L = c->lay;
  FusedState s{};
  s.preset = preset;
  uint32_t off = 0;
  s.pack.n_layers = L.n_layers;
  for (int l = 0; l < L.n_layers; ++l) {
    s.pack.off[l] = L.off[l];
    s.pack.in[l] = L.in[l];
    s.pack.layer_off[l] = off;
    off += uint32_t(L.in[l]) * uint32_t(L.out[l]) * 2u;
  }
  s.pack.off[L.n_layers] = L.off[L.n_layers];
  s.w_bytes = (off + 15u) & ~15u;
  // Operand formats. The FP16 path: every layer FP16. The BF16 path: the
  // training image all BF16; the inference image (the query and pdf passes)
  // runs the whole MLP on FP16 operands over the BF16 grid table: the encoder
  // packs the input tile in FP16 (the interpolated BF16 table values and the
  // direction encodings are then carried more precisely than in BF16).
  // Against the FP64 network on the FP32 weights, all-BF16 operands left a pdf
  // error of 1.8e-3 at the maximum over 65,536 queries; the hidden
  // activations of this bias-free ReLU network are O(1), within FP16's range,
  // and its 11 significant bits instead of BF16's 8 carry the precision.
  const bool all16 = c->cfg.path == NMG_PATH_FP16;
  const uint32_t all_layers = (1u << L.n_layers) - 1u;
  s.pack.fp16_layers[0] = all16 ? all_layers : 0u;
  s.pack.w0_lo_off[0] = 0;
  s.pack.fp16_layers[1] = all_layers;
  s.pack.w0_lo_off[1] = 0;
  s.w_bytes_inf = s.w_bytes;
  const size_t head = 256;
  const size_t bytes = head + size_t(s.w_bytes) + size_t(s.w_bytes_inf);
  void* mem = nullptr;
  cudaError_t e = cudaMalloc(&mem, bytes);
  if (e != cudaSuccess) return set_error(NMG_ERR_OOM, "fused workspace: %s", cudaGetErrorString(e));
  cudaMemset(mem, 0, bytes);
  // the state struct lives on the host; its device buffers follow a 256-byte header
  FusedState* hs = new FusedState(s);
  hs->err = reinterpret_cast<int*>(mem);
  hs->img_train = reinterpret_cast<uint8_t*>(mem) + head;
  hs->img_infer = hs->img_train + s.w_bytes;
  c->ws.fused_dev = mem;
  c->ws.fused = hs;
  c->ws.fused_bytes = bytes;
  return pack_images(c, 0);
}

void fused_release(nmg_ctx* c) {
  delete fstate(c);
  c->ws.fused = nullptr;
}

FusedArgs fused_make_args(nmg_ctx* c, bool infer_weights) {
  FusedState* s = fstate(c);
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.enc = c->enc;
  a.mix = c->mix;
  a.wimg = infer_weights ? s->img_infer : s->img_train;
  a.w_bytes = infer_weights ? s->w_bytes_inf : s->w_bytes;
  for (int l = 0; l < c->lay.n_layers; ++l) a.layer_off[l] = s->pack.layer_off[l];
  a.n_layers = c->lay.n_layers;
  a.fp16 = c->cfg.path == NMG_PATH_FP16;
  a.fp16_layers = s->pack.fp16_layers[infer_weights ? 1 : 0];
  a.w0_lo_off = s->pack.w0_lo_off[infer_weights ? 1 : 0];
  a.table = (infer_weights ? c->w16_inf : c->w16) + c->lay.n_mlp;
  a.lvl_hash = 0;
  for (int l = 0; l < c->enc.levels; ++l) {
    const uint32_t T = c->enc.offset[l + 1] - c->enc.offset[l];
    a.lvl_T[l] = T;
    const unsigned long long r = c->enc.res[l];
    if (c->enc.grid_hash && r * r * r > T) a.lvl_hash |= 1u << l;
  }
  a.n_out = c->lay.n_out;
  a.n_out_pad = c->lay.n_out_pad;
  a.selection = c->cfg.selection;
  a.err = s->err;
  return a;
}

nmg_status fused_query(nmg_ctx* c, const nmg_shading* in, const float* u4, const int* d_count, int n_max,
                       const nmg_query_out* out, cudaStream_t st) {
  if (!fstate(c)) return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
  FusedArgs a = fused_make_args(c, true);
  a.pos = in->pos;
  a.wo = in->wo;
  a.nrm = in->normal;
  a.rough = in->roughness;
  a.u4 = u4;
  a.d_count = d_count;
  a.n_max = n_max;
  a.dir = out->dir;
  a.pdf = out->pdf;
  a.lobe = out->lobe;
  a.raw = out->raw;
  a.sel = out->selection;
  return dispatch_query(c, a, st);
}

// Guide pdf at given directions in one pass: the query kernel with its
// sampling replaced by the pdf at wi (no raw outputs go through HBM).
nmg_status fused_pdf(nmg_ctx* c, const nmg_shading* in, const float* wi, const int* d_count, int n_max, float* pdf,
                     cudaStream_t st) {
  if (!fstate(c)) return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
  FusedArgs a = fused_make_args(c, true);
  a.pos = in->pos;
  a.wo = in->wo;
  a.nrm = in->normal;
  a.rough = in->roughness;
  a.wi = wi;
  a.d_count = d_count;
  a.n_max = n_max;
  a.pdf = pdf;
  return dispatch_query(c, a, st);
}

nmg_status fused_infer_raw(nmg_ctx* c, const float* x, const int* d_count, int n_max, int which, float* raw,
                           cudaStream_t st) {
  if (!fstate(c)) return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
  FusedArgs a = fused_make_args(c, which == 1);
  a.raw_mode = 1;
  a.x = x;
  a.d_count = d_count;
  a.n_max = n_max;
  a.raw = raw;
  return dispatch_query(c, a, st);
}

// Failure-detection self-test: one thread waits, through the same bounded
// mbarrier wait every fused kernel uses (tc::mbar_wait, about 2e9 SM cycles),
// on a barrier that nothing arrives at. The wait gives up, the kernel records
// code 9 in the context's device error flag, as a fused kernel does when one
// of its waits gives up, and returns; nothing else runs in it.
constexpr int kSelftestTimeoutCode = 9;
__global__ void k_selftest_wait_timeout(int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
    if (!tc::mbar_wait(&bar, 0)) atomicExch(err, kSelftestTimeoutCode);
  }
}

nmg_status fused_selftest_wait_timeout(nmg_ctx* c, cudaStream_t st) {
  FusedState* s = fstate(c);
  if (!s)
    return set_error(NMG_ERR_UNSUPPORTED,
                     "no fused kernel state (an FP32 configuration, or nmg_reserve not called): no device error flag");
  k_selftest_wait_timeout<<<1, 32, 0, st>>>(s->err);
  return check_launch("k_selftest_wait_timeout");
}

nmg_status fused_check_errors(nmg_ctx* c) {
  FusedState* s = fstate(c);
  if (!s) return NMG_OK;
  int e = 0;
  NMG_CUDA_TRY(cudaMemcpy(&e, s->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(s->err, 0, sizeof(int));
    return set_error(NMG_ERR_TIMEOUT, "a fused kernel gave up waiting (code %d)", e);
  }
  return NMG_OK;
}


// ---------------------------------------------------------------- autotuner
// Candidate CTA shapes of the fused query kernel: 4, 5 or 6 warpgroups
// (128-query tiles) per CTA, one CTA per SM. More warpgroups hide more
// gather and MMA latency but cap registers (128, 102, 85 per thread).
static const int kTileCandidates[] = {4, 5, 6, 7, 8, 9, 10, 11, 12};
static const int kTileCandidatesK16[] = {4, 7, 8};  // 128 TMEM columns per warpgroup

static std::string tune_cache_path() {
  const char* p = getenv("NMG_TUNE_CACHE");
  if (p && *p) return p;
  const char* h = getenv("HOME");
  return std::string(h && *h ? h : "/tmp") + "/.cache/nmg_tune.txt";
}

static std::string tune_key(nmg_ctx* c, int n) {
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, c->device);
  int bucket = 0;
  while ((1 << (bucket + 1)) <= n) ++bucket;  // log2 size class
  char buf[384];  // the device name alone can take 256 bytes
  snprintf(buf, sizeof(buf), "%s|sm%d%d|preset%d|fp16=%d|n2^%d", prop.name, prop.major, prop.minor, fstate(c)->preset,
           c->cfg.path == NMG_PATH_FP16, bucket);
  for (char* q = buf; *q; ++q)
    if (*q == ' ') *q = '_';
  return buf;
}

static int tune_cache_lookup(const std::string& key) {
  FILE* f = fopen(tune_cache_path().c_str(), "r");
  if (!f) return 0;
  char k[256];
  int v = 0, found = 0;
  while (fscanf(f, "%255s %d", k, &v) == 2)
    if (key == k) found = v;
  fclose(f);
  return found;
}

static void tune_cache_store(const std::string& key, int v) {
  std::string path = tune_cache_path();
  std::string dir = path.substr(0, path.find_last_of('/'));
  if (!dir.empty()) mkdir(dir.c_str(), 0755);
  FILE* f = fopen(path.c_str(), "a");
  if (!f) return;
  fprintf(f, "%s %d\n", key.c_str(), v);
  fclose(f);
}

nmg_status fused_autotune(nmg_ctx* c, const nmg_shading* in, const float* u4, int n, const nmg_query_out* out,
                          int use_cache, int* chosen, cudaStream_t st) {
  if (!fstate(c)) return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
  const std::string key = tune_key(c, n);
  if (use_cache) {
    const int v = tune_cache_lookup(key);
    if (v > 0) {
      c->query_wg = v;
      if (chosen) *chosen = v;
      return NMG_OK;
    }
  }
  cudaEvent_t e0, e1;
  NMG_CUDA_TRY(cudaEventCreate(&e0));
  NMG_CUDA_TRY(cudaEventCreate(&e1));
  float best_ms = 1e30f;
  int best = 4;
  const bool k16 = fstate(c)->preset == 2;
  const int* cand = k16 ? kTileCandidatesK16 : kTileCandidates;
  const int ncand = k16 ? int(sizeof(kTileCandidatesK16) / sizeof(int)) : int(sizeof(kTileCandidates) / sizeof(int));
  for (int i = 0; i < ncand; ++i) {
    c->query_wg = cand[i];
    nmg_status s = fused_query(c, in, u4, nullptr, n, out, st);  // warm-up (and shared-memory setup)
    if (s == NMG_ERR_UNSUPPORTED) continue;  // e.g. its shared memory does not fit this weight image
    if (s != NMG_OK) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return s;
    }
    cudaEventRecord(e0, st);
    for (int r = 0; r < 3; ++r) fused_query(c, in, u4, nullptr, n, out, st);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return set_error(NMG_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = cand[i];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->query_wg = best;
  if (chosen) *chosen = best;
  if (use_cache) tune_cache_store(key, best);
  return fused_check_errors(c);
}

}  // namespace nmg
