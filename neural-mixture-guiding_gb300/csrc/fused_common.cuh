// fused_common.cuh -- device helpers shared by the fused query and training
// kernels: the argument block, the row encoder that writes one input row
// into a 16-bit operand tile in core-matrix order, and warpgroup barriers.
#pragma once
#include "ctx.cuh"
#include "tcgen05.cuh"

namespace nmg {

constexpr int kRows = 128;      // rows per tile (MMA M)

struct FusedArgs {
  EncodingParams enc;
  MixOpts mix;
  const uint8_t* wimg;               // packed weight image
  uint32_t w_bytes;                  // image bytes (multiple of 16)
  uint32_t layer_off[kMaxLayers];    // byte offset of each layer in the image
  int n_layers;
  int fp16;                          // grid table and encoded features FP16 instead of BF16
  uint32_t fp16_layers;              // bit l: layer l's operands (its weights and input tile) are FP16
  uint32_t w0_lo_off;                // non-zero: byte offset of a second layer-0 image (the BF16 low
                                     // parts w - bf16(w)) whose products the first layer adds
  const uint16_t* table;             // 16-bit grid table [entries][F]
  uint32_t lvl_T[kMaxLevels];        // entries per level
  uint32_t lvl_hash;                 // bit l: level l is hashed (res^3 > T, T a power of two)
  int raw_mode;                      // 1: inputs are network input rows x, output raw only
  int n_out;                         // used outputs (4K [+1])
  int n_out_pad;
  int selection;
  const float* pos;
  const float* wo;
  const float* nrm;
  const float* rough;
  const float* u4;
  const float* wi;                   // non-NULL: evaluate the pdf at wi[n][3] instead of sampling
  const float* x;
  const int* d_count;
  int n_max;
  float* dir;
  float* pdf;
  int* lobe;
  float* raw;
  float* sel;
  int* err;
};

NMG_D bool layer_fp16(const FusedArgs& a, int l) { return ((a.fp16_layers >> l) & 1u) != 0; }

// Issues the MMAs of layer l (one thread): D[tmem] = A[a_addr] * W_l^T over
// the kin input columns, both operands K-major core-matrix tiles in shared
// memory (w_addr: the weight image). With a low-part image for layer 0 the
// same A also multiplies W0's low parts into the accumulator, which carries
// W0 = hi + lo to ~16 significant bits on BF16 operands.
NMG_D void issue_layer(const FusedArgs& a, int l, uint32_t tmem, uint32_t a_addr, uint32_t w_addr, int kin, int nout) {
  const uint32_t sbo = uint32_t(kin / 8) * 128u;
  const uint32_t idesc = tc::idesc_f16(kRows, nout, layer_fp16(a, l));
  const uint32_t b_addr = w_addr + a.layer_off[l];
  for (int kk = 0; kk < kin / 16; ++kk)
    tc::mma_f16(tmem, tc::smem_desc(a_addr + kk * 256u, 128u, sbo), tc::smem_desc(b_addr + kk * 256u, 128u, sbo),
                idesc, kk > 0 ? 1u : 0u);
  if (l == 0 && a.w0_lo_off) {
    const uint32_t lo_addr = w_addr + a.w0_lo_off;
    for (int kk = 0; kk < kin / 16; ++kk)
      tc::mma_f16(tmem, tc::smem_desc(a_addr + kk * 256u, 128u, sbo), tc::smem_desc(lo_addr + kk * 256u, 128u, sbo),
                  idesc, 1u);
  }
}

NMG_D int fused_count(const int* d_count, int n_max) {
  if (!d_count) return n_max;
  int n = *d_count;
  return n < 0 ? 0 : (n > n_max ? n_max : n);
}

NMG_D bool bar_red_and(int id, int count, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred pin, pout;\n\t"
      "setp.ne.u32 pin, %1, 0;\n\t"
      "bar.red.and.pred pout, %2, %3, pin;\n\t"
      "selp.u32 %0, 1, 0, pout;\n\t}"
      : "=r"(r)
      : "r"(uint32_t(v)), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

NMG_D uint32_t level_index(const FusedArgs& a, int l, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t T = a.lvl_T[l];
  if ((a.lvl_hash >> l) & 1u) return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (T - 1u);
  const uint32_t res = a.enc.res[l];
  uint32_t idx = x + y * res + z * (res * res);
  return idx < T ? idx : (idx < 2u * T ? idx - T : idx % T);
}

template <int BINS>
NMG_D void oneblob_fixed(float x, float* o) {
  const float nb = float(BINS);
  float left = quartic_cdf(-x, nb) + quartic_cdf(-x - 1.f, nb) + quartic_cdf(-x + 1.f, nb);
#pragma unroll
  for (int k = 0; k < BINS; ++k) {
    const float rb = float(k + 1) / nb;
    float right = quartic_cdf(rb - x, nb) + quartic_cdf(rb - x - 1.f, nb) + quartic_cdf(rb - x + 1.f, nb);
    o[k] = right - left;
    left = right;
  }
}

// ReLU of 8 accumulator values packed straight into a 16-byte tile chunk.
NMG_D void store_chunk_relu(uint8_t* tile, int row, int chunk, int chunks, const float* f, bool fp16) {
  uint4 v;
  v.x = tc::pack2_relu(f[0], f[1], fp16);
  v.y = tc::pack2_relu(f[2], f[3], fp16);
  v.z = tc::pack2_relu(f[4], f[5], fp16);
  v.w = tc::pack2_relu(f[6], f[7], fp16);
  *reinterpret_cast<uint4*>(tile + tc::cm_offset(row, chunk, chunks)) = v;
}

NMG_D void store_chunk(uint8_t* tile, int row, int chunk, int chunks, const float* f, bool fp16) {
  uint4 v;
  v.x = tc::pack2(f[0], f[1], fp16);
  v.y = tc::pack2(f[2], f[3], fp16);
  v.z = tc::pack2(f[4], f[5], fp16);
  v.w = tc::pack2(f[6], f[7], fp16);
  *reinterpret_cast<uint4*>(tile + tc::cm_offset(row, chunk, chunks)) = v;
}

template <int F>
NMG_D void load_feats(const uint16_t* table, uint32_t entry, float* v, bool fp16) {
  if (F == 2) {
    uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(table) + entry);
    float2 p = tc::unpack2(w, fp16);
    v[0] = p.x;
    v[1] = p.y;
  } else {
    uint2 w = __ldg(reinterpret_cast<const uint2*>(table) + entry);
    float2 p = tc::unpack2(w.x, fp16), q = tc::unpack2(w.y, fp16);
    v[0] = p.x;
    v[1] = p.y;
    v[2] = q.x;
    v[3] = q.y;
  }
}

// Features of grid level l at position p3 (F values into out). The cell and
// weights follow grid.h:221-385; the corner indices are formed from per-axis
// terms (x, y*P1, z*P2 for hashed levels, x, y*res, z*res^2 for dense ones),
// which equal grid_index's value for every corner, and the corner weight is
// (w_x' * w_y') * w_z' as in the reference. PAIR (F = 2): the x and x+1
// corners of a (y, z) pair that share an aligned 8-byte word (every other
// cell: for dense levels e1 = e0 + 1, for hashed ones e1 = e0 ^ 1 when x is
// even) are read with one 8-byte load -- a quarter fewer L1 requests: the
// query kernels take 648 instead of 678 us (warp-specialised) and 797
// instead of 834 us (one pipeline per warpgroup), the training step 0.492
// instead of 0.499 ms.
template <int F, bool SMOOTH, bool PAIR = false>
NMG_D void grid_level(const FusedArgs& a, int l, const float (&p3)[3], float* out) {
  float w[3];
  uint32_t g[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float pp = __fadd_rn(__fmul_rn(p3[d], a.enc.scale[l]), 0.5f);
    const float fl = floorf(pp);
    g[d] = uint32_t(int(fl));
    const float f = pp - fl;
    w[d] = SMOOTH ? f * f * (3.f - 2.f * f) : f;
  }
  const float wxy[4] = {(1.f - w[0]) * (1.f - w[1]), w[0] * (1.f - w[1]), (1.f - w[0]) * w[1], w[0] * w[1]};
  const float wz[2] = {1.f - w[2], w[2]};
  const uint32_t T = a.lvl_T[l];
  const uint32_t base = a.enc.offset[l];
  uint32_t e[8];
  if ((a.lvl_hash >> l) & 1u) {
    const uint32_t mask = T - 1u;
    const uint32_t hy0 = g[1] * 2654435761u, hz0 = g[2] * 805459861u;
    const uint32_t hx[2] = {g[0], g[0] + 1u};
    const uint32_t hy[2] = {hy0, hy0 + 2654435761u};
    const uint32_t hz[2] = {hz0, hz0 + 805459861u};
#pragma unroll
    for (int c = 0; c < 8; ++c) e[c] = base + ((hx[c & 1] ^ hy[(c >> 1) & 1] ^ hz[c >> 2]) & mask);
  } else {
    const uint32_t res = a.enc.res[l], r2 = res * res;
    const uint32_t dy0 = g[1] * res, dz0 = g[2] * r2;
    const uint32_t dx[2] = {g[0], g[0] + 1u};
    const uint32_t dy[2] = {dy0, dy0 + res};
    const uint32_t dz[2] = {dz0, dz0 + r2};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      uint32_t idx = dx[c & 1] + dy[(c >> 1) & 1] + dz[c >> 2];
      if (idx >= T) idx %= T;
      e[c] = base + idx;
    }
  }
  float acc[F];
#pragma unroll
  for (int k = 0; k < F; ++k) acc[k] = 0.f;
  if constexpr (PAIR && F == 2) {
    const bool fp16 = a.fp16 != 0;
    const uint32_t* tw = reinterpret_cast<const uint32_t*>(a.table);
#pragma unroll
    for (int c = 0; c < 8; c += 2) {
      uint32_t w0, w1;
      if ((e[c] ^ e[c + 1]) == 1u) {  // entries 2m and 2m+1
        const uint2 w = __ldg(reinterpret_cast<const uint2*>(tw + (e[c] & ~1u)));
        const bool lo0 = e[c] < e[c + 1];
        w0 = lo0 ? w.x : w.y;
        w1 = lo0 ? w.y : w.x;
      } else {
        w0 = __ldg(tw + e[c]);
        w1 = __ldg(tw + e[c + 1]);
      }
      const float2 v0 = tc::unpack2(w0, fp16), v1 = tc::unpack2(w1, fp16);
      const float wt0 = wxy[c & 3] * wz[c >> 2], wt1 = wxy[(c + 1) & 3] * wz[c >> 2];
      acc[0] = fmaf(wt0, v0.x, acc[0]);  // same corner order as below
      acc[1] = fmaf(wt0, v0.y, acc[1]);
      acc[0] = fmaf(wt1, v1.x, acc[0]);
      acc[1] = fmaf(wt1, v1.y, acc[1]);
    }
  } else {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float wt = wxy[c & 3] * wz[c >> 2];
      float v[F];
      load_feats<F>(a.table, e[c], v, a.fp16 != 0);
#pragma unroll
      for (int k = 0; k < F; ++k) acc[k] = fmaf(wt, v[k], acc[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < F; ++k) out[k] = acc[k];
}

// Encodes one input row x into `tile` row `row` (KC 16-byte chunks).
// UNROLL = false keeps one copy of the chunk body (smaller code for kernels
// whose instruction footprint matters more than the loop overhead). Levels
// are gathered one at a time: computing the corners of 2 or 4 levels first
// and issuing all their table loads back to back measured slower in both
// fused kernels.
template <int F, int LEVELS, int MODE, int SHDEG, int BINS, bool SMOOTH, bool UNROLL = true, bool PAIR = false>
NMG_D void encode_row(const FusedArgs& a, const float (&x)[10], uint8_t* tile, int row) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NGRID = LEVELS * F;
  constexpr int NPAD = (NGRID + NDIR + 15) / 16 * 16;
  constexpr int KC = NPAD / 8;
  constexpr int LPC = 8 / F;
  static_assert(NGRID % 8 == 0, "grid features must fill whole chunks");
  const bool fp16 = layer_fp16(a, 0);  // the tile's format is layer 0's operand format, not the table's
  const float p3[3] = {x[0], x[1], x[2]};
#pragma unroll(UNROLL ? NGRID / 8 : 1)
  for (int ch = 0; ch < NGRID / 8; ++ch) {
    float f[8];
#pragma unroll
    for (int j = 0; j < LPC; ++j) grid_level<F, SMOOTH, PAIR>(a, ch * LPC + j, p3, f + j * F);
    store_chunk(tile, row, ch, KC, f, fp16);
  }
  float d[NPAD - NGRID];
  sh_basis(SHDEG, x[3] * 2.f - 1.f, x[4] * 2.f - 1.f, x[5] * 2.f - 1.f, d);
  if (MODE == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) oneblob_fixed<BINS>(x[6 + k], d + SHDEG * SHDEG + k * BINS);
  } else {
    sh_basis(SHDEG, x[6] * 2.f - 1.f, x[7] * 2.f - 1.f, x[8] * 2.f - 1.f, d + SHDEG * SHDEG);
    oneblob_fixed<BINS>(x[9], d + 2 * SHDEG * SHDEG);
  }
#pragma unroll
  for (int k = NDIR; k < NPAD - NGRID; ++k) d[k] = 1.f;
#pragma unroll
  for (int ch = 0; ch < (NPAD - NGRID) / 8; ++ch) store_chunk(tile, row, NGRID / 8 + ch, KC, d + 8 * ch, fp16);
}

// encode_row for one of the two threads that share a row: half h writes the
// grid chunks ch with ch % 2 == h (each chunk 8 / F consecutive levels, so
// both halves get coarse and fine levels) and its share of the direction
// chunks: for input mode 1 half 0 the SH(wo) chunks and half 1 the rest
// (SH(normal), one-blob(roughness), padding), each computing only what it
// stores; for mode 0, whose encodings share chunks, both compute the whole
// direction part and split its chunks. Together the two calls write exactly
// what encode_row writes.
template <int F, int LEVELS, int MODE, int SHDEG, int BINS, bool SMOOTH, bool PAIR = false>
NMG_D void encode_row_half(const FusedArgs& a, const float (&x)[10], uint8_t* tile, int row, int h) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NGRID = LEVELS * F;
  constexpr int NPAD = (NGRID + NDIR + 15) / 16 * 16;
  constexpr int KC = NPAD / 8;
  constexpr int LPC = 8 / F;
  constexpr int GCH = NGRID / 8, DCH = (NPAD - NGRID) / 8;
  constexpr bool SPLIT_SH = MODE == 1 && (SHDEG * SHDEG) % 8 == 0;
  constexpr int DCH0 = SPLIT_SH ? SHDEG * SHDEG / 8 : (DCH + 1) / 2;  // direction chunks of half 0
  static_assert(NGRID % 16 == 0, "grid chunks split evenly over the two halves");
  const bool fp16 = layer_fp16(a, 0);
  const float p3[3] = {x[0], x[1], x[2]};
#pragma unroll 1
  for (int ch = h; ch < GCH; ch += 2) {
    float f[8];
#pragma unroll
    for (int j = 0; j < LPC; ++j) grid_level<F, SMOOTH, PAIR>(a, ch * LPC + j, p3, f + j * F);
    store_chunk(tile, row, ch, KC, f, fp16);
  }
  float d[NPAD - NGRID];
#pragma unroll
  for (int k = 0; k < NPAD - NGRID; ++k) d[k] = 1.f;
  if (MODE == 0) {
    sh_basis(SHDEG, x[3] * 2.f - 1.f, x[4] * 2.f - 1.f, x[5] * 2.f - 1.f, d);
#pragma unroll
    for (int k = 0; k < 3; ++k) oneblob_fixed<BINS>(x[6 + k], d + SHDEG * SHDEG + k * BINS);
  } else if (!SPLIT_SH || h == 0) {
    sh_basis(SHDEG, x[3] * 2.f - 1.f, x[4] * 2.f - 1.f, x[5] * 2.f - 1.f, d);
  }
  if (MODE == 1 && (!SPLIT_SH || h == 1)) {
    sh_basis(SHDEG, x[6] * 2.f - 1.f, x[7] * 2.f - 1.f, x[8] * 2.f - 1.f, d + SHDEG * SHDEG);
    oneblob_fixed<BINS>(x[9], d + 2 * SHDEG * SHDEG);
  }
#pragma unroll
  for (int ch = 0; ch < DCH; ++ch)
    if ((ch < DCH0) == (h == 0)) store_chunk(tile, row, GCH + ch, KC, d + 8 * ch, fp16);
}

// Loads network input row q (n_input <= 10 floats) with compile-time indices.
NMG_D void load_row(const float* x, long q, int n_input, float (&v)[10]) {
#pragma unroll
  for (int d = 0; d < 10; ++d) v[d] = d < n_input ? x[q * n_input + d] : 0.f;
}

NMG_D f3 face_fwd(f3 n, f3 v) { return dot3(n, v) > 0.f ? n : f3{-n.x, -n.y, -n.z}; }

// Output stage of one query from its raw network outputs r (registers):
// optional raw row, then (unless raw_mode) the mixture with the optional
// cosine lobe, and either the sampled direction with its pdf, lobe and
// selection probability, or (a.wi set) the pdf at the given direction.
// (The direction is stored per thread here: gathering a warp's directions
// into whole-sector float4 stores, as the 16-lobe epilogues do, kept three
// more values live across the pdf and made the 8-lobe consumers spill:
// query pass 0.647 -> 0.751 ms.)
template <int K, int NOUTMAX>
NMG_D void query_epilogue(const FusedArgs& a, long q, const float (&r)[NOUTMAX]) {
  if (a.raw) {
    float4* dst = reinterpret_cast<float4*>(a.raw + q * a.n_out_pad);
#pragma unroll
    for (int c = 0; c < NOUTMAX / 4; ++c)
      if (c * 4 < a.n_out_pad) dst[c] = make_float4(r[4 * c], r[4 * c + 1], r[4 * c + 2], r[4 * c + 3]);
  }
  if (a.raw_mode) return;
  Mix<K> m;
  mix_activate_regs<K, true>(m, r, a.mix.kappa_softplus);
  if (a.mix.cosine) mix_apply_cosine<K, true>(m, face_fwd(load3(a.nrm, q), load3(a.wo, q)));
  if (a.wi) {
    a.pdf[q] = mix_pdf<K, true>(m, load3(a.wi, q));
    return;
  }
  const float4 u = reinterpret_cast<const float4*>(a.u4)[q];
  const int sel = mix_select<K>(m, u.y);
  const f3 dv = mix_sample_lobe<K, true>(m, sel, u.z, u.w);
  store3(a.dir, q, dv);
  a.pdf[q] = mix_pdf<K, true>(m, dv);
  if (a.lobe) a.lobe[q] = sel;
  if (a.sel && a.selection) a.sel[q] = logistic<true>(r[4 * K < NOUTMAX ? 4 * K : 0]);
}

// query_epilogue for wide mixtures (K = 16) with the raw outputs left in
// TMEM: holding all K lobes (7 K floats) next to the 4 K raw outputs does not
// fit the registers of a 128-query warpgroup, so this variant keeps only the
// K lobe weights and derives each lobe again from its 4 raw outputs
// (tcgen05.ld of 16 columns = 4 lobes) when it is needed: once for the
// weights, once for the sampled lobe, once for the pdf. The lobe arithmetic
// is that of query_epilogue (same helpers, same order), so the results are
// the same. Warp-collective: every thread of the warpgroup calls it with its
// TMEM row address; rows past n (valid = false) compute and store nothing.
template <int K>
NMG_D void query_epilogue_streamed(const FusedArgs& a, long q, bool valid, uint32_t lane_addr) {
  static_assert(K % 4 == 0, "lobes come in groups of four (16 TMEM columns)");
  constexpr int G = K / 4;
  const bool cosine = a.mix.cosine != 0;
  f3 mb{0.f, 0.f, 1.f};
  if (cosine && valid) mb = unit3<true>(face_fwd(load3(a.nrm, q), load3(a.wo, q)));
  const float nb = prod_norm<true>(kCosineKappa);
  // lobe i of the 16-column group in v, as query_epilogue's activation (+ cosine product) makes it
  auto lobe = [&](const float (&v)[16], int j, float& lam, float& kap, f3& mu, float& nrm) {
    lobe_activate<true>(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3], a.mix.kappa_softplus, lam, kap, mu);
    nrm = vmf_norm<true>(kap);
    if (cosine) lobe_cosine<true>(mb, nb, lam, kap, mu, nrm);
  };
  // pass 1: weights
  float lw[K];
  float total = 0.f;
#pragma unroll
  for (int g = 0; g < G; ++g) {
    float v[16];
    tc::tmem_load<1>(lane_addr + 16 * g, v);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float lam, kap, nrm;
      f3 mu;
      lobe(v, j, lam, kap, mu, nrm);
      lw[4 * g + j] = lam;
      total += lam;
    }
  }
  if (cosine) total = fmaxf(total, NMG_EPS);  // distribution.h:191
  const float inv = 1.f / total;
#pragma unroll
  for (int i = 0; i < K; ++i) lw[i] *= inv;
  f3 d;
  int sel = 0;
  if (a.wi) {
    d = valid ? load3(a.wi, q) : f3{0.f, 0.f, 1.f};
  } else {
    // selection (distribution.h:132-140) and pass 2: the selected lobe, sampled
    const float4 u = valid ? reinterpret_cast<const float4*>(a.u4)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    float uu = u.y;
    sel = -1;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      if (sel < 0) {
        if (uu < lw[i])
          sel = i;
        else
          uu -= lw[i];
      }
    }
    sel = sel < 0 ? 0 : sel;
    // the selected lobe's four raw outputs, picked from each group as it is read (the reads are
    // warp-collective, the lobe is each thread's own), then that one lobe derived
    float rs[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) rs[k] = 0.f;
#pragma unroll
    for (int g = 0; g < G; ++g) {
      float v[16];
      tc::tmem_load<1>(lane_addr + 16 * g, v);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool pick = 4 * g + j == sel;
#pragma unroll
        for (int k = 0; k < 4; ++k) rs[k] = pick ? v[4 * j + k] : rs[k];
      }
    }
    float lam, ks, nrm;
    f3 ms;
    lobe(rs, 0, lam, ks, ms, nrm);
    d = vmf_sample_dir<true>(ks, ms, u.z, u.w);
  }
  // pass 3: pdf at d (distribution.h:113-119)
  float p = 0.f;
#pragma unroll
  for (int g = 0; g < G; ++g) {
    float v[16];
    tc::tmem_load<1>(lane_addr + 16 * g, v);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float lam, kap, nrm;
      f3 mu;
      lobe(v, j, lam, kap, mu, nrm);
      const float c = dot3(d, mu);
      const float vv = kap < NMG_EPS ? NMG_INV_4PI : __expf(kap * fminf(0.f, c - 1.f)) * nrm;
      p += lw[4 * g + j] * vv;
    }
  }
  float slogit = 0.f;
  if (a.sel && a.selection) {  // the selection logit follows the lobes (column 4K)
    float v[16];
    tc::tmem_load<1>(lane_addr + 4 * K, v);
    slogit = v[0];
  }
  if (a.wi) {
    if (valid) a.pdf[q] = p;
    return;
  }
  store3_warp(a.dir, q, d, valid);
  if (!valid) return;
  a.pdf[q] = p;
  if (a.lobe) a.lobe[q] = sel;
  if (a.sel && a.selection) a.sel[q] = logistic<true>(slogit);
}

// ------------------------------------------------------------ weight image
// Image 0 holds the training weights, image 1 the inference weights; each
// layer l of image i is converted to FP16 when bit l of fp16_layers[i] is
// set, else to BF16, and image i carries W0's BF16 low parts at w0_lo_off[i]
// when that is non-zero.
struct PackArgs {
  long off[kMaxLayers + 1];
  int in[kMaxLayers];
  uint32_t layer_off[kMaxLayers];
  int n_layers;
  uint32_t fp16_layers[2];
  uint32_t w0_lo_off[2];
};

struct FusedState {
  uint8_t* img_train;
  uint8_t* img_infer;
  int* err;
  uint32_t w_bytes;      // training image
  uint32_t w_bytes_inf;  // inference image
  PackArgs pack;
  int preset;  // 0 none, 1 hash-grid K8, 2 hash-grid K16, 3 reference K8
};

inline FusedState* fstate(nmg_ctx* c) { return reinterpret_cast<FusedState*>(c->ws.fused); }

FusedArgs fused_make_args(nmg_ctx* c, bool infer_weights);

// Query tilings >= 8 select a configuration of the warp-specialised kernel
// (fused_ws.cu): 8 = 4 encoder + 2 consumer warpgroups, 4 ring slots;
// 9 = 5 + 1, 5 slots; 10 = 6 + 2, 6 slots; 11 = 4 + 2, 8 slots;
// 12 = 4 + 2, 4 slots, hidden activations kept in the slot.
constexpr int kTilingWarpSpecialised = 8;
constexpr int kTilingPair = 7;  // two pipelines of two warpgroups, two threads per query (queries without raw outputs)
constexpr int kTilingLast = 12;
nmg_status launch_query_ws(int preset, int tiling, const FusedArgs& a, cudaStream_t st);

}  // namespace nmg
