// fused_train.cu -- the fused reduced-precision training step on tcgen05.
//
// One persistent CTA per SM: two pipelines (one for the K = 16 configuration)
// walking tiles of 128 training records, plus one MMA issuer warp. A pipeline
// is two warpgroups, so every record has two threads: warps w and w + 4 read
// the same TMEM lane quadrant, and each half of a row's pair takes half of
// every phase -- half the grid levels of the encoding, half the columns of
// each epilogue, half the mixture lobes of the loss (the two partial sums the
// loss needs cross through shared memory). All tensor-core work of the CTA is
// issued by one thread of the issuer warp, in each pipeline's order, so the
// shared weight-gradient accumulators see their MMAs in sequence; a pipeline
// signals "operands ready" on an mbarrier and waits on its "done" mbarrier
// (tcgen05.commit). For each tile, entirely on chip:
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
// TMEM (512 columns): one forward/data-gradient accumulator per pipeline
// (M = 128; 64 columns, 128 when the output layer is wider), then the shared
// weight-gradient accumulators dW0 | dW1 | dW2 | dW3^T (M = 64: rows live in
// lanes 0-15 of each 32-lane subpartition). The layer-0 data gradient is
// computed for the grid columns only, the only ones with parameters below.
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
#include "records.cuh"

namespace nmg {

constexpr uint32_t kTrainCols = 512;

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
  // Records mode (the kernel's REC instantiation): row q of the batch is the
  // path vertex vid[id_base + q] of the frame's radiance records rr (vertex
  // id = depth * pixels + pixel); the load stage computes its network input
  // and GuidedOutput (vertex_record) instead of reading x and rec.
  const uint32_t* vid;
  long id_base;
  uint32_t pixels;
  nmg_radiance_records rr;
};

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

// Number of tiles warpgroup g of this CTA processes (the same expression in
// the compute warpgroups and in the MMA issuer).
NMG_D int wg_tiles(int ntiles, int g, int nwg) {
  const int first = blockIdx.x * nwg + g, stride = gridDim.x * nwg;
  return first < ntiles ? (ntiles - 1 - first) / stride + 1 : 0;
}

// Signals the issuer that pipeline g's operands for its next MMA batch are in
// shared memory (and that its last TMEM reads are done): every thread makes
// its writes visible to the tensor core, the pipeline's two warpgroups
// synchronise (and agree on `ok`), and one thread arrives on the ready
// barrier.
NMG_D bool signal_ready(int g, bool leader, uint64_t* ready, bool ok) {
  tc::fence_proxy_async();
  tc::fence_before_sync();
  ok = bar_red_and(1 + g, 2 * kRows, ok);
  if (ok && leader) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(ready)) : "memory");
  return ok;
}

// Adds one record's grid-feature gradient df[F] of level lv into the table
// gradient gt with the corner weights of position p3 (grid.h:387-510).
template <int F, bool SMOOTH>
NMG_D void scatter_level(const FusedArgs& a, float* gt, int lv, const float (&p3)[3], const float (&df)[F]) {
  float w[3];
  uint32_t gc[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) pos_fract(p3[d], a.enc.scale[lv], SMOOTH ? 1 : 0, &w[d], &gc[d]);
  const float wxy[4] = {(1.f - w[0]) * (1.f - w[1]), w[0] * (1.f - w[1]), (1.f - w[0]) * w[1], w[0] * w[1]};
  const float wz[2] = {1.f - w[2], w[2]};
  if constexpr (F == 2) {
    // Corners x and x+1 of a (y, z) pair often land on adjacent entries (always for dense
    // levels, for even x on hashed ones: the x term of the hash is x itself); one 16-byte
    // vector reduction then updates both, halving those atomics' L2 requests.
#pragma unroll
    for (int c = 0; c < 8; c += 2) {
      const uint32_t yy = gc[1] + ((c >> 1) & 1), zz = gc[2] + (c >> 2);
      const uint32_t e0 = a.enc.offset[lv] + level_index(a, lv, gc[0], yy, zz);
      const uint32_t e1 = a.enc.offset[lv] + level_index(a, lv, gc[0] + 1u, yy, zz);
      const float wt0 = wxy[c & 3] * wz[c >> 2], wt1 = wxy[(c + 1) & 3] * wz[c >> 2];
      const float2 g0 = make_float2(wt0 * df[0], wt0 * df[1]), g1 = make_float2(wt1 * df[0], wt1 * df[1]);
      if ((e0 ^ e1) == 1u) {  // entries 2m and 2m+1: one aligned 16-byte pair
        const bool lo0 = e0 < e1;
        atomicAdd(reinterpret_cast<float4*>(gt + size_t(lo0 ? e0 : e1) * 2),
                  lo0 ? make_float4(g0.x, g0.y, g1.x, g1.y) : make_float4(g1.x, g1.y, g0.x, g0.y));
      } else {
        atomicAdd(reinterpret_cast<float2*>(gt + size_t(e0) * 2), g0);
        atomicAdd(reinterpret_cast<float2*>(gt + size_t(e1) * 2), g1);
      }
    }
  } else {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float wt = wxy[c & 3] * wz[c >> 2];
      const uint32_t e = a.enc.offset[lv] +
                         level_index(a, lv, gc[0] + (c & 1), gc[1] + ((c >> 1) & 1), gc[2] + ((c >> 2) & 1));
#pragma unroll
      for (int k = 0; k < F; k += 2)
        atomicAdd(reinterpret_cast<float2*>(gt + size_t(e) * F + k), make_float2(wt * df[k], wt * df[k + 1]));
    }
  }
}

// Scatter warps (SCAT): the CTA adds 7 warps (with the issuer warp they form
// two more warpgroups) that apply each tile's grid gradient to the table
// while the pipelines move on to their next tile. A pipeline stages its
// layer-0 data gradient in its third hidden tile (dead by then, rewritten
// only at the next tile's third forward layer) and arrives on sfull; the
// scatter warps arrive on sempty when they have read it.
// Registers: the 768-thread block launches at 80 per thread and moves 32 of
// them from each issuer/scatter thread to the compute threads.
constexpr int kScatThreadsPerCta = 6 * kRows;
constexpr int kScatRegLaunch = 80, kScatRegCompute = 96, kScatRegScatter = 48;
static_assert(4 * kRows * kScatRegCompute + 2 * kRows * kScatRegScatter == kScatThreadsPerCta * kScatRegLaunch,
              "register split must equal the launch allocation");

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH, int NWG, bool SCAT,
          bool REC>
__global__ void __launch_bounds__(SCAT ? kScatThreadsPerCta : 2 * NWG * kRows + 32, 1)
    k_fused_train(const __grid_constant__ TrainArgs ta) {
  static_assert(!SCAT || NWG == 2, "scatter warps pair with two pipelines");
  static_assert(K % 8 == 0, "each half of a row holds K / 2 lobes, a whole number of 16-column groups");
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  constexpr int NGRID = LEVELS * F;
  constexpr int DMAX = NOUTMAX > kWidth ? NOUTMAX : kWidth;
  constexpr uint32_t A_BYTES = kRows * NENC * 2;
  constexpr uint32_t H_BYTES = kRows * kWidth * 2;
  constexpr uint32_t D_BYTES = kRows * DMAX * 2;
  // per pipeline, after its operand tiles: each row's GuidedOutput (records
  // mode REC: computed at the load stage, read at the loss stage), by tile
  // parity each row's normalised position for the scatter warps, and the
  // loss's partial sums of both halves of each row
  constexpr uint32_t REC_BYTES = REC ? kRows * 8 * 4 : 0, P3_BYTES = SCAT ? 2 * kRows * 4 * 4 : 0;
  constexpr uint32_t XCH_BYTES = 2 * kRows * 2 * 4;
  constexpr uint32_t WG_BYTES = A_BYTES + 3 * H_BYTES + D_BYTES + REC_BYTES + P3_BYTES + XCH_BYTES;
  constexpr int NL = 4;  // three hidden layers
  // TMEM: one forward/data-gradient accumulator per pipeline, then the shared
  // weight-gradient accumulators (M = 64) dW0 | dW1 | dW2 | dW3^T.
  // (the accumulator holds a hidden layer's 64 columns or the output layer's
  // NOUTMAX: 80 for 16 lobes, so that two pipelines and the weight gradients
  // fit the 512 columns)
  constexpr uint32_t DCOLS = NOUTMAX <= kWidth ? kWidth : (NOUTMAX + 15) / 16 * 16;
  constexpr uint32_t CW0 = NWG * DCOLS, CW1 = CW0 + NENC, CW2 = CW1 + kWidth, CW3 = CW2 + kWidth;
  static_assert(CW3 + NOUTMAX <= kTrainCols, "TMEM holds 512 columns");
  static_assert(NGRID <= 64 && NGRID % 16 == 0, "grid features are read in 16-column groups");
  extern __shared__ __align__(1024) uint8_t smem[];
  const FusedArgs& a = ta.f;

  const uint32_t w_region = (a.w_bytes + 1023u) & ~1023u;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const bool issuer = warp == NWG * 8;
  const bool scatter = SCAT && warp > NWG * 8;
  const int g = (issuer || scatter) ? 0 : warp / 8;  // pipeline
  const int h = (warp / 4) & 1;                     // half of the row's pair
  const int t = threadIdx.x % kRows;                // row of the tile
  uint8_t* wsm = smem;
  uint8_t* A0 = smem + w_region + g * WG_BYTES;
  uint8_t* Hs = A0 + A_BYTES;  // three hidden tiles
  uint8_t* Dt = Hs + 3 * H_BYTES;
  float* s_rec = reinterpret_cast<float*>(Dt + D_BYTES);             // [kRows][8]
  float* s_p3 = reinterpret_cast<float*>(Dt + D_BYTES + REC_BYTES);  // [2][kRows][4]
  float2* s_xch = reinterpret_cast<float2*>(Dt + D_BYTES + REC_BYTES + P3_BYTES);  // [2 halves][kRows]
  // [0] weights, then ready[], done[], sfull[], sempty[]
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + w_region + NWG * WG_BYTES);
  uint64_t* ready = bars + 1;
  uint64_t* done = bars + 1 + NWG;
  uint64_t* sfull = bars + 1 + 2 * NWG;
  uint64_t* sempty = bars + 1 + 3 * NWG;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1 + 4 * NWG);
  constexpr int kScatThreads = SCAT ? 2 * kRows - 32 : 0;  // 7 warps after the issuer warp
  const bool fp16 = a.fp16 != 0;
  const int nout = a.n_out_pad;
  const int KC3 = nout / 8;

  if (threadIdx.x == 0) {
    tc::mbar_init(&bars[0], 1);
    for (int i = 0; i < NWG; ++i) {
      tc::mbar_init(&ready[i], 1);
      tc::mbar_init(&done[i], 1);
      tc::mbar_init(&sfull[i], 1);
      tc::mbar_init(&sempty[i], SCAT ? kScatThreads : 1);
    }
    tc::fence_mbar_init();
  }
  if (issuer) tc::tmem_alloc(tslot, kTrainCols);
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

  const uint32_t tbase = *tslot;
  const int n = fused_count(a.d_count, a.n_max);
  const int ntiles = (n + kRows - 1) / kRows;
  const float scale = n > 0 ? ta.loss_scale / float(n) : 0.f;          // reference gradient scale
  const float S = fp16 ? fminf(float(n), 256.f) : float(n > 0 ? n : 1);  // operand range factor
  const float inv_S = 1.f / S;
  const uint32_t w_addr = tc::smem_u32(wsm);
  double loss_acc = 0.0;
  int cta_tiles = 0;
  for (int i = 0; i < NWG; ++i) cta_tiles += wg_tiles(ntiles, i, NWG);
  if (issuer) {
    if constexpr (SCAT) tc::reg_dealloc<kScatRegScatter>();
    // ---------------------------------------------------- MMA issuer (one thread)
    if (lane == 0 && ok) {
      int remaining[NWG], step[NWG];
      uint32_t rph[NWG];
      uint32_t started = 0;  // bit l: layer l's weight-gradient accumulator holds a sum
      bool any = false;
      for (int i = 0; i < NWG; ++i) {
        remaining[i] = 8 * wg_tiles(ntiles, i, NWG);
        step[i] = 0;
        rph[i] = 0;
        any |= remaining[i] > 0;
      }
      long long last = clock64();
      while (any) {
        any = false;
        for (int i = 0; i < NWG; ++i) {
          if (remaining[i] <= 0) continue;
          any = true;
          if (!tc::mbar_test(&ready[i], rph[i])) continue;
          rph[i] ^= 1u;
          last = clock64();
          tc::fence_after_sync();
          uint8_t* gA0 = smem + w_region + i * WG_BYTES;
          uint8_t* gH = gA0 + A_BYTES;
          uint8_t* gD = gH + 3 * H_BYTES;
          const uint32_t tD = tbase + i * DCOLS;
          const int s = step[i];
          if (s < NL) {  // forward layer s
            const int kin = s == 0 ? NENC : kWidth;
            const uint32_t a_addr = tc::smem_u32(s == 0 ? gA0 : gH + (s - 1) * H_BYTES);
            issue_mma_kmajor(tD, a_addr, kin / 8, w_addr + a.layer_off[s], 128u, uint32_t(kin / 8) * 128u, 256u,
                             s == NL - 1 ? nout : kWidth, kin / 16, fp16, false);
          } else {  // backward layer l: weight gradient then data gradient
            const int l = NL - 1 - (s - NL);
            const int dchunks = l == NL - 1 ? KC3 : kWidth / 8;
            const int dwidth = l == NL - 1 ? nout : kWidth;
            const int in_w = l == 0 ? NENC : kWidth;
            const uint8_t* hin = l == 0 ? gA0 : gH + (l - 1) * H_BYTES;
            const bool acc = (started >> l) & 1u;
            if (l == NL - 1)
              issue_wgrad(tbase + CW3, tc::smem_u32(hin), kWidth / 8, tc::smem_u32(gD), dchunks, dwidth, fp16, acc);
            else
              issue_wgrad(tbase + (l == 0 ? CW0 : (l == 1 ? CW1 : CW2)), tc::smem_u32(gD), dchunks, tc::smem_u32(hin),
                          in_w / 8, in_w, fp16, acc);
            started |= 1u << l;
            // data gradient delta_l W_l (W_l's image as an MN-major operand); for l = 0 only the grid columns
            const uint32_t wk = uint32_t(in_w / 8) * 128u;
            issue_mma_kmajor(tD, tc::smem_u32(gD), dchunks, w_addr + a.layer_off[l], wk, 128u, 2u * wk,
                             l == 0 ? NGRID : in_w, dwidth / 16, fp16, true);
          }
          tc::mma_commit(&done[i]);
          step[i] = (s + 1) % (2 * NL);
          --remaining[i];
        }
        if (any && clock64() - last > 4000000000LL) {  // no warpgroup signalled for ~2 s
          atomicExch(a.err, 4);
          break;
        }
      }
    }
    __syncwarp();
    if constexpr (SCAT) tc::reg_alloc<kScatRegLaunch>();
  } else if (scatter) {
    // ------------------------------------------------------- scatter warps
    tc::reg_dealloc<kScatRegScatter>();
    // Tiles in the order the compute groups finish them (k-th tile of group
    // 0, then of group 1, ...); items (level, row) with rows fastest, so a
    // warp reads consecutive rows of the staged [feature][row] gradient.
    const int sidx = int(threadIdx.x) - (NWG * 8 + 1) * 32;
    float* gt = ta.grad + ta.n_mlp;
    for (int k = 0; ok; ++k) {
      bool any = false;
      for (int gg = 0; gg < NWG && ok; ++gg) {
        const int tile = blockIdx.x * NWG + gg + k * gridDim.x * NWG;
        if (tile >= ntiles) continue;
        any = true;
        if (!tc::mbar_wait(&sfull[gg], uint32_t(k) & 1u)) {
          ok = false;
          break;
        }
        const uint8_t* gbase = smem + w_region + gg * WG_BYTES;
        const float* dgs = reinterpret_cast<const float*>(gbase + A_BYTES + 2 * H_BYTES);
        const float* gp3 = reinterpret_cast<const float*>(gbase + A_BYTES + 3 * H_BYTES + D_BYTES + REC_BYTES) +
                           (k & 1) * kRows * 4;
        for (int item = sidx; item < kRows * LEVELS; item += kScatThreads) {
          const int r = item % kRows, lv = item / kRows;
          const long q = long(tile) * kRows + r;
          if (q < n) {
            const float p3[3] = {gp3[4 * r], gp3[4 * r + 1], gp3[4 * r + 2]};
            float df[F];
#pragma unroll
            for (int kk = 0; kk < F; ++kk) df[kk] = dgs[(F * lv + kk) * kRows + r];
            scatter_level<F, SMOOTH>(a, gt, lv, p3, df);
          }
        }
        tc::mbar_arrive(&sempty[gg]);
      }
      if (!any) break;
    }
    tc::reg_alloc<kScatRegLaunch>();
  } else {
    // ---------------------------------------- pipeline g, half h of every row
    if constexpr (SCAT) tc::reg_alloc<kScatRegCompute>();
    constexpr int KH = K / 2;          // lobes of each half: raw columns [2K h, 2K h + 2K)
    constexpr int HC = kWidth / 16;    // 8-column chunks of a hidden row per half
    constexpr int GCH = NGRID / 8;     // 8-column grid chunks; half h owns those with ch % 2 == h
    constexpr int LPC = 8 / F;         // levels per grid chunk
    uint32_t dph = 0;
    const bool leader = h == 0 && t == 0;
    const bool sel_on = a.selection != 0;
    const uint32_t tD = tbase + g * DCOLS;
    const uint32_t lane_addr = (uint32_t((warp & 3) * 32) << 16);
    for (int tile = blockIdx.x * NWG + g; tile < ntiles; tile += gridDim.x * NWG) {
      const int kt = (tile - (blockIdx.x * NWG + g)) / (gridDim.x * NWG);  // this pipeline's tile number
      const long q = long(tile) * kRows + t;
      const bool valid = q < n;
      float x[10];
#pragma unroll
      for (int d = 0; d < 10; ++d) x[d] = 0.f;
      if (valid) {
        if constexpr (REC) {
          // records mode: the vertex's network input and GuidedOutput from the radiance records
          // (both halves compute the input; half 0 keeps the GuidedOutput for the loss stage)
          const uint32_t v = ta.vid[ta.id_base + q];
          const uint32_t dd = v / ta.pixels;
          float out[7];
          vertex_record(ta.rr.depth[dd], ta.rr.product, a.enc, v - dd * ta.pixels, x, out);
          if (h == 0) {
#pragma unroll
            for (int j = 0; j < 7; ++j) s_rec[t * 8 + j] = out[j];
          }
        } else {
          load_row(ta.x, q, a.enc.n_input, x);
        }
      }
      if constexpr (SCAT) {  // the scatter warps read this tile's positions from here (buffer kt & 1)
        if (h == 0) {
          float* p3 = s_p3 + (kt & 1) * kRows * 4 + t * 4;
          p3[0] = x[0];
          p3[1] = x[1];
          p3[2] = x[2];
        }
      }
      encode_row_half<F, LEVELS, MODE, SHDEG, BINS, SMOOTH, true>(a, x, A0, t, h);
      ok = signal_ready(g, leader, &ready[g], ok);
      if (!ok) break;

      // ---------------------------------------------------------- forward
      float rh[2 * K];  // this half's lobes' raw outputs
      float sel_logit = 0.f;
      for (int l = 0; l < NL; ++l) {
        const bool fin = tc::mbar_wait(&done[g], dph);
        dph ^= 1u;
        tc::fence_after_sync();
        if (l < NL - 1) {
          float v[kWidth / 2];
          tc::tmem_load<kWidth / 32>(tD + lane_addr + uint32_t(h * (kWidth / 2)), v);
          uint8_t* H = Hs + l * H_BYTES;
          bool free_h = true;
          if (SCAT && l == 2 && kt > 0)  // the scatter warps still read the previous tile's gradient here
            free_h = tc::mbar_wait(&sempty[g], uint32_t(kt - 1) & 1u);
#pragma unroll
          for (int c = 0; c < HC; ++c) store_chunk_relu(H, t, h * HC + c, kWidth / 8, v + 8 * c, fp16);
          ok = signal_ready(g, leader, &ready[g], fin && free_h && ok);
          if (!ok) break;
        } else {
          tc::tmem_load<K / 8>(tD + lane_addr + uint32_t(h * 2 * K), rh);
          if (sel_on) {
            float v[16];
            tc::tmem_load<1>(tD + lane_addr + uint32_t(4 * K), v);
            sel_logit = v[0];
          }
          ok = fin && ok;
        }
      }
      if (!ok) {
        ok = bar_red_and(1 + g, 2 * kRows, false);
        break;
      }

      // ------------------------------------------------- loss and adjoint
      // each half takes its KH lobes; the lobe-weight total and the weighted
      // vMF sum of the other half come through shared memory
      {
        float rr[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) rr[j] = 0.f;
        if (valid) {
          if constexpr (REC) {
#pragma unroll
            for (int j = 0; j < 7; ++j) rr[j] = s_rec[t * 8 + j];
          } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) rr[j] = j < ta.rstride ? ta.rec[q * ta.rstride + j] : 0.f;
          }
        }
        HalfLoss<KH> hl;
        half_loss_lobes<KH, true>(hl, rh, rr, a.mix);
        const float2 mine = valid ? make_float2(hl.lt, hl.nt) : make_float2(0.f, 0.f);
        s_xch[h * kRows + t] = mine;
        ok = bar_red_and(1 + g, 2 * kRows, ok);  // a bar.red, like every other barrier of the pipeline
        if (!ok) break;
        const float2 other = s_xch[(1 - h) * kRows + t];
        float gh[4 * KH];
        float gsel = 0.f;
        const float l = sel_on ? half_loss_grad<KH, true, true>(hl, mine.x + other.x, mine.y + other.y, sel_logit, rr,
                                                                scale, a.mix, gh, &gsel)
                               : half_loss_grad<KH, true, false>(hl, mine.x + other.x, mine.y + other.y, 0.f, rr,
                                                                 scale, a.mix, gh, &gsel);
        if (valid && h == 0) loss_acc += double(l);
        // delta columns: half 0 its lobes' [0, 2K); half 1 its lobes' [2K, 4K),
        // the selection logit's gradient (column 4K) and zero padding to nout
        if (h == 0) {
#pragma unroll
          for (int c = 0; c < K / 4; ++c) {
            float fv[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) fv[i] = valid ? gh[8 * c + i] * S : 0.f;
            store_chunk(Dt, t, c, KC3, fv, fp16);
          }
        } else {
#pragma unroll
          for (int c = K / 4; c < NOUTMAX / 8; ++c) {
            if (c * 8 < nout) {
              float fv[8];
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                const int col = 8 * c + i;
                const float gv = col < 4 * K ? gh[col < 4 * K ? col - 2 * K : 0] : (col == 4 * K ? gsel : 0.f);
                fv[i] = valid ? gv * S : 0.f;
              }
              store_chunk(Dt, t, c, KC3, fv, fp16);
            }
          }
        }
      }
      ok = signal_ready(g, leader, &ready[g], ok);
      if (!ok) break;

      // ---------------------------------------------------------- backward
      for (int l = NL - 1; l >= 1; --l) {
        const bool fin = tc::mbar_wait(&done[g], dph);
        dph ^= 1u;
        tc::fence_after_sync();
        float v[kWidth / 2];
        tc::tmem_load<kWidth / 32>(tD + lane_addr + uint32_t(h * (kWidth / 2)), v);
        const uint8_t* H = Hs + (l - 1) * H_BYTES;
#pragma unroll
        for (int c = 0; c < HC; ++c) {
          float hv[8], fv[8];
          load_chunk(H, t, h * HC + c, kWidth / 8, hv, fp16);
#pragma unroll
          for (int i = 0; i < 8; ++i) fv[i] = hv[i] > 0.f ? v[8 * c + i] : 0.f;
          store_chunk(Dt, t, h * HC + c, kWidth / 8, fv, fp16);
        }
        ok = signal_ready(g, leader, &ready[g], fin && ok);
        if (!ok) break;
      }
      if (!ok) break;
      // layer 0: dL/d(grid features) -> table gradient (each half its own grid chunks)
      {
        const bool fin = tc::mbar_wait(&done[g], dph);
        dph ^= 1u;
        tc::fence_after_sync();
        float dg[NGRID];
        tc::tmem_load<NGRID / 16>(tD + lane_addr, dg);
        ok = bar_red_and(1 + g, 2 * kRows, fin && ok);
        if (!ok) break;
        if constexpr (SCAT) {
          // hand the gradient to the scatter warps through the third hidden tile
          float* dgs = reinterpret_cast<float*>(Hs + 2 * H_BYTES);
          static_assert(NGRID * kRows * 4 <= H_BYTES, "grid gradient staging fits a hidden tile");
#pragma unroll
          for (int ch = 0; ch < GCH; ++ch)
            if ((ch & 1) == h) {
#pragma unroll
              for (int i = 0; i < 8; ++i) dgs[(8 * ch + i) * kRows + t] = dg[8 * ch + i] * inv_S;
            }
          ok = bar_red_and(1 + g, 2 * kRows, ok);
          if (!ok) break;
          if (leader) tc::mbar_arrive(&sfull[g]);
          continue;
        }
        // Stage the row's grid gradient in the (now idle) delta tile, column t,
        // so the level loop below can index it: [feature][row] floats; each
        // half stages and scatters the levels of its own chunks.
        float* dgs = reinterpret_cast<float*>(Dt);
        static_assert(NGRID * kRows * 4 <= D_BYTES, "grid gradient staging fits the delta tile");
#pragma unroll
        for (int ch = 0; ch < GCH; ++ch)
          if ((ch & 1) == h) {
#pragma unroll
            for (int i = 0; i < 8; ++i) dgs[(8 * ch + i) * kRows + t] = dg[8 * ch + i] * inv_S;
          }
        if (valid) {
          const float p3[3] = {x[0], x[1], x[2]};
          float* gt = ta.grad + ta.n_mlp;
#pragma unroll 1
          for (int ch = h; ch < GCH; ch += 2) {
#pragma unroll 1
            for (int j = 0; j < LPC; ++j) {
              const int lv = ch * LPC + j;
              float df[F];
#pragma unroll
              for (int k = 0; k < F; ++k) df[k] = dgs[(F * lv + k) * kRows + t];
              scatter_level<F, SMOOTH>(a, gt, lv, p3, df);
            }
          }
        }
      }
    }
    if constexpr (SCAT) tc::reg_dealloc<kScatRegLaunch>();
  }

  // ---- flush the CTA's weight gradients (M = 64 accumulators) to global
  tc::fence_before_sync();
  ok = __syncthreads_and(ok) != 0;
  tc::fence_after_sync();
  if (ok && cta_tiles > 0 && !issuer && !scatter) {
    const int row = (warp & 3) * 16 + lane;  // valid for lane < 16
    const uint32_t qaddr = uint32_t((warp & 3) * 32) << 16;
    // one accumulator per layer m, compute warpgroup m % (2 NWG) flushing it;
    // the layer's TMEM column and width are compile-time constants (no
    // runtime-indexed local arrays: a build that held them on the stack read
    // every layer from column 0)
    const int cwg = warp / 4;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      if (m % (2 * NWG) != cwg) continue;
      const uint32_t col_m = m == 0 ? CW0 : (m == 1 ? CW1 : (m == 2 ? CW2 : CW3));
      const int width_m = m == 0 ? NENC : kWidth;
      const int ncols = m == 3 ? nout : width_m;
      const long off_m = ta.layer_elem_off[m];
      for (int c0 = 0; c0 < ncols; c0 += 16) {
        float v[16];
        tc::tmem_load<1>(tbase + qaddr + col_m + uint32_t(c0), v);
        if (lane < 16) {
          if (m < 3) {
            // dW_m[out = row][in = col]: a thread's 16 columns are contiguous, added as 4 float4
            // (the layer offsets and widths are multiples of 4 floats)
#pragma unroll
            for (int i = 0; i < 16; i += 4)
              if (c0 + i < ncols)
                atomicAdd(reinterpret_cast<float4*>(ta.grad + off_m + long(row) * width_m + c0 + i),
                          make_float4(v[i] * inv_S, v[i + 1] * inv_S, v[i + 2] * inv_S, v[i + 3] * inv_S));
          } else {
            // W3[out = col][in = row]: the 16 threads' rows are contiguous for each column
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (c0 + i < ncols) atomicAdd(ta.grad + off_m + long(c0 + i) * kWidth + row, v[i] * inv_S);
          }
        }
      }
    }
  }
  if (!ok && threadIdx.x == 0) atomicExch(a.err, 3);
  // loss partial sum of this CTA
  {
    __shared__ double red[SCAT ? kScatThreadsPerCta / 32 : NWG * 8 + 1];
    double v = (issuer || scatter) ? 0.0 : loss_acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int i = 0; i < int(blockDim.x / 32); ++i) s += red[i];
      ta.partials[blockIdx.x] = s;
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (issuer) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tbase, kTrainCols);
  }
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH, int NWG, bool SCAT,
          bool REC>
static nmg_status launch_train(const TrainArgs& a, int grid, cudaStream_t st) {
  constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  constexpr int DW = NOUTMAX > kWidth ? NOUTMAX : kWidth;
  auto kern = k_fused_train<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, NWG, SCAT, REC>;
  if constexpr (SCAT) {
    // the register split assumes the kernel was compiled to exactly its launch registers
    static int regs_ok = 0;
    if (regs_ok == 0) {
      cudaFuncAttributes attr;
      regs_ok = cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(kern)) == cudaSuccess &&
                        attr.numRegs == kScatRegLaunch
                    ? 1
                    : -1;
    }
    if (regs_ok < 0) return launch_train<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, NWG, false, REC>(a, grid, st);
  }
  const size_t smem = size_t((a.f.w_bytes + 1023u) & ~1023u) +
                      NWG * (size_t(kRows) * NENC * 2 + 3 * size_t(kRows) * kWidth * 2 + size_t(kRows) * DW * 2 +
                             (REC ? size_t(kRows) * 8 * 4 : 0) + (SCAT ? 2 * size_t(kRows) * 4 * 4 : 0) +
                             2 * size_t(kRows) * 2 * 4) +
                      256;
  nmg_status s = ensure_smem(reinterpret_cast<const void*>(kern), smem);
  if (s != NMG_OK) return s;
  kern<<<grid, SCAT ? kScatThreadsPerCta : 2 * NWG * kRows + 32, smem, st>>>(a);
  return check_launch("k_fused_train");
}

nmg_status fused_train_step(nmg_ctx* c, const float* x, const float* rec, const int* d_count, int n_max,
                            double* stats, cudaStream_t st) {
  return fused_train_step_src(c, x, rec, nullptr, d_count, n_max, stats, st);
}

nmg_status fused_train_step_src(nmg_ctx* c, const float* x, const float* rec, const TrainRecords* src,
                                const int* d_count, int n_max, double* stats, cudaStream_t st) {
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
  if (src) {
    a.vid = src->vid;
    a.id_base = src->id_base;
    a.pixels = src->pixels;
    a.rr = *src->rr;
  }
  a.rstride = c->lay.record_floats;
  a.loss_scale = c->cfg.loss_scale;
  a.grad = c->grad;
  a.n_mlp = c->lay.n_mlp;
  for (int l = 0; l < c->lay.n_layers; ++l) {
    // the weight-gradient flush adds float4 rows of the hidden layers
    NMG_REQUIRE(c->lay.off[l] % 4 == 0, "layer %d offset %ld not a multiple of 4", l, long(c->lay.off[l]));
    a.layer_elem_off[l] = c->lay.off[l];
  }
  a.partials = c->ws.partials;
  const int sms = sm_count();
  const int tiles = (n_max + kRows - 1) / kRows;
  const int per_cta = 2;  // pipelines (tiles in flight) per CTA
  int grid = (tiles + per_cta - 1) / per_cta < sms ? (tiles + per_cta - 1) / per_cta : sms;
  if (grid < 1) grid = 1;
  if (grid > c->ws.n_partials / 2) grid = c->ws.n_partials / 2;
  NMG_CUDA_TRY(cudaMemsetAsync(c->grad, 0, sizeof(float) * size_t(c->lay.n_params), st));
  NMG_CUDA_TRY(cudaMemsetAsync(c->ws.partials, 0, sizeof(double) * (c->ws.n_partials / 2), st));
  nmg_status r;
  // the records mode is its own instantiation: the load stage of the plain
  // one stays free of the record code
  const bool recs = src != nullptr;
  switch (s->preset) {
    case 1:
      r = recs ? launch_train<2, 16, 1, 4, 4, 8, 48, false, 2, true, true>(a, grid, st)
               : launch_train<2, 16, 1, 4, 4, 8, 48, false, 2, true, false>(a, grid, st);
      break;
    case 2:
      r = recs ? launch_train<2, 16, 1, 4, 4, 16, 80, false, 2, true, true>(a, grid, st)
               : launch_train<2, 16, 1, 4, 4, 16, 80, false, 2, true, false>(a, grid, st);
      break;
    case 3:
      r = recs ? launch_train<4, 8, 0, 2, 4, 8, 48, true, 2, true, true>(a, grid, st)
               : launch_train<4, 8, 0, 2, 4, 8, 48, true, 2, true, false>(a, grid, st);
      break;
    default: return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
  }
  if (r != NMG_OK) return r;
  r = optimizer_step(c, d_count, n_max, stats, st);
  if (r != NMG_OK) return r;
  return pack_images(c, st);
}

}  // namespace nmg
