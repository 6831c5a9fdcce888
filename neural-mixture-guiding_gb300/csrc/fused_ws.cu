// fused_ws.cu -- warp-specialised fused query kernel.
//
// The query pass spends most of its time on the hash-grid corner gathers: 128
// four-byte loads per query into the L2-resident table, which reach L1 as ~70
// separate 32-byte sector requests. An SM issues about one such request per
// cycle, and it only does so while enough of its threads are gathering. In
// the one-kernel-per-warpgroup design (fused.cu) every warpgroup alternates
// between gathering, the MLP chain and the mixture epilogue, so the request
// path idles whenever the groups happen to be in the other phases.
//
// Here the roles are split inside one persistent CTA per SM:
//   * E encoder warpgroups (few registers per thread after setmaxnreg) only
//     featurise and encode: thread t writes row t of a 128-query tile into a
//     shared-memory slot of a ring of S, then arrives on the slot's "full"
//     mbarrier (count 128);
//   * C consumer warpgroups (many registers) take the tiles in turn: one
//     elected thread issues the tcgen05 MMAs of the 4 layers (weights
//     resident in shared memory, accumulators in the group's TMEM columns),
//     the group's threads apply the ReLU epilogues into their own hidden
//     tile and finally run the mixture (activation, cosine lobe, selection,
//     vMF sampling, pdf) on the output row held in registers. The layer-0
//     MMA's commit also arrives on the slot's "empty" mbarrier, which hands
//     the slot back to the encoders as soon as the tensor core has read it.
// Tile j of a CTA lives in slot j % S, is encoded by warpgroup j % E and
// consumed by consumer j % C; the parities of round j / S drive the waits.
// The configurations (E, C, S and the register split) are the tiling ids
// 8-12 of nmg_set_query_tiling; the autotuner times them against the
// one-pipeline-per-warpgroup kernel.
//
// Every wait is bounded; on a timeout the kernel records an error and all
// roles leave through their own (bounded) waits. Each configuration's
// register split adds up to its launch allocation, and the host launches a
// configuration only after checking that the kernel was compiled to exactly
// that many registers per thread.
#include "api_common.cuh"
#include "ctx.cuh"
#include "fused_common.cuh"
#include "tcgen05.cuh"

namespace nmg {

// A warp-specialised configuration: E encoder and C consumer warpgroups, S
// ring slots, and the register split (launch / encoder / consumer registers
// per thread), which must add up to the launch allocation.
template <int E_, int C_, int S_, int RL_, int RE_, int RC_, bool HS_ = false>
struct WsCfg {
  static constexpr int E = E_, C = C_, S = S_, RL = RL_, RE = RE_, RC = RC_;
  // HS: hidden activations overwrite the input tile in its slot (no separate
  // hidden tiles, 32 KB less shared memory and so more L1 for the gathers);
  // the slot is then handed back after the last layer instead of the first.
  static constexpr bool HS = HS_;
  static constexpr int THREADS = (E + C) * kRows;
  static_assert(E * kRows * RE + C * kRows * RC == THREADS * RL, "register split must equal the launch allocation");
  static_assert(THREADS * RL <= 65536, "one CTA per SM");
  static_assert(S % E == 0, "each slot keeps one encoder warpgroup");
};
// Tiling ids of nmg_set_query_tiling.
using WsE4C2 = WsCfg<4, 2, 4, 80, 56, 128>;   // 8
using WsE5C1 = WsCfg<5, 1, 5, 80, 64, 160>;   // 9
using WsE6C2 = WsCfg<6, 2, 6, 64, 48, 112>;   // 10
using WsE4C2S8 = WsCfg<4, 2, 8, 80, 56, 128>; // 11
using WsE4C2HS = WsCfg<4, 2, 4, 80, 56, 128, true>;  // 12

template <int F, int LEVELS, int MODE, int SHDEG, int BINS>
struct WsShape {
  static constexpr int NDIR = MODE == 0 ? SHDEG * SHDEG + 3 * BINS : 2 * SHDEG * SHDEG + BINS;
  static constexpr int NENC = (LEVELS * F + NDIR + 15) / 16 * 16;
  static constexpr uint32_t TILE_IN = uint32_t(kRows) * NENC * 2;
  static constexpr uint32_t TILE_H = uint32_t(kRows) * kWidth * 2;
  // bytes of one ring slot: an input tile, or a hidden tile when it lives there
  template <bool HS> static constexpr uint32_t slot() { return HS && TILE_H > TILE_IN ? TILE_H : TILE_IN; }
};

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, class Cfg>
static size_t ws_smem_bytes(uint32_t w_bytes) {
  using Sh = WsShape<F, LEVELS, MODE, SHDEG, BINS>;
  return size_t((w_bytes + 1023u) & ~1023u) + Cfg::S * size_t(Sh::template slot<Cfg::HS>()) +
         (Cfg::HS ? 0 : Cfg::C * size_t(Sh::TILE_H)) + (2 * Cfg::S + 1 + Cfg::C) * 8 + 16;
}

// STREAM: the mixture epilogue re-reads the raw outputs from TMEM lobe group
// by lobe group (query_epilogue_streamed); 16-lobe queries without raw outputs.
template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH, class Cfg,
          bool STREAM = false>
__global__ void __launch_bounds__(Cfg::THREADS, 1) k_fused_query_ws(const __grid_constant__ FusedArgs a) {
  using Sh = WsShape<F, LEVELS, MODE, SHDEG, BINS>;
  constexpr int NENC = Sh::NENC;
  constexpr int S = Cfg::S;
  constexpr uint32_t SLOT = Sh::template slot<Cfg::HS>();
  constexpr int kWsEncoders = Cfg::E, kWsConsumers = Cfg::C;
  constexpr uint32_t COLS = NOUTMAX <= 64 ? 64 : 128;  // TMEM columns per consumer
  constexpr uint32_t TCOLS = COLS * kWsConsumers <= 64 ? 64 : (COLS * kWsConsumers <= 128 ? 128 : 256);
  static_assert(COLS * kWsConsumers <= 256, "TMEM columns");
  extern __shared__ __align__(1024) uint8_t smem[];

  const uint32_t w_region = (a.w_bytes + 1023u) & ~1023u;
  uint8_t* wsm = smem;
  uint8_t* slots = smem + w_region;
  uint8_t* hid = slots + S * SLOT;
  uint64_t* full = reinterpret_cast<uint64_t*>(hid + (Cfg::HS ? 0 : kWsConsumers * Sh::TILE_H));
  uint64_t* empty = full + S;
  uint64_t* wbar = empty + S;
  uint64_t* done = wbar + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + kWsConsumers);
  const int wg = threadIdx.x / kRows, t = threadIdx.x % kRows;
  const int alloc_warp = kWsEncoders * 4;  // first warp of the first consumer

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(&full[s], kRows);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(wbar, 1);
    for (int c = 0; c < kWsConsumers; ++c) tc::mbar_init(&done[c], 1);
    tc::fence_mbar_init();
  }
  if (int(threadIdx.x / 32) == alloc_warp) tc::tmem_alloc(tslot, TCOLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(wbar, a.w_bytes);
    for (uint32_t off = 0; off < a.w_bytes; off += 16384u) {
      const uint32_t nb = a.w_bytes - off < 16384u ? a.w_bytes - off : 16384u;
      tc::bulk_g2s(wsm + off, a.wimg + off, nb, wbar);
    }
  }
  const int n = fused_count(a.d_count, a.n_max);
  const long ntiles = (long(n) + kRows - 1) / kRows;
  bool ok = true;

  if (wg < kWsEncoders) {
    // ------------------------------------------------------------- encoders
    __syncwarp();
    tc::reg_dealloc<Cfg::RE>();
    for (int j = wg;; j += kWsEncoders) {
      const long tile = blockIdx.x + long(j) * gridDim.x;
      if (tile >= ntiles) break;
      const int s = j % S;
      const uint32_t r = uint32_t(j / S);
      if (!tc::mbar_wait(&empty[s], (r & 1u) ^ 1u)) {
        ok = false;
        break;
      }
      const long q = tile * kRows + t;
      float x[10];
#pragma unroll
      for (int d = 0; d < 10; ++d) x[d] = 0.f;
      if (q < n) {
        if (a.raw_mode)
          load_row(a.x, q, a.enc.n_input, x);
        else
          featurize<true>(a.enc, load3(a.pos, q), load3(a.wo, q), load3(a.nrm, q), a.rough[q], x);
      }
      encode_row<F, LEVELS, MODE, SHDEG, BINS, SMOOTH, false, true>(a, x, slots + s * SLOT, t);
      tc::fence_proxy_async();
      tc::mbar_arrive(&full[s]);
    }
    if (!ok) atomicExch(a.err, 5);
  } else {
    // ------------------------------------------------------------ consumers
    __syncwarp();
    tc::reg_alloc<Cfg::RC>();
    const int c = wg - kWsEncoders;
    const int bar = 1 + c;  // named barrier of this consumer warpgroup
    ok = bar_red_and(bar, kRows, tc::mbar_wait(wbar, 0));
    const uint32_t tmem = *tslot + uint32_t(c) * COLS;
    const uint32_t lane_addr = tmem + (uint32_t((t / 32) * 32) << 16);
    uint8_t* H = hid + c * Sh::TILE_H;  // with HS: set per tile to the tile's slot
    const uint32_t w_addr = tc::smem_u32(wsm);
    const int nl = a.n_layers;
    uint32_t phase = 0;
    // Issues layer l's MMAs (one elected thread): A = `a_addr` tile of kin columns.
    auto issue = [&](int l, uint32_t a_addr) {
      issue_layer(a, l, tmem, a_addr, w_addr, l == 0 ? NENC : kWidth, l == nl - 1 ? a.n_out_pad : kWidth);
    };
    // Every exit below follows a bar.red over the group (or depends only on
    // j), so the 128 threads always leave together. (Issuing the next tile's
    // layer 0 before this tile's mixture epilogue measured 10% slower, both
    // with the issuing thread waiting for the next slot and when it issues
    // only if that slot is already full.)
    for (int j = c;; j += kWsConsumers) {
      const long tile = blockIdx.x + long(j) * gridDim.x;
      if (tile >= ntiles) break;
      const int s = j % S;
      const uint32_t r = uint32_t(j / S);
      if (Cfg::HS) H = slots + s * SLOT;
      const uint32_t h_addr = tc::smem_u32(H);
      bool got = true;
      if (t == 0) {
        got = tc::mbar_wait(&full[s], r & 1u);
        if (got) {
          tc::fence_after_sync();
          issue(0, tc::smem_u32(slots + s * SLOT));
          if (!Cfg::HS) tc::mma_commit(&empty[s]);  // the slot is free once layer 0 has read it
          tc::mma_commit(&done[c]);
        }
      }
      ok = bar_red_and(bar, kRows, got && ok);
      if (!ok) break;
      float rr[NOUTMAX];
      bool last_ok = true;
      for (int l = 0; l < nl; ++l) {
        const bool last = l == nl - 1;
        const bool d = tc::mbar_wait(&done[c], phase);
        phase ^= 1u;
        tc::fence_after_sync();
        if (!last) {
          float v[kWidth];
          tc::tmem_load<kWidth / 16>(lane_addr, v);
#pragma unroll
          for (int cc = 0; cc < kWidth / 8; ++cc) store_chunk_relu(H, t, cc, kWidth / 8, v + 8 * cc, layer_fp16(a, l + 1));
          tc::fence_proxy_async();
          tc::fence_before_sync();
          ok = bar_red_and(bar, kRows, d);
          if (!ok) break;
          if (t == 0) {
            tc::fence_after_sync();
            issue(l + 1, h_addr);
            if (Cfg::HS && l + 1 == nl - 1) tc::mma_commit(&empty[s]);  // last reader of the slot
            tc::mma_commit(&done[c]);
          }
        } else {
          if constexpr (!STREAM) {
            tc::tmem_load_n<NOUTMAX / 16>(lane_addr, rr, (a.n_out_pad + 15) / 16);
            tc::fence_before_sync();
          }
          last_ok = d;
        }
      }
      if (!ok) break;
      const long q = tile * kRows + t;
      if constexpr (STREAM) {
        // warp-collective TMEM reads: the group agrees on ok first, and the accumulator must
        // outlive every thread's reads, so the group meets again before the next layer 0
        ok = bar_red_and(bar, kRows, last_ok);
        if (!ok) break;
        query_epilogue_streamed<K>(a, q, q < n, lane_addr);
        tc::fence_before_sync();
        ok = bar_red_and(bar, kRows, ok);
        if (!ok) break;
      } else {
        ok = last_ok;  // reconciled across the group at the next tile's barrier
        if (q < n && ok) query_epilogue<K, NOUTMAX>(a, q, rr);
      }
    }
    if (!ok && t == 0) atomicExch(a.err, 6);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (int(threadIdx.x / 32) == alloc_warp) {
    tc::fence_after_sync();
    tc::tmem_dealloc(*tslot, TCOLS);
  }
}

// Launch-time check of the register split: the kernel must have been
// compiled to exactly the launch registers per thread the split assumes.
template <class Kern>
static nmg_status ws_check_regs(Kern kern, int want) {
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(kern)) != cudaSuccess) return NMG_ERR_CUDA;
  return attr.numRegs == want ? NMG_OK : NMG_ERR_UNSUPPORTED;
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH, class Cfg,
          bool STREAM = false>
static nmg_status launch_ws(const FusedArgs& a, cudaStream_t st) {
  auto kern = k_fused_query_ws<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, Cfg, STREAM>;
  static int regs_ok = 0;  // 1: checked and usable, -1: unusable
  if (regs_ok == 0) regs_ok = ws_check_regs(kern, Cfg::RL) == NMG_OK ? 1 : -1;
  if (regs_ok < 0)
    return set_error(NMG_ERR_UNSUPPORTED, "warp-specialised query kernel not compiled to %d registers", Cfg::RL);
  const size_t smem = ws_smem_bytes<F, LEVELS, MODE, SHDEG, BINS, Cfg>(a.w_bytes);
  nmg_status s = ensure_smem(reinterpret_cast<const void*>(kern), smem);
  if (s != NMG_OK) return s;
  const long tiles = (long(a.n_max) + kRows - 1) / kRows;
  int grid = sm_count();
  if (tiles < grid) grid = int(tiles > 0 ? tiles : 1);
  kern<<<grid, Cfg::THREADS, smem, st>>>(a);
  return check_launch("k_fused_query_ws");
}

template <int F, int LEVELS, int MODE, int SHDEG, int BINS, int K, int NOUTMAX, bool SMOOTH>
static nmg_status launch_ws_tiling(int tiling, const FusedArgs& a, cudaStream_t st) {
  switch (tiling) {
    case 8: return launch_ws<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, WsE4C2>(a, st);
    case 9: return launch_ws<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, WsE5C1>(a, st);
    case 10: return launch_ws<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, WsE6C2>(a, st);
    case 11: return launch_ws<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, WsE4C2S8>(a, st);
    case 12: return launch_ws<F, LEVELS, MODE, SHDEG, BINS, K, NOUTMAX, SMOOTH, WsE4C2HS>(a, st);
  }
  return set_error(NMG_ERR_INVALID_ARG, "tiling %d is not a warp-specialised one", tiling);
}

nmg_status launch_query_ws(int preset, int tiling, const FusedArgs& a, cudaStream_t st) {
  switch (preset) {
    case 1: return launch_ws_tiling<2, 16, 1, 4, 4, 8, 48, false>(tiling, a, st);
    case 2:
      if (!a.raw && !a.raw_mode) return launch_ws<2, 16, 1, 4, 4, 16, 80, false, WsE4C2, true>(a, st);
      return launch_ws<2, 16, 1, 4, 4, 16, 80, false, WsE4C2>(a, st);
    case 3: return launch_ws_tiling<4, 8, 0, 2, 4, 8, 48, true>(tiling, a, st);
  }
  return set_error(NMG_ERR_UNSUPPORTED, "configuration has no fused kernel");
}

}  // namespace nmg
