// records.cu -- training records from the per-pixel radiance records of a
// frame (the reference's generate_training_data, train.cu:14-67), and one
// frame's training on them (the reference's trainStep, integrator.cpp:650-701).
//
// The integrator stores, for every pixel and path vertex, the raw vertex data
// (GuidedPixelStateBuffer::incrementDepth, workqueue.h:26-54) and adds the
// radiance arriving later to every earlier vertex (recordRadiance,
// workqueue.h:58-67). Once per frame a grid of training pixels (offset +
// stride over the image) turns each non-delta vertex into one GuidedInput /
// GuidedOutput pair (vertex_record, records.cuh): the local incident radiance
// L / thp (channels with thp > 1e-5) weighted by the MIS weight (and by the
// BSDF value with product sampling), its direction and pdfs, and the network
// inputs of the vertex. A record is dropped, as in train.cu:57-62, when its
// normalised position, its direction, its warped outgoing direction, its pdf
// or its local radiance (tested BEFORE the BSDF factor, which multiplies only
// the stored copy) has a NaN, or its pdf is zero; a NaN BSDF value alone keeps
// the record, with a NaN radiance, as it does in the reference.
//
// The extraction kernel runs one block per (group of 256 training pixels,
// depth), so that the vertices of different depths load in parallel, and
// appends with one atomic per block and round (block-aggregated: the append
// counter is a single address; one atomic per warp serialised on it), staging
// the block's rows in shared memory so that they leave as contiguous stores.
// The count stays on the device and can feed nmg_train_step directly.
// Measured for a 1920x1080 frame of 6 bounces: 715 us with one atomic per
// warp, 530 us per block, 495 us with the staged stores, 365 us once every
// field of a vertex is loaded before any is tested. (Counting every vertex
// first, then writing, measured 800 us: the second pass over the vertices
// costs more than it saves.)
#include <string.h>

#include "api_common.cuh"
#include "records.cuh"

namespace nmg {

struct RecordArgs {
  nmg_radiance_records r;
  nmg_train_pixels tp;
  EncodingParams enc;
  int selection;
  int capacity;
  float* x;
  float* rec;
  uint32_t* ids;
  int* count;
};

constexpr int kRecordThreads = 256;

// blockIdx.y is the depth. IDS: write 32-bit vertex ids instead of rows.
template <bool IDS>
__global__ void __launch_bounds__(kRecordThreads) k_extract_records(const __grid_constant__ RecordArgs a) {
  __shared__ int s_warp[2][kRecordThreads / 32];  // per warp: its count, then its offset (by round parity)
  __shared__ int s_base[2];                       // the block's first index for this round
  __shared__ int s_tot[2];                        // the block's record count for this round
  // The block's rows of one round, compacted, so that they leave as contiguous
  // coalesced stores (a thread storing its own 10- and 7-float rows would touch
  // ~40 sectors per warp store for 4 bytes of each)
  __shared__ float s_x[IDS ? 1 : kRecordThreads * 10], s_r[IDS ? 1 : kRecordThreads * 7];
  __shared__ uint32_t s_id[IDS ? kRecordThreads : 1];
  const long n = long(a.tp.train_res[0]) * a.tp.train_res[1];
  const uint32_t pixels = a.tp.res[0] * a.tp.res[1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ni = a.enc.n_input, rf = a.selection ? 7 : 6;
  const int d = blockIdx.y;
  // grid-stride over whole blocks, so that every thread reaches the block-wide barriers
  int round = 0;
  for (long base = long(blockIdx.x) * blockDim.x; base < n; base += long(gridDim.x) * blockDim.x, ++round) {
    const long tid = base + threadIdx.x;
    int pixel = -1;
    if (tid < n) {
      const uint32_t tx = uint32_t(tid % a.tp.train_res[0]), ty = uint32_t(tid / a.tp.train_res[0]);
      const uint32_t px = tx * a.tp.stride[0] + a.tp.offset[0], py = ty * a.tp.stride[1] + a.tp.offset[1];
      if (px < a.tp.res[0] && py < a.tp.res[1]) pixel = int(px + py * a.tp.res[0]);
    }
    bool keep = false;
    float xin[10], out[7];
    if (pixel >= 0 && d < int(a.r.cur_depth[pixel]))
      keep = vertex_record(a.r.depth[d], a.r.product, a.enc, uint32_t(pixel), xin, out);
    // block-aggregated append: the warps' counts, one atomic for the block, then each warp's offset.
    // A warp's slot is rewritten only by its own lane 0, after the next __ballot_sync, which every
    // lane of the warp reaches only after its reads; thread 0 rewrites the totals and the base only
    // after the next round's first barrier; the slots also alternate with the round's parity.
    const int sb = round & 1;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) s_warp[sb][warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < kRecordThreads / 32; ++w) {
        const int c = s_warp[sb][w];
        s_warp[sb][w] = tot;
        tot += c;
      }
      s_base[sb] = tot ? atomicAdd(a.count, tot) : 0;
      s_tot[sb] = tot;
    }
    __syncthreads();
    if (keep) {
      const int local = s_warp[sb][warp] + __popc(m & ((1u << lane) - 1u));
      if constexpr (IDS) {
        s_id[local] = vertex_id(d, uint32_t(pixel), pixels);
      } else {
#pragma unroll
        for (int k = 0; k < 10; ++k)
          if (k < ni) s_x[local * ni + k] = xin[k];
#pragma unroll
        for (int k = 0; k < 7; ++k)
          if (k < rf) s_r[local * rf + k] = out[k];
      }
    }
    __syncthreads();
    // the block's rows [base, base + tot), written out contiguously (up to the capacity); the staged rows
    // are rewritten only after the next round's two barriers, which every thread reaches after this copy
    const long rbase = s_base[sb];
    const int tot = s_tot[sb];
    const long rows = rbase + tot <= a.capacity ? tot : (rbase < a.capacity ? a.capacity - rbase : 0);
    if constexpr (IDS) {
      for (long i = threadIdx.x; i < rows; i += kRecordThreads) a.ids[rbase + i] = s_id[i];
    } else {
      for (long i = threadIdx.x; i < rows * ni; i += kRecordThreads) a.x[rbase * ni + i] = s_x[i];
      for (long i = threadIdx.x; i < rows * rf; i += kRecordThreads) a.rec[rbase * rf + i] = s_r[i];
    }
  }
}

// Record counts of a frame's training batches, as the reference's training
// loop sizes them (integrator.cpp:666-672): batch i holds min(N - i B, B) of
// the N stored records, rounded down to a multiple of 128, and the loop stops
// at the first batch below min_batch (the sizes only shrink with i, so every
// later batch is below it too). A count of 0 makes that batch's training step
// a no-op (no optimiser step).
__global__ void k_batch_counts(const int* __restrict__ d_count, int capacity, int batch, int batches, int min_batch,
                               int* __restrict__ counts) {
  int n = *d_count;
  n = n < 0 ? 0 : (n > capacity ? capacity : n);
  for (int i = threadIdx.x; i < batches; i += blockDim.x) {
    const long rem = long(n) - long(i) * batch;
    long c = rem < 0 ? 0 : (rem > batch ? batch : rem);
    c -= c % 128;
    counts[i] = (c > 0 && c >= min_batch) ? int(c) : 0;
  }
}

// Rows of one batch for the plain path: x[q][n_input] and rec[q][rf] of the
// vertices vid[base + q], q < *count.
__global__ void k_gather_rows(nmg_radiance_records rr, EncodingParams enc, int rf, const uint32_t* __restrict__ vid,
                              long base, uint32_t pixels, const int* __restrict__ count, int n_max,
                              float* __restrict__ x, float* __restrict__ rec) {
  int n = *count;
  n = n > n_max ? n_max : n;
  for (long q = long(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    const uint32_t v = vid[base + q], d = v / pixels;
    float xin[10], out[7];
    vertex_record(rr.depth[d], rr.product, enc, v - d * pixels, xin, out);
    for (int k = 0; k < enc.n_input; ++k) x[q * enc.n_input + k] = xin[k];
    for (int k = 0; k < rf; ++k) rec[q * rf + k] = out[k];
  }
}

static nmg_status check_records(const nmg_ctx* c, const nmg_radiance_records* r, const nmg_train_pixels* tp) {
  NMG_REQUIRE(r->max_depth >= 0 && r->max_depth <= NMG_MAX_TRAIN_DEPTH, "max_depth=%d (0..%d)", r->max_depth,
              NMG_MAX_TRAIN_DEPTH);
  NMG_REQUIRE(tp->stride[0] >= 1 && tp->stride[1] >= 1, "zero training-pixel stride");
  const long n = long(tp->train_res[0]) * tp->train_res[1];
  NMG_REQUIRE(n == 0 || r->cur_depth, "NULL cur_depth");
  for (int d = 0; d < r->max_depth; ++d) {
    const auto& R = r->depth[d];
    NMG_REQUIRE(R.L && R.thp && R.pos && R.dir && R.wi_pdf && R.mis_weight && R.wo && R.normal && R.roughness,
                "NULL record array at depth %d", d);
    NMG_REQUIRE(!c->cfg.selection || R.bsdf_pdf, "learned selection needs bsdf_pdf (depth %d)", d);
  }
  return NMG_OK;
}

static RecordArgs record_args(const nmg_ctx* c, const nmg_radiance_records* r, const nmg_train_pixels* tp,
                              int capacity, int* d_count) {
  RecordArgs a;
  memset(&a, 0, sizeof(a));
  a.r = *r;
  a.tp = *tp;
  a.enc = c->enc;
  a.selection = c->cfg.selection;
  a.capacity = capacity;
  a.count = d_count;
  return a;
}

// Blocks of the extraction grid along the pixels (the depths are its second
// dimension): about 8 blocks per SM in all.
static unsigned extraction_blocks(long n, int depths) {
  const long blocks = (n + kRecordThreads - 1) / kRecordThreads;
  const long cap = (152L * 8 + depths - 1) / depths;
  return unsigned(blocks > cap ? cap : (blocks > 0 ? blocks : 1));
}

}  // namespace nmg

using namespace nmg;

extern "C" nmg_status nmg_extract_records(nmg_ctx* c, const nmg_radiance_records* r, const nmg_train_pixels* tp,
                                          int capacity, float* x, float* records, int* d_count, nmg_stream stream) {
  NMG_REQUIRE(c && r && tp && x && records && d_count, "NULL argument");
  NMG_REQUIRE(capacity >= 0, "capacity=%d", capacity);
  NMG_TRY(check_records(c, r, tp));
  cudaStream_t st = (cudaStream_t)stream;
  NMG_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(int), st));
  const long n = long(tp->train_res[0]) * tp->train_res[1];
  if (n == 0 || r->max_depth == 0) return NMG_OK;
  RecordArgs a = record_args(c, r, tp, capacity, d_count);
  a.x = x;
  a.rec = records;
  const int depths = r->max_depth;
  k_extract_records<false><<<dim3(extraction_blocks(n, depths), unsigned(depths)), kRecordThreads, 0, st>>>(a);
  return check_launch("k_extract_records");
}

extern "C" nmg_status nmg_train_frame(nmg_ctx* c, const nmg_radiance_records* r, const nmg_train_pixels* tp,
                                      int capacity, uint32_t* vertex_ids, int* d_count, int batch_size,
                                      int max_batches, int min_batch, double* stats, nmg_stream stream) {
  NMG_REQUIRE(c && r && tp && vertex_ids && d_count, "NULL argument");
  NMG_REQUIRE(capacity >= 0, "capacity=%d", capacity);
  NMG_REQUIRE(batch_size > 0 && batch_size % 128 == 0, "batch_size=%d (a positive multiple of 128)", batch_size);
  NMG_REQUIRE(max_batches >= 1 && max_batches <= kMaxFrameBatches, "max_batches=%d (1..%d)", max_batches,
              kMaxFrameBatches);
  NMG_REQUIRE(min_batch >= 0, "min_batch=%d", min_batch);
  NMG_TRY(check_records(c, r, tp));
  const uint64_t pixels = uint64_t(tp->res[0]) * tp->res[1];
  NMG_REQUIRE(pixels * NMG_MAX_TRAIN_DEPTH < (1ull << 32), "image of %llu pixels: vertex ids need 32 bits",
              (unsigned long long)pixels);
  if (batch_size > c->ws.cap_b || !c->ws.batch_counts)
    return set_error(NMG_ERR_CAPACITY, "batch %d above reserved %d (call nmg_reserve)", batch_size, c->ws.cap_b);
  cudaStream_t st = (cudaStream_t)stream;
  NMG_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(int), st));
  if (stats) NMG_CUDA_TRY(cudaMemsetAsync(stats, 0, sizeof(double) * 2 * size_t(max_batches), st));
  const long n = long(tp->train_res[0]) * tp->train_res[1];
  if (n > 0 && r->max_depth > 0) {
    RecordArgs a = record_args(c, r, tp, capacity, d_count);
    a.ids = vertex_ids;
    const int depths = r->max_depth;
    k_extract_records<true><<<dim3(extraction_blocks(n, depths), unsigned(depths)), kRecordThreads, 0, st>>>(a);
    NMG_TRY(check_launch("k_extract_records"));
  }
  k_batch_counts<<<1, kMaxFrameBatches, 0, st>>>(d_count, capacity, batch_size, max_batches, min_batch,
                                                  c->ws.batch_counts);
  NMG_TRY(check_launch("k_batch_counts"));
  for (int i = 0; i < max_batches; ++i) {
    const int* count = c->ws.batch_counts + i;
    double* st_i = stats ? stats + 2 * i : nullptr;
    if (c->cfg.path == NMG_PATH_FP32) {
      k_gather_rows<<<152 * 4, 256, 0, st>>>(*r, c->enc, c->lay.record_floats, vertex_ids, long(i) * batch_size,
                                             uint32_t(pixels), count, batch_size, c->ws.x, c->ws.recs);
      NMG_TRY(check_launch("k_gather_rows"));
      NMG_TRY(plain_train_step(c, c->ws.x, c->ws.recs, count, batch_size, st_i, st));
    } else {
      const TrainRecords src{vertex_ids, long(i) * batch_size, uint32_t(pixels), r};
      NMG_TRY(fused_train_step_src(c, nullptr, nullptr, &src, count, batch_size, st_i, st));
    }
  }
  return NMG_OK;
}
