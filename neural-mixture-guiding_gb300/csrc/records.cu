// records.cu -- training records from the per-pixel radiance records of a
// frame (the reference's generate_training_data, train.cu:14-67).
//
// The integrator stores, for every pixel and path vertex, the raw vertex data
// (GuidedPixelStateBuffer::incrementDepth, workqueue.h:26-54) and adds the
// radiance arriving later to every earlier vertex (recordRadiance,
// workqueue.h:58-67). Once per frame a grid of training pixels (offset +
// stride over the image) turns each non-delta vertex into one GuidedInput /
// GuidedOutput pair: the local incident radiance L / thp (channels with
// thp > 1e-5) weighted by the MIS weight (and by the BSDF value with product
// sampling), its direction and pdfs, and the network inputs of the vertex.
// A record is dropped, as in train.cu:57-62, when its normalised position,
// its direction, its warped outgoing direction, its pdf or its local radiance
// (tested BEFORE the BSDF factor, which multiplies only the stored copy) has
// a NaN, or its pdf is zero; a NaN BSDF value alone keeps the record, with a
// NaN radiance, as it does in the reference. Here one thread per training
// pixel walks its vertices and appends
// the records with one atomic per block and vertex depth (block-aggregated:
// the append counter is a single address, and one atomic per warp and depth
// serialised on it: 715 -> 530 us for a 1920x1080 frame of 6 bounces), so the
// count can feed nmg_train_step's device count directly. (Counting every
// vertex first for one atomic per block and round, then writing, measured
// 800 us: the second pass over the vertices costs more than it saves.)
#include "api_common.cuh"
#include "ctx.cuh"

namespace nmg {

struct RecordArgs {
  nmg_radiance_records r;
  nmg_train_pixels tp;
  EncodingParams enc;
  int selection;
  int capacity;
  float* x;
  float* rec;
  int* count;
};

constexpr int kRecordThreads = 256;

__global__ void __launch_bounds__(kRecordThreads) k_extract_records(const __grid_constant__ RecordArgs a) {
  __shared__ int s_warp[2][kRecordThreads / 32];  // per warp: its count, then its offset (by depth parity)
  __shared__ int s_base[2];                       // the block's first index for this depth
  const long n = long(a.tp.train_res[0]) * a.tp.train_res[1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ni = a.enc.n_input, rf = a.selection ? 7 : 6;
  const int max_depth = a.r.max_depth < NMG_MAX_TRAIN_DEPTH ? a.r.max_depth : NMG_MAX_TRAIN_DEPTH;
  // grid-stride over whole blocks, so that every thread reaches the block-wide barriers
  for (long base = long(blockIdx.x) * blockDim.x; base < n; base += long(gridDim.x) * blockDim.x) {
    const long tid = base + threadIdx.x;
    int pixel = -1, depth = 0;
    if (tid < n) {
      const uint32_t tx = uint32_t(tid % a.tp.train_res[0]), ty = uint32_t(tid / a.tp.train_res[0]);
      const uint32_t px = tx * a.tp.stride[0] + a.tp.offset[0], py = ty * a.tp.stride[1] + a.tp.offset[1];
      if (px < a.tp.res[0] && py < a.tp.res[1]) {
        pixel = int(px + py * a.tp.res[0]);
        depth = int(a.r.cur_depth[pixel]);
        depth = depth < max_depth ? depth : max_depth;
      }
    }
    for (int d = 0; d < max_depth; ++d) {
      bool keep = false;
      float xin[10], out[7];
      if (pixel >= 0 && d < depth) {
        const auto& R = a.r.depth[d];
        keep = !R.delta || !R.delta[pixel];
        if (keep) {
          const f3 pos = load3(R.pos, pixel);
          const float th = R.dir[2 * pixel], ph = R.dir[2 * pixel + 1];
          const float wi_pdf = R.wi_pdf[pixel];
          const float mis = R.mis_weight[pixel];
          // local radiance (train.cu:44-49): L / thp per channel with thp > 1e-5,
          // times the MIS weight. The NaN test below reads this L; the BSDF value
          // multiplies only the stored copy (train.cu:50-53), as in the reference.
          float L[3], Lout[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float thp = R.thp[3 * pixel + c];
            L[c] = thp > NMG_EPS ? __fdiv_rn(R.L[3 * pixel + c], thp) : 0.f;
            L[c] = __fmul_rn(L[c], mis);
            Lout[c] = (a.r.product && R.bsdf_val) ? __fmul_rn(L[c], R.bsdf_val[3 * pixel + c]) : L[c];
          }
          // network inputs (train.cu:34-43): the position in the inflated box,
          // the outgoing direction and the auxiliary normal/roughness inputs
          float sw, cw, sp, cp;
          sincosf(R.wo[2 * pixel], &sw, &cw);
          sincosf(R.wo[2 * pixel + 1], &sp, &cp);
          const f3 wo{sw * cp, sw * sp, cw};
          const float nth = R.normal[2 * pixel], nph = R.normal[2 * pixel + 1];
          const float rough = R.roughness[pixel];
          // normalizeSpatialCoord (train.h:173-177), bit for bit
          const float p[3] = {pos.x, pos.y, pos.z};
          const float infl = aabb_inflation(a.enc.aabb);
          for (int k = 0; k < 3; ++k) xin[k] = normalize_coord(a.enc.aabb, infl, k, p[k]);
          xin[3] = (wo.x + 1.f) * 0.5f;
          xin[4] = (wo.y + 1.f) * 0.5f;
          xin[5] = (wo.z + 1.f) * 0.5f;
          if (a.enc.input_mode == 0) {
            xin[6] = nth * NMG_INV_PI;
            xin[7] = nph * NMG_INV_2PI;
            xin[8] = 1.f - expf(-rough);
          } else {
            float sn, cn, sq, cq;
            sincosf(nth, &sn, &cn);
            sincosf(nph, &sq, &cq);
            xin[6] = (sn * cq + 1.f) * 0.5f;
            xin[7] = (sn * sq + 1.f) * 0.5f;
            xin[8] = (cn + 1.f) * 0.5f;
            xin[9] = 1.f - expf(-rough);
          }
          out[0] = th;
          out[1] = ph;
          out[2] = Lout[0];
          out[3] = Lout[1];
          out[4] = Lout[2];
          out[5] = wi_pdf;
          out[6] = R.bsdf_pdf ? R.bsdf_pdf[pixel] : 0.f;
          // train.cu:57-62: NaN in the normalised position, the stored direction,
          // the warped outgoing direction (the networks here always take wo as an
          // input, as the reference's default product-sampling build does), the
          // pdf or the local radiance before the BSDF factor, or a zero pdf
          keep = !(isnan(xin[0]) || isnan(xin[1]) || isnan(xin[2]) || isnan(th) || isnan(ph) || isnan(xin[3]) ||
                   isnan(xin[4]) || isnan(xin[5]) || isnan(wi_pdf) || wi_pdf == 0.f || isnan(L[0]) ||
                   isnan(L[1]) || isnan(L[2]));
        }
      }
      // block-aggregated append: the warps' counts, one atomic for the block, then each warp's offset
      // (two barriers per depth). No barrier is needed after the offsets are read: a warp's slot is
      // rewritten only by its own lane 0, after the next __ballot_sync, which every lane of the warp
      // reaches only after its reads, and thread 0 rewrites the totals and the base only after the
      // next depth's first barrier; the slots also alternate with the depth's parity.
      const int sb = d & 1;
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
      }
      __syncthreads();
      if (keep) {
        const long idx = long(s_base[sb]) + s_warp[sb][warp] + __popc(m & ((1u << lane) - 1u));
        if (idx < a.capacity) {
          for (int k = 0; k < ni; ++k) a.x[idx * ni + k] = xin[k];
          for (int k = 0; k < rf; ++k) a.rec[idx * rf + k] = out[k];
        }
      }
    }
  }
}

}  // namespace nmg

using namespace nmg;

extern "C" nmg_status nmg_extract_records(nmg_ctx* c, const nmg_radiance_records* r, const nmg_train_pixels* tp,
                                          int capacity, float* x, float* records, int* d_count, nmg_stream stream) {
  NMG_REQUIRE(c && r && tp && x && records && d_count, "NULL argument");
  NMG_REQUIRE(capacity >= 0, "capacity=%d", capacity);
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
  cudaStream_t st = (cudaStream_t)stream;
  NMG_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(int), st));
  if (n == 0 || r->max_depth == 0) return NMG_OK;
  RecordArgs a;
  a.r = *r;
  a.tp = *tp;
  a.enc = c->enc;
  a.selection = c->cfg.selection;
  a.capacity = capacity;
  a.x = x;
  a.rec = records;
  a.count = d_count;
  long blocks = (n + kRecordThreads - 1) / kRecordThreads;
  if (blocks > 152L * 8) blocks = 152L * 8;
  k_extract_records<<<int(blocks), kRecordThreads, 0, st>>>(a);
  return check_launch("k_extract_records");
}
