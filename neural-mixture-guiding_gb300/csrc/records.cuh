// records.cuh -- the training record of one path vertex: the per-vertex
// body of the reference's generate_training_data (train.cu:29-65), shared by
// the record extraction kernels (records.cu) and the training kernel's load
// stage when it reads the radiance records directly (fused_train.cu).
#pragma once
#include "ctx.cuh"

namespace nmg {

// Vertex `pixel` of one depth's record arrays R: the network input row
// xin[n_input] and GuidedOutput out[6 | 7] {theta, phi, L / thp * mis
// [* bsdfVal], wiPdf[, bsdfPdf]}. Returns whether the reference keeps the
// vertex: not a delta lobe and, as in train.cu:57-62, no NaN in the
// normalised position, the stored direction, the warped outgoing direction
// (the networks here always take wo as an input, as the reference's default
// product-sampling build does), the pdf or L / thp * misWeight (tested
// before the BSDF factor, which multiplies only the stored copy,
// train.cu:50-53), and a non-zero pdf.
NMG_D bool vertex_record(const nmg_record_arrays& R, int product, const EncodingParams& enc, uint32_t pixel,
                         float* xin, float* out) {
  // every field is loaded before any is tested, so that the loads of a vertex
  // are in flight together (each array holds every pixel): testing the delta
  // flag or the throughput first serialised three memory latencies per vertex
  const bool delta = R.delta && R.delta[pixel];
  const f3 pos = load3(R.pos, pixel);
  const float th = R.dir[2 * pixel], ph = R.dir[2 * pixel + 1];
  const float wi_pdf = R.wi_pdf[pixel];
  const float mis = R.mis_weight[pixel];
  const f3 thp3 = load3(R.thp, pixel), L3 = load3(R.L, pixel);
  const bool use_bsdf = product && R.bsdf_val;
  const f3 bv3 = use_bsdf ? load3(R.bsdf_val, pixel) : f3{1.f, 1.f, 1.f};
  const float wo_t = R.wo[2 * pixel], wo_p = R.wo[2 * pixel + 1];
  const float nth = R.normal[2 * pixel], nph = R.normal[2 * pixel + 1];
  const float rough = R.roughness[pixel];
  const float bsdf_pdf = R.bsdf_pdf ? R.bsdf_pdf[pixel] : 0.f;
  // local radiance (train.cu:44-49): L / thp per channel with thp > 1e-5, times the MIS weight
  const float thp[3] = {thp3.x, thp3.y, thp3.z}, Lr[3] = {L3.x, L3.y, L3.z}, bv[3] = {bv3.x, bv3.y, bv3.z};
  float L[3], Lout[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    L[c] = thp[c] > NMG_EPS ? __fdiv_rn(Lr[c], thp[c]) : 0.f;
    L[c] = __fmul_rn(L[c], mis);
    Lout[c] = use_bsdf ? __fmul_rn(L[c], bv[c]) : L[c];
  }
  // network inputs (train.cu:34-43): the position in the inflated box, the
  // outgoing direction and the auxiliary normal/roughness inputs
  float sw, cw, sp, cp;
  sincosf(wo_t, &sw, &cw);
  sincosf(wo_p, &sp, &cp);
  const f3 wo{sw * cp, sw * sp, cw};
  // normalizeSpatialCoord (train.h:173-177), bit for bit
  const float p[3] = {pos.x, pos.y, pos.z};
  const float infl = aabb_inflation(enc.aabb);
#pragma unroll
  for (int k = 0; k < 3; ++k) xin[k] = normalize_coord(enc.aabb, infl, k, p[k]);
  xin[3] = (wo.x + 1.f) * 0.5f;
  xin[4] = (wo.y + 1.f) * 0.5f;
  xin[5] = (wo.z + 1.f) * 0.5f;
  if (enc.input_mode == 0) {
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
  out[6] = bsdf_pdf;
  return !delta && !(isnan(xin[0]) || isnan(xin[1]) || isnan(xin[2]) || isnan(th) || isnan(ph) || isnan(xin[3]) ||
                     isnan(xin[4]) || isnan(xin[5]) || isnan(wi_pdf) || wi_pdf == 0.f || isnan(L[0]) ||
                     isnan(L[1]) || isnan(L[2]));
}

// A vertex of the frame's radiance records as one 32-bit id: depth * pixels
// + pixel, pixels = the image's pixel count.
NMG_HD uint32_t vertex_id(int depth, uint32_t pixel, uint32_t pixels) { return uint32_t(depth) * pixels + pixel; }

}  // namespace nmg
