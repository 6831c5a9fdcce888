// ref_shim.cu -- extern "C" wrapper around the reference's OWN host-callable
// mixture code (TEST INFRASTRUCTURE ONLY).
//
// oracle/build_ref.sh compiles this file against the reference sources in
// place (src/render/guided/distribution.h, src/backend/src/util/vmf.h,
// src/render/guided/train.h, src/backend/src/util/math_utils.h) into
// oracle/_ref/libnmgref.so. Nothing here restates the mixture arithmetic:
// activation, pdf, sampling, the cosine-lobe product and gradients_probability
// are the reference's functions. Two things are written around them:
//   * ReplaySampler feeds given uniforms to MixedSphericalGaussianDistribution
//     ::sample (distribution.h:132-140), which otherwise draws them from the
//     renderer's per-pixel sampler;
//   * ref_loss_grad restates the per-sample body of the __global__ kernel
//     compute_dL_doutput_divergence (train.cu:80-123) around the compiled
//     gradients_probability and d_network_to_d_params, with the same __half
//     storage of raw outputs and gradients as the reference's training path.
// The reference fixes K = NUM_VMF_COMPONENTS = 8 at compile time
// (parameters.h:10), so these entry points handle K = 8 only.
#include "core/sampler.h"
#include "raytracing.h"
#include "render/guided/train.h"
#include "render/sampling.h"
#include "render/shared.h"
#include "util/math_utils.h"

namespace krr {
struct ReplaySampler {
  const float* u;
  int i;
  KRR_CALLABLE float get1D() { return u[i++]; }
  KRR_CALLABLE Vector2f get2D() {
    float a = u[i++];
    float b = u[i++];
    return {a, b};
  }
};
}  // namespace krr

// Route distribution.h's `Sampler&` parameter to the replay sampler; the
// renderer's Sampler class is already declared above, so only the text of
// distribution.h sees the rename.
#define Sampler ReplaySampler
#include "render/guided/distribution.h"
#undef Sampler

using namespace krr;
using Mix = MixedSphericalGaussianDistribution<NUM_VMF_COMPONENTS>;

extern "C" {

int ref_num_lobes(void) { return NUM_VMF_COMPONENTS; }

// Samples one direction per query with uniforms u4[q] = (u_guide, u_lobe,
// u_dir0, u_dir1). The selected lobe is reported as the lobe whose own
// VMFKernel::sample reproduces the direction bit for bit.
void ref_mixture_sample(const float* raw, int stride, long n, const float* u4, const float* cos_normal,
                        float* dir, float* pdf, int* lobe) {
  for (long q = 0; q < n; ++q) {
    Mix m(raw + q * stride);
    if (cos_normal) m.applyCosineLobe(Vector3f(cos_normal[3 * q], cos_normal[3 * q + 1], cos_normal[3 * q + 2]));
    ReplaySampler s{u4 + 4 * q + 1, 0};
    Vector3f d = m.sample(s);
    dir[3 * q] = d[0];
    dir[3 * q + 1] = d[1];
    dir[3 * q + 2] = d[2];
    pdf[q] = m.pdf(d);
    if (lobe) {
      lobe[q] = -1;
      Vector2f u2(u4[4 * q + 2], u4[4 * q + 3]);
      for (int i = 0; i < NUM_VMF_COMPONENTS; ++i) {
        Vector3f di = m.get(i).sample(u2);
        if (di[0] == d[0] && di[1] == d[1] && di[2] == d[2]) {
          lobe[q] = i;
          break;
        }
      }
    }
  }
}

void ref_mixture_pdf(const float* raw, int stride, long n, const float* wi, const float* cos_normal, float* pdf) {
  for (long q = 0; q < n; ++q) {
    Mix m(raw + q * stride);
    if (cos_normal) m.applyCosineLobe(Vector3f(cos_normal[3 * q], cos_normal[3 * q + 1], cos_normal[3 * q + 2]));
    pdf[q] = m.pdf(Vector3f(wi[3 * q], wi[3 * q + 1], wi[3 * q + 2]));
  }
}

// train.cu:80-123 per-sample body. raw: n x stride FP32 values that are
// rounded to __half on entry (network outputs are __half in the reference's
// training path); sample: n x 6 GuidedOutput {theta, phi, L rgb, wiPdf}.
// grad: n x stride FP32 copies of the __half gradients; loss: n floats.
void ref_loss_grad(const float* raw, int stride, long n, const float* sample, float loss_scale,
                   float* grad, float* loss) {
  const int N = NUM_VMF_COMPONENTS * N_DIM_VMF;
  for (long tid = 0; tid < n; ++tid) {
    precision_t data[N_DIM_PADDED_OUTPUT], gradient_data[N_DIM_PADDED_OUTPUT];
    for (int k = 0; k < N; ++k) data[k] = (precision_t)raw[tid * stride + k];
    float ls = loss_scale / (float)n;
    MixedSphericalGaussianDistribution<NUM_VMF_COMPONENTS> dist(data);
    const float* s = sample + tid * 6;
    Vector3f wi = utils::sphericalToCartesian(s[0], s[1]);
    Color L(s[2], s[3], s[4]);
    float Li = L.mean();
    float wiPdf = s[5] + M_EPSILON;
    float guidePdf = dist.gradients_probability(wi, gradient_data) + M_EPSILON;
    float prefix = -Li / wiPdf / guidePdf * ls;
    loss[tid] = -Li / wiPdf * logf(guidePdf);
    for (int sg = 0; sg < NUM_VMF_COMPONENTS; sg++) {
      precision_t* cur_params = data + sg * N_DIM_VMF;
      float lambda_r = cur_params[0], kappa_r = cur_params[1], theta_r = cur_params[2], phi_r = cur_params[3];
      precision_t* g = gradient_data + sg * N_DIM_VMF;
      g[0] = LR_LAMBDA * prefix * (float)g[0] * d_network_to_d_params(lambda_r, ACTIVATION_LAMBDA);
      g[1] = LR_KAPPA * prefix * (float)g[1] * d_network_to_d_params(kappa_r, ACTIVATION_KAPPA);
      g[2] = LR_THETA * prefix * (float)g[2] * M_PI * d_network_to_d_params(theta_r, ACTIVATION_THETA);
      g[3] = LR_PHI * prefix * (float)g[3] * M_2PI * d_network_to_d_params(phi_r, ACTIVATION_PHI);
    }
    for (int i = 0; i < N_DIM_OUTPUT; i++)
      if (isnan((float)gradient_data[i]) || isinf((float)gradient_data[i])) gradient_data[i] = (precision_t)0.f;
    for (int i = 0; i < N_DIM_OUTPUT; i++) gradient_data[i] = min(150.f, (float)gradient_data[i]);
    for (int k = 0; k < N; ++k) grad[tid * stride + k] = (float)gradient_data[k];
  }
}

}  // extern "C"
