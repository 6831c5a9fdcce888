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
//   * the __global__ kernels of train.cu (training-record extraction, the
//     KL loss and its adjoint, inference featurisation) are compiled as host
//     functions from the reference's own source and run once per thread
//     index (second half of this file).
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

}  // extern "C"

// ---------------------------------------------------------------------------
// The reference's own __global__ kernels of src/render/guided/train.cu, run
// on the host. Their bodies are compiled unchanged as host functions: the
// kernel qualifier is redefined to __host__ and the thread-index built-ins
// read host variables that the loops below set for every thread index, as a
// one-dimensional launch of 256-thread blocks would. Everything the bodies
// call is host-callable in the reference (KRR_CALLABLE): the mixture,
// TrainBuffer::push (atomic<int> falls back to std::atomic on the host),
// the SOA accessors, normalizeSpatialCoord and the warp_* helpers. The
// thread indices are visited in order, so pushes land in the reference's
// loop order (training pixel, then depth).
// ---------------------------------------------------------------------------
#include "render/guided/workqueue.h"
#include "render/wavefront/workqueue.h"

namespace nmg_host_launch {
uint3 thread_idx, block_idx;
dim3 block_dim;
inline void set(size_t tid) {
  thread_idx = make_uint3(unsigned(tid % 256), 0, 0);
  block_idx = make_uint3(unsigned(tid / 256), 0, 0);
  block_dim = dim3(256, 1, 1);
}
}  // namespace nmg_host_launch

#pragma push_macro("__global__")
#undef __global__
#define __global__ __host__
#define threadIdx ::nmg_host_launch::thread_idx
#define blockIdx ::nmg_host_launch::block_idx
#define blockDim ::nmg_host_launch::block_dim
// train.h already declares the kernels as __global__: the host definitions
// get names of their own
#define generate_training_data host_generate_training_data
#define compute_dL_doutput_divergence host_compute_dL_doutput_divergence
#define compute_dL_doutput_with_selection host_compute_dL_doutput_with_selection
#define generate_inference_data host_generate_inference_data
#include "render/guided/train.cu"
#undef generate_training_data
#undef compute_dL_doutput_divergence
#undef compute_dL_doutput_with_selection
#undef generate_inference_data
#undef threadIdx
#undef blockIdx
#undef blockDim
#pragma pop_macro("__global__")

namespace {
// Host memory for the reference's SOA containers (its Allocator is a
// polymorphic allocator over this interface, core/interop.h).
struct HostResource : krr::inter::memory_resource {
  void* do_allocate(size_t bytes, size_t alignment) override {
    return aligned_alloc(alignment < 16 ? 16 : alignment, (bytes + 15) / 16 * 16);
  }
  void do_deallocate(void* p, size_t, size_t) override { free(p); }
  bool do_is_equal(const memory_resource& o) const noexcept override { return this == &o; }
};
HostResource g_host_res;

// TrainBuffer keeps its storage pointers private and allocates them with
// cudaMalloc; this mirror of its member layout (train.h:158-162) points them
// at host arrays instead.
struct TrainBufferMirror {
  krr::atomic<int> mSize;
  GuidedInput* mInputs;
  GuidedOutput* mOutputs;
  int mMaxSize;
};
static_assert(sizeof(TrainBufferMirror) == sizeof(TrainBuffer), "TrainBuffer layout changed");
}  // namespace

extern "C" {

int ref_guided_input_floats(void) { return int(sizeof(GuidedInput) / sizeof(float)); }
int ref_guided_output_floats(void) { return int(sizeof(GuidedOutput) / sizeof(float)); }

// generate_training_data (train.cu:14-67) over a GuidedPixelStateBuffer whose
// per-depth field arrays are the caller's host arrays, laid out exactly as the
// reference's soac-generated SOA<RadianceRecordItem> stores them: per depth d
// and pixel p, L/thp/bsdf_val [d][p][3], pos [d][p][3], dir/wo/normal
// [d][p][2], wi_pdf/bsdf_pdf/mis_weight/roughness [d][p], delta [d][p] (bool).
// Depths beyond n_depth get no arrays (cur_depth must stay <= n_depth).
// Writes up to `capacity` GuidedInput rows to x and GuidedOutput rows to out;
// returns the number of records pushed.
int ref_generate_training_data(const float* L, const float* thp, const float* pos, const float* dir,
                               const float* wi_pdf, const float* bsdf_pdf, const float* mis_weight,
                               const unsigned char* delta, const float* bsdf_val, const float* wo,
                               const float* normal, const float* roughness, const unsigned* cur_depth,
                               int n_pixels, int n_depth, const unsigned* offset, const unsigned* stride,
                               const unsigned* train_res, const unsigned* res, const float* aabb, int capacity,
                               float* x, float* out) {
  GuidedPixelStateBuffer state;
  state.nAlloc = n_pixels;
  for (int d = 0; d < int(MAX_TRAIN_DEPTH); ++d) {
    auto& r = state.records[d];
    r.nAlloc = n_pixels;
    if (d >= n_depth) continue;
    const size_t p = size_t(d) * n_pixels;
    r.L = (Color*)(L + 3 * p);
    r.thp = (Color*)(thp + 3 * p);
    r.pos = (Vector3f*)(pos + 3 * p);
    r.dir = (Vector2f*)(dir + 2 * p);
    r.wiPdf = (float*)(wi_pdf + p);
    r.bsdfPdf = (float*)(bsdf_pdf + p);
    r.misWeight = (float*)(mis_weight + p);
    r.delta = (bool*)(delta + p);
    r.bsdfVal = (Color*)(bsdf_val + 3 * p);
    r.wo = (Vector2f*)(wo + 2 * p);
    r.normal = (Vector2f*)(normal + 2 * p);
    r.roughness = (float*)(roughness + p);
  }
  state.curDepth = (uint*)cur_depth;
  TrainBuffer tb;
  auto* m = reinterpret_cast<TrainBufferMirror*>(&tb);
  m->mSize.store(0);
  m->mInputs = reinterpret_cast<GuidedInput*>(x);
  m->mOutputs = reinterpret_cast<GuidedOutput*>(out);
  m->mMaxSize = capacity;
  const AABB box(Vector3f(aabb[0], aabb[1], aabb[2]), Vector3f(aabb[3], aabb[4], aabb[5]));
  const size_t n = size_t(train_res[0]) * train_res[1];
  for (size_t tid = 0; tid < n; ++tid) {
    nmg_host_launch::set(tid);
    host_generate_training_data(n, Vector2ui(offset[0], offset[1]), Vector2ui(stride[0], stride[1]),
                           Vector2ui(train_res[0], train_res[1]), Vector2ui(res[0], res[1]), &tb, &state, box);
  }
  return m->mSize.load();
}

// generate_inference_data (train.cu:174-191) over a ScatterRayQueue (the
// soac-generated SOA<ScatterRayWorkItem>, workitem.soa:89-94) filled on the
// host through the queue's own push(). Inputs: per query sd.pos, sd.wo
// (not necessarily unit), sd.frame.N [n][3] and sd.roughness [n]. Outputs:
// the network input rows x[n][N_DIM_INPUT] and, copied back out of the
// queue's own field arrays, the SOA leaves sd.pos / sd.wo / sd.frame.N
// ([n][3] each) and sd.roughness ([n]) with the bytes the queue holds.
int ref_generate_inference_data(const float* pos, const float* wo, const float* nrm, const float* rough, int n,
                                const float* aabb, float* x, float* soa_pos, float* soa_wo, float* soa_n,
                                float* soa_rough) {
  Allocator alloc(&g_host_res);
  ScatterRayQueue q(n, alloc);
  for (int i = 0; i < n; ++i) {
    ScatterRayWorkItem w = {};
    w.sd.pos = Vector3f(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    w.sd.wo = Vector3f(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    w.sd.frame.N = Vector3f(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    w.sd.roughness = rough[i];
    w.pixelId = unsigned(i);
    q.push(w);
  }
  static_assert(sizeof(Vector3f) == 3 * sizeof(float), "Vector3f is not a packed float triple");
  memcpy(soa_pos, q.sd.pos, sizeof(float) * 3 * size_t(n));
  memcpy(soa_wo, q.sd.wo, sizeof(float) * 3 * size_t(n));
  memcpy(soa_n, q.sd.frame.N, sizeof(float) * 3 * size_t(n));
  memcpy(soa_rough, q.sd.roughness, sizeof(float) * size_t(n));
  const AABB box(Vector3f(aabb[0], aabb[1], aabb[2]), Vector3f(aabb[3], aabb[4], aabb[5]));
  for (int i = 0; i < n; ++i) {
    nmg_host_launch::set(size_t(i));
    host_generate_inference_data(size_t(n), &q, x, box);
  }
  return N_DIM_INPUT;
}

// compute_dL_doutput_divergence (train.cu:69-124) itself: raw rows of
// N_DIM_PADDED_OUTPUT values rounded to precision_t (__half), GuidedOutput
// samples [n][6]; writes the __half gradient rows (as float) and the per-sample
// likelihood.
void ref_dL_doutput_divergence(const float* raw, int stride, long n, const float* sample, float loss_scale,
                               float* grad, float* loss) {
  std::vector<precision_t> pred(size_t(n) * N_DIM_PADDED_OUTPUT), dl(size_t(n) * N_DIM_PADDED_OUTPUT);
  for (long q = 0; q < n; ++q)
    for (int k = 0; k < N_DIM_PADDED_OUTPUT; ++k)
      pred[size_t(q) * N_DIM_PADDED_OUTPUT + k] = (precision_t)(k < stride ? raw[q * stride + k] : 0.f);
  std::vector<GuidedOutput> ref(n);
  for (long q = 0; q < n; ++q) memcpy(&ref[q], sample + 6 * q, sizeof(GuidedOutput));
  for (long tid = 0; tid < n; ++tid) {
    nmg_host_launch::set(size_t(tid));
    host_compute_dL_doutput_divergence(size_t(n), pred.data(), ref.data(), dl.data(), loss, loss_scale,
                                  EDivergence::KL);
  }
  const int N = NUM_VMF_COMPONENTS * N_DIM_VMF;
  for (long q = 0; q < n; ++q)
    for (int k = 0; k < N; ++k) grad[q * stride + k] = (float)dl[size_t(q) * N_DIM_PADDED_OUTPUT + k];
}

}  // extern "C"
