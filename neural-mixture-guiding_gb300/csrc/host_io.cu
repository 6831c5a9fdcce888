// host_io.cu -- query and training entry points on HOST buffers.
//
// A caller whose wavefront lives in host memory (the reference's CPU-side
// callers, or a renderer that keeps its queues on the host) would otherwise
// copy all inputs to the device, run the query, and copy the outputs back,
// one after another. These entry points split the wavefront into chunks and
// pipeline them on three streams: chunk i+1's inputs go host->device while
// chunk i is computed and chunk i-1's outputs go device->host. With pinned
// host buffers the copies overlap the fused kernel almost entirely.
//
// Ordering: the kernels run on the caller's stream after the work already
// queued there, and `stream` waits for the last output copy. The query
// inputs are staged in two alternating device buffers: a call's input copies
// wait only until the kernels of the call before the previous one have read
// its buffer, so they overlap whatever else the stream is still running (the
// previous query and the training step queued after it, for instance): the
// host input arrays must be ready when the call is made. The device staging
// buffers are allocated on the first call (sized to the reserved capacity)
// and reused; that first call is therefore not capturable.
//
// Outputs in pinned (page-locked, device-mapped) host memory are written by
// the query kernel itself through the mapping: its stores cross the host
// link as it produces them, with no staging, no copy after the last chunk
// and no copy stream in the way (a query pass plus training step of
// 1920x1080 queries measured 1.20 ms per step this way against 1.24 ms with
// staged outputs). Pageable outputs are staged and copied back.
#include <string.h>

#include <new>

#include "api_common.cuh"
#include "ctx.cuh"

namespace nmg {

// The first chunk's inputs and the last chunk's outputs cannot overlap a
// kernel, so more, smaller chunks shorten that exposed copy time, but every
// chunk is one more launch of the persistent query kernel, whose pipeline
// fill and last-round imbalance cost ~19 us per launch: a 1920x1080 query
// pass plus training step on host buffers measured 1.39 ms with 4 chunks,
// 1.41 with 2, 1.42 with 7 and 1.58 with 15 (even chunks), and 1.32 ms once
// the last of 4 chunks is half the size of the others. Below about 2^18
// queries a chunk leaves the persistent grid underfilled. With outputs
// written through the mapping there is no output copy at the end, and the
// chunks are of equal size. When the caller's stream still has work queued
// (back-to-back guiding steps), the input copies run under that work and
// need no chunks: 1920x1080 queries plus a training step measured 1.148 ms
// per step with one chunk and 1.171 with 2, against 1.093 ms with
// device-resident buffers.
constexpr int kAutoChunks = 4;
constexpr int kMaxChunks = 8;
constexpr int kMinChunk = 1 << 18;

struct HostIO {
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaEvent_t start = nullptr, done = nullptr;
  // recorded after the kernels that read each query input slot / the training input staging
  cudaEvent_t q_consumed[2] = {}, t_consumed = nullptr;
  cudaEvent_t in_ready[kMaxChunks] = {}, out_ready[kMaxChunks] = {};
  int cap_q = 0, cap_b = 0;
  int q_slot = 0;  // input slot of the next query call
  // query input staging (SoA, device), two slots
  float *pos[2] = {}, *wo[2] = {}, *nrm[2] = {}, *rough[2] = {}, *u4[2] = {};
  // query output staging (for pageable host outputs)
  float *dir = nullptr, *pdf = nullptr, *sel = nullptr;
  int* lobe = nullptr;
  // training staging
  float *x = nullptr, *rec = nullptr;
  double* stats = nullptr;  // [2] device copy of the step's statistics
};

static void free_staging_q(HostIO* h) {
  for (int s = 0; s < 2; ++s) {
    for (float* p : {h->pos[s], h->wo[s], h->nrm[s], h->rough[s], h->u4[s]}) cudaFree(p);
    h->pos[s] = h->wo[s] = h->nrm[s] = h->rough[s] = h->u4[s] = nullptr;
  }
  for (float* p : {h->dir, h->pdf, h->sel}) cudaFree(p);
  cudaFree(h->lobe);
  h->dir = h->pdf = h->sel = nullptr;
  h->lobe = nullptr;
  h->cap_q = 0;
}

static void free_staging_b(HostIO* h) {
  cudaFree(h->x);
  cudaFree(h->rec);
  cudaFree(h->stats);
  h->x = h->rec = nullptr;
  h->stats = nullptr;
  h->cap_b = 0;
}

void host_io_release(nmg_ctx* c) {
  HostIO* h = static_cast<HostIO*>(c->host_io);
  if (!h) return;
  free_staging_q(h);
  free_staging_b(h);
  if (h->h2d) cudaStreamDestroy(h->h2d);
  if (h->d2h) cudaStreamDestroy(h->d2h);
  if (h->start) cudaEventDestroy(h->start);
  if (h->done) cudaEventDestroy(h->done);
  for (cudaEvent_t e : h->q_consumed)
    if (e) cudaEventDestroy(e);
  if (h->t_consumed) cudaEventDestroy(h->t_consumed);
  for (int i = 0; i < kMaxChunks; ++i) {
    if (h->in_ready[i]) cudaEventDestroy(h->in_ready[i]);
    if (h->out_ready[i]) cudaEventDestroy(h->out_ready[i]);
  }
  delete h;
  c->host_io = nullptr;
}

static nmg_status host_io_get(nmg_ctx* c, HostIO** out) {
  HostIO* h = static_cast<HostIO*>(c->host_io);
  if (!h) {
    h = new (std::nothrow) HostIO();
    if (!h) return set_error(NMG_ERR_OOM, "host allocation failed");
    c->host_io = h;
    const unsigned ef = cudaEventDisableTiming;
    bool ok = cudaStreamCreateWithFlags(&h->h2d, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&h->d2h, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&h->start, ef) == cudaSuccess &&
              cudaEventCreateWithFlags(&h->done, ef) == cudaSuccess &&
              cudaEventCreateWithFlags(&h->q_consumed[0], ef) == cudaSuccess &&
              cudaEventCreateWithFlags(&h->q_consumed[1], ef) == cudaSuccess &&
              cudaEventCreateWithFlags(&h->t_consumed, ef) == cudaSuccess;
    for (int i = 0; ok && i < kMaxChunks; ++i)
      ok = cudaEventCreateWithFlags(&h->in_ready[i], ef) == cudaSuccess &&
           cudaEventCreateWithFlags(&h->out_ready[i], ef) == cudaSuccess;
    if (!ok) {
      host_io_release(c);
      return set_error(NMG_ERR_CUDA, "creating the copy streams failed");
    }
  }
  *out = h;
  return NMG_OK;
}

template <class T>
static bool alloc_n(T** p, size_t n) {
  return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T)) == cudaSuccess;
}

static nmg_status ensure_staging_q(HostIO* h, int cap) {
  if (h->cap_q >= cap) return NMG_OK;
  free_staging_q(h);
  const size_t n = size_t(cap);
  bool ok = alloc_n(&h->dir, 3 * n) && alloc_n(&h->pdf, n) && alloc_n(&h->sel, n) && alloc_n(&h->lobe, n);
  for (int s = 0; ok && s < 2; ++s)
    ok = alloc_n(&h->pos[s], 3 * n) && alloc_n(&h->wo[s], 3 * n) && alloc_n(&h->nrm[s], 3 * n) &&
         alloc_n(&h->rough[s], n) && alloc_n(&h->u4[s], 4 * n);
  if (!ok) {
    free_staging_q(h);
    return set_error(NMG_ERR_OOM, "query staging for %d queries", cap);
  }
  h->cap_q = cap;
  return NMG_OK;
}

static nmg_status ensure_staging_b(HostIO* h, int cap, int n_input, int rfloats) {
  if (h->cap_b >= cap) return NMG_OK;
  free_staging_b(h);
  const bool ok = alloc_n(&h->x, size_t(cap) * n_input) && alloc_n(&h->rec, size_t(cap) * rfloats) &&
                  alloc_n(&h->stats, 2);
  if (!ok) {
    free_staging_b(h);
    return set_error(NMG_ERR_OOM, "training staging for %d records", cap);
  }
  h->cap_b = cap;
  return NMG_OK;
}

#define NMG_CU(call)                                                                            \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return set_error(NMG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

static nmg_status h2d(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  NMG_CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
  return NMG_OK;
}
static nmg_status d2h(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  NMG_CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
  return NMG_OK;
}

// The device address of pinned host memory (NULL stays NULL), or nullptr
// with *ok = false when `p` is not page-locked and mapped.
template <class T>
static T* mapped(T* p, bool* ok) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();  // not a CUDA pointer: clear the (non-sticky) error
    *ok = false;
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) {
    *ok = false;
    return nullptr;
  }
  return static_cast<T*>(a.devicePointer);
}

}  // namespace nmg

using namespace nmg;

extern "C" {

nmg_status nmg_query_host(nmg_ctx* c, const nmg_shading* in, const float* u4, int n, const nmg_query_out* out,
                          nmg_stream stream) {
  NMG_REQUIRE(c && in && out, "NULL argument");
  NMG_REQUIRE(n >= 0 && n <= c->ws.cap_q, "n=%d outside 0..%d (call nmg_reserve)", n, c->ws.cap_q);
  if (n == 0) return NMG_OK;
  NMG_REQUIRE(in->pos && in->wo && in->normal && in->roughness && u4 && out->dir && out->pdf,
              "NULL shading array, uniforms or output");
  NMG_REQUIRE(!out->raw, "raw outputs are not returned by nmg_query_host (use nmg_query)");
  HostIO* h = nullptr;
  nmg_status s = host_io_get(c, &h);
  if (s != NMG_OK) return s;
  if ((s = ensure_staging_q(h, c->ws.cap_q)) != NMG_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  // outputs written through the mapping when every one given is pinned host memory
  bool direct = true;
  float* m_dir = mapped(out->dir, &direct);
  float* m_pdf = mapped(out->pdf, &direct);
  int* m_lobe = mapped(out->lobe, &direct);
  float* m_sel = mapped(out->selection, &direct);
  // inputs: only after the kernels that last read this slot (an event never recorded yet
  // is complete); staged outputs: after the stream's work
  const int slot = h->q_slot;
  h->q_slot ^= 1;
  NMG_CU(cudaStreamWaitEvent(h->h2d, h->q_consumed[slot], 0));
  if (!direct) {
    NMG_CU(cudaEventRecord(h->start, st));
    NMG_CU(cudaStreamWaitEvent(h->d2h, h->start, 0));
  }
  int limit = c->host_chunks;
  if (limit <= 0) {
    // automatic: with work still queued on `stream` the copies run under it, and one chunk
    // saves the per-launch cost; on an idle stream nothing hides the first chunk's copy
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const bool capturing = cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone;
    const cudaError_t q = capturing ? cudaSuccess : cudaStreamQuery(st);
    if (q == cudaErrorNotReady && cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
    limit = q == cudaErrorNotReady ? 1 : kAutoChunks;
  }
  int chunks = n / kMinChunk;
  chunks = chunks < 1 ? 1 : (chunks > limit ? limit : chunks);
  // staged outputs: the last chunk's are copied back after every kernel has run, so it gets
  // half an even share and the others split the rest
  const int last = chunks > 1 ? (direct ? n / chunks : n / (2 * chunks)) : n;
  const int per = chunks > 1 ? (n - last + chunks - 2) / (chunks - 1) : n;
  float *pos = h->pos[slot], *wo = h->wo[slot], *nrm = h->nrm[slot], *rough = h->rough[slot], *hu4 = h->u4[slot];
  for (int i = 0; i < chunks; ++i) {
    const size_t o = size_t(i) * per;
    if (o >= size_t(n)) break;
    const int m = i == chunks - 1 ? int(size_t(n) - o) : int(size_t(n) - o < size_t(per) ? size_t(n) - o : size_t(per));
    if (m <= 0) break;
    const size_t f = sizeof(float);
    if ((s = h2d(pos + 3 * o, in->pos + 3 * o, 3 * f * m, h->h2d)) != NMG_OK ||
        (s = h2d(wo + 3 * o, in->wo + 3 * o, 3 * f * m, h->h2d)) != NMG_OK ||
        (s = h2d(nrm + 3 * o, in->normal + 3 * o, 3 * f * m, h->h2d)) != NMG_OK ||
        (s = h2d(rough + o, in->roughness + o, f * m, h->h2d)) != NMG_OK ||
        (s = h2d(hu4 + 4 * o, u4 + 4 * o, 4 * f * m, h->h2d)) != NMG_OK)
      return s;
    NMG_CU(cudaEventRecord(h->in_ready[i], h->h2d));
    NMG_CU(cudaStreamWaitEvent(st, h->in_ready[i], 0));
    const nmg_shading din{pos + 3 * o, wo + 3 * o, nrm + 3 * o, rough + o};
    if (direct) {
      const nmg_query_out dout{m_dir + 3 * o, m_pdf + o, m_lobe ? m_lobe + o : nullptr, nullptr,
                               m_sel ? m_sel + o : nullptr};
      if ((s = nmg_query(c, &din, hu4 + 4 * o, nullptr, m, &dout, stream)) != NMG_OK) return s;
      continue;
    }
    const nmg_query_out dout{h->dir + 3 * o, h->pdf + o, out->lobe ? h->lobe + o : nullptr, nullptr,
                             out->selection ? h->sel + o : nullptr};
    if ((s = nmg_query(c, &din, hu4 + 4 * o, nullptr, m, &dout, stream)) != NMG_OK) return s;
    NMG_CU(cudaEventRecord(h->out_ready[i], st));
    NMG_CU(cudaStreamWaitEvent(h->d2h, h->out_ready[i], 0));
    if ((s = d2h(out->dir + 3 * o, h->dir + 3 * o, 3 * f * m, h->d2h)) != NMG_OK ||
        (s = d2h(out->pdf + o, h->pdf + o, f * m, h->d2h)) != NMG_OK)
      return s;
    if (out->lobe && (s = d2h(out->lobe + o, h->lobe + o, sizeof(int) * m, h->d2h)) != NMG_OK) return s;
    if (out->selection && (s = d2h(out->selection + o, h->sel + o, f * m, h->d2h)) != NMG_OK) return s;
  }
  NMG_CU(cudaEventRecord(h->q_consumed[slot], st));
  if (!direct) {
    NMG_CU(cudaEventRecord(h->done, h->d2h));
    NMG_CU(cudaStreamWaitEvent(st, h->done, 0));
  }
  return NMG_OK;
}

nmg_status nmg_set_host_chunks(nmg_ctx* c, int chunks) {
  NMG_REQUIRE(c != nullptr, "ctx is NULL");
  NMG_REQUIRE(chunks >= 0 && chunks <= kMaxChunks, "chunks=%d outside 0..%d (0 = automatic)", chunks, kMaxChunks);
  c->host_chunks = chunks;
  return NMG_OK;
}

int nmg_get_host_chunks(const nmg_ctx* c) { return c ? (c->host_chunks > 0 ? c->host_chunks : kAutoChunks) : -1; }

nmg_status nmg_train_step_host(nmg_ctx* c, const float* x, const float* records, int n, double* stats,
                               nmg_stream stream) {
  NMG_REQUIRE(c && x && records, "NULL argument");
  NMG_REQUIRE(n >= 0 && n <= c->ws.cap_b, "n=%d outside 0..%d (call nmg_reserve)", n, c->ws.cap_b);
  HostIO* h = nullptr;
  nmg_status s = host_io_get(c, &h);
  if (s != NMG_OK) return s;
  const int ni = c->enc.n_input, rf = c->lay.record_floats;
  if ((s = ensure_staging_b(h, c->ws.cap_b > 1 ? c->ws.cap_b : 1, ni, rf)) != NMG_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  NMG_CU(cudaStreamWaitEvent(h->h2d, h->t_consumed, 0));
  if ((s = h2d(h->x, x, sizeof(float) * size_t(n) * ni, h->h2d)) != NMG_OK ||
      (s = h2d(h->rec, records, sizeof(float) * size_t(n) * rf, h->h2d)) != NMG_OK)
    return s;
  NMG_CU(cudaEventRecord(h->in_ready[0], h->h2d));
  NMG_CU(cudaStreamWaitEvent(st, h->in_ready[0], 0));
  // statistics in pinned host memory are written by the kernel through the mapping
  bool direct = true;
  double* m_stats = mapped(stats, &direct);
  double* d_stats = stats ? (direct ? m_stats : h->stats) : nullptr;
  if ((s = nmg_train_step(c, h->x, h->rec, nullptr, n, d_stats, stream)) != NMG_OK) return s;
  NMG_CU(cudaEventRecord(h->t_consumed, st));
  if (stats && !direct) s = d2h(stats, h->stats, 2 * sizeof(double), st);
  return s;
}

}  // extern "C"
