// frame.cu -- one frame's bounce loop captured as a CUDA graph.
//
// The reference's wavefront integrator runs, per bounce, the guided query of
// that bounce's scatter queue and then (integrator.cpp:431-438, 463, 650-701)
// training steps on the records gathered so far. Queue lengths change from
// bounce to bounce and frame to frame, but they live in device memory
// (d_count), so the sequence of launches -- one fused query kernel per
// bounce, each followed by its training step -- is the same every frame.
// nmg_frame_capture records that sequence once into a CUDA graph; each
// nmg_frame_launch replays all of it with one host call. Every kernel reads
// its sizes and the optimiser step from device memory, so replays stay
// correct as counts and step numbers change.
#include <new>

#include "api_common.cuh"
#include "ctx.cuh"

struct nmg_frame {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int n_bounces = 0;
  int launches = 0;  // graph nodes (kernels and memsets) per replay
};

using namespace nmg;

static void frame_free(nmg_frame* f) {
  if (!f) return;
  if (f->exec) cudaGraphExecDestroy(f->exec);
  if (f->graph) cudaGraphDestroy(f->graph);
  delete f;
}

static nmg_status record_bounces(nmg_ctx* c, const nmg_bounce* b, int nb, cudaStream_t s) {
  for (int i = 0; i < nb; ++i) {
    nmg_status st = nmg_query(c, &b[i].in, b[i].u4, b[i].d_count, b[i].n_max, &b[i].out, s);
    if (st != NMG_OK) return st;
    if (b[i].train_x) {
      st = nmg_train_step(c, b[i].train_x, b[i].train_records, b[i].train_count, b[i].train_n_max, b[i].stats, s);
      if (st != NMG_OK) return st;
    }
  }
  return NMG_OK;
}

extern "C" {

nmg_status nmg_frame_capture(nmg_ctx* c, const nmg_bounce* bounces, int n_bounces, nmg_frame** out) {
  NMG_REQUIRE(c && bounces && out, "NULL argument");
  NMG_REQUIRE(n_bounces >= 1 && n_bounces <= 64, "n_bounces=%d (1..64)", n_bounces);
  *out = nullptr;
  for (int i = 0; i < n_bounces; ++i) {
    const nmg_bounce& b = bounces[i];
    NMG_REQUIRE(b.n_max >= 1 && b.n_max <= c->ws.cap_q, "bounce %d: n_max=%d outside 1..%d", i, b.n_max,
                c->ws.cap_q);
    NMG_REQUIRE(!b.train_x || (b.train_records && b.train_n_max >= 1 && b.train_n_max <= c->ws.cap_b),
                "bounce %d: training batch of %d outside 1..%d or without records", i, b.train_n_max, c->ws.cap_b);
  }
  nmg_frame* f = new (std::nothrow) nmg_frame();
  if (!f) return set_error(NMG_ERR_OOM, "host allocation failed");
  f->n_bounces = n_bounces;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    frame_free(f);
    return set_error(NMG_ERR_CUDA, "cudaStreamCreateWithFlags: %s", cudaGetErrorString(e));
  }
  // Relaxed mode: the first launch of a kernel may set its shared-memory
  // attribute, which is not a stream operation.
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    cudaStreamDestroy(s);
    frame_free(f);
    return set_error(NMG_ERR_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e));
  }
  nmg_status st = record_bounces(c, bounces, n_bounces, s);
  e = cudaStreamEndCapture(s, &f->graph);
  cudaStreamDestroy(s);
  if (st != NMG_OK) {
    frame_free(f);
    return st;
  }
  if (e != cudaSuccess) {
    frame_free(f);
    return set_error(NMG_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
  }
  size_t nodes = 0;
  cudaGraphGetNodes(f->graph, nullptr, &nodes);
  f->launches = int(nodes);
  e = cudaGraphInstantiate(&f->exec, f->graph, 0);
  if (e != cudaSuccess) {
    frame_free(f);
    return set_error(NMG_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  }
  *out = f;
  return NMG_OK;
}

nmg_status nmg_frame_launch(nmg_frame* f, nmg_stream stream) {
  NMG_REQUIRE(f && f->exec, "frame is NULL");
  NMG_CUDA_TRY(cudaGraphLaunch(f->exec, (cudaStream_t)stream));
  return NMG_OK;
}

int nmg_frame_nodes(const nmg_frame* f) { return f ? f->launches : 0; }

void nmg_frame_destroy(nmg_frame* f) { frame_free(f); }

nmg_status nmg_frame_run_eager(nmg_ctx* c, const nmg_bounce* bounces, int n_bounces, nmg_stream stream) {
  NMG_REQUIRE(c && bounces, "NULL argument");
  NMG_REQUIRE(n_bounces >= 1 && n_bounces <= 64, "n_bounces=%d (1..64)", n_bounces);
  return record_bounces(c, bounces, n_bounces, (cudaStream_t)stream);
}

}  // extern "C"
