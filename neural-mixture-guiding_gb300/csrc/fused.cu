// fused.cu -- placeholder until the tcgen05 kernels land.
#include "api_common.cuh"
#include "ctx.cuh"
namespace nmg {
nmg_status fused_reserve(nmg_ctx*) { return NMG_OK; }
nmg_status fused_query(nmg_ctx*, const nmg_shading*, const float*, const int*, int, const nmg_query_out*, cudaStream_t) {
  return set_error(NMG_ERR_UNSUPPORTED, "fused path not built");
}
nmg_status fused_infer_raw(nmg_ctx*, const float*, const int*, int, int, float*, cudaStream_t) {
  return set_error(NMG_ERR_UNSUPPORTED, "fused path not built");
}
nmg_status fused_train_step(nmg_ctx*, const float*, const float*, const int*, int, double*, cudaStream_t) {
  return set_error(NMG_ERR_UNSUPPORTED, "fused path not built");
}
}  // namespace nmg
