// ref_tcnn_layout.cu -- the parameter layout of tiny-cuda-nn 1.7's grid
// encoding as its own constructor computes it (TEST INFRASTRUCTURE ONLY).
//
// oracle/build_ref.sh compiles this file against the reference's unmodified
// tcnn headers. GridEncodingTemplated's constructor (grid.h:939-1000) sizes
// every level (the dense resolution^3 rounded up to a multiple of 8, capped
// by the hash table size) and lays the levels out back to back; nothing on
// the device is touched. The offsets and the parameter count it reports pin
// the table layout of the restated encoding and of the tcnn snapshot format.
// Linked with the vendored fmt's format.cc.
#include <tiny-cuda-nn/encodings/grid.h>

#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>
#include <algorithm>

using namespace tcnn;

// The class's other members reference six functions of tcnn's compiled
// sources: to_string(InterpolationType) (its encoding.cu, a several-minute
// compile of every encoding) and the device queries of its common.cu (which
// needs the CUDA driver library). The constructor reaches none of them, so
// stubs that abort stand in for them.
namespace tcnn {
std::string to_string(InterpolationType) { abort(); }
int cuda_device() { abort(); }
void set_cuda_device(int) { abort(); }
MemoryInfo cuda_memory_info() { abort(); }
size_t cuda_memory_granularity(int) { abort(); }
bool cuda_supports_virtual_memory(int) { abort(); }
}  // namespace tcnn

// tcnn's header-inline GPU memory arena references eight CUDA driver calls;
// the constructor never allocates, and this host-only build does not load
// the driver library, so they are stubs that abort too.
extern "C" {
CUresult cuGetErrorName(CUresult, const char**) { abort(); }
CUresult cuMemAddressFree(CUdeviceptr, size_t) { abort(); }
CUresult cuMemAddressReserve(CUdeviceptr*, size_t, size_t, CUdeviceptr, unsigned long long) { abort(); }
CUresult cuMemCreate(CUmemGenericAllocationHandle*, size_t, const CUmemAllocationProp*, unsigned long long) { abort(); }
CUresult cuMemMap(CUdeviceptr, size_t, size_t, CUmemGenericAllocationHandle, unsigned long long) { abort(); }
CUresult cuMemRelease(CUmemGenericAllocationHandle) { abort(); }
CUresult cuMemSetAccess(CUdeviceptr, size_t, const CUmemAccessDesc*, size_t) { abort(); }
CUresult cuMemUnmap(CUdeviceptr, size_t) { abort(); }
}

namespace {
template <uint32_t F>
int layout(int levels, int log2_hashmap, int base_res, float per_level_scale, int hash, int smoothstep,
           uint32_t* offsets, uint64_t* n_params) {
  GridEncodingTemplated<__half, 3, F, HashType::CoherentPrime> enc(
      uint32_t(levels) * F, uint32_t(log2_hashmap), uint32_t(base_res), per_level_scale, false,
      smoothstep ? InterpolationType::Smoothstep : InterpolationType::Linear, hash ? GridType::Hash : GridType::Dense);
  for (int l = 0; l <= levels; ++l) offsets[l] = uint32_t(enc.level_params_offset(uint32_t(l)));  // entries
  *n_params = enc.n_params();
  return 0;
}
}  // namespace

extern "C" int ref_tcnn_grid_layout(int feats, int levels, int log2_hashmap, int base_res, float per_level_scale,
                                    int hash, int smoothstep, uint32_t* offsets, uint64_t* n_params) {
  if (feats == 2) return layout<2>(levels, log2_hashmap, base_res, per_level_scale, hash, smoothstep, offsets, n_params);
  if (feats == 4) return layout<4>(levels, log2_hashmap, base_res, per_level_scale, hash, smoothstep, offsets, n_params);
  return -1;
}

// The MessagePack snapshot of a tcnn Trainer: the object Trainer::serialize
// builds (trainer.h:267-278: n_params, params_type, and the inference
// parameters as a binary blob, which gpu_memory_to_json_binary copies from the
// device) encoded by the reference's own nlohmann::json::to_msgpack. params
// holds n_params __half (params_type 0) or float (1) values. Returns the
// number of bytes written to out (at most cap), or -1 if cap is too small.
extern "C" long ref_tcnn_snapshot_msgpack(const void* params, uint64_t n_params, int params_type, uint8_t* out,
                                          long cap) {
  const size_t bytes = size_t(n_params) * (params_type == 0 ? sizeof(__half) : sizeof(float));
  const uint8_t* p = static_cast<const uint8_t*>(params);
  json data;
  data["n_params"] = size_t(n_params);
  // type_to_string<PARAMS_T>() (defined in tcnn's common.cu, not linked here): the two names
  // Trainer::deserialize accepts (trainer.h:283-288)
  data["params_type"] = params_type == 0 ? "__half" : "float";
  data["params_binary"] = nlohmann::json::binary_t(std::vector<uint8_t>(p, p + bytes));
  const std::vector<uint8_t> buf = json::to_msgpack(data);
  if (long(buf.size()) > cap) return -1;
  std::copy(buf.begin(), buf.end(), out);
  return long(buf.size());
}
