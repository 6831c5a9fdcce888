// tcnn_snapshot.cu -- parameters in tiny-cuda-nn's Trainer snapshot format.
//
// tcnn's Trainer::serialize (src/ext/tcnn/include/tiny-cuda-nn/trainer.h:267-278)
// returns a JSON object {"n_params": N, "params_type": "__half" | "float",
// "params_binary": <binary blob of the inference parameters>}, which tcnn
// users write with nlohmann::json::to_msgpack and read back with
// from_msgpack + Trainer::deserialize (trainer.h:280-305). The parameter
// vector is the GuidingNetwork's [MLP weights | encoding parameters]
// (src/render/guided/network.h:85-100), the layout this library uses, so a
// snapshot is a direct dump. Written here: a MessagePack map of those three
// keys (sorted, as nlohmann's std::map object writes them), the blob as
// MessagePack "bin"; read: any key order, "__half" or "float" blobs, the
// optional "optimizer" entry skipped.
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "api_common.cuh"
#include "ctx.cuh"

namespace nmg {
namespace {

void put_u8(std::vector<uint8_t>& o, uint8_t v) { o.push_back(v); }
void put_be(std::vector<uint8_t>& o, uint64_t v, int bytes) {
  for (int i = bytes - 1; i >= 0; --i) o.push_back(uint8_t(v >> (8 * i)));
}
void put_str(std::vector<uint8_t>& o, const char* s) {
  const size_t n = strlen(s);
  if (n < 32) {
    put_u8(o, uint8_t(0xa0 | n));
  } else {
    put_u8(o, 0xd9);
    put_u8(o, uint8_t(n));
  }
  o.insert(o.end(), s, s + n);
}
void put_uint(std::vector<uint8_t>& o, uint64_t v) {
  if (v < 128) {
    put_u8(o, uint8_t(v));
  } else if (v < 256) {
    put_u8(o, 0xcc);
    put_be(o, v, 1);
  } else if (v < 65536) {
    put_u8(o, 0xcd);
    put_be(o, v, 2);
  } else if (v <= 0xffffffffull) {
    put_u8(o, 0xce);
    put_be(o, v, 4);
  } else {
    put_u8(o, 0xcf);
    put_be(o, v, 8);
  }
}
void put_bin_header(std::vector<uint8_t>& o, uint64_t n) {
  if (n < 256) {
    put_u8(o, 0xc4);
    put_be(o, n, 1);
  } else if (n < 65536) {
    put_u8(o, 0xc5);
    put_be(o, n, 2);
  } else {
    put_u8(o, 0xc6);
    put_be(o, n, 4);
  }
}

// Minimal MessagePack reader over a byte buffer (the subset nlohmann writes
// for this object: maps, strings, unsigned/signed integers, bin/ext blobs,
// arrays, floats, booleans, nil).
struct Reader {
  const uint8_t* p;
  const uint8_t* end;
  bool ok = true;
  uint64_t be(int bytes) {
    if (end - p < bytes) {
      ok = false;
      return 0;
    }
    uint64_t v = 0;
    for (int i = 0; i < bytes; ++i) v = (v << 8) | *p++;
    return v;
  }
  uint8_t byte() { return uint8_t(be(1)); }
  bool str(std::string* s) {
    const uint8_t t = byte();
    uint64_t n;
    if ((t & 0xe0) == 0xa0) n = t & 0x1f;
    else if (t == 0xd9) n = be(1);
    else if (t == 0xda) n = be(2);
    else if (t == 0xdb) n = be(4);
    else return ok = false;
    if (uint64_t(end - p) < n) return ok = false;
    s->assign(reinterpret_cast<const char*>(p), size_t(n));
    p += n;
    return ok;
  }
  bool uint(uint64_t* v) {
    const uint8_t t = byte();
    if (t < 0x80) *v = t;
    else if (t == 0xcc) *v = be(1);
    else if (t == 0xcd) *v = be(2);
    else if (t == 0xce) *v = be(4);
    else if (t == 0xcf) *v = be(8);
    else return ok = false;
    return ok;
  }
  // bin8/16/32, or ext (nlohmann writes a binary with a subtype as ext)
  bool bin(const uint8_t** data, uint64_t* n) {
    const uint8_t t = byte();
    if (t == 0xc4) *n = be(1);
    else if (t == 0xc5) *n = be(2);
    else if (t == 0xc6) *n = be(4);
    else if (t == 0xc7) { *n = be(1); be(1); }
    else if (t == 0xc8) { *n = be(2); be(1); }
    else if (t == 0xc9) { *n = be(4); be(1); }
    else return ok = false;
    if (!ok || uint64_t(end - p) < *n) return ok = false;
    *data = p;
    p += *n;
    return ok;
  }
  // skips one value of any type
  bool skip(int depth = 0) {
    if (depth > 64) return ok = false;
    const uint8_t t = byte();
    if (!ok) return false;
    uint64_t n = 0;
    if (t < 0x80 || t >= 0xe0 || t == 0xc0 || t == 0xc2 || t == 0xc3) return true;
    if ((t & 0xf0) == 0x80) return skip_n(2 * uint64_t(t & 0x0f), depth);
    if ((t & 0xf0) == 0x90) return skip_n(t & 0x0f, depth);
    if ((t & 0xe0) == 0xa0) return adv(t & 0x1f);
    switch (t) {
      case 0xc4: return adv(be(1));
      case 0xc5: return adv(be(2));
      case 0xc6: return adv(be(4));
      case 0xc7: n = be(1); return adv(n + 1);
      case 0xc8: n = be(2); return adv(n + 1);
      case 0xc9: n = be(4); return adv(n + 1);
      case 0xca: return adv(4);
      case 0xcb: return adv(8);
      case 0xcc: case 0xd0: return adv(1);
      case 0xcd: case 0xd1: return adv(2);
      case 0xce: case 0xd2: return adv(4);
      case 0xcf: case 0xd3: return adv(8);
      case 0xd4: return adv(2);
      case 0xd5: return adv(3);
      case 0xd6: return adv(5);
      case 0xd7: return adv(9);
      case 0xd8: return adv(17);
      case 0xd9: return adv(be(1));
      case 0xda: return adv(be(2));
      case 0xdb: return adv(be(4));
      case 0xdc: return skip_n(be(2), depth);
      case 0xdd: return skip_n(be(4), depth);
      case 0xde: return skip_n(2 * be(2), depth);
      case 0xdf: return skip_n(2 * be(4), depth);
    }
    return ok = false;
  }
  bool adv(uint64_t n) {
    if (!ok || uint64_t(end - p) < n) return ok = false;
    p += n;
    return true;
  }
  bool skip_n(uint64_t n, int depth) {
    for (uint64_t i = 0; i < n && ok; ++i) skip(depth + 1);
    return ok;
  }
};

// IEEE binary16 <-> binary32 on the host, by the bit layouts.
uint16_t half_bits(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t mag = x & 0x7fffffffu;
  if (mag >= 0x7f800000u) return uint16_t(sign | (mag > 0x7f800000u ? 0x7e00u : 0x7c00u));  // NaN / Inf
  if (mag >= 0x477ff000u) return uint16_t(sign | 0x7c00u);  // rounds to >= 65520: overflow
  if (mag < 0x38800000u) {  // subnormal half (or zero): round the value scaled by 2^24
    if (mag < 0x33000000u) return uint16_t(sign);  // below half the smallest subnormal
    const uint32_t e = mag >> 23, m = (mag & 0x7fffffu) | 0x800000u;
    const int shift = int(126 - e);  // 14..24
    uint32_t r = m >> shift;
    const uint32_t rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
    if (rem > halfway || (rem == halfway && (r & 1u))) ++r;
    return uint16_t(sign | r);
  }
  // normal: rebias the exponent and round the mantissa to nearest even
  uint32_t r = ((mag - 0x38000000u) >> 13);
  const uint32_t rem = mag & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) ++r;
  return uint16_t(sign | r);
}

float half_value(uint16_t h) {
  const uint32_t sign = uint32_t(h & 0x8000u) << 16;
  const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) {
      x = sign;
    } else {  // subnormal: normalise
      int s = 0;
      uint32_t mm = m;
      while (!(mm & 0x400u)) {
        mm <<= 1;
        ++s;
      }
      x = sign | (uint32_t(127 - 15 - s + 1) << 23) | ((mm & 0x3ffu) << 13);
    }
  } else if (e == 31) {
    x = sign | 0x7f800000u | (m << 13);
  } else {
    x = sign | ((e + 112u) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &x, 4);
  return f;
}

}  // namespace
}  // namespace nmg

using namespace nmg;

extern "C" {

nmg_status nmg_export_tcnn(const nmg_ctx* c, const char* path, int params_type) {
  NMG_REQUIRE(c && path, "NULL argument");
  NMG_REQUIRE(params_type == 0 || params_type == 1, "params_type=%d (0 = __half, 1 = float)", params_type);
  const size_t n = size_t(c->lay.n_params);
  std::vector<float> p(n);
  NMG_CUDA_TRY(cudaMemcpy(p.data(), c->w_inf, n * sizeof(float), cudaMemcpyDeviceToHost));
  std::vector<uint8_t> o;
  o.reserve(64 + n * (params_type ? 4 : 2));
  put_u8(o, 0x83);  // map of 3, keys in std::map order
  put_str(o, "n_params");
  put_uint(o, n);
  put_str(o, "params_binary");
  put_bin_header(o, n * (params_type ? 4 : 2));
  for (size_t i = 0; i < n; ++i) {  // the blob is the raw little-endian device memory image
    if (params_type) {
      uint32_t b;
      memcpy(&b, &p[i], 4);
      for (int k = 0; k < 4; ++k) o.push_back(uint8_t(b >> (8 * k)));
    } else {
      const uint16_t h = half_bits(p[i]);
      o.push_back(uint8_t(h));
      o.push_back(uint8_t(h >> 8));
    }
  }
  put_str(o, "params_type");
  put_str(o, params_type ? "float" : "__half");
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(NMG_ERR_INVALID_ARG, "cannot open %s for writing", path);
  const bool w = fwrite(o.data(), 1, o.size(), f) == o.size();
  const bool cl = fclose(f) == 0;
  return w && cl ? NMG_OK : set_error(NMG_ERR_INVALID_ARG, "short write to %s", path);
}

nmg_status nmg_import_tcnn(nmg_ctx* c, const char* path, nmg_stream stream) {
  NMG_REQUIRE(c && path, "NULL argument");
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(NMG_ERR_INVALID_ARG, "cannot open %s", path);
  std::vector<uint8_t> buf;
  uint8_t tmp[1 << 16];
  size_t got;
  while ((got = fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
  fclose(f);
  Reader r{buf.data(), buf.data() + buf.size()};
  const uint8_t t = r.byte();
  uint64_t entries;
  if ((t & 0xf0) == 0x80) entries = t & 0x0f;
  else if (t == 0xde) entries = r.be(2);
  else if (t == 0xdf) entries = r.be(4);
  else return set_error(NMG_ERR_INVALID_ARG, "%s: not a MessagePack map", path);
  uint64_t n = 0;
  bool have_n = false;
  std::string type = "__half";
  const uint8_t* blob = nullptr;
  uint64_t blob_n = 0;
  for (uint64_t i = 0; i < entries && r.ok; ++i) {
    std::string key;
    if (!r.str(&key)) break;
    if (key == "n_params") have_n = r.uint(&n);
    else if (key == "params_type") r.str(&type);
    else if (key == "params_binary") r.bin(&blob, &blob_n);
    else r.skip();
  }
  if (!r.ok || !blob) return set_error(NMG_ERR_INVALID_ARG, "%s: malformed tcnn snapshot", path);
  const size_t np = size_t(c->lay.n_params);
  const size_t esz = type == "float" ? 4 : (type == "__half" ? 2 : 0);
  if (!esz) return set_error(NMG_ERR_INVALID_ARG, "%s: params_type %s (need __half or float)", path, type.c_str());
  if ((have_n && n != np) || blob_n != np * esz)
    return set_error(NMG_ERR_INVALID_ARG, "%s: %llu parameters, this network has %zu", path,
                     (unsigned long long)(blob_n / esz), np);
  std::vector<float> p(np);
  for (size_t i = 0; i < np; ++i) {
    const uint8_t* b = blob + i * esz;
    if (esz == 4) {
      const uint32_t v = uint32_t(b[0]) | uint32_t(b[1]) << 8 | uint32_t(b[2]) << 16 | uint32_t(b[3]) << 24;
      memcpy(&p[i], &v, 4);
    } else {
      p[i] = half_value(uint16_t(b[0] | b[1] << 8));
    }
  }
  float* d = nullptr;
  NMG_CUDA_TRY(cudaMalloc(&d, np * sizeof(float)));
  cudaError_t e = cudaMemcpy(d, p.data(), np * sizeof(float), cudaMemcpyHostToDevice);
  nmg_status s = e == cudaSuccess ? nmg_set_params(c, d, stream) : set_error(NMG_ERR_CUDA, "%s", cudaGetErrorString(e));
  if (s == NMG_OK) {
    e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) s = set_error(NMG_ERR_CUDA, "%s", cudaGetErrorString(e));
  }
  cudaFree(d);
  return s;
}

}  // extern "C"
