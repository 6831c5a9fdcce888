// tcgen05.cuh -- inline-PTX building blocks for the sm_103a tensor-core path:
// TMEM allocation, shared-memory matrix descriptors, tcgen05.mma (kind::f16,
// BF16/FP16 operands, FP32 accumulate in TMEM), commit to mbarriers, TMEM
// loads, 1-D bulk copies (cp.async.bulk) and bounded mbarrier waits.
//
// Operand layout used throughout (no swizzle): a matrix of R rows x C
// 16-bit elements is stored as 8x8 "core matrices" of 128 contiguous bytes
// (8 rows x 16 bytes). Core matrix (rg, cg) -- rows 8rg..8rg+7, columns
// 8cg..8cg+7 -- sits at byte (rg * (C/8) + cg) * 128 and its row r at +16r.
// As a K-major operand (rows = M or N, columns = K) the descriptor's
// leading-dimension byte offset is 128 (next core matrix along K) and the
// stride byte offset is (C/8) * 128 (next 8-row group). The same bytes read
// as an MN-major operand (rows = K, columns = M or N) have the roles
// exchanged; the weight-gradient products use that view.
#pragma once
#include <stdint.h>

#include "common.cuh"

namespace nmg {
namespace tc {

NMG_D uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// ------------------------------------------------------------------ mbarrier
NMG_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
NMG_D void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

NMG_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(1000000u)  // suspend up to 1 ms per attempt instead of spinning
      : "memory");
  return ok != 0;
}

// Non-blocking test of phase `parity` (for a thread that polls several
// barriers and must not be suspended on any one of them).
NMG_D bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of the barrier with a time limit (~1 s at the
// maximum SM clock). Returns false on timeout; the caller records the error
// and unwinds instead of hanging the GPU.
NMG_D bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > 2000000000LL) return false;
  }
  return true;
}

// Plain arrival (release at CTA scope).
NMG_D void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

NMG_D void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared completing on `bar` (both addresses
// 16-byte aligned, bytes a multiple of 16).
NMG_D void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// --------------------------------------------------------------------- TMEM
// Executed by one full warp. Writes the TMEM base address to *slot.
NMG_D void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
NMG_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

NMG_D void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
NMG_D void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Makes this thread's generic-proxy shared-memory writes visible to the
// tensor core (async proxy).
NMG_D void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ------------------------------------------------------------- descriptors
// Shared-memory matrix descriptor (sm_100 format): start address, leading
// and stride byte offsets (all >> 4), version 1, no swizzle.
NMG_D uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr & 0x3FFFFu) >> 4);
  d |= uint64_t((lbo & 0x3FFFFu) >> 4) << 16;
  d |= uint64_t((sbo & 0x3FFFFu) >> 4) << 32;
  d |= uint64_t(1) << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, absolute LBO mode, SWIZZLE_NONE
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator,
// A/B both BF16 (fp16 = false) or both FP16, dense, no negation.
// a_mn / b_mn select the MN-major view of an operand.
NMG_HD uint32_t idesc_f16(int M, int N, bool fp16, bool a_mn = false, bool b_mn = false) {
  const uint32_t ab = fp16 ? 0u : 1u;
  return (1u << 4)                      // D format: F32
         | (ab << 7) | (ab << 10)       // A, B format
         | (uint32_t(a_mn) << 15) | (uint32_t(b_mn) << 16)
         | (uint32_t(N >> 3) << 17)     // N / 8
         | (uint32_t(M >> 4) << 24);    // M / 16
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
NMG_D void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives once on `bar` when all MMAs issued so far by this thread complete.
NMG_D void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 lanes x 16 columns of 32-bit: thread t of the warp gets row (lane base
// + t), columns col..col+15.
NMG_D void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
NMG_D void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Register reallocation between warpgroups (all warps of the warpgroup
// execute it). The block's total stays what it was launched with: the
// caller checks the kernel's launch register count before using these.
template <int N> NMG_D void reg_dealloc() { asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(N)); }
template <int N> NMG_D void reg_alloc() { asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(N)); }

// Named barrier over `count` threads (a warpgroup = 128).
NMG_D void bar_sync(int id, int count) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }

// max(a,0), max(b,0) packed into one bf16x2 / f16x2 word in one instruction.
NMG_D uint32_t pack2_relu(float a, float b, bool fp16) {
  uint32_t r;
  if (fp16)  // saturating: a value beyond the FP16 range becomes +-65504, not infinity
    asm("cvt.rn.satfinite.relu.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  else
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

// Packs two floats into a bf16x2 / f16x2 word (low half = a).
NMG_D uint32_t pack2(float a, float b, bool fp16) {
  if (fp16) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  }
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}
NMG_D float2 unpack2(uint32_t w, bool fp16) {
  if (fp16) {
    __half2 h = *reinterpret_cast<__half2*>(&w);
    return __half22float2(h);
  }
  __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&w);
  return __bfloat1622float2(h);
}

// Byte offset of core-matrix row `row`, 16-byte chunk `chunk` in a tile of
// `chunks` chunks per row (no swizzle, see the header comment).
NMG_HD uint32_t cm_offset(int row, int chunk, int chunks) {
  return uint32_t(((row >> 3) * chunks + chunk) * 128 + (row & 7) * 16);
}

}  // namespace tc
}  // namespace nmg
