// Shared device helpers for the GB300 RMSD kernels (sm_103a).
//
// Contents:
//   * error-free FP32 transformations (TwoSum, exact products) used to carry
//     ~48-bit sums of FP32 partials without touching the FP64 pipe, which is
//     narrow on GB300;
//   * a warp "transpose reduction" that reduces 16 compensated values across
//     the 32 lanes with 16 shuffle rounds instead of 16 x 5;
//   * thin inline-PTX wrappers for mbarrier + 1-D bulk async copies
//     (cp.async.bulk, the TMA bulk engine) with bounded waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define GB_DEV __device__ __forceinline__

namespace gb {

constexpr unsigned FULL_MASK = 0xffffffffu;

// Error codes written to the device error word (bitwise OR).
constexpr int DEV_ERR_TIMEOUT = 1;   // an mbarrier wait exceeded its spin limit
constexpr int DEV_ERR_NONFINITE = 2; // QCP saw non-finite input

// ---------------------------------------------------------------------------
// Compensated FP32 arithmetic
// ---------------------------------------------------------------------------

// Knuth TwoSum: s + e == a + b exactly (round-to-nearest, no reassociation).
GB_DEV void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// A float pair carrying hi + lo.
struct CF {
  float hi, lo;
};

GB_DEV CF cf_zero() { return CF{0.f, 0.f}; }

// acc += p, keeping the rounding error of the leading add in lo.
GB_DEV void cf_add(CF& acc, float p) {
  float s, e;
  two_sum(acc.hi, p, s, e);
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, e);
}

// a + b for two compensated values.
GB_DEV CF cf_add2(CF a, CF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  CF r;
  r.hi = s;
  r.lo = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
  return r;
}

GB_DEV double cf_to_double(CF a) { return (double)a.hi + (double)a.lo; }

// Transpose reduction of 16 compensated values over a full warp.  On return
// lane l holds the warp-wide total of value index (l >> 1) in v[0]; both lanes
// 2k and 2k+1 hold value k.  The other entries of v are clobbered.
GB_DEV void warp_xpose_reduce16(CF (&v)[16], int lane) {
#pragma unroll
  for (int level = 0; level < 4; ++level) {
    const int mask = 16 >> level;     // 16, 8, 4, 2
    const int half = 8 >> level;      // 8, 4, 2, 1
    const bool upper = (lane & mask) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      CF keep = upper ? v[i + half] : v[i];
      CF send = upper ? v[i] : v[i + half];
      CF recv;
      recv.hi = __shfl_xor_sync(FULL_MASK, send.hi, mask);
      recv.lo = __shfl_xor_sync(FULL_MASK, send.lo, mask);
      v[i] = cf_add2(keep, recv);
    }
  }
  CF recv;
  recv.hi = __shfl_xor_sync(FULL_MASK, v[0].hi, 1);
  recv.lo = __shfl_xor_sync(FULL_MASK, v[0].lo, 1);
  v[0] = cf_add2(v[0], recv);
}

GB_DEV float warp_sum(float x) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) x += __shfl_xor_sync(FULL_MASK, x, m);
  return x;
}

GB_DEV double warp_sum_d(double x) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) x += __shfl_xor_sync(FULL_MASK, x, m);
  return x;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk async copy (TMA bulk engine), inline PTX
// ---------------------------------------------------------------------------

GB_DEV uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

GB_DEV void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

GB_DEV void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's prior generic-proxy shared-memory accesses before
// subsequent async-proxy (bulk copy) accesses.
GB_DEV void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

GB_DEV void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared, completion signalled on `bar` (tx bytes).
// dst, src must be 16-byte aligned and bytes a non-zero multiple of 16.
GB_DEV void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// 3-D tiled tensor copy global -> shared (TMA), completion on `bar`.  The
// tensor map lives in kernel parameter space (__grid_constant__).  The
// innermost coordinate x times the element size must be a multiple of 16.
GB_DEV void tma_load_3d(void* dst, const void* tmap, int32_t x, int32_t y, int32_t z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

GB_DEV bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: returns false (and sets the device error word) when the phase
// has not completed after `max_spins` try_wait rounds.  Every try_wait blocks
// for a bounded, hardware-defined time, so the overall wait is bounded too.
GB_DEV bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err, uint32_t max_spins = (1u << 24)) {
  for (uint32_t i = 0; i < max_spins; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  if (err) atomicOr(err, DEV_ERR_TIMEOUT);
  return false;
}

// try_wait with a suspend-time hint: the thread sleeps until the phase
// completes or about hint_ns nanoseconds have passed, and issues nothing
// meanwhile (a plain try_wait returns after a short hardware-defined time).
GB_DEV bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// Nanoseconds of the GPU's global timer.
GB_DEV uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait bounded in wall time: false (and DEV_ERR_TIMEOUT in *err) when the
// phase has not completed `limit_ns` nanoseconds after the first failed
// try_wait.  2^24 rounds of 64 try_waits stay as a backstop should the
// timer not advance.  The streaming kernels take the limit from their
// launch arguments (gbrmsd_set_wait_limit_ns).
GB_DEV bool mbar_wait_timed(uint64_t* bar, uint32_t parity, int* err, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t round = 0; round < (1u << 24); ++round) {
#pragma unroll 1
    for (int i = 0; i < 64; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) break;
  }
  if (err) atomicOr(err, DEV_ERR_TIMEOUT);
  return false;
}

// The same bound with sleeping try_waits (1 ms hint each): for waits that
// last a large part of a pipeline step, so that the waiting warps leave the
// issue slots to the warps with work.  2^24 rounds stay as the backstop.
GB_DEV bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, int* err, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t round = 0; round < (1u << 24); ++round) {
    if (mbar_try_wait_sleep(bar, parity, 1000000u)) return true;
    if (global_ns() - t0 > limit_ns) break;
  }
  if (err) atomicOr(err, DEV_ERR_TIMEOUT);
  return false;
}

GB_DEV float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }

GB_DEV float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

}  // namespace gb
