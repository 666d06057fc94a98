// lj_device.cuh -- device-side building blocks shared by the LJ kernels:
// fixed-point periodic coordinates, TMA bulk copies with mbarrier completion,
// time-bounded waits, compensated sums and FP64 block reductions.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lj_internal.h"

namespace ljgb {

// ---------------------------------------------------------------------------
// Fixed-point shadow positions.
//
// A coordinate x is stored as the int32 bits of u = llrint((x - origin) *
// 2^32 / P) mod 2^32, moved to the nearest multiple of 3.  For a periodic box
// P = L and origin = 0: the 32-bit wrapping difference qi - qj is then exactly
// the minimum-image separation in units of L/2^32, the role lround(r/L) plays
// in MDSystem.cu:31-33 and fast_round in MDSystem.cpp:273-277 (taking the low
// 32 bits of the rounded integer is the wrap into the box).  Keeping q on
// multiples of 3 makes a difference of exactly 2^31 (a separation of exactly
// L/2, where both images are equally near) impossible, since 3 does not
// divide 2^31; every ordered pair therefore sees the exact negative of its
// partner's separation, as the reference's antisymmetric rounding does.  The
// grid is 3 L/2^32 (2e-8 sigma at L = 27 sigma).  For walls / open boxes P is
// chosen at least twice the particle extent so no difference wraps.
// Cost: one FP64 multiply, one conversion and a few integer operations (FP64
// runs at 1/64 of the FP32 rate on this part).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t fixed_coord_scaled(double dx, double scale) {
  const double t = dx * scale;
  const uint32_t u = (uint32_t)(unsigned long long)llrint(t);
  const uint32_t r = u % 3u;
  const uint32_t q = r == 0u ? u : (r == 1u ? u - 1u : u + 1u);
  return (int32_t)q;
}

__device__ __forceinline__ int32_t fixed_coord(double x, double origin, double invP) {
  const double t = (x - origin) * (invP * 4294967296.0);
  const uint32_t u = (uint32_t)(unsigned long long)llrint(t);
  const uint32_t r = u % 3u;
  const uint32_t q = r == 0u ? u : (r == 1u ? u - 1u : u + 1u);
  return (int32_t)q;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk copy (cp.async.bulk, the non-tensor TMA path).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
          smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

// Global -> shared bulk copy of `bytes` (multiple of 16, both addresses
// 16-byte aligned), completion signalled on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
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

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for phase `parity` of `bar` to complete, giving up after
// kWaitLimitNs of wall time.  Returns false on timeout (the caller records
// LJ_DEVFLAG_TIMEOUT and leaves the kernel after draining its copies).
constexpr uint64_t kWaitLimitNs = 1500000000ull;  // 1.5 s

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_timer_ns() - t0 > kWaitLimitNs) return false;
  }
}

// ---------------------------------------------------------------------------
// Compensated summation (Knuth TwoSum): hi + lo carries the sum exactly up
// to the rounding of lo.
// ---------------------------------------------------------------------------
struct FloatAcc {
  float hi, lo;
};

__device__ __forceinline__ void two_sum_add(FloatAcc& a, float t) {
  float s = __fadd_rn(a.hi, t);
  float bp = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(t, bp));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, e);
}

// ---------------------------------------------------------------------------
// FP64 reductions.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of NV doubles per thread, result valid in thread 0.
// Fixed reduction order (warp tree, then warps in index order): the result
// is independent of scheduling.  `sh` needs NV * 32 doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k * 32 + warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += sh[k * 32 + w];
      v[k] = s;
    }
  }
  __syncthreads();
}

}  // namespace ljgb
