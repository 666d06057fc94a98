// lj_pairs.cu -- all-pairs Lennard-Jones force / energy / virial / RDF kernels.
//
// Replaces calculateForces + RDFmerger of the reference
// (src/library/MDSystem.cu:21-153) and the O(N^2) CPU loop of
// MDSystem::CalculateForces (src/library/MDSystem.cpp:253-310).  Same pair set
// (ordered pairs j != i, minimum image for periodic boxes, no cutoff), same
// physics (MDSystem.cu:44-53), redesigned for sm_103a:
//
//  * persistent stream-K grid: every CTA receives an equal share of the
//    (i-block, j-tile) sequence of all boxes, so the single wave fills all
//    SMs regardless of N (the reference launches ceil(N/256) CTAs);
//  * j-tiles of 16-byte records staged in shared memory by cp.async.bulk
//    (TMA bulk copies) into a STAGES-deep mbarrier ring, read back as
//    broadcast 128-bit shared loads;
//  * MIXED precision: positions as 32-bit fixed-point fractions of the box
//    whose wrapping integer difference is the minimum image (no rounding
//    instructions per pair), FP32 pair math, per-tile FP32 sums folded into
//    TwoSum-compensated accumulators;
//  * no per-pair global atomics: partial sums of each (CTA, i-block) segment
//    go to a partial buffer reduced deterministically in FP64 by the
//    integrator kernels; pair histograms (RDF) go to a shared-memory
//    histogram flushed once per CTA.
#include <cuda_runtime.h>

#include <cstdint>

#include "lj_device.cuh"
#include "lj_kernels.h"
#include "lj_schedule.h"
#include "lj_stepdev.cuh"

namespace ljgb {

namespace {

#ifndef LJ_CHUNK
#define LJ_CHUNK 32
#endif
constexpr int kChunk = LJ_CHUNK;  // pairs per compensated force partial sum
// CTA ranges start and end on multiples of kSplitGrain j records inside a
// tile; the unrolled chunk loop needs those to be whole chunks.
static_assert(kSplitGrain % kChunk == 0, "schedule cuts must fall on chunk boundaries");

// Wrapping difference of two fixed-point coordinates (the minimum image).
__device__ __forceinline__ int fixed_diff(int a, int b) { return (int)((unsigned)a - (unsigned)b); }

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The i record of a thread is held with x, y, z in slots 1..3 of an aligned
// register quadruple (.y, .z, .w), while the 128-bit shared loads of the j
// records put theirs in slots 0..2.  Each integer difference then reads its
// two operands from registers of opposite parity, which sit in different
// register-file banks: with both records in slots 0..2 every difference
// waited on a bank conflict (measured on GB300: 52.5 -> 49.4 cycles per
// 64-pair warp step of the packed loop).  i_record_slots123 places it.
__device__ __forceinline__ int4 i_record_slots123(const int4 q, int4* slot) {
  volatile int4* v = slot;
  v->x = 0;
  v->y = q.x;
  v->z = q.y;
  v->w = q.z;
  // volatile load: the compiler may not forward the stored registers
  int4 r;
  asm volatile("ld.volatile.shared.v4.s32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "r"((unsigned)__cvta_generic_to_shared(slot)));
  return r;
}

// One pair in the MIXED path.  d = qi - qj wraps to the minimum image (qi
// in slots 1..3, see i_record_slots123).
// s = (s/r)^8 [12 (s/r)^6 - 6] (sigma units), a += (s/r)^12, b += (s/r)^6.
template <bool MASKED>
__device__ __forceinline__ void pair_mixed(const int4 qi, const int4 qj, float k2inv, bool excl,
                                           float& fx, float& fy, float& fz, float& pa,
                                           float& pb) {
  const float dx = __int2float_rn(fixed_diff(qi.y, qj.x));
  const float dy = __int2float_rn(fixed_diff(qi.z, qj.y));
  const float dz = __int2float_rn(fixed_diff(qi.w, qj.z));
  const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
  // r2 is in fixed-point units^2, between ~1e14 and ~1.4e19: far from the
  // subnormal and 2^126 ranges, so the raw approximate reciprocal applies.
  float ri = k2inv * rcp_approx(r2);
  if (MASKED) ri = excl ? 0.0f : ri;
  const float r6 = ri * ri * ri;
  const float t = __fmaf_rn(12.0f, r6, -6.0f);
  const float s = r6 * ri * t;
  fx = __fmaf_rn(s, dx, fx);
  fy = __fmaf_rn(s, dy, fy);
  fz = __fmaf_rn(s, dz, fz);
  pa = __fmaf_rn(r6, r6, pa);
  pb += r6;
}

// Packed FP32x2 arithmetic (PTX .f32x2, sm_100 and later): one instruction
// applies the operation to two independent FP32 values held in a 64-bit
// register pair.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk2(f32x2 r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Two pairs (i, j0) and (i, j1) as the two lanes of FP32x2 operations (qi in
// slots 1..3): the
// same arithmetic as pair_mixed per lane, with half the instructions after
// the int -> float conversions.  The accumulators hold the j0 and j1 partial
// sums in their two lanes.
// On GB300 an FP32x2 instruction occupies both FMA sub-pipes (heavy and
// lite) for two cycles, so the FP32 throughput is that of two FFMAs; what it
// saves is issue slots.  The scalar loop issued ~23.7 warp-instructions per
// 32 pairs at 84% issue utilisation with the FMA pipes 64% busy; this one
// issues ~16.8 (ncu: 1.41e8 vs 1.98e8 per N=16384 launch) and ran 4.5%
// faster in the same step.  It needs ~80 registers, hence 6 (128-thread) or
// 3 (256-thread) resident CTAs per SM, and the integer differences stay on
// the ALU pipe, which has room here.
template <bool MASKED>
__device__ __forceinline__ void pair_mixed2(const int4 qi, const int4 qa, const int4 qb, f32x2 k2inv2, bool exa,
                                            bool exb, f32x2& fx, f32x2& fy, f32x2& fz, f32x2& pa, f32x2& pb) {
  const f32x2 dx = pk2(__int2float_rn(fixed_diff(qi.y, qa.x)), __int2float_rn(fixed_diff(qi.y, qb.x)));
  const f32x2 dy = pk2(__int2float_rn(fixed_diff(qi.z, qa.y)), __int2float_rn(fixed_diff(qi.z, qb.y)));
  const f32x2 dz = pk2(__int2float_rn(fixed_diff(qi.w, qa.z)), __int2float_rn(fixed_diff(qi.w, qb.z)));
  const f32x2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
  float r2a, r2b;
  upk2(r2, r2a, r2b);
  float ra = rcp_approx(r2a), rb = rcp_approx(r2b);
  if (MASKED) {
    ra = exa ? 0.0f : ra;
    rb = exb ? 0.0f : rb;
  }
  const f32x2 ri = mul2(pk2(ra, rb), k2inv2);
  const f32x2 r6 = mul2(mul2(ri, ri), ri);
  const f32x2 t = fma2(r6, pk2(12.0f, 12.0f), pk2(-6.0f, -6.0f));
  const f32x2 sf = mul2(mul2(r6, ri), t);
  fx = fma2(sf, dx, fx);
  fy = fma2(sf, dy, fy);
  fz = fma2(sf, dz, fz);
  pa = fma2(r6, r6, pa);
  pb = add2(pb, r6);
}

__device__ __forceinline__ float lane_sum(f32x2 v) {
  float a, b;
  upk2(v, a, b);
  return a + b;
}

// floor(x) for 0 <= x < 2^23: 2^23 + x rounded down is 2^23 + floor(x)
// exactly, read back from the float's bits (an FP32 add and an integer
// subtract instead of a round and a float -> int conversion).
__device__ __forceinline__ int floor_small(float x) {
  return __float_as_int(__fadd_rd(x, 8388608.0f)) - 0x4B000000;
}

// Histogram bin of a pair from its fixed-point separation (qi in slots 1..3);
// the arithmetic is exactly what the oracle's emu_rdf_* reproduces on the CPU
// (floor of the separately rounded products, clamped or dropped past the last
// bin).
__device__ __forceinline__ int pair_bin(const int4 qi, const int4 qj, float k2, const HistArgs& h) {
  const float dx = __int2float_rn((int)((unsigned)qj.x - (unsigned)qi.y));
  const float dy = __int2float_rn((int)((unsigned)qj.y - (unsigned)qi.z));
  const float dz = __int2float_rn((int)((unsigned)qj.z - (unsigned)qi.w));
  const float r2 = __fmul_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))), k2);
  if (h.mode == 2) {  // linear r bins, r < rmax (so r / w < nb, up to rounding)
    if (!(r2 < h.rmax2)) return -1;
    return min(floor_small(__fmul_rn(__fsqrt_rn(r2), h.inv_w)), h.nb - 1);
  }
  // r^2 bins; the quotient is capped at nb first, which keeps it in
  // floor_small's range and changes no bin
  const int fb = floor_small(fminf(__fmul_rn(r2, h.inv_w), (float)h.nb));
  if (h.mode == 0) return min(fb, h.nb - 1);  // clamp (MDSystem.cu:39)
  return fb < h.nb ? fb : -1;                  // drop (MDSystem.cpp:283)
}

}  // namespace

// ---------------------------------------------------------------------------
// MIXED-precision persistent pair kernel.
// THREADS threads, one i-particle each; TILE j-records per stage.
// ---------------------------------------------------------------------------
// EPI = 0: partial segments only.  EPI = MODE_EVN / MODE_TVN: the CTA that
// writes the last segment of an i-block also runs the second half of the
// Verlet step for that block (fused_block_step), and the CTA that finishes
// the last block runs the per-box observables (EVN) or the TVN scale (TVN).
// Completion is detected with atomic counters only; no CTA waits on another.
template <int THREADS, int TILE, int STAGES, bool FORCES, bool HIST, int EPI>
__device__ __forceinline__ void pairs_body(const PairArgs& a, const StateArgs& st, unsigned char* smem_raw) {
  int4* sq = reinterpret_cast<int4*>(smem_raw);
  unsigned* shist = reinterpret_cast<unsigned*>(smem_raw + sizeof(int4) * STAGES * TILE);
  __shared__ uint64_t bars[STAGES];
  __shared__ double shd[EPI ? 4 * 32 : 1];
  __shared__ int sflag;
  __shared__ int4 sirec[THREADS];  // i records on their way to slots 1..3

  const int g = blockIdx.x;
  const int tid = threadIdx.x;
  if (EPI && g == 0) {
    if (tid == 0) st.glob_cnt[st.ticket ^ 1] = 0;  // the other parity's ticket counter
    if (EPI == MODE_EVN) {
      // This step's observables are pending once the launch completes: its
      // parity's entry is read only after that (the next step's pair kernel,
      // a read-back), and this launch reads only the other parity's.
      const int par = st.ticket - 2;
      for (int sys = tid; sys < st.nsys; sys += THREADS) {
        st.sc[sys].obs_slot[par] = st.obs_slot;
        st.sc[sys].obs_pending[par] = MODE_EVN;
      }
    }
  }
  // This CTA's j range: from offset lo0 of its first tile to offset lo1 of
  // tile t1 (lo1 = 0: up to the end of tile t1 - 1).
  const int t0 = a.cta_tile_begin[g], t1 = a.cta_tile_begin[g + 1];
  const int lo0 = a.cta_lo ? a.cta_lo[g] : 0, lo1 = a.cta_lo ? a.cta_lo[g + 1] : 0;
  const int ntiles = t1 - t0 + (lo1 > 0 ? 1 : 0);
  if (ntiles <= 0) return;

  // Barrier-free j-tile pipeline: warps wait only for the data of the stage
  // they read (its mbarrier) and count themselves done with it in shared
  // memory; the last warp to finish a stage refills it with the tile STAGES
  // ahead (its lane 0 issues the bulk copy).  Warps therefore drift freely by
  // up to STAGES-1 tiles instead of meeting at a CTA barrier every tile.
  constexpr int NW = THREADS / 32;
  __shared__ int done_cnt[STAGES];
  __shared__ int prod[3];  // producer cursor: i-block, j-tile, tiles issued
  __shared__ volatile int sfail;
  const int lane = tid & 31;

  if (HIST) {
    for (int b = tid; b < a.hist.nb; b += THREADS) shist[b] = 0u;
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&bars[s], 1);
      done_cnt[s] = 0;
    }
    sfail = 0;
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    int pB = a.cta_block[g], pjt = a.cta_jt[g], issued = 0;
    const int pre = ntiles < STAGES ? ntiles : STAGES;
    for (; issued < pre; ++issued) {
      const BlockInfo bi = a.blocks[pB];
      const int j0 = pjt * TILE;
      const int cnt = min(TILE, bi.n_sys - j0);
      const int s = issued % STAGES;
      mbar_arrive_expect_tx(&bars[s], (uint32_t)cnt * 16u);
      bulk_g2s(sq + s * TILE, a.q + bi.p0 + j0, (uint32_t)cnt * 16u, &bars[s]);
      if (++pjt == bi.njt) { ++pB; pjt = 0; }
    }
    prod[0] = pB;
    prod[1] = pjt;
    prod[2] = issued;
  }
  __syncthreads();

  int B = a.cta_block[g], jt = a.cta_jt[g];
  BlockInfo bi = a.blocks[B];
  int i_local = bi.i0 + tid;
  bool valid_i = tid < bi.n_i;
  int4 qi = i_record_slots123(a.q[bi.p0 + (valid_i ? i_local : bi.i0)], &sirec[tid]);
  float k2inv = a.sc[bi.sys].k2inv;
  float k2 = a.sc[bi.sys].k2;
  FloatAcc acc[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) acc[c] = FloatAcc{0.f, 0.f};
  unsigned nclamp = 0;  // HIST, clamped r^2 bins: pairs in the last bin
  unsigned nself = 0;   // HIST: self pairs binned into bin 0

  // A warp whose wait times out (or that sees another warp's timeout) keeps
  // walking the tile sequence without computing, so every CTA-wide barrier
  // below is still reached by all warps; results of the launch are void.
  bool failed = false;
  for (int k = 0; k < ntiles; ++k) {
    const int s = k % STAGES;
    if (!failed) {
      const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bars[s], (uint32_t)((k / STAGES) & 1)));
      if (!ok) {
        failed = true;
        if (lane == 0) sfail = 1;
      } else if (sfail) {
        failed = true;
      }
    }
    const int j0 = jt * TILE;
    const int cnt = min(TILE, bi.n_sys - j0);
    const int jlo = k == 0 ? lo0 : 0;                        // multiples of kChunk
    const int jhi = (k == ntiles - 1 && lo1 > 0) ? lo1 : cnt;
    if (!failed) {
      const int4* st = sq + s * TILE;
      const bool masked = j0 < bi.i0 + bi.n_i && j0 + cnt > bi.i0;  // tile holds this block's own i's
      if (FORCES) {
        // Force sums are folded into the TwoSum accumulators every kChunk
        // pairs, so a large near-neighbour term rounds at most kChunk-1 later
        // additions.  Energy sums go chunk -> tile (plain FP32) -> TwoSum: a
        // chunk partial is never small next to the tile sum, so the far-field
        // (s/r)^6 tail is not truncated.
        float ta = 0.f, tb = 0.f;
        if (cnt == TILE) {
          // Full tile: unrolled chunks.  Only the diagonal tile (the j-range
          // holding this CTA's own i's) needs the self-pair excluded; it
          // keeps the unrolled loop and pays one compare + select per pair.
          const bool diag = masked;
#pragma unroll 1
          for (int c0 = jlo; c0 < jhi; c0 += kChunk) {
            const f32x2 k2i2 = pk2(k2inv, k2inv);
            f32x2 FX = 0ull, FY = 0ull, FZ = 0ull, PA = 0ull, PB = 0ull;
            if (!diag) {
#pragma unroll
              for (int jj = c0; jj < c0 + kChunk; jj += 2)
                pair_mixed2<false>(qi, st[jj], st[jj + 1], k2i2, false, false, FX, FY, FZ, PA, PB);
            } else {
              const int self = i_local - j0;  // tile-local index of this thread's i
#pragma unroll
              for (int jj = c0; jj < c0 + kChunk; jj += 2)
                pair_mixed2<true>(qi, st[jj], st[jj + 1], k2i2, jj == self, jj + 1 == self, FX, FY, FZ, PA, PB);
            }
            const float fx = lane_sum(FX), fy = lane_sum(FY), fz = lane_sum(FZ), pa = lane_sum(PA),
                        pb = lane_sum(PB);
            two_sum_add(acc[0], fx);
            two_sum_add(acc[1], fy);
            two_sum_add(acc[2], fz);
            ta += pa;
            tb += pb;
          }
        } else {
          // Ragged last tile of a box: packed pairs with the self pair
          // excluded, an odd last record on its own.
          const int self = i_local - j0;
          for (int c0 = jlo; c0 < jhi; c0 += kChunk) {
            const int c1 = min(jhi, c0 + kChunk);
            const f32x2 k2i2 = pk2(k2inv, k2inv);
            f32x2 FX = 0ull, FY = 0ull, FZ = 0ull, PA = 0ull, PB = 0ull;
            int jj = c0;
            for (; jj + 1 < c1; jj += 2)
              pair_mixed2<true>(qi, st[jj], st[jj + 1], k2i2, jj == self, jj + 1 == self, FX, FY, FZ, PA, PB);
            float fx = lane_sum(FX), fy = lane_sum(FY), fz = lane_sum(FZ), pa = lane_sum(PA), pb = lane_sum(PB);
            if (jj < c1) pair_mixed<true>(qi, st[jj], k2inv, jj == self, fx, fy, fz, pa, pb);
            two_sum_add(acc[0], fx);
            two_sum_add(acc[1], fy);
            two_sum_add(acc[2], fz);
            ta += pa;
            tb += pb;
          }
        }
        two_sum_add(acc[3], ta);
        two_sum_add(acc[4], tb);
      }
      if (HIST && valid_i) {
        // The self pair (separation 0) is binned with the others, into bin 0
        // in every mode, and taken out of bin 0 once at the end: no per-pair
        // index test.
        const int self = i_local - j0;
        if (self >= jlo && self < jhi) ++nself;
        if (a.hist.mode == 0) {
          // Clamped r^2 bins: most pairs of a box land in the last bin.  They
          // are counted in a register and added once per warp at the end
          // instead of by a same-address shared atomic per pair.
          const int last_bin = a.hist.nb - 1;
#pragma unroll 4
          for (int jj = jlo; jj < jhi; ++jj) {
            const int b = pair_bin(qi, st[jj], k2, a.hist);
            if (b == last_bin) ++nclamp;
            else atomicAdd(&shist[b], 1u);
          }
        } else {
#pragma unroll 4
          for (int jj = jlo; jj < jhi; ++jj) {
            const int b = pair_bin(qi, st[jj], k2, a.hist);
            if (b >= 0) atomicAdd(&shist[b], 1u);
          }
        }
      }
    }
    // This warp is done reading stage s; the last warp done refills it.
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      if (atomicAdd(&done_cnt[s], 1) == NW - 1) {
        done_cnt[s] = 0;
        const int issued = prod[2];
        if (issued < ntiles) {
          const int pB = prod[0], pjt = prod[1];
          const BlockInfo pbi = a.blocks[pB];
          const int pj0 = pjt * TILE;
          const int pcnt = min(TILE, pbi.n_sys - pj0);
          mbar_arrive_expect_tx(&bars[s], (uint32_t)pcnt * 16u);
          bulk_g2s(sq + s * TILE, a.q + pbi.p0 + pj0, (uint32_t)pcnt * 16u, &bars[s]);
          const bool wrap = (pjt + 1 == pbi.njt);
          prod[0] = wrap ? pB + 1 : pB;
          prod[1] = wrap ? 0 : pjt + 1;
          prod[2] = issued + 1;
        }
        __threadfence_block();
      }
    }
    const bool last = (k == ntiles - 1);
    const bool block_end = (jt + 1 == bi.njt);
    if (block_end || last) {
      if (FORCES && valid_i && !failed) {
        const int seg = bi.seg_first + (g - bi.g_first);
        float* out = a.partial + (size_t)seg * 5 * THREADS;
#pragma unroll
        for (int c = 0; c < 5; ++c) out[c * THREADS + tid] = acc[c].hi + acc[c].lo;
      }
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[c] = FloatAcc{0.f, 0.f};
      if (EPI) {
        // Last segment of block B?  (fence, then count; the CTA that
        // completes the count owns the block's epilogue)
        __threadfence();
        __syncthreads();
        if (tid == 0) sflag = !sfail && (atomicAdd(st.blk_cnt + B, 1) == bi.seg_count - 1);
        __syncthreads();
        if (sflag) {
          __threadfence();
          fused_block_step<EPI>(st, B, shd);
          __syncthreads();
          // No per-box stage here: TVN's chi is formed by k_tvn_close from
          // the blocks' sums, and EVN's observables were marked pending at
          // the launch's start.
          if (tid == 0) st.blk_cnt[B] = 0;
        }
      }
      if (block_end && !last) {
        ++B;
        bi = a.blocks[B];
        i_local = bi.i0 + tid;
        valid_i = tid < bi.n_i;
        qi = i_record_slots123(a.q[bi.p0 + (valid_i ? i_local : bi.i0)], &sirec[tid]);
        k2inv = a.sc[bi.sys].k2inv;
        k2 = a.sc[bi.sys].k2;
        jt = 0;
      }
    } else {
      ++jt;
    }
  }

  if (EPI) {
    // This CTA's pair work is done: the first CTAs to get here compute the
    // observables the previous step left pending (one box per ticket), in
    // time the SM would otherwise leave to the CTAs still busy.  The ticket
    // counters alternate by step parity; CTA 0 clears the other one at its
    // start, after the previous step's kernels have completed.
    __shared__ int ticket;
    __syncthreads();
    if (tid == 0) ticket = atomicAdd(st.glob_cnt + st.ticket, 1);
    __syncthreads();
    if (ticket < st.nsys && !sfail) pending_observables(st, ticket, gridDim.x, shd);
    // The dependent kernel of a fused TVN step (k_tvn_close) may be scheduled
    // from here on; it waits for this grid's completion before reading.
    if (EPI == MODE_TVN) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  }
  __syncthreads();
  if (sfail) {
    // Drain the copies still in flight before the CTA's shared memory goes away.
    if (tid == 0) {
      const int issued = prod[2];
      for (int kk = issued - STAGES < 0 ? 0 : issued - STAGES; kk < issued; ++kk)
        mbar_wait_bounded(&bars[kk % STAGES], (uint32_t)((kk / STAGES) & 1));
      atomicOr(a.status, LJ_DEVFLAG_TIMEOUT);
    }
    return;
  }
  if (HIST) {
    const unsigned wclamp = __reduce_add_sync(0xffffffffu, nclamp);
    const unsigned wself = __reduce_add_sync(0xffffffffu, nself);
    if (lane == 0) {
      if (wclamp) atomicAdd(&shist[a.hist.nb - 1], wclamp);
      if (wself) atomicSub(&shist[0], wself);
    }
    __syncthreads();
    for (int b = tid; b < a.hist.nb; b += THREADS)
      if (shist[b]) atomicAdd(a.hist.counts + b, (unsigned long long)shist[b]);
  }
}

template <int THREADS, int TILE, int STAGES, int MINB, bool FORCES, bool HIST>
__global__ void __launch_bounds__(THREADS, MINB) k_pairs_mixed(PairArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  pairs_body<THREADS, TILE, STAGES, FORCES, HIST, 0>(a, StateArgs{}, smem_raw);
}

template <int THREADS, int TILE, int STAGES, int MINB, int EPI>
__global__ void __launch_bounds__(THREADS, MINB) k_pairs_mixed_fused(FusedPairArgs f) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  pairs_body<THREADS, TILE, STAGES, true, false, EPI>(f.pair, f.st, smem_raw);
}

// ---------------------------------------------------------------------------
// All-FP64 persistent pair kernel (the comparator path): double positions,
// minimum image by rint, double accumulators.  Same schedule and partials
// layout (5 doubles per particle per segment).
// ---------------------------------------------------------------------------
template <int THREADS, int TILE, int STAGES>
__global__ void __launch_bounds__(THREADS) k_pairs_fp64(PairArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double4_32a* sx = reinterpret_cast<double4_32a*>(smem_raw);
  __shared__ uint64_t bars[STAGES];

  const int g = blockIdx.x;
  const int tid = threadIdx.x;
  const int t0 = a.cta_tile_begin[g], t1 = a.cta_tile_begin[g + 1];
  const int lo0 = a.cta_lo ? a.cta_lo[g] : 0, lo1 = a.cta_lo ? a.cta_lo[g + 1] : 0;
  const int ntiles = t1 - t0 + (lo1 > 0 ? 1 : 0);
  if (ntiles <= 0) return;
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  int pB = a.cta_block[g], pjt = a.cta_jt[g], issued = 0;
  if (tid == 0) {
    const int pre = ntiles < STAGES ? ntiles : STAGES;
    for (; issued < pre; ++issued) {
      const BlockInfo bi = a.blocks[pB];
      const int j0 = pjt * TILE;
      const int cnt = min(TILE, bi.n_sys - j0);
      const int s = issued % STAGES;
      mbar_arrive_expect_tx(&bars[s], (uint32_t)cnt * 32u);
      bulk_g2s(sx + s * TILE, a.xd + bi.p0 + j0, (uint32_t)cnt * 32u, &bars[s]);
      if (++pjt == bi.njt) { ++pB; pjt = 0; }
    }
  }

  int B = a.cta_block[g], jt = a.cta_jt[g];
  BlockInfo bi = a.blocks[B];
  int i_local = bi.i0 + tid;
  bool valid_i = tid < bi.n_i;
  double4_32a xi = a.xd[bi.p0 + (valid_i ? i_local : bi.i0)];
  BoxArgs box = a.boxes[bi.sys];
  double s2 = box.sigma * box.sigma;
  bool periodic = box.bc == 0;
  double ax = 0., ay = 0., az = 0., aa = 0., ab = 0.;

  int k = 0;
  bool failed = false;
  for (; k < ntiles; ++k) {
    const int s = k % STAGES;
    const bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((k / STAGES) & 1));
    const int j0 = jt * TILE;
    const int cnt = min(TILE, bi.n_sys - j0);
    const int jlo = k == 0 ? lo0 : 0;
    const int jhi = (k == ntiles - 1 && lo1 > 0) ? lo1 : cnt;
    if (ok) {
      const double4_32a* st = sx + s * TILE;
      for (int jj = jlo; jj < jhi; ++jj) {
        const double4_32a xj = st[jj];
        double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        if (periodic) {  // nearest image, ties away from zero (fast_round, MDSystem.cpp:732-739)
          dx = fma(-box.L, round(dx * box.invL), dx);
          dy = fma(-box.L, round(dy * box.invL), dy);
          dz = fma(-box.L, round(dz * box.invL), dz);
        }
        const double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
        double ri = s2 / r2;
        if (j0 + jj == i_local) ri = 0.0;
        const double r6 = ri * ri * ri;
        const double sf = r6 * ri * fma(12.0, r6, -6.0);
        ax = fma(sf, dx, ax);
        ay = fma(sf, dy, ay);
        az = fma(sf, dz, az);
        aa = fma(r6, r6, aa);
        ab += r6;
      }
    }
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    if (tid == 0 && issued < ntiles) {
      const BlockInfo pbi = a.blocks[pB];
      const int pj0 = pjt * TILE;
      const int pcnt = min(TILE, pbi.n_sys - pj0);
      mbar_arrive_expect_tx(&bars[s], (uint32_t)pcnt * 32u);
      bulk_g2s(sx + s * TILE, a.xd + pbi.p0 + pj0, (uint32_t)pcnt * 32u, &bars[s]);
      if (++pjt == pbi.njt) { ++pB; pjt = 0; }
      ++issued;
    }
    const bool last = (k == ntiles - 1);
    const bool block_end = (jt + 1 == bi.njt);
    if (block_end || last) {
      if (valid_i) {
        const int seg = bi.seg_first + (g - bi.g_first);
        double* out = reinterpret_cast<double*>(a.partial) + (size_t)seg * 5 * THREADS;
        out[0 * THREADS + tid] = ax;
        out[1 * THREADS + tid] = ay;
        out[2 * THREADS + tid] = az;
        out[3 * THREADS + tid] = aa;
        out[4 * THREADS + tid] = ab;
      }
      ax = ay = az = aa = ab = 0.;
      if (block_end && !last) {
        ++B;
        bi = a.blocks[B];
        i_local = bi.i0 + tid;
        valid_i = tid < bi.n_i;
        xi = a.xd[bi.p0 + (valid_i ? i_local : bi.i0)];
        box = a.boxes[bi.sys];
        s2 = box.sigma * box.sigma;
        periodic = box.bc == 0;
        jt = 0;
      }
    } else {
      ++jt;
    }
  }
  if (failed && tid == 0) {
    for (int kk = k; kk < issued; ++kk) mbar_wait_bounded(&bars[kk % STAGES], (uint32_t)((kk / STAGES) & 1));
    atomicOr(a.status, LJ_DEVFLAG_TIMEOUT);
  }
}

// ---------------------------------------------------------------------------
// Shape table and launchers.
// ---------------------------------------------------------------------------
namespace {

template <int THREADS, int TILE, int STAGES, int MINB, bool FORCES, bool HIST>
cudaError_t launch_mixed_t(const PairArgs& a, int grid, cudaStream_t st) {
  // <= 48 KB: 16 B x STAGES x TILE staging (+ the histogram's bins, at most
  // 16 KB), no opt-in needed.
  const size_t smem = sizeof(int4) * STAGES * TILE + (HIST ? hist_smem_bytes(a.hist.nb) : 0);
  k_pairs_mixed<THREADS, TILE, STAGES, MINB, FORCES, HIST><<<grid, THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int THREADS, int TILE, int STAGES, int MINB>
cudaError_t launch_fused_t(int mode, const FusedPairArgs& f, int grid, cudaStream_t st) {
  const size_t smem = sizeof(int4) * STAGES * TILE;
  if (mode == MODE_EVN) k_pairs_mixed_fused<THREADS, TILE, STAGES, MINB, MODE_EVN><<<grid, THREADS, smem, st>>>(f);
  else k_pairs_mixed_fused<THREADS, TILE, STAGES, MINB, MODE_TVN><<<grid, THREADS, smem, st>>>(f);
  return cudaGetLastError();
}

template <int THREADS, int TILE, int STAGES, int MINB>
cudaError_t occupancy_mixed_t(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      blocks_per_sm, k_pairs_mixed<THREADS, TILE, STAGES, MINB, true, false>, THREADS,
      sizeof(int4) * STAGES * TILE);
}

// Resident CTAs per SM of the histogram-only variant with nb bins.
template <int THREADS, int TILE, int STAGES, int MINB>
cudaError_t occupancy_hist_t(int nb, int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      blocks_per_sm, k_pairs_mixed<THREADS, TILE, STAGES, MINB, false, true>, THREADS,
      sizeof(int4) * STAGES * TILE + hist_smem_bytes(nb));
}

template <int THREADS, int TILE, int STAGES>
cudaError_t launch_fp64_t(const PairArgs& a, int grid, cudaStream_t st) {
  const size_t smem = sizeof(double4_32a) * STAGES * TILE;
  k_pairs_fp64<THREADS, TILE, STAGES><<<grid, THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int THREADS, int TILE, int STAGES>
cudaError_t occupancy_fp64_t(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pairs_fp64<THREADS, TILE, STAGES>,
                                                       THREADS, sizeof(double4_32a) * STAGES * TILE);
}

}  // namespace

// Kernel shapes the autotuner chooses among (threads = i-block size; MINB =
// resident CTAs per SM the register allocation must allow).
#define LJ_SHAPES(X)   \
  X(0, 128, 256, 3, 6)  \
  X(1, 128, 512, 3, 6)  \
  X(2, 256, 256, 3, 3)  \
  X(3, 256, 512, 3, 3)  \
  X(4, 384, 512, 3, 2)  \
  X(5, 64, 256, 3, 12)

const PairShape kShapes[] = {
#define LJ_SHAPE_ROW(i, T, TL, S, M) {T, TL, S},
    LJ_SHAPES(LJ_SHAPE_ROW)
#undef LJ_SHAPE_ROW
};
const int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

// FP64 i-block and j-tile match MIXED shape 0 so the histogram kernel can
// run on an FP64 handle's schedule.
constexpr int kFp64Threads = 128, kFp64Tile = 256, kFp64Stages = 3;

int fp64_block_threads() { return kFp64Threads; }
int fp64_tile() { return kFp64Tile; }

cudaError_t pair_occupancy(int prec, int shape, int* blocks_per_sm) {
  if (prec == 1) return occupancy_fp64_t<kFp64Threads, kFp64Tile, kFp64Stages>(blocks_per_sm);
  switch (shape) {
#define LJ_OCC_CASE(i, T, TL, S, M) \
  case i:                           \
    return occupancy_mixed_t<T, TL, S, M>(blocks_per_sm);
    LJ_SHAPES(LJ_OCC_CASE)
#undef LJ_OCC_CASE
  }
  return cudaErrorInvalidValue;
}

cudaError_t pair_hist_occupancy(int shape, int nb, int* blocks_per_sm) {
  switch (shape) {
#define LJ_HOCC_CASE(i, T, TL, S, M) \
  case i:                            \
    return occupancy_hist_t<T, TL, S, M>(nb, blocks_per_sm);
    LJ_SHAPES(LJ_HOCC_CASE)
#undef LJ_HOCC_CASE
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_pairs(int prec, int shape, bool forces, bool hist, const PairArgs& a, int grid,
                         cudaStream_t st) {
  if (prec == 1) return launch_fp64_t<kFp64Threads, kFp64Tile, kFp64Stages>(a, grid, st);
  switch (shape) {
#define LJ_LAUNCH_CASE(i, T, TL, S, M)                                                  \
  case i:                                                                               \
    if (forces && !hist) return launch_mixed_t<T, TL, S, M, true, false>(a, grid, st); \
    if (forces && hist) return launch_mixed_t<T, TL, S, M, true, true>(a, grid, st);   \
    return launch_mixed_t<T, TL, S, M, false, true>(a, grid, st);
    LJ_SHAPES(LJ_LAUNCH_CASE)
#undef LJ_LAUNCH_CASE
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_pairs_fused(int shape, int mode, const FusedPairArgs& f, int grid, cudaStream_t st) {
  switch (shape) {
#define LJ_FUSED_CASE(i, T, TL, S, M) \
  case i:                             \
    return launch_fused_t<T, TL, S, M>(mode, f, grid, st);
    LJ_SHAPES(LJ_FUSED_CASE)
#undef LJ_FUSED_CASE
  }
  return cudaErrorInvalidValue;
}

}  // namespace ljgb
