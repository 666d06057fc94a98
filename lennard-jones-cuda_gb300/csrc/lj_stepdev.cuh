// lj_stepdev.cuh -- device pieces of the Verlet step shared by the integrator
// kernels (lj_integrate.cu) and the fused epilogue of the pair kernel
// (lj_pairs.cu): boundaries, the fixed-point predictor, per-block segment
// reduction + kick, and the per-box observables of CalculateParameters.
#pragma once

#include <cuda_runtime.h>

#include "lj_device.cuh"
#include "lj_kernels.h"

namespace ljgb {

// Sign and order tests of FP64 values on their bit patterns (integer pipe;
// the FP64 pipe issues at 1/64 of the FP32 rate on this part).  For x not
// NaN: x < 0 exactly when the bits are negative as a signed integer and not
// those of -0.0; x > L (L > 0) exactly when the bits are larger than L's.
// For NaN both forms leave NaN behind, so results agree bit for bit.
__device__ __forceinline__ bool neg_bits(double x) {
  const long long b = __double_as_longlong(x);
  return b < 0 && b != (long long)0x8000000000000000ull;
}
__device__ __forceinline__ bool above_bits(double x, long long Lbits) { return __double_as_longlong(x) > Lbits; }

// ApplyBoundaryConditions (MDSystem.cpp:406-436) for one coordinate: wrap
// (periodic) or reflect the velocity (walls); open boxes leave both alone.
__device__ __forceinline__ void apply_bc1(int bc, double L, double& x, double& v) {
  const long long Lbits = __double_as_longlong(L);
  if (bc == 0) {
    if (neg_bits(x)) x += L;
    if (above_bits(x, Lbits)) x -= L;
  } else if (bc == 1) {
    // v = -v is a flip of the sign bit
    if (neg_bits(x) && neg_bits(v)) v = __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull);
    if (above_bits(x, Lbits) && __double_as_longlong(v) > 0)
      v = __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull);
  }
}

// ApplyBoundaryConditions for one particle.
__device__ __forceinline__ void apply_bc(int bc, double L, double (&x)[3], double (&v)[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) apply_bc1(bc, L, x[c], v[c]);
}

// x + dt v + dt^2 F / 2: the drift of MDSystem.cpp:445 / :472, and the
// predictor of the next step's positions.  Every kernel that drifts or
// predicts calls this one form, so a prediction and the drift it stands for
// agree bit for bit.
__device__ __forceinline__ double drift_pos(const BoxArgs& b, double x, double v, double f) {
  return fma(b.hdt2, f, fma(b.dt, v, x));
}

// chi = sqrt(T0 / Tkin) with Tkin = sum tv^2 / (3 N) (MDSystem.cpp:498-499),
// as rsqrt(Tkin / T0): no FP64 division on the step's critical path.
__device__ __forceinline__ double tvn_chi(const BoxArgs& b, double tv2, double* Tkin_out) {
  const double Tkin = tv2 * b.inv3N;
  *Tkin_out = Tkin;
  return b.T0 > 0 ? rsqrt(Tkin * b.invT0) : sqrt(b.T0 / Tkin);
}

// Walled boxes keep their fixed-point frame between frame updates (k_frame):
// a position outside [0, P/2) of it could wrap in the fixed-point
// differences, so it is flagged (the quantisation moves a coordinate by at
// most one unit, hence the slightly smaller bound).
__device__ __forceinline__ void check_wall_frame(const StateArgs& s, int bc, const DevScalars& sc, double x,
                                                 double y, double z) {
  if (bc != 1) return;
  const double ux = (x - sc.origin[0]) * sc.invP, uy = (y - sc.origin[1]) * sc.invP,
               uz = (z - sc.origin[2]) * sc.invP;
  constexpr double kHi = 0.4999;
  if (!(ux >= 0.0 && ux < kHi && uy >= 0.0 && uy < kHi && uz >= 0.0 && uz < kHi))
    atomicOr(s.status, LJ_DEVFLAG_ESCAPED);
}

__device__ __forceinline__ int4 shadow_of(const DevScalars& sc, double x, double y, double z) {
  return make_int4(fixed_coord(x, sc.origin[0], sc.invP), fixed_coord(y, sc.origin[1], sc.invP),
                   fixed_coord(z, sc.origin[2], sc.invP), 0);
}

// shadow_of for a box of boundary bc with the frame scale formed once; a
// periodic box's frame has origin 0, so its subtraction is skipped (x - 0 is
// x exactly): the same bits as shadow_of.
__device__ __forceinline__ int4 shadow_of_bc(const DevScalars& sc, int bc, double x, double y, double z) {
  const double scale = sc.invP * 4294967296.0;
  if (bc == 0) return make_int4(fixed_coord_scaled(x, scale), fixed_coord_scaled(y, scale), fixed_coord_scaled(z, scale), 0);
  return make_int4(fixed_coord_scaled(x - sc.origin[0], scale), fixed_coord_scaled(y - sc.origin[1], scale),
                   fixed_coord_scaled(z - sc.origin[2], scale), 0);
}

// Sum of blk_part[b][slot] over the blocks of one box, fixed order, valid in
// thread 0 (every CTA that calls this obtains the same bits).
__device__ __forceinline__ double box_sum(const StateArgs& s, int b0, int b1, int slot, double* sh) {
  double acc[1] = {0.0};
  for (int b = b0 + (int)threadIdx.x; b < b1; b += blockDim.x) acc[0] += __ldcg(s.blk_part + (size_t)b * 8 + slot);
  block_sum<1>(acc, sh);
  return acc[0];
}

// Sums of blk_part[b][0..2] (K, V, W) over the blocks of one box in one
// block reduction (fixed order); valid in thread 0.  sh: 3 x 32 doubles.
__device__ __forceinline__ void box_sum3(const StateArgs& s, int b0, int b1, double* sh, double (&out)[3],
                                         int slot = 0) {
  double acc[3] = {0.0, 0.0, 0.0};
  for (int b = b0 + (int)threadIdx.x; b < b1; b += blockDim.x) {
    const double* bp = s.blk_part + (size_t)b * 8 + slot;
    acc[0] += __ldcg(bp);
    acc[1] += __ldcg(bp + 1);
    acc[2] += __ldcg(bp + 2);
  }
  block_sum<3>(acc, sh);
  out[0] = acc[0];
  out[1] = acc[1];
  out[2] = acc[2];
}

// CalculateParameters (MDSystem.cpp:325-359) for box `sys`, plus t += dt for
// steps (MDSystem.cpp:582) and the optional per-step record.  Block-wide call;
// thread 0 writes.  sh: 3 x 32 doubles.
// rec_parity >= 0: the record's Tkin is Tkin_rec[rec_parity] (TVN steps
// whose observables were left pending), else the box's Tkin.
template <int MODE>
__device__ __forceinline__ void observables_box(const StateArgs& s, int sys, double* sh, int slot = 0,
                                                int rec_parity = -1) {
  const BoxArgs box = s.boxes[sys];
  const int b0 = s.sys_block_first[sys], b1 = s.sys_block_first[sys + 1];
  double kvw[3];
  box_sum3(s, b0, b1, sh, kvw, slot);
  const double K = kvw[0], V = kvw[1], W = kvw[2];
  if (threadIdx.x != 0) return;
  DevScalars& sc = s.sc[sys];
  const double N = (double)box.N;
  const double T = K * box.kT;                           // 2 K / 3 / N
  const double P = fma(W, 1. / 6., N * T) * box.kP;      // (W / 6 + N T) / (N / rho)
  const double U = K + V;
  sc.K = K;
  sc.V = V;
  sc.W = W;
  sc.T = T;
  sc.P_press = P;
  sc.U = U;
  if (MODE != MODE_TVN) sc.Tkin = 0.0;
  if (MODE != MODE_FORCES_ONLY) {
    sc.t += box.dt;
    sc.step += 1;
  }
  sc.av_iters += 1;
  sc.av_U += U;
  sc.av_p += P;
  sc.av_T += T;
  if (!isfinite(K) || !isfinite(V) || !isfinite(W)) atomicOr(s.status, LJ_DEVFLAG_NONFINITE);
  if (sc.rec_cap > 0 && MODE != MODE_FORCES_ONLY) {
    DevRecord& r = s.records[(size_t)sys * s.rec_stride + (size_t)(sc.rec_count % sc.rec_cap)];
    r.t = sc.t;
    r.K = K;
    r.V = V;
    r.T = T;
    r.P = P;
    r.U = U;
    r.W = W;
    r.Pshear = sc.Pshear;
    r.Tkin = (MODE == MODE_TVN && rec_parity >= 0) ? sc.Tkin_rec[rec_parity] : sc.Tkin;
    r.av_U = sc.av_U;
    r.av_T = sc.av_T;
    r.av_p = sc.av_p;
    r.av_iters = sc.av_iters;
    r.step = sc.step;
    sc.rec_count += 1;
  }
}

// Observables of the boxes whose fused step of parity `parity` left them
// pending (block partials K, V, W from k_tvn_close or the EVN epilogues, at
// obs_slot[parity]).  Called with a ticket from 0 .. tickets-1; ticket k
// takes boxes k, k + tickets, ...  Block-wide call.
__device__ __forceinline__ void pending_observables_parity(const StateArgs& s, int parity, int ticket, int tickets,
                                                           double* sh) {
  __shared__ int pend, slot;
  for (int sys = ticket; sys < s.nsys; sys += tickets) {
    if (threadIdx.x == 0) {
      pend = s.sc[sys].obs_pending[parity];
      slot = s.sc[sys].obs_slot[parity];
    }
    __syncthreads();
    if (pend == MODE_TVN) observables_box<MODE_TVN>(s, sys, sh, slot, parity);
    else if (pend == MODE_EVN) observables_box<MODE_EVN>(s, sys, sh, slot);
    if (pend && threadIdx.x == 0) s.sc[sys].obs_pending[parity] = 0;
    __syncthreads();
  }
}

// In a fused step's pair kernel: the previous step's (the other parity's).
static __device__ __noinline__ void pending_observables(const StateArgs& s, int ticket, int tickets, double* sh) {
  pending_observables_parity(s, (s.ticket - 2) ^ 1, ticket, tickets, sh);
}

// Everything still pending, the older step first: the step before the last
// fused one has parity s.ticket - 2 (the current parity), the last one the
// other.  Normally only the last is left; the next step's pair kernel
// consumes the one before it.
static __device__ __noinline__ void pending_observables_all(const StateArgs& s, int ticket, int tickets,
                                                            double* sh) {
  const int q = s.ticket - 2;
  pending_observables_parity(s, q, ticket, tickets, sh);
  pending_observables_parity(s, q ^ 1, ticket, tickets, sh);
}

// Sum of a particle's pair-kernel segments (5 values each).  The partials are
// FP32 values carrying TwoSum-compensated sums; they are added here in FP32
// TwoSum too (exact up to the low word's rounding) and converted to FP64 once,
// instead of ~10 conversions and additions per value on the FP64 pipe.
__device__ __forceinline__ void segment_sums(const StateArgs& s, const BlockInfo& bi, int tid, double (&S)[5]) {
  FloatAcc acc[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) acc[c] = FloatAcc{0.f, 0.f};
#pragma unroll 4
  for (int k = 0; k < bi.seg_count; ++k) {
    const size_t base = (size_t)(bi.seg_first + k) * 5 * s.bi_threads + tid;
#pragma unroll
    for (int c = 0; c < 5; ++c) two_sum_add(acc[c], __ldcg(s.partial + base + (size_t)c * s.bi_threads));
  }
#pragma unroll
  for (int c = 0; c < 5; ++c) S[c] = (double)acc[c].hi + (double)acc[c].lo;
}

// Fused second half of a step for block B, run by the CTA that wrote the last
// pair-kernel segment of the block (blockDim.x = the i-block length).
// Starts from the state at the beginning of the step (x_n, v_n, F_n); the
// forces of this step were computed at x_{n+1} = drift_pos(x_n, v_n, F_n),
// the predictor written by the previous step.
//   EVN (MDSystem.cpp:443-463): x_{n+1}; v_{n+1} = v_n + dt F_n/2 +
//       dt F_{n+1}/2; boundaries; the predictor of the next step into
//       q_next.  Block partials K, V, W at obs_slot .. obs_slot + 2 (the
//       slots alternate by step parity: the next step's epilogues write
//       while its first-finishing CTAs read this step's).
//   TVN (MDSystem.cpp:469-497): only what chi needs before any velocity can
//       be set -- F_{n+1} (kept in s.tf until k_tvn_close moves it to s.f),
//       e, w, and the half-kicked velocity's sum of squares in partial [3].
//       The drift, rescale, boundaries and predictor follow in k_tvn_close,
//       which runs on every SM at once.
// This code runs on whichever CTA finishes a block last, often several
// blocks on one SM at the end of the pair kernel, and FP64 runs at 1/64 of
// the FP32 rate here: the FP64 instruction count is kept to the minimum.
// Not inlined: compiled into the pair kernel's loop body, its register needs
// changed the allocation of the pair loop and cost 8% of the kernel's time
// (A/B on GB300, N=16384); as a call it leaves the loop as it is.
template <int MODE>
__device__ __noinline__ void fused_block_step(const StateArgs& s, int B, double* sh) {
  const BlockInfo bi = s.blocks[B];
  const int tid = threadIdx.x;
  const bool valid = tid < bi.n_i;
  const int p = bi.p0 + bi.i0 + tid;
  const BoxArgs box = s.boxes[bi.sys];
  const DevScalars& sc = s.sc[bi.sys];
  constexpr int NP = MODE == MODE_EVN ? 3 : 1;
  double part[NP];
#pragma unroll
  for (int c = 0; c < NP; ++c) part[c] = 0.0;
  if (valid) {
    double S[5];
    segment_sums(s, bi, tid, S);
    const double fs = sc.fscale;
    const double Fn1[3] = {fs * S[0], fs * S[1], fs * S[2]};
    const double e = box.eps4 * (S[3] - S[4]);
    const double w = box.eps4 * fma(12.0, S[3], -6.0 * S[4]);
    s.e[p] = e;
    s.w[p] = w;
    if constexpr (MODE == MODE_EVN) {
      double xp[3], vv = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {  // one component at a time: few live FP64 registers
        const size_t k = (size_t)c * s.npad + p;
        const double Fn = s.f[k];
        double v = s.v[k];
        double x = drift_pos(box, s.x[k], v, Fn);
        v = fma(box.hdt, Fn1[c], fma(box.hdt, Fn, v));
        apply_bc1(box.bc, box.L, x, v);
        s.f[k] = Fn1[c];
        s.x[k] = x;
        s.v[k] = v;
        xp[c] = drift_pos(box, x, v, Fn1[c]);
        vv = fma(v, v, vv);
      }
      check_wall_frame(s, box.bc, sc, xp[0], xp[1], xp[2]);
      s.q_next[p] = shadow_of_bc(sc, box.bc, xp[0], xp[1], xp[2]);
      part[0] = vv;  // K and V shares, halved once per block below
      part[1] = e;
      part[2] = w;
    } else {
      double tv2 = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t k = (size_t)c * s.npad + p;
        // v + dt/2 (F_n + F_{n+1})/2 as v + dt/4 (F_n + F_{n+1}): the same
        // bits (the halvings are exact), one FP64 operation fewer
        const double tv = fma(box.qdt, s.f[k] + Fn1[c], s.v[k]);
        s.tf[k] = Fn1[c];
        tv2 = fma(tv, tv, tv2);
      }
      part[0] = tv2;
    }
  }
  block_sum<NP>(part, sh);
  if (tid == 0) {
    if constexpr (MODE == MODE_EVN) {
      // halving the block sums gives the bits of summing halved terms
      s.blk_part[(size_t)B * 8 + s.obs_slot + 0] = 0.5 * part[0];
      s.blk_part[(size_t)B * 8 + s.obs_slot + 1] = 0.5 * part[1];
      s.blk_part[(size_t)B * 8 + s.obs_slot + 2] = part[2];
    } else {
      s.blk_part[(size_t)B * 8 + 3] = part[0];
    }
  }
}

}  // namespace ljgb
