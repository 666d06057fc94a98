// lj_integrate.cu -- FP64 integrator, boundary, observable and histogram kernels.
//
// Replaces the host loops of MDSystem::Integrate (src/library/MDSystem.cpp:438-510),
// ApplyBoundaryConditions (:406-436), CalculateParameters (:325-359),
// KineticTemperature (:361-373) and initvelo/updatevelo (:651-694).
//
// Layout: positions, velocities, forces are FP64, component-major
// (x[0..npad) | y | z) so every access of a warp is one coalesced 256-byte
// segment.  Work is split in the same i-blocks as the pair kernel (one CTA per
// block).  Every global sum is reduced in a fixed order (block partials, then
// blocks in index order), so results do not depend on scheduling.
#include <cuda_runtime.h>

#include <cstdint>

#include "lj_device.cuh"
#include "lj_kernels.h"
#include "lj_stepdev.cuh"

namespace ljgb {

namespace {

constexpr int kObsThreads = 256;

__device__ __forceinline__ void store_shadow(const StateArgs& s, const DevScalars& sc, int p, double x,
                                             double y, double z, const BoxArgs& box) {
  check_wall_frame(s, box.bc, sc, x, y, z);
  int4 q;
  q.x = fixed_coord(x, sc.origin[0], sc.invP);
  q.y = fixed_coord(y, sc.origin[1], sc.invP);
  q.z = fixed_coord(z, sc.origin[2], sc.invP);
  q.w = 0;
  s.q[p] = q;
  s.xd[p] = make_double4_32a(x, y, z, 0.0);
}

// Block-wide min/max of the positions (for the fixed-point frame of walls /
// open boxes); result in blk_part[B][0..5].
__device__ __forceinline__ void block_bbox(const StateArgs& s, int B, bool valid, const double (&x)[3],
                                           double* sh) {
  double lo[3], hi[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    lo[c] = valid ? x[c] : 1e300;
    hi[c] = valid ? x[c] : -1e300;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fmin(lo[c], __shfl_down_sync(0xffffffffu, lo[c], o));
      hi[c] = fmax(hi[c], __shfl_down_sync(0xffffffffu, hi[c], o));
    }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      sh[c * 32 + warp] = lo[c];
      sh[(3 + c) * 32 + warp] = hi[c];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int c = 0; c < 3; ++c) {
      double a = 1e300, b = -1e300;
      for (int w = 0; w < nw; ++w) {
        a = fmin(a, sh[c * 32 + w]);
        b = fmax(b, sh[(3 + c) * 32 + w]);
      }
      s.blk_part[(size_t)B * 8 + c] = a;
      s.blk_part[(size_t)B * 8 + 3 + c] = b;
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// First half of the Verlet step (MDSystem.cpp:443-454 EVN, :469-480 TVN):
//   x += dt v + dt^2 F/2;  EVN: v += dt F/2;  TVN: tF = F/2.
// Writes the position shadow for periodic boxes; for walls / open boxes it
// writes the block bounding box instead (the frame follows in k_frame).
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void k_drift(StateArgs s) {
  __shared__ double sh[6 * 32];
  const int B = blockIdx.x;
  const BlockInfo bi = s.blocks[B];
  const bool valid = (int)threadIdx.x < bi.n_i;
  const int p = bi.p0 + bi.i0 + threadIdx.x;
  const BoxArgs box = s.boxes[bi.sys];
  double x[3] = {0., 0., 0.};
  if (valid) {
    double v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * s.npad + p;
      const double f = s.f[k];
      v[c] = s.v[k];
      x[c] = drift_pos(box, s.x[k], v[c], f);
      s.x[k] = x[c];
      if (MODE == MODE_EVN) s.v[k] = fma(box.hdt, f, v[c]);
      if (MODE == MODE_TVN) s.tf[k] = 0.5 * f;
    }
    if (box.bc == 0) store_shadow(s, s.sc[bi.sys], p, x[0], x[1], x[2], box);
  }
  if (box.bc != 0) block_bbox(s, B, valid, x, sh);
}

// Bounding box of the current positions (initial / injected state).
__global__ void k_bbox(StateArgs s) {
  __shared__ double sh[6 * 32];
  const int B = blockIdx.x;
  const BlockInfo bi = s.blocks[B];
  const bool valid = (int)threadIdx.x < bi.n_i;
  const int p = bi.p0 + bi.i0 + threadIdx.x;
  double x[3] = {0., 0., 0.};
  if (valid)
#pragma unroll
    for (int c = 0; c < 3; ++c) x[c] = s.x[(size_t)c * s.npad + p];
  block_bbox(s, B, valid, x, sh);
}

// Fixed-point frame per box: origin and period P such that every position
// maps into [0, P/2) (no pair separation wraps), except for periodic boxes.
// Also the FP32 scale constants of the pair kernel.
//   periodic: origin 0, period L (the wrap is the minimum image);
//   walls:    the bounding box of the positions joined with [0, L], widened
//             by m = max(sigma, L/20) on every side, P = 2.002 x its largest
//             extent.  A wall turns a particle back within a step or two of
//             crossing it, so the frame stays valid while the fused step
//             keeps it fixed; a position outside it sets LJ_DEVFLAG_ESCAPED
//             (check_wall_frame, wherever a shadow is written);
//   open:     origin at the bounding-box minimum, P = 2.002 x the largest
//             extent, recomputed after every drift.
// The bounding box comes from the block partials blk_part[b][0..5]
// (k_bbox, or k_drift of the kernel-per-phase step).
__global__ void k_frame(StateArgs s, int only_nonperiodic) {
  __shared__ double sh[32];
  const int sys = blockIdx.x;
  const BoxArgs box = s.boxes[sys];
  if (only_nonperiodic && box.bc == 0) return;
  const int b0 = s.sys_block_first[sys], b1 = s.sys_block_first[sys + 1];
  double origin[3] = {0., 0., 0.};
  double P = box.L;
  if (box.bc != 0) {
    double lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
      // min/max over blocks (order-independent)
      double a = 1e300, b = -1e300;
      for (int k = b0 + (int)threadIdx.x; k < b1; k += blockDim.x) {
        a = fmin(a, s.blk_part[(size_t)k * 8 + c]);
        b = fmax(b, s.blk_part[(size_t)k * 8 + 3 + c]);
      }
      for (int o = 16; o > 0; o >>= 1) {
        a = fmin(a, __shfl_down_sync(0xffffffffu, a, o));
        b = fmax(b, __shfl_down_sync(0xffffffffu, b, o));
      }
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      __syncthreads();
      if (lane == 0) {
        sh[warp] = a;
        sh[16 + warp] = b;
      }
      __syncthreads();
      a = 1e300;
      b = -1e300;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        a = fmin(a, sh[w]);
        b = fmax(b, sh[16 + w]);
      }
      if (box.bc == 1) {
        a = fmin(a, 0.0) - box.wall_margin;
        b = fmax(b, box.L) + box.wall_margin;
      }
      lo[c] = a;
      hi[c] = b;
    }
    double ext = 0.0;
    for (int c = 0; c < 3; ++c) ext = fmax(ext, hi[c] - lo[c]);
    P = 2.002 * ext + 1e-3 * box.sigma;
    for (int c = 0; c < 3; ++c) origin[c] = lo[c];
  }
  if (threadIdx.x == 0) {
    DevScalars& sc = s.sc[sys];
    for (int c = 0; c < 3; ++c) sc.origin[c] = origin[c];
    sc.P = P;
    sc.invP = 1.0 / P;
    const double ks = P / (4294967296.0 * box.sigma);
    sc.k2 = (float)(ks * ks);
    sc.k2inv = (float)(1.0 / (ks * ks));
    sc.fscale = 4.0 * box.eps * ks / box.sigma;
  }
}

// Writes the fixed-point and FP64 shadows from the FP64 positions.
__global__ void k_quantize(StateArgs s, int only_nonperiodic) {
  const int B = blockIdx.x;
  const BlockInfo bi = s.blocks[B];
  if (only_nonperiodic && s.boxes[bi.sys].bc == 0) return;
  if ((int)threadIdx.x >= bi.n_i) return;
  const int p = bi.p0 + bi.i0 + threadIdx.x;
  store_shadow(s, s.sc[bi.sys], p, s.x[p], s.x[(size_t)s.npad + p], s.x[2 * (size_t)s.npad + p], s.boxes[bi.sys]);
}

// ---------------------------------------------------------------------------
// Sum of the pair-kernel segments into FP64 forces and per-particle sums,
// then (EVN) the second half-kick + boundaries, or (TVN) the averaged force
// and the half-kicked velocity whose kinetic temperature sets chi.
// Block partials: [0] K, [1] V, [2] W, [3] sum tv^2.
// ---------------------------------------------------------------------------
template <int MODE, int PREC>
__global__ void k_reduce(StateArgs s) {
  __shared__ double sh[4 * 32];
  const int B = blockIdx.x;
  const BlockInfo bi = s.blocks[B];
  const int tid = threadIdx.x;
  const bool valid = tid < bi.n_i;
  const int p = bi.p0 + bi.i0 + tid;
  const BoxArgs box = s.boxes[bi.sys];
  double part[4] = {0., 0., 0., 0.};
  if (valid) {
    double S[5] = {0., 0., 0., 0., 0.};
    if (PREC == 0) {
      segment_sums(s, bi, tid, S);
    } else {
      const double* pd = reinterpret_cast<const double*>(s.partial);
      for (int k = 0; k < bi.seg_count; ++k) {
        const size_t base = (size_t)(bi.seg_first + k) * 5 * s.bi_threads + tid;
#pragma unroll
        for (int c = 0; c < 5; ++c) S[c] += pd[base + (size_t)c * s.bi_threads];
      }
    }
    const double fs = (PREC == 0) ? s.sc[bi.sys].fscale : 4.0 * box.eps / (box.sigma * box.sigma);
    double F[3] = {fs * S[0], fs * S[1], fs * S[2]};
    const double e = box.eps4 * (S[3] - S[4]);
    const double w = box.eps4 * fma(12.0, S[3], -6.0 * S[4]);
    s.e[p] = e;
    s.w[p] = w;
    part[1] = 0.5 * e;
    part[2] = w;
    double x[3], v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * s.npad + p;
      s.f[k] = F[c];
      v[c] = s.v[k];
    }
    if (MODE == MODE_FORCES_ONLY) {
      part[0] = 0.5 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    } else if (MODE == MODE_EVN) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c] = fma(box.hdt, F[c], v[c]);
        x[c] = s.x[(size_t)c * s.npad + p];
      }
      apply_bc(box.bc, box.L, x, v);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        s.v[(size_t)c * s.npad + p] = v[c];
        if (box.bc == 0) s.x[(size_t)c * s.npad + p] = x[c];
      }
      part[0] = 0.5 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    } else {  // TVN
      double tv2 = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t k = (size_t)c * s.npad + p;
        const double tf = s.tf[k] + 0.5 * F[c];
        s.tf[k] = tf;
        const double tv = fma(box.hdt, tf, v[c]);
        tv2 = fma(tv, tv, tv2);
      }
      part[3] = tv2;
    }
  }
  block_sum<4>(part, sh);
  if (tid == 0) {
#pragma unroll
    for (int c = 0; c < 4; ++c) s.blk_part[(size_t)B * 8 + c] = part[c];
  }
}

// TVN velocity update (MDSystem.cpp:498-506): chi = sqrt(T0 / Tkin(tv)),
// v = (2 chi - 1) v + chi dt tF, then boundaries; block partial [0] = K.
__global__ void k_tvn_finish(StateArgs s) {
  __shared__ double sh[32];
  __shared__ double chi_sh;
  const int B = blockIdx.x;
  const BlockInfo bi = s.blocks[B];
  const int tid = threadIdx.x;
  const BoxArgs box = s.boxes[bi.sys];
  const int b0 = s.sys_block_first[bi.sys], b1 = s.sys_block_first[bi.sys + 1];
  const double tv2 = box_sum(s, b0, b1, 3, sh);
  if (tid == 0) {
    double Tkin;
    const double chi = tvn_chi(box, tv2, &Tkin);
    chi_sh = chi;
    if (B == b0) {
      s.sc[bi.sys].Tkin = Tkin;
      s.sc[bi.sys].chi = chi;
    }
  }
  __syncthreads();
  const double chi = chi_sh;
  double part[1] = {0.0};
  if (tid < bi.n_i) {
    const int p = bi.p0 + bi.i0 + tid;
    double x[3], v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * s.npad + p;
      v[c] = fma(2. * chi - 1., s.v[k], chi * box.dt * s.tf[k]);
      x[c] = s.x[k];
    }
    apply_bc(box.bc, box.L, x, v);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * s.npad + p;
      s.v[k] = v[c];
      if (box.bc == 0) s.x[k] = x[c];
    }
    part[0] = 0.5 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  }
  __syncthreads();
  block_sum<1>(part, sh);
  if (tid == 0) s.blk_part[(size_t)B * 8 + 0] = part[0];
}

// CalculateParameters (MDSystem.cpp:325-359) per box (one CTA per box).
template <int MODE>
__global__ void k_observables(StateArgs s) {
  __shared__ double sh[3 * 32];
  observables_box<MODE>(s, blockIdx.x, sh);
}

// Predictor of the fused step: the shadow of x + dt v + dt^2 F / 2 (the
// positions the next pair kernel evaluates), periodic and walled boxes.
__global__ void k_predict(StateArgs s) {
  const BlockInfo bi = s.blocks[blockIdx.x];
  if ((int)threadIdx.x >= bi.n_i) return;
  const int p = bi.p0 + bi.i0 + threadIdx.x;
  const BoxArgs box = s.boxes[bi.sys];
  double xp[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = (size_t)c * s.npad + p;
    xp[c] = drift_pos(box, s.x[k], s.v[k], s.f[k]);
  }
  const DevScalars& sc = s.sc[bi.sys];
  check_wall_frame(s, box.bc, sc, xp[0], xp[1], xp[2]);
  s.q[p] = shadow_of(sc, xp[0], xp[1], xp[2]);
}

// Close of a fused TVN step (MDSystem.cpp:469-506, :578-579).  The pair
// kernel's epilogue left F_{n+1} in s.tf (s.f still holds F_n), e and w, and
// each block's sum of the half-kicked velocities' squares; chi of the box is
// formed here from those.  Per particle: x_{n+1} = drift_pos(x_n, v_n, F_n),
// tF = F_n/2 + F_{n+1}/2, v = (2 chi - 1) v + chi dt tF, boundaries,
// F <- F_{n+1}, the next step's predictor, and block partials K, V, W.
// The observables of the step (sums over blocks, averages, record) are left
// pending in this step's parity entry: the next step's pair kernel computes
// them in a CTA that has finished its pair work (pending_observables), or
// the read-back launch / k_obs_finalize does before the host reads them.
// This takes a serial last-CTA stage off the step's critical path.
__global__ void k_tvn_close(StateArgs s) {
  __shared__ double sh[3 * 32];
  // Launched as a programmatic dependent of the pair kernel: the CTAs start
  // while the pair grid drains.  What the pair kernel does not write (the
  // block table, the box, x, v and F_n) is loaded before waiting for its
  // writes (F_{n+1} in tf, e, w, the blocks' sums) to become visible.
  const int B = blockIdx.x;
  const BlockInfo bi = s.blocks[B];
  const int tid = threadIdx.x;
  const BoxArgs box = s.boxes[bi.sys];
  const bool valid = tid < bi.n_i;
  const int p = bi.p0 + bi.i0 + (valid ? tid : 0);
  double xn[3], vn[3], fn[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = (size_t)c * s.npad + p;
    xn[c] = s.x[k];
    vn[c] = s.v[k];
    fn[c] = s.f[k];
  }
  const int b0 = s.sys_block_first[bi.sys], b1 = s.sys_block_first[bi.sys + 1];
  asm volatile("griddepcontrol.wait;" ::: "memory");
  DevScalars& sc = s.sc[bi.sys];
  // The pair kernel's results for this particle, loaded before chi's sum so
  // that both wait on memory together.
  double f1[3], ep = 0.0, wp = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) f1[c] = s.tf[(size_t)c * s.npad + p];
  if (valid) {
    ep = s.e[p];
    wp = s.w[p];
  }
  // chi of the box (MDSystem.cpp:498-499) from its blocks' sums of the
  // half-kicked velocities' squares (slot 3, written by the pair kernel's
  // block epilogues): every CTA of the box forms the same sum in the same
  // order (as k_tvn_finish does), so no CTA of the pair kernel has to wait
  // for the box's last block to compute it.
  __shared__ double chi_sh, tkin_sh;
  if (b1 - b0 <= 32) {
    // Boxes of at most 32 blocks (batches of small boxes): warp 0 alone.
    // box_sum would give every block value to one thread of warp 0 and zeros
    // to the other warps, then add 0 + w0 + 0 + ...: the same bits as
    // 0 + w0, with a quarter of the FP64 work (this kernel is FP64-bound on
    // batches).
    if (tid < 32) {
      double v = b0 + tid < b1 ? __ldcg(s.blk_part + (size_t)(b0 + tid) * 8 + 3) : 0.0;
      v = warp_sum(v);
      if (tid == 0) {
        double Tkin;
        chi_sh = tvn_chi(box, 0.0 + v, &Tkin);
        tkin_sh = Tkin;
      }
    }
    __syncthreads();
  } else {
    const double tv2 = box_sum(s, b0, b1, 3, sh);
    if (tid == 0) {
      double Tkin;
      chi_sh = tvn_chi(box, tv2, &Tkin);
      tkin_sh = Tkin;
    }
    __syncthreads();
  }
  const double chi = chi_sh;
  // chi dt tF with tF = (F_n + F_{n+1}) / 2 formed as (chi dt / 2)(F_n + F_{n+1}):
  // the same bits (the halvings are exact), one FP64 operation fewer
  const double a1 = 2. * chi - 1., b1h = 0.5 * (chi * box.dt);
  double part[3] = {0.0, 0.0, 0.0};
  if (valid) {
    double x[3], v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      x[c] = drift_pos(box, xn[c], vn[c], fn[c]);
      v[c] = fma(a1, vn[c], b1h * (fn[c] + f1[c]));
    }
    apply_bc(box.bc, box.L, x, v);
    double xp[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * s.npad + p;
      s.v[k] = v[c];
      s.x[k] = x[c];
      s.f[k] = f1[c];
      xp[c] = drift_pos(box, x[c], v[c], f1[c]);
    }
    check_wall_frame(s, box.bc, sc, xp[0], xp[1], xp[2]);
    s.q_next[p] = shadow_of_bc(sc, box.bc, xp[0], xp[1], xp[2]);
    part[0] = fma(v[0], v[0], fma(v[1], v[1], v[2] * v[2]));  // K and V shares, halved once per block below
    part[1] = ep;
    part[2] = wp;
  }
  block_sum<3>(part, sh);
  if (tid == 0) {
    // halving the block sums gives the bits of summing halved terms
    s.blk_part[(size_t)B * 8 + 0] = 0.5 * part[0];
    s.blk_part[(size_t)B * 8 + 1] = 0.5 * part[1];
    s.blk_part[(size_t)B * 8 + 2] = part[2];
    if (B == s.sys_block_first[bi.sys]) {
      const int par = s.ticket - 2;  // this step's parity
      sc.Tkin = tkin_sh;
      sc.Tkin_rec[par] = tkin_sh;
      sc.chi = chi;
      sc.obs_slot[par] = 0;
      sc.obs_pending[par] = MODE_TVN;
    }
  }
}

// Observables left pending by the last fused steps, EVN or TVN (one CTA per
// box).
__global__ void k_obs_finalize(StateArgs s) {
  __shared__ double sh[3 * 32];
  pending_observables_all(s, blockIdx.x, gridDim.x, sh);
}

// Subsystem counters of the fluctuation task (run-fluctuations-aux.h:124-273,
// GetNSubsystemBatch / GetNsubVzBatch): per particle and counter, the index
// of the first alpha whose subsystem contains it; the host turns the
// histogram into cumulative counts N(alpha_k).
//   slab (type t < 3):  k = (int)((x_t / L) / alpha_step)   (bin_trunc_div2)
//   cube (type 3):      k = max over axes of #{tl_j <= |x_c - L/2| / 0.5}
//   velocity (4 .. 6):  k = (int)((|v_c| / vmax) / alpha_step)
// (int)((a / b) / c) for b, c > 0: the bin index as the reference forms it
// (two separately rounded divisions, truncated toward zero), with the
// divisions skipped where they cannot change the result.  a * inv_bc
// (inv_bc = 1 / (b c) from the host) is within 1e-15 of that quotient,
// relatively; where q (1 - 1e-12) and q (1 + 1e-12) truncate to the same
// integer, so does the reference's quotient.  The divisions (a long FP64
// sequence each, at 1/64 of the FP32 rate on this part) run only next to a
// bin edge.
__device__ __forceinline__ int bin_trunc_div2(double a, double b, double c, double inv_bc) {
  const double q = a * inv_bc;
  const int lo = (int)(q * (1.0 - 1e-12)), hi = (int)(q * (1.0 + 1e-12));
  if (lo == hi) return lo;
  return (int)((a / b) / c);
}

// d >= e for non-negative, non-NaN doubles, on their bit patterns (integer
// pipe): such doubles order like their bits as signed integers.
__device__ __forceinline__ bool ge_nonneg(double d, double e) {
  return __double_as_longlong(d) >= __double_as_longlong(e);
}

// One launch per step, graph-capturable (everything that changes per step
// lives in st, the kCtr* words).  Whether the step is counted (every
// `every`-th step) is read at the start by every CTA; st is written only by
// the last CTA to finish, after every CTA has taken its ticket.  A counted
// step: each CTA histograms its particles in shared memory and writes its
// counts to part[block][bin]; the last CTA sums the blocks' counts into the
// step's ring row (written whole: no clearing pass) and advances the row.
__global__ void k_counters(StateArgs s, const CounterDev* cs, int nc, int nbins, int* st, int* ring, int* part,
                           int n) {
  extern __shared__ int shc[];
  __shared__ bool last;
  const int phase = st[kCtrPhase] + 1;
  const bool counted = phase >= st[kCtrEvery];
  if (counted) {
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) shc[b] = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
      const double L = s.boxes[0].L;
      double x[3], v[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        x[c] = s.x[(size_t)c * s.npad + i];
        v[c] = s.v[(size_t)c * s.npad + i];
      }
      for (int q = 0; q < nc; ++q) {
        const CounterDev& cd = cs[q];
        int k;
        if (cd.type < 3) {
          k = bin_trunc_div2(x[cd.type], L, cd.alpha_step, cd.inv_bc);
        } else if (cd.type == 3) {
          k = 0;
          for (int c = 0; c < 3; ++c) {
            const double d = fabs(x[c] - 0.5 * L) * 2.0;  // = / 0.5, exactly
            int kc = 0;
            while (kc < cd.nalpha && ge_nonneg(d, cd.tl[kc])) ++kc;
            k = kc > k ? kc : k;
          }
        } else {
          k = bin_trunc_div2(fabs(v[cd.type - 4]), cd.vmax, cd.alpha_step, cd.inv_bc);
        }
        if (k >= 0 && k < cd.nalpha) atomicAdd(&shc[cd.bin0 + k], 1);
      }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) part[(size_t)blockIdx.x * nbins + b] = shc[b];
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&st[kCtrTicket], 1) == (int)gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int row = st[kCtrNext];
  if (counted)
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
      int sum = 0;
      for (int k = 0; k < (int)gridDim.x; ++k) sum += __ldcg(part + (size_t)k * nbins + b);
      ring[(size_t)row * nbins + b] = sum;
    }
  if (threadIdx.x == 0) {
    st[kCtrTicket] = 0;
    st[kCtrPhase] = counted ? 0 : phase;
    if (counted) st[kCtrNext] = row + 1 == st[kCtrCap] ? 0 : row + 1;
  }
}

// |v| histogram (MDSystem.cpp:658-662): b = floor(sqrt(v.v)/step), b < nb.
// Products and sums rounded separately so the bins are reproducible on a CPU.
__global__ void k_velocity_hist(StateArgs s, double step, int nb, unsigned long long* counts) {
  __shared__ unsigned hist[kMaxHistBins];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) hist[b] = 0u;
  __syncthreads();
  const BlockInfo bi = s.blocks[blockIdx.x];
  int bin = -1;
  if ((int)threadIdx.x < bi.n_i) {
    const int p = bi.p0 + bi.i0 + threadIdx.x;
    const double vx = s.v[p], vy = s.v[(size_t)s.npad + p], vz = s.v[2 * (size_t)s.npad + p];
    double q = __dmul_rn(vx, vx);
    q = __dadd_rn(q, __dmul_rn(vy, vy));
    q = __dadd_rn(q, __dmul_rn(vz, vz));
    const double b = floor(__ddiv_rn(__dsqrt_rn(q), step));
    if (b < (double)nb) bin = (int)b;
  }
  // warp-aggregated: the lanes with the same bin add once (speeds cluster
  // in a few bins around sqrt(2 T))
  const unsigned peers = __match_any_sync(0xffffffffu, bin);
  if (bin >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&hist[bin], (unsigned)__popc(peers));
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (hist[b]) atomicAdd(counts + b, (unsigned long long)hist[b]);
}

// sysmode 0: v *= factor.  sysmode 1: block partial [0] = sum v^2 / 2 (for
// RenormalizeVelocities with Tkin recomputed).
__global__ void k_velocities(StateArgs s, int sysmode, double factor) {
  __shared__ double sh[32];
  const int B = blockIdx.x;
  const BlockInfo bi = s.blocks[B];
  double part[1] = {0.0};
  if ((int)threadIdx.x < bi.n_i) {
    const int p = bi.p0 + bi.i0 + threadIdx.x;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * s.npad + p;
      const double v = s.v[k];
      if (sysmode == 0) s.v[k] = v * factor;
      part[0] += v * v;
    }
    part[0] *= 0.5;
  }
  if (sysmode == 1) {
    block_sum<1>(part, sh);
    if (threadIdx.x == 0) s.blk_part[(size_t)B * 8 + 0] = part[0];
  }
}

// Interleaved (x,y,z per particle) <-> component-major, all boxes at once.
__global__ void k_unpack(const double* __restrict__ in, double* __restrict__ out, int n, int npad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int c = 0; c < 3; ++c) out[(size_t)c * npad + i] = in[3 * (size_t)i + c];
}

// Up to three component-major [3][npad] -> (N,3) transposes in one launch;
// blockIdx.y selects the array.  Thread k writes element k of the (N,3)
// output (consecutive threads, consecutive doubles: whole-line stores, which
// matters when the destination is host memory written over the chip-to-chip
// link) and gathers it from the device array.  With a mailbox, the row after
// the arrays copies the status words and the scalar block into the handle's
// page-locked mirrors (destinations may be mapped host memory: the host reads
// them after one synchronisation, with no copy operation queued); with
// mb.finalize it first computes the observables a fused TVN step left
// pending, as k_obs_finalize would, one CTA per box (one launch fewer per
// read-back after a step).  With mb.seq the last CTA to finish writes a
// completion word for the host to wait on.
__device__ __forceinline__ void mailbox_row(const Mailbox& mb, const StateArgs& s) {
  const int nb = mb.finalize ? s.nsys : 1;
  if ((int)blockIdx.x >= nb) return;
  if (mb.finalize) {
    // The observables k_obs_finalize would compute (box blockIdx.x), then
    // that box's scalar block; the status words follow once every box is
    // done, since a box's observables may flag the status.
    __shared__ double sh[3 * 32];
    __shared__ int last;
    pending_observables_all(s, blockIdx.x, nb, sh);
    const int wb = mb.sc_nwords / nb;
    for (int k = threadIdx.x; k < wb; k += blockDim.x) mb.sc_out[blockIdx.x * wb + k] = mb.sc[blockIdx.x * wb + k];
    if (nb > 1) {
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) last = atomicAdd(mb.ticket, 1) == nb - 1;
      __syncthreads();
      if (!last) return;
      if (threadIdx.x == 0) *mb.ticket = 0;
    }
  } else {
    for (int k = threadIdx.x; k < mb.sc_nwords; k += blockDim.x) mb.sc_out[k] = mb.sc[k];
  }
  if (threadIdx.x == 0) {
    mb.words_out[0] = *(volatile const int*)mb.status;
    if (mb.bad) {
      mb.words_out[1] = *mb.bad;
      *mb.bad = 0x7f7f7f7f;  // read: ready for the next upload's check
    }
  }
}

__global__ void k_pack_multi(XyzArrays a, int count, int n, int npad, Mailbox mb, StateArgs s) {
  if ((int)blockIdx.y == count) {
    mailbox_row(mb, s);
  } else {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < 3 * n) {
      const int i = k / 3, c = k - 3 * i;
      a.dst[blockIdx.y][k] = a.src[blockIdx.y][(size_t)c * npad + i];
    }
  }
  if (mb.seq) {
    // every thread's stores before its CTA's count (a fence orders only the
    // calling thread's own stores)
    __threadfence_system();
    __syncthreads();
    if (threadIdx.x == 0) {
      if (atomicAdd(mb.grid_ticket, 1) == (int)(gridDim.x * gridDim.y) - 1) {
        *mb.grid_ticket = 0;
        __threadfence_system();
        *(volatile int*)(mb.words_out + 2) = mb.seq;
      }
    }
  }
}

// First half of an upload: (N,3) positions (blockIdx.y = 0) and velocities
// (1), either possibly host memory mapped into the device's address space,
// read once with whole-line loads; each value is checked (lowest index of a
// non-finite value into *bad, velocities after the na position values) and
// written component-major into the staging buffer.
__global__ void k_upload_stage(const double* __restrict__ pos, const double* __restrict__ vel, int n, int npad,
                               double* __restrict__ spos, double* __restrict__ svel, int na, int* bad) {
  // k_upload_commit, launched as a programmatic dependent, may be scheduled
  // from here on: it waits for this grid's completion before reading.
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const double* src = blockIdx.y == 0 ? pos : vel;
  if (!src || k >= 3 * n) return;
  const double x = src[k];
  if (!isfinite(x)) atomicMin(bad, blockIdx.y == 0 ? k : na + k);
  const int i = k / 3, c = k - 3 * i;
  (blockIdx.y == 0 ? spos : svel)[(size_t)c * npad + i] = x;
}

// Second half, one thread per particle on the i-block decomposition: the
// staged arrays become the state unless a value was not finite (all or
// nothing).  With `predict` (periodic boxes on the fused step) the same thread
// then writes the next pair kernel's shadow x + dt v + dt^2 F / 2, as
// k_predict does, so the first step after an upload needs no predictor launch.
__global__ void k_upload_commit(StateArgs s, const double* __restrict__ spos, const double* __restrict__ svel,
                                const int* bad, int predict) {
  // Launched as a programmatic dependent of k_upload_stage: what the stage
  // does not write (block table, state, forces) is loaded before waiting for
  // its grid to complete.
  const BlockInfo bi = s.blocks[blockIdx.x];
  const bool valid = (int)threadIdx.x < bi.n_i;
  const int p = bi.p0 + bi.i0 + (valid ? (int)threadIdx.x : 0);
  double x[3], v[3], f[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = (size_t)c * s.npad + p;
    x[c] = s.x[k];
    v[c] = s.v[k];
    f[c] = predict ? s.f[k] : 0.0;
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (!valid) return;
  const bool ok = *bad == 0x7f7f7f7f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = (size_t)c * s.npad + p;
    if (ok && spos) {
      x[c] = spos[k];
      s.x[k] = x[c];
    }
    if (ok && svel) {
      v[c] = svel[k];
      s.v[k] = v[c];
    }
  }
  if (!predict) return;
  const BoxArgs box = s.boxes[bi.sys];
  double xp[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) xp[c] = drift_pos(box, x[c], v[c], f[c]);
  s.q[p] = shadow_of(s.sc[bi.sys], xp[0], xp[1], xp[2]);
}

// A wait that nothing completes: the pair kernels' bounded mbarrier wait must
// give up after its limit, flag LJ_DEVFLAG_TIMEOUT and let the kernel return.
__global__ void k_selftest_wait(int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!mbar_wait_bounded(&bar, 0)) atomicOr(status, LJ_DEVFLAG_TIMEOUT);
    mbar_inval(&bar);
  }
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
cudaError_t launch_selftest_wait(int* status, cudaStream_t st) {
  k_selftest_wait<<<1, 32, 0, st>>>(status);
  return cudaGetLastError();
}

cudaError_t launch_unpack(const double* in, double* out, int n, int npad, cudaStream_t st) {
  k_unpack<<<(n + 255) / 256, 256, 0, st>>>(in, out, n, npad);
  return cudaGetLastError();
}

cudaError_t launch_pack_multi(const XyzArrays& a, int count, int n, int npad, const Mailbox* mb, const StateArgs& s,
                              cudaStream_t st) {
  const int rows = count + (mb ? 1 : 0);
  if (rows <= 0) return cudaSuccess;
  int gx = (3 * n + 255) / 256;
  if (mb && mb->finalize && gx < s.nsys) gx = s.nsys;
  k_pack_multi<<<dim3(gx, rows), 256, 0, st>>>(a, count, n, npad, mb ? *mb : Mailbox{}, s);
  return cudaGetLastError();
}

cudaError_t launch_upload_stage(const double* pos, const double* vel, int n, int npad, double* spos, double* svel,
                                int* bad, cudaStream_t st) {
  if (!pos && !vel) return cudaSuccess;
  const int na = pos ? 3 * n : 0;
  k_upload_stage<<<dim3((3 * n + 255) / 256, 2), 256, 0, st>>>(pos, vel, n, npad, spos, svel, na, bad);
  return cudaGetLastError();
}

cudaError_t launch_upload_commit(const StateArgs& s, int nblocks, int bi, const double* spos, const double* svel,
                                 const int* bad, bool predict, cudaStream_t st) {
  // programmatic dependent of the stage launch queued just before it
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(bi);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_upload_commit, s, spos, svel, bad, predict ? 1 : 0);
}

cudaError_t launch_drift_mode(const StateArgs& s, int nblocks, int bi, int mode, cudaStream_t st) {
  if (mode == MODE_EVN) k_drift<MODE_EVN><<<nblocks, bi, 0, st>>>(s);
  else k_drift<MODE_TVN><<<nblocks, bi, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_bbox(const StateArgs& s, int nblocks, int bi, cudaStream_t st) {
  k_bbox<<<nblocks, bi, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_frame(const StateArgs& s, int nsys, bool only_nonperiodic, cudaStream_t st) {
  k_frame<<<nsys, kObsThreads, 0, st>>>(s, only_nonperiodic ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_quantize(const StateArgs& s, int nblocks, int bi, bool only_nonperiodic, cudaStream_t st) {
  k_quantize<<<nblocks, bi, 0, st>>>(s, only_nonperiodic ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_reduce(const StateArgs& s, int nblocks, int bi, int mode, cudaStream_t st) {
  if (s.prec == 0) {
    if (mode == MODE_FORCES_ONLY) k_reduce<MODE_FORCES_ONLY, 0><<<nblocks, bi, 0, st>>>(s);
    else if (mode == MODE_EVN) k_reduce<MODE_EVN, 0><<<nblocks, bi, 0, st>>>(s);
    else k_reduce<MODE_TVN, 0><<<nblocks, bi, 0, st>>>(s);
  } else {
    if (mode == MODE_FORCES_ONLY) k_reduce<MODE_FORCES_ONLY, 1><<<nblocks, bi, 0, st>>>(s);
    else if (mode == MODE_EVN) k_reduce<MODE_EVN, 1><<<nblocks, bi, 0, st>>>(s);
    else k_reduce<MODE_TVN, 1><<<nblocks, bi, 0, st>>>(s);
  }
  return cudaGetLastError();
}

cudaError_t launch_tvn_finish(const StateArgs& s, int nblocks, int bi, cudaStream_t st) {
  k_tvn_finish<<<nblocks, bi, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_observables(const StateArgs& s, int nsys, int mode, cudaStream_t st) {
  if (mode == MODE_FORCES_ONLY) k_observables<MODE_FORCES_ONLY><<<nsys, kObsThreads, 0, st>>>(s);
  else if (mode == MODE_EVN) k_observables<MODE_EVN><<<nsys, kObsThreads, 0, st>>>(s);
  else k_observables<MODE_TVN><<<nsys, kObsThreads, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_predict(const StateArgs& s, int nblocks, int bi, cudaStream_t st) {
  k_predict<<<nblocks, bi, 0, st>>>(s);
  return cudaGetLastError();
}

int counters_blocks(int n) { return (n + 255) / 256; }

cudaError_t launch_counters(const StateArgs& s, const CounterDev* cs, int nc, int nbins, int* state, int* ring,
                            int* part, int n, cudaStream_t st) {
  k_counters<<<counters_blocks(n), 256, sizeof(int) * nbins, st>>>(s, cs, nc, nbins, state, ring, part, n);
  return cudaGetLastError();
}

cudaError_t launch_obs_finalize(const StateArgs& s, int nsys, cudaStream_t st) {
  k_obs_finalize<<<nsys, kObsThreads, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_tvn_close(const StateArgs& s, int nblocks, int bi, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(bi);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_tvn_close, s);
}

cudaError_t launch_velocity_hist(const StateArgs& s, int nblocks, int bi, double step, int nb,
                                 unsigned long long* counts, cudaStream_t st) {
  k_velocity_hist<<<nblocks, bi, 0, st>>>(s, step, nb, counts);
  return cudaGetLastError();
}

cudaError_t launch_scale_velocities(const StateArgs& s, int nblocks, int bi, int sysmode, double factor,
                                    cudaStream_t st) {
  k_velocities<<<nblocks, bi, 0, st>>>(s, sysmode, factor);
  return cudaGetLastError();
}

}  // namespace ljgb
