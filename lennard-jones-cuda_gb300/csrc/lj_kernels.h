// lj_kernels.h -- launch interface of the LJ kernels (host side).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lj_internal.h"

namespace ljgb {

constexpr int kMaxHistBins = 4096;
// Shared-memory histogram of a pair-kernel CTA: nb 32-bit bins, rounded up to
// 16 bytes.
constexpr size_t hist_smem_bytes(int nb) { return (sizeof(unsigned) * (size_t)nb + 15) / 16 * 16; }

// Pair-histogram request.  mode 0: r^2 bins, clamp overflow to the last bin
// (MDSystem.cu:39); 1: r^2 bins, drop overflow (MDSystem.cpp:282-284);
// 2: linear r bins up to rmax (pairs with r >= rmax dropped).
struct HistArgs {
  int mode;
  int nb;
  float inv_w;   // 1/dr2 (modes 0,1) or 1/dr (mode 2)
  float rmax2;   // mode 2: rmax^2 in sigma^2
  unsigned long long* counts;  // nb counters (global, accumulated with atomics)
};

// Arguments of the persistent pair kernels (by value).
struct PairArgs {
  const int4* q;              // MIXED: fixed-point shadow (x, y, z, pad), all boxes
  const double4_32a* xd;          // FP64: position shadow (x, y, z, 0)
  const BlockInfo* blocks;    // i-blocks of the schedule
  const int* cta_tile_begin;  // G+1 tile ranges
  const int* cta_block;       // first i-block of each CTA
  const int* cta_jt;          // first j-tile (within that block) of each CTA
  const int* cta_lo;          // G+1 j offsets within the first tile (entry g+1: end in the
                              // last tile, 0 = whole tile); nullptr = whole tiles only
  const DevScalars* sc;       // per box frame / scalars
  const BoxArgs* boxes;       // per box constants
  float* partial;             // nseg x 5 x threads  (float, or double for FP64)
  int* status;                // device status word (timeouts)
  HistArgs hist;
};


struct PairShape {
  int threads;  // CTA size = i-block length (one i per thread)
  int tile;     // j records per staged tile
  int stages;   // depth of the bulk-copy ring
};

extern const PairShape kShapes[];
extern const int kNumShapes;
int fp64_block_threads();
int fp64_tile();

cudaError_t pair_occupancy(int prec, int shape, int* blocks_per_sm);
// Resident CTAs per SM of the MIXED histogram-only pair kernel with nb bins.
cudaError_t pair_hist_occupancy(int shape, int nb, int* blocks_per_sm);
cudaError_t launch_pairs(int prec, int shape, bool forces, bool hist, const PairArgs& a, int grid,
                         cudaStream_t st);
struct FusedPairArgs;
cudaError_t launch_pairs_fused(int shape, int mode, const FusedPairArgs& a, int grid, cudaStream_t st);

// ---------------------------------------------------------------------------
// Integrator / reduction kernels (lj_integrate.cu).  All operate on the
// i-block decomposition: grid = number of blocks, blockDim = BI.
// ---------------------------------------------------------------------------
struct StateArgs {
  double* x;        // 3 x Npad, component-major (x | y | z)
  double* v;        // 3 x Npad
  double* f;        // 3 x Npad, forces
  double* tf;       // 3 x Npad, TVN averaged force (F_old + F_new)/2
  double* e;        // Npad per-particle pair energy sum  4eps sum [(s/r)^12-(s/r)^6]
  double* w;        // Npad per-particle virial sum  sum r.f
  int4* q;          // fixed-point shadow
  double4_32a* xd;      // FP64 position shadow
  int npad;         // stride between components
  const BlockInfo* blocks;
  const BoxArgs* boxes;
  DevScalars* sc;
  const int* sys_block_first;  // nsys + 1
  double* blk_part;            // nblocks x 8 partial sums
  const float* partial;        // pair-kernel partials
  int prec;                    // LJ_PREC_*
  int bi_threads;              // threads of the pair kernel's i-block (partial stride)
  DevRecord* records;          // per box ring (rec_cap entries each)
  int rec_stride;              // ring capacity per box
  int* status;
  int4* q_next;                // fused step: predictor shadow for the next step
  int* blk_cnt;                // fused step: segments finished per i-block
  int* glob_cnt;               // fused step: [2 + parity] pending-observables tickets
  int nblocks;                 // i-blocks of all boxes
  int nsys;                    // boxes
  int obs_slot;                // fused EVN: first block-partial slot of this step's K, V, W (0 or 4, by parity)
  int ticket;                  // fused: glob_cnt index of this step's pending-observables tickets (2 or 3)
};

enum StepMode { MODE_FORCES_ONLY = 0, MODE_EVN = 1, MODE_TVN = 2 };

// The pair kernel with the second half of the Verlet step fused into the
// last CTA of every i-block (epi = MODE_EVN or MODE_TVN).
struct FusedPairArgs {
  PairArgs pair;
  StateArgs st;
};

cudaError_t launch_drift_mode(const StateArgs& s, int nblocks, int bi, int mode, cudaStream_t st);
cudaError_t launch_bbox(const StateArgs& s, int nblocks, int bi, cudaStream_t st);
cudaError_t launch_frame(const StateArgs& s, int nsys, bool only_nonperiodic, cudaStream_t st);
cudaError_t launch_quantize(const StateArgs& s, int nblocks, int bi, bool only_nonperiodic, cudaStream_t st);
cudaError_t launch_reduce(const StateArgs& s, int nblocks, int bi, int mode, cudaStream_t st);
cudaError_t launch_tvn_finish(const StateArgs& s, int nblocks, int bi, cudaStream_t st);
cudaError_t launch_observables(const StateArgs& s, int nsys, int mode, cudaStream_t st);
cudaError_t launch_velocity_hist(const StateArgs& s, int nblocks, int bi, double step, int nb,
                                 unsigned long long* counts, cudaStream_t st);
cudaError_t launch_predict(const StateArgs& s, int nblocks, int bi, cudaStream_t st);
cudaError_t launch_tvn_close(const StateArgs& s, int nblocks, int bi, cudaStream_t st);
cudaError_t launch_obs_finalize(const StateArgs& s, int nsys, cudaStream_t st);

// Fixed-point shadow of caller-owned float4 positions (lj_compat.cu), for the
// reference ABI and the allocation-free force entry point.  bbox writes one
// 8-double partial per kFloat4Threads positions (grid = ceil(n / 256)); frame
// reads nb such partials (non-periodic boxes) and clears *status if given.
constexpr int kFloat4Threads = 256;
cudaError_t launch_float4_bbox(const float4* pos, int n, double* blk, cudaStream_t st);
cudaError_t launch_float4_frame(const double* blk, int nb, int periodic, double L, DevScalars* sc, int* status,
                                cudaStream_t st);
cudaError_t launch_float4_quantize(const float4* pos, int n, const DevScalars* sc, int4* q, cudaStream_t st);

// Headless particle image (lj_render.cu): splat + shade into rgba (device).
cudaError_t launch_render(const double* x, int npad, int p0, int n, int axis, int W, int H, double L, double R,
                          unsigned long long* key, uint8_t* rgba, cudaStream_t st);

// Subsystem counters of the fluctuation runs (lj_counters_configure).
constexpr int kMaxCounterAlphas = 64;
struct CounterDev {
  int type;    // 0/1/2 slab x/y/z < alpha L; 3 cube around the centre; 4/5/6 |v_x|/|v_y|/|v_z| < alpha vmax
  int nalpha;  // alphas k = 0 .. nalpha-1
  int bin0;    // first bin of this counter in the per-step row
  int pad;
  double alpha_step;
  double vmax;
  double inv_bc;                 // 1 / (L alpha_step) (types 0-2) or 1 / (vmax alpha_step) (types 4-6)
  double tl[kMaxCounterAlphas];  // type 3: cube sides L alpha_k^(1/3)
};
// Device words of the counters (DevBuf<int> of kCtrWords): next ring row,
// steps since the last counted one, the interval, the ring's rows, and the
// per-launch ticket counter (0 between launches).
enum : int { kCtrNext = 0, kCtrPhase = 1, kCtrEvery = 2, kCtrCap = 3, kCtrTicket = 4, kCtrWords = 8 };
// One step of the counters in one launch (graph-capturable: everything that
// changes per step lives in `state`): the histogram of the counters' bin
// indices over the particles of box 0, per CTA into part (counters_blocks(n)
// x nbins ints), summed by the last CTA into the step's ring row when the
// step is counted.
int counters_blocks(int n);
cudaError_t launch_counters(const StateArgs& s, const CounterDev* cs, int nc, int nbins, int* state, int* ring,
                            int* part, int n, cudaStream_t st);
cudaError_t launch_unpack(const double* in, double* out, int n, int npad, cudaStream_t st);
cudaError_t launch_selftest_wait(int* status, cudaStream_t st);
// Up to three (N,3) interleaved <-> component-major [3][npad] transposes in one launch.
struct XyzArrays {
  const double* src[3];
  double* dst[3];
};
// Small device words copied by the pack launch: the status word (and the
// upload check's bad index, if bad is set, which is then reset to 0x7f7f7f7f)
// to words_out[0..1], and sc_nwords 32-bit words of the scalar block to sc_out.
struct Mailbox {
  const int* status;
  int* bad;
  int* words_out;
  const int* sc;
  int* sc_out;
  int sc_nwords;
  int finalize;  // != 0: compute the observables the last fused TVN step left pending first (one CTA per box)
  int* ticket;   // finalize with several boxes: the last box's CTA copies the status words (0 between launches)
  // seq != 0: the launch's last CTA writes seq into words_out[2] once every
  // store of the launch is visible to the host (grid_ticket: CTAs done, 0
  // between launches), so the host can wait on that word alone.
  int* grid_ticket;
  int seq;
};
// `s` is read only with mb->finalize.
cudaError_t launch_pack_multi(const XyzArrays& a, int count, int n, int npad, const Mailbox* mb, const StateArgs& s,
                              cudaStream_t st);
// Upload of (N,3) positions / velocities (either may be NULL; either may be
// mapped host memory), in two launches.  Stage: every value checked (*bad
// receives the lowest index of a non-finite value, velocities after the 3n
// position values; it must hold 0x7f7f7f7f before) and written component-major
// to spos / svel ([3][npad] each).  Commit (grid = i-blocks): the staged
// arrays become x / v only if every value was finite; with `predict`, also
// the fused step's shadow of x + dt v + dt^2 F / 2 into s.q (periodic boxes).
cudaError_t launch_upload_stage(const double* pos, const double* vel, int n, int npad, double* spos, double* svel,
                                int* bad, cudaStream_t st);
cudaError_t launch_upload_commit(const StateArgs& s, int nblocks, int bi, const double* spos, const double* svel,
                                 const int* bad, bool predict, cudaStream_t st);
cudaError_t launch_scale_velocities(const StateArgs& s, int nblocks, int bi, int sysmode, double target,
                                    cudaStream_t st);

}  // namespace ljgb
