// lj_adjoint.cu -- differentiable MD: gradients of a time-averaged loss of
// the EVN velocity-Verlet trajectory with respect to eps, sigma and the
// initial positions / velocities, by a discrete adjoint.
//
// The reference has no adjoint.  The dynamics differentiated are its EVN
// step (src/library/MDSystem.cpp:443-463, periodic boundaries :406-436) with
// all-pairs minimum-image forces, generalised from the hard-coded
// eps = sigma = 1 (MDSystem.cu:44-53, MDSystem.cpp:289-298) to explicit
// 4 eps [(sigma/r)^12 - (sigma/r)^6].  Everything is FP64: the gradients are
// checked against central finite differences of this same forward pass.
//
//   loss = (1/S) sum_{m=1..S} [ wK K_m/N + wV V_m/N + wP P_m ]
//
// Forward: S steps from (x_0, v_0), keeping (x, v, F) every k steps.
// Backward: segments of k steps from the last checkpoint down; each segment
// is replayed forward (bit-identical kernels) into a (k+1)-state buffer, then
// swept in reverse.  With Xb_{S+1} = bb_{S+1} = 0, for m = S..0:
//   bb_m = dl_m/dv_m + dt Xb_{m+1} + bb_{m+1}
//   z_m  = dt^2/2 Xb_{m+1} + dt/2 bb_{m+1} (+ dt/2 bb_m for m > 0)
//   Xb_m = dl_m/dx_m + Xb_{m+1} + H(x_m) z_m,   H = dF/dx (symmetric)
//   d/d(eps, sigma) += G(x_m)^T z_m + dl_m/d(eps, sigma),  G = dF/d(eps, sigma)
// dloss/dx_0 = Xb_0, dloss/dv_0 = bb_0.  One pair pass per reverse step
// gives F, dF/dsigma, H z and the energy / virial sums at x_m.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "lj_device.cuh"
#include "lj_gb300.h"
#include "lj_init.h"

namespace ljgb {
namespace {

constexpr int kAdjThreads = 128;  // i per CTA of the pair pass (and of the per-particle kernels)
constexpr int kAdjTile = 64;      // j records staged in shared memory per tile
constexpr int kParts = 12;        // per-i sums: F(3), dF/dsigma(3), Hz(3), e, w, dw/dsigma

struct AdjBox {
  int n, npad;
  double L, invL;
  double eps4, sigma2, inv_sigma;
};

// All-pairs pass over j in [blockIdx.y * jchunk, +jchunk) for the i of this
// CTA (one i per thread), minimum image d = d - L rint(d / L).  Per pair,
// with s6 = (sigma^2/r^2)^3, s12 = s6^2:
//   f = g d,  g = 4 eps (12 s12 - 6 s6) / r^2
//   dg/dsigma = 4 eps (144 s12 - 36 s6) / (sigma r^2)
//   H z: J (z_i - z_j),  J = g I + (g'/r) d d^T,  g'/r = 4 eps (-168 s12 + 48 s6) / r^4
// Partial sums go to part[blockIdx.y][c][i] (summed in a fixed order later).
template <bool HVP>
__global__ void __launch_bounds__(kAdjThreads) k_adj_pairs(AdjBox b, const double* __restrict__ x,
                                                           const double* __restrict__ z, int jchunk,
                                                           double* __restrict__ part) {
  __shared__ double sx[3][kAdjTile];
  __shared__ double sz[3][HVP ? kAdjTile : 1];
  const int i = blockIdx.x * kAdjThreads + threadIdx.x;
  const int j0 = blockIdx.y * jchunk;
  const int j1 = min(b.n, j0 + jchunk);
  const bool valid = i < b.n;
  double xi[3], zi[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    xi[c] = valid ? x[(size_t)c * b.npad + i] : 0.0;
    zi[c] = (HVP && valid) ? z[(size_t)c * b.npad + i] : 0.0;
  }
  double acc[kParts];
#pragma unroll
  for (int c = 0; c < kParts; ++c) acc[c] = 0.0;
  for (int t0 = j0; t0 < j1; t0 += kAdjTile) {
    const int cnt = min(kAdjTile, j1 - t0);
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += kAdjThreads) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sx[c][k] = x[(size_t)c * b.npad + t0 + k];
        if (HVP) sz[c][k] = z[(size_t)c * b.npad + t0 + k];
      }
    }
    __syncthreads();
    if (!valid) continue;
    for (int k = 0; k < cnt; ++k) {
      if (t0 + k == i) continue;
      double d[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double t = xi[c] - sx[c][k];
        d[c] = fma(-b.L, rint(t * b.invL), t);
      }
      const double r2 = fma(d[2], d[2], fma(d[1], d[1], d[0] * d[0]));
      const double inv = 1.0 / r2;
      const double s2 = b.sigma2 * inv;
      const double s6 = s2 * s2 * s2;
      const double s12 = s6 * s6;
      const double u = fma(12.0, s12, -6.0 * s6);
      const double g = b.eps4 * u * inv;
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] = fma(g, d[c], acc[c]);
      acc[9] += s12 - s6;
      acc[10] += u;
      if (HVP) {
        const double us = fma(144.0, s12, -36.0 * s6);
        const double gs = b.eps4 * us * inv * b.inv_sigma;
        const double h = b.eps4 * fma(-168.0, s12, 48.0 * s6) * inv * inv;
        double dz[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) dz[c] = zi[c] - sz[c][k];
        const double hd = h * fma(d[2], dz[2], fma(d[1], dz[1], d[0] * dz[0]));
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          acc[3 + c] = fma(gs, d[c], acc[3 + c]);
          acc[6 + c] = fma(g, dz[c], fma(hd, d[c], acc[6 + c]));
        }
        acc[11] += us;
      }
    }
  }
  if (!valid) return;
  acc[9] *= b.eps4;
  acc[10] *= b.eps4;
  acc[11] *= b.eps4 * b.inv_sigma;
  double* out = part + (size_t)blockIdx.y * kParts * b.npad + i;
#pragma unroll
  for (int c = 0; c < kParts; ++c)
    if (HVP || c < 3 || c == 9 || c == 10) out[(size_t)c * b.npad] = acc[c];
}

// Sum of part[js][c][i] over js = 0..JS-1 (fixed order).
__device__ __forceinline__ double part_sum(const double* part, int JS, int npad, int c, int i) {
  double s = 0.0;
  for (int js = 0; js < JS; ++js) s += part[((size_t)js * kParts + c) * npad + i];
  return s;
}

// x += dt v + dt^2 F / 2; v += dt F / 2; single +-L wrap.
__global__ void k_adj_drift(AdjBox b, double* x, double* v, const double* f, double dt) {
  const int i = blockIdx.x * kAdjThreads + threadIdx.x;
  if (i >= b.n) return;
  const double hdt = 0.5 * dt, hdt2 = 0.5 * dt * dt;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = (size_t)c * b.npad + i;
    const double fc = f[k], vc = v[k];
    double xc = fma(hdt2, fc, fma(dt, vc, x[k]));
    if (xc < 0.) xc += b.L;
    if (xc > b.L) xc -= b.L;
    x[k] = xc;
    v[k] = fma(hdt, fc, vc);
  }
}

// F = pair sums; with kick: v += dt F / 2.  Block partials (K, V, W) into
// blk[blockIdx.x * 3 + 0..2] when blk is non-null.
__global__ void k_adj_forces(AdjBox b, const double* part, int JS, double* f, double* v, double hdt, double* blk) {
  __shared__ double sh[3 * 32];
  const int i = blockIdx.x * kAdjThreads + threadIdx.x;
  double p[3] = {0.0, 0.0, 0.0};
  if (i < b.n) {
    double vv = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * b.npad + i;
      const double fc = part_sum(part, JS, b.npad, c, i);
      f[k] = fc;
      if (v) {
        const double vc = fma(hdt, fc, v[k]);
        v[k] = vc;
        vv = fma(vc, vc, vv);
      }
    }
    p[0] = 0.5 * vv;
    p[1] = 0.5 * part_sum(part, JS, b.npad, 9, i);
    p[2] = part_sum(part, JS, b.npad, 10, i);
  }
  if (!blk) return;
  block_sum<3>(p, sh);
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; ++c) blk[(size_t)blockIdx.x * 3 + c] = p[c];
}

// Reverse step m, first half: bb <- bb_m, z <- z_m (from Xb_{m+1}, bb_{m+1}).
// cv = dl_m/dv_m / v_m (0 for m = 0); first = (m == 0).
__global__ void k_adj_prep(AdjBox b, const double* vm, const double* Xb, double* bb, double* z, double cv,
                           double dt, int first) {
  const int i = blockIdx.x * kAdjThreads + threadIdx.x;
  if (i >= b.n) return;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = (size_t)c * b.npad + i;
    const double X = Xb[k], bn = bb[k];
    const double bm = fma(dt, X, fma(cv, vm[k], bn));
    const double y = fma(0.5 * dt * dt, X, 0.5 * dt * bn);
    z[k] = first ? y : fma(0.5 * dt, bm, y);
    bb[k] = bm;
  }
}

// Reverse step m, second half: Xb <- dl_m/dx_m + Xb + H z, with
// dl_m/dx_m = cF F + cA dF/dsigma (both 0 for m = 0).  Block partials
// (z.F, z.dF/dsigma, V, W, dW/dsigma) into blk[blockIdx.x * 5 + 0..4].
__global__ void k_adj_finish(AdjBox b, const double* part, int JS, const double* z, double* Xb, double cF,
                             double cA, double* blk) {
  __shared__ double sh[5 * 32];
  const int i = blockIdx.x * kAdjThreads + threadIdx.x;
  double p[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (i < b.n) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = (size_t)c * b.npad + i;
      const double F = part_sum(part, JS, b.npad, c, i);
      const double A = part_sum(part, JS, b.npad, 3 + c, i);
      const double Hz = part_sum(part, JS, b.npad, 6 + c, i);
      Xb[k] = fma(cF, F, fma(cA, A, Xb[k] + Hz));
      const double zc = z[k];
      p[0] = fma(zc, F, p[0]);
      p[1] = fma(zc, A, p[1]);
    }
    p[2] = 0.5 * part_sum(part, JS, b.npad, 9, i);
    p[3] = part_sum(part, JS, b.npad, 10, i);
    p[4] = part_sum(part, JS, b.npad, 11, i);
  }
  block_sum<5>(p, sh);
  if (threadIdx.x == 0)
    for (int c = 0; c < 5; ++c) blk[(size_t)blockIdx.x * 5 + c] = p[c];
}

// (N x 3 interleaved) <-> component-major device layout.
__global__ void k_adj_unpack(int n, int npad, const double* in, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int c = 0; c < 3; ++c) out[(size_t)c * npad + i] = in[(size_t)i * 3 + c];
}
__global__ void k_adj_pack(int n, int npad, const double* in, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int c = 0; c < 3; ++c) out[(size_t)i * 3 + c] = in[(size_t)c * npad + i];
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    void* q = nullptr;
    cudaError_t e = device_alloc(&q, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) {
      p = static_cast<T*>(q);
      n = count;
    }
    return e;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace
}  // namespace ljgb

using namespace ljgb;

struct lj_adjoint {
  int device = 0;
  int n = 0, npad = 0, nib = 0, JS = 1, jchunk = 0;
  AdjBox box{};
  double rho = 0, eps = 1, sigma = 1;
  double wK = 0.0, wV = 1.0, wP = 1.0;
  int every = 20;
  cudaStream_t stream = nullptr;
  DBuf<double> x, v, f, x0, v0, part, ckpt, seg, Xb, bb, z, blk, hostio;
  // last forward
  bool have_forward = false;
  double dt = 0.0;
  int S = 0;
  double loss = 0.0;
  std::vector<double> K, V, W;
  std::string err;
};

namespace {

lj_status afail(lj_adjoint* a, lj_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (a) a->err = buf;
  return code;
}

#define ADJ_CUDA(a, call)                                                                           \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return afail((a), e_ == cudaErrorMemoryAllocation ? LJ_ERR_OUT_OF_MEMORY : LJ_ERR_CUDA, "%s: %s", \
                   #call, cudaGetErrorString(e_));                                                  \
  } while (0)

size_t xyz(const lj_adjoint* a) { return (size_t)3 * a->npad; }

// F (and the energy sums) at the positions in x; kick v when v is non-null.
lj_status adj_forces(lj_adjoint* a, double* x, double* f, double* v, double* blk) {
  const dim3 grid(a->nib, a->JS);
  k_adj_pairs<false><<<grid, kAdjThreads, 0, a->stream>>>(a->box, x, nullptr, a->jchunk, a->part.p);
  k_adj_forces<<<a->nib, kAdjThreads, 0, a->stream>>>(a->box, a->part.p, a->JS, f, v, 0.5 * a->dt, blk);
  ADJ_CUDA(a, cudaGetLastError());
  return LJ_OK;
}

// One forward step of the current state (x, v, f); observables partials of
// step m into blk (nib x 3).
lj_status adj_step(lj_adjoint* a, double* blk) {
  k_adj_drift<<<a->nib, kAdjThreads, 0, a->stream>>>(a->box, a->x.p, a->v.p, a->f.p, a->dt);
  ADJ_CUDA(a, cudaGetLastError());
  return adj_forces(a, a->x.p, a->f.p, a->v.p, blk);
}

lj_status adj_copy(lj_adjoint* a, double* dst, const double* src, size_t count) {
  ADJ_CUDA(a, cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyDeviceToDevice, a->stream));
  return LJ_OK;
}

}  // namespace

extern "C" {

lj_status lj_adjoint_create(const lj_config* cfg, int32_t checkpoint_every, lj_adjoint** out) {
  if (!out) return LJ_ERR_INVALID;
  *out = nullptr;
  if (!cfg) return LJ_ERR_INVALID;
  if (cfg->n < 2 || !(cfg->density > 0) || !(cfg->epsilon > 0) || !(cfg->sigma > 0) || !(cfg->temperature >= 0))
    return LJ_ERR_INVALID;
  if (cfg->boundary != LJ_BC_PERIODIC || cfg->canonical) return LJ_ERR_UNSUPPORTED;
  if (checkpoint_every < 1) return LJ_ERR_INVALID;
  lj_adjoint* a = new lj_adjoint();
  a->device = cfg->device;
  a->n = cfg->n;
  a->npad = (cfg->n + 31) / 32 * 32;
  a->nib = (cfg->n + kAdjThreads - 1) / kAdjThreads;
  a->rho = cfg->density;
  a->eps = cfg->epsilon;
  a->sigma = cfg->sigma;
  a->every = checkpoint_every;
  const double L = std::cbrt((double)cfg->n / cfg->density);
  a->box = AdjBox{cfg->n, a->npad, L, 1.0 / L, 4.0 * cfg->epsilon, cfg->sigma * cfg->sigma, 1.0 / cfg->sigma};
  auto bail = [&](lj_status st) {
    lj_adjoint_destroy(a);
    return st;
  };
  DeviceGuard device_guard(a->device);
  if (!device_guard.ok()) return bail(LJ_ERR_NO_DEVICE);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, a->device) != cudaSuccess)
    return bail(LJ_ERR_NO_DEVICE);
  // j split: about four CTAs per SM, j chunks a multiple of 32 records
  const int want = std::max(1, (4 * sms + a->nib - 1) / a->nib);
  a->jchunk = std::max(32, ((a->n + want - 1) / want + 31) / 32 * 32);
  a->JS = (a->n + a->jchunk - 1) / a->jchunk;
  if (cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(LJ_ERR_CUDA);
  const size_t s3 = xyz(a);
  if (a->x.alloc(s3) || a->v.alloc(s3) || a->f.alloc(s3) || a->x0.alloc(s3) || a->v0.alloc(s3) || a->Xb.alloc(s3) ||
      a->bb.alloc(s3) || a->z.alloc(s3) || a->hostio.alloc(s3) ||
      a->part.alloc((size_t)a->JS * kParts * a->npad))
    return bail(LJ_ERR_OUT_OF_MEMORY);
  std::vector<double> pos((size_t)3 * a->n), vel((size_t)3 * a->n);
  if (!sample_initial_state(a->n, L, cfg->temperature, cfg->lattice, cfg->jitter, cfg->sigma, cfg->seed, pos.data(),
                            vel.data()))
    return bail(LJ_ERR_INVALID);
  lj_status st = lj_adjoint_set_state(a, pos.data(), vel.data());
  if (st) return bail(st);
  *out = a;
  return LJ_OK;
}

lj_status lj_adjoint_destroy(lj_adjoint* a) {
  if (!a) return LJ_OK;
  DeviceGuard device_guard(a->device);
  if (a->stream) cudaStreamSynchronize(a->stream);
  for (DBuf<double>* b : {&a->x, &a->v, &a->f, &a->x0, &a->v0, &a->part, &a->ckpt, &a->seg, &a->Xb, &a->bb, &a->z,
                          &a->blk, &a->hostio})
    b->free();
  if (a->stream) cudaStreamDestroy(a->stream);
  delete a;
  return LJ_OK;
}

const char* lj_adjoint_last_error(const lj_adjoint* a) { return a ? a->err.c_str() : ""; }

lj_status lj_adjoint_set_state(lj_adjoint* a, const double* pos, const double* vel) {
  if (!a) return LJ_ERR_INVALID;
  if (!pos || !vel) return afail(a, LJ_ERR_INVALID, "pos and vel must be non-NULL");
  DeviceGuard device_guard(a->device);
  const size_t bytes = sizeof(double) * 3 * a->n;
  const int g = (a->n + 255) / 256;
  ADJ_CUDA(a, cudaMemcpyAsync(a->hostio.p, pos, bytes, cudaMemcpyHostToDevice, a->stream));
  k_adj_unpack<<<g, 256, 0, a->stream>>>(a->n, a->npad, a->hostio.p, a->x0.p);
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  ADJ_CUDA(a, cudaMemcpyAsync(a->hostio.p, vel, bytes, cudaMemcpyHostToDevice, a->stream));
  k_adj_unpack<<<g, 256, 0, a->stream>>>(a->n, a->npad, a->hostio.p, a->v0.p);
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  a->have_forward = false;
  return LJ_OK;
}

lj_status lj_adjoint_set_loss(lj_adjoint* a, double w_kinetic, double w_potential, double w_pressure) {
  if (!a) return LJ_ERR_INVALID;
  if (!std::isfinite(w_kinetic) || !std::isfinite(w_potential) || !std::isfinite(w_pressure))
    return afail(a, LJ_ERR_INVALID, "loss weights must be finite");
  a->wK = w_kinetic;
  a->wV = w_potential;
  a->wP = w_pressure;
  a->have_forward = false;
  return LJ_OK;
}

lj_status lj_adjoint_forward(lj_adjoint* a, double dt, int32_t nsteps, double* loss) {
  if (!a) return LJ_ERR_INVALID;
  if (!(dt > 0) || !std::isfinite(dt)) return afail(a, LJ_ERR_INVALID, "dt must be > 0");
  if (nsteps < 1) return afail(a, LJ_ERR_INVALID, "nsteps must be >= 1");
  DeviceGuard device_guard(a->device);
  a->dt = dt;
  a->S = nsteps;
  a->have_forward = false;
  const size_t s3 = xyz(a);
  const int J = (nsteps + a->every - 1) / a->every;
  if (a->ckpt.alloc((size_t)J * 3 * s3) || a->seg.alloc((size_t)(a->every + 1) * 2 * s3) ||
      a->blk.alloc((size_t)(nsteps + 1) * a->nib * 5))
    return afail(a, LJ_ERR_OUT_OF_MEMORY, "cannot allocate %d checkpoints of %d particles", J, a->n);
  lj_status st;
  if ((st = adj_copy(a, a->x.p, a->x0.p, s3)) || (st = adj_copy(a, a->v.p, a->v0.p, s3))) return st;
  if ((st = adj_forces(a, a->x.p, a->f.p, nullptr, nullptr))) return st;
  for (int m = 0; m < nsteps; ++m) {
    if (m % a->every == 0) {
      double* c = a->ckpt.p + (size_t)(m / a->every) * 3 * s3;
      if ((st = adj_copy(a, c, a->x.p, s3)) || (st = adj_copy(a, c + s3, a->v.p, s3)) ||
          (st = adj_copy(a, c + 2 * s3, a->f.p, s3)))
        return st;
    }
    if ((st = adj_step(a, a->blk.p + (size_t)m * a->nib * 3))) return st;
  }
  std::vector<double> h((size_t)nsteps * a->nib * 3);
  ADJ_CUDA(a, cudaMemcpyAsync(h.data(), a->blk.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, a->stream));
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  const double N = (double)a->n;
  a->K.assign(nsteps, 0.0);
  a->V.assign(nsteps, 0.0);
  a->W.assign(nsteps, 0.0);
  double l = 0.0;
  for (int m = 0; m < nsteps; ++m) {
    double s[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < a->nib; ++b)
      for (int c = 0; c < 3; ++c) s[c] += h[((size_t)m * a->nib + b) * 3 + c];
    a->K[m] = s[0];
    a->V[m] = s[1];
    a->W[m] = s[2];
    const double T = 2. * s[0] / 3. / N;                // MDSystem.cpp:325-359
    const double P = (s[2] / 6. + N * T) / (N / a->rho);
    l += (a->wK * s[0] / N + a->wV * s[1] / N + a->wP * P) / nsteps;
  }
  if (!std::isfinite(l)) return afail(a, LJ_ERR_NONFINITE, "the loss is not finite");
  a->loss = l;
  a->have_forward = true;
  if (loss) *loss = l;
  return LJ_OK;
}

lj_status lj_adjoint_observables(lj_adjoint* a, double* K, double* V, double* W, int32_t max, int32_t* count) {
  if (!a) return LJ_ERR_INVALID;
  if (!a->have_forward) return afail(a, LJ_ERR_INVALID, "no forward pass");
  const int m = std::min<int>(max, a->S);
  for (int k = 0; k < m; ++k) {
    if (K) K[k] = a->K[k];
    if (V) V[k] = a->V[k];
    if (W) W[k] = a->W[k];
  }
  if (count) *count = a->S;
  return LJ_OK;
}

lj_status lj_adjoint_backward(lj_adjoint* a, double* d_epsilon, double* d_sigma, double* d_pos, double* d_vel) {
  if (!a) return LJ_ERR_INVALID;
  if (!a->have_forward) return afail(a, LJ_ERR_INVALID, "lj_adjoint_backward needs a forward pass first");
  DeviceGuard device_guard(a->device);
  const size_t s3 = xyz(a);
  const int S = a->S, k = a->every, J = (S + k - 1) / k;
  const double N = (double)a->n, dt = a->dt, rho = a->rho;
  const double cv = (a->wK / N + a->wP * rho * 2.0 / (3.0 * N)) / S;  // dl_m/dv_m = cv v_m
  const double cF = -a->wV / N / S;                                    // dl_m/dx_m = cF F + cA dF/dsigma
  const double cA = a->wP * rho / (6.0 * N) * (-2.0 * a->sigma) / S;
  ADJ_CUDA(a, cudaMemsetAsync(a->Xb.p, 0, sizeof(double) * s3, a->stream));
  ADJ_CUDA(a, cudaMemsetAsync(a->bb.p, 0, sizeof(double) * s3, a->stream));
  lj_status st;
  for (int j = J - 1; j >= 0; --j) {
    const int c0 = j * k, c1 = std::min(c0 + k, S);
    // replay the segment from its checkpoint (same kernels as the forward)
    const double* c = a->ckpt.p + (size_t)j * 3 * s3;
    if ((st = adj_copy(a, a->x.p, c, s3)) || (st = adj_copy(a, a->v.p, c + s3, s3)) ||
        (st = adj_copy(a, a->f.p, c + 2 * s3, s3)))
      return st;
    for (int m = c0; m <= c1; ++m) {
      if (m > c0 && (st = adj_step(a, nullptr))) return st;
      double* sl = a->seg.p + (size_t)(m - c0) * 2 * s3;
      if ((st = adj_copy(a, sl, a->x.p, s3)) || (st = adj_copy(a, sl + s3, a->v.p, s3))) return st;
    }
    // reverse sweep over m = c1 .. c0+1 (.. 0 in the first segment)
    for (int m = c1; m >= (j == 0 ? 0 : c0 + 1); --m) {
      const double* xm = a->seg.p + (size_t)(m - c0) * 2 * s3;
      const double* vm = xm + s3;
      k_adj_prep<<<a->nib, kAdjThreads, 0, a->stream>>>(a->box, vm, a->Xb.p, a->bb.p, a->z.p, m >= 1 ? cv : 0.0, dt,
                                                        m == 0 ? 1 : 0);
      k_adj_pairs<true><<<dim3(a->nib, a->JS), kAdjThreads, 0, a->stream>>>(a->box, xm, a->z.p, a->jchunk,
                                                                             a->part.p);
      k_adj_finish<<<a->nib, kAdjThreads, 0, a->stream>>>(a->box, a->part.p, a->JS, a->z.p, a->Xb.p,
                                                          m >= 1 ? cF : 0.0, m >= 1 ? cA : 0.0,
                                                          a->blk.p + (size_t)m * a->nib * 5);
      ADJ_CUDA(a, cudaGetLastError());
    }
  }
  // parameter gradients: fixed-order sums of the block partials
  std::vector<double> h((size_t)(S + 1) * a->nib * 5);
  ADJ_CUDA(a, cudaMemcpyAsync(h.data(), a->blk.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, a->stream));
  double de = 0.0, ds = 0.0;
  for (int m = 0; m <= S; ++m) {
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < a->nib; ++b)
      for (int q = 0; q < 5; ++q) s[q] += h[((size_t)m * a->nib + b) * 5 + q];
    de += s[0] / a->eps;  // G_eps^T z = z.F / eps
    ds += s[1];           // G_sigma^T z = z.dF/dsigma
    if (m >= 1) {         // explicit: dV/deps = V/eps, dV/dsigma = W/(2 sigma), dW/deps = W/eps
      de += (a->wV * s[2] / (N * a->eps) + a->wP * rho * s[3] / (6.0 * N * a->eps)) / S;
      ds += (a->wV * s[3] / (2.0 * a->sigma * N) + a->wP * rho * s[4] / (6.0 * N)) / S;
    }
  }
  if (d_epsilon) *d_epsilon = de;
  if (d_sigma) *d_sigma = ds;
  const int g = (a->n + 255) / 256;
  const size_t bytes = sizeof(double) * 3 * a->n;
  if (d_pos) {
    k_adj_pack<<<g, 256, 0, a->stream>>>(a->n, a->npad, a->Xb.p, a->hostio.p);
    ADJ_CUDA(a, cudaMemcpyAsync(d_pos, a->hostio.p, bytes, cudaMemcpyDeviceToHost, a->stream));
    ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  }
  if (d_vel) {
    k_adj_pack<<<g, 256, 0, a->stream>>>(a->n, a->npad, a->bb.p, a->hostio.p);
    ADJ_CUDA(a, cudaMemcpyAsync(d_vel, a->hostio.p, bytes, cudaMemcpyDeviceToHost, a->stream));
  }
  ADJ_CUDA(a, cudaStreamSynchronize(a->stream));
  if (!std::isfinite(de) || !std::isfinite(ds)) return afail(a, LJ_ERR_NONFINITE, "a gradient is not finite");
  return LJ_OK;
}

}  // extern "C"
