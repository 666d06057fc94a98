// lj_internal.h -- host/device shared structures of the LJ GB300 library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ljgb {

// Makes `device` current for the lifetime of the guard and puts the caller's
// device back afterwards: an lj_* call on a handle leaves the calling
// thread's current device as it found it.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
    if (prev_ != device) {
      err_ = cudaSetDevice(device);
      switched_ = err_ == cudaSuccess && prev_ >= 0;
    }
  }
  ~DeviceGuard() {
    if (switched_) cudaSetDevice(prev_);
  }
  bool ok() const { return err_ == cudaSuccess; }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

 private:
  int prev_ = -1;
  bool switched_ = false;
  cudaError_t err_ = cudaSuccess;
};

// Every device and page-locked host allocation the library makes goes
// through these two calls (lj_system.cpp).  lj_debug_fail_allocations arms a
// host-side countdown that makes them fail with cudaErrorMemoryAllocation
// without calling CUDA, so the out-of-memory paths can be tested without
// exhausting a GPU.
cudaError_t device_alloc(void** p, size_t bytes);
cudaError_t pinned_alloc(void** p, size_t bytes);

// Device-side status flags (DevScalars::status).
enum : int {
  LJ_DEVFLAG_TIMEOUT = 1,    // a bounded mbarrier wait gave up
  LJ_DEVFLAG_NONFINITE = 2,  // NaN/Inf observable
  LJ_DEVFLAG_ESCAPED = 4,    // a particle of a walled box left its fixed frame
};

// Per-system frame of the fixed-point shadow and the scalar state that the
// kernels update on the device.  One per simulated box; kept in device memory
// so captured step graphs read current values.
struct DevScalars {
  // fixed-point frame: q = frac((x - origin)/P) * 2^32
  double origin[3];
  double P, invP;
  float k2inv;    // 1 / (P / (2^32 sigma))^2  : sigma^2 / r^2 = k2inv / r2_fixed
  float k2;       // (P / (2^32 sigma))^2       : r^2 / sigma^2 = k2 * r2_fixed
  double fscale;  // F = fscale * sum s * d_fixed   (4 eps * k_sigma / sigma)
  // clock and running averages (MDSystem.h:80, 98-99)
  double t;
  long long step;
  double av_U, av_T, av_p;
  long long av_iters;
  // last observables (MDSystem.h:63-66)
  double K, V, T, P_press, U, W, Pshear, Tkin;
  // TVN scale of the last step
  double chi;
  int status;
  int rec_cap;
  long long rec_count;
  // Fused steps compute a step's observables late (inside the next step's
  // pair kernel, or in the read-back / k_obs_finalize), one entry per step
  // parity: obs_pending[p] is the step mode (MODE_EVN / MODE_TVN) of a box
  // whose K/V/W block partials from the step of parity p are written but not
  // yet summed, 0 if none; obs_slot[p] is the first of the three
  // block-partial slots that hold them; Tkin_rec[p] is the Tkin of that step
  // for its record.  A step marks its own parity's entry and the next step's
  // pair kernel consumes it, so the two never touch the same entry at once.
  double Tkin_rec[2];
  int obs_pending[2];
  int obs_slot[2];
};

// Observable record layout written by the device (matches lj_observables).
struct DevRecord {
  double t, K, V, T, P, U, W, Pshear, Tkin, av_U, av_T, av_p;
  long long av_iters, step;
};

// One i-block of the stream-K schedule: BI consecutive particles of one box.
struct BlockInfo {
  int sys;        // box index
  int i0;         // first box-local particle of the block
  int n_i;        // valid particles in the block (<= BI)
  int p0;         // global offset of the box's particle 0
  int n_sys;      // particles in the box
  int njt;        // j-tiles of the box
  int seg_first;  // first partial segment of this block
  int seg_count;  // segments of this block
  int g_first;    // first CTA that processes this block
  int pad;
};

// Per-box constants passed by value (captured into graphs).
struct BoxArgs {
  int N;
  int bc;
  int canonical;
  int pad;
  double L, invL;
  double eps, sigma;
  double dt, T0, rho;
  // Derived on the host from the fields above before every upload, so that
  // the step kernels multiply instead of divide (FP64 division is a long
  // dependent sequence on this part's narrow FP64 pipe).
  double hdt;    // dt / 2
  double qdt;    // dt / 4: the TVN kick dt/2 of the averaged force (F_n + F_{n+1}) / 2
  double hdt2;   // dt^2 / 2
  double eps4;   // 4 eps
  double kT;     // 2 / (3 N):  T = kT K
  double kP;     // rho / N:    P = (W / 6 + N T) kP
  double inv3N;  // 1 / (3 N):  Tkin = inv3N sum tv^2
  double invT0;  // 1 / T0 (0 when T0 = 0)
  double wall_margin;  // walls: m = max(sigma, L / 20), the frame's margin beyond [0, L] and the positions
};

}  // namespace ljgb
