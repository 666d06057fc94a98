// lj_compat.cu -- the reference's extern "C" CUDA entry points
// (src/library/MDSystem.cu:155-299, declared at MDSystem.cpp:10-25) on top of
// this library's sm_103a pair kernel.  See include/lj_reference_abi.h for the
// contract and the deliberate differences.
//
// calculateNForces: float4 positions -> fixed-point shadow (frame from L or
// from the bounding box for non-periodic boxes) -> persistent all-pairs
// kernel (forces, energies, virial and optionally the 256-bin r^2 RDF in one
// pass) -> per-particle float4 forces and one FP64 virial sum.  Work buffers
// are cached per particle count on a private stream.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lj_device.cuh"
#include "lj_gb300.h"
#include "lj_kernels.h"
#include "lj_reference_abi.h"
#include "lj_schedule.h"

namespace ljgb {
namespace {

constexpr int kRefBins = 256;  // NdNdr2 size (MDSystem.cpp:97)
constexpr int kBlk = kFloat4Threads;

// Force[i] = (F, sum_j r^-12 - r^-6); block partial of sum_j s r^2.
__global__ void k_ref_reduce(const float* partial, const BlockInfo* blocks, int bi_threads, const DevScalars* sc,
                             float4* force, double* blk) {
  __shared__ double sh[32];
  const BlockInfo bi = blocks[blockIdx.x];
  const int tid = threadIdx.x;
  double part[1] = {0.0};
  if (tid < bi.n_i) {
    double S[5] = {0, 0, 0, 0, 0};
    for (int k = 0; k < bi.seg_count; ++k) {
      const size_t base = (size_t)(bi.seg_first + k) * 5 * bi_threads + tid;
      for (int c = 0; c < 5; ++c) S[c] += (double)partial[base + (size_t)c * bi_threads];
    }
    const double fs = sc->fscale;
    force[bi.i0 + tid] = make_float4((float)(fs * S[0]), (float)(fs * S[1]), (float)(fs * S[2]), (float)(S[3] - S[4]));
    part[0] = 12.0 * S[3] - 6.0 * S[4];
  }
  block_sum<1>(part, sh);
  if (tid == 0) blk[(size_t)blockIdx.x * 8] = part[0];
}

// pressure = (4/6) sum_i sum_j s r^2   (MDSystem.cu:105-108, 136)
__global__ void k_ref_pressure(const double* blk, int nb, float* out) {
  __shared__ double sh[32];
  double acc[1] = {0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) acc[0] += blk[(size_t)b * 8];
  block_sum<1>(acc, sh);
  if (threadIdx.x == 0) *out = (float)(acc[0] * 4.0 / 6.0);
}

struct CompatCtx {
  int device = -1;  // the device that holds the buffers below
  int n = 0;
  int shape = -1;
  int nb_bbox = 0;
  Schedule sched;
  cudaStream_t stream = nullptr;
  int4* q = nullptr;
  DevScalars* sc = nullptr;
  BlockInfo* blocks = nullptr;
  int *ctb = nullptr, *clo = nullptr, *cb = nullptr, *cj = nullptr;
  float* partial = nullptr;
  double* blk = nullptr;
  unsigned long long* hist = nullptr;
  int* status = nullptr;
  float* pressure = nullptr;
  void release() {
    if (stream) cudaStreamSynchronize(stream);
    cudaFree(q);
    cudaFree(sc);
    cudaFree(blocks);
    cudaFree(ctb);
    cudaFree(clo);
    cudaFree(cb);
    cudaFree(cj);
    cudaFree(partial);
    cudaFree(blk);
    cudaFree(hist);
    cudaFree(status);
    cudaFree(pressure);
    if (stream) cudaStreamDestroy(stream);
    *this = CompatCtx();
  }
};

std::mutex g_mu;
CompatCtx g_ctx;
int g_status = 0;
std::string g_error;

bool record(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_status = e == cudaErrorMemoryAllocation ? LJ_ERR_OUT_OF_MEMORY : LJ_ERR_CUDA;
  g_error = std::string(what) + ": " + cudaGetErrorString(e);
  std::fprintf(stderr, "lj_gb300 reference ABI: %s\n", g_error.c_str());
  return false;
}

#define REF_CHECK(call) \
  if (!record((call), #call)) return false

bool ensure_ctx(int n, int block_hint) {
  int shape = 0;
  for (int k = 0; k < kNumShapes; ++k)
    if (std::abs(kShapes[k].threads - block_hint) < std::abs(kShapes[shape].threads - block_hint)) shape = k;
  int dev = 0, sms = 0, per_sm = 0;
  REF_CHECK(cudaGetDevice(&dev));
  if (g_ctx.n == n && g_ctx.shape == shape && g_ctx.stream && g_ctx.device == dev) return true;
  if (g_ctx.stream && g_ctx.device != dev) {
    // The caller switched devices: free the old buffers on their own device.
    REF_CHECK(cudaSetDevice(g_ctx.device));
    g_ctx.release();
    REF_CHECK(cudaSetDevice(dev));
  } else {
    g_ctx.release();
  }
  REF_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  REF_CHECK(pair_occupancy(0, shape, &per_sm));
  Schedule s;
  // at most 8 CTAs per i-block (a block's epilogue sums one segment per CTA)
  const int nb_i = (n + kShapes[shape].threads - 1) / kShapes[shape].threads;
  const int ctas = std::min(sms * per_sm, 8 * nb_i);
  if (!build_schedule(&n, 1, kShapes[shape].threads, kShapes[shape].tile, ctas, 8, &s)) {
    g_status = LJ_ERR_INVALID;
    g_error = "cannot build the pair schedule";
    return false;
  }
  CompatCtx c;
  c.device = dev;
  c.n = n;
  c.shape = shape;
  c.nb_bbox = (n + kBlk - 1) / kBlk;
  // Buffers of the new context; on any failure everything allocated so far
  // is freed and the layer is left without a context (the next call retries).
  auto build = [&]() -> bool {
    // A blocking stream: the reference's ABI is synchronous and its copies
    // (copyArrayToDevice, cudaMemcpy on the legacy stream) must be ordered
    // before this stream's kernels; a pageable cudaMemcpy can return before
    // its DMA has landed.
    REF_CHECK(cudaStreamCreateWithFlags(&c.stream, cudaStreamDefault));
    const int nb = (int)s.blocks.size();
    REF_CHECK(device_alloc((void**)&c.q, sizeof(int4) * n));
    REF_CHECK(device_alloc((void**)&c.sc, sizeof(DevScalars)));
    REF_CHECK(device_alloc((void**)&c.blocks, sizeof(BlockInfo) * nb));
    REF_CHECK(device_alloc((void**)&c.ctb, sizeof(int) * (s.G + 1)));
    REF_CHECK(device_alloc((void**)&c.clo, sizeof(int) * (s.G + 1)));
    REF_CHECK(device_alloc((void**)&c.cb, sizeof(int) * s.G));
    REF_CHECK(device_alloc((void**)&c.cj, sizeof(int) * s.G));
    REF_CHECK(device_alloc((void**)&c.partial, sizeof(float) * (size_t)s.nseg * 5 * s.BI));
    REF_CHECK(device_alloc((void**)&c.blk, sizeof(double) * 8 * (size_t)std::max(nb, c.nb_bbox)));
    REF_CHECK(device_alloc((void**)&c.hist, sizeof(unsigned long long) * kRefBins));
    REF_CHECK(device_alloc((void**)&c.status, sizeof(int)));
    REF_CHECK(device_alloc((void**)&c.pressure, sizeof(float)));
    REF_CHECK(cudaMemset(c.sc, 0, sizeof(DevScalars)));
    REF_CHECK(cudaMemset(c.status, 0, sizeof(int)));
    REF_CHECK(cudaMemcpy(c.blocks, s.blocks.data(), sizeof(BlockInfo) * nb, cudaMemcpyHostToDevice));
    REF_CHECK(cudaMemcpy(c.ctb, s.cta_tile_begin.data(), sizeof(int) * (s.G + 1), cudaMemcpyHostToDevice));
    REF_CHECK(cudaMemcpy(c.clo, s.cta_lo.data(), sizeof(int) * (s.G + 1), cudaMemcpyHostToDevice));
    REF_CHECK(cudaMemcpy(c.cb, s.cta_block.data(), sizeof(int) * s.G, cudaMemcpyHostToDevice));
    REF_CHECK(cudaMemcpy(c.cj, s.cta_jt.data(), sizeof(int) * s.G, cudaMemcpyHostToDevice));
    return true;
  };
  if (!build()) {
    c.release();
    return false;
  }
  c.sched = std::move(s);
  g_ctx = c;
  return true;
}

bool calc_forces(float* Pos, float* Force, float* host_pressure, int n, float L, int periodic, int* host_RDF,
                 float dr2, int block_size) {
  if (!Pos || !Force || !host_pressure || n < 2) {
    g_status = LJ_ERR_INVALID;
    g_error = "calculateNForces: null array or numBodies < 2";
    return false;
  }
  if (!ensure_ctx(n, block_size > 0 ? block_size : 128)) return false;
  CompatCtx& c = g_ctx;
  const float4* pos = reinterpret_cast<const float4*>(Pos);
  if (!periodic) REF_CHECK(launch_float4_bbox(pos, n, c.blk, c.stream));
  REF_CHECK(launch_float4_frame(c.blk, c.nb_bbox, periodic, (double)L, c.sc, nullptr, c.stream));
  REF_CHECK(launch_float4_quantize(pos, n, c.sc, c.q, c.stream));
  PairArgs a{};
  a.q = c.q;
  a.blocks = c.blocks;
  a.cta_tile_begin = c.ctb;
  a.cta_lo = c.clo;
  a.cta_block = c.cb;
  a.cta_jt = c.cj;
  a.sc = c.sc;
  a.partial = c.partial;
  a.status = c.status;
  a.hist = HistArgs{0, kRefBins, 1.0f / dr2, 0.0f, c.hist};
  const bool want_rdf = host_RDF != nullptr && dr2 > 0.0f;
  if (want_rdf) REF_CHECK(cudaMemsetAsync(c.hist, 0, sizeof(unsigned long long) * kRefBins, c.stream));
  REF_CHECK(launch_pairs(0, c.shape, true, want_rdf, a, c.sched.G, c.stream));
  const int nb = (int)c.sched.blocks.size();
  k_ref_reduce<<<nb, c.sched.BI, 0, c.stream>>>(c.partial, c.blocks, c.sched.BI, c.sc,
                                                  reinterpret_cast<float4*>(Force), c.blk);
  REF_CHECK(cudaGetLastError());
  k_ref_pressure<<<1, 256, 0, c.stream>>>(c.blk, nb, c.pressure);
  REF_CHECK(cudaGetLastError());
  REF_CHECK(cudaMemcpyAsync(host_pressure, c.pressure, sizeof(float), cudaMemcpyDeviceToHost, c.stream));
  unsigned long long h[kRefBins];
  if (want_rdf) REF_CHECK(cudaMemcpyAsync(h, c.hist, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
  int st = 0;
  REF_CHECK(cudaMemcpyAsync(&st, c.status, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  REF_CHECK(cudaStreamSynchronize(c.stream));
  if (st) {
    cudaMemset(c.status, 0, sizeof(int));
    g_status = LJ_ERR_DEVICE_TIMEOUT;
    g_error = "calculateNForces: a device-side wait timed out";
    return false;
  }
  if (want_rdf)
    for (int b = 0; b < kRefBins; ++b) host_RDF[b] = (int)h[b];
  return true;
}

}  // namespace
}  // namespace ljgb

using namespace ljgb;

extern "C" {

void allocateNBodyArrays(float* vel[2], int numBodies) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  const size_t bytes = sizeof(float) * 4 * (size_t)numBodies;
  vel[0] = vel[1] = nullptr;
  if (record(device_alloc((void**)&vel[0], bytes), "cudaMalloc") &&
      !record(device_alloc((void**)&vel[1], bytes), "cudaMalloc")) {
    cudaFree(vel[0]);
    vel[0] = nullptr;
  }
}

void allocateArray(float** dest, int number) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(device_alloc((void**)dest, sizeof(float) * 4 * (size_t)number), "cudaMalloc");
}

void deleteNBodyArrays(float* vel[2]) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(cudaFree(vel[0]), "cudaFree");
  record(cudaFree(vel[1]), "cudaFree");
}

void deleteArray(float* arr) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(cudaFree(arr), "cudaFree");
}

void allocateIntArray(int** dest, int number) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(device_alloc((void**)dest, sizeof(int) * (size_t)number), "cudaMalloc");
}

void deleteIntArray(int* arr) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(cudaFree(arr), "cudaFree");
}

void copyArrayFromDevice(float* host, const float* device, unsigned int pbo, int numBodies) {
  (void)pbo;
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(cudaMemcpy(host, device, sizeof(float) * 4 * (size_t)numBodies, cudaMemcpyDeviceToHost), "cudaMemcpy");
}

void copyArrayToDevice(float* device, const float* host, int numBodies) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(cudaMemcpy(device, host, sizeof(float) * 4 * (size_t)numBodies, cudaMemcpyHostToDevice), "cudaMemcpy");
}

void registerGLBufferObject(unsigned int pbo) { (void)pbo; }

void unregisterGLBufferObject(unsigned int pbo) { (void)pbo; }

void threadSync(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  record(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

void calculateNForces(float* Pos, float* Force, float* host_pressure, int numBodies, float host_L, int Lperiodic,
                      int* host_RDF, float host_dr2, int blockSize, int q) {
  (void)q;
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  calc_forces(Pos, Force, host_pressure, numBodies, host_L, Lperiodic, host_RDF, host_dr2, blockSize);
}

void threadExit(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_status = 0;
  g_ctx.release();
  record(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

int lj_reference_abi_status(void) { return g_status; }

const char* lj_reference_abi_error(void) { return g_error.c_str(); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Fixed-point shadow of caller-owned float4 positions, shared by the
// reference ABI above and the allocation-free force entry point
// (lj_noalloc.cu).
// ---------------------------------------------------------------------------
namespace ljgb {
namespace {

// Per-CTA bounding box of kFloat4Threads positions: blk[b*8 + 0..2] = min,
// blk[b*8 + 3..5] = max.
__global__ void k_float4_bbox(const float4* pos, int n, double* blk) {
  __shared__ double sh[6][32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  if (i < n) {
    const float4 p = pos[i];
    lo[0] = hi[0] = p.x;
    lo[1] = hi[1] = p.y;
    lo[2] = hi[2] = p.z;
  }
  for (int c = 0; c < 3; ++c)
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fmin(lo[c], __shfl_down_sync(0xffffffffu, lo[c], o));
      hi[c] = fmax(hi[c], __shfl_down_sync(0xffffffffu, hi[c], o));
    }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int c = 0; c < 3; ++c) {
      sh[c][warp] = lo[c];
      sh[3 + c][warp] = hi[c];
    }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; ++c) {
      double a = 1e300, b = -1e300;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        a = fmin(a, sh[c][w]);
        b = fmax(b, sh[3 + c][w]);
      }
      blk[(size_t)blockIdx.x * 8 + c] = a;
      blk[(size_t)blockIdx.x * 8 + 3 + c] = b;
    }
}

// One thread: frame of the fixed-point shadow (eps = sigma = 1).  Periodic:
// origin 0, period L.  Otherwise the bounding box's low corner and a period
// of twice its largest extent, so no separation wraps.  Clears *status when
// given.
__global__ void k_float4_frame(const double* blk, int nb, int periodic, double L, DevScalars* sc, int* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double origin[3] = {0, 0, 0};
  double P = L;
  if (!periodic) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int b = 0; b < nb; ++b)
      for (int c = 0; c < 3; ++c) {
        lo[c] = fmin(lo[c], blk[(size_t)b * 8 + c]);
        hi[c] = fmax(hi[c], blk[(size_t)b * 8 + 3 + c]);
      }
    double ext = 0;
    for (int c = 0; c < 3; ++c) {
      ext = fmax(ext, hi[c] - lo[c]);
      origin[c] = lo[c];
    }
    P = 2.002 * ext + 1e-3;
  }
  for (int c = 0; c < 3; ++c) sc->origin[c] = origin[c];
  sc->P = P;
  sc->invP = 1.0 / P;
  const double ks = P / 4294967296.0;
  sc->k2 = (float)(ks * ks);
  sc->k2inv = (float)(1.0 / (ks * ks));
  sc->fscale = 4.0 * ks;
  if (status) *status = 0;
}

__global__ void k_float4_quantize(const float4* pos, int n, const DevScalars* sc, int4* q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  q[i] = make_int4(fixed_coord(p.x, sc->origin[0], sc->invP), fixed_coord(p.y, sc->origin[1], sc->invP),
                   fixed_coord(p.z, sc->origin[2], sc->invP), 0);
}

}  // namespace

cudaError_t launch_float4_bbox(const float4* pos, int n, double* blk, cudaStream_t st) {
  k_float4_bbox<<<(n + kFloat4Threads - 1) / kFloat4Threads, kFloat4Threads, 0, st>>>(pos, n, blk);
  return cudaGetLastError();
}

cudaError_t launch_float4_frame(const double* blk, int nb, int periodic, double L, DevScalars* sc, int* status,
                                cudaStream_t st) {
  k_float4_frame<<<1, 32, 0, st>>>(blk, nb, periodic, L, sc, status);
  return cudaGetLastError();
}

cudaError_t launch_float4_quantize(const float4* pos, int n, const DevScalars* sc, int4* q, cudaStream_t st) {
  k_float4_quantize<<<(n + kFloat4Threads - 1) / kFloat4Threads, kFloat4Threads, 0, st>>>(pos, n, sc, q);
  return cudaGetLastError();
}

}  // namespace ljgb
