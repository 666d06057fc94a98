// lj_noalloc.cu -- all-pairs LJ forces without any device allocation.
//
// Some callers cannot allocate device memory: plug-ins hosted by another
// framework whose caching allocator has reserved the GPU's memory (a
// cudaMalloc of their own fails or fragments that pool), real-time loops
// that must not allocate after start-up (cudaMalloc and cudaFree can
// synchronise the whole device and stall every stream), and embedders whose
// rules give every byte of the GPU to their own allocator.  lj_forces_static serves them: the caller passes device input and
// output arrays only, and every intermediate buffer (fixed-point shadow, work
// schedule, per-segment partial sums, block sums, status word) lives in one
// file-scope __device__ array of fixed size that each GPU holds from the
// moment the library is loaded until the process exits.
//
// Limits and rules (also in include/lj_gb300.h):
//  * at most kStaticMaxParticles particles; larger calls are rejected with
//    LJ_ERR_INVALID and a message on stderr;
//  * all calls on a device share the one array and it keeps the last call's
//    contents: calls whose GPU work overlaps (two host threads, or two
//    streams) race and corrupt each other's results; serialise them;
//  * every call looks up the array's device address on the current device
//    (cudaGetSymbolAddress; the host-side name of a __device__ array is not a
//    device pointer), and the first call on a device also reads its SM count
//    and checks the kernel shape this file's scratch layout is sized for;
//    make that first call before any stream capture begins;
//  * every call ends by reading its status word and sums back to the host
//    on `stream` and synchronising it, so a call on a stream that is being
//    captured is rejected with LJ_ERR_UNSUPPORTED before anything is enqueued;
//  * the cached work schedule belongs to the array's current address: after
//    a cudaDeviceReset the next call finds a new address (or the same one
//    with the schedule gone) and uploads the schedule again.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "lj_device.cuh"
#include "lj_gb300.h"
#include "lj_kernels.h"

namespace ljgb {
namespace {

constexpr int kStaticMaxParticles = 16384;
constexpr int kBI = 128;                          // i-block of the pair-kernel shape used here
constexpr int kTile = 256;                        // j-tile of that shape
constexpr int kShape = 0;                         // kShapes[0] = {128, 256, 3}
constexpr int kMaxBlocks = kStaticMaxParticles / kBI;
constexpr int kMaxCtas = 1536;
constexpr int kMaxSegs = kMaxCtas + kMaxBlocks;
constexpr int kBboxThreads = kFloat4Threads;
constexpr int kMaxBbox = kStaticMaxParticles / kBboxThreads;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Byte layout of the scratch array.
constexpr size_t kOffFrame = 0;
constexpr size_t kOffStatus = kOffFrame + align256(sizeof(DevScalars));
constexpr size_t kOffQ = kOffStatus + 256;
constexpr size_t kOffBlocks = kOffQ + align256(sizeof(int4) * kStaticMaxParticles);
constexpr size_t kOffCtaBegin = kOffBlocks + align256(sizeof(BlockInfo) * kMaxBlocks);
constexpr size_t kOffCtaBlock = kOffCtaBegin + align256(sizeof(int) * (kMaxCtas + 1));
constexpr size_t kOffCtaJt = kOffCtaBlock + align256(sizeof(int) * kMaxCtas);
constexpr size_t kOffBlk = kOffCtaJt + align256(sizeof(int) * kMaxCtas);
constexpr size_t kOffSums = kOffBlk + align256(sizeof(double) * 8 * (kMaxBlocks > kMaxBbox ? kMaxBlocks : kMaxBbox));
constexpr size_t kOffPartial = kOffSums + 256;
constexpr size_t kScratchBytes = kOffPartial + align256(sizeof(float) * 5 * kBI * (size_t)kMaxSegs);

// The scratch (about 4.4 MB per GPU).
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

// force4[i] = (F, sum_j r^-12 - r^-6); block sums of V and W.
__global__ void k_static_reduce(const float* partial, const BlockInfo* blocks, const DevScalars* sc, float4* force,
                                double* blk) {
  __shared__ double sh[2 * 32];
  const BlockInfo bi = blocks[blockIdx.x];
  const int tid = threadIdx.x;
  double part[2] = {0.0, 0.0};
  if (tid < bi.n_i) {
    double S[5] = {0, 0, 0, 0, 0};
    for (int k = 0; k < bi.seg_count; ++k) {
      const size_t base = (size_t)(bi.seg_first + k) * 5 * kBI + tid;
      for (int c = 0; c < 5; ++c) S[c] += (double)partial[base + (size_t)c * kBI];
    }
    const double fs = sc->fscale;
    force[bi.i0 + tid] = make_float4((float)(fs * S[0]), (float)(fs * S[1]), (float)(fs * S[2]), (float)(S[3] - S[4]));
    part[0] = 2.0 * (S[3] - S[4]);          // V share: 4 eps (A - B) / 2
    part[1] = 4.0 * (12.0 * S[3] - 6.0 * S[4]);  // W share
  }
  block_sum<2>(part, sh);
  if (tid == 0) {
    blk[(size_t)blockIdx.x * 8] = part[0];
    blk[(size_t)blockIdx.x * 8 + 1] = part[1];
  }
}

__global__ void k_static_sums(const double* blk, int nb, double* sums) {
  __shared__ double sh[2 * 32];
  double acc[2] = {0.0, 0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    acc[0] += blk[(size_t)b * 8];
    acc[1] += blk[(size_t)b * 8 + 1];
  }
  block_sum<2>(acc, sh);
  if (threadIdx.x == 0) {
    sums[0] = acc[0];
    sums[1] = acc[1];
  }
}

// Host-side schedule for one box in fixed-size static storage (the same
// stream-K split as lj_schedule.cpp, restricted to a single box).
struct StaticPlan {
  int n = -1, G = 0, nblocks = 0, nseg = 0;
  BlockInfo blocks[kMaxBlocks];
  int cta_begin[kMaxCtas + 1];
  int cta_block[kMaxCtas];
  int cta_jt[kMaxCtas];
};

void plan_static(int n, int ctas, StaticPlan* s) {
  const int nb = (n + kBI - 1) / kBI, njt = (n + kTile - 1) / kTile;
  const int ntiles = nb * njt;
  int G = ctas < ntiles ? ctas : ntiles;
  if (G > 8 * nb) G = 8 * nb;  // at most 8 CTAs (segments) per i-block
  if (G > kMaxCtas) G = kMaxCtas;
  constexpr int kOverhead = 8;
  auto cost_before = [&](int t) -> long long {  // tiles are equal-cost except the ragged last of each block
    const int b = t / njt, jt = t % njt;
    const long long per_block = (long long)n + (long long)njt * kOverhead;
    const long long j = (long long)jt * kTile < n ? (long long)jt * kTile : n;
    return b * per_block + j + (long long)jt * kOverhead;
  };
  const long long total = (long long)nb * ((long long)n + (long long)njt * kOverhead);
  int t = 0;
  for (int g = 0; g < G; ++g) {
    const long long target = total * g / G;
    while (t < ntiles && cost_before(t) < target) ++t;
    s->cta_begin[g] = t;
  }
  s->cta_begin[0] = 0;
  for (int g = 1; g < G; ++g) s->cta_begin[g] = s->cta_begin[g] > s->cta_begin[g - 1] + 1 ? s->cta_begin[g] : s->cta_begin[g - 1] + 1;
  for (int g = 1; g < G; ++g) s->cta_begin[g] = s->cta_begin[g] < ntiles - (G - g) ? s->cta_begin[g] : ntiles - (G - g);
  s->cta_begin[G] = ntiles;
  for (int g = 0; g < G; ++g) {
    s->cta_block[g] = s->cta_begin[g] / njt;
    s->cta_jt[g] = s->cta_begin[g] % njt;
  }
  int seg = 0, g = 0;
  for (int b = 0; b < nb; ++b) {
    const int t0 = b * njt, t1 = (b + 1) * njt;
    while (g + 1 < G && s->cta_begin[g + 1] <= t0) ++g;
    int gh = g;
    while (gh + 1 < G && s->cta_begin[gh + 1] < t1) ++gh;
    BlockInfo& bi = s->blocks[b];
    bi = BlockInfo{};
    bi.sys = 0;
    bi.i0 = b * kBI;
    bi.n_i = n - b * kBI < kBI ? n - b * kBI : kBI;
    bi.p0 = 0;
    bi.n_sys = n;
    bi.njt = njt;
    bi.seg_first = seg;
    bi.seg_count = gh - g + 1;
    bi.g_first = g;
    seg += gh - g + 1;
  }
  s->n = n;
  s->G = G;
  s->nblocks = nb;
  s->nseg = seg;
}

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
unsigned char* g_static_ptr[kMaxDevices] = {nullptr};
int g_static_plan_n[kMaxDevices];
int g_static_sms[kMaxDevices];
int g_static_G[kMaxDevices];        // launch sizes of the plan each device holds
int g_static_nblocks[kMaxDevices];
StaticPlan g_static_plan;            // host staging of the plan being uploaded

int static_fail(int code, const char* msg) {
  std::fprintf(stderr, "lj_forces_static: %s\n", msg);
  return code;
}

}  // namespace
}  // namespace ljgb

using namespace ljgb;

extern "C" lj_status lj_forces_static(const float* pos4, float* force4, double* sums, int32_t n, float box,
                                      int32_t periodic, void* stream) {
  if (!pos4 || !force4) return (lj_status)static_fail(LJ_ERR_INVALID, "pos4 and force4 must be device pointers");
  if (n < 2) return (lj_status)static_fail(LJ_ERR_INVALID, "n must be >= 2");
  if (n > kStaticMaxParticles) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "n = %d exceeds the static scratch limit of %d particles; use lj_create / "
                  "calculateNForces for larger boxes", n, kStaticMaxParticles);
    return (lj_status)static_fail(LJ_ERR_INVALID, msg);
  }
  if (periodic && !(box > 0.0f)) return (lj_status)static_fail(LJ_ERR_INVALID, "box must be > 0 for a periodic box");
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return (lj_status)static_fail(LJ_ERR_UNSUPPORTED, "the stream is being captured (each call reads its results "
                                  "back to the host and synchronises the stream)");
  std::lock_guard<std::mutex> lk(g_static_mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return (lj_status)static_fail(LJ_ERR_NO_DEVICE, "no current CUDA device");
  // The device address of the scratch array on this device.  Looked up on
  // every call: a cudaDeviceReset by the embedding program gives the module
  // a new load, and the schedule cached in the array is then gone.
  void* addr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&addr, g_static_scratch);
  if (e != cudaSuccess) return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
  if (!g_static_ptr[dev]) {
    // The scratch layout is sized for kShapes[kShape]; refuse to launch if
    // that table entry no longer is the 128-thread, 256-record shape.
    if (kShape >= kNumShapes || kShapes[kShape].threads != kBI || kShapes[kShape].tile != kTile)
      return (lj_status)static_fail(LJ_ERR_INVALID, "pair-kernel shape 0 is not the 128-thread / 256-record "
                                    "shape the static scratch layout is sized for");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
    g_static_sms[dev] = sms;
  }
  if (g_static_ptr[dev] != static_cast<unsigned char*>(addr)) {
    g_static_ptr[dev] = static_cast<unsigned char*>(addr);
    g_static_plan_n[dev] = -1;
  }
  unsigned char* base = g_static_ptr[dev];
  DevScalars* sc = reinterpret_cast<DevScalars*>(base + kOffFrame);
  int* status = reinterpret_cast<int*>(base + kOffStatus);
  int4* q = reinterpret_cast<int4*>(base + kOffQ);
  BlockInfo* blocks = reinterpret_cast<BlockInfo*>(base + kOffBlocks);
  int* cta_begin = reinterpret_cast<int*>(base + kOffCtaBegin);
  int* cta_block = reinterpret_cast<int*>(base + kOffCtaBlock);
  int* cta_jt = reinterpret_cast<int*>(base + kOffCtaJt);
  double* blk = reinterpret_cast<double*>(base + kOffBlk);
  double* dsums = reinterpret_cast<double*>(base + kOffSums);
  float* partial = reinterpret_cast<float*>(base + kOffPartial);

  // The work schedule depends only on n (and the device); it stays in the
  // array until a call with another n replaces it.
  if (g_static_plan_n[dev] != n) {
    int per_sm = 0;
    e = pair_occupancy(0, kShape, &per_sm);
    if (e != cudaSuccess) return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
    plan_static(n, g_static_sms[dev] * per_sm, &g_static_plan);
    const StaticPlan& p = g_static_plan;
    if (p.G > kMaxCtas || p.nseg > kMaxSegs || p.nblocks > kMaxBlocks)
      return (lj_status)static_fail(LJ_ERR_INVALID, "work schedule exceeds the static scratch layout");
    if ((e = cudaMemcpyAsync(blocks, p.blocks, sizeof(BlockInfo) * p.nblocks, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(cta_begin, p.cta_begin, sizeof(int) * (p.G + 1), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(cta_block, p.cta_block, sizeof(int) * p.G, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(cta_jt, p.cta_jt, sizeof(int) * p.G, cudaMemcpyHostToDevice, st)) ||
        (e = cudaStreamSynchronize(st)))
      return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
    g_static_plan_n[dev] = n;
    g_static_G[dev] = p.G;
    g_static_nblocks[dev] = p.nblocks;
  }
  const int G = g_static_G[dev], nblocks = g_static_nblocks[dev];
  const float4* pos = reinterpret_cast<const float4*>(pos4);
  const int nbb = (n + kBboxThreads - 1) / kBboxThreads;
  if (!periodic && (e = launch_float4_bbox(pos, n, blk, st)) != cudaSuccess)
    return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
  if ((e = launch_float4_frame(blk, nbb, periodic ? 1 : 0, (double)box, sc, status, st)) != cudaSuccess ||
      (e = launch_float4_quantize(pos, n, sc, q, st)) != cudaSuccess)
    return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
  PairArgs a{};
  a.q = q;
  a.blocks = blocks;
  a.cta_tile_begin = cta_begin;
  a.cta_lo = nullptr;  // whole-tile ranges (the plan above cuts on tiles only)
  a.cta_block = cta_block;
  a.cta_jt = cta_jt;
  a.sc = sc;
  a.partial = partial;
  a.status = status;
  a.hist = HistArgs{0, 1, 1.0f, 0.0f, nullptr};
  if ((e = launch_pairs(0, kShape, true, false, a, G, st)) != cudaSuccess)
    return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
  k_static_reduce<<<nblocks, kBI, 0, st>>>(partial, blocks, sc, reinterpret_cast<float4*>(force4), blk);
  k_static_sums<<<1, 256, 0, st>>>(blk, nblocks, dsums);
  if ((e = cudaGetLastError()) != cudaSuccess) return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
  int hs = 0;
  double hsum[2] = {0, 0};
  if ((e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
      (e = cudaMemcpyAsync(hsum, dsums, sizeof(hsum), cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
    return (lj_status)static_fail(LJ_ERR_CUDA, cudaGetErrorString(e));
  if (hs & LJ_DEVFLAG_TIMEOUT) return (lj_status)static_fail(LJ_ERR_DEVICE_TIMEOUT, "a device-side wait timed out");
  if (sums) {
    sums[0] = hsum[0];
    sums[1] = hsum[1];
  }
  return LJ_OK;
}
