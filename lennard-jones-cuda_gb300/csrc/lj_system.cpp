// lj_system.cpp -- the lj_* C ABI: handle lifetime, device memory, step
// graphs, observables, histograms, autotuning and profiling.
//
// One lj_system owns one or more boxes (a batch shares one persistent pair
// launch per step).  Host code never loops over particles except to sample the
// initial state; all per-step work runs in the kernels of lj_pairs.cu and
// lj_integrate.cu, enqueued on the handle's stream as captured CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "lj_gb300.h"
#include "lj_init.h"
#include "lj_kernels.h"
#include "lj_schedule.h"

using namespace ljgb;

// ---- allocation hook -------------------------------------------------------
// g_alloc_budget < 0: allocations go to CUDA.  >= 0: that many more succeed,
// every later one fails with cudaErrorMemoryAllocation (no CUDA call made)
// until lj_debug_fail_allocations(-1).
static std::atomic<long long> g_alloc_budget{-1};

static bool allocation_refused() {
  long long b = g_alloc_budget.load();
  while (b >= 0) {
    if (b == 0) return true;
    if (g_alloc_budget.compare_exchange_weak(b, b - 1)) return false;
  }
  return false;
}

namespace ljgb {

cudaError_t device_alloc(void** p, size_t bytes) {
  *p = nullptr;
  if (allocation_refused()) return cudaErrorMemoryAllocation;
  return cudaMalloc(p, bytes);
}

cudaError_t pinned_alloc(void** p, size_t bytes) {
  *p = nullptr;
  if (allocation_refused()) return cudaErrorMemoryAllocation;
  return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

}  // namespace ljgb

extern "C" lj_status lj_debug_fail_allocations(int64_t after) {
  g_alloc_budget.store(after < 0 ? -1 : after);
  return LJ_OK;
}

namespace {

thread_local std::string g_create_error;

// Tile overhead in j-record units (barrier, compensation, refill) used to
// weight ragged tiles in the stream-K split.
constexpr int kTileOverhead = 8;
constexpr int kMaxSegmentsPerBlock = 8;

// Owned device array.  Movable, not copyable; freed on destruction (or
// explicitly).
// alloc() replaces the contents: on failure the buffer is left empty.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      free();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { free(); }
  cudaError_t alloc(size_t count) {
    free();
    if (count == 0) return cudaSuccess;
    void* q = nullptr;
    const cudaError_t e = device_alloc(&q, sizeof(T) * count);
    if (e != cudaSuccess) return e;
    p = static_cast<T*>(q);
    n = count;
    return cudaSuccess;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void swap(DevBuf& o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
  }
};

// Page-locked host memory: the device writes into it with asynchronous
// copies on the handle's stream, read by the host after one synchronisation.
template <typename T>
struct PinnedBuf {
  T* p = nullptr;
  size_t n = 0;
  void* dev = nullptr;  // the same memory's device address (mapped), nullptr if it has none
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  PinnedBuf(PinnedBuf&& o) noexcept : p(o.p), n(o.n), dev(o.dev) {
    o.p = nullptr;
    o.n = 0;
    o.dev = nullptr;
  }
  PinnedBuf& operator=(PinnedBuf&& o) noexcept {
    if (this != &o) {
      free();
      p = o.p;
      n = o.n;
      dev = o.dev;
      o.p = nullptr;
      o.n = 0;
      o.dev = nullptr;
    }
    return *this;
  }
  ~PinnedBuf() { free(); }
  cudaError_t alloc(size_t count) {
    free();
    if (count == 0) return cudaSuccess;
    void* q = nullptr;
    const cudaError_t e = pinned_alloc(&q, sizeof(T) * count);
    if (e != cudaSuccess) return e;
    p = static_cast<T*>(q);
    n = count;
    if (cudaHostGetDevicePointer(&dev, q, 0) != cudaSuccess) {
      dev = nullptr;
      (void)cudaGetLastError();
    }
    return cudaSuccess;
  }
  void free() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    dev = nullptr;
  }
};

// The device address of a caller's host buffer when it is page-locked and
// mapped into the current device's address space (lj_host_alloc memory,
// other page-locked allocations): kernels then read or write it directly
// (over NVLink-C2C on Grace) instead of a staged copy.  nullptr otherwise
// (pageable memory takes the staged path).
void* mapped_device_ptr(const void* host) {
  if (!host) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

struct GraphEntry {
  cudaGraph_t graph = nullptr;  // kept: exec-graph node updates name nodes of this graph
  cudaGraphExec_t exec = nullptr;
  int kernels = 0;
  bool profiled = false;
  cudaGraphNode_t ev_nodes[4] = {nullptr, nullptr, nullptr, nullptr};  // step start, pair start, pair end, step end
};

}  // namespace

struct lj_system {
  // configuration per box
  std::vector<lj_config> cfg;
  std::vector<BoxArgs> boxes;
  int nsys = 0;
  int ntotal = 0;  // particles over all boxes
  int npad = 0;
  int device = 0;
  int num_sms = 0;
  int prec = LJ_PREC_MIXED;
  bool any_nonperiodic = false;
  bool any_open = false;  // a box without walls (bc 2): its frame follows the particles

  // kernel shape / schedule
  int shape = 0;        // index into kShapes (MIXED)
  int forced_shape = -1;
  // Threads per particle: the most CTAs (j-range splits) one i-block is cut
  // into, each giving its particles one thread over part of the j range.
  int split_cap = kMaxSegmentsPerBlock;
  int forced_split = 0;  // > 0: set by lj_set_split_cap, kept by the autotuner
  bool tuned = false;
  Schedule sched;
  int BI = 128;
  int sched_shape = -1;  // shape and split cap the uploaded schedule was built for
  int sched_split = 0;

  // device memory
  DevBuf<double> x, v, f, tf, e, w;
  DevBuf<double> stage;          // 3 x (N,3) interleaved host-format arrays: positions, velocities, forces
  DevBuf<int> bad;               // lowest index of a non-finite uploaded value (INT_MAX: none)
  DevBuf<int> mb_ticket;         // read-back launch: [0] boxes finalized, [1] CTAs done (0 between launches)
  PinnedBuf<int> h_words;        // [0] status, [1] bad index: read back after one synchronisation;
                                 // [2] completion word of the last read-back launch
  int mb_seq = 0;                // last completion word queued
  int mb_wait = 0;               // completion word finish_status waits for (0: synchronise the stream)
  bool upload_check_pending = false;  // lj_set_state_async queued a finiteness check not yet read back
  bool bad_clean = false;             // s->bad holds 0x7f7f7f7f (reset by the read-back of a check)
  PinnedBuf<DevScalars> h_sc;    // per-box scalars read back
  DevBuf<int4> q, q2;  // fixed-point shadow, double-buffered for the fused step
  DevBuf<double4_32a> xd;
  DevBuf<int> blk_cnt, glob_cnt;  // fused-step completion counters
  int qpar = 0;             // which of q / q2 holds the current shadow
  bool obs_maybe_pending = false;  // a fused step left observables pending (DevScalars::obs_pending)
  bool pred_ready = false;  // current shadow = predictor x + dt v + dt^2 F/2 for pred_dt
  double pred_dt = 0.0;
  DevBuf<BlockInfo> blocks;
  DevBuf<int> cta_tile_begin, cta_lo, cta_block, cta_jt, sys_block_first;
  DevBuf<DevScalars> sc;
  DevBuf<BoxArgs> dboxes;
  DevBuf<double> blk_part;
  DevBuf<float> partial;  // sized in bytes/4 to also hold doubles
  DevBuf<int> status;
  DevBuf<DevRecord> records;
  DevBuf<unsigned long long> hist;
  int rec_cap = 0;

  // per-step subsystem counters (lj_counters_configure): one row of
  // counter_bins ints per step in a ring of counter_cap rows
  std::vector<CounterDev> counters;
  DevBuf<CounterDev> dcounters;
  DevBuf<int> counter_ring;
  DevBuf<int> counter_state;     // kCtr* words: the device's copy of the bookkeeping below
  DevBuf<int> counter_part;      // per-CTA counts of the counting launch
  int counter_bins = 0, counter_cap = 0;
  int counter_every = 1;         // count after every counter_every-th step
  long long counter_phase = 0;   // steps since the last counted one
  long long counter_head = 0, counter_tail = 0;  // rows written / rows read
  // RDF summed over steps (lj_rdf_accumulate), from its own shadow buffer
  bool rdf_acc = false;
  HistArgs rdf_args{};
  DevBuf<unsigned long long> rdf_sum;
  DevBuf<int4> qhist;
  long long rdf_samples = 0;
  // CTA ranges of the histogram-only pair pass: the same blocks and tiles as
  // `sched`, cut for the CTAs the histogram variant holds resident (more per
  // SM than the force kernel: fewer registers, a small shared histogram).
  Schedule hsched;
  int hist_shape = -1, hist_nb = -1;
  DevBuf<int> h_cta_tile_begin, h_cta_lo, h_cta_block, h_cta_jt;

  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;

  std::map<int, GraphEntry> graphs;
  std::vector<cudaEvent_t> graph_events;  // placeholders captured into profiled graphs

  // profiling
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  long long prof_steps = 0, prof_pairs = 0;
  double prof_step_ms = 0, prof_pair_ms = 0;

  long long launches = 0;
  std::string err;
};

extern "C" {
static lj_status enqueue_read(lj_system* s, double* pos, double* vel, double* force, bool scalars);
}

namespace {

lj_status fail(lj_system* s, lj_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  else g_create_error = buf;
  return code;
}

#define LJ_CUDA(sys, call)                                                                      \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return fail(sys, e_ == cudaErrorMemoryAllocation ? LJ_ERR_OUT_OF_MEMORY : LJ_ERR_CUDA,    \
                  "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

lj_status flush_observables(lj_system* s);

StateArgs state_args(lj_system* s) {
  StateArgs a{};
  a.x = s->x.p;
  a.v = s->v.p;
  a.f = s->f.p;
  a.tf = s->tf.p;
  a.e = s->e.p;
  a.w = s->w.p;
  a.q = s->qpar ? s->q2.p : s->q.p;
  a.q_next = s->qpar ? s->q.p : s->q2.p;
  a.xd = s->xd.p;
  a.npad = s->npad;
  a.blocks = s->blocks.p;
  a.boxes = s->dboxes.p;
  a.sc = s->sc.p;
  a.sys_block_first = s->sys_block_first.p;
  a.blk_part = s->blk_part.p;
  a.partial = s->partial.p;
  a.prec = s->prec;
  a.bi_threads = s->BI;
  a.records = s->records.p;
  a.rec_stride = s->rec_cap;
  a.status = s->status.p;
  a.blk_cnt = s->blk_cnt.p;
  a.glob_cnt = s->glob_cnt.p;
  a.nblocks = (int)s->sched.blocks.size();
  a.nsys = s->nsys;
  a.obs_slot = 4 * s->qpar;
  a.ticket = 2 + s->qpar;
  return a;
}

PairArgs pair_args(lj_system* s) {
  PairArgs a{};
  a.q = s->qpar ? s->q2.p : s->q.p;
  a.xd = s->xd.p;
  a.blocks = s->blocks.p;
  a.cta_tile_begin = s->cta_tile_begin.p;
  a.cta_block = s->cta_block.p;
  a.cta_jt = s->cta_jt.p;
  a.cta_lo = s->cta_lo.p;
  a.sc = s->sc.p;
  a.boxes = s->dboxes.p;
  a.partial = s->partial.p;
  a.status = s->status.p;
  a.hist = HistArgs{0, 1, 1.0f, 0.0f, nullptr};
  return a;
}

int nblocks(const lj_system* s) { return (int)s->sched.blocks.size(); }

void clear_graphs(lj_system* s) {
  for (auto& kv : s->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  s->graphs.clear();
  for (auto e : s->graph_events) cudaEventDestroy(e);
  s->graph_events.clear();
}

lj_status validate(const lj_config* c, lj_system* s) {
  if (!c) return fail(s, LJ_ERR_INVALID, "config is NULL");
  if (c->n < 2) return fail(s, LJ_ERR_INVALID, "n must be >= 2 (got %d)", c->n);
  if (!(c->density > 0) || !std::isfinite(c->density)) return fail(s, LJ_ERR_INVALID, "density must be > 0");
  if (!(c->temperature >= 0) || !std::isfinite(c->temperature))
    return fail(s, LJ_ERR_INVALID, "temperature must be >= 0");
  if (c->boundary < 0 || c->boundary > 2) return fail(s, LJ_ERR_INVALID, "boundary must be 0, 1 or 2");
  if (c->precision != LJ_PREC_MIXED && c->precision != LJ_PREC_FP64)
    return fail(s, LJ_ERR_INVALID, "precision must be LJ_PREC_MIXED or LJ_PREC_FP64");
  if (!(c->epsilon > 0) || !(c->sigma > 0)) return fail(s, LJ_ERR_INVALID, "epsilon and sigma must be > 0");
  if (c->lattice != LJ_LATTICE_SC && c->lattice != LJ_LATTICE_FCC)
    return fail(s, LJ_ERR_INVALID, "lattice must be LJ_LATTICE_SC or LJ_LATTICE_FCC");
  if (!(c->jitter >= 0)) return fail(s, LJ_ERR_INVALID, "jitter must be >= 0");
  return LJ_OK;
}

BoxArgs box_args(const lj_config& c) {
  BoxArgs b{};
  b.N = c.n;
  b.bc = c.boundary;
  b.canonical = c.canonical ? 1 : 0;
  b.L = std::cbrt((double)c.n / c.density);
  b.invL = 1.0 / b.L;
  b.eps = c.epsilon;
  b.sigma = c.sigma;
  b.dt = 0.0;
  b.T0 = c.temperature;
  b.rho = c.density;
  return b;
}

lj_status upload_boxes(lj_system* s) {
  s->any_nonperiodic = false;
  s->any_open = false;
  for (auto& b : s->boxes) {
    s->any_nonperiodic |= (b.bc != 0);
    b.hdt = 0.5 * b.dt;
    b.qdt = 0.25 * b.dt;
    b.hdt2 = 0.5 * b.dt * b.dt;
    b.eps4 = 4.0 * b.eps;
    b.kT = 2.0 / (3.0 * b.N);
    b.kP = b.rho / b.N;
    b.inv3N = 1.0 / (3.0 * b.N);
    b.invT0 = b.T0 > 0 ? 1.0 / b.T0 : 0.0;
    b.wall_margin = std::max(b.sigma, 0.05 * b.L);
    s->any_open |= (b.bc == 2);
  }
  LJ_CUDA(s, cudaMemcpyAsync(s->dboxes.p, s->boxes.data(), sizeof(BoxArgs) * s->nsys, cudaMemcpyHostToDevice,
                             s->stream));
  return LJ_OK;
}

// Builds the stream-K schedule for the active shape and split cap and
// uploads its tables.  All-or-nothing: the new tables are allocated and
// filled beside the old ones and swapped in only once complete, so a
// failure (an allocation, say) leaves the handle on its previous schedule,
// with shape and split cap put back to the ones that schedule was built for.
lj_status build_and_swap_schedule(lj_system* s) {
  int threads, tile, blocks_per_sm = 0;
  if (s->prec == LJ_PREC_FP64) {
    threads = fp64_block_threads();
    tile = fp64_tile();
  } else {
    threads = kShapes[s->shape].threads;
    tile = kShapes[s->shape].tile;
  }
  LJ_CUDA(s, pair_occupancy(s->prec, s->shape, &blocks_per_sm));
  if (blocks_per_sm < 1) return fail(s, LJ_ERR_NO_DEVICE, "pair kernel cannot be resident on this device");
  std::vector<int> n(s->nsys);
  for (int k = 0; k < s->nsys; ++k) n[k] = s->cfg[k].n;
  // At most kMaxSegmentsPerBlock CTAs per i-block: a small box spread over
  // the whole persistent grid leaves each block dozens of partial segments,
  // and the block epilogue that sums them serially becomes the step's tail
  // (N=2048 EVN: 34.1 -> 25.8 us per step with 8; N >= 8 x 128 x SMs x
  // occupancy / 128 is unaffected).
  long long nbt = 0;
  for (int k = 0; k < s->nsys; ++k) nbt += (n[k] + threads - 1) / threads;
  const int G = (int)std::min<long long>((long long)s->num_sms * blocks_per_sm, nbt * s->split_cap);
  Schedule sch;
  if (!build_schedule(n.data(), s->nsys, threads, tile, G, kTileOverhead, &sch))
    return fail(s, LJ_ERR_INVALID, "cannot build the pair schedule");
  const int nb = (int)sch.blocks.size();
  DevBuf<BlockInfo> blocks;
  DevBuf<int> ctb, clo, cb, cj, sbf, bcnt, gcnt;
  DevBuf<double> bpart;
  DevBuf<float> partial;
  LJ_CUDA(s, blocks.alloc(nb));
  LJ_CUDA(s, ctb.alloc(sch.G + 1));
  LJ_CUDA(s, clo.alloc(sch.G + 1));
  LJ_CUDA(s, cb.alloc(sch.G));
  LJ_CUDA(s, cj.alloc(sch.G));
  LJ_CUDA(s, sbf.alloc(s->nsys + 1));
  LJ_CUDA(s, bpart.alloc((size_t)nb * 8));
  LJ_CUDA(s, bcnt.alloc(nb));
  LJ_CUDA(s, gcnt.alloc(4));
  // partial: nseg x 5 x BI values of 8 bytes (FP64) or 4 bytes (MIXED)
  const size_t vals = (size_t)sch.nseg * 5 * threads;
  LJ_CUDA(s, partial.alloc(vals * (s->prec == LJ_PREC_FP64 ? 2 : 1)));
  LJ_CUDA(s, cudaMemsetAsync(bcnt.p, 0, sizeof(int) * nb, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(gcnt.p, 0, sizeof(int) * gcnt.n, s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(blocks.p, sch.blocks.data(), sizeof(BlockInfo) * nb, cudaMemcpyHostToDevice, s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(ctb.p, sch.cta_tile_begin.data(), sizeof(int) * (sch.G + 1), cudaMemcpyHostToDevice,
                             s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(clo.p, sch.cta_lo.data(), sizeof(int) * (sch.G + 1), cudaMemcpyHostToDevice, s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(cb.p, sch.cta_block.data(), sizeof(int) * sch.G, cudaMemcpyHostToDevice, s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(cj.p, sch.cta_jt.data(), sizeof(int) * sch.G, cudaMemcpyHostToDevice, s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(sbf.p, sch.sys_block_first.data(), sizeof(int) * (s->nsys + 1), cudaMemcpyHostToDevice,
                             s->stream));
  // also waits for all earlier work on the stream, which may still read the
  // old tables freed below
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  clear_graphs(s);  // captured graphs name the old tables
  s->blocks.swap(blocks);
  s->cta_tile_begin.swap(ctb);
  s->cta_lo.swap(clo);
  s->cta_block.swap(cb);
  s->cta_jt.swap(cj);
  s->sys_block_first.swap(sbf);
  s->blk_part.swap(bpart);
  s->blk_cnt.swap(bcnt);
  s->glob_cnt.swap(gcnt);
  s->partial.swap(partial);
  s->sched = std::move(sch);
  s->BI = threads;
  s->hist_shape = -1;  // the histogram pass re-cuts its ranges on next use
  s->pred_ready = false;
  s->sched_shape = s->shape;
  s->sched_split = s->split_cap;
  return LJ_OK;
}

lj_status setup_schedule(lj_system* s) {
  const lj_status st = build_and_swap_schedule(s);
  if (st != LJ_OK && s->sched_shape >= 0) {
    s->shape = s->sched_shape;
    s->split_cap = s->sched_split;
  }
  return st;
}

// ---- kernel sequences ----------------------------------------------------

lj_status enqueue_frame_all(lj_system* s) {
  s->pred_ready = false;  // the current shadow becomes the positions themselves
  StateArgs a = state_args(s);
  const int nb = nblocks(s);
  LJ_CUDA(s, launch_bbox(a, nb, s->BI, s->stream));
  LJ_CUDA(s, launch_frame(a, s->nsys, false, s->stream));
  LJ_CUDA(s, launch_quantize(a, nb, s->BI, false, s->stream));
  s->launches += 3;
  return LJ_OK;
}

lj_status enqueue_pairs(lj_system* s, bool forces, bool hist, const HistArgs* h) {
  PairArgs p = pair_args(s);
  if (h) p.hist = *h;
  LJ_CUDA(s, launch_pairs(s->prec, s->shape, forces, hist, p, s->sched.G, s->stream));
  s->launches += 1;
  return LJ_OK;
}

// Arguments and grid of a histogram-only pair pass over shadow q with
// histogram h, on `shape` (the geometry of the active schedule).  The CTA
// ranges are cut for as many CTAs as that variant holds resident with h.nb
// bins, and kept until the shape, the bin count or the schedule changes.
lj_status hist_pass_args(lj_system* s, int shape, const int4* q, const HistArgs& h, PairArgs* out, int* grid) {
  if (shape != s->hist_shape || h.nb != s->hist_nb) {
    int per_sm = 0;
    LJ_CUDA(s, pair_hist_occupancy(shape, h.nb, &per_sm));
    if (per_sm < 1) return fail(s, LJ_ERR_NO_DEVICE, "histogram pair kernel cannot be resident on this device");
    std::vector<int> n(s->nsys);
    for (int k = 0; k < s->nsys; ++k) n[k] = s->cfg[k].n;
    Schedule sch;
    if (!build_schedule(n.data(), s->nsys, kShapes[shape].threads, kShapes[shape].tile, s->num_sms * per_sm,
                        kTileOverhead, &sch))
      return fail(s, LJ_ERR_INVALID, "cannot build the histogram schedule");
    if (sch.BI != s->sched.BI || sch.TILE != s->sched.TILE || sch.blocks.size() != s->sched.blocks.size())
      return fail(s, LJ_ERR_INVALID, "histogram schedule does not match the pair schedule's blocks");
    // new range tables beside the old ones, swapped in once complete
    const int G = sch.G;
    DevBuf<int> ctb, clo, cb, cj;
    LJ_CUDA(s, ctb.alloc(G + 1));
    LJ_CUDA(s, clo.alloc(G + 1));
    LJ_CUDA(s, cb.alloc(G));
    LJ_CUDA(s, cj.alloc(G));
    LJ_CUDA(s, cudaMemcpyAsync(ctb.p, sch.cta_tile_begin.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice,
                               s->stream));
    LJ_CUDA(s, cudaMemcpyAsync(clo.p, sch.cta_lo.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice, s->stream));
    LJ_CUDA(s, cudaMemcpyAsync(cb.p, sch.cta_block.data(), sizeof(int) * G, cudaMemcpyHostToDevice, s->stream));
    LJ_CUDA(s, cudaMemcpyAsync(cj.p, sch.cta_jt.data(), sizeof(int) * G, cudaMemcpyHostToDevice, s->stream));
    LJ_CUDA(s, cudaStreamSynchronize(s->stream));
    s->h_cta_tile_begin.swap(ctb);
    s->h_cta_lo.swap(clo);
    s->h_cta_block.swap(cb);
    s->h_cta_jt.swap(cj);
    s->hsched = std::move(sch);
    // step graphs that accumulate the RDF name the old tables (freed on return)
    if (s->rdf_acc) clear_graphs(s);
    s->hist_shape = shape;
    s->hist_nb = h.nb;
  }
  PairArgs p = pair_args(s);
  p.q = q;
  p.hist = h;
  p.cta_tile_begin = s->h_cta_tile_begin.p;
  p.cta_lo = s->h_cta_lo.p;
  p.cta_block = s->h_cta_block.p;
  p.cta_jt = s->h_cta_jt.p;
  *out = p;
  *grid = s->hsched.G;
  return LJ_OK;
}

// Force evaluation + observables at the current positions (CalculateForces +
// CalculateParameters).
lj_status enqueue_compute_forces(lj_system* s) {
  lj_status st = flush_observables(s);
  if (st) return st;
  st = enqueue_frame_all(s);
  if (st) return st;
  st = enqueue_pairs(s, true, false, nullptr);
  if (st) return st;
  StateArgs a = state_args(s);
  LJ_CUDA(s, launch_reduce(a, nblocks(s), s->BI, MODE_FORCES_ONLY, s->stream));
  LJ_CUDA(s, launch_observables(a, s->nsys, MODE_FORCES_ONLY, s->stream));
  s->launches += 2;
  return LJ_OK;
}

cudaEvent_t next_event(lj_system* s) {
  if (s->ev_used == s->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    s->ev_pool.push_back(e);
  }
  return s->ev_pool[s->ev_used++];
}

// The kernels of one Verlet step, enqueued on s->stream (captured or not).
// ev (optional): events recorded at step start, pair start, pair end, step end.
lj_status enqueue_step(lj_system* s, int mode, cudaEvent_t* ev, bool capture, int* kernels) {
  if (!capture) {
    lj_status st = flush_observables(s);
    if (st) return st;
  }
  StateArgs a = state_args(s);
  const int nb = nblocks(s);
  int k = 0;
  const unsigned flags = capture ? cudaEventRecordExternal : cudaEventRecordDefault;
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[0], s->stream, flags));
  LJ_CUDA(s, launch_drift_mode(a, nb, s->BI, mode, s->stream));
  ++k;
  if (s->any_nonperiodic) {
    LJ_CUDA(s, launch_frame(a, s->nsys, true, s->stream));
    LJ_CUDA(s, launch_quantize(a, nb, s->BI, true, s->stream));
    k += 2;
  }
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[1], s->stream, flags));
  {
    PairArgs p = pair_args(s);
    LJ_CUDA(s, launch_pairs(s->prec, s->shape, true, false, p, s->sched.G, s->stream));
    ++k;
  }
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[2], s->stream, flags));
  LJ_CUDA(s, launch_reduce(a, nb, s->BI, mode, s->stream));
  ++k;
  if (mode == MODE_TVN) {
    LJ_CUDA(s, launch_tvn_finish(a, nb, s->BI, s->stream));
    ++k;
  }
  LJ_CUDA(s, launch_observables(a, s->nsys, mode, s->stream));
  ++k;
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[3], s->stream, flags));
  if (kernels) *kernels = k;
  return LJ_OK;
}

// Fused step: the pair kernel carries the second half of the Verlet step in
// the last CTA of each i-block (EVN: everything, one kernel per step; TVN: the
// chi reduction, then k_tvn_close applies the rescale).  Needs a constant
// shadow frame (periodic or walled boxes, not open ones) and the MIXED kernel.
bool use_fused(const lj_system* s) { return s->prec == LJ_PREC_MIXED && !s->any_open; }

lj_status enqueue_step_fused(lj_system* s, int mode, cudaEvent_t* ev, bool capture, int* kernels) {
  StateArgs a = state_args(s);
  const int nb = nblocks(s);
  const unsigned flags = capture ? cudaEventRecordExternal : cudaEventRecordDefault;
  int k = 0;
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[0], s->stream, flags));
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[1], s->stream, flags));
  FusedPairArgs f{};
  f.pair = pair_args(s);
  f.st = a;
  LJ_CUDA(s, launch_pairs_fused(s->shape, mode, f, s->sched.G, s->stream));
  ++k;
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[2], s->stream, flags));
  if (mode == MODE_TVN) {
    LJ_CUDA(s, launch_tvn_close(a, nb, s->BI, s->stream));
    ++k;
  }
  if (ev) LJ_CUDA(s, cudaEventRecordWithFlags(ev[3], s->stream, flags));
  if (kernels) *kernels = k;
  return LJ_OK;
}

int step_mode(const lj_system* s) {
  // A batch with mixed ensembles steps every box with its own flag inside the
  // kernels; the launch sequence only needs to know whether any box is TVN.
  for (const auto& b : s->boxes)
    if (b.canonical) return MODE_TVN;
  return MODE_EVN;
}

lj_status enqueue_after_step(lj_system* s, const PairArgs* hist, int hist_grid, int* kernels);

lj_status get_graph(lj_system* s, int mode, GraphEntry** out) {
  const bool fused = use_fused(s);
  const bool counters = s->counter_cap > 0, rdf = s->rdf_acc;
  const int key = mode * 128 + (rdf ? 64 : 0) + (counters ? 32 : 0) + (fused ? 8 : 0) + (fused && s->qpar ? 4 : 0) +
                  (s->any_nonperiodic ? 2 : 0) + (s->profiling ? 1 : 0);
  auto it = s->graphs.find(key);
  if (it != s->graphs.end()) {
    *out = &it->second;
    return LJ_OK;
  }
  // The RDF pass's range tables are built before the capture (building them
  // may allocate and synchronise).
  PairArgs hist{};
  int hist_grid = 0;
  if (rdf) {
    const int shape = (s->prec == LJ_PREC_MIXED) ? s->shape : 0;
    lj_status hst = hist_pass_args(s, shape, s->qhist.p, s->rdf_args, &hist, &hist_grid);
    if (hst) return hst;
  }
  GraphEntry ge;
  ge.profiled = s->profiling;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  if (ge.profiled)
    for (auto& e : ev) {
      LJ_CUDA(s, cudaEventCreate(&e));
    }
  cudaGraph_t g = nullptr;
  LJ_CUDA(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  lj_status st = fused ? enqueue_step_fused(s, mode, ge.profiled ? ev : nullptr, true, &ge.kernels)
                       : enqueue_step(s, mode, ge.profiled ? ev : nullptr, true, &ge.kernels);
  if (!st && (counters || rdf)) st = enqueue_after_step(s, &hist, hist_grid, &ge.kernels);
  cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
  if (st || ce != cudaSuccess) {  // nothing of a failed capture is kept
    if (g) cudaGraphDestroy(g);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (st) return st;
    LJ_CUDA(s, ce);
  }
  if (ge.profiled) {
    size_t nn = 0;
    LJ_CUDA(s, cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    LJ_CUDA(s, cudaGraphGetNodes(g, nodes.data(), &nn));
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      LJ_CUDA(s, cudaGraphNodeGetType(nd, &t));
      if (t != cudaGraphNodeTypeEventRecord) continue;
      cudaEvent_t e;
      LJ_CUDA(s, cudaGraphEventRecordNodeGetEvent(nd, &e));
      for (int k = 0; k < 4; ++k)
        if (e == ev[k]) ge.ev_nodes[k] = nd;
    }
  }
  LJ_CUDA(s, cudaGraphInstantiate(&ge.exec, g, 0));
  ge.graph = g;
  // The capture-time events stay alive with the graph; before every launch
  // the nodes are pointed at fresh events from the pool.
  for (auto& e : ev)
    if (e) s->graph_events.push_back(e);
  auto res = s->graphs.emplace(key, ge);
  *out = &res.first->second;
  return LJ_OK;
}

// Computes the observables that fused steps left pending (k_obs_finalize;
// entries a later pair kernel already consumed are skipped on the device).
// Called before anything reads or changes the observables, the running sums
// or the block partials; a read-back that returns the observables computes
// them in its own launch instead.
lj_status flush_observables(lj_system* s) {
  if (!s->obs_maybe_pending) return LJ_OK;
  s->obs_maybe_pending = false;
  LJ_CUDA(s, launch_obs_finalize(state_args(s), s->nsys, s->stream));
  s->launches += 1;
  return LJ_OK;
}

// Work after every step: the subsystem counters and the summed RDF, when
// enabled (plain launches after the step's graph).
// The per-step work that follows a step when counters or RDF accumulation are
// on, enqueued inside the step graph's capture (its per-step state -- ring
// row, counting phase -- lives on the device): the counters' bookkeeping and
// histogram, and the RDF of the step's positions (quantized into a shadow of
// their own: the step's shadow buffer holds the next step's prediction) added
// into the running sum.  `hist` are the histogram pass's arguments, prepared
// before the capture.
lj_status enqueue_after_step(lj_system* s, const PairArgs* hist, int hist_grid, int* kernels) {
  if (s->counter_cap > 0) {
    LJ_CUDA(s, launch_counters(state_args(s), s->dcounters.p, (int)s->counters.size(), s->counter_bins,
                               s->counter_state.p, s->counter_ring.p, s->counter_part.p, s->ntotal, s->stream));
    *kernels += 1;
  }
  if (s->rdf_acc) {
    StateArgs a = state_args(s);
    a.q = s->qhist.p;
    LJ_CUDA(s, launch_quantize(a, nblocks(s), s->BI, false, s->stream));
    const int shape = (s->prec == LJ_PREC_MIXED) ? s->shape : 0;
    LJ_CUDA(s, launch_pairs(LJ_PREC_MIXED, shape, false, true, *hist, hist_grid, s->stream));
    *kernels += 2;
  }
  return LJ_OK;
}

// The host's mirror of that bookkeeping, after every launched step: the same
// counting decision as k_counters, and one more RDF sample.
void after_step_host(lj_system* s) {
  if (s->counter_cap > 0 && ++s->counter_phase >= s->counter_every) {
    s->counter_phase = 0;
    s->counter_head += 1;
  }
  if (s->rdf_acc) s->rdf_samples += 1;
}

// Waits for the handle's stream and reports the device status word, read
// back by a copy enqueued behind the work (one synchronisation in all).
// Queues the copies of the status word (and a pending upload check's bad
// index) into h_words.
lj_status enqueue_status_read(lj_system* s) {
  LJ_CUDA(s, cudaMemcpyAsync(s->h_words.p, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  if (s->upload_check_pending)
    LJ_CUDA(s, cudaMemcpyAsync(s->h_words.p + 1, s->bad.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  return LJ_OK;
}

// Waits for the read-back launch's completion word when one was queued (it
// is written after every store of that launch, the last work queued; a word
// that does not come within 20 ms -- a long run of steps before it, or a
// failed launch -- falls back to synchronising the stream, which also
// reports errors), else synchronises the stream; then reports what the
// status words queued for h_words say.
static bool wait_completion_word(lj_system* s) {
  const int want = s->mb_wait;
  s->mb_wait = 0;
  if (!want) return false;
  const volatile int* w = s->h_words.p + 2;
  const auto t0 = std::chrono::steady_clock::now();
  for (unsigned it = 1;; ++it) {
    if (*w == want) {
      std::atomic_thread_fence(std::memory_order_acquire);
      return true;
    }
    if ((it & 255u) == 0 && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(20)) return false;
  }
}

lj_status finish_status(lj_system* s) {
  const bool upload = s->upload_check_pending;
  if (!wait_completion_word(s)) LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  s->upload_check_pending = false;
  if (upload && s->h_words.p[1] != 0x7f7f7f7f)
    return fail(s, LJ_ERR_INVALID, "an array queued by lj_set_state_async held a non-finite value (element %d of "
                "the staged upload); it was dropped and the state left as it was", s->h_words.p[1]);
  const int st = s->h_words.p[0];
  if (st) {
    // (on the handle's stream: it is non-blocking, so a legacy-stream memset
    // would not be ordered before the next launch)
    LJ_CUDA(s, cudaMemsetAsync(s->status.p, 0, sizeof(int), s->stream));
    // A failed launch may leave the fused-step counters mid-count.
    if (s->blk_cnt.p) LJ_CUDA(s, cudaMemsetAsync(s->blk_cnt.p, 0, sizeof(int) * s->blk_cnt.n, s->stream));
    if (s->glob_cnt.p) LJ_CUDA(s, cudaMemsetAsync(s->glob_cnt.p, 0, sizeof(int) * s->glob_cnt.n, s->stream));
    if (s->mb_ticket.p) LJ_CUDA(s, cudaMemsetAsync(s->mb_ticket.p, 0, 2 * sizeof(int), s->stream));
    s->pred_ready = false;
    if (st & LJ_DEVFLAG_TIMEOUT)
      return fail(s, LJ_ERR_DEVICE_TIMEOUT, "a device-side wait timed out; the results of that launch are void");
    if (st & LJ_DEVFLAG_NONFINITE)
      return fail(s, LJ_ERR_NONFINITE, "an observable became NaN/Inf (overlapping particles or blow-up)");
    if (st & LJ_DEVFLAG_ESCAPED)
      return fail(s, LJ_ERR_ESCAPED,
                  "a particle of a walled box went further than m = max(sigma, L/20) beyond the walls and the "
                  "positions it started from (blow-up)");
  }
  return LJ_OK;
}

lj_status sync_status(lj_system* s) {
  lj_status st = enqueue_status_read(s);
  if (st) return st;
  return finish_status(s);
}

lj_status check_status(lj_system* s) {
  lj_status fst = flush_observables(s);
  if (fst) return fst;
  return sync_status(s);
}

lj_status alloc_state(lj_system* s) {
  s->npad = (s->ntotal + 255) / 256 * 256;
  const size_t n3 = 3 * (size_t)s->npad;
  LJ_CUDA(s, s->x.alloc(n3));
  LJ_CUDA(s, s->v.alloc(n3));
  LJ_CUDA(s, s->f.alloc(n3));
  LJ_CUDA(s, s->tf.alloc(n3));
  LJ_CUDA(s, s->stage.alloc(4 * n3));  // uploads: 2 (N,3) + 2 component-major arrays; reads: 3 (N,3)
  LJ_CUDA(s, s->bad.alloc(1));
  LJ_CUDA(s, s->mb_ticket.alloc(2));
  LJ_CUDA(s, s->h_words.alloc(3));
  LJ_CUDA(s, s->h_sc.alloc(s->nsys));
  LJ_CUDA(s, s->e.alloc(s->npad));
  LJ_CUDA(s, s->w.alloc(s->npad));
  LJ_CUDA(s, s->q.alloc(s->npad));
  LJ_CUDA(s, s->q2.alloc(s->npad));
  LJ_CUDA(s, s->xd.alloc(s->npad));
  LJ_CUDA(s, s->sc.alloc(s->nsys));
  LJ_CUDA(s, s->dboxes.alloc(s->nsys));
  LJ_CUDA(s, s->status.alloc(1));
  LJ_CUDA(s, s->hist.alloc(kMaxHistBins));
  LJ_CUDA(s, cudaMemsetAsync(s->x.p, 0, sizeof(double) * n3, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->v.p, 0, sizeof(double) * n3, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->f.p, 0, sizeof(double) * n3, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->tf.p, 0, sizeof(double) * n3, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->q.p, 0, sizeof(int4) * s->npad, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->q2.p, 0, sizeof(int4) * s->npad, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->xd.p, 0, sizeof(double4_32a) * s->npad, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->sc.p, 0, sizeof(DevScalars) * s->nsys, s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->status.p, 0, sizeof(int), s->stream));
  LJ_CUDA(s, cudaMemsetAsync(s->mb_ticket.p, 0, 2 * sizeof(int), s->stream));
  return LJ_OK;
}

// Uploads an interleaved (N,3) host array of all boxes: one host->device copy
// into the staging buffer (direct DMA when the caller's buffer is pinned, see
// lj_host_alloc), then a device transpose into component-major storage.
lj_status upload_xyz(lj_system* s, const double* host, double* dev) {
  const size_t bytes = sizeof(double) * 3 * (size_t)s->ntotal;
  LJ_CUDA(s, cudaMemcpyAsync(s->stage.p, host, bytes, cudaMemcpyHostToDevice, s->stream));
  LJ_CUDA(s, launch_unpack(s->stage.p, dev, s->ntotal, s->npad, s->stream));
  s->launches += 1;
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  return LJ_OK;
}

// Per-box scalars into the pinned mirror h_sc (check_status semantics: one
// synchronisation, device status reported).
lj_status fetch_scalars(lj_system* s) {
  if (s->h_words.dev && s->h_sc.dev) {
    // one launch: pending observables, scalar block and status words
    lj_status st = enqueue_read(s, nullptr, nullptr, nullptr, true);
    if (st) return st;
    return finish_status(s);
  }
  lj_status st = flush_observables(s);
  if (st) return st;
  LJ_CUDA(s, cudaMemcpyAsync(s->h_sc.p, s->sc.p, sizeof(DevScalars) * s->nsys, cudaMemcpyDeviceToHost, s->stream));
  return sync_status(s);
}

lj_status read_scalars(lj_system* s, std::vector<DevScalars>& out) {
  lj_status st = flush_observables(s);
  if (st) return st;
  LJ_CUDA(s, cudaMemcpyAsync(s->h_sc.p, s->sc.p, sizeof(DevScalars) * s->nsys, cudaMemcpyDeviceToHost, s->stream));
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  out.assign(s->h_sc.p, s->h_sc.p + s->nsys);
  return LJ_OK;
}

lj_status write_scalars(lj_system* s, const std::vector<DevScalars>& in) {
  lj_status st = flush_observables(s);
  if (st) return st;
  LJ_CUDA(s, cudaMemcpyAsync(s->sc.p, in.data(), sizeof(DevScalars) * s->nsys, cudaMemcpyHostToDevice, s->stream));
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  return LJ_OK;
}

// A new schedule changes only how the pair sums are cut and rounded: the
// forces are recomputed for the next step, while the observables, the clock
// and the running averages stay as they were (the state did not change, so
// the recomputation is no new sample of the averages).
lj_status recompute_forces_keep_scalars(lj_system* s) {
  std::vector<DevScalars> sc;
  lj_status st = read_scalars(s, sc);
  if (st) return st;
  if ((st = enqueue_compute_forces(s))) return st;
  return write_scalars(s, sc);
}

void fill_obs(const DevScalars& d, lj_observables* o) {
  o->t = d.t;
  o->K = d.K;
  o->V = d.V;
  o->T = d.T;
  o->P = d.P_press;
  o->U = d.U;
  o->W = d.W;
  o->Pshear = d.Pshear;
  o->Tkin_tvn = d.Tkin;
  o->av_U_tot = d.av_U;
  o->av_T_tot = d.av_T;
  o->av_p_tot = d.av_p;
  o->av_iters = d.av_iters;
  o->step = d.step;
}

// Creates the handle for `nsys` boxes (a batch when nsys > 1); the initial
// state of every box is sampled from its own config.
lj_status create_impl(const lj_config* cfgs, int nsys, lj_system** out) {
  if (!out) return fail(nullptr, LJ_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!cfgs || nsys < 1) return fail(nullptr, LJ_ERR_INVALID, "no configuration");
  for (int k = 0; k < nsys; ++k) {
    lj_status st = validate(&cfgs[k], nullptr);
    if (st) return st;
    if (cfgs[k].precision != cfgs[0].precision || cfgs[k].device != cfgs[0].device ||
        (cfgs[k].canonical != 0) != (cfgs[0].canonical != 0))
      return fail(nullptr, LJ_ERR_INVALID, "all boxes of a batch must share precision, device and ensemble");
  }
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0)
    return fail(nullptr, LJ_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(ce));
  if (cfgs[0].device < 0 || cfgs[0].device >= ndev)
    return fail(nullptr, LJ_ERR_INVALID, "device %d out of range (%d devices)", cfgs[0].device, ndev);
  cudaDeviceProp prop;
  ce = cudaGetDeviceProperties(&prop, cfgs[0].device);
  if (ce != cudaSuccess) return fail(nullptr, LJ_ERR_NO_DEVICE, "%s", cudaGetErrorString(ce));
  if (prop.major != 10 || prop.minor != 3)
    return fail(nullptr, LJ_ERR_NO_DEVICE, "device %s is sm_%d%d; this library is built for sm_103a only",
                prop.name, prop.major, prop.minor);
  long long total = 0;
  for (int k = 0; k < nsys; ++k) total += cfgs[k].n;
  if (total > (1ll << 30)) return fail(nullptr, LJ_ERR_INVALID, "too many particles (%lld)", total);

  lj_system* s = new lj_system();
  s->nsys = nsys;
  s->cfg.assign(cfgs, cfgs + nsys);
  s->ntotal = (int)total;
  s->device = cfgs[0].device;
  s->num_sms = prop.multiProcessorCount;
  s->prec = cfgs[0].precision;
  for (int k = 0; k < nsys; ++k) s->boxes.push_back(box_args(cfgs[k]));
  auto bail = [&](lj_status st) {
    g_create_error = s->err;
    lj_destroy(s);
    return st;
  };
  DeviceGuard device_guard(s->device);
  if (!device_guard.ok()) return bail(fail(s, LJ_ERR_CUDA, "cudaSetDevice failed"));
  if (cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(s, LJ_ERR_CUDA, "cudaStreamCreate failed"));
  s->stream = s->own_stream;
  lj_status st = alloc_state(s);
  if (st) return bail(st);
  st = upload_boxes(s);
  if (st) return bail(st);
  // Shape: the reference's CUDABlockSize picks the nearest i-block size.
  s->shape = 0;
  if (cfgs[0].block_hint > 0 && s->prec == LJ_PREC_MIXED) {
    int best = 0;
    for (int k = 0; k < kNumShapes; ++k)
      if (std::abs(kShapes[k].threads - cfgs[0].block_hint) < std::abs(kShapes[best].threads - cfgs[0].block_hint))
        best = k;
    s->shape = best;
    s->forced_shape = best;
  }
  st = setup_schedule(s);
  if (st) return bail(st);
  // Initial state (host sampler), then forces and observables on the device.
  std::vector<double> pos(3 * (size_t)s->ntotal), vel(3 * (size_t)s->ntotal);
  size_t off = 0;
  for (int k = 0; k < nsys; ++k) {
    const lj_config& c = cfgs[k];
    if (!sample_initial_state(c.n, s->boxes[k].L, c.temperature, c.lattice, c.jitter, c.sigma, c.seed,
                              pos.data() + 3 * off, vel.data() + 3 * off))
      return bail(fail(s, LJ_ERR_INVALID, "initial-state sampling failed for box %d", k));
    off += c.n;
  }
  st = upload_xyz(s, pos.data(), s->x.p);
  if (st) return bail(st);
  st = upload_xyz(s, vel.data(), s->v.p);
  if (st) return bail(st);
  st = enqueue_compute_forces(s);
  if (st) return bail(st);
  st = check_status(s);
  if (st) return bail(st);
  // Reinitialize resets the averages after its CalculateParameters (MDSystem.cpp:112-113).
  std::vector<DevScalars> sc;
  st = read_scalars(s, sc);
  if (st) return bail(st);
  for (auto& d : sc) {
    d.av_U = d.av_T = d.av_p = 0.0;
    d.av_iters = 0;
  }
  st = write_scalars(s, sc);
  if (st) return bail(st);
  *out = s;
  return LJ_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

lj_status lj_config_default(lj_config* c) {
  if (!c) return LJ_ERR_INVALID;
  std::memset(c, 0, sizeof(*c));
  c->n = 128;
  c->temperature = 1.5;
  c->density = 0.2;
  c->canonical = 0;
  c->boundary = LJ_BC_PERIODIC;
  c->precision = LJ_PREC_MIXED;
  c->epsilon = 1.0;
  c->sigma = 1.0;
  c->lattice = LJ_LATTICE_SC;
  c->jitter = 0.0;
  c->seed = 1;
  c->block_hint = 0;
  c->device = 0;
  c->autotune = 1;
  return LJ_OK;
}

lj_status lj_create(const lj_config* cfg, lj_system** out) { return create_impl(cfg, 1, out); }

lj_status lj_batch_create(const lj_config* cfgs, int32_t nsys, lj_system** out) {
  return create_impl(cfgs, nsys, out);
}

lj_status lj_destroy(lj_system* s) {
  if (!s) return LJ_OK;
  DeviceGuard device_guard(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  clear_graphs(s);
  for (auto e : s->ev_pool) cudaEventDestroy(e);
  s->x.free();
  s->v.free();
  s->f.free();
  s->tf.free();
  s->e.free();
  s->w.free();
  s->stage.free();
  s->bad.free();
  s->h_words.free();
  s->h_sc.free();
  s->q.free();
  s->q2.free();
  s->xd.free();
  s->blk_cnt.free();
  s->glob_cnt.free();
  s->blocks.free();
  s->cta_tile_begin.free();
  s->dcounters.free();
  s->counter_ring.free();
  s->counter_state.free();
  s->counter_part.free();
  s->rdf_sum.free();
  s->qhist.free();
  s->h_cta_tile_begin.free();
  s->h_cta_lo.free();
  s->h_cta_block.free();
  s->h_cta_jt.free();
  s->cta_lo.free();
  s->cta_block.free();
  s->cta_jt.free();
  s->sys_block_first.free();
  s->sc.free();
  s->dboxes.free();
  s->blk_part.free();
  s->partial.free();
  s->status.free();
  s->records.free();
  s->hist.free();
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
  return LJ_OK;
}

const char* lj_last_error(const lj_system* s) { return s ? s->err.c_str() : g_create_error.c_str(); }

lj_status lj_get_info(const lj_system* s, int32_t* n, double* box) {
  if (!s) return LJ_ERR_INVALID;
  if (n) *n = s->cfg[0].n;
  if (box) *box = s->boxes[0].L;
  return LJ_OK;
}

lj_status lj_reinitialize(lj_system* s, const lj_config* cfg) {
  if (!s || !cfg) return LJ_ERR_INVALID;
  if (s->nsys != 1) return fail(s, LJ_ERR_UNSUPPORTED, "lj_reinitialize applies to single-box handles");
  lj_status st = validate(cfg, s);
  if (st) return st;
  lj_system* fresh = nullptr;
  st = create_impl(cfg, 1, &fresh);
  if (st) return fail(s, st, "%s", g_create_error.c_str());
  // Swap the new state into the caller's handle (the handle pointer stays valid).
  cudaStream_t user_stream = (s->stream != s->own_stream) ? s->stream : nullptr;
  std::swap(*s, *fresh);
  lj_destroy(fresh);
  if (user_stream) s->stream = user_stream;
  return LJ_OK;
}

// Both arrays go to the staging buffer in one pass and are checked there on
// the device; the state is written only if every value is finite, so a
// rejected call leaves it unchanged.  One synchronisation (the caller's
// buffers are free on return).
// Queues the upload of pos / vel: the finiteness check (lowest bad index into
// s->bad) with the transpose into the staging buffer, then the commit.
// A check still pending from an earlier queued upload keeps its index, so a
// rejection is never lost (later uploads are then dropped too).
// Page-locked mapped caller buffers are read by the kernels directly; others
// are copied to the staging buffer first.  Staging buffer: [0, 6 npad) the
// copied (N,3) host arrays, [6 npad, 12 npad) the component-major arrays
// checked before they are committed.
static lj_status enqueue_upload(lj_system* s, const double* pos, const double* vel) {
  s->pred_ready = false;
  const size_t n3 = 3 * (size_t)s->ntotal;
  const size_t pad3 = 3 * (size_t)s->npad;
  const double* src_pos = static_cast<const double*>(mapped_device_ptr(pos));
  const double* src_vel = static_cast<const double*>(mapped_device_ptr(vel));
  if (!s->upload_check_pending && !s->bad_clean)
    LJ_CUDA(s, cudaMemsetAsync(s->bad.p, 0x7f, sizeof(int), s->stream));
  s->bad_clean = false;
  if (pos && !src_pos) {
    LJ_CUDA(s, cudaMemcpyAsync(s->stage.p, pos, sizeof(double) * n3, cudaMemcpyHostToDevice, s->stream));
    src_pos = s->stage.p;
  }
  if (vel && !src_vel) {
    LJ_CUDA(s, cudaMemcpyAsync(s->stage.p + pad3, vel, sizeof(double) * n3, cudaMemcpyHostToDevice, s->stream));
    src_vel = s->stage.p + pad3;
  }
  double* spos = pos ? s->stage.p + 2 * pad3 : nullptr;
  double* svel = vel ? s->stage.p + 3 * pad3 : nullptr;
  LJ_CUDA(s, launch_upload_stage(pos ? src_pos : nullptr, vel ? src_vel : nullptr, s->ntotal, s->npad, spos, svel,
                                 s->bad.p, s->stream));
  // Periodic boxes on the fused step keep a fixed frame: the commit also
  // writes the predictor for the last step size used, so the next step needs
  // no predictor launch (a walled box's frame is rebuilt around the new
  // positions first, and its predictor follows at the step).
  const bool predict = use_fused(s) && !s->any_nonperiodic && s->boxes[0].dt > 0;
  LJ_CUDA(s, launch_upload_commit(state_args(s), nblocks(s), s->BI, spos, svel, s->bad.p, predict, s->stream));
  s->launches += 2;
  if (predict) {
    s->pred_ready = true;
    s->pred_dt = s->boxes[0].dt;
  }
  return LJ_OK;
}

lj_status lj_set_state(lj_system* s, const double* pos, const double* vel) {
  if (!s) return LJ_ERR_INVALID;
  if (!pos && !vel) return LJ_OK;
  DeviceGuard device_guard(s->device);
  lj_status fst = flush_observables(s);
  if (fst) return fst;
  // a rejection still pending from lj_set_state_async is reported first
  if (s->upload_check_pending && (fst = sync_status(s))) return fst;
  const size_t n3 = 3 * (size_t)s->ntotal;
  if ((fst = enqueue_upload(s, pos, vel))) return fst;
  LJ_CUDA(s, cudaMemcpyAsync(s->h_words.p + 1, s->bad.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  const int bad = s->h_words.p[1];
  if (bad != 0x7f7f7f7f) {
    const bool is_pos = pos && (size_t)bad < n3;
    return fail(s, LJ_ERR_INVALID, "%s of particle %zu is not finite", is_pos ? "position" : "velocity",
                ((size_t)bad % n3) / 3);
  }
  // A walled box keeps its fixed-point frame between steps: rebuild it
  // around the new positions.
  if (pos && s->any_nonperiodic) return enqueue_frame_all(s);
  return LJ_OK;
}

lj_status lj_set_state_async(lj_system* s, const double* pos, const double* vel) {
  if (!s) return LJ_ERR_INVALID;
  if (!pos && !vel) return LJ_OK;
  DeviceGuard device_guard(s->device);
  lj_status st = flush_observables(s);
  if (st) return st;
  if ((st = enqueue_upload(s, pos, vel))) return st;
  s->upload_check_pending = true;
  // A walled box keeps its fixed-point frame between steps: rebuild it
  // around the new positions (around the old ones if the upload is dropped).
  if (pos && s->any_nonperiodic) return enqueue_frame_all(s);
  return LJ_OK;
}

// Queues the read-back of the requested arrays behind the pending work, with
// the status words and, with `scalars`, the per-box scalar block into h_sc:
// one pack launch writes page-locked mapped destinations directly and the
// status words and scalars into the handle's mapped mirrors; other
// destinations get staged copies.  The caller finishes with finish_status.
static lj_status enqueue_read(lj_system* s, double* pos, double* vel, double* force, bool scalars) {
  const size_t n3 = 3 * (size_t)s->ntotal;
  const double* src[3] = {s->x.p, s->v.p, s->f.p};
  double* dst[3] = {pos, vel, force};
  XyzArrays xa{};
  double* host[3] = {nullptr, nullptr, nullptr};
  int na = 0;
  for (int k = 0; k < 3; ++k) {
    if (!dst[k]) continue;
    xa.src[na] = src[k];
    double* d = static_cast<double*>(mapped_device_ptr(dst[k]));
    if (d) {
      xa.dst[na] = d;
    } else {
      xa.dst[na] = s->stage.p + na * n3;
      host[na] = dst[k];
    }
    ++na;
  }
  const bool mailbox = s->h_words.dev && (!scalars || s->h_sc.dev);
  Mailbox mb{};
  if (mailbox) {
    mb.status = s->status.p;
    mb.bad = s->upload_check_pending ? s->bad.p : nullptr;
    if (mb.bad) s->bad_clean = true;  // the pack launch resets it after reading
    mb.words_out = static_cast<int*>(s->h_words.dev);
    if (scalars) {
      mb.sc = reinterpret_cast<const int*>(s->sc.p);
      mb.sc_out = static_cast<int*>(s->h_sc.dev);
      mb.sc_nwords = (int)(sizeof(DevScalars) * s->nsys / sizeof(int));
      // the pending observables are computed by the same launch
      mb.finalize = s->obs_maybe_pending ? 1 : 0;
      mb.ticket = s->mb_ticket.p;
      s->obs_maybe_pending = false;
    }
    // nothing is queued behind this launch (every destination is mapped):
    // the host may wait on its completion word alone
    bool staged = false;
    for (int k = 0; k < na; ++k) staged |= host[k] != nullptr;
    if (!staged) {
      s->mb_seq = s->mb_seq == INT32_MAX ? 1 : s->mb_seq + 1;
      mb.seq = s->mb_seq;
      mb.grid_ticket = s->mb_ticket.p + 1;
      // cleared by the host before the launch is queued: page-locked memory
      // comes back from the allocator holding what an earlier handle left
      *(volatile int*)(s->h_words.p + 2) = 0;
    }
  }
  if (scalars && !mailbox) {
    lj_status st = flush_observables(s);
    if (st) return st;
  }
  LJ_CUDA(s, launch_pack_multi(xa, na, s->ntotal, s->npad, mailbox ? &mb : nullptr, state_args(s), s->stream));
  if (na > 0 || mailbox) s->launches += 1;
  s->mb_wait = mb.seq;
  for (int k = 0; k < na; ++k)
    if (host[k])
      LJ_CUDA(s, cudaMemcpyAsync(host[k], xa.dst[k], sizeof(double) * n3, cudaMemcpyDeviceToHost, s->stream));
  if (!mailbox) {
    if (scalars)
      LJ_CUDA(s, cudaMemcpyAsync(s->h_sc.p, s->sc.p, sizeof(DevScalars) * s->nsys, cudaMemcpyDeviceToHost,
                                 s->stream));
    return enqueue_status_read(s);
  }
  return LJ_OK;
}

// All requested arrays are packed and copied behind the pending work; one
// synchronisation, which also reports the device status.
lj_status lj_get_state(lj_system* s, double* pos, double* vel, double* force) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = flush_observables(s);
  if (st) return st;
  if ((st = enqueue_read(s, pos, vel, force, false))) return st;
  return finish_status(s);
}

// lj_get_state and lj_get_observables behind a single synchronisation.
lj_status lj_get_state_observables(lj_system* s, double* pos, double* vel, double* force, lj_observables* out) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st;
  if (!out && (st = flush_observables(s))) return st;
  if ((st = enqueue_read(s, pos, vel, force, out != nullptr))) return st;
  if ((st = finish_status(s))) return st;
  if (out) fill_obs(s->h_sc.p[0], out);
  return LJ_OK;
}

// One host round trip of a caller that keeps the state on the host: queued
// upload, steps, and the read-back with the observables, one synchronisation.
lj_status lj_step_io(lj_system* s, const double* pos_in, const double* vel_in, double dt, int32_t nsteps,
                     double* pos_out, double* vel_out, double* force_out, lj_observables* out) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = lj_set_state_async(s, pos_in, vel_in);
  if (st) return st;
  if ((st = lj_step(s, dt, nsteps))) return st;
  return lj_get_state_observables(s, pos_out, vel_out, force_out, out);
}

lj_status lj_get_pair_sums(lj_system* s, double* e, double* w) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  if (e) LJ_CUDA(s, cudaMemcpy(e, s->e.p, sizeof(double) * s->ntotal, cudaMemcpyDeviceToHost));
  if (w) LJ_CUDA(s, cudaMemcpy(w, s->w.p, sizeof(double) * s->ntotal, cudaMemcpyDeviceToHost));
  return LJ_OK;
}

lj_status lj_compute_forces(lj_system* s) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  return enqueue_compute_forces(s);
}

lj_status lj_step(lj_system* s, double dt, int32_t nsteps) {
  if (!s) return LJ_ERR_INVALID;
  if (nsteps < 0) return fail(s, LJ_ERR_INVALID, "nsteps must be >= 0");
  if (!(dt > 0) || !std::isfinite(dt)) return fail(s, LJ_ERR_INVALID, "dt must be > 0");
  if (nsteps == 0) return LJ_OK;
  DeviceGuard device_guard(s->device);
  bool changed = false;
  for (auto& b : s->boxes)
    if (b.dt != dt) {
      b.dt = dt;
      changed = true;
    }
  if (changed) {
    lj_status st = upload_boxes(s);
    if (st) return st;
  }
  const int mode = step_mode(s);
  const bool fused = use_fused(s);
  if (!fused) {
    lj_status st = flush_observables(s);
    if (st) return st;
  }
  if (fused && (!s->pred_ready || s->pred_dt != dt)) {
    LJ_CUDA(s, launch_predict(state_args(s), nblocks(s), s->BI, s->stream));
    s->launches += 1;
    s->pred_ready = true;
    s->pred_dt = dt;
  }
  for (int k = 0; k < nsteps; ++k) {
    GraphEntry* ge = nullptr;
    lj_status st = get_graph(s, mode, &ge);
    if (st) return st;
    if (ge->profiled) {
      for (int e = 0; e < 4; ++e) {
        cudaEvent_t ev = next_event(s);
        if (!ev) return fail(s, LJ_ERR_CUDA, "cudaEventCreate failed");
        if (ge->ev_nodes[e]) LJ_CUDA(s, cudaGraphExecEventRecordNodeSetEvent(ge->exec, ge->ev_nodes[e], ev));
      }
    }
    LJ_CUDA(s, cudaGraphLaunch(ge->exec, s->stream));
    s->launches += ge->kernels;
    if (fused) s->qpar ^= 1;  // the step wrote the next predictor into the other buffer
    if (fused) s->obs_maybe_pending = true;
    after_step_host(s);
  }
  return LJ_OK;
}

lj_status lj_sync(lj_system* s) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  return check_status(s);
}

lj_status lj_get_observables(lj_system* s, lj_observables* out) {
  if (!s || !out) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = fetch_scalars(s);
  if (st) return st;
  fill_obs(s->h_sc.p[0], out);
  return LJ_OK;
}

lj_status lj_batch_observables(lj_system* s, lj_observables* out) {
  if (!s || !out) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = fetch_scalars(s);
  if (st) return st;
  for (int k = 0; k < s->nsys; ++k) fill_obs(s->h_sc.p[k], out + k);
  return LJ_OK;
}

lj_status lj_set_recording(lj_system* s, int32_t cap) {
  if (!s || cap < 0) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  // The new ring is allocated before the old one is let go: if that fails,
  // recording goes on as before.
  DevBuf<DevRecord> ring;
  LJ_CUDA(s, ring.alloc((size_t)cap * s->nsys));
  std::vector<DevScalars> sc;
  lj_status st = read_scalars(s, sc);
  if (st) return st;
  for (auto& d : sc) {
    d.rec_cap = cap;
    d.rec_count = 0;
  }
  clear_graphs(s);  // records pointer and stride are captured
  s->records.swap(ring);
  s->rec_cap = cap;
  return write_scalars(s, sc);
}

// Copies box `box`'s ring of per-step records (rec_cap entries at
// records + box * rec_cap, written by the step epilogues), oldest first.
static lj_status read_records(lj_system* s, int box, lj_observables* out, int32_t max, int32_t* count) {
  if (!s || !count || max < 0 || box < 0 || box >= s->nsys) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  *count = 0;
  if (s->rec_cap == 0) return LJ_OK;
  std::vector<DevScalars> sc;
  if ((st = read_scalars(s, sc))) return st;
  std::vector<DevRecord> rec(s->rec_cap);
  LJ_CUDA(s, cudaMemcpy(rec.data(), s->records.p + (size_t)box * s->rec_cap, sizeof(DevRecord) * s->rec_cap,
                        cudaMemcpyDeviceToHost));
  const long long total = sc[box].rec_count;
  const long long have = std::min<long long>(total, s->rec_cap);
  const long long first = total - have;
  int n = 0;
  for (long long k = first; k < total && n < max; ++k, ++n) {
    const DevRecord& r = rec[k % s->rec_cap];
    lj_observables& o = out[n];
    o.t = r.t;
    o.K = r.K;
    o.V = r.V;
    o.T = r.T;
    o.P = r.P;
    o.U = r.U;
    o.W = r.W;
    o.Pshear = r.Pshear;
    o.Tkin_tvn = r.Tkin;
    o.av_U_tot = r.av_U;
    o.av_T_tot = r.av_T;
    o.av_p_tot = r.av_p;
    o.av_iters = r.av_iters;
    o.step = r.step;
  }
  *count = n;
  return LJ_OK;
}

lj_status lj_get_records(lj_system* s, lj_observables* out, int32_t max, int32_t* count) {
  return read_records(s, 0, out, max, count);
}

lj_status lj_batch_records(lj_system* s, int32_t box, lj_observables* out, int32_t max, int32_t* count) {
  return read_records(s, box, out, max, count);
}

lj_status lj_reset_averaging(lj_system* s) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  std::vector<DevScalars> sc;
  lj_status st = read_scalars(s, sc);
  if (st) return st;
  for (auto& d : sc) {
    d.av_U = d.av_T = d.av_p = 0.0;
    d.av_iters = 0;
  }
  return write_scalars(s, sc);
}

lj_status lj_set_canonical(lj_system* s, int32_t canonical) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  for (int k = 0; k < s->nsys; ++k) {
    s->cfg[k].canonical = canonical ? 1 : 0;
    s->boxes[k].canonical = canonical ? 1 : 0;
  }
  return upload_boxes(s);
}

lj_status lj_set_boundary(lj_system* s, int32_t bc) {
  if (!s) return LJ_ERR_INVALID;
  if (bc < 0 || bc > 2) return fail(s, LJ_ERR_INVALID, "boundary must be 0, 1 or 2");
  DeviceGuard device_guard(s->device);
  for (int k = 0; k < s->nsys; ++k) {
    s->cfg[k].boundary = bc;
    s->boxes[k].bc = bc;
  }
  lj_status st = upload_boxes(s);
  if (st) return st;
  // The shadow frame depends on the boundary; rebuild it from the positions.
  return enqueue_frame_all(s);
}

lj_status lj_set_temperature(lj_system* s, double T0) {
  if (!s || !(T0 >= 0)) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  for (int k = 0; k < s->nsys; ++k) {
    s->cfg[k].temperature = T0;
    s->boxes[k].T0 = T0;
  }
  return upload_boxes(s);
}

lj_status lj_set_time(lj_system* s, double t) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  std::vector<DevScalars> sc;
  lj_status st = read_scalars(s, sc);
  if (st) return st;
  for (auto& d : sc) d.t = t;
  return write_scalars(s, sc);
}

lj_status lj_renormalize_velocities(lj_system* s, int32_t recalc) {
  if (!s) return LJ_ERR_INVALID;
  if (s->nsys != 1) return fail(s, LJ_ERR_UNSUPPORTED, "renormalization applies to single-box handles");
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  std::vector<DevScalars> sc;
  if ((st = read_scalars(s, sc))) return st;
  const double T0 = s->boxes[0].T0, N = s->cfg[0].n;
  double Tkin = sc[0].T;
  StateArgs a = state_args(s);
  if (recalc) {
    LJ_CUDA(s, launch_scale_velocities(a, nblocks(s), s->BI, 1, 1.0, s->stream));
    s->launches += 1;
    std::vector<double> part((size_t)nblocks(s) * 8);
    LJ_CUDA(s, cudaMemcpyAsync(part.data(), s->blk_part.p, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                               s->stream));
    LJ_CUDA(s, cudaStreamSynchronize(s->stream));
    double K = 0;
    for (int b = 0; b < nblocks(s); ++b) K += part[(size_t)b * 8];
    Tkin = 2.0 * K / 3.0 / N;  // KineticTemperature = sum v^2/(3N)
  }
  if (!(Tkin > 0)) return fail(s, LJ_ERR_INVALID, "kinetic temperature is zero; cannot rescale");
  LJ_CUDA(s, launch_scale_velocities(a, nblocks(s), s->BI, 0, std::sqrt(T0 / Tkin), s->stream));
  s->launches += 1;
  s->pred_ready = false;
  // MDSystem.cpp:386-388: K *= T0/Tkin; T = T0; U = K + V.
  sc[0].K *= T0 / Tkin;
  sc[0].T = T0;
  sc[0].U = sc[0].K + sc[0].V;
  return write_scalars(s, sc);
}

lj_status lj_renormalize_velocities_to_energy(lj_system* s, double ust) {
  if (!s) return LJ_ERR_INVALID;
  if (s->nsys != 1) return fail(s, LJ_ERR_UNSUPPORTED, "renormalization applies to single-box handles");
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  std::vector<DevScalars> sc;
  if ((st = read_scalars(s, sc))) return st;
  const double Kold = sc[0].K;
  const double Kdes = ust * s->cfg[0].n - sc[0].V;
  if (!(Kold > 0) || !(Kdes >= 0))
    return fail(s, LJ_ERR_INVALID, "target energy %.6g per particle is below the potential energy", ust);
  StateArgs a = state_args(s);
  LJ_CUDA(s, launch_scale_velocities(a, nblocks(s), s->BI, 0, std::sqrt(Kdes / Kold), s->stream));
  s->launches += 1;
  s->pred_ready = false;
  sc[0].K = Kdes;
  sc[0].U = sc[0].K + sc[0].V;
  return write_scalars(s, sc);
}

float lj_reference_rdf_dr2(int32_t n) {
  // MDSystem.cpp:93-95, with the float member's roundings.
  if (n < 1) return 0.0f;
  const double a = 0.2 * std::sqrt(100. / n);
  float dr2 = (float)(a > 0.05 ? a : 0.05);
  if (250 * dr2 < 25.0) dr2 = (float)(25.0 / 250);
  return dr2;
}

lj_status lj_rdf_counts(lj_system* s, int32_t mode, int32_t nbins, double width, uint64_t* counts) {
  if (!s || !counts) return LJ_ERR_INVALID;
  if (mode < 0 || mode > 2) return fail(s, LJ_ERR_INVALID, "unknown RDF mode %d", mode);
  if (nbins < 1 || nbins > kMaxHistBins) return fail(s, LJ_ERR_INVALID, "nbins must be in [1, %d]", kMaxHistBins);
  if (!(width > 0)) return fail(s, LJ_ERR_INVALID, "bin width must be > 0");
  if (s->nsys != 1) return fail(s, LJ_ERR_UNSUPPORTED, "RDF counts apply to single-box handles");
  DeviceGuard device_guard(s->device);
  lj_status st = enqueue_frame_all(s);
  if (st) return st;
  LJ_CUDA(s, cudaMemsetAsync(s->hist.p, 0, sizeof(unsigned long long) * nbins, s->stream));
  HistArgs h{};
  h.mode = mode;
  h.nb = nbins;
  const double sig = s->cfg[0].sigma;
  // bins in reduced units: width / sigma^2 (r^2 bins) or width / sigma (r bins)
  if (mode == 2) {
    h.inv_w = (float)(sig / width);
    const double rmax = nbins * width / sig;
    h.rmax2 = (float)(rmax * rmax);
  } else {
    h.inv_w = (float)(sig * sig / width);
    h.rmax2 = 0.0f;
  }
  h.counts = s->hist.p;
  // The histogram path always runs on the fixed-point shadow.
  // FP64 handles schedule 128-particle i-blocks and 256-record j-tiles,
  // the geometry of MIXED shape 0, so that shape reads their tables.
  const int shape = (s->prec == LJ_PREC_MIXED) ? s->shape : 0;
  PairArgs p;
  int grid = 0;
  st = hist_pass_args(s, shape, pair_args(s).q, h, &p, &grid);
  if (st) return st;
  LJ_CUDA(s, launch_pairs(LJ_PREC_MIXED, shape, false, true, p, grid, s->stream));
  s->launches += 1;
  LJ_CUDA(s, cudaMemcpyAsync(counts, s->hist.p, sizeof(unsigned long long) * nbins, cudaMemcpyDeviceToHost,
                             s->stream));
  return check_status(s);
}

lj_status lj_velocity_counts(lj_system* s, double step, int32_t nbins, uint64_t* counts) {
  if (!s || !counts) return LJ_ERR_INVALID;
  if (nbins < 1 || nbins > kMaxHistBins) return fail(s, LJ_ERR_INVALID, "nbins must be in [1, %d]", kMaxHistBins);
  if (!(step > 0)) return fail(s, LJ_ERR_INVALID, "step must be > 0");
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaMemsetAsync(s->hist.p, 0, sizeof(unsigned long long) * nbins, s->stream));
  StateArgs a = state_args(s);
  LJ_CUDA(s, launch_velocity_hist(a, nblocks(s), s->BI, step, nbins, s->hist.p, s->stream));
  s->launches += 1;
  LJ_CUDA(s, cudaMemcpyAsync(counts, s->hist.p, sizeof(unsigned long long) * nbins, cudaMemcpyDeviceToHost,
                             s->stream));
  return check_status(s);
}

lj_status lj_counters_configure(lj_system* s, const lj_counter* counters, int32_t ncounters, int32_t ring_steps) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  if (s->counter_cap > 0) clear_graphs(s);  // the step graphs hold the counters' launches
  s->counters.clear();
  s->counter_cap = 0;
  s->counter_bins = 0;
  s->counter_head = s->counter_tail = 0;
  s->counter_phase = 0;
  if (ncounters == 0) return LJ_OK;
  if (!counters || ncounters < 0) return fail(s, LJ_ERR_INVALID, "counters must be non-NULL");
  if (ring_steps < 1) return fail(s, LJ_ERR_INVALID, "ring_steps must be >= 1");
  if (s->nsys != 1) return fail(s, LJ_ERR_UNSUPPORTED, "subsystem counters apply to single-box handles");
  const double L = s->boxes[0].L;
  int bins = 0;
  for (int q = 0; q < ncounters; ++q) {
    const lj_counter& c = counters[q];
    if (c.type < 0 || c.type > 6) return fail(s, LJ_ERR_INVALID, "counter %d: unknown type %d", q, c.type);
    if (c.nalpha < 1 || c.nalpha > kMaxCounterAlphas)
      return fail(s, LJ_ERR_INVALID, "counter %d: nalpha must be in [1, %d]", q, kMaxCounterAlphas);
    if (!(c.alpha_step > 0)) return fail(s, LJ_ERR_INVALID, "counter %d: alpha_step must be > 0", q);
    if (c.type >= 4 && !(c.vmax > 0)) return fail(s, LJ_ERR_INVALID, "counter %d: vmax must be > 0", q);
    CounterDev d{};
    d.type = c.type;
    d.nalpha = c.nalpha;
    d.bin0 = bins;
    d.alpha_step = c.alpha_step;
    d.vmax = c.vmax;
    d.inv_bc = 1.0 / ((c.type >= 4 ? c.vmax : L) * c.alpha_step);
    // cube sides from the accumulated alphas, as the reference's loop forms them
    double alpha = c.alpha_step;
    for (int k = 0; k < c.nalpha; ++k, alpha += c.alpha_step) d.tl[k] = L * std::pow(alpha, 1. / 3.);
    s->counters.push_back(d);
    bins += c.nalpha;
  }
  s->counter_bins = bins;
  // counting starts only once both buffers exist (counter_cap > 0); on a
  // failure the handle is left with no counters
  int words[kCtrWords] = {0};
  words[kCtrNext] = 0;
  words[kCtrPhase] = 0;
  words[kCtrEvery] = s->counter_every;
  words[kCtrCap] = ring_steps;
  words[kCtrTicket] = 0;
  cudaError_t e = s->dcounters.alloc(s->counters.size());
  if (e == cudaSuccess) e = s->counter_ring.alloc((size_t)bins * ring_steps);
  if (e == cudaSuccess) e = s->counter_state.alloc(kCtrWords);
  if (e == cudaSuccess) e = s->counter_part.alloc((size_t)counters_blocks(s->ntotal) * bins);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->dcounters.p, s->counters.data(), sizeof(CounterDev) * s->counters.size(),
                        cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->counter_state.p, words, sizeof(words), cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    s->counters.clear();
    s->counter_bins = 0;
    s->dcounters.free();
    s->counter_ring.free();
    s->counter_state.free();
    s->counter_part.free();
  }
  LJ_CUDA(s, e);
  s->counter_cap = ring_steps;
  clear_graphs(s);  // the step graphs now count
  return LJ_OK;
}

lj_status lj_counters_set_interval(lj_system* s, int32_t every) {
  if (!s) return LJ_ERR_INVALID;
  if (every < 1) return fail(s, LJ_ERR_INVALID, "the counting interval must be >= 1 step");
  DeviceGuard device_guard(s->device);
  s->counter_every = every;
  s->counter_phase = 0;
  if (s->counter_state.p) {
    // the device's copy, behind the queued steps (phase and interval words)
    const int words[2] = {0, every};
    static_assert(kCtrEvery == kCtrPhase + 1, "phase and interval words are adjacent");
    LJ_CUDA(s, cudaMemcpyAsync(s->counter_state.p + kCtrPhase, words, sizeof(words), cudaMemcpyHostToDevice,
                               s->stream));
    LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  }
  return LJ_OK;
}

lj_status lj_counters_read(lj_system* s, int32_t* counts, int32_t max_steps, int32_t* nsteps) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  const long long avail = s->counter_head - s->counter_tail;
  if (nsteps) *nsteps = (int32_t)std::min<long long>(avail, INT32_MAX);
  if (avail > s->counter_cap) {
    s->counter_tail = s->counter_head;
    return fail(s, LJ_ERR_INVALID, "%lld steps since the last read overflowed the counter ring of %d steps", avail,
                s->counter_cap);
  }
  if (!counts) return LJ_OK;
  const int n = (int)std::min<long long>(avail, max_steps);
  const int B = s->counter_bins;
  // the rows are contiguous in the ring up to its end, then from its start
  for (int k = 0; k < n;) {
    const long long row = (s->counter_tail + k) % s->counter_cap;
    const int run = (int)std::min<long long>(n - k, s->counter_cap - row);
    LJ_CUDA(s, cudaMemcpyAsync(counts + (size_t)k * B, s->counter_ring.p + (size_t)row * B,
                               sizeof(int) * B * (size_t)run, cudaMemcpyDeviceToHost, s->stream));
    k += run;
  }
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  // cumulative over each counter's alphas: N(alpha_k) = sum of bins <= k
  for (int k = 0; k < n; ++k)
    for (const CounterDev& d : s->counters) {
      int32_t* r = counts + (size_t)k * B + d.bin0;
      for (int a = 1; a < d.nalpha; ++a) r[a] += r[a - 1];
    }
  s->counter_tail += n;
  if (nsteps) *nsteps = n;
  return LJ_OK;
}

lj_status lj_rdf_accumulate(lj_system* s, int32_t enable, int32_t mode, int32_t nbins, double width) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  if (s->rdf_acc) clear_graphs(s);  // the step graphs hold the accumulation's launches
  s->rdf_acc = false;
  s->rdf_samples = 0;
  if (!enable) return LJ_OK;
  if (mode < 0 || mode > 2) return fail(s, LJ_ERR_INVALID, "unknown RDF mode %d", mode);
  if (nbins < 1 || nbins > kMaxHistBins) return fail(s, LJ_ERR_INVALID, "nbins must be in [1, %d]", kMaxHistBins);
  if (!(width > 0)) return fail(s, LJ_ERR_INVALID, "bin width must be > 0");
  if (s->nsys != 1) return fail(s, LJ_ERR_UNSUPPORTED, "RDF accumulation applies to single-box handles");
  LJ_CUDA(s, s->rdf_sum.alloc(nbins));
  LJ_CUDA(s, s->qhist.alloc(s->npad));
  LJ_CUDA(s, cudaMemsetAsync(s->rdf_sum.p, 0, sizeof(unsigned long long) * nbins, s->stream));
  HistArgs h{};
  h.mode = mode;
  h.nb = nbins;
  const double sig = s->cfg[0].sigma;
  if (mode == 2) {
    h.inv_w = (float)(sig / width);
    const double rmax = nbins * width / sig;
    h.rmax2 = (float)(rmax * rmax);
  } else {
    h.inv_w = (float)(sig * sig / width);
    h.rmax2 = 0.0f;
  }
  h.counts = s->rdf_sum.p;
  s->rdf_args = h;
  s->rdf_acc = true;
  clear_graphs(s);  // the step graphs now accumulate
  return LJ_OK;
}

lj_status lj_rdf_accumulated(lj_system* s, uint64_t* counts, int64_t* nsamples, int32_t reset) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  if (!s->rdf_acc) return fail(s, LJ_ERR_INVALID, "RDF accumulation is not enabled");
  if (counts)
    LJ_CUDA(s, cudaMemcpy(counts, s->rdf_sum.p, sizeof(unsigned long long) * s->rdf_args.nb, cudaMemcpyDeviceToHost));
  if (nsamples) *nsamples = s->rdf_samples;
  if (reset) {
    LJ_CUDA(s, cudaMemsetAsync(s->rdf_sum.p, 0, sizeof(unsigned long long) * s->rdf_args.nb, s->stream));
    s->rdf_samples = 0;
  }
  return LJ_OK;
}

lj_status lj_render(lj_system* s, int32_t box, int32_t axis, int32_t width, int32_t height, double radius,
                    uint8_t* rgba) {
  if (!s || !rgba) return LJ_ERR_INVALID;
  if (box < 0 || box >= s->nsys) return fail(s, LJ_ERR_INVALID, "box %d out of range", box);
  if (axis < 0 || axis > 2) return fail(s, LJ_ERR_INVALID, "axis must be 0, 1 or 2");
  if (width < 1 || height < 1 || (long long)width * height > (1ll << 26))
    return fail(s, LJ_ERR_INVALID, "image size must be 1 .. 2^26 pixels");
  if (!(radius > 0)) return fail(s, LJ_ERR_INVALID, "radius must be > 0");
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  const size_t npix = (size_t)width * height;
  DevBuf<unsigned long long> key;
  DevBuf<uint8_t> img;
  LJ_CUDA(s, key.alloc(npix));
  LJ_CUDA(s, img.alloc(4 * npix));
  int p0 = 0;
  for (int k = 0; k < box; ++k) p0 += s->cfg[k].n;
  LJ_CUDA(s, launch_render(s->x.p, s->npad, p0, s->cfg[box].n, axis, width, height, s->boxes[box].L,
                           radius * s->cfg[box].sigma, key.p, img.p, s->stream));
  s->launches += 2;
  LJ_CUDA(s, cudaMemcpyAsync(rgba, img.p, 4 * npix, cudaMemcpyDeviceToHost, s->stream));
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  return LJ_OK;
}

lj_status lj_tune_info(lj_system* s, int32_t* nshapes, int32_t* active, int32_t k, int32_t* threads, int32_t* ipt,
                       int32_t* tile) {
  if (!s) return LJ_ERR_INVALID;
  if (nshapes) *nshapes = kNumShapes;
  if (active) *active = s->shape;
  if (k >= 0 && k < kNumShapes) {
    if (threads) *threads = kShapes[k].threads;
    if (ipt) *ipt = 1;
    if (tile) *tile = kShapes[k].tile;
  }
  return LJ_OK;
}

lj_status lj_set_kernel_shape(lj_system* s, int32_t shape) {
  if (!s) return LJ_ERR_INVALID;
  if (shape < -1 || shape >= kNumShapes) return fail(s, LJ_ERR_INVALID, "shape %d out of range", shape);
  if (s->prec == LJ_PREC_FP64) return LJ_OK;  // one FP64 shape
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  const int old_forced = s->forced_shape;
  s->forced_shape = shape;
  s->shape = shape < 0 ? 0 : shape;
  lj_status st = setup_schedule(s);
  if (st) {
    s->forced_shape = old_forced;
    return st;
  }
  // The i-block length changed: rebuild shadows and the per-block sums.
  return recompute_forces_keep_scalars(s);
}

lj_status lj_set_split_cap(lj_system* s, int32_t cap) {
  if (!s) return LJ_ERR_INVALID;
  if (cap < 0 || cap > 1024) return fail(s, LJ_ERR_INVALID, "split cap %d out of range [0, 1024]", cap);
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  const int old_forced = s->forced_split;
  s->forced_split = cap;
  s->split_cap = cap > 0 ? cap : kMaxSegmentsPerBlock;
  lj_status st = setup_schedule(s);
  if (st) {
    s->forced_split = old_forced;
    return st;
  }
  // The partial segments were re-cut: rebuild the per-block sums.
  return recompute_forces_keep_scalars(s);
}

lj_status lj_split_info(lj_system* s, int32_t* cap, int32_t* ctas, int32_t* max_segments) {
  if (!s) return LJ_ERR_INVALID;
  if (cap) *cap = s->split_cap;
  if (ctas) *ctas = s->sched.G;
  if (max_segments) {
    int m = 0;
    for (const BlockInfo& b : s->sched.blocks) m = std::max(m, b.seg_count);
    *max_segments = m;
  }
  return LJ_OK;
}

lj_status lj_autotune(lj_system* s) {
  if (!s) return LJ_ERR_INVALID;
  if (s->prec == LJ_PREC_FP64) return LJ_OK;  // one FP64 shape
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);
  if (st) return st;
  // Every shape is timed on whole steps of this very system (the fused step
  // ranks shapes differently from the bare pair kernel); the state is
  // snapshotted first and restored after each trial.
  const size_t n3 = 3 * (size_t)s->npad;
  std::vector<DevBuf<double>> snap(6);
  DevBuf<int4> snap_q, snap_q2;
  DevBuf<DevScalars> snap_sc;
  DevBuf<DevRecord> snap_rec;
  double* cur[6] = {s->x.p, s->v.p, s->f.p, s->tf.p, s->e.p, s->w.p};
  const size_t cnt[6] = {n3, n3, n3, n3, (size_t)s->npad, (size_t)s->npad};
  for (int k = 0; k < 6; ++k) {
    LJ_CUDA(s, snap[k].alloc(cnt[k]));
    LJ_CUDA(s, cudaMemcpyAsync(snap[k].p, cur[k], sizeof(double) * cnt[k], cudaMemcpyDeviceToDevice, s->stream));
  }
  LJ_CUDA(s, snap_q.alloc(s->npad));
  LJ_CUDA(s, snap_q2.alloc(s->npad));
  LJ_CUDA(s, snap_sc.alloc(s->nsys));
  LJ_CUDA(s, cudaMemcpyAsync(snap_q.p, s->q.p, sizeof(int4) * s->npad, cudaMemcpyDeviceToDevice, s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(snap_q2.p, s->q2.p, sizeof(int4) * s->npad, cudaMemcpyDeviceToDevice, s->stream));
  LJ_CUDA(s, cudaMemcpyAsync(snap_sc.p, s->sc.p, sizeof(DevScalars) * s->nsys, cudaMemcpyDeviceToDevice, s->stream));
  if (s->rec_cap > 0) {
    LJ_CUDA(s, snap_rec.alloc(s->records.n));
    LJ_CUDA(s, cudaMemcpyAsync(snap_rec.p, s->records.p, sizeof(DevRecord) * s->records.n, cudaMemcpyDeviceToDevice,
                               s->stream));
  }
  const int qpar = s->qpar;
  const bool was_profiling = s->profiling;
  s->profiling = false;
  auto restore = [&]() -> lj_status {
    for (int k = 0; k < 6; ++k)
      LJ_CUDA(s, cudaMemcpyAsync(cur[k], snap[k].p, sizeof(double) * cnt[k], cudaMemcpyDeviceToDevice, s->stream));
    LJ_CUDA(s, cudaMemcpyAsync(s->q.p, snap_q.p, sizeof(int4) * s->npad, cudaMemcpyDeviceToDevice, s->stream));
    LJ_CUDA(s, cudaMemcpyAsync(s->q2.p, snap_q2.p, sizeof(int4) * s->npad, cudaMemcpyDeviceToDevice, s->stream));
    LJ_CUDA(s, cudaMemcpyAsync(s->sc.p, snap_sc.p, sizeof(DevScalars) * s->nsys, cudaMemcpyDeviceToDevice, s->stream));
    if (s->rec_cap > 0)
      LJ_CUDA(s, cudaMemcpyAsync(s->records.p, snap_rec.p, sizeof(DevRecord) * s->records.n,
                                 cudaMemcpyDeviceToDevice, s->stream));
    // the fused steps' ticket counters follow the step parity restored here
    LJ_CUDA(s, cudaMemsetAsync(s->glob_cnt.p, 0, sizeof(int) * s->glob_cnt.n, s->stream));
    LJ_CUDA(s, cudaStreamSynchronize(s->stream));
    s->qpar = qpar;
    return LJ_OK;
  };
  // On a failure part-way (an allocation of a trial schedule, say), the
  // handle goes back to its own shape and split cap where it can, and to the
  // snapshotted state, before the error is returned.
  const int orig_shape = s->shape, orig_split = s->split_cap;
  auto give_up = [&](lj_status err) -> lj_status {
    const std::string msg = s->err;
    s->profiling = was_profiling;
    s->shape = orig_shape;
    s->split_cap = orig_split;
    if (s->sched_shape != orig_shape || s->sched_split != orig_split) setup_schedule(s);
    if (restore() == LJ_OK && enqueue_compute_forces(s) == LJ_OK &&
        cudaMemcpyAsync(s->sc.p, snap_sc.p, sizeof(DevScalars) * s->nsys, cudaMemcpyDeviceToDevice, s->stream) ==
            cudaSuccess)
      cudaStreamSynchronize(s->stream);
    s->err = msg;
    return err;
  };
  double dt = s->boxes[0].dt > 0 ? s->boxes[0].dt : 0.005;
  struct Events {  // destroyed on every return path
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Events() {
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
  } ev;
  LJ_CUDA(s, cudaEventCreate(&ev.e0));
  LJ_CUDA(s, cudaEventCreate(&ev.e1));
  cudaEvent_t e0 = ev.e0, e1 = ev.e1;
  // Two dimensions: the CTA shape (threads, j-tile, stages) and the threads
  // per particle (the split cap: CTAs an i-block may be cut into).  A cap
  // only matters while it keeps the grid below SMs x resident CTAs; larger
  // caps give the same schedule and are skipped.
  static const int kSplitCaps[] = {1, 2, 4, 8, 16, 32};
  int best = 0, best_split = s->split_cap;
  float best_ms = 1e30f;
  for (int k = 0; k < kNumShapes; ++k) {
    int prev_G = -1;
    for (int cap : kSplitCaps) {
      if (s->forced_split > 0 && cap != kSplitCaps[0]) break;
      s->shape = k;
      s->split_cap = s->forced_split > 0 ? s->forced_split : cap;
      if ((st = setup_schedule(s))) return give_up(st);
      if (s->sched.G == prev_G) break;
      prev_G = s->sched.G;
      if ((st = restore())) return give_up(st);
      if ((st = enqueue_compute_forces(s))) return give_up(st);
      // two warm-up steps (timed, to size the rounds), then the fastest of
      // three rounds of about 1 ms each (2..10 steps): neighbouring shapes
      // differ by ~1%, about the spread of a single short round
      LJ_CUDA(s, cudaEventRecord(e0, s->stream));
      if ((st = lj_step(s, dt, 2))) return give_up(st);
      LJ_CUDA(s, cudaEventRecord(e1, s->stream));
      LJ_CUDA(s, cudaEventSynchronize(e1));
      float warm_ms = 0;
      LJ_CUDA(s, cudaEventElapsedTime(&warm_ms, e0, e1));
      const int reps = std::max(2, std::min(10, (int)(1.0f / std::max(warm_ms * 0.5f, 1e-3f))));
      float ms = 1e30f;
      for (int round = 0; round < 3; ++round) {
        LJ_CUDA(s, cudaEventRecord(e0, s->stream));
        if ((st = lj_step(s, dt, reps))) return give_up(st);
        LJ_CUDA(s, cudaEventRecord(e1, s->stream));
        LJ_CUDA(s, cudaEventSynchronize(e1));
        float r_ms = 0;
        LJ_CUDA(s, cudaEventElapsedTime(&r_ms, e0, e1));
        ms = std::min(ms, r_ms / reps);
      }
      if ((st = check_status(s))) return give_up(st);
      if (ms < best_ms) {
        best_ms = ms;
        best = k;
        best_split = s->split_cap;
      }
    }
  }
  s->shape = best;
  s->split_cap = best_split;
  s->profiling = was_profiling;
  if ((st = setup_schedule(s))) return give_up(st);
  s->tuned = true;
  if ((st = restore())) return st;
  // The restored shadow and sums belong to the old i-block length: rebuild
  // forces, then put back the observables and running sums.
  if ((st = enqueue_compute_forces(s))) return st;
  LJ_CUDA(s, cudaMemcpyAsync(s->sc.p, snap_sc.p, sizeof(DevScalars) * s->nsys, cudaMemcpyDeviceToDevice, s->stream));
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  return LJ_OK;
}

lj_status lj_selftest_device_timeout(lj_system* s) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = check_status(s);  // earlier errors are reported as such
  if (st) return st;
  LJ_CUDA(s, launch_selftest_wait(s->status.p, s->stream));
  s->launches += 1;
  st = sync_status(s);
  if (st == LJ_ERR_DEVICE_TIMEOUT) return LJ_OK;
  if (st) return st;
  return fail(s, LJ_ERR_CUDA, "the bounded device wait returned without reporting its timeout");
}

lj_status lj_profile_enable(lj_system* s, int32_t on) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  s->profiling = on != 0;
  s->ev_used = 0;
  s->prof_steps = s->prof_pairs = 0;
  s->prof_step_ms = s->prof_pair_ms = 0;
  return LJ_OK;
}

lj_status lj_profile_read(lj_system* s, int64_t* pair_launches, double* pair_ms, int64_t* steps, double* step_ms) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  // Events are used four per step: step start, pair start, pair end, step end.
  for (size_t k = 0; k + 3 < s->ev_used; k += 4) {
    float a = 0, b = 0;
    LJ_CUDA(s, cudaEventElapsedTime(&a, s->ev_pool[k + 1], s->ev_pool[k + 2]));
    LJ_CUDA(s, cudaEventElapsedTime(&b, s->ev_pool[k], s->ev_pool[k + 3]));
    s->prof_pair_ms += a;
    s->prof_step_ms += b;
    s->prof_pairs += 1;
    s->prof_steps += 1;
  }
  s->ev_used = 0;
  if (pair_launches) *pair_launches = s->prof_pairs;
  if (pair_ms) *pair_ms = s->prof_pair_ms;
  if (steps) *steps = s->prof_steps;
  if (step_ms) *step_ms = s->prof_step_ms;
  return LJ_OK;
}

lj_status lj_get_stream(lj_system* s, void** stream) {
  if (!s || !stream) return LJ_ERR_INVALID;
  *stream = (void*)s->stream;
  return LJ_OK;
}

lj_status lj_set_stream(lj_system* s, void* stream) {
  if (!s) return LJ_ERR_INVALID;
  DeviceGuard device_guard(s->device);
  lj_status st = flush_observables(s);
  if (st) return st;
  LJ_CUDA(s, cudaStreamSynchronize(s->stream));
  s->stream = stream ? (cudaStream_t)stream : s->own_stream;
  clear_graphs(s);
  return LJ_OK;
}

int64_t lj_kernel_launch_count(const lj_system* s) { return s ? s->launches : 0; }

lj_status lj_batch_info(const lj_system* s, int32_t* nsys, int32_t* offsets) {
  if (!s) return LJ_ERR_INVALID;
  if (nsys) *nsys = s->nsys;
  if (offsets) {
    int32_t o = 0;
    for (int k = 0; k < s->nsys; ++k) {
      offsets[k] = o;
      o += s->cfg[k].n;
    }
    offsets[s->nsys] = o;
  }
  return LJ_OK;
}

const char* lj_version(void) { return "lj_gb300 1.0 (sm_103a)"; }

void* lj_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (bytes == 0 || pinned_alloc(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void lj_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

lj_status lj_sample_initial_state(const lj_config* cfg, double* pos, double* vel) {
  lj_status st = validate(cfg, nullptr);
  if (st) return st;
  if (!pos || !vel) return fail(nullptr, LJ_ERR_INVALID, "pos and vel must be non-NULL");
  const double L = std::cbrt((double)cfg->n / cfg->density);
  if (!sample_initial_state(cfg->n, L, cfg->temperature, cfg->lattice, cfg->jitter, cfg->sigma, cfg->seed, pos, vel))
    return fail(nullptr, LJ_ERR_INVALID, "initial-state sampling failed");
  return LJ_OK;
}

lj_status lj_schedule_plan(const int32_t* n, int32_t nsys, int32_t block, int32_t tile, int32_t ctas,
                           int32_t* out_ctas, int32_t* out_nseg, int32_t* cta_tile_begin, int32_t* cta_lo,
                           int32_t* block_info, int32_t max_blocks) {
  Schedule sch;
  if (!build_schedule(n, nsys, block, tile, ctas, kTileOverhead, &sch))
    return fail(nullptr, LJ_ERR_INVALID, "invalid schedule request");
  if (out_ctas) *out_ctas = sch.G;
  if (out_nseg) *out_nseg = sch.nseg;
  if (cta_tile_begin)
    for (int g = 0; g <= sch.G; ++g) cta_tile_begin[g] = sch.cta_tile_begin[g];
  if (cta_lo)
    for (int g = 0; g <= sch.G; ++g) cta_lo[g] = sch.cta_lo[g];
  if (block_info) {
    const int nb = std::min<int>(max_blocks, (int)sch.blocks.size());
    for (int b = 0; b < nb; ++b) {
      const BlockInfo& bi = sch.blocks[b];
      int32_t* o = block_info + 8 * b;
      o[0] = bi.sys;
      o[1] = bi.i0;
      o[2] = bi.n_i;
      o[3] = bi.p0;
      o[4] = bi.njt;
      o[5] = bi.seg_first;
      o[6] = bi.seg_count;
      o[7] = bi.g_first;
    }
  }
  return LJ_OK;
}

}  // extern "C"
