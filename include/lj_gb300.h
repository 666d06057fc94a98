/*
 * lj_gb300.h -- C ABI of the GB300-native Lennard-Jones MD hot path.
 *
 * One handle (lj_system) owns one simulation box on one GPU: FP64 positions
 * and velocities resident in HBM, the FP32/fixed-point shadow the pair
 * kernel reads, forces, observables and the step graphs.  Every entry point
 * returns an lj_status (0 = LJ_OK) and never exits the process; the message
 * of the last failure on a handle is available from lj_last_error().
 *
 * It replaces, in the reference (vlvovch/lennard-jones-cuda):
 *   - the host integrator and observables of class MDSystem
 *     (src/library/MDSystem.cpp:325-359 CalculateParameters,
 *      :406-436 ApplyBoundaryConditions, :438-583 Integrate),
 *   - the CUDA force path behind the extern "C" block of
 *     src/library/MDSystem.cu:155-299 (calculateNForces, allocate/copy),
 *     whose exact signatures are kept separately in lj_reference_abi.h,
 *   - the RDF and velocity histograms (MDSystem.cpp:93-97, 633-694).
 * Each declaration cites the reference interface it stands in for.
 *
 * Units are reduced LJ units (m = 1); epsilon and sigma default to 1, the
 * reference's hard-coded values (MDSystem.cu:44-53, MDSystem.cpp:289-298).
 * Arrays are interleaved (x, y, z) per particle, N x 3 doubles.
 */
#ifndef LJ_GB300_H
#define LJ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Opaque handle: one box (or a batch of boxes) resident on one GPU. */
typedef struct lj_system lj_system;

typedef enum {
  LJ_OK = 0,
  LJ_ERR_INVALID = 1,     /* bad argument (null pointer, N < 2, rho <= 0, ...) */
  LJ_ERR_CUDA = 2,        /* a CUDA runtime call failed (message holds the CUDA error) */
  LJ_ERR_NO_DEVICE = 3,   /* no usable sm_103 device, or the kernels were not built for it */
  LJ_ERR_DEVICE_TIMEOUT = 4, /* a bounded device-side wait gave up; results of that launch are void */
  LJ_ERR_NONFINITE = 5,   /* an observable became NaN/Inf (overlapping particles, blow-up) */
  LJ_ERR_UNSUPPORTED = 6, /* requested mode is not provided (e.g. the CPU hardware mode) */
  LJ_ERR_OUT_OF_MEMORY = 7,
  LJ_ERR_ESCAPED = 8      /* a particle of a hard-wall box went more than max(sigma, L/20) beyond
                             the walls and its starting bounding box (blow-up); no counterpart in
                             the reference, whose walls have no frame to leave */
} lj_status;

/* Boundary conditions, MDSystem.h:24: 0 periodic, 1 hard wall, 2 none. */
enum { LJ_BC_PERIODIC = 0, LJ_BC_WALL = 1, LJ_BC_NONE = 2 };

/* Arithmetic of the pair loop.  MIXED: fixed-point positions, FP32 pair math
 * with compensated per-particle sums, FP64 positions/velocities/reductions.
 * FP64: every pair computed in double (the all-FP64 comparator path). */
enum { LJ_PREC_MIXED = 0, LJ_PREC_FP64 = 1 };

/* Initial lattice: SC is the reference's cell-centred simple-cubic lattice
 * (MDSystem.cpp:150-167); FCC fills ceil((N/4)^(1/3))^3 cells in lattice order. */
enum { LJ_LATTICE_SC = 0, LJ_LATTICE_FCC = 1 };

/* RDF bin layouts.  R2_CLAMP: the reference GPU rule, bins in r^2 with the
 * overflow counted in the last bin (MDSystem.cu:39).  R2_DROP: the reference
 * CPU rule, overflow dropped (MDSystem.cpp:282-284).  R_LINEAR: bins linear
 * in r up to rmax, pairs beyond rmax dropped. */
enum { LJ_RDF_R2_CLAMP = 0, LJ_RDF_R2_DROP = 1, LJ_RDF_R_LINEAR = 2 };

/* MDSystem::MDSystemConfiguration (MDSystem.h:10-41) plus the parameters the
 * reference hard-codes or seeds from the clock. */
typedef struct {
  int32_t n;            /* N, number of particles (MDSystem.h:12) */
  double temperature;   /* T0 (MDSystem.h:15) */
  double density;       /* rho (MDSystem.h:18); box side L = (N/rho)^(1/3) */
  int32_t canonical;    /* 0 EVN velocity Verlet, 1 TVN (MDSystem.h:21) */
  int32_t boundary;     /* LJ_BC_* (MDSystem.h:25) */
  int32_t precision;    /* LJ_PREC_* */
  double epsilon;       /* LJ energy scale, 1 in the reference */
  double sigma;         /* LJ length scale, 1 in the reference */
  int32_t lattice;      /* LJ_LATTICE_* */
  double jitter;        /* uniform displacement half-width in sigma, 0 = none */
  uint64_t seed;        /* seed of the initial-condition generator */
  int32_t block_hint;   /* CUDABlockSize (MDSystem.h:29); 0 = use the autotuned shape */
  int32_t device;       /* CUDA device ordinal */
  int32_t autotune;     /* reserved (kept for the layout); shapes and the split cap are
                           timed when the caller runs lj_autotune */
} lj_config;

/* Thermodynamic state after the last force evaluation / step.  Same
 * definitions as MDSystem::CalculateParameters (MDSystem.cpp:325-359):
 * K = sum v^2/2, V = 4 eps sum_{i<j}[(s/r)^12-(s/r)^6], T = 2K/(3N),
 * P = (W/6 + N T)/(N/rho) with W = sum over ordered pairs of r.f, U = K + V. */
typedef struct {
  double t;          /* simulation time (MDSystem.h:80) */
  double K, V, T, P, U;
  double W;          /* virial sum over ordered pairs, r_ij . f_ij */
  double Pshear;     /* off-diagonal stress: always 0.  The reference computes it on its
                        CPU path only (MDSystem.cpp:259, 299, 309, 335); its GPU path
                        never updates it. */
  double Tkin_tvn;   /* TVN: kinetic temperature of the half-kicked velocities, else 0 */
  double av_U_tot, av_T_tot, av_p_tot; /* running sums, MDSystem.h:98 */
  int64_t av_iters;  /* MDSystem.h:99 */
  int64_t step;      /* steps taken since creation */
} lj_observables;

/* Fills *cfg with MDSystemConfiguration's defaults (MDSystem.h:32-40):
 * N=128, T0=1.5, rho=0.2, EVN, periodic; plus eps=sigma=1, SC lattice,
 * no jitter, seed 1, mixed precision, device 0, autotune field 1. */
lj_status lj_config_default(lj_config* cfg);

/* MDSystem::MDSystem / Reinitialize (MDSystem.cpp:55-114): allocates the box
 * on cfg->device, samples the seeded initial state (lattice, jitter, Maxwell
 * speeds, zero momentum, exact-T0 rescale), computes forces and observables
 * and resets the running averages. */
lj_status lj_create(const lj_config* cfg, lj_system** out);

/* MDSystem::~MDSystem (MDSystem.cpp:218-230), without the process-wide
 * device reset the reference performs through threadExit(). */
lj_status lj_destroy(lj_system* sys);

/* Message of the last failed call on sys (or of the last failed lj_create
 * when sys is NULL).  Valid until the next call on the same handle. */
const char* lj_last_error(const lj_system* sys);

/* Box side L and particle count. */
lj_status lj_get_info(const lj_system* sys, int32_t* n, double* box);

/* Reinitialize with a new configuration on the same handle
 * (MDSystem::Reinitialize, MDSystem.cpp:66-114). */
lj_status lj_reinitialize(lj_system* sys, const lj_config* cfg);

/* Inject positions/velocities (N x 3 doubles, either may be NULL) -- the
 * reference's writes into h_Pos/h_Vel followed by setArray (MDSystem.cpp:615-630).
 * Forces are NOT recomputed; call lj_compute_forces. */
lj_status lj_set_state(lj_system* sys, const double* pos, const double* vel);

/* lj_set_state without its synchronisation: the upload, its finiteness check
 * and the unpack are queued on the handle's stream and the call returns.
 * For a host loop that uploads, steps and reads back every step
 * (lj_set_state_async + lj_step + lj_get_state_observables: one host
 * synchronisation per step).  The caller keeps pos / vel unchanged until the
 * next synchronising call (lj_sync, lj_get_*) returns.  A non-finite value
 * drops the upload on the device (the state stays as it was, and later
 * queued uploads are dropped too) and is reported as LJ_ERR_INVALID by that
 * next synchronising call.  No counterpart in the reference. */
lj_status lj_set_state_async(lj_system* sys, const double* pos, const double* vel);

/* One host round trip for a caller that keeps the state on the host (the
 * reference's host loop: write h_Pos/h_Vel, Integrate(dt), read them back,
 * MDSystem.cpp:438-583, 586-630): lj_set_state_async(pos_in, vel_in), then
 * lj_step(dt, nsteps), then lj_get_state_observables(pos_out, vel_out,
 * force_out, obs) -- one host synchronisation.  Any array may be NULL;
 * outputs may be the input buffers.  Page-locked host buffers (lj_host_alloc)
 * are read and written by the kernels directly, others through staged
 * copies.  No counterpart in the reference. */
lj_status lj_step_io(lj_system* sys, const double* pos_in, const double* vel_in, double dt, int32_t nsteps,
                     double* pos_out, double* vel_out, double* force_out, lj_observables* obs);

/* Read back state (N x 3 doubles each, any may be NULL) -- getArray(0/1)
 * (MDSystem.cpp:586-613) and h_Force. */
lj_status lj_get_state(lj_system* sys, double* pos, double* vel, double* force);

/* Per-particle pair sums of the last force evaluation, N doubles each (any
 * may be NULL): e_i = sum_j 4eps[(s/r)^12-(s/r)^6] (the reference's Force.w
 * times 4 eps), w_i = sum_j r_ij.f_ij. */
lj_status lj_get_pair_sums(lj_system* sys, double* e, double* w);

/* MDSystem::CalculateForces + CalculateParameters (MDSystem.cpp:232-359):
 * forces, V, virial at the current positions, then K, T, P, U; the running
 * averages advance by one sample like CalculateParameters does. */
lj_status lj_compute_forces(lj_system* sys);

/* MDSystem::Integrate(dt) nsteps times (MDSystem.cpp:438-583): velocity
 * Verlet (EVN) or constant-kinetic-temperature Verlet (TVN), boundary
 * handling, observables and running averages every step.  Enqueued on the
 * handle's stream as CUDA graphs; returns once enqueued.  Errors of the
 * device work surface at the next lj_sync / lj_get_* call. */
lj_status lj_step(lj_system* sys, double dt, int32_t nsteps);

/* Waits for queued work and reports device-side failures (timeouts, NaN). */
lj_status lj_sync(lj_system* sys);

/* Observables after the last step / force evaluation (synchronises). */
lj_status lj_get_observables(lj_system* sys, lj_observables* out);

/* lj_get_state and lj_get_observables in one call with one synchronisation:
 * what a host loop that mirrors the state every step (the reference's
 * Integrate followed by getArray, MDSystem.cpp:438-583, 586-613) needs.  Any
 * pointer may be NULL. */
lj_status lj_get_state_observables(lj_system* sys, double* pos, double* vel, double* force,
                                   lj_observables* out);

/* Per-step observable records.  lj_set_recording(sys, cap) keeps the last
 * cap steps (0 disables); lj_get_records copies up to max records, oldest
 * first, and returns their count in *count. */
lj_status lj_set_recording(lj_system* sys, int32_t cap);
lj_status lj_get_records(lj_system* sys, lj_observables* out, int32_t max, int32_t* count);

/* MDSystem::resetAveraging (MDSystem.cpp:701-705). */
lj_status lj_reset_averaging(lj_system* sys);

/* Setters of MDSystem.h:160-163 (setCanonical, setBoundaryCondition) and the
 * time step counter's clock (MDSystem::t). */
lj_status lj_set_canonical(lj_system* sys, int32_t canonical);
lj_status lj_set_boundary(lj_system* sys, int32_t bc);
lj_status lj_set_temperature(lj_system* sys, double T0);
lj_status lj_set_time(lj_system* sys, double t);

/* MDSystem::RenormalizeVelocities (MDSystem.cpp:375-389): scale velocities by
 * sqrt(T0/Tkin); recalc = 1 measures Tkin from the velocities, 0 uses the
 * current observable T.  MDSystem::RenormalizeVelocitiesToEnergy
 * (MDSystem.cpp:391-404): scale so that K = u*N - V. */
lj_status lj_renormalize_velocities(lj_system* sys, int32_t recalc);
lj_status lj_renormalize_velocities_to_energy(lj_system* sys, double ust);

/* Pair histogram at the current positions (ordered pairs, as the reference's
 * NdNdr2 filled inside CalculateForces, MDSystem.cu:39-42 / MDSystem.cpp:281-285).
 * mode LJ_RDF_R2_*: bins of width `width` in r^2 (the reference's rdf_dr2);
 * LJ_RDF_R_LINEAR: bins of width `width` in r, r < nbins*width.
 * nbins <= 4096.  counts: nbins uint64. */
lj_status lj_rdf_counts(lj_system* sys, int32_t mode, int32_t nbins, double width,
                        uint64_t* counts);

/* The reference's RDF bin width for N (MDSystem.cpp:93-95), as the float it stores. */
float lj_reference_rdf_dr2(int32_t n);

/* Speed histogram of initvelo/updatevelo (MDSystem.cpp:651-694): counts of
 * floor(|v|/step) for bins < nbins.  counts: nbins uint64. */
lj_status lj_velocity_counts(lj_system* sys, double step, int32_t nbins, uint64_t* counts);

/* Selects the pair-kernel shape by index (see lj_tune_info) or -1 for the
 * autotuned choice; lj_autotune times every shape now and keeps the fastest.
 * Changing the shape (or the split cap below) recomputes the forces for the
 * next step; the observables, the clock and the running averages are kept. */
lj_status lj_autotune(lj_system* sys);
lj_status lj_set_kernel_shape(lj_system* sys, int32_t shape);
/* Shape table: count, and for shape k its threads per CTA, i-particles per
 * thread and j-tile length; *active = shape in use. */
lj_status lj_tune_info(lj_system* sys, int32_t* nshapes, int32_t* active, int32_t k,
                       int32_t* threads, int32_t* ipt, int32_t* tile);

/* Threads per particle.  The reference gives each particle one thread over
 * all j (MDSystem.cu:74-111, 113-138); here an i-block's j range is cut over
 * up to `cap` CTAs, i.e. up to `cap` threads per particle, each summing a
 * j sub-range into its own partial segment.  lj_autotune searches the cap
 * together with the shape (caps 1..32 that change the grid); lj_set_split_cap
 * fixes it (0: back to the default 8, searched again by lj_autotune).
 * lj_split_info reports the cap in use, the CTAs of the persistent grid and
 * the most segments any i-block has. */
lj_status lj_set_split_cap(lj_system* sys, int32_t cap);
lj_status lj_split_info(lj_system* sys, int32_t* cap, int32_t* ctas, int32_t* max_segments);

/* Device-time profiling.  When enabled, each pair-kernel launch inside
 * lj_step / lj_compute_forces is bracketed by CUDA events on the handle's
 * stream; lj_profile_read returns the launch count and summed milliseconds
 * of the pair kernel and of the whole step graph since the last reset. */
lj_status lj_profile_enable(lj_system* sys, int32_t on);
lj_status lj_profile_read(lj_system* sys, int64_t* pair_launches, double* pair_ms,
                          int64_t* steps, double* step_ms);

/* The CUDA stream the handle enqueues on (cudaStream_t as void*).  A caller
 * may substitute its own stream; NULL restores the handle's private stream. */
lj_status lj_get_stream(lj_system* sys, void** stream);
lj_status lj_set_stream(lj_system* sys, void* stream);

/* Self-test of the device-side wait limit (no counterpart in the reference,
 * whose kernels have no waits).  Runs the bounded mbarrier wait of the pair
 * kernels on a barrier that nothing completes: it must give up after its
 * 1.5 s limit, flag LJ_DEVFLAG_TIMEOUT and return, and the host must report
 * LJ_ERR_DEVICE_TIMEOUT.  Returns LJ_OK when that happened (the handle stays
 * usable), LJ_ERR_CUDA otherwise.  Takes about 1.5 s. */
lj_status lj_selftest_device_timeout(lj_system* sys);

/* Number of kernels the library launched on this handle since creation. */
int64_t lj_kernel_launch_count(const lj_system* sys);

/* ---- Batched replicas ----------------------------------------------------
 * One handle for nsys independent boxes (uneven N, rho, T0, boundaries),
 * advanced together: one persistent pair launch per step covers every box.
 * No counterpart in the reference, which runs one MDSystem per process with
 * process-global device state (MDSystem.cu:9-18).  All boxes share
 * precision, device and ensemble (canonical flag). */
lj_status lj_batch_create(const lj_config* cfgs, int32_t nsys, lj_system** out);
/* Observables of every box (nsys entries), synchronising. */
lj_status lj_batch_observables(lj_system* sys, lj_observables* out);
/* Per-step records of box `box` of a batch (lj_set_recording keeps cap steps
 * of every box), oldest first, like lj_get_records (which reads box 0). */
lj_status lj_batch_records(lj_system* sys, int32_t box, lj_observables* out, int32_t max, int32_t* count);
/* Number of boxes and the particle offset of each (offsets: nsys + 1 entries). */
lj_status lj_batch_info(const lj_system* sys, int32_t* nsys, int32_t* offsets);

/* ---- Host-side helpers (no device needed) -------------------------------- */

/* The seeded initial state lj_create samples for cfg (N x 3 each): lattice,
 * jitter, Maxwell speeds, zero momentum, exact T0 (MDSystem.cpp:147-216,
 * 375-389). */
lj_status lj_sample_initial_state(const lj_config* cfg, double* pos, double* vel);

/* The stream-K work split the pair kernel uses for boxes n[0..nsys) with
 * i-blocks of `block` particles, j-tiles of `tile` and at most `ctas` CTAs.
 * Writes the CTA count, the number of partial segments, the CTA ranges
 * (ctas+1 entries each: CTA g covers j from offset cta_lo[g] of flattened
 * tile cta_tile_begin[g] up to offset cta_lo[g+1] of tile
 * cta_tile_begin[g+1], offsets multiples of 32; cta_lo may be NULL) and, per
 * i-block, 8 ints: box, first particle, particles, box offset, j-tiles, first
 * segment, segments, first CTA. */
lj_status lj_schedule_plan(const int32_t* n, int32_t nsys, int32_t block, int32_t tile, int32_t ctas,
                           int32_t* out_ctas, int32_t* out_nseg, int32_t* cta_tile_begin, int32_t* cta_lo,
                           int32_t* block_info, int32_t max_blocks);

/* All-pairs LJ forces for callers that cannot allocate device memory
 * (plug-ins inside a framework whose caching allocator has reserved the GPU's
 * memory, loops that must not allocate after start-up because cudaMalloc and
 * cudaFree can synchronise the device, embedders whose allocator owns the
 * GPU).  No counterpart in the reference.  pos4: device float4[n] positions
 * (w ignored); force4: device float4[n] out, xyz = force (eps = sigma = 1),
 * w = sum_j (r^-12 - r^-6), as calculateNForces writes Force; sums (host,
 * may be NULL): {V, W} with V = 4 sum_{i<j}[r^-12 - r^-6] and W = sum over
 * ordered pairs of r.f.  Minimum image when periodic != 0 (box side `box`).
 * Enqueued on `stream` (NULL: default stream) and synchronised before
 * returning.  Allocates nothing: every intermediate lives in one fixed
 * __device__ array (about 4.4 MB per GPU, held from library load to process
 * exit), so n is limited to 16384 (larger n: LJ_ERR_INVALID).  All calls on
 * a device share that array and it keeps the last call's contents: calls
 * whose GPU work overlaps race.  The first call on a device looks up the
 * array's address and the device's SM count; make it before any stream
 * capture.  Every call reads its results back to the host and synchronises
 * `stream`, so a call on a stream that is being captured returns
 * LJ_ERR_UNSUPPORTED and enqueues nothing.  After a cudaDeviceReset the next
 * call sets the array up again. */
lj_status lj_forces_static(const float* pos4, float* force4, double* sums, int32_t n, float box,
                           int32_t periodic, void* stream);

/* ---- Per-step subsystem counts and summed RDF (task drivers) --------------
 * The fluctuation task of the reference (src/tasks/run-fluctuations/
 * run-fluctuations.cpp:87-174 with run-fluctuations-aux.h:124-273) counts,
 * after every step, the particles of nested subsystems and averages the RDF;
 * it copies all positions to the host for that every step.  Here the counts
 * are made on the GPU after every lj_step step into a ring that the host
 * reads every few hundred steps.  Single-box handles only. */
typedef struct {
  int32_t type;       /* 0/1/2: slab x/y/z < alpha L (GetNSubsystemBatch types 0-2);
                         3: cube of volume alpha L^3 around the box centre (type 3);
                         4/5/6: |v_x|/|v_y|/|v_z| < alpha vmax (GetNsubVzBatch types 0-2) */
  int32_t nalpha;     /* alpha_k = (k+1) alpha_step, k < nalpha (<= 64) */
  double alpha_step;
  double vmax;        /* types 4-6 (the reference uses 3 sqrt(T0)) */
} lj_counter;
/* Enables the counters (ncounters = 0 disables them); ring_steps rows are
 * kept between reads. */
lj_status lj_counters_configure(lj_system* sys, const lj_counter* counters, int32_t ncounters, int32_t ring_steps);
/* Counts after every `every`-th step only (default 1; kept across
 * lj_counters_configure calls), counted from this call or the last
 * configure: the semi-grand-canonical task of the reference
 * (src/tasks/semiGCEfluctuations/semiGCEfluctuations.cpp:70-80) samples every
 * 200 steps. */
lj_status lj_counters_set_interval(lj_system* sys, int32_t every);
/* Copies the rows of the counted steps since the last read, oldest first: per step
 * and counter, the cumulative counts N(alpha_0) .. N(alpha_{nalpha-1}).  With
 * counts = NULL only *nsteps is set.  More steps than ring_steps since the
 * last read is an error (LJ_ERR_INVALID) and drops them. */
lj_status lj_counters_read(lj_system* sys, int32_t* counts, int32_t max_steps, int32_t* nsteps);
/* Adds the RDF counts (modes and bins as lj_rdf_counts) of the state after
 * every step into a device histogram; enable = 0 stops and clears. */
lj_status lj_rdf_accumulate(lj_system* sys, int32_t enable, int32_t mode, int32_t nbins, double width);
/* The summed counts and the number of steps summed; reset != 0 clears both. */
lj_status lj_rdf_accumulated(lj_system* sys, uint64_t* counts, int64_t* nsamples, int32_t reset);

/* ---- Headless particle image ---------------------------------------------
 * Stand-in for the reference's OpenGL viewer (src/gui/MDSystemGL.cpp:32-160,
 * orange spheres of radius 0.5 sigma): a GPU splat of box `box` viewed along
 * `axis` (0/1/2, viewer on its positive side) into width x height RGBA8
 * pixels (host buffer, 4 bytes per pixel, row 0 at the top), spheres of
 * `radius` sigma shaded by their view-facing normal, background black.  No
 * graphics API is involved. */
lj_status lj_render(lj_system* sys, int32_t box, int32_t axis, int32_t width, int32_t height, double radius,
                    uint8_t* rgba);

/* ---- Differentiable MD (adjoint) ----------------------------------------
 * No counterpart in the reference (its dynamics are not differentiable).
 * Gradients of a time-averaged trajectory loss
 *   loss = (1/S) sum_{m=1..S} [ wK K_m/N + wV V_m/N + wP P_m ]
 * over S EVN velocity-Verlet steps (MDSystem.cpp:443-463) of a periodic box,
 * with respect to eps, sigma and the initial positions and velocities, by a
 * discrete adjoint: FP64 forward pass keeping (x, v, F) every
 * `checkpoint_every` steps, then a reverse sweep that replays each segment
 * from its checkpoint and applies the force Jacobian-vector product
 * (Hessian . vector) on the GPU.  Everything runs in FP64; the gradients are
 * those of this forward pass (the same equations as lj_step with
 * LJ_PREC_FP64, summed in a different order). */
typedef struct lj_adjoint lj_adjoint;

/* cfg: n, density, temperature, epsilon, sigma, lattice, jitter, seed and
 * device as for lj_create (the initial state is sampled the same way);
 * boundary must be LJ_BC_PERIODIC and canonical 0 (LJ_ERR_UNSUPPORTED
 * otherwise: wall reflections and the TVN rescale are not differentiated).
 * Default loss weights: wK = 0, wV = 1, wP = 1. */
lj_status lj_adjoint_create(const lj_config* cfg, int32_t checkpoint_every, lj_adjoint** out);
lj_status lj_adjoint_destroy(lj_adjoint* adj);
const char* lj_adjoint_last_error(const lj_adjoint* adj);
/* Initial state (N x 3 each, interleaved). */
lj_status lj_adjoint_set_state(lj_adjoint* adj, const double* pos, const double* vel);
lj_status lj_adjoint_set_loss(lj_adjoint* adj, double w_kinetic, double w_potential, double w_pressure);
/* Runs nsteps steps of size dt from the initial state; writes the loss. */
lj_status lj_adjoint_forward(lj_adjoint* adj, double dt, int32_t nsteps, double* loss);
/* K, V, W after each step of the last forward pass (any may be NULL). */
lj_status lj_adjoint_observables(lj_adjoint* adj, double* K, double* V, double* W, int32_t max, int32_t* count);
/* dloss/deps, dloss/dsigma, dloss/dpos (N x 3), dloss/dvel (N x 3) of the last
 * forward pass (any output may be NULL). */
lj_status lj_adjoint_backward(lj_adjoint* adj, double* d_epsilon, double* d_sigma, double* d_pos, double* d_vel);

/* Page-locked host memory for lj_set_state / lj_get_state buffers: copies
 * from and to it run as direct DMA.  NULL on failure; free with lj_host_free. */
void* lj_host_alloc(size_t bytes);
void lj_host_free(void* ptr);

/* Out-of-memory testing hook (host side; no counterpart in the reference,
 * whose checkCudaErrors(cudaMalloc(...)) exits the process on a failed
 * allocation, MDSystem.cu:167-173).  after >= 0: the next `after` device or
 * page-locked host allocations of this library succeed and every later one
 * fails with LJ_ERR_OUT_OF_MEMORY (the reference ABI: status
 * LJ_ERR_OUT_OF_MEMORY) without calling CUDA, until lj_debug_fail_allocations(-1)
 * turns the hook off.  Process-wide.  A call that fails this way leaves its
 * handle as it was: creation frees what it had allocated, a new schedule,
 * histogram range table, record ring or counter table replaces the old one
 * only once complete, and an interrupted autotune puts the state back. */
lj_status lj_debug_fail_allocations(int64_t after);

/* Library version string and the device architecture it was built for. */
const char* lj_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LJ_GB300_H */
