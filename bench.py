"""Benchmark: pair-interactions/s of the Lennard-Jones MD step on GB300.

Workload (the dense-liquid mixed-precision configuration): N = 16384
particles, periodic box at rho* = 0.85, T* = 1.0, FCC lattice with seeded
+-0.02 sigma jitter, Maxwell velocities, dt = 0.005, TVN constant-kinetic-
temperature dynamics, no cutoff (all N(N-1) ordered pairs per step, the
count the reference kernel evaluates).  A step is one full Verlet+TVN step
(drift, all-pairs forces, reductions, thermostat, observables).

Prints one JSON line (rank 0):
  value       pair-interactions/s of the mixed FP32/FP64 path, inputs resident
              in HBM, device-timed per step with CUDA events, L2 flushed
              between timed steps;
  e2e         the same metric through the public C ABI with host buffers:
              every step uploads positions+velocities from pinned host memory,
              steps, and reads positions+velocities+observables back;
  fp64        the all-FP64 GPU path on the same box (the 3x comparator);
  accuracy    per-particle force error of the mixed path vs FP64;
  roofline    pair kernel vs the FP32 peak (38 flops per ordered pair);
  cpu_baseline the reference's CPU algorithm (float-storage restatement of
              MDSystem.cpp's CPU path) on the host cores, a bounded sample;
  configs     the other configurations, measured briefly on the same GPU:
              256 batched replicas (aggregate steps/s and pair-interactions/s),
              N = 262144 (pair-interactions/s, FP32 fraction, subset force
              error vs the FP64 oracle) and the adjoint at N = 2048 (forward
              and backward time of 200 steps).

--impl reference times that CPU implementation alone on the same workload.
Multi-GPU (torchrun): every rank runs an independent replica (the path has
no data exchange between boxes), value = total over ranks, scaling "weak".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "lennard-jones-cuda_gb300"), os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N = 16384
RHO = 0.85
T0 = 1.0
DT = 0.005
JITTER = 0.02
SEED = 2
FLOPS_PER_PAIR = 38  # algorithmic FP32 flops per ordered pair, FMA = 2, rcp = 1
WORKLOAD = "lj-dense-liquid-tvn N=16384 rho*=0.85 T*=1.0 FCC+0.02 dt=0.005"


def bench_config(world: int) -> dict:
    """The workload description both arms print (identical keys and values)."""
    return {"workload": WORKLOAD, "n": N, "rho": RHO, "T": T0, "dt": DT, "ensemble": "TVN",
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "GPU arm: flushed (256 MB write) before every timed step"}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock and throttle-reason samples taken while the timed
    region runs.  The sampler is started and its first line awaited before
    the region begins (nvidia-smi needs ~0.1-0.5 s to come up); only samples
    stamped inside the region (plus one interval after it) are summarised."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    INTERVAL_MS = 20

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []  # (monotonic time, line)
        self.t_begin = self.t_end = None
        self._first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", str(self.INTERVAL_MS)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self._first.wait(timeout=5.0)
        except (OSError, FileNotFoundError):
            self.proc = None
        self.t_begin = time.monotonic()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))
            self._first.set()

    def __exit__(self, *exc):
        self.t_end = time.monotonic()
        if self.proc:
            time.sleep(self.INTERVAL_MS * 1e-3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t_hi = (self.t_end or time.monotonic()) + self.INTERVAL_MS * 1e-3
        for t, ln in self.lines:
            if self.t_begin is not None and not (self.t_begin <= t <= t_hi):
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "interval_ms": self.INTERVAL_MS,
                "region_s": (self.t_end - self.t_begin) if self.t_end and self.t_begin else None}


# ---------------------------------------------------------------------------
# CPU arm: the reference's CPU algorithm (faithful float-storage restatement)
# ---------------------------------------------------------------------------
def cpu_state():
    """The workload's seeded initial state as float4 arrays, drawn by the
    oracle's restatement of the library's sampler (the same numbers; the CPU
    arm never loads the product library)."""
    import oracle
    pos, vel, L = oracle.sample_state(N, RHO, T0, lattice=1, jitter=JITTER, seed=SEED)
    p4 = np.zeros((N, 4), np.float32)
    p4[:, :3] = pos
    p4[:, 3] = np.float32(L / 150.0)
    v4 = np.zeros((N, 4), np.float32)
    v4[:, :3] = vel
    return p4, v4


def cpu_baseline(max_seconds=12.0, max_steps=None, threads=None):
    """Times MDSystem.cpp's CPU Integrate (restated in oracle/lj_oracle.c,
    parallel over i) on this host: full N=16384 TVN steps until max_seconds."""
    import oracle
    oracle.build()
    threads = threads or oracle.default_threads()
    p4, v4 = cpu_state()
    r = oracle.R32System(N, T0, RHO, True, 0, p4, v4)
    r.calculate_forces(threads)
    r.calculate_parameters()
    steps, t0 = 0, time.perf_counter()
    while True:
        r.integrate(DT, threads)
        steps += 1
        el = time.perf_counter() - t0
        if el >= max_seconds or (max_steps and steps >= max_steps):
            break
    rate = N * (N - 1) * steps / el
    return {"value": rate, "unit": "pair-interactions/s", "cores": threads, "kind": "port",
            "sample": "%d full TVN steps of the N=16384 workload (%.1f s), reference CPU algorithm "
                      "(float storage, MDSystem.cpp:237-583) restated in C, OpenMP over i" % (steps, el),
            "seconds": el, "steps": steps}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def make_system(ljgb, prec, device):
    return ljgb.System(n=N, density=RHO, temperature=T0, canonical=1, lattice=ljgb.LATTICE_FCC, jitter=JITTER,
                       seed=SEED, precision=prec, device=device)


def timed_steps(torch, s, steps, warmup, flush, dt=DT):
    """Per-step CUDA-event timing on the library's stream, L2 flushed before
    every timed step (flush writes a buffer larger than L2)."""
    ext = torch.cuda.ExternalStream(s.stream())
    for _ in range(warmup):
        with torch.cuda.stream(ext):
            flush.zero_()
        s.integrate(dt)
    s.sync()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    c0 = s.launch_count()
    for k in range(steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            starts[k].record(ext)
        s.integrate(dt)
        with torch.cuda.stream(ext):
            ends[k].record(ext)
    s.sync()
    launches = s.launch_count() - c0
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    return sum(ms), ms, launches


def e2e_steps(ljgb, s, steps, warmup):
    """Through the public API with host buffers: every step is one lj_step_io
    call -- upload of pos+vel from page-locked host memory (queued; the
    kernels read it over NVLink-C2C), one step, read-back of pos+vel (written
    by the pack kernel into host memory) and of the observables, one host
    synchronisation, which also reports the upload's finiteness check."""
    pos = ljgb.pinned((N, 3))
    vel = ljgb.pinned((N, 3))
    s.get_state_into(pos, vel, None)
    for _ in range(warmup):
        s.step_io(DT, 1, pos, vel, pos, vel)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.step_io(DT, 1, pos, vel, pos, vel)
    el = time.perf_counter() - t0
    # the box's device scalar block (208 B: observables, clock, averages), the
    # status word and the upload check's result
    obs_bytes = 208 + 4 + 4
    return el, {"h2d_bytes_per_step": 2 * N * 3 * 8, "d2h_bytes_per_step": 2 * N * 3 * 8 + obs_bytes}


def fp32_peak_nominal(device):
    """SMs x 128 FP32 lanes x 2 flops x maximum SM clock."""
    import torch
    props = torch.cuda.get_device_properties(device)
    mhz = None
    try:
        out = subprocess.run(["nvidia-smi", "-i", str(device), "--query-gpu=clocks.max.sm",
                              "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=20)
        mhz = float(out.stdout.strip().splitlines()[0])
    except Exception:
        mhz = 2070.0
    return props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12, props.multi_processor_count, mhz


def read_traffic():
    """Per-launch DRAM bytes of the pair kernel from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "pairs_mixed_fused_n16384_ncu.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1].split()[0])
    except OSError:
        pass
    return None


def accuracy(ljgb, oracle, device):
    """Mixed vs FP64 forces on the benchmark state: all particles vs the GPU
    FP64 path, and 512 seeded rows vs the CPU FP64 oracle."""
    a = make_system(ljgb, 0, device)
    b = make_system(ljgb, 1, device)
    pos, _, Fa = a.get_state()
    _, _, Fb = b.get_state()
    ea, _ = a.pair_sums()
    oa, ob = a.observables(), b.observables()
    d = np.linalg.norm(Fa - Fb, axis=1)
    mag = np.linalg.norm(Fb, axis=1)
    rms = float(np.sqrt(np.mean(mag ** 2)))
    rel = d / mag
    rows = (4096, 4608)
    r = oracle.f64_forces(pos, a.L, True, rows=rows)
    magc = np.linalg.norm(r["F"], axis=1)
    dc = np.linalg.norm(Fa[rows[0]:rows[1]] - r["F"], axis=1)
    # The plain per-particle error |dF_i|/|F_i| exceeds 1e-5 only where the
    # pair forces on a particle nearly cancel (|F_i| well below rms|F|): the
    # count, the fraction and the largest |F_i|/rms|F| among those particles.
    over = rel > 1e-5
    out = {
        "vs": "all-FP64 GPU path (all N) and FP64 CPU oracle (512 rows)",
        "force_rel_median": float(np.median(rel)), "force_rel_p99": float(np.percentile(rel, 99)),
        "force_rel_max": float(rel.max()), "force_rms_rel_max": float(d.max() / rms),
        "force_rel_over_1e-5": {"count": int(over.sum()), "fraction": float(over.mean()),
                                "max_abs_F_over_rms": float((mag[over] / rms).max()) if over.any() else None,
                                "median_abs_F_over_rms": float(np.median(mag[over] / rms)) if over.any() else None,
                                "median_abs_F_over_rms_all": float(np.median(mag / rms))},
        "gate_max": float((d / np.maximum(mag, rms)).max()),
        "oracle_gate_max": float((dc / np.maximum(magc, rms)).max()),
        "V_rel": abs(oa["V"] - ob["V"]) / abs(ob["V"]), "W_rel": abs(oa["W"] - ob["W"]) / abs(ob["W"]),
        "gate": "every particle |dF_i| <= 1e-5 max(|F_i|, rms|F|), median |dF_i|/|F_i| <= 1e-5",
    }
    out["gate_pass"] = bool(out["gate_max"] <= 1e-5 and out["oracle_gate_max"] <= 1e-5
                            and out["force_rel_median"] <= 1e-5)
    a.close()
    b.close()
    return out


def batch_configs(ljgb, seed=3, k=256):
    """The batched-replicas configuration: 256 boxes, N in [200, 4000),
    rho* in [0.01, 1.1], T* in [0.7, 2.0], half periodic and half hard-wall,
    FCC + 0.02 jitter, TVN."""
    return ljgb.replica_batch_configs(seed, k)


def extra_configs(torch, ljgb, oracle, dev, flush, peak):
    """Short measurements of the other configurations (rank 0)."""
    out = {}
    # 256 batched replicas, dt = 0.004, TVN, one persistent pair launch per step
    cfgs = batch_configs(ljgb)
    b = ljgb.System(batch=cfgs)
    b.autotune()
    steps = 20
    ms, _, launches = timed_steps(torch, b, steps, 3, flush, dt=0.004)
    pairs = float(sum(c.n * (c.n - 1) for c in cfgs))
    # per-replica U/N and P, averaged over every step the replicas ran (the
    # device's running sums, MDSystem.cpp:355-358)
    obs = b.batch_observables()
    per_replica = {
        "steps_averaged": int(obs[0]["av_iters"]),
        "n": [int(c.n) for c in cfgs],
        "U_per_N": [float("%.6g" % (o["av_U_tot"] / max(1, o["av_iters"]) / c.n)) for o, c in zip(obs, cfgs)],
        "P": [float("%.6g" % (o["av_p_tot"] / max(1, o["av_iters"]))) for o in obs]}
    out["batch_256"] = {
        "workload": "256 replicas, N U[200,4000) (sum %d), rho* U[0.01,1.1], T* U[0.7,2.0], half walls, TVN, "
                    "dt=0.004" % sum(c.n for c in cfgs),
        "ms_per_step": ms / steps, "steps_per_s": 1e3 * steps / ms, "replica_steps_per_s": 256e3 * steps / ms,
        "pair_interactions_per_s": pairs * steps / (ms * 1e-3), "gpu_launches_per_step": launches / steps,
        "l2": "flushed before every timed step", "per_replica": per_replica}
    b.close()
    # one large box: N = 262144, rho* = 1.1, T* = 1.0, FCC + 0.01, dt = 0.004, TVN
    n = 262144
    g = ljgb.System(n=n, density=1.1, temperature=1.0, canonical=1, lattice=ljgb.LATTICE_FCC, jitter=0.01,
                    seed=262144, device=dev, autotune=0)
    pos, _, F = g.get_state()
    g.autotune()  # as the main configuration does (a few seconds at this size)
    i0 = int(np.random.default_rng(4096).integers(0, n - 4096))
    r = oracle.f64_forces(pos, g.L, True, rows=(i0, i0 + 4096))
    d = np.linalg.norm(F[i0:i0 + 4096] - r["F"], axis=1)
    mag = np.linalg.norm(r["F"], axis=1)
    rms = float(np.sqrt(np.mean(mag ** 2)))
    steps = 5
    ms, _, _ = timed_steps(torch, g, steps, 2, flush, dt=0.004)
    g.profile(True)
    g.integrate(0.004, steps)
    prof = g.profile_read()
    g.profile(False)
    pair_ms = prof["pair_ms"] / max(1, prof["pair_launches"])
    tune = g.tune_info()
    g.close()
    out["large_262144"] = {
        "workload": "N=262144 rho*=1.1 T*=1.0 FCC+0.01 dt=0.004 TVN", "ms_per_step": ms / steps,
        "kernel_shape": tune["shapes"][tune["active"]],
        "pair_interactions_per_s": n * (n - 1) * steps / (ms * 1e-3), "pair_kernel_ms": pair_ms,
        "fp32_frac": FLOPS_PER_PAIR * n * (n - 1) / (pair_ms * 1e-3) / 1e12 / peak,
        "subset_vs_fp64_oracle": {"rows": [i0, i0 + 4096], "gate_max": float((d / np.maximum(mag, rms)).max()),
                                  "rel_median": float(np.median(d / mag))}}
    # adjoint: N = 2048, rho* = 0.85, 200 EVN steps, checkpoints every 20, FP64
    a = ljgb.Adjoint(n=2048, density=0.85, temperature=1.0, lattice=ljgb.LATTICE_FCC, jitter=0.02, seed=2048,
                     checkpoint_every=20)
    a.forward(0.005, 200)
    a.backward()
    t0 = time.perf_counter()
    a.forward(0.005, 200)
    t1 = time.perf_counter()
    a.backward()
    t2 = time.perf_counter()
    a.close()
    out["adjoint_2048"] = {"workload": "N=2048 rho*=0.85 T*=1.0 dt=0.005, 200 EVN steps, checkpoints every 20, "
                                       "loss <V/N + P>, FP64", "forward_ms": (t1 - t0) * 1e3,
                           "backward_ms": (t2 - t1) * 1e3, "timing": "host wall clock, synchronised"}
    return out


def max_over_ranks(ms: float, device: str) -> float:
    """The slowest rank's timed region (every rank calls this)."""
    import torch
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, pairs_per_step: int, steps: int, total_ms: float) -> float:
    """Whole-job pair-interactions/s: every rank runs its own box (replicas,
    weak scaling) and the job takes as long as the slowest rank."""
    return world * pairs_per_step * steps / (total_ms * 1e-3)


def ref_gpu_kernel(torch, ljgb, dev, flush, pair_ms, steps=20, block=256):
    """The reference's GPU force kernel, restated in comparator/ref_nbody.cu
    (FP32 nbody tiles, lround minimum image, a global RDF atomic per pair),
    timed on the bench state: informational, beside the library's pair
    kernel."""
    import comparator
    lib = comparator.load()
    s = make_system(ljgb, 0, dev)
    pos, _, _ = s.get_state()
    L = s.L
    s.close()
    p4 = torch.zeros((N, 4), dtype=torch.float32, device="cuda")
    p4[:, :3] = torch.from_numpy(pos.astype(np.float32)).cuda()
    f4 = torch.zeros_like(p4)
    scratch = torch.zeros(int(lib.ljref_scratch_bytes(N, block)) // 4 + 4, dtype=torch.int32, device="cuda")
    dr2 = float(ljgb.reference_rdf_dr2(N))
    stream = torch.cuda.current_stream()

    def run():
        rc = lib.ljref_forces(p4.data_ptr(), f4.data_ptr(), N, L, 1, dr2, block, scratch.data_ptr(),
                              stream.cuda_stream)
        if rc != 0:
            raise RuntimeError("ljref_forces failed: cuda error %d" % rc)

    for _ in range(3):
        run()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        flush.zero_()
        a.record()
        run()
        b.record()
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    return {"kind": "restatement of the reference's calculateForces kernel (MDSystem.cu:21-153, "
                    "comparator/ref_nbody.cu), block %d, RDF counted per pair" % block,
            "ms_per_eval": ms, "pair_interactions_per_s": N * (N - 1) / (ms * 1e-3),
            "library_pair_kernel_speedup": ms / pair_ms,
            "note": "force evaluation only (the reference's host-side Verlet step and per-call allocations "
                    "are not timed); L2 flushed before every launch"}


def gpu_arm(args, rank, world, local_rank):
    import torch
    import ljgb
    import oracle
    ljgb.load()
    oracle.build()
    dev = local_rank
    torch.cuda.set_device(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > L2

    s = make_system(ljgb, 0, dev)
    s.autotune()
    tune = s.tune_info()
    shape = tune["shapes"][tune["active"]]

    dist = world > 1
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        total_ms, per_step, launches = timed_steps(torch, s, args.steps, args.warmup, flush)
    torch.cuda.synchronize()
    if dist:
        total_ms = max_over_ranks(total_ms, "cuda")
    pairs_step = N * (N - 1)
    value = replica_value(world, pairs_step, args.steps, total_ms)
    ms_step = total_ms / args.steps

    # pair-kernel duration inside the same step graph (event nodes around it)
    s.profile(True)
    ext = torch.cuda.ExternalStream(s.stream())
    for _ in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        s.integrate(DT)
    prof = s.profile_read()
    s.profile(False)
    pair_ms = prof["pair_ms"] / max(1, prof["pair_launches"])
    step_ms_prof = prof["step_ms"] / max(1, prof["steps"])

    # e2e through the C ABI with host buffers
    e2e_s, e2e_bytes = e2e_steps(ljgb, s, args.steps, args.warmup)
    e2e_value = world * pairs_step * args.steps / e2e_s
    s.close()

    result = None
    if rank == 0:
        # FP64 comparator (same workload, fewer steps)
        f = make_system(ljgb, 1, dev)
        k64 = max(3, min(args.steps, 20))
        ms64, _, _ = timed_steps(torch, f, k64, 2, flush)
        f.close()
        fp64_value = pairs_step * k64 / (ms64 * 1e-3)
        acc = accuracy(ljgb, oracle, dev)
        peak, sms, mhz = fp32_peak_nominal(dev)
        achieved = FLOPS_PER_PAIR * pairs_step / (pair_ms * 1e-3) / 1e12
        traffic = read_traffic()
        cpu = cpu_baseline(max_seconds=args.cpu_seconds)
        extra = extra_configs(torch, ljgb, oracle, dev, flush, peak) if not args.no_extra else None
        refk = ref_gpu_kernel(torch, ljgb, dev, flush, pair_ms)
        result = {
            "metric": "pair-interactions/s, N=16384, FP32-mixed vs FP64 same GB300 @ force rel err<=1e-5",
            "value": value, "unit": "pair-interactions/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-pairs/f64-state", "data": "synthetic (seeded FCC+jitter)",
            "config": bench_config(world), "kernel_shape": shape,
            "steps_per_s": 1e3 / ms_step,
            "e2e": {"value": e2e_value, "unit": "pair-interactions/s", "h2d_bytes_per_step":
                    e2e_bytes["h2d_bytes_per_step"], "d2h_bytes_per_step": e2e_bytes["d2h_bytes_per_step"],
                    "ms_per_step": e2e_s * 1e3 / args.steps},
            "fp64": {"value": fp64_value, "unit": "pair-interactions/s", "ms_per_step": ms64 / k64, "steps": k64,
                     "mixed_over_fp64": value / world / fp64_value},
            "accuracy": acc,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_pairs_mixed_fused", "flops_per_pair": FLOPS_PER_PAIR,
                         "pair_kernel_ms": pair_ms, "step_ms_profiled": step_ms_prof,
                         "step_frac": FLOPS_PER_PAIR * pairs_step / (ms_step * 1e-3) / 1e12 / peak,
                         "peak_source": "nominal FP32: %d SMs x 128 lanes x 2 x %.0f MHz (MEASURED_PEAKS.json "
                                        "has no FP32 figure)" % (sms, mhz)},
            "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "ref_gpu_kernel": refk,
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        if extra:
            result["configs"] = extra
    return result


def reference_arm(args, rank, world):
    if rank != 0:
        return None
    # Each step is a bounded sample of one N=16384 step of the reference CPU
    # algorithm: its force loop (MDSystem.cpp:237-311, restated bit-exactly)
    # over a slice of the rows, rotating through all N rows, sized so that
    # warm-up + steps stay within about 150 s.  The O(N) integration of a
    # step is left out of the sample (well under 0.1% of a step at this N).
    import oracle
    oracle.build()
    threads = oracle.default_threads()
    p4, v4 = cpu_state()
    r = oracle.R32System(N, T0, RHO, True, 0, p4, v4)
    t0 = time.perf_counter()
    r.calculate_forces(threads)                      # calibration: one full force evaluation
    full = time.perf_counter() - t0
    budget = 150.0
    rows = max(64, min(N, int(N * budget / max(args.steps + args.warmup, 1) / max(full, 1e-6))))
    cursor = [0]

    def step():
        i0 = cursor[0]
        i1 = min(N, i0 + rows)
        r.force_rows(i0, i1, threads)
        cursor[0] = 0 if i1 >= N else i1
        return (i1 - i0) * (N - 1)

    for _ in range(args.warmup):
        step()
    pairs = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pairs += step()
    el = time.perf_counter() - t0
    value = pairs / el
    sample = ("force loop of the N=16384 workload over %d rows per step (%d ordered pairs), rotating through "
              "all rows; MDSystem.cpp CPU path restated bit-exactly in C (oracle/lj_oracle.c), OpenMP over i"
              % (rows, rows * (N - 1)))
    return {
        "metric": "pair-interactions/s, N=16384, FP32-mixed vs FP64 same GB300 @ force rel err<=1e-5",
        "impl": "reference", "value": value, "unit": "pair-interactions/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el * 1e3 / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-storage/f64-temporaries",
        "data": "synthetic (seeded FCC+jitter)", "config": bench_config(world),
        "cpu_baseline": {"value": value, "unit": "pair-interactions/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "pair-interactions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own sources are not present on this machine; the bit-exact C restatement of "
                "its CPU path runs instead (pinned to the reference by tests/golden)",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-extra", action="store_true", help="skip the other configurations")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        res = reference_arm(args, rank, world)
    else:
        if world > 1:
            import torch
            torch.cuda.set_device(local_rank)
            torch.distributed.init_process_group("nccl")
        res = gpu_arm(args, rank, world, local_rank)
        if world > 1:
            import torch
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
    if rank == 0 and res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
