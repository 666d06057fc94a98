"""Command-line driver: one box, n steps, printed observables.

    python lennard-jones-cuda_gb300/ljgb/run_case.py --n 16384 --rho 0.85 --T 1.0 \\
        --tvn --fcc --jitter 0.02 --steps 10

The counterpart of the reference's task drivers (src/tasks/*) for quick runs
and for profiling a fixed workload (every step is one CUDA-graph launch of
the drift / pair / reduce / thermostat / observable kernels).
"""
import argparse
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import ljgb  # noqa: E402


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--rho", type=float, default=0.85)
    ap.add_argument("--T", type=float, default=1.0)
    ap.add_argument("--dt", type=float, default=0.005)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--tvn", action="store_true")
    ap.add_argument("--fcc", action="store_true")
    ap.add_argument("--jitter", type=float, default=0.02)
    ap.add_argument("--bc", type=int, default=0)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--shape", type=int, default=-1, help="pair-kernel shape (-1: autotune)")
    ap.add_argument("--time-shapes", action="store_true", help="print the pair-kernel time of every shape")
    ap.add_argument("--adjoint", type=int, default=0, metavar="K",
                    help="run the adjoint instead (EVN, FP64, checkpoints every K steps): forward + backward "
                         "of loss = <V/N + P> over --steps steps")
    ap.add_argument("--rdf", type=int, default=-1, metavar="MODE",
                    help="after the steps, time --calls RDF passes (0: clamped r^2 bins, 1: r^2 bins with overflow "
                         "dropped, 2: linear r bins to L/2)")
    ap.add_argument("--velo", action="store_true", help="after the steps, time --calls speed histograms")
    ap.add_argument("--calls", type=int, default=20)
    ap.add_argument("--batch", type=int, default=0, metavar="K",
                    help="run the batched-replicas workload instead: K boxes (N in [200, 4000), rho* in [0.01, 1.1], "
                         "T* in [0.7, 2.0], half hard-wall, TVN, dt 0.004); --shape as above")
    a = ap.parse_args(argv)
    if a.batch > 0:
        cfgs = ljgb.replica_batch_configs(3, a.batch)
        b = ljgb.System(batch=cfgs)
        if a.shape >= 0:
            b.set_kernel_shape(a.shape)
        else:
            b.autotune()
        b.integrate(0.004, 2)
        b.profile(True)
        b.integrate(0.004, a.steps)
        p = b.profile_read()
        b.profile(False)
        obs = b.batch_observables()
        pairs = float(sum(c.n * (c.n - 1) for c in cfgs))
        step_ms = p["step_ms"] / max(1, p["steps"])
        print("batch of %d boxes (sum N %d): pair kernel %.4f ms, step %.4f ms, %.3e pair-interactions/s, "
              "U/N of box 0 %.6f, tune %s" % (a.batch, sum(c.n for c in cfgs), p["pair_ms"] / max(1, p["pair_launches"]),
                                              step_ms, pairs / (step_ms * 1e-3), obs[0]["U"] / cfgs[0].n,
                                              {k: v for k, v in b.tune_info().items() if k != "shapes"}))
        b.close()
        return
    if a.adjoint > 0:
        adj = ljgb.Adjoint(n=a.n, density=a.rho, temperature=a.T, lattice=ljgb.LATTICE_FCC if a.fcc else
                           ljgb.LATTICE_SC, jitter=a.jitter, seed=a.seed, checkpoint_every=a.adjoint)
        adj.set_loss(0.0, 1.0, 1.0)
        t0 = time.perf_counter()
        loss = adj.forward(a.dt, a.steps)
        t1 = time.perf_counter()
        de, ds, dx, _ = adj.backward()
        t2 = time.perf_counter()
        print("adjoint n=%d steps=%d loss=%.10f dloss/deps=%.6e dloss/dsigma=%.6e |dloss/dx0|max=%.3e "
              "forward=%.3fs backward=%.3fs" % (a.n, a.steps, loss, de, ds, abs(dx).max(), t1 - t0, t2 - t1))
        return
    s = ljgb.System(n=a.n, density=a.rho, temperature=a.T, canonical=int(a.tvn), boundary=a.bc,
                    lattice=ljgb.LATTICE_FCC if a.fcc else ljgb.LATTICE_SC, jitter=a.jitter, seed=a.seed,
                    precision=ljgb.PREC_FP64 if a.fp64 else ljgb.PREC_MIXED)
    if a.time_shapes and not a.fp64:
        info = s.tune_info()
        for k, sh in enumerate(info["shapes"]):
            s.set_kernel_shape(k)
            s.integrate(a.dt, 3)
            s.profile(True)
            s.integrate(a.dt, a.steps)
            p = s.profile_read()
            s.profile(False)
            pairs = a.n * (a.n - 1)
            ms = p["pair_ms"] / max(1, p["pair_launches"])
            print("shape %d %s: pair kernel %.4f ms (%.3e pairs/s), step %.4f ms" % (
                k, sh, ms, pairs / (ms * 1e-3), p["step_ms"] / max(1, p["steps"])))
    if not a.fp64:
        if a.shape >= 0:
            s.set_kernel_shape(a.shape)
        else:
            s.autotune()
    t0 = time.perf_counter()
    s.integrate(a.dt, a.steps)
    o = s.observables()
    el = time.perf_counter() - t0
    print("n=%d steps=%d t=%.4f U/N=%.8f T=%.6f P=%.6f wall=%.3fs shape=%s" % (
        a.n, a.steps, o["t"], o["U"] / a.n, o["T"], o["P"], el, s.tune_info()["active"]))
    if a.rdf >= 0:
        nb, width = (200, (s.L / 2) / 200) if a.rdf == 2 else (256, ljgb.reference_rdf_dr2(a.n))
        s.rdf_counts(a.rdf, nb, width)
        t0 = time.perf_counter()
        for _ in range(a.calls):
            c = s.rdf_counts(a.rdf, nb, width)
        ms = (time.perf_counter() - t0) * 1e3 / a.calls
        print("rdf mode %d: %d bins, %.4f ms per call (host clock, synchronised), %d pairs counted, last bin %d" % (
            a.rdf, nb, ms, int(c.sum()), int(c[-1])))
    if a.velo:
        s.velocity_counts()
        t0 = time.perf_counter()
        for _ in range(a.calls):
            c = s.velocity_counts()
        ms = (time.perf_counter() - t0) * 1e3 / a.calls
        print("speed histogram: %.4f ms per call (host clock, synchronised), %d counted" % (ms, int(c.sum())))
    s.close()


if __name__ == "__main__":
    main()
