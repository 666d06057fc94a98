"""The benchmark configurations end to end (GPU tests).

Each test runs one configuration of the path as specified -- sizes,
densities, temperatures, lattices, ensembles, step counts -- through the C ABI
and checks it against the FP64 oracle or the all-FP64 GPU path:

  * plain method: N=400, rho*=0.05, T*=1.4, SC lattice +-0.05 sigma jitter,
    Maxwell velocities, dt=0.005, EVN, 1000 steps, FP64; per-step K, V, W
    against the FP64 oracle and a 200-bin RDF to r = L/2;
  * dense liquid: N=16384, rho*=0.85, T*=1.0, FCC +-0.02, dt=0.005, TVN,
    10^4 steps; mixed precision step by step (first 10 steps) against the
    all-FP64 run, then time averages of U/N, P and g(r) against it;
  * batched replicas: 256 boxes, 5000 TVN steps; per-replica averages of a
    sample against all-FP64 runs;
  * large single system: N=262144, rho*=1.1 (solid), T*=1.0, FCC +-0.01,
    dt=0.004, TVN; forces on a 4096-particle seeded subset against the FP64
    oracle, then TVN steps;
  * energy drift of the mixed path against the FP64 path over 1e5 EVN steps.
"""
import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu


def test_plain_method_configuration(ljgb_mod, oracle_mod):
    N, rho, T0, dt, S = 400, 0.05, 1.4, 0.005, 1000
    cfg = ljgb_mod.config(n=N, density=rho, temperature=T0, canonical=0, lattice=ljgb_mod.LATTICE_SC,
                          jitter=0.05, seed=400, precision=ljgb_mod.PREC_FP64)
    pos, vel = ljgb_mod.sample_initial_state(cfg)
    assert np.abs(vel.sum(0)).max() < 1e-10                          # zero net momentum
    assert 0.5 * (vel * vel).sum() * 2 / 3 / N == pytest.approx(T0, rel=1e-12)
    s = ljgb_mod.System(cfg=cfg)
    s.set_recording(S)
    s.integrate(dt, S)
    rec = s.records()
    assert len(rec) == S and rec[-1]["step"] == S
    o = oracle_mod.F64System(pos, vel, s.L, rho, T0, False, 0)
    K, V, W = np.zeros(S), np.zeros(S), np.zeros(S)
    for m in range(S):
        o.step(dt)
        K[m], V[m], W[m] = o.K, o.V, o.W
    for key, ref in (("K", K), ("V", V), ("W", W)):
        got = np.array([r[key] for r in rec])
        err = np.abs(got - ref).max() / np.abs(ref).max()
        print("plain method: per-step %s max rel deviation from the FP64 oracle over %d steps: %.2e" % (key, S, err))
        assert err < 3e-9, key
    # 200-bin RDF to r = L/2 of the final state (exact counts, device binning rule)
    p, _, _ = s.get_state()
    dr = (s.L / 2) / 200
    got = s.rdf_counts(ljgb_mod.RDF_R_LINEAR, 200, dr)
    ks = s.L / (4294967296.0 * 1.0)
    want = oracle_mod.emu_rdf_r(oracle_mod.emu_fixed(p, s.L), np.float32(ks * ks), np.float32(1.0 / dr),
                                np.float32((200 * dr) ** 2), 200)
    assert np.array_equal(got, want)
    # every pair closer than L/2 is counted once per ordered pair
    d = p[:, None, :] - p[None, :, :]
    d -= s.L * np.round(d / s.L)
    r = np.sqrt((d * d).sum(-1))[~np.eye(N, dtype=bool)]
    assert abs(int(got.sum()) - int((r < s.L / 2).sum())) <= 4


def time_average(x):
    """Mean and its error the way the reference's TimeAverage forms them
    (src/tasks/auxiliary/time-average-aux.h:27-67): the error of the mean
    scaled by the square root of the statistical inefficiency."""
    import tasks
    m = tasks.moments(x)
    return m["mean"], m["mean_err"] * np.sqrt(tasks.inefficiency(x))


def block_time_average(x, block=100):
    """TimeAverage of the means of consecutive `block`-step blocks.  The
    inefficiency formula assumes exponentially decaying correlations; per-step
    U and P of a TVN run also carry step-to-step (anti)correlations from the
    thermostat, which make the lag-1 estimate of a per-step series useless
    (s = 1 where runs that differ by a 1e-9 perturbation disagree by 40
    errors).  Block means remove those; their inefficiency then measures the
    slow correlations."""
    x = np.asarray(x, np.float64)
    nb = len(x) // block
    return time_average(x[:nb * block].reshape(nb, block).mean(1))


def test_dense_liquid_configuration(ljgb_mod):
    """N=16384, rho*=0.85, T*=1.0, FCC +-0.02, dt=0.005, TVN for 10^4 steps,
    mixed precision against the all-FP64 run: step by step for the first 10
    steps, then time averages of U/N, P and g(r) over steps 1001..10000
    within their statistical errors."""
    N, rho, T0, dt = 16384, 0.85, 1.0, 0.005
    S, S_eq, blk = 10000, 1000, 100
    kw = dict(n=N, density=rho, temperature=T0, canonical=1, lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=2)
    mixed = ljgb_mod.System(**kw, precision=ljgb_mod.PREC_MIXED)
    fp64 = ljgb_mod.System(**kw, precision=ljgb_mod.PREC_FP64)
    L = mixed.L
    # step by step, first 10 steps
    for k in range(10):
        mixed.integrate(dt)
        fp64.integrate(dt)
        pm, vm, fm = mixed.get_state()
        pd, vd, fd = fp64.get_state()
        dp = pm - pd
        dp -= L * np.round(dp / L)
        om, od = mixed.observables(), fp64.observables()
        err = U.force_errors(fm, fd)
        print("dense liquid step %d: |dx| %.2e |dv| %.2e force gate %.2e dU/N %.2e dP %.2e" % (
            k + 1, np.abs(dp).max(), np.abs(vm - vd).max(), err["gate_max"], abs(om["U"] - od["U"]) / N,
            abs(om["P"] - od["P"])))
        assert np.abs(dp).max() < 1e-6 * L
        assert np.abs(vm - vd).max() < 1e-5
        assert err["gate_max"] < 1e-5
        assert om["T"] == pytest.approx(od["T"], rel=1e-7)
        assert om["U"] == pytest.approx(od["U"], rel=1e-6)
        assert om["P"] == pytest.approx(od["P"], rel=1e-5)
    # Both runs continue to step S.  The trajectories decorrelate; the
    # averages after equilibration must agree within their statistical
    # errors: U/N and P from the per-step records, g(r) summed on the device
    # after every step (100 linear bins to L/2) and read every 100 steps.
    nbr = 100
    width = (L / 2) / nbr
    # ordered pairs per step of an ideal gas in each shell: N rho 4/3 pi (r1^3 - r0^3)
    edges = width * np.arange(nbr + 1)
    ideal = N * rho * 4.0 / 3.0 * np.pi * (edges[1:] ** 3 - edges[:-1] ** 3)
    g, series = {}, {}
    for name, s in (("mixed", mixed), ("fp64", fp64)):
        s.set_recording(S - S_eq)
        s.rdf_accumulate(True, mode=ljgb_mod.RDF_R_LINEAR, nbins=nbr, width=width)
        done, blocks = 10, []
        while done < S:
            k = blk - done % blk
            s.integrate(dt, k)
            c, ns = s.rdf_accumulated(reset=True)
            assert ns == k
            done += k
            if done > S_eq:
                blocks.append(c.astype(np.float64) / ns / ideal)
        s.rdf_accumulate(False)
        g[name] = np.array(blocks)
        rec = s.records(max_records=S - S_eq)
        assert len(rec) == S - S_eq and rec[0]["step"] == S_eq + 1 and rec[-1]["step"] == S
        series[name] = (np.array([r["U"] for r in rec]) / N, np.array([r["P"] for r in rec]),
                        np.array([r["T"] for r in rec]))
    assert len(g["mixed"]) == (S - S_eq) // blk
    # g(r): per-bin time averages of the 100-step block means
    gm = np.array([time_average(col) for col in g["mixed"].T])
    gd = np.array([time_average(col) for col in g["fp64"].T])
    err_g = np.hypot(gm[:, 1], gd[:, 1])
    dev_g = np.abs(gm[:, 0] - gd[:, 0]) / (err_g + 1e-3 * gd[:, 0].max())
    print("dense liquid g(r) over steps %d..%d: first peak g=%.4f at r=%.3f, max |mixed - fp64| / error %.2f "
          "(max |dg| %.2e)" % (S_eq + 1, S, gd[:, 0].max(), (gd[:, 0].argmax() + 0.5) * width, dev_g.max(),
                               np.abs(gm[:, 0] - gd[:, 0]).max()))
    assert 2.0 < gd[:, 0].max() < 4.0 and abs(gd[-10:, 0].mean() - 1.0) < 0.05
    assert dev_g.max() < 5
    for q, label, floor in ((0, "U/N", 1e-4), (1, "P", 1e-3)):
        am, em = block_time_average(series["mixed"][q])
        ad, ed = block_time_average(series["fp64"][q])
        print("dense liquid <%s> over steps %d..%d: %.7f +- %.1e (mixed), %.7f +- %.1e (fp64), "
              "difference %.2f sigma" % (label, S_eq + 1, S, am, em, ad, ed, abs(am - ad) / np.hypot(em, ed)))
        assert abs(am - ad) < 4 * np.hypot(em, ed) + floor, label
    # TVN holds the kinetic temperature of both runs at T0
    for name in ("mixed", "fp64"):
        assert abs(series[name][2].mean() - T0) < 5e-3, name


def test_batched_replicas_configuration(ljgb_mod):
    """256 replicas (N uniform in [200, 4000), rho* in [0.01, 1.1], T* in
    [0.7, 2.0], periodic and hard-wall boxes alternating), dt=0.004, 5000 TVN
    steps in one launch per step, autotuned and graph-captured.  Every
    replica stays finite, in its box and at its temperature.  For a seeded
    sample of 8 replicas (4 periodic, 4 walled) the time averages of U/N and
    P over steps 1001..5000 agree with all-FP64 runs of the same replicas
    within statistical error.

    Many replicas are still relaxing after 1000 steps (a gas below T_c
    condensing, a walled box building its wall layers), so the averages are
    over a non-stationary stretch.  Their statistical error is measured
    directly: each sampled replica runs R times in FP64, the copies differing
    by 1e-9 in one velocity component, which the dynamics amplifies into
    independent trajectories of the same relaxation.  The mixed run is one
    more such draw: |mixed - mean_FP64| <= 5 sqrt(sd^2 (1 + 1/R) + e^2) +
    floor, with sd the spread of the FP64 copies and e the mixed run's
    block TimeAverage error."""
    S, S_eq, dt, R = 5000, 1000, 0.004, 6
    cfgs = ljgb_mod.replica_batch_configs(seed=3, k=256)
    b = ljgb_mod.System(batch=cfgs)
    b.autotune()
    b.set_recording(S - S_eq)
    b.integrate(dt, S)
    obs = b.batch_observables()
    p, _, _ = b.get_state()
    for k, (c, o) in enumerate(zip(cfgs, obs)):
        assert o["step"] == S and np.isfinite(o["U"]) and np.isfinite(o["P"]), k
        L = (c.n / c.density) ** (1 / 3)
        pk = p[b.offsets[k]:b.offsets[k + 1]]
        if c.boundary == 1:
            assert pk.min() > -0.5 and pk.max() < L + 0.5, k
        # TVN holds the kinetic temperature at T0 in every replica
        Tk = np.array([r["T"] for r in b.batch_records(k, max_records=S - S_eq)])
        assert len(Tk) == S - S_eq and abs(Tk.mean() - c.temperature) < 0.03 * c.temperature, k
    rng = np.random.default_rng(8)
    sample = sorted(list(rng.choice(np.arange(0, 256, 2), 4, replace=False)) +
                    list(rng.choice(np.arange(1, 256, 2), 4, replace=False)))
    ref_cfgs = ljgb_mod.replica_batch_configs(seed=3, k=256)
    sel = [ref_cfgs[k] for k in sample for _ in range(R)]
    for c in sel:
        c.precision = ljgb_mod.PREC_FP64
    d = ljgb_mod.System(batch=sel)
    pd, vd, _ = d.get_state()
    for j in range(len(sample)):
        for r in range(1, R):
            vd[d.offsets[j * R + r], 0] += 1e-9 * r
    d.set_state(None, vd)
    d.calculate_forces()
    d.set_recording(S - S_eq)
    d.integrate(dt, S)
    worst = 0.0
    for j, k in enumerate(sample):
        c = cfgs[k]
        rm = b.batch_records(k, max_records=S - S_eq)
        assert len(rm) == S - S_eq and rm[-1]["step"] == S
        line = []
        for key, scale, floor in (("U", 1.0 / c.n, 1e-4), ("P", 1.0, 1e-4)):
            am, em = block_time_average(np.array([r[key] for r in rm]) * scale)
            ens = []
            for r in range(R):
                rd = d.batch_records(j * R + r, max_records=S - S_eq)
                assert len(rd) == S - S_eq and rd[-1]["step"] == S
                ens.append(np.mean([x[key] for x in rd]) * scale)
            mu, sd = float(np.mean(ens)), float(np.std(ens, ddof=1))
            sig = np.sqrt(sd * sd * (1 + 1.0 / R) + em * em)
            dev = abs(am - mu) / (sig + floor)
            worst = max(worst, dev)
            line.append("<%s> %.6f (block error %.1e) / FP64 %.6f, spread %.1e over %d runs (%.2f sigma)" % (
                "U/N" if key == "U" else "P", am, em, mu, sd, R, dev))
            assert abs(am - mu) < 5 * sig + floor, (k, key, line[-1])
        print("replica %3d (N=%d rho*=%.3f T*=%.3f %s): %s" % (k, c.n, c.density, c.temperature,
                                                             "wall" if c.boundary else "periodic", "; ".join(line)))
    print("batched replicas: largest mixed-vs-FP64 deviation %.2f sigma" % worst)


def test_large_single_system_configuration(ljgb_mod, oracle_mod):
    N, rho, T0, dt = 262144, 1.1, 1.0, 0.004
    s = ljgb_mod.System(n=N, density=rho, temperature=T0, canonical=1, lattice=ljgb_mod.LATTICE_FCC, jitter=0.01,
                        seed=262144)
    pos, _, F = s.get_state()
    i0 = int(np.random.default_rng(4096).integers(0, N - 4096))
    r = oracle_mod.f64_forces(pos, s.L, True, rows=(i0, i0 + 4096))
    err = U.force_errors(F[i0:i0 + 4096], r["F"])
    print("large system: 4096 rows from %d vs FP64 oracle: %s" % (i0, err))
    assert err["gate_max"] <= 1e-5 and err["rel_median"] <= 1e-5
    e, _ = s.pair_sums()
    assert np.abs(e[i0:i0 + 4096] - r["e"]).max() <= 1e-5 * np.abs(r["e"]).max()
    s.integrate(dt, 20)
    o = s.observables()
    assert o["step"] == 20 and np.isfinite(o["U"])
    # TVN: chi = sqrt(T0 / Tkin) of the half-kicked velocities keeps both near T0
    assert o["Tkin_tvn"] == pytest.approx(T0, rel=0.02)
    assert abs(o["T"] - T0) < 0.05


def test_energy_drift_mixed_vs_fp64(ljgb_mod):
    """EVN, N=2048, rho*=0.85, T*=1.0, dt=0.005, 1e5 steps: the drift of the
    total energy per particle of the mixed path against the all-FP64 path."""
    N, rho, dt, S, every = 2048, 0.85, 0.005, 100000, 1000
    kw = dict(n=N, density=rho, temperature=1.0, canonical=0, lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=5)
    fit = {}
    for name, prec in (("mixed", ljgb_mod.PREC_MIXED), ("fp64", ljgb_mod.PREC_FP64)):
        s = ljgb_mod.System(**kw, precision=prec)
        s.integrate(dt, 2000)                      # equilibrate from the lattice
        u = []
        for _ in range(S // every):
            s.integrate(dt, every)
            u.append(s.observables()["U"] / N)
        u = np.array(u)
        t = dt * every * np.arange(1, len(u) + 1)
        slope, icpt = np.polyfit(t, u, 1)
        resid = u - (slope * t + icpt)
        fit[name] = (slope, resid.std(), u.max() - u.min())
        print("energy drift %s: dU/N/dt %.3e per tau, residual %.2e, range %.2e over %d steps" % (
            name, slope, resid.std(), u.max() - u.min(), S))
    (sm, rm, _), (sd, rd, _) = fit["mixed"], fit["fp64"]
    T = dt * S
    # No extra drift: over the whole run the mixed path's drift exceeds the
    # FP64 path's by less than the fluctuation level.  (The FP64 path drifts
    # too: the minimum-image force jumps where a pair crosses L/2, and Verlet
    # does not conserve energy across such a jump.)
    assert abs(sm) * T < abs(sd) * T + 5 * max(rm, rd) + 1e-5
