"""Integrator, boundaries, observables and running averages (GPU tests).

Step-by-step parity of the device velocity Verlet (EVN) and constant-kinetic-
temperature Verlet (TVN) with the FP64 oracle restatement of
MDSystem::Integrate (MDSystem.cpp:438-583), on identical seeded states,
through the C ABI.
"""
import os

import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu

GOLDEN = U.golden_states()


def run_pair(ljgb, oracle_mod, pos, vel, N, rho, T0, canonical, bc, dt, steps, prec):
    s = ljgb.System(n=N, density=rho, temperature=T0, boundary=bc, canonical=int(canonical), precision=prec)
    s.set_state(pos, vel)
    s.calculate_forces()
    o = oracle_mod.F64System(pos, vel, s.L, rho, T0, canonical, bc, nthreads=4)
    for k in range(steps):
        s.integrate(dt)
        o.step(dt)
    p, v, f = s.get_state()
    return s, o, p, v, f


@pytest.mark.parametrize("prec", [0, 1], ids=["mixed", "fp64"])
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_trajectory_matches_fp64_oracle(ljgb_mod, oracle_mod, path, prec):
    g = dict(np.load(path))
    N, rho, T0, bc = int(g["N"]), float(g["rho"]), float(g["T0"]), int(g["bc"])
    rng = np.random.default_rng(0)
    pos = g["pos0"][:, :3].astype(np.float64) + rng.uniform(-1e-7, 1e-7, (N, 3))  # no exact half-box ties
    vel = g["vel0"][:, :3].astype(np.float64)
    steps = 20
    s, o, p, v, f = run_pair(ljgb_mod, oracle_mod, pos, vel, N, rho, T0, bool(g["canonical"]), bc,
                             float(g["dt"]), steps, prec)
    tol = 1e-6 if prec == 0 else 1e-11
    assert np.abs(p - o.pos).max() < tol * max(1.0, s.L)
    assert np.abs(v - o.vel).max() < tol * 10
    obs = s.observables()
    for k in ("K", "V", "T", "P", "U"):
        assert obs[k] == pytest.approx(getattr(o, k), rel=tol * 10, abs=tol * 10 * N), k
    assert obs["t"] == pytest.approx(o.t, rel=1e-14)
    assert obs["step"] == steps


@pytest.mark.parametrize("prec", [0, 1], ids=["mixed", "fp64"])
def test_tvn_dense_liquid(ljgb_mod, oracle_mod, prec):
    N, rho, T0 = 2048, 0.85, 1.0
    pos, vel, L = U.lattice_state(N, rho, 1.3, "fcc", 0.02, seed=3)
    s, o, p, v, f = run_pair(ljgb_mod, oracle_mod, pos, vel, N, rho, T0, True, 0, 0.005, 10, prec)
    obs = s.observables()
    assert np.abs(v - o.vel).max() < (2e-6 if prec == 0 else 1e-11)
    # the TVN scale was computed from the half-kicked velocities
    assert obs["Tkin_tvn"] > 0
    assert obs["T"] == pytest.approx(o.T, rel=1e-8)


def test_records_and_time(ljgb_mod):
    N, rho = 400, 0.05
    pos, vel, L = U.lattice_state(N, rho, 1.4, "sc", 0.05, seed=1)
    s = ljgb_mod.System(n=N, density=rho, temperature=1.4)
    s.set_state(pos, vel)
    s.calculate_forces()
    s.set_recording(64)
    s.integrate(0.005, 100)
    rec = s.records()
    assert len(rec) == 64
    steps = [r["step"] for r in rec]
    assert steps == list(range(37, 101))
    assert rec[-1]["t"] == pytest.approx(100 * 0.005)
    obs = s.observables()
    assert obs["U"] == rec[-1]["U"] and obs["step"] == 100
    # running averages advance every step (CalculateParameters, MDSystem.cpp:355-358)
    assert obs["av_iters"] == 101
    assert rec[-1]["av_U_tot"] == obs["av_U_tot"]


def test_energy_conservation_and_momentum(ljgb_mod):
    """EVN, periodic, config-1 point (N=400, rho=0.05, T=1.4), 2000 steps."""
    N, rho = 400, 0.05
    pos, vel, L = U.lattice_state(N, rho, 1.4, "sc", 0.05, seed=1)
    drift = {}
    for prec in (0, 1):
        s = ljgb_mod.System(n=N, density=rho, temperature=1.4, precision=prec)
        s.set_state(pos, vel)
        s.calculate_forces()
        U0 = s.observables()["U"]
        s.set_recording(2000)
        s.integrate(0.002, 2000)
        Us = np.array([r["U"] for r in s.records()])
        _, v, _ = s.get_state()
        # FP32 per-particle sums round independently, so the pair forces do
        # not cancel to the last bit: total momentum random-walks at ~1e-6 over
        # this run in the mixed path; FP64 sums cancel to round-off.
        assert np.abs(v.sum(0)).max() < (3e-5 if prec == 0 else 1e-10)
        drift[prec] = np.abs(Us - U0).max() / N
    assert drift[1] < 2e-3
    assert drift[0] < 2e-3
    assert abs(drift[0] - drift[1]) < 1e-4


def test_wall_energy_conservation_fused_vs_fp64(ljgb_mod):
    """EVN between hard walls (N=500, rho*=0.3, T*=1.4, 2000 steps): a wall
    flips a velocity component and keeps K, so U is conserved as in a
    periodic box.  The fused mixed path (fixed wall frame) and the FP64
    kernel-per-phase path conserve it alike."""
    N, rho = 500, 0.3
    drift = {}
    for prec in (0, 1):
        s = ljgb_mod.System(n=N, density=rho, temperature=1.4, boundary=1, lattice=ljgb_mod.LATTICE_FCC,
                            jitter=0.05, seed=11, precision=prec)
        U0 = s.observables()["U"]
        s.set_recording(2000)
        s.integrate(0.002, 2000)
        Us = np.array([r["U"] for r in s.records()])
        p, _, _ = s.get_state()
        assert p.min() > -0.5 and p.max() < s.L + 0.5
        drift[prec] = np.abs(Us - U0).max() / N
    assert drift[0] < 2e-3 and drift[1] < 2e-3
    assert abs(drift[0] - drift[1]) < 2e-4


def test_wall_keeps_particles_in_box(ljgb_mod):
    N, rho = 500, 0.3
    s = ljgb_mod.System(n=N, density=rho, temperature=2.0, boundary=1, jitter=0.05, seed=7)
    s.integrate(0.005, 400)
    p, v, _ = s.get_state()
    assert p.min() > -0.5 and p.max() < s.L + 0.5


def test_periodic_wrap(ljgb_mod):
    N, rho = 300, 0.1
    s = ljgb_mod.System(n=N, density=rho, temperature=3.0, seed=4)
    s.integrate(0.005, 300)
    p, _, _ = s.get_state()
    assert p.min() >= -1e-9 and p.max() <= s.L + 1e-9


def test_renormalize_and_reset(ljgb_mod):
    s = ljgb_mod.System(n=512, density=0.5, temperature=1.2, seed=3)
    s.integrate(0.005, 50)
    s.renormalize_velocities(True)
    _, v, _ = s.get_state()
    assert np.sum(v * v) / 3 / 512 == pytest.approx(1.2, rel=1e-12)
    assert s.observables()["T"] == 1.2
    o = s.observables()
    s.renormalize_velocities_to_energy(o["V"] / 512 + 1.0)
    _, v, _ = s.get_state()
    assert 0.5 * np.sum(v * v) == pytest.approx(512.0, rel=1e-12)
    s.reset_averaging()
    assert s.observables()["av_iters"] == 0
    s.set_time(3.0)
    s.integrate(0.01, 2)
    assert s.observables()["t"] == pytest.approx(3.02)


def test_set_canonical_and_boundary_switch(ljgb_mod, oracle_mod):
    N, rho = 600, 0.4
    pos, vel, L = U.lattice_state(N, rho, 1.0, "sc", 0.05, seed=12)
    s = ljgb_mod.System(n=N, density=rho, temperature=1.0)
    s.set_state(pos, vel)
    s.calculate_forces()
    o = oracle_mod.F64System(pos, vel, L, rho, 1.0, False, 0, nthreads=4)
    for k in range(6):
        s.integrate(0.005)
        o.step(0.005)
    s.set_canonical(True)
    o.canonical = True
    s.set_boundary(1)
    o.bc = 1
    s.calculate_forces()
    o.compute_forces()
    for k in range(6):
        s.integrate(0.005)
        o.step(0.005)
    p, v, _ = s.get_state()
    assert np.abs(v - o.vel).max() < 2e-6


def test_launch_count_and_graph_reuse(ljgb_mod):
    s = ljgb_mod.System(n=1000, density=0.8, temperature=1.0, canonical=1)
    c0 = s.launch_count()
    s.integrate(0.005, 10)
    s.sync()
    # fused TVN, periodic: one predictor, then pair kernel (+ epilogue) and
    # k_tvn_close per step; the last step's observables are computed by one
    # k_obs_finalize when the host syncs (earlier steps' inside the next
    # step's pair kernel)
    assert s.launch_count() - c0 == 1 + 2 * 10 + 1
    c1 = s.launch_count()
    s.integrate(0.005, 10)
    assert s.launch_count() - c1 == 2 * 10     # prediction carried over from the last step
    e = ljgb_mod.System(n=1000, density=0.8, temperature=1.0, canonical=0)
    c2 = e.launch_count()
    e.integrate(0.005, 10)
    assert e.launch_count() - c2 == 1 + 10     # fused EVN: one kernel per step
    w = ljgb_mod.System(n=1000, density=0.8, temperature=1.0, canonical=0, boundary=1)
    c3 = w.launch_count()
    w.integrate(0.005, 10)
    assert w.launch_count() - c3 == 1 + 10     # walls keep a fixed frame: fused as well
    o = ljgb_mod.System(n=1000, density=0.8, temperature=1.0, canonical=0, boundary=2)
    c4 = o.launch_count()
    o.integrate(0.005, 10)
    # open box: drift, frame, quantize, pairs, reduce, observables per step
    assert o.launch_count() - c4 == 6 * 10


@pytest.mark.parametrize("boundary", [0, 1])
def test_fused_matches_unfused_path(ljgb_mod, boundary):
    """The fused step (periodic and walled boxes) and the kernel-per-phase
    step (taken by FP64 and open boxes) integrate the same equations: compare
    the fused mixed path with the FP64 path over 30 steps of both ensembles.
    With walls, one particle starts outside the box moving away from it: the
    frame takes in the starting positions, and the wall turns it back."""
    N, rho = 3000, 0.8
    pos, vel, L = U.lattice_state(N, rho, 1.1, "fcc", 0.02, seed=21)
    if boundary == 1:
        pos[7] = (L + 0.3, 0.5 * L, -0.2)
        vel[7] = (2.0, 0.0, -1.0)
    for canonical in (0, 1):
        out = []
        for prec in (0, 1):
            s = ljgb_mod.System(n=N, density=rho, temperature=1.0, canonical=canonical, precision=prec,
                                boundary=boundary)
            s.set_state(pos, vel)
            s.calculate_forces()
            s.integrate(0.004, 15)
            s.integrate(0.004, 15)
            out.append((s.get_state(), s.observables()))
        (p0, v0, f0), o0 = out[0]
        (p1, v1, f1), o1 = out[1]
        assert np.abs(p0 - p1).max() < 1e-6 * L
        assert np.abs(v0 - v1).max() < 1e-5
        for k in ("K", "V", "T", "P", "U", "t"):
            assert o0[k] == pytest.approx(o1[k], rel=1e-6, abs=1e-6), (canonical, k)
        assert o0["step"] == o1["step"] == 30 and o0["av_iters"] == o1["av_iters"] == 31
        if boundary == 1:
            assert p0[7, 0] < L + 0.3 + 0.1 and v0[7, 0] < 0    # turned back by the wall at x = L


@pytest.mark.parametrize("shape", range(6))
def test_fused_step_every_shape(ljgb_mod, shape):
    """Every pair-kernel shape (i-blocks of 64 to 384 particles, ragged last
    blocks) runs the fused step -- block epilogues, per-parity pending
    observables, TVN chi in the close kernel -- as the FP64 path steps the same
    box, periodic and walled, in both ensembles."""
    N, rho = 3001, 0.8
    pos, vel, L = U.lattice_state(N, rho, 1.1, "fcc", 0.02, seed=31)
    for boundary in (0, 1):
        for canonical in (0, 1):
            out = []
            for prec in (0, 1):
                s = ljgb_mod.System(n=N, density=rho, temperature=1.0, canonical=canonical, precision=prec,
                                    boundary=boundary)
                if prec == 0:
                    s.set_kernel_shape(shape)
                s.set_state(pos, vel)
                s.calculate_forces()
                s.integrate(0.004, 7)
                s.integrate(0.004, 8)
                out.append((s.get_state(), s.observables()))
                s.close()
            (p0, v0, _), o0 = out[0]
            (p1, v1, _), o1 = out[1]
            assert np.abs(p0 - p1).max() < 1e-6 * L, (boundary, canonical)
            assert np.abs(v0 - v1).max() < 1e-5, (boundary, canonical)
            for k in ("K", "V", "T", "P", "U", "t"):
                assert o0[k] == pytest.approx(o1[k], rel=1e-6, abs=1e-6), (boundary, canonical, k)
            assert o0["step"] == o1["step"] == 15 and o0["av_iters"] == o1["av_iters"] == 16


def test_autotune_keeps_the_state(ljgb_mod):
    s = ljgb_mod.System(n=2000, density=0.85, temperature=1.0, canonical=1, lattice=1, jitter=0.02)
    s.set_recording(8)
    s.integrate(0.005, 5)
    p0, v0, f0 = s.get_state()
    o0 = s.observables()
    r0 = s.records()
    s.autotune()
    p1, v1, f1 = s.get_state()
    o1 = s.observables()
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)
    assert np.abs(f0 - f1).max() <= 1e-5 * np.abs(f0).max()   # recomputed with the chosen shape
    for k in ("t", "step", "av_iters", "av_U_tot", "av_p_tot", "av_T_tot", "K", "U"):
        assert o0[k] == o1[k], k
    assert s.records() == r0
    s.integrate(0.005, 3)
    assert s.observables()["step"] == 8


def test_set_state_checks_and_round_trips(ljgb_mod):
    """lj_set_state checks finiteness on the device and leaves the state
    unchanged when it rejects a call; set/get round-trip bit for bit."""
    s = ljgb_mod.System(n=700, density=0.6, temperature=1.0, lattice=ljgb_mod.LATTICE_FCC, jitter=0.05)
    s.integrate(0.005, 3)
    p0, v0, f0 = s.get_state()
    bad_v = v0.copy()
    bad_v[5, 1] = np.nan
    with pytest.raises(ljgb_mod.LJError, match="velocity of particle 5"):
        s.set_state(p0 + 0.01, bad_v)
    bad_p = p0.copy()
    bad_p[3, 2] = np.inf
    with pytest.raises(ljgb_mod.LJError, match="position of particle 3"):
        s.set_state(bad_p, v0)
    p1, v1, f1 = s.get_state()
    assert np.array_equal(p1, p0) and np.array_equal(v1, v0) and np.array_equal(f1, f0)
    rng = np.random.default_rng(1)
    p2 = p0 + rng.normal(scale=1e-3, size=p0.shape)
    v2 = v0 * 1.01
    s.set_state(p2, None)
    s.set_state(None, v2)
    p3, v3, _ = s.get_state()
    assert np.array_equal(p3, p2) and np.array_equal(v3, v2)
    s.integrate(0.005, 2)
    assert s.observables()["step"] == 5


@pytest.mark.parametrize("boundary", [0, 1])
def test_set_state_async(ljgb_mod, boundary):
    """lj_set_state_async queues what lj_set_state does: an upload/step/read
    loop with one synchronisation per step gives the same trajectory, bit for
    bit, as the synchronous uploads; a non-finite upload is dropped on the
    device and reported by the next synchronising call."""
    kw = dict(n=900, density=0.7, temperature=1.1, canonical=1, boundary=boundary,
              lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=4)
    a, b = ljgb_mod.System(**kw), ljgb_mod.System(**kw)
    pa, va = ljgb_mod.pinned((900, 3)), ljgb_mod.pinned((900, 3))
    pb, vb = ljgb_mod.pinned((900, 3)), ljgb_mod.pinned((900, 3))
    a.get_state_into(pa, va, None)
    b.get_state_into(pb, vb, None)
    for _ in range(6):
        va *= 0.999                      # the host changes the state between steps
        vb *= 0.999
        a.set_state_async_from(pa, va)
        b.set_state_from(pb, vb)
        a.integrate(0.005)
        b.integrate(0.005)
        oa = a.get_state_observables_into(pa, va, None)
        ob = b.get_state_observables_into(pb, vb, None)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)
        assert oa["U"] == ob["U"] and oa["step"] == ob["step"]
    p0, v0, f0 = a.get_state()
    bad = ljgb_mod.pinned((900, 3))
    bad[:] = v0
    bad[17, 0] = np.nan
    a.set_state_async_from(None, bad)    # queued; the check runs on the device
    with pytest.raises(ljgb_mod.LJError, match="lj_set_state_async"):
        a.sync()
    p1, v1, f1 = a.get_state()
    assert np.array_equal(p1, p0) and np.array_equal(v1, v0) and np.array_equal(f1, f0)
    a.integrate(0.005, 2)
    assert np.isfinite(a.observables()["U"])
    a.close()
    b.close()


@pytest.mark.parametrize("boundary", [0, 1])
def test_step_io_matches_separate_calls(ljgb_mod, boundary):
    """lj_step_io (queued upload, steps, read-back and observables, one
    synchronisation) gives what lj_set_state + lj_step +
    lj_get_state_observables give, bit for bit: with page-locked buffers (the
    kernels read and write them directly) and with pageable ones (staged
    copies).  A non-finite input is reported by the same call."""
    n = 1100
    kw = dict(n=n, density=0.75, temperature=1.2, canonical=1, boundary=boundary,
              lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=9)
    a, b, c = ljgb_mod.System(**kw), ljgb_mod.System(**kw), ljgb_mod.System(**kw)
    pa, va = ljgb_mod.pinned((n, 3)), ljgb_mod.pinned((n, 3))
    pc, vc = np.zeros((n, 3)), np.zeros((n, 3))
    a.get_state_into(pa, va, None)
    c.get_state_into(pc, vc, None)
    pb, vb, _ = b.get_state()
    for _ in range(5):
        va *= 0.999
        vb *= 0.999
        vc *= 0.999
        oa = a.step_io(0.005, 2, pa, va, pa, va)
        oc = c.step_io(0.005, 2, pc, vc, pc, vc)
        b.set_state(pb, vb)
        b.integrate(0.005, 2)
        ob = b.get_state_observables_into(pb, vb, None)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)
        assert np.array_equal(pc, pb) and np.array_equal(vc, vb)
        assert oa["U"] == ob["U"] == oc["U"] and oa["step"] == ob["step"] == oc["step"]
    fa = ljgb_mod.pinned((n, 3))
    a.step_io(0.005, 1, None, None, None, None, fa)
    b.integrate(0.005, 1)
    _, _, fb = b.get_state()
    assert np.array_equal(fa, fb)
    va[3, 2] = np.inf
    with pytest.raises(ljgb_mod.LJError, match="lj_set_state_async"):
        a.step_io(0.005, 1, pa, va, pa, va)
    a.integrate(0.005, 1)
    assert np.isfinite(a.observables()["U"])
    for s in (a, b, c):
        s.close()


def test_read_back_waits_for_its_own_launch(ljgb_mod):
    """A read-back into page-locked buffers waits on a completion word its
    launch writes after its last store.  Behind a long run of steps (here
    ~30 ms, past the word's 20 ms limit) the wait falls back to a stream
    synchronisation; a new handle whose page-locked mirrors come from memory
    an earlier handle used must not see that handle's words.  Both give what
    separate calls give, bit for bit."""
    n = 16384
    kw = dict(n=n, density=0.85, temperature=1.0, canonical=1, lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=4)
    a, b = ljgb_mod.System(**kw), ljgb_mod.System(**kw)
    pa, va = ljgb_mod.pinned((n, 3)), ljgb_mod.pinned((n, 3))
    a.get_state_into(pa, va, None)
    oa = a.step_io(0.005, 150, pa, va, pa, va)
    b.integrate(0.005, 150)
    pb, vb, _ = b.get_state()
    ob = b.observables()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    assert oa["U"] == ob["U"] and oa["step"] == ob["step"] == 150
    # short calls: the completion word itself
    for _ in range(3):
        oa = a.step_io(0.005, 1, pa, va, pa, va)
        b.integrate(0.005, 1)
        ob = b.get_state_observables_into(pb, vb, None)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb) and oa["U"] == ob["U"]
    a.close()
    b.close()
    # fresh handles, created and read one after another
    small = dict(n=700, density=0.6, temperature=1.1, canonical=0, lattice=ljgb_mod.LATTICE_FCC, jitter=0.02)
    for seed in range(4):
        c = ljgb_mod.System(seed=seed, **small)
        c.integrate(0.005, 3)
        oc = c.observables()
        d = ljgb_mod.System(seed=seed, **small)
        d.integrate(0.005, 3)
        d.sync()
        od = d.observables()
        assert oc["U"] == od["U"] and oc["step"] == od["step"] == 3, seed
        c.close()
        d.close()


def test_upload_writes_the_predictor(ljgb_mod):
    """On periodic boxes the upload's commit also writes the fused step's
    predictor, so the step after an upload launches no predictor kernel; a
    round trip of the state through host memory then leaves the trajectory
    bit-identical to a twin that never left the GPU."""
    kw = dict(n=1500, density=0.8, temperature=1.0, canonical=1, lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=3)
    a, b = ljgb_mod.System(**kw), ljgb_mod.System(**kw)
    a.integrate(0.005, 3)
    b.integrate(0.005, 3)
    for _ in range(4):
        p, v, _ = a.get_state()
        c0 = a.launch_count()
        a.set_state_async_from(p, v)
        a.integrate(0.005)
        b.integrate(0.005)
        a.sync()
        b.sync()
        # stage + commit, pairs + TVN close, the step's observables at the sync
        assert a.launch_count() - c0 == 2 + 2 + 1
    pa, va, fa = a.get_state()
    pb, vb, fb = b.get_state()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
    assert a.observables()["U"] == b.observables()["U"]
    a.close()
    b.close()


def test_walls_frame_follows_set_state(ljgb_mod):
    """A walled box's fixed frame is rebuilt around positions set from the
    host, even far outside the walls; the wall turns the particle back."""
    N, rho = 864, 0.5
    s = ljgb_mod.System(n=N, density=rho, temperature=1.0, boundary=1, lattice=ljgb_mod.LATTICE_FCC, jitter=0.02)
    p, v, _ = s.get_state()
    L = s.L
    p[11] = (L + 4.0, 0.5 * L, 0.5 * L)      # 4 sigma beyond the wall, moving away
    v[11] = (1.5, 0.0, 0.0)
    s.set_state(p, v)
    s.calculate_forces()
    s.integrate(0.005, 400)
    p1, v1, _ = s.get_state()
    assert p1[11, 0] < L + 4.0 + 0.05 and v1[11, 0] < 0
    assert np.all(p1 > -1.5) and np.all(p1 < L + 4.1)


def test_device_wait_limit_reports_and_recovers(ljgb_mod):
    """The pair kernels' bounded mbarrier wait, on a barrier nothing
    completes: it gives up after its 1.5 s limit, the host reports
    LJ_ERR_DEVICE_TIMEOUT (the self-test returns normally), and the same
    handle steps on.  No fault and no hang are involved."""
    import time
    s = ljgb_mod.System(n=500, density=0.8, temperature=1.0, canonical=1)
    s.integrate(0.005, 2)
    t0 = time.perf_counter()
    s.selftest_device_timeout()
    el = time.perf_counter() - t0
    assert 1.4 < el < 30
    s.integrate(0.005, 3)
    o = s.observables()
    assert o["step"] == 5 and np.isfinite(o["U"])


@pytest.mark.parametrize("canonical", [0, 1], ids=["evn", "tvn"])
def test_combined_state_observables_read(ljgb_mod, canonical):
    """lj_get_state_observables returns exactly what lj_get_state followed by
    lj_get_observables return, on a handle whose last steps left their
    observables pending (fused steps), after a state upload and a step."""
    N, rho, T0 = 1000, 0.8, 1.2
    pos, vel, L = U.lattice_state(N, rho, T0, "fcc", 0.02, seed=5)
    a = ljgb_mod.System(n=N, density=rho, temperature=T0, canonical=canonical)
    b = ljgb_mod.System(n=N, density=rho, temperature=T0, canonical=canonical)
    for s in (a, b):
        s.set_state(pos, vel)
        s.integrate(0.005, 3)
    pa, va, fa = (np.zeros((N, 3)) for _ in range(3))
    oa = a.get_state_observables_into(pa, va, fa)
    pb, vb, fb = b.get_state()
    ob = b.observables()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
    assert oa == ob
    # upload, one step, combined read: positions only, then nothing but the observables
    for s in (a, b):
        s.set_state_from(pa, va)
        s.integrate(0.005)
    p2 = np.zeros((N, 3))
    oa = a.get_state_observables_into(p2, None, None)
    pb, _, _ = b.get_state()
    ob = b.observables()
    assert np.array_equal(p2, pb) and oa == ob
    assert a.get_state_observables_into() == ob
    a.close()
    b.close()
