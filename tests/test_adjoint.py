"""Differentiable MD: the discrete adjoint of the EVN velocity-Verlet
trajectory loss (lj_adjoint_*, include/ljgb/Adjoint.hpp).

CPU: the numpy restatement of the forward pass and its adjoint recursion
(oracle/adjoint.py) against central finite differences, and the C++
Function API compiling against the library.  GPU: the CUDA adjoint against
the numpy adjoint (small N), against the FP64 lj_step trajectory, and the
differentiable-MD configuration -- N=2048, rho*=0.85, T*=1.0, dt=0.005,
200 EVN steps, checkpoints every 20, loss = <V/N + P> -- against FP64
central finite differences on eps, sigma and 32 seeded initial coordinates.
"""
import os
import subprocess

import numpy as np
import pytest

import lj_testutil as U

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _fd(f, h):
    return (f(h) - f(-h)) / (2 * h)


def test_oracle_adjoint_matches_finite_differences():
    import adjoint as A
    N, rho, dt, S = 108, 0.85, 0.005, 30
    pos, vel, _ = U.lattice_state(N, rho, 1.0, "fcc", 0.02, seed=5)
    rng = np.random.default_rng(0)
    for wts in [(0.0, 1.0, 1.0), (1.0, 0.0, 0.0), (0.3, 0.7, 0.2)]:
        t = A.Trajectory(pos, vel, rho, 1.0, 1.0, wts)
        t.forward(dt, S)
        de, ds, dx, dv = t.backward()
        # h small enough that no pair crosses the minimum-image switch at r = L/2
        # (a kink of the force) between the two evaluations
        h = 1e-6
        fe = _fd(lambda e: A.loss_of(pos, vel, rho, 1 + e, 1.0, dt, S, wts), h)
        fs = _fd(lambda e: A.loss_of(pos, vel, rho, 1.0, 1 + e, dt, S, wts), h)
        assert de == pytest.approx(fe, rel=1e-6, abs=1e-9)
        assert ds == pytest.approx(fs, rel=1e-6, abs=1e-9)
        for _ in range(3):
            i, c = int(rng.integers(N)), int(rng.integers(3))

            def lx(e):
                p = pos.copy()
                p[i, c] += e
                return A.loss_of(p, vel, rho, 1.0, 1.0, dt, S, wts)

            def lv(e):
                v = vel.copy()
                v[i, c] += e
                return A.loss_of(pos, v, rho, 1.0, 1.0, dt, S, wts)
            assert dx[i, c] == pytest.approx(_fd(lx, h), rel=1e-5, abs=1e-8)
            assert dv[i, c] == pytest.approx(_fd(lv, h), rel=1e-5, abs=1e-8)


def _build_driver(ljlib, tmp_path):
    exe = str(tmp_path / "adjoint_driver")
    libdir = os.path.dirname(ljlib._name)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                           os.path.join(REPO, "tests", "adjoint", "adjoint_driver.cpp"), "-o", exe,
                           "-L", libdir, "-llj_gb300", "-Wl,-rpath," + libdir])
    return exe


def test_function_api_compiles_and_links(ljlib, tmp_path):
    assert os.path.exists(_build_driver(ljlib, tmp_path))


def test_adjoint_rejects_unsupported_dynamics(ljgb_mod):
    with pytest.raises(ljgb_mod.LJError):
        ljgb_mod.Adjoint(n=64, boundary=1)       # walls: reflections are not differentiated
    with pytest.raises(ljgb_mod.LJError):
        ljgb_mod.Adjoint(n=64, canonical=1)      # TVN rescale is not differentiated
    with pytest.raises(ljgb_mod.LJError):
        ljgb_mod.Adjoint(n=64, checkpoint_every=0)


@pytest.mark.gpu
@pytest.mark.parametrize("every", [7, 40])
def test_gpu_adjoint_matches_oracle_adjoint(ljgb_mod, every):
    """Same loss and gradients as the numpy adjoint, for checkpoint intervals
    that split the 40 steps unevenly (7) and not at all (40)."""
    import adjoint as A
    N, rho, dt, S = 108, 0.85, 0.005, 40
    wts = (0.3, 0.7, 0.2)
    pos, vel, _ = U.lattice_state(N, rho, 1.0, "fcc", 0.02, seed=9)
    t = A.Trajectory(pos, vel, rho, 1.1, 0.95, wts)
    loss_ref = t.forward(dt, S)
    de_r, ds_r, dx_r, dv_r = t.backward()
    adj = ljgb_mod.Adjoint(n=N, density=rho, temperature=1.0, epsilon=1.1, sigma=0.95, checkpoint_every=every)
    adj.set_state(pos, vel)
    adj.set_loss(*wts)
    loss = adj.forward(dt, S)
    assert loss == pytest.approx(loss_ref, rel=1e-11)
    obs = adj.observables()
    K_r, V_r, W_r = (np.array([o[k] for o in t.obs]) for k in range(3))
    assert np.allclose(obs["K"], K_r, rtol=1e-11) and np.allclose(obs["V"], V_r, rtol=1e-11)
    assert np.allclose(obs["W"], W_r, rtol=1e-10)
    de, ds, dx, dv = adj.backward()
    assert de == pytest.approx(de_r, rel=1e-9)
    assert ds == pytest.approx(ds_r, rel=1e-9)
    assert np.abs(dx - dx_r).max() <= 1e-9 * np.abs(dx_r).max()
    assert np.abs(dv - dv_r).max() <= 1e-9 * np.abs(dv_r).max()
    # backward is repeatable and independent of the checkpoint interval
    de2, ds2, dx2, _ = adj.backward()
    assert (de2, ds2) == (de, ds) and np.array_equal(dx2, dx)


@pytest.mark.gpu
def test_gpu_adjoint_forward_is_the_fp64_step(ljgb_mod):
    """The adjoint's forward pass integrates the same trajectory as lj_step
    with LJ_PREC_FP64 (EVN, periodic): per-step K, V, W agree to rounding."""
    N, rho, dt, S = 500, 0.8, 0.005, 50
    pos, vel, _ = U.lattice_state(N, rho, 1.0, "fcc", 0.02, seed=4)
    s = ljgb_mod.System(n=N, density=rho, temperature=1.0, canonical=0, precision=ljgb_mod.PREC_FP64)
    s.set_state(pos, vel)
    s.calculate_forces()
    s.set_recording(S)
    s.integrate(dt, S)
    rec = s.records()
    adj = ljgb_mod.Adjoint(n=N, density=rho, temperature=1.0)
    adj.set_state(pos, vel)
    adj.forward(dt, S)
    obs = adj.observables()
    for key, arr in (("K", obs["K"]), ("V", obs["V"]), ("W", obs["W"])):
        ref = np.array([r[key] for r in rec])
        assert np.allclose(arr, ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max()), key


@pytest.mark.gpu
def test_function_api_runs(ljgb_mod, ljlib, tmp_path):
    """ljgb::TrajectoryLoss from C++: the same numbers as the Python binding
    of the same C ABI, and a finite difference along a random direction of
    one particle's initial position (N=2048, 20 steps)."""
    out = subprocess.run([_build_driver(ljlib, tmp_path), "2048"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = {}
    for line in out.stdout.splitlines():
        head, *kv = line.split()
        lines[head] = {k: float(v) for k, v in (x.split("=", 1) for x in kv)}
    a = ljgb_mod.Adjoint(n=2048, density=0.85, temperature=1.0, lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=7,
                         checkpoint_every=5)
    a.set_loss(0.0, 1.0, 1.0)
    loss = a.forward(0.005, 20)
    de, ds, dp, dv = a.backward()
    got = lines["adjoint"]
    assert (got["loss"], got["deps"], got["dsigma"], got["dpos0"], got["dvel0"]) == (loss, de, ds, dp[0, 0], dv[0, 0])
    d = lines["direction"]
    assert d["adj"] == pytest.approx(d["fd"], rel=1e-3), out.stdout


@pytest.mark.gpu
def test_differentiable_md_configuration(ljgb_mod):
    """N=2048, periodic, rho*=0.85, T*=1.0, dt=0.005, EVN, checkpoints every
    20 steps; loss = time-averaged V/N + P.  Adjoint gradients w.r.t. eps,
    sigma and 32 seeded initial coordinates against FP64 central differences.

    The all-pairs minimum-image model (no cutoff, MDSystem.cpp:264-300)
    switches a pair's image where its separation crosses L/2 and the force
    jumps there, so the loss is only piecewise smooth: a finite difference
    whose two runs put some pair on different sides of the switch at some
    step measures a slope that includes those jumps.  Such events grow with
    the length of the run and with the number of coordinates perturbed.  Over
    20 steps with one coordinate perturbed they are rare (agreement 1e-11 to
    1e-5); over the configuration's 200 steps (h = 1e-4) the finite
    differences themselves scatter by ~1e-3 with h, which sets the tolerance
    there.  Exactness of the adjoint itself is checked against the numpy
    adjoint (test_gpu_adjoint_matches_oracle_adjoint, 1e-9)."""
    N, rho, dt = 2048, 0.85, 0.005
    cfg = ljgb_mod.config(n=N, density=rho, temperature=1.0, canonical=0, lattice=ljgb_mod.LATTICE_FCC,
                          jitter=0.02, seed=2048)
    pos, vel = ljgb_mod.sample_initial_state(cfg)
    rng = np.random.default_rng(32)
    picks = [(int(i), int(c)) for i, c in zip(rng.choice(N, 32, replace=False), rng.integers(0, 3, 32))]

    def run(S, eps=1.0, sigma=1.0, p=pos):
        a = ljgb_mod.Adjoint(ljgb_mod.config(n=N, density=rho, temperature=1.0, canonical=0, epsilon=eps,
                                             sigma=sigma), checkpoint_every=20)
        a.set_state(p, vel)
        a.set_loss(0.0, 1.0, 1.0)
        return a, a.forward(dt, S)

    for S, h, tol, tol_x in ((200, 1e-4, 5e-3, 5e-3), (20, 1e-6, 5e-5, 2e-4)):
        adj, loss = run(S)
        de, ds, dx, _ = adj.backward()
        rows = [("eps", de, (run(S, eps=1 + h)[1] - run(S, eps=1 - h)[1]) / (2 * h)),
                ("sigma", ds, (run(S, sigma=1 + h)[1] - run(S, sigma=1 - h)[1]) / (2 * h))]
        for i, c in picks:
            p1 = pos.copy()
            p1[i, c] += h
            p2 = pos.copy()
            p2[i, c] -= h
            rows.append(("x[%d,%d]" % (i, c), dx[i, c], (run(S, p=p1)[1] - run(S, p=p2)[1]) / (2 * h)))
        gmax = np.abs(dx).max()
        print("S=%d h=%.0e loss %.12f max|dloss/dx0| %.3e" % (S, h, loss, gmax))
        for name, a, f in rows:
            print("  %-12s adjoint % .10e  fd % .10e  rel %.2e" % (name, a, f, abs(a - f) / max(abs(f), 1e-300)))
        for name, a, f in rows:
            bound = tol * abs(f) if name in ("eps", "sigma") else tol_x * gmax
            assert abs(a - f) <= bound, (S, name, a, f)
