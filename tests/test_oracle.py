"""The CPU oracle pinned against the reference (CPU-only tests).

The golden fixtures were produced by the reference's own MDSystem.cpp
(tests/golden/make_golden.py).  The faithful float-storage restatement
(oracle R32System) must reproduce them bit for bit; the FP64 restatement must
agree within the reference's float-storage error; analytic known answers pin
the physics independently of both.
"""
import os

import numpy as np
import pytest

import lj_testutil as U

GOLDEN = U.golden_states()
SCALARS = ("U", "T", "K", "V", "P", "Pshear", "t", "L", "av_U", "av_T", "av_p", "av_iters", "rdf_dr2")


def load_case(path):
    return dict(np.load(path))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_r32_port_matches_reference_bit_for_bit(path, oracle_mod):
    g = load_case(path)
    N, rho, T0 = int(g["N"]), float(g["rho"]), float(g["T0"])
    r = oracle_mod.R32System(N, T0, rho, bool(g["canonical"]), int(g["bc"]), g["pos0"], g["vel0"])
    r.calculate_forces()
    r.calculate_parameters()
    assert np.array_equal(r.frc[:, :3], g["frc0"][:, :3])
    sc = r.scalars()
    for k, want in zip(SCALARS, g["scalars0"]):
        if k in ("U", "T", "K", "V", "P", "Pshear", "L", "rdf_dr2"):
            assert sc[k] == want, k
    assert np.array_equal(r.rdf_counts(), g["rdf0"])
    # initvelo (MDSystem.cpp:651-669): dens / step / N at step*(0.5+i)
    counts = r.velocity_counts(0.12, 101)
    assert np.array_equal(counts / 0.12 / N, g["velo_y"])
    dt, every = float(g["dt"]), int(g["every"])
    for k in range(g["traj_pos"].shape[0]):
        for _ in range(every):
            r.integrate(dt)
        assert np.array_equal(r.pos[:, :3], g["traj_pos"][k][:, :3]), "pos at record %d" % k
        assert np.array_equal(r.vel[:, :3], g["traj_vel"][k][:, :3]), "vel at record %d" % k
        assert np.array_equal(r.frc[:, :3], g["traj_frc"][k][:, :3]), "frc at record %d" % k
        assert np.array_equal(r.rdf_counts(), g["traj_rdf"][k])
        sc = r.scalars()
        for name, want in zip(SCALARS, g["traj_scalars"][k]):
            assert sc[name] == want, (name, k)


@pytest.mark.parametrize("path", GOLDEN[:2], ids=lambda p: os.path.basename(p)[:-4])
def test_r32_threaded_forces_identical(path, oracle_mod):
    g = load_case(path)
    r = oracle_mod.R32System(int(g["N"]), float(g["T0"]), float(g["rho"]), bool(g["canonical"]),
                             int(g["bc"]), g["pos0"], g["vel0"])
    r.calculate_forces(nthreads=4)
    assert np.array_equal(r.frc[:, :3], g["frc0"][:, :3])
    assert np.array_equal(r.rdf_counts(), g["rdf0"])
    assert r.scalars()["V"] == pytest.approx(g["scalars0"][3], rel=1e-13)


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_f64_oracle_agrees_with_reference_within_float_storage(path, oracle_mod):
    g = load_case(path)
    N, rho = int(g["N"]), float(g["rho"])
    L = (N / rho) ** (1.0 / 3.0)
    pos = g["pos0"][:, :3].astype(np.float64)
    r = oracle_mod.f64_forces(pos, L, periodic=int(g["bc"]) == 0, nthreads=2)
    Fref = g["frc0"][:, :3].astype(np.float64)
    rms = np.sqrt(np.mean(np.sum(r["F"] ** 2, 1)))
    err = np.linalg.norm(r["F"] - Fref, axis=1) / rms
    # the reference stores positions/forces as float: its own error vs FP64
    assert err.max() < 2e-4
    V_ref, P_ref = g["scalars0"][3], g["scalars0"][4]
    assert r["V"] == pytest.approx(V_ref, rel=1e-6, abs=1e-6)
    # P after CalculateParameters = (W/6 + N T) / (N / rho)
    T = g["scalars0"][1]
    P = (r["W"] / 6.0 + N * T) / (N / rho)
    assert P == pytest.approx(P_ref, rel=1e-5, abs=1e-6)


def test_known_answers_two_body(oracle_mod):
    L = 50.0
    rmin = 2.0 ** (1.0 / 6.0)
    pos = np.array([[10.0, 10.0, 10.0], [10.0 + rmin, 10.0, 10.0]])
    r = oracle_mod.f64_forces(pos, L, True)
    assert r["V"] == pytest.approx(-1.0, abs=1e-14)
    assert np.abs(r["F"]).max() < 1e-13
    pos[1, 0] = 11.0
    r = oracle_mod.f64_forces(pos, L, True)
    assert r["V"] == pytest.approx(0.0, abs=1e-14)
    assert r["F"][0, 0] == pytest.approx(-24.0, abs=1e-12)   # pushed away from particle 1
    assert r["F"][1, 0] == pytest.approx(24.0, abs=1e-12)
    # virial sum over ordered pairs: 2 * r f = 2 * 24
    assert r["W"] == pytest.approx(48.0, abs=1e-11)


def test_known_answer_minimum_image_and_scaling(oracle_mod):
    L = 10.0
    pos = np.array([[0.4, 5.0, 5.0], [L - 0.6, 5.0, 5.0]])   # separated by 1.0 through the wall
    r = oracle_mod.f64_forces(pos, L, True)
    assert r["V"] == pytest.approx(0.0, abs=1e-13)
    assert r["F"][0, 0] == pytest.approx(24.0, abs=1e-10)   # image of 1 sits at x = -0.6
    r_open = oracle_mod.f64_forces(pos, L, False)          # no minimum image without PBC
    assert abs(r_open["F"][0, 0]) < 1e-3
    # eps, sigma: u(r) = 4 eps [(s/r)^12 - (s/r)^6] at r = s
    pos2 = np.array([[1.0, 1.0, 1.0], [1.0, 1.0, 3.0]])
    r2 = oracle_mod.f64_forces(pos2, 100.0, True, eps=3.0, sigma=2.0)
    assert r2["V"] == pytest.approx(0.0, abs=1e-13)
    assert r2["F"][0, 2] == pytest.approx(-24.0 * 3.0 / 2.0, abs=1e-12)


def test_f64_integrator_conserves_energy_and_momentum(oracle_mod):
    g = load_case(GOLDEN[0])
    N, rho = int(g["N"]), float(g["rho"])
    L = (N / rho) ** (1.0 / 3.0)
    s = oracle_mod.F64System(g["pos0"][:, :3], g["vel0"][:, :3], L, rho, float(g["T0"]), False, 0, nthreads=2)
    U0 = s.U
    p0 = s.vel.sum(0)
    for _ in range(50):
        s.step(0.002)
    assert abs(s.U - U0) / N < 1e-4
    assert np.abs(s.vel.sum(0) - p0).max() < 1e-10


def test_f64_tvn_holds_kinetic_temperature(oracle_mod):
    g = load_case(GOLDEN[1])
    N, rho, T0 = int(g["N"]), float(g["rho"]), float(g["T0"])
    L = (N / rho) ** (1.0 / 3.0)
    s = oracle_mod.F64System(g["pos0"][:, :3], g["vel0"][:, :3], L, rho, T0, True, 0, nthreads=2)
    for _ in range(5):
        s.step(0.005)
    # v_new = (2chi-1) v + chi dt tF = chi tv + (chi-1)(v - ...) -> T stays within O(dt^2) of T0
    assert abs(s.T - T0) < 0.05


def test_wall_reflection_rule(oracle_mod):
    # A particle outside [0, L] moving outwards is reflected; one moving inwards is not.
    L = 5.0
    pos = np.array([[-0.1, 2.0, 2.0], [5.1, 2.0, 2.0]])
    vel = np.array([[-1.0, 0.0, 0.0], [-1.0, 0.0, 0.0]])
    s = oracle_mod.F64System(pos, vel, L, 2 / L ** 3, 1.0, False, 1, nthreads=1)
    s.pos, s.vel = pos.copy(), vel.copy()
    s.boundary()
    assert s.vel[0, 0] == 1.0 and s.vel[1, 0] == -1.0


def test_emulated_rdf_matches_numpy(oracle_mod):
    rng = np.random.default_rng(7)
    N, L = 300, 9.0
    pos = rng.uniform(0, L, (N, 3))
    q = oracle_mod.emu_fixed(pos, L)
    k2 = np.float32((L / 4294967296.0) ** 2)
    inv_dr2 = np.float32(1.0 / 0.1)
    counts = oracle_mod.emu_rdf_r2(q, k2, inv_dr2, 256, mode=0, nthreads=2)
    assert counts.sum() == N * (N - 1)
    # float64 minimum-image distances put almost every pair in the same bin
    d = pos[:, None, :] - pos[None, :, :]
    d -= L * np.round(d / L)
    r2 = np.sum(d * d, -1)[~np.eye(N, dtype=bool)]
    b = np.minimum(np.floor(r2 / 0.1), 255).astype(int)
    ref = np.bincount(b, minlength=256)
    assert np.abs(ref - counts.astype(np.int64)).sum() <= 4
    drop = oracle_mod.emu_rdf_r2(q, k2, inv_dr2, 256, mode=1, nthreads=2)
    assert np.array_equal(drop[:255], counts[:255]) and drop.sum() <= counts.sum()


def test_emulated_velocity_histogram(oracle_mod):
    rng = np.random.default_rng(3)
    vel = rng.normal(0, 1.2, (1000, 3))
    c = oracle_mod.emu_velocity_counts(vel, 0.12, 101)
    ref = np.bincount(np.floor(np.sqrt(np.sum(vel * vel, 1)) / 0.12).astype(int), minlength=200)[:101]
    assert np.array_equal(c.astype(np.int64), ref)


@pytest.mark.parametrize("n,rho,T0,lattice,jitter,seed", [(16384, 0.85, 1.0, 1, 0.02, 2), (400, 0.05, 1.4, 0, 0.05, 400),
                                                          (262144, 1.1, 1.0, 1, 0.01, 262144), (1000, 0.3, 2.0, 0, 0.0, 9)])
def test_oracle_initial_state_is_the_library_sampler(ljlib, n, rho, T0, lattice, jitter, seed):
    """oracle.sample_state (the CPU baseline's start, drawn without loading
    the product library) gives the state lj_sample_initial_state draws."""
    import ljgb
    import oracle
    cfg = ljgb.config(n=n, density=rho, temperature=T0, lattice=lattice, jitter=jitter, seed=seed)
    p, v = ljgb.sample_initial_state(cfg)
    po, vo, L = oracle.sample_state(n, rho, T0, lattice, jitter, seed)
    assert L == pytest.approx((n / rho) ** (1 / 3), rel=1e-14)
    # identical draws; the last bits may differ where a compiler contracts a
    # multiply-add on one side only
    assert np.abs(p - po).max() <= 1e-12 * L
    assert np.abs(v - vo).max() <= 1e-12
