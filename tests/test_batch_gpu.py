"""Batched replicas (GPU tests): many independent boxes with uneven N, rho*,
T* and boundaries advanced together -- one persistent pair launch per step
covers every box.  Each box must evolve exactly as it would alone (same
initial state from the same config, same equations), up to the summation
order of the FP32 pair sums, and as the FP64 oracle steps it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_cfgs(ljgb, k, seed=3, canonical=1, n_range=(200, 1500), bc_mix=True):
    rng = np.random.default_rng(seed)
    cfgs = []
    for i in range(k):
        cfgs.append(ljgb.config(n=int(rng.integers(*n_range)), density=float(rng.uniform(0.05, 1.0)),
                                temperature=float(rng.uniform(0.7, 2.0)), canonical=canonical,
                                boundary=(i % 2) if bc_mix else 0, lattice=ljgb.LATTICE_FCC, jitter=0.02,
                                seed=100 + i))
    return cfgs


@pytest.mark.parametrize("canonical", [1, 0], ids=["tvn", "evn"])
def test_batch_matches_individual_boxes(ljgb_mod, canonical):
    cfgs = make_cfgs(ljgb_mod, 8, canonical=canonical)
    b = ljgb_mod.System(batch=cfgs)
    assert b.nsys == 8
    b.integrate(0.004, 20)
    pb, vb, _ = b.get_state()
    ob = b.batch_observables()
    for k, c in enumerate(cfgs):
        s = ljgb_mod.System(cfg=c)
        s.integrate(0.004, 20)
        p, v, _ = s.get_state()
        o = s.observables()
        sl = slice(b.offsets[k], b.offsets[k + 1])
        assert np.abs(pb[sl] - p).max() < 1e-6 * s.L, k
        assert np.abs(vb[sl] - v).max() < 1e-5, k
        for key in ("K", "V", "T", "P", "U", "t"):
            assert ob[k][key] == pytest.approx(o[key], rel=1e-6, abs=1e-6), (k, key)
        assert ob[k]["step"] == 20


@pytest.mark.parametrize("canonical", [1, 0], ids=["tvn", "evn"])
def test_batch_boxes_match_fp64_oracle(ljgb_mod, oracle_mod, canonical):
    """Each box of a batch (uneven N, rho*, T*, periodic and hard-wall boxes)
    against the FP64 oracle restatement of the reference's step, directly:
    20 steps of dt 0.004 from the batch's own initial state."""
    cfgs = make_cfgs(ljgb_mod, 6, seed=17, canonical=canonical, n_range=(200, 900))
    b = ljgb_mod.System(batch=cfgs)
    p0, v0, _ = b.get_state()
    oracles = []
    for k, c in enumerate(cfgs):
        sl = slice(b.offsets[k], b.offsets[k + 1])
        L = (c.n / c.density) ** (1 / 3)
        oracles.append(oracle_mod.F64System(p0[sl], v0[sl], L, c.density, c.temperature, bool(canonical),
                                            c.boundary, nthreads=4))
    steps = 20
    b.integrate(0.004, steps)
    for o in oracles:
        for _ in range(steps):
            o.step(0.004)
    p, v, _ = b.get_state()
    obs = b.batch_observables()
    for k, (c, o) in enumerate(zip(cfgs, oracles)):
        sl = slice(b.offsets[k], b.offsets[k + 1])
        L = (c.n / c.density) ** (1 / 3)
        assert np.abs(p[sl] - o.pos).max() < 1e-6 * max(1.0, L), k
        assert np.abs(v[sl] - o.vel).max() < 1e-5, k
        for key in ("K", "V", "T", "P", "U"):
            assert obs[k][key] == pytest.approx(getattr(o, key), rel=1e-5, abs=1e-5 * c.n), (k, key)
        assert obs[k]["step"] == steps


def test_batch_periodic_only_uses_fused_step(ljgb_mod):
    cfgs = make_cfgs(ljgb_mod, 6, bc_mix=False)
    b = ljgb_mod.System(batch=cfgs)
    c0 = b.launch_count()
    b.integrate(0.004, 10)
    b.sync()
    # predictor, then pairs + TVN close per step, and the last step's
    # observables (k_obs_finalize) at the sync
    assert b.launch_count() - c0 == 1 + 2 * 10 + 1
    ob = b.batch_observables()
    for k, c in enumerate(cfgs):
        s = ljgb_mod.System(cfg=c)
        s.integrate(0.004, 10)
        assert ob[k]["U"] == pytest.approx(s.observables()["U"], rel=1e-6, abs=1e-6)


def test_batch_256_replicas_run(ljgb_mod):
    """The replica configuration's shape: 256 boxes, N in [200, 4000),
    rho* in [0.01, 1.1], T* in [0.7, 2.0], half periodic, half walls, TVN."""
    rng = np.random.default_rng(3)
    cfgs = [ljgb_mod.config(n=int(rng.integers(200, 4000)), density=float(rng.uniform(0.01, 1.1)),
                            temperature=float(rng.uniform(0.7, 2.0)), canonical=1, boundary=i % 2,
                            lattice=ljgb_mod.LATTICE_FCC, jitter=0.02, seed=1000 + i) for i in range(256)]
    b = ljgb_mod.System(batch=cfgs)
    b.autotune()
    b.integrate(0.004, 20)
    obs = b.batch_observables()
    assert len(obs) == 256
    for c, o in zip(cfgs, obs):
        assert np.isfinite(o["U"]) and o["step"] == 20
        # TVN keeps the kinetic temperature of the half-kicked velocities at T0
        assert o["Tkin_tvn"] > 0
        assert abs(o["T"] - c.temperature) < 0.25 * c.temperature
    p, _, _ = b.get_state()
    for k in range(256):
        L = (cfgs[k].n / cfgs[k].density) ** (1 / 3)
        pk = p[b.offsets[k]:b.offsets[k + 1]]
        assert pk.min() > -1.0 and pk.max() < L + 1.0


def test_batch_rejects_mixed_ensembles(ljgb_mod):
    cfgs = make_cfgs(ljgb_mod, 2)
    cfgs[1].canonical = 0
    with pytest.raises(ljgb_mod.LJError):
        ljgb_mod.System(batch=cfgs)
