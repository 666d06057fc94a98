"""RDF and velocity histograms (GPU tests): exact integer parity.

The device bins pairs from the fixed-point separation in FP32 and speeds in
FP64 with separately rounded operations; the oracle's emu_* functions repeat
that arithmetic on the CPU, so the counts must agree exactly.
"""
import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu


def k2_of(L, sigma=1.0):
    ks = L / (4294967296.0 * sigma)
    return np.float32(ks * ks)


@pytest.mark.parametrize("N,rho", [(400, 0.05), (2048, 0.85), (999, 0.5)])
def test_rdf_r2_counts_exact(ljgb_mod, oracle_mod, N, rho):
    pos, vel, L = U.lattice_state(N, rho, 1.0, "fcc", 0.05, seed=N)
    s = ljgb_mod.System(n=N, density=rho)
    s.set_state(pos, vel)
    dr2 = ljgb_mod.reference_rdf_dr2(N)
    q = oracle_mod.emu_fixed(pos, L)
    for mode in (0, 1):
        got = s.rdf_counts(mode, 256, dr2)
        want = oracle_mod.emu_rdf_r2(q, k2_of(L), np.float32(1.0 / dr2), 256, mode)
        assert np.array_equal(got, want), mode
    assert s.rdf_counts(0, 256, dr2).sum() == N * (N - 1)


@pytest.mark.parametrize("dr2", [0.1, 1.2])
def test_rdf_r2_large_box_clamp_dominant_or_rare(ljgb_mod, oracle_mod, dr2):
    """N=16384 over the whole persistent grid (ranges cut inside tiles): with
    dr2 = 0.1 about 97% of the pairs fall in the clamp bin, with dr2 = 1.2
    almost none; the last bin is counted per thread and added per warp."""
    N, rho = 16384, 0.85
    pos, vel, L = U.lattice_state(N, rho, 1.0, "fcc", 0.05, seed=7)
    s = ljgb_mod.System(n=N, density=rho)
    s.set_state(pos, vel)
    q = oracle_mod.emu_fixed(pos, L)
    for mode in (0, 1):
        got = s.rdf_counts(mode, 256, dr2)
        want = oracle_mod.emu_rdf_r2(q, k2_of(L), np.float32(1.0 / dr2), 256, mode)
        assert np.array_equal(got, want), mode
    assert got[:255].sum() <= N * (N - 1)
    s.close()


def test_rdf_counts_same_on_every_shape(ljgb_mod, oracle_mod):
    """The histogram pass cuts its own CTA ranges for the active shape's
    blocks and tiles; changing the shape (or the bin count) re-cuts them."""
    N, rho = 3000, 0.85
    pos, vel, L = U.lattice_state(N, rho, 1.0, "fcc", 0.05, seed=9)
    s = ljgb_mod.System(n=N, density=rho)
    s.set_state(pos, vel)
    q = oracle_mod.emu_fixed(pos, L)
    dr2 = ljgb_mod.reference_rdf_dr2(N)
    want0 = oracle_mod.emu_rdf_r2(q, k2_of(L), np.float32(1.0 / dr2), 256, 0)
    want_wide = oracle_mod.emu_rdf_r2(q, k2_of(L), np.float32(1.0 / 0.5), 64, 1)
    for shape in range(len(s.tune_info()["shapes"])):
        s.set_kernel_shape(shape)
        s.set_state(pos, vel)
        assert np.array_equal(s.rdf_counts(0, 256, dr2), want0), shape
        assert np.array_equal(s.rdf_counts(1, 64, 0.5), want_wide), shape
    s.close()


def test_rdf_linear_r_to_half_box(ljgb_mod, oracle_mod):
    """Config-1 output: a 200-bin RDF to r = L/2."""
    N, rho = 400, 0.05
    pos, vel, L = U.lattice_state(N, rho, 1.4, "sc", 0.05, seed=1)
    s = ljgb_mod.System(n=N, density=rho, temperature=1.4)
    s.set_state(pos, vel)
    dr = (L / 2) / 200
    got = s.rdf_counts(ljgb_mod.RDF_R_LINEAR, 200, dr)
    inv_dr = np.float32(1.0 / dr)
    rmax = 200 * dr
    want = oracle_mod.emu_rdf_r(oracle_mod.emu_fixed(pos, L), k2_of(L), inv_dr, np.float32(rmax * rmax), 200)
    assert np.array_equal(got, want)


def test_rdf_after_steps_and_fp64_handle(ljgb_mod, oracle_mod):
    N, rho = 1000, 0.7
    for prec in (0, 1):
        s = ljgb_mod.System(n=N, density=rho, temperature=1.0, precision=prec, lattice=1, jitter=0.02)
        s.integrate(0.005, 20)
        pos, _, _ = s.get_state()
        dr2 = ljgb_mod.reference_rdf_dr2(N)
        got = s.rdf_counts(0, 256, dr2)
        want = oracle_mod.emu_rdf_r2(oracle_mod.emu_fixed(pos, s.L), k2_of(s.L), np.float32(1.0 / dr2), 256, 0)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("N", [100, 4000])
def test_velocity_counts_exact(ljgb_mod, oracle_mod, N):
    s = ljgb_mod.System(n=N, density=0.5, temperature=1.7, seed=N)
    s.integrate(0.005, 5)
    _, vel, _ = s.get_state()
    for step, nb in ((0.12, 101), (0.05, 300)):
        got = s.velocity_counts(step, nb)
        want = oracle_mod.emu_velocity_counts(vel, step, nb)
        assert np.array_equal(got, want)


def test_histogram_argument_checks(ljgb_mod):
    s = ljgb_mod.System(n=64, density=0.5)
    with pytest.raises(ljgb_mod.LJError):
        s.rdf_counts(0, 0, 0.1)
    with pytest.raises(ljgb_mod.LJError):
        s.rdf_counts(0, 100000, 0.1)
    with pytest.raises(ljgb_mod.LJError):
        s.velocity_counts(-1.0, 10)
