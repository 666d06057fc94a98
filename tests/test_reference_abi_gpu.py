"""The reference's own extern "C" entry points (MDSystem.cu:155-299) served by
this library (GPU tests): the call sequence MDSystem::CalculateForces makes
in GPU mode (MDSystem.cpp:240-251), on the golden states."""
import ctypes as C
import os

import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu

GOLDEN = U.golden_states()


def calculate_n_forces(L, pos4, box, periodic, dr2, block=256):
    n = pos4.shape[0]
    d_pos, d_frc = C.c_void_p(), C.c_void_p()
    L.allocateArray(C.byref(d_pos), n)
    L.allocateArray(C.byref(d_frc), n)
    assert L.lj_reference_abi_status() == 0
    p = np.ascontiguousarray(pos4, np.float32)
    L.copyArrayToDevice(d_pos, p.ctypes.data, n)
    pressure = C.c_float(0)
    rdf = np.zeros(256, np.int32)
    L.calculateNForces(d_pos, d_frc, C.byref(pressure), n, C.c_float(box), int(periodic), rdf.ctypes.data,
                       C.c_float(dr2), block, 1)
    assert L.lj_reference_abi_status() == 0, L.lj_reference_abi_error()
    f = np.zeros((n, 4), np.float32)
    L.copyArrayFromDevice(f.ctypes.data, d_frc, 0, n)
    L.deleteArray(d_pos)
    L.deleteArray(d_frc)
    return f, pressure.value, rdf


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_calculate_n_forces_matches_reference(ljlib, oracle_mod, path):
    g = dict(np.load(path))
    N, rho, bc = int(g["N"]), float(g["rho"]), int(g["bc"])
    L = (N / rho) ** (1.0 / 3.0)
    dr2 = float(g["scalars0"][-1])
    f, pressure, rdf = calculate_n_forces(ljlib, g["pos0"], np.float32(L), bc == 0, dr2)
    # vs the FP64 oracle at the same (float) positions
    pos = g["pos0"][:, :3].astype(np.float64)
    r = oracle_mod.f64_forces(pos, float(np.float32(L)), bc == 0)
    rms = np.sqrt(np.mean(np.sum(r["F"] ** 2, 1)))
    assert (np.linalg.norm(f[:, :3] - r["F"], axis=1) / rms).max() < 1e-5
    # Force.w = sum_j (r^-12 - r^-6), V = 2 sum_i Force.w (MDSystem.cpp:340-346)
    assert 2.0 * f[:, 3].astype(np.float64).sum() == pytest.approx(r["V"], rel=1e-5, abs=1e-4)
    # pressure = virial part, W / 6
    assert pressure == pytest.approx(r["W"] / 6.0, rel=1e-5, abs=1e-4)
    # the reference's float CPU path agrees within its float storage
    Fref = g["frc0"][:, :3].astype(np.float64)
    assert (np.linalg.norm(f[:, :3] - Fref, axis=1) / rms).max() < 2e-4
    # RDF: 256 r^2 bins, overflow in the last bin; totals are exact, bins can
    # move across a bin edge only for pairs whose r^2 rounds differently.
    assert rdf.sum() == N * (N - 1)
    ref_rdf = g["rdf0"].astype(np.int64)
    inside = ref_rdf[:255].sum()
    assert np.abs(rdf[:255] - ref_rdf[:255]).sum() <= max(4, 1e-4 * inside)


def test_threadexit_releases_and_recovers(ljlib):
    g = dict(np.load(GOLDEN[0]))
    N, rho = int(g["N"]), float(g["rho"])
    L = (N / rho) ** (1.0 / 3.0)
    f1, p1, _ = calculate_n_forces(ljlib, g["pos0"], np.float32(L), True, 0.1)
    ljlib.threadExit()
    assert ljlib.lj_reference_abi_status() == 0
    f2, p2, _ = calculate_n_forces(ljlib, g["pos0"], np.float32(L), True, 0.1, block=64)
    assert np.abs(f1 - f2).max() <= 1e-5 * np.abs(f1).max()
    assert p1 == pytest.approx(p2, rel=1e-6)


def test_bad_arguments_do_not_exit(ljlib):
    pressure = C.c_float(0)
    ljlib.calculateNForces(None, None, C.byref(pressure), 1, C.c_float(1.0), 1, None, C.c_float(0.1), 256, 1)
    assert ljlib.lj_reference_abi_status() != 0
