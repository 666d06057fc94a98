"""lj_forces_static: the force entry point that allocates nothing.

Callers that cannot allocate device memory pass only their device input and
output arrays; the library keeps every intermediate in one fixed __device__
array.  This file is collected last so that, if it fails, a run stopping at
the first failure has already run every other test.  It must pass both alone
in a fresh process and after the other tests (which leave the array holding
another call's contents, or none).
"""
import ctypes as C
import os

import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu

GOLDEN = U.golden_states()


def bind(lib):
    f = lib.lj_forces_static
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.c_int32, C.c_void_p]
    return f


def device_array(lib, n):
    p = C.c_void_p()
    lib.allocateArray(C.byref(p), n)
    assert lib.lj_reference_abi_status() == 0
    return p


def run_existing(lib, d_pos, n, box, periodic):
    """The existing entry point: calculateNForces (the reference's ABI)."""
    d_frc = device_array(lib, n)
    pressure = C.c_float(0)
    lib.calculateNForces(d_pos, d_frc, C.byref(pressure), n, C.c_float(box), int(periodic), None, C.c_float(0.1),
                         128, 1)
    assert lib.lj_reference_abi_status() == 0, lib.lj_reference_abi_error()
    f = np.zeros((n, 4), np.float32)
    lib.copyArrayFromDevice(f.ctypes.data, d_frc, 0, n)
    lib.deleteArray(d_frc)
    return f, pressure.value


def run_static(lib, fn, d_pos, n, box, periodic):
    d_frc = device_array(lib, n)
    sums = np.zeros(2)
    rc = fn(d_pos, d_frc, sums.ctypes.data, n, C.c_float(box), int(periodic), None)
    f = np.zeros((n, 4), np.float32)
    lib.copyArrayFromDevice(f.ctypes.data, d_frc, 0, n)
    lib.deleteArray(d_frc)
    return rc, f, sums


def compare(f_static, f_ref, sums, pressure):
    mag = np.linalg.norm(f_ref[:, :3].astype(np.float64), axis=1)
    rms = np.sqrt(np.mean(mag ** 2))
    d = np.linalg.norm(f_static[:, :3].astype(np.float64) - f_ref[:, :3], axis=1)
    assert (d / np.maximum(mag, rms)).max() <= 1e-5          # the suite's force tolerance
    w = f_ref[:, 3].astype(np.float64)
    assert np.abs(f_static[:, 3] - w).max() <= 1e-5 * np.abs(w).max()
    assert sums[1] / 6.0 == pytest.approx(pressure, rel=1e-5)  # calculateNForces' pressure = W / 6
    assert sums[0] == pytest.approx(2.0 * w.sum(), rel=1e-5, abs=1e-4)


def test_static_matches_existing_entry_point_twice(ljlib):
    fn = bind(ljlib)
    cases = []
    for path in GOLDEN[:2]:
        g = dict(np.load(path))
        n, rho, bc = int(g["N"]), float(g["rho"]), int(g["bc"])
        cases.append((np.ascontiguousarray(g["pos0"], np.float32), n, np.float32((n / rho) ** (1 / 3)), bc == 0))
    # two calls in a row with different inputs, then the first again: the
    # array keeps the previous call's contents and must not leak into a result
    for pos4, n, box, periodic in cases + cases[:1]:
        d_pos = device_array(ljlib, n)
        ljlib.copyArrayToDevice(d_pos, pos4.ctypes.data, n)
        f_ref, pressure = run_existing(ljlib, d_pos, n, box, periodic)
        rc, f_static, sums = run_static(ljlib, fn, d_pos, n, box, periodic)
        assert rc == 0
        compare(f_static, f_ref, sums, pressure)
        ljlib.deleteArray(d_pos)


def test_static_dense_box_two_calls(ljlib):
    fn = bind(ljlib)
    n = 4000
    pos, _, L = U.lattice_state(n, 0.85, 1.0, "fcc", 0.02, seed=11)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos
    d_pos = device_array(ljlib, n)
    ljlib.copyArrayToDevice(d_pos, pos4.ctypes.data, n)
    f_ref, pressure = run_existing(ljlib, d_pos, n, np.float32(L), True)
    for _ in range(2):
        rc, f_static, sums = run_static(ljlib, fn, d_pos, n, np.float32(L), True)
        assert rc == 0
        compare(f_static, f_ref, sums, pressure)
    ljlib.deleteArray(d_pos)


@pytest.mark.parametrize("n", [16384, 16383])
def test_static_at_the_size_limit_against_fp64_oracle(ljlib, oracle_mod, n):
    """At the documented maximum (and one below, a ragged last i-block) the
    scratch regions are fullest.  Two calls in a row against calculateNForces
    and, on a seeded subset of 2048 rows, against the FP64 oracle on the same
    float positions (force gate |dF_i| <= 1e-5 max(|F_i|, rms|F|), median
    |dF_i|/|F_i| <= 1e-5; sum_j (r^-12 - r^-6) to 1e-5 of its largest)."""
    fn = bind(ljlib)
    pos, _, L = U.lattice_state(n, 0.85, 1.0, "fcc", 0.02, seed=n)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos
    box = np.float32(L)
    d_pos = device_array(ljlib, n)
    ljlib.copyArrayToDevice(d_pos, pos4.ctypes.data, n)
    f_ref, pressure = run_existing(ljlib, d_pos, n, box, True)
    i0 = int(np.random.default_rng(n).integers(0, n - 2048))
    r = oracle_mod.f64_forces(pos4[:, :3].astype(np.float64), float(box), True, rows=(i0, i0 + 2048))
    for _ in range(2):
        rc, f_static, sums = run_static(ljlib, fn, d_pos, n, box, True)
        assert rc == 0
        compare(f_static, f_ref, sums, pressure)
        err = U.force_errors(f_static[i0:i0 + 2048, :3].astype(np.float64), r["F"])
        print("lj_forces_static n=%d rows %d..%d vs FP64 oracle: %s" % (n, i0, i0 + 2048, err))
        assert err["gate_max"] <= 1e-5 and err["rel_median"] <= 1e-5
        # Force.w = sum_j (r^-12 - r^-6); the oracle's e_i = 4 sum_j (r^-12 - r^-6)
        w = f_static[i0:i0 + 2048, 3].astype(np.float64)
        assert np.abs(4.0 * w - r["e"]).max() <= 1e-5 * np.abs(r["e"]).max()
    ljlib.deleteArray(d_pos)


def test_static_rejects_a_capturing_stream(ljlib):
    """Each call reads its results back and synchronises its stream, which a
    stream capture cannot hold: on a capturing stream the call returns
    LJ_ERR_UNSUPPORTED and enqueues nothing, so the caller's capture stays
    valid."""
    torch = pytest.importorskip("torch")
    fn = bind(ljlib)
    n = 256
    d_pos, d_frc = device_array(ljlib, n), device_array(ljlib, n)
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    x = torch.zeros(4, device="cuda")
    with torch.cuda.graph(g, stream=side):
        rc = fn(d_pos, d_frc, None, n, C.c_float(10.0), 1, C.c_void_p(side.cuda_stream))
        x += 1.0
    assert rc == 6  # LJ_ERR_UNSUPPORTED
    g.replay()
    torch.cuda.synchronize()
    assert float(x.sum()) == 4.0
    ljlib.deleteArray(d_pos)
    ljlib.deleteArray(d_frc)


def test_static_works_while_every_allocation_fails(ljlib):
    """With the library's allocation hook refusing every device and host
    allocation (lj_debug_fail_allocations(0)), the entry point still works:
    it allocates nothing."""
    fn = bind(ljlib)
    n = 1500
    pos, _, L = U.lattice_state(n, 0.8, 1.0, "fcc", 0.02, seed=21)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos
    d_pos, d_frc = device_array(ljlib, n), device_array(ljlib, n)
    ljlib.copyArrayToDevice(d_pos, pos4.ctypes.data, n)
    f_ref, pressure = run_existing(ljlib, d_pos, n, np.float32(L), True)
    ljlib.lj_debug_fail_allocations(0)
    try:
        for _ in range(2):
            sums = np.zeros(2)
            assert fn(d_pos, d_frc, sums.ctypes.data, n, C.c_float(L), 1, None) == 0
    finally:
        ljlib.lj_debug_fail_allocations(-1)
    f = np.zeros((n, 4), np.float32)
    ljlib.copyArrayFromDevice(f.ctypes.data, d_frc, 0, n)
    compare(f, f_ref, sums, pressure)
    ljlib.deleteArray(d_pos)
    ljlib.deleteArray(d_frc)


def test_static_rejects_oversized_box(ljlib):
    fn = bind(ljlib)
    d = device_array(ljlib, 4)
    rc = fn(d, d, None, 16385, C.c_float(30.0), 1, None)
    assert rc == 1  # LJ_ERR_INVALID, nothing launched
    ljlib.deleteArray(d)
