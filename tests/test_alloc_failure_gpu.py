"""Out-of-memory handling (GPU tests; no GPU fault is involved).

The reference aborts the process when a device allocation fails
(checkCudaErrors(cudaMalloc(...)), src/library/MDSystem.cu:167-173).  This
library returns LJ_ERR_OUT_OF_MEMORY and leaves the handle as it was.
lj_debug_fail_allocations(k) lets the next k allocations of the library
succeed and makes every later one fail on the host, without calling CUDA, so
each allocation of each entry point can be made to fail in turn.  After a
failure the handle must go on exactly as a twin that never saw one (same
schedule, same state: bit-identical trajectories), and a failed creation
must leave no device memory behind.
"""
import ctypes as C

import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu

OOM = 7      # LJ_ERR_OUT_OF_MEMORY
DT = 0.005


@pytest.fixture
def hook(ljlib):
    """lj_debug_fail_allocations, switched off again after the test."""
    yield ljlib.lj_debug_fail_allocations
    ljlib.lj_debug_fail_allocations(-1)


def _free_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _expect_oom(fn, *args):
    import ljgb
    with pytest.raises(ljgb.LJError) as e:
        fn(*args)
    assert e.value.code == OOM, str(e.value)


def _cfg(ljgb, n=1000, **kw):
    base = dict(n=n, density=0.8, temperature=1.0, canonical=1, lattice=ljgb.LATTICE_FCC, jitter=0.02, seed=7)
    base.update(kw)
    return ljgb.config(**base)


def _create_until_success(ljlib, hook, create, limit=200):
    """Runs create() with the k-th allocation failing, k = 0, 1, ..., until it
    succeeds; returns (number of failing k, the successful handle)."""
    k = 0
    while True:
        hook(k)
        rc, h = create()
        hook(-1)
        if rc == 0:
            return k, h
        assert rc == OOM, (k, rc)
        assert not h, "a failed creation returned a handle"
        k += 1
        assert k < limit


@pytest.mark.parametrize("nboxes", [1, 3])
def test_creation_fails_cleanly_at_every_allocation(ljgb_mod, ljlib, hook, nboxes):
    cfgs = [_cfg(ljgb_mod, n=600 + 150 * b, boundary=b % 2, seed=11 + b) for b in range(nboxes)]
    arr = (ljgb_mod.Config * nboxes)(*cfgs)

    def create():
        h = ljgb_mod._P()
        rc = ljlib.lj_batch_create(arr, nboxes, C.byref(h)) if nboxes > 1 else ljlib.lj_create(arr, C.byref(h))
        return rc, h.value

    # once without failures: lazy CUDA set-up and module loading happen here
    rc, h = create()
    assert rc == 0
    ljlib.lj_destroy(h)
    free0 = _free_bytes()
    fails, h = _create_until_success(ljlib, hook, create)
    ljlib.lj_destroy(h)
    free1 = _free_bytes()
    print("lj_%screate: %d allocations, each failed in turn; free device memory %+.1f MiB"
          % ("batch_" if nboxes > 1 else "", fails, (free1 - free0) / 2 ** 20))
    assert fails >= 15                                  # every buffer of the handle
    assert abs(free1 - free0) <= 8 << 20                # nothing left behind by the failures
    # and the library works as before
    s = ljgb_mod.System(batch=cfgs) if nboxes > 1 else ljgb_mod.System(cfg=cfgs[0])
    s.integrate(DT, 5)
    assert all(np.isfinite(o["U"]) for o in s.batch_observables())
    s.close()


def _twins(ljgb_mod, **kw):
    a = ljgb_mod.System(cfg=_cfg(ljgb_mod, **kw))
    b = ljgb_mod.System(cfg=_cfg(ljgb_mod, **kw))
    return a, b


def _same_trajectory(a, b, steps=10):
    a.integrate(DT, steps)
    b.integrate(DT, steps)
    pa, va, fa = a.get_state()
    pb, vb, fb = b.get_state()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
    assert a.observables()["U"] == b.observables()["U"]


def test_failed_schedule_rebuild_keeps_the_old_schedule(ljgb_mod, ljlib, hook):
    """lj_set_kernel_shape and lj_set_split_cap build a new work schedule
    (ten device tables): whichever allocation fails, the handle keeps its
    schedule, its shape and its split cap, and steps on bit-identically."""
    a, b = _twins(ljgb_mod, n=3000)
    info0 = a.tune_info()
    for k in (0, 1, 4, 9):
        hook(k)
        _expect_oom(a.set_kernel_shape, (info0["active"] + 1) % 6)
        hook(-1)
        hook(k)
        _expect_oom(a.set_split_cap, 3)
        hook(-1)
        info = a.tune_info()
        assert (info["active"], info["split_cap"], info["ctas"]) == (info0["active"], info0["split_cap"],
                                                                     info0["ctas"]), k
    _same_trajectory(a, b)
    shape0 = info0["active"]
    # the same calls succeed once allocations do
    a.set_kernel_shape((shape0 + 1) % 6)
    a.set_split_cap(3)
    a.integrate(DT, 3)
    assert np.isfinite(a.observables()["U"])
    a.close()
    b.close()


def test_failed_histogram_and_recording_setup_leave_the_handle_as_it_was(ljgb_mod, ljlib, hook):
    a, b = _twins(ljgb_mod, n=2000)
    a.set_recording(50)
    b.set_recording(50)
    a.integrate(DT, 20)
    b.integrate(DT, 20)
    want = b.rdf_counts(ljgb_mod.RDF_R_LINEAR, 120, 0.05)
    for k in (0, 2):
        hook(k)
        _expect_oom(a.rdf_counts, ljgb_mod.RDF_R_LINEAR, 120, 0.05)   # histogram range tables
        hook(-1)
    hook(0)
    _expect_oom(a.set_recording, 400)                                  # a larger record ring
    _expect_oom(a.rdf_accumulate, True, ljgb_mod.RDF_R_LINEAR, 100, 0.05)
    _expect_oom(a.counters_configure, [(0, 10, 0.1, 0.0)])
    _expect_oom(a.render, 0, 2, 64, 64)
    hook(-1)
    assert np.array_equal(a.rdf_counts(ljgb_mod.RDF_R_LINEAR, 120, 0.05), want)
    # the old record ring goes on recording; accumulation and counters are off
    _same_trajectory(a, b, steps=30)
    ra, rb = a.records(max_records=50), b.records(max_records=50)
    assert len(ra) == len(rb) == 50 and [r["U"] for r in ra] == [r["U"] for r in rb]
    with pytest.raises(ljgb_mod.LJError):
        a.rdf_accumulated()
    # and each succeeds once allocations do
    a.set_recording(400)
    a.rdf_accumulate(True, mode=ljgb_mod.RDF_R_LINEAR, nbins=100, width=0.05)
    a.integrate(DT, 4)
    c, ns = a.rdf_accumulated()
    assert ns == 4 and c.sum() > 0
    assert a.render(0, 2, 64, 64).shape == (64, 64, 4)
    a.close()
    b.close()


def test_failed_autotune_puts_the_state_back(ljgb_mod, ljlib, hook):
    """lj_autotune snapshots the state, then builds and times a schedule per
    shape and split cap.  A failure part-way returns the error with the
    state as it was before the call (and the handle stepping on)."""
    a = ljgb_mod.System(cfg=_cfg(ljgb_mod, n=2500))
    a.integrate(DT, 10)
    for k in (0, 3, 12, 30):
        p0, v0, _ = a.get_state()
        o0 = a.observables()
        hook(k)
        _expect_oom(a.autotune)
        hook(-1)
        p1, v1, _ = a.get_state()
        o1 = a.observables()
        assert np.array_equal(p0, p1) and np.array_equal(v0, v1), k
        assert o1["step"] == o0["step"] and o1["U"] == pytest.approx(o0["U"], rel=1e-12), k
        a.integrate(DT, 5)
        assert np.isfinite(a.observables()["U"])
    a.autotune()
    a.integrate(DT, 5)
    assert np.isfinite(a.observables()["U"])
    a.close()


def test_failed_adjoint_allocations(ljgb_mod, ljlib, hook):
    cfg = _cfg(ljgb_mod, n=256, canonical=0, density=0.85)

    def create():
        h = ljgb_mod._P()
        rc = ljlib.lj_adjoint_create(C.byref(cfg), 5, C.byref(h))
        return rc, h.value

    fails, h = _create_until_success(ljlib, hook, create)
    ljlib.lj_adjoint_destroy(h)
    assert fails >= 10
    adj = ljgb_mod.Adjoint(cfg=cfg, checkpoint_every=5)
    hook(0)
    _expect_oom(adj.forward, DT, 20)                 # checkpoints
    hook(-1)
    loss = adj.forward(DT, 20)
    assert np.isfinite(loss)
    d_eps, d_sigma, _, _ = adj.backward()
    assert np.isfinite(d_eps) and np.isfinite(d_sigma)
    adj.close()


def test_failed_reference_abi_allocations(ljlib, hook):
    """The reference ABI records the failure in its status word instead of
    exiting; calculateNForces builds its work context again on the next call."""
    n = 500
    pos, _, L = U.lattice_state(n, 0.8, 1.0, "fcc", 0.02, seed=3)
    p4 = np.zeros((n, 4), np.float32)
    p4[:, :3] = pos
    hook(0)
    d = C.c_void_p()
    ljlib.allocateArray(C.byref(d), n)
    assert ljlib.lj_reference_abi_status() == OOM
    hook(-1)
    d_pos, d_frc = C.c_void_p(), C.c_void_p()
    ljlib.allocateArray(C.byref(d_pos), n)
    ljlib.allocateArray(C.byref(d_frc), n)
    assert ljlib.lj_reference_abi_status() == 0
    ljlib.copyArrayToDevice(d_pos, p4.ctypes.data, n)
    pressure = C.c_float()
    for k in (0, 3, 8):
        ljlib.threadExit()                           # drop the cached work context: the call builds a new one
        hook(k)
        ljlib.calculateNForces(d_pos, d_frc, C.byref(pressure), n, C.c_float(L), 1, None, C.c_float(0.1), 128, 0)
        hook(-1)
        assert ljlib.lj_reference_abi_status() == OOM, k
    ljlib.calculateNForces(d_pos, d_frc, C.byref(pressure), n, C.c_float(L), 1, None, C.c_float(0.1), 128, 0)
    assert ljlib.lj_reference_abi_status() == 0
    f = np.zeros((n, 4), np.float32)
    ljlib.copyArrayFromDevice(f.ctypes.data, d_frc, 0, n)
    assert np.isfinite(f).all() and np.abs(f[:, :3]).max() > 0
    ljlib.deleteArray(d_pos)
    ljlib.deleteArray(d_frc)


def test_pinned_host_allocation_failure(ljlib, hook):
    hook(0)
    assert not ljlib.lj_host_alloc(4096)
    hook(-1)
    p = ljlib.lj_host_alloc(4096)
    assert p
    ljlib.lj_host_free(p)
