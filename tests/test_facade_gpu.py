"""The MDSystem C++ class (include/ljgb/MDSystem.hpp) used the way the
reference's task drivers use it: compiled against the header and linked to
liblj_gb300.so (CPU: compile/link; GPU: run and check the physics)."""
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "facade", "facade_driver.cpp")


def build_driver(ljlib, tmp_path):
    exe = str(tmp_path / "facade_driver")
    libdir = os.path.dirname(ljlib._name)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), SRC, "-o", exe,
                           "-L", libdir, "-llj_gb300", "-Wl,-rpath," + libdir])
    return exe


def test_driver_compiles_and_links(ljlib, tmp_path):
    exe = build_driver(ljlib, tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_driver_runs(ljlib, tmp_path):
    exe = build_driver(ljlib, tmp_path)
    out = subprocess.run([exe, "200"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = {}
    for line in out.stdout.splitlines():
        head, *kv = line.split()
        lines[head] = dict(x.split("=", 1) for x in kv if "=" in x)
    init, tvn, evn, rdf, velo, multi = (lines[k] for k in ("init", "tvn", "evn", "rdf", "velo", "multi"))
    assert float(init["T"]) == pytest.approx(1.312, rel=1e-9)          # exact-T0 initial state
    assert float(init["L"]) == pytest.approx((512 / 0.316) ** (1 / 3), rel=1e-9)
    assert float(tvn["T"]) == pytest.approx(1.312, rel=0.02)          # TVN holds T near T0
    assert int(tvn["av_iters"]) == 200
    assert int(evn["av_iters"]) == 200
    assert abs(float(evn["<T>"]) - 1.312) < 0.2
    assert int(rdf["total"]) == 512 * 511                             # every ordered pair binned (clamp rule)
    assert 1.0 < float(rdf["peak_r"]) < 1.3                            # first shell of the LJ fluid
    assert float(velo["norm"]) == pytest.approx(1.0, abs=0.02)        # velocity density integrates to ~1
    assert float(multi["t"]) == pytest.approx(0.005 * 450, rel=1e-9)
    assert int(multi["av_iters"]) == 250


GOLDEN = ("n400_evn_gas", "n256_tvn_liquid", "n216_evn_liquid", "n125_wall", "n64_open")


def _build_golden_driver(ljlib, tmp_path):
    exe = str(tmp_path / "golden_driver")
    libdir = os.path.dirname(ljlib._name)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                           os.path.join(REPO, "tests", "facade", "golden_driver.cpp"), "-o", exe,
                           "-L", libdir, "-llj_gb300", "-Wl,-rpath," + libdir])
    return exe


def test_golden_driver_compiles_and_links(ljlib, tmp_path):
    assert os.path.exists(_build_golden_driver(ljlib, tmp_path))


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN)
def test_facade_rdf_and_velocity_pinned_to_reference(ljlib, tmp_path, case):
    """RDF(), initvelo(), getvelo() and updatevelo() of the facade on the
    golden states against the reference's own outputs (MDSystem.cpp:633-694,
    recorded in tests/golden/<case>.npz by the reference's CPU MDSystem).

    The bin positions must be identical.  The normalisation constants are
    pinned independently of the binning: every RDF value divided by its
    count equals the reference's value divided by the reference's count (to
    the float rounding of the reference's count / bin-width division; exactly
    where the counts agree), and
    every velocity-density value times (bin width x N) -- times 2 after one
    updatevelo (the running mean of two histograms) -- is an integer count.
    The counts themselves agree with the reference's except for the pairs
    or particles that fall on the other side of a bin edge (the device bins
    FP64-state separations, the reference float ones): at most a few."""
    z = np.load(os.path.join(REPO, "tests", "golden", case + ".npz"))
    N = int(z["N"])
    exe = _build_golden_driver(ljlib, tmp_path)
    pf, vf = tmp_path / "pos.f32", tmp_path / "vel.f32"
    z["pos0"].astype(np.float32).tofile(pf)
    z["vel0"].astype(np.float32).tofile(vf)
    args = [exe, str(N), "%.17g" % float(z["T0"]), "%.17g" % float(z["rho"]), str(int(z["canonical"])),
            str(int(z["bc"])), "%.17g" % float(z["dt"]), str(int(z["steps"])), str(pf), str(vf)]
    out = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = {}
    for line in out.stdout.splitlines():
        head, *vals = line.split()
        if head == "scalars":
            rows[head] = {k: float(v) for k, v in (x.split("=", 1) for x in vals)}
        elif head != "status":
            rows[head] = np.array([float(v) for v in vals])
    sc0 = dict(zip(("U", "T", "K", "V", "P", "Pshear", "t", "L", "av_U", "av_T", "av_p", "av_iters", "rdf_dr2"),
                   z["scalars0"]))
    assert rows["scalars"]["rdf_dr2"] == sc0["rdf_dr2"]                 # same float bin width
    assert rows["scalars"]["L"] == pytest.approx(sc0["L"], rel=1e-12)
    # ---- RDF (MDSystem.cpp:633-649): 256 r^2 bins ----
    np.testing.assert_allclose(rows["rdf_x"], z["rdf_x"], rtol=1e-15, atol=0)
    cnt, ref_cnt = rows["rdf_counts"], z["rdf0"].astype(np.float64)
    y, ref_y = rows["rdf_y"], z["rdf_y"]
    assert len(y) == len(ref_y) == 256
    both = (cnt > 0) & (ref_cnt > 0)
    both[255] = False          # overflow bin: clamped on the device, dropped by the reference CPU path
    assert both.sum() > 10
    # MDSystem.cpp:643 divides the int count by the float bin width in float
    # (int / float), so y / count carries that one float rounding (2^-24)
    np.testing.assert_allclose(y[both] / cnt[both], ref_y[both] / ref_cnt[both], rtol=1.2e-7)
    same = both & (cnt == ref_cnt)
    np.testing.assert_allclose(y[same], ref_y[same], rtol=1e-12)
    moved = np.abs(cnt[:255] - ref_cnt[:255]).sum()
    assert moved <= max(4, 1e-4 * N * (N - 1)), moved
    assert cnt.sum() == N * (N - 1)                                       # every ordered pair, clamp rule
    # ---- velocity density (MDSystem.cpp:651-694): 101 bins of 0.12 ----
    step = 0.12
    np.testing.assert_allclose(rows["velo_x"], z["velo_x"], rtol=1e-15)
    for name, ref_name, k in (("velo_y", "velo_y", 1), ("velo_upd_y", "velo_upd_y", 2)):
        got_c = rows[name] * step * N * k
        ref_c = z[ref_name] * step * N * k
        assert np.abs(got_c - np.rint(got_c)).max() < 1e-9, name           # normalisation pinned
        assert np.abs(ref_c - np.rint(ref_c)).max() < 1e-9, name
        diff = np.abs(np.rint(got_c) - np.rint(ref_c)).sum()
        assert np.rint(got_c).sum() == k * N, name                         # every particle counted
        print("%s %s: %d of %d counts in another bin than the reference's" % (case, name, diff, k * N))
        assert diff <= 4, name
