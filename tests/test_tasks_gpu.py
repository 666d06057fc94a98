"""Task-driver support on the GPU: the per-step subsystem counters and the
RDF summed over steps, against the numpy restatement of the reference's
counting functions (oracle/tasks.py) and the exact RDF emulation, on the
positions and velocities of the same steps; the task executables end to end."""
import numpy as np
import pytest

import lj_testutil as U

pytestmark = pytest.mark.gpu


def test_subsystem_counters_match_reference_counting(ljgb_mod):
    import tasks
    N, rho, T0 = 400, 0.05, 1.4
    s = ljgb_mod.System(n=N, density=rho, temperature=T0, canonical=1, precision=ljgb_mod.PREC_FP64)
    vmax = 3.0 * np.sqrt(T0)
    spec = [(0, 19, 0.05, 0.0), (1, 19, 0.05, 0.0), (2, 19, 0.05, 0.0), (3, 19, 0.05, 0.0),
            (6, 20, 0.05, vmax), (2, 1, 0.5, 0.0)]
    s.counters_configure(spec, ring_steps=16)
    expect = []
    for _ in range(6):
        s.integrate(0.005)
        p, v, _ = s.get_state()
        row = np.concatenate([tasks.subsystem_counts(p, s.L, 0.05, t) for t in range(4)] +
                             [tasks.velocity_counts(v, vmax, 0.05, 2), tasks.subsystem_counts(p, s.L, 0.5, 2)[:1]])
        expect.append(row)
    got = s.counters_read()
    assert got.shape == (6, 19 * 4 + 20 + 1)
    assert np.array_equal(got, np.array(expect))
    assert s.counters_read().shape[0] == 0          # read clears
    # the cube of volume fraction 1 holds nothing beyond the box: last alpha < 1
    assert got[:, 3 * 19 + 18].max() <= N


def test_counters_every_kth_step(ljgb_mod):
    """lj_counters_set_interval: the central cubes counted after every 3rd
    step only, against the restated GetNsub on the states of those steps."""
    import tasks
    N = 512
    s = ljgb_mod.System(n=N, density=0.316, temperature=1.312)
    s.counters_configure([(3, 19, 0.05, 0.0)], ring_steps=4)
    s.counters_set_interval(3)
    expect = []
    for _ in range(4):
        s.integrate(0.005, 3)
        p, _, _ = s.get_state()
        expect.append([tasks.gce_nsub(p, s.L, f) for f in tasks.gce_fractions()])
    s.integrate(0.005, 2)                       # not a multiple of 3: no row
    got = s.counters_read()
    assert np.array_equal(got, np.array(expect))
    s.integrate(0.005, 1)                       # the 15th step counts
    assert s.counters_read().shape == (1, 19)
    with pytest.raises(ljgb_mod.LJError):
        s.counters_set_interval(0)


def test_counter_ring_overflow_is_reported(ljgb_mod):
    s = ljgb_mod.System(n=256, density=0.5, temperature=1.0)
    s.counters_configure([(0, 4, 0.25, 0.0)], ring_steps=4)
    s.integrate(0.005, 6)
    with pytest.raises(ljgb_mod.LJError):
        s.counters_read()
    s.integrate(0.005, 3)
    assert s.counters_read().shape == (3, 4)


@pytest.mark.parametrize("prec", [0, 1], ids=["mixed", "fp64"])
def test_rdf_summed_over_steps(ljgb_mod, oracle_mod, prec):
    N, rho = 1000, 0.7
    s = ljgb_mod.System(n=N, density=rho, temperature=1.0, canonical=1, precision=prec, lattice=1, jitter=0.02)
    nb, w = 167, 0.03
    s.rdf_accumulate(True, ljgb_mod.RDF_R_LINEAR, nb, w)
    want = np.zeros(nb, np.uint64)
    ks = s.L / 4294967296.0
    for _ in range(3):
        s.integrate(0.005)
        p, _, _ = s.get_state()
        want += oracle_mod.emu_rdf_r(oracle_mod.emu_fixed(p, s.L), np.float32(ks * ks), np.float32(1.0 / w),
                                     np.float32((nb * w) ** 2), nb).astype(np.uint64)
    got, n = s.rdf_accumulated(reset=True)
    assert n == 3
    assert np.array_equal(got, want)
    s.integrate(0.005, 2)
    assert s.rdf_accumulated()[1] == 2


def _run_task(name, text, tmp_path):
    import os
    import subprocess
    import ljgb.build as b
    f = tmp_path / "params.txt"
    f.write_text(text)
    r = subprocess.run([os.path.join(b.BIN_DIR, name), str(f)], cwd=tmp_path, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def _table(path):
    return np.loadtxt(path, skiprows=1, ndmin=2)


def test_run_isotherm_driver(ljlib, tmp_path):
    """Three TVN densities at T*=1.4 (N=256), 2 tau equilibration, 6 tau
    production: one row per density with the reference's columns."""
    r = _run_task("ljgb-run-isotherm", "# isotherm\nN 256\nT* 1.4\nrho*_min 0.1\nrho*_max 0.31\ndrho* 0.1\n"
                  "teq 2.\ntfin 8.\ndt* 0.004\nuseCUDA 1\noutput_prefix iso\n", tmp_path)
    files = list(tmp_path.glob("iso.*.N256.Tst1.4.dat"))
    assert len(files) == 1
    head = files[0].read_text().splitlines()[0].split()
    assert head == ["rho*", "t*", "T*", "<u*>", "d<u*>", "teq_u*", "<p*>", "d<p*>", "teq_p*", "<Z>", "d<Z>",
                    "w[N]", "dw[N]"]
    t = _table(files[0])
    assert t.shape == (3, 13)
    assert np.allclose(t[:, 0], [0.1, 0.2, 0.3])
    assert np.allclose(t[:, 1], 8.0 - 0.004, atol=0.005)
    assert np.all(np.abs(t[:, 2] - 1.4) < 0.15)                      # TVN holds T* near 1.4
    assert np.all(np.isfinite(t)) and np.all(t[:, [4, 7, 10]] > 0)   # errors
    assert np.all(np.diff(t[:, 6]) > 0)                              # p* rises with density
    # near-critical isotherm (T*=1.4, T_c ~ 1.3): Z = p/(rho T) falls from ~0.7 at rho*=0.1 to ~0.5 at 0.3
    assert np.all((t[:, 9] > 0.3) & (t[:, 9] < 1.0)) and np.all(np.diff(t[:, 9]) < 0)
    # a console line every 1000 observations (1500 per density)
    assert sum(1 for line in r.stdout.splitlines() if line.split()[:1] and line.split()[0] in ("0.1", "0.2", "0.3")) == 3


@pytest.mark.parametrize("ensemble", ["tvn", "evn"])
def test_run_fluctuations_driver(ljlib, tmp_path, ensemble):
    """N=400 fluctuation run (the sample inputs' N and u*), 2000 production
    steps: the time-dependence table, the averaged RDF and the five
    fluctuation tables with the reference's layout."""
    canon = "1" if ensemble == "tvn" else "0"
    _run_task("ljgb-run-fluctuations", "N 400\nT* 1.4\nu* 1.708\nrho* 0.3\nteq 1.\ntfin 9.\ndt* 0.004\n"
              "canonical %s\nsubvolume_spacing 0.05\noutput_prefix fl\n" % canon, tmp_path)
    key = "Tst1.4" if ensemble == "tvn" else "ust1.708"
    pre = list(tmp_path.glob("fl.*.N400.%s.rhost0.3.TimeDep.txt" % key))
    assert len(pre) == 1
    base = str(pre[0])[:-len(".TimeDep.txt")]
    td = _table(base + ".TimeDep.txt")
    assert td.shape == (2, 13)
    assert np.allclose(td[:, 0], [1.0 + 4.0, 1.0 + 8.0], atol=0.01)
    if ensemble == "evn":
        assert np.allclose(td[:, 1], 1.708, atol=2e-3)            # energy per particle conserved
    else:
        assert np.all(np.abs(td[:, 2] - 1.4) < 0.15)
    assert np.all(np.abs(td[:, 10:13]) < 1e-6)                     # zero net momentum
    g = _table(base + ".RDF.dat")
    assert g.shape == (256, 2)
    r, gr = g[:, 0], g[:, 1]
    assert np.all(gr[r < 0.8] < 1e-3)                               # hard core
    far = (r > 2.5) & (r < 3.5)
    assert abs(gr[far].mean() - 1.0) < 0.15                         # g(r) -> 1
    # first shell; the last bin collects every pair beyond its edge (the GPU
    # clamp rule of the reference, MDSystem.cu:39), as in the reference's output
    assert 1.2 < gr[:-1].max() < 4.0 and gr[-1] > 10
    for ax in "XYZ":
        f = _table(base + ".flucs%s.dat" % ax)
        assert f.shape == (19, 6)
        assert np.allclose(f[:, 1], f[:, 0] * 400, rtol=0.15, atol=4)  # <N> ~ alpha N
        assert np.all((f[:, 3] > 0.05) & (f[:, 3] < 5))              # w[N]/(1-alpha)
    cube = _table(base + ".flucsCube.dat")
    assert cube.shape == (19, 6) and np.all(np.diff(cube[:, 1]) > 0)
    vz = _table(base + ".flucsVz.dat")
    assert vz.shape == (20, 7)
    assert np.allclose(vz[:, 0], np.sqrt(1.4) * 3 * 0.05 * np.arange(1, 21), rtol=1e-5)  # 6 printed digits
    assert np.all(np.diff(vz[:, 1]) >= 0) and vz[-1, 2] > 0.95         # nearly all |v_z| < 3 sqrt(T*)


def test_semigce_fluctuations_driver(ljlib, tmp_path):
    """The semi-grand-canonical fluctuation task, shortened (500 TVN steps,
    30 EVN events of 20 steps): the reference's console block every 10
    events, and its statistics recomputed from the dumped per-event counts
    with the restated NumberStatistics formulas."""
    import tasks
    r = _run_task("ljgb-semiGCEfluctuations", "N 512\nequilibration_steps 500\nsteps_per_event 20\nevents 30\n"
                  "print_every 10\ndump_counts 1\noutput_prefix gce\n", tmp_path)
    blocks = [b.splitlines() for b in r.stdout.strip().split("\n\n")]
    assert len(blocks) == 3 and all(len(b) == 19 for b in blocks)
    rows = [[float(x) for x in line.replace("+-", " ").split()] for line in blocks[-1]]
    assert all(int(row[0]) == 30 for row in rows)
    counts = np.loadtxt(tmp_path / "gce.counts.dat", ndmin=2)
    assert counts.shape == (30, 19)
    assert np.all(np.diff(counts, axis=1) >= 0) and counts.max() <= 512
    fr = tasks.gce_fractions()
    for k, (f, row) in enumerate(zip(fr, rows)):
        x = counts[:, k]
        m = tasks.moments(x)
        want = [m["mean"], m["mean_err"], m["w"], m["w_err"], m["w"] / (1 - f), m["w_err"] / (1 - f)]
        got = row[1:7]
        if m["var"] > 0:
            assert np.allclose(got, want, rtol=1e-5, atol=2e-6), (f, got, want)
        assert abs(m["mean"] - f * 512) < 0.25 * f * 512 + 10           # <N> ~ f N
        if m["var"] > 0 and abs(1 - 2 * f) > 1e-3:
            cr = tasks.cumulant_ratios(x, shift=x[0])
            assert row[7] == pytest.approx(cr["skew"] / (1 - 2 * f), rel=1e-5, abs=2e-6)
            assert row[8] == pytest.approx(cr["skew_err"] / (1 - 2 * f), rel=1e-5, abs=2e-6)


@pytest.mark.parametrize("axis,W,H", [(2, 96, 96), (0, 80, 64)])
def test_headless_render_matches_restatement(ljgb_mod, axis, W, H):
    """The GPU splat image is pixel-identical to the CPU restatement of the
    same rules (oracle/render.py) on the same positions."""
    import render
    s = ljgb_mod.System(n=200, density=0.3, temperature=1.0, lattice=ljgb_mod.LATTICE_FCC, jitter=0.05)
    s.integrate(0.005, 20)
    p, _, _ = s.get_state()
    img = s.render(0, axis, W, H, 0.5)
    want = render.render(p, s.L, axis, W, H, 0.5)
    assert img.shape == (H, W, 4)
    assert np.array_equal(img, want)
    lit = (img[:, :, 0] > 0).mean()
    assert 0.2 < lit < 1.0                              # particles cover part of the view
    assert set(np.unique(img[:, :, 2])) == {0}          # orange: no blue channel
