"""Task-driver building blocks on the CPU: the statistics of
include/ljgb/Statistics.hpp against the numpy restatement of the reference's
NumberStatistics / TimeAverage (oracle/tasks.py), the parameter-file reader
of include/ljgb/Parameters.hpp on the reference's file format, and the task
executables being built."""
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(REPO, "include")


_BUILT = {}


def _compile(tmp_path, name):
    """g++ build of tests/tasks/<name>.cpp, once per test session."""
    if name not in _BUILT:
        exe = str(tmp_path / name)
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", INC,
                               os.path.join(REPO, "tests", "tasks", name + ".cpp"), "-o", exe])
        _BUILT[name] = exe
    return _BUILT[name]


def _parse(line):
    return {k: v for k, v in (x.split("=", 1) for x in line.split())}


@pytest.mark.parametrize("kind", ["ar1", "counts", "energy"])
def test_statistics_match_reference_formulas(tmp_path, kind):
    import tasks
    rng = np.random.default_rng(7)
    n = 5000
    if kind == "ar1":          # exponentially correlated series
        x = np.zeros(n)
        for k in range(1, n):
            x[k] = 0.9 * x[k - 1] + rng.normal()
        x += 3.0
    elif kind == "counts":     # integer particle counts
        x = rng.binomial(400, 0.35, n).astype(float)
    else:                      # U/N-like: large mean, small spread
        x = -5.3 + 1e-3 * np.cumsum(rng.normal(size=n)) / np.sqrt(n)
    exe = _compile(tmp_path, "stats_check")
    out = subprocess.run([exe], input="\n".join("%.17g" % v for v in x), capture_output=True, text=True, check=True)
    got = {k: float(v) for k, v in _parse(out.stdout).items()}
    ref = tasks.moments(x)
    assert got["n"] == n
    for k in ("mean", "var", "mean_err", "w", "w_err"):
        assert got[k] == pytest.approx(ref[k], rel=1e-9), k
    # Statistics.hpp sums powers about the first observation: the reference
    # with SetMeanShift(x[0])
    cr = tasks.cumulant_ratios(x, shift=x[0])
    for k in ("skew", "skew_err", "kurt", "kurt_err"):
        assert got[k] == pytest.approx(cr[k], rel=1e-7), k
    s = tasks.inefficiency(x)
    assert got["s"] == pytest.approx(s, rel=1e-6)
    assert got["ta_err"] == pytest.approx(ref["mean_err"] * np.sqrt(s), rel=1e-6)
    if kind == "ar1":  # s ~ 2/(-ln 0.9) ~ 19 for an AR(1) with coefficient 0.9
        assert 12 < s < 28


STATS_GOLDEN = os.path.join(REPO, "tests", "golden", "stats_reference.npz")
STATS_SERIES = ("counts_binomial", "counts_correlated", "ar1_pressure", "energy_shifted", "gamma_skewed",
                "anticorrelated", "short")


@pytest.mark.parametrize("name", STATS_SERIES)
def test_statistics_pinned_to_reference(tmp_path, name):
    """The numpy restatement (oracle/tasks.py) and Statistics.hpp against the
    reference's own TimeAverage / NumberStatistics run on the same series
    (fixtures written by tests/golden/make_stats_golden.py)."""
    import tasks
    z = np.load(STATS_GOLDEN)
    fields = [str(f) for f in z["fields"]]
    x = z[name + "__x"]
    ref = dict(zip(fields, z[name + "__ref"]))              # as the task drivers call it
    first = dict(zip(fields, z[name + "__ref_first"]))      # power sums about x[0]
    assert ref["n"] == len(x)
    # mean, variance, error of the mean, scaled variance and its error
    m = tasks.moments(x)
    for k in ("mean", "var", "mean_err", "w", "w_err"):
        assert m[k] == pytest.approx(ref[k], rel=1e-9), k
    # cumulant ratios: the restatement's moment sums about a given shift
    # reproduce the reference's with the same shift
    with np.errstate(invalid="ignore", divide="ignore"):   # the constant-free short series
        cr = tasks.cumulant_ratios(x, shift=x[0])
    for k in ("skew", "skew_err", "kurt", "kurt_err"):
        if np.isfinite(first[k]):
            assert cr[k] == pytest.approx(first[k], rel=1e-10, abs=1e-15), k
    # statistical inefficiency: the reference's where it is finite; 1 where
    # its logarithm's argument is negative (NaN there, a stated difference)
    s = tasks.inefficiency(x)
    if np.isfinite(ref["s"]):
        assert s == pytest.approx(ref["s"], rel=1e-9)
        assert m["mean_err"] * np.sqrt(s) == pytest.approx(ref["ta_err"], rel=1e-9)
    else:
        assert s == 1.0
    # include/ljgb/Statistics.hpp (moments summed about the first observation)
    exe = _compile(tmp_path, "stats_check")
    out = subprocess.run([exe], input="\n".join("%.17g" % v for v in x), capture_output=True, text=True, check=True)
    got = {k: float(v) for k, v in _parse(out.stdout).items()}
    assert got["n"] == len(x)
    for k in ("mean", "var", "mean_err", "w", "w_err", "skew", "skew_err", "kurt", "kurt_err"):
        if np.isfinite(first[k]):
            assert got[k] == pytest.approx(first[k], rel=1e-9, abs=1e-15), k
    if np.isfinite(ref["s"]):
        assert got["s"] == pytest.approx(ref["s"], rel=1e-9)
        assert got["ta_err"] == pytest.approx(ref["ta_err"], rel=1e-9)
    else:
        assert got["s"] == 1.0


def test_parameter_file_format(tmp_path):
    exe = _compile(tmp_path, "params_check")
    f = tmp_path / "p.txt"
    f.write_text("# Sample input file\n# Format: <parameter-name> <parameter-value>\n\n"
                 "# The number of particles\nN 256\n\nT* 0.9   # trailing comment\nrho*_min 0.01 rho*_max 0.71\n"
                 "output_prefix myrun\nteq 5.\n")
    out = subprocess.run([exe, str(f)], capture_output=True, text=True, check=True).stdout.splitlines()
    kv = dict(line.split("=", 1) for line in out)
    assert kv["output_prefix"] == "myrun"
    assert float(kv["N"]) == 256 and float(kv["T*"]) == 0.9 and float(kv["teq"]) == 5.0
    assert float(kv["rho*_min"]) == 0.01 and float(kv["rho*_max"]) == 0.71
    assert float(kv["useCUDA"]) == 1                     # default kept
    full = kv["full"]
    assert full.startswith("myrun.") and ".N256.ust" in full
    bad = tmp_path / "bad.txt"
    bad.write_text("N abc\n")
    assert subprocess.run([exe, str(bad)], capture_output=True).returncode == 2
    assert subprocess.run([exe, str(tmp_path / "missing.txt")], capture_output=True).returncode == 2


def test_task_executables_are_built(ljlib):
    import ljgb.build as b
    for name in b.TASKS:
        assert os.access(os.path.join(b.BIN_DIR, name), os.X_OK), name


def test_gce_cube_count_is_the_type3_counter():
    """GetNsub of the semi-grand-canonical task (cube of volume fraction f
    around the centre) is the cumulative type-3 subsystem count at the same
    accumulated fractions: the GPU counter serves both tasks."""
    import tasks
    fr = tasks.gce_fractions()
    assert len(fr) == 19 and fr[-1] < 1.0 and fr[9] != 0.5   # accumulated, as the reference's loop
    assert fr == tasks.alphas(0.05, False)
    rng = np.random.default_rng(3)
    L = 11.7
    pos = rng.uniform(0, L, size=(3000, 3))
    cum = tasks.subsystem_counts(pos, L, 0.05, 3)
    assert [tasks.gce_nsub(pos, L, f) for f in fr] == list(cum)
