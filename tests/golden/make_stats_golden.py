"""Generates tests/golden/stats_reference.npz from the reference itself.

Runs the reference's own TimeAverage / NumberStatistics
(src/tasks/auxiliary/time-average-aux.h:27-67,
src/extra/sample-moments/NumberStatistics.h of vlvovch/lennard-jones-cuda,
compiled where they lie into oracle/_ref/ref_stats by oracle/build_ref.sh) on
seeded series shaped like the task drivers' observables, and records its
mean, variance, errors, scaled variance, statistical inefficiency, skewness
and kurtosis, once as the task drivers call it (no mean shift, except the
U/N-like series) and once with NumberStatistics::SetMeanShift(first
observation).  These fixtures pin the numpy restatement (oracle/tasks.py) and
include/ljgb/Statistics.hpp to the reference (tests/test_tasks.py).

Usage (needs the reference sources, given as LJ_REFERENCE_DIR or the first
argument; not run by the test suite):
    python tests/golden/make_stats_golden.py <reference checkout>
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle as O  # noqa: E402

FIELDS = ("n", "mean", "var", "mean_err", "w", "w_err", "s", "ta_err", "skew", "skew_err", "kurt", "kurt_err")


def _ar1(rng, n, phi, mean, sd):
    x = np.empty(n)
    x[0] = rng.normal()
    e = rng.normal(size=n) * np.sqrt(1.0 - phi * phi)
    for k in range(1, n):
        x[k] = phi * x[k - 1] + e[k]
    return mean + sd * x


def series():
    """name -> (series, mean shift or None).  Integer counts like the
    subsystem counters, AR(1) series like P or T, a U/N-like series with a
    large mean (summed about its first observation, the reference's
    SetMeanShift guard), a skewed one, an anticorrelated one (the
    reference's inefficiency is NaN there) and a short one."""
    rng = np.random.default_rng(20240611)
    out = {}
    out["counts_binomial"] = (rng.binomial(400, 0.35, 6000).astype(np.float64), None)
    slow = _ar1(rng, 8000, 0.97, 0.0, 6.0)
    out["counts_correlated"] = (np.rint(130.0 + slow + rng.normal(size=8000) * 3.0), None)
    out["ar1_pressure"] = (_ar1(rng, 5000, 0.9, 2.31, 0.37), None)
    e = _ar1(rng, 4000, 0.95, -5.2731, 0.011)
    out["energy_shifted"] = (e, float(e[0]))
    out["gamma_skewed"] = (rng.gamma(2.5, 1.7, 7000), None)
    out["anticorrelated"] = (_ar1(rng, 3000, -0.5, 10.0, 1.0), None)
    out["short"] = (np.array([1.0, 2.0, 3.0, 4.0, 2.0, 3.0]), None)
    return out


def run_reference(exe, x, shift):
    cmd = [exe] + ([] if shift is None else ["%.17g" % shift])
    r = subprocess.run(cmd, input="\n".join("%.17g" % v for v in x), capture_output=True, text=True, check=True)
    kv = dict(t.split("=", 1) for t in r.stdout.split())
    return np.array([float(kv[f]) for f in FIELDS])


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else None
    O.build_ref(ref_dir)
    exe = os.path.join(O.HERE, "_ref", "ref_stats")
    if not os.path.exists(exe):
        raise SystemExit("reference sources unavailable; cannot regenerate the statistics fixtures")
    out = {"fields": np.array(FIELDS)}
    for name, (x, shift) in series().items():
        out[name + "__x"] = x
        out[name + "__shift"] = np.array([np.nan if shift is None else shift])
        out[name + "__ref"] = run_reference(exe, x, shift)
        # the same with the power sums taken about the first observation,
        # the summation include/ljgb/Statistics.hpp uses
        out[name + "__ref_first"] = run_reference(exe, x, float(x[0]))
        print(name, dict(zip(FIELDS, out[name + "__ref"])))
    np.savez_compressed(os.path.join(HERE, "stats_reference.npz"), **out)


if __name__ == "__main__":
    main()
