"""numpy restatement of the reference's task-driver statistics (test
infrastructure only: tests/ import it as the checker; the product library
never imports, links or calls it).

  * subsystem_counts: GetNSubsystemBatch
    (src/tasks/run-fluctuations/include/run-fluctuations-aux.h:186-240);
  * velocity_counts: GetNsubVzBatch (run-fluctuations-aux.h:242-273);
  * NumberStatistics moments / mean error / scaled variance and its error
    (src/extra/sample-moments/NumberStatistics.h: moments from sums of N^k,
    error of the mean sqrt(var/n), central-moment covariances after Kendall &
    Stuart, scaled variance kappa_2/<N>);
  * TimeAverage statistical inefficiency s = 2 / ln(var / (<N_t N_{t-1}> -
    <N>^2)), s = 1 if negative (src/tasks/auxiliary/time-average-aux.h:27-67,
    after Allen & Tildesley, Computer Simulation of Liquids, pp. 194-195);
  * cumulant ratios kappa_r / kappa_q and their errors the way
    NumberStatistics.h:470-560 forms them: moments from plain sums of N^k
    (CalculateMoments, :563-599), each cumulant a sum of products of central
    moments, and the error summed term by term over the pairs of factors
    with the Kendall & Stuart central-moment covariances (:208-225);
  * gce_nsub: GetNsub of src/tasks/semiGCEfluctuations/
    semiGCEfluctuations.cpp:7-25 (particles in the cube of volume fraction f
    around the box centre).

Parity is pinned: tests/golden/stats_reference.npz holds the reference's own
TimeAverage / NumberStatistics outputs on seeded series (compiled from its
headers by oracle/build_ref.sh into oracle/_ref/ref_stats and run by
tests/golden/make_stats_golden.py); tests/test_tasks.py checks these
functions and include/ljgb/Statistics.hpp against them.
"""
from __future__ import annotations

import numpy as np


def alphas(step, upper_inclusive):
    """The reference's alpha loop: alpha = step, 2 step, ... accumulated in
    floating point, < 1 - 1e-9 (coordinates) or <= 1 + 1e-9 (velocities)."""
    out = []
    a = step
    while (a <= 1.0 + 1e-9) if upper_inclusive else (a < 1.0 - 1e-9):
        out.append(a)
        a += step
    return out


def subsystem_counts(pos, L, alpha_step, type_):
    """Cumulative counts N(alpha_k) for type 0/1/2 (slab) or 3 (central cube)."""
    al = alphas(alpha_step, False)
    cnts = np.zeros(len(al), np.int64)
    if type_ == 3:
        tls = np.array([L * a ** (1.0 / 3.0) for a in al])
        d = np.abs(pos - 0.5 * L) / 0.5
        ind = np.searchsorted(tls, d, side="right").max(axis=1)
    else:
        ind = ((pos[:, type_] / L) / alpha_step).astype(np.int64)
    for k in ind:
        if 0 <= k < len(al):
            cnts[k] += 1
    return np.cumsum(cnts)


def velocity_counts(vel, vmax, alpha_step, component):
    al = alphas(alpha_step, True)
    cnts = np.zeros(len(al), np.int64)
    ind = ((np.abs(vel[:, component]) / vmax) / alpha_step).astype(np.int64)
    for k in ind:
        if 0 <= k < len(al):
            cnts[k] += 1
    return np.cumsum(cnts)


def moments(x):
    """mean, biased variance, error of the mean, scaled variance and its error."""
    x = np.asarray(x, np.float64)
    n = len(x)
    m = x.mean()
    mu = [np.mean((x - m) ** k) for k in range(5)]
    var = mu[2]
    mean_err = np.sqrt(var / n)
    # cov(m2, m2) = (mu4 - mu2^2)/n; cov(m2, mean) = mu3/n (Kendall & Stuart)
    c1, c2 = var, m
    c1dev = (mu[4] - mu[2] ** 2) / n
    c2dev = mean_err ** 2
    c12 = mu[3] / n
    w = c1 / c2
    w_err = abs(w) * np.sqrt(c1dev / c1 / c1 + c2dev / c2 / c2 - 2.0 * c12 / c1 / c2)
    return dict(mean=m, var=var, mean_err=mean_err, w=w, w_err=w_err)


def inefficiency(x):
    """s = 2 / ln(var / corr), s = 1 if negative; also s = 1 where corr <= 0
    or var / corr <= 1, where the reference's formula gives NaN / infinity
    (a deliberate difference, stated in include/ljgb/Statistics.hpp)."""
    x = np.asarray(x, np.float64)
    n = len(x)
    m = x.mean()
    var = np.mean(x * x) - m * m
    corr = np.sum(x[1:] * x[:-1]) / (n - 1) - m * m
    if not corr > 0 or not var / corr > 1:
        return 1.0
    s = 2.0 / np.log(var / corr)
    return 1.0 if s < 0 else s


def gce_nsub(pos, L, fraction):
    """GetNsub: |x_c - L/2| < L f^(1/3) / 2 in all three coordinates."""
    tL = L * fraction ** (1.0 / 3.0)
    d = np.abs(pos - 0.5 * L)
    return int(np.sum(np.all(d < 0.5 * tL, axis=1)))


def gce_fractions():
    """The task's fraction loop: 0.05, 0.10, ... accumulated, <= 1."""
    out, t = [], 0.05
    while t <= 1.0:
        out.append(t)
        t += 0.05
    return out


# kappa_r as sums of products of central moments: (coefficient, [orders])
_CUMULANT_TERMS = {2: [(1, [2])], 3: [(1, [3])], 4: [(1, [4]), (-3, [2, 2])]}


class _Moments:
    def __init__(self, x, nmax=8, shift=0.0):
        # shift: SetMeanShift (NumberStatistics.h:322-345), subtracted from
        # every observation before its powers are summed
        x = np.asarray(x, np.float64) - shift
        self.n = float(len(x))
        raw = [np.sum(x ** k) / len(x) for k in range(nmax + 1)]
        from math import comb
        self.mu = [1.0, 0.0]
        for r in range(2, nmax + 1):
            self.mu.append(sum(comb(r, i) * raw[r - i] * raw[1] ** i * (-1.0) ** i for i in range(r + 1)))

    def cov(self, r, q):
        mu = self.mu
        if r <= 1 or q <= 1:
            return 0.0
        c = mu[r + q] - mu[r] * mu[q] + r * q * mu[2] * mu[r - 1] * mu[q - 1]
        c -= r * mu[r - 1] * mu[q + 1] + q * mu[r + 1] * mu[q - 1]
        return c / self.n

    def cumulant(self, r):
        return sum(coef * np.prod([self.mu[m] for m in ms]) for coef, ms in _CUMULANT_TERMS[r])

    def _partials(self, r):
        """(d kappa_r / d mu_m) contributions, one per factor of each term."""
        out = []
        for coef, ms in _CUMULANT_TERMS[r]:
            full = coef * np.prod([self.mu[m] for m in ms])
            for m in ms:
                out.append((m, full / self.mu[m]))
        return out

    def ratio_error(self, r, q):
        num, den = self.cumulant(r), self.cumulant(q)
        a = [(m, t / den) for m, t in self._partials(r)] + \
            [(m, -t * num / den / den) for m, t in self._partials(q)]
        return float(np.sqrt(sum(t1 * t2 * self.cov(m1, m2) for m1, t1 in a for m2, t2 in a)))


def cumulant_ratios(x, shift=0.0):
    """skewness kappa_3/kappa_2, kurtosis kappa_4/kappa_2 and their errors."""
    m = _Moments(x, shift=shift)
    return dict(skew=m.cumulant(3) / m.cumulant(2), skew_err=m.ratio_error(3, 2),
                kurt=m.cumulant(4) / m.cumulant(2), kurt_err=m.ratio_error(4, 2))
