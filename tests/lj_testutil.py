"""Shared helpers of the test suite: seeded states and error statistics."""
import numpy as np


def lattice_state(N, rho, T0, lattice="fcc", jitter=0.02, seed=1):
    """Seeded lattice + uniform jitter + Gaussian velocities (zero momentum,
    exact T0), FP64 (N,3) arrays and the box side."""
    rng = np.random.default_rng(seed)
    L = (N / rho) ** (1.0 / 3.0)
    if lattice == "sc":
        ns = int(np.ceil(N ** (1.0 / 3.0) - 1e-12))
        n = np.arange(N)
        dL = L / ns
        p = np.stack([(n % ns + 0.5) * dL, ((n // ns) % ns + 0.5) * dL, (n // ns ** 2 + 0.5) * dL], 1)
    else:
        nc = int(np.ceil((N / 4) ** (1.0 / 3.0) - 1e-12))
        while 4 * nc ** 3 < N:
            nc += 1
        a = L / nc
        basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
        k = np.arange(N)
        c = k // 4
        cell = np.stack([c % nc, (c // nc) % nc, c // nc ** 2], 1)
        p = (cell + basis[k % 4] + 0.25) * a
    p = p + rng.uniform(-jitter, jitter, p.shape)
    v = rng.normal(0.0, np.sqrt(T0), (N, 3))
    v -= v.mean(0)
    v *= np.sqrt(T0 / (np.sum(v * v) / 3.0 / N))
    return p, v, L


def force_errors(F, Fref):
    """Per-particle |dF_i|/|F_i| and |dF_i|/rms|F| statistics."""
    d = np.linalg.norm(F - Fref, axis=1)
    mag = np.linalg.norm(Fref, axis=1)
    rms = np.sqrt(np.mean(mag ** 2))
    rel = d / np.maximum(mag, 1e-300)
    relrms = d / rms
    mixed = d / np.maximum(mag, rms)
    return dict(rel_median=float(np.median(rel)), rel_p99=float(np.percentile(rel, 99)),
                rel_max=float(rel.max()), rms_max=float(relrms.max()), rms_median=float(np.median(relrms)),
                gate_max=float(mixed.max()))


def golden_states():
    """The golden MDSystem state fixtures (tests/golden/n*.npz, written by the
    reference's CPU MDSystem); tests/golden/stats_*.npz pin the statistics."""
    import glob
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    return sorted(p for p in glob.glob(os.path.join(here, "*.npz")) if not os.path.basename(p).startswith("stats_"))
