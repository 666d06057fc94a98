"""Generates the golden fixtures under tests/golden/ from the reference itself.

Runs the reference's own CPU MDSystem (src/library/MDSystem.cpp of
vlvovch/lennard-jones-cuda, compiled from its sources by oracle/build_ref.sh
into oracle/_ref/) on seeded injected states and records its outputs:
forces, observables, RDF counts, velocity histograms and trajectories.
The reference has no tests or golden vectors of its own, so these fixtures
are what pins the oracle restatement (oracle/lj_oracle.c) to the reference.

Usage (needs the reference sources, given as LJ_REFERENCE_DIR or the first
argument; not run by the test suite):
    python tests/golden/make_golden.py <reference checkout>
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle as O  # noqa: E402


def lattice_state(N, rho, T0, lattice, jitter, seed):
    """Seeded lattice + jitter + Gaussian velocities (zero momentum, exact T0),
    as float4 arrays (w of the position = L/150 like MDSystem.cpp:168)."""
    rng = np.random.default_rng(seed)
    L = (N / rho) ** (1.0 / 3.0)
    if lattice == "sc":
        ns = int(np.ceil(N ** (1.0 / 3.0) - 1e-12))
        n = np.arange(N)
        dL = L / ns
        p = np.stack([(n % ns + 0.5) * dL, ((n // ns) % ns + 0.5) * dL, (n // ns ** 2 + 0.5) * dL], 1)
    else:
        nc = int(np.ceil((N / 4) ** (1.0 / 3.0) - 1e-12))
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
    p4 = np.zeros((N, 4), np.float32)
    p4[:, :3] = p
    p4[:, 3] = np.float32(L / 150.0)
    v4 = np.zeros((N, 4), np.float32)
    v4[:, :3] = v
    return p4, v4


CASES = [
    # name, N, rho, T0, canonical, bc, lattice, jitter, seed, dt, steps, record_every
    ("n400_evn_gas", 400, 0.05, 1.4, False, 0, "sc", 0.05, 1, 0.005, 60, 20),
    ("n256_tvn_liquid", 256, 0.85, 1.0, True, 0, "fcc", 0.02, 2, 0.005, 40, 20),
    ("n216_evn_liquid", 216, 0.8, 1.2, False, 0, "sc", 0.05, 5, 0.004, 40, 20),
    ("n125_wall", 125, 0.5, 1.2, False, 1, "sc", 0.05, 3, 0.005, 40, 20),
    ("n64_open", 64, 0.3, 1.5, True, 2, "sc", 0.05, 4, 0.005, 30, 15),
]

SCALARS = ("U", "T", "K", "V", "P", "Pshear", "t", "L", "av_U", "av_T", "av_p", "av_iters", "rdf_dr2")


def make_case(name, N, rho, T0, canonical, bc, lattice, jitter, seed, dt, steps, every):
    p4, v4 = lattice_state(N, rho, T0, lattice, jitter, seed)
    ref = O.RefSystem(N, T0, rho, canonical, bc)
    ref.set_state(p4, v4)
    ref.calculate_forces()
    ref.calculate_parameters()
    ref.initvelo(12.0, 0.12)
    g0 = ref.get()
    rx, ry = ref.rdf()
    vx, vy = ref.getvelo()
    out = dict(N=N, rho=rho, T0=T0, canonical=int(canonical), bc=bc, dt=dt, steps=steps, every=every,
               pos0=p4, vel0=v4, frc0=g0["frc"], rdf0=g0["rdf"], rdf_x=rx, rdf_y=ry, velo_x=vx,
               velo_y=vy, scalars0=np.array([g0[k] for k in SCALARS]))
    traj_pos, traj_vel, traj_frc, traj_sc, traj_rdf = [], [], [], [], []
    for k in range(steps // every):
        ref.integrate(dt, every)
        g = ref.get()
        traj_pos.append(g["pos"])
        traj_vel.append(g["vel"])
        traj_frc.append(g["frc"])
        traj_rdf.append(g["rdf"])
        traj_sc.append([g[s] for s in SCALARS])
    ref.updatevelo()
    ux, uy = ref.getvelo()
    out.update(traj_pos=np.array(traj_pos), traj_vel=np.array(traj_vel), traj_frc=np.array(traj_frc),
               traj_rdf=np.array(traj_rdf), traj_scalars=np.array(traj_sc), velo_upd_y=uy)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def main():
    if not O.ref_available() and not O.build_ref(sys.argv[1] if len(sys.argv) > 1 else None):
        raise SystemExit("reference sources unavailable; cannot regenerate golden fixtures")
    for case in CASES:
        make_case(*case)
        print("wrote", case[0])


if __name__ == "__main__":
    main()
