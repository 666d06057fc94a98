"""FP64 numpy restatement of the differentiable trajectory loss and its
discrete adjoint (test infrastructure only: tests/ import it as the checker;
the product library never imports, links or calls it).

The dynamics are the reference's EVN velocity Verlet with periodic
boundaries, unit masses and all-pairs minimum-image Lennard-Jones forces,
generalised from the reference's hard-coded eps = sigma = 1 to explicit
4 eps [(sigma/r)^12 - (sigma/r)^6]:
  * step: src/library/MDSystem.cpp:443-463 (x += dt v + dt^2 F/2,
    v += dt F/2, boundaries :406-436, forces, v += dt F/2);
  * forces, energy and virial: MDSystem.cpp:237-323 (the pair loop) with
    the CUDA kernel's per-particle virial Force.w (src/library/MDSystem.cu:44-53);
  * observables: MDSystem.cpp:325-359 (T = 2K/3/N, P = (W/6 + N T)/(N/rho)).
The reference has no adjoint; the loss and the backward recursion below are
this project's own (derived from the step equations above):

  loss = (1/S) sum_{m=1..S} [ wK K_m/N + wV V_m/N + wP P_m ]

  reverse sweep over m = S..0 with Xb_{S+1} = bb_{S+1} = 0:
    bb_m = dl_m/dv_m + dt Xb_{m+1} + bb_{m+1}
    y_m  = dt^2/2 Xb_{m+1} + dt/2 bb_{m+1}
    z_m  = y_m + dt/2 bb_m   (m > 0),   z_0 = y_0
    Xb_m = dl_m/dx_m + Xb_{m+1} + H(x_m) z_m          (H = dF/dx, symmetric)
    d/d(eps, sigma) += G(x_m)^T z_m + dl_m/d(eps, sigma) (G = dF/d(eps, sigma))
  dloss/dx_0 = Xb_0, dloss/dv_0 = bb_0.
"""
from __future__ import annotations

import numpy as np


def pair_terms(x, L, eps, sigma, z=None):
    """Per-particle sums over all minimum-image partners j != i.

    Returns F (force), A = dF/dsigma, Hz = (dF/dx) z (or None), and the
    scalars e_i = 4 eps sum (s12 - s6), w_i = 4 eps sum (12 s12 - 6 s6)
    (r . f per ordered pair) and ws_i = dw_i/dsigma."""
    d = x[:, None, :] - x[None, :, :]
    d -= L * np.rint(d / L)
    r2 = (d * d).sum(-1)
    np.fill_diagonal(r2, np.inf)
    inv = 1.0 / r2
    s6 = (sigma * sigma * inv) ** 3
    s12 = s6 * s6
    e4 = 4.0 * eps
    g = e4 * (12 * s12 - 6 * s6) * inv            # f_ij = g d_ij
    gs = e4 * (144 * s12 - 36 * s6) * inv / sigma  # dg/dsigma
    F = (g[..., None] * d).sum(1)
    A = (gs[..., None] * d).sum(1)
    e = e4 * (s12 - s6).sum(1)
    w = e4 * (12 * s12 - 6 * s6).sum(1)
    ws = (e4 * (144 * s12 - 36 * s6) / sigma).sum(1)
    Hz = None
    if z is not None:
        h = e4 * (-168 * s12 + 48 * s6) * inv * inv  # g'(r) / r
        dz = z[:, None, :] - z[None, :, :]
        ddz = (d * dz).sum(-1)
        Hz = (g[..., None] * dz + (h * ddz)[..., None] * d).sum(1)
    return F, A, Hz, e, w, ws


def wrap(x, L):
    """Single +-L wrap of ApplyBoundaryConditions (MDSystem.cpp:406-436)."""
    x = np.where(x < 0.0, x + L, x)
    return np.where(x > L, x - L, x)


class Trajectory:
    """Forward run keeping every state (small N only)."""

    def __init__(self, x0, v0, rho, eps=1.0, sigma=1.0, weights=(0.0, 1.0, 1.0)):
        self.x0 = np.array(x0, dtype=np.float64)
        self.v0 = np.array(v0, dtype=np.float64)
        self.N = len(self.x0)
        self.rho = float(rho)
        self.L = (self.N / self.rho) ** (1.0 / 3.0)
        self.eps, self.sigma = float(eps), float(sigma)
        self.wK, self.wV, self.wP = map(float, weights)

    def forward(self, dt, S):
        N, L, rho = self.N, self.L, self.rho
        x, v = self.x0.copy(), self.v0.copy()
        F = pair_terms(x, L, self.eps, self.sigma)[0]
        self.xs, self.vs = [x.copy()], [v.copy()]
        self.obs = []
        loss = 0.0
        for _ in range(S):
            x = x + dt * v + 0.5 * dt * dt * F
            v = v + 0.5 * dt * F
            x = wrap(x, L)
            F, _, _, e, w, _ = pair_terms(x, L, self.eps, self.sigma)
            v = v + 0.5 * dt * F
            K = 0.5 * (v * v).sum()
            V = 0.5 * e.sum()
            W = w.sum()
            T = 2.0 * K / 3.0 / N
            P = (W / 6.0 + N * T) / (N / rho)
            self.obs.append((K, V, W, T, P))
            loss += (self.wK * K / N + self.wV * V / N + self.wP * P) / S
            self.xs.append(x.copy())
            self.vs.append(v.copy())
        self.dt, self.S = dt, S
        return loss

    def backward(self):
        """Returns (dloss/deps, dloss/dsigma, dloss/dx0 (N,3), dloss/dv0 (N,3))."""
        N, L, rho, dt, S = self.N, self.L, self.rho, self.dt, self.S
        eps, sigma = self.eps, self.sigma
        Xb = np.zeros((N, 3))
        bb = np.zeros((N, 3))
        deps = dsig = 0.0
        cv = (self.wK / N + self.wP * rho * 2.0 / (3.0 * N)) / S
        for m in range(S, -1, -1):
            x, v = self.xs[m], self.vs[m]
            bb_m = (cv * v if m >= 1 else 0.0) + dt * Xb + bb
            y = 0.5 * dt * dt * Xb + 0.5 * dt * bb
            z = y + 0.5 * dt * bb_m if m > 0 else y
            F, A, Hz, e, w, ws = pair_terms(x, L, eps, sigma, z)
            dlx = ((-self.wV / N) * F + (self.wP * rho / (6.0 * N)) * (-2.0 * sigma) * A) / S if m >= 1 else 0.0
            Xb = dlx + Xb + Hz
            bb = bb_m
            deps += (z * F).sum() / eps
            dsig += (z * A).sum()
            if m >= 1:
                V, W, Ws = 0.5 * e.sum(), w.sum(), ws.sum()
                deps += (self.wV * V / (N * eps) + self.wP * rho * W / (6.0 * N * eps)) / S
                dsig += (self.wV * W / (2.0 * sigma * N) + self.wP * rho * Ws / (6.0 * N)) / S
        return deps, dsig, Xb, bb


def loss_of(x0, v0, rho, eps, sigma, dt, S, weights=(0.0, 1.0, 1.0)):
    return Trajectory(x0, v0, rho, eps, sigma, weights).forward(dt, S)
