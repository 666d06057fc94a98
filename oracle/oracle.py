"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker or the timed CPU baseline.  The product
library (lennard-jones-cuda_gb300/) never imports, links or calls it.

Wraps
  * oracle/liblj_oracle.so   -- lj_oracle.c: the faithful float-storage
    restatement of the reference CPU path (``R32System``), the FP64
    restatement (``f64_forces``, ``F64System``) and the device-decision
    emulation used for exact histogram parity (``emu_*``);
  * oracle/_ref/libmdsystem_ref.so -- the reference's own MDSystem.cpp built
    from its sources by build_ref.sh (``RefSystem``), present only where the
    reference sources were available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblj_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libmdsystem_ref.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile lj_oracle.c with gcc (OpenMP, no FP contraction) if needed."""
    src = os.path.join(HERE, "lj_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                               "-o", LIB_PATH, src])
    return LIB_PATH


def reference_dir(ref_dir: str = None):
    """The vlvovch/lennard-jones-cuda checkout to build oracle/_ref from:
    ref_dir, else LJ_REFERENCE_DIR; None unless it holds the reference's
    src/library/MDSystem.cpp."""
    d = ref_dir or os.environ.get("LJ_REFERENCE_DIR")
    if d and os.path.isfile(os.path.join(d, "src", "library", "MDSystem.cpp")):
        return d
    return None


def build_ref(ref_dir: str = None) -> bool:
    """Build oracle/_ref from the reference sources when they are present
    (see reference_dir); True if the reference library exists afterwards."""
    d = reference_dir(ref_dir)
    if d is not None:
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), d])
    return os.path.exists(REF_PATH)


def sample_state(n, density, temperature, lattice=1, jitter=0.0, seed=1):
    """The seeded initial state of a workload ((n,3) positions, velocities,
    box side): lattice 0 = simple cubic, 1 = FCC."""
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    L = C.c_double()
    if lib().init_sample_state(int(n), float(density), float(temperature), int(lattice), float(jitter), int(seed),
                               pos, vel, C.byref(L)):
        raise ValueError("bad initial-state arguments")
    return pos, vel, L.value


class _R32State(C.Structure):
    _fields_ = [("N", C.c_int), ("T0", C.c_double), ("rho", C.c_double), ("canonical", C.c_int),
                ("bc", C.c_int), ("L", C.c_double), ("t", C.c_double), ("U", C.c_double),
                ("T", C.c_double), ("K", C.c_double), ("V", C.c_double), ("P", C.c_double),
                ("Pshear", C.c_double), ("av_U_tot", C.c_double), ("av_T_tot", C.c_double),
                ("av_p_tot", C.c_double), ("av_iters", C.c_int), ("rdf_dr2", C.c_float),
                ("rdf", C.c_int * 256), ("pos", C.c_void_p), ("vel", C.c_void_p),
                ("frc", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(_R32State)
        L.init_sample_state.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_uint64,
                                        _f64p, _f64p, C.POINTER(C.c_double)]
        L.init_sample_state.restype = C.c_int
        L.r32_rdf_dr2.argtypes = [C.c_int]
        L.r32_rdf_dr2.restype = C.c_float
        L.r32_calculate_forces.argtypes = [P, C.c_void_p, C.c_int]
        L.r32_force_rows.argtypes = [P, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.r32_force_rows.restype = C.c_double
        L.r32_calculate_parameters.argtypes = [P]
        L.r32_kinetic_temperature.argtypes = [P, C.c_void_p]
        L.r32_kinetic_temperature.restype = C.c_double
        L.r32_renormalize_velocities.argtypes = [P, C.c_int]
        L.r32_renormalize_velocities_to_energy.argtypes = [P, C.c_double]
        L.r32_apply_boundary_conditions.argtypes = [P]
        L.r32_integrate.argtypes = [P, C.c_double, C.c_int]
        L.r32_velocity_counts.argtypes = [P, C.c_double, C.c_int, _i32p]
        L.f64_forces_rows.argtypes = [C.c_int, _f64p, C.c_double, C.c_int, C.c_double, C.c_double,
                                      C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                      _f64p, C.c_int]
        L.emu_fixed_coord.argtypes = [C.c_double, C.c_double]
        L.emu_fixed_coord.restype = C.c_uint32
        L.emu_rdf_r2.argtypes = [C.c_int, _u32p, C.c_float, C.c_float, C.c_int, C.c_int, _u64p,
                                 C.c_int]
        L.emu_rdf_r.argtypes = [C.c_int, _u32p, C.c_float, C.c_float, C.c_float, C.c_int, _u64p,
                                C.c_int]
        L.emu_velocity_counts.argtypes = [C.c_int, _f64p, C.c_double, C.c_int, _u64p]
        _lib = L
    return _lib


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)))


# --------------------------------------------------------------------------
# Faithful float-storage restatement of the reference CPU path
# --------------------------------------------------------------------------
class R32System:
    """MDSystem (CPU mode) restated: float[4N] pos/vel/frc, double scalars.

    Mirrors MDSystem.cpp; state is injected through ``pos``/``vel`` the way
    callers write h_Pos/h_Vel.
    """

    def __init__(self, N, T0, rho, canonical=False, bc=0, pos4=None, vel4=None):
        self.N = int(N)
        self.pos = np.zeros((self.N, 4), np.float32)
        self.vel = np.zeros((self.N, 4), np.float32)
        self.frc = np.zeros((self.N, 4), np.float32)
        s = _R32State()
        s.N, s.T0, s.rho = self.N, float(T0), float(rho)
        s.canonical, s.bc = int(bool(canonical)), int(bc)
        s.L = (self.N / float(rho)) ** (1.0 / 3.0)
        s.T = float(T0)
        s.rdf_dr2 = lib().r32_rdf_dr2(self.N)
        s.pos = self.pos.ctypes.data
        s.vel = self.vel.ctypes.data
        s.frc = self.frc.ctypes.data
        self.s = s
        if pos4 is not None:
            self.pos[:] = pos4
        if vel4 is not None:
            self.vel[:] = vel4

    @property
    def L(self):
        return self.s.L

    def calculate_forces(self, nthreads=1):
        lib().r32_calculate_forces(C.byref(self.s), self.frc.ctypes.data, int(nthreads))

    def force_rows(self, i0, i1, nthreads=1):
        """The force loop over rows [i0, i1) only (a timing sample)."""
        return lib().r32_force_rows(C.byref(self.s), self.frc.ctypes.data, int(i0), int(i1), int(nthreads))

    def calculate_parameters(self):
        lib().r32_calculate_parameters(C.byref(self.s))

    def integrate(self, dt, nthreads=1):
        lib().r32_integrate(C.byref(self.s), float(dt), int(nthreads))

    def renormalize(self, recalc=True):
        lib().r32_renormalize_velocities(C.byref(self.s), int(recalc))

    def renormalize_to_energy(self, ust):
        lib().r32_renormalize_velocities_to_energy(C.byref(self.s), float(ust))

    def velocity_counts(self, step=0.12, nbins=101):
        out = np.zeros(nbins, np.int32)
        lib().r32_velocity_counts(C.byref(self.s), float(step), int(nbins), out)
        return out

    def scalars(self):
        s = self.s
        return dict(U=s.U, T=s.T, K=s.K, V=s.V, P=s.P, Pshear=s.Pshear, t=s.t, L=s.L,
                    av_U=s.av_U_tot, av_T=s.av_T_tot, av_p=s.av_p_tot, av_iters=s.av_iters,
                    rdf_dr2=s.rdf_dr2)

    def rdf_counts(self):
        return np.array(self.s.rdf[:], np.int64)


# --------------------------------------------------------------------------
# True FP64 restatement
# --------------------------------------------------------------------------
def f64_forces(pos, L, periodic=True, eps=1.0, sigma=1.0, rows=None, nthreads=None):
    """All-pairs LJ forces in double.  pos: (N,3) float64.

    Returns dict(F=(n,3), e=(n,), w=(n,), V, W, Pshear_pair) for rows
    ``rows=(i0, i1)`` (default all).  e_i = sum_j 4eps[(s/r)^12-(s/r)^6],
    w_i = sum_j r_ij.f_ij; V = sum_i e_i / 2 over the rows, W = sum_i w_i.
    """
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    N = pos.shape[0]
    i0, i1 = (0, N) if rows is None else rows
    n = i1 - i0
    F = np.zeros((N, 3), np.float64)
    e = np.zeros(N, np.float64)
    w = np.zeros(N, np.float64)
    out3 = np.zeros(3, np.float64)
    lib().f64_forces_rows(N, pos.ravel(), float(L), int(bool(periodic)), float(eps), float(sigma),
                          int(i0), int(i1), F.ctypes.data, e.ctypes.data, w.ctypes.data, out3,
                          int(nthreads or default_threads()))
    return dict(F=F[i0:i1].copy(), e=e[i0:i1].copy(), w=w[i0:i1].copy(), V=out3[0], W=out3[1],
                Pshear_pair=out3[2], n=n)


class F64System:
    """Double-storage restatement of Integrate/ApplyBoundaryConditions/
    CalculateParameters (MDSystem.cpp:325-359, 406-510) with explicit eps, sigma."""

    def __init__(self, pos, vel, L, rho, T0, canonical=False, bc=0, eps=1.0, sigma=1.0,
                 nthreads=None):
        self.pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3).copy()
        self.vel = np.ascontiguousarray(vel, np.float64).reshape(-1, 3).copy()
        self.N = self.pos.shape[0]
        self.L, self.rho, self.T0 = float(L), float(rho), float(T0)
        self.canonical, self.bc = bool(canonical), int(bc)
        self.eps, self.sigma = float(eps), float(sigma)
        self.t = 0.0
        self.nthreads = nthreads or default_threads()
        self.compute_forces()
        self.parameters()

    def compute_forces(self):
        r = f64_forces(self.pos, self.L, self.bc == 0, self.eps, self.sigma,
                       nthreads=self.nthreads)
        self.F = r["F"]
        self.V = r["V"]
        self.W = r["W"]
        self.e = r["e"]

    def parameters(self):
        self.K = float(0.5 * np.sum(self.vel * self.vel))
        self.T = 2.0 * self.K / 3.0 / self.N
        self.P = (self.W / 6.0 + self.N * self.T) / (self.N / self.rho)
        self.U = self.K + self.V

    def boundary(self):
        if self.bc == 0:
            self.pos = np.where(self.pos < 0.0, self.pos + self.L, self.pos)
            self.pos = np.where(self.pos > self.L, self.pos - self.L, self.pos)
        elif self.bc == 1:
            flip = ((self.pos < 0.0) & (self.vel < 0.0)) | ((self.pos > self.L) & (self.vel > 0.0))
            self.vel = np.where(flip, -self.vel, self.vel)

    def step(self, dt):
        dt = float(dt)
        if not self.canonical:
            self.pos += dt * self.vel + dt * dt * self.F / 2.0
            self.vel += dt * self.F / 2.0
            self.compute_forces()
            self.vel += dt * self.F / 2.0
        else:
            self.pos += dt * self.vel + dt * dt * self.F / 2.0
            tF = 0.5 * self.F
            self.compute_forces()
            tF = tF + 0.5 * self.F
            tv = self.vel + dt * tF / 2.0
            Tkin = float(np.sum(tv * tv)) / 3.0 / self.N
            chi = np.sqrt(self.T0 / Tkin)
            self.vel = (2.0 * chi - 1.0) * self.vel + chi * dt * tF
        self.boundary()
        self.parameters()
        self.t += dt


# --------------------------------------------------------------------------
# Device-decision emulation (exact histogram parity)
# --------------------------------------------------------------------------
def emu_fixed(pos, L):
    """FP64 positions -> the device's uint32 shadow: low 32 bits of
    rint(x * (1/L) * 2^32), moved to the nearest multiple of 3."""
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    scale = (1.0 / L) * 4294967296.0
    u = (np.rint(pos * scale).astype(np.int64) & 0xFFFFFFFF).astype(np.uint64)
    r = u % 3
    q = np.where(r == 0, u, np.where(r == 1, u - 1, u + 1))
    return q.astype(np.uint32)


def emu_rdf_r2(q, k2, inv_dr2, nb=256, mode=0, nthreads=None):
    q = np.ascontiguousarray(q, np.uint32).reshape(-1, 3)
    out = np.zeros(nb, np.uint64)
    lib().emu_rdf_r2(q.shape[0], q.ravel(), float(k2), float(inv_dr2), int(nb), int(mode), out,
                     int(nthreads or default_threads()))
    return out


def emu_rdf_r(q, k2, inv_dr, rmax2, nb, nthreads=None):
    q = np.ascontiguousarray(q, np.uint32).reshape(-1, 3)
    out = np.zeros(nb, np.uint64)
    lib().emu_rdf_r(q.shape[0], q.ravel(), float(k2), float(inv_dr), float(rmax2), int(nb), out,
                    int(nthreads or default_threads()))
    return out


def emu_velocity_counts(vel, step, nb):
    vel = np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
    out = np.zeros(nb, np.uint64)
    lib().emu_velocity_counts(vel.shape[0], vel.ravel(), float(step), int(nb), out)
    return out


# --------------------------------------------------------------------------
# The reference's own CPU MDSystem (oracle/_ref)
# --------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_create.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_int]
        R.ref_create.restype = C.c_void_p
        R.ref_destroy.argtypes = [C.c_void_p]
        R.ref_set_state.argtypes = [C.c_void_p, _f32p, _f32p]
        R.ref_set_forces.argtypes = [C.c_void_p, _f32p]
        for name in ("ref_calculate_forces", "ref_calculate_parameters", "ref_updatevelo",
                     "ref_reset_averaging"):
            getattr(R, name).argtypes = [C.c_void_p]
        R.ref_integrate.argtypes = [C.c_void_p, C.c_double, C.c_int]
        R.ref_renormalize.argtypes = [C.c_void_p, C.c_int]
        R.ref_renormalize_to_energy.argtypes = [C.c_void_p, C.c_double]
        R.ref_set_canonical.argtypes = [C.c_void_p, C.c_int]
        R.ref_set_bc.argtypes = [C.c_void_p, C.c_int]
        R.ref_set_time.argtypes = [C.c_void_p, C.c_double]
        R.ref_get.argtypes = [C.c_void_p, _f32p, _f32p, _f32p, _f64p, _i32p]
        R.ref_rdf.argtypes = [C.c_void_p, _f64p, _f64p]
        R.ref_initvelo.argtypes = [C.c_void_p, C.c_double, C.c_double]
        R.ref_getvelo.argtypes = [C.c_void_p, _f64p, _f64p, C.c_int]
        R.ref_getvelo.restype = C.c_int
        R.ref_maxwell.argtypes = [C.c_void_p, C.c_double]
        R.ref_maxwell.restype = C.c_double
        _ref = R
    return _ref


_REF_SCALARS = ("U", "T", "K", "V", "P", "Pshear", "t", "L", "av_U", "av_T", "av_p", "av_iters",
                "rdf_dr2")


class RefSystem:
    """The reference's MDSystem (CPU mode) with injected state."""

    def __init__(self, N, T0, rho, canonical=False, bc=0):
        self.N = int(N)
        self.h = ref_lib().ref_create(self.N, float(T0), float(rho), int(bool(canonical)), int(bc))

    def __del__(self):
        if getattr(self, "h", None):
            ref_lib().ref_destroy(self.h)
            self.h = None

    def set_state(self, pos4, vel4):
        ref_lib().ref_set_state(self.h, np.ascontiguousarray(pos4, np.float32),
                                np.ascontiguousarray(vel4, np.float32))

    def set_forces(self, frc4):
        ref_lib().ref_set_forces(self.h, np.ascontiguousarray(frc4, np.float32))

    def calculate_forces(self):
        ref_lib().ref_calculate_forces(self.h)

    def calculate_parameters(self):
        ref_lib().ref_calculate_parameters(self.h)

    def integrate(self, dt, nsteps=1):
        ref_lib().ref_integrate(self.h, float(dt), int(nsteps))

    def get(self):
        p = np.zeros((self.N, 4), np.float32)
        v = np.zeros((self.N, 4), np.float32)
        f = np.zeros((self.N, 4), np.float32)
        sc = np.zeros(13, np.float64)
        rdf = np.zeros(256, np.int32)
        ref_lib().ref_get(self.h, p, v, f, sc, rdf)
        return dict(pos=p, vel=v, frc=f, rdf=rdf, **dict(zip(_REF_SCALARS, sc.tolist())))

    def rdf(self):
        x = np.zeros(256)
        y = np.zeros(256)
        ref_lib().ref_rdf(self.h, x, y)
        return x, y

    def initvelo(self, vmax=12.0, step=0.12):
        ref_lib().ref_initvelo(self.h, float(vmax), float(step))

    def updatevelo(self):
        ref_lib().ref_updatevelo(self.h)

    def getvelo(self):
        x = np.zeros(4096)
        y = np.zeros(4096)
        n = ref_lib().ref_getvelo(self.h, x, y, 4096)
        return x[:n].copy(), y[:n].copy()
