"""ljgb -- Python front end of liblj_gb300.so (the lj_* C ABI).

A thin ctypes layer: every call goes through the exported C functions of
include/lj_gb300.h; the compute runs in the library's sm_103a kernels.
Importing this module never falls back to a CPU implementation: if the
shared library cannot be loaded, or no GB300 is present, the calls raise.

The Python names mirror the reference's MDSystem API
(src/library/MDSystem.h:104-163): ``System.calculate_forces`` is
CalculateForces + CalculateParameters, ``System.integrate`` is Integrate,
``System.rdf_counts`` fills NdNdr2, and so on.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB_PATH

LJ_OK, LJ_ERR_INVALID, LJ_ERR_CUDA, LJ_ERR_NO_DEVICE = 0, 1, 2, 3
LJ_ERR_DEVICE_TIMEOUT, LJ_ERR_NONFINITE, LJ_ERR_UNSUPPORTED, LJ_ERR_OUT_OF_MEMORY = 4, 5, 6, 7
LJ_ERR_ESCAPED = 8
BC_PERIODIC, BC_WALL, BC_NONE = 0, 1, 2
PREC_MIXED, PREC_FP64 = 0, 1
LATTICE_SC, LATTICE_FCC = 0, 1
RDF_R2_CLAMP, RDF_R2_DROP, RDF_R_LINEAR = 0, 1, 2


class LJError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("lj_gb300 error %d: %s" % (code, msg))
        self.code = code


class Config(C.Structure):
    """lj_config (include/lj_gb300.h)."""
    _fields_ = [("n", C.c_int32), ("temperature", C.c_double), ("density", C.c_double),
                ("canonical", C.c_int32), ("boundary", C.c_int32), ("precision", C.c_int32),
                ("epsilon", C.c_double), ("sigma", C.c_double), ("lattice", C.c_int32),
                ("jitter", C.c_double), ("seed", C.c_uint64), ("block_hint", C.c_int32),
                ("device", C.c_int32), ("autotune", C.c_int32)]


class Observables(C.Structure):
    """lj_observables (include/lj_gb300.h)."""
    _fields_ = [("t", C.c_double), ("K", C.c_double), ("V", C.c_double), ("T", C.c_double),
                ("P", C.c_double), ("U", C.c_double), ("W", C.c_double), ("Pshear", C.c_double),
                ("Tkin_tvn", C.c_double), ("av_U_tot", C.c_double), ("av_T_tot", C.c_double),
                ("av_p_tot", C.c_double), ("av_iters", C.c_int64), ("step", C.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Counter(C.Structure):
    """lj_counter (include/lj_gb300.h): type 0-2 slab, 3 cube, 4-6 |v| component."""
    _fields_ = [("type", C.c_int32), ("nalpha", C.c_int32), ("alpha_step", C.c_double), ("vmax", C.c_double)]


_lib = None
_P = C.c_void_p
_dp = C.POINTER(C.c_double)


def _declare(L):
    sig = {
        "lj_config_default": (C.c_int, [C.POINTER(Config)]),
        "lj_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
        "lj_batch_create": (C.c_int, [C.POINTER(Config), C.c_int32, C.POINTER(_P)]),
        "lj_destroy": (C.c_int, [_P]),
        "lj_last_error": (C.c_char_p, [_P]),
        "lj_get_info": (C.c_int, [_P, C.POINTER(C.c_int32), _dp]),
        "lj_reinitialize": (C.c_int, [_P, C.POINTER(Config)]),
        "lj_set_state": (C.c_int, [_P, _P, _P]),
        "lj_set_state_async": (C.c_int, [_P, _P, _P]),
        "lj_step_io": (C.c_int, [_P, _P, _P, C.c_double, C.c_int32, _P, _P, _P, C.POINTER(Observables)]),
        "lj_get_state": (C.c_int, [_P, _P, _P, _P]),
        "lj_get_pair_sums": (C.c_int, [_P, _P, _P]),
        "lj_compute_forces": (C.c_int, [_P]),
        "lj_step": (C.c_int, [_P, C.c_double, C.c_int32]),
        "lj_sync": (C.c_int, [_P]),
        "lj_get_observables": (C.c_int, [_P, C.POINTER(Observables)]),
        "lj_get_state_observables": (C.c_int, [_P, _P, _P, _P, C.POINTER(Observables)]),
        "lj_batch_observables": (C.c_int, [_P, C.POINTER(Observables)]),
        "lj_batch_info": (C.c_int, [_P, C.POINTER(C.c_int32), _P]),
        "lj_set_recording": (C.c_int, [_P, C.c_int32]),
        "lj_get_records": (C.c_int, [_P, C.POINTER(Observables), C.c_int32, C.POINTER(C.c_int32)]),
        "lj_batch_records": (C.c_int, [_P, C.c_int32, C.POINTER(Observables), C.c_int32, C.POINTER(C.c_int32)]),
        "lj_debug_fail_allocations": (C.c_int, [C.c_int64]),
        "lj_reset_averaging": (C.c_int, [_P]),
        "lj_set_canonical": (C.c_int, [_P, C.c_int32]),
        "lj_set_boundary": (C.c_int, [_P, C.c_int32]),
        "lj_set_temperature": (C.c_int, [_P, C.c_double]),
        "lj_set_time": (C.c_int, [_P, C.c_double]),
        "lj_renormalize_velocities": (C.c_int, [_P, C.c_int32]),
        "lj_renormalize_velocities_to_energy": (C.c_int, [_P, C.c_double]),
        "lj_rdf_counts": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_double, _P]),
        "lj_reference_rdf_dr2": (C.c_float, [C.c_int32]),
        "lj_velocity_counts": (C.c_int, [_P, C.c_double, C.c_int32, _P]),
        "lj_autotune": (C.c_int, [_P]),
        "lj_set_split_cap": (C.c_int, [_P, C.c_int32]),
        "lj_split_info": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "lj_set_kernel_shape": (C.c_int, [_P, C.c_int32]),
        "lj_tune_info": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32,
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "lj_profile_enable": (C.c_int, [_P, C.c_int32]),
        "lj_profile_read": (C.c_int, [_P, C.POINTER(C.c_int64), _dp, C.POINTER(C.c_int64), _dp]),
        "lj_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
        "lj_set_stream": (C.c_int, [_P, _P]),
        "lj_kernel_launch_count": (C.c_int64, [_P]),
        "lj_version": (C.c_char_p, []),
        "lj_sample_initial_state": (C.c_int, [C.POINTER(Config), _P, _P]),
        "lj_host_alloc": (_P, [C.c_size_t]),
        "lj_host_free": (None, [_P]),
        "lj_schedule_plan": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P, _P, _P, C.c_int32]),
        # the reference's own ABI (include/lj_reference_abi.h)
        "allocateArray": (None, [C.POINTER(_P), C.c_int]),
        "deleteArray": (None, [_P]),
        "allocateIntArray": (None, [C.POINTER(_P), C.c_int]),
        "deleteIntArray": (None, [_P]),
        "copyArrayToDevice": (None, [_P, _P, C.c_int]),
        "copyArrayFromDevice": (None, [_P, _P, C.c_uint, C.c_int]),
        "calculateNForces": (None, [_P, _P, C.POINTER(C.c_float), C.c_int, C.c_float, C.c_int, _P,
                                    C.c_float, C.c_int, C.c_int]),
        "threadSync": (None, []),
        "threadExit": (None, []),
        "lj_counters_configure": (C.c_int, [_P, _P, C.c_int32, C.c_int32]),
        "lj_counters_read": (C.c_int, [_P, _P, C.c_int32, C.POINTER(C.c_int32)]),
        "lj_counters_set_interval": (C.c_int, [_P, C.c_int32]),
        "lj_selftest_device_timeout": (C.c_int, [_P]),
        "lj_rdf_accumulate": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_double]),
        "lj_rdf_accumulated": (C.c_int, [_P, _P, C.POINTER(C.c_int64), C.c_int32]),
        "lj_render": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, _P]),
        "lj_adjoint_create": (C.c_int, [C.POINTER(Config), C.c_int32, C.POINTER(_P)]),
        "lj_adjoint_destroy": (C.c_int, [_P]),
        "lj_adjoint_last_error": (C.c_char_p, [_P]),
        "lj_adjoint_set_state": (C.c_int, [_P, _P, _P]),
        "lj_adjoint_set_loss": (C.c_int, [_P, C.c_double, C.c_double, C.c_double]),
        "lj_adjoint_forward": (C.c_int, [_P, C.c_double, C.c_int32, _dp]),
        "lj_adjoint_observables": (C.c_int, [_P, _P, _P, _P, C.c_int32, C.POINTER(C.c_int32)]),
        "lj_adjoint_backward": (C.c_int, [_P, _dp, _dp, _P, _P]),
        "lj_reference_abi_status": (C.c_int, []),
        "lj_reference_abi_error": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def load(build: bool = True) -> C.CDLL:
    """Load liblj_gb300.so (building it first when missing or stale).

    LJGB_LIBRARY=<path> loads another build of the same library instead
    (for example one compiled with different kernel options)."""
    global _lib
    if _lib is None:
        path = os.environ.get("LJGB_LIBRARY")
        if path is None:
            if build:
                _build.build()
            path = LIB_PATH
        if not os.path.exists(path):
            raise OSError("%s not built: run ljgb.build.build()" % path)
        L = C.CDLL(path)
        _declare(L)
        _lib = L
    return _lib


def _check(code: int, handle=None):
    if code != LJ_OK:
        msg = load().lj_last_error(handle)
        raise LJError(code, msg.decode() if msg else "")


def config(**kw) -> Config:
    """lj_config with the reference defaults (MDSystem.h:32-40), overridden by kw."""
    c = Config()
    _check(load().lj_config_default(C.byref(c)))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise AttributeError("lj_config has no field %r" % k)
        setattr(c, k, v)
    return c


def _f64(a, n3):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.size != n3:
        raise ValueError("expected %d values, got %d" % (n3, a.size))
    return a


class PinnedArray(np.ndarray):
    """numpy array over page-locked host memory (lj_host_alloc)."""

    def __del__(self):
        ptr = getattr(self, "_lj_ptr", None)
        if ptr:
            load().lj_host_free(ptr)
            self._lj_ptr = None


def pinned(shape, dtype=np.float64) -> np.ndarray:
    """Page-locked host array for lj_set_state / lj_get_state buffers."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    ptr = load().lj_host_alloc(nbytes)
    if not ptr:
        raise MemoryError("lj_host_alloc(%d) failed" % nbytes)
    buf = (C.c_char * nbytes).from_address(ptr)
    arr = np.frombuffer(buf, dtype=dtype).reshape(shape).view(PinnedArray)
    arr._lj_ptr = ptr
    return arr


def replica_batch_configs(seed: int = 3, k: int = 256):
    """The batched-replicas workload: k boxes with N uniform in [200, 4000),
    rho* in [0.01, 1.1], T* in [0.7, 2.0], periodic and hard-wall boxes
    alternating, FCC + 0.02 sigma jitter, TVN (seeded)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [config(n=int(rng.integers(200, 4000)), density=float(rng.uniform(0.01, 1.1)),
                   temperature=float(rng.uniform(0.7, 2.0)), canonical=1, boundary=i % 2,
                   lattice=LATTICE_FCC, jitter=0.02, seed=1000 + i) for i in range(k)]


def reference_rdf_dr2(n: int) -> float:
    return float(load().lj_reference_rdf_dr2(int(n)))


def write_ppm(path: str, rgba) -> None:
    """Writes an RGBA image (System.render) as a binary PPM (P6) file."""
    rgba = np.asarray(rgba, np.uint8)
    h, w = rgba.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgba[:, :, :3]).tobytes())


def sample_initial_state(cfg: Config):
    """The seeded initial state lj_create samples (host side, no GPU)."""
    pos = np.zeros((cfg.n, 3))
    vel = np.zeros((cfg.n, 3))
    _check(load().lj_sample_initial_state(C.byref(cfg), pos.ctypes.data, vel.ctypes.data))
    return pos, vel


def schedule_plan(n: Sequence[int], block: int, tile: int, ctas: int):
    """Stream-K split of the pair work (host side, no GPU)."""
    n = np.ascontiguousarray(n, np.int32)
    G = C.c_int32()
    nseg = C.c_int32()
    nb = int(sum((int(x) + block - 1) // block for x in n))
    ctb = np.zeros(ctas + 1, np.int32)
    clo = np.zeros(ctas + 1, np.int32)
    info = np.zeros((nb, 8), np.int32)
    _check(load().lj_schedule_plan(n.ctypes.data, len(n), block, tile, ctas, C.byref(G), C.byref(nseg),
                                   ctb.ctypes.data, clo.ctypes.data, info.ctypes.data, nb))
    return dict(ctas=G.value, nseg=nseg.value, cta_tile_begin=ctb[:G.value + 1].copy(),
                cta_lo=clo[:G.value + 1].copy(), blocks=info)


class System:
    """One box (or a batch of boxes) on the GPU: the lj_system handle."""

    def __init__(self, cfg: Optional[Config] = None, batch: Optional[Sequence[Config]] = None, **kw):
        L = load()
        h = _P()
        if batch is not None:
            arr = (Config * len(batch))(*batch)
            _check(L.lj_batch_create(arr, len(batch), C.byref(h)))
            self.nsys = len(batch)
            self.cfgs = list(batch)
        else:
            cfg = cfg if cfg is not None else config(**kw)
            _check(L.lj_create(C.byref(cfg), C.byref(h)))
            self.nsys = 1
            self.cfgs = [cfg]
        self.h = h
        n = C.c_int32()
        box = C.c_double()
        _check(L.lj_get_info(h, C.byref(n), C.byref(box)), h)
        offs = np.zeros(self.nsys + 1, np.int32)
        ns = C.c_int32()
        _check(L.lj_batch_info(h, C.byref(ns), offs.ctypes.data), h)
        self.offsets = offs
        self.ntotal = int(offs[-1])
        self.n = int(n.value)
        self.L = float(box.value)

    # -- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            load().lj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _c(self, code):
        _check(code, self.h)

    # -- state -----------------------------------------------------------
    def set_state(self, pos=None, vel=None):
        n3 = 3 * self.ntotal
        p = _f64(pos, n3) if pos is not None else None
        v = _f64(vel, n3) if vel is not None else None
        self._c(load().lj_set_state(self.h, p.ctypes.data if p is not None else None,
                                    v.ctypes.data if v is not None else None))

    def get_state(self):
        pos = np.zeros((self.ntotal, 3))
        vel = np.zeros((self.ntotal, 3))
        frc = np.zeros((self.ntotal, 3))
        self._c(load().lj_get_state(self.h, pos.ctypes.data, vel.ctypes.data, frc.ctypes.data))
        return pos, vel, frc

    def get_state_into(self, pos=None, vel=None, frc=None):
        """Read state into caller buffers (e.g. pinned host memory)."""
        ptr = lambda a: a.ctypes.data if a is not None else None
        self._c(load().lj_get_state(self.h, ptr(pos), ptr(vel), ptr(frc)))

    def get_state_observables_into(self, pos=None, vel=None, frc=None) -> dict:
        """State into caller buffers plus the observables, one synchronisation."""
        ptr = lambda a: a.ctypes.data if a is not None else None
        o = Observables()
        self._c(load().lj_get_state_observables(self.h, ptr(pos), ptr(vel), ptr(frc), C.byref(o)))
        return o.as_dict()

    def set_state_from(self, pos=None, vel=None):
        ptr = lambda a: a.ctypes.data if a is not None else None
        self._c(load().lj_set_state(self.h, ptr(pos), ptr(vel)))

    def set_state_async_from(self, pos=None, vel=None):
        """lj_set_state_async: queued upload; pos / vel must stay unchanged
        (and alive) until the next synchronising call returns."""
        ptr = lambda a: a.ctypes.data if a is not None else None
        self._c(load().lj_set_state_async(self.h, ptr(pos), ptr(vel)))

    def step_io(self, dt: float, nsteps: int = 1, pos_in=None, vel_in=None, pos_out=None, vel_out=None,
                frc_out=None) -> dict:
        """lj_step_io: queued upload of pos_in / vel_in, nsteps steps, the
        state into the *_out buffers and the observables, one
        synchronisation.  Inputs must stay alive and unchanged until it
        returns (it returns after the synchronisation)."""
        ptr = lambda a: a.ctypes.data if a is not None else None
        o = Observables()
        self._c(load().lj_step_io(self.h, ptr(pos_in), ptr(vel_in), float(dt), int(nsteps), ptr(pos_out),
                                  ptr(vel_out), ptr(frc_out), C.byref(o)))
        return o.as_dict()

    def pair_sums(self):
        e = np.zeros(self.ntotal)
        w = np.zeros(self.ntotal)
        self._c(load().lj_get_pair_sums(self.h, e.ctypes.data, w.ctypes.data))
        return e, w

    # -- dynamics --------------------------------------------------------
    def calculate_forces(self):
        self._c(load().lj_compute_forces(self.h))

    def integrate(self, dt: float, nsteps: int = 1):
        self._c(load().lj_step(self.h, float(dt), int(nsteps)))

    def sync(self):
        self._c(load().lj_sync(self.h))

    def observables(self) -> dict:
        o = Observables()
        self._c(load().lj_get_observables(self.h, C.byref(o)))
        return o.as_dict()

    def batch_observables(self):
        arr = (Observables * self.nsys)()
        self._c(load().lj_batch_observables(self.h, arr))
        return [a.as_dict() for a in arr]

    def set_recording(self, cap: int):
        self._c(load().lj_set_recording(self.h, int(cap)))

    def records(self, max_records: int = 1 << 20):
        arr = (Observables * max_records)()
        cnt = C.c_int32()
        self._c(load().lj_get_records(self.h, arr, max_records, C.byref(cnt)))
        return [arr[k].as_dict() for k in range(cnt.value)]

    def batch_records(self, box: int, max_records: int = 1 << 20):
        arr = (Observables * max_records)()
        cnt = C.c_int32()
        self._c(load().lj_batch_records(self.h, int(box), arr, max_records, C.byref(cnt)))
        return [arr[k].as_dict() for k in range(cnt.value)]

    def reset_averaging(self):
        self._c(load().lj_reset_averaging(self.h))

    def set_canonical(self, on: bool):
        self._c(load().lj_set_canonical(self.h, int(bool(on))))

    def set_boundary(self, bc: int):
        self._c(load().lj_set_boundary(self.h, int(bc)))

    def set_temperature(self, T0: float):
        self._c(load().lj_set_temperature(self.h, float(T0)))

    def set_time(self, t: float):
        self._c(load().lj_set_time(self.h, float(t)))

    def renormalize_velocities(self, recalc: bool = True):
        self._c(load().lj_renormalize_velocities(self.h, int(bool(recalc))))

    def renormalize_velocities_to_energy(self, ust: float):
        self._c(load().lj_renormalize_velocities_to_energy(self.h, float(ust)))

    # -- histograms ------------------------------------------------------
    def rdf_counts(self, mode: int = RDF_R2_CLAMP, nbins: int = 256, width: Optional[float] = None):
        if width is None:
            width = reference_rdf_dr2(self.n)
        out = np.zeros(nbins, np.uint64)
        self._c(load().lj_rdf_counts(self.h, int(mode), int(nbins), float(width), out.ctypes.data))
        return out

    def velocity_counts(self, step: float = 0.12, nbins: int = 101):
        out = np.zeros(nbins, np.uint64)
        self._c(load().lj_velocity_counts(self.h, float(step), int(nbins), out.ctypes.data))
        return out

    # -- tuning / profiling ----------------------------------------------
    def autotune(self):
        self._c(load().lj_autotune(self.h))

    def counters_configure(self, counters, ring_steps: int = 1000):
        """counters: sequence of (type, nalpha, alpha_step, vmax)."""
        arr = (Counter * max(1, len(counters)))(*[Counter(*c) for c in counters])
        self.counter_bins = sum(int(c[1]) for c in counters)
        self._c(load().lj_counters_configure(self.h, arr, len(counters), int(ring_steps)))

    def selftest_device_timeout(self):
        """Runs a device wait that nothing completes; raises unless its
        timeout was reported (the handle stays usable)."""
        self._c(load().lj_selftest_device_timeout(self.h))

    def counters_set_interval(self, every: int):
        """Count after every `every`-th step only."""
        self._c(load().lj_counters_set_interval(self.h, int(every)))

    def counters_read(self, max_steps: int = 1 << 20):
        n = C.c_int32()
        self._c(load().lj_counters_read(self.h, None, 0, C.byref(n)))
        m = min(n.value, max_steps)
        out = np.zeros((m, self.counter_bins), np.int32)
        self._c(load().lj_counters_read(self.h, out.ctypes.data, m, C.byref(n)))
        return out[:n.value]

    def rdf_accumulate(self, enable: bool, mode: int = 2, nbins: int = 200, width: float = 0.05):
        self._rdf_nbins = nbins
        self._c(load().lj_rdf_accumulate(self.h, int(bool(enable)), mode, nbins, width))

    def rdf_accumulated(self, reset: bool = False):
        out = np.zeros(self._rdf_nbins, np.uint64)
        n = C.c_int64()
        self._c(load().lj_rdf_accumulated(self.h, out.ctypes.data, C.byref(n), int(bool(reset))))
        return out, n.value

    def render(self, box: int = 0, axis: int = 2, width: int = 512, height: int = 512, radius: float = 0.5):
        """Headless particle image (lj_render): (height, width, 4) uint8 RGBA."""
        img = np.zeros((height, width, 4), np.uint8)
        self._c(load().lj_render(self.h, box, axis, width, height, radius, img.ctypes.data))
        return img

    def set_kernel_shape(self, shape: int):
        self._c(load().lj_set_kernel_shape(self.h, int(shape)))

    def tune_info(self):
        ns, act = C.c_int32(), C.c_int32()
        shapes = []
        L = load()
        self._c(L.lj_tune_info(self.h, C.byref(ns), C.byref(act), -1, None, None, None))
        for k in range(ns.value):
            th, ipt, tl = C.c_int32(), C.c_int32(), C.c_int32()
            self._c(L.lj_tune_info(self.h, None, None, k, C.byref(th), C.byref(ipt), C.byref(tl)))
            shapes.append(dict(threads=th.value, ipt=ipt.value, tile=tl.value))
        cap, ctas, segs = C.c_int32(), C.c_int32(), C.c_int32()
        self._c(L.lj_split_info(self.h, C.byref(cap), C.byref(ctas), C.byref(segs)))
        return dict(active=act.value, shapes=shapes, split_cap=cap.value, ctas=ctas.value,
                    max_segments=segs.value)

    def set_split_cap(self, cap: int):
        """Most CTAs (threads per particle) an i-block's j range is cut over;
        0 restores the default, which lj_autotune searches."""
        self._c(load().lj_set_split_cap(self.h, int(cap)))

    def profile(self, on: bool):
        self._c(load().lj_profile_enable(self.h, int(bool(on))))

    def profile_read(self):
        pl, st = C.c_int64(), C.c_int64()
        pm, sm = C.c_double(), C.c_double()
        self._c(load().lj_profile_read(self.h, C.byref(pl), C.byref(pm), C.byref(st), C.byref(sm)))
        return dict(pair_launches=pl.value, pair_ms=pm.value, steps=st.value, step_ms=sm.value)

    def stream(self) -> int:
        p = _P()
        self._c(load().lj_get_stream(self.h, C.byref(p)))
        return p.value or 0

    def set_stream(self, ptr: Optional[int]):
        self._c(load().lj_set_stream(self.h, ptr))

    def launch_count(self) -> int:
        return int(load().lj_kernel_launch_count(self.h))


class Adjoint:
    """Differentiable trajectory loss (lj_adjoint_*): FP64 forward pass with
    checkpoints and the discrete adjoint (force Hessian-vector products on
    the GPU).  loss = (1/S) sum_m [wK K_m/N + wV V_m/N + wP P_m]."""

    def __init__(self, cfg: Optional[Config] = None, checkpoint_every: int = 20, **kw):
        L = load()
        cfg = cfg if cfg is not None else config(**kw)
        h = _P()
        code = L.lj_adjoint_create(C.byref(cfg), int(checkpoint_every), C.byref(h))
        if code != LJ_OK:
            raise LJError(code, "lj_adjoint_create failed")
        self.h = h
        self.cfg = cfg
        self.n = cfg.n

    def _c(self, code):
        if code != LJ_OK:
            msg = load().lj_adjoint_last_error(self.h)
            raise LJError(code, msg.decode() if msg else "")

    def set_state(self, pos, vel):
        p = _f64(pos, 3 * self.n)
        v = _f64(vel, 3 * self.n)
        self._c(load().lj_adjoint_set_state(self.h, p.ctypes.data, v.ctypes.data))

    def set_loss(self, w_kinetic=0.0, w_potential=1.0, w_pressure=1.0):
        self._c(load().lj_adjoint_set_loss(self.h, w_kinetic, w_potential, w_pressure))

    def forward(self, dt: float, nsteps: int) -> float:
        out = C.c_double()
        self._c(load().lj_adjoint_forward(self.h, dt, int(nsteps), C.byref(out)))
        return out.value

    def observables(self):
        cnt = C.c_int32()
        self._c(load().lj_adjoint_observables(self.h, None, None, None, 0, C.byref(cnt)))
        K, V, W = (np.zeros(cnt.value) for _ in range(3))
        self._c(load().lj_adjoint_observables(self.h, K.ctypes.data, V.ctypes.data, W.ctypes.data, cnt.value, None))
        return dict(K=K, V=V, W=W)

    def backward(self):
        de, ds = C.c_double(), C.c_double()
        dp = np.zeros((self.n, 3))
        dv = np.zeros((self.n, 3))
        self._c(load().lj_adjoint_backward(self.h, C.byref(de), C.byref(ds), dp.ctypes.data, dv.ctypes.data))
        return de.value, ds.value, dp, dv

    def close(self):
        if getattr(self, "h", None):
            load().lj_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
