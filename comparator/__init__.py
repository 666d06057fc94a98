"""Timing comparator: the reference's GPU force kernel restated for GB300
(comparator/ref_nbody.cu, after src/library/MDSystem.cu:21-153).

Measurement infrastructure only, kept outside the product package: the
bench reports its time beside the library's pair kernel, and one GPU test
checks it against the FP64 oracle.  liblj_gb300.so neither links nor calls
it.  build() compiles it for sm_103a into comparator/libljref_nbody.so.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ref_nbody.cu")
LIB_PATH = os.path.join(HERE, "libljref_nbody.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17", "-Xcompiler",
           "-fPIC", "-shared", SRC, "-o", tmp, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("comparator build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def load() -> C.CDLL:
    """The comparator library with its entry points declared."""
    lib = C.CDLL(build())
    lib.ljref_scratch_bytes.restype = C.c_size_t
    lib.ljref_scratch_bytes.argtypes = [C.c_int, C.c_int]
    lib.ljref_forces.restype = C.c_int
    lib.ljref_forces.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_int, C.c_float, C.c_int,
                                 C.c_void_p, C.c_void_p]
    lib.ljref_results.restype = C.c_int
    lib.ljref_results.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return lib
