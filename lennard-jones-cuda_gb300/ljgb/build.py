"""In-tree build of liblj_gb300.so for sm_103a.

Each translation unit is compiled by nvcc in parallel (one -gencode, no
cmake), then linked into a shared library next to this package:
lennard-jones-cuda_gb300/liblj_gb300.so.  The library exports the C ABI of
include/lj_gb300.h and include/lj_reference_abi.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # lennard-jones-cuda_gb300/
REPO = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "liblj_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [
    "lj_pairs.cu",
    "lj_integrate.cu",
    "lj_compat.cu",
    "lj_noalloc.cu",
    "lj_adjoint.cu",
    "lj_render.cu",
    "lj_system.cpp",
    "lj_schedule.cpp",
    "lj_init.cpp",
    "MDSystem.cpp",
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _flags():
    extra = os.environ.get("LJGB_NVCC_FLAGS", "").split()
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE, "-I", CSRC,
                   "-Xptxas", "-warn-spills"] + extra


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc()] + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"] if src.endswith(".cu") else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    for d in (CSRC, INCLUDE, os.path.join(PKG_DIR, "tasks")):
        for root, _, files in os.walk(d):
            for f in files:
                if os.path.getmtime(os.path.join(root, f)) > t:
                    return True
    return os.path.getmtime(os.path.abspath(__file__)) > t


def build(force: bool = False, verbose: bool = False, out: str = None, build_dir: str = None) -> str:
    """Compile the CUDA/C++ sources into liblj_gb300.so (skipped when fresh).

    out / build_dir place a variant build elsewhere (extra nvcc flags come
    from LJGB_NVCC_FLAGS)."""
    global BUILD_DIR
    lib_path = out or LIB_PATH
    if out is None and not force and not _stale():
        return LIB_PATH
    saved = BUILD_DIR
    BUILD_DIR = build_dir or BUILD_DIR
    try:
        return _build_into(lib_path, verbose)
    finally:
        BUILD_DIR = saved


def _build_into(lib_path: str, verbose: bool) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = lib_path + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib_path)
    if lib_path == LIB_PATH:
        build_tasks()
    return lib_path


TASKS = {"ljgb-run-isotherm": "run_isotherm.cpp", "ljgb-run-fluctuations": "run_fluctuations.cpp",
         "ljgb-semiGCEfluctuations": "run_semigce_fluctuations.cpp"}
TASK_DIR = os.path.join(PKG_DIR, "tasks")
BIN_DIR = os.path.join(PKG_DIR, "bin")


def build_tasks() -> list:
    """The task-driver executables (C++ over the lj_* ABI), next to the
    library in lennard-jones-cuda_gb300/bin/."""
    os.makedirs(BIN_DIR, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    outs = []

    def one(item):
        name, src = item
        out = os.path.join(BIN_DIR, name)
        cmd = [cxx, "-std=c++17", "-O2", "-I", INCLUDE, os.path.join(TASK_DIR, src), "-o", out, "-L", PKG_DIR,
               "-llj_gb300", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("task build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return out

    with cf.ThreadPoolExecutor(max_workers=len(TASKS)) as ex:
        outs = list(ex.map(one, TASKS.items()))
    return outs


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
