"""The drop-in claim at the C ABI (CPU test): the reference's own, unmodified
src/library/MDSystem.cpp and splinefunction.cpp, compiled with
-DUSE_CUDA_TOOLKIT as its CMake build does (CMakeLists.txt:31), link against
liblj_gb300.so with no unresolved symbol, and the extern "C" block they
declare (MDSystem.cpp:9-25) agrees, declaration by declaration, with
include/lj_reference_abi.h.

The reference sources are read where they lie (LJ_REFERENCE_DIR, or a
checkout named "reference" beside this repository); the test is skipped
where they are absent.  Nothing of them is copied into the repository: the
declaration block is extracted into the test's temporary directory.
"""
import os
import re
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ref_dir():
    import oracle
    d = oracle.reference_dir(os.environ.get("LJ_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO), "reference"))
    if d is None:
        pytest.skip("reference sources not available")
    return d


def _extern_c_block(ref):
    """The declarations MDSystem.cpp makes under USE_CUDA_TOOLKIT."""
    src = open(os.path.join(ref, "src", "library", "MDSystem.cpp")).read()
    m = re.search(r"#ifdef USE_CUDA_TOOLKIT\s*(extern \"C\"\s*\{.*?\})\s*#else", src, re.S)
    assert m, "extern \"C\" block not found in MDSystem.cpp"
    return m.group(1)


def test_reference_declarations_match_header(tmp_path):
    """A C function declared twice with different parameter types is a
    compile error in C++ ("conflicting declaration of C function"): the
    header followed by the reference's own block compiles cleanly only if
    every signature agrees."""
    ref = _ref_dir()
    block = _extern_c_block(ref)
    names = re.findall(r"\b(\w+)\s*\(", re.sub(r"//[^\n]*", "", block))
    assert {"allocateArray", "deleteArray", "calculateNForces", "copyArrayFromDevice", "copyArrayToDevice",
            "threadExit"} <= set(names)
    header = open(os.path.join(REPO, "include", "lj_reference_abi.h")).read()
    for n in names:
        assert re.search(r"\b%s\s*\(" % n, header), "%s is declared by the reference but not by the header" % n
    tu = tmp_path / "decl_check.cpp"
    tu.write_text('#include "lj_reference_abi.h"\n' + block + "\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Werror", "-I", os.path.join(REPO, "include"),
                        str(tu)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_mdsystem_links_against_library(ljlib, tmp_path):
    ref = _ref_dir()
    lib = os.path.join(ref, "src", "library")
    libdir = os.path.dirname(ljlib._name)
    exe = str(tmp_path / "reference_on_gb300")
    cmd = ["g++", "-std=c++11", "-O2", "-w", "-DUSE_CUDA_TOOLKIT", "-I", lib, "-I", os.path.join(ref, "thirdparty"),
           os.path.join(lib, "MDSystem.cpp"), os.path.join(lib, "splinefunction.cpp"),
           os.path.join(REPO, "tests", "dropin", "dropin_main.cpp"), "-o", exe,
           "-L", libdir, "-llj_gb300", "-Wl,-rpath," + libdir, "-Wl,--no-undefined",
           "-Wl,--no-allow-shlib-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # every CUDA entry point the reference object needs is defined by the
    # library (not by the C++ runtime or left to the loader)
    und = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
    nm = subprocess.run(["nm", "-D", "--defined-only", ljlib._name], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in nm.splitlines() if line.strip()}
    for sym in ("allocateArray", "deleteArray", "calculateNForces", "copyArrayFromDevice", "copyArrayToDevice",
                "threadExit"):
        assert re.search(r"\b%s\b" % sym, und), sym
        assert sym in exported, sym
