"""The MDSystem C++ class (include/ljgb/MDSystem.hpp) used the way the
reference's task drivers use it: compiled against the header and linked to
liblj_gb300.so (CPU: compile/link; GPU: run and check the physics)."""
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "facade", "facade_driver.cpp")


def build_driver(ljlib, tmp_path):
    exe = str(tmp_path / "facade_driver")
    libdir = os.path.dirname(ljlib._name)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), SRC, "-o", exe,
                           "-L", libdir, "-llj_gb300", "-Wl,-rpath," + libdir])
    return exe


def test_driver_compiles_and_links(ljlib, tmp_path):
    exe = build_driver(ljlib, tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_driver_runs(ljlib, tmp_path):
    exe = build_driver(ljlib, tmp_path)
    out = subprocess.run([exe, "200"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = {}
    for line in out.stdout.splitlines():
        head, *kv = line.split()
        lines[head] = dict(x.split("=", 1) for x in kv if "=" in x)
    init, tvn, evn, rdf, velo, multi = (lines[k] for k in ("init", "tvn", "evn", "rdf", "velo", "multi"))
    assert float(init["T"]) == pytest.approx(1.312, rel=1e-9)          # exact-T0 initial state
    assert float(init["L"]) == pytest.approx((512 / 0.316) ** (1 / 3), rel=1e-9)
    assert float(tvn["T"]) == pytest.approx(1.312, rel=0.02)          # TVN holds T near T0
    assert int(tvn["av_iters"]) == 200
    assert int(evn["av_iters"]) == 200
    assert abs(float(evn["<T>"]) - 1.312) < 0.2
    assert int(rdf["total"]) == 512 * 511                             # every ordered pair binned (clamp rule)
    assert 1.0 < float(rdf["peak_r"]) < 1.3                            # first shell of the LJ fluid
    assert float(velo["norm"]) == pytest.approx(1.0, abs=0.02)        # velocity density integrates to ~1
    assert float(multi["t"]) == pytest.approx(0.005 * 450, rel=1e-9)
    assert int(multi["av_iters"]) == 250
