"""The C ABI without a GPU: exported symbols, host-side sampler and the
stream-K schedule (CPU-only tests)."""
import ctypes
import glob
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    """Function names declared in include/*.h (C declarations only)."""
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{]*)\)\s*;", src):
            name = m.group(1)
            if name in ("if", "while", "for", "return", "sizeof"):
                continue
            names.add(name)
    return sorted(names)


def test_headers_declare_the_reference_abi():
    names = declared_functions()
    for ref in ("calculateNForces", "allocateArray", "deleteArray", "copyArrayToDevice",
                "copyArrayFromDevice", "threadExit", "threadSync", "allocateNBodyArrays",
                "deleteNBodyArrays", "registerGLBufferObject", "unregisterGLBufferObject"):
        assert ref in names
    assert "lj_create" in names and "lj_step" in names


def test_library_exports_every_declared_symbol(ljlib):
    out = subprocess.run(["nm", "-D", "--defined-only", ljlib._name], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert hasattr(ljlib, n)


def test_config_defaults_match_reference(ljlib):
    import ljgb
    c = ljgb.config()
    # MDSystemConfiguration() defaults (MDSystem.h:32-40)
    assert (c.n, c.temperature, c.density, c.canonical, c.boundary) == (128, 1.5, 0.2, 0, 0)
    assert (c.epsilon, c.sigma) == (1.0, 1.0)


def test_reference_rdf_bin_width(ljlib, oracle_mod):
    import ljgb
    for n in (50, 100, 128, 400, 1000, 16384):
        assert ljgb.reference_rdf_dr2(n) == oracle_mod.lib().r32_rdf_dr2(n)


def test_invalid_config_is_rejected_without_exit(ljlib):
    import ljgb
    for kw in (dict(n=1), dict(density=0.0), dict(boundary=3), dict(precision=7), dict(sigma=-1.0)):
        with pytest.raises(ljgb.LJError) as e:
            ljgb.System(**kw)
        assert e.value.code == ljgb.LJ_ERR_INVALID


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="checks the no-GPU error path")
def test_create_without_gpu_reports_no_device(ljlib):
    import ljgb
    with pytest.raises(ljgb.LJError) as e:
        ljgb.System(n=64)
    assert e.value.code == ljgb.LJ_ERR_NO_DEVICE


@pytest.mark.parametrize("lattice", [0, 1])
def test_initial_state_properties(ljlib, lattice):
    import ljgb
    c = ljgb.config(n=500, temperature=1.3, density=0.8, lattice=lattice, jitter=0.05, seed=11)
    pos, vel = ljgb.sample_initial_state(c)
    L = (500 / 0.8) ** (1 / 3)
    assert np.all(pos > -0.05 - 1e-12) and np.all(pos < L + 0.05 + 1e-12)
    assert np.abs(vel.sum(0)).max() < 1e-10                       # zero momentum
    assert np.sum(vel * vel) / 3 / 500 == pytest.approx(1.3, rel=1e-13)  # exact T0
    pos2, vel2 = ljgb.sample_initial_state(c)
    assert np.array_equal(pos, pos2) and np.array_equal(vel, vel2)  # seeded
    c.seed = 12
    pos3, _ = ljgb.sample_initial_state(c)
    assert not np.array_equal(pos, pos3)
    # lattice sites without jitter are distinct and at least a lattice spacing apart
    c.jitter = 0.0
    p0, _ = ljgb.sample_initial_state(c)
    d = p0[:, None, :] - p0[None, :, :]
    r = np.sqrt((d * d).sum(-1)) + np.eye(500) * 1e9
    assert r.min() > 0.5


def test_initial_speeds_are_maxwellian(ljlib):
    import ljgb
    c = ljgb.config(n=20000, temperature=1.0, density=0.5, seed=3)
    _, vel = ljgb.sample_initial_state(c)
    s = np.sqrt((vel * vel).sum(1))
    # Maxwell at T=1: <v> = sqrt(8/pi), <v^2> = 3
    assert s.mean() == pytest.approx(np.sqrt(8 / np.pi), rel=0.02)
    assert np.mean(s ** 2) == pytest.approx(3.0, rel=1e-12)


@pytest.mark.parametrize("n,block,tile,ctas", [
    ([16384], 128, 256, 1824), ([400], 128, 256, 1824), ([1000, 37, 4000, 200], 64, 256, 608),
    ([5], 128, 256, 1824), ([262144], 128, 256, 1824), ([777], 256, 512, 300)])
def test_schedule_covers_every_pair_once(ljlib, n, block, tile, ctas):
    import ljgb
    s = ljgb.schedule_plan(n, block, tile, ctas)
    G, ctb, blocks = s["ctas"], s["cta_tile_begin"], s["blocks"]
    assert G <= ctas and ctb[0] == 0 and np.all(np.diff(ctb) >= 1)
    njt = blocks[:, 4]
    assert ctb[-1] == njt.sum()
    # every (block, tile) belongs to exactly one CTA, and the segment of (g, b)
    # = seg_first[b] + g - g_first[b] is unique and inside the block's range
    tile_first = np.concatenate([[0], np.cumsum(njt)])
    seen = set()
    for g in range(G):
        for t in range(ctb[g], ctb[g + 1]):
            b = int(np.searchsorted(tile_first, t, side="right") - 1)
            seg = blocks[b, 5] + g - blocks[b, 7]
            assert blocks[b, 5] <= seg < blocks[b, 5] + blocks[b, 6]
            seen.add((b, seg))
    assert len({sg for _, sg in seen}) == s["nseg"]
    # balance: the costliest CTA is within two tiles of the mean
    cost = []
    for g in range(G):
        c = 0
        for t in range(ctb[g], ctb[g + 1]):
            b = int(np.searchsorted(tile_first, t, side="right") - 1)
            jt = t - tile_first[b]
            nsys = n[blocks[b, 0]]
            c += min(tile, nsys - jt * tile) + 8
        cost.append(c)
    assert max(cost) <= np.mean(cost) + 2 * (tile + 8)


def test_schedule_rejects_bad_input(ljlib):
    import ljgb
    with pytest.raises(ljgb.LJError):
        ljgb.schedule_plan([0], 128, 256, 10)
