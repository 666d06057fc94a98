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
    ([16384], 128, 256, 1216), ([16384], 128, 256, 1824), ([400], 128, 256, 1824),
    ([1000, 37, 4000, 200], 64, 256, 608), ([5], 128, 256, 1824), ([262144], 128, 256, 1824),
    ([777], 256, 512, 300), ([1000, 37, 4000, 200], 128, 512, 2000),
    ([16384], 384, 512, 304), ([262144], 384, 512, 304), ([1000, 37, 4000, 200], 384, 512, 304)])
def test_schedule_covers_every_pair_once(ljlib, n, block, tile, ctas):
    """Every (i-block, j) belongs to exactly one CTA, CTA ranges are cut on
    32-record chunks, each (CTA, block) pair has its own segment in the
    block's range, and the work per CTA is equal to within about one chunk."""
    import ljgb
    grain = 32
    s = ljgb.schedule_plan(n, block, tile, ctas)
    G, ctb, clo, blocks = s["ctas"], s["cta_tile_begin"], s["cta_lo"], s["blocks"]
    assert G <= ctas and ctb[0] == 0 and clo[0] == 0 and clo[G] == 0
    njt = blocks[:, 4]
    nsys = np.array([n[k] for k in blocks[:, 0]])
    assert ctb[-1] == njt.sum()
    assert np.all(clo % grain == 0) and np.all((clo >= 0) & (clo < tile))
    tile_first = np.concatenate([[0], np.cumsum(njt)])
    chunk_first = np.concatenate([[0], np.cumsum((nsys + grain - 1) // grain)])
    # global chunk index of each CTA's first j: strictly increasing, 0 .. total
    bstart = np.searchsorted(tile_first, ctb[:G], side="right") - 1
    jstart = (ctb[:G] - tile_first[bstart]) * tile + clo[:G]
    assert np.all(jstart < nsys[bstart])
    C = np.concatenate([chunk_first[bstart] + jstart // grain, [chunk_first[-1]]])
    assert C[0] == 0 and np.all(np.diff(C) >= 1)
    # segments: CTAs meeting block b are g_first .. g_first + seg_count - 1
    seg_first, seg_count, g_first = blocks[:, 5], blocks[:, 6], blocks[:, 7]
    assert seg_first[0] == 0 and np.all(seg_first[1:] == seg_first[:-1] + seg_count[:-1])
    assert s["nseg"] == seg_first[-1] + seg_count[-1]
    for b in range(len(blocks)):
        meet = np.nonzero((C[:-1] < chunk_first[b + 1]) & (C[1:] > chunk_first[b]))[0]
        assert meet[0] == g_first[b] and len(meet) == seg_count[b] and np.all(np.diff(meet) == 1)
    # the kernel's walk of each CTA (small cases) lands on the same j ranges
    if G * 8 < 20000:
        cover = {}
        for g in range(G):
            t0, t1, lo0, lo1 = ctb[g], ctb[g + 1], clo[g], clo[g + 1]
            ntiles = t1 - t0 + (1 if lo1 > 0 else 0)
            b = int(np.searchsorted(tile_first, t0, side="right") - 1)
            jt = t0 - tile_first[b]
            for k in range(ntiles):
                cnt = min(tile, nsys[b] - jt * tile)
                jlo = lo0 if k == 0 else 0
                jhi = lo1 if (k == ntiles - 1 and lo1 > 0) else cnt
                assert 0 <= jlo < jhi <= cnt
                cover.setdefault(b, []).append((jt * tile + jlo, jt * tile + jhi))
                if jt + 1 == njt[b]:
                    b, jt = b + 1, 0
                else:
                    jt += 1
        for b in range(len(blocks)):
            iv = sorted(cover[b])
            assert iv[0][0] == 0 and iv[-1][1] == nsys[b]
            assert all(iv[k][1] == iv[k + 1][0] for k in range(len(iv) - 1))
    # balance in cost units (j records + 8 per tile started): within ~2 chunks
    cost_first = np.concatenate([[0], np.cumsum(nsys + njt * 8)])
    def cost_at(c):
        b = np.searchsorted(chunk_first, c, side="right") - 1
        b = np.minimum(b, len(blocks) - 1)
        j = np.minimum((c - chunk_first[b]) * grain, nsys[b])
        return cost_first[b] + j + (j + tile - 1) // tile * 8
    cost = np.diff(cost_at(C))
    assert cost.max() <= cost.mean() + 2 * (grain + 8)


@pytest.mark.parametrize("n", [200, 1500, 3001, 7777, 16384])
@pytest.mark.parametrize("cap", [1, 2, 3, 8, 32])
def test_split_cap_bounds_threads_per_particle(ljlib, n, cap):
    """A handle with split cap k runs min(SMs x resident CTAs, k x i-blocks)
    CTAs.  Every i-block of one box costs the same (all j), so the equal-cost
    cuts give no block more than k segments: at most k threads per particle."""
    import ljgb
    nbt = (n + 127) // 128
    for tile in (256, 512):
        s = ljgb.schedule_plan([n], 128, tile, min(912, nbt * cap))
        seg = s["blocks"][:, 6]
        assert seg.max() <= cap and seg.min() >= 1


def test_schedule_rejects_bad_input(ljlib):
    import ljgb
    with pytest.raises(ljgb.LJError):
        ljgb.schedule_plan([0], 128, 256, 10)
