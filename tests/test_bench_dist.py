"""The multi-GPU (replica) logic of bench.py on CPU: two gloo ranks agree on
the slowest rank's time, the whole-job value counts every rank's box, and the
reference arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [120.0, 250.0][rank]
    slowest = bench.max_over_ranks(local_ms, "cpu")
    value = bench.replica_value(world, 16384 * 16383, 200, slowest)
    torch.distributed.barrier()
    torch.distributed.destroy_process_group()
    out.put((rank, slowest, value))


def test_two_rank_max_and_value():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [250.0, 250.0]
    assert res[0][2] == res[1][2] == pytest.approx(2 * 16384 * 16383 * 200 / 0.250)


def test_reference_arm_runs_on_rank_zero_only():
    import sys
    sys.path.insert(0, REPO)
    import bench

    class A:
        steps, warmup = 1, 1
    assert bench.reference_arm(A(), rank=1, world=2) is None


def test_clock_samples_kept_only_inside_the_timed_region():
    """bench.ClockSampler summarises the nvidia-smi lines stamped between the
    start and the end of the timed region (plus one sampling interval): the
    median SM clock, the maximum, and any throttle reason seen active."""
    import sys
    sys.path.insert(0, REPO)
    import bench
    c = bench.ClockSampler(0)
    c.t_begin, c.t_end = 10.0, 11.0
    line = "0, {sm}, 2070, 900.5, 0x0, {hw}, Not Active, Not Active, {pc}"
    c.lines = [
        (9.5, line.format(sm=800, hw="Active", pc="Not Active")),       # before: ignored
        (10.1, line.format(sm=2070, hw="Not Active", pc="Not Active")),
        (10.5, line.format(sm=2055, hw="Not Active", pc="Active")),
        (11.01, line.format(sm=2070, hw="Not Active", pc="Not Active")),  # within one interval after
        (11.5, line.format(sm=700, hw="Active", pc="Not Active")),      # after: ignored
        (10.7, "garbage"),
    ]
    s = c.summary()
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["region_s"] == pytest.approx(1.0)


def test_reference_arm_line_without_the_product_library():
    """`bench.py --impl reference` (rank 0, one process): K timed steps and W
    warm-up steps as asked, the same config as the GPU arm, and the product
    library never loaded into the process."""
    import json
    import subprocess
    import sys
    code = ("import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '3', '--warmup', '1'];"
            "sys.path.insert(0, %r); import bench; bench.main();"
            "maps = open('/proc/self/maps').read();"
            "print(json.dumps({'lj_loaded': 'liblj_gb300' in maps, 'ljgb_imported': 'ljgb' in sys.modules}))"
            % REPO)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[-1]
    import bench
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 1
    assert line["config"] == bench.bench_config(1)
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert probe == {"lj_loaded": False, "ljgb_imported": False}
