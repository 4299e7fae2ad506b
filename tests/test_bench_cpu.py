"""bench.py's host side: the CPU reference arm prints one valid JSON line, alone and as rank 0 of
a two-rank gloo job (the other rank exits without work)."""
import json
import os
import subprocess
import sys

from conftest import ROOT

REQUIRED = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
            "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}


def run(cmd, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=e)


def test_reference_arm_prints_one_line():
    r = run([sys.executable, "bench.py", "--impl", "reference", "--bodies", "16", "--steps", "1", "--warmup", "1"])
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert REQUIRED <= set(d)
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"


def test_reference_arm_two_ranks_gloo():
    r = run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
             "--master-addr", "127.0.0.1", "--master-port", "29531", "bench.py", "--impl", "reference",
             "--gpus", "2", "--bodies", "16", "--steps", "1", "--warmup", "1"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    assert json.loads(lines[0])["n_gpus"] == 2


def test_rank_reductions_gloo(tmp_path):
    """max / sum over ranks used for the timed region, on two gloo ranks."""
    code = r'''
import os, sys
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r = dist.get_rank()
assert bench.max_over_ranks(dist, 1.0 + r) == 2.0
assert bench.sum_over_ranks(dist, 10.0 * (r + 1)) == 30.0
dist.destroy_process_group()
''' % ROOT
    script = tmp_path / "reduce.py"
    script.write_text(code)
    r = run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
             "--master-addr", "127.0.0.1", "--master-port", "29532", str(script)])
    assert r.returncode == 0, r.stderr[-2000:]


def test_threaded_oracle_batch_equals_single_runs():
    """The CPU baseline's threaded batch (oracle.simulate_batch: one body per task on host
    threads) gives each body bitwise what a single run of the restatement gives."""
    import numpy as np

    import oracle
    from bounce_softbody_gb300 import meshes

    descs = meshes.batch_bodies(count=5, lo=3, hi=7, seed=2)
    xs, vs, its, _ = oracle.simulate_batch(descs, 3, bits=32, threads=3)
    for d, x, v, it in zip(descs, xs, vs, its):
        xr, vr, itr, _ = oracle.simulate(d, 3, kind="port", bits=32)
        assert np.array_equal(x, xr) and np.array_equal(v, vr) and np.array_equal(it, itr), d.name
