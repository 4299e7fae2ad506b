"""bench.py's host side: the CPU reference arm prints one valid JSON line, alone and as rank 0 of
a two-rank gloo job (the other rank exits without work); the rank reductions; the split of one
body list over ranks by device footprint and the per-rank stats gather on two gloo ranks; the
algorithmic byte counts of the rooflines."""
import json
import os
import subprocess
import sys

import pytest

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


def test_split_over_two_ranks_gloo(tmp_path):
    """bench.py --split on two gloo ranks: every rank computes the same footprint split of one body
    list (host only), the shares are disjoint and cover the list, the estimated bytes per rank are
    balanced to within the largest body, and the per-rank stats gather reaches every rank."""
    code = r'''
import os, sys
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
from bounce_softbody_gb300 import b3g, meshes
dist.init_process_group("gloo")
r, w = dist.get_rank(), dist.get_world_size()
descs = meshes.batch_bodies(24, lo=4, hi=14, seed=3)
mine, per_rank = bench.split_workload(descs, w, r)
shares = bench.gather_rank_stats(dist, {"rank": r, "bodies": mine, "per_rank": per_rank}, w)
assert [s["rank"] for s in shares] == list(range(w))
assert all(s["per_rank"] == per_rank for s in shares)          # the same split everywhere
allb = sorted(k for s in shares for k in s["bodies"])
assert allb == list(range(len(descs))), allb                     # disjoint and complete
sizes = [b3g.estimate_bytes(d) for d in descs]
assert sum(per_rank) == sum(sizes)
assert max(per_rank) - min(per_rank) <= max(sizes)               # greedy bound
for s in shares:
    assert sum(sizes[k] for k in s["bodies"]) == per_rank[s["rank"]]
class A: pass
a = A(); a.workload, a.split, a.bodies = "batch", True, 24
d2, cfg = bench.workload(a, r, w)
assert cfg["bodies_this_rank"] == len(mine) and len(d2) == len(mine)
dist.destroy_process_group()
''' % ROOT
    script = tmp_path / "split.py"
    script.write_text(code)
    r = run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
             "--master-addr", "127.0.0.1", "--master-port", "29533", str(script)])
    assert r.returncode == 0, r.stderr[-3000:]


def test_partition_rule():
    """b3g_partition_bodies: largest first to the least-loaded rank, ties to the lowest rank."""
    from bounce_softbody_gb300 import b3g

    owner = b3g.partition([5, 9, 3, 9, 1], 2)
    # order 9(1), 9(3), 5(0), 3(2), 1(4): 1->0, 3->1, 0->0 (9 vs 9: rank 0), 2->1, 4->1
    assert list(owner) == [0, 0, 1, 1, 1]
    assert list(b3g.partition([7, 7, 7], 1)) == [0, 0, 0]
    assert len(b3g.partition([], 4)) == 0
    with pytest.raises(b3g.B3gError):
        b3g.partition([1, 2], 0)


def test_algorithmic_byte_counts_follow_their_units():
    """The roofline's algorithmic bytes, per unit, as the design notes state them: SpMV
    40·nnzb + n + 24·n; a PCG iteration that plus 36·n (direction and product in the SpMV sweep)
    and 96·n (update); the final update 112·n; the assembly 212·T + 48·n (elements and state
    gathers) + 40·nnzb + 112·T + 105·n (rows). The counts come from a Kuhn block's mesh."""
    import numpy as np
    sys.path.insert(0, str(ROOT))
    import bench
    from bounce_softbody_gb300 import meshes
    d = meshes.tet_grid(5, 4, 6, pin="y0")
    n, nt = d.x.shape[0], d.tets.shape[0]
    pairs = {(int(t[a]), int(t[b])) for t in d.tets for a in range(4) for b in range(4) if a != b}
    nnzb = n + len(pairs)
    info = {"vertices": n, "tets": nt, "nnzb": nnzb}
    assert bench.spmv_bytes(info) == 40 * nnzb + n + 24 * n
    assert bench.iteration_bytes(info) == 40 * nnzb + n + 24 * n + 36 * n + 96 * n
    assert bench.final_bytes(info) == 112 * n
    assert bench.assembly_bytes(info) == 212 * nt + 48 * n + 40 * nnzb + 112 * nt + 105 * n
    assert np.isclose(nt, 6 * 4 * 3 * 5)
