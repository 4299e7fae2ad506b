"""Serving loop (b3g_server_*): continuous batching of step requests over many bodies.

Checks through the C ABI that a body's results do not depend on the mix it is served in (bitwise:
every launch uses one kernel and each body's team size depends only on its own size), that
evicting idle bodies under a tight memory budget and restoring them later changes nothing
(contacts included), that a body larger than the budget is rejected while the rest are served,
and the bookkeeping of requests and statistics."""
import threading
import time

import numpy as np
import pytest

from bounce_softbody_gb300 import b3g, meshes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def descs_mix():
    out = [meshes.tet_grid(18, 16, 17, seed=3, E=3e5, nu=0.35, pin="x0", name="big0")]  # >= 4096: cluster team
    out.append(meshes.cloth_grid(24, side=0.8, height=0.53, name="cloth24"))            # falls onto the sphere
    out += meshes.batch_bodies(count=4, lo=4, hi=9, seed=29)
    return out


def cfg():
    return b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)


def serve(ctx, descs, plan, budget=8 << 30, max_active=64, concurrent=True):
    """Run `plan` (list of (body, steps) requests, submission order) on a new server and return
    (states, results, stats)."""
    srv = b3g.Server(ctx, budget, max_active, DT, cfg())
    ids = [srv.add_body(d) for d in descs]
    assert ids == list(range(len(descs)))
    if concurrent:
        srv.start()

        def client():
            for b, s in plan:
                srv.submit(b, s)
                time.sleep(0.0005)

        t = threading.Thread(target=client)
        t.start()
        t.join()
    else:
        for b, s in plan:
            srv.submit(b, s)
        srv.start()
    res = srv.drain(timeout=300)
    stats = srv.stats()
    states = [srv.state(k) for k in range(len(descs))]
    srv.close()
    return states, res, stats


def interleaved_plan(nbodies, splits, seed):
    rng = np.random.default_rng(seed)
    queues = [list(splits[k % len(splits)]) for k in range(nbodies)]
    plan = []
    while any(queues):
        k = int(rng.choice([i for i in range(nbodies) if queues[i]]))
        plan.append((k, queues[k].pop(0)))
    return plan


def test_alone_equals_mix_bitwise():
    ctx = b3g.Context(0)
    descs = descs_mix()
    total = 8
    plan = interleaved_plan(len(descs), [[3, 1, 4], [2, 2, 2, 2], [8], [1, 5, 2]], seed=5)
    mix, res, stats = serve(ctx, descs, plan)
    assert all(r["status"] == "done" for r in res)
    assert len(res) == len(plan)
    assert stats["completed"] == len(plan)
    assert stats["vertex_steps"] == total * sum(d.n for d in descs)
    for k, d in enumerate(descs):
        alone, res_a, _ = serve(ctx, [d], [(0, total)], concurrent=False)
        assert res_a[0]["status"] == "done"
        assert np.array_equal(mix[k][0], alone[0][0]), d.name
        assert np.array_equal(mix[k][1], alone[0][1]), d.name
        moved = np.abs(mix[k][0].astype(np.float64) - d.x).max()
        assert np.isfinite(mix[k][0]).all() and moved > 1e-4, d.name
    ctx.close()


def test_served_body_matches_batched_step():
    """The server's step is the batch kernel's: its result agrees with b3g_step_batch to rounding."""
    ctx = b3g.Context(0)
    descs = descs_mix()[:3]
    states, _, _ = serve(ctx, descs, [(k, 3) for k in range(len(descs))], concurrent=False)
    bodies = [b3g.Body(ctx, d) for d in descs]
    b3g.step_batch(ctx, bodies, DT, 3, cfg(), stats=False)
    for k, d in enumerate(descs):
        xr, vr = bodies[k].state()
        disp = np.linalg.norm(xr.astype(np.float64) - d.x)
        assert np.linalg.norm(states[k][0].astype(np.float64) - xr) <= 1e-5 * max(disp, 1e-12), d.name
        assert np.linalg.norm(states[k][1] - vr) <= 1e-4 * max(np.linalg.norm(vr), 1e-12), d.name
        bodies[k].close()
    ctx.close()


def test_eviction_restores_state_exactly():
    ctx = b3g.Context(0)
    descs = [meshes.cloth_grid(20, side=0.7, height=0.52, name=f"cloth{k}") for k in range(2)]
    descs += meshes.batch_bodies(count=3, lo=5, hi=8, seed=41)
    # round robin, one step per request, so bodies go idle between their requests
    plan = [(k, 1) for _ in range(6) for k in range(len(descs))]
    roomy, res_r, st_r = serve(ctx, descs, plan, concurrent=False)
    assert st_r["evictions"] == 0
    # room for about two bodies at a time: most requests need an eviction
    probe = b3g.Body(ctx, descs[0])
    one = probe.device_bytes()
    probe.close()
    tight, res_t, st_t = serve(ctx, descs, plan, budget=int(2.6 * one), max_active=2, concurrent=False)
    assert st_t["evictions"] >= len(plan) // 2
    assert st_t["resident_bytes"] <= int(2.6 * one)
    assert all(r["status"] == "done" for r in res_t)
    for k, d in enumerate(descs):
        assert np.array_equal(roomy[k][0], tight[k][0]), d.name
        assert np.array_equal(roomy[k][1], tight[k][1]), d.name
    # the cloths reached the sphere, so contact state crossed the evictions
    for k in range(2):
        y = tight[k][0][:, 1]
        assert y.min() < 0.52 - 1e-3
    ctx.close()


def test_oversized_body_rejected_others_served():
    ctx = b3g.Context(0)
    small = meshes.batch_bodies(count=2, lo=4, hi=5, seed=7)
    big = meshes.tet_grid(30, 30, 30, name="big30")
    probe = b3g.Body(ctx, small[0])
    budget = 4 * max(probe.device_bytes(), 1 << 20)
    probe.close()
    states, res, stats = serve(ctx, small + [big], [(0, 2), (2, 2), (1, 2)], budget=budget, concurrent=False)
    by = {r["body_id"]: r for r in res}
    assert by[2]["status"] == "rejected"
    assert by[0]["status"] == "done" and by[1]["status"] == "done"
    assert stats["rejected"] == 1
    assert np.array_equal(states[2][0], big.x.astype(np.float32))  # never stepped
    ctx.close()


def test_request_bookkeeping_and_latency():
    ctx = b3g.Context(0)
    descs = meshes.batch_bodies(count=6, lo=4, hi=8, seed=13)
    srv = b3g.Server(ctx, 4 << 30, 16, DT, cfg())
    for d in descs:
        srv.add_body(d)
    with pytest.raises(b3g.B3gError, match="unknown body"):
        srv.submit(len(descs), 1)
    with pytest.raises(b3g.B3gError, match="at least one step"):
        srv.submit(0, 0)
    srv.start()
    rids = [srv.submit(k % len(descs), 1 + k % 3) for k in range(18)]
    assert rids == sorted(rids) and len(set(rids)) == len(rids)
    res = srv.drain(timeout=120)
    assert sorted(r["request_id"] for r in res) == rids
    for r in res:
        assert r["status"] == "done"
        assert r["latency_seconds"] >= r["queue_seconds"] >= 0.0
        assert r["pcg_iterations"] >= r["steps"]
    # one body serves its requests in arrival order
    for k in range(len(descs)):
        mine = [r["request_id"] for r in res if r["body_id"] == k]
        assert mine == sorted(mine)
    st = srv.stats()
    assert st["completed"] == 18 and st["waiting"] == 0
    assert st["iterations"] >= max(sum(1 + j % 3 for j in range(18) if j % len(descs) == k) for k in range(len(descs)))
    assert 0.0 < st["step_ms_p50"] <= st["step_ms_p99"]
    assert srv.pending() == 0
    srv.close()
    ctx.close()
