"""The persistent batch kernel (b3g_step_batch) against the per-body path and the oracle."""
import os

import numpy as np
import pytest

import oracle
from bounce_softbody_gb300 import b3g, meshes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def small_batch(count=20, lo=4, hi=11, seed=11):
    return meshes.batch_bodies(count=count, lo=lo, hi=hi, seed=seed)


def disp_rel(x, xr, x0):
    return float(np.linalg.norm(np.asarray(x, np.float64) - xr) / max(np.linalg.norm(xr - x0), 1e-30))


def test_batch_matches_single_body_path(ctx):
    """Each body of a batch ends where the per-op single-body path takes it (5 steps).

    Both paths stop at the same relative residual (1e-5), but the per-op path accumulates the
    solution in FP64 (iterative refinement) and the batch kernel in FP32, so a solve may stop one
    iteration apart: velocities agree to the solve tolerance times the conditioning (1e-3
    relative), positions (which add the velocity times h to the unchanged start) to 1e-5 of the
    displacement."""
    descs = small_batch()
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    batch = [b3g.Body(ctx, d) for d in descs]
    alone = [b3g.Body(ctx, d) for d in descs]
    for _ in range(5):
        st = b3g.step_batch(ctx, batch, DT, 1, cfg)
        for b in alone:
            b.step(DT, cfg, stats=False)
    for k, d in enumerate(descs):
        xb, vb = batch[k].state()
        xa, va = alone[k].state()
        assert disp_rel(xb, xa.astype(np.float64), d.x) < 1e-5, d.name
        assert np.linalg.norm(vb - va) <= 1e-3 * max(np.linalg.norm(va), 1e-12), d.name
        assert st[k]["solve_status"] in ("converged", "max_iterations")


def test_batch_matches_oracle(ctx):
    descs = small_batch(count=6, seed=5)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    bodies = [b3g.Body(ctx, d) for d in descs]
    st = b3g.step_batch(ctx, bodies, DT, 10, cfg)
    for k, d in enumerate(descs):
        x, v = bodies[k].state()
        xr, vr, it, _ = oracle.simulate(d, 10, kind="port", bits=64)
        assert disp_rel(x, xr, d.x) < 1e-4, d.name
        assert np.linalg.norm(v - vr) < 1e-3 * np.linalg.norm(vr), d.name
        assert abs(st[k]["pcg_iterations"] - int(it[-1])) <= 3
        assert st[k]["total_steps"] == 10


@pytest.mark.parametrize("schedule", ["2,8192", "4,8192", "8,8192"])
def test_batch_cluster_teams_match_single_body_path(ctx, schedule, monkeypatch):
    """Bodies above the cluster threshold are stepped by clusters of CTAs (DSMEM reductions)."""
    monkeypatch.setenv("B3G_BATCH_SCHEDULE", schedule)
    descs = [meshes.tet_grid(28, 26, 24, seed=3, E=3e5, nu=0.35, pin="x0", name="big0"),
             meshes.tet_grid(26, 25, 27, seed=4, E=8e4, nu=0.25, pin="z1", name="big1")]
    descs += small_batch(count=6, seed=8)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    batch = [b3g.Body(ctx, d) for d in descs]
    alone = [b3g.Body(ctx, d) for d in descs]
    for _ in range(3):
        b3g.step_batch(ctx, batch, DT, 1, cfg)
        for b in alone:
            b.step(DT, cfg, stats=False)
    sched = b3g.batch_schedule(ctx)
    assert sched["cluster"] == int(schedule.split(",")[0]) and sched["cluster_bodies"] == 2
    for k, d in enumerate(descs):
        xb, vb = batch[k].state()
        xa, va = alone[k].state()
        assert disp_rel(xb, xa.astype(np.float64), d.x) < 1e-5, d.name
        assert np.linalg.norm(vb - va) <= 1e-4 * max(np.linalg.norm(va), 1e-12), d.name


@pytest.mark.parametrize("cluster_env", ["0"])
def test_batch_is_deterministic(ctx, cluster_env, monkeypatch):
    """Two batches from the same state give bitwise equal states (no float atomics)."""
    monkeypatch.setenv("B3G_AUTOTUNE", cluster_env)
    descs = small_batch(count=8, seed=21)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    out = []
    for _ in range(2):
        bodies = [b3g.Body(ctx, d) for d in descs]
        b3g.step_batch(ctx, bodies, DT, 4, cfg)
        out.append([b.state() for b in bodies])
        for b in bodies:
            b.close()
    for (x1, v1), (x2, v2) in zip(out[0], out[1]):
        assert np.array_equal(x1, x2) and np.array_equal(v1, v2)


def mixed_bodies():
    """Every element kind: tetrahedra; membrane triangles and springs with sphere contact;
    Baraff-Witkin stretch and shear with a mouse spring."""
    return [meshes.batch_bodies(count=1, lo=6, hi=9, seed=21)[0],
            meshes.cloth_grid(12, side=1.2, height=0.56, sphere_radius=0.5, contact_radius=0.05),
            meshes.bw_cloth(8, pinned="edges", stretch_ks=5e4, shear_ks=1e3, shear_kd=10.0, mouse=True),
            meshes.batch_bodies(count=1, lo=10, hi=14, seed=22)[0]]


@pytest.mark.parametrize("split,mixed", [("0.5,1,2", False), ("0.3,2,1", False), ("0.1,1,2", True)],
                         ids=["tets-half", "tets-third", "mixed-kinds"])
def test_split_assembly_is_bitwise_equal(ctx, split, mixed, monkeypatch):
    """The split assembly (the second body group's element launch on a second stream beside the
    first group's row launch) computes every element and row exactly as the two whole-batch
    launches do: bitwise equal states after several steps, graph-replayed and timed. Batches of
    tetrahedra only split by default; a batch of mixed element kinds only when asked to, which
    it then also handles."""
    monkeypatch.setenv("B3G_AUTOTUNE", "0")
    descs = mixed_bodies() if mixed else small_batch(count=12, seed=29)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    out = []
    for env, timed in (("0", False), (split, False), (split, True)):
        monkeypatch.setenv("B3G_ASM_SPLIT", env)
        bodies = [b3g.Body(ctx, d) for d in descs]
        b3g.batch_set_launch_timing(ctx, timed)
        b3g.step_batch(ctx, bodies, DT, 4, cfg, stats=False)
        b3g.batch_set_launch_timing(ctx, False)
        sp = b3g.batch_assembly_split(ctx)
        assert (sp["elem_mid"] > 0) == (env != "0") and (sp["slice_mid"] > 0) == (env != "0")
        out.append([b.state() for b in bodies])
        for b in bodies:
            b.close()
    for run in out[1:]:
        for (x1, v1), (x2, v2) in zip(out[0], run):
            assert np.array_equal(x1, x2) and np.array_equal(v1, v2)


def test_launch_timing_mode_same_results(ctx):
    """Timed batched steps (direct launches with events around the assembly and PCG launches)
    compute exactly what the graph-replayed steps compute, and report positive launch times."""
    descs = small_batch(count=8, seed=23)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    ref = [b3g.Body(ctx, d) for d in descs]
    tim = [b3g.Body(ctx, d) for d in descs]
    b3g.step_batch(ctx, ref, DT, 3, cfg, stats=False)
    b3g.batch_set_launch_timing(ctx, True)
    b3g.batch_launch_times(ctx, reset=True)
    b3g.step_batch(ctx, tim, DT, 3, cfg, stats=False)
    t = b3g.batch_launch_times(ctx, reset=True)
    b3g.batch_set_launch_timing(ctx, False)
    assert t["steps"] == 3 and t["assembly_ms"] > 0 and t["pcg_ms"] > 0
    for a, b in zip(ref, tim):
        xa, va = a.state()
        xb, vb = b.state()
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    for b in ref + tim:
        b.close()


def test_queued_force_uploads_overlap_and_match(ctx):
    """Page-locked force arrays are copied on the context's upload stream into two staging
    buffers taken in turn, overlapping the step queued before. Five steps queued without any
    synchronisation, each with its own forces, end bitwise where the per-body calls take the
    same bodies."""
    torch = pytest.importorskip("torch")
    descs = meshes.batch_bodies(count=6, lo=3, hi=9, seed=31)
    cfg = b3g.solver_config()
    rng = np.random.default_rng(5)
    nsteps = 5
    a = [b3g.Body(ctx, d) for d in descs]
    b = [b3g.Body(ctx, d) for d in descs]
    total = sum(x.n for x in a)
    forces = [rng.uniform(-2.0, 2.0, 3 * total).astype(np.float32) for _ in range(nsteps)]
    pinned = [torch.from_numpy(f.copy()).pin_memory() for f in forces]
    for p in pinned:
        b3g.batch_apply_forces(ctx, a, p.data_ptr())
        b3g.step_batch(ctx, a, DT, 1, cfg, stats=False)
    for f in forces:
        off = 0
        for body in b:
            body.apply_forces(f[off:off + 3 * body.n].reshape(body.n, 3))
            off += 3 * body.n
        b3g.step_batch(ctx, b, DT, 1, cfg, stats=False)
    ctx.synchronize()
    for x, y in zip(a, b):
        xa, va = x.state()
        xb, vb = y.state()
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    for body in a + b:
        body.close()


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "page_locked"])
def test_batch_host_transfers_match_per_body_calls(ctx, pinned):
    """b3g_batch_apply_forces / b3g_batch_get_state (one launch each way over a cached body
    table; page-locked host arrays are read and written by the launch directly, others go through
    one staging copy) against the per-body calls: bitwise the same state, also after the body list
    changes and after a listed body is destroyed."""
    descs = meshes.batch_bodies(count=7, lo=3, hi=9, seed=13)
    cfg = b3g.solver_config()
    if pinned:
        torch = pytest.importorskip("torch")

        def host(a):
            t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).pin_memory()
            return t, t.numpy()
    else:
        def host(a):
            a = np.ascontiguousarray(a, np.float32)
            return a, a

    def run(batched, order, forces):
        bodies = [b3g.Body(ctx, d) for d in descs]
        sel = [bodies[k] for k in order]
        n = [b.n for b in sel]
        for f in forces:
            if batched:
                keep, fa = host(f)
                b3g.batch_apply_forces(ctx, sel, fa.ctypes.data)
                ctx.synchronize()
            else:
                off = 0
                for b, m in zip(sel, n):
                    b.apply_forces(f[off:off + 3 * m].reshape(m, 3))
                    off += 3 * m
            b3g.step_batch(ctx, bodies, DT, 1, cfg, stats=False)
        kx, x = host(np.zeros(3 * sum(n), np.float32))
        kv, v = host(np.zeros(3 * sum(n), np.float32))
        if batched:
            b3g.batch_get_state(ctx, sel, x.ctypes.data, v.ctypes.data)
        else:
            off = 0
            for b, m in zip(sel, n):
                xb, vb = b.state()
                x[off:off + 3 * m], v[off:off + 3 * m] = xb.ravel(), vb.ravel()
                off += 3 * m
        return bodies, np.array(x), np.array(v)

    for order in ([0, 1, 2, 3, 4, 5, 6], [5, 2, 6]):
        total = sum(descs[k].n for k in order)
        forces = [np.random.default_rng(1 + s).standard_normal(3 * total).astype(np.float32) for s in range(3)]
        b1, x1, v1 = run(True, order, forces)
        b2, x2, v2 = run(False, order, forces)
        assert np.array_equal(x1, x2) and np.array_equal(v1, v2), order
        assert np.abs(v1).max() > 0
        # a listed body goes away: the next batched call rebuilds its table
        b1[order[0]].close()
        rest = [b1[k] for k in order[1:]]
        kxs, xs = host(np.zeros(3 * sum(b.n for b in rest), np.float32))
        kvs, vs = host(np.zeros(3 * sum(b.n for b in rest), np.float32))
        b3g.batch_get_state(ctx, rest, xs.ctypes.data, vs.ctypes.data)
        m = rest[0].n
        xr, vr = rest[0].state()
        assert np.array_equal(xs[:3 * m], xr.ravel()) and np.array_equal(vs[:3 * m], vr.ravel())
        for b in b1 + b2:
            b.close()


def test_mixed_batch_matches_oracle(ctx):
    """One batch of every element kind (tetrahedra; membrane triangles and springs with sphere
    contact; Baraff-Witkin stretch and shear with a mouse spring): the flat element launch
    dispatches each body's elements by kind over one numbering, the flat row launch serves slices
    of all of them; each body against the FP64 oracle within 20x the oracle's own FP32 spread."""
    descs = mixed_bodies()
    steps = 4
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    bodies = [b3g.Body(ctx, d) for d in descs]
    b3g.step_batch(ctx, bodies, DT, steps, cfg, stats=False)
    for g, d in zip(bodies, descs):
        x, v = g.state()
        x64, v64, _, _ = oracle.simulate(d, steps, kind="port", bits=64)
        x32, v32, _, _ = oracle.simulate(d, steps, kind="port", bits=32)
        assert disp_rel(x, x64, d.x) < max(1e-4, 20 * disp_rel(x32, x64, d.x)), d.name
        fv = float(np.linalg.norm(v32 - v64) / max(np.linalg.norm(v64), 1e-30))
        assert np.linalg.norm(v - v64) <= max(1e-3, 20 * fv) * np.linalg.norm(v64), d.name
        g.close()


@pytest.mark.parametrize("pinned", [False, True])
def test_async_state_read_is_a_snapshot(ctx, pinned):
    """b3g_batch_get_state_async: the host arrays receive the state at the call, even though the
    next step is queued before the copy is waited for; they match b3g_batch_get_state."""
    descs = small_batch(count=7, seed=21)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    bodies = [b3g.Body(ctx, d) for d in descs]
    n3 = 3 * sum(d.n for d in descs)
    if pinned:
        torch = pytest.importorskip("torch")
        xa = torch.zeros(n3, dtype=torch.float32).pin_memory()
        va = torch.zeros(n3, dtype=torch.float32).pin_memory()
        xp, vp = xa.data_ptr(), va.data_ptr()
        get = lambda t: t.numpy().copy()  # noqa: E731
    else:
        xa, va = np.zeros(n3, np.float32), np.zeros(n3, np.float32)
        xp, vp = xa.ctypes.data, va.ctypes.data
        get = lambda a: a.copy()  # noqa: E731
    b3g.step_batch(ctx, bodies, DT, 2, cfg, stats=False)
    xs, vs = np.zeros(n3, np.float32), np.zeros(n3, np.float32)
    b3g.batch_get_state(ctx, bodies, xs.ctypes.data, vs.ctypes.data)
    b3g.batch_get_state_async(ctx, bodies, xp, vp)
    b3g.step_batch(ctx, bodies, DT, 1, cfg, stats=False)  # queued behind the snapshot
    b3g.batch_wait_state(ctx)
    assert np.array_equal(get(xa), xs) and np.array_equal(get(va), vs)
    # a second read after the step: the new state
    b3g.batch_get_state_async(ctx, bodies, xp, vp)
    b3g.batch_wait_state(ctx)
    b3g.batch_get_state(ctx, bodies, xs.ctypes.data, vs.ctypes.data)
    assert np.array_equal(get(xa), xs) and not np.array_equal(xs, np.zeros_like(xs))
    for b in bodies:
        b.close()
