"""b3g_step_batch_noalloc: the batched step for callers that cannot call cudaMalloc while they
step (engines that forbid device allocation after load or keep a fixed device-memory budget,
real-time loops that cannot take the device-wide synchronisation of cudaMalloc / cudaFree). It
keeps its per-batch tables in a fixed device array of the library instead of allocating them.

These tests call it through the C ABI and compare it with b3g_step_batch, which allocates its
tables, on identical bodies: several steps per call, one and two Newton iterations, the three
precisions, and two different body lists taking turns on the shared array. They also check that
it refuses batches larger than its array. This file is collected last on purpose, so that a run
stopping at the first failure has run every other test before it."""
import numpy as np
import pytest

from bounce_softbody_gb300 import b3g, meshes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def list_a():
    descs = [meshes.tet_grid(18, 16, 17, seed=3, E=3e5, nu=0.35, pin="x0", name="big0")]  # >= 4096: cluster team
    descs += meshes.batch_bodies(count=10, lo=4, hi=11, seed=17)
    return descs


def list_b():
    descs = [meshes.tet_grid(17, 17, 15, seed=5, E=1e5, nu=0.3, pin="y0", name="big1")]
    descs += meshes.batch_bodies(count=7, lo=4, hi=9, seed=29)
    return descs


def _compare(ref, new, descs, st_ref, st_new, total, xtol, vtol, tag):
    for k, d in enumerate(descs):
        xr, vr = ref[k].state()
        xn, vn = new[k].state()
        disp = np.linalg.norm(xr.astype(np.float64) - d.x)
        # team sizes and the assembly launches may differ between the two entry points, so
        # reduction groupings (and last bits) may too
        assert np.linalg.norm(xn.astype(np.float64) - xr) <= xtol * max(disp, 1e-12), (tag, d.name)
        assert np.linalg.norm(vn - vr) <= vtol * max(np.linalg.norm(vr), 1e-12), (tag, d.name)
        assert abs(st_new[k]["pcg_iterations"] - st_ref[k]["pcg_iterations"]) <= 2, (tag, d.name)
        assert st_new[k]["solve_status"] in ("converged", "max_iterations"), (tag, d.name)
        assert st_new[k]["total_steps"] == st_ref[k]["total_steps"] == total, (tag, d.name)


@pytest.fixture
def same_schedule(monkeypatch):
    # b3g_step_batch with the allocation-free call's fixed size rule instead of the autotuner's pick
    monkeypatch.setenv("B3G_BATCH_SCHEDULE", "4,4096")


def test_noalloc_matches_allocating_batch_two_calls():
    ctx = b3g.Context(0)
    descs = list_a()
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    ref = [b3g.Body(ctx, d) for d in descs]
    new = [b3g.Body(ctx, d) for d in descs]
    for call in range(2):
        st_ref = b3g.step_batch(ctx, ref, DT, 1, cfg)
        st_new = b3g.step_batch_noalloc(ctx, new, DT, 1, cfg)
        _compare(ref, new, descs, st_ref, st_new, call + 1, 1e-5, 1e-4, f"call {call}")
    for b in ref + new:
        b.close()
    ctx.close()


@pytest.mark.parametrize("newton", [1, 2])
def test_noalloc_several_steps_per_call(same_schedule, newton):
    ctx = b3g.Context(0)
    descs = list_a()
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5, force_iterations=newton,
                            newton_tolerance=1e-6)
    ref = [b3g.Body(ctx, d) for d in descs]
    new = [b3g.Body(ctx, d) for d in descs]
    for call in range(2):
        st_ref = b3g.step_batch(ctx, ref, DT, 3, cfg)
        st_new = b3g.step_batch_noalloc(ctx, new, DT, 3, cfg)
        _compare(ref, new, descs, st_ref, st_new, 3 * (call + 1), 1e-5, 1e-4, f"newton {newton} call {call}")
    for b in ref + new:
        b.close()
    ctx.close()


@pytest.mark.parametrize("precision,xtol,vtol", [(b3g.PRECISION_FP64, 1e-6, 1e-5), (b3g.PRECISION_BF16, 1e-4, 1e-3)])
def test_noalloc_other_precisions(same_schedule, precision, xtol, vtol):
    """FP64 solves agree to the float rounding of the stored state (positions and velocities are
    float in every precision); BF16 blocks to their looser solve."""
    ctx = b3g.Context(0)
    descs = list_a()
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5, precision=precision)
    ref = [b3g.Body(ctx, d) for d in descs]
    new = [b3g.Body(ctx, d) for d in descs]
    # the first step in a precision creates the bodies' solver buffers for it (b3g_step_batch does)
    b3g.step_batch(ctx, ref, DT, 1, cfg)
    b3g.step_batch(ctx, new, DT, 1, cfg)
    for call in range(2):
        st_ref = b3g.step_batch(ctx, ref, DT, 2, cfg)
        st_new = b3g.step_batch_noalloc(ctx, new, DT, 2, cfg)
        _compare(ref, new, descs, st_ref, st_new, 1 + 2 * (call + 1), xtol, vtol, f"{precision} call {call}")
    for b in ref + new:
        b.close()
    ctx.close()


def test_noalloc_two_body_lists_take_turns(same_schedule):
    """Two lists of different bodies step in turn through the one shared array: each call must
    step exactly its own bodies."""
    ctx = b3g.Context(0)
    da, db = list_a(), list_b()
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    ref_a = [b3g.Body(ctx, d) for d in da]
    ref_b = [b3g.Body(ctx, d) for d in db]
    new_a = [b3g.Body(ctx, d) for d in da]
    new_b = [b3g.Body(ctx, d) for d in db]
    counts = {"a": 0, "b": 0}
    for tag, steps in (("a", 1), ("b", 2), ("a", 2), ("b", 1), ("a", 1)):
        descs, ref, new = (da, ref_a, new_a) if tag == "a" else (db, ref_b, new_b)
        st_ref = b3g.step_batch(ctx, ref, DT, steps, cfg)
        st_new = b3g.step_batch_noalloc(ctx, new, DT, steps, cfg)
        counts[tag] += steps
        _compare(ref, new, descs, st_ref, st_new, counts[tag], 1e-5, 1e-4, f"list {tag}")
    for b in ref_a + ref_b + new_a + new_b:
        b.close()
    ctx.close()


def test_noalloc_rejects_batches_beyond_its_array():
    ctx = b3g.Context(0)
    tiny = meshes.tet_grid(2, 2, 2, pin="y0")
    bodies = [b3g.Body(ctx, tiny) for _ in range(513)]
    with pytest.raises(b3g.B3gError, match="at most 512 bodies"):
        b3g.step_batch_noalloc(ctx, bodies, DT, 1)
    for b in bodies:
        b.close()
    ctx.close()
