"""b3g_step_batch_noalloc: the batched step for callers that cannot allocate device memory while
they step (a frame captured into a CUDA graph, engines with a no-allocation-after-load rule or a
fixed memory budget). It keeps its per-batch tables in a fixed device array of the library
instead of allocating them; these tests check it through the C ABI against b3g_step_batch, which
allocates its tables, on identical bodies, two calls in a row, and that it refuses batches larger
than its array."""
import numpy as np
import pytest

from bounce_softbody_gb300 import b3g, meshes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def bodies_mix():
    descs = [meshes.tet_grid(18, 16, 17, seed=3, E=3e5, nu=0.35, pin="x0", name="big0")]  # >= 4096: cluster team
    descs += meshes.batch_bodies(count=10, lo=4, hi=11, seed=17)
    return descs


def test_noalloc_matches_allocating_batch_two_calls():
    ctx = b3g.Context(0)
    descs = bodies_mix()
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    ref = [b3g.Body(ctx, d) for d in descs]
    new = [b3g.Body(ctx, d) for d in descs]
    for call in range(2):
        st_ref = b3g.step_batch(ctx, ref, DT, 1, cfg)
        st_new = b3g.step_batch_noalloc(ctx, new, DT, 1, cfg)
        for k, d in enumerate(descs):
            xr, vr = ref[k].state()
            xn, vn = new[k].state()
            disp = np.linalg.norm(xr.astype(np.float64) - d.x)
            # same tolerance as the other batch tests: team sizes may differ, so reduction
            # groupings (and last bits) may too
            assert np.linalg.norm(xn.astype(np.float64) - xr) <= 1e-5 * max(disp, 1e-12), (call, d.name)
            assert np.linalg.norm(vn - vr) <= 1e-4 * max(np.linalg.norm(vr), 1e-12), (call, d.name)
            assert abs(st_new[k]["pcg_iterations"] - st_ref[k]["pcg_iterations"]) <= 2
            assert st_new[k]["solve_status"] in ("converged", "max_iterations")
            assert st_new[k]["total_steps"] == call + 1
    for b in ref + new:
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
