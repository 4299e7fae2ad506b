"""Degenerate bodies through the per-op and the batched path: free particles (backward Euler in
closed form), a body of static vertices only, a single tetrahedron, a batch mixing them with an
ordinary block, and empty or zero-step batch calls."""
import numpy as np
import pytest

import edge_bodies as eb
import oracle
from bounce_softbody_gb300 import b3g, meshes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def cfg():
    return b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)


@pytest.mark.parametrize("damping", [0.0, 0.02])
def test_free_particles_fall_in_closed_form(ctx, damping):
    """No element: A = (1 + h c) I and one PCG iteration solves it; both paths give
    v' = v + h (g - c v) / (1 + h c), x' = x + h v' to float rounding."""
    desc = eb.particles(damping=damping)
    steps = 6
    xf, vf = eb.free_fall(desc, steps, DT)
    g = b3g.Body(ctx, desc)
    its = [g.step(DT, cfg())["pcg_iterations"] for _ in range(steps)]
    x, v = g.state()
    b = b3g.Body(ctx, desc)
    st = b3g.step_batch(ctx, [b], DT, steps, cfg())
    xb, vb = b.state()
    for got_x, got_v in ((x, v), (xb, vb)):
        np.testing.assert_allclose(got_x, xf, rtol=0, atol=2e-6)
        np.testing.assert_allclose(got_v, vf, rtol=0, atol=2e-6)
    assert its == [1] * steps and st[0]["pcg_iterations"] == 1
    g.close()
    b.close()


def test_all_static_body_does_not_move(ctx):
    desc = eb.all_static()
    g = b3g.Body(ctx, desc)
    s = [g.step(DT, cfg()) for _ in range(3)][-1]
    x, v = g.state()
    b = b3g.Body(ctx, desc)
    sb = b3g.step_batch(ctx, [b], DT, 3, cfg())[0]
    xb, vb = b.state()
    for xx, vv, st in ((x, v, s), (xb, vb, sb)):
        assert np.array_equal(xx, desc.x.astype(np.float32)) and not np.any(vv)
        assert st["pcg_iterations"] == 0 and st["solve_status"] == "converged"
    g.close()
    b.close()


def test_single_tetrahedron_matches_oracle(ctx):
    desc = eb.single_tet()
    steps = 10
    x64, v64, it64, _ = oracle.simulate(desc, steps, kind="port", bits=64)
    g = b3g.Body(ctx, desc)
    its = [g.step(DT, cfg())["pcg_iterations"] for _ in range(steps)]
    x, v = g.state()
    g.close()
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64 - desc.x) < 1e-4
    assert np.linalg.norm(v - v64) / np.linalg.norm(v64) < 1e-3
    assert max(abs(a - int(b)) for a, b in zip(its, it64)) <= 1


def test_batch_of_degenerate_and_ordinary_bodies(ctx):
    """One batch of free particles, a static body, a single tetrahedron and an ordinary block:
    each body as the per-op path steps it alone."""
    descs = [eb.particles(n=5), eb.all_static(), eb.single_tet(),
             meshes.tet_grid(7, 6, 8, seed=3, E=1e5, nu=0.3, pin="y0", name="block")]
    steps = 5
    batch = [b3g.Body(ctx, d) for d in descs]
    b3g.step_batch(ctx, batch, DT, steps, cfg())
    for d, b in zip(descs, batch):
        g = b3g.Body(ctx, d)
        for _ in range(steps):
            g.step(DT, cfg(), stats=False)
        xa, va = g.state()
        xb, vb = b.state()
        disp = max(np.linalg.norm(xa - d.x), 1e-12)
        assert np.linalg.norm(xb - xa) / disp < 1e-5, d.name
        assert np.linalg.norm(vb - va) <= 1e-3 * max(np.linalg.norm(va), 1e-12), d.name
        g.close()
        b.close()


def test_empty_and_zero_step_batches(ctx):
    desc = meshes.tet_grid(4, 4, 4, seed=1, E=1e5, nu=0.3, pin="y0")
    g = b3g.Body(ctx, desc)
    x0, v0 = g.state()
    assert b3g.step_batch(ctx, [], DT, 3, cfg()) == []
    assert b3g.step_batch(ctx, [g], DT, 0, cfg(), stats=False) is None
    x, v = g.state()
    assert np.array_equal(x, x0) and np.array_equal(v, v0)
    g.close()
