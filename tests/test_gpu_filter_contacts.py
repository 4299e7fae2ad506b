"""Filtered contacts (B3G_CONTACT_FILTER, an opt-in extension of b3g_body_step and
b3g_step_batch) against the oracle's restatement of the same mode: overlapping dynamic vertices
constrained along the contact normal through the solver's pre-filter instead of penalty springs."""
import numpy as np
import pytest

import oracle
from bounce_softbody_gb300 import b3g, meshes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def rel_disp(x, xr, x0):
    return float(np.linalg.norm(np.asarray(x, np.float64) - xr) / max(np.linalg.norm(xr - x0), 1e-30))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def filt_config(**kw):
    kw.setdefault("max_pcg_iterations", 200)
    kw.setdefault("pcg_tolerance", 1e-5)
    return b3g.solver_config(contact_mode=b3g.CONTACT_FILTER, **kw)


def gpu_run(ctx, desc, steps, cfg):
    g = b3g.Body(ctx, desc)
    its = [g.step(DT, cfg)["pcg_iterations"] for _ in range(steps)]
    x, v = g.state()
    g.close()
    return x, v, its


def check_against_oracle(x, v, desc, steps, newton_iters=1):
    """Within 20x the oracle's own FP32-vs-FP64 spread on this scene (contacts amplify rounding:
    a vertex at the overlap threshold may be constrained in one run and free in another)."""
    x64, v64, _, _ = oracle.simulate(desc, steps, kind="port", bits=64, contact_mode=1, newton_iters=newton_iters)
    x32, v32, _, _ = oracle.simulate(desc, steps, kind="port", bits=32, contact_mode=1, newton_iters=newton_iters)
    assert rel_disp(x, x64, desc.x) < max(1e-4, 20 * rel_disp(x32, x64, desc.x)), desc.name
    assert rel(v, v64) < max(1e-3, 20 * rel(v32, v64)), desc.name
    return x64, v64


@pytest.mark.parametrize("tilt", [0.0, 0.05])
def test_filtered_block_on_floor_matches_oracle(ctx, tilt):
    """The 50 kg block the penalty contact cannot carry: held (flat floor) or sliding without
    friction (tilted floor), as the oracle's filtered contacts do."""
    desc = meshes.block_on_floor(tilt=tilt)
    steps = 40
    x, v, its = gpu_run(ctx, desc, steps, filt_config())
    check_against_oracle(x, v, desc, steps)
    assert x[:, 1].min() > -0.05 and max(its) < 200


def test_filtered_contacts_fp64_newton(ctx):
    """FP64 precision and three Newton iterations (z in the first one only)."""
    desc = meshes.block_on_floor(a=4, b=3, c=4)
    steps = 20
    cfg = filt_config(precision=b3g.PRECISION_FP64, force_iterations=3)
    x, v, _ = gpu_run(ctx, desc, steps, cfg)
    x64, v64 = check_against_oracle(x, v, desc, steps, newton_iters=3)
    assert rel_disp(x, x64, desc.x) < 1e-4


def test_filter_mode_without_contact_spheres_is_the_default_path(ctx):
    desc = meshes.tet_grid(5, 5, 5, seed=3, E=1e5, nu=0.3, pin="y0")
    cfg0 = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    a = gpu_run(ctx, desc, 4, cfg0)
    b = gpu_run(ctx, desc, 4, filt_config())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_filter_mode_is_refused_by_the_server_and_the_allocation_free_step(ctx):
    desc = meshes.block_on_floor(a=3, b=3, c=3)
    g = b3g.Body(ctx, desc)
    with pytest.raises(b3g.B3gError, match="b3g_body_step and b3g_step_batch only"):
        b3g.Server(ctx, 1 << 28, 8, DT, config=filt_config())
    with pytest.raises(b3g.B3gError, match="b3g_body_step and b3g_step_batch only"):
        b3g.step_batch_noalloc(ctx, [g], DT, 1, filt_config())
    bad = b3g.solver_config()
    bad.contact_mode = 7
    with pytest.raises(b3g.B3gError, match="unknown contact mode"):
        g.step(DT, bad)
    g.close()


@pytest.mark.parametrize("newton,precision", [(1, b3g.PRECISION_FP32), (3, b3g.PRECISION_FP64)])
def test_batched_filtered_contacts_match_oracle(ctx, newton, precision):
    """b3g_step_batch in the filtered mode: blocks on a flat and a tilted floor, batched with a body
    without contact spheres (stepped in the default form), against the oracle's filtered mode.
    One Newton iteration runs the flat element / row launches (the vertex constraints in the
    element launch), several the whole-step team launch."""
    descs = [meshes.block_on_floor(tilt=0.05), meshes.block_on_floor(a=4, b=3, c=4, tilt=0.0, seed=6),
             meshes.tet_grid(5, 5, 5, seed=3, E=1e5, nu=0.3, pin="y0", name="free")]
    steps = 20
    cfg = filt_config(force_iterations=newton, precision=precision)
    bodies = [b3g.Body(ctx, d) for d in descs]
    st = b3g.step_batch(ctx, bodies, DT, steps, cfg)
    for k, d in enumerate(descs):
        x, v = bodies[k].state()
        check_against_oracle(x, v, d, steps, newton_iters=newton)
        assert st[k]["total_steps"] == steps
    # the blocks rest on / slide along the floor instead of sinking through it
    for k in (0, 1):
        assert bodies[k].state()[0][:, 1].min() > -0.05
    # the body without contact spheres steps exactly as in the default mode
    plain = b3g.Body(ctx, descs[2])
    b3g.step_batch(ctx, [plain], DT, steps, b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5,
                                                               force_iterations=newton, precision=precision))
    alone = b3g.Body(ctx, descs[2])
    b3g.step_batch(ctx, [alone], DT, steps, cfg)
    assert np.array_equal(plain.state()[0], alone.state()[0])
    for b in bodies + [plain, alone]:
        b.close()
