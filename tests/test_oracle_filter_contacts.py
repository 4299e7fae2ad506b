"""Filtered contacts (contact_mode 1), an extension of the restatement: dynamic vertices that
overlap a static shape are constrained along its normal through the solver's pre-filter
(S = I - n n^T, z = (vt - v.n) n) instead of penalty springs. The reference has no such mode, so
these tests check the restatement's own physics; the CUDA path is compared with it in
test_gpu_filter_contacts.py."""
import numpy as np

import oracle
from bounce_softbody_gb300 import meshes


def floor_top_under(x, desc):
    """Height of the tilted floor's top face under each vertex (x, z)."""
    sh = desc.world_shapes[0]
    qx, qy, qz, qw = sh.rotation
    # rotation about z only: the top face's normal and a point on it
    ang = 2.0 * np.arctan2(qz, qw)
    n = np.array([-np.sin(ang), np.cos(ang), 0.0])
    p0 = np.asarray(sh.translation) + sh.p[1] * n
    # n . (q - p0) = 0 with q = (x, y, z): y = p0.y + (n.x (p0.x - x)) / n.y
    return p0[1] + n[0] * (p0[0] - x[:, 0]) / n[1]


def test_filtered_contacts_hold_a_heavy_block():
    desc = meshes.block_on_floor(tilt=0.0)
    r = desc.sphere_radius[0]
    # the reference's penalty contact lets the 50 kg block sink through the floor
    x0, _, _, _ = oracle.simulate(desc, 60, kind="port", bits=64, contact_mode=0)
    assert x0[:, 1].min() < -0.5
    # filtered contacts: the block comes to rest on the floor, its spheres touching the top face
    x, v, it, _ = oracle.simulate(desc, 90, kind="port", bits=64, contact_mode=1)
    gap = x[:, 1] - r - floor_top_under(x, desc)
    assert -2e-3 < gap.min() < 1e-3
    assert np.abs(v).max() < 0.02
    assert it.max() < 200


def test_filtered_contacts_are_frictionless():
    """On a floor tilted by t rad the block keeps touching it (no normal velocity) and slides
    downhill with acceleration g sin t: the constraint has no tangential part."""
    tilt, steps, h = 0.05, 90, 1.0 / 60.0
    desc = meshes.block_on_floor(tilt=tilt)
    x, v, _, _ = oracle.simulate(desc, steps, kind="port", bits=64, contact_mode=1)
    n = np.array([-np.sin(tilt), np.cos(tilt), 0.0])
    down = -np.array([np.cos(tilt), np.sin(tilt), 0.0])
    # the vertices touching the floor move along it (a vertex that did not overlap at the start
    # of a step is free during it and may dip in; the next step's constraint lifts it out)
    touch = x[:, 1] - desc.sphere_radius[0] - floor_top_under(x, desc) < 2e-3
    assert touch.sum() >= 20
    assert float(np.abs(v[touch] @ n).mean()) < 0.01
    # contacts exist from the end of the first step on
    expect = 9.8 * np.sin(tilt) * (steps - 1) * h
    assert abs(float((v @ down).mean()) / expect - 1.0) < 0.05


def test_filtered_contacts_without_spheres_change_nothing():
    """A body without contact spheres steps bitwise the same in both modes."""
    desc = meshes.tet_grid(4, 4, 4, seed=2, E=1e5, nu=0.3, pin="y0")
    a = oracle.simulate(desc, 5, kind="port", bits=64, contact_mode=0)
    b = oracle.simulate(desc, 5, kind="port", bits=64, contact_mode=1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_filtered_contacts_newton_iterations():
    """z acts in the first Newton iteration only: three Newton iterations reach the one-iteration
    state up to the Newton tolerance's change (the block settles either way)."""
    desc = meshes.block_on_floor(a=4, b=3, c=4)
    x1, v1, _, _ = oracle.simulate(desc, 30, kind="port", bits=64, contact_mode=1)
    x3, v3, _, _ = oracle.simulate(desc, 30, kind="port", bits=64, contact_mode=1, newton_iters=3)
    assert np.linalg.norm(x3 - x1) / np.linalg.norm(x1 - desc.x) < 0.05


def test_constrained_vertices_end_the_step_at_the_target_normal_velocity():
    """The filtered system's solution has no component along a constrained vertex's normal
    (n^T py = 0 when S = I - n n^T), so dv.n = z.n and a vertex that overlaps the floor at the
    start of a step ends it with v.n = vt = min(0.2 (r - dist), 0.2) / h, recomputed here from the
    floor's geometry, to the PCG's tolerance."""
    tilt, h, s = 0.05, 1.0 / 60.0, 12
    desc = meshes.block_on_floor(tilt=tilt)
    r = desc.sphere_radius[0]
    n = np.array([-np.sin(tilt), np.cos(tilt), 0.0])
    xs, vs, _, _ = oracle.simulate(desc, s, kind="port", bits=64, contact_mode=1, sub_tol=1e-8)
    x1, v1, _, _ = oracle.simulate(desc, s + 1, kind="port", bits=64, contact_mode=1, sub_tol=1e-8)
    sh = desc.world_shapes[0]
    top = np.asarray(sh.translation) + sh.p[1] * n          # a point of the top face
    dist = (xs - top) @ n                                   # sphere centre above the face
    inside = np.abs((xs - np.asarray(sh.translation)) @ np.array([np.cos(tilt), np.sin(tilt), 0.0])) < 0.9
    cons = (dist < r) & inside
    assert cons.sum() >= 20
    vt = np.minimum(0.2 * (r - dist[cons]), 0.2) / h
    # measured: 2e-11 m/s against targets of 0.002-0.024 m/s
    np.testing.assert_allclose(v1[cons] @ n, vt, rtol=0, atol=1e-8)
