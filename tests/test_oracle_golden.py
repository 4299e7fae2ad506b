"""The oracle (C restatement) against golden vectors produced by the reference library itself.

FP64 restatement vs FP64 reference: the same arithmetic up to summation order, so agreement to
~1e-9 relative, or to within 10x the reference's own FP64 spread when its input moves by one ulp
(stored in the fixture) where the scene amplifies rounding (contacts; a PCG stopped at a loose
tolerance on a stiff cloth). FP32 restatement vs FP32 reference: both sit on the float noise
floor; the bound is a multiple of the reference's own FP32-vs-FP64 spread.
"""
import numpy as np
import pytest
from conftest import GOLDEN_CASES, load_golden

import oracle


def rel_disp(x, xr, x0):
    return float(np.linalg.norm(x - xr) / max(np.linalg.norm(xr - x0), 1e-30))


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_port_matches_reference_golden(name):
    desc, z, st = load_golden(name)
    for s in [int(k) for k in z["steps"]]:
        rx, rv = z[f"ref64_x_{s}"], z[f"ref64_v_{s}"]
        # the reference's own FP32-vs-FP64 spread: its float noise floor on this input
        floor_x = max(rel_disp(z[f"ref32_x_{s}"], rx, desc.x), 1e-7)
        floor_v = max(rel(z[f"ref32_v_{s}"], rv), 1e-6)
        # the FP64 reference's own spread when its input moves by one ulp: how much this scene
        # (contacts, a PCG stopped at a loose tolerance) amplifies rounding
        ulp_x = rel_disp(z[f"ref64ulp_x_{s}"], rx, desc.x)
        ulp_v = rel(z[f"ref64ulp_v_{s}"], rv)
        x64, v64, it64, _ = oracle.simulate(desc, s, kind="port", bits=64, **st)
        ref_it = z[f"ref64_it_{s}"]
        if np.array_equal(it64, ref_it):
            # FP64 restatement vs FP64 reference: summation-order rounding only, amplified at most
            # as much as the scene amplifies it, far below the FP32 floor
            assert rel_disp(x64, rx, desc.x) < max(1e-9, 1e-3 * floor_x, 10 * ulp_x), (name, s)
            assert rel(v64, rv) < max(1e-7, 1e-3 * floor_v, 10 * ulp_v), (name, s)
        else:
            # a step whose residual ends on the stopping threshold (delta <= tol^2 delta0) can stop
            # one PCG iteration apart under a different summation order; the two solutions then
            # differ by one iteration's update, a residual below the tolerance
            assert np.abs(it64.astype(int) - ref_it.astype(int)).max() <= 1, (name, s)
            assert rel_disp(x64, rx, desc.x) < max(1e-9, 1e-3 * floor_x, 0.1 * st["sub_tol"]), (name, s)
            assert rel(v64, rv) < max(1e-7, 1e-3 * floor_v, st["sub_tol"]), (name, s)
        x32, v32, it32, _ = oracle.simulate(desc, s, kind="port", bits=32, **st)
        assert rel_disp(x32, rx, desc.x) < 10 * floor_x + 1e-6, (name, s)
        assert rel(v32, rv) < 10 * floor_v + 1e-5, (name, s)
        assert np.abs(it32.astype(int) - z[f"ref32_it_{s}"].astype(int)).max() <= 2, (name, s)


def test_golden_inputs_match_generators():
    """The committed inputs are the generators' output (seeded, platform independent)."""
    from bounce_softbody_gb300 import meshes

    desc, _, _ = load_golden("tet10")
    g = meshes.config_tet10()
    np.testing.assert_array_equal(desc.tets, g.tets)
    np.testing.assert_allclose(desc.x, g.x, rtol=0, atol=1e-15)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness not built here")
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_port_matches_reference_live(seed):
    """Where the reference is compiled (not on the GPU host), compare on fresh random bodies."""
    from bounce_softbody_gb300 import meshes

    rng = np.random.default_rng(seed)
    a, b, c = (int(k) for k in rng.integers(3, 7, size=3))
    desc = meshes.tet_grid(a, b, c, seed=seed, E=float(10 ** rng.uniform(4, 6)), nu=float(rng.uniform(0.2, 0.45)),
                           pin=["x0", "y0", "z1"][seed], kdamp=0.005 * seed)
    xr, vr, itr, _ = oracle.simulate(desc, 6, kind="ref", bits=64)
    xp, vp, itp, _ = oracle.simulate(desc, 6, kind="port", bits=64)
    assert rel_disp(xp, xr, desc.x) < 1e-9
    assert np.array_equal(itp, itr)


@pytest.mark.parametrize("case", ["bw_pinned", "cloth12"])
def test_port_ray_cast_matches_reference_golden(case):
    """b3Body::RayCastSingle: the restatement's brute-force closest hit against the reference's
    tree query (tests/golden/ray_casts.npz): the same triangles hit, fractions and normals equal
    up to the trajectory's own FP64 rounding spread."""
    import os
    from conftest import GOLDEN

    z = np.load(os.path.join(GOLDEN, "ray_casts.npz"))
    desc, _, st = load_golden(case)
    steps = int(z[f"{case}_steps"])
    hit, tri, frac, normal, _ = oracle.ray_cast(desc, steps, z[f"{case}_seg"], kind="port", bits=64, **st)
    assert np.array_equal(hit, z[f"{case}_ref64_hit"])
    assert np.array_equal(tri[hit], z[f"{case}_ref64_tri"][hit])
    assert np.abs(frac - z[f"{case}_ref64_frac"]).max() < 1e-6
    assert np.abs(normal - z[f"{case}_ref64_normal"]).max() < 1e-6
    assert hit.sum() == 64  # every aimed segment hits, the 16 others miss
