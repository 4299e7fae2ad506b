"""The CUDA step (through the C ABI) against golden vectors produced by the reference itself
(FP32 and FP64 builds of the reference, tests/golden/make_golden.py).

Bound: positions within 1e-4 of the FP64 reference relative to the displacement (or 20x the
reference's own FP32-vs-FP64 spread where the scene amplifies rounding), velocities within 1e-3
relative (or 20x that spread); PCG iteration counts within 3 of the FP32 reference's.
"""
import numpy as np
import pytest
from conftest import BW_CASES, GOLDEN_CASES, SHAPE_CASES, load_golden

from bounce_softbody_gb300 import b3g

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def rel_disp(x, xr, x0):
    return float(np.linalg.norm(np.asarray(x, np.float64) - xr) / max(np.linalg.norm(xr - x0), 1e-30))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_gpu_matches_reference_golden(ctx, name):
    desc, z, st = load_golden(name)
    cfg = b3g.solver_config(force_iterations=st["newton_iters"], max_pcg_iterations=st["max_sub"],
                            pcg_tolerance=st["sub_tol"])
    g = b3g.Body(ctx, desc)
    done = 0
    for s in [int(k) for k in z["steps"]]:
        its = []
        while done < s:
            its.append(g.step(DT, cfg)["pcg_iterations"])
            done += 1
        x, v = g.state()
        rx, rv = z[f"ref64_x_{s}"], z[f"ref64_v_{s}"]
        floor_x = rel_disp(z[f"ref32_x_{s}"], rx, desc.x)
        floor_v = rel(z[f"ref32_v_{s}"], rv)
        assert rel_disp(x, rx, desc.x) < max(1e-4, 20 * floor_x), (name, s)
        assert rel(v, rv) < max(1e-3, 20 * floor_v), (name, s)
        ref_it = int(z[f"ref32_it_{s}"][-1])
        # contact scenes are chaotic: their iteration counts wander with the trajectory
        slack = max(3, int(0.35 * ref_it)) if ("contact" in name or name.startswith("shape_")) else 3
        assert abs(its[-1] - ref_it) <= slack, (name, s, its[-1])
    g.close()


@pytest.mark.parametrize("group", [SHAPE_CASES, BW_CASES], ids=["shapes", "cloth_forces"])
def test_batched_group_matches_reference_golden(ctx, group):
    """Scenes of one kind stepped together by the persistent batch kernels (one launch for the
    group: the five world-shape kinds, or the four Baraff-Witkin / mouse-spring cloths) against
    the same golden vectors, each at its own snapshot steps."""
    loaded = [load_golden(name) for name in group]
    st = loaded[0][2]
    cfg = b3g.solver_config(max_pcg_iterations=st["max_sub"], pcg_tolerance=st["sub_tol"])
    bodies = [b3g.Body(ctx, desc) for desc, _, _ in loaded]
    snaps = sorted({int(k) for _, z, _ in loaded for k in z["steps"]})
    done = 0
    for s in snaps:
        b3g.step_batch(ctx, bodies, DT, s - done, cfg, stats=False)
        done = s
        for (desc, z, _), g, name in zip(loaded, bodies, group):
            if s not in [int(k) for k in z["steps"]]:
                continue
            x, v = g.state()
            rx, rv = z[f"ref64_x_{s}"], z[f"ref64_v_{s}"]
            floor_x = rel_disp(z[f"ref32_x_{s}"], rx, desc.x)
            floor_v = rel(z[f"ref32_v_{s}"], rv)
            assert rel_disp(x, rx, desc.x) < max(1e-4, 20 * floor_x), (name, s)
            assert rel(v, rv) < max(1e-3, 20 * floor_v), (name, s)
    for g in bodies:
        g.close()
