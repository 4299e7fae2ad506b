import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path through the C ABI)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    from bounce_softbody_gb300 import b3g

    c = b3g.Context(0)
    yield c
    c.close()


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SHAPE_CASES = ["shape_capsule", "shape_box", "shape_triangle", "shape_mesh", "shape_sdf"]
BW_CASES = ["bw_pinned", "bw_stretch_map", "bw_shear", "bw_mouse"]
GOLDEN_CASES = ["tet10", "tet10_bodystep", "tet4", "tet6_newton", "single_tet", "cloth12", "cloth12_contact"] + \
    SHAPE_CASES + BW_CASES


def load_golden(name):
    """A golden fixture made by the reference itself: (BodyDesc, arrays, run settings)."""
    import numpy as np

    from bounce_softbody_gb300 import meshes

    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    kw = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    gravity = kw.pop("gravity")
    world = kw.pop("world_spheres")
    sr = kw.pop("sphere_radius", None)
    sf = kw.pop("sphere_friction", None)
    shapes = []
    k = 0
    while f"shape{k}_type" in z.files:
        fields = {f[len(f"shape{k}_"):]: z[f] for f in z.files if f.startswith(f"shape{k}_")}
        t = int(fields.pop("type"))
        for f in ("radius", "friction", "invert"):
            if f in fields:
                fields[f] = fields[f].item()
        shapes.append(meshes.WorldShape(t, **fields))
        k += 1
    for f in ("tri_Ex", "tri_Ey", "tri_Es", "tri_nuxy", "tri_nuyx", "tri_kdamp"):
        kw.setdefault(f, None)  # mass-only triangle fixtures
    desc = meshes.BodyDesc(**kw, sphere_radius=sr, sphere_friction=sf, world_spheres=world, gravity=gravity, name=name,
                           world_shapes=shapes)
    st = z["settings"]
    settings = dict(max_sub=int(st[0]), sub_tol=float(st[1]), newton_iters=int(st[2]))
    return desc, z, settings
