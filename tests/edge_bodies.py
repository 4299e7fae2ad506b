"""Degenerate bodies shared by the edge-case tests: free particles (no element), a body whose
vertices are all static, and a single tetrahedron."""
import numpy as np

from bounce_softbody_gb300 import meshes


def _z():
    return np.zeros(0, np.float64)


def particles(n: int = 37, seed: int = 1, damping: float = 0.0) -> meshes.BodyDesc:
    """n dynamic particles without elements or fixtures (unit masses, the reference's rule for a
    dynamic particle without mass), random positions and velocities."""
    rng = np.random.default_rng(seed)
    return meshes.BodyDesc(
        x=rng.uniform(-1.0, 1.0, (n, 3)), v=rng.uniform(-0.5, 0.5, (n, 3)), type=np.full(n, 2, np.int32),
        damping=np.full(n, damping), tets=np.zeros((0, 4), np.uint32), tet_E=_z(), tet_nu=_z(), tet_kdamp=_z(),
        tet_density=_z(), tris=np.zeros((0, 3), np.uint32), tri_Ex=None, tri_Ey=None, tri_Es=None, tri_nuxy=None,
        tri_nuyx=None, tri_kdamp=None, tri_density=_z(), springs=np.zeros((0, 2), np.uint32), spring_L0=_z(),
        spring_ks=_z(), spring_kd=_z(), name=f"particles{n}")


def all_static(seed: int = 2) -> meshes.BodyDesc:
    d = meshes.tet_grid(4, 3, 5, seed=seed, E=1e5, nu=0.3, pin="none", name="static")
    d.type[:] = 0
    return d


def single_tet() -> meshes.BodyDesc:
    """One tetrahedron, vertex 0 static."""
    d = meshes.tet_grid(2, 2, 2, seed=5, E=5e4, nu=0.3, pin="none", name="tet1")
    keep = d.tets[0].astype(np.int64)
    x = d.x[keep]
    d.x, d.v = x, np.zeros_like(x)
    d.type, d.damping = np.array([0, 2, 2, 2], np.int32), d.damping[keep]
    d.tets = np.array([[0, 1, 2, 3]], np.uint32)
    for f in ("tet_E", "tet_nu", "tet_kdamp", "tet_density"):
        setattr(d, f, getattr(d, f)[:1])
    return d


def free_fall(desc, steps: int, h: float):
    """Closed form of backward Euler for unit-mass particles with mass damping c and gravity g:
    (1 + h c) dv = h (g - c v)."""
    x, v = desc.x.copy(), desc.v.copy()
    c = desc.damping[:, None]
    for _ in range(steps):
        v = v + h * (desc.gravity - c * v) / (1.0 + h * c)
        x = x + h * v
    return x, v
