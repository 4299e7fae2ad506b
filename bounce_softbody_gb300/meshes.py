"""Seeded body generators for the workloads this library is measured on.

Every generator returns a :class:`BodyDesc` of plain numpy arrays in the layout the C ABI
(``include/b3g.h``, ``b3g_body_desc``) takes: vertex arrays, element index arrays and
per-element material arrays. The same arrays feed the CUDA path and the CPU oracle, so both
see identical inputs.

The tetrahedral grids split every cell into 6 tetrahedra along its main diagonal (the Kuhn or
Freudenthal split); the reference's testbed ``GridTetMesh`` uses 5 per cell
(examples/testbed/framework/uniform_body.h:424-517), and the workloads here ask for 6.
Cloth grids split each cell into 2 triangles and add structural (distance-1) and bending
(distance-2) springs, with rest lengths measured on the initial positions like
``b3SpringForceDef::Initialize`` (src/bounce_softbody/dynamics/forces/spring_force.cpp:25-35).
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import Optional

import numpy as np

STATIC, KINEMATIC, DYNAMIC = 0, 1, 2  # b3ParticleType (include/bounce_softbody/dynamics/particle.h:31-36)


SHAPE_SPHERE, SHAPE_CAPSULE, SHAPE_BOX, SHAPE_TRIANGLE, SHAPE_MESH, SHAPE_SDF = range(6)
NULL_VERTEX = 0xFFFFFFFF


@dataclasses.dataclass
class WorldShape:
    """A static world fixture's shape (b3g_world_shape). `p` per type: sphere center; capsule
    center1, center2; box half extents; triangle vertex1..3. Box, mesh and SDF carry a transform
    (rotation quaternion x, y, z, w and translation); a mesh its vertices, triangles, optional
    wing vertices (NULL_VERTEX = open edge) and scale; an SDF its voxel grid (grid[0] fastest),
    grid AABB in the shape frame and the invert flag."""
    type: int
    radius: float = 0.0
    friction: float = 0.0
    p: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(9))
    rotation: np.ndarray = dataclasses.field(default_factory=lambda: np.array([0.0, 0.0, 0.0, 1.0]))
    translation: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(3))
    scale: np.ndarray = dataclasses.field(default_factory=lambda: np.ones(3))
    vertices: Optional[np.ndarray] = None     # (V, 3)
    triangles: Optional[np.ndarray] = None    # (T, 3) uint32
    wings: Optional[np.ndarray] = None        # (T, 3) uint32
    voxels: Optional[np.ndarray] = None       # (D, H, W) signed distances
    grid_lower: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(3))
    grid_upper: np.ndarray = dataclasses.field(default_factory=lambda: np.ones(3))
    invert: bool = False


def mesh_wings(triangles: np.ndarray) -> np.ndarray:
    """Wing vertex of every triangle edge as b3Mesh::BuildAdjacency sets it (mesh.cpp:40-94):
    for edge (v_j, v_j+1) of triangle t the vertex opposite the shared edge of the first other
    triangle, in index order, that holds the reversed edge; NULL_VERTEX when there is none."""
    T = np.asarray(triangles, np.int64)
    holders = {}  # directed edge -> triangles holding it, ascending, with the edge's position
    for t in range(T.shape[0]):
        for j in range(3):
            holders.setdefault((int(T[t, j]), int(T[t, (j + 1) % 3])), []).append((t, j))
    wings = np.full(T.shape, NULL_VERTEX, np.uint32)
    for t in range(T.shape[0]):
        for j in range(3):
            for t2, j2 in holders.get((int(T[t, (j + 1) % 3]), int(T[t, j])), []):
                if t2 != t:
                    wings[t, j] = T[t2, (j2 + 2) % 3]
                    break
    return wings


@dataclasses.dataclass
class BodyDesc:
    x: np.ndarray                      # (n, 3) float64 positions (also the rest state)
    v: np.ndarray                      # (n, 3) float64 velocities
    type: np.ndarray                   # (n,) int32 particle types
    damping: np.ndarray                # (n,) float64 mass damping
    tets: np.ndarray                   # (T, 4) uint32
    tet_E: np.ndarray                  # (T,) Young modulus
    tet_nu: np.ndarray                 # (T,) Poisson ratio
    tet_kdamp: np.ndarray              # (T,) stiffness damping
    tet_density: np.ndarray            # (T,) density of the mass fixture
    tris: np.ndarray                   # (Tr, 3) uint32
    tri_Ex: Optional[np.ndarray]       # the five element arrays None = mass fixtures only
    tri_Ey: Optional[np.ndarray]
    tri_Es: Optional[np.ndarray]
    tri_nuxy: Optional[np.ndarray]
    tri_nuyx: Optional[np.ndarray]
    tri_kdamp: Optional[np.ndarray]
    tri_density: np.ndarray
    springs: np.ndarray                # (S, 2) uint32
    spring_L0: np.ndarray
    spring_ks: np.ndarray
    spring_kd: np.ndarray
    sphere_radius: Optional[np.ndarray] = None    # (n,) per-vertex contact radius
    sphere_friction: Optional[np.ndarray] = None  # (n,)
    world_spheres: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 5)))
    gravity: np.ndarray = dataclasses.field(default_factory=lambda: np.array([0.0, -9.8, 0.0]))
    name: str = "body"
    world_shapes: list = dataclasses.field(default_factory=list)   # WorldShape, after the spheres
    # Baraff-Witkin cloth forces and mouse springs (b3StretchForceDef, b3ShearForceDef,
    # b3MouseForceDef). uv None = the defs' Initialize from the initial positions.
    stretch_tris: np.ndarray = dataclasses.field(default_factory=lambda: _empty_elems(3))
    stretch_uv: Optional[np.ndarray] = None      # (St, 6): u1, v1, u2, v2, u3, v3
    stretch_params: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 6)))
    shear_tris: np.ndarray = dataclasses.field(default_factory=lambda: _empty_elems(3))
    shear_uv: Optional[np.ndarray] = None
    shear_params: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 2)))
    mouse_ids: np.ndarray = dataclasses.field(default_factory=lambda: _empty_elems(4))
    mouse_params: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 6)))

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def tet_rest(self) -> np.ndarray:
        return self.x[self.tets.astype(np.int64)]

    @property
    def tri_rest(self) -> np.ndarray:
        return self.x[self.tris.astype(np.int64)]


def _empty_elems(k):
    return np.zeros((0, k), np.uint32)


def _z():
    return np.zeros(0, np.float64)


def kuhn_cells(a: int, b: int, c: int) -> np.ndarray:
    """Tetrahedra of an a x b x c vertex grid, 6 per cell, vertex id = i + a*(j + b*k).

    Each cell is split along the diagonal from corner (0,0,0) to (1,1,1): one tetrahedron per
    ordering of the three axes. Orientation is made positive (det > 0) on the regular grid.
    """
    i, j, k = np.meshgrid(np.arange(a - 1), np.arange(b - 1), np.arange(c - 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()

    def vid(di, dj, dk):
        return (i + di) + a * ((j + dj) + b * (k + dk))

    axes = np.eye(3, dtype=np.int64)
    tets = []
    for perm in itertools.permutations(range(3)):
        p0 = np.zeros(3, np.int64)
        p1 = p0 + axes[perm[0]]
        p2 = p1 + axes[perm[1]]
        p3 = p2 + axes[perm[2]]
        corners = [p0, p1, p2, p3]
        e = np.stack([corners[1] - p0, corners[2] - p0, corners[3] - p0])
        if np.linalg.det(e.astype(np.float64)) < 0:
            corners[1], corners[2] = corners[2], corners[1]
        tets.append(np.stack([vid(*q) for q in corners], axis=1))
    # cell-major order: the 6 tetrahedra of a cell are adjacent
    t = np.stack(tets, axis=1).reshape(-1, 4)
    return t.astype(np.uint32)


def tet_grid(a: int, b: int, c: int, spacing: float = 0.1, jitter: float = 0.01, seed: int = 0,
             E: float = 1e5, nu: float = 0.3, density: float = 1000.0, damping: float = 0.01,
             pin: str = "y0", kdamp: float = 0.0, origin=(0.0, 0.0, 0.0),
             rng: Optional[np.random.Generator] = None, name: str = "") -> BodyDesc:
    """Kuhn-split tetrahedral block of a x b x c vertices.

    Rest positions are the grid points jittered by seeded uniform noise of +-jitter*spacing
    per coordinate. ``pin`` selects the static vertices: "y0" (grid layer j = 0), one of
    "x0", "x1", "y1", "z0", "z1" (a face of the block) or "none".
    """
    rng = rng if rng is not None else np.random.default_rng(seed)
    i, j, k = np.meshgrid(np.arange(a), np.arange(b), np.arange(c), indexing="ij")
    # vertex id = i + a*(j + b*k): iterate k slowest
    i = np.transpose(i, (2, 1, 0)).ravel()
    j = np.transpose(j, (2, 1, 0)).ravel()
    k = np.transpose(k, (2, 1, 0)).ravel()
    x = np.stack([i, j, k], axis=1).astype(np.float64) * spacing + np.asarray(origin, np.float64)
    x += rng.uniform(-jitter * spacing, jitter * spacing, size=x.shape)
    n = x.shape[0]
    types = np.full(n, DYNAMIC, np.int32)
    faces = {"x0": i == 0, "x1": i == a - 1, "y0": j == 0, "y1": j == b - 1, "z0": k == 0, "z1": k == c - 1}
    if pin != "none":
        types[faces[pin]] = STATIC
    tets = kuhn_cells(a, b, c)
    T = tets.shape[0]
    return BodyDesc(
        x=x, v=np.zeros_like(x), type=types, damping=np.full(n, damping),
        tets=tets, tet_E=np.full(T, E), tet_nu=np.full(T, nu), tet_kdamp=np.full(T, kdamp),
        tet_density=np.full(T, density),
        tris=_empty_elems(3), tri_Ex=_z(), tri_Ey=_z(), tri_Es=_z(), tri_nuxy=_z(), tri_nuyx=_z(),
        tri_kdamp=_z(), tri_density=_z(),
        springs=_empty_elems(2), spring_L0=_z(), spring_ks=_z(), spring_kd=_z(),
        name=name or f"tet{a}x{b}x{c}",
    )


def cloth_grid(m: int = 128, side: float = 2.0, height: float = 1.0, E_t: float = 50.0,
               nu: float = 0.3, areal_density: float = 0.2, ks: float = 1e3, kd: float = 5.0,
               contact_radius: float = 0.01, friction: float = 0.3, sphere_radius: float = 0.5,
               sphere_center=(0.0, 0.0, 0.0), pinned_corners: int = 2, damping: float = 0.0,
               name: str = "") -> BodyDesc:
    """m x m cloth in the y = height plane centred over a static sphere.

    Triangle elements carry membrane stiffness E*t = ``E_t`` in both directions, shear modulus
    E*t / (2(1+nu)) and Poisson ratio nu (b3TriangleElementForce has no thickness parameter).
    Springs: structural (grid neighbours) and bending (distance 2) with stiffness ``ks`` and
    damping ``kd``. Every vertex carries a contact sphere of ``contact_radius``.
    """
    h = side / (m - 1)
    jj, ii = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()  # vertex id = i + m*j
    x = np.stack([-0.5 * side + ii * h, np.full(ii.shape, height), -0.5 * side + jj * h], axis=1)
    n = m * m
    types = np.full(n, DYNAMIC, np.int32)
    if pinned_corners >= 1:
        types[0] = STATIC
    if pinned_corners >= 2:
        types[m - 1] = STATIC
    ci, cj = np.meshgrid(np.arange(m - 1), np.arange(m - 1), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    v00 = ci + m * cj
    v10 = v00 + 1
    v01 = v00 + m
    v11 = v01 + 1
    tris = np.concatenate([np.stack([v00, v01, v10], 1), np.stack([v10, v01, v11], 1)]).astype(np.uint32)
    Tr = tris.shape[0]
    springs = []
    for di, dj in ((1, 0), (0, 1)):
        for d in (1, 2):
            mi = (ii + d * di < m) & (jj + d * dj < m)
            a0 = (ii + m * jj)[mi]
            springs.append(np.stack([a0, a0 + d * di + m * d * dj], 1))
    springs = np.concatenate(springs).astype(np.uint32)
    L0 = np.linalg.norm(x[springs[:, 0]] - x[springs[:, 1]], axis=1)
    S = springs.shape[0]
    Es = E_t / (2.0 * (1.0 + nu))
    return BodyDesc(
        x=x, v=np.zeros_like(x), type=types, damping=np.full(n, damping),
        tets=_empty_elems(4), tet_E=_z(), tet_nu=_z(), tet_kdamp=_z(), tet_density=_z(),
        tris=tris, tri_Ex=np.full(Tr, E_t), tri_Ey=np.full(Tr, E_t), tri_Es=np.full(Tr, Es),
        tri_nuxy=np.full(Tr, nu), tri_nuyx=np.full(Tr, nu), tri_kdamp=np.zeros(Tr),
        tri_density=np.full(Tr, areal_density),
        springs=springs, spring_L0=L0, spring_ks=np.full(S, ks), spring_kd=np.full(S, kd),
        sphere_radius=np.full(n, contact_radius), sphere_friction=np.full(n, friction),
        world_spheres=np.array([[*sphere_center, sphere_radius, friction]], np.float64),
        name=name or f"cloth{m}",
    )


def bw_cloth(m: int = 10, side: float = 2.0, height: float = 1.0, density: float = 0.2,
             stretch_ks: float = 1e5, stretch_kd: float = 0.0, shear_ks: float = 0.0, shear_kd: float = 0.0,
             pinned: str = "edges", mouse: bool = False, mouse_ks: float = 1e5, mouse_kd: float = 1e3,
             mouse_offset=(0.0, -0.3, 0.0), damping: float = 0.0, name: str = "") -> BodyDesc:
    """m x m cloth of the reference testbed's kind: triangle mass fixtures of ``density`` and one
    Baraff-Witkin stretch force per triangle (b_u = b_v = 1, rest frame from Initialize), as
    UniformBody builds a ClothDef with createElements = false; optionally one shear force per
    triangle and a mouse spring as BodyDragger makes it: a static particle at the centre of a
    triangle moved by ``mouse_offset``, weights (1/3, 1/3, 1/3), length 0.

    ``pinned``: "edges" (the border, as PinnedCloth), "row" (the first row, as StretchMapping),
    "corners" (two corners) or "none".
    """
    h = side / (m - 1)
    jj, ii = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()  # vertex id = i + m*j
    x = np.stack([-0.5 * side + ii * h, np.full(ii.shape, height), -0.5 * side + jj * h], axis=1)
    n = m * m
    types = np.full(n, DYNAMIC, np.int32)
    if pinned == "edges":
        types[(ii == 0) | (ii == m - 1) | (jj == 0) | (jj == m - 1)] = STATIC
    elif pinned == "row":
        types[jj == 0] = STATIC
    elif pinned == "corners":
        types[0] = STATIC
        types[m - 1] = STATIC
    ci, cj = np.meshgrid(np.arange(m - 1), np.arange(m - 1), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    v00 = ci + m * cj
    v10 = v00 + 1
    v01 = v00 + m
    v11 = v01 + 1
    tris = np.concatenate([np.stack([v00, v01, v10], 1), np.stack([v10, v01, v11], 1)]).astype(np.uint32)
    Tr = tris.shape[0]
    stretch = np.tile([stretch_ks, stretch_kd, 1.0, stretch_ks, stretch_kd, 1.0], (Tr, 1)).astype(np.float64)
    desc = BodyDesc(
        x=x, v=np.zeros_like(x), type=types, damping=np.full(n, damping),
        tets=_empty_elems(4), tet_E=_z(), tet_nu=_z(), tet_kdamp=_z(), tet_density=_z(),
        tris=tris, tri_Ex=None, tri_Ey=None, tri_Es=None, tri_nuxy=None, tri_nuyx=None, tri_kdamp=None,
        tri_density=np.full(Tr, density),
        springs=_empty_elems(2), spring_L0=_z(), spring_ks=_z(), spring_kd=_z(),
        stretch_tris=tris.copy(), stretch_params=stretch,
        name=name or f"bwcloth{m}",
    )
    if shear_ks > 0.0 or shear_kd > 0.0:
        desc.shear_tris = tris.copy()
        desc.shear_params = np.tile([shear_ks, shear_kd], (Tr, 1)).astype(np.float64)
    if mouse:
        t = tris[Tr // 2 + (m - 1) // 2]
        c = x[t.astype(np.int64)].mean(axis=0) + np.asarray(mouse_offset, np.float64)
        desc.x = np.concatenate([x, c[None, :]])
        desc.v = np.zeros_like(desc.x)
        desc.type = np.concatenate([types, np.array([STATIC], np.int32)])
        desc.damping = np.full(n + 1, damping)
        desc.mouse_ids = np.array([[n, t[0], t[1], t[2]]], np.uint32)
        desc.mouse_params = np.array([[1.0 / 3.0, 1.0 / 3.0, 1.0 - 2.0 / 3.0, mouse_ks, mouse_kd, 0.0]])
    return desc


def batch_bodies(count: int = 512, lo: int = 4, hi: int = 40, seed: int = 3, spacing: float = 0.1,
                 density: float = 1000.0, damping: float = 0.01) -> list[BodyDesc]:
    """Independent tetrahedral blocks of uneven size.

    Sizes a, b, c ~ U{lo..hi}; Young modulus log-uniform in [1e4, 1e6]; Poisson ratio
    U[0.2, 0.45]; rest positions jittered by +-1% of the spacing; one random face pinned.
    """
    rng = np.random.default_rng(seed)
    faces = ["x0", "x1", "y0", "y1", "z0", "z1"]
    out = []
    for bidx in range(count):
        a, b, c = (int(s) for s in rng.integers(lo, hi + 1, size=3))
        E = float(10.0 ** rng.uniform(4.0, 6.0))
        nu = float(rng.uniform(0.2, 0.45))
        face = faces[int(rng.integers(0, 6))]
        out.append(tet_grid(a, b, c, spacing=spacing, jitter=0.01, E=E, nu=nu, density=density,
                            damping=damping, pin=face, rng=rng, name=f"batch{bidx}_{a}x{b}x{c}"))
    return out


def config_tet10(seed: int = 0) -> BodyDesc:
    """10x10x10 vertex block, 4374 tets, E=1e5, nu=0.3, rho=1000, damping 0.01, y=0 pinned."""
    return tet_grid(10, 10, 10, spacing=0.1, jitter=0.01, seed=seed, E=1e5, nu=0.3,
                    density=1000.0, damping=0.01, pin="y0", name="tet10")


def config_tet64(seed: int = 0) -> BodyDesc:
    """64^3 vertex block (262,144 vertices, 1,500,282 tets), E=1e6, nu=0.45."""
    return tet_grid(64, 64, 64, spacing=0.1, jitter=0.01, seed=seed, E=1e6, nu=0.45,
                    density=1000.0, damping=0.01, pin="y0", name="tet64")


def config_cloth128() -> BodyDesc:
    """128^2 cloth (16,384 vertices, 32,258 triangles, 64,768 springs) over a r=0.5 sphere."""
    return cloth_grid(128, name="cloth128")


def serving_bodies(count: int = 256, seed: int = 5) -> list[BodyDesc]:
    """Bodies of a serving stream: half tetrahedral blocks, half cloths (seeded).

    A block has a vertex count log-uniform in [1e3, 1e5], split into a x b x c with aspect ratios
    up to about 1.4, Young modulus log-uniform in [1e4, 1e6], Poisson ratio U[0.2, 0.45] and one
    random face pinned. A cloth is an m x m grid with m log-uniform in [32, 256], membrane
    stiffness E*t U[25, 100], springs of stiffness 1e3 and damping 5, two corners pinned, over a
    static sphere with contacts and friction 0.3.
    """
    rng = np.random.default_rng(seed)
    faces = ["x0", "x1", "y0", "y1", "z0", "z1"]
    out = []
    for k in range(count):
        if rng.random() < 0.5:
            nv = float(np.exp(rng.uniform(np.log(1e3), np.log(1e5))))
            f = np.exp(rng.uniform(-0.33, 0.33, size=3))
            f /= np.cbrt(np.prod(f))
            a, b, c = (max(4, int(round(np.cbrt(nv) * s))) for s in f)
            E = float(10.0 ** rng.uniform(4.0, 6.0))
            nu = float(rng.uniform(0.2, 0.45))
            face = faces[int(rng.integers(0, 6))]
            out.append(tet_grid(a, b, c, E=E, nu=nu, pin=face, rng=rng, name=f"serve{k}_tet{a}x{b}x{c}"))
        else:
            m = int(round(np.exp(rng.uniform(np.log(32), np.log(256)))))
            E_t = float(rng.uniform(25.0, 100.0))
            out.append(cloth_grid(m, E_t=E_t, name=f"serve{k}_cloth{m}"))
    return out


def _quat_axis_angle(axis, angle):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    return np.array([*(np.sin(0.5 * angle) * axis), np.cos(0.5 * angle)])


def block_on_floor(a: int = 5, b: int = 4, c: int = 5, tilt: float = 0.05, seed: int = 4, E: float = 2e5,
                   nu: float = 0.33, radius: float = 0.03, friction: float = 0.3) -> BodyDesc:
    """A free Kuhn tet block (spacing 0.1, density 1000: about 50 kg for 5 x 4 x 5 vertices) with a
    contact sphere of `radius` on every vertex, resting with its lowest layer on a static box floor
    (1 x 0.05 x 1 half extents, tilted `tilt` rad about z) that its spheres already overlap. The
    reference's penalty contact (stiffness 1000) cannot carry its weight: the block sinks through
    the floor; filtered contacts hold it."""
    d = tet_grid(a, b, c, seed=seed, E=E, nu=nu, pin="none", name=f"floor{a}{b}{c}")
    d.sphere_radius = np.full(d.n, radius)
    d.sphere_friction = np.full(d.n, friction)
    d.world_shapes = [WorldShape(SHAPE_BOX, radius=0.0, friction=0.5, p=np.array([1.0, 0.05, 1.0, 0, 0, 0, 0, 0, 0]),
                                 rotation=_quat_axis_angle([0, 0, 1], tilt), translation=np.array([0.2, -0.07, 0.2]))]
    return d


def shape_scene(kind: str, m: int = 12, height: float = 0.05) -> BodyDesc:
    """An m x m cloth (side 0.8, contact radius 0.01, friction 0.3, two corners pinned) hanging
    just above one static world shape of the given kind: "capsule" (horizontal, r = 0.2), "box"
    (0.4 x 0.1 x 0.4 half extents, tilted 0.3 rad about z), "triangle" (a large tilted
    triangle), "mesh" (a 6 x 6 bumpy height-field mesh with wing vertices, scaled and rotated)
    or "sdf" (a 16^3 voxel grid of the signed distance to a sphere of radius 0.3). The cloth's
    lowest vertex starts `height` above the shape's top."""
    cloth = cloth_grid(m, side=0.8, height=0.0, contact_radius=0.01, friction=0.3, name=f"{kind}{m}")
    cloth.world_spheres = np.zeros((0, 5))
    fr = 0.4
    if kind == "capsule":
        sh = WorldShape(SHAPE_CAPSULE, radius=0.2, friction=fr, p=np.array([-0.5, 0, 0.05, 0.5, 0, -0.05, 0, 0, 0]))
        top = 0.2
    elif kind == "box":
        sh = WorldShape(SHAPE_BOX, radius=0.0, friction=fr, p=np.array([0.4, 0.1, 0.4, 0, 0, 0, 0, 0, 0]),
                        rotation=_quat_axis_angle([0, 0, 1], 0.3), translation=np.array([0.0, 0.0, 0.0]))
        top = 0.1 * np.cos(0.3) + 0.4 * np.sin(0.3)
    elif kind == "triangle":
        sh = WorldShape(SHAPE_TRIANGLE, radius=0.0, friction=fr,
                        p=np.array([-1.2, -0.05, -1.0, 1.2, 0.05, -1.0, 0.0, 0.0, 1.3]))
        top = 0.05 * 0.4 / 1.2  # the plane's height under the cloth's highest corner
    elif kind == "mesh":
        g = 6
        xs = np.linspace(-0.6, 0.6, g)
        X, Z = np.meshgrid(xs, xs, indexing="ij")
        Y = 0.05 * np.sin(3.0 * X) * np.cos(2.0 * Z)
        verts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
        tris = []
        for i in range(g - 1):
            for j in range(g - 1):
                a, b, c, d = i * g + j, (i + 1) * g + j, i * g + j + 1, (i + 1) * g + j + 1
                tris += [[a, c, b], [b, c, d]]
        tris = np.array(tris, np.uint32)
        sh = WorldShape(SHAPE_MESH, radius=0.0, friction=fr, vertices=verts, triangles=tris, wings=mesh_wings(tris),
                        scale=np.array([1.1, 1.0, 0.9]), rotation=_quat_axis_angle([0, 1, 0], 0.2),
                        translation=np.array([0.0, -0.02, 0.0]))
        top = 0.05 - 0.02
    elif kind == "sdf":
        n = 16
        lo, hi = -0.5, 0.5
        ax = np.linspace(lo, hi, n)
        Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")  # voxels (k, j, i): x fastest
        vox = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - 0.3
        sh = WorldShape(SHAPE_SDF, radius=0.0, friction=fr, voxels=vox, grid_lower=np.full(3, lo),
                        grid_upper=np.full(3, hi), rotation=np.array([0.0, 0.0, 0.0, 1.0]))
        top = 0.3
    else:
        raise ValueError(kind)
    cloth.x = cloth.x.copy()
    cloth.x[:, 1] = top + 0.01 + height
    cloth.world_shapes = [sh]
    return cloth
