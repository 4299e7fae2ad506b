"""Cloth (triangles, springs, sphere contact, friction), Baraff-Witkin stretch / shear forces and
mouse springs, precision variants, preconditioners, Newton iterations and the particle API of the
CUDA path, against the oracle."""
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


def gpu_run(ctx, desc, steps, cfg):
    g = b3g.Body(ctx, desc)
    its = [g.step(DT, cfg)["pcg_iterations"] for _ in range(steps)]
    x, v = g.state()
    m = g.masses()
    g.close()
    return x, v, its, m


@pytest.mark.parametrize("m,steps,height", [(12, 6, 0.52), (24, 8, 0.52), (32, 4, 0.53)])
def test_cloth_contact_friction_matches_oracle(ctx, m, steps, height):
    """Cloth over a sphere: triangle elements, structural and bending springs, penalty contact
    and Coulomb friction impulses (the reference's contact semantics). The scene is chaotic
    (tension-only springs start at rest length), so parity is checked over a short horizon
    against the float noise floor the reference itself shows between FP32 and FP64."""
    desc = meshes.cloth_grid(m, side=1.2, height=height, sphere_radius=0.5, contact_radius=0.05)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    x, v, its, m_gpu = gpu_run(ctx, desc, steps, cfg)
    x64, v64, it64, _ = oracle.simulate(desc, steps, kind="port", bits=64)
    x32, v32, _, _ = oracle.simulate(desc, steps, kind="port", bits=32)
    # the cloth touched the sphere: some vertex ended inside the contact shell
    r = np.linalg.norm(x64 - desc.world_spheres[0, :3], axis=1)
    assert r.min() < 0.5 + 0.05 + 1e-3
    floor_x = rel_disp(x32, x64, desc.x)
    assert rel_disp(x, x64, desc.x) < max(1e-4, 20 * floor_x)
    floor_v = rel(v32, v64)
    assert rel(v, v64) < max(1e-3, 20 * floor_v)


def test_lumped_masses_match_oracle_rule(ctx):
    desc = meshes.cloth_grid(8, side=1.0)
    g = b3g.Body(ctx, desc)
    m = g.masses()
    g.close()
    area = 0.5 * (1.0 / 7) ** 2
    expected = np.zeros(desc.n)
    for t in desc.tris:
        expected[t] += desc.tri_density[0] * area / 3
    expected[desc.type != 2] = 0.0
    np.testing.assert_allclose(m, expected, rtol=1e-5)


@pytest.mark.parametrize("precision", [b3g.PRECISION_FP64, b3g.PRECISION_BF16])
def test_precision_variants_reach_tolerance(ctx, precision):
    """FP64 PCG and BF16-stored blocks (FP32 refinement) both end within 1e-4 of the FP64 oracle."""
    desc = meshes.tet_grid(8, 8, 8, seed=5, E=1e6, nu=0.45, pin="y0")
    cfg = b3g.solver_config(max_pcg_iterations=1000, pcg_tolerance=1e-5, precision=precision, refresh_period=25)
    x, v, its, _ = gpu_run(ctx, desc, 10, cfg)
    x64, v64, _, _ = oracle.simulate(desc, 10, kind="port", bits=64, max_sub=1000)
    assert rel_disp(x, x64, desc.x) < 1e-4
    assert rel(v, v64) < 1e-3


def test_block_jacobi_converges_to_same_state(ctx):
    desc = meshes.tet_grid(7, 9, 6, seed=2, E=2e5, nu=0.4, pin="x0")
    cfg_j = b3g.solver_config(max_pcg_iterations=500, pcg_tolerance=1e-7)
    cfg_b = b3g.solver_config(max_pcg_iterations=500, pcg_tolerance=1e-7, preconditioner=b3g.PRECOND_BLOCK_JACOBI)
    xj, vj, itj, _ = gpu_run(ctx, desc, 5, cfg_j)
    xb, vb, itb, _ = gpu_run(ctx, desc, 5, cfg_b)
    assert rel_disp(xb, xj.astype(np.float64), desc.x) < 1e-5
    assert itb[-1] <= itj[-1] + 2


def test_newton_iterations_match_oracle(ctx):
    desc = meshes.tet_grid(6, 6, 6, seed=9, E=5e4, nu=0.3, pin="y0", kdamp=0.01)
    cfg = b3g.solver_config(force_iterations=3, max_pcg_iterations=200, pcg_tolerance=1e-6)
    x, v, its, _ = gpu_run(ctx, desc, 8, cfg)
    x64, v64, _, _ = oracle.simulate(desc, 8, kind="port", bits=64, newton_iters=3, sub_tol=1e-6)
    assert rel_disp(x, x64, desc.x) < 1e-4
    assert rel(v, v64) < 1e-3


def test_stiffness_damping_matches_oracle(ctx):
    desc = meshes.tet_grid(6, 7, 5, seed=4, E=1e5, nu=0.3, pin="z0", kdamp=0.02)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    x, v, _, _ = gpu_run(ctx, desc, 10, cfg)
    x64, v64, _, _ = oracle.simulate(desc, 10, kind="port", bits=64)
    assert rel_disp(x, x64, desc.x) < 1e-4


def test_particle_api_forces_translations_types(ctx):
    """ApplyForce / ApplyTranslation act for one step and are then cleared; SetType(static)
    zeroes the velocity and pins the vertex."""
    desc = meshes.tet_grid(5, 5, 5, seed=1, pin="y0")
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    g = b3g.Body(ctx, desc)
    g.step(DT, cfg)
    x1, v1 = g.state()
    f = np.zeros((desc.n, 3), np.float32)
    top = np.where(desc.x[:, 1] > desc.x[:, 1].max() - 1e-3)[0]
    f[top, 0] = 50.0
    g.apply_forces(f)
    t = np.zeros((desc.n, 3), np.float32)
    t[desc.type == 0, 2] = 0.01  # move the pinned layer (translation applies to every vertex)
    g.apply_translations(t)
    g.step(DT, cfg)
    x2, v2 = g.state()
    assert x2[top, 0].mean() > x1[top, 0].mean()
    pinned = desc.type == 0
    np.testing.assert_allclose(x2[pinned, 2] - x1[pinned, 2], 0.01, atol=1e-6)
    # forces and translations were cleared: a third step moves pinned vertices no more
    g.step(DT, cfg)
    x3, _ = g.state()
    np.testing.assert_allclose(x3[pinned], x2[pinned], atol=1e-7)
    types = desc.type.copy()
    types[top] = 0
    g.set_types(types)
    _, v4 = g.state()
    assert np.abs(v4[top]).max() == 0.0
    g.step(DT, cfg)
    x5, v5 = g.state()
    np.testing.assert_allclose(x5[top], x3[top], atol=1e-7)
    assert g.masses()[top].max() == 0.0
    g.close()


def test_rotations_roundtrip_and_determinism(ctx):
    """The per-tet rotation state is device resident, readable and restorable; restoring state
    and rotations reproduces the next step bitwise (checkpoint / resume)."""
    desc = meshes.tet_grid(6, 6, 6, seed=3, pin="y0")
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    g = b3g.Body(ctx, desc)
    for _ in range(4):
        g.step(DT, cfg)
    x, v = g.state()
    q = g.rotations()
    assert np.allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-5)
    g.step(DT, cfg)
    xa, va = g.state()
    g.set_state(x, v)
    g.set_rotations(q)
    g.step(DT, cfg)
    xb, vb = g.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    g.close()


def _quat_mat(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def test_rotations_come_back_in_element_order(ctx):
    """Tetrahedra are stored grouped by vertex-offset signature, not in the caller's order; the
    rotations read back are in the caller's order. The tetrahedra of a block are shuffled, the
    body steps (the last step extracts each rotation from the deformation gradient of the state
    it starts from), and every returned rotation is the polar rotation of its own tetrahedron's
    gradient (numpy SVD), to the float tolerance of the iteration."""
    desc = meshes.tet_grid(6, 5, 7, seed=4, pin="y0")
    rng = np.random.default_rng(2)
    perm = rng.permutation(desc.tets.shape[0])
    for k in ("tets", "tet_E", "tet_nu", "tet_kdamp", "tet_density"):
        setattr(desc, k, np.asarray(getattr(desc, k))[perm].copy())
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    g = b3g.Body(ctx, desc)
    for _ in range(3):
        g.step(DT, cfg)
    x, _ = g.state()
    g.step(DT, cfg)
    q = g.rotations()
    rest = np.asarray(desc.x, np.float64)
    cur = np.asarray(x, np.float64)
    worst = 0.0
    for e, t in enumerate(np.asarray(desc.tets)):
        Dm = np.stack([rest[t[k]] - rest[t[0]] for k in (1, 2, 3)], axis=1)
        Ds = np.stack([cur[t[k]] - cur[t[0]] for k in (1, 2, 3)], axis=1)
        F = Ds @ np.linalg.inv(Dm)
        U, _, Vt = np.linalg.svd(F)
        R = U @ Vt
        worst = max(worst, float(np.abs(_quat_mat(q[e]) - R).max()))
    assert worst < 1e-4, worst
    g.close()


def test_nonfinite_input_reports_status(ctx):
    """A NaN external force makes the solve report NONFINITE instead of failing silently."""
    desc = meshes.tet_grid(4, 4, 4, seed=1, pin="y0")
    g = b3g.Body(ctx, desc)
    f = np.zeros((desc.n, 3), np.float32)
    f[-1, 0] = np.nan
    g.apply_forces(f)
    st = g.step(DT, b3g.solver_config(max_pcg_iterations=50, pcg_tolerance=1e-5))
    assert st["solve_status"] == "nonfinite"
    g.close()


def test_invalid_meshes_are_rejected(ctx):
    desc = meshes.tet_grid(3, 3, 3, pin="y0")
    bad = meshes.tet_grid(3, 3, 3, pin="y0")
    bad.tets = bad.tets.copy()
    bad.tets[0, 0] = desc.n + 5
    with pytest.raises(b3g.B3gError, match="references vertex"):
        b3g.Body(ctx, bad)
    deg = meshes.tet_grid(3, 3, 3, pin="y0")
    deg.tets = deg.tets.copy()
    deg.tets[1, 1] = deg.tets[1, 0]
    with pytest.raises(b3g.B3gError, match="repeats vertex"):
        b3g.Body(ctx, deg)


def test_zero_dt_skips_the_solve(ctx):
    desc = meshes.tet_grid(4, 4, 4, pin="y0")
    g = b3g.Body(ctx, desc)
    x0, v0 = g.state()
    g.step(0.0)
    x1, v1 = g.state()
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)
    g.close()


def test_invalid_world_shapes_are_rejected(ctx):
    """b3g_body_create validates world shapes: fixture count, types, mesh indices, SDF grids."""
    base = meshes.shape_scene("capsule", m=4)
    cases = []
    many = meshes.shape_scene("capsule", m=4)
    many.world_shapes = [meshes.WorldShape(meshes.SHAPE_SPHERE, radius=0.1, p=np.zeros(9)) for _ in range(17)]
    cases.append((many, "at most 16 world fixtures"))
    bad_type = meshes.shape_scene("capsule", m=4)
    bad_type.world_shapes = [meshes.WorldShape(9)]
    cases.append((bad_type, "unknown shape type"))
    bad_mesh = meshes.shape_scene("mesh", m=4)
    sh = bad_mesh.world_shapes[0]
    sh.triangles = sh.triangles.copy()
    sh.triangles[0, 0] = 1000
    cases.append((bad_mesh, "vertex out of range"))
    bad_sdf = meshes.shape_scene("sdf", m=4)
    bad_sdf.world_shapes[0].voxels = np.zeros((1, 4, 4))
    cases.append((bad_sdf, "at least 2 voxels"))
    for desc, msg in cases:
        with pytest.raises(b3g.B3gError, match=msg):
            b3g.Body(ctx, desc)
    b3g.Body(ctx, base).close()


def _bw_variant(kind):
    """Baraff-Witkin and mouse-spring scenes beyond the golden fixtures."""
    if kind == "uv_compressed":
        # explicit (u, v) frames: rest lengths 0.9 of the mesh along u and 1.1 along v, and b_u,
        # b_v away from 1, so both branches of the stretch Jacobian (|w| > b or not) are taken
        d = meshes.bw_cloth(8, pinned="row", stretch_ks=2e4, stretch_kd=5.0)
        tri = d.stretch_tris.astype(np.int64)
        ab = d.x[tri[:, 1]] - d.x[tri[:, 0]]
        ac = d.x[tri[:, 2]] - d.x[tri[:, 0]]
        u2 = np.linalg.norm(ab, axis=1)
        uv = np.zeros((tri.shape[0], 6))
        uv[:, 2] = 0.9 * u2
        uv[:, 4] = 0.9 * np.einsum("ij,ij->i", ac, ab) / u2
        uv[:, 5] = 1.1 * np.linalg.norm(np.cross(ab, ac), axis=1) / u2
        d.stretch_uv = uv
        d.stretch_params[:, 2] = 1.05
        d.stretch_params[:, 5] = 0.95
        d.stretch_params[:, 3] = 5e3
        return d, {}
    if kind == "mouse_repeat":
        # a mouse spring whose triangle names one vertex twice, with a rest length
        d = meshes.bw_cloth(8, pinned="edges", stretch_ks=5e4, mouse=True, mouse_offset=(0.1, -0.4, 0.0))
        d.mouse_ids[0, 3] = d.mouse_ids[0, 2]
        d.mouse_params[0, :3] = [0.5, 0.25, 0.25]
        d.mouse_params[0, 5] = 0.1
        return d, {}
    if kind == "shear_newton":
        d = meshes.bw_cloth(8, pinned="row", stretch_ks=1e4, shear_ks=2e3, shear_kd=20.0)
        return d, dict(newton_iters=3, sub_tol=1e-6)
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["uv_compressed", "mouse_repeat", "shear_newton"])
def test_cloth_forces_match_oracle(ctx, kind):
    """Stretch / shear / mouse-spring variants against the FP64 oracle (pinned to the reference by
    the golden fixtures), within 20x the oracle's own FP32-vs-FP64 spread."""
    desc, kw = _bw_variant(kind)
    steps = 12
    cfg = b3g.solver_config(force_iterations=kw.get("newton_iters", 1), max_pcg_iterations=200,
                            pcg_tolerance=kw.get("sub_tol", 1e-5))
    x, v, its, _ = gpu_run(ctx, desc, steps, cfg)
    x64, v64, _, _ = oracle.simulate(desc, steps, kind="port", bits=64, **kw)
    x32, v32, _, _ = oracle.simulate(desc, steps, kind="port", bits=32, **kw)
    assert np.abs(x64 - desc.x).max() > 1e-3  # the cloth moved
    assert rel_disp(x, x64, desc.x) < max(1e-4, 20 * rel_disp(x32, x64, desc.x)), kind
    assert rel(v, v64) < max(1e-3, 20 * rel(v32, v64)), kind


def test_cloth_forces_fp64_precision(ctx):
    """The FP64 solver path with stretch, shear and a mouse spring against the FP64 reference
    golden vectors: far inside the FP32 floor."""
    from conftest import load_golden

    for name in ("bw_shear", "bw_mouse"):
        desc, z, st = load_golden(name)
        cfg = b3g.solver_config(max_pcg_iterations=st["max_sub"], pcg_tolerance=st["sub_tol"],
                                precision=b3g.PRECISION_FP64)
        s = int(z["steps"][0])
        x, v, _, _ = gpu_run(ctx, desc, s, cfg)
        rx = z[f"ref64_x_{s}"]
        floor_x = rel_disp(z[f"ref32_x_{s}"], rx, desc.x)
        ulp_x = rel_disp(z[f"ref64ulp_x_{s}"], rx, desc.x)
        # FP32 input rounding of the positions bounds how close a float-input body can get
        assert rel_disp(x, rx, desc.x) < max(0.2 * floor_x, 10 * ulp_x, 1e-6), name


def test_invalid_cloth_forces_are_rejected(ctx):
    """b3g_body_create validates stretch / shear / mouse inputs and mass-only triangles."""
    cases = []
    d = meshes.bw_cloth(4)
    d.x[int(d.stretch_tris[0, 2])] = d.x[int(d.stretch_tris[0, 0])] + 0.5 * (
        d.x[int(d.stretch_tris[0, 1])] - d.x[int(d.stretch_tris[0, 0])])
    cases.append((d, "degenerate"))
    d = meshes.bw_cloth(4)
    d.stretch_tris = d.stretch_tris.copy()
    d.stretch_tris[1, 1] = 999
    cases.append((d, "stretch force 1 references vertex 999"))
    d = meshes.bw_cloth(4, shear_ks=1.0)
    d.shear_uv = np.zeros((d.shear_tris.shape[0], 6))
    cases.append((d, "det = 0"))
    d = meshes.bw_cloth(4, mouse=True)
    d.mouse_ids = d.mouse_ids.copy()
    d.mouse_ids[0, 0] = d.n
    cases.append((d, "mouse spring 0 references vertex"))
    d = meshes.bw_cloth(4, mouse=True)
    d.mouse_params = d.mouse_params.copy()
    d.mouse_params[0, 3] = np.inf
    cases.append((d, "non-finite"))
    d = meshes.bw_cloth(4)
    d.tri_Ex = np.ones(d.tris.shape[0])
    cases.append((d, "all or none"))
    for desc, msg in cases:
        with pytest.raises(b3g.B3gError, match=msg):
            b3g.Body(ctx, desc)
    b3g.Body(ctx, meshes.bw_cloth(4, mouse=True, shear_ks=1.0)).close()


@pytest.mark.parametrize("case", ["bw_pinned", "cloth12"])
def test_ray_cast_matches_reference_golden(ctx, case):
    """b3g_body_ray_cast after stepping a golden body against b3Body::RayCastSingle of the FP64
    reference on its own trajectory: the same triangles hit; fractions and normals within the
    reference's own FP32-vs-FP64 spread plus float rounding of the segment."""
    import os
    from conftest import GOLDEN, load_golden

    z = np.load(os.path.join(GOLDEN, "ray_casts.npz"))
    desc, _, st = load_golden(case)
    steps = int(z[f"{case}_steps"])
    cfg = b3g.solver_config(max_pcg_iterations=st["max_sub"], pcg_tolerance=st["sub_tol"])
    g = b3g.Body(ctx, desc)
    for _ in range(steps):
        g.step(DT, cfg)
    hit, tri, frac, normal = g.ray_cast(z[f"{case}_seg"])
    g.close()
    rh = z[f"{case}_ref64_hit"]
    assert np.array_equal(hit, rh)
    assert np.array_equal(tri[hit], z[f"{case}_ref64_tri"][hit])
    spread = np.abs(z[f"{case}_ref32_frac"] - z[f"{case}_ref64_frac"]).max()
    assert np.abs(frac[hit] - z[f"{case}_ref64_frac"][hit]).max() < max(20 * spread, 1e-4)
    nspread = np.abs(z[f"{case}_ref32_normal"] - z[f"{case}_ref64_normal"]).max()
    assert np.abs(normal[hit] - z[f"{case}_ref64_normal"][hit]).max() < max(20 * nspread, 1e-3)


def test_ray_cast_edge_cases(ctx):
    """No triangles, zero-length and non-finite segments, nearest of two stacked layers, normal
    facing the segment's start from either side, ties to the lowest triangle index."""
    # two parallel unit triangles at y = 0 and y = 1, and a duplicate of the lower one
    x = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1], [0, 1, 0], [1, 1, 0], [0, 1, 1]], np.float64)
    tris = np.array([[0, 2, 1], [3, 5, 4], [0, 2, 1]], np.uint32)
    desc = meshes.BodyDesc(x=x, v=np.zeros_like(x), type=np.zeros(6, np.int32), damping=np.zeros(6),
                           tets=np.zeros((0, 4), np.uint32), tet_E=np.zeros(0), tet_nu=np.zeros(0),
                           tet_kdamp=np.zeros(0), tet_density=np.zeros(0), tris=tris, tri_Ex=None, tri_Ey=None,
                           tri_Es=None, tri_nuxy=None, tri_nuyx=None, tri_kdamp=None, tri_density=np.ones(3),
                           springs=np.zeros((0, 2), np.uint32), spring_L0=np.zeros(0), spring_ks=np.zeros(0),
                           spring_kd=np.zeros(0))
    g = b3g.Body(ctx, desc)
    seg = np.array([[0.2, 2.0, 0.2, 0.2, -1.0, 0.2],     # from above: the upper layer first
                    [0.2, -1.0, 0.2, 0.2, 2.0, 0.2],     # from below: the lower layers, tie -> index 0
                    [0.2, 0.5, 0.2, 0.2, 0.5, 0.2],      # zero length
                    [0.9, 2.0, 0.9, 0.9, -1.0, 0.9],     # outside both triangles
                    [0.2, 2.0, 0.2, 0.2, 1.5, 0.2]])     # ends before the upper layer
    hit, tri, frac, normal = g.ray_cast(seg)
    assert hit.tolist() == [True, True, False, False, False]
    assert tri[:2].tolist() == [1, 0]
    np.testing.assert_allclose(frac[:2], [1.0 / 3.0, 1.0 / 3.0], rtol=1e-6)
    np.testing.assert_allclose(normal[0], [0, 1, 0], atol=1e-6)   # faces the start above
    np.testing.assert_allclose(normal[1], [0, -1, 0], atol=1e-6)  # faces the start below
    with pytest.raises(b3g.B3gError, match="not finite"):
        g.ray_cast(np.array([[np.nan, 0, 0, 0, 1, 0]]))
    assert g.ray_cast(np.zeros((0, 6)))[0].size == 0
    g.close()
    # a body without triangles never hits
    t = meshes.tet_grid(3, 3, 3)
    g = b3g.Body(ctx, t)
    assert not g.ray_cast(np.array([[0.1, 5, 0.1, 0.1, -5, 0.1]]))[0].any()
    g.close()


def test_body_outliving_its_context_is_detached(ctx):
    """Destroying a context first releases its bodies' device memory and detaches them: a later
    b3g_body_destroy only frees the host object, and other calls report an error."""
    lib = b3g.load_library()
    c2 = b3g.Context(0)
    g = b3g.Body(c2, meshes.tet_grid(3, 3, 3))
    assert lib.b3g_context_destroy(c2.handle) == 0
    c2.handle = None
    with pytest.raises(b3g.B3gError, match="context was destroyed"):
        g.step(DT, b3g.solver_config())
    g.close()


@pytest.mark.parametrize("scene", ["sphere", "capsule"])
def test_contact_checkpoint_resumes_bitwise(ctx, scene):
    """Checkpoint / resume of a cloth in contact through the C ABI: positions, velocities and the
    contact state (b3g_body_get/set_contacts: exists, friction flag, normal force, normal per
    vertex and fixture) restored into a fresh body continue bit for bit; without the contact state
    the continuation differs (contacts created at the end of a step act in the next)."""
    if scene == "sphere":
        desc = meshes.cloth_grid(24, side=1.2, height=0.52, sphere_radius=0.5, contact_radius=0.05)
    else:
        desc = meshes.shape_scene("capsule", m=12, height=0.002)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=1e-5)
    a = b3g.Body(ctx, desc)
    for _ in range(4):
        a.step(DT, cfg)
    x, v = a.state()
    c = a.contacts()
    assert c["fixtures"] >= 1 and c["exists"].sum() > 0 and c["apply_friction"].sum() > 0
    for _ in range(4):
        a.step(DT, cfg)
    xa, va = a.state()
    b = b3g.Body(ctx, desc)
    b.set_state(x, v)
    b.set_contacts(c)
    assert all(np.array_equal(b.contacts()[k], c[k]) for k in ("exists", "apply_friction", "normal_force", "normal"))
    for _ in range(4):
        b.step(DT, cfg)
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    d = b3g.Body(ctx, desc)  # state without the contacts
    d.set_state(x, v)
    for _ in range(4):
        d.step(DT, cfg)
    xd, _ = d.state()
    assert not np.array_equal(xa, xd)
    bad = dict(c, exists=np.full_like(c["exists"], 2))
    with pytest.raises(b3g.B3gError):
        d.set_contacts(bad)
    for g in (a, b, d):
        g.close()
