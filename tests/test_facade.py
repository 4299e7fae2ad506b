"""The C++ façade (include/b3g_body.hpp): a Bounce Softbody-style program built against it and
linked with libb3g.so gives the same state as the C ABI used directly."""
import os
import subprocess

import numpy as np
import pytest
from conftest import ROOT

from bounce_softbody_gb300 import b3g, meshes

LIBDIR = os.path.join(ROOT, "bounce_softbody_gb300", "_lib")


def build_demo(tmp_path):
    exe = str(tmp_path / "facade_demo")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "facade_demo.cpp"), "-L", LIBDIR, "-lb3g",
                        f"-Wl,-rpath,{LIBDIR}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles_and_links(tmp_path):
    build_demo(tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("shapes,mode", [(False, 0), (True, 0), (True, 1)], ids=["tets", "shapes", "shapes_filter"])
def test_facade_matches_c_abi(tmp_path, ctx, shapes, mode):
    exe = build_demo(tmp_path)
    desc = meshes.tet_grid(6, 5, 7, seed=4, E=2e5, nu=0.33, pin="none" if shapes else "y0")
    if shapes:
        # what facade_demo.cpp builds with "shapes": contact spheres, a box floor, a capsule
        desc.sphere_radius = np.full(desc.n, 0.03)
        desc.sphere_friction = np.full(desc.n, 0.3)
        desc.world_shapes = [
            meshes.WorldShape(meshes.SHAPE_BOX, radius=0.0, friction=0.5, p=np.array([1.0, 0.05, 1.0, 0, 0, 0, 0, 0, 0]),
                              rotation=np.array([0.0, 0.0, 0.0499792, 0.9987503]), translation=np.array([0.2, -0.07, 0.2])),
            meshes.WorldShape(meshes.SHAPE_CAPSULE, radius=0.12, friction=0.2,
                              p=np.array([0.6, 0.0, -0.1, 0.6, 0.0, 0.8, 0, 0, 0])),
        ]
    steps, dt, tol = 8, 1.0 / 60.0, 1e-5
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([desc.n, desc.tets.shape[0]], np.uint32).tofile(f)
        desc.x.astype(np.float32).tofile(f)
        desc.type.astype(np.int32).tofile(f)
        desc.tets.astype(np.uint32).tofile(f)
        np.array([desc.tet_E[0], desc.tet_nu[0], desc.tet_density[0], desc.damping[0]], np.float32).tofile(f)
        np.array([steps], np.uint32).tofile(f)
        np.array([dt, tol], np.float32).tofile(f)
    out = tmp_path / "out.bin"
    extra = (["shapes"] if shapes else []) + (["filter"] if mode == 1 else [])
    r = subprocess.run([exe, str(inp), str(out)] + extra, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    res = np.fromfile(out, np.float32).reshape(2, desc.n, 3)
    g = b3g.Body(ctx, desc)
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=tol, contact_mode=mode)
    for _ in range(steps):
        g.step(dt, cfg)
    x, v = g.state()
    g.close()
    # same library, same inputs: identical results
    assert np.array_equal(res[0], x) and np.array_equal(res[1], v)


@pytest.mark.gpu
def test_facade_cloth_forces_match_c_abi(tmp_path, ctx):
    """facade_demo.cpp "cloth": triangle mass fixtures + stretch + shear forces, a mouse spring
    for 6 steps (then DestroyForce), 6 steps more and a RayCastSingle pick, against the same
    scene through the C ABI
    (meshes.bw_cloth; the mouse spring dropped by rebuilding the body from the state reached,
    with the initial rest frames and masses). The facade computes the (u, v) frames in float
    (b3StretchForceDef::Initialize), the C ABI in double, so the two agree to float rounding
    rather than bitwise."""
    exe = build_demo(tmp_path)
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, "-", str(out), "cloth"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    desc = meshes.bw_cloth(10, pinned="edges", stretch_ks=1e5, shear_ks=1e3, shear_kd=10.0, mouse=True)
    x_init = desc.x.copy()
    raw = np.fromfile(out, np.float32)
    res, pick = raw[: 6 * desc.n].reshape(2, desc.n, 3), raw[6 * desc.n:]
    dt, tol = 1.0 / 60.0, 1e-5
    cfg = b3g.solver_config(max_pcg_iterations=200, pcg_tolerance=tol)
    g = b3g.Body(ctx, desc)
    masses = g.masses()
    for _ in range(6):
        g.step(dt, cfg)
    x, v = g.state()
    g.close()
    # the rest frames of the initial cloth (what Initialize gave), then the state reached
    tri = desc.stretch_tris.astype(np.int64)
    ab = x_init[tri[:, 1]] - x_init[tri[:, 0]]
    ac = x_init[tri[:, 2]] - x_init[tri[:, 0]]
    uv = np.zeros((tri.shape[0], 6))
    uv[:, 2] = np.linalg.norm(ab, axis=1)
    uv[:, 4] = np.einsum("ij,ij->i", ac, ab / uv[:, 2:3])
    uv[:, 5] = np.linalg.norm(np.cross(ab, ac), axis=1) / uv[:, 2]
    desc.stretch_uv, desc.shear_uv = uv, uv.copy()
    desc.x, desc.v = x.astype(np.float64), v.astype(np.float64)
    desc.mouse_ids, desc.mouse_params = desc.mouse_ids[:0], desc.mouse_params[:0]
    g = b3g.Body(ctx, desc, masses=masses)
    for _ in range(6):
        g.step(dt, cfg)
    x, v = g.state()
    hit, tri, frac, normal = g.ray_cast(np.array([[0.05, 3.0, 0.03, 0.05, -3.0, 0.03]]))
    g.close()
    assert np.linalg.norm(res[0] - x) <= 1e-4 * np.linalg.norm(x - x_init) + 1e-6
    assert np.linalg.norm(res[1] - v) <= 1e-3 * np.linalg.norm(v) + 1e-5
    # RayCastSingle through the facade: the same triangle as the C ABI's ray cast
    assert pick[0] == 1.0 and hit[0]
    assert int(pick[1]) == tri[0]
    assert abs(pick[2] - frac[0]) < 1e-5
    np.testing.assert_allclose(pick[3:], normal[0], atol=1e-4)


# ---------------------------------------------------------------- the sparse layer (b3g_sparse.hpp)
def build_sparse_demo(tmp_path):
    exe = str(tmp_path / "sparse_demo")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "sparse_demo.cpp"), "-L", LIBDIR, "-lb3g",
                        f"-Wl,-rpath,{LIBDIR}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_sparse_facade_compiles_and_links(tmp_path):
    build_sparse_demo(tmp_path)


@pytest.mark.gpu
def test_sparse_facade_matches_reference(tmp_path):
    """The reference's own expressions (A = M - h dfdv - h^2 dfdx, pA = S A S^T + I - S, ...),
    b3SparseSolveCG and b3SparseSolveBE with a C++ b3SparseForceModel, written against the façade,
    against the reference's outputs in tests/golden/sparse_tet10.npz (tolerances of
    tests/test_gpu_sparse.py)."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "sparse_tet10.npz"))
    n = int(z["n"])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n], np.uint32).tofile(f)
        np.array([float(z["h"])], np.float32).tofile(f)
        for m in ("dfdx", "dfdv"):
            np.array([len(z[f"{m}_rows"])], np.uint32).tofile(f)
            z[f"{m}_rows"].astype(np.uint32).tofile(f)
            z[f"{m}_cols"].astype(np.uint32).tofile(f)
            z[f"{m}_vals"].astype(np.float32).tofile(f)
        for k in ("f", "x", "v", "fe", "y", "z", "u"):
            z[k].astype(np.float32).tofile(f)
        z["mass"].astype(np.float32).tofile(f)
        z["dynamic"].astype(np.int32).tofile(f)
        np.array([int(z["cg_max"])], np.uint32).tofile(f)
        np.array([float(z["cg_tol"])], np.float32).tofile(f)
    out = tmp_path / "out.bin"
    exe = build_sparse_demo(tmp_path)
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    res = np.fromfile(out, np.float32)
    vecs = res[:6 * 3 * n].reshape(6, n, 3)
    its = res[6 * 3 * n:]

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(np.asarray(b, np.float64)))

    assert rel(vecs[0], z["ref32_spmv"][0]) < 2e-5  # A u
    assert rel(vecs[1], z["ref32_spmv"][1]) < 2e-5  # pA u
    assert rel(vecs[2], z["ref32_pb"]) < 2e-5
    floor = rel(z["ref32_cg_x"], z["ref64_cg_x"])
    assert rel(vecs[3], z["ref64_cg_x"]) < max(1e-4, 20 * floor)
    assert abs(its[0] - int(z["ref32_cg_iterations"])) <= 3
    x64 = z["ref64_be_x"]
    fx = np.linalg.norm(z["ref32_be_x"].astype(np.float64) - x64) / np.linalg.norm(x64 - z["x"])
    assert np.linalg.norm(vecs[4] - x64) / np.linalg.norm(x64 - z["x"]) < max(1e-4, 20 * fx)
    assert rel(vecs[5], z["ref64_be_v"]) < max(1e-3, 20 * rel(z["ref32_be_v"], z["ref64_be_v"]))
    assert its[1] == 1 and abs(its[2] - int(z["ref32_be_max_sub"])) <= 3
