"""Generates the golden fixtures of tests/golden/ by running the reference library itself.

The reference is compiled from its own sources by oracle/Makefile (target `ref`, float and
double builds) and driven through oracle/ref_harness.cpp. Each fixture stores the inputs (so the
tests need neither the reference nor the mesh generators to reproduce them) and the reference's
positions, velocities and PCG iteration counts after a number of steps.

Run here, where the reference sources exist:  python tests/golden/make_golden.py [case ...]
(cases: the names in CASES, "ray_casts", "sparse_tet10")
"""
import copy
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402
from bounce_softbody_gb300 import meshes  # noqa: E402


def single_tet():
    d = meshes.tet_grid(2, 2, 2, pin="none", E=2e4, nu=0.3, damping=0.0, name="single_tet")
    keep = d.tets[:1]
    used = np.unique(keep)
    remap = {int(v): k for k, v in enumerate(used)}
    d.x = d.x[used]
    d.v = np.zeros_like(d.x)
    d.type = np.array([0, 0, 0, 2], np.int32)[: len(used)]
    d.damping = np.zeros(len(used))
    d.tets = np.array([[remap[int(v)] for v in keep[0]]], np.uint32)
    for f in ("tet_E", "tet_nu", "tet_kdamp", "tet_density"):
        setattr(d, f, getattr(d, f)[:1])
    return d


CASES = [
    # name, body factory, steps snapshots, run settings
    ("tet10", meshes.config_tet10, [1, 10, 120], dict(max_sub=200, sub_tol=1e-5)),
    ("tet10_bodystep", meshes.config_tet10, [10], dict(max_sub=40, use_body_step=True)),
    ("tet4", lambda: meshes.tet_grid(4, 4, 4, seed=2, E=1e5, nu=0.3, pin="y0"), [20], dict(max_sub=200, sub_tol=1e-5)),
    ("tet6_newton", lambda: meshes.tet_grid(6, 6, 6, seed=9, E=5e4, nu=0.3, pin="y0", kdamp=0.01), [8],
     dict(max_sub=200, sub_tol=1e-6, newton_iters=3)),
    ("single_tet", single_tet, [10], dict(max_sub=50, sub_tol=1e-6)),
    # cloth over a sphere is chaotic (tension-only springs start exactly at rest length, so float
    # rounding decides which engage): the reference's own FP32 and FP64 builds separate within
    # tens of steps, so the fixture keeps a short horizon
    ("cloth12", lambda: meshes.cloth_grid(12, side=1.2, height=0.56, sphere_radius=0.5, contact_radius=0.05), [5, 10],
     dict(max_sub=200, sub_tol=1e-5)),
    ("cloth12_contact", lambda: meshes.cloth_grid(12, side=1.2, height=0.52, sphere_radius=0.5, contact_radius=0.05),
     [3, 6], dict(max_sub=200, sub_tol=1e-5)),
    # a 10 x 10 cloth falling onto each kind of static world shape (the reference's own
    # b3CapsuleShape, b3BoxShape, b3TriangleShape, b3MeshShape with wing vertices and b3SDFShape),
    # in contact from step 2; short horizon for the same reason as the sphere cloth
] + [(f"shape_{k}", (lambda k=k: meshes.shape_scene(k, m=10, height=0.002)), [2, 4], dict(max_sub=200, sub_tol=1e-5))
     for k in ("capsule", "box", "triangle", "mesh", "sdf")] + [
    # Baraff-Witkin cloth of the reference testbed (triangle mass fixtures + b3StretchForce per
    # triangle): pinned border (PinnedCloth), pinned row with stretch damping (StretchMapping),
    # stretch + b3ShearForce, and a BodyDragger mouse spring pulling the pinned cloth's centre
    ("bw_pinned", lambda: meshes.bw_cloth(10, pinned="edges", stretch_ks=1e5), [10, 40],
     dict(max_sub=200, sub_tol=1e-5)),
    ("bw_stretch_map", lambda: meshes.bw_cloth(10, pinned="row", stretch_ks=1e4, stretch_kd=10.0), [10, 40],
     dict(max_sub=200, sub_tol=1e-5)),
    ("bw_shear", lambda: meshes.bw_cloth(10, pinned="row", stretch_ks=1e4, shear_ks=1e3, shear_kd=10.0), [10, 40],
     dict(max_sub=200, sub_tol=1e-5)),
    ("bw_mouse", lambda: meshes.bw_cloth(10, pinned="edges", stretch_ks=1e5, mouse=True), [5, 20],
     dict(max_sub=200, sub_tol=1e-5)),
]

SHAPE_FIELDS = ["type", "radius", "friction", "p", "rotation", "translation", "scale", "vertices", "triangles",
                "wings", "voxels", "grid_lower", "grid_upper", "invert"]

FIELDS = ["x", "v", "type", "damping", "tets", "tet_E", "tet_nu", "tet_kdamp", "tet_density", "tris", "tri_Ex",
          "tri_Ey", "tri_Es", "tri_nuxy", "tri_nuyx", "tri_kdamp", "tri_density", "springs", "spring_L0",
          "spring_ks", "spring_kd", "world_spheres", "gravity", "stretch_tris", "stretch_params", "shear_tris",
          "shear_params", "mouse_ids", "mouse_params"]


# b3Body::RayCastSingle on golden bodies after some steps: (golden case, steps). Segments pass
# through interior points of random triangles (barycentric weights >= 0.15, away from edges) from
# random directions (a few stop short of far layers); 8 segments far above the cloth and 8 that
# end before reaching it miss.
RAY_CASES = [("bw_pinned", 10), ("cloth12", 5)]


def ray_segments(x, tris, rng, count=64):
    t = rng.choice(len(tris), count, replace=False)
    b = rng.uniform(0.15, 0.7, (count, 2))
    b = np.where(b.sum(1, keepdims=True) > 0.85, b * 0.85 / b.sum(1, keepdims=True), b)
    w = np.stack([1 - b[:, 0] - b[:, 1], b[:, 0], b[:, 1]], 1)
    q = (w[:, :, None] * x[tris[t].astype(np.int64)]).sum(1)
    dirn = rng.normal(size=(count, 3))
    dirn /= np.linalg.norm(dirn, axis=1, keepdims=True)
    length = rng.uniform(0.2, 1.0, (count, 1))
    p1 = q + length * dirn
    p2 = q - rng.uniform(0.3, 1.5, (count, 1)) * length * dirn
    miss = np.concatenate([q[:8] + [0, 5, 0], q[:8] + [1, 6, 0]], 1)
    short = np.concatenate([p1[8:16], p1[8:16] + 0.2 * (q[8:16] - p1[8:16])], 1)
    return np.concatenate([np.concatenate([p1, p2], 1), miss, short])


def make_rays():
    out = {}
    for case, steps in RAY_CASES:
        z = np.load(os.path.join(HERE, f"{case}.npz"))
        desc = next(make for name, make, _, _ in CASES if name == case)()
        kw = next(k for name, _, _, k in CASES if name == case)
        seg = ray_segments(z[f"ref64_x_{steps}"], desc.tris, np.random.default_rng(1))
        out[f"{case}_steps"] = np.array(steps)
        out[f"{case}_seg"] = seg
        for bits in (32, 64):
            hit, tri, frac, normal, _ = oracle.ray_cast(desc, steps, seg, kind="ref", bits=bits, **kw)
            out[f"{case}_ref{bits}_hit"] = hit
            out[f"{case}_ref{bits}_tri"] = tri
            out[f"{case}_ref{bits}_frac"] = frac
            out[f"{case}_ref{bits}_normal"] = normal
    np.savez_compressed(os.path.join(HERE, "ray_casts.npz"), **out)
    print("wrote ray_casts", {k: v.shape for k, v in out.items() if k.endswith("_seg")})


def sparse_body():
    """The 10^3 block of the single-body workload with stiffness damping 0.01 (so that dfdv carries
    the full pattern, not only mass damping)."""
    return meshes.tet_grid(10, 10, 10, spacing=0.1, jitter=0.01, seed=0, E=1e5, nu=0.3, density=1000.0,
                           damping=0.01, pin="y0", kdamp=0.01, name="sparse_tet10")


def make_sparse():
    """sparse_tet10.npz: the reference's force model evaluated at the 10^3 block's state after 10
    steps (f, dfdx, dfdv from its FP32 build), then the reference's own container operators
    (b3Mul SpMV of ten matrix expressions, diag x dense, b3Dot, b3LengthSquared), the
    backward-Euler system and its pre-filter (sparse_force_solver.cpp:165-174),
    b3SparseSolveCG from x = 0 and one b3SparseSolveBE iteration driven by a force model that
    replays f, dfdx and dfdv; by its FP32 build and by its FP64 build on the same (float-valued)
    inputs."""
    body = sparse_body()
    steps, h = 10, 1.0 / 60.0
    jac = oracle.ref_jacobians(body, steps, dt=h, bits=32)
    n = body.n
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)  # noqa: E731
    rng = np.random.default_rng(11)
    eye = np.eye(3)
    M = np.stack([m * eye for m in jac["mass"]]).transpose(0, 2, 1).reshape(n, 9)
    S = np.stack([eye * dyn for dyn in jac["dynamic"]]).reshape(n, 9)
    y = f32(rng.normal(scale=1e-4, size=(n, 3)))
    z = f32(rng.normal(scale=1e-3, size=(n, 3)) * jac["dynamic"][:, None])
    u = f32(rng.normal(size=(n, 3)))
    D = f32(rng.normal(size=(n, 9)))
    s = 0.75
    out = {"n": np.array(n), "h": np.array(h), "steps": np.array(steps), "s": np.array(s),
           "cg_max": np.array(200), "cg_tol": np.array(1e-5)}
    for m in ("dfdx", "dfdv"):
        out[f"{m}_rows"] = jac[f"{m}_rows"].astype(np.uint16)
        out[f"{m}_cols"] = jac[f"{m}_cols"].astype(np.uint16)
        out[f"{m}_vals"] = jac[f"{m}_vals"].astype(np.float32)
    for k in ("x", "v", "f", "fe"):
        out[k] = jac[k].astype(np.float32)
    out["mass"] = jac["mass"].astype(np.float32)
    out["dynamic"] = jac["dynamic"].astype(np.int8)
    out.update(y=y.astype(np.float32), z=z.astype(np.float32), u=u.astype(np.float32), D=D.astype(np.float32))
    for bits in (32, 64):
        r = oracle.ref_sparse_ops(n, h, jac, M, S, y, z, u, D, s, 200, 1e-5, bits=bits)
        t = np.float32 if bits == 32 else np.float64
        out[f"ref{bits}_spmv"] = r["spmv"].astype(t)
        for k in ("b", "pb", "diag_u", "cg_x", "be_x", "be_v"):
            out[f"ref{bits}_{k}"] = r[k].astype(t)
        for k in ("dot_u_pb", "len2_pb", "cg_iterations", "cg_error", "be_iterations", "be_error", "be_min_sub",
                  "be_max_sub"):
            out[f"ref{bits}_{k}"] = np.array(r[k])
        if bits == 32:
            # pA's pattern and its diagonal blocks (the full matrix is checked through its products)
            rp, cols = r["pA_row_ptr"], r["pA_cols"]
            out["ref32_pA_row_ptr"] = rp.astype(np.uint32)
            out["ref32_pA_cols"] = cols.astype(np.uint16)
            diag = np.zeros((n, 9))
            for i in range(n):
                k = rp[i] + int(np.nonzero(cols[rp[i]:rp[i + 1]] == i)[0][0])
                diag[i] = r["pA_vals"][k]
            out["ref32_pA_diag"] = diag.astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "sparse_tet10.npz"), **out)
    print("wrote sparse_tet10", {k: v.shape for k, v in out.items() if k.endswith("_vals")},
          "cg iterations", int(out["ref32_cg_iterations"]), int(out["ref64_cg_iterations"]))


def main():
    if not oracle.build_ref():
        raise SystemExit("the reference harness could not be built (reference sources absent)")
    only = set(sys.argv[1:])  # case names to regenerate (default: all)
    for name, make, snaps, kw in CASES:
        if only and name not in only:
            continue
        body = make()
        # absent fields (None: mass-only triangles) stay out of the file
        out = {f"in_{f}": np.asarray(getattr(body, f)) for f in FIELDS if getattr(body, f) is not None}
        if body.sphere_radius is not None:
            out["in_sphere_radius"] = body.sphere_radius
            out["in_sphere_friction"] = body.sphere_friction
        for k, sh in enumerate(body.world_shapes):
            for f in SHAPE_FIELDS:
                val = getattr(sh, f)
                if val is not None:
                    out[f"shape{k}_{f}"] = np.asarray(val)
        out["steps"] = np.array(snaps)
        out["settings"] = np.array([kw.get("max_sub", 200), kw.get("sub_tol", 1.1920928955078125e-07),
                                    kw.get("newton_iters", 1), 1 if kw.get("use_body_step") else 0], np.float64)
        for bits in (32, 64):
            for s in snaps:
                x, v, it, _ = oracle.simulate(body, s, kind="ref", bits=bits, **kw)
                out[f"ref{bits}_x_{s}"] = x
                out[f"ref{bits}_v_{s}"] = v
                out[f"ref{bits}_it_{s}"] = it
        # the FP64 reference's own sensitivity to rounding: the same run from positions moved by
        # one unit in the last place (a PCG stopped at a loose tolerance amplifies such changes)
        rng = np.random.default_rng(7)
        moved = copy.deepcopy(body)
        moved.x = body.x * (1.0 + np.ldexp(1.0, -52) * rng.choice([-1.0, 1.0], size=body.x.shape))
        for s in snaps:
            x, v, _, _ = oracle.simulate(moved, s, kind="ref", bits=64, **kw)
            out[f"ref64ulp_x_{s}"] = x
            out[f"ref64ulp_v_{s}"] = v
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print("wrote", name, {k: v.shape for k, v in out.items() if k.startswith("ref64_x")})
    if not only or "ray_casts" in only:
        make_rays()
    if not only or "sparse_tet10" in only:
        make_sparse()


if __name__ == "__main__":
    main()
