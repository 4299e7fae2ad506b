"""ctypes front-end of the oracle (test infrastructure only).

Two CPU implementations of the implicit body step sit behind the same call:

* ``port``: the restatement in ``oracle/b3_oracle.c`` (built by ``make -C oracle port``), float
  or double. It exists on every machine, the GPU host included.
* ``ref``: the reference library compiled from its own sources with ``oracle/ref_harness.cpp``
  (``make -C oracle ref``), float or double. It exists only where the reference sources were
  present at build time; it is never shipped.

Only tests, the smoke check and the CPU-baseline leg of bench.py use this module, and only as
the checker; the product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFOUT = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)
_ip = C.POINTER(C.c_int32)


class _Shape(C.Structure):
    """Mirror of RefShape (oracle/ref_harness.cpp) and b3o_shape (oracle/b3_oracle.c)."""
    _fields_ = [
        ("type", C.c_int32), ("radius", C.c_double), ("friction", C.c_double), ("p", C.c_double * 9),
        ("rotation", C.c_double * 4), ("translation", C.c_double * 3), ("scale", C.c_double * 3),
        ("vertex_count", C.c_uint32), ("vertices", _dp), ("triangle_count", C.c_uint32), ("triangles", _up),
        ("wings", _up), ("grid", C.c_uint32 * 3), ("voxels", _dp), ("grid_lower", C.c_double * 3),
        ("grid_upper", C.c_double * 3), ("invert", C.c_int32),
    ]


class _Desc(C.Structure):
    """Mirror of RefDesc (oracle/ref_harness.cpp) and b3o_desc (oracle/b3_oracle.c)."""
    _fields_ = [
        ("n", C.c_uint32), ("x", _dp), ("v", _dp), ("type", _ip), ("damping", _dp),
        ("tet_count", C.c_uint32), ("tets", _up), ("tet_rest", _dp), ("tet_E", _dp), ("tet_nu", _dp),
        ("tet_kdamp", _dp), ("tet_density", _dp),
        ("tri_count", C.c_uint32), ("tris", _up), ("tri_rest", _dp), ("tri_Ex", _dp), ("tri_Ey", _dp),
        ("tri_Es", _dp), ("tri_nuxy", _dp), ("tri_nuyx", _dp), ("tri_kdamp", _dp), ("tri_density", _dp),
        ("spring_count", C.c_uint32), ("springs", _up), ("spring_L0", _dp), ("spring_ks", _dp),
        ("spring_kd", _dp),
        ("sphere_radius", _dp), ("sphere_friction", _dp),
        ("world_sphere_count", C.c_uint32), ("world_spheres", _dp),
        ("gravity", C.c_double * 3),
        ("world_shape_count", C.c_uint32), ("world_shapes", C.POINTER(_Shape)),
        ("stretch_count", C.c_uint32), ("stretch_tris", _up), ("stretch_uv", _dp), ("stretch_params", _dp),
        ("shear_count", C.c_uint32), ("shear_tris", _up), ("shear_uv", _dp), ("shear_params", _dp),
        ("mouse_count", C.c_uint32), ("mouse_ids", _up), ("mouse_params", _dp),
    ]


class _Run(C.Structure):
    _fields_ = [
        ("steps", C.c_uint32), ("dt", C.c_double), ("newton_iters", C.c_uint32), ("max_sub", C.c_uint32),
        ("sub_tol", C.c_double), ("use_body_step", C.c_int32),
        ("x_out", _dp), ("v_out", _dp), ("sub_iters_out", _up), ("seconds_out", _dp),
        ("contact_mode", C.c_int32),
    ]


_libs: dict = {}
_lock = threading.Lock()


def build_port() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def reference_root() -> Optional[str]:
    """The reference project's sources: $B3G_REFERENCE, else the read-only checkout this recipe
    was written against; None where neither exists (the GPU host, for one)."""
    for cand in (os.environ.get("B3G_REFERENCE"), "/root/reference"):
        if cand and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None


def build_ref() -> bool:
    """Build the reference harness if the reference sources are present; return availability."""
    root = reference_root()
    if root is None:
        return ref_available()
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF={root}"], check=True)
    return ref_available()


def ref_available() -> bool:
    return os.path.exists(os.path.join(REFOUT, "libb3ref32.so")) and os.path.exists(
        os.path.join(REFOUT, "libb3ref64.so"))


def _lib(kind: str, bits: int):
    key = (kind, bits)
    with _lock:
        if key in _libs:
            return _libs[key]
        if kind == "port":
            path = os.path.join(BUILD, f"libb3oracle{bits}.so")
            if not os.path.exists(path):
                build_port()
            lib = C.CDLL(path)
            lib.b3o_simulate.argtypes = [C.POINTER(_Desc), C.POINTER(_Run)]
            lib.b3o_simulate.restype = C.c_int
            lib.b3o_simulate_batch.argtypes = [C.POINTER(_Desc), C.POINTER(_Run), C.c_uint32, C.c_uint32,
                                               C.POINTER(C.c_double)]
            lib.b3o_simulate_batch.restype = C.c_int
        elif kind == "ref":
            path = os.path.join(REFOUT, f"libb3ref{bits}.so")
            if not os.path.exists(path):
                raise FileNotFoundError(f"reference harness not built: {path}")
            lib = C.CDLL(path)
            lib.ref_simulate.argtypes = [C.POINTER(_Desc), C.POINTER(_Run)]
            lib.ref_simulate.restype = C.c_int
        else:
            raise ValueError(kind)
        _libs[key] = lib
        return lib


def _arr(a, dtype):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=dtype)


def _ptr(a, ctype):
    if a is None or a.size == 0:
        return C.cast(None, ctype)
    return a.ctypes.data_as(ctype)


def _make_desc(body):
    keep = []

    def d(a):
        a = _arr(a, np.float64)
        keep.append(a)
        return _ptr(a, _dp)

    def u(a):
        a = _arr(a, np.uint32)
        keep.append(a)
        return _ptr(a, _up)

    tt = _arr(body.type, np.int32)
    keep.append(tt)
    desc = _Desc()
    desc.n = body.n
    desc.x = d(body.x)
    desc.v = d(body.v)
    desc.type = tt.ctypes.data_as(_ip)
    desc.damping = d(body.damping)
    desc.tet_count = body.tets.shape[0]
    desc.tets = u(body.tets)
    desc.tet_rest = C.cast(None, _dp)
    desc.tet_E, desc.tet_nu, desc.tet_kdamp, desc.tet_density = (
        d(body.tet_E), d(body.tet_nu), d(body.tet_kdamp), d(body.tet_density))
    desc.tri_count = body.tris.shape[0]
    desc.tris = u(body.tris)
    desc.tri_rest = C.cast(None, _dp)
    desc.tri_Ex, desc.tri_Ey, desc.tri_Es = d(body.tri_Ex), d(body.tri_Ey), d(body.tri_Es)
    desc.tri_nuxy, desc.tri_nuyx = d(body.tri_nuxy), d(body.tri_nuyx)
    desc.tri_kdamp, desc.tri_density = d(body.tri_kdamp), d(body.tri_density)
    desc.spring_count = body.springs.shape[0]
    desc.springs = u(body.springs)
    desc.spring_L0, desc.spring_ks, desc.spring_kd = d(body.spring_L0), d(body.spring_ks), d(body.spring_kd)
    desc.sphere_radius = d(body.sphere_radius) if body.sphere_radius is not None else C.cast(None, _dp)
    desc.sphere_friction = d(body.sphere_friction) if body.sphere_friction is not None else C.cast(None, _dp)
    desc.world_sphere_count = body.world_spheres.shape[0]
    desc.world_spheres = d(body.world_spheres)
    for k in range(3):
        desc.gravity[k] = float(body.gravity[k])
    shapes = list(getattr(body, "world_shapes", []) or [])
    desc.world_shape_count = len(shapes)
    if shapes:
        arr = (_Shape * len(shapes))()
        keep.append(arr)
        for w, sh in zip(arr, shapes):
            w.type = int(sh.type)
            w.radius, w.friction = float(sh.radius), float(sh.friction)
            p = np.zeros(9)
            p[:len(np.ravel(sh.p))] = np.ravel(sh.p)
            for k in range(9):
                w.p[k] = float(p[k])
            for k in range(4):
                w.rotation[k] = float(sh.rotation[k])
            for k in range(3):
                w.translation[k] = float(sh.translation[k])
                w.scale[k] = float(sh.scale[k])
                w.grid_lower[k] = float(sh.grid_lower[k])
                w.grid_upper[k] = float(sh.grid_upper[k])
            if sh.vertices is not None:
                w.vertex_count = int(np.asarray(sh.vertices).shape[0])
                w.vertices = d(np.asarray(sh.vertices))
            if sh.triangles is not None:
                w.triangle_count = int(np.asarray(sh.triangles).shape[0])
                w.triangles = u(np.asarray(sh.triangles))
            if sh.wings is not None:
                w.wings = u(np.asarray(sh.wings))
            if sh.voxels is not None:
                vox = np.asarray(sh.voxels)
                w.grid[0], w.grid[1], w.grid[2] = vox.shape[2], vox.shape[1], vox.shape[0]
                w.voxels = d(vox)
            w.invert = 1 if sh.invert else 0
        desc.world_shapes = C.cast(arr, C.POINTER(_Shape))
    else:
        desc.world_shapes = C.cast(None, C.POINTER(_Shape))
    st = getattr(body, "stretch_tris", None)
    if st is not None and len(st):
        desc.stretch_count = len(st)
        desc.stretch_tris = u(st)
        desc.stretch_uv = d(body.stretch_uv)
        desc.stretch_params = d(body.stretch_params)
    sh = getattr(body, "shear_tris", None)
    if sh is not None and len(sh):
        desc.shear_count = len(sh)
        desc.shear_tris = u(sh)
        desc.shear_uv = d(body.shear_uv)
        desc.shear_params = d(body.shear_params)
    ms = getattr(body, "mouse_ids", None)
    if ms is not None and len(ms):
        desc.mouse_count = len(ms)
        desc.mouse_ids = u(ms)
        desc.mouse_params = d(body.mouse_params)
    return desc, keep


def simulate(body, steps: int, dt: float = 1.0 / 60.0, newton_iters: int = 1, max_sub: int = 200,
             sub_tol: float = 1e-5, kind: str = "port", bits: int = 32, use_body_step: bool = False,
             threads: int = 1, contact_mode: int = 0):
    """Run ``steps`` implicit steps on a CPU implementation. Returns (x, v, iters, seconds).

    contact_mode 1 (filtered contacts) exists in the restatement only: the reference has no such
    mode."""
    if contact_mode and kind != "port":
        raise ValueError("filtered contacts are an extension of the restatement")
    lib = _lib(kind, bits)
    desc, keep = _make_desc(body)
    n = body.n
    x = np.zeros((n, 3))
    v = np.zeros((n, 3))
    it = np.zeros(max(steps, 1), np.uint32)
    sec = np.zeros(1)
    run = _Run()
    run.steps, run.dt, run.newton_iters, run.max_sub = steps, dt, newton_iters, max_sub
    run.sub_tol = sub_tol
    run.use_body_step = 1 if use_body_step else 0
    run.contact_mode = contact_mode
    run.x_out, run.v_out = x.ctypes.data_as(_dp), v.ctypes.data_as(_dp)
    run.sub_iters_out = it.ctypes.data_as(_up)
    run.seconds_out = sec.ctypes.data_as(_dp)
    fn = lib.b3o_simulate if kind == "port" else lib.ref_simulate
    rc = fn(C.byref(desc), C.byref(run))
    if rc != 0:
        raise RuntimeError(f"oracle {kind}{bits} failed with {rc}")
    del keep
    return x, v, it[:steps].copy(), float(sec[0])


class _Hit(C.Structure):
    """Mirror of RefHit (oracle/ref_harness.cpp) and b3o_hit (oracle/b3_oracle.c)."""
    _fields_ = [("hit", C.c_int32), ("triangle", C.c_uint32), ("fraction", C.c_double), ("normal", C.c_double * 3)]


def ray_cast(body, steps: int, segments, dt: float = 1.0 / 60.0, newton_iters: int = 1, max_sub: int = 200,
             sub_tol: float = 1e-5, kind: str = "port", bits: int = 64):
    """b3Body::RayCastSingle for each segment (rows p1, p2) after ``steps`` steps.

    Returns (hit bool array, triangle index array, fraction array, normal array, positions)."""
    lib = _lib(kind, bits)
    fn = lib.b3o_ray_cast if kind == "port" else lib.ref_ray_cast
    fn.argtypes = [C.POINTER(_Desc), C.POINTER(_Run), C.c_uint32, _dp, C.POINTER(_Hit)]
    fn.restype = C.c_int
    desc, keep = _make_desc(body)
    seg = np.ascontiguousarray(np.asarray(segments, np.float64).reshape(-1, 6))
    out = (_Hit * max(len(seg), 1))()
    x = np.zeros((body.n, 3))
    run = _Run()
    run.steps, run.dt, run.newton_iters, run.max_sub, run.sub_tol = steps, dt, newton_iters, max_sub, sub_tol
    run.x_out = x.ctypes.data_as(_dp)
    rc = fn(C.byref(desc), C.byref(run), len(seg), seg.ctypes.data_as(_dp), out)
    if rc != 0:
        raise RuntimeError(f"ray cast {kind}{bits} failed with {rc}")
    del keep
    hits = list(out)[: len(seg)]
    return (np.array([h.hit != 0 for h in hits]), np.array([h.triangle for h in hits], np.int64),
            np.array([h.fraction for h in hits]), np.array([list(h.normal) for h in hits]).reshape(-1, 3), x)


def simulate_batch(bodies, steps: int, dt: float = 1.0 / 60.0, newton_iters: int = 1, max_sub: int = 200,
                   sub_tol: float = 1e-5, bits: int = 32, threads: int = 0):
    """Step independent bodies on `threads` host threads with the restatement.

    Returns (xs, vs, iters, step_seconds); step_seconds covers the stepping phase only (the bodies
    are built before the clock starts)."""
    lib = _lib("port", bits)
    threads = threads or (os.cpu_count() or 1)
    count = len(bodies)
    descs = (_Desc * count)()
    runs = (_Run * count)()
    keep = []
    outs = []
    for k, body in enumerate(bodies):
        d, kk = _make_desc(body)
        keep.append(kk)
        descs[k] = d
        x = np.zeros((body.n, 3))
        v = np.zeros((body.n, 3))
        it = np.zeros(max(steps, 1), np.uint32)
        outs.append((x, v, it))
        r = runs[k]
        r.steps, r.dt, r.newton_iters, r.max_sub, r.sub_tol, r.use_body_step = steps, dt, newton_iters, max_sub, sub_tol, 0
        r.x_out, r.v_out = x.ctypes.data_as(_dp), v.ctypes.data_as(_dp)
        r.sub_iters_out = it.ctypes.data_as(_up)
        r.seconds_out = C.cast(None, _dp)
    sec = C.c_double(0.0)
    rc = lib.b3o_simulate_batch(descs, runs, count, threads, C.byref(sec))
    if rc != 0:
        raise RuntimeError(f"oracle batch failed with {rc}")
    del keep
    return [o[0] for o in outs], [o[1] for o in outs], [o[2][:steps] for o in outs], float(sec.value)


# ---------------------------------------------------------------- sparse containers and solvers
class _Jac(C.Structure):
    """Mirror of RefJacobians (oracle/ref_harness.cpp)."""
    _fields_ = [("capacity", C.c_uint32), ("dfdx_count", C.c_uint32), ("dfdv_count", C.c_uint32),
                ("dfdx_rows", _up), ("dfdx_cols", _up), ("dfdx_vals", _dp),
                ("dfdv_rows", _up), ("dfdv_cols", _up), ("dfdv_vals", _dp),
                ("x", _dp), ("v", _dp), ("f", _dp), ("fe", _dp), ("mass", _dp), ("dynamic", _ip)]


class _SpIn(C.Structure):
    """Mirror of RefSparseIn (oracle/ref_harness.cpp)."""
    _fields_ = [("n", C.c_uint32), ("h", C.c_double),
                ("dfdx_count", C.c_uint32), ("dfdx_rows", _up), ("dfdx_cols", _up), ("dfdx_vals", _dp),
                ("dfdv_count", C.c_uint32), ("dfdv_rows", _up), ("dfdv_cols", _up), ("dfdv_vals", _dp),
                ("f", _dp), ("x0", _dp), ("v0", _dp), ("fe", _dp), ("M", _dp), ("S", _dp), ("y", _dp), ("z", _dp),
                ("u", _dp), ("D", _dp), ("s", C.c_double), ("cg_max_iterations", C.c_uint32),
                ("cg_tolerance", C.c_double), ("capacity", C.c_uint32)]


class _SpOut(C.Structure):
    """Mirror of RefSparseOut (oracle/ref_harness.cpp)."""
    _fields_ = [("spmv", _dp), ("b", _dp), ("pb", _dp), ("diag_u", _dp), ("dot_u_pb", C.c_double),
                ("len2_pb", C.c_double), ("pA_row_ptr", _up), ("pA_cols", _up), ("pA_vals", _dp),
                ("pA_count", C.c_uint32), ("cg_x", _dp), ("cg_iterations", C.c_uint32), ("cg_error", C.c_double),
                ("be_x", _dp), ("be_v", _dp), ("be_iterations", C.c_uint32), ("be_error", C.c_double),
                ("be_min_sub", C.c_uint32), ("be_max_sub", C.c_uint32)]


# names of the SpMV products of RefSparseOut::spmv, in order
SPARSE_PRODUCTS = ["A", "pA", "D_dfdx", "dfdx_D", "s_dfdx", "dfdx_plus_dfdv", "dfdx_minus_dfdv", "dfdx_plus_D",
                   "D_minus_dfdx", "zero_dfdx"]


def ref_jacobians(body, steps: int, dt: float = 1.0 / 60.0, max_sub: int = 200, sub_tol: float = 1e-5,
                  bits: int = 32, capacity: Optional[int] = None) -> dict:
    """The reference's force model evaluated once at the state after `steps` steps: f, dfdx and
    dfdv (COO in the reference's row-list order, 9 values per block in b3Mat33 column order), the
    state, external forces, masses and the dynamic flags, by input vertex index."""
    lib = _lib("ref", bits)
    fn = lib.ref_jacobians
    fn.argtypes = [C.POINTER(_Desc), C.POINTER(_Run), C.POINTER(_Jac)]
    fn.restype = C.c_int
    desc, keep = _make_desc(body)
    n = body.n
    cap = capacity or 64 * n
    arrs = {k: np.zeros(cap, np.uint32) for k in ("dfdx_rows", "dfdx_cols", "dfdv_rows", "dfdv_cols")}
    arrs.update({k: np.zeros(9 * cap) for k in ("dfdx_vals", "dfdv_vals")})
    arrs.update({k: np.zeros(3 * n) for k in ("x", "v", "f", "fe")})
    arrs["mass"] = np.zeros(n)
    arrs["dynamic"] = np.zeros(n, np.int32)
    jac = _Jac()
    jac.capacity = cap
    for k, a in arrs.items():
        setattr(jac, k, a.ctypes.data_as(_up if a.dtype == np.uint32 else (_ip if a.dtype == np.int32 else _dp)))
    run = _Run()
    run.steps, run.dt, run.newton_iters, run.max_sub, run.sub_tol = steps, dt, 1, max_sub, sub_tol
    if fn(C.byref(desc), C.byref(run), C.byref(jac)) != 0:
        raise RuntimeError("ref_jacobians: COO capacity too small")
    del keep
    out = {}
    for m in ("dfdx", "dfdv"):
        c = getattr(jac, f"{m}_count")
        out[f"{m}_rows"] = arrs[f"{m}_rows"][:c].copy()
        out[f"{m}_cols"] = arrs[f"{m}_cols"][:c].copy()
        out[f"{m}_vals"] = arrs[f"{m}_vals"][:9 * c].reshape(c, 9).copy()
    for k in ("x", "v", "f", "fe"):
        out[k] = arrs[k].reshape(n, 3).copy()
    out["mass"], out["dynamic"] = arrs["mass"], arrs["dynamic"]
    return out


def ref_sparse_ops(n: int, h: float, jac: dict, M, S, y, z, u, D, s: float, cg_max: int, cg_tol: float,
                   bits: int = 32) -> dict:
    """The reference's container operators, b3SparseSolveCG and a one-iteration b3SparseSolveBE on
    the given matrices (see RefSparseIn / RefSparseOut in oracle/ref_harness.cpp)."""
    lib = _lib("ref", bits)
    fn = lib.ref_sparse_ops
    fn.argtypes = [C.POINTER(_SpIn), C.POINTER(_SpOut)]
    fn.restype = C.c_int
    keep = []

    def d(a):
        a = np.ascontiguousarray(a, np.float64).ravel()
        keep.append(a)
        return a.ctypes.data_as(_dp)

    def u32(a):
        a = np.ascontiguousarray(a, np.uint32).ravel()
        keep.append(a)
        return a.ctypes.data_as(_up)

    si = _SpIn()
    si.n, si.h = n, h
    for m in ("dfdx", "dfdv"):
        setattr(si, f"{m}_count", len(jac[f"{m}_rows"]))
        setattr(si, f"{m}_rows", u32(jac[f"{m}_rows"]))
        setattr(si, f"{m}_cols", u32(jac[f"{m}_cols"]))
        setattr(si, f"{m}_vals", d(jac[f"{m}_vals"]))
    si.f, si.x0, si.v0, si.fe = d(jac["f"]), d(jac["x"]), d(jac["v"]), d(jac["fe"])
    si.M, si.S, si.y, si.z, si.u, si.D = d(M), d(S), d(y), d(z), d(u), d(D)
    si.s, si.cg_max_iterations, si.cg_tolerance = s, cg_max, cg_tol
    cap = len(jac["dfdx_rows"]) + len(jac["dfdv_rows"]) + n
    si.capacity = cap
    o = {"spmv": np.zeros(10 * 3 * n), "b": np.zeros(3 * n), "pb": np.zeros(3 * n), "diag_u": np.zeros(3 * n),
         "pA_row_ptr": np.zeros(n + 1, np.uint32), "pA_cols": np.zeros(cap, np.uint32), "pA_vals": np.zeros(9 * cap),
         "cg_x": np.zeros(3 * n), "be_x": np.zeros(3 * n), "be_v": np.zeros(3 * n)}
    so = _SpOut()
    for k, a in o.items():
        setattr(so, k, a.ctypes.data_as(_up if a.dtype == np.uint32 else _dp))
    if fn(C.byref(si), C.byref(so)) != 0:
        raise RuntimeError("ref_sparse_ops: CSR capacity too small")
    del keep
    c = so.pA_count
    res = {"spmv": o["spmv"].reshape(10, n, 3), "b": o["b"].reshape(n, 3), "pb": o["pb"].reshape(n, 3),
           "diag_u": o["diag_u"].reshape(n, 3), "dot_u_pb": so.dot_u_pb, "len2_pb": so.len2_pb,
           "pA_row_ptr": o["pA_row_ptr"], "pA_cols": o["pA_cols"][:c].copy(),
           "pA_vals": o["pA_vals"][:9 * c].reshape(c, 9).copy(),
           "cg_x": o["cg_x"].reshape(n, 3), "cg_iterations": so.cg_iterations, "cg_error": so.cg_error,
           "be_x": o["be_x"].reshape(n, 3), "be_v": o["be_v"].reshape(n, 3), "be_iterations": so.be_iterations,
           "be_error": so.be_error, "be_min_sub": so.be_min_sub, "be_max_sub": so.be_max_sub}
    return res
