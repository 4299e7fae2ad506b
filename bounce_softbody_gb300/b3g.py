"""ctypes binding of the C ABI in include/b3g.h (libb3g.so, built in-tree by build.py).

This is the Python face of the drop-in boundary: the same calls a C/C++ host makes. There is no
CPU fallback: if libb3g.so is missing, or no GPU is usable, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libb3g.so")

STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
PRECISION_FP32, PRECISION_FP64, PRECISION_BF16 = 0, 1, 2
PRECOND_JACOBI, PRECOND_BLOCK_JACOBI = 0, 1
CONTACT_PENALTY, CONTACT_FILTER = 0, 1
SOLVE_STATUS = {0: "converged", 1: "max_iterations", 2: "nonfinite", 3: "breakdown", 4: "device_timeout"}

_fp = C.POINTER(C.c_float)
_up = C.POINTER(C.c_uint32)
_ip = C.POINTER(C.c_int32)


class WorldShapeC(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("radius", C.c_float), ("friction", C.c_float), ("p", C.c_float * 9),
        ("rotation", C.c_float * 4), ("translation", C.c_float * 3), ("scale", C.c_float * 3),
        ("vertex_count", C.c_uint32), ("vertices", _fp), ("triangle_count", C.c_uint32), ("triangles", _up),
        ("wings", _up), ("grid", C.c_uint32 * 3), ("voxels", _fp), ("grid_lower", C.c_float * 3),
        ("grid_upper", C.c_float * 3), ("invert", C.c_int32),
    ]


class RayHit(C.Structure):
    """b3g_ray_hit (include/b3g.h)."""
    _fields_ = [("hit", C.c_int32), ("triangle", C.c_uint32), ("fraction", C.c_float), ("normal", C.c_float * 3)]


class BodyDescC(C.Structure):
    _fields_ = [
        ("vertex_count", C.c_uint32), ("positions", _fp), ("velocities", _fp), ("types", _ip),
        ("damping", _fp), ("masses", _fp),
        ("tet_count", C.c_uint32), ("tets", _up), ("tet_rest", _fp), ("tet_young", _fp),
        ("tet_poisson", _fp), ("tet_stiffness_damping", _fp), ("tet_density", _fp),
        ("tri_count", C.c_uint32), ("tris", _up), ("tri_rest", _fp), ("tri_young_x", _fp),
        ("tri_young_y", _fp), ("tri_shear", _fp), ("tri_poisson_xy", _fp), ("tri_poisson_yx", _fp),
        ("tri_stiffness_damping", _fp), ("tri_density", _fp),
        ("spring_count", C.c_uint32), ("springs", _up), ("spring_rest_length", _fp),
        ("spring_stiffness", _fp), ("spring_damping", _fp),
        ("sphere_radius", _fp), ("sphere_friction", _fp),
        ("world_sphere_count", C.c_uint32), ("world_spheres", _fp),
        ("gravity", C.c_float * 3),
        ("world_shape_count", C.c_uint32), ("world_shapes", C.POINTER(WorldShapeC)),
        ("stretch_count", C.c_uint32), ("stretch_tris", _up), ("stretch_uv", _fp), ("stretch_params", _fp),
        ("shear_count", C.c_uint32), ("shear_tris", _up), ("shear_uv", _fp), ("shear_params", _fp),
        ("mouse_count", C.c_uint32), ("mouse_ids", _up), ("mouse_params", _fp),
    ]


class SolverConfig(C.Structure):
    _fields_ = [
        ("force_iterations", C.c_uint32), ("max_pcg_iterations", C.c_uint32),
        ("pcg_tolerance", C.c_double), ("newton_tolerance", C.c_double),
        ("refresh_period", C.c_uint32), ("precision", C.c_int32), ("preconditioner", C.c_int32),
        ("contact_mode", C.c_int32),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("newton_iterations", C.c_uint32), ("pcg_iterations", C.c_uint32),
        ("min_pcg_iterations", C.c_uint32), ("solve_status", C.c_int32),
        ("residual_ratio", C.c_double), ("newton_error", C.c_double),
        ("total_pcg_iterations", C.c_uint64), ("total_steps", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {"newton_iterations": self.newton_iterations, "pcg_iterations": self.pcg_iterations,
                "min_pcg_iterations": self.min_pcg_iterations,
                "solve_status": SOLVE_STATUS.get(self.solve_status, str(self.solve_status)),
                "residual_ratio": self.residual_ratio, "newton_error": self.newton_error,
                "total_pcg_iterations": int(self.total_pcg_iterations), "total_steps": int(self.total_steps)}


class RequestResult(C.Structure):
    _fields_ = [
        ("request_id", C.c_uint64), ("body_id", C.c_uint32), ("steps", C.c_uint32),
        ("status", C.c_int32), ("reserved", C.c_int32), ("pcg_iterations", C.c_uint64),
        ("queue_seconds", C.c_double), ("latency_seconds", C.c_double),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_uint64), ("vertex_steps", C.c_uint64), ("admitted", C.c_uint64),
        ("completed", C.c_uint64), ("rejected", C.c_uint64), ("evictions", C.c_uint64),
        ("resident_bytes", C.c_uint64), ("waiting", C.c_uint64), ("gpu_seconds", C.c_double),
        ("wall_seconds", C.c_double), ("step_ms_p50", C.c_double), ("step_ms_p99", C.c_double),
        ("cluster_ctas", C.c_uint32), ("cluster_threshold", C.c_uint32),
    ]


REQUEST_STATUS = {0: "done", 1: "rejected", 2: "device_timeout"}

# every entry point of include/b3g.h with its ctypes signature
SIGNATURES = {
    "b3g_solver_config_default": (None, [C.POINTER(SolverConfig)]),
    "b3g_last_error": (C.c_char_p, []),
    "b3g_version": (C.c_char_p, []),
    "b3g_context_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "b3g_context_destroy": (C.c_int, [C.c_void_p]),
    "b3g_context_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "b3g_context_synchronize": (C.c_int, [C.c_void_p]),
    "b3g_body_create": (C.c_int, [C.c_void_p, C.POINTER(BodyDescC), C.POINTER(C.c_void_p)]),
    "b3g_body_destroy": (C.c_int, [C.c_void_p]),
    "b3g_body_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "b3g_body_device_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "b3g_body_step": (C.c_int, [C.c_void_p, C.c_float, C.POINTER(SolverConfig), C.POINTER(StepStats)]),
    "b3g_step_batch": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, C.c_float,
                                 C.POINTER(SolverConfig), C.c_uint32, C.POINTER(StepStats)]),
    "b3g_batch_schedule": (C.c_int, [C.c_void_p, _ip, C.c_uint32]),
    "b3g_step_batch_noalloc": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, C.c_float,
                                         C.POINTER(SolverConfig), C.c_uint32, C.POINTER(StepStats)]),
    "b3g_batch_phase_cycles": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int]),
    "b3g_batch_set_launch_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "b3g_batch_launch_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int]),
    "b3g_batch_element_launch_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "b3g_batch_assembly_split": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    "b3g_batch_apply_forces": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, _fp]),
    "b3g_batch_get_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, _fp, _fp]),
    "b3g_batch_get_state_async": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, _fp, _fp]),
    "b3g_batch_wait_state": (C.c_int, [C.c_void_p]),
    "b3g_body_get_state": (C.c_int, [C.c_void_p, _fp, _fp]),
    "b3g_body_set_state": (C.c_int, [C.c_void_p, _fp, _fp]),
    "b3g_body_apply_forces": (C.c_int, [C.c_void_p, _fp]),
    "b3g_body_apply_translations": (C.c_int, [C.c_void_p, _fp]),
    "b3g_body_set_types": (C.c_int, [C.c_void_p, _ip]),
    "b3g_body_get_rotations": (C.c_int, [C.c_void_p, _fp]),
    "b3g_body_set_rotations": (C.c_int, [C.c_void_p, _fp]),
    "b3g_body_get_masses": (C.c_int, [C.c_void_p, _fp]),
    "b3g_body_get_stats": (C.c_int, [C.c_void_p, C.POINTER(StepStats)]),
    "b3g_body_ray_cast": (C.c_int, [C.c_void_p, _fp, C.c_uint32, C.POINTER(RayHit)]),
    "b3g_server_create": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_float, C.POINTER(SolverConfig),
                                    C.POINTER(C.c_void_p)]),
    "b3g_server_add_body": (C.c_int, [C.c_void_p, C.POINTER(BodyDescC), _up]),
    "b3g_server_start": (C.c_int, [C.c_void_p]),
    "b3g_server_submit": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64)]),
    "b3g_server_poll": (C.c_int, [C.c_void_p, C.POINTER(RequestResult), C.c_uint32, _up]),
    "b3g_server_pending": (C.c_int, [C.c_void_p, _up]),
    "b3g_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "b3g_server_reset_stats": (C.c_int, [C.c_void_p]),
    "b3g_server_get_state": (C.c_int, [C.c_void_p, C.c_uint32, _fp, _fp]),
    "b3g_server_destroy": (C.c_int, [C.c_void_p]),
    "b3g_body_contact_fixtures": (C.c_int, [C.c_void_p, _up]),
    "b3g_body_get_contacts": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8), C.POINTER(C.c_uint8), _fp, _fp]),
    "b3g_body_set_contacts": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8), C.POINTER(C.c_uint8), _fp, _fp]),
    "b3g_body_desc_estimate_bytes": (C.c_int, [C.POINTER(BodyDescC), C.POINTER(C.c_uint64)]),
    "b3g_partition_bodies": (C.c_int, [C.POINTER(C.c_uint64), C.c_uint32, C.c_uint32, _up]),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Load libb3g.so; raise if it is absent (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libb3g.so not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class B3gError(RuntimeError):
    pass


def _check(rc: int, what: str):
    if rc != 0:
        msg = load_library().b3g_last_error().decode(errors="replace")
        raise B3gError(f"{what} failed ({rc}): {msg}")


def solver_config(force_iterations: int = 1, max_pcg_iterations: int = 200, pcg_tolerance: float = 1e-5,
                  refresh_period: int = 50, precision: int = PRECISION_FP32,
                  preconditioner: int = PRECOND_JACOBI, newton_tolerance: Optional[float] = None,
                  contact_mode: int = 0) -> SolverConfig:
    """b3g_solver_config; contact_mode CONTACT_PENALTY (the reference's) or CONTACT_FILTER."""
    lib = load_library()
    c = SolverConfig()
    lib.b3g_solver_config_default(C.byref(c))
    c.force_iterations = force_iterations
    c.max_pcg_iterations = max_pcg_iterations
    c.pcg_tolerance = pcg_tolerance
    c.refresh_period = refresh_period
    c.precision = precision
    c.preconditioner = preconditioner
    c.contact_mode = contact_mode
    if newton_tolerance is not None:
        c.newton_tolerance = newton_tolerance
    return c


class Context:
    """A b3g context. Bodies and servers made on it register here; close() closes them first, so a
    body never outlives the context its device memory and stream belong to."""

    def __init__(self, device: int = 0):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.b3g_context_create(device, C.byref(h)), "b3g_context_create")
        self.handle = h
        self.device = device
        self._dependents = weakref.WeakSet()

    def stream(self) -> int:
        s = C.c_void_p()
        _check(load_library().b3g_context_stream(self.handle, C.byref(s)), "b3g_context_stream")
        return s.value or 0

    def synchronize(self):
        _check(load_library().b3g_context_synchronize(self.handle), "b3g_context_synchronize")

    def close(self):
        if self.handle:
            # servers first (their worker thread steps bodies of this context), then bodies
            deps = sorted(list(self._dependents), key=lambda o: 0 if isinstance(o, Server) else 1)
            for o in deps:
                o.close()
            load_library().b3g_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t):
    if a is None or a.size == 0:
        return C.cast(None, t)
    return a.ctypes.data_as(t)


def _desc_struct(desc, masses=None):
    """A b3g_body_desc pointing into numpy copies of a meshes.BodyDesc; returns (struct, arrays to keep alive)."""
    keep = []

    def f(a):
        a = _f32(a)
        keep.append(a)
        return _ptr(a, _fp)

    def u(a):
        a = np.ascontiguousarray(a, dtype=np.uint32)
        keep.append(a)
        return _ptr(a, _up)

    d = BodyDescC()
    d.vertex_count = desc.n
    d.positions = f(desc.x)
    d.velocities = f(desc.v)
    types = np.ascontiguousarray(desc.type, dtype=np.int32)
    keep.append(types)
    d.types = types.ctypes.data_as(_ip)
    d.damping = f(desc.damping)
    d.masses = f(masses) if masses is not None else C.cast(None, _fp)
    d.tet_count = desc.tets.shape[0]
    d.tets = u(desc.tets)
    d.tet_rest = C.cast(None, _fp)
    d.tet_young, d.tet_poisson = f(desc.tet_E), f(desc.tet_nu)
    d.tet_stiffness_damping, d.tet_density = f(desc.tet_kdamp), f(desc.tet_density)
    d.tri_count = desc.tris.shape[0]
    d.tris = u(desc.tris)
    d.tri_rest = C.cast(None, _fp)
    d.tri_young_x, d.tri_young_y, d.tri_shear = f(desc.tri_Ex), f(desc.tri_Ey), f(desc.tri_Es)
    d.tri_poisson_xy, d.tri_poisson_yx = f(desc.tri_nuxy), f(desc.tri_nuyx)
    d.tri_stiffness_damping, d.tri_density = f(desc.tri_kdamp), f(desc.tri_density)
    d.spring_count = desc.springs.shape[0]
    d.springs = u(desc.springs)
    d.spring_rest_length, d.spring_stiffness, d.spring_damping = (
        f(desc.spring_L0), f(desc.spring_ks), f(desc.spring_kd))
    d.sphere_radius = f(desc.sphere_radius) if desc.sphere_radius is not None else C.cast(None, _fp)
    d.sphere_friction = f(desc.sphere_friction) if desc.sphere_friction is not None else C.cast(None, _fp)
    d.world_sphere_count = desc.world_spheres.shape[0]
    d.world_spheres = f(desc.world_spheres)
    for k in range(3):
        d.gravity[k] = float(desc.gravity[k])
    shapes = list(getattr(desc, "world_shapes", []) or [])
    d.world_shape_count = len(shapes)
    if shapes:
        arr = (WorldShapeC * len(shapes))()
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
                w.vertices = f(np.asarray(sh.vertices))
            if sh.triangles is not None:
                w.triangle_count = int(np.asarray(sh.triangles).shape[0])
                w.triangles = u(np.asarray(sh.triangles))
            if sh.wings is not None:
                w.wings = u(np.asarray(sh.wings))
            if sh.voxels is not None:
                vox = np.asarray(sh.voxels)
                w.grid[0], w.grid[1], w.grid[2] = vox.shape[2], vox.shape[1], vox.shape[0]
                w.voxels = f(vox)
            w.invert = 1 if sh.invert else 0
        d.world_shapes = C.cast(arr, C.POINTER(WorldShapeC))
    else:
        d.world_shapes = C.cast(None, C.POINTER(WorldShapeC))
    st = getattr(desc, "stretch_tris", None)
    if st is not None and len(st):
        d.stretch_count = len(st)
        d.stretch_tris = u(st)
        d.stretch_uv = f(desc.stretch_uv)
        d.stretch_params = f(desc.stretch_params)
    sh = getattr(desc, "shear_tris", None)
    if sh is not None and len(sh):
        d.shear_count = len(sh)
        d.shear_tris = u(sh)
        d.shear_uv = f(desc.shear_uv)
        d.shear_params = f(desc.shear_params)
    ms = getattr(desc, "mouse_ids", None)
    if ms is not None and len(ms):
        d.mouse_count = len(ms)
        d.mouse_ids = u(ms)
        d.mouse_params = f(desc.mouse_params)
    return d, keep


def estimate_bytes(desc) -> int:
    """b3g_body_desc_estimate_bytes: device bytes of a body made from desc (host only)."""
    d, keep = _desc_struct(desc)
    out = C.c_uint64()
    _check(load_library().b3g_body_desc_estimate_bytes(C.byref(d), C.byref(out)), "b3g_body_desc_estimate_bytes")
    del keep
    return int(out.value)


def partition(sizes, ranks: int) -> np.ndarray:
    """b3g_partition_bodies: the GPU of each body for a split of `sizes` (bytes) over `ranks`."""
    b = np.ascontiguousarray(np.asarray(sizes, np.uint64).reshape(-1))
    out = np.zeros(max(b.size, 1), np.uint32)
    _check(load_library().b3g_partition_bodies(b.ctypes.data_as(C.POINTER(C.c_uint64)), b.size, ranks,
                                               out.ctypes.data_as(_up)), "b3g_partition_bodies")
    return out[:b.size]


class Body:
    """One body on the GPU, created from a meshes.BodyDesc (or anything with its fields)."""

    def __init__(self, ctx: Context, desc, masses=None):
        lib = load_library()
        self.ctx = ctx
        d, keep = _desc_struct(desc, masses)
        h = C.c_void_p()
        _check(lib.b3g_body_create(ctx.handle, C.byref(d), C.byref(h)), "b3g_body_create")
        del keep
        self.handle = h
        ctx._dependents.add(self)
        self.n = desc.n
        self.tet_count = desc.tets.shape[0]

    def info(self) -> dict:
        a = (C.c_uint64 * 6)()
        _check(load_library().b3g_body_info(self.handle, a), "b3g_body_info")
        return dict(zip(["vertices", "tets", "tris", "springs", "nnzb", "slots"], list(a)))

    def device_bytes(self) -> int:
        b = C.c_uint64()
        _check(load_library().b3g_body_device_bytes(self.handle, C.byref(b)), "b3g_body_device_bytes")
        return int(b.value)

    def step(self, dt: float, config: Optional[SolverConfig] = None, stats: bool = True) -> Optional[dict]:
        cfg = config if config is not None else solver_config()
        st = StepStats()
        _check(load_library().b3g_body_step(self.handle, dt, C.byref(cfg), C.byref(st) if stats else None),
               "b3g_body_step")
        return st.as_dict() if stats else None

    def state(self):
        x = np.zeros((self.n, 3), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        _check(load_library().b3g_body_get_state(self.handle, x.ctypes.data_as(_fp), v.ctypes.data_as(_fp)),
               "b3g_body_get_state")
        return x, v

    def set_state(self, x=None, v=None):
        xa, va = _f32(x), _f32(v)
        _check(load_library().b3g_body_set_state(self.handle, _ptr(xa, _fp), _ptr(va, _fp)), "b3g_body_set_state")

    def apply_forces(self, f):
        fa = _f32(f)
        _check(load_library().b3g_body_apply_forces(self.handle, fa.ctypes.data_as(_fp)), "b3g_body_apply_forces")
        self.ctx.synchronize()

    def apply_translations(self, t):
        ta = _f32(t)
        _check(load_library().b3g_body_apply_translations(self.handle, ta.ctypes.data_as(_fp)),
               "b3g_body_apply_translations")
        self.ctx.synchronize()

    def set_types(self, types):
        t = np.ascontiguousarray(types, dtype=np.int32)
        _check(load_library().b3g_body_set_types(self.handle, t.ctypes.data_as(_ip)), "b3g_body_set_types")

    def rotations(self) -> np.ndarray:
        q = np.zeros((self.tet_count, 4), np.float32)
        _check(load_library().b3g_body_get_rotations(self.handle, q.ctypes.data_as(_fp)), "b3g_body_get_rotations")
        return q

    def set_rotations(self, q):
        qa = _f32(q)
        _check(load_library().b3g_body_set_rotations(self.handle, qa.ctypes.data_as(_fp)), "b3g_body_set_rotations")

    def ray_cast(self, segments):
        """b3Body::RayCastSingle for each row (p1, p2) of ``segments`` against the body's triangle
        fixtures. Returns (hit bool array, triangle index array, fraction array, normal array)."""
        seg = np.ascontiguousarray(np.asarray(segments, np.float32).reshape(-1, 6))
        out = (RayHit * max(len(seg), 1))()
        _check(load_library().b3g_body_ray_cast(self.handle, seg.ctypes.data_as(_fp), len(seg), out),
               "b3g_body_ray_cast")
        hits = list(out)[: len(seg)]
        return (np.array([h.hit != 0 for h in hits], bool), np.array([h.triangle for h in hits], np.int64),
                np.array([h.fraction for h in hits], np.float32),
                np.array([list(h.normal) for h in hits], np.float32).reshape(-1, 3))

    def masses(self) -> np.ndarray:
        m = np.zeros(self.n, np.float32)
        _check(load_library().b3g_body_get_masses(self.handle, m.ctypes.data_as(_fp)), "b3g_body_get_masses")
        return m

    def stats(self) -> dict:
        st = StepStats()
        _check(load_library().b3g_body_get_stats(self.handle, C.byref(st)), "b3g_body_get_stats")
        return st.as_dict()

    def contacts(self) -> dict:
        """b3g_body_get_contacts: per (vertex, fixture) exists, apply_friction, normal_force, normal."""
        lib = load_library()
        k = C.c_uint32()
        _check(lib.b3g_body_contact_fixtures(self.handle, C.byref(k)), "b3g_body_contact_fixtures")
        c = self.n * k.value
        out = {"fixtures": k.value, "exists": np.zeros(c, np.uint8), "apply_friction": np.zeros(c, np.uint8),
               "normal_force": np.zeros(c, np.float32), "normal": np.zeros((c, 3), np.float32)}
        u8 = C.POINTER(C.c_uint8)
        _check(lib.b3g_body_get_contacts(self.handle, out["exists"].ctypes.data_as(u8),
                                         out["apply_friction"].ctypes.data_as(u8),
                                         out["normal_force"].ctypes.data_as(_fp), out["normal"].ctypes.data_as(_fp)),
               "b3g_body_get_contacts")
        return out

    def set_contacts(self, c: dict):
        u8 = C.POINTER(C.c_uint8)
        ex = np.ascontiguousarray(c["exists"], np.uint8)
        ap = np.ascontiguousarray(c["apply_friction"], np.uint8)
        nf = np.ascontiguousarray(c["normal_force"], np.float32)
        nn = np.ascontiguousarray(c["normal"], np.float32)
        _check(load_library().b3g_body_set_contacts(self.handle, ex.ctypes.data_as(u8), ap.ctypes.data_as(u8),
                                                    nf.ctypes.data_as(_fp), nn.ctypes.data_as(_fp)),
               "b3g_body_set_contacts")

    def close(self):
        if self.handle:
            load_library().b3g_body_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def step_batch(ctx: Context, bodies: Sequence[Body], dt: float, steps: int = 1,
               config: Optional[SolverConfig] = None, stats: bool = True):
    lib = load_library()
    cfg = config if config is not None else solver_config()
    arr = (C.c_void_p * len(bodies))(*[b.handle for b in bodies])
    st = (StepStats * len(bodies))()
    _check(lib.b3g_step_batch(ctx.handle, arr, len(bodies), dt, C.byref(cfg), steps, st if stats else None),
           "b3g_step_batch")
    return [s.as_dict() for s in st] if stats else None


def step_batch_noalloc(ctx: Context, bodies: Sequence[Body], dt: float, steps: int = 1,
                       config: Optional[SolverConfig] = None, stats: bool = True):
    """b3g_step_batch_noalloc: the batched step with no device (or host) allocation in the call."""
    lib = load_library()
    cfg = config if config is not None else solver_config()
    arr = (C.c_void_p * len(bodies))(*[b.handle for b in bodies])
    st = (StepStats * max(len(bodies), 1))()
    _check(lib.b3g_step_batch_noalloc(ctx.handle, arr, len(bodies), dt, C.byref(cfg), steps, st if stats else None),
           "b3g_step_batch_noalloc")
    return [s.as_dict() for s in st[:len(bodies)]] if stats else None


def batch_schedule(ctx: Context) -> dict:
    """b3g_batch_schedule: the schedule of the context's current batch and the autotuner's timings."""
    buf = np.zeros(512, np.int32)
    _check(load_library().b3g_batch_schedule(ctx.handle, buf.ctypes.data_as(_ip), buf.size), "b3g_batch_schedule")
    n = int(buf[5])
    cands = [((int(buf[7 + 2 * k]) // 1000000) % 100, int(buf[7 + 2 * k]) % 1000000,
              "lpt" if int(buf[7 + 2 * k]) >= 100000000 else "size", buf[8 + 2 * k] / 1000.0)
             for k in range(min(n, (buf.size - 7) // 2))]
    return {"cluster": int(buf[0]), "threshold": int(buf[1]), "cluster_bodies": int(buf[2]),
            "ctas": int(buf[3]), "autotuned": bool(buf[4]), "order": "lpt" if int(buf[6]) else "size",
            "candidates_ms": cands}


def batch_assembly_split(ctx: Context) -> dict:
    """b3g_batch_assembly_split: where the second body group of the split assembly starts."""
    a = (C.c_uint32 * 4)()
    _check(load_library().b3g_batch_assembly_split(ctx.handle, a), "b3g_batch_assembly_split")
    return {"elem_mid": int(a[0]), "slice_mid": int(a[1]), "element_ctas_per_sm": int(a[2]),
            "row_ctas_per_sm": int(a[3])}


def batch_apply_forces(ctx: Context, bodies: Sequence[Body], forces_ptr: int):
    """forces_ptr: host address of the concatenated forces (3 floats per vertex, list order)."""
    arr = (C.c_void_p * len(bodies))(*[b.handle for b in bodies])
    _check(load_library().b3g_batch_apply_forces(ctx.handle, arr, len(bodies), C.cast(forces_ptr, _fp)),
           "b3g_batch_apply_forces")


def batch_get_state(ctx: Context, bodies: Sequence[Body], x_ptr: int, v_ptr: int):
    """Copy every body's positions / velocities into concatenated host arrays (addresses)."""
    arr = (C.c_void_p * len(bodies))(*[b.handle for b in bodies])
    _check(load_library().b3g_batch_get_state(ctx.handle, arr, len(bodies), C.cast(x_ptr, _fp), C.cast(v_ptr, _fp)),
           "b3g_batch_get_state")


def batch_get_state_async(ctx: Context, bodies: Sequence[Body], x_ptr: int, v_ptr: int):
    """b3g_batch_get_state_async: the same copy on the context's second stream; the host arrays
    are filled once batch_wait_state returns."""
    arr = (C.c_void_p * len(bodies))(*[b.handle for b in bodies])
    _check(load_library().b3g_batch_get_state_async(ctx.handle, arr, len(bodies), C.cast(x_ptr, _fp),
                                                    C.cast(v_ptr, _fp)), "b3g_batch_get_state_async")


def batch_wait_state(ctx: Context):
    _check(load_library().b3g_batch_wait_state(ctx.handle), "b3g_batch_wait_state")


def batch_set_launch_timing(ctx: Context, on: bool):
    _check(load_library().b3g_batch_set_launch_timing(ctx.handle, 1 if on else 0), "b3g_batch_set_launch_timing")


def batch_launch_times(ctx: Context, reset: bool = True) -> dict:
    """Accumulated device ms of the assembly and PCG launches of timed batched steps, and the
    element launch's part of the assembly ms."""
    lib = load_library()
    el = C.c_double(0.0)
    _check(lib.b3g_batch_element_launch_ms(ctx.handle, C.byref(el)), "b3g_batch_element_launch_ms")
    a = (C.c_double * 3)()
    _check(lib.b3g_batch_launch_times(ctx.handle, a, 1 if reset else 0), "b3g_batch_launch_times")
    return {"assembly_ms": a[0], "pcg_ms": a[1], "steps": int(a[2]), "elements_ms": el.value}


PHASES = ["elements", "assembly", "spmv", "update", "direction", "final", "-", "-"]


def batch_phase_cycles(ctx: Context, reset: bool = True) -> dict:
    a = (C.c_uint64 * 8)()
    _check(load_library().b3g_batch_phase_cycles(ctx.handle, a, 1 if reset else 0), "b3g_batch_phase_cycles")
    return {PHASES[k]: int(a[k]) for k in range(6)}


class Server:
    """Continuous-batching request loop over many bodies (b3g_server_*).

    Register bodies with add_body, start the worker, submit (body, steps) requests from any
    thread and poll finished ones. Close before the context."""

    def __init__(self, ctx: Context, memory_budget_bytes: int, max_active: int, dt: float,
                 config: Optional[SolverConfig] = None):
        lib = load_library()
        self.ctx = ctx
        cfg = config if config is not None else solver_config()
        h = C.c_void_p()
        _check(lib.b3g_server_create(ctx.handle, int(memory_budget_bytes), int(max_active), float(dt),
                                     C.byref(cfg), C.byref(h)), "b3g_server_create")
        self.handle = h
        ctx._dependents.add(self)
        self.sizes = []

    def add_body(self, desc, masses=None) -> int:
        d, keep = _desc_struct(desc, masses)
        out = C.c_uint32()
        _check(load_library().b3g_server_add_body(self.handle, C.byref(d), C.byref(out)), "b3g_server_add_body")
        del keep
        self.sizes.append(desc.n)
        return int(out.value)

    def start(self):
        _check(load_library().b3g_server_start(self.handle), "b3g_server_start")

    def submit(self, body_id: int, steps: int) -> int:
        rid = C.c_uint64()
        _check(load_library().b3g_server_submit(self.handle, int(body_id), int(steps), C.byref(rid)),
               "b3g_server_submit")
        return int(rid.value)

    def poll(self, capacity: int = 1024) -> list:
        buf = (RequestResult * capacity)()
        n = C.c_uint32()
        _check(load_library().b3g_server_poll(self.handle, buf, capacity, C.byref(n)), "b3g_server_poll")
        return [{"request_id": int(r.request_id), "body_id": int(r.body_id), "steps": int(r.steps),
                 "status": REQUEST_STATUS.get(r.status, str(r.status)), "pcg_iterations": int(r.pcg_iterations),
                 "queue_seconds": r.queue_seconds, "latency_seconds": r.latency_seconds}
                for r in buf[:n.value]]

    def pending(self) -> int:
        n = C.c_uint32()
        _check(load_library().b3g_server_pending(self.handle, C.byref(n)), "b3g_server_pending")
        return int(n.value)

    def drain(self, timeout: float = 600.0, poll_interval: float = 0.001) -> list:
        """Wait until every submitted request has finished; return the finished requests."""
        import time
        out = []
        t0 = time.monotonic()
        while True:
            out += self.poll()
            if self.pending() == 0:
                return out + self.poll()
            if time.monotonic() - t0 > timeout:
                raise B3gError(f"server requests not finished after {timeout} s")
            time.sleep(poll_interval)

    def stats(self) -> dict:
        st = ServerStats()
        _check(load_library().b3g_server_get_stats(self.handle, C.byref(st)), "b3g_server_get_stats")
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def reset_stats(self):
        _check(load_library().b3g_server_reset_stats(self.handle), "b3g_server_reset_stats")

    def state(self, body_id: int):
        n = self.sizes[body_id]
        x = np.empty((n, 3), np.float32)
        v = np.empty((n, 3), np.float32)
        _check(load_library().b3g_server_get_state(self.handle, int(body_id), _ptr(x, _fp), _ptr(v, _fp)),
               "b3g_server_get_state")
        return x, v

    def close(self):
        if self.handle:
            load_library().b3g_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
