"""ctypes binding of include/b3g_sparse.h: the reference's sparse value types (b3DenseVec3,
b3DiagMat33, b3SparseMat33) and solvers (b3SparseSolveCG, b3SparseSolveBE with a force-model
callback), device-resident, on a b3g context. Blocks are 9 floats in b3Mat33 order (column-major),
vectors 3 floats per entry, as in the C ABI."""
from __future__ import annotations

import ctypes as C
from typing import Callable, Optional

import numpy as np

from .b3g import B3gError, Context, SOLVE_STATUS, _check, load_library

_fp = C.POINTER(C.c_float)
_up = C.POINTER(C.c_uint32)
_vp = C.c_void_p


class SolveCGInput(C.Structure):
    _fields_ = [("A", _vp), ("b", _vp), ("max_iterations", C.c_uint32), ("tolerance", C.c_float)]


class SolveCGOutput(C.Structure):
    _fields_ = [("x", _vp), ("iterations", C.c_uint32), ("error", C.c_double), ("status", C.c_int32)]


class ForceSolverData(C.Structure):
    _fields_ = [("h", C.c_float), ("inv_h", C.c_float), ("x", _vp), ("v", _vp), ("f", _vp), ("dfdx", _vp),
                ("dfdv", _vp)]


APPLY_FORCES = C.CFUNCTYPE(None, _vp, C.POINTER(ForceSolverData))


class ForceModelC(C.Structure):
    _fields_ = [("apply_forces", APPLY_FORCES), ("user", _vp)]


class SolveBEInput(C.Structure):
    _fields_ = [("h", C.c_float), ("inv_h", C.c_float), ("force_model", ForceModelC), ("dof_count", C.c_uint32),
                ("x0", _vp), ("v0", _vp), ("fe", _vp), ("M", _vp), ("y", _vp), ("S", _vp), ("z", _vp),
                ("max_iterations", C.c_uint32), ("tolerance", C.c_float), ("max_sub_iterations", C.c_uint32),
                ("sub_tolerance", C.c_float)]


class SolveBEOutput(C.Structure):
    _fields_ = [("x", _vp), ("v", _vp), ("iterations", C.c_uint32), ("error", C.c_double),
                ("min_sub_iterations", C.c_uint32), ("max_sub_iterations", C.c_uint32), ("status", C.c_int32)]


_i = C.c_int
SIGNATURES = {
    "b3g_dense_vec3_create": (_i, [_vp, C.c_uint32, C.POINTER(_vp)]),
    "b3g_dense_vec3_destroy": (_i, [_vp]),
    "b3g_dense_vec3_size": (_i, [_vp, _up]),
    "b3g_dense_vec3_set": (_i, [_vp, _fp]),
    "b3g_dense_vec3_get": (_i, [_vp, _fp]),
    "b3g_dense_vec3_set_zero": (_i, [_vp]),
    "b3g_dense_vec3_copy": (_i, [_vp, _vp]),
    "b3g_dense_vec3_add": (_i, [_vp, _vp, _vp]),
    "b3g_dense_vec3_sub": (_i, [_vp, _vp, _vp]),
    "b3g_dense_vec3_scale": (_i, [_vp, C.c_float, _vp]),
    "b3g_dense_vec3_negate": (_i, [_vp, _vp]),
    "b3g_dense_vec3_dot": (_i, [_vp, _vp, C.POINTER(C.c_double)]),
    "b3g_dense_vec3_length_squared": (_i, [_vp, C.POINTER(C.c_double)]),
    "b3g_dense_vec3_add_values": (_i, [_vp, C.c_uint32, _up, _fp]),
    "b3g_dense_vec3_set_values": (_i, [_vp, C.c_uint32, _up, _fp]),
    "b3g_dense_vec3_device": (_i, [_vp, C.POINTER(_vp)]),
    "b3g_diag_mat33_create": (_i, [_vp, C.c_uint32, C.POINTER(_vp)]),
    "b3g_diag_mat33_destroy": (_i, [_vp]),
    "b3g_diag_mat33_size": (_i, [_vp, _up]),
    "b3g_diag_mat33_set": (_i, [_vp, _fp]),
    "b3g_diag_mat33_get": (_i, [_vp, _fp]),
    "b3g_diag_mat33_set_zero": (_i, [_vp]),
    "b3g_diag_mat33_set_identity": (_i, [_vp]),
    "b3g_diag_mat33_copy": (_i, [_vp, _vp]),
    "b3g_diag_mat33_transpose": (_i, [_vp, _vp]),
    "b3g_diag_mat33_add": (_i, [_vp, _vp, _vp]),
    "b3g_diag_mat33_sub": (_i, [_vp, _vp, _vp]),
    "b3g_diag_mat33_scale": (_i, [_vp, C.c_float, _vp]),
    "b3g_diag_mat33_negate": (_i, [_vp, _vp]),
    "b3g_diag_mat33_mul_vec": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_create": (_i, [_vp, C.c_uint32, C.POINTER(_vp)]),
    "b3g_sparse_mat33_destroy": (_i, [_vp]),
    "b3g_sparse_mat33_size": (_i, [_vp, _up, C.POINTER(C.c_uint64)]),
    "b3g_sparse_mat33_add_blocks": (_i, [_vp, C.c_uint32, _up, _up, _fp]),
    "b3g_sparse_mat33_set_blocks": (_i, [_vp, C.c_uint32, _up, _up, _fp]),
    "b3g_sparse_mat33_get_block": (_i, [_vp, C.c_uint32, C.c_uint32, _fp]),
    "b3g_sparse_mat33_export": (_i, [_vp, _up, _up, _fp, C.c_uint64, C.POINTER(C.c_uint64)]),
    "b3g_sparse_mat33_to_dense": (_i, [_vp, _fp]),
    "b3g_sparse_mat33_clear": (_i, [_vp]),
    "b3g_sparse_mat33_zero_values": (_i, [_vp]),
    "b3g_sparse_mat33_copy": (_i, [_vp, _vp]),
    "b3g_sparse_mat33_add": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_sub": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_add_diag": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_sub_diag": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_diag_add": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_diag_sub": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_scale": (_i, [_vp, C.c_float, _vp]),
    "b3g_sparse_mat33_diag_mul": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_mul_diag": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_mat33_mul_vec": (_i, [_vp, _vp, _vp]),
    "b3g_sparse_solve_cg": (_i, [C.POINTER(SolveCGOutput), C.POINTER(SolveCGInput)]),
    "b3g_sparse_solve_be": (_i, [C.POINTER(SolveBEOutput), C.POINTER(SolveBEInput)]),
}

_bound = None


def lib():
    global _bound
    if _bound is None:
        L = load_library()
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _bound = L
    return _bound


def _f32(a, count):
    a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
    if a.size != count:
        raise ValueError(f"expected {count} floats, got {a.size}")
    return a


class _Handle:
    _destroy = ""

    def __init__(self, ctx: Context, n: int, create: str):
        self.ctx = ctx
        self.n = int(n)
        h = _vp()
        _check(getattr(lib(), create)(ctx.handle, self.n, C.byref(h)), create)
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            getattr(lib(), self._destroy)(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DenseVec3(_Handle):
    """b3DenseVec3 on the device."""
    _destroy = "b3g_dense_vec3_destroy"

    def __init__(self, ctx: Context, n: int, values=None):
        super().__init__(ctx, n, "b3g_dense_vec3_create")
        if values is not None:
            self.set(values)

    def set(self, values):
        a = _f32(values, 3 * self.n)
        _check(lib().b3g_dense_vec3_set(self.handle, a.ctypes.data_as(_fp)), "b3g_dense_vec3_set")

    def get(self) -> np.ndarray:
        a = np.zeros((self.n, 3), np.float32)
        _check(lib().b3g_dense_vec3_get(self.handle, a.ctypes.data_as(_fp)), "b3g_dense_vec3_get")
        return a

    def add_values(self, index, values, op="add"):
        idx = np.ascontiguousarray(np.asarray(index, np.uint32).reshape(-1))
        val = _f32(values, 3 * idx.size)
        fn = lib().b3g_dense_vec3_add_values if op == "add" else lib().b3g_dense_vec3_set_values
        _check(fn(self.handle, idx.size, idx.ctypes.data_as(_up), val.ctypes.data_as(_fp)), "dense_vec3 values")

    def dot(self, other: "DenseVec3") -> float:
        out = C.c_double()
        _check(lib().b3g_dense_vec3_dot(self.handle, other.handle, C.byref(out)), "b3g_dense_vec3_dot")
        return out.value

    def length_squared(self) -> float:
        out = C.c_double()
        _check(lib().b3g_dense_vec3_length_squared(self.handle, C.byref(out)), "b3g_dense_vec3_length_squared")
        return out.value


def vec_op(name: str, *args):
    """A b3g_dense_vec3_* operation on handles / scalars in C-ABI order."""
    conv = [a.handle if isinstance(a, _Handle) else a for a in args]
    _check(getattr(lib(), "b3g_dense_vec3_" + name)(*conv), "b3g_dense_vec3_" + name)


class DiagMat33(_Handle):
    """b3DiagMat33 on the device."""
    _destroy = "b3g_diag_mat33_destroy"

    def __init__(self, ctx: Context, n: int, blocks=None):
        super().__init__(ctx, n, "b3g_diag_mat33_create")
        if blocks is not None:
            self.set(blocks)

    def set(self, blocks):
        a = _f32(blocks, 9 * self.n)
        _check(lib().b3g_diag_mat33_set(self.handle, a.ctypes.data_as(_fp)), "b3g_diag_mat33_set")

    def get(self) -> np.ndarray:
        a = np.zeros((self.n, 9), np.float32)
        _check(lib().b3g_diag_mat33_get(self.handle, a.ctypes.data_as(_fp)), "b3g_diag_mat33_get")
        return a


def diag_op(name: str, *args):
    conv = [a.handle if isinstance(a, _Handle) else a for a in args]
    _check(getattr(lib(), "b3g_diag_mat33_" + name)(*conv), "b3g_diag_mat33_" + name)


class SparseMat33(_Handle):
    """b3SparseMat33 on the device."""
    _destroy = "b3g_sparse_mat33_destroy"

    def __init__(self, ctx: Context, n: int):
        super().__init__(ctx, n, "b3g_sparse_mat33_create")

    def add_blocks(self, rows, cols, blocks, op="add"):
        r = np.ascontiguousarray(np.asarray(rows, np.uint32).reshape(-1))
        c = np.ascontiguousarray(np.asarray(cols, np.uint32).reshape(-1))
        b = _f32(blocks, 9 * r.size)
        fn = lib().b3g_sparse_mat33_add_blocks if op == "add" else lib().b3g_sparse_mat33_set_blocks
        _check(fn(self.handle, r.size, r.ctypes.data_as(_up), c.ctypes.data_as(_up), b.ctypes.data_as(_fp)),
               "sparse_mat33 blocks")

    def size(self):
        n, nb = C.c_uint32(), C.c_uint64()
        _check(lib().b3g_sparse_mat33_size(self.handle, C.byref(n), C.byref(nb)), "b3g_sparse_mat33_size")
        return n.value, nb.value

    def get_block(self, i, j) -> np.ndarray:
        a = np.zeros(9, np.float32)
        _check(lib().b3g_sparse_mat33_get_block(self.handle, i, j, a.ctypes.data_as(_fp)), "get_block")
        return a

    def export(self):
        _, nb = self.size()
        rp = np.zeros(self.n + 1, np.uint32)
        cols = np.zeros(max(nb, 1), np.uint32)
        blk = np.zeros((max(nb, 1), 9), np.float32)
        cnt = C.c_uint64()
        _check(lib().b3g_sparse_mat33_export(self.handle, rp.ctypes.data_as(_up), cols.ctypes.data_as(_up),
                                             blk.ctypes.data_as(_fp), max(nb, 1), C.byref(cnt)), "export")
        return rp, cols[:cnt.value], blk[:cnt.value]

    def to_dense(self) -> np.ndarray:
        a = np.zeros(9 * self.n * self.n, np.float32)
        _check(lib().b3g_sparse_mat33_to_dense(self.handle, a.ctypes.data_as(_fp)), "to_dense")
        return a.reshape(3 * self.n, 3 * self.n, order="F")


def sp_op(name: str, *args):
    conv = [a.handle if isinstance(a, _Handle) else a for a in args]
    _check(getattr(lib(), "b3g_sparse_mat33_" + name)(*conv), "b3g_sparse_mat33_" + name)


def solve_cg(A: SparseMat33, b: DenseVec3, x: DenseVec3, max_iterations: int, tolerance: float) -> dict:
    """b3SparseSolveCG: x holds the initial guess and receives the solution."""
    ci = SolveCGInput(A.handle, b.handle, max_iterations, tolerance)
    co = SolveCGOutput()
    co.x = x.handle
    _check(lib().b3g_sparse_solve_cg(C.byref(co), C.byref(ci)), "b3g_sparse_solve_cg")
    return {"iterations": co.iterations, "error": co.error, "status": SOLVE_STATUS.get(co.status, co.status)}


class ForceSolverView:
    """What a Python force model receives: handles of the solver's containers."""

    def __init__(self, ctx: Context, data: ForceSolverData, n: int):
        self.h, self.inv_h = data.h, data.inv_h
        self.x = _borrowed(DenseVec3, ctx, data.x, n)
        self.v = _borrowed(DenseVec3, ctx, data.v, n)
        self.f = _borrowed(DenseVec3, ctx, data.f, n)
        self.dfdx = _borrowed(SparseMat33, ctx, data.dfdx, n)
        self.dfdv = _borrowed(SparseMat33, ctx, data.dfdv, n)


def _borrowed(cls, ctx, handle, n):
    o = cls.__new__(cls)
    o.ctx, o.n, o.handle = ctx, n, _vp(handle)
    o.close = lambda: None  # owned by the solver
    o.__del__ = lambda: None
    return o


def solve_be(ctx: Context, apply_forces: Callable[[ForceSolverView], None], h: float, x0: DenseVec3,
             v0: DenseVec3, fe: DenseVec3, M: DiagMat33, y: DenseVec3, S: DiagMat33, z: DenseVec3, x: DenseVec3,
             v: DenseVec3, max_iterations: int = 1, tolerance: float = 1.1920928955078125e-07,
             max_sub_iterations: int = 20, sub_tolerance: float = 1.1920928955078125e-07) -> dict:
    """b3SparseSolveBE with a Python force model (called once per Newton iteration)."""
    n = x0.n
    errors = []

    def cb(user, data_p):
        try:
            apply_forces(ForceSolverView(ctx, data_p.contents, n))
        except Exception as exc:  # surfaced after the call
            errors.append(exc)

    fn = APPLY_FORCES(cb)
    bi = SolveBEInput()
    bi.h, bi.inv_h = h, 1.0 / h
    bi.force_model = ForceModelC(fn, None)
    bi.dof_count = n
    bi.x0, bi.v0, bi.fe, bi.M, bi.y, bi.S, bi.z = (x0.handle, v0.handle, fe.handle, M.handle, y.handle, S.handle,
                                                    z.handle)
    bi.max_iterations, bi.tolerance = max_iterations, tolerance
    bi.max_sub_iterations, bi.sub_tolerance = max_sub_iterations, sub_tolerance
    bo = SolveBEOutput()
    bo.x, bo.v = x.handle, v.handle
    bo.min_sub_iterations, bo.max_sub_iterations = 0xFFFFFFFF, 0
    rc = lib().b3g_sparse_solve_be(C.byref(bo), C.byref(bi))
    if errors:
        raise errors[0]
    _check(rc, "b3g_sparse_solve_be")
    return {"iterations": bo.iterations, "error": bo.error, "min_sub": bo.min_sub_iterations,
            "max_sub": bo.max_sub_iterations, "status": SOLVE_STATUS.get(bo.status, bo.status)}


__all__ = ["DenseVec3", "DiagMat33", "SparseMat33", "vec_op", "diag_op", "sp_op", "solve_cg", "solve_be",
           "B3gError"]
