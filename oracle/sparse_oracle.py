"""numpy restatement of the reference's sparse containers and solvers (test infrastructure only).

Restates, in float64 with scipy's block-sparse matrices:

* the backward-Euler system build and pre-filter of b3SparseSolveBE
  (src/bounce_softbody/sparse/sparse_force_solver.cpp:165-174):
  A = M - h dfdv - h^2 dfdx, b = M (v0 - v) + h (fe + f) + h dfdx (x0 - x + h v + y),
  pA = S A S^T + I - S, pb = S (b - A z);
* the Jacobi-preconditioned CG of b3SparseSolveCG (src/bounce_softbody/sparse/sparse_solver.cpp:28-109):
  scalar Jacobi from the diagonal entries of each diagonal block, stop at the loop top when
  iteration == max or delta <= tol^2 delta0, true residual recomputed when iteration % 50 == 0;
* one Newton iteration of b3SparseSolveBE (sparse_force_solver.cpp:176-226): dv = y' + z,
  v = v0 + dv, x = x0 + h v + y, error = |dv|^2.

Blocks are 9 values in b3Mat33 order (column-major, include/bounce_softbody/common/math/mat33.h:25):
entry (r, c) of a block is value[3 c + r]. Used by tests to pin the golden vectors of
tests/golden/sparse_tet10.npz (made by the reference itself) and to check the GPU containers.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def blocks_rowmajor(vals) -> np.ndarray:
    """(k, 9) b3Mat33-ordered values -> (k, 3, 3) with [r, c]."""
    return np.asarray(vals, np.float64).reshape(-1, 3, 3).transpose(0, 2, 1)


def coo_matrix(n, rows, cols, vals) -> sp.csr_matrix:
    """The (3n x 3n) matrix of 3x3 blocks at (rows[k], cols[k]); repeated blocks add up, as
    b3SparseMat33::operator()(i, j) += does (sparse_mat33.h:268-288)."""
    B = blocks_rowmajor(vals)
    r = np.asarray(rows, np.int64)
    c = np.asarray(cols, np.int64)
    ii = (3 * r[:, None, None] + np.arange(3)[None, :, None]).repeat(3, 2)
    jj = (3 * c[:, None, None] + np.arange(3)[None, None, :]).repeat(3, 1)
    return sp.csr_matrix((B.ravel(), (ii.ravel(), jj.ravel())), shape=(3 * n, 3 * n))


def diag_matrix(blocks9) -> sp.csr_matrix:
    """A b3DiagMat33 (n blocks of 9 values) as a block-diagonal matrix."""
    B = blocks_rowmajor(blocks9)
    return sp.csr_matrix(sp.block_diag([sp.coo_matrix(b) for b in B], format="csr"))


def system(n, h, dfdx, dfdv, f, x0, v0, x, v, fe, M, S, y, z):
    """A, b, pA, pb of sparse_force_solver.cpp:165-174 (dfdx, dfdv, M, S: scipy matrices)."""
    A = M - h * dfdv - (h * h) * dfdx
    b = M @ (v0 - v).ravel() + h * (fe + f).ravel() + h * (dfdx @ (x0 - x + h * v + y).ravel())
    I = sp.identity(3 * n, format="csr")
    pA = S @ A @ S.T + I - S
    pb = S @ (b - A @ z.ravel())
    return A, b.reshape(n, 3), pA.tocsr(), pb.reshape(n, 3)


def jacobi(A: sp.csr_matrix) -> np.ndarray:
    """invM = diag(1 / a.x.x, 1 / a.y.y, 1 / a.z.z) of each diagonal block (sparse_solver.cpp:38-55)."""
    return 1.0 / A.diagonal()


def solve_cg(A: sp.csr_matrix, b, max_iterations: int, tolerance: float, x0=None, refresh: int = 50):
    """b3SparseSolveCG. Returns (x, iterations, error = delta at exit)."""
    b = np.asarray(b, np.float64).ravel()
    x = np.zeros_like(b) if x0 is None else np.asarray(x0, np.float64).ravel().copy()
    inv = jacobi(A)
    r = b - A @ x
    d = inv * r
    delta = float(r @ d)
    delta0 = delta
    it = 0
    while True:
        if it == max_iterations or delta <= tolerance * tolerance * delta0:
            break
        q = A @ d
        alpha = delta / float(d @ q)
        x = x + alpha * d
        r = b - A @ x if it % refresh == 0 else r - alpha * q
        s = inv * r
        old = delta
        delta = float(r @ s)
        d = s + (delta / old) * d
        it += 1
    return x.reshape(-1, 3), it, delta


def solve_be_one(n, h, dfdx, dfdv, f, x0, v0, fe, M, S, y, z, max_sub, sub_tol):
    """One Newton iteration of b3SparseSolveBE from x = x0, v = v0, initial guess 0.
    Returns (x, v, sub_iterations, error)."""
    A, b, pA, pb = system(n, h, dfdx, dfdv, f, x0, v0, x0, v0, fe, M, S, y, z)
    py, it, _ = solve_cg(pA, pb, max_sub, sub_tol)
    dv = py + z
    v = v0 + dv
    x = x0 + h * v + y
    return x, v, it, float((dv * dv).sum())
