"""The golden vectors of the sparse container / solver boundary (tests/golden/sparse_tet10.npz,
made by the reference's own FP32 and FP64 builds) pinned against the numpy restatement in
oracle/sparse_oracle.py: the block layout, the backward-Euler system and pre-filter, every SpMV
product, Jacobi PCG and one backward-Euler iteration. CPU only."""
import os

import numpy as np
import pytest
import scipy.sparse as sp

import sparse_oracle as so
from conftest import GOLDEN

PRODUCTS = ["A", "pA", "D_dfdx", "dfdx_D", "s_dfdx", "dfdx_plus_dfdv", "dfdx_minus_dfdv", "dfdx_plus_D",
            "D_minus_dfdx", "zero_dfdx"]


@pytest.fixture(scope="module")
def g():
    z = np.load(os.path.join(GOLDEN, "sparse_tet10.npz"))
    return {k: z[k] for k in z.files}


def inputs(g):
    n, h = int(g["n"]), float(g["h"])
    f64 = lambda k: g[k].astype(np.float64)  # noqa: E731
    dfdx = so.coo_matrix(n, g["dfdx_rows"], g["dfdx_cols"], f64("dfdx_vals"))
    dfdv = so.coo_matrix(n, g["dfdv_rows"], g["dfdv_cols"], f64("dfdv_vals"))
    eye = np.eye(3)
    M = sp.csr_matrix(sp.diags(np.repeat(f64("mass"), 3)))
    S = sp.csr_matrix(sp.diags(np.repeat(g["dynamic"].astype(np.float64), 3)))
    D = so.diag_matrix(f64("D"))
    return n, h, dfdx, dfdv, M, S, D


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_golden_products_match_restatement(g):
    n, h, dfdx, dfdv, M, S, D = inputs(g)
    f64 = lambda k: g[k].astype(np.float64)  # noqa: E731
    A, b, pA, pb = so.system(n, h, dfdx, dfdv, f64("f"), f64("x"), f64("v"), f64("x"), f64("v"), f64("fe"), M, S,
                             f64("y"), f64("z"))
    u = f64("u").ravel()
    s = float(g["s"])
    mats = {"A": A, "pA": pA, "D_dfdx": D @ dfdx, "dfdx_D": dfdx @ D, "s_dfdx": s * dfdx,
            "dfdx_plus_dfdv": dfdx + dfdv, "dfdx_minus_dfdv": dfdx - dfdv, "dfdx_plus_D": dfdx + D,
            "D_minus_dfdx": D - dfdx, "zero_dfdx": 0 * dfdx}
    for k, name in enumerate(PRODUCTS):
        ref64 = g["ref64_spmv"][k].ravel()
        mine = mats[name] @ u
        assert rel(mine, ref64) < 1e-12, name
        # the FP32 build agrees to float rounding
        assert rel(g["ref32_spmv"][k].ravel(), ref64) < 1e-5, name
    assert rel(b, g["ref64_b"]) < 1e-12
    assert rel(pb, g["ref64_pb"]) < 1e-12
    assert rel((D @ u).reshape(n, 3), g["ref64_diag_u"]) < 1e-12
    assert abs(float(u @ pb.ravel()) - float(g["ref64_dot_u_pb"])) <= 1e-12 * abs(float(g["ref64_dot_u_pb"]))
    assert abs(float((pb * pb).sum()) - float(g["ref64_len2_pb"])) <= 1e-12 * float(g["ref64_len2_pb"])
    # pA's pattern and diagonal blocks (FP32 build)
    rp, cols = g["ref32_pA_row_ptr"].astype(np.int64), g["ref32_pA_cols"].astype(np.int64)
    pat = sp.csr_matrix((np.ones(len(cols)), cols, rp), shape=(n, n))
    blk = sp.csr_matrix(abs(pA)).tocoo()
    mine_pat = sp.csr_matrix((np.ones(blk.nnz), (blk.row // 3, blk.col // 3)), shape=(n, n))
    mine_pat.data[:] = 1.0
    # the reference keeps zero blocks that the filter produced (pinned rows and columns)
    assert (mine_pat - mine_pat.multiply(pat)).nnz == 0
    diag = np.stack([pA[3 * i:3 * i + 3, 3 * i:3 * i + 3].toarray() for i in range(n)])
    assert rel(diag, so.blocks_rowmajor(g["ref32_pA_diag"])) < 1e-6


def test_golden_cg_and_be_match_restatement(g):
    n, h, dfdx, dfdv, M, S, D = inputs(g)
    f64 = lambda k: g[k].astype(np.float64)  # noqa: E731
    A, b, pA, pb = so.system(n, h, dfdx, dfdv, f64("f"), f64("x"), f64("v"), f64("x"), f64("v"), f64("fe"), M, S,
                             f64("y"), f64("z"))
    x, it, err = so.solve_cg(pA, pb, int(g["cg_max"]), float(g["cg_tol"]))
    assert it == int(g["ref64_cg_iterations"])
    assert rel(x, g["ref64_cg_x"]) < 1e-10
    assert abs(err - float(g["ref64_cg_error"])) <= 1e-8 * float(g["ref64_cg_error"])
    xb, vb, itb, errb = so.solve_be_one(n, h, dfdx, dfdv, f64("f"), f64("x"), f64("v"), f64("fe"), M, S, f64("y"),
                                        f64("z"), int(g["cg_max"]), float(g["cg_tol"]))
    assert itb == int(g["ref64_be_max_sub"]) == int(g["ref64_be_min_sub"])
    # one Newton iteration whose |dv|^2 is above the outer tolerance: the loop counts it and ends
    # at maxIterations (sparse_force_solver.cpp:205-228)
    assert int(g["ref64_be_iterations"]) == 1
    assert rel(xb, g["ref64_be_x"]) < 1e-12
    assert rel(vb, g["ref64_be_v"]) < 1e-10
    assert abs(errb - float(g["ref64_be_error"])) <= 1e-9 * float(g["ref64_be_error"])
    # the reference's float build: same iteration counts within a few, same solution to float noise
    assert abs(int(g["ref32_cg_iterations"]) - it) <= 3
    assert rel(g["ref32_cg_x"], x) < 1e-3
