"""The sparse container / solver boundary (include/b3g_sparse.h) through the C ABI, against the
reference's own outputs recorded in tests/golden/sparse_tet10.npz (the 10^3 block's Jacobians
after 10 steps, the reference's container operators, b3SparseSolveCG and b3SparseSolveBE).

Tolerances: products and sums of the FP32 containers within 2e-5 of the norm of the reference's
FP32 result (float rounding of differently ordered sums); the CG and backward-Euler solutions
within 20x the reference's own FP32-vs-FP64 distance (a solve stopped at 1e-5 amplifies
rounding by the condition number), PCG iterations within 3 of the reference's FP32 build."""
import os

import numpy as np
import pytest

from bounce_softbody_gb300 import b3g
from bounce_softbody_gb300.b3g_sparse import (DenseVec3, DiagMat33, SparseMat33, diag_op, solve_be, solve_cg,
                                              sp_op, vec_op)
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

PRODUCTS = ["A", "pA", "D_dfdx", "dfdx_D", "s_dfdx", "dfdx_plus_dfdv", "dfdx_minus_dfdv", "dfdx_plus_D",
            "D_minus_dfdx", "zero_dfdx"]
TOL = 2e-5


@pytest.fixture(scope="module")
def g():
    z = np.load(os.path.join(GOLDEN, "sparse_tet10.npz"))
    return {k: z[k] for k in z.files}


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def eye_blocks(scale):
    e = np.zeros((len(scale), 9), np.float32)
    e[:, 0] = e[:, 4] = e[:, 8] = scale
    return e


class Setup:
    def __init__(self, ctx, g):
        n = int(g["n"])
        self.n, self.h = n, float(g["h"])
        self.dfdx = SparseMat33(ctx, n)
        self.dfdx.add_blocks(g["dfdx_rows"], g["dfdx_cols"], g["dfdx_vals"])
        self.dfdv = SparseMat33(ctx, n)
        self.dfdv.add_blocks(g["dfdv_rows"], g["dfdv_cols"], g["dfdv_vals"])
        self.M = DiagMat33(ctx, n, eye_blocks(g["mass"]))
        self.S = DiagMat33(ctx, n, eye_blocks(g["dynamic"].astype(np.float32)))
        self.D = DiagMat33(ctx, n, g["D"])
        vec = lambda k: DenseVec3(ctx, n, g[k])  # noqa: E731
        self.x, self.v, self.f, self.fe = vec("x"), vec("v"), vec("f"), vec("fe")
        self.y, self.z, self.u = vec("y"), vec("z"), vec("u")
        self.ctx = ctx

    def new_vec(self):
        return DenseVec3(self.ctx, self.n)

    def new_sp(self):
        return SparseMat33(self.ctx, self.n)


def spmv(S, m):
    out = S.new_vec()
    sp_op("mul_vec", out, m, S.u)
    return out.get()


def system(S):
    """A, b, pA, pb built with the container operations, as sparse_force_solver.cpp:165-174 does."""
    h = S.h
    t1, A, t3 = S.new_sp(), S.new_sp(), S.new_sp()
    sp_op("scale", t1, h, S.dfdv)
    sp_op("diag_sub", A, S.M, t1)           # M - h dfdv (b3Sub(out, D, B) on a fresh out)
    sp_op("scale", t3, h * h, S.dfdx)
    sp_op("sub", A, A, t3)                  # - h^2 dfdx
    ST = DiagMat33(S.ctx, S.n)
    diag_op("transpose", ST, S.S)
    I = DiagMat33(S.ctx, S.n)
    diag_op("set_identity", I)
    pA = S.new_sp()
    sp_op("diag_mul", pA, S.S, A)
    sp_op("mul_diag", pA, pA, ST)
    sp_op("add_diag", pA, pA, I)
    sp_op("sub_diag", pA, pA, S.S)
    # b = M (v0 - v) + h (fe + f) + h dfdx (x0 - x + h v + y), here x = x0, v = v0
    dv, Mdv, ff, w, hv, q, b = (S.new_vec() for _ in range(7))
    vec_op("sub", dv, S.v, S.v)
    diag_op("mul_vec", Mdv, S.M, dv)
    vec_op("add", ff, S.fe, S.f)
    vec_op("scale", ff, h, ff)
    vec_op("sub", w, S.x, S.x)
    vec_op("scale", hv, h, S.v)
    vec_op("add", w, w, hv)
    vec_op("add", w, w, S.y)
    hdfdx = S.new_sp()
    sp_op("scale", hdfdx, h, S.dfdx)
    sp_op("mul_vec", q, hdfdx, w)
    vec_op("add", b, Mdv, ff)
    vec_op("add", b, b, q)
    Az, r, pb = S.new_vec(), S.new_vec(), S.new_vec()
    sp_op("mul_vec", Az, A, S.z)
    vec_op("sub", r, b, Az)
    diag_op("mul_vec", pb, S.S, r)
    return A, b, pA, pb


def test_container_products_match_reference(ctx, g):
    S = Setup(ctx, g)
    A, b, pA, pb = system(S)
    got = {"A": spmv(S, A), "pA": spmv(S, pA)}
    t = S.new_sp()
    sp_op("diag_mul", t, S.D, S.dfdx)
    got["D_dfdx"] = spmv(S, t)
    t = S.new_sp()
    sp_op("mul_diag", t, S.dfdx, S.D)
    got["dfdx_D"] = spmv(S, t)
    t = S.new_sp()
    sp_op("scale", t, float(g["s"]), S.dfdx)
    got["s_dfdx"] = spmv(S, t)
    t = S.new_sp()
    sp_op("add", t, S.dfdx, S.dfdv)
    got["dfdx_plus_dfdv"] = spmv(S, t)
    t = S.new_sp()
    sp_op("sub", t, S.dfdx, S.dfdv)
    got["dfdx_minus_dfdv"] = spmv(S, t)
    t = S.new_sp()
    sp_op("add_diag", t, S.dfdx, S.D)
    got["dfdx_plus_D"] = spmv(S, t)
    t = S.new_sp()
    sp_op("diag_sub", t, S.D, S.dfdx)
    got["D_minus_dfdx"] = spmv(S, t)
    t = S.new_sp()
    sp_op("scale", t, 0.0, S.dfdx)      # b3Mul with s = 0 leaves the fresh matrix empty
    assert t.size()[1] == 0
    got["zero_dfdx"] = spmv(S, t)
    for k, name in enumerate(PRODUCTS):
        ref = g["ref32_spmv"][k]
        if name == "zero_dfdx":
            assert not np.any(got[name]) and not np.any(ref)
            continue
        assert rel(got[name], ref) < TOL, (name, rel(got[name], ref))
        assert rel(got[name], g["ref64_spmv"][k]) < TOL, name
    assert rel(b.get(), g["ref32_b"]) < TOL
    assert rel(pb.get(), g["ref32_pb"]) < TOL
    du = S.new_vec()
    diag_op("mul_vec", du, S.D, S.u)
    assert rel(du.get(), g["ref32_diag_u"]) < 1e-6
    assert abs(S.u.dot(pb) - float(g["ref64_dot_u_pb"])) <= TOL * abs(float(g["ref64_dot_u_pb"]))
    assert abs(pb.length_squared() - float(g["ref64_len2_pb"])) <= TOL * float(g["ref64_len2_pb"])
    # pA's blocks: the reference's pattern exactly, its diagonal blocks to float rounding
    rp, cols, blk = pA.export()
    assert np.array_equal(rp, g["ref32_pA_row_ptr"]) and np.array_equal(cols, g["ref32_pA_cols"])
    diag = np.stack([blk[rp[i] + int(np.nonzero(cols[rp[i]:rp[i + 1]] == i)[0][0])] for i in range(S.n)])
    assert rel(diag, g["ref32_pA_diag"]) < 1e-6
    for i in (0, 17, 555, 999):
        assert np.allclose(pA.get_block(i, i), g["ref32_pA_diag"][i], rtol=1e-6, atol=1e-6 * np.abs(diag).max())
    # the dense export (CreateMatrix, column-major) agrees with the blocks
    dense = S.dfdx.to_dense()
    rr, cc, bb = S.dfdx.export()
    i = 7
    for k in range(rr[i], rr[i + 1]):
        j = cols_k = int(cc[k])
        np.testing.assert_array_equal(dense[3 * i:3 * i + 3, 3 * j:3 * j + 3], bb[k].reshape(3, 3).T)
        assert cols_k < S.n


def test_cg_matches_reference(ctx, g):
    S = Setup(ctx, g)
    _, _, pA, pb = system(S)
    x = S.new_vec()
    out = solve_cg(pA, pb, x, int(g["cg_max"]), float(g["cg_tol"]))
    floor = rel(g["ref32_cg_x"], g["ref64_cg_x"])
    assert abs(out["iterations"] - int(g["ref32_cg_iterations"])) <= 3
    assert out["status"] == "converged"
    assert rel(x.get(), g["ref64_cg_x"]) < max(1e-4, 20 * floor)
    # error is r.M^-1.r at exit, the reference's delta_new
    assert 0.0 < out["error"] <= 10 * float(g["ref32_cg_error"])


def test_be_with_replayed_force_model_matches_reference(ctx, g):
    S = Setup(ctx, g)
    calls = []

    def model(data):
        calls.append(data.h)
        data.dfdx.add_blocks(g["dfdx_rows"], g["dfdx_cols"], g["dfdx_vals"])
        data.dfdv.add_blocks(g["dfdv_rows"], g["dfdv_cols"], g["dfdv_vals"])
        data.f.add_values(np.arange(S.n), g["f"])
        # the model sees the Newton iterate: x = x0, v = v0 in the first iteration
        assert np.array_equal(data.x.get(), g["x"]) and np.array_equal(data.v.get(), g["v"])

    xo, vo = S.new_vec(), S.new_vec()
    out = solve_be(ctx, model, S.h, S.x, S.v, S.fe, S.M, S.y, S.S, S.z, xo, vo, max_iterations=1,
                   max_sub_iterations=int(g["cg_max"]), sub_tolerance=float(g["cg_tol"]))
    assert len(calls) == 1 and abs(calls[0] - S.h) < 1e-9
    assert out["iterations"] == int(g["ref32_be_iterations"]) == 1
    assert abs(out["max_sub"] - int(g["ref32_be_max_sub"])) <= 3 and out["min_sub"] == out["max_sub"]
    x64, v64 = g["ref64_be_x"], g["ref64_be_v"]
    fx = np.linalg.norm(g["ref32_be_x"].astype(np.float64) - x64) / np.linalg.norm(x64 - g["x"])
    fv = rel(g["ref32_be_v"], v64)
    x = xo.get()
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64 - g["x"]) < max(1e-4, 20 * fx)
    assert rel(vo.get(), v64) < max(1e-3, 20 * fv)
    assert out["error"] > 0.0 and abs(out["error"] - float(g["ref64_be_error"])) <= 1e-2 * float(g["ref64_be_error"])


def test_queued_writes_apply_in_call_order(ctx):
    """Repeated writes to one block or entry take effect in call order (add, set, add), and a new
    block grows the pattern without disturbing the others."""
    n = 40
    m = SparseMat33(ctx, n)
    rng = np.random.default_rng(3)
    b1, b2, b3 = (rng.normal(size=9).astype(np.float32) for _ in range(3))
    m.add_blocks([3, 3], [5, 5], np.stack([b1, b2]))
    m.add_blocks([3], [5], b3[None], op="set")
    m.add_blocks([3, 39], [5, 0], np.stack([b1, b2]))
    np.testing.assert_allclose(m.get_block(3, 5), b3 + b1, rtol=1e-6)
    np.testing.assert_array_equal(m.get_block(39, 0), b2)
    np.testing.assert_array_equal(m.get_block(0, 39), np.zeros(9, np.float32))
    n_rows, nb = m.size()
    assert n_rows == n and nb == n + 2  # the diagonal of every row plus the two written blocks
    v = DenseVec3(ctx, n)
    v.add_values([1, 1, 2], [[1, 2, 3], [10, 20, 30], [5, 5, 5]])
    v.add_values([1], [[7, 7, 7]], op="set")
    got = v.get()
    np.testing.assert_array_equal(got[1], [7, 7, 7])
    np.testing.assert_array_equal(got[2], [5, 5, 5])
    # SpMV of a random matrix against numpy (blocks are column-major b3Mat33)
    rows = rng.integers(0, n, 300)
    cols = rng.integers(0, n, 300)
    blocks = rng.normal(size=(300, 9)).astype(np.float32)
    a = SparseMat33(ctx, n)
    a.add_blocks(rows, cols, blocks)
    dense = np.zeros((3 * n, 3 * n))
    for r, c, b in zip(rows, cols, blocks.astype(np.float64)):
        dense[3 * r:3 * r + 3, 3 * c:3 * c + 3] += b.reshape(3, 3).T
    np.testing.assert_allclose(a.to_dense(), dense, rtol=1e-5, atol=1e-5)
    u = DenseVec3(ctx, n, rng.normal(size=(n, 3)))
    out = DenseVec3(ctx, n)
    sp_op("mul_vec", out, a, u)
    np.testing.assert_allclose(out.get().ravel(), dense @ u.get().ravel().astype(np.float64), rtol=1e-4, atol=1e-4)
    with pytest.raises(b3g.B3gError):
        sp_op("mul_vec", u, a, u)  # out must not be the input
    with pytest.raises(b3g.B3gError):
        a.add_blocks([n], [0], np.zeros((1, 9)))  # row outside the matrix


def test_edge_cases_and_errors(ctx):
    """Empty containers, mismatched sizes, aliasing, the reference's b3Sub(out, D, B) and s = 0
    quirks, a CG already converged, and a backward-Euler solve with a force model that writes
    nothing (free particles under gravity in closed form)."""
    # zero-sized containers work and do nothing
    e0 = DenseVec3(ctx, 0)
    m0 = SparseMat33(ctx, 0)
    out0 = DenseVec3(ctx, 0)
    sp_op("mul_vec", out0, m0, e0)
    assert e0.dot(e0) == 0.0 and m0.size() == (0, 0)
    # mismatched sizes are rejected
    a, b = DenseVec3(ctx, 4), DenseVec3(ctx, 5)
    with pytest.raises(b3g.B3gError):
        vec_op("add", a, a, b)
    with pytest.raises(b3g.B3gError):
        a.dot(b)
    # aliasing: out = a + out gives the sum
    rng = np.random.default_rng(1)
    va, vb = rng.normal(size=(4, 3)), rng.normal(size=(4, 3))
    a.set(va)
    c = DenseVec3(ctx, 4, vb)
    vec_op("add", c, a, c)
    np.testing.assert_allclose(c.get(), (va + vb).astype(np.float32), rtol=1e-6)
    # b3Sub(out, D, B) keeps out's other blocks and sets its diagonal to D
    n = 3
    eye9 = np.eye(3, dtype=np.float32).reshape(9)
    out = SparseMat33(ctx, n)
    blk = rng.normal(size=9).astype(np.float32)
    out.add_blocks([0], [2], blk[None])
    B = SparseMat33(ctx, n)
    bb = rng.normal(size=9).astype(np.float32)
    B.add_blocks([1], [1], bb[None])
    D = DiagMat33(ctx, n, np.tile(2.0 * eye9, (n, 1)))
    sp_op("diag_sub", out, D, B)
    np.testing.assert_array_equal(out.get_block(0, 2), blk)
    np.testing.assert_allclose(out.get_block(1, 1), 2.0 * eye9 - bb, rtol=1e-6)
    np.testing.assert_allclose(out.get_block(0, 0), 2.0 * eye9, rtol=1e-6)
    # b3Mul(out, 0, B) leaves out as it was
    before = out.export()
    sp_op("scale", out, 0.0, B)
    after = out.export()
    assert all(np.array_equal(x, y) for x, y in zip(before, after))
    # a CG whose right-hand side is zero stops at once
    I = SparseMat33(ctx, n)
    I.add_blocks(np.arange(n), np.arange(n), np.tile(eye9, (n, 1)))
    zb, x = DenseVec3(ctx, n), DenseVec3(ctx, n)
    res = solve_cg(I, zb, x, 10, 1e-5)
    assert res["iterations"] == 0 and not np.any(x.get())
    with pytest.raises(b3g.B3gError):
        solve_cg(I, zb, zb, 10, 1e-5)     # x must not be b
    with pytest.raises(b3g.B3gError):
        solve_cg(I, zb, x, 10, 1.5)       # tolerance outside (0, 1)
    # backward Euler with no internal forces: v = v0 + h g, x = x0 + h v (one PCG iteration)
    m, h, grav = 2.0, 1.0 / 60.0, np.array([0.0, -9.8, 0.0])
    x0 = DenseVec3(ctx, n, rng.normal(size=(n, 3)))
    v0 = DenseVec3(ctx, n, rng.normal(size=(n, 3)))
    fe = DenseVec3(ctx, n, np.tile(m * grav, (n, 1)))
    M = DiagMat33(ctx, n, np.tile(m * eye9, (n, 1)))
    S = DiagMat33(ctx, n, np.tile(eye9, (n, 1)))
    y, z = DenseVec3(ctx, n), DenseVec3(ctx, n)
    xo, vo = DenseVec3(ctx, n), DenseVec3(ctx, n)
    out = solve_be(ctx, lambda data: None, h, x0, v0, fe, M, y, S, z, xo, vo, max_iterations=1,
                   max_sub_iterations=20, sub_tolerance=1e-6)
    v_exp = v0.get().astype(np.float64) + h * grav
    np.testing.assert_allclose(vo.get(), v_exp, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(xo.get(), x0.get().astype(np.float64) + h * v_exp, rtol=1e-6, atol=1e-7)
    assert out["max_sub"] == 1 and out["status"] == "converged"
