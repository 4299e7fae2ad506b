/*
 * b3g sparse containers and solvers: the reference's integrator seam on the GPU.
 *
 * Device-resident counterparts of the reference's value types and solvers (paths inside the
 * reference project):
 *   b3g_dense_vec3    b3DenseVec3   include/bounce_softbody/sparse/dense_vec3.h:24-208
 *   b3g_diag_mat33    b3DiagMat33   include/bounce_softbody/sparse/diag_mat33.h:27-190
 *   b3g_sparse_mat33  b3SparseMat33 include/bounce_softbody/sparse/sparse_mat33.h:94-646
 *   b3g_sparse_solve_cg   b3SparseSolveCG  include/bounce_softbody/sparse/sparse_solver.h:28-47
 *                                          (src/bounce_softbody/sparse/sparse_solver.cpp:28-109)
 *   b3g_sparse_solve_be   b3SparseSolveBE  include/bounce_softbody/sparse/sparse_force_solver.h:52-97
 *                                          (src/bounce_softbody/sparse/sparse_force_solver.cpp:104-232)
 *   b3g_sparse_force_model b3SparseForceModel sparse_force_solver.h:31-49
 *
 * Every container belongs to one context and lives on its device; operations are ordered on the
 * context's stream and are asynchronous unless they return a value to the host (get, dot,
 * export, solver outputs), which makes them wait. Host arrays of blocks hold 9 floats per block in
 * b3Mat33 order (column-major: column x, then y, then z, so entry (r, c) is at 3 c + r); host
 * arrays of vectors hold 3 floats per entry like b3Vec3 arrays.
 *
 * Element writes of a force model ("(*dfdx)(i, j) += K", "(*f)[i] += g") are b3g_*_add_* calls:
 * they queue on the host and are applied on the device, in call order per entry, by the next
 * operation that reads the container. A sparse matrix stores the diagonal block of every row (a
 * zero block when never written); an empty matrix (no write yet) has no blocks at all.
 * An output container may be one of the operands.
 */
#ifndef B3G_SPARSE_H
#define B3G_SPARSE_H

#include "b3g.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct b3g_dense_vec3 b3g_dense_vec3;
typedef struct b3g_diag_mat33 b3g_diag_mat33;
typedef struct b3g_sparse_mat33 b3g_sparse_mat33;

/* ---------------------------------------------------------------- b3DenseVec3 (dense_vec3.h) */
/* b3DenseVec3(n), zero-filled. */
B3G_API int b3g_dense_vec3_create(b3g_context* ctx, uint32_t n, b3g_dense_vec3** out);
B3G_API int b3g_dense_vec3_destroy(b3g_dense_vec3* v);
B3G_API int b3g_dense_vec3_size(const b3g_dense_vec3* v, uint32_t* n);
/* Whole-vector host transfers (3 n floats). */
B3G_API int b3g_dense_vec3_set(b3g_dense_vec3* v, const float* xyz);
B3G_API int b3g_dense_vec3_get(b3g_dense_vec3* v, float* xyz);
/* SetZero (dense_vec3.h:86). */
B3G_API int b3g_dense_vec3_set_zero(b3g_dense_vec3* v);
/* operator= / Copy (dense_vec3.h:57-84). */
B3G_API int b3g_dense_vec3_copy(b3g_dense_vec3* out, const b3g_dense_vec3* a);
/* b3Add, b3Sub, b3Mul(out, s, v), b3Negate (dense_vec3.h:116-150). */
B3G_API int b3g_dense_vec3_add(b3g_dense_vec3* out, const b3g_dense_vec3* a, const b3g_dense_vec3* b);
B3G_API int b3g_dense_vec3_sub(b3g_dense_vec3* out, const b3g_dense_vec3* a, const b3g_dense_vec3* b);
B3G_API int b3g_dense_vec3_scale(b3g_dense_vec3* out, float s, const b3g_dense_vec3* a);
B3G_API int b3g_dense_vec3_negate(b3g_dense_vec3* out, const b3g_dense_vec3* a);
/* b3Dot and b3LengthSquared (dense_vec3.h:151-175): each entry's three-component term in float,
 * the terms summed in FP64 in a fixed order (deterministic); waits. */
B3G_API int b3g_dense_vec3_dot(const b3g_dense_vec3* a, const b3g_dense_vec3* b, double* out);
B3G_API int b3g_dense_vec3_length_squared(const b3g_dense_vec3* a, double* out);
/* operator[] writes: v[index[k]] += values[3k..3k+2] (add) or = (set), in call order. */
B3G_API int b3g_dense_vec3_add_values(b3g_dense_vec3* v, uint32_t count, const uint32_t* index, const float* values);
B3G_API int b3g_dense_vec3_set_values(b3g_dense_vec3* v, uint32_t count, const uint32_t* index, const float* values);
/* The device array behind the vector (4 floats per entry: x, y, z, unused), for callers that
 * write it with their own kernels on the context's stream; queued writes are applied first. */
B3G_API int b3g_dense_vec3_device(b3g_dense_vec3* v, void** device_ptr);

/* ---------------------------------------------------------------- b3DiagMat33 (diag_mat33.h) */
B3G_API int b3g_diag_mat33_create(b3g_context* ctx, uint32_t n, b3g_diag_mat33** out);
B3G_API int b3g_diag_mat33_destroy(b3g_diag_mat33* m);
B3G_API int b3g_diag_mat33_size(const b3g_diag_mat33* m, uint32_t* n);
/* Whole-matrix host transfers (9 n floats, b3Mat33 order). */
B3G_API int b3g_diag_mat33_set(b3g_diag_mat33* m, const float* blocks);
B3G_API int b3g_diag_mat33_get(b3g_diag_mat33* m, float* blocks);
/* SetZero, SetIdentity (diag_mat33.h:89-107), operator= / Copy. */
B3G_API int b3g_diag_mat33_set_zero(b3g_diag_mat33* m);
B3G_API int b3g_diag_mat33_set_identity(b3g_diag_mat33* m);
B3G_API int b3g_diag_mat33_copy(b3g_diag_mat33* out, const b3g_diag_mat33* a);
/* b3Transpose, b3Add, b3Sub, b3Mul(out, s, A), b3Negate (diag_mat33.h:109-162). */
B3G_API int b3g_diag_mat33_transpose(b3g_diag_mat33* out, const b3g_diag_mat33* a);
B3G_API int b3g_diag_mat33_add(b3g_diag_mat33* out, const b3g_diag_mat33* a, const b3g_diag_mat33* b);
B3G_API int b3g_diag_mat33_sub(b3g_diag_mat33* out, const b3g_diag_mat33* a, const b3g_diag_mat33* b);
B3G_API int b3g_diag_mat33_scale(b3g_diag_mat33* out, float s, const b3g_diag_mat33* a);
B3G_API int b3g_diag_mat33_negate(b3g_diag_mat33* out, const b3g_diag_mat33* a);
/* b3Mul(b3DenseVec3& out, const b3DiagMat33& A, const b3DenseVec3& v) (diag_mat33.h:149). */
B3G_API int b3g_diag_mat33_mul_vec(b3g_dense_vec3* out, const b3g_diag_mat33* a, const b3g_dense_vec3* v);

/* ---------------------------------------------------------------- b3SparseMat33 (sparse_mat33.h) */
/* b3SparseMat33(n): n x n blocks, no entries. */
B3G_API int b3g_sparse_mat33_create(b3g_context* ctx, uint32_t n, b3g_sparse_mat33** out);
B3G_API int b3g_sparse_mat33_destroy(b3g_sparse_mat33* m);
/* Rows (rowCount) and stored blocks (the diagonal of every row included once any block exists). */
B3G_API int b3g_sparse_mat33_size(b3g_sparse_mat33* m, uint32_t* n, uint64_t* blocks);
/* operator()(i, j) += / = block (sparse_mat33.h:268-288) for `count` blocks, in call order:
 * rows[k], cols[k], blocks + 9 k. An absent (i, j) is created, as operator() creates it. */
B3G_API int b3g_sparse_mat33_add_blocks(b3g_sparse_mat33* m, uint32_t count, const uint32_t* rows,
                                        const uint32_t* cols, const float* blocks);
B3G_API int b3g_sparse_mat33_set_blocks(b3g_sparse_mat33* m, uint32_t count, const uint32_t* rows,
                                        const uint32_t* cols, const float* blocks);
/* operator()(i, j) const (sparse_mat33.h:258): the block, zero when absent; waits. */
B3G_API int b3g_sparse_mat33_get_block(b3g_sparse_mat33* m, uint32_t i, uint32_t j, float block[9]);
/* Every stored block as CSR with ascending columns per row: row_ptr (n + 1 entries), cols and
 * blocks (9 floats each) for at most `capacity` blocks; *count receives the number of blocks
 * (B3G_ERROR_INVALID_ARGUMENT when it exceeds capacity). Waits. */
B3G_API int b3g_sparse_mat33_export(b3g_sparse_mat33* m, uint32_t* row_ptr, uint32_t* cols, float* blocks,
                                    uint64_t capacity, uint64_t* count);
/* CreateMatrix (sparse_mat33.h:418-450): the dense (3n x 3n) matrix, column-major; waits. */
B3G_API int b3g_sparse_mat33_to_dense(b3g_sparse_mat33* m, float* out);
/* Destroy + b3SparseMat33(n): remove every block. */
B3G_API int b3g_sparse_mat33_clear(b3g_sparse_mat33* m);
/* Every stored block set to zero, the blocks kept (equal to clear for every product and sum). */
B3G_API int b3g_sparse_mat33_zero_values(b3g_sparse_mat33* m);
/* operator= / Copy (sparse_mat33.h:188-230). */
B3G_API int b3g_sparse_mat33_copy(b3g_sparse_mat33* out, const b3g_sparse_mat33* a);
/* b3Add / b3Sub (sparse_mat33.h:452-462): out = a +- b over the union of their blocks. */
B3G_API int b3g_sparse_mat33_add(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_sparse_mat33* b);
B3G_API int b3g_sparse_mat33_sub(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_sparse_mat33* b);
/* b3Add / b3Sub with a diagonal (sparse_mat33.h:464-492): out = a + d, a - d, d + a, and
 * b3Sub(out, d, b): the diagonal of `out` is set to d (its other blocks are kept) and b is
 * subtracted, as the reference does. */
B3G_API int b3g_sparse_mat33_add_diag(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d);
B3G_API int b3g_sparse_mat33_sub_diag(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d);
B3G_API int b3g_sparse_mat33_diag_add(b3g_sparse_mat33* out, const b3g_diag_mat33* d, const b3g_sparse_mat33* a);
B3G_API int b3g_sparse_mat33_diag_sub(b3g_sparse_mat33* out, const b3g_diag_mat33* d, const b3g_sparse_mat33* b);
/* b3Mul(out, s, B) (sparse_mat33.h:514-533): out = s B; for s == 0 the reference returns before
 * touching `out`, and so does this call. */
B3G_API int b3g_sparse_mat33_scale(b3g_sparse_mat33* out, float s, const b3g_sparse_mat33* b);
/* b3Mul(out, D, B) = D_i B_ij and b3Mul(out, A, D) = A_ij D_j (sparse_mat33.h:535-576). */
B3G_API int b3g_sparse_mat33_diag_mul(b3g_sparse_mat33* out, const b3g_diag_mat33* d, const b3g_sparse_mat33* b);
B3G_API int b3g_sparse_mat33_mul_diag(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d);
/* b3Mul(b3DenseVec3& out, const b3SparseMat33& A, const b3DenseVec3& v) (sparse_mat33.h:494-512):
 * the SpMV, one warp per 32 block rows, 16-byte block and column loads. out must not be v. */
B3G_API int b3g_sparse_mat33_mul_vec(b3g_dense_vec3* out, b3g_sparse_mat33* a, const b3g_dense_vec3* v);

/* ---------------------------------------------------------------- b3SparseSolveCG (sparse_solver.h) */
/* b3SolveCGInput / b3SolveCGOutput. */
typedef struct b3g_solve_cg_input
{
	b3g_sparse_mat33* A;           /* A in A x = b (positive definite) */
	const b3g_dense_vec3* b;
	uint32_t max_iterations;
	float tolerance;               /* stop when r.M^-1.r <= tolerance^2 r0.M^-1.r0 */
} b3g_solve_cg_input;

typedef struct b3g_solve_cg_output
{
	b3g_dense_vec3* x;             /* solution; holds the initial guess on entry */
	uint32_t iterations;
	double error;                  /* r.M^-1.r at exit (the reference's delta_new) */
	int32_t status;                /* b3g_solve_status (the reference always returns true) */
} b3g_solve_cg_output;

/* Jacobi-preconditioned CG exactly as the reference runs it (scalar Jacobi from the diagonal
 * entries of each diagonal block, exit test at the loop top, true residual recomputed when
 * iteration % 50 == 0), FP32 vectors and blocks with FP64 sums of the dot products, as
 * hand-written kernels on the context's stream. Waits. */
B3G_API int b3g_sparse_solve_cg(b3g_solve_cg_output* output, const b3g_solve_cg_input* input);

/* ---------------------------------------------------------------- b3SparseSolveBE (sparse_force_solver.h) */
/* b3SparseForceSolverData: what a force model receives. x and v are the Newton iterate (read them
 * with b3g_dense_vec3_get or on the device); f, dfdx and dfdv start empty (zero) in every Newton
 * iteration and collect the model's writes. */
typedef struct b3g_sparse_force_solver_data
{
	float h, inv_h;
	b3g_dense_vec3* x;
	b3g_dense_vec3* v;
	b3g_dense_vec3* f;
	b3g_sparse_mat33* dfdx;
	b3g_sparse_mat33* dfdv;
} b3g_sparse_force_solver_data;

/* b3SparseForceModel::ApplyForces as a C callback: called on the host thread that called
 * b3g_sparse_solve_be, once per Newton iteration. */
typedef void (*b3g_apply_forces_fn)(void* user, const b3g_sparse_force_solver_data* data);

typedef struct b3g_sparse_force_model
{
	b3g_apply_forces_fn apply_forces;
	void* user;
} b3g_sparse_force_model;

/* b3SolveBEInput (sparse_force_solver.h:52-82). */
typedef struct b3g_solve_be_input
{
	float h, inv_h;
	b3g_sparse_force_model force_model;
	uint32_t dof_count;
	const b3g_dense_vec3* x0;      /* x(t) */
	const b3g_dense_vec3* v0;      /* v(t) */
	const b3g_dense_vec3* fe;      /* external forces over [t, t + h] */
	const b3g_diag_mat33* M;       /* mass matrix */
	const b3g_dense_vec3* y;       /* translation: x(t + h) += y */
	const b3g_diag_mat33* S;       /* constraint filter */
	const b3g_dense_vec3* z;       /* desired sub-solver solution (usually zero) */
	uint32_t max_iterations;       /* Newton iterations */
	float tolerance;               /* |dv|^2 <= tolerance^2 (|dv0|^2 after the first) */
	uint32_t max_sub_iterations;
	float sub_tolerance;
} b3g_solve_be_input;

/* b3SolveBEOutput (sparse_force_solver.h:84-94). min / max_sub_iterations are folded into the
 * values the caller sets (b3ForceSolver starts them at UINT32_MAX and 0). */
typedef struct b3g_solve_be_output
{
	b3g_dense_vec3* x;             /* x(t + h) */
	b3g_dense_vec3* v;             /* v(t + h) */
	uint32_t iterations;
	double error;
	uint32_t min_sub_iterations;
	uint32_t max_sub_iterations;
	int32_t status;                /* b3g_solve_status of the last PCG solve */
} b3g_solve_be_output;

/* Backward-Euler Newton loop of the reference: per iteration the force model fills f, dfdx and
 * dfdv; A = M - h dfdv - h^2 dfdx, b = M (v0 - v) + h (fe + f) + h dfdx (x0 - x + h v + y), the
 * pre-filter pA = S A S^T + I - S, pb = S (b - A z) (one fused kernel over the union of the two
 * matrices' blocks), then b3g_sparse_solve_cg's kernels from the previous solution (zeroed once
 * per call), v += dv = y' + z, x = x0 + h v + y. Waits. */
B3G_API int b3g_sparse_solve_be(b3g_solve_be_output* output, const b3g_solve_be_input* input);

#ifdef __cplusplus
}
#endif

#endif /* B3G_SPARSE_H */
