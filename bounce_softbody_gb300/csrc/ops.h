// Host-callable launchers of the per-op kernels (kernels.cu) and of the persistent batch
// kernel (persistent.cu).
#pragma once

#include "internal.h"

#include <cuda_runtime.h>

// Threads per CTA of the batch kernel's team launches (the PCG launch and the team assembly).
// On the 512-body batch with every body on a cluster, 256-thread CTAs at 4 per SM (clusters of
// 8) measured 1 % faster than 512-thread CTAs at 2 per SM (clusters of 4); with small bodies on
// single CTAs it was the other way round.
#ifndef B3G_PCG_THREADS
#define B3G_PCG_THREADS 256
#endif

namespace b3g {

// Storage / arithmetic of the PCG: matrix storage type and vector type.
enum Prec
{
	kP32 = 0,   // float blocks, float vectors, double dot products
	kP64 = 1,   // double blocks and vectors
	kPBF = 2    // bf16 blocks in the iteration, float blocks for the residual refresh, float vectors
};

struct StepParamsHost
{
	float h;
	int first_newton;
};

cudaError_t op_begin(const DevBody& B, cudaStream_t st, int max_it, double tol2, int refresh, double newton_tol2);
cudaError_t op_newton_begin(const DevBody& B, cudaStream_t st);
cudaError_t op_elements(const DevBody& B, const StepParamsHost& P, cudaStream_t st);
cudaError_t op_assemble(const DevBody& B, const StepParamsHost& P, int prec, bool init, cudaStream_t st);
// filtered contacts: contact update and per-vertex constraints (B.filt) at the start of a step
cudaError_t op_contact_filter(const DevBody& B, float h, cudaStream_t st);
cudaError_t op_pcg_init(const DevBody& B, int prec, cudaStream_t st);
// iteration j (0-based) of the current solve; refresh = the true-residual refresh period
cudaError_t op_pcg_iteration(const DevBody& B, int prec, int j, int refresh, cudaStream_t st);
// Iterations of j that launch the true-residual refresh kernel (bit k: iteration j0 + k) for a
// chunk of `count` iterations from j0; and the launch geometry of the iteration kernels computed
// once outside any stream capture.
unsigned pcg_resid_mask(int prec, int j0, int count, int refresh);
void op_pcg_prime(const DevBody& B, int prec);
// BF16 mode of the per-op step: a flexible CG (Notay's FCG with one stored direction) on the FP32
// blocks whose preconditioner is an inner Jacobi-PCG solve with the BF16 blocks.
//   Bin: the inner solve's view (pb = the outer residual, py = z, its own r s d d2 q and scalars,
//        no float-float solution); inner_begin starts it (max_it iterations, tolerance tol2) unless
//        the outer solve is done (outer_sc), inner_iteration runs iteration j.
//   Bo:  the outer view of outer iteration k (d = p_prev, d2 = p, q = q of this iteration), z the
//        inner solution, q_prev the previous iteration's q: p = z - (z.q_prev / p_prev.q_prev)
//        p_prev, q = A p, alpha = p.r / p.q, then the body step's update and true-residual refresh.
cudaError_t op_fcg_inner_begin(const DevBody& Bin, const Scalars* outer_sc, int max_it, double tol2, cudaStream_t st);
cudaError_t op_fcg_inner_iteration(const DevBody& Bin, int j, cudaStream_t st);
cudaError_t op_fcg_outer(const DevBody& Bo, const float* z, const float* q_prev, FcgScalars* f, double* part, int k,
                         cudaStream_t st);
// mode 0: write the Newton iterate (xi, vi); mode 1: write the state and finish the step
cudaError_t op_final(const DevBody& B, const StepParamsHost& P, int prec, int mode, cudaStream_t st);
// finish a multi-Newton step: iterate -> state, friction, clear, new contacts
cudaError_t op_post(const DevBody& B, float h, cudaStream_t st);
// dt <= 0: no solve, only contact bookkeeping and clearing (body.cpp:552-604)
cudaError_t op_nostep(const DevBody& B, cudaStream_t st);
// clear a float array on the device
cudaError_t op_fill_f32(float* p, size_t count, float value, cudaStream_t st);

// One body of a batched host transfer: its state arrays and its place in the flat host array.
struct XferBody
{
	float* x;
	float* v;
	float* fext;
	unsigned long long off;  // first float of the body in the flat array
	unsigned n3;             // 3 * vertices
	unsigned pad;
};
// fext of every body += src[off .. off + n3) (one launch for the whole batch)
cudaError_t op_batch_scatter_add(const XferBody* table, uint32_t count, uint32_t max_n3, const float* src,
                                 cudaStream_t st);
// dst_x / dst_v[off .. off + n3) = x / v of every body (either may be null)
cudaError_t op_batch_gather(const XferBody* table, uint32_t count, uint32_t max_n3, float* dst_x, float* dst_v,
                            cudaStream_t st);
// Closest triangle-fixture hit of `count` segments (6 floats each, device): keys[r] (device,
// count entries) is reduced to fraction bits << 32 | triangle, then decoded into hits (device).
cudaError_t op_ray_cast(const DevBody& B, int ntri, const float* segments, uint32_t count, unsigned long long* keys,
                        b3g_ray_hit* hits, cudaStream_t st);

// Persistent batch kernel: every body listed in `big` (teams of `cluster` CTAs) and in `small`
// (one CTA each) steps `steps` times in one launch.
struct BatchArgs
{
	const DevBody* bodies;   // device array of all bodies of the batch
	const int* big;          // device array: indices of bodies stepped by whole clusters
	int nbig;
	const int* small;        // device array: indices of bodies stepped by single CTAs
	int nsmall;
	unsigned* queue;         // device: four work counters (two per launch), cleared by op_batch
	int steps;
	float h;
	int newton;
	int max_iter;
	double tol2;
	int refresh;
	double newton_tol2;
	int prec;
	int cluster;             // CTAs per cluster: 1, 2, 4 or 8
	int ctas;                // CTAs of the launch (multiple of cluster)
	unsigned long long* prof; // optional phase cycle counters (8 per CTA), null = off
	int part = 0;            // single-Newton steps: 0 both launches, 1 assembly only, 2 PCG only
	cudaEvent_t ev_rows = nullptr;  // if set, recorded between the element and the row launches
	// single-Newton steps: the elements, then the rows, of all bodies in two flat launches before
	// the PCG launch. elem_off[k] / slice_off[k]: first element / row slice of bodies[k] in the
	// flat numbering (count + 1 entries each; elements of a body: tetrahedra, triangles, springs,
	// stretch/shear triangles, mouse springs). Null = the team launches do both, as for several
	// Newton iterations.
	const unsigned* elem_off = nullptr;
	const unsigned* slice_off = nullptr;
	unsigned nelem = 0;
	unsigned nslices = 0;
	int nbodies = 0;
	int tets_only = 0;       // every body has tetrahedra only and no contact spheres
	int filter = 0;          // filtered contacts: bodies with a filt buffer; their vertices follow
	                         // their elements in the flat element numbering
	// Split assembly (side stream set): bodies below the flat element offset elem_mid (slice
	// offset slice_mid) form group 1, the rest group 2; group 2's elements run on `side`,
	// forked and joined through ev_fork / ev_join, concurrently with group 1's rows. CTAs per SM
	// of the element and row launches (0: their defaults).
	cudaStream_t side = nullptr;
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
	unsigned elem_mid = 0, slice_mid = 0;
	int split_elem_per_sm = 0, split_rows_per_sm = 0;
};
cudaError_t op_batch(const BatchArgs& A, cudaStream_t st);
// Co-resident clusters of the batch kernel for this precision and cluster size (0 on error).
int batch_max_clusters(int prec, int cluster);

} // namespace b3g
