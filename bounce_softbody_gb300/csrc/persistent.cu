// Dispatch of the persistent batch kernel (persistent.cuh) to its per-precision instantiations.
#include "persistent.cuh"

namespace b3g {

namespace {

constexpr int kElemThreads = 256;

// The elements of every body of a batch (tetrahedra, triangles, springs, stretch / shear
// triangles, mouse springs, then the vertices of bodies with filtered contacts; first Newton
// iteration of a step), one per thread over a flat
// numbering (elem_off: first element of each body). Its own launch runs at its own register
// budget (3 CTAs per SM) instead of the 128 registers the row assembly needs: the tetrahedra's
// rotation extraction, a dependent chain, wants the extra warps. The state it reads was written
// by earlier launches, so plain (L1) loads. TETS: every body has tetrahedra only (and no filtered
// contacts), so only the tetrahedron code is compiled, which fits four CTAs per SM.
#ifndef B3G_ELEM_TETS_MIN_BLOCKS
#define B3G_ELEM_TETS_MIN_BLOCKS 4
#endif
template <bool TETS>
__global__ void __launch_bounds__(kElemThreads, TETS ? B3G_ELEM_TETS_MIN_BLOCKS : 3) k_batch_elements(BatchParams P)
{
	StepParams sp;
	sp.h = P.h;
	sp.first_newton = 1;
	for (unsigned g = P.g_begin + blockIdx.x * blockDim.x + threadIdx.x; g < P.nelem; g += gridDim.x * blockDim.x)
	{
		const int b = flat_body(P.elem_off, P.nbodies, g);
		const DevBody& B = P.bodies[b];
		int e = (int)(g - __ldg(P.elem_off + b));
		if (TETS || e < B.nt)
		{
			tet_element<LdPlain>(B, e, sp);
			continue;
		}
		e -= B.nt;
		if (e < B.ntr)
		{
			tri_element<LdPlain>(B, e, sp);
			continue;
		}
		e -= B.ntr;
		if (e < B.ns)
		{
			spring_element<LdPlain>(B, e, sp);
			continue;
		}
		e -= B.ns;
		if (e < B.nbw)
		{
			bw_element<LdPlain>(B, e, sp);
			continue;
		}
		e -= B.nbw;
		if (e < B.nms)
		{
			mouse_element<LdPlain>(B, e, sp);
			continue;
		}
		// filtered contacts: the body's vertices follow its elements in the numbering; the
		// contact update and each vertex's constraint at the step's start (no element reads them)
		contact_filter_vertex(B, e - B.nms, P.h);
	}
}

int elem_grid(unsigned nelem, int per_sm)
{
	static const int sms = [] {
		int dev = 0, n = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
		return n > 0 ? n : 1;
	}();
	const unsigned cap = (unsigned)(per_sm * sms);
	const unsigned g = (nelem + kElemThreads - 1) / kElemThreads;
	return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

} // namespace

int batch_max_clusters(int prec, int cluster)
{
	if (prec == kP64) return max_clusters_f64(cluster);
	if (prec == kPBF) return max_clusters_bf16(cluster);
	return max_clusters_f32(cluster);
}

cudaError_t op_batch(const BatchArgs& A, cudaStream_t st)
{
	BatchParams P;
	P.bodies = A.bodies;
	P.big = A.big;
	P.nbig = A.nbig;
	P.small = A.small;
	P.nsmall = A.nsmall;
	P.queue = A.queue;
	P.steps = A.steps;
	P.h = A.h;
	P.newton = A.newton < 1 ? 1 : A.newton;
	P.max_iter = A.max_iter;
	P.tol2 = A.tol2;
	P.refresh = A.refresh;
	P.newton_tol2 = A.newton_tol2;
	P.prof = A.prof;
	P.elem_off = A.elem_off;
	P.slice_off = A.slice_off;
	P.nelem = A.nelem;
	P.nslices = A.nslices;
	P.nbodies = A.nbodies;
	P.tets_only = A.tets_only;
	P.filter = A.filter;
	P.g_begin = 0;
	P.s_begin = 0;
	P.rows_per_sm = 0;
	// a single Newton iteration with the flat numbering: elements and rows in two flat launches,
	// then the PCG launch (which knows from `flat` to sum delta0 itself)
	P.flat = (P.newton == 1 && A.elem_off && A.slice_off && A.nslices > 0) ? 1 : 0;
	if (A.part != 2)
	{
		// two counters per launch; the solve-only part reuses what the assembly part cleared
		cudaError_t e = cudaMemsetAsync(A.queue, 0, 4 * sizeof(unsigned), st);
		if (e != cudaSuccess) return e;
		if (P.flat)
		{
			// the batch's elements are all tetrahedra when every body qualifies for the
			// tetrahedra-only row form
			auto elements = [&](const BatchParams& Q, int per_sm, cudaStream_t s) -> cudaError_t {
				const unsigned count = Q.nelem - Q.g_begin;
				if (count == 0) return cudaSuccess;
				if (Q.tets_only)
					k_batch_elements<true><<<elem_grid(count, per_sm > 0 ? per_sm : B3G_ELEM_TETS_MIN_BLOCKS), kElemThreads, 0, s>>>(Q);
				else
					k_batch_elements<false><<<elem_grid(count, per_sm > 0 ? per_sm : 3), kElemThreads, 0, s>>>(Q);
				return cudaGetLastError();
			};
			auto rows = [&](const BatchParams& Q, cudaStream_t s) -> cudaError_t {
				return A.prec == kP64 ? launch_rows_f64(Q, s) : (A.prec == kPBF ? launch_rows_bf16(Q, s) : launch_rows_f32(Q, s));
			};
			if (A.side && A.elem_mid > 0 && A.elem_mid < A.nelem && A.slice_mid > 0 && A.slice_mid < A.nslices)
			{
				// two body groups: group 1's elements alone, then group 2's elements on the side
				// stream while group 1's rows run here (an ALU-bound and a latency-bound launch
				// sharing the SMs), then group 2's rows
				BatchParams E1 = P, E2 = P, R1 = P, R2 = P;
				E1.nelem = A.elem_mid;
				E2.g_begin = A.elem_mid;
				R1.nslices = A.slice_mid;
				R2.s_begin = A.slice_mid;
				R1.rows_per_sm = A.split_rows_per_sm;
				e = elements(E1, 0, st);
				if (e == cudaSuccess) e = cudaEventRecord(A.ev_fork, st);
				if (e == cudaSuccess) e = cudaStreamWaitEvent(A.side, A.ev_fork, 0);
				if (e == cudaSuccess) e = elements(E2, A.split_elem_per_sm, A.side);
				if (e == cudaSuccess) e = cudaEventRecord(A.ev_join, A.side);
				if (e == cudaSuccess) e = rows(R1, st);
				if (e == cudaSuccess) e = cudaStreamWaitEvent(st, A.ev_join, 0);
				if (e == cudaSuccess) e = rows(R2, st);
			}
			else
			{
				e = elements(P, 0, st);
				if (e == cudaSuccess && A.ev_rows) e = cudaEventRecord(A.ev_rows, st);
				if (e == cudaSuccess) e = rows(P, st);
			}
			if (e != cudaSuccess || A.part == 1) return e;
		}
	}
	if (A.prec == kP64) return launch_batch_f64(P, A.cluster, A.ctas, A.part, st);
	if (A.prec == kPBF) return launch_batch_bf16(P, A.cluster, A.ctas, A.part, st);
	return launch_batch_f32(P, A.cluster, A.ctas, A.part, st);
}

} // namespace b3g
