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
	for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < P.nelem; g += gridDim.x * blockDim.x)
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
			if (A.nelem > 0)
			{
				// the batch's elements are all tetrahedra when every body qualifies for the
				// tetrahedra-only row form
				if (P.tets_only)
					k_batch_elements<true><<<elem_grid(A.nelem, B3G_ELEM_TETS_MIN_BLOCKS), kElemThreads, 0, st>>>(P);
				else
					k_batch_elements<false><<<elem_grid(A.nelem, 3), kElemThreads, 0, st>>>(P);
			}
			e = cudaGetLastError();
			if (e == cudaSuccess && A.ev_rows) e = cudaEventRecord(A.ev_rows, st);
			if (e == cudaSuccess)
				e = A.prec == kP64 ? launch_rows_f64(P, st)
				                   : (A.prec == kPBF ? launch_rows_bf16(P, st) : launch_rows_f32(P, st));
			if (e != cudaSuccess || A.part == 1) return e;
		}
	}
	if (A.prec == kP64) return launch_batch_f64(P, A.cluster, A.ctas, A.part, st);
	if (A.prec == kPBF) return launch_batch_bf16(P, A.cluster, A.ctas, A.part, st);
	return launch_batch_f32(P, A.cluster, A.ctas, A.part, st);
}

} // namespace b3g
