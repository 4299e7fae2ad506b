// Dispatch of the persistent batch kernel (persistent.cuh) to its per-precision instantiations.
#include "persistent.cuh"

namespace b3g {

namespace {

constexpr int kTetThreads = 256;

// The tetrahedra of every body of a batch, first Newton iteration of a step, one per thread over
// a flat numbering (tet_off: first tetrahedron of each body). Separate from the team launch so
// that it runs at its own register budget (80, 3 CTAs per SM) instead of the 128 the row
// assembly needs: the rotation extraction's dependent chain wants the extra warps. The state it
// reads was written by earlier launches, so plain (L1) loads.
__global__ void __launch_bounds__(kTetThreads, 3)
k_batch_tets(const DevBody* __restrict__ bodies, const unsigned* __restrict__ tet_off, int nbodies, unsigned ntets,
             float h)
{
	StepParams sp;
	sp.h = h;
	sp.first_newton = 1;
	for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < ntets; g += gridDim.x * blockDim.x)
	{
		// the body whose range holds g: the last k with tet_off[k] <= g
		int lo = 0, hi = nbodies - 1;
		while (lo < hi)
		{
			const int mid = (lo + hi + 1) >> 1;
			if (__ldg(tet_off + mid) <= g) lo = mid;
			else hi = mid - 1;
		}
		tet_element<LdPlain>(bodies[lo], (int)(g - __ldg(tet_off + lo)), sp);
	}
}

int tet_grid(unsigned ntets)
{
	static const int cap = [] {
		int dev = 0, sms = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		return 3 * (sms > 0 ? sms : 1);
	}();
	const unsigned g = (ntets + kTetThreads - 1) / kTetThreads;
	return (int)(g < (unsigned)cap ? (g > 0 ? g : 1) : cap);
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
	P.tets_done = 0;
	if (A.part != 2)
	{
		// two counters per launch; the solve-only part reuses what the assembly part cleared
		cudaError_t e = cudaMemsetAsync(A.queue, 0, 4 * sizeof(unsigned), st);
		if (e != cudaSuccess) return e;
		if (P.newton == 1 && A.tet_off && A.ntets > 0)
		{
			k_batch_tets<<<tet_grid(A.ntets), kTetThreads, 0, st>>>(A.bodies, A.tet_off, A.nbodies, A.ntets, A.h);
			e = cudaGetLastError();
			if (e != cudaSuccess) return e;
			P.tets_done = 1;
		}
	}
	if (A.prec == kP64) return launch_batch_f64(P, A.cluster, A.ctas, A.part, st);
	if (A.prec == kPBF) return launch_batch_bf16(P, A.cluster, A.ctas, A.part, st);
	return launch_batch_f32(P, A.cluster, A.ctas, A.part, st);
}

} // namespace b3g
