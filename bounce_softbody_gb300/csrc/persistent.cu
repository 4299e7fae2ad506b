// Dispatch of the persistent batch kernel (persistent.cuh) to its per-precision instantiations.
#include "persistent.cuh"

namespace b3g {

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
	if (A.part != 2)
	{
		// two counters per launch; the solve-only part reuses what the assembly part cleared
		cudaError_t e = cudaMemsetAsync(A.queue, 0, 4 * sizeof(unsigned), st);
		if (e != cudaSuccess) return e;
	}
	if (A.prec == kP64) return launch_batch_f64(P, A.cluster, A.ctas, A.part, st);
	if (A.prec == kPBF) return launch_batch_bf16(P, A.cluster, A.ctas, A.part, st);
	return launch_batch_f32(P, A.cluster, A.ctas, A.part, st);
}

} // namespace b3g
