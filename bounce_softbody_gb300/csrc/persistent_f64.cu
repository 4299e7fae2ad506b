// The persistent batch kernel instantiated for f64 matrix blocks (double blocks, double vectors).
#include "persistent.cuh"

namespace b3g {

cudaError_t launch_batch_f64(const BatchParams& P, int cluster, int ctas, int part, cudaStream_t st)
{
	return launch_prec<double, double>(P, cluster, ctas, 0, part, st);
}

cudaError_t launch_rows_f64(const BatchParams& P, cudaStream_t st) { return launch_rows<double, double>(P, st); }

int max_clusters_f64(int cluster) { return max_clusters_prec<double, double>(cluster); }

} // namespace b3g
