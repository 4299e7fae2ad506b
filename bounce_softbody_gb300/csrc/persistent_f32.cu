// The persistent batch kernel instantiated for f32 matrix blocks (float blocks, float vectors).
#include "persistent.cuh"

namespace b3g {

cudaError_t launch_batch_f32(const BatchParams& P, int cluster, int ctas, int part, cudaStream_t st)
{
	return launch_prec<float, float>(P, cluster, ctas, 0, part, st);
}

cudaError_t launch_rows_f32(const BatchParams& P, cudaStream_t st) { return launch_rows<float, float>(P, st); }

int max_clusters_f32(int cluster) { return max_clusters_prec<float, float>(cluster); }

} // namespace b3g
