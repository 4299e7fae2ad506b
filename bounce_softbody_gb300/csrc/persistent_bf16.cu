// The persistent batch kernel instantiated for bf16 matrix blocks (__nv_bfloat16 blocks, float vectors).
#include "persistent.cuh"

namespace b3g {

cudaError_t launch_batch_bf16(const BatchParams& P, int cluster, int ctas, int part, cudaStream_t st)
{
	return launch_prec<__nv_bfloat16, float>(P, cluster, ctas, 1, part, st);
}

cudaError_t launch_rows_bf16(const BatchParams& P, cudaStream_t st) { return launch_rows<__nv_bfloat16, float>(P, st); }

int max_clusters_bf16(int cluster) { return max_clusters_prec<__nv_bfloat16, float>(cluster); }

} // namespace b3g
