// The reference's sparse value types and solvers on the GPU (include/b3g_sparse.h):
// b3DenseVec3, b3DiagMat33, b3SparseMat33 with their operator sets, b3SparseSolveCG and
// b3SparseSolveBE with the b3SparseForceModel seam.
//
// Layouts (the same as a body's, internal.h): a sparse matrix is sliced block-ELL with 32 rows
// per slice (one warp per slice, one lane per block row, the diagonal block first in each row,
// 9 value planes p = 3 row + col); a dense vector is 4 floats per entry; a diagonal matrix is 9
// planes of n floats. The block pattern is kept on the host (rows of column ids) and changes
// only when a write names a new (i, j) or an operation needs the union of two patterns; values
// live on the device only. Writes queued by the add / set calls are applied on the device in
// call order per entry (one thread per written block, its writes in order), so results do not
// depend on thread scheduling. The CG reuses the per-op PCG kernels of the body step
// (kernels.cu) on this layout.
#include "api_internal.h"
#include "device.cuh"
#include "../../include/b3g_sparse.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <numeric>
#include <utility>
#include <vector>

using namespace b3g;

namespace b3g {

struct SparseObject
{
	b3g_context* ctx = nullptr;
	virtual ~SparseObject() {}
	virtual void release_device() = 0;
};

} // namespace b3g

namespace {

constexpr int kT = 256;

int grid_of(size_t items, int per)
{
	size_t g = (items + per - 1) / per;
	if (g < 1) g = 1;
	if (g > 4096) g = 4096;
	return (int)g;
}

// A device buffer that only grows.
struct DevBuf
{
	void* p = nullptr;
	size_t bytes = 0;
	cudaError_t ensure(size_t need)
	{
		if (need <= bytes) return cudaSuccess;
		if (p) cudaFree(p);
		p = nullptr;
		bytes = 0;
		cudaError_t e = cudaMalloc(&p, need);
		if (e == cudaSuccess) bytes = need;
		return e;
	}
	void release()
	{
		if (p) cudaFree(p);
		p = nullptr;
		bytes = 0;
	}
};

std::atomic<uint64_t> g_pattern_ids(1);

// Block pattern of a sparse matrix: host rows (diagonal first, then ascending columns) and the
// SELL-32 slot layout on the device.
struct SpPattern
{
	int device = 0;
	uint32_t n = 0;
	std::vector<int> rp;     // n + 1
	std::vector<int> cols;   // per row: the diagonal, then the other columns ascending
	int nslices = 0;
	size_t nslots = 0;
	std::vector<int> slice_ptr;
	int* d_slice_ptr = nullptr;
	int* d_col = nullptr;
	uint64_t id = 0;

	~SpPattern()
	{
		if (d_slice_ptr || d_col)
		{
			cudaSetDevice(device);
			cudaFree(d_slice_ptr);
			cudaFree(d_col);
		}
	}
	size_t slot(int i, int k) const { return block_slot((size_t)slice_ptr[i >> 5], k, i & 31); }
	// position of column j in row i, -1 when absent
	int find(int i, int j) const
	{
		const int b = rp[i], e = rp[i + 1];
		if (b == e) return -1;
		if (j == i) return 0;
		const int* lo = cols.data() + b + 1;
		const int* hi = cols.data() + e;
		const int* p = std::lower_bound(lo, hi, j);
		return (p != hi && *p == j) ? (int)(p - (cols.data() + b)) : -1;
	}
	uint64_t blocks() const { return (uint64_t)cols.size(); }
};

typedef std::shared_ptr<SpPattern> PatPtr;

// The pattern of the given (row, column) pairs plus every diagonal block. Sorts `pairs`.
int make_pattern(int device, uint32_t n, std::vector<std::pair<int, int>>& pairs, PatPtr* out)
{
	for (uint32_t i = 0; i < n; ++i) pairs.push_back({(int)i, (int)i});
	std::sort(pairs.begin(), pairs.end());
	pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
	auto P = std::make_shared<SpPattern>();
	P->device = device;
	P->n = n;
	P->id = g_pattern_ids.fetch_add(1);
	P->rp.assign(n + 1, 0);
	for (auto& pr : pairs) P->rp[pr.first + 1] += 1;
	for (uint32_t i = 0; i < n; ++i) P->rp[i + 1] += P->rp[i];
	P->cols.resize(pairs.size());
	{
		// pairs are sorted and hold every (i, i): row i is pairs[rp[i] .. rp[i + 1]), diagonal first
		size_t k = 0;
		for (uint32_t i = 0; i < n; ++i)
		{
			size_t w = (size_t)P->rp[i];
			P->cols[w++] = (int)i;
			for (; k < pairs.size() && pairs[k].first == (int)i; ++k)
				if (pairs[k].second != (int)i) P->cols[w++] = pairs[k].second;
		}
	}
	P->nslices = (int)((n + kSlice - 1) / kSlice);
	P->slice_ptr.assign(P->nslices + 1, 0);
	for (int s = 0; s < P->nslices; ++s)
	{
		int w = 1;
		for (int l = 0; l < kSlice; ++l)
		{
			const uint32_t i = (uint32_t)s * kSlice + l;
			if (i < n) w = std::max(w, P->rp[i + 1] - P->rp[i]);
		}
		w = (w + kGroup - 1) / kGroup * kGroup;
		P->slice_ptr[s + 1] = P->slice_ptr[s] + kSlice * w;
	}
	P->nslots = (size_t)P->slice_ptr[P->nslices];
	std::vector<int> col(std::max<size_t>(P->nslots, 1));
	for (int s = 0; s < P->nslices; ++s)
	{
		const int w = (P->slice_ptr[s + 1] - P->slice_ptr[s]) / kSlice;
		for (int l = 0; l < kSlice; ++l)
		{
			const uint32_t i = (uint32_t)s * kSlice + l;
			const int row = (int)std::min<uint32_t>(i, n ? n - 1 : 0);
			const int len = i < n ? P->rp[i + 1] - P->rp[i] : 0;
			for (int k = 0; k < w; ++k)
				col[block_slot((size_t)P->slice_ptr[s], k, l)] = k < len ? P->cols[P->rp[i] + k] : row;
		}
	}
	cudaError_t e = cudaMalloc(&P->d_slice_ptr, P->slice_ptr.size() * sizeof(int));
	if (e == cudaSuccess) e = cudaMalloc(&P->d_col, col.size() * sizeof(int));
	if (e == cudaSuccess)
		e = cudaMemcpy(P->d_slice_ptr, P->slice_ptr.data(), P->slice_ptr.size() * sizeof(int), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(P->d_col, col.data(), col.size() * sizeof(int), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return cuda_fail(e, "sparse pattern");
	*out = P;
	return B3G_OK;
}

void pattern_pairs(const SpPattern* P, std::vector<std::pair<int, int>>& out)
{
	if (!P) return;
	for (uint32_t i = 0; i < P->n; ++i)
		for (int k = P->rp[i]; k < P->rp[i + 1]; ++k) out.push_back({(int)i, P->cols[k]});
}

// For every slot of `to`: the slot of the same block in `from`, -1 when absent (padding too).
std::vector<int> slot_map(const SpPattern* to, const SpPattern* from)
{
	std::vector<int> m(std::max<size_t>(to->nslots, 1), -1);
	if (!from) return m;
	for (uint32_t i = 0; i < to->n; ++i)
		for (int k = 0; k < to->rp[i + 1] - to->rp[i]; ++k)
		{
			const int kf = from->find((int)i, to->cols[to->rp[i] + k]);
			if (kf >= 0) m[to->slot((int)i, k)] = (int)from->slot((int)i, kf);
		}
	return m;
}

// b3Mat33 order (column-major) <-> plane order p = 3 r + c
inline int plane_of_b3(int idx) { return 3 * (idx % 3) + idx / 3; }

// ------------------------------------------------------------------ kernels
__global__ void k_vec_pack(float* __restrict__ d, const float* __restrict__ xyz, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		reinterpret_cast<float4*>(d)[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
}

__global__ void k_vec_unpack(float* __restrict__ xyz, const float* __restrict__ d, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 v = reinterpret_cast<const float4*>(d)[i];
		xyz[3 * i] = v.x;
		xyz[3 * i + 1] = v.y;
		xyz[3 * i + 2] = v.z;
	}
}

// out = a * A + b * B (B may be null)
__global__ void k_vec_axpby(float* out, float a, const float* A, float b, const float* B, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 x = reinterpret_cast<const float4*>(A)[i];
		float4 o;
		if (B)
		{
			const float4 y = reinterpret_cast<const float4*>(B)[i];
			o = make_float4(a * x.x + b * y.x, a * x.y + b * y.y, a * x.z + b * y.z, 0.0f);
		}
		else
			o = make_float4(a * x.x, a * x.y, a * x.z, 0.0f);
		reinterpret_cast<float4*>(out)[i] = o;
	}
}

// out = A + B, A - B exactly as single float operations (no fused multiply)
__global__ void k_vec_addsub(float* out, const float* A, const float* B, int sign, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 x = reinterpret_cast<const float4*>(A)[i];
		const float4 y = reinterpret_cast<const float4*>(B)[i];
		reinterpret_cast<float4*>(out)[i] = sign > 0 ? make_float4(x.x + y.x, x.y + y.y, x.z + y.z, 0.0f)
		                                             : make_float4(x.x - y.x, x.y - y.y, x.z - y.z, 0.0f);
	}
}

// per-CTA partial sums of a.b over entries (each entry's term in float, the sum in FP64)
__global__ void __launch_bounds__(kT) k_vec_dot_partials(const float* A, const float* B, int n, double* partials)
{
	__shared__ double sh[kT / 32];
	double s = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 x = reinterpret_cast<const float4*>(A)[i];
		const float4 y = reinterpret_cast<const float4*>(B)[i];
		s += (double)(x.x * y.x + x.y * y.y + x.z * y.z);
	}
	s = warp_sum(s);
	if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double t = 0.0;
		for (int k = 0; k < kT / 32; ++k) t += sh[k];
		partials[blockIdx.x] = t;
	}
}

__global__ void k_sum_partials(const double* partials, int count, double* out)
{
	__shared__ double sh[32];
	double s = 0.0;
	for (int k = threadIdx.x; k < count; k += blockDim.x) s += partials[k];
	s = warp_sum(s);
	if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double t = 0.0;
		for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
		*out = t;
	}
}

// queued writes of a dense vector: one thread per written entry, its writes in call order
__global__ void k_vec_apply(float* d, int m, const int* __restrict__ idx, const int* __restrict__ seg,
                            const uint8_t* __restrict__ op, const float* __restrict__ val)
{
	for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < m; u += gridDim.x * blockDim.x)
	{
		float4 v = reinterpret_cast<float4*>(d)[idx[u]];
		for (int e = seg[u]; e < seg[u + 1]; ++e)
		{
			const float a = val[3 * e], b = val[3 * e + 1], c = val[3 * e + 2];
			if (op[e]) v = make_float4(a, b, c, 0.0f);
			else v = make_float4(v.x + a, v.y + b, v.z + c, 0.0f);
		}
		reinterpret_cast<float4*>(d)[idx[u]] = v;
	}
}

// diagonal matrices: 9 planes of n floats
__global__ void k_diag_pack(float* d, const float* blocks, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		for (int r = 0; r < 3; ++r)
			for (int c = 0; c < 3; ++c) d[(3 * r + c) * (size_t)n + i] = blocks[9 * (size_t)i + 3 * c + r];
}

__global__ void k_diag_unpack(float* blocks, const float* d, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		for (int r = 0; r < 3; ++r)
			for (int c = 0; c < 3; ++c) blocks[9 * (size_t)i + 3 * c + r] = d[(3 * r + c) * (size_t)n + i];
}

// mode 0: out = a A + b B (B may be null); 1: transpose; 2: identity; 3: zero
__global__ void k_diag_op(float* out, const float* A, const float* B, float a, float b, int mode, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		float t[9];
		for (int p = 0; p < 9; ++p)
		{
			if (mode == 0) t[p] = B ? a * A[p * (size_t)n + i] + b * B[p * (size_t)n + i] : a * A[p * (size_t)n + i];
			else if (mode == 1) t[p] = A[(3 * (p % 3) + p / 3) * (size_t)n + i];
			else if (mode == 2) t[p] = (p % 4 == 0) ? 1.0f : 0.0f;
			else t[p] = 0.0f;
		}
		for (int p = 0; p < 9; ++p) out[p * (size_t)n + i] = t[p];
	}
}

// A + B, A - B of diagonal matrices as single float operations
__global__ void k_diag_addsub(float* out, const float* A, const float* B, int sign, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		for (int p = 0; p < 9; ++p)
		{
			const float x = A[p * (size_t)n + i], y = B[p * (size_t)n + i];
			out[p * (size_t)n + i] = sign > 0 ? x + y : x - y;
		}
}

__global__ void k_diag_mul_vec(float* out, const float* D, const float* v, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 x = reinterpret_cast<const float4*>(v)[i];
		float o[3];
		for (int r = 0; r < 3; ++r)
			o[r] = D[(3 * r) * (size_t)n + i] * x.x + D[(3 * r + 1) * (size_t)n + i] * x.y +
			       D[(3 * r + 2) * (size_t)n + i] * x.z;
		reinterpret_cast<float4*>(out)[i] = make_float4(o[0], o[1], o[2], 0.0f);
	}
}

__device__ __forceinline__ void ld_block(const float* P, size_t ns, size_t s, float a[9])
{
#pragma unroll
	for (int p = 0; p < 9; ++p) a[p] = P[p * ns + s];
}

__device__ __forceinline__ void ld_diag(const float* D, int n, int i, float a[9])
{
#pragma unroll
	for (int p = 0; p < 9; ++p) a[p] = D[p * (size_t)n + i];
}

__device__ __forceinline__ void mul33(const float a[9], const float b[9], float o[9])
{
#pragma unroll
	for (int r = 0; r < 3; ++r)
#pragma unroll
		for (int c = 0; c < 3; ++c) o[3 * r + c] = a[3 * r] * b[c] + a[3 * r + 1] * b[3 + c] + a[3 * r + 2] * b[6 + c];
}

// queued writes of a sparse matrix: one thread per written block, its writes in call order
__global__ void k_sp_apply(float* val, size_t ns, int m, const int* __restrict__ slot, const int* __restrict__ seg,
                           const uint8_t* __restrict__ op, const float* __restrict__ blk)
{
	for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < m; u += gridDim.x * blockDim.x)
	{
		const size_t s = (size_t)slot[u];
		float a[9];
		ld_block(val, ns, s, a);
		for (int e = seg[u]; e < seg[u + 1]; ++e)
#pragma unroll
			for (int p = 0; p < 9; ++p) a[p] = op[e] ? blk[9 * (size_t)e + p] : a[p] + blk[9 * (size_t)e + p];
#pragma unroll
		for (int p = 0; p < 9; ++p) val[p * ns + s] = a[p];
	}
}

// values of a grown pattern: new slot s takes old slot map[s] (zero when -1)
__global__ void k_sp_remap(float* out, size_t ns_out, const float* in, size_t ns_in, const int* __restrict__ map)
{
	for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < ns_out; s += (size_t)gridDim.x * blockDim.x)
	{
		const int m = map[s];
#pragma unroll
		for (int p = 0; p < 9; ++p) out[p * ns_out + s] = m >= 0 ? in[p * ns_in + m] : 0.0f;
	}
}

// Blockwise combination over the output pattern, warp per slice and lane per row:
//   out_ij = alpha [DL_i] A_ij [DR_j] + beta B_ij, on the diagonal also + gamma G_i,
// or, with gset, the A term's diagonal block replaced by G_i. A / B blocks are found through
// slot maps (null = the same pattern as the output). Each operation is one float operation per
// entry where the reference does one (scalar x block, block + block).
struct Combine
{
	int n;
	const int* slice_ptr;
	const int* col;
	size_t ns;
	float* out;
	const float* A;
	size_t nsA;
	const int* mapA;
	float alpha;
	int scaleA;        // multiply the A term by alpha (otherwise alpha is 1)
	const float* DL;
	const float* DR;
	const float* B;
	size_t nsB;
	const int* mapB;
	float beta;        // +1 or -1 (added or subtracted)
	const float* G;
	float gamma;       // +1 or -1
	int gset;
};

__global__ void __launch_bounds__(kT) k_sp_combine(Combine C)
{
	const int lane = threadIdx.x & 31;
	const int nsl = (C.n + kSlice - 1) / kSlice;
	for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < nsl; sl += (gridDim.x * blockDim.x) >> 5)
	{
		const int i = sl * kSlice + lane;
		if (i >= C.n) continue;
		const int base = C.slice_ptr[sl], w = (C.slice_ptr[sl + 1] - base) / kSlice;
		for (int k = 0; k < w; ++k)
		{
			const size_t s = block_slot((size_t)base, k, lane);
			float o[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
			if (C.A)
			{
				const int sa = C.mapA ? C.mapA[s] : (int)s;
				if (sa >= 0)
				{
					float a[9];
					ld_block(C.A, C.nsA, (size_t)sa, a);
					if (C.DL)
					{
						float d[9], t[9];
						ld_diag(C.DL, C.n, i, d);
						mul33(d, a, t);
#pragma unroll
						for (int p = 0; p < 9; ++p) a[p] = t[p];
					}
					if (C.DR)
					{
						float d[9], t[9];
						ld_diag(C.DR, C.n, C.col[s], d);
						mul33(a, d, t);
#pragma unroll
						for (int p = 0; p < 9; ++p) a[p] = t[p];
					}
#pragma unroll
					for (int p = 0; p < 9; ++p) o[p] = C.scaleA ? C.alpha * a[p] : a[p];
				}
			}
			if (k == 0 && C.G)
			{
				float g[9];
				ld_diag(C.G, C.n, i, g);
#pragma unroll
				for (int p = 0; p < 9; ++p) o[p] = C.gset ? g[p] : (C.gamma > 0.0f ? o[p] + g[p] : o[p] - g[p]);
			}
			if (C.B)
			{
				const int sb = C.mapB ? C.mapB[s] : (int)s;
				if (sb >= 0)
				{
					float b[9];
					ld_block(C.B, C.nsB, (size_t)sb, b);
#pragma unroll
					for (int p = 0; p < 9; ++p) o[p] = C.beta > 0.0f ? o[p] + b[p] : o[p] - b[p];
				}
			}
#pragma unroll
			for (int p = 0; p < 9; ++p) C.out[p * C.ns + s] = o[p];
		}
	}
}

// out = A v: the SpMV of the body step (16-byte loads of four blocks' planes and column ids,
// the matrix streamed evict-first so the gathered vector stays in L2)
__global__ void __launch_bounds__(kT) k_sp_mul_vec(int n, const int* slice_ptr, const int* col, size_t ns,
                                                   const float* A, const float* v, float* out)
{
	const int lane = threadIdx.x & 31;
	const int nsl = (n + kSlice - 1) / kSlice;
	for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < nsl; sl += (gridDim.x * blockDim.x) >> 5)
	{
		const int i = sl * kSlice + lane;
		if (i >= n) continue;
		const int base = slice_ptr[sl], w = (slice_ptr[sl + 1] - base) / kSlice;
		float o[3];
		spmv_row<float, float>(A, col, (int)ns, base, w, lane, v, o);
		vst(out, i, o);
	}
}

// scalar Jacobi of the reference's CG (sparse_solver.cpp:38-55) from the diagonal blocks
__global__ void k_sp_jacobi(int n, const int* slice_ptr, size_t ns, const float* A, float* minv)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const size_t s = block_slot((size_t)slice_ptr[i >> 5], 0, i & 31);
		reinterpret_cast<float4*>(minv)[i] =
		    make_float4(1.0f / A[0 * ns + s], 1.0f / A[4 * ns + s], 1.0f / A[8 * ns + s], 0.0f);
	}
}

// Backward-Euler system over the union pattern P of dfdx and dfdv (sparse_force_solver.cpp:165-174),
// warp per slice and lane per row:
//   A_ij = (delta_ij M_i - h dfdv_ij) - h^2 dfdx_ij
//   b_i = (M_i (v0_i - v_i) + h (fe_i + f_i)) + h sum_j dfdx_ij w_j,  w = ((x0 - x) + h v) + y
//   pA_ij = (S_i A_ij) S_j^T, on the diagonal ((.) + I) - S_i;  pb_i = S_i (b_i - sum_j A_ij z_j)
// and the scalar Jacobi of pA. Values of pA are written in P's layout.
struct BeSystem
{
	int n;
	const int* slice_ptr;
	const int* col;
	size_t ns;
	const int* mapX;
	const float* X;
	size_t nsX;
	const int* mapV;
	const float* V;
	size_t nsV;
	const float* M;
	const float* S;
	float h, hh;
	const float* v0;
	const float* v;
	const float* fe;
	const float* f;
	const float* w;
	const float* z;
	float* pA;
	float* pb;
	float* minv;
};

__global__ void __launch_bounds__(kT) k_be_system(BeSystem E)
{
	const int lane = threadIdx.x & 31;
	const int nsl = (E.n + kSlice - 1) / kSlice;
	for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < nsl; sl += (gridDim.x * blockDim.x) >> 5)
	{
		const int i = sl * kSlice + lane;
		if (i >= E.n) continue;
		const int base = E.slice_ptr[sl], w = (E.slice_ptr[sl + 1] - base) / kSlice;
		float Si[9], Mi[9];
		ld_diag(E.S, E.n, i, Si);
		ld_diag(E.M, E.n, i, Mi);
		float dxw[3] = {0, 0, 0}, az[3] = {0, 0, 0};
		for (int k = 0; k < w; ++k)
		{
			const size_t s = block_slot((size_t)base, k, lane);
			const int j = E.col[s];
			float x[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, vv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
			const int sx = E.mapX[s], sv = E.mapV[s];
			if (sx >= 0) ld_block(E.X, E.nsX, (size_t)sx, x);
			if (sv >= 0) ld_block(E.V, E.nsV, (size_t)sv, vv);
			float a[9];
#pragma unroll
			for (int p = 0; p < 9; ++p) a[p] = ((k == 0 ? Mi[p] : 0.0f) - E.h * vv[p]) - E.hh * x[p];
			const float4 wj = reinterpret_cast<const float4*>(E.w)[j];
			const float4 zj = reinterpret_cast<const float4*>(E.z)[j];
#pragma unroll
			for (int r = 0; r < 3; ++r)
			{
				dxw[r] += x[3 * r] * wj.x + x[3 * r + 1] * wj.y + x[3 * r + 2] * wj.z;
				az[r] += a[3 * r] * zj.x + a[3 * r + 1] * zj.y + a[3 * r + 2] * zj.z;
			}
			float Sj[9], t[9], u[9];
			ld_diag(E.S, E.n, j, Sj);
			mul33(Si, a, t);
			// (S_i A_ij) S_j^T
#pragma unroll
			for (int r = 0; r < 3; ++r)
#pragma unroll
				for (int c = 0; c < 3; ++c) u[3 * r + c] = t[3 * r] * Sj[3 * c] + t[3 * r + 1] * Sj[3 * c + 1] + t[3 * r + 2] * Sj[3 * c + 2];
			if (k == 0)
			{
#pragma unroll
				for (int p = 0; p < 9; ++p) u[p] = (u[p] + (p % 4 == 0 ? 1.0f : 0.0f)) - Si[p];
				reinterpret_cast<float4*>(E.minv)[i] = make_float4(1.0f / u[0], 1.0f / u[4], 1.0f / u[8], 0.0f);
			}
#pragma unroll
			for (int p = 0; p < 9; ++p) E.pA[p * E.ns + s] = u[p];
		}
		const float4 v0 = reinterpret_cast<const float4*>(E.v0)[i];
		const float4 vi = reinterpret_cast<const float4*>(E.v)[i];
		const float4 fe = reinterpret_cast<const float4*>(E.fe)[i];
		const float4 fi = reinterpret_cast<const float4*>(E.f)[i];
		const float dv[3] = {v0.x - vi.x, v0.y - vi.y, v0.z - vi.z};
		const float ff[3] = {fe.x + fi.x, fe.y + fi.y, fe.z + fi.z};
		float r[3];
#pragma unroll
		for (int c = 0; c < 3; ++c)
		{
			const float b = (Mi[3 * c] * dv[0] + Mi[3 * c + 1] * dv[1] + Mi[3 * c + 2] * dv[2] + E.h * ff[c]) + E.h * dxw[c];
			r[c] = b - az[c];
		}
		float pb[3];
#pragma unroll
		for (int c = 0; c < 3; ++c) pb[c] = Si[3 * c] * r[0] + Si[3 * c + 1] * r[1] + Si[3 * c + 2] * r[2];
		vst(E.pb, i, pb);
	}
}

// w = ((x0 - x) + h v) + y
__global__ void k_be_w(float* w, const float* x0, const float* x, const float* v, const float* y, float h, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 a = reinterpret_cast<const float4*>(x0)[i], b = reinterpret_cast<const float4*>(x)[i];
		const float4 c = reinterpret_cast<const float4*>(v)[i], d = reinterpret_cast<const float4*>(y)[i];
		reinterpret_cast<float4*>(w)[i] =
		    make_float4(((a.x - b.x) + h * c.x) + d.x, ((a.y - b.y) + h * c.y) + d.y, ((a.z - b.z) + h * c.z) + d.z, 0.0f);
	}
}

// dv = y' + z, v += dv, x = (x0 + h v) + y; per-CTA partials of |dv|^2
__global__ void __launch_bounds__(kT) k_be_update(float* x, float* v, const float* x0, const float* y, const float* py,
                                                  const float* z, float h, int n, double* partials)
{
	__shared__ double sh[kT / 32];
	double s = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const float4 p = reinterpret_cast<const float4*>(py)[i], q = reinterpret_cast<const float4*>(z)[i];
		const float4 dv = make_float4(p.x + q.x, p.y + q.y, p.z + q.z, 0.0f);
		float4 vi = reinterpret_cast<const float4*>(v)[i];
		vi = make_float4(vi.x + dv.x, vi.y + dv.y, vi.z + dv.z, 0.0f);
		const float4 a = reinterpret_cast<const float4*>(x0)[i], b = reinterpret_cast<const float4*>(y)[i];
		reinterpret_cast<float4*>(v)[i] = vi;
		reinterpret_cast<float4*>(x)[i] = make_float4((a.x + h * vi.x) + b.x, (a.y + h * vi.y) + b.y, (a.z + h * vi.z) + b.z, 0.0f);
		s += (double)(dv.x * dv.x + dv.y * dv.y + dv.z * dv.z);
	}
	s = warp_sum(s);
	if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double t = 0.0;
		for (int k = 0; k < kT / 32; ++k) t += sh[k];
		partials[blockIdx.x] = t;
	}
}

} // namespace

// ------------------------------------------------------------------ objects
struct b3g_dense_vec3 : public SparseObject
{
	uint32_t n = 0;
	float* d = nullptr;        // 4 n
	DevBuf stage;              // host transfers and queued writes
	std::vector<uint32_t> q_idx;
	std::vector<uint8_t> q_op;
	std::vector<float> q_val;  // 3 per queued write
	void release_device() override
	{
		if (d) cudaFree(d);
		d = nullptr;
		stage.release();
	}
};

struct b3g_diag_mat33 : public SparseObject
{
	uint32_t n = 0;
	float* d = nullptr;        // 9 planes of n
	DevBuf stage;
	void release_device() override
	{
		if (d) cudaFree(d);
		d = nullptr;
		stage.release();
	}
};

struct b3g_sparse_mat33 : public SparseObject
{
	uint32_t n = 0;
	PatPtr pat;                // null: no blocks
	float* val = nullptr;      // 9 planes of pat->nslots
	DevBuf stage;
	std::vector<uint32_t> q_i, q_j;
	std::vector<uint8_t> q_op;
	std::vector<float> q_blk;  // 9 per queued write, b3Mat33 order
	void release_device() override
	{
		if (val) cudaFree(val);
		val = nullptr;
		pat.reset();
		stage.release();
	}
};

namespace b3g {

// Solver workspace of a context: CG vectors and scalars, the Newton iterate and the system of the
// backward-Euler solve, the force model's containers (kept between calls with their patterns).
struct SparseWork
{
	uint32_t n = 0;
	DevBuf vecs;               // r d d2 q s minv py w pb: 9 x 4 n floats
	Scalars* sc = nullptr;
	double* partials = nullptr;
	double* sum = nullptr;
	DevBuf pA;                 // BE system values
	PatPtr sys;                // union pattern of dfdx and dfdv
	uint64_t sys_x = 0, sys_v = 0;
	DevBuf maps;               // slot maps into dfdx and dfdv
	b3g_dense_vec3* xi = nullptr;
	b3g_dense_vec3* vi = nullptr;
	b3g_dense_vec3* fi = nullptr;
	b3g_sparse_mat33* dfdx = nullptr;
	b3g_sparse_mat33* dfdv = nullptr;
};

} // namespace b3g

namespace {

template <class T>
T* register_obj(b3g_context* ctx, T* o)
{
	o->ctx = ctx;
	ctx->live_sparse.push_back(o);
	return o;
}

void unregister_obj(SparseObject* o)
{
	if (!o->ctx) return;
	auto& L = o->ctx->live_sparse;
	L.erase(std::remove(L.begin(), L.end(), o), L.end());
}

int check_ctx(const SparseObject* o)
{
	if (!o) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	if (!o->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "the container's context was destroyed");
	cudaSetDevice(o->ctx->device);
	return B3G_OK;
}

int same_ctx(const SparseObject* a, const SparseObject* b)
{
	if (a->ctx != b->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "containers of different contexts");
	return B3G_OK;
}

inline cudaStream_t stream_of(const SparseObject* o) { return o->ctx->stream; }

int vec_flush(b3g_dense_vec3* v)
{
	if (v->q_idx.empty()) return B3G_OK;
	const size_t E = v->q_idx.size();
	std::vector<int> ord(E);
	std::iota(ord.begin(), ord.end(), 0);
	std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return v->q_idx[a] < v->q_idx[b]; });
	std::vector<int> idx, seg;
	std::vector<uint8_t> op(E);
	std::vector<float> val(3 * E);
	for (size_t e = 0; e < E; ++e)
	{
		const int o = ord[e];
		if (idx.empty() || (uint32_t)idx.back() != v->q_idx[o])
		{
			idx.push_back((int)v->q_idx[o]);
			seg.push_back((int)e);
		}
		op[e] = v->q_op[o];
		for (int c = 0; c < 3; ++c) val[3 * e + c] = v->q_val[3 * (size_t)o + c];
	}
	seg.push_back((int)E);
	const size_t m = idx.size();
	const size_t bytes = (m + seg.size()) * sizeof(int) + E * 3 * sizeof(float) + E;
	cudaError_t e = v->stage.ensure(bytes + 64);
	if (e != cudaSuccess) return cuda_fail(e, "dense_vec3 queued writes");
	char* base = (char*)v->stage.p;
	int* d_idx = (int*)base;
	int* d_seg = d_idx + m;
	float* d_val = (float*)(d_seg + seg.size());
	uint8_t* d_op = (uint8_t*)(d_val + 3 * E);
	cudaStream_t st = stream_of(v);
	e = cudaMemcpyAsync(d_idx, idx.data(), m * sizeof(int), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_seg, seg.data(), seg.size() * sizeof(int), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_val, val.data(), val.size() * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_op, op.data(), E, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
	{
		k_vec_apply<<<grid_of(m, kT), kT, 0, st>>>(v->d, (int)m, d_idx, d_seg, d_op, d_val);
		e = cudaGetLastError();
	}
	// the pageable copies above are staged before they return: the host vectors may go
	v->q_idx.clear();
	v->q_op.clear();
	v->q_val.clear();
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "dense_vec3 queued writes");
}

// replaces m's pattern by P, carrying the values of the blocks both have
int sp_set_pattern(b3g_sparse_mat33* m, const PatPtr& P)
{
	float* nv = nullptr;
	cudaError_t e = cudaMalloc(&nv, 9 * std::max<size_t>(P->nslots, 1) * sizeof(float));
	if (e != cudaSuccess) return cuda_fail(e, "sparse_mat33 values");
	cudaStream_t st = stream_of(m);
	if (m->pat && m->val)
	{
		std::vector<int> map = slot_map(P.get(), m->pat.get());
		int* d_map = nullptr;
		e = cudaMalloc(&d_map, map.size() * sizeof(int));
		if (e == cudaSuccess) e = cudaMemcpyAsync(d_map, map.data(), map.size() * sizeof(int), cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess)
		{
			k_sp_remap<<<grid_of(P->nslots, kT), kT, 0, st>>>(nv, P->nslots, m->val, m->pat->nslots, d_map);
			e = cudaGetLastError();
		}
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		cudaFree(d_map);
	}
	else
		e = cudaMemsetAsync(nv, 0, 9 * std::max<size_t>(P->nslots, 1) * sizeof(float), st);
	if (e != cudaSuccess)
	{
		cudaFree(nv);
		return cuda_fail(e, "sparse_mat33 pattern change");
	}
	if (m->val)
	{
		cudaStreamSynchronize(st);
		cudaFree(m->val);
	}
	m->val = nv;
	m->pat = P;
	return B3G_OK;
}

int sp_flush(b3g_sparse_mat33* m)
{
	if (m->q_i.empty()) return B3G_OK;
	const size_t E = m->q_i.size();
	// new blocks grow the pattern
	std::vector<std::pair<int, int>> extra;
	for (size_t e = 0; e < E; ++e)
		if (!m->pat || m->pat->find((int)m->q_i[e], (int)m->q_j[e]) < 0) extra.push_back({(int)m->q_i[e], (int)m->q_j[e]});
	if (!extra.empty())
	{
		pattern_pairs(m->pat.get(), extra);
		PatPtr P;
		int rc = make_pattern(m->ctx->device, m->n, extra, &P);
		if (rc != B3G_OK) return rc;
		rc = sp_set_pattern(m, P);
		if (rc != B3G_OK) return rc;
	}
	const SpPattern* P = m->pat.get();
	std::vector<int> slot(E);
	for (size_t e = 0; e < E; ++e) slot[e] = (int)P->slot((int)m->q_i[e], P->find((int)m->q_i[e], (int)m->q_j[e]));
	std::vector<int> ord(E);
	std::iota(ord.begin(), ord.end(), 0);
	std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return slot[a] < slot[b]; });
	std::vector<int> us, seg;
	std::vector<uint8_t> op(E);
	std::vector<float> blk(9 * E);
	for (size_t e = 0; e < E; ++e)
	{
		const int o = ord[e];
		if (us.empty() || us.back() != slot[o])
		{
			us.push_back(slot[o]);
			seg.push_back((int)e);
		}
		op[e] = m->q_op[o];
		for (int t = 0; t < 9; ++t) blk[9 * e + plane_of_b3(t)] = m->q_blk[9 * (size_t)o + t];
	}
	seg.push_back((int)E);
	const size_t U = us.size();
	const size_t bytes = (U + seg.size()) * sizeof(int) + blk.size() * sizeof(float) + E;
	cudaError_t e = m->stage.ensure(bytes + 64);
	if (e != cudaSuccess) return cuda_fail(e, "sparse_mat33 queued writes");
	char* base = (char*)m->stage.p;
	int* d_us = (int*)base;
	int* d_seg = d_us + U;
	float* d_blk = (float*)(d_seg + seg.size());
	uint8_t* d_op = (uint8_t*)(d_blk + blk.size());
	cudaStream_t st = stream_of(m);
	e = cudaMemcpyAsync(d_us, us.data(), U * sizeof(int), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_seg, seg.data(), seg.size() * sizeof(int), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_blk, blk.data(), blk.size() * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_op, op.data(), E, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
	{
		k_sp_apply<<<grid_of(U, kT), kT, 0, st>>>(m->val, P->nslots, (int)U, d_us, d_seg, d_op, d_blk);
		e = cudaGetLastError();
	}
	m->q_i.clear();
	m->q_j.clear();
	m->q_op.clear();
	m->q_blk.clear();
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "sparse_mat33 queued writes");
}

int sp_queue(b3g_sparse_mat33* m, uint32_t count, const uint32_t* rows, const uint32_t* cols, const float* blocks,
             uint8_t op)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (count && (!rows || !cols || !blocks)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null array");
	for (uint32_t k = 0; k < count; ++k)
		if (rows[k] >= m->n || cols[k] >= m->n)
			return fail(B3G_ERROR_INVALID_ARGUMENT, "block %u at (%u, %u) is outside a %u x %u block matrix", k, rows[k],
			            cols[k], m->n, m->n);
	m->q_i.insert(m->q_i.end(), rows, rows + count);
	m->q_j.insert(m->q_j.end(), cols, cols + count);
	m->q_op.insert(m->q_op.end(), count, op);
	m->q_blk.insert(m->q_blk.end(), blocks, blocks + 9 * (size_t)count);
	return B3G_OK;
}

int vec_queue(b3g_dense_vec3* v, uint32_t count, const uint32_t* index, const float* values, uint8_t op)
{
	int rc = check_ctx(v);
	if (rc != B3G_OK) return rc;
	if (count && (!index || !values)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null array");
	for (uint32_t k = 0; k < count; ++k)
		if (index[k] >= v->n) return fail(B3G_ERROR_INVALID_ARGUMENT, "entry %u indexes %u of %u", k, index[k], v->n);
	v->q_idx.insert(v->q_idx.end(), index, index + count);
	v->q_op.insert(v->q_op.end(), count, op);
	v->q_val.insert(v->q_val.end(), values, values + 3 * (size_t)count);
	return B3G_OK;
}

// The union pattern of a and b (a itself when both share it) and the slot maps into each.
int union_of(b3g_context* ctx, uint32_t n, const PatPtr& a, const PatPtr& b, PatPtr* out)
{
	if (a && b && a == b)
	{
		*out = a;
		return B3G_OK;
	}
	if (a && !b)
	{
		*out = a;
		return B3G_OK;
	}
	if (b && !a)
	{
		*out = b;
		return B3G_OK;
	}
	std::vector<std::pair<int, int>> pairs;
	pattern_pairs(a.get(), pairs);
	pattern_pairs(b.get(), pairs);
	return make_pattern(ctx->device, n, pairs, out);
}

// out's pattern := P (values of out not carried); maps of a and b into P uploaded to `maps`.
struct MapSet
{
	int* mA = nullptr;
	int* mB = nullptr;
	DevBuf buf;
};

int upload_maps(b3g_context* ctx, const PatPtr& P, const SpPattern* a, const SpPattern* b, MapSet& M)
{
	std::vector<int> ma, mb;
	const size_t ns = std::max<size_t>(P->nslots, 1);
	const bool needA = a && a != P.get(), needB = b && b != P.get();
	if (needA) ma = slot_map(P.get(), a);
	if (needB) mb = slot_map(P.get(), b);
	cudaError_t e = M.buf.ensure(2 * ns * sizeof(int));
	if (e != cudaSuccess) return cuda_fail(e, "sparse maps");
	M.mA = needA ? (int*)M.buf.p : nullptr;
	M.mB = needB ? (int*)M.buf.p + ns : nullptr;
	if (needA) e = cudaMemcpyAsync(M.mA, ma.data(), ns * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
	if (e == cudaSuccess && needB) e = cudaMemcpyAsync(M.mB, mb.data(), ns * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "sparse maps");
}

// out := combination over pattern P of (a, b) as described by C (C's output fields are filled
// here). out may be a or b: the result goes to a new value array first.
int sp_combine(b3g_sparse_mat33* out, const PatPtr& P, const b3g_sparse_mat33* a, const b3g_sparse_mat33* b,
               Combine C)
{
	b3g_context* ctx = out->ctx;
	MapSet M;
	int rc = upload_maps(ctx, P, a ? a->pat.get() : nullptr, b ? b->pat.get() : nullptr, M);
	if (rc != B3G_OK) return rc;
	float* nv = nullptr;
	const size_t ns = std::max<size_t>(P->nslots, 1);
	cudaError_t e = cudaMalloc(&nv, 9 * ns * sizeof(float));
	if (e != cudaSuccess)
	{
		M.buf.release();
		return cuda_fail(e, "sparse_mat33 values");
	}
	C.n = (int)out->n;
	C.slice_ptr = P->d_slice_ptr;
	C.col = P->d_col;
	C.ns = P->nslots;
	C.out = nv;
	if (a && a->pat)
	{
		C.A = a->val;
		C.nsA = a->pat->nslots;
		C.mapA = M.mA;
	}
	else
		C.A = nullptr;
	if (b && b->pat)
	{
		C.B = b->val;
		C.nsB = b->pat->nslots;
		C.mapB = M.mB;
	}
	else
		C.B = nullptr;
	cudaStream_t st = ctx->stream;
	if (out->n > 0) k_sp_combine<<<grid_of((size_t)P->nslices * 32, kT), kT, 0, st>>>(C);
	e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the maps and the old values may go
	M.buf.release();
	if (e != cudaSuccess)
	{
		cudaFree(nv);
		return cuda_fail(e, "sparse_mat33 operation");
	}
	if (out->val) cudaFree(out->val);
	out->val = nv;
	out->pat = P;
	return B3G_OK;
}

Combine combine_defaults()
{
	Combine C;
	std::memset(&C, 0, sizeof(C));
	C.alpha = 1.0f;
	C.beta = 1.0f;
	C.gamma = 1.0f;
	return C;
}

int check_vec(const b3g_dense_vec3* v, uint32_t n, const char* what)
{
	int rc = check_ctx(v);
	if (rc != B3G_OK) return rc;
	if (v->n != n) return fail(B3G_ERROR_INVALID_ARGUMENT, "%s has %u entries, expected %u", what, v->n, n);
	return B3G_OK;
}

int check_diag(const b3g_diag_mat33* m, uint32_t n, const char* what)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (m->n != n) return fail(B3G_ERROR_INVALID_ARGUMENT, "%s has %u entries, expected %u", what, m->n, n);
	return B3G_OK;
}

int check_sp(const b3g_sparse_mat33* m, uint32_t n, const char* what)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (m->n != n) return fail(B3G_ERROR_INVALID_ARGUMENT, "%s has %u rows, expected %u", what, m->n, n);
	return B3G_OK;
}

int reduce_dot(b3g_context* ctx, const float* a, const float* b, uint32_t n, double* out)
{
	cudaStream_t st = ctx->stream;
	double* buf = nullptr;
	const int g = grid_of(n, kT);
	cudaError_t e = cudaMallocAsync(&buf, (g + 1) * sizeof(double), st);
	if (e != cudaSuccess) return cuda_fail(e, "dot");
	k_vec_dot_partials<<<g, kT, 0, st>>>(a, b, (int)n, buf);
	k_sum_partials<<<1, 256, 0, st>>>(buf, g, buf + g);
	e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaMemcpyAsync(out, buf + g, sizeof(double), cudaMemcpyDeviceToHost, st);
	cudaFreeAsync(buf, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "dot");
}

} // namespace

void release_sparse(b3g_context* c)
{
	for (SparseObject* o : c->live_sparse)
	{
		o->release_device();
		o->ctx = nullptr;
	}
	c->live_sparse.clear();
	if (c->sparse_work)
	{
		// the workspace's own containers were detached above; they are not the caller's
		SparseWork* w = c->sparse_work;
		delete w->xi;
		delete w->vi;
		delete w->fi;
		delete w->dfdx;
		delete w->dfdv;
		w->vecs.release();
		w->pA.release();
		w->maps.release();
		w->sys.reset();
		if (w->sc) cudaFree(w->sc);
		if (w->partials) cudaFree(w->partials);
		delete w;
		c->sparse_work = nullptr;
	}
}

// ------------------------------------------------------------------ b3DenseVec3
extern "C" int b3g_dense_vec3_create(b3g_context* ctx, uint32_t n, b3g_dense_vec3** out)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*out = nullptr;
	cudaSetDevice(ctx->device);
	b3g_dense_vec3* v = new b3g_dense_vec3();
	v->n = n;
	cudaError_t e = cudaMalloc(&v->d, 4 * std::max<size_t>(n, 1) * sizeof(float));
	if (e == cudaSuccess) e = cudaMemsetAsync(v->d, 0, 4 * std::max<size_t>(n, 1) * sizeof(float), ctx->stream);
	if (e != cudaSuccess)
	{
		if (v->d) cudaFree(v->d);
		delete v;
		return cuda_fail(e, "dense_vec3_create");
	}
	*out = register_obj(ctx, v);
	return B3G_OK;
}

extern "C" int b3g_dense_vec3_destroy(b3g_dense_vec3* v)
{
	if (!v) return B3G_OK;
	if (v->ctx)
	{
		cudaSetDevice(v->ctx->device);
		cudaStreamSynchronize(v->ctx->stream);
		v->release_device();
		unregister_obj(v);
	}
	delete v;
	return B3G_OK;
}

extern "C" int b3g_dense_vec3_size(const b3g_dense_vec3* v, uint32_t* n)
{
	if (!v || !n) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*n = v->n;
	return B3G_OK;
}

extern "C" int b3g_dense_vec3_set(b3g_dense_vec3* v, const float* xyz)
{
	int rc = check_ctx(v);
	if (rc != B3G_OK) return rc;
	if (!xyz && v->n) return fail(B3G_ERROR_INVALID_ARGUMENT, "null array");
	v->q_idx.clear();  // the whole vector is replaced: earlier queued writes are void
	v->q_op.clear();
	v->q_val.clear();
	if (!v->n) return B3G_OK;
	cudaStream_t st = stream_of(v);
	cudaError_t e = v->stage.ensure(3 * (size_t)v->n * sizeof(float));
	if (e == cudaSuccess) e = cudaMemcpyAsync(v->stage.p, xyz, 3 * (size_t)v->n * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
	{
		k_vec_pack<<<grid_of(v->n, kT), kT, 0, st>>>(v->d, (const float*)v->stage.p, (int)v->n);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "dense_vec3_set");
}

extern "C" int b3g_dense_vec3_get(b3g_dense_vec3* v, float* xyz)
{
	int rc = check_ctx(v);
	if (rc != B3G_OK) return rc;
	if (!xyz && v->n) return fail(B3G_ERROR_INVALID_ARGUMENT, "null array");
	rc = vec_flush(v);
	if (rc != B3G_OK || !v->n) return rc;
	cudaStream_t st = stream_of(v);
	cudaError_t e = v->stage.ensure(3 * (size_t)v->n * sizeof(float));
	if (e == cudaSuccess)
	{
		k_vec_unpack<<<grid_of(v->n, kT), kT, 0, st>>>((float*)v->stage.p, v->d, (int)v->n);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(xyz, v->stage.p, 3 * (size_t)v->n * sizeof(float), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "dense_vec3_get");
}

extern "C" int b3g_dense_vec3_set_zero(b3g_dense_vec3* v)
{
	int rc = check_ctx(v);
	if (rc != B3G_OK) return rc;
	v->q_idx.clear();
	v->q_op.clear();
	v->q_val.clear();
	cudaError_t e = cudaMemsetAsync(v->d, 0, 4 * (size_t)v->n * sizeof(float), stream_of(v));
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "dense_vec3_set_zero");
}

static int vec_binary(b3g_dense_vec3* out, const b3g_dense_vec3* a, const b3g_dense_vec3* b, int mode, float s)
{
	int rc = check_ctx(out);
	if (rc == B3G_OK) rc = check_vec(a, out->n, "operand a");
	if (rc == B3G_OK && b) rc = check_vec(b, out->n, "operand b");
	if (rc == B3G_OK) rc = same_ctx(out, a);
	if (rc == B3G_OK && b) rc = same_ctx(out, b);
	if (rc == B3G_OK) rc = vec_flush(const_cast<b3g_dense_vec3*>(a));
	if (rc == B3G_OK && b) rc = vec_flush(const_cast<b3g_dense_vec3*>(b));
	if (rc == B3G_OK && out != a && out != b)
	{
		out->q_idx.clear();
		out->q_op.clear();
		out->q_val.clear();
	}
	if (rc == B3G_OK) rc = vec_flush(out);
	if (rc != B3G_OK || !out->n) return rc;
	cudaStream_t st = stream_of(out);
	const int g = grid_of(out->n, kT);
	if (mode == 0) k_vec_addsub<<<g, kT, 0, st>>>(out->d, a->d, b->d, +1, (int)out->n);
	else if (mode == 1) k_vec_addsub<<<g, kT, 0, st>>>(out->d, a->d, b->d, -1, (int)out->n);
	else k_vec_axpby<<<g, kT, 0, st>>>(out->d, s, a->d, 0.0f, nullptr, (int)out->n);
	cudaError_t e = cudaGetLastError();
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "dense_vec3 operation");
}

extern "C" int b3g_dense_vec3_copy(b3g_dense_vec3* out, const b3g_dense_vec3* a)
{
	return vec_binary(out, a, nullptr, 2, 1.0f);
}
extern "C" int b3g_dense_vec3_add(b3g_dense_vec3* out, const b3g_dense_vec3* a, const b3g_dense_vec3* b)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return vec_binary(out, a, b, 0, 0.0f);
}
extern "C" int b3g_dense_vec3_sub(b3g_dense_vec3* out, const b3g_dense_vec3* a, const b3g_dense_vec3* b)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return vec_binary(out, a, b, 1, 0.0f);
}
extern "C" int b3g_dense_vec3_scale(b3g_dense_vec3* out, float s, const b3g_dense_vec3* a)
{
	return vec_binary(out, a, nullptr, 2, s);
}
extern "C" int b3g_dense_vec3_negate(b3g_dense_vec3* out, const b3g_dense_vec3* a)
{
	return vec_binary(out, a, nullptr, 2, -1.0f);
}

extern "C" int b3g_dense_vec3_dot(const b3g_dense_vec3* a, const b3g_dense_vec3* b, double* out)
{
	if (!out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	int rc = check_ctx(a);
	if (rc == B3G_OK) rc = check_vec(b, a->n, "operand b");
	if (rc == B3G_OK) rc = same_ctx(a, b);
	if (rc == B3G_OK) rc = vec_flush(const_cast<b3g_dense_vec3*>(a));
	if (rc == B3G_OK) rc = vec_flush(const_cast<b3g_dense_vec3*>(b));
	if (rc != B3G_OK) return rc;
	*out = 0.0;
	if (!a->n) return B3G_OK;
	return reduce_dot(a->ctx, a->d, b->d, a->n, out);
}

extern "C" int b3g_dense_vec3_length_squared(const b3g_dense_vec3* a, double* out)
{
	return b3g_dense_vec3_dot(a, a, out);
}

extern "C" int b3g_dense_vec3_add_values(b3g_dense_vec3* v, uint32_t count, const uint32_t* index, const float* values)
{
	return vec_queue(v, count, index, values, 0);
}

extern "C" int b3g_dense_vec3_set_values(b3g_dense_vec3* v, uint32_t count, const uint32_t* index, const float* values)
{
	return vec_queue(v, count, index, values, 1);
}

extern "C" int b3g_dense_vec3_device(b3g_dense_vec3* v, void** device_ptr)
{
	if (!device_ptr) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	int rc = check_ctx(v);
	if (rc == B3G_OK) rc = vec_flush(v);
	if (rc != B3G_OK) return rc;
	*device_ptr = v->d;
	return B3G_OK;
}

// ------------------------------------------------------------------ b3DiagMat33
extern "C" int b3g_diag_mat33_create(b3g_context* ctx, uint32_t n, b3g_diag_mat33** out)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*out = nullptr;
	cudaSetDevice(ctx->device);
	b3g_diag_mat33* m = new b3g_diag_mat33();
	m->n = n;
	cudaError_t e = cudaMalloc(&m->d, 9 * std::max<size_t>(n, 1) * sizeof(float));
	if (e == cudaSuccess) e = cudaMemsetAsync(m->d, 0, 9 * std::max<size_t>(n, 1) * sizeof(float), ctx->stream);
	if (e != cudaSuccess)
	{
		if (m->d) cudaFree(m->d);
		delete m;
		return cuda_fail(e, "diag_mat33_create");
	}
	*out = register_obj(ctx, m);
	return B3G_OK;
}

extern "C" int b3g_diag_mat33_destroy(b3g_diag_mat33* m)
{
	if (!m) return B3G_OK;
	if (m->ctx)
	{
		cudaSetDevice(m->ctx->device);
		cudaStreamSynchronize(m->ctx->stream);
		m->release_device();
		unregister_obj(m);
	}
	delete m;
	return B3G_OK;
}

extern "C" int b3g_diag_mat33_size(const b3g_diag_mat33* m, uint32_t* n)
{
	if (!m || !n) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*n = m->n;
	return B3G_OK;
}

extern "C" int b3g_diag_mat33_set(b3g_diag_mat33* m, const float* blocks)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (!blocks && m->n) return fail(B3G_ERROR_INVALID_ARGUMENT, "null array");
	if (!m->n) return B3G_OK;
	cudaStream_t st = stream_of(m);
	cudaError_t e = m->stage.ensure(9 * (size_t)m->n * sizeof(float));
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(m->stage.p, blocks, 9 * (size_t)m->n * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
	{
		k_diag_pack<<<grid_of(m->n, kT), kT, 0, st>>>(m->d, (const float*)m->stage.p, (int)m->n);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "diag_mat33_set");
}

extern "C" int b3g_diag_mat33_get(b3g_diag_mat33* m, float* blocks)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (!blocks && m->n) return fail(B3G_ERROR_INVALID_ARGUMENT, "null array");
	if (!m->n) return B3G_OK;
	cudaStream_t st = stream_of(m);
	cudaError_t e = m->stage.ensure(9 * (size_t)m->n * sizeof(float));
	if (e == cudaSuccess)
	{
		k_diag_unpack<<<grid_of(m->n, kT), kT, 0, st>>>((float*)m->stage.p, m->d, (int)m->n);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(blocks, m->stage.p, 9 * (size_t)m->n * sizeof(float), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "diag_mat33_get");
}

static int diag_op(b3g_diag_mat33* out, const b3g_diag_mat33* a, const b3g_diag_mat33* b, float s, float t, int mode)
{
	int rc = check_ctx(out);
	if (rc == B3G_OK && a) rc = check_diag(a, out->n, "operand a");
	if (rc == B3G_OK && b) rc = check_diag(b, out->n, "operand b");
	if (rc == B3G_OK && a) rc = same_ctx(out, a);
	if (rc == B3G_OK && b) rc = same_ctx(out, b);
	if (rc != B3G_OK || !out->n) return rc;
	cudaStream_t st = stream_of(out);
	const int g = grid_of(out->n, kT);
	if (mode == 1 && a == out)
	{
		// transpose in place through a copy
		cudaError_t e = out->stage.ensure(9 * (size_t)out->n * sizeof(float));
		if (e == cudaSuccess) e = cudaMemcpyAsync(out->stage.p, a->d, 9 * (size_t)out->n * sizeof(float), cudaMemcpyDeviceToDevice, st);
		if (e != cudaSuccess) return cuda_fail(e, "diag_mat33 transpose");
		k_diag_op<<<g, kT, 0, st>>>(out->d, (const float*)out->stage.p, nullptr, 1.0f, 0.0f, 1, (int)out->n);
	}
	else if (mode == 4)
		k_diag_addsub<<<g, kT, 0, st>>>(out->d, a->d, b->d, s > 0.0f ? +1 : -1, (int)out->n);
	else
		k_diag_op<<<g, kT, 0, st>>>(out->d, a ? a->d : nullptr, b ? b->d : nullptr, s, t, mode, (int)out->n);
	cudaError_t e = cudaGetLastError();
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "diag_mat33 operation");
}

extern "C" int b3g_diag_mat33_set_zero(b3g_diag_mat33* m) { return diag_op(m, nullptr, nullptr, 0, 0, 3); }
extern "C" int b3g_diag_mat33_set_identity(b3g_diag_mat33* m) { return diag_op(m, nullptr, nullptr, 0, 0, 2); }
extern "C" int b3g_diag_mat33_copy(b3g_diag_mat33* out, const b3g_diag_mat33* a)
{
	if (!a) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return diag_op(out, a, nullptr, 1.0f, 0.0f, 0);
}
extern "C" int b3g_diag_mat33_transpose(b3g_diag_mat33* out, const b3g_diag_mat33* a)
{
	if (!a) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return diag_op(out, a, nullptr, 1.0f, 0.0f, 1);
}
extern "C" int b3g_diag_mat33_add(b3g_diag_mat33* out, const b3g_diag_mat33* a, const b3g_diag_mat33* b)
{
	if (!a || !b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return diag_op(out, a, b, 1.0f, 1.0f, 4);
}
extern "C" int b3g_diag_mat33_sub(b3g_diag_mat33* out, const b3g_diag_mat33* a, const b3g_diag_mat33* b)
{
	if (!a || !b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return diag_op(out, a, b, -1.0f, -1.0f, 4);
}
extern "C" int b3g_diag_mat33_scale(b3g_diag_mat33* out, float s, const b3g_diag_mat33* a)
{
	if (!a) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return diag_op(out, a, nullptr, s, 0.0f, 0);
}
extern "C" int b3g_diag_mat33_negate(b3g_diag_mat33* out, const b3g_diag_mat33* a)
{
	if (!a) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	return diag_op(out, a, nullptr, -1.0f, 0.0f, 0);
}

extern "C" int b3g_diag_mat33_mul_vec(b3g_dense_vec3* out, const b3g_diag_mat33* a, const b3g_dense_vec3* v)
{
	int rc = check_ctx(out);
	if (rc == B3G_OK) rc = check_diag(a, out->n, "matrix");
	if (rc == B3G_OK) rc = check_vec(v, out->n, "vector");
	if (rc == B3G_OK) rc = same_ctx(out, a);
	if (rc == B3G_OK) rc = same_ctx(out, v);
	if (rc == B3G_OK) rc = vec_flush(const_cast<b3g_dense_vec3*>(v));
	if (rc == B3G_OK && out != v)
	{
		out->q_idx.clear();
		out->q_op.clear();
		out->q_val.clear();
	}
	if (rc != B3G_OK || !out->n) return rc;
	k_diag_mul_vec<<<grid_of(out->n, kT), kT, 0, stream_of(out)>>>(out->d, a->d, v->d, (int)out->n);
	cudaError_t e = cudaGetLastError();
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "diag_mat33_mul_vec");
}

// ------------------------------------------------------------------ b3SparseMat33
extern "C" int b3g_sparse_mat33_create(b3g_context* ctx, uint32_t n, b3g_sparse_mat33** out)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (n > (1u << 30)) return fail(B3G_ERROR_INVALID_ARGUMENT, "too many rows (%u)", n);
	cudaSetDevice(ctx->device);
	b3g_sparse_mat33* m = new b3g_sparse_mat33();
	m->n = n;
	*out = register_obj(ctx, m);
	return B3G_OK;
}

extern "C" int b3g_sparse_mat33_destroy(b3g_sparse_mat33* m)
{
	if (!m) return B3G_OK;
	if (m->ctx)
	{
		cudaSetDevice(m->ctx->device);
		cudaStreamSynchronize(m->ctx->stream);
		m->release_device();
		unregister_obj(m);
	}
	delete m;
	return B3G_OK;
}

extern "C" int b3g_sparse_mat33_size(b3g_sparse_mat33* m, uint32_t* n, uint64_t* blocks)
{
	int rc = check_ctx(m);
	if (rc == B3G_OK) rc = sp_flush(m);
	if (rc != B3G_OK) return rc;
	if (n) *n = m->n;
	if (blocks) *blocks = m->pat ? m->pat->blocks() : 0;
	return B3G_OK;
}

extern "C" int b3g_sparse_mat33_add_blocks(b3g_sparse_mat33* m, uint32_t count, const uint32_t* rows,
                                          const uint32_t* cols, const float* blocks)
{
	return sp_queue(m, count, rows, cols, blocks, 0);
}

extern "C" int b3g_sparse_mat33_set_blocks(b3g_sparse_mat33* m, uint32_t count, const uint32_t* rows,
                                          const uint32_t* cols, const float* blocks)
{
	return sp_queue(m, count, rows, cols, blocks, 1);
}

// every value plane to the host (synchronous)
static int sp_download(b3g_sparse_mat33* m, std::vector<float>& h)
{
	h.assign(9 * m->pat->nslots, 0.0f);
	cudaStream_t st = stream_of(m);
	cudaError_t e = cudaMemcpyAsync(h.data(), m->val, h.size() * sizeof(float), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "sparse_mat33 download");
}

extern "C" int b3g_sparse_mat33_get_block(b3g_sparse_mat33* m, uint32_t i, uint32_t j, float block[9])
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (!block) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (i >= m->n || j >= m->n) return fail(B3G_ERROR_INVALID_ARGUMENT, "(%u, %u) outside %u rows", i, j, m->n);
	rc = sp_flush(m);
	if (rc != B3G_OK) return rc;
	for (int t = 0; t < 9; ++t) block[t] = 0.0f;
	const int k = m->pat ? m->pat->find((int)i, (int)j) : -1;
	if (k < 0) return B3G_OK;
	const size_t s = m->pat->slot((int)i, k), ns = m->pat->nslots;
	float a[9];
	cudaStream_t st = stream_of(m);
	cudaError_t e = cudaSuccess;
	for (int p = 0; p < 9 && e == cudaSuccess; ++p)
		e = cudaMemcpyAsync(a + p, m->val + p * ns + s, sizeof(float), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return cuda_fail(e, "sparse_mat33_get_block");
	for (int t = 0; t < 9; ++t) block[t] = a[plane_of_b3(t)];
	return B3G_OK;
}

extern "C" int b3g_sparse_mat33_export(b3g_sparse_mat33* m, uint32_t* row_ptr, uint32_t* cols, float* blocks,
                                      uint64_t capacity, uint64_t* count)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (!row_ptr || !count) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	rc = sp_flush(m);
	if (rc != B3G_OK) return rc;
	const uint64_t nb = m->pat ? m->pat->blocks() : 0;
	*count = nb;
	if (nb > capacity) return fail(B3G_ERROR_INVALID_ARGUMENT, "%llu blocks do not fit a capacity of %llu",
	                                (unsigned long long)nb, (unsigned long long)capacity);
	if (nb && (!cols || !blocks)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null array");
	row_ptr[0] = 0;
	if (!m->pat)
	{
		for (uint32_t i = 0; i < m->n; ++i) row_ptr[i + 1] = 0;
		return B3G_OK;
	}
	std::vector<float> h;
	rc = sp_download(m, h);
	if (rc != B3G_OK) return rc;
	const SpPattern* P = m->pat.get();
	const size_t ns = P->nslots;
	uint64_t c = 0;
	std::vector<std::pair<int, int>> row;
	for (uint32_t i = 0; i < m->n; ++i)
	{
		row.clear();
		for (int k = 0; k < P->rp[i + 1] - P->rp[i]; ++k) row.push_back({P->cols[P->rp[i] + k], k});
		std::sort(row.begin(), row.end());
		for (auto& e : row)
		{
			const size_t s = P->slot((int)i, e.second);
			cols[c] = (uint32_t)e.first;
			for (int t = 0; t < 9; ++t) blocks[9 * c + t] = h[plane_of_b3(t) * ns + s];
			++c;
		}
		row_ptr[i + 1] = (uint32_t)c;
	}
	return B3G_OK;
}

extern "C" int b3g_sparse_mat33_to_dense(b3g_sparse_mat33* m, float* out)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	if (!out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	rc = sp_flush(m);
	if (rc != B3G_OK) return rc;
	const size_t AM = 3 * (size_t)m->n;
	std::fill(out, out + AM * AM, 0.0f);
	if (!m->pat) return B3G_OK;
	std::vector<float> h;
	rc = sp_download(m, h);
	if (rc != B3G_OK) return rc;
	const SpPattern* P = m->pat.get();
	for (uint32_t i = 0; i < m->n; ++i)
		for (int k = 0; k < P->rp[i + 1] - P->rp[i]; ++k)
		{
			const size_t s = P->slot((int)i, k);
			const size_t j = (size_t)P->cols[P->rp[i] + k];
			for (int r = 0; r < 3; ++r)
				for (int c = 0; c < 3; ++c) out[(3 * i + r) + AM * (3 * j + c)] = h[(3 * r + c) * P->nslots + s];
		}
	return B3G_OK;
}

extern "C" int b3g_sparse_mat33_clear(b3g_sparse_mat33* m)
{
	int rc = check_ctx(m);
	if (rc != B3G_OK) return rc;
	cudaStreamSynchronize(stream_of(m));
	m->release_device();
	m->q_i.clear();
	m->q_j.clear();
	m->q_op.clear();
	m->q_blk.clear();
	return B3G_OK;
}

extern "C" int b3g_sparse_mat33_zero_values(b3g_sparse_mat33* m)
{
	int rc = check_ctx(m);
	if (rc == B3G_OK) rc = sp_flush(m);
	if (rc != B3G_OK || !m->pat) return rc;
	cudaError_t e = cudaMemsetAsync(m->val, 0, 9 * m->pat->nslots * sizeof(float), stream_of(m));
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "sparse_mat33_zero_values");
}

// the common front of the matrix operations: checks, queued writes applied, out's own queue
// dropped when out is overwritten
static int sp_prepare(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_sparse_mat33* b,
                      const b3g_diag_mat33* d)
{
	int rc = check_ctx(out);
	if (rc == B3G_OK && a) rc = check_sp(a, out->n, "operand a");
	if (rc == B3G_OK && b) rc = check_sp(b, out->n, "operand b");
	if (rc == B3G_OK && d) rc = check_diag(d, out->n, "diagonal operand");
	if (rc == B3G_OK && a) rc = same_ctx(out, a);
	if (rc == B3G_OK && b) rc = same_ctx(out, b);
	if (rc == B3G_OK && d) rc = same_ctx(out, d);
	if (rc == B3G_OK && a) rc = sp_flush(const_cast<b3g_sparse_mat33*>(a));
	if (rc == B3G_OK && b) rc = sp_flush(const_cast<b3g_sparse_mat33*>(b));
	if (rc == B3G_OK) rc = sp_flush(out);
	return rc;
}

extern "C" int b3g_sparse_mat33_copy(b3g_sparse_mat33* out, const b3g_sparse_mat33* a)
{
	if (!a) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	int rc = sp_prepare(out, a, nullptr, nullptr);
	if (rc != B3G_OK || out == a) return rc;
	if (!a->pat)
	{
		out->release_device();
		return B3G_OK;
	}
	return sp_combine(out, a->pat, a, nullptr, combine_defaults());
}

static int sp_addsub(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_sparse_mat33* b, float sign)
{
	if (!a || !b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	int rc = sp_prepare(out, a, b, nullptr);
	if (rc != B3G_OK) return rc;
	if (!a->pat && !b->pat)
	{
		out->release_device();
		return B3G_OK;
	}
	PatPtr P;
	rc = union_of(out->ctx, out->n, a->pat, b->pat, &P);
	if (rc != B3G_OK) return rc;
	Combine C = combine_defaults();
	C.beta = sign;
	return sp_combine(out, P, a, b, C);
}

extern "C" int b3g_sparse_mat33_add(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_sparse_mat33* b)
{
	return sp_addsub(out, a, b, 1.0f);
}
extern "C" int b3g_sparse_mat33_sub(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_sparse_mat33* b)
{
	return sp_addsub(out, a, b, -1.0f);
}

// out = a +- d (gset = 0), or out's diagonal := d then - a (the reference's b3Sub(out, D, B))
static int sp_with_diag(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d, float gamma,
                        float beta, int gset)
{
	if (!a || !d) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	int rc = sp_prepare(out, a, nullptr, d);
	if (rc != B3G_OK) return rc;
	if (out->n == 0) return B3G_OK;
	Combine C = combine_defaults();
	C.G = d->d;
	C.gamma = gamma;
	C.gset = gset;
	if (!gset)
	{
		// the diagonal pattern is always present, so a's pattern (or the diagonal alone) serves
		PatPtr P = a->pat;
		if (!P)
		{
			std::vector<std::pair<int, int>> none;
			rc = make_pattern(out->ctx->device, out->n, none, &P);
			if (rc != B3G_OK) return rc;
		}
		return sp_combine(out, P, a, nullptr, C);
	}
	// out(i, i) = d_i over out's current blocks, then out -= a
	PatPtr P;
	PatPtr base = out->pat;
	if (!base)
	{
		std::vector<std::pair<int, int>> none;
		rc = make_pattern(out->ctx->device, out->n, none, &base);
		if (rc != B3G_OK) return rc;
	}
	rc = union_of(out->ctx, out->n, base, a->pat, &P);
	if (rc != B3G_OK) return rc;
	C.beta = beta;
	// the A term is out itself (its diagonal replaced by d), the B term the subtracted matrix
	b3g_sparse_mat33* cur = out;
	if (!out->pat)
	{
		C.G = d->d;
		return sp_combine(out, P, nullptr, a, C);
	}
	return sp_combine(out, P, cur, a, C);
}

extern "C" int b3g_sparse_mat33_add_diag(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d)
{
	return sp_with_diag(out, a, d, 1.0f, 1.0f, 0);
}
extern "C" int b3g_sparse_mat33_sub_diag(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d)
{
	return sp_with_diag(out, a, d, -1.0f, 1.0f, 0);
}
extern "C" int b3g_sparse_mat33_diag_add(b3g_sparse_mat33* out, const b3g_diag_mat33* d, const b3g_sparse_mat33* a)
{
	return sp_with_diag(out, a, d, 1.0f, 1.0f, 0);
}
extern "C" int b3g_sparse_mat33_diag_sub(b3g_sparse_mat33* out, const b3g_diag_mat33* d, const b3g_sparse_mat33* b)
{
	return sp_with_diag(out, b, d, 1.0f, -1.0f, 1);
}

extern "C" int b3g_sparse_mat33_scale(b3g_sparse_mat33* out, float s, const b3g_sparse_mat33* b)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	int rc = sp_prepare(out, b, nullptr, nullptr);
	if (rc != B3G_OK) return rc;
	if (s == 0.0f) return B3G_OK;  // sparse_mat33.h:518-521: out is left as it is
	if (!b->pat)
	{
		out->release_device();
		return B3G_OK;
	}
	Combine C = combine_defaults();
	C.alpha = s;
	C.scaleA = 1;
	return sp_combine(out, b->pat, b, nullptr, C);
}

static int sp_diag_mul(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d, bool left)
{
	if (!a || !d) return fail(B3G_ERROR_INVALID_ARGUMENT, "null container");
	int rc = sp_prepare(out, a, nullptr, d);
	if (rc != B3G_OK) return rc;
	if (!a->pat)
	{
		out->release_device();
		return B3G_OK;
	}
	Combine C = combine_defaults();
	if (left) C.DL = d->d;
	else C.DR = d->d;
	return sp_combine(out, a->pat, a, nullptr, C);
}

extern "C" int b3g_sparse_mat33_diag_mul(b3g_sparse_mat33* out, const b3g_diag_mat33* d, const b3g_sparse_mat33* b)
{
	return sp_diag_mul(out, b, d, true);
}
extern "C" int b3g_sparse_mat33_mul_diag(b3g_sparse_mat33* out, const b3g_sparse_mat33* a, const b3g_diag_mat33* d)
{
	return sp_diag_mul(out, a, d, false);
}

extern "C" int b3g_sparse_mat33_mul_vec(b3g_dense_vec3* out, b3g_sparse_mat33* a, const b3g_dense_vec3* v)
{
	int rc = check_ctx(out);
	if (rc == B3G_OK) rc = check_sp(a, out->n, "matrix");
	if (rc == B3G_OK) rc = check_vec(v, out->n, "vector");
	if (rc == B3G_OK) rc = same_ctx(out, a);
	if (rc == B3G_OK) rc = same_ctx(out, v);
	if (rc != B3G_OK) return rc;
	if (out == v) return fail(B3G_ERROR_INVALID_ARGUMENT, "b3g_sparse_mat33_mul_vec: out must not be the input vector");
	rc = sp_flush(a);
	if (rc == B3G_OK) rc = vec_flush(const_cast<b3g_dense_vec3*>(v));
	if (rc != B3G_OK) return rc;
	out->q_idx.clear();
	out->q_op.clear();
	out->q_val.clear();
	cudaStream_t st = stream_of(out);
	cudaError_t e;
	if (!a->pat) e = cudaMemsetAsync(out->d, 0, 4 * (size_t)out->n * sizeof(float), st);  // out.SetZero()
	else
	{
		const SpPattern* P = a->pat.get();
		k_sp_mul_vec<<<grid_of((size_t)P->nslices * 32, kT), kT, 0, st>>>((int)a->n, P->d_slice_ptr, P->d_col, P->nslots,
		                                                                   a->val, v->d, out->d);
		e = cudaGetLastError();
	}
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "sparse_mat33_mul_vec");
}

// ------------------------------------------------------------------ solvers
namespace {

int work_for(b3g_context* ctx, uint32_t n, SparseWork** out)
{
	if (!ctx->sparse_work) ctx->sparse_work = new SparseWork();
	SparseWork* w = ctx->sparse_work;
	cudaError_t e = w->vecs.ensure(9 * 4 * std::max<size_t>(n, 1) * sizeof(float));
	if (e == cudaSuccess && !w->sc) e = cudaMalloc(&w->sc, sizeof(Scalars));
	if (e == cudaSuccess && !w->partials)
	{
		e = cudaMalloc(&w->partials, (kMaxPartials + 1) * sizeof(double));
		if (e == cudaSuccess) e = cudaMemset(w->partials, 0, (kMaxPartials + 1) * sizeof(double));
		w->sum = w->partials + kMaxPartials;
	}
	if (e != cudaSuccess) return cuda_fail(e, "sparse solver workspace");
	*out = w;
	return B3G_OK;
}

float* work_vec(SparseWork* w, uint32_t n, int k) { return (float*)w->vecs.p + (size_t)k * 4 * std::max<size_t>(n, 1); }

// The PCG of the body step on a matrix in pattern P with values A: x (in/out, 4-wide) solves
// A x = b; minv is filled by the caller. Waits; returns the final scalars.
int run_cg(b3g_context* ctx, SparseWork* w, const SpPattern* P, const float* A, uint32_t n, const float* b, float* x,
           float* minv, uint32_t max_it, double tol, Scalars* out)
{
	DevBody D;
	std::memset(&D, 0, sizeof(D));
	D.n = (int)n;
	D.nslices = P->nslices;
	D.nslots = (int)P->nslots;
	D.slice_ptr = P->d_slice_ptr;
	D.col = P->d_col;
	D.A32 = const_cast<float*>(A);
	D.Minv = minv;
	D.precond = B3G_PRECOND_JACOBI;
	D.pb = const_cast<float*>(b);
	D.r = work_vec(w, n, 0);
	D.d = work_vec(w, n, 1);
	D.d2 = work_vec(w, n, 2);
	D.q = work_vec(w, n, 3);
	D.s = work_vec(w, n, 4);
	D.py = x;
	D.xff = nullptr;
	D.sc = w->sc;
	D.partials = w->partials;
	cudaStream_t st = ctx->stream;
	const int refresh = 50;  // sparse_solver.cpp:83
	cudaError_t e = op_begin(D, st, (int)max_it, tol * tol, refresh, 0.0);
	if (e == cudaSuccess) e = op_pcg_init(D, kP32, st);
	int done = 0;
	for (uint32_t it = 0; it < max_it && e == cudaSuccess && !done; it += kPcgChunk)
	{
		for (uint32_t j = it; j < std::min<uint32_t>(it + kPcgChunk, max_it) && e == cudaSuccess; ++j)
			e = op_pcg_iteration(D, kP32, (int)j, refresh, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(&ctx->h_scalars->done, &w->sc->done, sizeof(int), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		done = ctx->h_scalars->done;
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_scalars, w->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return cuda_fail(e, "sparse CG");
	*out = *ctx->h_scalars;
	return B3G_OK;
}

} // namespace

extern "C" int b3g_sparse_solve_cg(b3g_solve_cg_output* output, const b3g_solve_cg_input* input)
{
	if (!output || !input || !input->A || !input->b || !output->x) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	b3g_sparse_mat33* A = input->A;
	int rc = check_ctx(A);
	if (rc == B3G_OK) rc = check_vec(input->b, A->n, "b");
	if (rc == B3G_OK) rc = check_vec(output->x, A->n, "x");
	if (rc == B3G_OK) rc = same_ctx(A, input->b);
	if (rc == B3G_OK) rc = same_ctx(A, output->x);
	if (rc != B3G_OK) return rc;
	if (!(input->tolerance > 0.0f && input->tolerance < 1.0f))
		return fail(B3G_ERROR_INVALID_ARGUMENT, "tolerance must lie in (0, 1) (sparse_solver.cpp:36)");
	if (output->x == input->b) return fail(B3G_ERROR_INVALID_ARGUMENT, "x must not be b");
	rc = sp_flush(A);
	if (rc == B3G_OK) rc = vec_flush(const_cast<b3g_dense_vec3*>(input->b));
	if (rc == B3G_OK) rc = vec_flush(output->x);
	if (rc != B3G_OK) return rc;
	output->iterations = 0;
	output->error = 0.0;
	output->status = B3G_SOLVE_CONVERGED;
	const uint32_t n = A->n;
	if (n == 0) return B3G_OK;
	b3g_context* ctx = A->ctx;
	PatPtr P = A->pat;
	if (!P)
	{
		// no blocks: A = 0, the reference's Jacobi divides by zero; the diagonal pattern keeps
		// the kernels' layout valid and the status reports it
		std::vector<std::pair<int, int>> none;
		rc = make_pattern(ctx->device, n, none, &P);
		if (rc != B3G_OK) return rc;
		rc = sp_set_pattern(A, P);
		if (rc != B3G_OK) return rc;
	}
	SparseWork* w;
	rc = work_for(ctx, n, &w);
	if (rc != B3G_OK) return rc;
	float* minv = work_vec(w, n, 5);
	k_sp_jacobi<<<grid_of(n, kT), kT, 0, ctx->stream>>>((int)n, P->d_slice_ptr, P->nslots, A->val, minv);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return cuda_fail(e, "sparse CG");
	Scalars sc;
	rc = run_cg(ctx, w, P.get(), A->val, n, input->b->d, output->x->d, minv, input->max_iterations, input->tolerance, &sc);
	if (rc != B3G_OK) return rc;
	output->iterations = (uint32_t)sc.iter;
	output->error = sc.delta;
	output->status = sc.status;
	return B3G_OK;
}

extern "C" int b3g_sparse_solve_be(b3g_solve_be_output* output, const b3g_solve_be_input* in)
{
	if (!output || !in || !output->x || !output->v || !in->x0 || !in->v0 || !in->fe || !in->M || !in->y || !in->S ||
	    !in->z || !in->force_model.apply_forces)
		return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	const uint32_t n = in->dof_count;
	int rc = check_vec(in->x0, n, "x0");
	if (rc == B3G_OK) rc = check_vec(in->v0, n, "v0");
	if (rc == B3G_OK) rc = check_vec(in->fe, n, "fe");
	if (rc == B3G_OK) rc = check_vec(in->y, n, "y");
	if (rc == B3G_OK) rc = check_vec(in->z, n, "z");
	if (rc == B3G_OK) rc = check_vec(output->x, n, "x");
	if (rc == B3G_OK) rc = check_vec(output->v, n, "v");
	if (rc == B3G_OK) rc = check_diag(in->M, n, "M");
	if (rc == B3G_OK) rc = check_diag(in->S, n, "S");
	if (rc != B3G_OK) return rc;
	b3g_context* ctx = in->x0->ctx;
	const SparseObject* objs[] = {in->v0, in->fe, in->y, in->z, output->x, output->v, in->M, in->S};
	for (const SparseObject* o : objs)
		if (o->ctx != ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "containers of different contexts");
	if (!(in->h > 0.0f)) return fail(B3G_ERROR_INVALID_ARGUMENT, "h must be > 0");
	if (!(in->sub_tolerance > 0.0f && in->sub_tolerance < 1.0f))
		return fail(B3G_ERROR_INVALID_ARGUMENT, "sub_tolerance must lie in (0, 1) (sparse_solver.cpp:36)");
	const b3g_dense_vec3* vin[] = {in->x0, in->v0, in->fe, in->y, in->z};
	for (const b3g_dense_vec3* v : vin)
	{
		rc = vec_flush(const_cast<b3g_dense_vec3*>(v));
		if (rc != B3G_OK) return rc;
	}
	SparseWork* w;
	rc = work_for(ctx, n, &w);
	if (rc != B3G_OK) return rc;
	// the force model's containers and the iterate, kept in the workspace (patterns reused)
	auto ensure_vec = [&](b3g_dense_vec3** v) -> int {
		if (*v && (*v)->n == n) return B3G_OK;
		if (*v) b3g_dense_vec3_destroy(*v);
		*v = nullptr;
		return b3g_dense_vec3_create(ctx, n, v);
	};
	auto ensure_sp = [&](b3g_sparse_mat33** m) -> int {
		if (*m && (*m)->n == n) return B3G_OK;
		if (*m) b3g_sparse_mat33_destroy(*m);
		*m = nullptr;
		return b3g_sparse_mat33_create(ctx, n, m);
	};
	rc = ensure_vec(&w->xi);
	if (rc == B3G_OK) rc = ensure_vec(&w->vi);
	if (rc == B3G_OK) rc = ensure_vec(&w->fi);
	if (rc == B3G_OK) rc = ensure_sp(&w->dfdx);
	if (rc == B3G_OK) rc = ensure_sp(&w->dfdv);
	if (rc != B3G_OK) return rc;
	cudaStream_t st = ctx->stream;
	float* py = work_vec(w, n, 6);
	float* wv = work_vec(w, n, 7);
	float* pb = work_vec(w, n, 8);
	float* minv = work_vec(w, n, 5);
	cudaError_t e = cudaMemsetAsync(py, 0, 4 * (size_t)std::max<uint32_t>(n, 1) * sizeof(float), st);
	if (e != cudaSuccess) return cuda_fail(e, "sparse BE");
	rc = b3g_dense_vec3_copy(w->xi, in->x0);
	if (rc == B3G_OK) rc = b3g_dense_vec3_copy(w->vi, in->v0);
	if (rc != B3G_OK) return rc;
	const float h = in->h;
	const double eps2 = (double)in->tolerance * (double)in->tolerance;
	double error = 0.0, error0 = 0.0;
	uint32_t iteration = 0;
	int status = B3G_SOLVE_CONVERGED;
	while (iteration < in->max_iterations)
	{
		rc = b3g_dense_vec3_set_zero(w->fi);
		if (rc == B3G_OK) rc = b3g_sparse_mat33_zero_values(w->dfdx);
		if (rc == B3G_OK) rc = b3g_sparse_mat33_zero_values(w->dfdv);
		if (rc != B3G_OK) return rc;
		b3g_sparse_force_solver_data data;
		data.h = h;
		data.inv_h = in->inv_h;
		data.x = w->xi;
		data.v = w->vi;
		data.f = w->fi;
		data.dfdx = w->dfdx;
		data.dfdv = w->dfdv;
		in->force_model.apply_forces(in->force_model.user, &data);
		rc = vec_flush(w->fi);
		if (rc == B3G_OK) rc = sp_flush(w->dfdx);
		if (rc == B3G_OK) rc = sp_flush(w->dfdv);
		if (rc == B3G_OK) rc = vec_flush(w->xi);
		if (rc == B3G_OK) rc = vec_flush(w->vi);
		if (rc != B3G_OK) return rc;
		// the union of the two Jacobians' patterns and the maps into each, rebuilt when either
		// pattern changed
		const uint64_t idx = w->dfdx->pat ? w->dfdx->pat->id : 0, idv = w->dfdv->pat ? w->dfdv->pat->id : 0;
		if (!w->sys || w->sys_x != idx || w->sys_v != idv || w->sys->n != n)
		{
			PatPtr P;
			std::vector<std::pair<int, int>> pairs;
			pattern_pairs(w->dfdx->pat.get(), pairs);
			pattern_pairs(w->dfdv->pat.get(), pairs);
			rc = make_pattern(ctx->device, n, pairs, &P);
			if (rc != B3G_OK) return rc;
			std::vector<int> mx = slot_map(P.get(), w->dfdx->pat.get());
			std::vector<int> mv = slot_map(P.get(), w->dfdv->pat.get());
			const size_t ns = std::max<size_t>(P->nslots, 1);
			e = w->maps.ensure(2 * ns * sizeof(int));
			if (e == cudaSuccess) e = cudaMemcpy(w->maps.p, mx.data(), ns * sizeof(int), cudaMemcpyHostToDevice);
			if (e == cudaSuccess) e = cudaMemcpy((int*)w->maps.p + ns, mv.data(), ns * sizeof(int), cudaMemcpyHostToDevice);
			if (e == cudaSuccess) e = w->pA.ensure(9 * ns * sizeof(float));
			if (e != cudaSuccess) return cuda_fail(e, "sparse BE system");
			w->sys = P;
			w->sys_x = idx;
			w->sys_v = idv;
		}
		const SpPattern* P = w->sys.get();
		const size_t ns = std::max<size_t>(P->nslots, 1);
		BeSystem E;
		E.n = (int)n;
		E.slice_ptr = P->d_slice_ptr;
		E.col = P->d_col;
		E.ns = P->nslots;
		E.mapX = (const int*)w->maps.p;
		E.X = w->dfdx->val;
		E.nsX = w->dfdx->pat ? w->dfdx->pat->nslots : 0;
		E.mapV = (const int*)w->maps.p + ns;
		E.V = w->dfdv->val;
		E.nsV = w->dfdv->pat ? w->dfdv->pat->nslots : 0;
		E.M = in->M->d;
		E.S = in->S->d;
		E.h = h;
		E.hh = h * h;
		E.v0 = in->v0->d;
		E.v = w->vi->d;
		E.fe = in->fe->d;
		E.f = w->fi->d;
		E.w = wv;
		E.z = in->z->d;
		E.pA = (float*)w->pA.p;
		E.pb = pb;
		E.minv = minv;
		if (n > 0)
		{
			k_be_w<<<grid_of(n, kT), kT, 0, st>>>(wv, in->x0->d, w->xi->d, w->vi->d, in->y->d, h, (int)n);
			k_be_system<<<grid_of((size_t)P->nslices * 32, kT), kT, 0, st>>>(E);
		}
		e = cudaGetLastError();
		if (e != cudaSuccess) return cuda_fail(e, "sparse BE system");
		Scalars sc;
		std::memset(&sc, 0, sizeof(sc));
		if (n > 0)
		{
			rc = run_cg(ctx, w, P, (const float*)w->pA.p, n, pb, py, minv, in->max_sub_iterations, in->sub_tolerance, &sc);
			if (rc != B3G_OK) return rc;
		}
		status = sc.status;
		const uint32_t sub = (uint32_t)sc.iter;
		output->min_sub_iterations = std::min(output->min_sub_iterations, sub);
		output->max_sub_iterations = std::max(output->max_sub_iterations, sub);
		const int g = grid_of(n, kT);
		if (n > 0)
		{
			k_be_update<<<g, kT, 0, st>>>(w->xi->d, w->vi->d, in->x0->d, in->y->d, py, in->z->d, h, (int)n, w->partials);
			k_sum_partials<<<1, 256, 0, st>>>(w->partials, g, w->sum);
			e = cudaGetLastError();
			double err = 0.0;
			if (e == cudaSuccess) e = cudaMemcpyAsync(&err, w->sum, sizeof(double), cudaMemcpyDeviceToHost, st);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			if (e != cudaSuccess) return cuda_fail(e, "sparse BE update");
			error = err;
		}
		else
			error = 0.0;
		// sparse_force_solver.cpp:205-228
		if (iteration == 0)
		{
			error0 = error;
			if (error <= eps2) break;
		}
		else if (error <= eps2 * error0)
			break;
		++iteration;
	}
	rc = b3g_dense_vec3_copy(output->x, w->xi);
	if (rc == B3G_OK) rc = b3g_dense_vec3_copy(output->v, w->vi);
	if (rc != B3G_OK) return rc;
	e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return cuda_fail(e, "sparse BE");
	output->iterations = iteration;
	output->error = error;
	output->status = status;
	return B3G_OK;
}
