// Per-op kernels of the single-body ("plain") path: one kernel per phase, grid-wide
// deterministic reductions (per-CTA partials summed in a fixed order by the last CTA to
// arrive), solver decisions taken on the device in Scalars.
#include "device.cuh"
#include "ops.h"

#include <cstdlib>
#include <utility>

#include <algorithm>

namespace b3g {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

int grid_for(int items, int per_block)
{
	int g = (items + per_block - 1) / per_block;
	if (g < 1) g = 1;
	if (g > kMaxPartials) g = kMaxPartials;
	return g;
}

// Sum `v` over the whole grid. Returns true in thread 0 of the last CTA to arrive, with the
// total in *total; the partials are summed in CTA order, so the result does not depend on
// arrival order.
__device__ bool grid_reduce(double v, double* partials, unsigned* counter, double* total)
{
	__shared__ double sh[32];
	__shared__ int last;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	v = warp_sum(v);
	if (lane == 0) sh[warp] = v;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double s = 0.0;
		for (int k = 0; k < nw; ++k) s += sh[k];
		partials[blockIdx.x] = s;
		__threadfence();
		unsigned prev = atomicAdd(counter, 1u);
		last = (prev == gridDim.x - 1) ? 1 : 0;
	}
	__syncthreads();
	if (!last) return false;
	__threadfence();
	double s = 0.0;
	for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) s += ((volatile double*)partials)[k];
	s = warp_sum(s);
	__syncthreads();
	if (lane == 0) sh[warp] = s;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double t = 0.0;
		for (int k = 0; k < nw; ++k) t += sh[k];
		*total = t;
		*counter = 0u;
	}
	return threadIdx.x == 0;
}

__device__ __forceinline__ bool finite_d(double x) { return isfinite(x); }

// PCG exit test at the top of the reference loop (sparse_solver.cpp:65-73), taken after the
// iteration counter moved.
__device__ void decide_after_reduction(Scalars* sc, double delta_new, bool bf16_mode, bool was_refresh)
{
	double delta_old = sc->delta;
	sc->delta = delta_new;
	sc->beta = delta_new / delta_old;
	sc->iter += 1;
	if (!finite_d(delta_new))
	{
		sc->status = B3G_SOLVE_NONFINITE;
		sc->done = 1;
		return;
	}
	bool conv = delta_new <= sc->tol2 * sc->delta0;
	if (bf16_mode && conv && !was_refresh)
	{
		// the recursive residual of the bf16 iteration drifts from the true one: confirm with a
		// true-residual refresh on the next iteration before stopping
		sc->pending_check = 1;
		conv = false;
	}
	if (conv)
	{
		sc->status = B3G_SOLVE_CONVERGED;
		sc->done = 1;
	}
	else if (sc->iter >= sc->max_iter)
	{
		sc->status = B3G_SOLVE_MAX_ITERATIONS;
		sc->done = 1;
	}
	if (was_refresh) sc->pending_check = 0;
}

__device__ __forceinline__ bool refresh_now(const Scalars* sc)
{
	return (sc->refresh > 0 && (sc->iter % sc->refresh) == 0) || sc->pending_check;
}

// ------------------------------------------------------------------ kernels
__global__ void k_begin(Scalars* sc, int max_it, double tol2, int refresh, double newton_tol2)
{
	sc->iter = 0;
	sc->max_iter = max_it;
	sc->done = 0;
	sc->status = B3G_SOLVE_CONVERGED;
	sc->tol2 = tol2;
	sc->refresh = refresh;
	sc->newton_iter = 0;
	sc->newton_done = 0;
	sc->newton_tol2 = newton_tol2;
	sc->newton_err = 0.0;
	sc->newton_err0 = 0.0;
	sc->min_it = 0x7fffffff;
	sc->max_it = 0;
	sc->counter = 0u;
	sc->pending_check = 0;
	sc->fault = 0;
	sc->delta = sc->delta0 = 0.0;
	sc->alpha = sc->beta = sc->dq = 0.0;
}

__global__ void k_newton_begin(Scalars* sc)
{
	sc->iter = 0;
	sc->done = 0;
	sc->pending_check = 0;
	sc->status = B3G_SOLVE_CONVERGED;
}

__global__ void __launch_bounds__(kThreads) k_tets(DevBody B, StepParams P)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.nt; e += gridDim.x * blockDim.x) tet_element(B, e, P);
}

__global__ void __launch_bounds__(kThreads) k_tris(DevBody B, StepParams P)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.ntr; e += gridDim.x * blockDim.x) tri_element(B, e, P);
}

__global__ void __launch_bounds__(kThreads) k_springs(DevBody B, StepParams P)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B.ns; e += gridDim.x * blockDim.x) spring_element(B, e, P);
}

// stretch/shear triangles and mouse springs in one launch: the triangles, then the springs
__global__ void __launch_bounds__(kThreads) k_cloth_forces(DevBody B, StepParams P)
{
	const int total = B.nbw + B.nms;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x)
	{
		if (e < B.nbw) bw_element(B, e, P);
		else mouse_element(B, e - B.nbw, P);
	}
}

// ------------------------------------------------------------------ ray casts
// b3TriangleShape::RayCast (triangle_shape.cpp:314-387) for the segment p1 + t d, t in [0, 1].
// Returns the fraction and the plane offset num = n . (A - p1), whose sign orients the normal.
__device__ __forceinline__ bool ray_triangle(float3 p1, float3 d, float3 A, float3 B, float3 C, float& t, float& num,
                                             float3& n)
{
	if (dot3(d, d) < kFltEps * kFltEps) return false;
	const float3 AB = B - A, AC = C - A;
	n = normalize3(cross3(AB, AC));
	num = dot3(n, A - p1);
	const float den = dot3(n, d);
	if (den == 0.0f) return false;
	t = num / den;
	if (t < 0.0f || 1.0f < t) return false;
	const float3 Q = p1 + t * d;
	const float3 QA = A - Q, QB = B - Q, QC = C - Q;
	const float3 N = cross3(AB, AC);
	const float u = dot3(cross3(QB, QC), N);
	const float v = dot3(cross3(QC, QA), N);
	const float w = dot3(cross3(QA, QB), N);
	return u >= 0.0f && v >= 0.0f && w >= 0.0f;
}

__device__ __forceinline__ unsigned long long ray_key(float t, unsigned tri)
{
	// a hit has 0 <= t <= 1, and non-negative floats order like their bit patterns; fmaxf maps
	// -0 (which passes the t < 0 test) to +0
	return ((unsigned long long)__float_as_uint(fmaxf(t, 0.0f)) << 32) | tri;
}

// grid.x strides over triangles, grid.y over segments; one 64-bit atomicMin per warp and segment
__global__ void __launch_bounds__(kThreads) k_ray_cast(DevBody B, int ntri, const float* __restrict__ seg,
                                                        unsigned count, unsigned long long* keys)
{
	const int lane = threadIdx.x & 31;
	for (unsigned r = blockIdx.y; r < count; r += gridDim.y)
	{
		const float3 p1 = f3(seg[6 * r], seg[6 * r + 1], seg[6 * r + 2]);
		const float3 d = f3(seg[6 * r + 3], seg[6 * r + 4], seg[6 * r + 5]) - p1;
		const int stride = gridDim.x * blockDim.x;
		for (int base = blockIdx.x * blockDim.x; base < ntri; base += stride)
		{
			const int e = base + threadIdx.x;
			unsigned long long key = ~0ull;
			if (e < ntri)
			{
				const uint4 id = B.tri[e];
				float t, num;
				float3 n;
				if (ray_triangle(p1, d, ld3(B.x, id.x), ld3(B.x, id.y), ld3(B.x, id.z), t, num, n))
					key = ray_key(t, (unsigned)e);
			}
#pragma unroll
			for (int o = 16; o > 0; o >>= 1)
			{
				const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
				key = other < key ? other : key;
			}
			if (lane == 0 && key != ~0ull) atomicMin(keys + r, key);
		}
	}
}

// One thread per segment: the winner's normal, oriented as the reference orients it.
__global__ void k_ray_finish(DevBody B, const float* __restrict__ seg, unsigned count,
                             const unsigned long long* __restrict__ keys, b3g_ray_hit* hits)
{
	const unsigned r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= count) return;
	b3g_ray_hit o;
	o.hit = 0;
	o.triangle = 0;
	o.fraction = 0.0f;
	o.normal[0] = o.normal[1] = o.normal[2] = 0.0f;
	const unsigned long long key = keys[r];
	if (key != ~0ull)
	{
		const unsigned e = (unsigned)(key & 0xffffffffu);
		const uint4 id = B.tri[e];
		const float3 p1 = f3(seg[6 * r], seg[6 * r + 1], seg[6 * r + 2]);
		const float3 d = f3(seg[6 * r + 3], seg[6 * r + 4], seg[6 * r + 5]) - p1;
		float t, num;
		float3 n;
		ray_triangle(p1, d, ld3(B.x, id.x), ld3(B.x, id.y), ld3(B.x, id.z), t, num, n);
		if (num > 0.0f) n = -n;
		o.hit = 1;
		o.triangle = e;
		o.fraction = __uint_as_float((unsigned)(key >> 32));
		o.normal[0] = n.x;
		o.normal[1] = n.y;
		o.normal[2] = n.z;
	}
	hits[r] = o;
}

__device__ void pcg_start(Scalars* sc, double delta0)
{
	sc->delta = delta0;
	sc->delta0 = delta0;
	sc->iter = 0;
	sc->pending_check = 0;
	if (!finite_d(delta0))
	{
		sc->status = B3G_SOLVE_NONFINITE;
		sc->done = 1;
	}
	else if (delta0 <= sc->tol2 * delta0)
	{
		sc->status = B3G_SOLVE_CONVERGED;
		sc->done = 1;
	}
	else if (sc->max_iter <= 0)
	{
		sc->status = B3G_SOLVE_MAX_ITERATIONS;
		sc->done = 1;
	}
	else
		sc->done = 0;
}

// Filtered contacts: the contact update and each vertex's constraint at the start of a step
__global__ void __launch_bounds__(kThreads) k_contact_filter(DevBody B, float h)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x)
		contact_filter_vertex(B, i, h);
}

template <class TA, class TV, bool FILTER>
__global__ void __launch_bounds__(kThreads) k_assemble(DevBody B, StepParams P, int init)
{
	const int lane = threadIdx.x & 31;
	double part = 0.0;
	for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < B.nslices; s += (gridDim.x * blockDim.x) >> 5)
		part += assemble_row<TA, TV, LdPlain, FILTER>(B, s, lane, P, init != 0);
	if (!init) return;
	double total;
	if (grid_reduce(part, B.partials, &B.sc->counter, &total)) pcg_start(B.sc, total);
}

// r = pb - A py, s = M^-1 r, d = s (warm start from the previous Newton iteration's solution)
template <class TA, class TV>
__global__ void __launch_bounds__(kThreads) k_pcg_init(DevBody B, const TA* A)
{
	const int lane = threadIdx.x & 31;
	double part = 0.0;
	for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < B.nslices; sl += (gridDim.x * blockDim.x) >> 5)
	{
		const int i = sl * kSlice + lane;
		if (i >= B.n) continue;
		const int base = B.slice_ptr[sl], w = (B.slice_ptr[sl + 1] - base) / kSlice;
		TV b[3], rr[3], ss[3];
		vld<TV, LdPlain>((const TV*)B.pb, i, b);
		if (B.xff)
		{
			// refinement: b - A x from the float-float solution in float-float, rounded once
			float qh[3], ql[3];
			spmv_row_ff(B.A32, B.col, B.nslots, base, w, lane, B.xff, qh, ql);
#pragma unroll
			for (int c = 0; c < 3; ++c) rr[c] = (TV)ff_residual((float)b[c], qh[c], ql[c]);
		}
		else
		{
			TV q[3];
			spmv_row<TA, TV>(A, B.col, B.nslots, base, w, lane, (const TV*)B.py, q);
#pragma unroll
			for (int c = 0; c < 3; ++c) rr[c] = b[c] - q[c];
		}
		precond_row<TV>(B, i, rr, ss);
		vst((TV*)B.r, i, rr);
		vst((TV*)B.s, i, ss);
		vst((TV*)B.d, i, ss);
		part += dot3<TV>(rr, ss);
	}
	double total;
	if (grid_reduce(part, B.partials, &B.sc->counter, &total)) pcg_start(B.sc, total);
}

// d' = s + beta d (d' = s on a solve's first iteration), q = A d' and alpha = delta / d'.q.
// q is formed by linearity, q = A s + beta q (the previous q, which is A d): the SpMV gathers only
// s, and each row updates its own d and q. Reads the direction from B.d and writes the new one to
// B.d2; the host swaps the two buffers every iteration.
#ifndef B3G_SPMV_MIN_BLOCKS
#define B3G_SPMV_MIN_BLOCKS 4   // 64 registers: 4 CTAs (32 warps) per SM hide more gather latency
#endif
template <class TA, class TV>
__global__ void __launch_bounds__(kThreads, B3G_SPMV_MIN_BLOCKS) k_dir_spmv_dot(DevBody B, const TA* A)
{
	if (B.sc->done) return;
	const int lane = threadIdx.x & 31;
	const bool first = B.sc->iter == 0;
	const TV beta = (TV)B.sc->beta;
	double part = 0.0;
	for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < B.nslices; sl += (gridDim.x * blockDim.x) >> 5)
	{
		const int i = sl * kSlice + lane;
		if (i >= B.n) continue;
		const int base = B.slice_ptr[sl], w = (B.slice_ptr[sl + 1] - base) / kSlice;
		TV o[3], dn[3];
		spmv_row<TA, TV>(A, B.col, B.nslots, base, w, lane, (const TV*)B.s, o);
		vld<TV, LdPlain>((const TV*)B.s, i, dn);
		if (!first)
		{
			TV dp[3], qp[3];
			vld<TV, LdPlain>((const TV*)B.d, i, dp);
			vld<TV, LdPlain>((const TV*)B.q, i, qp);
#pragma unroll
			for (int c = 0; c < 3; ++c)
			{
				dn[c] = dn[c] + beta * dp[c];
				o[c] = o[c] + beta * qp[c];
			}
		}
		vst((TV*)B.q, i, o);
		vst((TV*)B.d2, i, dn);
		part += dot3<TV>(dn, o);
	}
	double total;
	if (grid_reduce(part, B.partials, &B.sc->counter, &total))
	{
		Scalars* sc = B.sc;
		sc->dq = total;
		if (!finite_d(total))
		{
			sc->status = B3G_SOLVE_NONFINITE;
			sc->done = 1;
		}
		else if (!(total > 0.0))
		{
			sc->status = B3G_SOLVE_BREAKDOWN;
			sc->done = 1;
		}
		else
			sc->alpha = sc->delta / total;
	}
}

// x += alpha d' (d' in B.d2); unless this is a refresh iteration: r -= alpha q, s = M^-1 r, delta = r.s
template <class TV>
__global__ void __launch_bounds__(kThreads) k_update(DevBody B, int bf16_mode)
{
	Scalars* sc = B.sc;
	if (sc->done) return;
	const bool refresh = refresh_now(sc);
	const TV alpha = (TV)sc->alpha;
	double part = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x)
	{
		TV d[3], r[3], q[3], s[3];
		vld<TV, LdPlain>((const TV*)B.d2, i, d);  // this iteration's direction
		if (!refresh)
		{
			vld<TV, LdPlain>((const TV*)B.r, i, r);
			vld<TV, LdPlain>((const TV*)B.q, i, q);
		}
		if (B.xff)
		{
			// refinement: the solution accumulates in float-float (the product alpha d and its
			// rounding error are both added)
			float xh[3], xl[3];
			ff_ld(B.xff, i, xh, xl);
#pragma unroll
			for (int c = 0; c < 3; ++c)
			{
				const float p = __fmul_rn((float)alpha, (float)d[c]);
				ff_add(xh[c], xl[c], p, fmaf((float)alpha, (float)d[c], -p));
			}
			ff_st(B.xff, i, xh, xl);
		}
		else
		{
			TV x[3];
			vld<TV, LdPlain>((const TV*)B.py, i, x);
#pragma unroll
			for (int c = 0; c < 3; ++c) x[c] += alpha * d[c];
			vst((TV*)B.py, i, x);
		}
		if (refresh) continue;
#pragma unroll
		for (int c = 0; c < 3; ++c) r[c] -= alpha * q[c];
		precond_row<TV>(B, i, r, s);
		vst((TV*)B.r, i, r);
		vst((TV*)B.s, i, s);
		part += dot3<TV>(r, s);
	}
	if (refresh) return;
	double total;
	if (grid_reduce(part, B.partials, &sc->counter, &total)) decide_after_reduction(sc, total, bf16_mode != 0, false);
}

// refresh iteration: r = b - A x (sparse_solver.cpp:83-90), s = M^-1 r, delta = r.s
template <class TA, class TV>
__global__ void __launch_bounds__(kThreads) k_resid(DevBody B, const TA* A, int bf16_mode)
{
	Scalars* sc = B.sc;
	if (sc->done) return;
	if (!refresh_now(sc)) return;
	const int lane = threadIdx.x & 31;
	double part = 0.0;
	for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < B.nslices; sl += (gridDim.x * blockDim.x) >> 5)
	{
		const int i = sl * kSlice + lane;
		if (i >= B.n) continue;
		const int base = B.slice_ptr[sl], w = (B.slice_ptr[sl + 1] - base) / kSlice;
		TV b[3], rr[3], ss[3];
		vld<TV, LdPlain>((const TV*)B.pb, i, b);
		if (B.xff)
		{
			// refinement: b - A x from the float-float solution in float-float, rounded once
			float qh[3], ql[3];
			spmv_row_ff(B.A32, B.col, B.nslots, base, w, lane, B.xff, qh, ql);
#pragma unroll
			for (int c = 0; c < 3; ++c) rr[c] = (TV)ff_residual((float)b[c], qh[c], ql[c]);
		}
		else
		{
			TV q[3];
			spmv_row<TA, TV>(A, B.col, B.nslots, base, w, lane, (const TV*)B.py, q);
#pragma unroll
			for (int c = 0; c < 3; ++c) rr[c] = b[c] - q[c];
		}
		precond_row<TV>(B, i, rr, ss);
		vst((TV*)B.r, i, rr);
		vst((TV*)B.s, i, ss);
		part += dot3<TV>(rr, ss);
	}
	double total;
	if (grid_reduce(part, B.partials, &sc->counter, &total)) decide_after_reduction(sc, total, bf16_mode != 0, true);
}

// v = v + dv, x = x0 + h v + y, Newton error |dv|^2 (sparse_force_solver.cpp:194-223).
// mode 1 also finishes the step: friction, clearing of external forces and translations,
// new contacts (body.cpp:572-603).
template <class TV, bool FILTER>
__global__ void __launch_bounds__(kThreads) k_final(DevBody B, StepParams P, int mode)
{
	double part = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x)
		part += final_vertex<TV, LdPlain, FILTER>(B, i, P.h, P.first_newton != 0, mode == 1);
	double total;
	if (grid_reduce(part, B.partials, &B.sc->counter, &total))
	{
		Scalars* sc = B.sc;
		sc->newton_err = total;
		if (sc->newton_iter == 0) sc->newton_err0 = total;
		int it = sc->iter;
		sc->min_it = it < sc->min_it ? it : sc->min_it;
		sc->max_it = it > sc->max_it ? it : sc->max_it;
		// sparse_force_solver.cpp:205-223
		if (sc->newton_iter == 0) sc->newton_done = total <= sc->newton_tol2 ? 1 : 0;
		else sc->newton_done = total <= sc->newton_tol2 * sc->newton_err0 ? 1 : 0;
		sc->newton_iter += 1;
		sc->total_iters += (unsigned long long)it;
		if (mode == 1) sc->total_steps += 1ull;
	}
}

__global__ void __launch_bounds__(kThreads) k_post(DevBody B, float h)
{
	if (blockIdx.x == 0 && threadIdx.x == 0) B.sc->total_steps += 1ull;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x) post_vertex(B, i, h);
}

__global__ void __launch_bounds__(kThreads) k_nostep(DevBody B)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x)
	{
		float3 x = ld3(B.x, i);
		if (B.contacts)
			for (int k = 0; k < B.nw; ++k)
			{
				const int c = i * B.nw + k;
				if (B.c_exists[c] && (B.type[i] != B3G_DYNAMIC || !aabb_overlap(x, B.srad[i], B.shapes[k]))) B.c_exists[c] = 0;
				else if (B.c_exists[c])
				{
					B.c_nf[c] = 0.0f;
					B.c_apply[c] = 0;
				}
			}
		st3(B.fext, i, f3(0, 0, 0));
		st3(B.trans, i, f3(0, 0, 0));
		if (B.contacts) find_new_contacts(B, i, x);
	}
}

__global__ void k_accumulate(float* dst, const float* src, size_t n)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] += src[i];
}

// b3Particle::SetType (particle.cpp:58-87) for every vertex whose type changes: external force
// and translation cleared, velocity zeroed for static vertices, contacts destroyed.
__global__ void k_set_types(DevBody B, const int8_t* nt)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x)
	{
		int8_t t = nt[i];
		if (t == B.type[i]) continue;
		st3(B.fext, i, f3(0, 0, 0));
		st3(B.trans, i, f3(0, 0, 0));
		if (t == B3G_STATIC) st3(B.v, i, f3(0, 0, 0));
		for (int k = 0; k < B.nw; ++k) B.c_exists[i * B.nw + k] = 0;
		((int8_t*)B.type)[i] = t;
	}
}

__global__ void k_fill(float* p, size_t n, float v)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

// ------------------------------------------------------------------ BF16 mode: flexible outer CG
// Sum two values over the whole grid (like grid_reduce); true in thread 0 of the last CTA to
// arrive, with the totals in *ta, *tb, summed in CTA order.
__device__ bool grid_reduce2(double a, double b, double* partials, unsigned* counter, double* ta, double* tb)
{
	__shared__ double sa[32], sb[32];
	__shared__ int last;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	a = warp_sum(a);
	b = warp_sum(b);
	if (lane == 0)
	{
		sa[warp] = a;
		sb[warp] = b;
	}
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double x = 0.0, y = 0.0;
		for (int k = 0; k < nw; ++k)
		{
			x += sa[k];
			y += sb[k];
		}
		partials[2 * blockIdx.x] = x;
		partials[2 * blockIdx.x + 1] = y;
		__threadfence();
		unsigned prev = atomicAdd(counter, 1u);
		last = (prev == gridDim.x - 1) ? 1 : 0;
	}
	__syncthreads();
	if (!last) return false;
	__threadfence();
	double x = 0.0, y = 0.0;
	for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x)
	{
		x += ((volatile double*)partials)[2 * k];
		y += ((volatile double*)partials)[2 * k + 1];
	}
	x = warp_sum(x);
	y = warp_sum(y);
	__syncthreads();
	if (lane == 0)
	{
		sa[warp] = x;
		sb[warp] = y;
	}
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double u = 0.0, v = 0.0;
		for (int k = 0; k < nw; ++k)
		{
			u += sa[k];
			v += sb[k];
		}
		*ta = u;
		*tb = v;
		*counter = 0u;
	}
	return threadIdx.x == 0;
}

// Start of an inner BF16 solve M_bf16 z = r from z = 0: r_in = r, s = M^-1 r, d = s, delta0. If
// the outer solve is already done the inner one is marked done at once (every later launch of the
// outer iteration returns immediately).
__global__ void __launch_bounds__(kThreads) k_fcg_inner_init(DevBody B, const Scalars* outer)
{
	if (outer->done)
	{
		if (blockIdx.x == 0 && threadIdx.x == 0) B.sc->done = 1;
		return;
	}
	double part = 0.0;
	const float zero[3] = {0.0f, 0.0f, 0.0f};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x)
	{
		float r[3], sv[3];
		vld<float, LdPlain>((const float*)B.pb, i, r);
		precond_row<float>(B, i, r, sv);
		vst((float*)B.r, i, r);
		vst((float*)B.s, i, sv);
		vst((float*)B.d, i, sv);
		vst((float*)B.py, i, zero);
		part += dot3<float>(r, sv);
	}
	double total;
	if (grid_reduce(part, B.partials, &B.sc->counter, &total)) pcg_start(B.sc, total);
}

// gamma = z . q_prev (the flexible CG's orthogonalisation against the previous direction)
__global__ void __launch_bounds__(kThreads) k_fcg_gamma(DevBody B, const float* z, const float* q_prev,
                                                        FcgScalars* f, double* part)
{
	if (B.sc->done) return;
	double a = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += gridDim.x * blockDim.x)
	{
		float zz[3], qq[3];
		vld<float, LdPlain>(z, i, zz);
		vld<float, LdPlain>(q_prev, i, qq);
		a += dot3<float>(zz, qq);
	}
	double ta, tb;
	if (grid_reduce2(a, 0.0, part, &f->counter, &ta, &tb)) f->gamma = ta;
}

// p = z + beta p_prev with beta = -gamma / (p_prev . q_prev) (p = z on the first iteration), formed
// on the fly for every gathered column; q = A p with the FP32 blocks; p.q and p.r; alpha = p.r / p.q.
// p_prev is B.d, p is written to B.d2, q to B.q.
__global__ void __launch_bounds__(kThreads, B3G_SPMV_MIN_BLOCKS) k_fcg_dir_spmv(DevBody B, const float* z,
                                                                              FcgScalars* f, double* part, int first)
{
	Scalars* sc = B.sc;
	if (sc->done) return;
	const int lane = threadIdx.x & 31;
	const float beta = first ? 0.0f : (float)(-f->gamma / f->pq_prev);
	double pq = 0.0, pr = 0.0;
	for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < B.nslices; sl += (gridDim.x * blockDim.x) >> 5)
	{
		const int i = sl * kSlice + lane;
		if (i >= B.n) continue;
		const int base = B.slice_ptr[sl], w = (B.slice_ptr[sl + 1] - base) / kSlice;
		float o[3], dn[3], r[3];
		spmv_row_dir<float, float>(B.A32, B.col, B.nslots, base, w, lane, z, (const float*)B.d, beta, first != 0, o, dn);
		vld<float, LdPlain>((const float*)B.r, i, r);
		vst((float*)B.q, i, o);
		vst((float*)B.d2, i, dn);
		pq += dot3<float>(dn, o);
		pr += dot3<float>(dn, r);
	}
	double tq, tr;
	if (grid_reduce2(pq, pr, part, &f->counter, &tq, &tr))
	{
		f->pq_prev = tq;
		f->pq = tq;
		f->rho = tr;
		sc->dq = tq;
		if (!finite_d(tq) || !finite_d(tr))
		{
			sc->status = B3G_SOLVE_NONFINITE;
			sc->done = 1;
		}
		else if (!(tq > 0.0))
		{
			sc->status = B3G_SOLVE_BREAKDOWN;
			sc->done = 1;
		}
		else
			sc->alpha = tr / tq;
	}
}

StepParams dev_params(const StepParamsHost& P)
{
	StepParams p;
	p.h = P.h;
	p.first_newton = P.first_newton;
	return p;
}

int slice_grid(const DevBody& B) { return grid_for(B.nslices, kWarps); }

// Grid of the per-vertex kernels (vector update, final update): at most two CTAs per SM, each
// thread striding over several vertices. One vertex per thread (1024 CTAs on the 64³ block) made
// the vector update 1.6x slower: every CTA pays the reduction's fence and its atomic on one
// counter. Measured per 64³ step: 17.9 ms (one vertex a thread), 17.3 (4 CTAs/SM), 16.7 (2),
// 17.3 (1). B3G_VERTEX_CTAS overrides the cap (tuning knob, read once).
int vertex_grid(const DevBody& B)
{
	static const int cap = [] {
		const char* e = std::getenv("B3G_VERTEX_CTAS");
		if (e) return std::atoi(e);
		int dev = 0, sms = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		return 2 * sms;
	}();
	const int g = grid_for(B.n, kThreads);
	return cap > 0 && cap < g ? cap : g;
}

// SpMV grid: every CTA resident at once and the same whole number of slices per warp, so that
// no partial second wave trails the launch (64³ block: 8192 slices, 608 resident CTAs of 8 warps
// -> 2 slices a warp on 512 CTAs; measured 6 % faster per step than one slice a warp on 1024
// CTAs). B3G_SPMV_CTAS overrides the CTA count (tuning knob, read once).
template <class TA, class TV>
int spmv_grid(const DevBody& B)
{
	static const int cap = [] {
		const char* e = std::getenv("B3G_SPMV_CTAS");
		return e ? std::atoi(e) : 0;
	}();
	const int g = slice_grid(B);
	if (cap > 0) return cap < g ? cap : g;
	static const int resident = [] {
		int dev = 0, sms = 0, per_sm = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dir_spmv_dot<TA, TV>, kThreads, 0);
		return sms * per_sm;
	}();
	if (resident <= 0 || g <= resident) return g;
	const int per_warp = (B.nslices + resident * kWarps - 1) / (resident * kWarps);
	return (B.nslices + per_warp * kWarps - 1) / (per_warp * kWarps);
}

template <class TA, class TV>
cudaError_t launch_spmv(const DevBody& B, const TA* A, cudaStream_t st)
{
	k_dir_spmv_dot<TA, TV><<<spmv_grid<TA, TV>(B), kThreads, 0, st>>>(B, A);
	return cudaGetLastError();
}

} // namespace

cudaError_t op_begin(const DevBody& B, cudaStream_t st, int max_it, double tol2, int refresh, double newton_tol2)
{
	k_begin<<<1, 1, 0, st>>>(B.sc, max_it, tol2, refresh, newton_tol2);
	return cudaGetLastError();
}

cudaError_t op_ray_cast(const DevBody& B, int ntri, const float* segments, uint32_t count, unsigned long long* keys,
                        b3g_ray_hit* hits, cudaStream_t st)
{
	if (count == 0) return cudaSuccess;
	cudaError_t e = cudaMemsetAsync(keys, 0xff, count * sizeof(unsigned long long), st);
	if (e != cudaSuccess) return e;
	if (ntri > 0)
	{
		// enough CTAs over the triangles to fill the GPU for one segment, fewer per segment when
		// there are many segments
		static const int sms = [] {
			int dev = 0, n = 0;
			cudaGetDevice(&dev);
			cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
			return n > 0 ? n : 1;
		}();
		const int per_seg = std::max(1, std::min(grid_for(ntri, kThreads), 4 * sms / (int)std::min<uint32_t>(count, 64)));
		dim3 grid((unsigned)per_seg, std::min<uint32_t>(count, 65535u));
		k_ray_cast<<<grid, kThreads, 0, st>>>(B, ntri, segments, count, keys);
	}
	k_ray_finish<<<(count + 127) / 128, 128, 0, st>>>(B, segments, count, keys, hits);
	return cudaGetLastError();
}

cudaError_t op_newton_begin(const DevBody& B, cudaStream_t st)
{
	k_newton_begin<<<1, 1, 0, st>>>(B.sc);
	return cudaGetLastError();
}

cudaError_t op_elements(const DevBody& B, const StepParamsHost& Ph, cudaStream_t st)
{
	StepParams P = dev_params(Ph);
	if (B.nt > 0) k_tets<<<grid_for(B.nt, kThreads), kThreads, 0, st>>>(B, P);
	if (B.ntr > 0) k_tris<<<grid_for(B.ntr, kThreads), kThreads, 0, st>>>(B, P);
	if (B.ns > 0) k_springs<<<grid_for(B.ns, kThreads), kThreads, 0, st>>>(B, P);
	if (B.nbw + B.nms > 0) k_cloth_forces<<<grid_for(B.nbw + B.nms, kThreads), kThreads, 0, st>>>(B, P);
	return cudaGetLastError();
}

cudaError_t op_assemble(const DevBody& B, const StepParamsHost& Ph, int prec, bool init, cudaStream_t st)
{
	StepParams P = dev_params(Ph);
	int g = slice_grid(B);
	const int in = init ? 1 : 0;
	if (B.filt)
	{
		if (prec == kP64) k_assemble<double, double, true><<<g, kThreads, 0, st>>>(B, P, in);
		else if (prec == kPBF) k_assemble<__nv_bfloat16, float, true><<<g, kThreads, 0, st>>>(B, P, in);
		else k_assemble<float, float, true><<<g, kThreads, 0, st>>>(B, P, in);
	}
	else if (prec == kP64) k_assemble<double, double, false><<<g, kThreads, 0, st>>>(B, P, in);
	else if (prec == kPBF) k_assemble<__nv_bfloat16, float, false><<<g, kThreads, 0, st>>>(B, P, in);
	else k_assemble<float, float, false><<<g, kThreads, 0, st>>>(B, P, in);
	return cudaGetLastError();
}

cudaError_t op_contact_filter(const DevBody& B, float h, cudaStream_t st)
{
	k_contact_filter<<<vertex_grid(B), kThreads, 0, st>>>(B, h);
	return cudaGetLastError();
}

cudaError_t op_pcg_init(const DevBody& B, int prec, cudaStream_t st)
{
	int g = slice_grid(B);
	if (prec == kP64) k_pcg_init<double, double><<<g, kThreads, 0, st>>>(B, (const double*)B.Alo);
	else k_pcg_init<float, float><<<g, kThreads, 0, st>>>(B, B.A32);
	return cudaGetLastError();
}

unsigned pcg_resid_mask(int prec, int j0, int count, int refresh)
{
	unsigned m = 0;
	for (int k = 0; k < count && k < 32; ++k)
		if (prec == kPBF || (refresh > 0 && (j0 + k) % refresh == 0)) m |= 1u << k;
	return m;
}

void op_pcg_prime(const DevBody& B, int prec)
{
	(void)slice_grid(B);
	(void)vertex_grid(B);
	if (prec == kP64) (void)spmv_grid<double, double>(B);
	else if (prec == kPBF) (void)spmv_grid<__nv_bfloat16, float>(B);
	else (void)spmv_grid<float, float>(B);
}

cudaError_t op_pcg_iteration(const DevBody& D, int prec, int j, int refresh, cudaStream_t st)
{
	// direction buffers alternate: iteration j reads the direction from one and writes the new
	// one to the other
	DevBody B = D;
	if (j & 1) std::swap(B.d, B.d2);
	// the true-residual refresh runs when the iteration counter is a multiple of the period; in
	// bf16 mode it may also be requested by a pending convergence check, so it is always launched
	const bool resid = prec == kPBF || (refresh > 0 && j % refresh == 0);
	int gs = slice_grid(B), gv = vertex_grid(B);
	if (prec == kP64)
	{
		const double* A = (const double*)B.Alo;
		cudaError_t e = launch_spmv<double, double>(B, A, st);
		if (e != cudaSuccess) return e;
		k_update<double><<<gv, kThreads, 0, st>>>(B, 0);
		if (resid) k_resid<double, double><<<gs, kThreads, 0, st>>>(B, A, 0);
	}
	else if (prec == kPBF)
	{
		cudaError_t e = launch_spmv<__nv_bfloat16, float>(B, (const __nv_bfloat16*)B.Alo, st);
		if (e != cudaSuccess) return e;
		k_update<float><<<gv, kThreads, 0, st>>>(B, 1);
		k_resid<float, float><<<gs, kThreads, 0, st>>>(B, B.A32, 1);
	}
	else
	{
		cudaError_t e = launch_spmv<float, float>(B, B.A32, st);
		if (e != cudaSuccess) return e;
		k_update<float><<<gv, kThreads, 0, st>>>(B, 0);
		if (resid) k_resid<float, float><<<gs, kThreads, 0, st>>>(B, B.A32, 0);
	}
	return cudaGetLastError();
}

cudaError_t op_fcg_inner_begin(const DevBody& Bin, const Scalars* outer_sc, int max_it, double tol2, cudaStream_t st)
{
	k_begin<<<1, 1, 0, st>>>(Bin.sc, max_it, tol2, 0, 0.0);
	k_fcg_inner_init<<<vertex_grid(Bin), kThreads, 0, st>>>(Bin, outer_sc);
	return cudaGetLastError();
}

cudaError_t op_fcg_inner_iteration(const DevBody& Din, int j, cudaStream_t st)
{
	// the inner iteration of the body step's PCG with the BF16 blocks: fused direction / SpMV /
	// d.q, then x (= z) += alpha d, r -= alpha q, s = M^-1 r, r.s and the exit test; no refresh
	DevBody B = Din;
	if (j & 1) std::swap(B.d, B.d2);
	cudaError_t e = launch_spmv<__nv_bfloat16, float>(B, (const __nv_bfloat16*)B.Alo, st);
	if (e != cudaSuccess) return e;
	k_update<float><<<vertex_grid(B), kThreads, 0, st>>>(B, 0);
	return cudaGetLastError();
}

cudaError_t op_fcg_outer(const DevBody& Bo, const float* z, const float* q_prev, FcgScalars* f, double* part, int k,
                         cudaStream_t st)
{
	if (k > 0) k_fcg_gamma<<<vertex_grid(Bo), kThreads, 0, st>>>(Bo, z, q_prev, f, part);
	k_fcg_dir_spmv<<<spmv_grid<float, float>(Bo), kThreads, 0, st>>>(Bo, z, f, part, k == 0 ? 1 : 0);
	// x += alpha p (float-float), r -= alpha q, s = M^-1 r, r.s and the exit test; the true residual
	// r = b - A x (float-float) replaces the recursive one when the iteration is a refresh
	k_update<float><<<vertex_grid(Bo), kThreads, 0, st>>>(Bo, 0);
	k_resid<float, float><<<slice_grid(Bo), kThreads, 0, st>>>(Bo, Bo.A32, 0);
	return cudaGetLastError();
}

cudaError_t op_final(const DevBody& B, const StepParamsHost& Ph, int prec, int mode, cudaStream_t st)
{
	StepParams P = dev_params(Ph);
	int g = vertex_grid(B);
	if (B.filt)
	{
		if (prec == kP64) k_final<double, true><<<g, kThreads, 0, st>>>(B, P, mode);
		else k_final<float, true><<<g, kThreads, 0, st>>>(B, P, mode);
	}
	else if (prec == kP64) k_final<double, false><<<g, kThreads, 0, st>>>(B, P, mode);
	else k_final<float, false><<<g, kThreads, 0, st>>>(B, P, mode);
	return cudaGetLastError();
}

cudaError_t op_post(const DevBody& B, float h, cudaStream_t st)
{
	k_post<<<vertex_grid(B), kThreads, 0, st>>>(B, h);
	return cudaGetLastError();
}

cudaError_t op_nostep(const DevBody& B, cudaStream_t st)
{
	k_nostep<<<vertex_grid(B), kThreads, 0, st>>>(B);
	return cudaGetLastError();
}

// grid.y walks the bodies, grid.x (with a stride) the floats of one body
__global__ void __launch_bounds__(kThreads) k_batch_scatter_add(const XferBody* __restrict__ table, unsigned count,
                                                                 const float* __restrict__ src)
{
	for (unsigned b = blockIdx.y; b < count; b += gridDim.y)
	{
		const XferBody t = table[b];
		const float* s = src + t.off;
		for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < t.n3; k += gridDim.x * blockDim.x)
			t.fext[k] += s[k];
	}
}

__global__ void __launch_bounds__(kThreads) k_batch_gather(const XferBody* __restrict__ table, unsigned count,
                                                            float* __restrict__ dx, float* __restrict__ dv)
{
	for (unsigned b = blockIdx.y; b < count; b += gridDim.y)
	{
		const XferBody t = table[b];
		for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < t.n3; k += gridDim.x * blockDim.x)
		{
			if (dx) dx[t.off + k] = t.x[k];
			if (dv) dv[t.off + k] = t.v[k];
		}
	}
}

static dim3 xfer_grid(uint32_t count, uint32_t max_n3)
{
	return dim3((unsigned)std::max(1u, std::min<uint32_t>((max_n3 + kThreads - 1) / kThreads, 64u)),
	            std::min<uint32_t>(std::max(count, 1u), 65535u));
}

cudaError_t op_batch_scatter_add(const XferBody* table, uint32_t count, uint32_t max_n3, const float* src,
                                 cudaStream_t st)
{
	if (count == 0) return cudaSuccess;
	k_batch_scatter_add<<<xfer_grid(count, max_n3), kThreads, 0, st>>>(table, count, src);
	return cudaGetLastError();
}

cudaError_t op_batch_gather(const XferBody* table, uint32_t count, uint32_t max_n3, float* dst_x, float* dst_v,
                            cudaStream_t st)
{
	if (count == 0) return cudaSuccess;
	k_batch_gather<<<xfer_grid(count, max_n3), kThreads, 0, st>>>(table, count, dst_x, dst_v);
	return cudaGetLastError();
}

cudaError_t op_accumulate(float* dst, const float* src, size_t count, cudaStream_t st)
{
	if (count == 0) return cudaSuccess;
	int g = (int)((count + kThreads - 1) / kThreads);
	if (g > 4096) g = 4096;
	k_accumulate<<<g, kThreads, 0, st>>>(dst, src, count);
	return cudaGetLastError();
}

cudaError_t op_set_types(const DevBody& B, const int8_t* new_types, cudaStream_t st)
{
	k_set_types<<<vertex_grid(B), kThreads, 0, st>>>(B, new_types);
	return cudaGetLastError();
}

cudaError_t op_fill_f32(float* p, size_t count, float value, cudaStream_t st)
{
	if (count == 0) return cudaSuccess;
	int g = (int)((count + kThreads - 1) / kThreads);
	if (g > 4096) g = 4096;
	k_fill<<<g, kThreads, 0, st>>>(p, count, value);
	return cudaGetLastError();
}

} // namespace b3g
