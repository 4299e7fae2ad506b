// Persistent batch kernel: many independent bodies step in one launch.
//
// A body is owned by a team: either a thread-block cluster of CL CTAs (large bodies) or a
// single CTA (small bodies). The team runs the whole implicit step of its body without leaving
// the kernel: element phase, row assembly, PCG, final update. Team-wide synchronisation is the
// hardware cluster barrier (or __syncthreads for one CTA); dot products are reduced per warp by
// shuffles, per CTA through shared memory and across the cluster through distributed shared
// memory, always in the same order, so every thread of the team holds the same bitwise value
// and takes the same solver decisions without a round trip to global memory. There is no
// spin-wait anywhere: the only inter-CTA waits are hardware barriers between CTAs that the
// cluster launch guarantees to be co-resident.
//
// Work distribution: bodies are sorted by size (largest first). Clusters first take large bodies
// from a global counter; when those run out every CTA takes small bodies on its own.
//
// This header holds the kernel templates; persistent_{f32,f64,bf16}.cu instantiate one
// precision each (compiled in parallel) and persistent.cu dispatches.
#pragma once

#include "device.cuh"
#include "ops.h"

#include <atomic>
#include <cooperative_groups.h>
#include <type_traits>
#include <utility>

namespace cg = cooperative_groups;

namespace b3g {

struct BatchParams
{
	const DevBody* bodies;
	const int* big;
	int nbig;
	const int* small;
	int nsmall;
	unsigned* queue;
	int steps;
	float h;
	int newton;
	int max_iter;
	double tol2;
	int refresh;
	double newton_tol2;
	unsigned long long* prof;  // optional: kPhases cycle counters per CTA
	// flat: the single Newton iteration's elements and rows ran in the flat launches (their
	// numbering below); the PCG launch then starts by summing delta0 = r.s itself
	int flat;
	const unsigned* elem_off;
	const unsigned* slice_off;
	unsigned nelem;
	unsigned nslices;
	int nbodies;
	int tets_only;   // every body: tetrahedra only, no contact spheres (the row assembly's short form)
	int filter;      // filtered contacts: bodies with a constraint buffer (filt) are stepped in that mode
	// flat launches over part of the numbering: elements [g_begin, nelem), slices [s_begin,
	// nslices); rows_per_sm > 0 caps the row launch at that many CTAs per SM (0: all resident)
	unsigned g_begin;
	unsigned s_begin;
	int rows_per_sm;
};

namespace {

// resident CTAs per SM the team assembly's register budget is sized for (128 registers a thread)
#ifndef B3G_BATCH_MIN_BLOCKS
#define B3G_BATCH_MIN_BLOCKS (B3G_PCG_THREADS >= 512 ? 1 : 2)
#endif

constexpr int kPThreads = B3G_PCG_THREADS;  // ops.h
constexpr int kPWarps = kPThreads / 32;

struct TeamShared
{
	double wp[2][kPWarps];
	double slot[2];
	int item;
	int pad;
};

template <int CL>
struct Team
{
	TeamShared* sh;
	int parity;
	int rank;

	__device__ void sync()
	{
		if (CL == 1) __syncthreads();
		else cg::this_cluster().sync();
	}
	__device__ int tid() const { return rank * kPThreads + (int)threadIdx.x; }
	__device__ int nthreads() const { return CL * kPThreads; }
	__device__ int warp() const { return rank * kPWarps + ((int)threadIdx.x >> 5); }
	__device__ int nwarps() const { return CL * kPWarps; }

	// Team-wide sum; every thread of the team returns the same value (fixed summation order).
	__device__ double reduce(double v)
	{
		const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
		v = warp_sum(v);
		if (lane == 0) sh->wp[parity][w] = v;
		__syncthreads();
		double t = 0.0;
#pragma unroll
		for (int k = 0; k < kPWarps; ++k) t += sh->wp[parity][k];
		if (CL > 1)
		{
			if (threadIdx.x == 0) sh->slot[parity] = t;
			cg::cluster_group cl = cg::this_cluster();
			cl.sync();
			double u = 0.0;
			if (lane < CL) u = *cl.map_shared_rank(&sh->slot[parity], lane);
			t = warp_sum(u);
		}
		parity ^= 1;
		return t;
	}
};


// Phases timed by the optional instrumentation (cycles of thread 0 of each CTA, barriers and
// reductions included in the phase that ends with them). The direction update runs inside the
// SpMV sweep, so kPhDir stays zero; its slot keeps the numbering the host reads.
enum { kPhElem = 0, kPhAsm = 1, kPhSpmv = 2, kPhUpdate = 3, kPhDir = 4, kPhFinal = 5, kPhIdle = 6, kPhases = 8 };

struct PhaseClock
{
	unsigned long long* slot;
	long long t;
	__device__ void start(unsigned long long* p)
	{
		slot = p ? p + (size_t)blockIdx.x * kPhases : nullptr;
		if (slot) t = clock64();
	}
	__device__ void tick(int phase)
	{
		if (!slot) return;
		long long now = clock64();
		if (threadIdx.x == 0) slot[phase] += (unsigned long long)(now - t);
		t = now;
	}
};

// PCG update of two rows (slices sl and sl + stride of one warp) with every load issued before
// the first store: x += alpha d and, unless this is a refresh iteration, r -= alpha q,
// s = M^-1 r. Returns the rows' r.s.
template <class TV, class LD>
__device__ __forceinline__ double update_two(const DevBody& B, TV* __restrict__ py, const TV* __restrict__ d,
                                             TV* __restrict__ r, const TV* __restrict__ q, TV* __restrict__ s,
                                             int i0, int i1, bool ok1, TV alpha, bool refresh)
{
	const int ii[2] = {i0, i1};
	const bool ok[2] = {true, ok1};
	TV x[2][3], dd[2][3], rr[2][3], qq[2][3];
#pragma unroll
	for (int u = 0; u < 2; ++u)
		if (ok[u])
		{
			vld<TV, LD>(py, ii[u], x[u]);
			vld<TV, LD>(d, ii[u], dd[u]);
			if (!refresh)
			{
				vld<TV, LD>(r, ii[u], rr[u]);
				vld<TV, LD>(q, ii[u], qq[u]);
			}
		}
	double part = 0.0;
#pragma unroll
	for (int u = 0; u < 2; ++u)
	{
		if (!ok[u]) continue;
		TV nx[3];
#pragma unroll
		for (int c = 0; c < 3; ++c) nx[c] = x[u][c] + alpha * dd[u][c];
		vst(py, ii[u], nx);
		if (refresh) continue;
		TV nr[3], ss[3];
#pragma unroll
		for (int c = 0; c < 3; ++c) nr[c] = rr[u][c] - alpha * qq[u][c];
		precond_row<TV, LD>(B, ii[u], nr, ss);
		vst(r, ii[u], nr);
		vst(s, ii[u], ss);
		part += dot3<TV>(nr, ss);
	}
	return part;
}

// r = pb - A x, s = M^-1 r for the rows of one warp's slices (init / refresh); optionally d = s
template <class TA, class TV, class LD>
__device__ __forceinline__ double residual_rows(const DevBody& B, const TA* A, const TV* x, int s0, int stride,
                                                bool set_d)
{
	const int lane = threadIdx.x & 31;
	double part = 0.0;
	for (int sl = s0; sl < B.nslices; sl += stride)
	{
		const int i = sl * kSlice + lane;
		if (i >= B.n) continue;
		const int base = B.slice_ptr[sl], w = (B.slice_ptr[sl + 1] - base) / kSlice;
		TV o[3], b[3], rr[3], ss[3];
		spmv_row<TA, TV, LD, MatVia<LD>>(A, B.col, B.nslots, base, w, lane, x, o);
		vld<TV, LD>((const TV*)B.pb, i, b);
#pragma unroll
		for (int c = 0; c < 3; ++c) rr[c] = b[c] - o[c];
		precond_row<TV, LD>(B, i, rr, ss);
		vst((TV*)B.r, i, rr);
		vst((TV*)B.s, i, ss);
		if (set_d) vst((TV*)B.d, i, ss);
		part += dot3<TV>(rr, ss);
	}
	return part;
}

// The direction and A times it by linearity, for the rows of one warp's slices: d = s + beta d
// and q = A s + beta q (d = s, q = A s on a solve's first iteration), and this warp's part of
// d.q. The SpMV gathers only s, which the update sweep finished before its reduction (a team
// barrier), so no direction sweep and no barrier of its own precede it. d and q stay row-local.
template <class TA, class TV, class LD>
__device__ __forceinline__ double spmv_lin_rows(const DevBody& B, const TA* A, const TV* s, TV* d, TV* q, TV beta,
                                                bool first, int s0, int stride)
{
	const int lane = threadIdx.x & 31;
	double part = 0.0;
	for (int sl = s0; sl < B.nslices; sl += stride)
	{
		const int i = sl * kSlice + lane;
		if (i >= B.n) continue;
		const int base = B.slice_ptr[sl], w = (B.slice_ptr[sl + 1] - base) / kSlice;
		TV o[3], dd[3];
		spmv_row<TA, TV, LD, MatVia<LD>>(A, B.col, B.nslots, base, w, lane, s, o);
		vld<TV, LD>(s, i, dd);
		if (!first)
		{
			TV dp[3], qp[3];
			vld<TV, LD>(d, i, dp);
			vld<TV, LD>(q, i, qp);
#pragma unroll
			for (int c = 0; c < 3; ++c)
			{
				dd[c] = dd[c] + beta * dp[c];
				o[c] = o[c] + beta * qp[c];
			}
		}
		vst(q, i, o);
		vst(d, i, dd);
		part += dot3<TV>(dd, o);
	}
	return part;
}

// Filtered-contact forms of the row assembly and of the final update, out of line so that the
// default forms inlined in the team kernels keep their register allocation.
template <class TA, class TV, class LD>
__device__ __noinline__ double assemble_row_filtered(const DevBody& B, int sl, int lane, const StepParams& sp,
                                                     bool init)
{
	return assemble_row<TA, TV, LD, true>(B, sl, lane, sp, init);
}

__device__ __noinline__ void contact_filter_vertex_ool(const DevBody& B, int i, float h)
{
	contact_filter_vertex(B, i, h);
}

template <class TV, class LD>
__device__ __noinline__ double final_vertex_filtered(const DevBody& B, int i, float h, bool first, bool finish)
{
	return final_vertex<TV, LD, true>(B, i, h, first, finish);
}

// Result of one PCG solve of a team.
struct SolveOut
{
	int iter;
	int status;
	double delta;
};

// The preconditioned CG of one body by one team, from r, s, d, py set up by the assembly (or a
// warm start) with r.s = delta0 (sparse_solver.cpp:57-108 with the true-residual refresh).
template <int CL, class TA, class TV, class LD>
__device__ SolveOut team_pcg(Team<CL>& T, const DevBody& B, const BatchParams& P, bool bf16, double delta0,
                             PhaseClock& pc)
{
	const int lane = threadIdx.x & 31;
	const TA* Asp = (sizeof(TA) == sizeof(float) && !bf16) ? (const TA*)B.A32 : (const TA*)B.Alo;
	TV* py = (TV*)B.py;
	TV* r = (TV*)B.r;
	TV* s = (TV*)B.s;
	TV* d = (TV*)B.d;
	TV* q = (TV*)B.q;
	SolveOut out;
	out.status = B3G_SOLVE_CONVERGED;
	out.iter = 0;
	double delta = delta0;
	bool pending = false;
	bool done;
	if (!isfinite(delta0))
	{
		out.status = B3G_SOLVE_NONFINITE;
		done = true;
	}
	else if (delta0 <= P.tol2 * delta0)
	{
		out.status = B3G_SOLVE_CONVERGED;
		done = true;
	}
	else if (P.max_iter <= 0)
	{
		out.status = B3G_SOLVE_MAX_ITERATIONS;
		done = true;
	}
	else
		done = false;
	int iter = 0;
	TV bt = (TV)0;
	while (!done)
	{
		// d = s + beta d, q = A d (as A s + beta q), alpha = delta / d.q
		double part = spmv_lin_rows<TA, TV, LD>(B, Asp, s, d, q, bt, iter == 0, T.warp(), T.nwarps());
		const double dq = T.reduce(part);
		pc.tick(kPhSpmv);
		if (!isfinite(dq))
		{
			out.status = B3G_SOLVE_NONFINITE;
			break;
		}
		if (!(dq > 0.0))
		{
			out.status = B3G_SOLVE_BREAKDOWN;
			break;
		}
		const TV alpha = (TV)(delta / dq);
		const bool refresh = (P.refresh > 0 && (iter % P.refresh) == 0) || pending;
		part = 0.0;
		for (int sl = T.warp(); sl < B.nslices; sl += T.nwarps())
		{
			const int i0 = sl * kSlice + lane;
			if (i0 >= B.n) continue;
			part += update_two<TV, LD>(B, py, d, r, q, s, i0, i0, false, alpha, refresh);
		}
		if (refresh)
		{
			// sparse_solver.cpp:83-90: r = b - A x with the full-precision blocks
			T.sync();
			part = (sizeof(TA) == sizeof(double))
			           ? residual_rows<TA, TV, LD>(B, Asp, py, T.warp(), T.nwarps(), false)
			           : residual_rows<float, TV, LD>(B, B.A32, py, T.warp(), T.nwarps(), false);
		}
		const double dn = T.reduce(part);
		pc.tick(kPhUpdate);
		const double beta = dn / delta;
		delta = dn;
		iter += 1;
		if (!isfinite(dn))
		{
			out.status = B3G_SOLVE_NONFINITE;
			break;
		}
		bool conv = dn <= P.tol2 * delta0;
		if (bf16 && conv && !refresh)
		{
			pending = true;
			conv = false;
		}
		if (refresh) pending = false;
		if (conv)
		{
			out.status = B3G_SOLVE_CONVERGED;
			break;
		}
		if (iter >= P.max_iter)
		{
			out.status = B3G_SOLVE_MAX_ITERATIONS;
			break;
		}
		bt = (TV)beta;
	}
	out.iter = iter;
	out.delta = delta;
	return out;
}

// Element phase and row assembly of one Newton iteration; returns the team's r.s (the PCG's
// delta0). k > 0 warm-starts from the previous solution: r = pb - A py.
template <int CL, class TA, class TV, class LD>
__device__ double team_assemble(Team<CL>& T, const DevBody& B, const BatchParams& P, bool bf16, int k, PhaseClock& pc)
{
	const int lane = threadIdx.x & 31;
	StepParams sp;
	sp.h = P.h;
	sp.first_newton = k == 0 ? 1 : 0;
	if (k == 0 && B.filt)
	{
		// filtered contacts: the contact update and each vertex's constraint at the step's start
		for (int i = T.tid(); i < B.n; i += T.nthreads()) contact_filter_vertex_ool(B, i, P.h);
		T.sync();
	}
	for (int e = T.tid(); e < B.nt; e += T.nthreads()) tet_element<LD>(B, e, sp);
	for (int e = T.tid(); e < B.ntr; e += T.nthreads()) tri_element<LD>(B, e, sp);
	for (int e = T.tid(); e < B.ns; e += T.nthreads()) spring_element<LD>(B, e, sp);
	for (int e = T.tid(); e < B.nbw; e += T.nthreads()) bw_element<LD>(B, e, sp);
	for (int e = T.tid(); e < B.nms; e += T.nthreads()) mouse_element<LD>(B, e, sp);
	T.sync();
	pc.tick(kPhElem);
	double part = 0.0;
	for (int sl = T.warp(); sl < B.nslices; sl += T.nwarps())
		part += B.filt ? assemble_row_filtered<TA, TV, LD>(B, sl, lane, sp, k == 0)
		               : assemble_row<TA, TV, LD>(B, sl, lane, sp, k == 0);
	if (k > 0)
	{
		const TA* Asp = (sizeof(TA) == sizeof(float) && !bf16) ? (const TA*)B.A32 : (const TA*)B.Alo;
		T.sync();
		part = (sizeof(TA) == sizeof(double))
		           ? residual_rows<TA, TV, LD>(B, Asp, (const TV*)B.py, T.warp(), T.nwarps(), true)
		           : residual_rows<float, TV, LD>(B, B.A32, (const TV*)B.py, T.warp(), T.nwarps(), true);
	}
	const double delta0 = T.reduce(part);
	pc.tick(kPhAsm);
	return delta0;
}

// Final update of a single-Newton step (state, friction, clearing, new contacts) and the
// step's statistics.
template <int CL, class TV, class LD>
__device__ void team_finish(Team<CL>& T, const DevBody& B, const BatchParams& P, const SolveOut& so, double delta0,
                            int newton_iters, int min_it, int max_it, unsigned long long iters_all, double err,
                            PhaseClock& pc)
{
	T.sync();
	if (T.tid() == 0)
	{
		Scalars* sc = B.sc;
		sc->iter = so.iter;
		sc->delta = so.delta;
		sc->delta0 = delta0;
		sc->status = so.status;
		sc->min_it = min_it;
		sc->max_it = max_it;
		sc->newton_iter = newton_iters;
		sc->newton_err = err;
		sc->done = 1;
		if (sc->fault) sc->status = B3G_SOLVE_DEVICE_TIMEOUT;
		sc->total_iters += iters_all;
		sc->total_steps += 1ull;
	}
}

// The whole implicit step of one body by one team (any number of Newton iterations); mirrors
// the per-op path of kernels.cu phase for phase (same device functions, same reduction
// decisions).
template <int CL, class TA, class TV>
__device__ void team_step(Team<CL>& T, const DevBody& B, const BatchParams& P, bool bf16)
{
	// A single-CTA team reads what its own threads wrote behind __syncthreads: ordinary (L1)
	// loads are coherent there. Cluster teams read other SMs' writes: L2-coherent loads.
	typedef typename std::conditional<CL == 1, LdPlain, LdCG>::type LD;
	const int lane = threadIdx.x & 31;
	const float h = P.h;
	int min_it = 0x7fffffff, max_it = 0, newton_done_at = 0;
	double delta0 = 0.0, err = 0.0, err0 = 0.0;
	unsigned long long iters_all = 0ull;
	SolveOut so;
	so.iter = 0;
	so.status = B3G_SOLVE_CONVERGED;
	so.delta = 0.0;
	PhaseClock pc;
	pc.start(P.prof);
	if (T.tid() == 0) B.sc->fault = 0;  // ordered before any SpMV by the element-phase barrier
	for (int k = 0; k < P.newton; ++k)
	{
		const bool finish = P.newton == 1;
		delta0 = team_assemble<CL, TA, TV, LD>(T, B, P, bf16, k, pc);
		so = team_pcg<CL, TA, TV, LD>(T, B, P, bf16, delta0, pc);
		min_it = so.iter < min_it ? so.iter : min_it;
		max_it = so.iter > max_it ? so.iter : max_it;
		iters_all += (unsigned long long)so.iter;
		// every thread finished its PCG reads before the final update rewrites x / v
		T.sync();
		double part = 0.0;
		for (int sl = T.warp(); sl < B.nslices; sl += T.nwarps())
		{
			const int i = sl * kSlice + lane;
			if (i < B.n)
				part += B.filt ? final_vertex_filtered<TV, LD>(B, i, h, k == 0, finish)
				               : final_vertex<TV, LD>(B, i, h, k == 0, finish);
		}
		err = T.reduce(part);
		pc.tick(kPhFinal);
		if (k == 0) err0 = err;
		newton_done_at = k + 1;
		if (finish) break;
		const bool ndone = k == 0 ? err <= P.newton_tol2 : err <= P.newton_tol2 * err0;
		if (ndone || k == P.newton - 1)
		{
			T.sync();
			for (int sl = T.warp(); sl < B.nslices; sl += T.nwarps())
			{
				const int i = sl * kSlice + lane;
				if (i < B.n) post_vertex<LD>(B, i, h);
			}
			break;
		}
	}
	team_finish<CL, TV, LD>(T, B, P, so, delta0, newton_done_at, min_it, max_it, iters_all, err, pc);
}

// Single-Newton step split in two launches so that each part runs with its own register budget
// (the element and assembly code needs 128 registers a thread, the PCG far fewer, and more warps
// per SM hide more of its memory latency). Part 1: elements and assembly; the PCG's delta0 goes
// to the body's scalars.
template <int CL, class TA, class TV>
__device__ void team_step_assemble(Team<CL>& T, const DevBody& B, const BatchParams& P, bool bf16)
{
	typedef typename std::conditional<CL == 1, LdPlain, LdCG>::type LD;
	PhaseClock pc;
	pc.start(P.prof);
	if (T.tid() == 0) B.sc->fault = 0;
	const double delta0 = team_assemble<CL, TA, TV, LD>(T, B, P, bf16, 0, pc);
	if (T.tid() == 0) B.sc->delta0 = delta0;
}

// Part 2: the PCG, the final update and the statistics.
template <int CL, class TA, class TV>
__device__ void team_step_solve(Team<CL>& T, const DevBody& B, const BatchParams& P, bool bf16)
{
	typedef typename std::conditional<CL == 1, LdPlain, LdCG>::type LD;
	const int lane = threadIdx.x & 31;
	PhaseClock pc;
	pc.start(P.prof);
	double delta0;
	if (P.flat)
	{
		// the flat row launch left r and s: delta0 = r.s, summed in the order the team assembly
		// sums it (each warp its slices, then the team), so it is the same value bitwise
		double part = 0.0;
		for (int sl = T.warp(); sl < B.nslices; sl += T.nwarps())
		{
			const int i = sl * kSlice + lane;
			if (i >= B.n) continue;
			TV rr[3], ss[3];
			vld<TV, LD>((const TV*)B.r, i, rr);
			vld<TV, LD>((const TV*)B.s, i, ss);
			part += dot3<TV>(rr, ss);
		}
		delta0 = T.reduce(part);
		if (T.tid() == 0)
		{
			B.sc->fault = 0;
			B.sc->delta0 = delta0;
		}
	}
	else
		delta0 = __ldcg(&B.sc->delta0);
	const SolveOut so = team_pcg<CL, TA, TV, LD>(T, B, P, bf16, delta0, pc);
	T.sync();
	double part = 0.0;
	for (int sl = T.warp(); sl < B.nslices; sl += T.nwarps())
	{
		const int i = sl * kSlice + lane;
		if (i < B.n)
			part += B.filt ? final_vertex_filtered<TV, LD>(B, i, P.h, true, true) : final_vertex<TV, LD>(B, i, P.h, true, true);
	}
	const double err = T.reduce(part);
	pc.tick(kPhFinal);
	team_finish<CL, TV, LD>(T, B, P, so, delta0, 1, so.iter, so.iter, (unsigned long long)so.iter, err, pc);
}

__device__ void load_body(DevBody* dst, const DevBody* src)
{
	const int words = (int)(sizeof(DevBody) / sizeof(int));
	const int* s = (const int*)src;
	int* d = (int*)dst;
	for (int k = threadIdx.x; k < words; k += blockDim.x) d[k] = __ldcg(s + k);
}

#ifndef B3G_SOLVE_MIN_BLOCKS  // resident CTAs per SM of the PCG launch (64 registers a thread)
#define B3G_SOLVE_MIN_BLOCKS (B3G_PCG_THREADS >= 512 ? 2 : 4)
#endif

// Launch phases: the whole step (any number of Newton iterations), or the two parts of a
// single-Newton step. Each part takes its work from its own pair of counters.
enum { kPhaseWhole = 0, kPhaseAssemble = 1, kPhaseSolve = 2 };

template <int CL, class TA, class TV, int PH>
__device__ __forceinline__ void team_run(Team<CL>& T, const DevBody& B, const BatchParams& P, bool bf16)
{
	if (PH == kPhaseWhole) team_step<CL, TA, TV>(T, B, P, bf16);
	else if (PH == kPhaseAssemble) team_step_assemble<CL, TA, TV>(T, B, P, bf16);
	else team_step_solve<CL, TA, TV>(T, B, P, bf16);
}

template <int CL, class TA, class TV, int PH>
__global__ void __launch_bounds__(kPThreads, PH == kPhaseSolve ? B3G_SOLVE_MIN_BLOCKS : B3G_BATCH_MIN_BLOCKS)
k_batch(BatchParams P, int bf16)
{
	__shared__ TeamShared sh;
	__shared__ __align__(16) DevBody sb;
	unsigned* queue = P.queue + (PH == kPhaseSolve ? 2 : 0);

	if (CL > 1)
	{
		cg::cluster_group cl = cg::this_cluster();
		Team<CL> T;
		T.sh = &sh;
		T.parity = 0;
		T.rank = (int)cl.block_rank();
		for (;;)
		{
			if (T.rank == 0 && threadIdx.x == 0) sh.item = (int)atomicAdd(queue, 1u);
			cl.sync();
			const int item = *cl.map_shared_rank(&sh.item, 0);
			cl.sync();
			if (item >= P.nbig) break;
			load_body(&sb, P.bodies + P.big[item]);
			__syncthreads();
			for (int st = 0; st < P.steps; ++st) team_run<CL, TA, TV, PH>(T, sb, P, bf16 != 0);
			cl.sync();
		}
	}
	Team<1> T1;
	T1.sh = &sh;
	T1.parity = 0;
	T1.rank = 0;
	for (;;)
	{
		if (threadIdx.x == 0) sh.item = (int)atomicAdd(queue + 1, 1u);
		__syncthreads();
		const int item = sh.item;
		__syncthreads();
		if (item >= P.nsmall) break;
		load_body(&sb, P.bodies + P.small[item]);
		__syncthreads();
		for (int st = 0; st < P.steps; ++st) team_run<1, TA, TV, PH>(T1, sb, P, bf16 != 0);
		__syncthreads();
	}
}

// Clusters of more than 8 CTAs are a non-portable size the kernel has to opt in to.
template <int CL, class TA, class TV, int PH>
cudaError_t allow_cluster()
{
	if (CL <= 8) return cudaSuccess;
	return cudaFuncSetAttribute(k_batch<CL, TA, TV, PH>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
}

template <int CL, class TA, class TV, int PH>
cudaError_t launch_ph(const BatchParams& P, int ctas, int bf16, cudaStream_t st)
{
	cudaError_t e = allow_cluster<CL, TA, TV, PH>();
	if (e != cudaSuccess) return e;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)ctas, 1, 1);
	cfg.blockDim = dim3(kPThreads, 1, 1);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = CL;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, k_batch<CL, TA, TV, PH>, P, bf16);
}

template <int CL, class TA, class TV, int PH>
int max_clusters_ph()
{
	if (allow_cluster<CL, TA, TV, PH>() != cudaSuccess) return 0;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(CL * 64, 1, 1);
	cfg.blockDim = dim3(kPThreads, 1, 1);
	cfg.dynamicSmemBytes = 0;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = CL;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	int n = 0;
	if (cudaOccupancyMaxActiveClusters(&n, k_batch<CL, TA, TV, PH>, &cfg) != cudaSuccess) return 0;
	return n;
}

// Co-resident clusters of the solve launch (more CTAs per SM than the assembly launch), queried
// once per instantiation.
template <int CL, class TA, class TV>
int solve_clusters()
{
	static std::atomic<int> cached(-1);
	int m = cached.load(std::memory_order_relaxed);
	if (m < 0)
	{
		m = max_clusters_ph<CL, TA, TV, kPhaseSolve>();
		cached.store(m, std::memory_order_relaxed);
	}
	return m;
}

// One step: the whole-step kernel for several Newton iterations, else the assembly launch
// (`ctas` CTAs) followed by the solve launch (as many CTAs as fit). part 1 / 2 issues only the
// assembly / solve launch of a single-Newton step (timed separately), 0 both.
template <int CL, class TA, class TV>
cudaError_t launch_cl(const BatchParams& P, int ctas, int bf16, int part, cudaStream_t st)
{
	if (P.newton > 1) return launch_ph<CL, TA, TV, kPhaseWhole>(P, ctas, bf16, st);
	if (part != 2 && !P.flat)
	{
		cudaError_t e = launch_ph<CL, TA, TV, kPhaseAssemble>(P, ctas, bf16, st);
		if (e != cudaSuccess || part == 1) return e;
	}
	const int m = solve_clusters<CL, TA, TV>();
	return launch_ph<CL, TA, TV, kPhaseSolve>(P, m > 0 ? m * CL : ctas, bf16, st);
}

// The body of flat item g: the last k with off[k] <= g.
__device__ __forceinline__ int flat_body(const unsigned* __restrict__ off, int nbodies, unsigned g)
{
	int lo = 0, hi = nbodies - 1;
	while (lo < hi)
	{
		const int mid = (lo + hi + 1) >> 1;
		if (__ldg(off + mid) <= g) lo = mid;
		else hi = mid - 1;
	}
	return lo;
}

// The row assembly of every body of a batch, one warp per slice over a flat numbering of all
// bodies' slices: no team, no barrier, and the load spreads evenly over the GPU whatever the
// bodies' sizes (the team launch's tail was set by its largest bodies). Element records come from
// the flat element launch before it, state from earlier launches: plain loads. The PCG launch
// sums delta0 = r.s per body itself.
#ifndef B3G_ROWS_THREADS
#define B3G_ROWS_THREADS 256     // threads per CTA of the flat row launch
#endif
#ifndef B3G_ROWS_MIN_BLOCKS
#define B3G_ROWS_MIN_BLOCKS 2    // resident CTAs per SM its register budget is sized for
#endif
constexpr int kRowsWarps = B3G_ROWS_THREADS / 32;

#ifndef B3G_ROWS_TETS_MIN_BLOCKS
#define B3G_ROWS_TETS_MIN_BLOCKS 3  // the tetrahedra-only row assembly fits more CTAs per SM
#endif

// FILT: some bodies have filtered contacts (their filt buffer set); each body takes its own form
template <class TA, class TV, bool TETS, bool FILT = false>
__global__ void __launch_bounds__(B3G_ROWS_THREADS, TETS ? B3G_ROWS_TETS_MIN_BLOCKS : B3G_ROWS_MIN_BLOCKS)
k_batch_rows(BatchParams P)
{
	// each warp's body descriptor, copied to shared memory: the row code's stores to global
	// memory cannot alias it there, so its fields need not be re-read after each store
	static_assert(sizeof(DevBody) % 8 == 0, "DevBody is copied in 8-byte words");
	__shared__ DevBody s_body[kRowsWarps];
	const int lane = threadIdx.x & 31;
	DevBody& B = s_body[threadIdx.x >> 5];
	StepParams sp;
	sp.h = P.h;
	sp.first_newton = 1;
	const unsigned nw = gridDim.x * kRowsWarps;
	for (unsigned g = P.s_begin + blockIdx.x * kRowsWarps + (threadIdx.x >> 5); g < P.nslices; g += nw)
	{
		const int b = flat_body(P.slice_off, P.nbodies, g);
		__syncwarp();
		{
			const unsigned long long* src = reinterpret_cast<const unsigned long long*>(P.bodies + b);
			unsigned long long* dst = reinterpret_cast<unsigned long long*>(&B);
			for (int w = lane; w < (int)(sizeof(DevBody) / 8); w += 32) dst[w] = __ldg(src + w);
		}
		__syncwarp();
		const int sl = (int)(g - __ldg(P.slice_off + b));
		if (FILT && B.filt) assemble_row_filtered<TA, TV, LdPlain>(B, sl, lane, sp, true);
		else assemble_row<TA, TV, LdPlain, false, TETS>(B, sl, lane, sp, true);
	}
}

template <class TA, class TV, bool TETS, bool FILT>
cudaError_t launch_rows_t(const BatchParams& P, cudaStream_t st)
{
	static const std::pair<int, int> resident = [] {  // SMs, resident CTAs per SM
		int dev = 0, sms = 0, per_sm = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_rows<TA, TV, TETS, FILT>, B3G_ROWS_THREADS, 0);
		return std::make_pair(std::max(1, sms), std::max(per_sm, 1));
	}();
	const int cap = resident.first * (P.rows_per_sm > 0 ? std::min(P.rows_per_sm, resident.second) : resident.second);
	const unsigned need = (P.nslices - P.s_begin + kRowsWarps - 1) / kRowsWarps;
	const int grid = (int)std::max(1u, std::min(need, (unsigned)cap));
	k_batch_rows<TA, TV, TETS, FILT><<<grid, B3G_ROWS_THREADS, 0, st>>>(P);
	return cudaGetLastError();
}

// the tetrahedra-only kernel when every body of the batch qualifies (P.tets_only), the kernel
// with both row forms when some body has filtered contacts (P.filter)
template <class TA, class TV>
cudaError_t launch_rows(const BatchParams& P, cudaStream_t st)
{
	if (P.filter) return launch_rows_t<TA, TV, false, true>(P, st);
	return P.tets_only ? launch_rows_t<TA, TV, true, false>(P, st) : launch_rows_t<TA, TV, false, false>(P, st);
}

template <class TA, class TV>
cudaError_t launch_prec(const BatchParams& P, int cluster, int ctas, int bf16, int part, cudaStream_t st)
{
	switch (cluster)
	{
	case 1: return launch_cl<1, TA, TV>(P, ctas, bf16, part, st);
	case 2: return launch_cl<2, TA, TV>(P, ctas, bf16, part, st);
	case 4: return launch_cl<4, TA, TV>(P, ctas, bf16, part, st);
	case 8: return launch_cl<8, TA, TV>(P, ctas, bf16, part, st);
	case 16: return launch_cl<16, TA, TV>(P, ctas, bf16, part, st);
	default: return cudaErrorInvalidValue;
	}
}

// Co-resident clusters of the assembly (and whole-step) launch; also primes the solve launch's
// count so that no occupancy query happens while a stream is being captured.
template <int CL, class TA, class TV>
int max_clusters()
{
	solve_clusters<CL, TA, TV>();
	return max_clusters_ph<CL, TA, TV, kPhaseAssemble>();
}

template <class TA, class TV>
int max_clusters_prec(int cluster)
{
	switch (cluster)
	{
	case 1: return max_clusters<1, TA, TV>();
	case 2: return max_clusters<2, TA, TV>();
	case 4: return max_clusters<4, TA, TV>();
	case 8: return max_clusters<8, TA, TV>();
	case 16: return max_clusters<16, TA, TV>();
	default: return 0;
	}
}

} // namespace

// per-precision entry points (persistent_f32.cu, persistent_f64.cu, persistent_bf16.cu)
cudaError_t launch_batch_f32(const BatchParams& P, int cluster, int ctas, int part, cudaStream_t st);
cudaError_t launch_batch_f64(const BatchParams& P, int cluster, int ctas, int part, cudaStream_t st);
cudaError_t launch_batch_bf16(const BatchParams& P, int cluster, int ctas, int part, cudaStream_t st);
cudaError_t launch_rows_f32(const BatchParams& P, cudaStream_t st);
cudaError_t launch_rows_f64(const BatchParams& P, cudaStream_t st);
cudaError_t launch_rows_bf16(const BatchParams& P, cudaStream_t st);
int max_clusters_f32(int cluster);
int max_clusters_f64(int cluster);
int max_clusters_bf16(int cluster);

} // namespace b3g
