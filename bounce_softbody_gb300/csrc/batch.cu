// Batched stepping of many independent bodies (b3g_step_batch): one persistent launch
// (persistent.cu) per call, captured once into a CUDA graph and replayed.
//
// Schedule: bodies are sorted by vertex count, largest first. Bodies with at least `threshold`
// vertices are stepped by clusters of `cluster` CTAs, the rest by single CTAs. The schedule
// (cluster size, threshold) is chosen per batch by an autotuner on the first call: it snapshots
// the mutable state of every body, times one step of each candidate schedule with CUDA events,
// restores the snapshot and keeps the fastest. Set B3G_AUTOTUNE=0 to use the size heuristic, or
// B3G_BATCH_SCHEDULE="cluster,threshold" to force a schedule.
#include "api_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

using namespace b3g;

struct Snapshot
{
	void* dst;
	const void* src;
	size_t bytes;
};

struct BatchCache
{
	std::vector<b3g_body*> bodies;
	int prec = 0, precond = 0;
	DevBody* d_bodies = nullptr;
	int* d_order = nullptr;      // cluster-stepped bodies, then the others, each longest first
	unsigned* d_queue = nullptr;
	std::vector<int> order;
	std::vector<int> iters;      // PCG iterations of each body's last step (0 = not known yet)
	int lpt = 0;                 // queues ordered by estimated solve time (1) or by size (0)
	int cluster = 1;
	int threshold = 1 << 30;
	int nbig = 0;
	int ctas = 0;
	bool tuned = false;
	// graph of (memset queue, batch launch) for one step with the current parameters
	cudaGraphExec_t graph = nullptr;
	float g_h = 0.0f;
	int g_steps = 0, g_newton = 0, g_max_iter = 0, g_refresh = 0;
	double g_tol2 = 0.0, g_ntol2 = 0.0;
	std::vector<std::pair<int, double>> tune_log;  // (cluster * 1e6 + threshold, ms)
	unsigned long long* d_prof = nullptr;          // phase cycle counters when B3G_PHASE_PROFILE=1
	unsigned* d_flat_off = nullptr;                 // flat numbering: element offsets, then slice offsets
	unsigned nelem = 0, nslices = 0;
	// split assembly: flat element / slice offsets of the first body of group 2 (0: no split),
	// CTAs per SM of group 2's element launch and of group 1's row launch
	unsigned elem_mid = 0, slice_mid = 0;
	int split_elem_per_sm = 0, split_rows_per_sm = 0;
	int tets_only = 0;   // every body: tetrahedra only, no contact spheres
	int filter = 0;      // filtered contacts: bodies with contact spheres carry a constraint buffer
};

namespace {

void free_cache(BatchCache* c)
{
	if (!c) return;
	if (c->graph) cudaGraphExecDestroy(c->graph);
	cudaFree(c->d_bodies);
	cudaFree(c->d_order);
	cudaFree(c->d_queue);
	cudaFree(c->d_prof);
	cudaFree(c->d_flat_off);
	delete c;
}

int schedule_ctas(int prec, int cluster, int sms)
{
	int m = batch_max_clusters(prec, cluster);
	if (m <= 0) m = std::max(1, sms / cluster);
	return m * cluster;
}

BatchArgs make_args(BatchCache* c, float h, int steps, const b3g_solver_config& cfg)
{
	BatchArgs A;
	A.bodies = c->d_bodies;
	A.big = c->d_order;
	A.nbig = c->nbig;
	A.small = c->d_order + c->nbig;
	A.nsmall = (int)c->order.size() - c->nbig;
	A.queue = c->d_queue;
	A.steps = steps;
	A.h = h;
	A.newton = (int)std::max<uint32_t>(1u, cfg.force_iterations);
	A.max_iter = (int)cfg.max_pcg_iterations;
	A.tol2 = cfg.pcg_tolerance * cfg.pcg_tolerance;
	A.refresh = (int)cfg.refresh_period;
	A.newton_tol2 = cfg.newton_tolerance * cfg.newton_tolerance;
	A.prec = c->prec;
	A.cluster = c->cluster;
	A.ctas = c->ctas;
	A.prof = c->d_prof;
	A.elem_off = c->d_flat_off;
	A.slice_off = c->d_flat_off ? c->d_flat_off + c->bodies.size() + 1 : nullptr;
	A.nelem = c->nelem;
	A.nslices = c->nslices;
	A.nbodies = (int)c->bodies.size();
	A.tets_only = c->tets_only;
	A.filter = c->filter;
	A.elem_mid = c->elem_mid;
	A.slice_mid = c->slice_mid;
	A.split_elem_per_sm = c->split_elem_per_sm;
	A.split_rows_per_sm = c->split_rows_per_sm;
	return A;
}

// Estimated solve time of body k on a team of `warps` warps, in units of one warp's pass over one
// slice: every PCG iteration is a sweep of ceil(slices / warps) passes plus about two passes'
// worth of team barriers and reductions. Iteration counts come from a step already taken; before
// one is known every body counts one iteration, so the order is by size.
double est_time(const BatchCache* c, int k, int warps)
{
	const double slices = std::ceil((double)c->bodies[k]->n / kSlice);
	const double it = c->iters.empty() || c->iters[k] <= 0 ? 1.0 : (double)c->iters[k];
	return it * (2.0 + std::ceil(slices / warps));
}

// Bodies of at least `threshold` vertices are stepped by clusters of `cluster` CTAs, the others by
// single CTAs. Each queue runs largest first, or with lpt longest estimated solve first
// (longest-processing-time order), so that a small body with many PCG iterations does not start
// last and trail the launch; the autotuner tries both.
void set_schedule(BatchCache* c, int cluster, int threshold, int sms, cudaStream_t st, int lpt = 0)
{
	c->cluster = cluster;
	c->threshold = threshold;
	c->lpt = lpt;
	constexpr int kCtaWarps = 8;  // warps of one CTA of the PCG launch
	std::vector<int> big, small;
	for (int k = 0; k < (int)c->bodies.size(); ++k)
		((cluster > 1 && (int)c->bodies[k]->n >= threshold) ? big : small).push_back(k);
	auto by_time = [&](std::vector<int>& v, int warps) {
		std::vector<double> t(c->bodies.size());
		for (int k : v) t[k] = lpt ? est_time(c, k, warps) : (double)c->bodies[k]->n;
		std::stable_sort(v.begin(), v.end(), [&](int a, int b) {
			if (t[a] != t[b]) return t[a] > t[b];
			return c->bodies[a]->n > c->bodies[b]->n;
		});
	};
	by_time(big, kCtaWarps * cluster);
	by_time(small, kCtaWarps);
	c->order = big;
	c->order.insert(c->order.end(), small.begin(), small.end());
	c->nbig = (int)big.size();
	c->ctas = schedule_ctas(c->prec, cluster, sms);
	if (!c->order.empty())
		cudaMemcpyAsync(c->d_order, c->order.data(), c->order.size() * sizeof(int), cudaMemcpyHostToDevice, st);
	if (c->graph)
	{
		cudaGraphExecDestroy(c->graph);
		c->graph = nullptr;
	}
}

// PCG iterations of every body's last step (the solver scalars on the device)
int read_iters(b3g_context* ctx, BatchCache* c)
{
	cudaStream_t st = ctx->stream;
	const uint32_t count = (uint32_t)c->bodies.size();
	c->iters.assign(count, 0);
	cudaError_t e = cudaSuccess;
	for (uint32_t k0 = 0; k0 < count && e == cudaSuccess; k0 += 1024)
	{
		const uint32_t m = std::min<uint32_t>(1024, count - k0);
		for (uint32_t k = 0; k < m && e == cudaSuccess; ++k)
			e = cudaMemcpyAsync(ctx->h_scalars + k, c->bodies[k0 + k]->d.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		for (uint32_t k = 0; k < m && e == cudaSuccess; ++k) c->iters[k0 + k] = ctx->h_scalars[k].iter;
	}
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "batch iteration counts");
}

// the mutable per-body state a step changes
std::vector<Snapshot> snapshot_list(BatchCache* c, char* store, size_t* total)
{
	std::vector<Snapshot> L;
	size_t off = 0;
	auto add = [&](const void* p, size_t bytes) {
		if (!bytes) return;
		L.push_back(Snapshot{store ? store + off : nullptr, p, bytes});
		off += (bytes + 255) & ~(size_t)255;
	};
	for (b3g_body* b : c->bodies)
	{
		const DevBody& d = b->d;
		size_t v3 = 3 * (size_t)b->n * sizeof(float);
		add(d.x, v3);
		add(d.v, v3);
		add(d.fext, v3);
		add(d.trans, v3);
		add(d.tet_q, (size_t)b->nt * sizeof(float4));
		add(d.c_exists, (size_t)b->n * b->nw);
		add(d.c_apply, (size_t)b->n * b->nw);
		add(d.c_nf, (size_t)b->n * b->nw * sizeof(float));
		add(d.c_normal, 3 * (size_t)b->n * b->nw * sizeof(float));
		add(d.sc, sizeof(Scalars));
	}
	*total = off;
	return L;
}

cudaError_t run_once(BatchCache* c, const BatchArgs& A, cudaStream_t st) { return op_batch(A, st); }

int autotune(b3g_context* ctx, BatchCache* c, float h, const b3g_solver_config& cfg)
{
	cudaStream_t st = ctx->stream;
	size_t total = 0;
	snapshot_list(c, nullptr, &total);
	char* store = nullptr;
	cudaError_t e = cudaMalloc(&store, std::max<size_t>(total, 256));
	if (e != cudaSuccess)
	{
		cudaGetLastError();
		return B3G_OK;  // not enough memory to tune: keep the heuristic
	}
	std::vector<Snapshot> L = snapshot_list(c, store, &total);
	for (const Snapshot& s : L) cudaMemcpyAsync(s.dst, s.src, s.bytes, cudaMemcpyDeviceToDevice, st);

	int maxn = 0;
	for (b3g_body* b : c->bodies) maxn = std::max(maxn, (int)b->n);
	// candidates: (cluster size, size threshold of cluster-stepped bodies, queue order)
	struct Cand
	{
		int cl, thr, lpt;
	};
	std::vector<Cand> cands;
	cands.push_back({1, 1 << 30, 0});
	cands.push_back({1, 1 << 30, 1});
	// threshold 1: every body stepped by a cluster. Small bodies on single CTAs run after the
	// clusters have drained the queue of large ones and can trail the launch; on a cluster they
	// take their turn in the same queue (512-body batch: PCG launch 28.6 -> 27.9 ms)
	const int thresholds[] = {1, 1024, 2048, 4096, 8192, 16384, 32768};
	const int clusters[] = {2, 4, 8, 16};
	for (int cl : clusters)
		if (batch_max_clusters(c->prec, cl) > 0)  // 16-CTA clusters need hardware support
			for (int t : thresholds)
				if (t <= maxn)
					for (int o = 0; o < 2; ++o) cands.push_back({cl, t, o});
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	float best = 1e30f;
	Cand best_c = {c->cluster, c->threshold, c->lpt};
	for (auto& cd : cands)
	{
		set_schedule(c, cd.cl, cd.thr, ctx->sm_count, st, cd.lpt);
		BatchArgs A = make_args(c, h, 1, cfg);
		e = run_once(c, A, st);  // warm-up
		if (e == cudaSuccess && c->iters.empty())
		{
			// the first warm-up step gives every body's iteration count, which the estimated
			// solve times of the lpt order use
			int rc = read_iters(ctx, c);
			if (rc != B3G_OK)
			{
				e = cudaErrorUnknown;
				break;
			}
			set_schedule(c, cd.cl, cd.thr, ctx->sm_count, st, cd.lpt);
			A = make_args(c, h, 1, cfg);
		}
		for (const Snapshot& s : L) cudaMemcpyAsync((void*)s.src, s.dst, s.bytes, cudaMemcpyDeviceToDevice, st);
		cudaEventRecord(e0, st);
		if (e == cudaSuccess) e = run_once(c, A, st);
		cudaEventRecord(e1, st);
		for (const Snapshot& s : L) cudaMemcpyAsync((void*)s.src, s.dst, s.bytes, cudaMemcpyDeviceToDevice, st);
		if (e == cudaSuccess) e = cudaEventSynchronize(e1);
		if (e != cudaSuccess) break;
		float ms = 0.0f;
		cudaEventElapsedTime(&ms, e0, e1);
		c->tune_log.push_back({cd.lpt * 100000000 + cd.cl * 1000000 + std::min(cd.thr, 999999), (double)ms});
		if (ms < best)
		{
			best = ms;
			best_c = cd;
		}
	}
	cudaStreamSynchronize(st);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(store);
	if (e != cudaSuccess) return cuda_fail(e, "batch autotune");
	set_schedule(c, best_c.cl, best_c.thr, ctx->sm_count, st, best_c.lpt);
	c->tuned = true;
	return B3G_OK;
}

int build_cache(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, int prec, int precond, int filter,
                BatchCache** out)
{
	BatchCache* c = new BatchCache();
	c->bodies.assign(bodies, bodies + count);
	c->prec = prec;
	c->precond = precond;
	std::vector<DevBody> h(count);
	for (uint32_t k = 0; k < count; ++k)
	{
		h[k] = dev_for(bodies[k], prec, precond);
		// filtered contacts for the bodies with contact spheres (their buffers exist: b3g_step_batch)
		h[k].filt = filter && bodies[k]->d.contacts ? bodies[k]->filt : nullptr;
		if (h[k].filt) c->filter = 1;
	}
	c->order.resize(count);
	std::iota(c->order.begin(), c->order.end(), 0);
	std::stable_sort(c->order.begin(), c->order.end(), [&](int a, int b) { return bodies[a]->n > bodies[b]->n; });
	cudaError_t e = cudaMalloc(&c->d_bodies, std::max<size_t>(1, count) * sizeof(DevBody));
	if (e == cudaSuccess) e = cudaMalloc(&c->d_order, std::max<size_t>(1, count) * sizeof(int));
	if (e == cudaSuccess) e = cudaMalloc(&c->d_queue, 4 * sizeof(unsigned));
	// flat numbering of all bodies' elements and row slices (count + 1 offsets each)
	std::vector<unsigned> off(2 * (size_t)(count + 1), 0);
	uint64_t ne = 0, nsl = 0;
	for (uint32_t k = 0; k < count; ++k)
	{
		off[k] = (unsigned)ne;
		off[count + 1 + k] = (unsigned)nsl;
		ne += (uint64_t)h[k].nt + h[k].ntr + h[k].ns + h[k].nbw + h[k].nms + (h[k].filt ? (uint64_t)h[k].n : 0u);
		nsl += (uint64_t)h[k].nslices;
	}
	off[count] = (unsigned)ne;
	off[2 * (size_t)count + 1] = (unsigned)nsl;
	c->tets_only = 1;
	for (uint32_t k = 0; k < count; ++k)
		if (h[k].ntr || h[k].ns || h[k].nbw || h[k].nms || h[k].contacts || h[k].filt) c->tets_only = 0;
	if (e == cudaSuccess && count && ne < (1ull << 32) && nsl < (1ull << 32))
	{
		e = cudaMalloc(&c->d_flat_off, off.size() * sizeof(unsigned));
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(c->d_flat_off, off.data(), off.size() * sizeof(unsigned), cudaMemcpyHostToDevice,
			                    ctx->stream);
		c->nelem = (unsigned)ne;
		c->nslices = (unsigned)nsl;
		// split assembly: group 2 starts at the first body whose elements begin past half of all
		// elements; its element launch takes one CTA per SM beside two of group 1's row launch
		// (64 + 2 x 80 registers a thread of 256-thread CTAs fit one SM's register file). Only
		// for tetrahedra-only batches, whose kernels are that small; B3G_ASM_SPLIT =
		// "fraction,element CTAs per SM,row CTAs per SM" overrides it, "0" turns it off.
		const char* se = std::getenv("B3G_ASM_SPLIT");
		double frac = c->tets_only ? 0.5 : 0.0;
		int ecta = 1, rcta = 2;
		if (se) std::sscanf(se, "%lf,%d,%d", &frac, &ecta, &rcta);
		if (frac > 0.0 && frac < 1.0)
		{
			for (uint32_t k = 1; k < count; ++k)
				if ((double)off[k] >= frac * (double)ne)
				{
					c->elem_mid = off[k];
					c->slice_mid = off[count + 1 + k];
					break;
				}
			c->split_elem_per_sm = std::max(0, ecta);
			c->split_rows_per_sm = std::max(0, rcta);
		}
	}
	if (e == cudaSuccess && count)
		e = cudaMemcpyAsync(c->d_bodies, h.data(), count * sizeof(DevBody), cudaMemcpyHostToDevice, ctx->stream);
	if (e == cudaSuccess && count)
		e = cudaMemcpyAsync(c->d_order, c->order.data(), count * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
	if (e != cudaSuccess)
	{
		free_cache(c);
		return cuda_fail(e, "batch setup");
	}
	const char* pe = std::getenv("B3G_PHASE_PROFILE");
	if (pe && pe[0] == '1')
	{
		const size_t bytes = 8 * 4096 * sizeof(unsigned long long);
		if (cudaMalloc(&c->d_prof, bytes) == cudaSuccess) cudaMemset(c->d_prof, 0, bytes);
		else cudaGetLastError();
	}
	// size heuristic: clusters of 4 for bodies of 16k vertices or more
	int maxn = 0;
	for (uint32_t k = 0; k < count; ++k) maxn = std::max(maxn, (int)bodies[k]->n);
	if (maxn >= 16384) set_schedule(c, 4, 16384, ctx->sm_count, ctx->stream);
	else set_schedule(c, 1, 1 << 30, ctx->sm_count, ctx->stream);
	*out = c;
	return B3G_OK;
}

} // namespace

void destroy_batch_cache(b3g_context* c)
{
	free_cache(c->batch);
	c->batch = nullptr;
}

void forget_body_in_batch_cache(b3g_context* c, b3g_body* b)
{
	if (!c->batch) return;
	for (b3g_body* x : c->batch->bodies)
		if (x == b)
		{
			destroy_batch_cache(c);
			return;
		}
}

// each body's solver scalars through the context's pinned buffer, 1024 at a time
static int read_batch_stats(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, b3g_step_stats* stats)
{
	cudaStream_t st = ctx->stream;
	cudaError_t e = cudaSuccess;
	for (uint32_t k0 = 0; k0 < count && e == cudaSuccess; k0 += 1024)
	{
		uint32_t m = std::min<uint32_t>(1024, count - k0);
		for (uint32_t k = 0; k < m && e == cudaSuccess; ++k)
			e = cudaMemcpyAsync(ctx->h_scalars + k, bodies[k0 + k]->d.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		for (uint32_t k = 0; k < m && e == cudaSuccess; ++k) stats_from(ctx->h_scalars[k], stats + k0 + k);
	}
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "batch stats");
}

extern "C" int b3g_step_batch(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float dt,
                              const b3g_solver_config* cfg_in, uint32_t steps, b3g_step_stats* stats)
{
	if (!ctx || (!bodies && count)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (count == 0 || steps == 0) return B3G_OK;
	b3g_solver_config cfg;
	if (cfg_in) cfg = *cfg_in;
	else b3g_solver_config_default(&cfg);
	int rc = check_config(&cfg, true);
	if (rc != B3G_OK) return rc;
	const int filter = cfg.contact_mode == B3G_CONTACT_FILTER ? 1 : 0;
	for (uint32_t k = 0; k < count; ++k)
	{
		if (!bodies[k]) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u is null", k);
		if (bodies[k]->ctx != ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u belongs to another context", k);
		for (uint32_t j = 0; j < k; ++j)
			if (bodies[j] == bodies[k]) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u is listed twice", k);
	}
	cudaSetDevice(ctx->device);
	cudaStream_t st = ctx->stream;
	if (!(dt > 0.0f))
	{
		for (uint32_t s = 0; s < steps; ++s)
			for (uint32_t k = 0; k < count; ++k)
			{
				rc = b3g_body_step(bodies[k], dt, &cfg, nullptr);
				if (rc != B3G_OK) return rc;
			}
		if (stats) std::memset(stats, 0, count * sizeof(*stats));
		return b3g_context_synchronize(ctx);
	}
	const int prec = prec_of(&cfg);
	int want_filter = 0;
	for (uint32_t k = 0; k < count; ++k)
	{
		rc = ensure_precision(bodies[k], prec);
		if (rc == B3G_OK && filter && bodies[k]->d.contacts)
		{
			rc = ensure_filter(bodies[k]);
			want_filter = 1;
		}
		if (rc != B3G_OK) return rc;
	}
	BatchCache* c = ctx->batch;
	bool same = c && c->prec == prec && c->precond == cfg.preconditioner && c->filter == want_filter &&
	            c->bodies.size() == count && std::equal(c->bodies.begin(), c->bodies.end(), bodies);
	if (!same)
	{
		destroy_batch_cache(ctx);
		rc = build_cache(ctx, bodies, count, prec, cfg.preconditioner, filter, &c);
		if (rc != B3G_OK) return rc;
		ctx->batch = c;
		const char* env = std::getenv("B3G_AUTOTUNE");
		const char* forced = std::getenv("B3G_BATCH_SCHEDULE");  // "cluster,threshold[,lpt]"
		int fc = 0, ft = 0, fo = 0;
		if (forced && std::sscanf(forced, "%d,%d,%d", &fc, &ft, &fo) >= 2 &&
		    (fc == 1 || fc == 2 || fc == 4 || fc == 8 || fc == 16))
			set_schedule(c, fc, ft > 0 ? ft : (1 << 30), ctx->sm_count, ctx->stream, fo ? 1 : 0);
		else if (!(env && env[0] == '0'))
		{
			rc = autotune(ctx, c, dt, cfg);
			if (rc != B3G_OK) return rc;
		}
	}
	BatchArgs A = make_args(c, dt, 1, cfg);
	if (c->elem_mid > 0 && A.newton == 1)
	{
		// the split assembly's second stream and fork / join events, made once per context
		cudaError_t e = cudaSuccess;
		if (!ctx->side_stream) e = cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking);
		if (e == cudaSuccess && !ctx->ev_fork) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
		if (e == cudaSuccess && !ctx->ev_join) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
		if (e != cudaSuccess) return cuda_fail(e, "split assembly stream");
		A.side = ctx->side_stream;
		A.ev_fork = ctx->ev_fork;
		A.ev_join = ctx->ev_join;
	}
	if (ctx->launch_timing && A.newton == 1)
	{
		// timed steps: the two launches of each step bracketed by events, no graph
		for (cudaEvent_t& ev : ctx->tev)
			if (!ev && cudaEventCreate(&ev) != cudaSuccess) return cuda_fail(cudaGetLastError(), "timing events");
		for (uint32_t s = 0; s < steps; ++s)
		{
			cudaError_t e = cudaEventRecord(ctx->tev[0], st);
			A.part = 1;
			A.ev_rows = A.side ? nullptr : ctx->tev[3];  // no single element/row boundary when split
			if (e == cudaSuccess) e = op_batch(A, st);
			A.ev_rows = nullptr;
			if (e == cudaSuccess) e = cudaEventRecord(ctx->tev[1], st);
			A.part = 2;
			if (e == cudaSuccess) e = op_batch(A, st);
			if (e == cudaSuccess) e = cudaEventRecord(ctx->tev[2], st);
			if (e == cudaSuccess) e = cudaEventSynchronize(ctx->tev[2]);
			if (e != cudaSuccess) return cuda_fail(e, "timed batch step");
			float m1 = 0.0f, m2 = 0.0f, m3 = 0.0f;
			cudaEventElapsedTime(&m1, ctx->tev[0], ctx->tev[1]);
			cudaEventElapsedTime(&m2, ctx->tev[1], ctx->tev[2]);
			if (!A.side) cudaEventElapsedTime(&m3, ctx->tev[0], ctx->tev[3]);
			ctx->t_assembly_ms += m1;
			ctx->t_elements_ms += m3;
			ctx->t_pcg_ms += m2;
			ctx->t_steps += 1;
		}
		A.part = 0;
		return stats ? read_batch_stats(ctx, bodies, count, stats) : B3G_OK;
	}
	const bool graph_ok = c->graph && c->g_h == dt && c->g_newton == A.newton && c->g_max_iter == A.max_iter &&
	                      c->g_tol2 == A.tol2 && c->g_refresh == A.refresh && c->g_ntol2 == A.newton_tol2;
	cudaError_t e = cudaSuccess;
	if (!graph_ok)
	{
		if (c->graph)
		{
			cudaGraphExecDestroy(c->graph);
			c->graph = nullptr;
		}
		cudaGraph_t g = nullptr;
		e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
		if (e == cudaSuccess)
		{
			cudaError_t le = op_batch(A, st);
			e = cudaStreamEndCapture(st, &g);
			if (le != cudaSuccess) e = le;
		}
		if (e == cudaSuccess) e = cudaGraphInstantiate(&c->graph, g, 0);
		if (g) cudaGraphDestroy(g);
		if (e != cudaSuccess) return cuda_fail(e, "batch graph");
		c->g_h = dt;
		c->g_newton = A.newton;
		c->g_max_iter = A.max_iter;
		c->g_tol2 = A.tol2;
		c->g_refresh = A.refresh;
		c->g_ntol2 = A.newton_tol2;
	}
	for (uint32_t s = 0; s < steps && e == cudaSuccess; ++s) e = cudaGraphLaunch(c->graph, st);
	if (e != cudaSuccess) return cuda_fail(e, "batch launch");
	if (stats) return read_batch_stats(ctx, bodies, count, stats);
	return B3G_OK;
}

extern "C" int b3g_batch_set_launch_timing(b3g_context* ctx, int on)
{
	if (!ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "null context");
	ctx->launch_timing = on != 0;
	return B3G_OK;
}

extern "C" int b3g_batch_launch_times(b3g_context* ctx, double out[3], int reset)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	out[0] = ctx->t_assembly_ms;
	out[1] = ctx->t_pcg_ms;
	out[2] = (double)ctx->t_steps;
	if (reset)
	{
		ctx->t_assembly_ms = ctx->t_pcg_ms = ctx->t_elements_ms = 0.0;
		ctx->t_steps = 0;
	}
	return B3G_OK;
}

extern "C" int b3g_batch_element_launch_ms(b3g_context* ctx, double* out)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*out = ctx->t_elements_ms;
	return B3G_OK;
}

extern "C" int b3g_batch_assembly_split(b3g_context* ctx, uint32_t out[4])
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (!ctx->batch) return fail(B3G_ERROR_INVALID_ARGUMENT, "no batch has been stepped on this context");
	const BatchCache* c = ctx->batch;
	out[0] = c->elem_mid;
	out[1] = c->slice_mid;
	out[2] = (uint32_t)c->split_elem_per_sm;
	out[3] = (uint32_t)c->split_rows_per_sm;
	return B3G_OK;
}

extern "C" int b3g_batch_schedule(b3g_context* ctx, int32_t* out, uint32_t capacity)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (!ctx->batch) return fail(B3G_ERROR_INVALID_ARGUMENT, "no batch has been stepped on this context");
	BatchCache* c = ctx->batch;
	std::vector<int32_t> v = {c->cluster, c->threshold == (1 << 30) ? -1 : c->threshold, c->nbig, c->ctas,
	                          c->tuned ? 1 : 0, (int32_t)c->tune_log.size(), c->lpt};
	for (auto& t : c->tune_log)
	{
		v.push_back(t.first);
		v.push_back((int32_t)(t.second * 1000.0));  // microseconds
	}
	for (uint32_t k = 0; k < capacity && k < v.size(); ++k) out[k] = v[k];
	return B3G_OK;
}

// The transfer table of a body list (rebuilt when the list differs from the last call's) and a
// staging buffer of at least `floats` floats.
static int prepare_xfer(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, size_t floats_per_total)
{
	bool same = ctx->xfer_bodies.size() == count;
	for (uint32_t k = 0; same && k < count; ++k) same = ctx->xfer_bodies[k] == bodies[k];
	cudaStream_t st = ctx->stream;
	cudaError_t e = cudaSuccess;
	if (!same)
	{
		std::vector<XferBody> t(count);
		uint64_t off = 0;
		uint32_t mx = 0;
		for (uint32_t k = 0; k < count; ++k)
		{
			b3g_body* b = bodies[k];
			if (!b || b->ctx != ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u is null or of another context", k);
			t[k] = XferBody{b->d.x, b->d.v, b->d.fext, off, 3u * b->n, 0u};
			off += 3ull * b->n;
			mx = std::max(mx, 3u * b->n);
		}
		if (count > ctx->xfer_table_cap)
		{
			e = cudaStreamSynchronize(st);
			if (ctx->xfer_table) cudaFree(ctx->xfer_table);
			ctx->xfer_table = nullptr;
			ctx->xfer_table_cap = 0;
			if (e == cudaSuccess) e = cudaMalloc(&ctx->xfer_table, count * sizeof(XferBody));
			if (e != cudaSuccess) return cuda_fail(e, "batch transfer table");
			ctx->xfer_table_cap = count;
		}
		// earlier transfers on the stream may still read the old table; the copy from pageable
		// memory completes before the call returns, so `t` may go
		e = cudaStreamSynchronize(st);
		if (e == cudaSuccess) e = cudaMemcpy(ctx->xfer_table, t.data(), count * sizeof(XferBody), cudaMemcpyHostToDevice);
		if (e != cudaSuccess) return cuda_fail(e, "batch transfer table");
		ctx->xfer_bodies.assign(bodies, bodies + count);
		ctx->xfer_total = off;
		ctx->xfer_max_n3 = mx;
	}
	const size_t need = floats_per_total * ctx->xfer_total;
	if (need > ctx->xfer_cap)
	{
		e = cudaStreamSynchronize(st);
		if (ctx->xfer) cudaFree(ctx->xfer);
		ctx->xfer = nullptr;
		ctx->xfer_cap = 0;
		if (e == cudaSuccess) e = cudaMalloc(&ctx->xfer, need * sizeof(float));
		if (e != cudaSuccess) return cuda_fail(e, "batch transfer staging");
		ctx->xfer_cap = need;
	}
	return B3G_OK;
}

// The device address of `floats` floats of page-locked host memory at p (cudaHostAlloc /
// cudaHostRegister, which the GPU reads and writes directly over the CPU-GPU link), or null when
// p is not such memory or the range is not one mapping.
static float* mapped_host(const float* p, uint64_t floats)
{
	if (!p || floats == 0) return nullptr;
	cudaPointerAttributes a0, a1;
	if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, p + floats - 1) != cudaSuccess)
	{
		cudaGetLastError();
		return nullptr;
	}
	if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
		return nullptr;
	float* d = (float*)a0.devicePointer;
	return (float*)a1.devicePointer == d + (floats - 1) ? d : nullptr;
}

extern "C" int b3g_batch_apply_forces(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, const float* forces)
{
	if (!ctx || (!bodies && count) || (!forces && count)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (count == 0) return B3G_OK;
	cudaSetDevice(ctx->device);
	int rc = prepare_xfer(ctx, bodies, count, 2);
	if (rc != B3G_OK) return rc;
	cudaStream_t st = ctx->stream;
	cudaError_t e = cudaSuccess;
	const float* src = mapped_host(forces, ctx->xfer_total);
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	if (src) e = cudaStreamIsCapturing(st, &cap);
	if (e != cudaSuccess) return cuda_fail(e, "batch_apply_forces");
	if (src && cap == cudaStreamCaptureStatusNone)
	{
		// page-locked host memory: the array is copied on the upload stream into one of two
		// staging buffers as soon as that buffer's previous scatter has run, so the copy overlaps
		// whatever the context stream is doing (the step before); the context stream waits for
		// the copy and adds every body's slice to its fext
		const size_t total = ctx->xfer_total;
		if (total > ctx->up_cap)
		{
			if (ctx->up_stream) e = cudaStreamSynchronize(ctx->up_stream);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			if (ctx->up_buf) cudaFree(ctx->up_buf);
			ctx->up_buf = nullptr;
			ctx->up_cap = 0;
			ctx->up_used_pending[0] = ctx->up_used_pending[1] = false;
			if (e == cudaSuccess) e = cudaMalloc(&ctx->up_buf, 2 * total * sizeof(float));
			if (e != cudaSuccess) return cuda_fail(e, "force upload buffers");
			ctx->up_cap = total;
		}
		if (!ctx->up_stream) e = cudaStreamCreateWithFlags(&ctx->up_stream, cudaStreamNonBlocking);
		for (int k = 0; k < 2 && e == cudaSuccess; ++k)
		{
			if (!ctx->ev_up_copied[k]) e = cudaEventCreateWithFlags(&ctx->ev_up_copied[k], cudaEventDisableTiming);
			if (e == cudaSuccess && !ctx->ev_up_used[k])
				e = cudaEventCreateWithFlags(&ctx->ev_up_used[k], cudaEventDisableTiming);
		}
		if (e != cudaSuccess) return cuda_fail(e, "force upload stream");
		const int k = ctx->up_next;
		ctx->up_next ^= 1;
		float* buf = ctx->up_buf + (size_t)k * ctx->up_cap;
		if (ctx->up_used_pending[k]) e = cudaStreamWaitEvent(ctx->up_stream, ctx->ev_up_used[k], 0);
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(buf, forces, total * sizeof(float), cudaMemcpyHostToDevice, ctx->up_stream);
		if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_up_copied[k], ctx->up_stream);
		if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ctx->ev_up_copied[k], 0);
		if (e == cudaSuccess) e = op_batch_scatter_add(ctx->xfer_table, count, ctx->xfer_max_n3, buf, st);
		if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_up_used[k], st);
		ctx->up_used_pending[k] = e == cudaSuccess;
		return e == cudaSuccess ? B3G_OK : cuda_fail(e, "batch_apply_forces");
	}
	// pageable memory: one copy of the whole array into the staging buffer first; a stream being
	// captured: one launch reads the page-locked array directly
	if (!src)
	{
		e = cudaMemcpyAsync(ctx->xfer, forces, ctx->xfer_total * sizeof(float), cudaMemcpyHostToDevice, st);
		src = ctx->xfer;
	}
	if (e == cudaSuccess) e = op_batch_scatter_add(ctx->xfer_table, count, ctx->xfer_max_n3, src, st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "batch_apply_forces");
}

extern "C" int b3g_batch_get_state(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float* positions,
                                   float* velocities)
{
	if (!ctx || (!bodies && count)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (count == 0 || (!positions && !velocities)) return B3G_OK;
	cudaSetDevice(ctx->device);
	int rc = prepare_xfer(ctx, bodies, count, 2);
	if (rc != B3G_OK) return rc;
	cudaStream_t st = ctx->stream;
	// one launch packs every body's x and v, straight into page-locked host arrays or into the
	// staging buffer followed by one copy each
	float* mx = mapped_host(positions, ctx->xfer_total);
	float* mv = mapped_host(velocities, ctx->xfer_total);
	float* sx = mx ? mx : ctx->xfer;
	float* sv = mv ? mv : ctx->xfer + ctx->xfer_total;
	const size_t bytes = ctx->xfer_total * sizeof(float);
	cudaError_t e = op_batch_gather(ctx->xfer_table, count, ctx->xfer_max_n3, positions ? sx : nullptr,
	                                velocities ? sv : nullptr, st);
	if (e == cudaSuccess && positions && !mx) e = cudaMemcpyAsync(positions, sx, bytes, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess && velocities && !mv) e = cudaMemcpyAsync(velocities, sv, bytes, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "batch_get_state");
}

extern "C" int b3g_batch_get_state_async(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float* positions,
                                         float* velocities)
{
	if (!ctx || (!bodies && count)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (count == 0 || (!positions && !velocities)) return B3G_OK;
	cudaSetDevice(ctx->device);
	int rc = prepare_xfer(ctx, bodies, count, 2);
	if (rc != B3G_OK) return rc;
	cudaError_t e = cudaSuccess;
	if (!ctx->copy_stream)
	{
		e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
		if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_snap, cudaEventDisableTiming);
		if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_copied, cudaEventDisableTiming);
		if (e != cudaSuccess) return cuda_fail(e, "batch_get_state_async streams");
	}
	const size_t need = 2 * ctx->xfer_total;
	if (need > ctx->snap_cap)
	{
		e = cudaStreamSynchronize(ctx->copy_stream);  // the old snapshot may still be in flight
		if (ctx->snap) cudaFree(ctx->snap);
		ctx->snap = nullptr;
		ctx->snap_cap = 0;
		ctx->copy_pending = false;
		if (e == cudaSuccess) e = cudaMalloc(&ctx->snap, need * sizeof(float));
		if (e != cudaSuccess) return cuda_fail(e, "batch_get_state_async snapshot");
		ctx->snap_cap = need;
	}
	cudaStream_t st = ctx->stream;
	// the previous copy must have left the snapshot before the gather overwrites it
	if (ctx->copy_pending) e = cudaStreamWaitEvent(st, ctx->ev_copied, 0);
	float* sx = ctx->snap;
	float* sv = ctx->snap + ctx->xfer_total;
	const size_t bytes = ctx->xfer_total * sizeof(float);
	if (e == cudaSuccess)
		e = op_batch_gather(ctx->xfer_table, count, ctx->xfer_max_n3, positions ? sx : nullptr, velocities ? sv : nullptr, st);
	if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_snap, st);
	if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_snap, 0);
	if (e == cudaSuccess && positions) e = cudaMemcpyAsync(positions, sx, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream);
	if (e == cudaSuccess && velocities) e = cudaMemcpyAsync(velocities, sv, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream);
	if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_copied, ctx->copy_stream);
	if (e != cudaSuccess) return cuda_fail(e, "batch_get_state_async");
	ctx->copy_pending = true;
	return B3G_OK;
}

extern "C" int b3g_batch_wait_state(b3g_context* ctx)
{
	if (!ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "null context");
	if (!ctx->copy_pending) return B3G_OK;
	// later work on the context stream is ordered after the copy, and the host waits for it
	cudaError_t e = cudaStreamWaitEvent(ctx->stream, ctx->ev_copied, 0);
	if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev_copied);
	ctx->copy_pending = false;
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "batch_wait_state");
}

extern "C" int b3g_batch_phase_cycles(b3g_context* ctx, uint64_t out[8], int reset)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	for (int k = 0; k < 8; ++k) out[k] = 0;
	BatchCache* c = ctx->batch;
	if (!c || !c->d_prof) return B3G_OK;
	std::vector<unsigned long long> h(8 * 4096);
	cudaError_t e = cudaMemcpyAsync(h.data(), c->d_prof, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
	                                ctx->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
	if (e == cudaSuccess && reset) e = cudaMemsetAsync(c->d_prof, 0, h.size() * sizeof(unsigned long long), ctx->stream);
	if (e != cudaSuccess) return cuda_fail(e, "phase cycles");
	for (size_t k = 0; k < h.size(); ++k) out[k % 8] += h[k];
	return B3G_OK;
}

// ------------------------------------------------------------------ allocation-free batch step
// b3g_step_batch allocates its per-batch tables (body descriptors, size order, work counters) with
// cudaMalloc on first use. Some callers cannot allocate device memory when they step: a frame
// being captured into a CUDA graph (cudaMalloc is not allowed while a stream is capturing),
// engines that forbid allocation after load or run under a fixed device-memory budget (and
// cudaMalloc / cudaFree synchronise the device, stalling a frame). b3g_step_batch_noalloc keeps
// those tables in this file-scope device array instead: room for kNoAllocMaxBodies bodies per
// call, held by every GPU that loads the library until the process exits.
constexpr uint32_t kNoAllocMaxBodies = 512;
constexpr size_t noalloc_round(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kNoAllocOrderOffset = noalloc_round(kNoAllocMaxBodies * sizeof(DevBody));
constexpr size_t kNoAllocQueueOffset = kNoAllocOrderOffset + noalloc_round(kNoAllocMaxBodies * sizeof(int));
constexpr size_t kNoAllocScratchBytes = kNoAllocQueueOffset + 256;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host side: the array's name is only a host stand-in for the device copy, so each device's real
// address is looked up once (with that device current) and kept here. The host staging arrays are
// static too, so a call allocates nothing on the host either.
static std::mutex g_noalloc_mutex;
static unsigned char* g_noalloc_dev[kNoAllocMaxDevices] = {};
static DevBody g_noalloc_host_bodies[kNoAllocMaxBodies];
static int g_noalloc_host_order[kNoAllocMaxBodies];

static int noalloc_setup(int device, unsigned char** out)
{
	if (device < 0 || device >= kNoAllocMaxDevices) return fail(B3G_ERROR_UNSUPPORTED, "device %d out of range", device);
	if (!g_noalloc_dev[device])
	{
		unsigned char* ptr = nullptr;
		cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
		if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the allocation-free scratch");
		e = cudaMemset(ptr + kNoAllocQueueOffset, 0, 256);
		if (e != cudaSuccess) return cuda_fail(e, "clearing the allocation-free scratch");
		g_noalloc_dev[device] = ptr;
	}
	*out = g_noalloc_dev[device];
	return B3G_OK;
}

extern "C" int b3g_step_batch_noalloc(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float dt,
                                      const b3g_solver_config* cfg_in, uint32_t steps, b3g_step_stats* stats)
{
	if (!ctx || (!bodies && count)) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (count > kNoAllocMaxBodies)
		return fail(B3G_ERROR_UNSUPPORTED, "b3g_step_batch_noalloc takes at most %u bodies per call (got %u)",
		            kNoAllocMaxBodies, count);
	if (count == 0 || steps == 0) return B3G_OK;
	if (!(dt > 0.0f)) return fail(B3G_ERROR_INVALID_ARGUMENT, "b3g_step_batch_noalloc needs dt > 0");
	b3g_solver_config cfg;
	if (cfg_in) cfg = *cfg_in;
	else b3g_solver_config_default(&cfg);
	int rc = check_config(&cfg);
	if (rc != B3G_OK) return rc;
	const int prec = prec_of(&cfg);
	for (uint32_t k = 0; k < count; ++k)
	{
		const b3g_body* b = bodies[k];
		if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u is null", k);
		if (b->ctx != ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u belongs to another context", k);
		if (!b->prec[prec].mem)
			return fail(B3G_ERROR_INVALID_ARGUMENT,
			            "body %u has no solver buffers for this precision yet; step it once with this precision "
			            "through b3g_body_step or b3g_step_batch first",
			            k);
		for (uint32_t j = 0; j < k; ++j)
			if (bodies[j] == bodies[k]) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u is listed twice", k);
	}
	if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(B3G_ERROR_CUDA, "cudaSetDevice");
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	unsigned char* scratch = nullptr;
	rc = noalloc_setup(ctx->device, &scratch);
	if (rc != B3G_OK) return rc;
	cudaStream_t st = ctx->stream;

	// descriptors and the size order (largest first), staged through the static host arrays
	int maxn = 0;
	for (uint32_t k = 0; k < count; ++k)
	{
		g_noalloc_host_bodies[k] = dev_for(bodies[k], prec, cfg.preconditioner);
		g_noalloc_host_order[k] = (int)k;
		maxn = std::max(maxn, (int)bodies[k]->n);
	}
	std::stable_sort(g_noalloc_host_order, g_noalloc_host_order + count,
	                 [&](int a, int b) { return bodies[a]->n > bodies[b]->n; });
	DevBody* d_bodies = (DevBody*)scratch;
	int* d_order = (int*)(scratch + kNoAllocOrderOffset);
	unsigned* d_queue = (unsigned*)(scratch + kNoAllocQueueOffset);
	cudaError_t e = cudaMemcpyAsync(d_bodies, g_noalloc_host_bodies, count * sizeof(DevBody), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(d_order, g_noalloc_host_order, count * sizeof(int), cudaMemcpyHostToDevice, st);
	if (e != cudaSuccess) return cuda_fail(e, "b3g_step_batch_noalloc upload");

	// fixed size rule, no autotuning (which would need a state snapshot): clusters of 4 CTAs for
	// bodies of 4096 vertices or more, single CTAs below
	const int cluster = maxn >= 4096 ? 4 : 1;
	const int threshold = 4096;
	int nbig = 0;
	if (cluster > 1)
		for (uint32_t k = 0; k < count; ++k)
			if ((int)bodies[k]->n >= threshold) ++nbig;
	int m = batch_max_clusters(prec, cluster);
	if (m <= 0) m = std::max(1, ctx->sm_count / cluster);
	BatchArgs A;
	A.bodies = d_bodies;
	A.big = d_order;
	A.nbig = nbig;
	A.small = d_order + nbig;
	A.nsmall = (int)count - nbig;
	A.queue = d_queue;  // op_batch clears the work counters before each step's launches
	A.steps = 1;        // one step per op_batch: a single-Newton step is two launches (assembly, then PCG)
	A.h = dt;
	A.newton = (int)std::max<uint32_t>(1u, cfg.force_iterations);
	A.max_iter = (int)cfg.max_pcg_iterations;
	A.tol2 = cfg.pcg_tolerance * cfg.pcg_tolerance;
	A.refresh = (int)cfg.refresh_period;
	A.newton_tol2 = cfg.newton_tolerance * cfg.newton_tolerance;
	A.prec = prec;
	A.cluster = cluster;
	A.ctas = m * cluster;
	A.prof = nullptr;
	for (uint32_t s = 0; s < steps && e == cudaSuccess; ++s) e = op_batch(A, st);
	if (e != cudaSuccess) return cuda_fail(e, "b3g_step_batch_noalloc launch");
	if (stats)
	{
		for (uint32_t k0 = 0; k0 < count && e == cudaSuccess; k0 += 1024)
		{
			uint32_t mm = std::min<uint32_t>(1024, count - k0);
			for (uint32_t k = 0; k < mm && e == cudaSuccess; ++k)
				e = cudaMemcpyAsync(ctx->h_scalars + k, bodies[k0 + k]->d.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			for (uint32_t k = 0; k < mm && e == cudaSuccess; ++k) stats_from(ctx->h_scalars[k], stats + k0 + k);
		}
		if (e != cudaSuccess) return cuda_fail(e, "b3g_step_batch_noalloc stats");
	}
	return B3G_OK;
}
