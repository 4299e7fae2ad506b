// Serving loop: step requests for many bodies, continuously batched into the persistent batch
// kernel (persistent.cu).
//
// A client registers bodies (host copies of their descriptions) and submits requests "step body
// b n times". A worker thread repeats: admit waiting requests (a body must be resident on the
// device; a body that is not is created if its device footprint fits the memory budget, evicting
// idle resident bodies least recently used first, their state saved to the host and restored when
// they return), launch one batched step of every body with an active request, then retire
// finished requests. Requests that arrive while a step runs join at the next iteration, so work
// of different requests overlaps on the device. A body serves its requests in arrival order, one
// at a time. The schedule (team size per body) depends only on the body's own size, so a body's
// results are the same whether it is stepped alone or in any mix.
#include "api_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace b3g;

namespace {

double now_s()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct HostDesc
{
	uint32_t n = 0, nt = 0, ntr = 0, ns = 0, nw = 0;
	std::vector<float> x, v, damping, masses;
	std::vector<int32_t> types;
	std::vector<uint32_t> tets, tris, springs;
	std::vector<float> tet_rest, tet_E, tet_nu, tet_kd, tet_rho;
	std::vector<float> tri_rest, tri_Ex, tri_Ey, tri_Es, tri_nxy, tri_nyx, tri_kd, tri_rho;
	std::vector<float> spr_L0, spr_ks, spr_kd;
	std::vector<float> srad, sfric, world;
	uint32_t nst = 0, nsh = 0, nms = 0;
	std::vector<uint32_t> st_tris, sh_tris, ms_ids;
	std::vector<float> st_uv, st_par, sh_uv, sh_par, ms_par;
	float gravity[3] = {0, 0, 0};
	// world shapes; their arrays are owned by `owned`, and the pointers in `shapes` point into
	// those arrays' heap buffers (which stay put when a HostDesc is moved)
	struct Owned
	{
		std::vector<float> vertices, voxels;
		std::vector<uint32_t> triangles, wings;
	};
	std::vector<b3g_world_shape> shapes;
	std::vector<Owned> owned;
};

template <class T>
void copy_opt(std::vector<T>& dst, const T* src, size_t count)
{
	if (src && count) dst.assign(src, src + count);
	else dst.clear();
}

void capture(HostDesc& h, const b3g_body_desc* d)
{
	const uint32_t n = d->vertex_count;
	h.n = n;
	h.nt = d->tet_count;
	h.ntr = d->tri_count;
	h.ns = d->spring_count;
	h.nw = d->world_sphere_count;
	copy_opt(h.x, d->positions, 3 * (size_t)n);
	if (d->velocities) copy_opt(h.v, d->velocities, 3 * (size_t)n);
	else h.v.assign(3 * (size_t)n, 0.0f);
	if (d->damping) copy_opt(h.damping, d->damping, n);
	else h.damping.assign(n, 0.0f);
	copy_opt(h.types, d->types, n);
	copy_opt(h.masses, d->masses, n);
	copy_opt(h.tets, d->tets, 4 * (size_t)h.nt);
	copy_opt(h.tris, d->tris, 3 * (size_t)h.ntr);
	copy_opt(h.springs, d->springs, 2 * (size_t)h.ns);
	if (d->tet_rest) copy_opt(h.tet_rest, d->tet_rest, 12 * (size_t)h.nt);
	else
	{
		h.tet_rest.resize(12 * (size_t)h.nt);
		for (uint32_t e = 0; e < h.nt; ++e)
			for (int k = 0; k < 4; ++k)
				for (int c = 0; c < 3; ++c) h.tet_rest[12 * e + 3 * k + c] = d->positions[3 * d->tets[4 * e + k] + c];
	}
	copy_opt(h.tet_E, d->tet_young, h.nt);
	copy_opt(h.tet_nu, d->tet_poisson, h.nt);
	copy_opt(h.tet_kd, d->tet_stiffness_damping, h.nt);
	copy_opt(h.tet_rho, d->tet_density, h.nt);
	if (d->tri_rest) copy_opt(h.tri_rest, d->tri_rest, 9 * (size_t)h.ntr);
	else
	{
		h.tri_rest.resize(9 * (size_t)h.ntr);
		for (uint32_t e = 0; e < h.ntr; ++e)
			for (int k = 0; k < 3; ++k)
				for (int c = 0; c < 3; ++c) h.tri_rest[9 * e + 3 * k + c] = d->positions[3 * d->tris[3 * e + k] + c];
	}
	copy_opt(h.tri_Ex, d->tri_young_x, h.ntr);
	copy_opt(h.tri_Ey, d->tri_young_y, h.ntr);
	copy_opt(h.tri_Es, d->tri_shear, h.ntr);
	copy_opt(h.tri_nxy, d->tri_poisson_xy, h.ntr);
	copy_opt(h.tri_nyx, d->tri_poisson_yx, h.ntr);
	copy_opt(h.tri_kd, d->tri_stiffness_damping, h.ntr);
	copy_opt(h.tri_rho, d->tri_density, h.ntr);
	copy_opt(h.spr_L0, d->spring_rest_length, h.ns);
	copy_opt(h.spr_ks, d->spring_stiffness, h.ns);
	copy_opt(h.spr_kd, d->spring_damping, h.ns);
	if (d->sphere_radius)
	{
		copy_opt(h.srad, d->sphere_radius, n);
		if (d->sphere_friction) copy_opt(h.sfric, d->sphere_friction, n);
		else h.sfric.assign(n, 0.0f);
	}
	copy_opt(h.world, d->world_spheres, 5 * (size_t)h.nw);
	h.nst = d->stretch_count;
	h.nsh = d->shear_count;
	h.nms = d->mouse_count;
	copy_opt(h.st_tris, d->stretch_tris, 3 * (size_t)h.nst);
	copy_opt(h.st_uv, d->stretch_uv, 6 * (size_t)h.nst);
	copy_opt(h.st_par, d->stretch_params, 6 * (size_t)h.nst);
	copy_opt(h.sh_tris, d->shear_tris, 3 * (size_t)h.nsh);
	copy_opt(h.sh_uv, d->shear_uv, 6 * (size_t)h.nsh);
	copy_opt(h.sh_par, d->shear_params, 2 * (size_t)h.nsh);
	copy_opt(h.ms_ids, d->mouse_ids, 4 * (size_t)h.nms);
	copy_opt(h.ms_par, d->mouse_params, (size_t)kMouseFloats * h.nms);
	for (int k = 0; k < 3; ++k) h.gravity[k] = d->gravity[k];
	h.shapes.clear();
	h.owned.clear();
	if (d->world_shapes)
	{
		h.owned.resize(d->world_shape_count);
		for (uint32_t k = 0; k < d->world_shape_count; ++k)
		{
			b3g_world_shape w = d->world_shapes[k];
			HostDesc::Owned& o = h.owned[k];
			const size_t nvox = (size_t)w.grid[0] * w.grid[1] * w.grid[2];
			if (w.vertices) o.vertices.assign(w.vertices, w.vertices + 3 * (size_t)w.vertex_count);
			if (w.triangles) o.triangles.assign(w.triangles, w.triangles + 3 * (size_t)w.triangle_count);
			if (w.wings) o.wings.assign(w.wings, w.wings + 3 * (size_t)w.triangle_count);
			if (w.voxels) o.voxels.assign(w.voxels, w.voxels + nvox);
			w.vertices = w.vertices ? o.vertices.data() : nullptr;
			w.triangles = w.triangles ? o.triangles.data() : nullptr;
			w.wings = w.wings ? o.wings.data() : nullptr;
			w.voxels = w.voxels ? o.voxels.data() : nullptr;
			h.shapes.push_back(w);
		}
	}
}

template <class T>
const T* ptr_or_null(const std::vector<T>& v)
{
	return v.empty() ? nullptr : v.data();
}

b3g_body_desc make_desc(const HostDesc& h)
{
	b3g_body_desc d = {};
	d.vertex_count = h.n;
	d.positions = h.x.data();
	d.velocities = h.v.data();
	d.types = h.types.data();
	d.damping = h.damping.data();
	d.masses = ptr_or_null(h.masses);
	d.tet_count = h.nt;
	d.tets = ptr_or_null(h.tets);
	d.tet_rest = ptr_or_null(h.tet_rest);
	d.tet_young = ptr_or_null(h.tet_E);
	d.tet_poisson = ptr_or_null(h.tet_nu);
	d.tet_stiffness_damping = ptr_or_null(h.tet_kd);
	d.tet_density = ptr_or_null(h.tet_rho);
	d.tri_count = h.ntr;
	d.tris = ptr_or_null(h.tris);
	d.tri_rest = ptr_or_null(h.tri_rest);
	d.tri_young_x = ptr_or_null(h.tri_Ex);
	d.tri_young_y = ptr_or_null(h.tri_Ey);
	d.tri_shear = ptr_or_null(h.tri_Es);
	d.tri_poisson_xy = ptr_or_null(h.tri_nxy);
	d.tri_poisson_yx = ptr_or_null(h.tri_nyx);
	d.tri_stiffness_damping = ptr_or_null(h.tri_kd);
	d.tri_density = ptr_or_null(h.tri_rho);
	d.spring_count = h.ns;
	d.springs = ptr_or_null(h.springs);
	d.spring_rest_length = ptr_or_null(h.spr_L0);
	d.spring_stiffness = ptr_or_null(h.spr_ks);
	d.spring_damping = ptr_or_null(h.spr_kd);
	d.sphere_radius = ptr_or_null(h.srad);
	d.sphere_friction = ptr_or_null(h.sfric);
	d.world_sphere_count = h.nw;
	d.world_spheres = ptr_or_null(h.world);
	for (int k = 0; k < 3; ++k) d.gravity[k] = h.gravity[k];
	d.world_shape_count = (uint32_t)h.shapes.size();
	d.world_shapes = ptr_or_null(h.shapes);
	d.stretch_count = h.nst;
	d.stretch_tris = ptr_or_null(h.st_tris);
	d.stretch_uv = ptr_or_null(h.st_uv);
	d.stretch_params = ptr_or_null(h.st_par);
	d.shear_count = h.nsh;
	d.shear_tris = ptr_or_null(h.sh_tris);
	d.shear_uv = ptr_or_null(h.sh_uv);
	d.shear_params = ptr_or_null(h.sh_par);
	d.mouse_count = h.nms;
	d.mouse_ids = ptr_or_null(h.ms_ids);
	d.mouse_params = ptr_or_null(h.ms_par);
	return d;
}

// Device bytes of a body that has not been created yet (partition.cpp); once a body has been
// created its exact size is used instead.
uint64_t estimate_bytes(const HostDesc& h) { return estimate_desc_bytes(make_desc(h)); }

// default team size of large bodies, 64 warps (B3G_SERVER_CLUSTER overrides)
constexpr int kServerCluster = 2048 / B3G_PCG_THREADS;
constexpr uint32_t kServerThreshold = 4096;

struct Request
{
	uint64_t id = 0;
	uint32_t body = 0;
	uint32_t steps = 0, remaining = 0;
	double t_arrival = 0, t_start = 0, t_finish = 0;
	int32_t status = 0;
	uint64_t pcg_iterations = 0;
	uint64_t iters0 = 0;         // the body's PCG iteration total when the request started
};

struct SBody
{
	HostDesc h;
	b3g_body* body = nullptr;
	uint64_t bytes = 0;          // device bytes: exact once created, estimated before
	std::deque<uint64_t> queue;  // its requests, arrival order; front is the active one when started
	bool active = false;
	uint64_t last_used = 0;
	std::vector<char> saved;     // device state saved at eviction, empty if never evicted
};

} // namespace

struct b3g_server
{
	b3g_context* ctx = nullptr;
	b3g_solver_config cfg;
	float dt = 0;
	uint64_t budget = 0, resident_bytes = 0;
	uint32_t max_active = 0;
	int cluster = kServerCluster;
	std::mutex mu;
	std::condition_variable cv;
	std::vector<SBody> bodies;
	std::deque<uint64_t> waiting;                 // requests not started, arrival order
	std::unordered_map<uint64_t, Request> reqs;   // every request not yet polled
	std::deque<uint64_t> done;                    // finished, not yet polled
	uint64_t next_id = 1, iteration = 0, iteration_base = 0;
	std::thread worker;
	bool stop = false, running = false;
	int error = 0;
	std::string error_msg;
	// device table of the active bodies' descriptors, sized for max_active
	DevBody* d_table = nullptr;
	int* d_order = nullptr;
	unsigned* d_queue = nullptr;
	DevBody* h_table = nullptr;  // pinned
	int* h_order = nullptr;      // pinned
	unsigned* d_flat_off = nullptr;  // flat numbering: element offsets, then slice offsets
	unsigned* h_flat_off = nullptr;  // pinned
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;
	// statistics
	std::vector<float> step_ms;
	uint64_t vertex_steps = 0, admitted = 0, rejected = 0, evictions = 0, completed = 0;
	double t_first = 0, t_last = 0;
};

namespace {

// The device state a step changes; everything else of a body is rebuilt from its description.
// Vertex state, element rotations, contacts (found at the end of a step, used by the next) and
// the solver's counters.
struct Part
{
	void* dev;
	size_t bytes;
};

std::vector<Part> mutable_parts(const b3g_body* b)
{
	const DevBody& d = b->d;
	const size_t v3 = 3 * (size_t)b->n * sizeof(float), c = (size_t)b->n * b->nw;
	std::vector<Part> L = {{d.x, v3},
	                       {d.v, v3},
	                       {d.fext, v3},
	                       {d.trans, v3},
	                       {d.tet_q, (size_t)b->nt * sizeof(float4)},
	                       {d.c_exists, c},
	                       {d.c_apply, c},
	                       {d.c_nf, c * sizeof(float)},
	                       {d.c_normal, 3 * c * sizeof(float)},
	                       {d.sc, sizeof(Scalars)}};
	return L;
}

int save_state(b3g_body* b, std::vector<char>& blob, cudaStream_t st)
{
	size_t total = 0;
	for (const Part& p : mutable_parts(b)) total += p.bytes;
	blob.resize(total);
	size_t off = 0;
	cudaError_t e = cudaSuccess;
	for (const Part& p : mutable_parts(b))
	{
		if (p.bytes && e == cudaSuccess) e = cudaMemcpyAsync(blob.data() + off, p.dev, p.bytes, cudaMemcpyDeviceToHost, st);
		off += p.bytes;
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "server eviction");
}

int restore_state(b3g_body* b, const std::vector<char>& blob, cudaStream_t st)
{
	size_t off = 0;
	cudaError_t e = cudaSuccess;
	for (const Part& p : mutable_parts(b))
	{
		if (p.bytes && e == cudaSuccess) e = cudaMemcpyAsync(p.dev, blob.data() + off, p.bytes, cudaMemcpyHostToDevice, st);
		off += p.bytes;
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "server restore");
}

int make_resident(b3g_server* s, uint32_t bi)
{
	SBody& B = s->bodies[bi];
	if (B.body) return B3G_OK;
	const uint64_t need = B.bytes;  // exact once the body has been created, estimated before
	// evict idle resident bodies, least recently used first, until the new one fits
	while (s->resident_bytes + need > s->budget)
	{
		int victim = -1;
		for (size_t k = 0; k < s->bodies.size(); ++k)
		{
			SBody& o = s->bodies[k];
			if (!o.body || o.active) continue;
			if (victim < 0 || o.last_used < s->bodies[victim].last_used) victim = (int)k;
		}
		if (victim < 0) return B3G_ERROR_OUT_OF_MEMORY;  // wait for a body to go idle
		SBody& o = s->bodies[victim];
		int rc = save_state(o.body, o.saved, s->ctx->stream);
		if (rc != B3G_OK) return rc;
		b3g_body_destroy(o.body);
		o.body = nullptr;
		s->resident_bytes -= o.bytes;
		s->evictions++;
	}
	b3g_body_desc d = make_desc(B.h);
	int rc = b3g_body_create(s->ctx, &d, &B.body);
	if (rc != B3G_OK) return rc;
	if (!B.saved.empty())
	{
		rc = restore_state(B.body, B.saved, s->ctx->stream);
		if (rc != B3G_OK) return rc;
	}
	uint64_t bytes = 0;
	b3g_body_device_bytes(B.body, &bytes);
	B.bytes = bytes;
	s->resident_bytes += bytes;
	return B3G_OK;
}

// Start waiting requests whose body is free; called with the lock held.
void admit(b3g_server* s)
{
	uint32_t active = 0, ready = 0;  // ready: idle bodies with a request waiting
	for (const SBody& b : s->bodies)
	{
		active += b.active ? 1 : 0;
		ready += !b.active && !b.queue.empty() ? 1 : 0;
	}
	for (auto it = s->waiting.begin(); it != s->waiting.end() && active < s->max_active && ready > 0;)
	{
		Request& r = s->reqs[*it];
		SBody& B = s->bodies[r.body];
		if (B.active || B.queue.front() != r.id)
		{
			++it;
			continue;
		}
		--ready;  // the oldest waiting request of an idle body
		if (B.bytes > s->budget && !B.body)
		{
			r.status = B3G_REQUEST_REJECTED;  // can never fit the budget
			r.t_finish = now_s();
			B.queue.pop_front();
			s->done.push_back(r.id);
			s->rejected++;
			it = s->waiting.erase(it);
			continue;
		}
		int rc = make_resident(s, r.body);
		if (rc == B3G_ERROR_OUT_OF_MEMORY)
		{
			++it;  // back-pressure: try again when a body goes idle
			continue;
		}
		if (rc != B3G_OK)
		{
			s->error = rc;
			s->error_msg = b3g_last_error();
			return;
		}
		Scalars sc;
		rc = read_scalars(B.body, &sc);
		if (rc != B3G_OK)
		{
			s->error = rc;
			s->error_msg = b3g_last_error();
			return;
		}
		r.iters0 = sc.total_iters;
		B.active = true;
		r.t_start = now_s();
		s->admitted++;
		++active;
		it = s->waiting.erase(it);
	}
}

// Descriptor table of the active bodies, largest first; called with the lock held.
int prepare(b3g_server* s, const std::vector<uint32_t>& act, int* nbig)
{
	const int prec = prec_of(&s->cfg);
	for (size_t k = 0; k < act.size(); ++k)
	{
		SBody& B = s->bodies[act[k]];
		if (!B.body->prec[prec].mem)
		{
			// solver vectors of another precision than FP32 are made on the body's first step
			int rc = ensure_precision(B.body, prec);
			if (rc != B3G_OK) return rc;
			uint64_t bytes = 0;
			b3g_body_device_bytes(B.body, &bytes);
			s->resident_bytes += bytes - B.bytes;
			B.bytes = bytes;
		}
		s->h_table[k] = dev_for(B.body, prec, s->cfg.preconditioner);
		s->h_order[k] = (int)k;
	}
	// the flat numbering of the active bodies' elements and row slices for the flat launches
	const size_t na = act.size();
	uint64_t ne = 0, nsl = 0;
	for (size_t k = 0; k < na; ++k)
	{
		const DevBody& D = s->h_table[k];
		s->h_flat_off[k] = (unsigned)ne;
		s->h_flat_off[na + 1 + k] = (unsigned)nsl;
		ne += (uint64_t)D.nt + D.ntr + D.ns + D.nbw + D.nms;
		nsl += (uint64_t)D.nslices;
	}
	s->h_flat_off[na] = (unsigned)ne;
	s->h_flat_off[2 * na + 1] = (unsigned)nsl;
	std::stable_sort(s->h_order, s->h_order + act.size(),
	                 [&](int a, int b) { return s->bodies[act[a]].h.n > s->bodies[act[b]].h.n; });
	// One schedule for every launch: bodies of kServerThreshold vertices or more are stepped by
	// clusters of s->cluster CTAs, the rest by single CTAs, always by the same kernel, so a body's
	// arithmetic does not depend on which other bodies share the launch.
	*nbig = 0;
	for (uint32_t k : act)
		if (s->bodies[k].h.n >= kServerThreshold) ++*nbig;
	return B3G_OK;
}

// One step of the prepared bodies; runs without the lock.
int step_active(b3g_server* s, int count, int nbig)
{
	const int prec = prec_of(&s->cfg);
	cudaStream_t st = s->ctx->stream;
	cudaError_t e = cudaMemcpyAsync(s->d_table, s->h_table, count * sizeof(DevBody), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_order, s->h_order, count * sizeof(int), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(s->d_flat_off, s->h_flat_off, 2 * (count + 1) * sizeof(unsigned), cudaMemcpyHostToDevice,
		                    st);
	if (e != cudaSuccess) return cuda_fail(e, "server upload");
	int m = batch_max_clusters(prec, s->cluster);
	if (m <= 0) m = std::max(1, s->ctx->sm_count / s->cluster);
	BatchArgs A;
	A.bodies = s->d_table;
	A.big = s->d_order;
	A.nbig = nbig;
	A.small = s->d_order + nbig;
	A.nsmall = count - nbig;
	A.queue = s->d_queue;
	A.steps = 1;
	A.h = s->dt;
	A.newton = (int)std::max<uint32_t>(1u, s->cfg.force_iterations);
	A.max_iter = (int)s->cfg.max_pcg_iterations;
	A.tol2 = s->cfg.pcg_tolerance * s->cfg.pcg_tolerance;
	A.refresh = (int)s->cfg.refresh_period;
	A.newton_tol2 = s->cfg.newton_tolerance * s->cfg.newton_tolerance;
	A.prec = prec;
	A.cluster = s->cluster;
	A.ctas = m * s->cluster;
	A.prof = nullptr;
	A.elem_off = s->d_flat_off;
	A.slice_off = s->d_flat_off + count + 1;
	A.nelem = s->h_flat_off[count];
	A.nslices = s->h_flat_off[2 * count + 1];
	A.nbodies = count;
	cudaEventRecord(s->ev0, st);
	e = op_batch(A, st);
	cudaEventRecord(s->ev1, st);
	if (e == cudaSuccess) e = cudaEventSynchronize(s->ev1);
	if (e != cudaSuccess) return cuda_fail(e, "server step");
	float ms = 0;
	cudaEventElapsedTime(&ms, s->ev0, s->ev1);
	s->step_ms.push_back(ms);
	return B3G_OK;
}

void worker_loop(b3g_server* s)
{
	cudaSetDevice(s->ctx->device);
	std::vector<uint32_t> act;
	for (;;)
	{
		int nbig = 0;
		{
			std::unique_lock<std::mutex> lk(s->mu);
			for (;;)
			{
				if (s->stop) return;
				admit(s);
				if (s->error) return;
				act.clear();
				for (uint32_t k = 0; k < s->bodies.size(); ++k)
					if (s->bodies[k].active) act.push_back(k);
				if (!act.empty()) break;
				s->cv.wait_for(lk, std::chrono::milliseconds(5));
			}
			int rc = prepare(s, act, &nbig);
			if (rc != B3G_OK)
			{
				s->error = rc;
				s->error_msg = b3g_last_error();
				return;
			}
		}
		int rc = step_active(s, (int)act.size(), nbig);
		std::lock_guard<std::mutex> lk(s->mu);
		if (rc != B3G_OK)
		{
			s->error = rc;
			s->error_msg = b3g_last_error();
			return;
		}
		s->iteration++;
		const double t = now_s();
		for (uint32_t k : act)
		{
			SBody& B = s->bodies[k];
			Request& r = s->reqs[B.queue.front()];
			s->vertex_steps += B.h.n;
			B.last_used = s->iteration;
			if (--r.remaining == 0)
			{
				Scalars sc;
				rc = read_scalars(B.body, &sc);
				if (rc != B3G_OK)
				{
					s->error = rc;
					s->error_msg = b3g_last_error();
					return;
				}
				r.pcg_iterations = sc.total_iters - r.iters0;
				r.status = sc.fault ? B3G_REQUEST_DEVICE_TIMEOUT : B3G_REQUEST_DONE;
				r.t_finish = t;
				s->done.push_back(r.id);
				s->completed++;
				B.queue.pop_front();
				B.active = false;
			}
		}
		s->t_last = t;
	}
}

} // namespace

extern "C" {

int b3g_server_create(b3g_context* ctx, uint64_t memory_budget_bytes, uint32_t max_active, float dt,
                      const b3g_solver_config* cfg, b3g_server** out)
{
	if (!ctx || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (max_active == 0) return fail(B3G_ERROR_INVALID_ARGUMENT, "max_active must be positive");
	if (!(dt > 0.0f)) return fail(B3G_ERROR_INVALID_ARGUMENT, "dt must be > 0");
	b3g_server* s = new b3g_server();
	s->ctx = ctx;
	if (cfg) s->cfg = *cfg;
	else b3g_solver_config_default(&s->cfg);
	int rc = check_config(&s->cfg);
	if (rc != B3G_OK)
	{
		delete s;
		return rc;
	}
	s->dt = dt;
	s->budget = memory_budget_bytes;
	s->max_active = max_active;
	cudaSetDevice(ctx->device);
	if (const char* env = std::getenv("B3G_SERVER_CLUSTER"))
	{
		const int c = std::atoi(env);
		if (c == 1 || c == 2 || c == 4 || c == 8 || c == 16) s->cluster = c;
	}
	while (s->cluster > 1 && batch_max_clusters(prec_of(&s->cfg), s->cluster) <= 0) s->cluster /= 2;
	cudaError_t e = cudaMalloc(&s->d_table, max_active * sizeof(DevBody));
	if (e == cudaSuccess) e = cudaMalloc(&s->d_order, max_active * sizeof(int));
	if (e == cudaSuccess) e = cudaMalloc(&s->d_flat_off, 2 * (max_active + 1) * sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMallocHost(&s->h_flat_off, 2 * (max_active + 1) * sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMalloc(&s->d_queue, 4 * sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMallocHost(&s->h_table, max_active * sizeof(DevBody));
	if (e == cudaSuccess) e = cudaMallocHost(&s->h_order, max_active * sizeof(int));
	if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
	if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
	if (e != cudaSuccess)
	{
		cudaFree(s->d_table);
		cudaFree(s->d_order);
		cudaFree(s->d_flat_off);
		cudaFree(s->d_queue);
		cudaFreeHost(s->h_table);
		cudaFreeHost(s->h_order);
		cudaFreeHost(s->h_flat_off);
		delete s;
		return cuda_fail(e, "server setup");
	}
	*out = s;
	return B3G_OK;
}

int b3g_server_add_body(b3g_server* s, const b3g_body_desc* desc, uint32_t* body_id)
{
	if (!s || !desc || !body_id) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (desc->vertex_count == 0 || !desc->positions || !desc->types)
		return fail(B3G_ERROR_INVALID_ARGUMENT, "positions and types are required");
	std::lock_guard<std::mutex> lk(s->mu);
	s->bodies.emplace_back();
	capture(s->bodies.back().h, desc);
	s->bodies.back().bytes = estimate_bytes(s->bodies.back().h);
	*body_id = (uint32_t)(s->bodies.size() - 1);
	return B3G_OK;
}

int b3g_server_start(b3g_server* s)
{
	if (!s) return fail(B3G_ERROR_INVALID_ARGUMENT, "null server");
	std::lock_guard<std::mutex> lk(s->mu);
	if (s->running) return B3G_OK;
	s->stop = false;
	s->running = true;
	s->worker = std::thread(worker_loop, s);
	return B3G_OK;
}

int b3g_server_submit(b3g_server* s, uint32_t body_id, uint32_t steps, uint64_t* request_id)
{
	if (!s) return fail(B3G_ERROR_INVALID_ARGUMENT, "null server");
	std::lock_guard<std::mutex> lk(s->mu);
	if (body_id >= s->bodies.size()) return fail(B3G_ERROR_INVALID_ARGUMENT, "unknown body %u", body_id);
	if (steps == 0) return fail(B3G_ERROR_INVALID_ARGUMENT, "a request needs at least one step");
	if (s->error) return fail(s->error, "server stopped: %s", s->error_msg.c_str());
	Request r;
	r.id = s->next_id++;
	r.body = body_id;
	r.steps = r.remaining = steps;
	r.t_arrival = now_s();
	if (s->t_first == 0) s->t_first = r.t_arrival;
	s->reqs[r.id] = r;
	s->bodies[body_id].queue.push_back(r.id);
	s->waiting.push_back(r.id);
	if (request_id) *request_id = r.id;
	s->cv.notify_one();
	return B3G_OK;
}

int b3g_server_poll(b3g_server* s, b3g_request_result* out, uint32_t capacity, uint32_t* count)
{
	if (!s || (!out && capacity) || !count) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	std::lock_guard<std::mutex> lk(s->mu);
	uint32_t n = 0;
	while (n < capacity && !s->done.empty())
	{
		const Request& r = s->reqs[s->done.front()];
		b3g_request_result& o = out[n++];
		o.request_id = r.id;
		o.body_id = r.body;
		o.steps = r.steps;
		o.status = r.status;
		o.pcg_iterations = r.pcg_iterations;
		o.queue_seconds = r.t_start > 0 ? r.t_start - r.t_arrival : r.t_finish - r.t_arrival;
		o.latency_seconds = r.t_finish - r.t_arrival;
		s->reqs.erase(s->done.front());
		s->done.pop_front();
	}
	*count = n;
	if (s->error) return fail(s->error, "server stopped: %s", s->error_msg.c_str());
	return B3G_OK;
}

int b3g_server_pending(b3g_server* s, uint32_t* pending)
{
	if (!s || !pending) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	std::lock_guard<std::mutex> lk(s->mu);
	*pending = (uint32_t)(s->reqs.size() - s->done.size());
	if (s->error) return fail(s->error, "server stopped: %s", s->error_msg.c_str());
	return B3G_OK;
}

int b3g_server_get_stats(b3g_server* s, b3g_server_stats* out)
{
	if (!s || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	std::lock_guard<std::mutex> lk(s->mu);
	std::memset(out, 0, sizeof(*out));
	out->iterations = s->iteration - s->iteration_base;
	out->cluster_ctas = (uint32_t)s->cluster;
	out->cluster_threshold = kServerThreshold;
	out->vertex_steps = s->vertex_steps;
	out->admitted = s->admitted;
	out->completed = s->completed;
	out->rejected = s->rejected;
	out->evictions = s->evictions;
	out->resident_bytes = s->resident_bytes;
	out->waiting = s->waiting.size();
	double total = 0;
	for (float m : s->step_ms) total += m;
	out->gpu_seconds = total / 1e3;
	out->wall_seconds = s->t_last > s->t_first ? s->t_last - s->t_first : 0;
	if (!s->step_ms.empty())
	{
		std::vector<float> v = s->step_ms;
		std::sort(v.begin(), v.end());
		out->step_ms_p50 = v[(v.size() - 1) / 2];
		out->step_ms_p99 = v[std::min(v.size() - 1, (size_t)(0.99 * (double)(v.size() - 1) + 0.5))];
	}
	return B3G_OK;
}

int b3g_server_reset_stats(b3g_server* s)
{
	if (!s) return fail(B3G_ERROR_INVALID_ARGUMENT, "null server");
	std::lock_guard<std::mutex> lk(s->mu);
	s->step_ms.clear();
	s->vertex_steps = s->admitted = s->completed = s->rejected = s->evictions = 0;
	s->iteration_base = s->iteration;
	s->t_first = s->t_last = 0;
	return B3G_OK;
}

int b3g_server_get_state(b3g_server* s, uint32_t body_id, float* positions, float* velocities)
{
	if (!s) return fail(B3G_ERROR_INVALID_ARGUMENT, "null server");
	std::lock_guard<std::mutex> lk(s->mu);
	if (body_id >= s->bodies.size()) return fail(B3G_ERROR_INVALID_ARGUMENT, "unknown body %u", body_id);
	SBody& B = s->bodies[body_id];
	if (B.active) return fail(B3G_ERROR_INVALID_ARGUMENT, "body %u is being stepped", body_id);
	if (B.body) return b3g_body_get_state(B.body, positions, velocities);
	// not resident: the state saved at its eviction (positions then velocities lead the saved
	// parts), else the state it was registered with
	const size_t bytes = 3 * (size_t)B.h.n * sizeof(float);
	const char* x = B.saved.empty() ? (const char*)B.h.x.data() : B.saved.data();
	const char* v = B.saved.empty() ? (const char*)B.h.v.data() : B.saved.data() + bytes;
	if (positions) std::memcpy(positions, x, bytes);
	if (velocities) std::memcpy(velocities, v, bytes);
	return B3G_OK;
}

int b3g_server_destroy(b3g_server* s)
{
	if (!s) return B3G_OK;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
		s->cv.notify_all();
	}
	if (s->worker.joinable()) s->worker.join();
	cudaSetDevice(s->ctx->device);
	for (SBody& b : s->bodies)
		if (b.body) b3g_body_destroy(b.body);
	cudaEventDestroy(s->ev0);
	cudaEventDestroy(s->ev1);
	cudaFree(s->d_table);
	cudaFree(s->d_order);
	cudaFree(s->d_flat_off);
	cudaFree(s->d_queue);
	cudaFreeHost(s->h_table);
	cudaFreeHost(s->h_order);
	cudaFreeHost(s->h_flat_off);
	delete s;
	return B3G_OK;
}

} // extern "C"
