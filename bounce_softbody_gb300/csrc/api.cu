// C ABI of b3g (include/b3g.h): contexts, bodies, the single-body step (per-op kernels) and
// state transfer. The batch entry point lives in batch.cu.
#include "api_internal.h"
#include "forces.h"
#include "shapes.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace b3g;

namespace {

thread_local std::string g_error;

} // namespace

namespace b3g {

int fail(int code, const char* fmt, ...)
{
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	std::vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_error = buf;
	return code;
}

int cuda_fail(cudaError_t e, const char* where)
{
	return fail(e == cudaErrorMemoryAllocation ? B3G_ERROR_OUT_OF_MEMORY : B3G_ERROR_CUDA, "%s: %s", where,
	            cudaGetErrorString(e));
}

// ------------------------------------------------------------------ host-side element setup
namespace {

struct V3h
{
	float x, y, z;
};
V3h sub(V3h a, V3h b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3h cross(V3h a, V3h b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float dot(V3h a, V3h b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3h normalize(V3h a)
{
	float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
	if (l > 1.1920928955078125e-7f)
	{
		float s = 1.0f / l;
		a = {a.x * s, a.y * s, a.z * s};
	}
	return a;
}
V3h ld(const float* p) { return {p[0], p[1], p[2]}; }

// column-major dense products (math.h b3Mul / b3Transpose of the reference)
void dmul(float* out, const float* A, int m, int n, const float* B, int p)
{
	for (int i = 0; i < m; ++i)
		for (int j = 0; j < p; ++j)
		{
			float s = 0.0f;
			for (int k = 0; k < n; ++k) s += A[i + m * k] * B[k + n * j];
			out[i + m * j] = s;
		}
}
void dtr(float* out, const float* A, int m, int n)
{
	for (int i = 0; i < m; ++i)
		for (int j = 0; j < n; ++j) out[j + n * i] = A[i + m * j];
}

// tetrahedron_element_force.cpp:219-265: invE = adj(E) / det(E), volume |det| / 6,
// Lame parameters of the isotropic D.
void tet_setup(const float r[12], float E, float nu, float invE[9], float* vol, float* lam, float* mu)
{
	V3h x1 = ld(r), x2 = ld(r + 3), x3 = ld(r + 6), x4 = ld(r + 9);
	V3h e1 = sub(x2, x1), e2 = sub(x3, x1), e3 = sub(x4, x1);
	float det = dot(e1, cross(e2, e3));
	*vol = std::fabs(det) / 6.0f;
	float id = 1.0f / det;
	V3h c0 = cross(e2, e3), c1 = cross(e3, e1), c2 = cross(e1, e2);
	const V3h c[3] = {c0, c1, c2};
	for (int j = 0; j < 3; ++j)
		for (int rr = 0; rr < 3; ++rr)
		{
			const float* cj = &c[rr].x;
			invE[3 * j + rr] = id * cj[j];
		}
	*lam = (nu * E) / ((1.0f + nu) * (1.0f - 2.0f * nu));
	*mu = E / (2.0f * (1.0f + nu));
}

// mat33.h:310 b3ComputeBasis
void compute_basis(V3h a, V3h* b, V3h* c)
{
	const float sqrt_inv3 = std::sqrt(1.0f / 3.0f);
	if (std::fabs(a.x) >= sqrt_inv3) *b = {a.y, -a.x, 0.0f};
	else *b = {0.0f, a.z, -a.y};
	*b = normalize(*b);
	*c = cross(a, *b);
}

// triangle_element_force.cpp:208-279: rest 2-D coordinates, invS, K0 = A B^T C B in 2x2 blocks
bool tri_setup(const float r[9], float Ex, float Ey, float Es, float nxy, float nyx, float x2d[6], float invS[4],
               float K[36])
{
	V3h p1 = ld(r), p2 = ld(r + 3), p3 = ld(r + 6);
	V3h n = normalize(cross(sub(p2, p1), sub(p3, p1)));
	V3h px, py;
	compute_basis(n, &px, &py);
	const V3h ps[3] = {p1, p2, p3};
	for (int k = 0; k < 3; ++k)
	{
		x2d[2 * k] = px.x * ps[k].x + px.y * ps[k].y + px.z * ps[k].z;
		x2d[2 * k + 1] = py.x * ps[k].x + py.y * ps[k].y + py.z * ps[k].z;
	}
	float e1x = x2d[2] - x2d[0], e1y = x2d[3] - x2d[1];
	float e2x = x2d[4] - x2d[0], e2y = x2d[5] - x2d[1];
	float det = e1x * e2y - e1y * e2x;
	if (det == 0.0f) return false;
	float A = 0.5f * std::fabs(det);
	// The reference multiplies the adjugate by det instead of dividing by it
	// (triangle_element_force.cpp:260-265), so its rest-shape matrix is det^2 S^-1 and the
	// element stiffness scales accordingly. Kept as the reference computes it, for parity.
	invS[0] = det * e2y;
	invS[1] = det * -e1y;
	invS[2] = det * -e2x;
	invS[3] = det * e1x;
	float s = 1.0f - nxy * nyx;
	float C[9] = {Ex / s, Ey * nxy / s, 0.0f, Ex * nyx / s, Ey / s, 0.0f, 0.0f, 0.0f, Es};
	float n2x = invS[0], n3x = invS[1], n1x = -n2x - n3x;
	float n2y = invS[2], n3y = invS[3], n1y = -n2y - n3y;
	float Bm[18] = {n1x, 0, n1y, 0, n1y, n1x, n2x, 0, n2y, 0, n2y, n2x, n3x, 0, n3y, 0, n3y, n3x};
	float BT[18], BTC[18], Kd[36];
	dtr(BT, Bm, 3, 6);
	dmul(BTC, BT, 6, 3, C, 3);
	dmul(Kd, BTC, 6, 3, Bm, 6);
	for (int i = 0; i < 36; ++i) Kd[i] *= A;
	for (int i = 0; i < 6; ++i)
		for (int j = 0; j < 6; ++j) K[4 * ((i / 2) + 3 * (j / 2)) + 2 * (j % 2) + (i % 2)] = Kd[i + 6 * j];
	return true;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

struct Carver
{
	size_t off = 0;
	char* base = nullptr;
	template <class T>
	T* take(size_t count)
	{
		size_t o = off;
		off = align_up(off + std::max<size_t>(count, 1) * sizeof(T));
		return base ? (T*)(base + o) : nullptr;
	}
};

} // namespace

// b3Body::ResetMass (body.cpp:394-466): fixture lists are walked newest first.
void reset_mass(b3g_body* b)
{
	const uint32_t n = b->n;
	std::vector<float>& m = b->h_mass;
	std::vector<float>& im = b->h_invmass;
	m.assign(n, 0.0f);
	im.assign(n, 0.0f);
	for (uint32_t i = 0; i < n; ++i)
	{
		m[i] = b->h_type[i] == B3G_DYNAMIC ? 1.0f : 0.0f;
		im[i] = m[i];
	}
	if (b->h_given_mass.size() == n)
	{
		for (uint32_t i = 0; i < n; ++i)
		{
			if (b->h_type[i] != B3G_DYNAMIC) { m[i] = 0.0f; im[i] = 0.0f; continue; }
			m[i] = b->h_given_mass[i] > 0.0f ? b->h_given_mass[i] : 1.0f;
			im[i] = 1.0f / m[i];
		}
		return;
	}
	for (uint32_t e = 0; e < b->ntr_fix; ++e)
		for (int k = 0; k < 3; ++k) m[b->h_tris[3 * e + k]] = 0.0f;
	for (uint32_t e = 0; e < b->nt; ++e)
		for (int k = 0; k < 4; ++k) m[b->h_tets[4 * e + k]] = 0.0f;
	const float inv3 = 1.0f / 3.0f, inv4 = 1.0f / 4.0f;
	for (uint32_t e = b->ntr_fix; e-- > 0;)
	{
		float mm = b->h_tri_mass[e];
		for (int k = 0; k < 3; ++k) m[b->h_tris[3 * e + k]] += inv3 * mm;
	}
	for (uint32_t e = b->nt; e-- > 0;)
	{
		float mm = b->h_tet_mass[e];
		for (int k = 0; k < 4; ++k) m[b->h_tets[4 * e + k]] += inv4 * mm;
	}
	for (uint32_t i = 0; i < n; ++i)
	{
		if (b->h_type[i] != B3G_DYNAMIC) { m[i] = 0.0f; im[i] = 0.0f; continue; }
		if (m[i] > 0.0f) im[i] = 1.0f / m[i];
		else { m[i] = 1.0f; im[i] = 1.0f; }
	}
}

int upload_masses(b3g_body* b)
{
	cudaStream_t st = b->ctx->stream;
	cudaError_t e = cudaMemcpyAsync((void*)b->d.mass, b->h_mass.data(), b->n * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync((void*)b->d.invmass, b->h_invmass.data(), b->n * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "uploading masses");
}

// Solver vectors and low-precision matrix storage of one precision, allocated on first use.
int ensure_precision(b3g_body* b, int prec)
{
	PrecBuffers& pb = b->prec[prec];
	if (pb.mem) return B3G_OK;
	const size_t vs = prec == kP64 ? sizeof(double) : sizeof(float);
	const size_t np = (size_t)b->d.npad;
	size_t bytes = 0;
	bytes += align_up(7 * 4 * np * vs);           // pb r d d2 q s py, 4-wide per vertex
	bytes += align_up(12 * np * vs);              // Minv: 4 (scalar Jacobi) or 12 (block Jacobi) per vertex
	size_t alo = 0;
	if (prec == kP64) alo = 9 * (size_t)b->d.nslots * sizeof(double);
	if (prec == kPBF) alo = 9 * (size_t)b->d.nslots * sizeof(__nv_bfloat16);
	bytes += align_up(alo);
	const size_t xff = prec == kP64 ? 0 : 8 * np * sizeof(float);  // float-float solution for refinement
	bytes += align_up(xff);
	// BF16: the flexible outer CG's workspace (7 vectors, inner scalars, outer scalars, partials)
	const size_t fcg = prec == kPBF ? align_up(7 * 4 * np * vs) + align_up(sizeof(Scalars)) +
	                                      align_up(sizeof(FcgScalars)) + align_up(2 * kMaxPartials * sizeof(double))
	                                : 0;
	bytes += fcg;
	char* mem = nullptr;
	cudaError_t e = cudaMalloc(&mem, bytes);
	if (e != cudaSuccess) return cuda_fail(e, "allocating solver vectors");
	e = cudaMemsetAsync(mem, 0, bytes, b->ctx->stream);
	if (e != cudaSuccess)
	{
		cudaFree(mem);
		return cuda_fail(e, "clearing solver vectors");
	}
	pb.mem = mem;
	pb.bytes = bytes;
	char* p = mem;
	for (int k = 0; k < 7; ++k)
	{
		pb.vec[k] = p;
		p += 4 * np * vs;
	}
	p = mem + align_up(7 * 4 * np * vs);
	pb.minv = p;
	p += align_up(12 * np * vs);
	pb.alo = alo ? p : nullptr;
	p += align_up(alo);
	pb.xff = xff ? (float*)p : nullptr;
	p += align_up(xff);
	if (fcg)
	{
		for (int k = 0; k < 7; ++k) pb.fcg_vec[k] = p + k * 4 * np * vs;
		p += align_up(7 * 4 * np * vs);
		pb.fcg_inner = (Scalars*)p;
		p += align_up(sizeof(Scalars));
		pb.fcg = (FcgScalars*)p;
		p += align_up(sizeof(FcgScalars));
		pb.fcg_part = (double*)p;
	}
	return B3G_OK;
}

DevBody dev_for(const b3g_body* b, int prec, int precond, bool refine)
{
	DevBody d = b->d;
	const PrecBuffers& pb = b->prec[prec];
	d.pb = pb.vec[0];
	d.r = pb.vec[1];
	d.d = pb.vec[2];
	d.d2 = pb.vec[3];
	d.q = pb.vec[4];
	d.s = pb.vec[5];
	d.py = pb.vec[6];
	d.Minv = pb.minv;
	d.Alo = pb.alo;
	d.xff = refine ? pb.xff : nullptr;
	d.precond = precond;
	return d;
}

int prec_of(const b3g_solver_config* c)
{
	if (c->precision == B3G_PRECISION_FP64) return kP64;
	if (c->precision == B3G_PRECISION_BF16_BLOCKS) return kPBF;
	return kP32;
}

// The per-vertex constraint buffer of filtered contacts, made on the first step in that mode.
int ensure_filter(b3g_body* b)
{
	if (b->filt) return B3G_OK;
	cudaError_t e = cudaMalloc(&b->filt, std::max<size_t>(1, (size_t)b->d.n) * sizeof(float4));
	if (e != cudaSuccess)
	{
		b->filt = nullptr;
		return cuda_fail(e, "filtered contacts");
	}
	return B3G_OK;
}

int check_config(const b3g_solver_config* c, bool filter_ok)
{
	if (c->contact_mode != B3G_CONTACT_PENALTY && c->contact_mode != B3G_CONTACT_FILTER)
		return fail(B3G_ERROR_INVALID_ARGUMENT, "unknown contact mode %d", c->contact_mode);
	if (c->contact_mode == B3G_CONTACT_FILTER && !filter_ok)
		return fail(B3G_ERROR_UNSUPPORTED, "filtered contacts are stepped by b3g_body_step and b3g_step_batch only");
	if (c->precision < 0 || c->precision > 2) return fail(B3G_ERROR_INVALID_ARGUMENT, "unknown precision %d", c->precision);
	if (c->preconditioner < 0 || c->preconditioner > 1)
		return fail(B3G_ERROR_INVALID_ARGUMENT, "unknown preconditioner %d", c->preconditioner);
	if (!(c->pcg_tolerance > 0.0 && c->pcg_tolerance < 1.0))
		return fail(B3G_ERROR_INVALID_ARGUMENT, "pcg_tolerance must lie in (0, 1)");
	return B3G_OK;
}

void stats_from(const Scalars& sc, b3g_step_stats* st)
{
	st->newton_iterations = (uint32_t)sc.newton_iter;
	st->pcg_iterations = (uint32_t)sc.max_it;
	st->min_pcg_iterations = sc.min_it == 0x7fffffff ? 0u : (uint32_t)sc.min_it;
	st->solve_status = sc.fault ? B3G_SOLVE_DEVICE_TIMEOUT : sc.status;
	st->residual_ratio = sc.delta0 > 0.0 ? std::sqrt(std::max(0.0, sc.delta / sc.delta0)) : 0.0;
	st->newton_error = sc.newton_err;
	st->total_pcg_iterations = sc.total_iters;
	st->total_steps = sc.total_steps;
}

int read_scalars(b3g_body* b, Scalars* out)
{
	cudaStream_t st = b->ctx->stream;
	cudaError_t e = cudaMemcpyAsync(b->ctx->h_scalars, b->d.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return cuda_fail(e, "reading solver scalars");
	*out = *b->ctx->h_scalars;
	return B3G_OK;
}

} // namespace b3g

// ------------------------------------------------------------------ C ABI
extern "C" {

void b3g_solver_config_default(b3g_solver_config* c)
{
	if (!c) return;
	c->force_iterations = 1;
	c->max_pcg_iterations = 20;           // b3SolveBEInput default maxSubIterations
	c->pcg_tolerance = 1.1920928955078125e-7;   // FLT_EPSILON
	c->newton_tolerance = 1.1920928955078125e-7;
	c->refresh_period = 50;
	c->precision = B3G_PRECISION_FP32;
	c->preconditioner = B3G_PRECOND_JACOBI;
	c->contact_mode = B3G_CONTACT_PENALTY;
}

const char* b3g_last_error(void) { return g_error.c_str(); }

const char* b3g_version(void) { return "b3g 0.1 sm_103a"; }

int b3g_context_create(int device, b3g_context** out)
{
	if (!out) return fail(B3G_ERROR_INVALID_ARGUMENT, "out is null");
	*out = nullptr;
	int count = 0;
	cudaError_t e = cudaGetDeviceCount(&count);
	if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
	if (device < 0 || device >= count) return fail(B3G_ERROR_INVALID_ARGUMENT, "device %d of %d", device, count);
	e = cudaSetDevice(device);
	if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
	b3g_context* c = new (std::nothrow) b3g_context();
	if (!c) return fail(B3G_ERROR_OUT_OF_MEMORY, "context");
	c->device = device;
	e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_scalars, sizeof(Scalars) * 1024);
	if (e != cudaSuccess)
	{
		if (c->stream) cudaStreamDestroy(c->stream);
		delete c;
		return cuda_fail(e, "context setup");
	}
	cudaDeviceProp prop;
	if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) c->sm_count = prop.multiProcessorCount;
	*out = c;
	return B3G_OK;
}

static void release_body_memory(b3g_body* b);

int b3g_context_destroy(b3g_context* c)
{
	if (!c) return B3G_OK;
	cudaSetDevice(c->device);
	cudaStreamSynchronize(c->stream);
	destroy_batch_cache(c);
	release_sparse(c);
	for (b3g_body* b : c->live_bodies)
	{
		release_body_memory(b);
		b->ctx = nullptr;
	}
	c->live_bodies.clear();
	if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
	if (c->snap) cudaFree(c->snap);
	if (c->ev_snap) cudaEventDestroy(c->ev_snap);
	if (c->ev_copied) cudaEventDestroy(c->ev_copied);
	if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
	if (c->up_stream) cudaStreamSynchronize(c->up_stream);
	for (int k = 0; k < 2; ++k)
	{
		if (c->ev_up_copied[k]) cudaEventDestroy(c->ev_up_copied[k]);
		if (c->ev_up_used[k]) cudaEventDestroy(c->ev_up_used[k]);
	}
	if (c->up_buf) cudaFree(c->up_buf);
	if (c->up_stream) cudaStreamDestroy(c->up_stream);
	if (c->side_stream) cudaStreamSynchronize(c->side_stream);
	if (c->ev_fork) cudaEventDestroy(c->ev_fork);
	if (c->ev_join) cudaEventDestroy(c->ev_join);
	if (c->side_stream) cudaStreamDestroy(c->side_stream);
	if (c->xfer) cudaFree(c->xfer);
	if (c->xfer_table) cudaFree(c->xfer_table);
	for (cudaEvent_t& e : c->tev)
		if (e) cudaEventDestroy(e);
	if (c->h_scalars) cudaFreeHost(c->h_scalars);
	cudaStreamDestroy(c->stream);
	delete c;
	return B3G_OK;
}

int b3g_context_stream(b3g_context* c, void** stream)
{
	if (!c || !stream) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*stream = (void*)c->stream;
	return B3G_OK;
}

int b3g_context_synchronize(b3g_context* c)
{
	if (!c) return fail(B3G_ERROR_INVALID_ARGUMENT, "null context");
	cudaError_t e = cudaStreamSynchronize(c->stream);
	if (e == cudaSuccess && c->up_stream) e = cudaStreamSynchronize(c->up_stream);
	if (e == cudaSuccess && c->copy_stream)
	{
		e = cudaStreamSynchronize(c->copy_stream);
		c->copy_pending = false;
	}
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "synchronize");
}

int b3g_body_create(b3g_context* ctx, const b3g_body_desc* d, b3g_body** out)
{
	if (!ctx || !d || !out) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*out = nullptr;
	const uint32_t n = d->vertex_count;
	if (n == 0 || !d->positions || !d->types) return fail(B3G_ERROR_INVALID_ARGUMENT, "positions and types are required");
	if (d->tet_count && (!d->tets || !d->tet_young || !d->tet_poisson))
		return fail(B3G_ERROR_INVALID_ARGUMENT, "tetrahedra need tets, tet_young and tet_poisson");
	// triangles are mass fixtures (b3TriangleFixture) and, when the five material arrays are
	// given, membrane elements (b3TriangleElementForce) too
	const bool tri_elements = d->tri_young_x || d->tri_young_y || d->tri_shear || d->tri_poisson_xy || d->tri_poisson_yx;
	if (d->tri_count && (!d->tris || (tri_elements && !(d->tri_young_x && d->tri_young_y && d->tri_shear &&
	                                                   d->tri_poisson_xy && d->tri_poisson_yx))))
		return fail(B3G_ERROR_INVALID_ARGUMENT, "triangles need tris and all or none of their five material arrays");
	for (uint64_t k = 0; k < 3 * (uint64_t)d->tri_count; ++k)
		if (d->tris[k] >= n)
			return fail(B3G_ERROR_INVALID_ARGUMENT, "triangle %u references vertex %u >= vertex_count %u",
			            (uint32_t)(k / 3), d->tris[k], n);
	if (d->spring_count && (!d->springs || !d->spring_rest_length || !d->spring_stiffness || !d->spring_damping))
		return fail(B3G_ERROR_INVALID_ARGUMENT, "springs need springs, rest lengths, stiffness and damping");
	std::vector<DevShape> shapes;
	std::vector<float> shape_data;
	ClothForces cf;
	{
		char msg[256];
		if (build_shapes(d, shapes, shape_data, msg, sizeof(msg)) != 0)
			return fail(B3G_ERROR_INVALID_ARGUMENT, "%s", msg);
		if (build_cloth_forces(d, cf, msg, sizeof(msg)) != 0) return fail(B3G_ERROR_INVALID_ARGUMENT, "%s", msg);
	}
	const uint32_t nbw = (uint32_t)cf.bw.size(), nms = (uint32_t)cf.ms.size();
	for (uint32_t i = 0; i < n; ++i)
		if (d->types[i] < 0 || d->types[i] > 2) return fail(B3G_ERROR_INVALID_ARGUMENT, "vertex %u has type %d", i, d->types[i]);
	if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(B3G_ERROR_CUDA, "cudaSetDevice");

	b3g_body* b = new (std::nothrow) b3g_body();
	if (!b) return fail(B3G_ERROR_OUT_OF_MEMORY, "body");
	b->ctx = ctx;
	b->n = n;
	b->nt = d->tet_count;
	b->ntr_fix = d->tri_count;
	b->ntr = tri_elements ? d->tri_count : 0;
	b->ns = d->spring_count;
	b->nw = d->sphere_radius ? (uint32_t)shapes.size() : 0;

	char err[256];
	// device storage order of the tetrahedra (b->tet_order[k] = element at position k)
	b->tet_order = tet_storage_order(b->nt, d->tets);
	std::vector<uint32_t> tet_rank(b->nt);
	for (uint32_t k = 0; k < b->nt; ++k) tet_rank[b->tet_order[k]] = k;
	Pattern P;
	if (!build_pattern(n, b->nt, d->tets, b->ntr, d->tris, b->ns, d->springs, nbw, cf.bw_ids.data(), nms,
	                   cf.ms_ids.data(), tet_rank.data(), &P, err, sizeof(err)))
	{
		delete b;
		return fail(B3G_ERROR_INVALID_ARGUMENT, "%s", err);
	}
	b->nnzb = P.nnzb;

	// element constants on the host
	b->h_type.assign(d->types, d->types + n);
	b->h_tets.assign(d->tets, d->tets + 4 * (size_t)b->nt);
	b->h_tris.assign(d->tris, d->tris + 3 * (size_t)b->ntr_fix);
	if (d->masses) b->h_given_mass.assign(d->masses, d->masses + n);
	std::vector<uint4> tet(b->nt);
	std::vector<float> tet_invE(9 * (size_t)b->nt);
	std::vector<float4> tet_mat(b->nt), tet_q(b->nt);
	b->h_tet_mass.resize(b->nt);
	for (uint32_t e = 0; e < b->nt; ++e)
	{
		const uint32_t* t = d->tets + 4 * e;
		const uint32_t k_e = tet_rank[e];
		tet[k_e] = make_uint4(t[0], t[1], t[2], t[3]);
		float r[12];
		for (int k = 0; k < 4; ++k)
			for (int c = 0; c < 3; ++c) r[3 * k + c] = d->tet_rest ? d->tet_rest[12 * e + 3 * k + c] : d->positions[3 * t[k] + c];
		float vol, lam, mu, ie[9];
		tet_setup(r, d->tet_young[e], d->tet_poisson[e], ie, &vol, &lam, &mu);
		if (!(vol > 0.0f) || !std::isfinite(ie[0]))
		{
			free_pattern(&P);
			delete b;
			return fail(B3G_ERROR_INVALID_ARGUMENT, "tetrahedron %u is degenerate", e);
		}
		for (int q = 0; q < 9; ++q) tet_invE[(size_t)q * b->nt + k_e] = ie[q];
		float kd = d->tet_stiffness_damping ? d->tet_stiffness_damping[e] : 0.0f;
		tet_mat[k_e] = make_float4(vol, lam, mu, kd);
		tet_q[k_e] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
		// tetrahedron_fixture.cpp:34-45 (same volume as the element's)
		float dens = d->tet_density ? d->tet_density[e] : 0.0f;
		b->h_tet_mass[e] = dens * vol;
	}
	std::vector<uint4> tri(b->ntr_fix);  // every triangle fixture (the ray cast's targets)
	std::vector<float> tri_x(6 * (size_t)b->ntr), tri_invS(4 * (size_t)b->ntr), tri_K(36 * (size_t)b->ntr), tri_kd(b->ntr);
	b->h_tri_mass.resize(b->ntr_fix);
	for (uint32_t e = 0; e < b->ntr_fix; ++e)
	{
		const uint32_t* t = d->tris + 3 * e;
		float r[9];
		for (int k = 0; k < 3; ++k)
			for (int c = 0; c < 3; ++c) r[3 * k + c] = d->tri_rest ? d->tri_rest[9 * e + 3 * k + c] : d->positions[3 * t[k] + c];
		tri[e] = make_uint4(t[0], t[1], t[2], 0);
		if (tri_elements)
		{
			if (!tri_setup(r, d->tri_young_x[e], d->tri_young_y[e], d->tri_shear[e], d->tri_poisson_xy[e],
			               d->tri_poisson_yx[e], &tri_x[6 * (size_t)e], &tri_invS[4 * (size_t)e], &tri_K[36 * (size_t)e]))
			{
				free_pattern(&P);
				delete b;
				return fail(B3G_ERROR_INVALID_ARGUMENT, "triangle %u is degenerate", e);
			}
			tri_kd[e] = d->tri_stiffness_damping ? d->tri_stiffness_damping[e] : 0.0f;
		}
		// triangle_fixture.cpp:33-36 area = |cross| / 2
		V3h a = ld(r), bb = ld(r + 3), c = ld(r + 6);
		V3h N = cross(sub(bb, a), sub(c, a));
		float area = 0.5f * std::sqrt(dot(N, N));
		float dens = d->tri_density ? d->tri_density[e] : 0.0f;
		b->h_tri_mass[e] = dens * area;
	}
	reset_mass(b);

	// device arena
	const int np = P.npad;
	float* shape_dev = nullptr;  // mesh triangles and SDF voxels of the world shapes
	auto carve = [&](Carver& C, DevBody& D) {
		D.slice_ptr = C.take<int>(P.nslices + 1);
		D.col = C.take<int>(P.nslots);
		D.rowlen = C.take<uint8_t>(np);
		D.A32 = C.take<float>(9 * (size_t)P.nslots);
		D.tet_cstart = C.take<uint32_t>(P.tet.items);
		D.tet_ccnt = C.take<uint16_t>(P.tet.items);
		D.tet_clist = C.take<uint32_t>(P.tet.len);
		D.blk_cstart = C.take<uint32_t>(P.blk.items);
		D.blk_ccnt = C.take<uint16_t>(P.blk.items);
		D.blk_clist = C.take<uint32_t>(P.blk.len);
		D.vt_start = C.take<uint32_t>(P.vt.items);
		D.vt_cnt = C.take<uint16_t>(P.vt.items);
		D.vt_list = C.take<uint32_t>(P.vt.len);
		D.vb_start = C.take<uint32_t>(P.vb.items);
		D.vb_cnt = C.take<uint16_t>(P.vb.items);
		D.vb_list = C.take<uint32_t>(P.vb.len);
		D.x = C.take<float>(3 * (size_t)n);
		D.v = C.take<float>(3 * (size_t)n);
		D.fext = C.take<float>(3 * (size_t)n);
		D.trans = C.take<float>(3 * (size_t)n);
		D.xi = C.take<float>(3 * (size_t)n);
		D.vi = C.take<float>(3 * (size_t)n);
		D.mass = C.take<float>(n);
		D.invmass = C.take<float>(n);
		D.damping = C.take<float>(n);
		D.type = C.take<int8_t>(n);
		D.tet = C.take<uint4>(b->nt);
		D.tet_invE = C.take<float>(9 * (size_t)b->nt);
		D.tet_mat = C.take<float4>(b->nt);
		D.tet_q = C.take<float4>(b->nt);
		D.tet_rec = C.take<float4>(4 * (size_t)b->nt);
		D.tet_bc = C.take<float>(12 * (size_t)b->nt);
		D.tri = C.take<uint4>(b->ntr_fix);
		D.tri_x = C.take<float>(6 * (size_t)b->ntr);
		D.tri_invS = C.take<float>(4 * (size_t)b->ntr);
		D.tri_K = C.take<float>(36 * (size_t)b->ntr);
		D.tri_kd = C.take<float>(b->ntr);
		D.spr = C.take<uint2>(b->ns);
		D.spr_L0 = C.take<float>(b->ns);
		D.spr_ks = C.take<float>(b->ns);
		D.spr_kd = C.take<float>(b->ns);
		D.bw = C.take<uint4>(nbw);
		D.bw_c = C.take<float>((size_t)kBwFloats * nbw);
		D.ms = C.take<uint4>(nms);
		D.ms_c = C.take<float>((size_t)kMouseFloats * nms);
		D.blocks = C.take<float>(9 * (9 * (size_t)b->ntr + b->ns + 9 * (size_t)nbw + 16 * (size_t)nms));
		D.bvec = C.take<float>(3 * (3 * (size_t)b->ntr + b->ns + 3 * (size_t)nbw + 4 * (size_t)nms));
		D.srad = C.take<float>(b->nw ? n : 0);
		D.sfric = C.take<float>(b->nw ? n : 0);
		D.c_exists = C.take<uint8_t>((size_t)n * b->nw);
		D.c_apply = C.take<uint8_t>((size_t)n * b->nw);
		D.c_nf = C.take<float>((size_t)n * b->nw);
		D.c_normal = C.take<float>(3 * (size_t)n * b->nw);
		D.shapes = C.take<DevShape>(b->nw);
		shape_dev = C.take<float>(b->nw ? shape_data.size() : 0);
		D.sc = C.take<Scalars>(1);
		D.partials = C.take<double>(kMaxPartials);
		D.team_partials = C.take<double>(kMaxPartials);
		b->staging = C.take<float>(3 * (size_t)n);
	};
	DevBody D{};
	Carver sizer;
	carve(sizer, D);
	char* mem = nullptr;
	cudaError_t ce = cudaMalloc(&mem, sizer.off);
	if (ce != cudaSuccess)
	{
		free_pattern(&P);
		delete b;
		return cuda_fail(ce, "allocating body");
	}
	b->arena = mem;
	b->arena_bytes = sizer.off;
	Carver C;
	C.base = mem;
	carve(C, D);
	D.n = (int)n;
	D.nslices = P.nslices;
	D.npad = np;
	D.nslots = P.nslots;
	D.nt = (int)b->nt;
	D.ntr = (int)b->ntr;
	D.ns = (int)b->ns;
	D.nw = (int)b->nw;
	D.nbw = (int)nbw;
	D.nms = (int)nms;
	D.maxw = P.maxw;
	D.contacts = b->nw > 0 ? 1 : 0;
	if (b->nw) bind_shape_data(shapes, shape_dev);
	D.gravity[0] = d->gravity[0];
	D.gravity[1] = d->gravity[1];
	D.gravity[2] = d->gravity[2];
	D.precond = B3G_PRECOND_JACOBI;
	// the ratio the element kernel stores in each record (mu > 0 ? lambda / mu : 0), when it is
	// the same for every tetrahedron
	D.tet_ratio = -1.0f;
	for (uint32_t k = 0; k < b->nt; ++k)
	{
		const float r = tet_mat[k].z > 0.0f ? tet_mat[k].y / tet_mat[k].z : 0.0f;
		if (k == 0) D.tet_ratio = r;
		else if (r != D.tet_ratio)
		{
			D.tet_ratio = -1.0f;
			break;
		}
	}
	b->d = D;

	cudaStream_t st = ctx->stream;
	std::vector<int8_t> type8(n);
	for (uint32_t i = 0; i < n; ++i) type8[i] = (int8_t)d->types[i];
	std::vector<float> zeros3(3 * (size_t)n, 0.0f), damping(n, 0.0f);
	if (d->damping) damping.assign(d->damping, d->damping + n);
	std::vector<uint2> spr(b->ns);
	for (uint32_t e = 0; e < b->ns; ++e) spr[e] = make_uint2(d->springs[2 * e], d->springs[2 * e + 1]);
	std::vector<int8_t> hold;  // keep host buffers alive until the stream is synchronised
	auto up = [&](const void* dst, const void* src, size_t bytes) {
		if (ce != cudaSuccess || bytes == 0 || !src) return;
		ce = cudaMemcpyAsync((void*)dst, src, bytes, cudaMemcpyHostToDevice, st);
	};
	ce = cudaMemsetAsync(mem, 0, sizer.off, st);
	up(D.slice_ptr, P.slice_ptr, (P.nslices + 1) * sizeof(int));
	up(D.col, P.col, P.nslots * sizeof(int));
	up(D.rowlen, P.rowlen, np);
	auto up_lists = [&](const uint32_t* ds, const uint16_t* dc, const uint32_t* dl, const Pattern::Lists& L) {
		up(ds, L.start, L.items * sizeof(uint32_t));
		up(dc, L.cnt, L.items * sizeof(uint16_t));
		up(dl, L.list, L.len * sizeof(uint32_t));
	};
	up_lists(D.tet_cstart, D.tet_ccnt, D.tet_clist, P.tet);
	up_lists(D.blk_cstart, D.blk_ccnt, D.blk_clist, P.blk);
	up_lists(D.vt_start, D.vt_cnt, D.vt_list, P.vt);
	up_lists(D.vb_start, D.vb_cnt, D.vb_list, P.vb);
	up(D.x, d->positions, 3 * (size_t)n * sizeof(float));
	up(D.v, d->velocities ? (const void*)d->velocities : (const void*)zeros3.data(), 3 * (size_t)n * sizeof(float));
	up(D.mass, b->h_mass.data(), n * sizeof(float));
	up(D.invmass, b->h_invmass.data(), n * sizeof(float));
	up(D.damping, damping.data(), n * sizeof(float));
	up(D.type, type8.data(), n);
	up(D.tet, tet.data(), b->nt * sizeof(uint4));
	up(D.tet_invE, tet_invE.data(), tet_invE.size() * sizeof(float));
	up(D.tet_mat, tet_mat.data(), b->nt * sizeof(float4));
	up(D.tet_q, tet_q.data(), b->nt * sizeof(float4));
	up(D.tri, tri.data(), b->ntr_fix * sizeof(uint4));
	up(D.tri_x, tri_x.data(), tri_x.size() * sizeof(float));
	up(D.tri_invS, tri_invS.data(), tri_invS.size() * sizeof(float));
	up(D.tri_K, tri_K.data(), tri_K.size() * sizeof(float));
	up(D.tri_kd, tri_kd.data(), tri_kd.size() * sizeof(float));
	up(D.spr, spr.data(), b->ns * sizeof(uint2));
	up(D.spr_L0, d->spring_rest_length, b->ns * sizeof(float));
	up(D.spr_ks, d->spring_stiffness, b->ns * sizeof(float));
	up(D.spr_kd, d->spring_damping, b->ns * sizeof(float));
	up(D.bw, cf.bw.data(), nbw * sizeof(uint4));
	up(D.bw_c, cf.bw_c.data(), cf.bw_c.size() * sizeof(float));
	up(D.ms, cf.ms.data(), nms * sizeof(uint4));
	up(D.ms_c, cf.ms_c.data(), cf.ms_c.size() * sizeof(float));
	if (b->nw)
	{
		up(D.srad, d->sphere_radius, n * sizeof(float));
		if (d->sphere_friction) up(D.sfric, d->sphere_friction, n * sizeof(float));
		up(D.shapes, shapes.data(), shapes.size() * sizeof(DevShape));
		up(shape_dev, shape_data.data(), shape_data.size() * sizeof(float));
	}
	if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
	free_pattern(&P);
	if (ce != cudaSuccess)
	{
		cudaFree(mem);
		delete b;
		return cuda_fail(ce, "uploading body");
	}
	int rc = ensure_precision(b, kP32);
	if (rc != B3G_OK)
	{
		cudaFree(mem);
		delete b;
		return rc;
	}
	ctx->live_bodies.push_back(b);
	*out = b;
	return B3G_OK;
}

// Device memory of a body (its context is current and its stream idle).
static void release_body_memory(b3g_body* b)
{
	for (int k = 0; k < 3; ++k)
		if (b->prec[k].mem) cudaFree(b->prec[k].mem);
	if (b->arena) cudaFree(b->arena);
	if (b->ray_buf) cudaFree(b->ray_buf);
	if (b->filt) cudaFree(b->filt);
	for (auto& g : b->chunk_graphs) cudaGraphExecDestroy(g.exec);
	b->chunk_graphs.clear();
	for (auto& g : b->fcg_graphs) cudaGraphExecDestroy(g.exec);
	b->fcg_graphs.clear();
	for (int k = 0; k < 3; ++k) b->prec[k] = PrecBuffers();
	b->arena = nullptr;
	b->ray_buf = nullptr;
	b->ray_cap = 0;
	b->filt = nullptr;
}

int b3g_body_destroy(b3g_body* b)
{
	if (!b) return B3G_OK;
	b3g_context* c = b->ctx;
	if (!c)
	{
		// its context was destroyed first and already released the device memory
		delete b;
		return B3G_OK;
	}
	cudaSetDevice(c->device);
	cudaStreamSynchronize(c->stream);
	forget_body_in_batch_cache(c, b);
	if (std::find(c->xfer_bodies.begin(), c->xfer_bodies.end(), b) != c->xfer_bodies.end())
		c->xfer_bodies.clear();  // a later body at the same address must not reuse the table
	c->live_bodies.erase(std::remove(c->live_bodies.begin(), c->live_bodies.end(), b), c->live_bodies.end());
	release_body_memory(b);
	delete b;
	return B3G_OK;
}

int b3g_body_info(const b3g_body* b, uint64_t info[6])
{
	if (!b || !info) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	info[0] = b->n;
	info[1] = b->nt;
	info[2] = b->ntr;
	info[3] = b->ns;
	info[4] = b->nnzb;
	info[5] = (uint64_t)b->d.nslots;
	return B3G_OK;
}

int b3g_body_device_bytes(const b3g_body* b, uint64_t* bytes)
{
	if (!b || !bytes) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	uint64_t t = b->arena_bytes;
	for (int k = 0; k < 3; ++k) t += b->prec[k].bytes;
	*bytes = t;
	return B3G_OK;
}

// kPcgChunk iterations of the per-op PCG from iteration j0 (a multiple of kPcgChunk, so even):
// one replay of the chunk's CUDA graph, captured on first use. The kernels decide on the device
// whether the solve already finished; the host only checks between chunks. A chunk's launches
// depend on j0 only through which iterations refresh, so a handful of graphs serve every chunk.
static cudaError_t pcg_chunk(b3g_body* b, const DevBody& D, int prec, int precond, int j0, int refresh,
                             cudaStream_t st)
{
	const unsigned mask = pcg_resid_mask(prec, j0, kPcgChunk, refresh);
	for (const auto& g : b->chunk_graphs)
		if (g.prec == prec && g.precond == precond && g.refresh == refresh && g.resid_mask == mask)
			return cudaGraphLaunch(g.exec, st);
	op_pcg_prime(D, prec);
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	cudaError_t e = cudaStreamIsCapturing(st, &cs);
	if (e == cudaSuccess && cs == cudaStreamCaptureStatusNone) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
	else e = cudaErrorStreamCaptureUnsupported;
	if (e != cudaSuccess)
	{
		// no graph (the stream is captured by someone else, or capture is unavailable): launch
		// the chunk's kernels one by one
		cudaGetLastError();
		e = cudaSuccess;
		for (int k = 0; k < kPcgChunk && e == cudaSuccess; ++k) e = op_pcg_iteration(D, prec, j0 + k, refresh, st);
		return e;
	}
	for (int k = 0; k < kPcgChunk && e == cudaSuccess; ++k) e = op_pcg_iteration(D, prec, j0 + k, refresh, st);
	cudaGraph_t graph = nullptr;
	const cudaError_t ec = cudaStreamEndCapture(st, &graph);
	if (e == cudaSuccess) e = ec;
	cudaGraphExec_t exec = nullptr;
	if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
	if (graph) cudaGraphDestroy(graph);
	if (e != cudaSuccess) return e;
	b->chunk_graphs.push_back({prec, precond, refresh, mask, exec});
	return cudaGraphLaunch(exec, st);
}

// Inner BF16 PCG iterations per outer iteration of the BF16 mode (B3G_BF16_INNER overrides).
static int bf16_inner_iterations()
{
	static const int m = [] {
		const char* e = std::getenv("B3G_BF16_INNER");
		const int v = e ? std::atoi(e) : 0;
		return v > 0 ? v : 20;
	}();
	return m;
}

// The BF16 mode's solve: a flexible CG on the FP32 blocks (float-float solution, the true residual
// refreshed every refresh_period outer iterations) preconditioned by a fixed number of Jacobi-PCG
// iterations with the BF16 blocks (from z = 0). The matrix is read mostly as BF16: per outer
// iteration one FP32 product and bf16_inner_iterations() BF16 products. Unlike refining a BF16
// PCG, this converges when the BF16 rounding of the matrix times its condition number exceeds
// one: the outer iteration only needs the inner solve to be a fair approximation of A^-1.
// max_pcg_iterations bounds the outer iterations; the step's PCG statistics count them.
static cudaError_t run_bf16_fcg(b3g_body* b, const DevBody& D, const b3g_solver_config& cfg, cudaStream_t st)
{
	const PrecBuffers& pb = b->prec[kPBF];
	DevBody Bin = D;
	Bin.pb = D.r;  // the inner solve's right-hand side is the outer residual
	Bin.py = pb.fcg_vec[0];
	Bin.r = pb.fcg_vec[1];
	Bin.s = pb.fcg_vec[2];
	Bin.d = pb.fcg_vec[3];
	Bin.d2 = pb.fcg_vec[4];
	Bin.q = pb.fcg_vec[5];
	Bin.xff = nullptr;
	Bin.sc = pb.fcg_inner;
	const int m = bf16_inner_iterations();
	Scalars* hs = b->ctx->h_scalars;
	// one outer iteration's launches: the inner solve, then the outer direction, product and update
	auto launch = [&](int k) -> cudaError_t {
		cudaError_t e = op_fcg_inner_begin(Bin, D.sc, m, 0.0, st);
		for (int j = 0; j < m && e == cudaSuccess; ++j) e = op_fcg_inner_iteration(Bin, j, st);
		// p and p_prev alternate between d and d2, q and q_prev between q and the workspace's
		DevBody Bo = D;
		if (k & 1) std::swap(Bo.d, Bo.d2);
		float* qa = (float*)D.q;
		float* qb = (float*)pb.fcg_vec[6];
		Bo.q = (k & 1) ? qb : qa;
		if (e == cudaSuccess) e = op_fcg_outer(Bo, (const float*)Bin.py, (k & 1) ? qa : qb, pb.fcg, pb.fcg_part, k, st);
		return e;
	};
	// ... replayed as a CUDA graph per variant (first, odd, even), captured on first use; launched
	// directly when the stream is being captured by the caller
	auto run = [&](int k) -> cudaError_t {
		const int variant = k == 0 ? 0 : ((k & 1) ? 1 : 2);
		for (const auto& g : b->fcg_graphs)
			if (g.variant == variant && g.inner == m && g.precond == D.precond) return cudaGraphLaunch(g.exec, st);
		op_pcg_prime(Bin, kPBF);
		op_pcg_prime(D, kP32);
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		cudaError_t e = cudaStreamIsCapturing(st, &cs);
		if (e != cudaSuccess || cs != cudaStreamCaptureStatusNone ||
		    cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
		{
			cudaGetLastError();
			return launch(k);
		}
		e = launch(k);
		cudaGraph_t graph = nullptr;
		const cudaError_t ec = cudaStreamEndCapture(st, &graph);
		if (e == cudaSuccess) e = ec;
		cudaGraphExec_t exec = nullptr;
		if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
		if (graph) cudaGraphDestroy(graph);
		if (e != cudaSuccess) return e;
		b->fcg_graphs.push_back({variant, m, D.precond, exec});
		return cudaGraphLaunch(exec, st);
	};
	cudaError_t e = cudaSuccess;
	for (int k = 0; k < (int)cfg.max_pcg_iterations && e == cudaSuccess; ++k)
	{
		e = run(k);
		if (e == cudaSuccess) e = cudaMemcpyAsync(&hs->done, &D.sc->done, sizeof(int), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e == cudaSuccess && hs->done) break;
	}
	return e;
}

int b3g_body_step(b3g_body* b, float dt, const b3g_solver_config* cfg_in, b3g_step_stats* stats)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null body");
	if (!b->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "the body's context was destroyed");
	b3g_solver_config cfg;
	if (cfg_in) cfg = *cfg_in;
	else b3g_solver_config_default(&cfg);
	int rc = check_config(&cfg, true);
	if (rc != B3G_OK) return rc;
	cudaSetDevice(b->ctx->device);
	cudaStream_t st = b->ctx->stream;
	cudaError_t e;
	if (!(dt > 0.0f))
	{
		e = op_nostep(b->d, st);
		if (e != cudaSuccess) return cuda_fail(e, "step");
		if (stats)
		{
			std::memset(stats, 0, sizeof(*stats));
			e = cudaStreamSynchronize(st);
			if (e != cudaSuccess) return cuda_fail(e, "step");
		}
		return B3G_OK;
	}
	const int prec = prec_of(&cfg);
	rc = ensure_precision(b, prec);
	if (rc != B3G_OK) return rc;
	DevBody D = dev_for(b, prec, cfg.preconditioner, true);
	if (cfg.contact_mode == B3G_CONTACT_FILTER && b->d.contacts)
	{
		rc = ensure_filter(b);
		if (rc != B3G_OK) return rc;
		D.filt = b->filt;
	}
	const int newton = (int)std::max<uint32_t>(1u, cfg.force_iterations);
	e = op_begin(D, st, (int)cfg.max_pcg_iterations, cfg.pcg_tolerance * cfg.pcg_tolerance, (int)cfg.refresh_period,
	             cfg.newton_tolerance * cfg.newton_tolerance);
	const int chunk = kPcgChunk;
	Scalars* hs = b->ctx->h_scalars;
	for (int k = 0; k < newton && e == cudaSuccess; ++k)
	{
		StepParamsHost P{dt, k == 0 ? 1 : 0};
		if (k > 0) e = op_newton_begin(D, st);
		else if (D.filt && e == cudaSuccess) e = op_contact_filter(D, dt, st);
		if (e == cudaSuccess) e = op_elements(D, P, st);
		if (e == cudaSuccess) e = op_assemble(D, P, prec, k == 0, st);
		if (e == cudaSuccess && k > 0) e = op_pcg_init(D, prec, st);
		// the host first asks whether the solve ended one chunk before the previous step's solve
		// did: the chunks before that queue back to back (a chunk launched after the end returns
		// at once from every kernel)
		const int quiet = std::max(0, b->pcg_chunks_hint - 1);
		int chunks = 0;
		if (prec == kPBF && e == cudaSuccess) e = run_bf16_fcg(b, D, cfg, st);
		for (int it = 0; prec != kPBF && it < (int)cfg.max_pcg_iterations && e == cudaSuccess; it += chunk)
		{
			if (it + chunk <= (int)cfg.max_pcg_iterations)
				e = pcg_chunk(b, D, prec, (int)cfg.preconditioner, it, (int)cfg.refresh_period, st);
			else
				for (int j = 0; it + j < (int)cfg.max_pcg_iterations && e == cudaSuccess; ++j)
					e = op_pcg_iteration(D, prec, it + j, (int)cfg.refresh_period, st);
			if (e != cudaSuccess) break;
			if (++chunks <= quiet) continue;
			e = cudaMemcpyAsync(&hs->done, &D.sc->done, sizeof(int), cudaMemcpyDeviceToHost, st);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			if (e == cudaSuccess && hs->done) break;
		}
		if (k == 0) b->pcg_chunks_hint = chunks;
		if (e != cudaSuccess) break;
		const bool single = newton == 1;
		e = op_final(D, P, prec, single ? 1 : 0, st);
		if (e != cudaSuccess || single) break;
		e = cudaMemcpyAsync(&hs->newton_done, &D.sc->newton_done, sizeof(int), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e == cudaSuccess && (hs->newton_done || k == newton - 1))
		{
			e = op_post(D, dt, st);
			break;
		}
	}
	if (e != cudaSuccess) return cuda_fail(e, "step");
	if (stats)
	{
		Scalars sc;
		rc = read_scalars(b, &sc);
		if (rc != B3G_OK) return rc;
		stats_from(sc, stats);
		b->last = *stats;
	}
	return B3G_OK;
}

int b3g_body_get_stats(b3g_body* b, b3g_step_stats* stats)
{
	if (!b || !stats) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	Scalars sc;
	int rc = read_scalars(b, &sc);
	if (rc != B3G_OK) return rc;
	stats_from(sc, stats);
	return B3G_OK;
}

int b3g_body_get_state(b3g_body* b, float* positions, float* velocities)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null body");
	if (!b->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "the body's context was destroyed");
	cudaStream_t st = b->ctx->stream;
	cudaError_t e = cudaSuccess;
	size_t bytes = 3 * (size_t)b->n * sizeof(float);
	if (positions) e = cudaMemcpyAsync(positions, b->d.x, bytes, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess && velocities) e = cudaMemcpyAsync(velocities, b->d.v, bytes, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "get_state");
}

int b3g_body_set_state(b3g_body* b, const float* positions, const float* velocities)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null body");
	if (!b->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "the body's context was destroyed");
	cudaStream_t st = b->ctx->stream;
	cudaError_t e = cudaSuccess;
	size_t bytes = 3 * (size_t)b->n * sizeof(float);
	if (positions) e = cudaMemcpyAsync(b->d.x, positions, bytes, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess && velocities) e = cudaMemcpyAsync(b->d.v, velocities, bytes, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "set_state");
}

int b3g_body_apply_forces(b3g_body* b, const float* forces)
{
	if (!b || !forces) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	cudaStream_t st = b->ctx->stream;
	size_t count = 3 * (size_t)b->n;
	cudaError_t e = cudaMemcpyAsync(b->staging, forces, count * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = op_accumulate(b->d.fext, b->staging, count, st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "apply_forces");
}

int b3g_body_apply_translations(b3g_body* b, const float* translations)
{
	if (!b || !translations) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	cudaStream_t st = b->ctx->stream;
	size_t count = 3 * (size_t)b->n;
	cudaError_t e = cudaMemcpyAsync(b->staging, translations, count * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = op_accumulate(b->d.trans, b->staging, count, st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "apply_translations");
}

int b3g_body_set_types(b3g_body* b, const int32_t* types)
{
	if (!b || !types) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	for (uint32_t i = 0; i < b->n; ++i)
		if (types[i] < 0 || types[i] > 2) return fail(B3G_ERROR_INVALID_ARGUMENT, "vertex %u has type %d", i, types[i]);
	cudaStream_t st = b->ctx->stream;
	std::vector<int8_t> t8(b->n);
	for (uint32_t i = 0; i < b->n; ++i) t8[i] = (int8_t)types[i];
	// staging holds 12 bytes per vertex: enough for the new types
	cudaError_t e = cudaMemcpyAsync(b->staging, t8.data(), b->n, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = op_set_types(b->d, (const int8_t*)b->staging, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return cuda_fail(e, "set_types");
	b->h_type.assign(types, types + b->n);
	reset_mass(b);
	return upload_masses(b);
}

// rotations in the caller's element order; the device keeps them in storage order
int b3g_body_get_rotations(b3g_body* b, float* q)
{
	if (!b || !q) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	cudaStream_t st = b->ctx->stream;
	std::vector<float4> stored(b->nt);
	cudaError_t e = cudaMemcpyAsync(stored.data(), b->d.tet_q, b->nt * sizeof(float4), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return cuda_fail(e, "get_rotations");
	for (uint32_t k = 0; k < b->nt; ++k) std::memcpy(q + 4 * (size_t)b->tet_order[k], &stored[k], sizeof(float4));
	return B3G_OK;
}

int b3g_body_set_rotations(b3g_body* b, const float* q)
{
	if (!b || !q) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	cudaStream_t st = b->ctx->stream;
	std::vector<float4> stored(b->nt);
	for (uint32_t k = 0; k < b->nt; ++k) std::memcpy(&stored[k], q + 4 * (size_t)b->tet_order[k], sizeof(float4));
	cudaError_t e = cudaMemcpyAsync(b->d.tet_q, stored.data(), b->nt * sizeof(float4), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "set_rotations");
}

int b3g_body_contact_fixtures(const b3g_body* b, uint32_t* fixtures)
{
	if (!b || !fixtures) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*fixtures = b->d.contacts ? b->nw : 0u;
	return B3G_OK;
}

// vertex-major per (vertex, fixture): exists, apply friction, accumulated normal force, normal
int b3g_body_get_contacts(b3g_body* b, uint8_t* exists, uint8_t* apply_friction, float* normal_force, float* normals)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null body");
	if (!b->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "the body's context was destroyed");
	const size_t c = b->d.contacts ? (size_t)b->n * b->nw : 0;
	if (!c) return B3G_OK;
	cudaStream_t st = b->ctx->stream;
	cudaError_t e = cudaSuccess;
	if (exists) e = cudaMemcpyAsync(exists, b->d.c_exists, c, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess && apply_friction) e = cudaMemcpyAsync(apply_friction, b->d.c_apply, c, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess && normal_force)
		e = cudaMemcpyAsync(normal_force, b->d.c_nf, c * sizeof(float), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess && normals) e = cudaMemcpyAsync(normals, b->d.c_normal, 3 * c * sizeof(float), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "get_contacts");
}

int b3g_body_set_contacts(b3g_body* b, const uint8_t* exists, const uint8_t* apply_friction, const float* normal_force,
                          const float* normals)
{
	if (!b) return fail(B3G_ERROR_INVALID_ARGUMENT, "null body");
	if (!b->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "the body's context was destroyed");
	const size_t c = b->d.contacts ? (size_t)b->n * b->nw : 0;
	if (!c) return B3G_OK;
	if (exists)
		for (size_t k = 0; k < c; ++k)
			if (exists[k] > 1) return fail(B3G_ERROR_INVALID_ARGUMENT, "exists[%zu] is %u (0 or 1)", k, exists[k]);
	if (apply_friction)
		for (size_t k = 0; k < c; ++k)
			if (apply_friction[k] > 1)
				return fail(B3G_ERROR_INVALID_ARGUMENT, "apply_friction[%zu] is %u (0 or 1)", k, apply_friction[k]);
	cudaStream_t st = b->ctx->stream;
	cudaError_t e = cudaSuccess;
	if (exists) e = cudaMemcpyAsync(b->d.c_exists, exists, c, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess && apply_friction) e = cudaMemcpyAsync(b->d.c_apply, apply_friction, c, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess && normal_force)
		e = cudaMemcpyAsync(b->d.c_nf, normal_force, c * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess && normals) e = cudaMemcpyAsync(b->d.c_normal, normals, 3 * c * sizeof(float), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "set_contacts");
}

int b3g_body_ray_cast(b3g_body* b, const float* segments, uint32_t count, b3g_ray_hit* hits)
{
	if (!b || (count && (!segments || !hits))) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (!b->ctx) return fail(B3G_ERROR_INVALID_ARGUMENT, "the body's context was destroyed");
	if (count == 0) return B3G_OK;
	for (uint64_t k = 0; k < 6 * (uint64_t)count; ++k)
		if (!std::isfinite(segments[k])) return fail(B3G_ERROR_INVALID_ARGUMENT, "segment %u is not finite", (uint32_t)(k / 6));
	cudaSetDevice(b->ctx->device);
	cudaStream_t st = b->ctx->stream;
	auto layout = [](uint32_t cap, size_t* off_keys, size_t* off_hits) {
		*off_keys = align_up(6 * sizeof(float) * (size_t)cap);
		*off_hits = *off_keys + align_up(sizeof(unsigned long long) * (size_t)cap);
		return *off_hits + align_up(sizeof(b3g_ray_hit) * (size_t)cap);
	};
	size_t off_keys, off_hits;
	if (count > b->ray_cap)
	{
		uint32_t cap = std::max<uint32_t>(count, 64);
		cudaError_t e = cudaStreamSynchronize(st);
		if (e != cudaSuccess) return cuda_fail(e, "ray cast");
		if (b->ray_buf) cudaFree(b->ray_buf);
		b->ray_buf = nullptr;
		b->ray_cap = 0;
		e = cudaMalloc(&b->ray_buf, layout(cap, &off_keys, &off_hits));
		if (e != cudaSuccess) return cuda_fail(e, "allocating ray cast scratch");
		b->ray_cap = cap;
	}
	layout(b->ray_cap, &off_keys, &off_hits);
	float* dseg = (float*)b->ray_buf;
	unsigned long long* keys = (unsigned long long*)(b->ray_buf + off_keys);
	b3g_ray_hit* dhits = (b3g_ray_hit*)(b->ray_buf + off_hits);
	cudaError_t e = cudaMemcpyAsync(dseg, segments, 6 * sizeof(float) * (size_t)count, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = op_ray_cast(b->d, (int)b->ntr_fix, dseg, count, keys, dhits, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(hits, dhits, sizeof(b3g_ray_hit) * (size_t)count, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return e == cudaSuccess ? B3G_OK : cuda_fail(e, "ray cast");
}

int b3g_body_get_masses(b3g_body* b, float* masses)
{
	if (!b || !masses) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	std::memcpy(masses, b->h_mass.data(), b->n * sizeof(float));
	return B3G_OK;
}

} // extern "C"
