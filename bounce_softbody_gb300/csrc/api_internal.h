// Host-side objects behind the opaque handles of include/b3g.h.
#pragma once

#include "internal.h"
#include "ops.h"

#include <cuda_runtime.h>

#include <vector>

struct BatchCache;
namespace b3g {
struct SparseObject;
struct SparseWork;
}

struct b3g_context
{
	int device = 0;
	int sm_count = 0;
	cudaStream_t stream = nullptr;
	b3g::Scalars* h_scalars = nullptr;   // pinned, 1024 entries
	BatchCache* batch = nullptr;
	// b3g_batch_set_launch_timing: batched steps launch directly (no graph) with events around
	// the assembly and PCG launches; device milliseconds accumulate here
	bool launch_timing = false;
	cudaEvent_t tev[4] = {nullptr, nullptr, nullptr, nullptr};
	double t_assembly_ms = 0.0, t_pcg_ms = 0.0, t_elements_ms = 0.0;
	unsigned long long t_steps = 0;
	// batched host transfers (b3g_batch_apply_forces / b3g_batch_get_state): one contiguous
	// device staging buffer, one copy each way and one scatter / gather launch per call; the
	// body table is rebuilt when the body list changes
	float* xfer = nullptr;
	size_t xfer_cap = 0;                 // floats
	b3g::XferBody* xfer_table = nullptr;
	uint32_t xfer_table_cap = 0;
	std::vector<b3g_body*> xfer_bodies;
	uint32_t xfer_max_n3 = 0;
	uint64_t xfer_total = 0;             // floats of the flat host array (3 per vertex)
	// live bodies: destroying the context releases their device memory and detaches them, so a
	// later b3g_body_destroy only frees the host object
	std::vector<b3g_body*> live_bodies;
	// asynchronous state reads (b3g_batch_get_state_async): a device snapshot of the bodies' x and
	// v copied to the host on a second stream, so that the copy overlaps the next step
	cudaStream_t copy_stream = nullptr;
	// overlapped force uploads from page-locked host arrays: an upload stream, two device staging
	// buffers taken in turn (up_cap floats each), and per buffer the events "copied" (upload
	// stream) and "consumed" (context stream, after the scatter that reads it)
	cudaStream_t up_stream = nullptr;
	float* up_buf = nullptr;
	size_t up_cap = 0;
	cudaEvent_t ev_up_copied[2] = {nullptr, nullptr}, ev_up_used[2] = {nullptr, nullptr};
	bool up_used_pending[2] = {false, false};
	int up_next = 0;
	// the batched step's split assembly: a second stream and its fork / join events
	cudaStream_t side_stream = nullptr;
	cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
	cudaEvent_t ev_snap = nullptr, ev_copied = nullptr;
	float* snap = nullptr;
	size_t snap_cap = 0;                 // floats
	bool copy_pending = false;
	// containers of include/b3g_sparse.h made on this context (released with it), and the
	// workspace of its solvers
	std::vector<b3g::SparseObject*> live_sparse;
	b3g::SparseWork* sparse_work = nullptr;
};

namespace b3g {

// Solver vectors and low-precision matrix storage for one precision mode.
struct PrecBuffers
{
	char* mem = nullptr;
	size_t bytes = 0;
	void* vec[7] = {};   // pb r d d2 q s py
	void* minv = nullptr;
	void* alo = nullptr;
	float* xff = nullptr;  // float-float solution (FP32 and BF16 modes), 8 floats per vertex
	// BF16 mode of the per-op step (flexible outer CG around inner BF16 PCG solves): the inner
	// solution z, the inner r s d d2 q, the outer q of the previous iteration (7 vectors, 4-wide),
	// the inner solve's scalars, the outer's extra scalars and their reduction partials
	void* fcg_vec[7] = {};
	Scalars* fcg_inner = nullptr;
	FcgScalars* fcg = nullptr;
	double* fcg_part = nullptr;
};

} // namespace b3g

struct b3g_body
{
	b3g_context* ctx = nullptr;
	uint32_t n = 0, nt = 0, ntr = 0, ns = 0, nw = 0;
	uint32_t ntr_fix = 0;  // triangle mass fixtures (ntr of them are also membrane elements)
	uint64_t nnzb = 0;
	b3g::DevBody d{};
	char* arena = nullptr;
	size_t arena_bytes = 0;
	float* staging = nullptr;            // 3 floats per vertex of upload space
	b3g::PrecBuffers prec[3];
	// host copies needed by ResetMass / SetType
	std::vector<int32_t> h_type;
	std::vector<uint32_t> h_tets, h_tris;
	std::vector<uint32_t> tet_order;     // device storage order: element at each position
	std::vector<float> h_tet_mass, h_tri_mass, h_given_mass;
	std::vector<float> h_mass, h_invmass;
	b3g_step_stats last{};
	// ray cast scratch (segments, reduction keys, hits), grown on demand
	char* ray_buf = nullptr;
	uint32_t ray_cap = 0;
	// per-vertex constraints of filtered contacts, made on the first step in that mode
	float4* filt = nullptr;
	// the per-op PCG's chunks of kPcgChunk iterations, captured into CUDA graphs once per kind:
	// precision, preconditioner, refresh period and which iterations of the chunk refresh
	struct ChunkGraph
	{
		int prec, precond, refresh;
		unsigned resid_mask;
		cudaGraphExec_t exec;
	};
	std::vector<ChunkGraph> chunk_graphs;
	// the BF16 mode's outer iterations captured into CUDA graphs: variant 0 = the first outer
	// iteration, 1 / 2 = later odd / even ones (buffers alternate), for `inner` inner iterations
	struct FcgGraph
	{
		int variant, inner, precond;
		cudaGraphExec_t exec;
	};
	std::vector<FcgGraph> fcg_graphs;
	int pcg_chunks_hint = 0;  // chunks the previous step's first solve launched
};

namespace b3g {

int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* where);
void reset_mass(b3g_body* b);
int upload_masses(b3g_body* b);
int ensure_precision(b3g_body* b, int prec);
// refine: the per-op path's iterative refinement (float-float solution and refresh residual)
DevBody dev_for(const b3g_body* b, int prec, int precond, bool refine = false);
int prec_of(const b3g_solver_config* c);
// filter_ok: the caller steps filtered contacts (b3g_body_step, b3g_step_batch)
int check_config(const b3g_solver_config* c, bool filter_ok = false);
// the per-vertex constraint buffer of filtered contacts (made on first use)
int ensure_filter(b3g_body* b);
void stats_from(const Scalars& sc, b3g_step_stats* st);
int read_scalars(b3g_body* b, Scalars* out);

// device bytes of a body made from d, estimated on the host (partition.cpp)
uint64_t estimate_desc_bytes(const b3g_body_desc& d);

cudaError_t op_accumulate(float* dst, const float* src, size_t count, cudaStream_t st);
cudaError_t op_set_types(const DevBody& B, const int8_t* new_types, cudaStream_t st);

} // namespace b3g

void destroy_batch_cache(b3g_context* c);
// frees the device memory of every sparse container of the context and detaches them
void release_sparse(b3g_context* c);
void forget_body_in_batch_cache(b3g_context* c, b3g_body* b);
