// Internal layout of a body on the device, shared by the host builder (pattern.cpp), the
// kernels (kernels.cu, persistent.cu) and the C ABI (api.cu).
//
// Matrix storage: sliced block-ELL with 32 rows per slice ("SELL-32", one warp per slice, one
// lane per block row). Slice s owns slots [slice_ptr[s], slice_ptr[s+1]) = width_s * 32 slots,
// width_s a multiple of kGroup = 4. The k-th block of row i = 32 s + lane sits in
//   block_slot(s, k, lane) = slice_ptr[s] + 128 (k / 4) + 4 lane + k % 4,
// so one lane's four consecutive blocks are adjacent: a lane loads each of the 9 value planes of
// a group of four blocks, and their column ids, as single 16-byte vectors, and a warp's loads
// cover 512 consecutive bytes. Plane p (entry p = 3 * row + col of a 3x3 block) of every slot
// lives at p * nslots + slot. Slots past the end of a row hold zero blocks whose column is the
// row itself. The diagonal block is always k = 0.
// Per-slot contribution lists use the item index list_item(s, k, lane) = slice_ptr[s] + 32 k +
// lane (same range, different order) so that a warp reading the lists of its 32 rows at one k
// touches consecutive words.
//
// Solver vectors are 4-wide per vertex (x, y, z, unused) so a neighbour's value is one 16-byte
// load: component c of vertex i at 4 i + c. Vertex state (x, v, external force, translation)
// stays 3 floats per vertex, like b3Vec3 arrays.
#pragma once

#include <stdint.h>
#include <stddef.h>

#include <vector>

#include "../../include/b3g.h"

#include <vector_types.h>

#ifdef __CUDACC__
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#define B3G_HD __host__ __device__ __forceinline__
#else
#define B3G_HD inline
#endif

namespace b3g {

constexpr int kSlice = 32;
constexpr int kPcgChunk = 8;     // per-op PCG iterations between host checks of convergence
constexpr int kGroup = 4;

B3G_HD size_t block_slot(size_t base, int k, int lane) { return base + 128 * (size_t)(k >> 2) + 4 * lane + (k & 3); }
constexpr int kMaxWorld = 16;   // world fixtures per body
constexpr int kMaxTeamCtas = 16;

// Device-resident solver scalars of one body; everything the PCG decides is taken here.
struct Scalars
{
	double delta;      // r.s of the current residual
	double delta0;     // r0.s0
	double dq;         // d.q
	double alpha, beta;
	double tol2;       // pcg_tolerance^2
	double newton_err, newton_err0;
	double newton_tol2;
	int iter;          // PCG iteration of the current solve
	int max_iter;
	int done;          // current PCG solve finished
	int status;        // b3g_solve_status
	int newton_iter;
	int newton_done;
	int min_it, max_it;
	int refresh;       // refresh period
	unsigned counter;  // arrival counter of the deterministic grid reduction (plain path)
	int pending_check; // bf16 mode: recursive residual met the tolerance, confirm with a refresh
	int fault;         // a bounded device wait expired (the step's results are not valid)
	unsigned long long total_iters;  // PCG iterations of every step since creation
	unsigned long long total_steps;
};

// Scalars of the flexible outer CG of the BF16 mode (per-op path): z.q_prev, p.r, p.q of this
// iteration and of the previous one, and the arrival counter of its two-value reductions.
struct FcgScalars
{
	double gamma;      // z . q_prev
	double rho;        // p . r
	double pq;         // p . q
	double pq_prev;    // p_prev . q_prev
	unsigned counter;
	int pad;
};

// One static world shape (b3WorldFixture + b3Shape) on the device. Geometry is in world space
// except where the shape keeps a frame (box, sdf: rotation q, translation t; mesh triangles are
// stored transformed). lo / hi: the fixture's AABB as the reference computes it, for contact
// creation and persistence.
struct DevShape
{
	int type;                   // b3g_shape_type
	float radius;               // b3Shape::m_radius
	float friction;
	int count;                  // mesh: triangles
	float a[3], b[3], c[3];     // sphere: a center; capsule: a, b; triangle: a, b, c; box: a extents
	float q[4];                 // box, sdf, mesh: rotation (x, y, z, w)
	float t[3];                 // box, sdf, mesh: translation
	float lo[3], hi[3];         // fixture AABB
	float inv_scale[3];         // mesh: 1 / scale (query box in the unscaled mesh frame)
	int dims[3];                // sdf: voxels along x, y, z
	int invert;                 // sdf
	float glo[3], ghi[3];       // sdf: grid AABB in the shape frame
	const float* data;          // mesh: kMeshTriFloats per triangle; sdf: voxels
};

// Per mesh triangle: world-space vertices (9), world-space wing vertices (9), wing flags (3),
// unscaled mesh-frame AABB lower and upper (6), pad (1)
constexpr int kMeshTriFloats = 28;

// Baraff-Witkin triangle records (stretch_force.cpp:62-107, shear_force.cpp:51-92): alpha,
// inv_det, du1, dv1, du2, dv2, dwu/dx (3), dwv/dx (3), then stiffness_u, damping_u, b_u,
// stiffness_v, damping_v, b_v (stretch) or stiffness, damping (shear).
constexpr int kBwFloats = 20;
constexpr int kMouseFloats = 6;
constexpr uint32_t kForceStretch = 0, kForceShear = 1;

// Everything a kernel needs about one body. Passed by value to the per-op kernels and read
// from a device array by the persistent batch kernel.
struct DevBody
{
	int n, nslices, npad, nslots;
	int nt, ntr, ns, nw;
	int nbw, nms;               // stretch/shear triangles, mouse springs
	int maxw;                   // widest slice
	int contacts;               // per-vertex contact spheres present

	// matrix structure
	const int* slice_ptr;       // nslices + 1
	const int* col;             // nslots
	const uint8_t* rowlen;      // npad (0 for padding rows)
	float* A32;                 // 9 * nslots
	void* Alo;                  // 9 * nslots of the precision's storage type (double / bf16), or null
	void* Minv;                 // 4 per vertex (scalar Jacobi) or 12 (three rows, block Jacobi), vector type

	// contribution lists in element order (deterministic), interleaved across the 32 lanes of a
	// slice: entry t of item j (a slot, or a row) sits at start[j] + 32 t, so a warp reading entry
	// t of its 32 items touches 128 consecutive bytes
	const uint32_t* tet_cstart; // per slot
	const uint16_t* tet_ccnt;   // per slot
	const uint32_t* tet_clist;  // e << 4 | a << 2 | b
	const uint32_t* blk_cstart; // per slot
	const uint16_t* blk_ccnt;
	const uint32_t* blk_clist;  // block index << 1 | negate
	const uint32_t* vt_start;   // per row (npad)
	const uint16_t* vt_cnt;
	const uint32_t* vt_list;    // 4 e + a
	const uint32_t* vb_start;   // per row (npad)
	const uint16_t* vb_cnt;
	const uint32_t* vb_list;    // vector index << 1 | negate

	// vertex state
	float* x;
	float* v;
	float* fext;
	float* trans;
	float* xi;                  // Newton iterate (force_iterations > 1)
	float* vi;
	const float* mass;
	const float* invmass;
	const float* damping;
	const int8_t* type;

	// tetrahedra
	// tetrahedra in device storage order (tet_storage_order); the per-tet arrays are planes of
	// nt entries, so that consecutive tetrahedra's values are consecutive words
	const uint4* tet;
	const float* tet_invE;      // 9 planes: plane 3 j + r = invE(r, j) (column-major like b3Mat33)
	const float4* tet_mat;      // volume, lambda, mu, stiffness damping
	float4* tet_q;              // rotation quaternion (x, y, z, w)
	float4* tet_rec;            // 4 planes, plane a: (sqrt(c mu) R g_a, lambda / mu), c = (h^2 + h kd) V
	float* tet_bc;              // 12 planes, plane 3 a + c: h * (f + dfdx w) of local vertex a

	// triangles
	const uint4* tri;           // 3 ids + pad
	const float* tri_x;         // 6 per tri: rest 2-D coordinates
	const float* tri_invS;      // 4 per tri (column-major 2x2)
	const float* tri_K;         // 36 per tri: 9 blocks of 2x2, block (a, b) at 4 (a + 3 b)
	const float* tri_kd;

	// springs
	const uint2* spr;
	const float* spr_L0;
	const float* spr_ks;
	const float* spr_kd;

	// Baraff-Witkin stretch and shear triangles, mouse springs
	const uint4* bw;            // 3 ids, kind in w (kForceStretch / kForceShear)
	const float* bw_c;          // kBwFloats per element (bw_setup)
	const uint4* ms;            // 4 ids: the dragged particle, then the triangle
	const float* ms_c;          // kMouseFloats per element: w2, w3, w4, stiffness, damping, length

	// explicit (non-tetrahedral) contributions. Blocks, 9 floats each: tri (a, b) at 9 e + 3 a + b,
	// spring at 9 Tr + s, stretch/shear (a, b) at 9 Tr + S + 9 e + 3 a + b, mouse (a, b) at
	// 9 Tr + S + 9 Bw + 16 e + 4 a + b. Vectors, 3 floats each: tri (a) at 3 e + a, spring at
	// 3 Tr + s, stretch/shear (a) at 3 Tr + S + 3 e + a, mouse (a) at 3 Tr + S + 3 Bw + 4 e + a.
	float* blocks;
	float* bvec;

	// contacts
	const float* srad;
	const float* sfric;
	const struct DevShape* shapes; // nw static world shapes (device array)
	uint8_t* c_exists;          // n * nw
	uint8_t* c_apply;
	float* c_nf;                // accumulated normal force
	float* c_normal;            // 3 per contact
	// filtered contacts (B3G_CONTACT_FILTER, per-op step only; null otherwise): per vertex the
	// constrained normal n (zero when free) and the normal velocity change zn of z = zn n
	float4* filt;

	// solver vectors (vector type), planar
	void* pb;
	void* r;
	void* d;
	void* d2;                   // second direction buffer (persistent kernel ping-pong)
	void* q;
	void* s;
	void* py;
	float* xff;                 // float-float solution for iterative refinement (per-op path, FP32
	                            // and BF16 modes): 8 floats per vertex, (hi x, y, z, 0) then
	                            // (lo x, y, z, 0); null = the solution is py

	float gravity[3];

	Scalars* sc;
	double* partials;           // reduction scratch of the per-op kernels (kMaxPartials)
	double* team_partials;      // reduction scratch of the grid team (persistent kernel)
	int precond;                // b3g_preconditioner
	float tet_ratio;            // lambda / mu when every tetrahedron has the same ratio, else -1
};

constexpr int kMaxPartials = 4096;

// Host-side result of the pattern builder (pattern.cpp).
struct Pattern
{
	int n = 0, nslices = 0, npad = 0, nslots = 0, maxw = 0;
	uint64_t nnzb = 0;
	int* slice_ptr = nullptr;
	int* col = nullptr;
	uint8_t* rowlen = nullptr;
	// interleaved lists (see DevBody): start / count per item, entries at start + 32 t
	struct Lists
	{
		uint32_t* start = nullptr;
		uint16_t* cnt = nullptr;
		uint32_t* list = nullptr;
		uint64_t len = 0;    // entries including the padding of each group of 32 items
		uint64_t items = 0;
	};
	Lists tet, blk, vt, vb;
};

// Builds the SELL-32 pattern and every contribution list. Returns false with a message on a
// malformed mesh (vertex index out of range, degenerate element). tet_rank (may be null: the
// identity) maps each tetrahedron to its position in device storage; the lists name that
// position, while each slot still lists its contributions in the caller's element order.
bool build_pattern(uint32_t n, uint32_t nt, const uint32_t* tets, uint32_t ntr, const uint32_t* tris,
                   uint32_t ns, const uint32_t* springs, uint32_t nbw, const uint32_t* bw, uint32_t nms,
                   const uint32_t* ms, const uint32_t* tet_rank, Pattern* out, char* err, size_t errlen);

// Device storage order of a body's tetrahedra (order[k] = the element stored at position k).
// When the mesh has few distinct vertex-offset signatures (t1 - t0, t2 - t0, t3 - t0), as a
// structured grid has, the tetrahedra are grouped by signature and ordered by first vertex
// within a group: rows that are neighbours in the vertex numbering then read neighbouring
// records. Any other mesh keeps its own order.
std::vector<uint32_t> tet_storage_order(uint32_t nt, const uint32_t* tets);
void free_pattern(Pattern* p);

} // namespace b3g
