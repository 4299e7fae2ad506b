/*
 * b3g — GB300-native implicit soft-body step behind a plain C ABI.
 *
 * This is the drop-in boundary for the implicit (backward-Euler) step of Bounce Softbody.
 * Every entry point takes plain pointers and sizes; host pointers unless the name says
 * "device". All functions return a b3g_status; b3g_last_error() gives the message of the last
 * failure on the calling thread. Nothing here falls back to the CPU: without a usable GPU the
 * context cannot be created and every call fails with B3G_ERROR_CUDA.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   b3g_body_create            b3Body::CreateParticle / CreateForce / CreateTetrahedron /
 *                              CreateTriangle / CreateSphere / CreateFixture and ResetMass
 *                              (include/bounce_softbody/dynamics/body.h:68-110,
 *                               src/bounce_softbody/dynamics/body.cpp:62-466)
 *   b3g_body_step              b3Body::Step(dt, forceIterations, forceSubIterations)
 *                              (include/bounce_softbody/dynamics/body.h:153,
 *                               src/bounce_softbody/dynamics/body.cpp:552-604), which runs
 *                              b3SparseSolveBE (include/bounce_softbody/sparse/sparse_force_solver.h:97)
 *                              and b3SparseSolveCG (include/bounce_softbody/sparse/sparse_solver.h:47)
 *   b3g_step_batch             no single counterpart: many independent b3Body::Step calls
 *   b3g_body_get_state /       b3Particle::GetPosition / GetVelocity / SetPosition / SetVelocity
 *   b3g_body_set_state         (include/bounce_softbody/dynamics/particle.h:75-90)
 *   b3g_body_apply_forces      b3Particle::ApplyForce (particle.h:96)
 *   b3g_body_apply_translations b3Particle::ApplyTranslation (particle.h:104)
 *   b3g_body_set_types         b3Particle::SetType (particle.h:72, src/bounce_softbody/dynamics/particle.cpp:58-87)
 *   b3g_body_get_rotations     b3TetrahedronElementForce::m_q, the warm-started element rotation
 *                              (include/bounce_softbody/dynamics/forces/tetrahedron_element_force.h:154)
 *   b3g_body_get_stats         b3_forceSolverIterations / Min / MaxSubIterations
 *                              (src/bounce_softbody/dynamics/force_solver.cpp:29-34)
 * The sparse containers and the CG / backward-Euler solvers as calls of their own
 * (b3SparseMat33, b3DenseVec3, b3DiagMat33, b3SparseSolveCG, b3SparseSolveBE with a force-model
 * callback) are in b3g_sparse.h.
 */
#ifndef B3G_H
#define B3G_H

#include <stdint.h>

#if defined(__GNUC__)
#define B3G_API __attribute__((visibility("default")))
#else
#define B3G_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct b3g_context b3g_context;
typedef struct b3g_body b3g_body;

typedef enum b3g_status
{
	B3G_OK = 0,
	B3G_ERROR_INVALID_ARGUMENT = 1,
	B3G_ERROR_CUDA = 2,
	B3G_ERROR_OUT_OF_MEMORY = 3,
	B3G_ERROR_UNSUPPORTED = 4
} b3g_status;

/* How the last PCG solve of a step ended (the reference has no such report:
 * b3SparseSolveCG always returns true, src/bounce_softbody/sparse/sparse_solver.cpp:108). */
typedef enum b3g_solve_status
{
	B3G_SOLVE_CONVERGED = 0,      /* delta <= tol^2 * delta0 */
	B3G_SOLVE_MAX_ITERATIONS = 1, /* stopped at the iteration cap (the reference's usual exit) */
	B3G_SOLVE_NONFINITE = 2,      /* a reduction produced NaN or Inf; state left unchanged */
	B3G_SOLVE_BREAKDOWN = 3,      /* d.Ad <= 0: the filtered system is not positive definite */
	B3G_SOLVE_DEVICE_TIMEOUT = 4  /* a bounded device wait expired; the step's results are not valid */
} b3g_solve_status;

/* b3ParticleType (include/bounce_softbody/dynamics/particle.h:31-36). */
enum { B3G_STATIC = 0, B3G_KINEMATIC = 1, B3G_DYNAMIC = 2 };

typedef enum b3g_precision
{
	B3G_PRECISION_FP32 = 0,        /* FP32 blocks and vectors, FP64 dot products for alpha/beta */
	B3G_PRECISION_FP64 = 1,        /* everything in FP64 */
	B3G_PRECISION_BF16_BLOCKS = 2  /* BF16 matrix blocks, FP32 accumulation, FP32 outer refinement */
} b3g_precision;

typedef enum b3g_preconditioner
{
	B3G_PRECOND_JACOBI = 0,        /* the reference's scalar Jacobi (sparse_solver.cpp:38-55) */
	B3G_PRECOND_BLOCK_JACOBI = 1   /* inverse of each 3x3 diagonal block */
} b3g_preconditioner;

/* How vertex spheres touching static world shapes are resolved. */
typedef enum b3g_contact_mode
{
	/* the reference's penalty spring and friction impulse
	 * (sphere_shape_contact.cpp:53-189) */
	B3G_CONTACT_PENALTY = 0,
	/* opt-in extension of b3g_body_step and b3g_step_batch (the server and the allocation-free
	 * step refuse it): an overlapping dynamic vertex is constrained along the
	 * contact normal n through the solver's pre-filter (S = I - n n^T, z = (vt - v.n) n in
	 * pA = S A S^T + I - S, pb = S (b - A z), dv = y + z; sparse_force_solver.cpp:170-190), vt the
	 * Baumgarte velocity min(0.2 C, 0.2) / h of the penalty force's depth C; inelastic and
	 * frictionless */
	B3G_CONTACT_FILTER = 1
} b3g_contact_mode;

/* Static world shapes the body's vertex spheres collide with (b3WorldFixture with a b3Shape,
 * include/bounce_softbody/collision/shapes/). All in world space unless noted. */
typedef enum b3g_shape_type
{
	B3G_SHAPE_SPHERE = 0,     /* b3SphereShape: p[0..2] center */
	B3G_SHAPE_CAPSULE = 1,    /* b3CapsuleShape: p[0..2] center1, p[3..5] center2 */
	B3G_SHAPE_BOX = 2,        /* b3BoxShape: p[0..2] extents, transform */
	B3G_SHAPE_TRIANGLE = 3,   /* b3TriangleShape: p[0..8] vertex1..3 (no wing vertices) */
	B3G_SHAPE_MESH = 4,       /* b3MeshShape: mesh, scale, transform */
	B3G_SHAPE_SDF = 5         /* b3SDFShape: voxel grid of signed distances, transform, invert */
} b3g_shape_type;

typedef struct b3g_world_shape
{
	int32_t type;             /* b3g_shape_type */
	float radius;             /* b3Shape::m_radius */
	float friction;           /* b3WorldFixtureDef::friction */
	float p[9];               /* per type, see b3g_shape_type */
	float rotation[4];        /* box, mesh, sdf: b3Transform::rotation quaternion (x, y, z, w) */
	float translation[3];     /* box, mesh, sdf: b3Transform::translation */
	float scale[3];           /* mesh: b3MeshShape::m_scale */
	uint32_t vertex_count;    /* mesh: b3Mesh::vertexCount */
	const float* vertices;    /* mesh: 3 per vertex, mesh frame */
	uint32_t triangle_count;  /* mesh: b3Mesh::triangleCount (at most 1,048,576) */
	const uint32_t* triangles; /* mesh: v1, v2, v3 per triangle (b3Triangle) */
	const uint32_t* wings;    /* mesh: u1, u2, u3 per triangle, the wing vertex of edge v1v2 / v2v3 /
	                             v3v1 or 0xFFFFFFFF (b3Mesh::BuildAdjacency); NULL = all edges open */
	uint32_t grid[3];         /* sdf: voxels along x, y, z (b3VoxelGrid width, height, depth), >= 2 */
	const float* voxels;      /* sdf: grid[0]*grid[1]*grid[2] signed distances, x fastest */
	float grid_lower[3];      /* sdf: the grid's AABB in the shape frame */
	float grid_upper[3];
	int32_t invert;           /* sdf: b3SDFShape::m_invert */
} b3g_world_shape;

/* One body. Arrays are host memory, read once by b3g_body_create. Per-element material arrays
 * hold one value per element. Vertex ids index the arrays of this body. */
typedef struct b3g_body_desc
{
	uint32_t vertex_count;
	const float* positions;        /* 3 per vertex, also the rest state when *_rest is NULL */
	const float* velocities;       /* 3 per vertex, NULL = zero */
	const int32_t* types;          /* B3G_STATIC / B3G_KINEMATIC / B3G_DYNAMIC */
	const float* damping;          /* mass damping per vertex, NULL = zero (b3ParticleDef::damping) */
	const float* masses;           /* NULL = lumped from fixture densities as b3Body::ResetMass does */

	uint32_t tet_count;
	const uint32_t* tets;          /* 4 vertex ids per tetrahedron */
	const float* tet_rest;         /* 12 per tetrahedron, NULL = positions */
	const float* tet_young;        /* b3TetrahedronElementForceDef::youngModulus */
	const float* tet_poisson;      /* ::poissonRatio */
	const float* tet_stiffness_damping; /* ::stiffnessDamping, NULL = zero */
	const float* tet_density;      /* b3TetrahedronFixtureDef::density, NULL = zero */

	uint32_t tri_count;            /* b3TriangleFixtures; with the five material arrays also
	                                  b3TriangleElementForces, all five NULL = mass fixtures only */
	const uint32_t* tris;          /* 3 vertex ids per triangle */
	const float* tri_rest;         /* 9 per triangle, NULL = positions */
	const float* tri_young_x;      /* b3TriangleElementForceDef::youngModulusX */
	const float* tri_young_y;      /* ::youngModulusY */
	const float* tri_shear;        /* ::shearModulus */
	const float* tri_poisson_xy;   /* ::poissonRationXY */
	const float* tri_poisson_yx;   /* ::poissonRationYX */
	const float* tri_stiffness_damping; /* NULL = zero */
	const float* tri_density;      /* b3TriangleFixtureDef::density, NULL = zero */

	uint32_t spring_count;
	const uint32_t* springs;       /* 2 vertex ids per spring */
	const float* spring_rest_length; /* b3SpringForceDef::length */
	const float* spring_stiffness;   /* ::stiffness */
	const float* spring_damping;     /* ::dampingStiffness */

	const float* sphere_radius;    /* per-vertex b3SphereFixture radius, NULL = no contacts */
	const float* sphere_friction;  /* per-vertex friction */
	uint32_t world_sphere_count;   /* static b3SphereShape world fixtures (shorthand, see below) */
	const float* world_spheres;    /* 5 per shape: center x, y, z, radius, friction */

	float gravity[3];              /* b3Body::SetGravity */

	uint32_t world_shape_count;    /* further static world fixtures of any shape; together with the
	                                  world spheres at most 16 fixtures, spheres first */
	const b3g_world_shape* world_shapes;

	/* Baraff-Witkin cloth forces (src/bounce_softbody/dynamics/forces/stretch_force.cpp,
	 * shear_force.cpp) and mouse springs (mouse_force.cpp). uv: u1, v1, u2, v2, u3, v3 per
	 * element as b3StretchForceDef / b3ShearForceDef hold them; NULL = Initialize() from the
	 * elements' positions. */
	uint32_t stretch_count;
	const uint32_t* stretch_tris;    /* 3 vertex ids per element */
	const float* stretch_uv;         /* 6 per element or NULL */
	const float* stretch_params;     /* 6 per element: stiffness_u, damping_stiffness_u, b_u,
	                                    stiffness_v, damping_stiffness_v, b_v */
	uint32_t shear_count;
	const uint32_t* shear_tris;      /* 3 vertex ids per element */
	const float* shear_uv;           /* 6 per element or NULL */
	const float* shear_params;       /* 2 per element: stiffness, dampingStiffness */
	uint32_t mouse_count;
	const uint32_t* mouse_ids;       /* 4 per element: p1 (the dragged particle), p2, p3, p4 */
	const float* mouse_params;       /* 6 per element: w2, w3, w4, stiffness, dampingStiffness, length */
} b3g_body_desc;

/* Solver settings of one step. b3g_solver_config_default() gives the reference's: one Newton
 * iteration, FLT_EPSILON tolerances, true-residual refresh every 50 PCG iterations, scalar
 * Jacobi, FP32. */
typedef struct b3g_solver_config
{
	uint32_t force_iterations;     /* Newton iterations (Step's forceIterations) */
	uint32_t max_pcg_iterations;   /* Step's forceSubIterations */
	double pcg_tolerance;          /* stop when r.M^-1.r <= tol^2 * r0.M^-1.r0 (b3SolveBEInput::subTolerance) */
	double newton_tolerance;       /* b3SolveBEInput::tolerance */
	uint32_t refresh_period;       /* recompute r = b - A x when iteration % period == 0 */
	int32_t precision;             /* b3g_precision */
	int32_t preconditioner;        /* b3g_preconditioner */
	int32_t contact_mode;          /* b3g_contact_mode (B3G_CONTACT_PENALTY, the reference's) */
} b3g_solver_config;

typedef struct b3g_step_stats
{
	uint32_t newton_iterations;    /* b3_forceSolverIterations */
	uint32_t pcg_iterations;       /* max over Newton iterations (b3_forceSolverMaxSubIterations) */
	uint32_t min_pcg_iterations;   /* b3_forceSolverMinSubIterations */
	int32_t solve_status;          /* b3g_solve_status of the last PCG solve */
	double residual_ratio;         /* sqrt(delta / delta0) at exit of the last PCG solve */
	double newton_error;           /* |dv|^2 of the last Newton iteration */
	uint64_t total_pcg_iterations; /* PCG iterations of every step since the body was created */
	uint64_t total_steps;          /* steps with dt > 0 since the body was created */
} b3g_step_stats;

B3G_API void b3g_solver_config_default(b3g_solver_config* config);
B3G_API const char* b3g_last_error(void);
B3G_API const char* b3g_version(void);

/* A context owns one CUDA stream on one device; bodies belong to one context. */
B3G_API int b3g_context_create(int device, b3g_context** out);
B3G_API int b3g_context_destroy(b3g_context* ctx);
/* The CUDA stream (cudaStream_t) every call of this context is ordered on. */
B3G_API int b3g_context_stream(b3g_context* ctx, void** stream);
B3G_API int b3g_context_synchronize(b3g_context* ctx);

B3G_API int b3g_body_create(b3g_context* ctx, const b3g_body_desc* desc, b3g_body** out);
B3G_API int b3g_body_destroy(b3g_body* body);
/* Sizes: vertex count, tetrahedra, triangles, springs, nonzero 3x3 blocks of A, padded slots. */
B3G_API int b3g_body_info(const b3g_body* body, uint64_t info[6]);
/* Device bytes held by the body (state, matrix, element data, solver vectors). */
B3G_API int b3g_body_device_bytes(const b3g_body* body, uint64_t* bytes);

/* One b3Body::Step on the GPU. Asynchronous on the context stream unless stats is non-NULL,
 * in which case the call waits and fills stats. dt <= 0 skips the solve like the reference. */
B3G_API int b3g_body_step(b3g_body* body, float dt, const b3g_solver_config* config, b3g_step_stats* stats);

/* `steps` steps of `count` independent bodies of one context in one persistent launch per
 * size bucket (captured once in a CUDA graph and replayed). stats, if non-NULL, receives the
 * last step's statistics of each body (count entries) and makes the call wait. */
B3G_API int b3g_step_batch(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float dt,
                   const b3g_solver_config* config, uint32_t steps, b3g_step_stats* stats);

/* Like b3g_step_batch, without allocating anything. No counterpart in the reference.
 * For callers that cannot call cudaMalloc while they step: engines that forbid device allocation
 * after load or run under a fixed device-memory budget, and real-time loops that cannot afford the
 * device-wide synchronisation cudaMalloc / cudaFree bring. b3g_step_batch allocates per-batch
 * tables on first use; this entry point keeps them in a fixed device array of the library instead
 * (held by every GPU that loads the library until exit), for at most 512 bodies per call (more
 * fails with B3G_ERROR_UNSUPPORTED). Differences from b3g_step_batch: each body must already have
 * solver buffers for the requested precision (FP32 always does; FP64 / BF16 after a first step in
 * that precision), where b3g_step_batch creates them; dt must be > 0 (b3g_step_batch steps each
 * body alone for dt <= 0); the schedule is a fixed size rule (clusters of 4 CTAs of 256 threads
 * for bodies of 4096 vertices or more, single CTAs below), not autotuned. The first call on a device looks the
 * array up and clears it (set-up): make that first call before any stream capture. Each call
 * copies the body descriptors to the device from static host arrays of the library, which the
 * next call rewrites. Every call reuses the same device array, so calls whose work overlaps on the
 * GPU (other streams, other contexts on the same device) race; calls on one stream are ordered. */
B3G_API int b3g_step_batch_noalloc(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float dt,
                                   const b3g_solver_config* config, uint32_t steps, b3g_step_stats* stats);

/* Schedule of the context's current batch: cluster size, size threshold of cluster-stepped bodies
 * (-1 = none), bodies stepped by clusters, CTAs per launch, autotuned (0/1), number of timed
 * candidates, queue order (0: largest first, 1: longest estimated solve first), then per
 * candidate (code = order * 1e8 + cluster * 1e6 + threshold, microseconds). */
B3G_API int b3g_batch_schedule(b3g_context* ctx, int32_t* out, uint32_t capacity);

/* Split assembly of the context's current batch (single Newton iteration, tetrahedra-only
 * bodies): the flat element and row-slice offsets where the second body group starts (0 = no
 * split), the CTAs per SM of that group's element launch, which runs on a second stream beside
 * the first group's row launch, and of that row launch. */
B3G_API int b3g_batch_assembly_split(b3g_context* ctx, uint32_t out[4]);

/* Cycles spent per phase of the batch kernel, summed over CTAs (elements, assembly, SpMV, update,
 * direction, final update, -, -). Only counted when the environment variable B3G_PHASE_PROFILE=1
 * is set when the batch is first stepped; zeros otherwise. reset != 0 clears the counters. */
B3G_API int b3g_batch_phase_cycles(b3g_context* ctx, uint64_t out[8], int reset);

/* Launch timing of batched steps (measurement aid, no reference counterpart). While on, a
 * single-Newton b3g_step_batch launches its two kernels (elements + assembly, then PCG + final
 * update) directly instead of replaying its graph, records CUDA events around each and waits
 * for them; b3g_batch_launch_times returns the accumulated device milliseconds of the assembly
 * launches and of the PCG launches and the number of timed steps (out[0..2]). */
B3G_API int b3g_batch_set_launch_timing(b3g_context* ctx, int on);
B3G_API int b3g_batch_launch_times(b3g_context* ctx, double out[3], int reset);
/* The element launch's share of the assembly milliseconds above (the rest is the row assembly),
 * accumulated and reset with them. */
B3G_API int b3g_batch_element_launch_ms(b3g_context* ctx, double* out);

/* Host-buffer transfers for a list of bodies of one context; the host arrays are the bodies'
 * arrays concatenated in list order (3 floats per vertex). Pinned host memory makes them
 * asynchronous copies; get waits for the copies. apply_forces from pinned memory copies on an
 * upload stream of the context into one of two device buffers taken in turn, so the copy
 * overlaps the step queued before it; the host array must stay unchanged until the step queued
 * after the call has completed (or b3g_context_synchronize). */
B3G_API int b3g_batch_apply_forces(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, const float* forces);
B3G_API int b3g_batch_get_state(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float* positions,
                                float* velocities);

/* ---------------------------------------------------------------- several GPUs
 * Bodies never interact (b3Body::Step, src/bounce_softbody/dynamics/body.cpp:552-604, touches one
 * body), so a body list spreads over GPUs with no exchange between them: one context per GPU,
 * each stepping its share. No reference counterpart (the reference is single-threaded). Neither
 * call needs a GPU. */
/* Device bytes a body made from desc would take, estimated from its counts (slightly high by
 * design; b3g_body_device_bytes gives the exact figure once the body exists). */
B3G_API int b3g_body_desc_estimate_bytes(const b3g_body_desc* desc, uint64_t* bytes);
/* Split `count` bodies of the given device bytes over `ranks` GPUs: largest first, each to the
 * GPU with the fewest bytes so far (ties: lowest rank). rank_of[k] receives body k's GPU. The
 * split is deterministic, so every rank computes the same one. */
B3G_API int b3g_partition_bodies(const uint64_t* bytes, uint32_t count, uint32_t ranks, uint32_t* rank_of);

/* b3g_batch_get_state without waiting (no reference counterpart): one launch snapshots every
 * body's x and v on the device, and a second stream of the context copies the snapshot to the
 * host arrays, so that the copy overlaps the work queued next (the next step). The arrays are
 * filled once b3g_batch_wait_state (or b3g_context_synchronize) returns; they must stay valid
 * and untouched until then. Page-locked arrays (cudaHostAlloc / cudaHostRegister) make the copy
 * asynchronous; with pageable ones the call waits for it. A later call on the context reuses
 * the snapshot only after the previous copy has left it. */
B3G_API int b3g_batch_get_state_async(b3g_context* ctx, b3g_body* const* bodies, uint32_t count, float* positions,
                                      float* velocities);
B3G_API int b3g_batch_wait_state(b3g_context* ctx);

/* Host <-> device state transfer (3 floats per vertex each; either pointer may be NULL). */
B3G_API int b3g_body_get_state(b3g_body* body, float* positions, float* velocities);
B3G_API int b3g_body_set_state(b3g_body* body, const float* positions, const float* velocities);
/* Accumulate external forces / translations for the next step; both are cleared by the step
 * like b3Body::Step clears b3Particle::m_force and m_translation (body.cpp:577-581). */
B3G_API int b3g_body_apply_forces(b3g_body* body, const float* forces);
B3G_API int b3g_body_apply_translations(b3g_body* body, const float* translations);
/* b3Particle::SetType for every vertex whose type changes (masses are re-lumped). */
B3G_API int b3g_body_set_types(b3g_body* body, const int32_t* types);
/* Element rotations as quaternions (x, y, z, w), 4 floats per tetrahedron. */
B3G_API int b3g_body_get_rotations(b3g_body* body, float* quaternions);
B3G_API int b3g_body_set_rotations(b3g_body* body, const float* quaternions);
/* Contact state between steps, for checkpoint / resume: the b3SphereAndShapeContact of each vertex
 * sphere and world fixture (m_manifold's normal, m_normalForce, m_applyFriction and whether the
 * contact exists; include/bounce_softbody/dynamics/contacts/sphere_shape_contact.h:50-52, created by
 * b3ContactManager::FindNewContacts, src/bounce_softbody/dynamics/contacts/contact_manager.cpp:65-82).
 * Arrays are vertex-major: entry v * fixtures + k for vertex v and fixture k (world spheres first,
 * then world shapes); normals hold 3 floats per entry. fixtures is 0 for a body without vertex
 * spheres. Any array may be NULL (not transferred). set_contacts takes flags of 0 or 1. */
B3G_API int b3g_body_contact_fixtures(const b3g_body* body, uint32_t* fixtures);
B3G_API int b3g_body_get_contacts(b3g_body* body, uint8_t* exists, uint8_t* apply_friction, float* normal_force,
                                  float* normals);
B3G_API int b3g_body_set_contacts(b3g_body* body, const uint8_t* exists, const uint8_t* apply_friction,
                                  const float* normal_force, const float* normals);
/* Lumped vertex masses as b3Body::ResetMass computed them (1 float per vertex). */
B3G_API int b3g_body_get_masses(b3g_body* body, float* masses);
/* Statistics of the body's last step (waits for it). */
B3G_API int b3g_body_get_stats(b3g_body* body, b3g_step_stats* stats);

/* One segment's closest hit on the body's triangle fixtures (b3BodyRayCastSingleOutput,
 * include/bounce_softbody/dynamics/body.h:52-57): the triangle is its index in desc.tris. */
typedef struct b3g_ray_hit
{
	int32_t hit;          /* 1 if the segment hits a triangle */
	uint32_t triangle;    /* index into b3g_body_desc::tris */
	float fraction;       /* p1 + fraction (p2 - p1) is the hit point, in [0, 1] */
	float normal[3];      /* the triangle's unit normal, facing p1 */
} b3g_ray_hit;

/* b3Body::RayCastSingle (src/bounce_softbody/dynamics/body.cpp:468-521) for `count` segments
 * (6 floats each: p1, p2) against every triangle fixture at the body's current positions, with
 * b3TriangleShape::RayCast (src/bounce_softbody/collision/shapes/triangle_shape.cpp:314-387); the
 * smallest fraction wins, ties go to the lowest triangle index. Synchronous: hits are in host
 * memory on return. */
B3G_API int b3g_body_ray_cast(b3g_body* body, const float* segments, uint32_t count, b3g_ray_hit* hits);

/* ---------------------------------------------------------------- serving
 * A server steps many bodies on request, continuously batched: a worker thread repeatedly admits
 * waiting requests, steps every body with an active request once in one batched launch (the
 * kernel of b3g_step_batch) and retires finished requests; requests that arrive meanwhile join at
 * the next launch. Bodies stay resident on the device between requests while their device
 * footprint fits `memory_budget_bytes`; beyond it idle bodies are evicted least recently used
 * first (their state is kept on the host and restored exactly when they return) and requests wait
 * for room. A body serves its requests one at a time in arrival order. Team sizes depend only on
 * each body's own size, so a body's results do not depend on the mix it is stepped in.
 * No reference counterpart: the reference steps one body per b3Body::Step call
 * (src/bounce_softbody/dynamics/body.cpp:552); this is the request loop a service would put around it. */
typedef struct b3g_server b3g_server;

typedef enum b3g_request_status
{
	B3G_REQUEST_DONE = 0,
	B3G_REQUEST_REJECTED = 1,          /* the body alone exceeds the memory budget */
	B3G_REQUEST_DEVICE_TIMEOUT = 2     /* a bounded device wait expired during one of its steps */
} b3g_request_status;

typedef struct b3g_request_result
{
	uint64_t request_id;
	uint32_t body_id;
	uint32_t steps;
	int32_t status;                /* b3g_request_status */
	int32_t reserved;
	uint64_t pcg_iterations;       /* PCG iterations of the request's steps */
	double queue_seconds;          /* arrival to first step */
	double latency_seconds;        /* arrival to completion */
} b3g_request_result;

typedef struct b3g_server_stats
{
	uint64_t iterations;           /* batched launches */
	uint64_t vertex_steps;         /* vertices x steps completed */
	uint64_t admitted, completed, rejected, evictions;
	uint64_t resident_bytes;       /* device bytes of the resident bodies */
	uint64_t waiting;              /* requests not yet started */
	double gpu_seconds;            /* summed device time of the launches */
	double wall_seconds;           /* first arrival to last completed launch */
	double step_ms_p50, step_ms_p99; /* device time per launch */
	uint32_t cluster_ctas;         /* CTAs of the team of a large body */
	uint32_t cluster_threshold;    /* vertices from which a body is large */
} b3g_server_stats;

/* config NULL = b3g_solver_config_default; max_active bounds the bodies of one launch. */
B3G_API int b3g_server_create(b3g_context* ctx, uint64_t memory_budget_bytes, uint32_t max_active, float dt,
                              const b3g_solver_config* config, b3g_server** out);
/* Register a body (its arrays are copied; nothing is allocated on the device yet). */
B3G_API int b3g_server_add_body(b3g_server* server, const b3g_body_desc* desc, uint32_t* body_id);
/* Start the worker thread. Requests submitted before it starts wait. */
B3G_API int b3g_server_start(b3g_server* server);
/* Queue `steps` steps of a body; thread-safe. */
B3G_API int b3g_server_submit(b3g_server* server, uint32_t body_id, uint32_t steps, uint64_t* request_id);
/* Take up to `capacity` finished requests in completion order. */
B3G_API int b3g_server_poll(b3g_server* server, b3g_request_result* out, uint32_t capacity, uint32_t* count);
/* Requests submitted and not yet finished. */
B3G_API int b3g_server_pending(b3g_server* server, uint32_t* pending);
B3G_API int b3g_server_get_stats(b3g_server* server, b3g_server_stats* stats);
/* Restart the statistics (counters, launch times, the wall clock from the next arrival). */
B3G_API int b3g_server_reset_stats(b3g_server* server);
/* State of a body that has no active request (3 floats per vertex each; either may be NULL). */
B3G_API int b3g_server_get_state(b3g_server* server, uint32_t body_id, float* positions, float* velocities);
/* Stop the worker after its current launch and free every body of the server. */
B3G_API int b3g_server_destroy(b3g_server* server);

#ifdef __cplusplus
}
#endif

#endif /* B3G_H */
