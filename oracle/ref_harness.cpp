// Test infrastructure only: a harness around the reference library compiled from its own
// sources (see oracle/Makefile). Nothing in the product links or loads this file.
//
// It builds a b3Body from flat arrays in O(n) and steps it exactly like b3Body::Step
// (src/bounce_softbody/dynamics/body.cpp:552-604), except that the PCG tolerance can be set:
// b3ForceSolver::Solve (src/bounce_softbody/dynamics/force_solver.cpp:88-180) never sets
// b3SolveBEInput::subTolerance, so b3Body::Step always runs with FLT_EPSILON. The harness
// therefore re-does the pack/unpack of force_solver.cpp:100-179 itself and calls the
// reference's own b3SparseSolveBE (src/bounce_softbody/sparse/sparse_force_solver.cpp:104)
// with the tolerance it is given. With use_body_step=1 it calls b3Body::Step unchanged.
//
// Compiled with -Dprivate=public -Dprotected=public so that fixtures can be linked into the
// body lists without the O(n^2) duplicate scans of b3Body::CreateTetrahedron/CreateTriangle
// (body.cpp:209-219, 278-289); b3Body::ResetMass (body.cpp:394-466) then runs once.

#include <bounce_softbody/bounce_softbody.h>
#include <bounce_softbody/dynamics/body_solver.h>
#include <bounce_softbody/dynamics/force_solver.h>
#include <bounce_softbody/dynamics/time_step.h>
#include <bounce_softbody/dynamics/contacts/sphere_shape_contact.h>
#include <bounce_softbody/sparse/sparse_force_solver.h>
#include <bounce_softbody/sparse/dense_vec3.h>
#include <bounce_softbody/sparse/diag_mat33.h>
#include <bounce_softbody/sparse/sparse_mat33.h>
#include <bounce_softbody/collision/shapes/sphere_shape.h>
#include <bounce_softbody/collision/shapes/capsule_shape.h>
#include <bounce_softbody/collision/shapes/box_shape.h>
#include <bounce_softbody/collision/shapes/triangle_shape.h>
#include <bounce_softbody/collision/shapes/mesh_shape.h>
#include <bounce_softbody/collision/shapes/sdf_shape.h>
#include <bounce_softbody/collision/geometry/mesh.h>
#include <bounce_softbody/collision/geometry/sdf.h>

#include <algorithm>
#include <chrono>
#include <new>
#include <vector>
#include <stdint.h>
#include <string.h>

extern "C" {

// A static world fixture's shape; p per type: sphere center; capsule center1, center2; box half
// extents; triangle vertex1..3 (mirror of b3o_shape in b3_oracle.c).
struct RefShape
{
	int32_t type;  // 0 sphere, 1 capsule, 2 box, 3 triangle, 4 mesh, 5 sdf
	double radius, friction;
	double p[9];
	double rotation[4], translation[3], scale[3];
	uint32_t vertex_count;
	const double* vertices;
	uint32_t triangle_count;
	const uint32_t* triangles;
	const uint32_t* wings;  // null = all edges open
	uint32_t grid[3];
	const double* voxels;
	double grid_lower[3], grid_upper[3];
	int32_t invert;
};

// Flat description of one body. Arrays are double on this boundary whatever `scalar` is.
struct RefDesc
{
	uint32_t n;
	const double* x;        // 3n initial positions
	const double* v;        // 3n initial velocities
	const int32_t* type;    // n, b3ParticleType values (0 static, 1 kinematic, 2 dynamic)
	const double* damping;  // n mass damping

	uint32_t tet_count;
	const uint32_t* tets;       // 4 per tet
	const double* tet_rest;     // 12 per tet (rest vertices); null = initial positions
	const double* tet_E;
	const double* tet_nu;
	const double* tet_kdamp;
	const double* tet_density;

	uint32_t tri_count;
	const uint32_t* tris;       // 3 per triangle
	const double* tri_rest;     // 9 per triangle; null = initial positions
	const double* tri_Ex;
	const double* tri_Ey;
	const double* tri_Es;
	const double* tri_nuxy;
	const double* tri_nuyx;
	const double* tri_kdamp;
	const double* tri_density;

	uint32_t spring_count;
	const uint32_t* springs;    // 2 per spring
	const double* spring_L0;
	const double* spring_ks;
	const double* spring_kd;

	const double* sphere_radius;   // n, null = no sphere fixtures
	const double* sphere_friction; // n

	uint32_t world_sphere_count;
	const double* world_spheres;   // 5 per shape: cx, cy, cz, radius, friction

	double gravity[3];

	uint32_t world_shape_count;
	const RefShape* world_shapes;

	// cloth forces (b3StretchForceDef, b3ShearForceDef, b3MouseForceDef); uv null = the defs'
	// Initialize from the initial positions
	uint32_t stretch_count;
	const uint32_t* stretch_tris;   // 3 per force
	const double* stretch_uv;       // 6 per force: u1, v1, u2, v2, u3, v3
	const double* stretch_params;   // 6 per force: ks_u, kd_u, b_u, ks_v, kd_v, b_v
	uint32_t shear_count;
	const uint32_t* shear_tris;
	const double* shear_uv;
	const double* shear_params;     // 2 per force: stiffness, dampingStiffness
	uint32_t mouse_count;
	const uint32_t* mouse_ids;      // 4 per force: p1..p4
	const double* mouse_params;     // 6 per force: w2, w3, w4, stiffness, dampingStiffness, length
};

struct RefRun
{
	uint32_t steps;
	double dt;
	uint32_t newton_iters;
	uint32_t max_sub;
	double sub_tol;
	int32_t use_body_step;

	double* x_out;              // 3n
	double* v_out;              // 3n
	uint32_t* sub_iters_out;    // steps (max PCG iterations of each step), may be null
	double* seconds_out;        // wall time of the stepping loop
	int32_t contact_mode;       // unused: the reference has penalty contacts only
};

} // extern "C"

// Defined in src/bounce_softbody/dynamics/force_solver.cpp:29-34 without a header declaration.
extern uint32 b3_forceSolverIterations;
extern uint32 b3_forceSolverMinSubIterations;
extern uint32 b3_forceSolverMaxSubIterations;

namespace {

struct HarnessModel : public b3SparseForceModel
{
	void ApplyForces(const b3SparseForceSolverData* data) override
	{
		for (uint32 i = 0; i < particleCount; ++i) particles[i]->ApplyForces(data);
		for (uint32 i = 0; i < forceCount; ++i) forces[i]->ApplyForces(data);
		for (uint32 i = 0; i < contactCount; ++i) contacts[i]->ApplyForces(data);
	}

	uint32 particleCount = 0;
	b3Particle** particles = nullptr;
	uint32 forceCount = 0;
	b3Force** forces = nullptr;
	uint32 contactCount = 0;
	b3SphereAndShapeContact** contacts = nullptr;
};

// One step of the body with an explicit PCG tolerance; the order of operations is the one of
// b3Body::Step / b3Body::Solve / b3BodySolver::Solve / b3ForceSolver::Solve.
uint32 HarnessStep(b3Body* body, scalar dt, uint32 newtonIters, uint32 maxSub, scalar subTol)
{
	body->m_contactManager.UpdateContacts();
	for (b3Force* f = body->m_forceList; f; f = f->m_next) f->ClearForces();

	uint32 subIters = 0;
	if (dt > scalar(0))
	{
		std::vector<b3Particle*> particles;
		std::vector<b3Force*> forces;
		std::vector<b3SphereAndShapeContact*> contacts;
		for (b3Particle* p = body->m_particleList; p; p = p->m_next)
		{
			p->m_solverId = (uint32)particles.size();
			particles.push_back(p);
		}
		for (b3Force* f = body->m_forceList; f; f = f->m_next) forces.push_back(f);
		for (b3SphereAndShapeContact* c = body->m_contactManager.m_contactList; c; c = c->m_next) contacts.push_back(c);

		uint32 n = (uint32)particles.size();
		b3DenseVec3 x0(n), v0(n), fe(n), y(n), x(n), v(n), z(n);
		b3DiagMat33 M(n), S(n);
		b3Vec3 g = body->m_gravity;
		for (uint32 i = 0; i < n; ++i)
		{
			b3Particle* p = particles[i];
			x0[i] = p->m_position;
			v0[i] = p->m_velocity;
			fe[i] = p->m_force;
			y[i] = p->m_translation;
			z[i].SetZero();
			if (p->m_type == e_dynamicParticle)
			{
				M[i] = b3Mat33Diagonal(p->m_mass);
				fe[i] += p->m_mass * g;
				S[i].SetIdentity();
			}
			else
			{
				M[i] = b3Mat33Diagonal(scalar(1));
				S[i].SetZero();
			}
		}

		HarnessModel model;
		model.particleCount = n;
		model.particles = particles.data();
		model.forceCount = (uint32)forces.size();
		model.forces = forces.data();
		model.contactCount = (uint32)contacts.size();
		model.contacts = contacts.data();

		b3SolveBEInput in;
		in.forceModel = &model;
		in.h = dt;
		in.inv_h = scalar(1) / dt;
		in.dofCount = n;
		in.x0 = &x0;
		in.v0 = &v0;
		in.fe = &fe;
		in.M = &M;
		in.y = &y;
		in.S = &S;
		in.z = &z;
		in.maxIterations = newtonIters;
		in.maxSubIterations = maxSub;
		in.subTolerance = subTol;

		b3SolveBEOutput out;
		out.x = &x;
		out.v = &v;
		out.minSubIterations = B3_MAX_U32;
		out.maxSubIterations = 0;
		b3SparseSolveBE(&out, &in);
		subIters = out.maxSubIterations;

		for (uint32 i = 0; i < n; ++i)
		{
			particles[i]->m_position = x[i];
			particles[i]->m_velocity = v[i];
		}

		b3TimeStep step;
		step.dt = dt;
		step.inv_dt = scalar(1) / dt;
		step.forceIterations = newtonIters;
		step.forceSubIterations = maxSub;
		for (b3SphereAndShapeContact* c : contacts) c->ApplyFriction(step, g);
	}

	for (b3Particle* p = body->m_particleList; p; p = p->m_next)
	{
		p->m_force.SetZero();
		p->m_translation.SetZero();
	}

	for (b3TriangleFixture* t = body->m_triangleList; t; t = t->m_next)
	{
		b3Vec3 vc = (t->m_p1->m_velocity + t->m_p2->m_velocity + t->m_p3->m_velocity) / scalar(3);
		t->Synchronize(dt * vc);
	}

	body->m_contactManager.FindNewContacts();
	return subIters;
}

inline b3Vec3 V3(const double* p) { return b3Vec3(scalar(p[0]), scalar(p[1]), scalar(p[2])); }

// Owns the shapes a body's world fixtures were cloned from and the meshes and SDFs the clones
// point to.
struct ShapeStore
{
	std::vector<b3Shape*> shapes;
	std::vector<b3Mesh*> meshes;
	std::vector<b3SDF*> sdfs;
	~ShapeStore()
	{
	
		for (b3Mesh* m : meshes)
		{
			delete[] m->vertices;
			delete[] m->triangles;
			delete m;
		}
		for (b3SDF* f : sdfs) delete f;
	}
};

static b3Transform Xf(const RefShape& w)
{
	b3Transform xf;
	xf.translation = V3(w.translation);
	xf.rotation = b3Quat(b3Vec3(scalar(w.rotation[0]), scalar(w.rotation[1]), scalar(w.rotation[2])), scalar(w.rotation[3]));
	return xf;
}

// The reference's own shape objects for one world shape description.
static b3Shape* MakeShape(const RefShape& w, ShapeStore& store)
{
	b3Shape* out = nullptr;
	switch (w.type)
	{
	case 0:
	{
		b3SphereShape* sh = new b3SphereShape();
		sh->m_center = V3(w.p);
		out = sh;
		break;
	}
	case 1:
	{
		b3CapsuleShape* sh = new b3CapsuleShape();
		sh->m_center1 = V3(w.p);
		sh->m_center2 = V3(w.p + 3);
		out = sh;
		break;
	}
	case 2:
	{
		b3BoxShape* sh = new b3BoxShape();
		sh->m_extents = V3(w.p);
		sh->m_xf = Xf(w);
		out = sh;
		break;
	}
	case 3:
	{
		b3TriangleShape* sh = new b3TriangleShape();
		sh->Set(V3(w.p), V3(w.p + 3), V3(w.p + 6));
		out = sh;
		break;
	}
	case 4:
	{
		b3Mesh* m = new b3Mesh();
		m->vertexCount = w.vertex_count;
		m->vertices = new b3Vec3[w.vertex_count];
		for (uint32_t v = 0; v < w.vertex_count; ++v) m->vertices[v] = V3(w.vertices + 3 * v);
		m->triangleCount = w.triangle_count;
		m->triangles = new b3Triangle[w.triangle_count];
		for (uint32_t t = 0; t < w.triangle_count; ++t)
		{
			b3Triangle& T = m->triangles[t];
			T.v1 = w.triangles[3 * t];
			T.v2 = w.triangles[3 * t + 1];
			T.v3 = w.triangles[3 * t + 2];
			T.u1 = w.wings ? w.wings[3 * t] : B3_NULL_VERTEX;
			T.u2 = w.wings ? w.wings[3 * t + 1] : B3_NULL_VERTEX;
			T.u3 = w.wings ? w.wings[3 * t + 2] : B3_NULL_VERTEX;
		}
		m->BuildTree();
		store.meshes.push_back(m);
		b3MeshShape* sh = new b3MeshShape();
		sh->m_mesh = m;
		sh->m_scale = V3(w.scale);
		sh->m_xf = Xf(w);
		out = sh;
		break;
	}
	case 5:
	{
		b3SDF* f = new b3SDF();
		f->mesh = nullptr;
		b3AABB aabb;
		aabb.lowerBound = V3(w.grid_lower);
		aabb.upperBound = V3(w.grid_upper);
		f->voxelGrid.Create(aabb, w.grid[0], w.grid[1], w.grid[2]);
		const uint32_t nv = w.grid[0] * w.grid[1] * w.grid[2];
		for (uint32_t k = 0; k < nv; ++k) f->voxelGrid.SetVoxel(k, scalar(w.voxels[k]));
		store.sdfs.push_back(f);
		b3SDFShape* sh = new b3SDFShape();
		sh->m_sdf = f;
		sh->m_xf = Xf(w);
		sh->m_invert = w.invert != 0;
		out = sh;
		break;
	}
	default: return nullptr;
	}
	out->m_radius = scalar(w.radius);
	store.shapes.push_back(out);
	return out;
}

b3Body* BuildBody(const RefDesc* d, std::vector<b3Particle*>& ps, ShapeStore& store,
                  std::vector<b3TriangleFixture*>* tris_out = nullptr)
{
	// b3Body embeds a 1 MiB stack allocator: keep it on the heap.
	b3Body* body = new b3Body();
	body->SetGravity(V3(d->gravity));

	ps.resize(d->n);
	for (uint32_t i = 0; i < d->n; ++i)
	{
		b3ParticleDef pd;
		pd.type = (b3ParticleType)d->type[i];
		pd.position = V3(d->x + 3 * i);
		pd.velocity = V3(d->v + 3 * i);
		pd.damping = d->damping ? scalar(d->damping[i]) : scalar(0);
		ps[i] = body->CreateParticle(pd);
	}

	for (uint32_t e = 0; e < d->tet_count; ++e)
	{
		const uint32_t* t = d->tets + 4 * e;
		b3Vec3 r[4];
		for (int k = 0; k < 4; ++k)
			r[k] = d->tet_rest ? V3(d->tet_rest + 12 * e + 3 * k) : V3(d->x + 3 * t[k]);

		b3TetrahedronFixtureDef fd;
		fd.p1 = ps[t[0]]; fd.p2 = ps[t[1]]; fd.p3 = ps[t[2]]; fd.p4 = ps[t[3]];
		fd.v1 = r[0]; fd.v2 = r[1]; fd.v3 = r[2]; fd.v4 = r[3];
		fd.density = scalar(d->tet_density[e]);
		void* mem = body->m_blockAllocator.Allocate(sizeof(b3TetrahedronFixture));
		b3TetrahedronFixture* f = new (mem) b3TetrahedronFixture(fd, body);
		f->m_prev = nullptr;
		f->m_next = body->m_tetrahedronList;
		if (body->m_tetrahedronList) body->m_tetrahedronList->m_prev = f;
		body->m_tetrahedronList = f;
		++body->m_tetrahedronCount;

		b3TetrahedronElementForceDef ed;
		ed.p1 = ps[t[0]]; ed.p2 = ps[t[1]]; ed.p3 = ps[t[2]]; ed.p4 = ps[t[3]];
		ed.v1 = r[0]; ed.v2 = r[1]; ed.v3 = r[2]; ed.v4 = r[3];
		ed.youngModulus = scalar(d->tet_E[e]);
		ed.poissonRatio = scalar(d->tet_nu[e]);
		ed.stiffnessDamping = d->tet_kdamp ? scalar(d->tet_kdamp[e]) : scalar(0);
		body->CreateForce(ed);
	}

	for (uint32_t e = 0; e < d->tri_count; ++e)
	{
		const uint32_t* t = d->tris + 3 * e;
		b3Vec3 r[3];
		for (int k = 0; k < 3; ++k)
			r[k] = d->tri_rest ? V3(d->tri_rest + 9 * e + 3 * k) : V3(d->x + 3 * t[k]);

		b3TriangleFixtureDef fd;
		fd.p1 = ps[t[0]]; fd.p2 = ps[t[1]]; fd.p3 = ps[t[2]];
		fd.v1 = r[0]; fd.v2 = r[1]; fd.v3 = r[2];
		fd.density = scalar(d->tri_density[e]);
		void* mem = body->m_blockAllocator.Allocate(sizeof(b3TriangleFixture));
		b3TriangleFixture* f = new (mem) b3TriangleFixture(fd, body);
		f->m_proxyId = body->m_tree.CreateProxy(f->ComputeAABB(), f);
		f->m_prev = nullptr;
		f->m_next = body->m_triangleList;
		if (body->m_triangleList) body->m_triangleList->m_prev = f;
		body->m_triangleList = f;
		++body->m_triangleCount;
		if (tris_out) tris_out->push_back(f);

		if (!d->tri_Ex) continue;  // a mass fixture without an element force
		b3TriangleElementForceDef ed;
		ed.p1 = ps[t[0]]; ed.p2 = ps[t[1]]; ed.p3 = ps[t[2]];
		ed.v1 = r[0]; ed.v2 = r[1]; ed.v3 = r[2];
		ed.youngModulusX = scalar(d->tri_Ex[e]);
		ed.youngModulusY = scalar(d->tri_Ey[e]);
		ed.shearModulus = scalar(d->tri_Es[e]);
		ed.poissonRationXY = scalar(d->tri_nuxy[e]);
		ed.poissonRationYX = scalar(d->tri_nuyx[e]);
		ed.stiffnessDamping = d->tri_kdamp ? scalar(d->tri_kdamp[e]) : scalar(0);
		body->CreateForce(ed);
	}

	for (uint32_t e = 0; e < d->spring_count; ++e)
	{
		b3SpringForceDef sd;
		sd.p1 = ps[d->springs[2 * e + 0]];
		sd.p2 = ps[d->springs[2 * e + 1]];
		sd.length = scalar(d->spring_L0[e]);
		sd.stiffness = scalar(d->spring_ks[e]);
		sd.dampingStiffness = scalar(d->spring_kd[e]);
		body->CreateForce(sd);
	}

	for (uint32_t e = 0; e < d->stretch_count; ++e)
	{
		const uint32_t* t = d->stretch_tris + 3 * e;
		const double* c = d->stretch_params + 6 * e;
		b3StretchForceDef fd;
		if (d->stretch_uv)
		{
			const double* uv = d->stretch_uv + 6 * e;
			fd.u1 = scalar(uv[0]); fd.v1 = scalar(uv[1]);
			fd.u2 = scalar(uv[2]); fd.v2 = scalar(uv[3]);
			fd.u3 = scalar(uv[4]); fd.v3 = scalar(uv[5]);
		}
		else
			fd.Initialize(V3(d->x + 3 * t[0]), V3(d->x + 3 * t[1]), V3(d->x + 3 * t[2]));
		fd.p1 = ps[t[0]]; fd.p2 = ps[t[1]]; fd.p3 = ps[t[2]];
		fd.stiffness_u = scalar(c[0]);
		fd.damping_stiffness_u = scalar(c[1]);
		fd.b_u = scalar(c[2]);
		fd.stiffness_v = scalar(c[3]);
		fd.damping_stiffness_v = scalar(c[4]);
		fd.b_v = scalar(c[5]);
		body->CreateForce(fd);
	}

	for (uint32_t e = 0; e < d->shear_count; ++e)
	{
		const uint32_t* t = d->shear_tris + 3 * e;
		b3ShearForceDef fd;
		if (d->shear_uv)
		{
			const double* uv = d->shear_uv + 6 * e;
			fd.u1 = scalar(uv[0]); fd.v1 = scalar(uv[1]);
			fd.u2 = scalar(uv[2]); fd.v2 = scalar(uv[3]);
			fd.u3 = scalar(uv[4]); fd.v3 = scalar(uv[5]);
		}
		else
			fd.Initialize(V3(d->x + 3 * t[0]), V3(d->x + 3 * t[1]), V3(d->x + 3 * t[2]));
		fd.p1 = ps[t[0]]; fd.p2 = ps[t[1]]; fd.p3 = ps[t[2]];
		fd.stiffness = scalar(d->shear_params[2 * e]);
		fd.dampingStiffness = scalar(d->shear_params[2 * e + 1]);
		body->CreateForce(fd);
	}

	for (uint32_t e = 0; e < d->mouse_count; ++e)
	{
		const uint32_t* t = d->mouse_ids + 4 * e;
		const double* c = d->mouse_params + 6 * e;
		b3MouseForceDef fd;
		fd.p1 = ps[t[0]]; fd.p2 = ps[t[1]]; fd.p3 = ps[t[2]]; fd.p4 = ps[t[3]];
		fd.w2 = scalar(c[0]);
		fd.w3 = scalar(c[1]);
		fd.w4 = scalar(c[2]);
		fd.stiffness = scalar(c[3]);
		fd.dampingStiffness = scalar(c[4]);
		fd.length = scalar(c[5]);
		body->CreateForce(fd);
	}

	body->ResetMass();

	if (d->sphere_radius)
	{
		for (uint32_t i = 0; i < d->n; ++i)
		{
			b3SphereFixtureDef sd;
			sd.p = ps[i];
			sd.radius = scalar(d->sphere_radius[i]);
			sd.friction = scalar(d->sphere_friction[i]);
			void* mem = body->m_blockAllocator.Allocate(sizeof(b3SphereFixture));
			b3SphereFixture* s = new (mem) b3SphereFixture(sd, body);
			s->m_prev = nullptr;
			s->m_next = body->m_sphereList;
			if (body->m_sphereList) body->m_sphereList->m_prev = s;
			body->m_sphereList = s;
			++body->m_sphereCount;
		}
	}

	for (uint32_t k = 0; k < d->world_sphere_count; ++k)
	{
		const double* w = d->world_spheres + 5 * k;
		b3SphereShape* shape = new b3SphereShape();
		shape->m_center = V3(w);
		shape->m_radius = scalar(w[3]);
		store.shapes.push_back(shape);
		b3WorldFixtureDef wd;
		wd.shape = shape;
		wd.friction = scalar(w[4]);
		body->CreateFixture(wd);
	}
	for (uint32_t k = 0; k < d->world_shape_count; ++k)
	{
		b3Shape* shape = MakeShape(d->world_shapes[k], store);
		if (!shape) continue;
		b3WorldFixtureDef wd;
		wd.shape = shape;
		wd.friction = scalar(d->world_shapes[k].friction);
		body->CreateFixture(wd);
	}
	return body;
}

} // namespace

extern "C" {

// Returns 0 on success.
int ref_simulate(const RefDesc* d, RefRun* run)
{
	std::vector<b3Particle*> ps;
	ShapeStore shapes;
	b3Body* body = BuildBody(d, ps, shapes);

	auto t0 = std::chrono::steady_clock::now();
	for (uint32_t s = 0; s < run->steps; ++s)
	{
		uint32 it;
		if (run->use_body_step)
		{
			body->Step(scalar(run->dt), run->newton_iters, run->max_sub);
			it = b3_forceSolverMaxSubIterations;
			b3_forceSolverMaxSubIterations = 0;
			b3_forceSolverMinSubIterations = B3_MAX_U32;
		}
		else
		{
			it = HarnessStep(body, scalar(run->dt), run->newton_iters, run->max_sub, scalar(run->sub_tol));
		}
		if (run->sub_iters_out) run->sub_iters_out[s] = it;
	}
	auto t1 = std::chrono::steady_clock::now();
	if (run->seconds_out) *run->seconds_out = std::chrono::duration<double>(t1 - t0).count();

	for (uint32_t i = 0; i < d->n; ++i)
	{
		b3Vec3 x = ps[i]->GetPosition();
		b3Vec3 v = ps[i]->GetVelocity();
		run->x_out[3 * i + 0] = x.x; run->x_out[3 * i + 1] = x.y; run->x_out[3 * i + 2] = x.z;
		run->v_out[3 * i + 0] = v.x; run->v_out[3 * i + 1] = v.y; run->v_out[3 * i + 2] = v.z;
	}

	delete body;

	return 0;
}

struct RefHit
{
	int32_t hit;
	uint32_t triangle;   // index of the triangle fixture in RefDesc::tris
	double fraction;
	double normal[3];
};

// b3Body::RayCastSingle (src/bounce_softbody/dynamics/body.cpp:468-521) on the body after
// run->steps harness steps, for `count` segments (p1, p2: 6 doubles each).
int ref_ray_cast(const RefDesc* d, RefRun* run, uint32_t count, const double* segs, RefHit* out)
{
	std::vector<b3Particle*> ps;
	std::vector<b3TriangleFixture*> tris;
	ShapeStore shapes;
	b3Body* body = BuildBody(d, ps, shapes, &tris);
	for (uint32_t s = 0; s < run->steps; ++s)
	{
		uint32 it = HarnessStep(body, scalar(run->dt), run->newton_iters, run->max_sub, scalar(run->sub_tol));
		if (run->sub_iters_out) run->sub_iters_out[s] = it;
	}
	for (uint32_t r = 0; r < count; ++r)
	{
		b3BodyRayCastSingleOutput o;
		RefHit h = {};
		if (body->RayCastSingle(&o, V3(segs + 6 * r), V3(segs + 6 * r + 3)))
		{
			h.hit = 1;
			h.triangle = (uint32_t)(std::find(tris.begin(), tris.end(), o.triangle) - tris.begin());
			h.fraction = o.fraction;
			h.normal[0] = o.normal.x;
			h.normal[1] = o.normal.y;
			h.normal[2] = o.normal.z;
		}
		out[r] = h;
	}
	if (run->x_out)
		for (uint32_t i = 0; i < d->n; ++i)
		{
			b3Vec3 x = ps[i]->GetPosition();
			run->x_out[3 * i + 0] = x.x; run->x_out[3 * i + 1] = x.y; run->x_out[3 * i + 2] = x.z;
		}
	delete body;
	return 0;
}

int ref_scalar_size(void) { return (int)sizeof(scalar); }

} // extern "C"
