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
#include <bounce_softbody/sparse/sparse_solver.h>
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

// ---------------------------------------------------------------- sparse containers and solvers
// Golden vectors for the container / solver boundary (b3SparseMat33, b3DenseVec3, b3DiagMat33,
// b3SparseSolveCG, b3SparseSolveBE). Block values cross this boundary as 9 doubles per block in
// b3Mat33 order (column-major: column x, then y, then z).

struct RefJacobians
{
	uint32_t capacity;       // entries the COO arrays hold
	uint32_t dfdx_count;     // entries written (one per nonzero block, in the matrix's row-list order)
	uint32_t dfdv_count;
	uint32_t* dfdx_rows;     // capacity
	uint32_t* dfdx_cols;
	double* dfdx_vals;       // 9 * capacity
	uint32_t* dfdv_rows;
	uint32_t* dfdv_cols;
	double* dfdv_vals;
	double* x;               // 3n: state the forces are evaluated at (x0 = x, v0 = v)
	double* v;
	double* f;               // 3n: internal forces
	double* fe;              // 3n: external forces incl. m g (force_solver.cpp:116)
	double* mass;            // n: M[i] = mass I (dynamic) or I (force_solver.cpp:113, 125)
	int32_t* dynamic;        // n: S[i] = I (1) or 0 (0) (force_solver.cpp:119, 128)
};

static void put_block(double* out, const b3Mat33& a)
{
	out[0] = a.x.x; out[1] = a.x.y; out[2] = a.x.z;
	out[3] = a.y.x; out[4] = a.y.y; out[5] = a.y.z;
	out[6] = a.z.x; out[7] = a.z.y; out[8] = a.z.z;
}

static b3Mat33 get_block(const double* in)
{
	b3Mat33 a;
	a.x = b3Vec3(scalar(in[0]), scalar(in[1]), scalar(in[2]));
	a.y = b3Vec3(scalar(in[3]), scalar(in[4]), scalar(in[5]));
	a.z = b3Vec3(scalar(in[6]), scalar(in[7]), scalar(in[8]));
	return a;
}

// Steps the body run->steps harness steps, then evaluates the force model once at the resulting
// state exactly as the first Newton iteration of the next step does (after UpdateContacts and
// ClearForces, sparse_force_solver.cpp:137-161). Vertex indices are the input's, not the
// reference's solver ids. Returns 0, or 1 if the COO arrays are too small.
int ref_jacobians(const RefDesc* d, RefRun* run, RefJacobians* out)
{
	std::vector<b3Particle*> ps;
	ShapeStore shapes;
	b3Body* body = BuildBody(d, ps, shapes);
	for (uint32_t s = 0; s < run->steps; ++s)
		HarnessStep(body, scalar(run->dt), run->newton_iters, run->max_sub, scalar(run->sub_tol));

	body->m_contactManager.UpdateContacts();
	for (b3Force* f = body->m_forceList; f; f = f->m_next) f->ClearForces();
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
	const uint32 n = (uint32)particles.size();
	// solver id -> input index
	std::vector<uint32_t> input_of(n);
	for (uint32_t i = 0; i < d->n; ++i) input_of[ps[i]->m_solverId] = i;

	b3DenseVec3 x(n), v(n), fi(n);
	fi.SetZero();
	b3SparseMat33 dfdx(n), dfdv(n);
	const b3Vec3 g = body->m_gravity;
	for (uint32 k = 0; k < n; ++k)
	{
		b3Particle* p = particles[k];
		const uint32_t i = input_of[k];
		x[k] = p->m_position;
		v[k] = p->m_velocity;
		b3Vec3 fe = p->m_force;
		const bool dyn = p->m_type == e_dynamicParticle;
		if (dyn) fe += p->m_mass * g;
		out->fe[3 * i + 0] = fe.x; out->fe[3 * i + 1] = fe.y; out->fe[3 * i + 2] = fe.z;
		out->mass[i] = dyn ? p->m_mass : 1.0;
		out->dynamic[i] = dyn ? 1 : 0;
		out->x[3 * i + 0] = x[k].x; out->x[3 * i + 1] = x[k].y; out->x[3 * i + 2] = x[k].z;
		out->v[3 * i + 0] = v[k].x; out->v[3 * i + 1] = v[k].y; out->v[3 * i + 2] = v[k].z;
	}
	HarnessModel model;
	model.particleCount = n;
	model.particles = particles.data();
	model.forceCount = (uint32)forces.size();
	model.forces = forces.data();
	model.contactCount = (uint32)contacts.size();
	model.contacts = contacts.data();
	b3SparseForceSolverData data;
	data.h = scalar(run->dt);
	data.inv_h = scalar(1) / scalar(run->dt);
	data.x = &x;
	data.v = &v;
	data.f = &fi;
	data.dfdx = &dfdx;
	data.dfdv = &dfdv;
	model.ApplyForces(&data);

	for (uint32 k = 0; k < n; ++k)
	{
		const uint32_t i = input_of[k];
		out->f[3 * i + 0] = fi[k].x; out->f[3 * i + 1] = fi[k].y; out->f[3 * i + 2] = fi[k].z;
	}
	int rc = 0;
	auto dump = [&](const b3SparseMat33& m, uint32_t* rows, uint32_t* cols, double* vals, uint32_t* count) {
		uint32_t c = 0;
		for (uint32 r = 0; r < n; ++r)
			for (b3RowEntry* e = m.rows[r].head; e; e = e->next)
			{
				if (c == out->capacity)
				{
					rc = 1;
					continue;
				}
				rows[c] = input_of[r];
				cols[c] = input_of[e->column];
				put_block(vals + 9 * (size_t)c, e->value);
				++c;
			}
		*count = c;
	};
	dump(dfdx, out->dfdx_rows, out->dfdx_cols, out->dfdx_vals, &out->dfdx_count);
	dump(dfdv, out->dfdv_rows, out->dfdv_cols, out->dfdv_vals, &out->dfdv_count);
	delete body;
	return rc;
}

struct RefSparseIn
{
	uint32_t n;
	double h;
	uint32_t dfdx_count;
	const uint32_t* dfdx_rows;
	const uint32_t* dfdx_cols;
	const double* dfdx_vals;
	uint32_t dfdv_count;
	const uint32_t* dfdv_rows;
	const uint32_t* dfdv_cols;
	const double* dfdv_vals;
	const double* f;        // 3n
	const double* x0;       // 3n; also the Newton iterate x of the first iteration
	const double* v0;       // 3n; also v
	const double* fe;       // 3n
	const double* M;        // 9n
	const double* S;        // 9n
	const double* y;        // 3n
	const double* z;        // 3n
	const double* u;        // 3n test vector
	const double* D;        // 9n test diagonal
	double s;               // test scalar
	uint32_t cg_max_iterations;
	double cg_tolerance;
	uint32_t capacity;      // entries the CSR output of pA holds
};

struct RefSparseOut
{
	// SpMV (b3Mul) of u with: A, pA, D dfdx, dfdx D, s dfdx, dfdx + dfdv, dfdx - dfdv, dfdx + D,
	// D - dfdx (b3Sub(out, D, B) on a fresh out), 0 dfdx (b3Mul with s = 0 leaves out empty)
	double* spmv;           // 10 * 3n
	double* b;              // 3n right-hand side (sparse_force_solver.cpp:167)
	double* pb;             // 3n
	double* diag_u;         // 3n: D u (b3Mul(b3DenseVec3&, const b3DiagMat33&, const b3DenseVec3&))
	double dot_u_pb;        // b3Dot(u, pb)
	double len2_pb;         // b3LengthSquared(pb)
	// pA as CSR, columns ascending within a row
	uint32_t* pA_row_ptr;   // n + 1
	uint32_t* pA_cols;      // capacity
	double* pA_vals;        // 9 * capacity
	uint32_t pA_count;
	// b3SparseSolveCG(pA, pb) from x = 0
	double* cg_x;           // 3n
	uint32_t cg_iterations;
	double cg_error;
	// b3SparseSolveBE, one Newton iteration, with a force model that replays dfdx, dfdv and f
	double* be_x;           // 3n
	double* be_v;           // 3n
	uint32_t be_iterations;
	double be_error;
	uint32_t be_min_sub, be_max_sub;
};

namespace {

void load_coo(b3SparseMat33& m, uint32_t count, const uint32_t* rows, const uint32_t* cols, const double* vals)
{
	for (uint32_t k = 0; k < count; ++k) m(rows[k], cols[k]) += get_block(vals + 9 * (size_t)k);
}

void load_vec(b3DenseVec3& v, const double* p)
{
	for (uint32 i = 0; i < v.n; ++i) v[i] = V3(p + 3 * i);
}

void store_vec(double* p, const b3DenseVec3& v)
{
	for (uint32 i = 0; i < v.n; ++i)
	{
		p[3 * i + 0] = v[i].x; p[3 * i + 1] = v[i].y; p[3 * i + 2] = v[i].z;
	}
}

struct ReplayModel : public b3SparseForceModel
{
	void ApplyForces(const b3SparseForceSolverData* data) override
	{
		load_coo(*data->dfdx, in->dfdx_count, in->dfdx_rows, in->dfdx_cols, in->dfdx_vals);
		load_coo(*data->dfdv, in->dfdv_count, in->dfdv_rows, in->dfdv_cols, in->dfdv_vals);
		for (uint32 i = 0; i < in->n; ++i) (*data->f)[i] += V3(in->f + 3 * i);
	}
	const RefSparseIn* in = nullptr;
};

} // namespace

// The reference's own container operators, CG and backward-Euler solve on given matrices. Returns
// 0, or 1 if the CSR output of pA is too small.
int ref_sparse_ops(const RefSparseIn* in, RefSparseOut* out)
{
	const uint32 n = in->n;
	const scalar h = scalar(in->h);
	b3SparseMat33 dfdx(n), dfdv(n);
	load_coo(dfdx, in->dfdx_count, in->dfdx_rows, in->dfdx_cols, in->dfdx_vals);
	load_coo(dfdv, in->dfdv_count, in->dfdv_rows, in->dfdv_cols, in->dfdv_vals);
	b3DenseVec3 fi(n), x0(n), v0(n), fe(n), y(n), z(n), u(n);
	load_vec(fi, in->f);
	load_vec(x0, in->x0);
	load_vec(v0, in->v0);
	load_vec(fe, in->fe);
	load_vec(y, in->y);
	load_vec(z, in->z);
	load_vec(u, in->u);
	b3DiagMat33 M(n), S(n), D(n);
	for (uint32 i = 0; i < n; ++i)
	{
		M[i] = get_block(in->M + 9 * (size_t)i);
		S[i] = get_block(in->S + 9 * (size_t)i);
		D[i] = get_block(in->D + 9 * (size_t)i);
	}
	const b3DenseVec3& x = x0;
	const b3DenseVec3& v = v0;

	// sparse_force_solver.cpp:165-174
	b3DiagMat33 ST(n);
	b3Transpose(ST, S);
	b3DiagMat33 I(n);
	I.SetIdentity();
	b3SparseMat33 A = M - h * dfdv - (h * h) * dfdx;
	b3DenseVec3 b = M * (v0 - v) + h * (fe + fi) + h * dfdx * (x0 - x + h * v + y);
	b3SparseMat33 pA = S * A * ST + I - S;
	b3DenseVec3 pb = S * (b - A * z);

	const size_t n3 = 3 * (size_t)n;
	const scalar s = scalar(in->s);
	store_vec(out->spmv + 0 * n3, A * u);
	store_vec(out->spmv + 1 * n3, pA * u);
	store_vec(out->spmv + 2 * n3, (D * dfdx) * u);
	store_vec(out->spmv + 3 * n3, (dfdx * D) * u);
	store_vec(out->spmv + 4 * n3, (s * dfdx) * u);
	store_vec(out->spmv + 5 * n3, (dfdx + dfdv) * u);
	store_vec(out->spmv + 6 * n3, (dfdx - dfdv) * u);
	store_vec(out->spmv + 7 * n3, (dfdx + D) * u);
	store_vec(out->spmv + 8 * n3, (D - dfdx) * u);
	store_vec(out->spmv + 9 * n3, (scalar(0) * dfdx) * u);
	store_vec(out->b, b);
	store_vec(out->pb, pb);
	store_vec(out->diag_u, D * u);
	out->dot_u_pb = b3Dot(u, pb);
	out->len2_pb = b3LengthSquared(pb);

	int rc = 0;
	uint32_t c = 0;
	out->pA_row_ptr[0] = 0;
	for (uint32 r = 0; r < n; ++r)
	{
		std::vector<std::pair<uint32, b3Mat33>> row;
		for (b3RowEntry* e = pA.rows[r].head; e; e = e->next) row.push_back({e->column, e->value});
		std::sort(row.begin(), row.end(), [](const std::pair<uint32, b3Mat33>& a, const std::pair<uint32, b3Mat33>& b) {
			return a.first < b.first;
		});
		for (auto& e : row)
		{
			if (c == in->capacity)
			{
				rc = 1;
				continue;
			}
			out->pA_cols[c] = e.first;
			put_block(out->pA_vals + 9 * (size_t)c, e.second);
			++c;
		}
		out->pA_row_ptr[r + 1] = c;
	}
	out->pA_count = c;

	b3DenseVec3 xcg(n);
	xcg.SetZero();
	b3SolveCGInput ci;
	ci.A = &pA;
	ci.b = &pb;
	ci.maxIterations = in->cg_max_iterations;
	ci.tolerance = scalar(in->cg_tolerance);
	b3SolveCGOutput co;
	co.x = &xcg;
	b3SparseSolveCG(&co, &ci);
	store_vec(out->cg_x, xcg);
	out->cg_iterations = co.iterations;
	out->cg_error = co.error;

	ReplayModel model;
	model.in = in;
	b3DenseVec3 xb(n), vb(n);
	b3SolveBEInput bi;
	bi.h = h;
	bi.inv_h = scalar(1) / h;
	bi.forceModel = &model;
	bi.dofCount = n;
	bi.x0 = &x0;
	bi.v0 = &v0;
	bi.fe = &fe;
	bi.M = &M;
	bi.y = &y;
	bi.S = &S;
	bi.z = &z;
	bi.maxIterations = 1;
	bi.maxSubIterations = in->cg_max_iterations;
	bi.subTolerance = scalar(in->cg_tolerance);
	b3SolveBEOutput bo;
	bo.x = &xb;
	bo.v = &vb;
	bo.minSubIterations = B3_MAX_U32;
	bo.maxSubIterations = 0;
	b3SparseSolveBE(&bo, &bi);
	store_vec(out->be_x, xb);
	store_vec(out->be_v, vb);
	out->be_iterations = bo.iterations;
	out->be_error = bo.error;
	out->be_min_sub = bo.minSubIterations;
	out->be_max_sub = bo.maxSubIterations;
	return rc;
}

int ref_scalar_size(void) { return (int)sizeof(scalar); }

} // extern "C"
