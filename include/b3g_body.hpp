// b3g_body.hpp — the reference's body / particle / force API over the b3g C ABI (header-only).
//
// A program written against Bounce Softbody's b3Body (include/bounce_softbody/dynamics/body.h)
// builds against this header and links libb3g.so instead: the same class and definition names,
// the same creation calls and the same Step(dt, forceIterations, forceSubIterations). The body's
// state lives on the GPU; particles read it back on demand.
//
// What maps where:
//   b3Body::CreateParticle / CreateForce / DestroyForce / CreateTetrahedron / CreateTriangle /
//   CreateSphere / CreateFixture / SetGravity
//                                   recorded on the host; the device body (b3g_body_create) is
//                                   built at the first Step and rebuilt after topology changes.
//                                   Forces: tetrahedron and triangle elements, springs,
//                                   Baraff-Witkin stretch and shear, mouse springs.
//   b3Body::Step                    b3g_body_step (uploads pending forces / translations first)
//   b3Particle::Get/SetPosition, Get/SetVelocity, ApplyForce, ApplyTranslation, SetType
//                                   b3g_body_get_state / set_state / apply_* / set_types
//   b3_forceSolver*Iterations       b3Body::GetStepStats()
// Extensions (no reference counterpart): SetSolverTolerance (the reference's Step always runs the
// PCG at FLT_EPSILON), SetPrecision, SetPreconditioner, SetContactMode (filtered contacts).
//   b3Body::RayCastSingle            b3g_body_ray_cast
// Not provided: debug draw, DestroyParticle and the Destroy* calls of fixtures.
#pragma once

#include "b3g.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

typedef float scalar;
typedef uint32_t uint32;

struct b3Vec3
{
	b3Vec3() : x(0), y(0), z(0) {}
	b3Vec3(scalar _x, scalar _y, scalar _z) : x(_x), y(_y), z(_z) {}
	void SetZero() { x = y = z = 0; }
	void Set(scalar _x, scalar _y, scalar _z) { x = _x; y = _y; z = _z; }
	b3Vec3 operator+(const b3Vec3& b) const { return b3Vec3(x + b.x, y + b.y, z + b.z); }
	b3Vec3 operator-(const b3Vec3& b) const { return b3Vec3(x - b.x, y - b.y, z - b.z); }
	b3Vec3& operator+=(const b3Vec3& b) { x += b.x; y += b.y; z += b.z; return *this; }
	scalar x, y, z;
};
inline b3Vec3 operator*(scalar s, const b3Vec3& v) { return b3Vec3(s * v.x, s * v.y, s * v.z); }
inline scalar b3Dot(const b3Vec3& a, const b3Vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline b3Vec3 b3Cross(const b3Vec3& a, const b3Vec3& b)
{
	return b3Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline scalar b3Length(const b3Vec3& v) { return std::sqrt(b3Dot(v, v)); }
inline scalar b3Distance(const b3Vec3& a, const b3Vec3& b)
{
	b3Vec3 d = a - b;
	return std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
}

enum b3ParticleType
{
	e_staticParticle,
	e_kinematicParticle,
	e_dynamicParticle
};

struct b3ParticleDef
{
	b3ParticleType type = e_staticParticle;
	b3Vec3 position;
	b3Vec3 velocity;
	scalar damping = 0;
	uint32 userIndex = 0xFFFFFFFFu;
	void* userData = nullptr;
};

class b3Body;

class b3Particle
{
public:
	void SetType(b3ParticleType type);
	b3ParticleType GetType() const { return m_type; }
	void SetPosition(const b3Vec3& position);
	const b3Vec3& GetPosition() const;
	void SetVelocity(const b3Vec3& velocity);
	const b3Vec3& GetVelocity() const;
	scalar GetMass() const;
	void ApplyForce(const b3Vec3& force);
	const b3Vec3& GetForce() const { return m_force; }
	void ApplyImpulse(const b3Vec3& impulse);
	void ApplyTranslation(const b3Vec3& translation);
	const b3Vec3& GetTranslation() const { return m_translation; }
	scalar GetDamping() const { return m_damping; }
	void SetUserIndex(uint32 i) { m_userIndex = i; }
	uint32 GetUserIndex() const { return m_userIndex; }
	void SetUserData(void* p) { m_userData = p; }
	void* GetUserData() const { return m_userData; }

private:
	friend class b3Body;
	b3Body* m_body = nullptr;
	uint32 m_index = 0;
	b3ParticleType m_type = e_staticParticle;
	scalar m_damping = 0;
	b3Vec3 m_force, m_translation;
	uint32 m_userIndex = 0xFFFFFFFFu;
	void* m_userData = nullptr;
};

enum b3ForceType
{
	e_stretchForce,
	e_shearForce,
	e_springForce,
	e_mouseForce,
	e_triangleElementForce,
	e_tetrahedronElementForce
};

struct b3ForceDef
{
	b3ForceType type;
	uint32 userIndex = 0xFFFFFFFFu;
};

struct b3SpringForceDef : public b3ForceDef
{
	b3SpringForceDef() { type = e_springForce; }
	// spring_force.cpp:25-35: rest length from the particles' current positions
	void Initialize(b3Particle* particle1, b3Particle* particle2, scalar ks, scalar kd)
	{
		p1 = particle1;
		p2 = particle2;
		length = b3Distance(p1->GetPosition(), p2->GetPosition());
		stiffness = ks;
		dampingStiffness = kd;
	}
	b3Particle* p1 = nullptr;
	b3Particle* p2 = nullptr;
	scalar length = 0;
	scalar stiffness = 0;
	scalar dampingStiffness = 0;
};

struct b3TriangleElementForceDef : public b3ForceDef
{
	b3TriangleElementForceDef() { type = e_triangleElementForce; }
	b3Particle *p1 = nullptr, *p2 = nullptr, *p3 = nullptr;
	b3Vec3 v1, v2, v3;
	scalar youngModulusX = 100, youngModulusY = 100, shearModulus = 50;
	scalar poissonRationXY = 0.2f, poissonRationYX = 0.2f;
	scalar stiffnessDamping = 0;
};

// Baraff-Witkin stretch and shear triangles (stretch_force.h, shear_force.h): rest (u, v)
// coordinates of the three particles, from Initialize or set directly.
struct b3StretchForceDef : public b3ForceDef
{
	b3StretchForceDef() { type = e_stretchForce; }
	// stretch_force.cpp:36-60
	void Initialize(const b3Vec3& A, const b3Vec3& B, const b3Vec3& C)
	{
		b3Vec3 AB = B - A, AC = C - A;
		u1 = 0;
		v1 = 0;
		u2 = b3Length(AB);
		v2 = 0;
		b3Vec3 n_AB(AB.x / u2, AB.y / u2, AB.z / u2);
		u3 = b3Dot(AC, n_AB);
		v3 = b3Length(b3Cross(AB, AC)) / u2;
	}
	b3Particle *p1 = nullptr, *p2 = nullptr, *p3 = nullptr;
	scalar u1 = 0, v1 = 0, u2 = 0, v2 = 0, u3 = 0, v3 = 0;
	scalar stiffness_u = 0, damping_stiffness_u = 0, b_u = 1;
	scalar stiffness_v = 0, damping_stiffness_v = 0, b_v = 1;
};

struct b3ShearForceDef : public b3ForceDef
{
	b3ShearForceDef() { type = e_shearForce; }
	// shear_force.cpp:25-49 (the stretch definition's frame)
	void Initialize(const b3Vec3& A, const b3Vec3& B, const b3Vec3& C)
	{
		b3StretchForceDef s;
		s.Initialize(A, B, C);
		u1 = s.u1; v1 = s.v1; u2 = s.u2; v2 = s.v2; u3 = s.u3; v3 = s.v3;
	}
	b3Particle *p1 = nullptr, *p2 = nullptr, *p3 = nullptr;
	scalar u1 = 0, v1 = 0, u2 = 0, v2 = 0, u3 = 0, v3 = 0;
	scalar stiffness = 0, dampingStiffness = 0;
};

// Mouse spring (mouse_force.h): particle 1 held at `length` from the point with barycentric
// weights w2, w3, w4 on the triangle (p2, p3, p4).
struct b3MouseForceDef : public b3ForceDef
{
	b3MouseForceDef() { type = e_mouseForce; }
	b3Particle *p1 = nullptr, *p2 = nullptr, *p3 = nullptr, *p4 = nullptr;
	scalar w2 = 0, w3 = 0, w4 = 0;
	scalar length = 0, stiffness = 0, dampingStiffness = 0;
};

struct b3TetrahedronElementForceDef : public b3ForceDef
{
	b3TetrahedronElementForceDef() { type = e_tetrahedronElementForce; }
	b3Particle *p1 = nullptr, *p2 = nullptr, *p3 = nullptr, *p4 = nullptr;
	b3Vec3 v1, v2, v3, v4;
	scalar youngModulus = 500, poissonRatio = 0.3f, stiffnessDamping = 0;
};

struct b3Force
{
	b3ForceType type;
	uint32 index;
};

struct b3FixtureDef
{
	scalar radius = 0, density = 0, friction = 0;
	uint32 userIndex = 0xFFFFFFFFu;
};
struct b3SphereFixtureDef : public b3FixtureDef
{
	b3Particle* p = nullptr;
};
// A triangle fixture (b3TriangleFixture): the handle CreateTriangle returns and ray casts report.
struct b3TriangleFixture
{
	b3Particle *m_p1 = nullptr, *m_p2 = nullptr, *m_p3 = nullptr;
	scalar m_density = 0;
};

// b3BodyRayCastSingleOutput (include/bounce_softbody/dynamics/body.h:52-57)
struct b3BodyRayCastSingleOutput
{
	b3TriangleFixture* triangle = nullptr;
	scalar fraction = 0;
	b3Vec3 normal;
};

struct b3TriangleFixtureDef : public b3FixtureDef
{
	b3Particle *p1 = nullptr, *p2 = nullptr, *p3 = nullptr;
	b3Vec3 v1, v2, v3;
};
struct b3TetrahedronFixtureDef : public b3FixtureDef
{
	b3Particle *p1 = nullptr, *p2 = nullptr, *p3 = nullptr, *p4 = nullptr;
	b3Vec3 v1, v2, v3, v4;
};

// Static world shapes (include/bounce_softbody/collision/shapes/): the same member names; the
// geometry is read when the fixture is created.
struct b3Quat
{
	b3Vec3 v;
	scalar s = 1;
	b3Quat() {}
	b3Quat(const b3Vec3& _v, scalar _s) : v(_v), s(_s) {}
};
struct b3Transform
{
	b3Vec3 translation;
	b3Quat rotation;
	void SetIdentity()
	{
		translation = b3Vec3(0, 0, 0);
		rotation = b3Quat();
	}
};
class b3Shape
{
public:
	enum Type { e_sphere = 0, e_capsule = 1, e_triangle = 2, e_box = 3, e_mesh = 4, e_sdf = 5 };
	virtual ~b3Shape() {}
	Type GetType() const { return m_type; }
	Type m_type = e_sphere;
	scalar m_radius = 0;
};
struct b3SphereShape : public b3Shape
{
	b3SphereShape() { m_type = e_sphere; }
	b3Vec3 m_center;
};
struct b3CapsuleShape : public b3Shape
{
	b3CapsuleShape() : m_center1(0, 1, 0), m_center2(0, -1, 0) { m_type = e_capsule; }
	b3Vec3 m_center1, m_center2;
};
struct b3BoxShape : public b3Shape
{
	b3BoxShape() { m_type = e_box; m_xf.SetIdentity(); }
	b3Vec3 m_extents;
	b3Transform m_xf;
};
struct b3TriangleShape : public b3Shape
{
	b3TriangleShape() { m_type = e_triangle; }
	void Set(const b3Vec3& v1, const b3Vec3& v2, const b3Vec3& v3)
	{
		m_vertex1 = v1;
		m_vertex2 = v2;
		m_vertex3 = v3;
	}
	b3Vec3 m_vertex1, m_vertex2, m_vertex3;
};
// b3Triangle / b3Mesh (collision/geometry/mesh.h): wing vertex 0xFFFFFFFF = open edge
struct b3Triangle
{
	uint32 v1, v2, v3;
	uint32 u1 = 0xFFFFFFFFu, u2 = 0xFFFFFFFFu, u3 = 0xFFFFFFFFu;
};
struct b3Mesh
{
	uint32 vertexCount = 0;
	b3Vec3* vertices = nullptr;
	uint32 triangleCount = 0;
	b3Triangle* triangles = nullptr;
};
struct b3MeshShape : public b3Shape
{
	b3MeshShape() : m_scale(1, 1, 1) { m_type = e_mesh; m_xf.SetIdentity(); }
	const b3Mesh* m_mesh = nullptr;
	b3Transform m_xf;
	b3Vec3 m_scale;
};
// b3SDF (collision/geometry/sdf.h): a voxel grid of signed distances over an AABB, x fastest
struct b3SDF
{
	uint32 width = 0, height = 0, depth = 0;
	const scalar* voxels = nullptr;
	b3Vec3 lowerBound, upperBound;
};
struct b3SDFShape : public b3Shape
{
	b3SDFShape() { m_type = e_sdf; m_xf.SetIdentity(); }
	const b3SDF* m_sdf = nullptr;
	b3Transform m_xf;
	bool m_invert = false;
};
struct b3WorldFixtureDef
{
	const b3Shape* shape = nullptr;
	scalar friction = 0.5f;
};

class b3Body
{
public:
	explicit b3Body(int device = 0)
	{
		check(b3g_context_create(device, &m_ctx), "b3g_context_create");
		b3g_solver_config_default(&m_cfg);
	}
	~b3Body()
	{
		for (b3Particle* p : m_particles) delete p;
		for (b3Force* f : m_forceHandles) delete f;
		for (b3TriangleFixture* t : m_triFixture) delete t;
		if (m_body) b3g_body_destroy(m_body);
		if (m_ctx) b3g_context_destroy(m_ctx);
	}
	b3Body(const b3Body&) = delete;
	b3Body& operator=(const b3Body&) = delete;

	b3Particle* CreateParticle(const b3ParticleDef& def)
	{
		fetch();
		b3Particle* p = new b3Particle();
		p->m_body = this;
		p->m_index = (uint32)m_particles.size();
		p->m_type = def.type;
		p->m_damping = def.damping;
		p->m_userIndex = def.userIndex;
		p->m_userData = def.userData;
		m_particles.push_back(p);
		m_x.push_back(def.position);
		m_v.push_back(def.velocity);  // as the reference constructor: SetType(static) zeroes it
		m_topologyDirty = true;
		return p;
	}

	b3Force* CreateForce(const b3ForceDef& def)
	{
		b3Force* f = new b3Force();
		f->type = def.type;
		switch (def.type)
		{
		case e_tetrahedronElementForce:
		{
			const b3TetrahedronElementForceDef& d = (const b3TetrahedronElementForceDef&)def;
			f->index = (uint32)m_tetE.size();
			const b3Particle* ps[4] = {d.p1, d.p2, d.p3, d.p4};
			const b3Vec3 vs[4] = {d.v1, d.v2, d.v3, d.v4};
			for (int k = 0; k < 4; ++k)
			{
				m_tets.push_back(ps[k]->m_index);
				push3(m_tetRest, vs[k]);
			}
			m_tetE.push_back(d.youngModulus);
			m_tetNu.push_back(d.poissonRatio);
			m_tetKd.push_back(d.stiffnessDamping);
			m_tetDensity.push_back(0);
			break;
		}
		case e_triangleElementForce:
		{
			const b3TriangleElementForceDef& d = (const b3TriangleElementForceDef&)def;
			const uint32 a[3] = {d.p1->m_index, d.p2->m_index, d.p3->m_index};
			const b3Vec3 vs[3] = {d.v1, d.v2, d.v3};
			size_t e = find_tri(a, true);  // a mass fixture of the same particles without an element
			if (e == m_triEx.size())
			{
				for (int k = 0; k < 3; ++k) m_tris.push_back(a[k]);
				m_triRest.resize(m_triRest.size() + 9);
				m_triEx.push_back(0);
				m_triEy.push_back(0);
				m_triEs.push_back(0);
				m_triNxy.push_back(0);
				m_triNyx.push_back(0);
				m_triKd.push_back(0);
				m_triDensity.push_back(0);
				m_triElem.push_back(0);
				m_triFixture.push_back(nullptr);
			}
			for (int k = 0; k < 3; ++k)
				for (int c = 0; c < 3; ++c) m_triRest[9 * e + 3 * k + c] = (&vs[k].x)[c];
			m_triEx[e] = d.youngModulusX;
			m_triEy[e] = d.youngModulusY;
			m_triEs[e] = d.shearModulus;
			m_triNxy[e] = d.poissonRationXY;
			m_triNyx[e] = d.poissonRationYX;
			m_triKd[e] = d.stiffnessDamping;
			m_triElem[e] = 1;
			f->index = (uint32)e;
			break;
		}
		case e_stretchForce:
		{
			const b3StretchForceDef& d = (const b3StretchForceDef&)def;
			f->index = (uint32)m_stParams.size() / 6;
			for (const b3Particle* p : {d.p1, d.p2, d.p3}) m_stTris.push_back(p->m_index);
			for (scalar c : {d.u1, d.v1, d.u2, d.v2, d.u3, d.v3}) m_stUv.push_back(c);
			for (scalar c : {d.stiffness_u, d.damping_stiffness_u, d.b_u, d.stiffness_v, d.damping_stiffness_v, d.b_v})
				m_stParams.push_back(c);
			break;
		}
		case e_shearForce:
		{
			const b3ShearForceDef& d = (const b3ShearForceDef&)def;
			f->index = (uint32)m_shParams.size() / 2;
			for (const b3Particle* p : {d.p1, d.p2, d.p3}) m_shTris.push_back(p->m_index);
			for (scalar c : {d.u1, d.v1, d.u2, d.v2, d.u3, d.v3}) m_shUv.push_back(c);
			m_shParams.push_back(d.stiffness);
			m_shParams.push_back(d.dampingStiffness);
			break;
		}
		case e_mouseForce:
		{
			const b3MouseForceDef& d = (const b3MouseForceDef&)def;
			f->index = (uint32)m_msParams.size() / 6;
			for (const b3Particle* p : {d.p1, d.p2, d.p3, d.p4}) m_msIds.push_back(p->m_index);
			for (scalar c : {d.w2, d.w3, d.w4, d.stiffness, d.dampingStiffness, d.length}) m_msParams.push_back(c);
			break;
		}
		case e_springForce:
		{
			const b3SpringForceDef& d = (const b3SpringForceDef&)def;
			f->index = (uint32)m_sprL0.size();
			m_springs.push_back(d.p1->m_index);
			m_springs.push_back(d.p2->m_index);
			m_sprL0.push_back(d.length);
			m_sprKs.push_back(d.stiffness);
			m_sprKd.push_back(d.dampingStiffness);
			break;
		}
		default:
			delete f;
			throw std::invalid_argument("b3g: unknown force type");
		}
		m_forceHandles.push_back(f);
		m_topologyDirty = true;
		return f;
	}

	// b3Body::DestroyForce: the force's entries leave the arrays; handles behind it move down.
	void DestroyForce(b3Force* force)
	{
		auto it = std::find(m_forceHandles.begin(), m_forceHandles.end(), force);
		if (it == m_forceHandles.end()) throw std::invalid_argument("b3g: DestroyForce of an unknown force");
		const uint32 e = force->index;
		auto drop = [e](auto& v, size_t w) { v.erase(v.begin() + w * e, v.begin() + w * (e + 1)); };
		bool shift = true;
		switch (force->type)
		{
		case e_tetrahedronElementForce:
			drop(m_tets, 4); drop(m_tetRest, 12); drop(m_tetE, 1); drop(m_tetNu, 1); drop(m_tetKd, 1);
			drop(m_tetDensity, 1);
			break;
		case e_triangleElementForce:
			if (m_triFixture[e])
			{
				// the mass fixture stays
				m_triElem[e] = 0;
				m_triEx[e] = m_triEy[e] = m_triEs[e] = m_triNxy[e] = m_triNyx[e] = m_triKd[e] = 0;
				shift = false;
				break;
			}
			drop(m_tris, 3); drop(m_triRest, 9); drop(m_triEx, 1); drop(m_triEy, 1); drop(m_triEs, 1);
			drop(m_triNxy, 1); drop(m_triNyx, 1); drop(m_triKd, 1); drop(m_triDensity, 1); drop(m_triElem, 1);
			drop(m_triFixture, 1);
			break;
		case e_springForce:
			drop(m_springs, 2); drop(m_sprL0, 1); drop(m_sprKs, 1); drop(m_sprKd, 1);
			break;
		case e_stretchForce:
			drop(m_stTris, 3); drop(m_stUv, 6); drop(m_stParams, 6);
			break;
		case e_shearForce:
			drop(m_shTris, 3); drop(m_shUv, 6); drop(m_shParams, 2);
			break;
		case e_mouseForce:
			drop(m_msIds, 4); drop(m_msParams, 6);
			break;
		}
		if (shift)
			for (b3Force* h : m_forceHandles)
				if (h != force && h->type == force->type && h->index > e) --h->index;
		m_forceHandles.erase(it);
		delete force;
		m_topologyDirty = true;
	}

	// Tetrahedron fixtures carry the density of the lumped mass (b3Body::ResetMass) and pair with
	// the element force of the same particles, which must exist (a tetrahedron fixture alone is
	// not modelled; destroying the element drops its fixture's mass too).
	void CreateTetrahedron(const b3TetrahedronFixtureDef& def)
	{
		uint32 a[4] = {def.p1->m_index, def.p2->m_index, def.p3->m_index, def.p4->m_index};
		for (size_t e = 0; e < m_tetE.size(); ++e)
			if (same_set(&m_tets[4 * e], a, 4))
			{
				m_tetDensity[e] = def.density;
				m_topologyDirty = true;
				return;
			}
		throw std::invalid_argument("b3g: CreateTetrahedron needs the tetrahedron element force created first");
	}
	// A triangle fixture pairs with the element force of the same particles when there is one;
	// otherwise it is a mass fixture of its own (cloth held by stretch and shear forces).
	b3TriangleFixture* CreateTriangle(const b3TriangleFixtureDef& def)
	{
		const uint32 a[3] = {def.p1->m_index, def.p2->m_index, def.p3->m_index};
		size_t e = find_tri(a, false);
		if (e == m_triEx.size())
		{
			for (int k = 0; k < 3; ++k) m_tris.push_back(a[k]);
			for (const b3Vec3* v : {&def.v1, &def.v2, &def.v3}) push3(m_triRest, *v);
			for (std::vector<float>* v : {&m_triEx, &m_triEy, &m_triEs, &m_triNxy, &m_triNyx, &m_triKd})
				v->push_back(0);
			m_triDensity.push_back(0);
			m_triElem.push_back(0);
			m_triFixture.push_back(nullptr);
		}
		b3TriangleFixture* t = new b3TriangleFixture();
		t->m_p1 = def.p1;
		t->m_p2 = def.p2;
		t->m_p3 = def.p3;
		t->m_density = def.density;
		m_triFixture[e] = t;
		m_triDensity[e] = def.density;
		m_topologyDirty = true;
		return t;
	}
	void CreateSphere(const b3SphereFixtureDef& def)
	{
		if (m_sphereRadius.size() < m_particles.size())
		{
			m_sphereRadius.resize(m_particles.size(), 0);
			m_sphereFriction.resize(m_particles.size(), 0);
		}
		m_sphereRadius[def.p->m_index] = def.radius;
		m_sphereFriction[def.p->m_index] = def.friction;
		m_topologyDirty = true;
	}
	void CreateFixture(const b3WorldFixtureDef& def)
	{
		const b3Shape* sh = def.shape;
		if (sh->m_type == b3Shape::e_sphere)
		{
			const b3SphereShape* sp = static_cast<const b3SphereShape*>(sh);
			m_world.push_back(sp->m_center.x);
			m_world.push_back(sp->m_center.y);
			m_world.push_back(sp->m_center.z);
			m_world.push_back(sp->m_radius);
			m_world.push_back(def.friction);
			m_topologyDirty = true;
			return;
		}
		b3g_world_shape w{};
		w.radius = sh->m_radius;
		w.friction = def.friction;
		w.rotation[3] = 1;
		auto set_xf = [&](const b3Transform& xf) {
			w.rotation[0] = xf.rotation.v.x;
			w.rotation[1] = xf.rotation.v.y;
			w.rotation[2] = xf.rotation.v.z;
			w.rotation[3] = xf.rotation.s;
			w.translation[0] = xf.translation.x;
			w.translation[1] = xf.translation.y;
			w.translation[2] = xf.translation.z;
		};
		auto set_p = [&](int at, const b3Vec3& v) {
			w.p[at] = v.x;
			w.p[at + 1] = v.y;
			w.p[at + 2] = v.z;
		};
		m_shapeData.emplace_back();
		ShapeData& own = m_shapeData.back();
		switch (sh->m_type)
		{
		case b3Shape::e_capsule:
		{
			const b3CapsuleShape* c = static_cast<const b3CapsuleShape*>(sh);
			w.type = B3G_SHAPE_CAPSULE;
			set_p(0, c->m_center1);
			set_p(3, c->m_center2);
			break;
		}
		case b3Shape::e_box:
		{
			const b3BoxShape* b = static_cast<const b3BoxShape*>(sh);
			w.type = B3G_SHAPE_BOX;
			set_p(0, b->m_extents);
			set_xf(b->m_xf);
			break;
		}
		case b3Shape::e_triangle:
		{
			const b3TriangleShape* t = static_cast<const b3TriangleShape*>(sh);
			w.type = B3G_SHAPE_TRIANGLE;
			set_p(0, t->m_vertex1);
			set_p(3, t->m_vertex2);
			set_p(6, t->m_vertex3);
			break;
		}
		case b3Shape::e_mesh:
		{
			const b3MeshShape* m = static_cast<const b3MeshShape*>(sh);
			w.type = B3G_SHAPE_MESH;
			set_xf(m->m_xf);
			w.scale[0] = m->m_scale.x;
			w.scale[1] = m->m_scale.y;
			w.scale[2] = m->m_scale.z;
			for (uint32 v = 0; v < m->m_mesh->vertexCount; ++v) push3(own.f, m->m_mesh->vertices[v]);
			for (uint32 t = 0; t < m->m_mesh->triangleCount; ++t)
			{
				const b3Triangle& T = m->m_mesh->triangles[t];
				own.u.insert(own.u.end(), {T.v1, T.v2, T.v3});
				own.u2.insert(own.u2.end(), {T.u1, T.u2, T.u3});
			}
			w.vertex_count = m->m_mesh->vertexCount;
			w.triangle_count = m->m_mesh->triangleCount;
			break;
		}
		case b3Shape::e_sdf:
		{
			const b3SDFShape* f = static_cast<const b3SDFShape*>(sh);
			w.type = B3G_SHAPE_SDF;
			set_xf(f->m_xf);
			const b3SDF* g = f->m_sdf;
			w.grid[0] = g->width;
			w.grid[1] = g->height;
			w.grid[2] = g->depth;
			own.f.assign(g->voxels, g->voxels + (size_t)g->width * g->height * g->depth);
			w.grid_lower[0] = g->lowerBound.x;
			w.grid_lower[1] = g->lowerBound.y;
			w.grid_lower[2] = g->lowerBound.z;
			w.grid_upper[0] = g->upperBound.x;
			w.grid_upper[1] = g->upperBound.y;
			w.grid_upper[2] = g->upperBound.z;
			w.invert = f->m_invert ? 1 : 0;
			break;
		}
		default: break;
		}
		m_shapes.push_back(w);
		m_topologyDirty = true;
	}

	void SetGravity(const b3Vec3& g)
	{
		m_gravity = g;
		m_topologyDirty = true;
	}
	b3Vec3 GetGravity() const { return m_gravity; }

	// b3Body::Step (body.cpp:552-604) on the GPU.
	void Step(scalar dt, uint32 forceIterations, uint32 forceSubIterations)
	{
		build();
		flush_inputs();
		m_cfg.force_iterations = forceIterations;
		m_cfg.max_pcg_iterations = forceSubIterations;
		check(b3g_body_step(m_body, dt, &m_cfg, &m_stats), "b3g_body_step");
		for (b3Particle* p : m_particles)
		{
			p->m_force.SetZero();
			p->m_translation.SetZero();
		}
		m_hostFresh = false;
	}

	// b3Body::RayCastSingle (body.cpp:468-521): the closest triangle hit by the segment p1 -> p2,
	// at the current positions (b3g_body_ray_cast). Triangles created only as element forces (no
	// fixture) are hit too, and then reported with a null fixture.
	bool RayCastSingle(b3BodyRayCastSingleOutput* output, const b3Vec3& p1, const b3Vec3& p2) const
	{
		b3Body* self = const_cast<b3Body*>(this);
		self->build();
		self->flush_state();  // pending forces and translations stay for the next Step
		const float seg[6] = {p1.x, p1.y, p1.z, p2.x, p2.y, p2.z};
		b3g_ray_hit h;
		check(b3g_body_ray_cast(m_body, seg, 1, &h), "b3g_body_ray_cast");
		if (!h.hit) return false;
		output->triangle = m_triFixture[h.triangle];
		output->fraction = h.fraction;
		output->normal.Set(h.normal[0], h.normal[1], h.normal[2]);
		return true;
	}

	scalar GetEnergy() const
	{
		const_cast<b3Body*>(this)->fetch();
		scalar E = 0;
		for (size_t i = 0; i < m_particles.size(); ++i)
			E += mass_of(i) * (m_v[i].x * m_v[i].x + m_v[i].y * m_v[i].y + m_v[i].z * m_v[i].z);
		return scalar(0.5) * E;
	}

	uint32 GetParticleCount() const { return (uint32)m_particles.size(); }
	b3Particle* GetParticle(uint32 i) { return m_particles[i]; }
	const b3g_step_stats& GetStepStats() const { return m_stats; }
	void SetSolverTolerance(double pcgTolerance) { m_cfg.pcg_tolerance = pcgTolerance; }
	void SetPrecision(b3g_precision p) { m_cfg.precision = p; }
	void SetPreconditioner(b3g_preconditioner p) { m_cfg.preconditioner = p; }
	void SetContactMode(b3g_contact_mode m) { m_cfg.contact_mode = m; }
	b3g_body* GetDeviceBody()
	{
		build();
		return m_body;
	}

private:
	friend class b3Particle;

	static void check(int rc, const char* what)
	{
		if (rc != B3G_OK) throw std::runtime_error(std::string(what) + ": " + b3g_last_error());
	}
	static void push3(std::vector<float>& v, const b3Vec3& p)
	{
		v.push_back(p.x);
		v.push_back(p.y);
		v.push_back(p.z);
	}
	static bool same_set(const uint32* a, const uint32* b, int k)
	{
		for (int i = 0; i < k; ++i)
		{
			bool found = false;
			for (int j = 0; j < k; ++j) found = found || a[i] == b[j];
			if (!found) return false;
		}
		return true;
	}
	scalar mass_of(size_t i) const { return i < m_mass.size() ? m_mass[i] : 0; }
	// the triangle entry of these particles that lacks an element (want_fixture_only) or a
	// fixture; the entry count when there is none
	size_t find_tri(const uint32* a, bool want_fixture_only) const
	{
		for (size_t e = 0; e < m_triEx.size(); ++e)
			if (same_set(&m_tris[3 * e], a, 3) && (want_fixture_only ? !m_triElem[e] : !m_triFixture[e])) return e;
		return m_triEx.size();
	}

	// device -> host state, when the host copy is stale
	void fetch()
	{
		if (!m_body || m_hostFresh) return;
		std::vector<float> x(3 * m_x.size()), v(3 * m_v.size());
		check(b3g_body_get_state(m_body, x.data(), v.data()), "b3g_body_get_state");
		for (size_t i = 0; i < m_x.size(); ++i)
		{
			m_x[i].Set(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
			m_v[i].Set(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
		}
		m_hostFresh = true;
	}

	void build()
	{
		if (m_body && !m_topologyDirty) return;
		fetch();
		std::vector<float> x, v, damping;
		std::vector<int32_t> types;
		for (size_t i = 0; i < m_particles.size(); ++i)
		{
			push3(x, m_x[i]);
			push3(v, m_v[i]);
			damping.push_back(m_particles[i]->m_damping);
			types.push_back((int32_t)m_particles[i]->m_type);
		}
		b3g_body_desc d = {};
		d.vertex_count = (uint32)m_particles.size();
		d.positions = x.data();
		d.velocities = v.data();
		d.types = types.data();
		d.damping = damping.data();
		d.tet_count = (uint32)m_tetE.size();
		d.tets = m_tets.data();
		d.tet_rest = m_tetRest.data();
		d.tet_young = m_tetE.data();
		d.tet_poisson = m_tetNu.data();
		d.tet_stiffness_damping = m_tetKd.data();
		d.tet_density = m_tetDensity.data();
		d.tri_count = (uint32)m_triEx.size();
		d.tris = m_tris.data();
		d.tri_rest = m_triRest.data();
		// without any element the triangles are mass fixtures only (no element work on the GPU);
		// mixed bodies give fixture-only entries zero stiffness
		if (std::find(m_triElem.begin(), m_triElem.end(), 1) != m_triElem.end())
		{
			d.tri_young_x = m_triEx.data();
			d.tri_young_y = m_triEy.data();
			d.tri_shear = m_triEs.data();
			d.tri_poisson_xy = m_triNxy.data();
			d.tri_poisson_yx = m_triNyx.data();
			d.tri_stiffness_damping = m_triKd.data();
		}
		d.tri_density = m_triDensity.data();
		d.stretch_count = (uint32)m_stParams.size() / 6;
		d.stretch_tris = m_stTris.data();
		d.stretch_uv = m_stUv.data();
		d.stretch_params = m_stParams.data();
		d.shear_count = (uint32)m_shParams.size() / 2;
		d.shear_tris = m_shTris.data();
		d.shear_uv = m_shUv.data();
		d.shear_params = m_shParams.data();
		d.mouse_count = (uint32)m_msParams.size() / 6;
		d.mouse_ids = m_msIds.data();
		d.mouse_params = m_msParams.data();
		d.spring_count = (uint32)m_sprL0.size();
		d.springs = m_springs.data();
		d.spring_rest_length = m_sprL0.data();
		d.spring_stiffness = m_sprKs.data();
		d.spring_damping = m_sprKd.data();
		std::vector<float> rad, fr;
		if (!m_sphereRadius.empty())
		{
			rad = m_sphereRadius;
			fr = m_sphereFriction;
			rad.resize(m_particles.size(), 0);
			fr.resize(m_particles.size(), 0);
			d.sphere_radius = rad.data();
			d.sphere_friction = fr.data();
		}
		d.world_sphere_count = (uint32)(m_world.size() / 5);
		d.world_spheres = m_world.data();
		// shape arrays point into m_shapeData (kept beside m_shapes, in the same order)
		for (size_t k = 0; k < m_shapes.size(); ++k)
		{
			b3g_world_shape& w = m_shapes[k];
			ShapeData& own = m_shapeData[k];
			if (w.type == B3G_SHAPE_MESH)
			{
				w.vertices = own.f.data();
				w.triangles = own.u.data();
				w.wings = own.u2.data();
			}
			if (w.type == B3G_SHAPE_SDF) w.voxels = own.f.data();
		}
		d.world_shape_count = (uint32)m_shapes.size();
		d.world_shapes = m_shapes.data();
		d.gravity[0] = m_gravity.x;
		d.gravity[1] = m_gravity.y;
		d.gravity[2] = m_gravity.z;
		if (m_body) b3g_body_destroy(m_body);
		m_body = nullptr;
		check(b3g_body_create(m_ctx, &d, &m_body), "b3g_body_create");
		m_mass.assign(m_particles.size(), 0);
		check(b3g_body_get_masses(m_body, m_mass.data()), "b3g_body_get_masses");
		m_topologyDirty = false;
		m_hostFresh = true;
		m_stateDirty = false;
	}

	// pending host-side changes -> device, before a step
	// host-side SetPosition / SetVelocity -> device
	void flush_state()
	{
		if (m_stateDirty)
		{
			std::vector<float> x, v;
			for (size_t i = 0; i < m_x.size(); ++i)
			{
				push3(x, m_x[i]);
				push3(v, m_v[i]);
			}
			check(b3g_body_set_state(m_body, x.data(), v.data()), "b3g_body_set_state");
			m_stateDirty = false;
		}
	}

	void flush_inputs()
	{
		flush_state();
		bool f = false, t = false;
		for (b3Particle* p : m_particles)
		{
			f = f || p->m_force.x != 0 || p->m_force.y != 0 || p->m_force.z != 0;
			t = t || p->m_translation.x != 0 || p->m_translation.y != 0 || p->m_translation.z != 0;
		}
		if (f)
		{
			std::vector<float> a;
			for (b3Particle* p : m_particles) push3(a, p->m_force);
			check(b3g_body_apply_forces(m_body, a.data()), "b3g_body_apply_forces");
		}
		if (t)
		{
			std::vector<float> a;
			for (b3Particle* p : m_particles) push3(a, p->m_translation);
			check(b3g_body_apply_translations(m_body, a.data()), "b3g_body_apply_translations");
		}
	}

	b3g_context* m_ctx = nullptr;
	b3g_body* m_body = nullptr;
	b3g_solver_config m_cfg;
	b3g_step_stats m_stats{};
	bool m_topologyDirty = true, m_hostFresh = true, m_stateDirty = false;
	b3Vec3 m_gravity;
	std::vector<b3Particle*> m_particles;
	std::vector<b3Force*> m_forceHandles;
	std::vector<b3Vec3> m_x, m_v;
	std::vector<float> m_mass;
	std::vector<uint32> m_tets, m_tris, m_springs;
	std::vector<float> m_tetRest, m_tetE, m_tetNu, m_tetKd, m_tetDensity;
	std::vector<float> m_triRest, m_triEx, m_triEy, m_triEs, m_triNxy, m_triNyx, m_triKd, m_triDensity;
	std::vector<uint8_t> m_triElem;                // per triangle entry: has an element force
	std::vector<b3TriangleFixture*> m_triFixture;  // per triangle entry: its fixture or null
	std::vector<float> m_sprL0, m_sprKs, m_sprKd;
	std::vector<uint32> m_stTris, m_shTris, m_msIds;
	std::vector<float> m_stUv, m_stParams, m_shUv, m_shParams, m_msParams;
	std::vector<float> m_sphereRadius, m_sphereFriction, m_world;
	struct ShapeData
	{
		std::vector<float> f;          // mesh vertices or SDF voxels
		std::vector<uint32_t> u, u2;   // mesh triangles and wing vertices
	};
	std::vector<b3g_world_shape> m_shapes;
	std::vector<ShapeData> m_shapeData;
};

inline void b3Particle::SetType(b3ParticleType type)
{
	if (m_type == type) return;
	m_type = type;
	m_force.SetZero();
	m_translation.SetZero();
	b3Body* b = m_body;
	if (!b->m_body)
	{
		if (type == e_staticParticle) b->m_v[m_index].SetZero();
		b->m_topologyDirty = true;
		return;
	}
	b->fetch();
	if (type == e_staticParticle) b->m_v[m_index].SetZero();
	std::vector<int32_t> types;
	for (b3Particle* p : b->m_particles) types.push_back((int32_t)p->m_type);
	b3Body::check(b3g_body_set_types(b->m_body, types.data()), "b3g_body_set_types");
	b3Body::check(b3g_body_get_masses(b->m_body, b->m_mass.data()), "b3g_body_get_masses");
}
inline void b3Particle::SetPosition(const b3Vec3& position)
{
	m_body->fetch();
	m_body->m_x[m_index] = position;
	m_body->m_stateDirty = m_body->m_body != nullptr;
}
inline const b3Vec3& b3Particle::GetPosition() const
{
	m_body->fetch();
	return m_body->m_x[m_index];
}
inline void b3Particle::SetVelocity(const b3Vec3& velocity)
{
	if (m_type == e_staticParticle) return;
	m_body->fetch();
	m_body->m_v[m_index] = velocity;
	m_body->m_stateDirty = m_body->m_body != nullptr;
}
inline const b3Vec3& b3Particle::GetVelocity() const
{
	m_body->fetch();
	return m_body->m_v[m_index];
}
inline scalar b3Particle::GetMass() const { return m_body->mass_of(m_index); }
inline void b3Particle::ApplyForce(const b3Vec3& force)
{
	if (m_type != e_dynamicParticle) return;
	m_force += force;
}
inline void b3Particle::ApplyImpulse(const b3Vec3& impulse)
{
	if (m_type != e_dynamicParticle) return;
	m_body->fetch();
	const scalar m = m_body->mass_of(m_index);
	if (m > 0) m_body->m_v[m_index] += (scalar(1) / m) * impulse;
	m_body->m_stateDirty = m_body->m_body != nullptr;
}
inline void b3Particle::ApplyTranslation(const b3Vec3& translation) { m_translation += translation; }
