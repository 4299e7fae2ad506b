// Drives the implicit step through include/b3g_body.hpp the way a Bounce Softbody program does:
// CreateParticle / CreateForce / CreateTetrahedron / SetGravity / Step. Reads a tetrahedral mesh
// (binary: n, T, positions, types, tets, E, nu, density, damping, steps, dt, tol) from argv[1],
// writes the final positions and velocities (binary floats) to argv[2]. With a third argument
// "shapes" every particle also gets a contact sphere (radius 0.03, friction 0.3) and the body
// collides with a static b3BoxShape floor and a b3CapsuleShape ("shapes filter": the same with
// filtered contacts, SetContactMode); with "cloth" it runs the Baraff-Witkin cloth scene below
// instead (argv[1] is not read).
#include "b3g_body.hpp"

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

// The reference testbed's pinned cloth (examples/testbed/tests/pinned_cloth.h with
// UniformBody's ClothDef, createElements = false): an m x m grid of triangle fixtures of density
// 0.2 held by one b3StretchForce each (stiffness 1e5), border pinned, plus one b3ShearForce per
// triangle. A BodyDragger-style b3MouseForce pulls the centre towards a static particle for
// `drag` steps, is destroyed, and the cloth runs `steps - drag` steps more; then a vertical ray
// picks the cloth (b3Body::RayCastSingle). Output: positions, velocities, then hit flag, triangle
// index, fraction and normal.
static int cloth(const char* out_path, uint32 m, uint32 steps, uint32 drag, float dt, float tol)
{
	b3Body body;
	body.SetGravity(b3Vec3(0, -9.8f, 0));
	const float side = 2.0f, h = side / (m - 1);
	std::vector<b3Particle*> ps;
	for (uint32 j = 0; j < m; ++j)
		for (uint32 i = 0; i < m; ++i)
		{
			b3ParticleDef pd;
			pd.type = (i == 0 || j == 0 || i == m - 1 || j == m - 1) ? e_staticParticle : e_dynamicParticle;
			pd.position.Set(-0.5f * side + i * h, 1.0f, -0.5f * side + j * h);
			ps.push_back(body.CreateParticle(pd));
		}
	// cells in the order of meshes.bw_cloth (cell column i outer), lower triangles first
	std::vector<uint32> tris;
	for (int upper = 0; upper < 2; ++upper)
		for (uint32 i = 0; i + 1 < m; ++i)
			for (uint32 j = 0; j + 1 < m; ++j)
			{
				uint32 v00 = i + m * j, v10 = v00 + 1, v01 = v00 + m, v11 = v01 + 1;
				if (upper) tris.insert(tris.end(), {v10, v01, v11});
				else tris.insert(tris.end(), {v00, v01, v10});
			}
	const uint32 T = (uint32)tris.size() / 3;
	std::vector<b3TriangleFixture*> fixtures;
	for (uint32 e = 0; e < T; ++e)
	{
		b3Particle *p1 = ps[tris[3 * e]], *p2 = ps[tris[3 * e + 1]], *p3 = ps[tris[3 * e + 2]];
		b3TriangleFixtureDef td;
		td.p1 = p1; td.p2 = p2; td.p3 = p3;
		td.v1 = p1->GetPosition(); td.v2 = p2->GetPosition(); td.v3 = p3->GetPosition();
		td.density = 0.2f;
		fixtures.push_back(body.CreateTriangle(td));
		b3StretchForceDef sd;
		sd.Initialize(td.v1, td.v2, td.v3);
		sd.p1 = p1; sd.p2 = p2; sd.p3 = p3;
		sd.stiffness_u = sd.stiffness_v = 1e5f;
		body.CreateForce(sd);
		b3ShearForceDef hd;
		hd.Initialize(td.v1, td.v2, td.v3);
		hd.p1 = p1; hd.p2 = p2; hd.p3 = p3;
		hd.stiffness = 1e3f;
		hd.dampingStiffness = 10.0f;
		body.CreateForce(hd);
	}
	// BodyDragger::StartDragging (examples/testbed/framework/body_dragger.cpp): a static particle
	// at the picked point, tied to the triangle's barycentre
	const uint32 t = T / 2 + (m - 1) / 2;
	b3Particle *q1 = ps[tris[3 * t]], *q2 = ps[tris[3 * t + 1]], *q3 = ps[tris[3 * t + 2]];
	b3Vec3 c = (1.0f / 3.0f) * (q1->GetPosition() + q2->GetPosition() + q3->GetPosition());
	b3ParticleDef md;
	md.type = e_staticParticle;
	md.position = c + b3Vec3(0.0f, -0.3f, 0.0f);
	ps.push_back(body.CreateParticle(md));
	b3MouseForceDef mf;
	mf.p1 = ps.back(); mf.p2 = q1; mf.p3 = q2; mf.p4 = q3;
	mf.w2 = 1.0f / 3.0f; mf.w3 = 1.0f / 3.0f; mf.w4 = 1.0f - 2.0f / 3.0f;
	mf.stiffness = 1e5f;
	mf.dampingStiffness = 1e3f;
	mf.length = 0.0f;
	b3Force* mouse = body.CreateForce(mf);
	body.SetSolverTolerance(tol);
	for (uint32 s = 0; s < steps; ++s)
	{
		if (s == drag) body.DestroyForce(mouse);  // BodyDragger::StopDragging
		body.Step(dt, 1, 200);
	}
	// picking as BodyDragger::StartDragging does it: a ray from above through the cloth's centre
	b3BodyRayCastSingleOutput hit;
	float pick[6] = {0, 0, 0, 0, 0, 0};
	if (body.RayCastSingle(&hit, b3Vec3(0.05f, 3.0f, 0.03f), b3Vec3(0.05f, -3.0f, 0.03f)))
	{
		pick[0] = 1.0f;
		pick[1] = (float)(std::find(fixtures.begin(), fixtures.end(), hit.triangle) - fixtures.begin());
		pick[2] = hit.fraction;
		pick[3] = hit.normal.x;
		pick[4] = hit.normal.y;
		pick[5] = hit.normal.z;
	}
	FILE* o = std::fopen(out_path, "wb");
	if (!o) return 6;
	for (int pass = 0; pass < 2; ++pass)
		for (b3Particle* p : ps)
		{
			const b3Vec3& w = pass == 0 ? p->GetPosition() : p->GetVelocity();
			float xyz[3] = {w.x, w.y, w.z};
			std::fwrite(xyz, 4, 3, o);
		}
	std::fwrite(pick, 4, 6, o);
	std::fclose(o);
	std::printf("cloth steps=%u pcg=%u\n", steps, body.GetStepStats().pcg_iterations);
	return 0;
}

int main(int argc, char** argv)
{
	if (argc < 3) return 2;
	if (argc > 3 && std::string(argv[3]) == "cloth") return cloth(argv[2], 10, 12, 6, 1.0f / 60.0f, 1e-5f);
	FILE* f = std::fopen(argv[1], "rb");
	if (!f) return 3;
	uint32 n = 0, T = 0, steps = 0;
	float E = 0, nu = 0, density = 0, damping = 0, dt = 0, tol = 0;
	if (std::fread(&n, 4, 1, f) != 1 || std::fread(&T, 4, 1, f) != 1) return 4;
	std::vector<float> x(3 * n);
	std::vector<int32_t> type(n);
	std::vector<uint32> tets(4 * T);
	size_t ok = std::fread(x.data(), 4, x.size(), f) + std::fread(type.data(), 4, n, f) + std::fread(tets.data(), 4, tets.size(), f);
	ok += std::fread(&E, 4, 1, f) + std::fread(&nu, 4, 1, f) + std::fread(&density, 4, 1, f) + std::fread(&damping, 4, 1, f);
	ok += std::fread(&steps, 4, 1, f) + std::fread(&dt, 4, 1, f) + std::fread(&tol, 4, 1, f);
	std::fclose(f);
	if (ok != x.size() + n + tets.size() + 7) return 5;

	b3Body body;
	body.SetGravity(b3Vec3(0, -9.8f, 0));
	std::vector<b3Particle*> ps(n);
	for (uint32 i = 0; i < n; ++i)
	{
		b3ParticleDef pd;
		pd.type = (b3ParticleType)type[i];
		pd.position.Set(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
		pd.damping = damping;
		ps[i] = body.CreateParticle(pd);
	}
	for (uint32 e = 0; e < T; ++e)
	{
		b3Particle* q[4] = {ps[tets[4 * e]], ps[tets[4 * e + 1]], ps[tets[4 * e + 2]], ps[tets[4 * e + 3]]};
		b3TetrahedronElementForceDef fd;
		fd.p1 = q[0]; fd.p2 = q[1]; fd.p3 = q[2]; fd.p4 = q[3];
		fd.v1 = q[0]->GetPosition(); fd.v2 = q[1]->GetPosition(); fd.v3 = q[2]->GetPosition(); fd.v4 = q[3]->GetPosition();
		fd.youngModulus = E;
		fd.poissonRatio = nu;
		body.CreateForce(fd);
		b3TetrahedronFixtureDef td;
		td.p1 = q[0]; td.p2 = q[1]; td.p3 = q[2]; td.p4 = q[3];
		td.v1 = fd.v1; td.v2 = fd.v2; td.v3 = fd.v3; td.v4 = fd.v4;
		td.density = density;
		body.CreateTetrahedron(td);
	}
	if (argc > 3 && std::string(argv[3]) == "shapes")
	{
		for (uint32 i = 0; i < n; ++i)
		{
			b3SphereFixtureDef sd;
			sd.p = ps[i];
			sd.radius = 0.03f;
			sd.friction = 0.3f;
			body.CreateSphere(sd);
		}
		b3BoxShape floor;
		floor.m_extents = b3Vec3(1.0f, 0.05f, 1.0f);
		floor.m_xf.translation = b3Vec3(0.2f, -0.07f, 0.2f);
		floor.m_xf.rotation = b3Quat(b3Vec3(0.0f, 0.0f, 0.0499792f), 0.9987503f);
		b3WorldFixtureDef fd;
		fd.shape = &floor;
		fd.friction = 0.5f;
		body.CreateFixture(fd);
		b3CapsuleShape pole;
		pole.m_center1 = b3Vec3(0.6f, 0.0f, -0.1f);
		pole.m_center2 = b3Vec3(0.6f, 0.0f, 0.8f);
		pole.m_radius = 0.12f;
		fd.shape = &pole;
		fd.friction = 0.2f;
		body.CreateFixture(fd);
		if (argc > 4 && std::string(argv[4]) == "filter") body.SetContactMode(B3G_CONTACT_FILTER);
	}
	body.SetSolverTolerance(tol);
	for (uint32 s = 0; s < steps; ++s) body.Step(dt, 1, 200);
	FILE* o = std::fopen(argv[2], "wb");
	if (!o) return 6;
	for (uint32 i = 0; i < n; ++i)
	{
		const b3Vec3& p = ps[i]->GetPosition();
		float xyz[3] = {p.x, p.y, p.z};
		std::fwrite(xyz, 4, 3, o);
	}
	for (uint32 i = 0; i < n; ++i)
	{
		const b3Vec3& v = ps[i]->GetVelocity();
		float xyz[3] = {v.x, v.y, v.z};
		std::fwrite(xyz, 4, 3, o);
	}
	std::fclose(o);
	std::printf("steps=%u pcg=%u energy=%g\n", steps, body.GetStepStats().pcg_iterations, (double)body.GetEnergy());
	return 0;
}
