// Drives the implicit step through include/b3g_body.hpp the way a Bounce Softbody program does:
// CreateParticle / CreateForce / CreateTetrahedron / SetGravity / Step. Reads a tetrahedral mesh
// (binary: n, T, positions, types, tets, E, nu, density, damping, steps, dt, tol) from argv[1],
// writes the final positions and velocities (binary floats) to argv[2]. With a third argument
// "shapes" every particle also gets a contact sphere (radius 0.03, friction 0.3) and the body
// collides with a static b3BoxShape floor and a b3CapsuleShape.
#include "b3g_body.hpp"

#include <cstdio>
#include <string>
#include <vector>

int main(int argc, char** argv)
{
	if (argc < 3) return 2;
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
