// The sparse layer of the reference written as a Bounce Softbody program would write it, built
// against include/b3g_sparse.hpp and linked with libb3g.so (tests/test_facade.py runs it).
//
// Input (binary): n, h, then per matrix (dfdx, dfdv) a block count and rows, cols, 9 values per
// block (b3Mat33 order); then f, x, v, fe, y, z, u (3 n floats each), mass (n), dynamic (n
// int32), cg max iterations, cg tolerance. Output (binary floats): A u, pA u, pb, the CG solution,
// the backward-Euler x and v, then iterations (CG, BE Newton, BE max sub) as floats.
#include "b3g_sparse.hpp"

#include <cstdio>
#include <vector>

namespace {

struct Coo
{
	std::vector<uint32_t> rows, cols;
	std::vector<float> vals;
};

template <class T>
void read(FILE* f, T* p, size_t count)
{
	if (std::fread(p, sizeof(T), count, f) != count) throw std::runtime_error("short input");
}

void load(b3SparseMat33& m, const Coo& c)
{
	for (size_t k = 0; k < c.rows.size(); ++k)
	{
		b3Mat33 b;
		std::copy(&c.vals[9 * k], &c.vals[9 * k] + 9, &b.x.x);
		m(c.rows[k], c.cols[k]) += b;
	}
}

// a force model that adds recorded Jacobians and forces, as the reference's models add theirs
struct Replay : public b3SparseForceModel
{
	void ApplyForces(const b3SparseForceSolverData* data) override
	{
		load(*data->dfdx, *dfdx);
		load(*data->dfdv, *dfdv);
		for (uint32 i = 0; i < n; ++i) (*data->f)[i] += (*f)[i];
	}
	const Coo* dfdx;
	const Coo* dfdv;
	const std::vector<b3Vec3>* f;
	uint32 n;
};

void write(FILE* o, const b3DenseVec3& v)
{
	for (uint32 i = 0; i < v.n; ++i)
	{
		const b3Vec3& e = v[i];
		std::fwrite(&e.x, sizeof(float), 3, o);
	}
}

} // namespace

int main(int argc, char** argv)
{
	if (argc < 3) return 2;
	FILE* in = std::fopen(argv[1], "rb");
	if (!in) return 2;
	uint32_t n;
	float h;
	read(in, &n, 1);
	read(in, &h, 1);
	Coo coo[2];
	for (Coo& c : coo)
	{
		uint32_t cnt;
		read(in, &cnt, 1);
		c.rows.resize(cnt);
		c.cols.resize(cnt);
		c.vals.resize(9 * (size_t)cnt);
		read(in, c.rows.data(), cnt);
		read(in, c.cols.data(), cnt);
		read(in, c.vals.data(), c.vals.size());
	}
	std::vector<b3Vec3> hv[7];
	for (auto& a : hv)
	{
		a.resize(n);
		read(in, &a[0].x, 3 * (size_t)n);
	}
	std::vector<float> mass(n);
	std::vector<int32_t> dyn(n);
	read(in, mass.data(), n);
	read(in, dyn.data(), n);
	uint32_t cg_max;
	float cg_tol;
	read(in, &cg_max, 1);
	read(in, &cg_tol, 1);
	std::fclose(in);

	b3DenseVec3 fi(n), x0(n), v0(n), fe(n), y(n), z(n), u(n);
	b3DenseVec3* vs[7] = {&fi, &x0, &v0, &fe, &y, &z, &u};
	for (int k = 0; k < 7; ++k)
		for (uint32 i = 0; i < n; ++i) (*vs[k])[i] = hv[k][i];
	b3DiagMat33 M(n), S(n);
	for (uint32 i = 0; i < n; ++i)
	{
		M[i] = b3Mat33Diagonal(mass[i]);
		S[i] = b3Mat33Diagonal(dyn[i] ? scalar(1) : scalar(0));
	}
	b3SparseMat33 dfdx(n), dfdv(n);
	load(dfdx, coo[0]);
	load(dfdv, coo[1]);
	const b3DenseVec3& x = x0;
	const b3DenseVec3& v = v0;

	// sparse_force_solver.cpp:142-174, written the same way
	b3DiagMat33 ST(n);
	b3Transpose(ST, S);
	b3DiagMat33 I(n);
	I.SetIdentity();
	b3SparseMat33 A = M - h * dfdv - (h * h) * dfdx;
	b3DenseVec3 b = M * (v0 - v) + h * (fe + fi) + h * dfdx * (x0 - x + h * v + y);
	b3SparseMat33 pA = S * A * ST + I - S;
	b3DenseVec3 pb = S * (b - A * z);

	FILE* o = std::fopen(argv[2], "wb");
	if (!o) return 2;
	write(o, A * u);
	write(o, pA * u);
	write(o, pb);

	b3DenseVec3 xcg(n);
	xcg.SetZero();
	b3SolveCGInput ci;
	ci.A = &pA;
	ci.b = &pb;
	ci.maxIterations = cg_max;
	ci.tolerance = cg_tol;
	b3SolveCGOutput co;
	co.x = &xcg;
	b3SparseSolveCG(&co, &ci);
	write(o, xcg);

	Replay model;
	model.dfdx = &coo[0];
	model.dfdv = &coo[1];
	model.f = &hv[0];
	model.n = n;
	b3DenseVec3 xb(n), vb(n);
	b3SolveBEInput bi;
	bi.h = h;
	bi.inv_h = 1.0f / h;
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
	bi.maxSubIterations = cg_max;
	bi.subTolerance = cg_tol;
	b3SolveBEOutput bo;
	bo.x = &xb;
	bo.v = &vb;
	bo.minSubIterations = 0xFFFFFFFFu;
	bo.maxSubIterations = 0;
	b3SparseSolveBE(&bo, &bi);
	write(o, xb);
	write(o, vb);
	const float its[3] = {(float)co.iterations, (float)bo.iterations, (float)bo.maxSubIterations};
	std::fwrite(its, sizeof(float), 3, o);
	std::fclose(o);
	std::printf("cg %u iterations, be %u / %u\n", co.iterations, bo.iterations, bo.maxSubIterations);
	return 0;
}
