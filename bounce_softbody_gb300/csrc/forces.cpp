// Host setup of the Baraff-Witkin cloth forces and mouse springs.
//
// The per-element constants follow the reference's constructors
// (src/bounce_softbody/dynamics/forces/stretch_force.cpp:62-107 and shear_force.cpp:51-92):
// with du1 = u2 - u1, dv1 = v2 - v1, du2 = u3 - u1, dv2 = v3 - v1 and det = du1 dv2 - du2 dv1,
//   dwu/dx = (dv1 - dv2, dv2, -dv1) / det,  dwv/dx = (du2 - du1, -du2, du1) / det,
//   alpha = |det| / 2.
// They are formed in double and stored as floats.
#include "forces.h"

#include <cmath>
#include <cstdio>

namespace b3g {

namespace {

// b3StretchForceDef::Initialize / b3ShearForceDef::Initialize (stretch_force.cpp:36-60,
// shear_force.cpp:25-49): vertex 1 at the origin, vertex 2 on the u axis, vertex 3 above it.
// Returns false for a degenerate triangle.
bool initialize_uv(const float* A, const float* B, const float* C, double uv[6])
{
	double ab[3], ac[3];
	for (int k = 0; k < 3; ++k)
	{
		ab[k] = (double)B[k] - A[k];
		ac[k] = (double)C[k] - A[k];
	}
	const double u2 = std::sqrt(ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2]);
	if (!(u2 > 0.0)) return false;
	const double cr[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
	const double a2 = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
	if (!(a2 > 0.0)) return false;
	uv[0] = 0.0;
	uv[1] = 0.0;
	uv[2] = u2;
	uv[3] = 0.0;
	uv[4] = (ac[0] * ab[0] + ac[1] * ab[1] + ac[2] * ab[2]) / u2;
	uv[5] = a2 / u2;
	return true;
}

// The constructor's constants into rec[0..11]. Returns false when det == 0.
bool uv_record(const double uv[6], float* rec)
{
	const double du1 = uv[2] - uv[0], dv1 = uv[3] - uv[1];
	const double du2 = uv[4] - uv[0], dv2 = uv[5] - uv[1];
	const double det = du1 * dv2 - du2 * dv1;
	if (!(det != 0.0) || !std::isfinite(det)) return false;
	const double inv_det = 1.0 / det;
	const double r[12] = {0.5 * std::fabs(det), inv_det, du1, dv1, du2, dv2,
	                      inv_det * (dv1 - dv2), inv_det * dv2, -inv_det * dv1,
	                      inv_det * (du2 - du1), -inv_det * du2, inv_det * du1};
	for (int k = 0; k < 12; ++k) rec[k] = (float)r[k];
	return true;
}

bool all_finite(const float* p, size_t count)
{
	for (size_t k = 0; k < count; ++k)
		if (!std::isfinite(p[k])) return false;
	return true;
}

} // namespace

int build_cloth_forces(const b3g_body_desc* d, ClothForces& out, char* msg, size_t cap)
{
	out = ClothForces();
	const uint32_t n = d->vertex_count;
	const uint32_t nst = d->stretch_count, nsh = d->shear_count, nm = d->mouse_count;
	if (nst && (!d->stretch_tris || !d->stretch_params))
	{
		std::snprintf(msg, cap, "stretch forces need stretch_tris and stretch_params");
		return 1;
	}
	if (nsh && (!d->shear_tris || !d->shear_params))
	{
		std::snprintf(msg, cap, "shear forces need shear_tris and shear_params");
		return 1;
	}
	if (nm && (!d->mouse_ids || !d->mouse_params))
	{
		std::snprintf(msg, cap, "mouse springs need mouse_ids and mouse_params");
		return 1;
	}
	const uint32_t nbw = nst + nsh;
	out.bw_ids.resize(3 * (size_t)nbw);
	out.bw.resize(nbw);
	out.bw_c.assign((size_t)kBwFloats * nbw, 0.0f);
	for (uint32_t e = 0; e < nbw; ++e)
	{
		const bool shear = e >= nst;
		const uint32_t k = shear ? e - nst : e;
		const char* what = shear ? "shear force" : "stretch force";
		const uint32_t* ids = (shear ? d->shear_tris : d->stretch_tris) + 3 * (size_t)k;
		const float* uvf = shear ? d->shear_uv : d->stretch_uv;
		const float* par = shear ? d->shear_params + 2 * (size_t)k : d->stretch_params + 6 * (size_t)k;
		for (int a = 0; a < 3; ++a)
			if (ids[a] >= n)
			{
				std::snprintf(msg, cap, "%s %u references vertex %u >= vertex_count %u", what, k, ids[a], n);
				return 1;
			}
		double uv[6];
		if (uvf)
		{
			for (int c = 0; c < 6; ++c) uv[c] = uvf[6 * (size_t)k + c];
		}
		else if (!initialize_uv(d->positions + 3 * (size_t)ids[0], d->positions + 3 * (size_t)ids[1],
		                        d->positions + 3 * (size_t)ids[2], uv))
		{
			std::snprintf(msg, cap, "%s %u is degenerate (no (u, v) frame)", what, k);
			return 1;
		}
		float* rec = &out.bw_c[(size_t)kBwFloats * e];
		if (!uv_record(uv, rec))
		{
			std::snprintf(msg, cap, "%s %u has a degenerate (u, v) triangle (det = 0)", what, k);
			return 1;
		}
		const int np = shear ? 2 : 6;
		if (!all_finite(par, np))
		{
			std::snprintf(msg, cap, "%s %u has a non-finite parameter", what, k);
			return 1;
		}
		for (int c = 0; c < np; ++c) rec[12 + c] = par[c];
		for (int a = 0; a < 3; ++a) out.bw_ids[3 * (size_t)e + a] = ids[a];
		out.bw[e] = uint4{ids[0], ids[1], ids[2], shear ? kForceShear : kForceStretch};
	}
	out.ms_ids.assign(d->mouse_ids, d->mouse_ids + 4 * (size_t)nm);
	out.ms.resize(nm);
	out.ms_c.assign(d->mouse_params, d->mouse_params + (size_t)kMouseFloats * nm);
	for (uint32_t e = 0; e < nm; ++e)
	{
		const uint32_t* ids = d->mouse_ids + 4 * (size_t)e;
		for (int a = 0; a < 4; ++a)
			if (ids[a] >= n)
			{
				std::snprintf(msg, cap, "mouse spring %u references vertex %u >= vertex_count %u", e, ids[a], n);
				return 1;
			}
		if (!all_finite(d->mouse_params + (size_t)kMouseFloats * e, kMouseFloats))
		{
			std::snprintf(msg, cap, "mouse spring %u has a non-finite parameter", e);
			return 1;
		}
		out.ms[e] = uint4{ids[0], ids[1], ids[2], ids[3]};
	}
	return 0;
}

} // namespace b3g
