// Host setup of the Baraff-Witkin stretch and shear triangles and of mouse springs (forces.cpp).
#pragma once

#include "internal.h"

#include <vector>

namespace b3g {

struct ClothForces
{
	std::vector<uint32_t> bw_ids;   // 3 per stretch/shear triangle: stretch first, then shear
	std::vector<uint4> bw;          // the same ids with the kind in w
	std::vector<float> bw_c;        // kBwFloats per triangle
	std::vector<uint32_t> ms_ids;   // 4 per mouse spring
	std::vector<uint4> ms;
	std::vector<float> ms_c;        // kMouseFloats per mouse spring
};

// Validates the desc's stretch, shear and mouse arrays and computes the element records: the
// (u, v) frame of b3StretchForceDef::Initialize when no coordinates are given, then the
// constants of the b3StretchForce / b3ShearForce constructors. Returns nonzero with a message
// on invalid input (a degenerate (u, v) triangle, a missing array, a vertex id out of range).
int build_cloth_forces(const b3g_body_desc* d, ClothForces& out, char* msg, size_t cap);

} // namespace b3g
