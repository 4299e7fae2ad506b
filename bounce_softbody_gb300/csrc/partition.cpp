// Host-only helpers for placing independent bodies on several GPUs: a body's device footprint
// estimated from its description, and a split of a body list over GPUs by those footprints.
// Bodies never interact (b3Body::Step touches one body only, src/bounce_softbody/dynamics/
// body.cpp:552-604), so a split needs no exchange between GPUs. Nothing here touches a GPU.
#include "api_internal.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace b3g {

// Device bytes of a body made from d, from its counts and the layout of the body's arena and
// FP32 solver vectors (api.cu): about 15 matrix blocks per vertex for tetrahedral meshes and 11
// for cloth with bending springs, a quarter more for the padding of the sliced layout and the
// interleaved contribution lists. Meant to be slightly high; once a body has been created
// b3g_body_device_bytes gives its exact size.
uint64_t estimate_desc_bytes(const b3g_body_desc& d)
{
	const double n = d.vertex_count, nt = d.tet_count, ntr = d.tri_count, ns = d.spring_count;
	const double nw = (double)d.world_sphere_count + d.world_shape_count;
	const double nbw = (double)d.stretch_count + d.shear_count, nms = d.mouse_count;
	const double npad = 32.0 * std::ceil(n / 32.0);
	const double nnzb = (d.tet_count ? 15.0 * n : (d.tri_count || d.spring_count || nbw ? 11.0 * n : n)) + 16 * nms;
	const double slots = 1.25 * nnzb + 128.0;
	double b = slots * (4 + 36 + 4 + 2 + 4 + 2);                                       // col, blocks, list heads
	b += 1.4 * 4.0 * (16 * nt + 9 * ntr + 4 * ns + 4 * nt + 3 * ntr + 2 * ns);          // contribution lists
	b += npad * (1 + 6 + 6) + n * (6 * 12 + 13 + 12);                                   // row lists, vertex state
	b += nt * (16 + 36 + 16 + 16 + 64 + 48) + ntr * (16 + 24 + 16 + 144 + 4) + ns * 20;  // elements
	b += 36 * (9 * ntr + ns) + 12 * (3 * ntr + ns);                                     // explicit blocks
	b += nbw * (16 + 4 * kBwFloats + 36 * 9 + 12 * 3 + 1.4 * 4 * 12) +                  // cloth forces
	     nms * (16 + 4 * kMouseFloats + 36 * 16 + 12 * 4 + 1.4 * 4 * 20);
	b += nw * n * 18 + (nw ? 8 * n : 0);                                                // contacts
	b += 160 * npad;                                                                    // FP32 solver vectors
	for (uint32_t k = 0; k < d.world_shape_count && d.world_shapes; ++k)                // mesh triangles, voxels
	{
		const b3g_world_shape& w = d.world_shapes[k];
		b += 4.0 * kMeshTriFloats * w.triangle_count + 4.0 * w.grid[0] * w.grid[1] * w.grid[2];
	}
	return (uint64_t)(1.15 * b) + (64u << 10);
}

} // namespace b3g

using namespace b3g;

extern "C" int b3g_body_desc_estimate_bytes(const b3g_body_desc* desc, uint64_t* bytes)
{
	if (!desc || !bytes) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	*bytes = estimate_desc_bytes(*desc);
	return B3G_OK;
}

extern "C" int b3g_partition_bodies(const uint64_t* bytes, uint32_t count, uint32_t ranks, uint32_t* rank_of)
{
	if ((!bytes || !rank_of) && count) return fail(B3G_ERROR_INVALID_ARGUMENT, "null argument");
	if (ranks == 0) return fail(B3G_ERROR_INVALID_ARGUMENT, "ranks must be at least 1");
	// largest first (ties: lower index first), each to the GPU with the fewest bytes so far
	// (ties: lowest rank): the greedy longest-processing-time rule, deterministic
	std::vector<uint32_t> order(count);
	std::iota(order.begin(), order.end(), 0u);
	std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return bytes[a] > bytes[b]; });
	std::vector<uint64_t> load(ranks, 0);
	for (uint32_t k : order)
	{
		uint32_t best = 0;
		for (uint32_t r = 1; r < ranks; ++r)
			if (load[r] < load[best]) best = r;
		rank_of[k] = best;
		load[best] += bytes[k];
	}
	return B3G_OK;
}
