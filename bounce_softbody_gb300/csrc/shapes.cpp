// Host setup of a body's static world shapes (b3WorldFixture + b3Shape): validation, the
// fixture AABBs exactly as the reference computes them (they decide contact creation and
// persistence), mesh triangles transformed to world space with their wing vertices, and SDF
// voxels. The device side (collide routines) is in device.cuh.
#include "shapes.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace b3g {

namespace {

struct V3
{
	float x, y, z;
};
V3 v3(const float* p) { return V3{p[0], p[1], p[2]}; }
V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 scl(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
V3 vmin(V3 a, V3 b) { return V3{std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
V3 vmax(V3 a, V3 b) { return V3{std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// quat.h:75-79 b3Quat::Rotate
V3 qrot(const float q[4], V3 v)
{
	const V3 u{q[0], q[1], q[2]};
	const V3 t = scl(2.0f, cross(u, v));
	return add(add(v, scl(q[3], t)), cross(u, t));
}
// transform.h b3Mul(xf, v)
V3 xform(const float q[4], const float t[3], V3 v) { return add(qrot(q, v), v3(t)); }

void put(float* dst, V3 v)
{
	dst[0] = v.x;
	dst[1] = v.y;
	dst[2] = v.z;
}

struct Box
{
	V3 lo, hi;
};
void extend(Box& b, float r)
{
	b.lo = sub(b.lo, V3{r, r, r});
	b.hi = add(b.hi, V3{r, r, r});
}

// aabb.h:321-336 b3AABB::Transform: the center transformed, the half extents dotted with the
// columns of |R| (R = quat.h:133-146 GetRotationMatrix)
Box transform_box(Box b, const float q[4], const float t[3])
{
	const V3 lc = scl(0.5f, add(b.lo, b.hi));
	const V3 lr = scl(0.5f, sub(b.hi, b.lo));
	const V3 c = xform(q, t, lc);
	const float x = q[0], y = q[1], z = q[2], w = q[3];
	const float x2 = x + x, y2 = y + y, z2 = z + z;
	const float xx = x * x2, xy = x * y2, xz = x * z2;
	const float yy = y * y2, yz = y * z2, zz = z * z2;
	const float wx = w * x2, wy = w * y2, wz = w * z2;
	const V3 cx{std::fabs(1.0f - (yy + zz)), std::fabs(xy + wz), std::fabs(xz - wy)};
	const V3 cy{std::fabs(xy - wz), std::fabs(1.0f - (xx + zz)), std::fabs(yz + wx)};
	const V3 cz{std::fabs(xz + wy), std::fabs(yz - wx), std::fabs(1.0f - (xx + yy))};
	const V3 r{dot(lr, cx), dot(lr, cy), dot(lr, cz)};
	return Box{sub(c, r), add(c, r)};
}

constexpr float kLinearSlop = 0.005f;  // settings.h:70 B3_LINEAR_SLOP
constexpr uint32_t kNullVertex = 0xFFFFFFFFu;
constexpr uint32_t kMaxMeshTriangles = 1u << 20;

int bad(char* msg, size_t cap, const char* text, uint32_t k)
{
	std::snprintf(msg, cap, "world shape %u: %s", k, text);
	return 1;
}

} // namespace

int build_shapes(const b3g_body_desc* d, std::vector<DevShape>& shapes, std::vector<float>& data, char* msg,
                 size_t cap)
{
	shapes.clear();
	data.clear();
	const uint32_t total = d->world_sphere_count + d->world_shape_count;
	if (total > (uint32_t)kMaxWorld)
	{
		std::snprintf(msg, cap, "at most %d world fixtures (spheres and shapes), got %u", kMaxWorld, total);
		return 1;
	}
	if (d->world_sphere_count && !d->world_spheres)
	{
		std::snprintf(msg, cap, "world_spheres is null");
		return 1;
	}
	if (d->world_shape_count && !d->world_shapes)
	{
		std::snprintf(msg, cap, "world_shapes is null");
		return 1;
	}
	// sphere_shape.cpp:42-48 ComputeAABB
	for (uint32_t k = 0; k < d->world_sphere_count; ++k)
	{
		const float* w = d->world_spheres + 5 * k;
		DevShape S{};
		S.type = B3G_SHAPE_SPHERE;
		S.radius = w[3];
		S.friction = w[4];
		std::memcpy(S.a, w, 3 * sizeof(float));
		const V3 c = v3(w), r{w[3], w[3], w[3]};
		put(S.lo, sub(c, r));
		put(S.hi, add(c, r));
		S.q[3] = 1.0f;
		shapes.push_back(S);
	}
	std::vector<size_t> data_at(d->world_shape_count, 0);
	for (uint32_t k = 0; k < d->world_shape_count; ++k)
	{
		const b3g_world_shape& W = d->world_shapes[k];
		const uint32_t id = d->world_sphere_count + k;
		DevShape S{};
		S.type = W.type;
		S.radius = W.radius;
		S.friction = W.friction;
		std::memcpy(S.q, W.rotation, 4 * sizeof(float));
		std::memcpy(S.t, W.translation, 3 * sizeof(float));
		if (!(W.radius >= 0.0f)) return bad(msg, cap, "radius must be >= 0", id);
		Box box{};
		switch (W.type)
		{
		case B3G_SHAPE_SPHERE:
		{
			// sphere_shape.cpp:42-48
			std::memcpy(S.a, W.p, 3 * sizeof(float));
			const V3 c = v3(W.p), r{W.radius, W.radius, W.radius};
			box = Box{sub(c, r), add(c, r)};
			break;
		}
		case B3G_SHAPE_CAPSULE:
		{
			// capsule_shape.cpp:40-50
			std::memcpy(S.a, W.p, 3 * sizeof(float));
			std::memcpy(S.b, W.p + 3, 3 * sizeof(float));
			const V3 r{W.radius, W.radius, W.radius};
			box = Box{sub(vmin(v3(W.p), v3(W.p + 3)), r), add(vmax(v3(W.p), v3(W.p + 3)), r)};
			break;
		}
		case B3G_SHAPE_BOX:
		{
			// box_shape.cpp:40-61: the 8 corners transformed, extended by the radius
			std::memcpy(S.a, W.p, 3 * sizeof(float));
			const V3 e = v3(W.p);
			if (!(e.x >= 0.0f && e.y >= 0.0f && e.z >= 0.0f)) return bad(msg, cap, "box extents must be >= 0", id);
			const V3 corners[8] = {{-e.x, -e.y, -e.z}, {-e.x, -e.y, e.z}, {-e.x, e.y, -e.z}, {-e.x, e.y, e.z},
			                       {e.x, -e.y, -e.z},  {e.x, -e.y, e.z},  {e.x, e.y, -e.z},  {e.x, e.y, e.z}};
			box.lo = box.hi = xform(W.rotation, W.translation, corners[0]);
			for (int c = 1; c < 8; ++c)
			{
				const V3 v = xform(W.rotation, W.translation, corners[c]);
				box.lo = vmin(box.lo, v);
				box.hi = vmax(box.hi, v);
			}
			extend(box, W.radius);
			break;
		}
		case B3G_SHAPE_TRIANGLE:
		{
			// triangle_shape.cpp:51-63
			std::memcpy(S.a, W.p, 3 * sizeof(float));
			std::memcpy(S.b, W.p + 3, 3 * sizeof(float));
			std::memcpy(S.c, W.p + 6, 3 * sizeof(float));
			const V3 A = v3(W.p), B = v3(W.p + 3), C = v3(W.p + 6), r{W.radius, W.radius, W.radius};
			box = Box{sub(vmin(A, vmin(B, C)), r), add(vmax(A, vmax(B, C)), r)};
			break;
		}
		case B3G_SHAPE_MESH:
		{
			if (!W.vertices || !W.triangles || W.vertex_count == 0 || W.triangle_count == 0)
				return bad(msg, cap, "a mesh needs vertices and triangles", id);
			if (W.triangle_count > kMaxMeshTriangles) return bad(msg, cap, "a mesh has at most 1,048,576 triangles", id);
			if (W.scale[0] == 0.0f || W.scale[1] == 0.0f || W.scale[2] == 0.0f)
				return bad(msg, cap, "mesh scale components must be nonzero", id);
			for (uint32_t t = 0; t < 3 * W.triangle_count; ++t)
				if (W.triangles[t] >= W.vertex_count) return bad(msg, cap, "mesh triangle vertex out of range", id);
			if (W.wings)
				for (uint32_t t = 0; t < 3 * W.triangle_count; ++t)
					if (W.wings[t] != kNullVertex && W.wings[t] >= W.vertex_count)
						return bad(msg, cap, "mesh wing vertex out of range", id);
			for (int c = 0; c < 3; ++c) S.inv_scale[c] = 1.0f / W.scale[c];
			S.count = (int)W.triangle_count;
			// mesh_shape.cpp:129-162 GetChildTriangle: b3Mul(xf, b3Mul(scale, v))
			auto world = [&](uint32_t v) {
				const V3 p = v3(W.vertices + 3 * v);
				return xform(W.rotation, W.translation, V3{W.scale[0] * p.x, W.scale[1] * p.y, W.scale[2] * p.z});
			};
			data_at[k] = data.size();
			for (uint32_t t = 0; t < W.triangle_count; ++t)
			{
				float rec[kMeshTriFloats] = {};
				const uint32_t* tv = W.triangles + 3 * t;
				for (int c = 0; c < 3; ++c) put(rec + 3 * c, world(tv[c]));
				for (int c = 0; c < 3; ++c)
				{
					const uint32_t u = W.wings ? W.wings[3 * t + c] : kNullVertex;
					if (u != kNullVertex)
					{
						put(rec + 9 + 3 * c, world(u));
						rec[18 + c] = 1.0f;
					}
				}
				// mesh.h:102-117 GetTriangleAABB (mesh frame, unscaled), extended by the slop
				const V3 A = v3(W.vertices + 3 * tv[0]), B = v3(W.vertices + 3 * tv[1]), C = v3(W.vertices + 3 * tv[2]);
				Box tb{vmin(A, vmin(B, C)), vmax(A, vmax(B, C))};
				extend(tb, kLinearSlop);
				put(rec + 21, tb.lo);
				put(rec + 24, tb.hi);
				data.insert(data.end(), rec, rec + kMeshTriFloats);
			}
			// mesh_shape.cpp:46-52 ComputeAABB: every vertex scaled and transformed, extended
			box.lo = box.hi = world(0);
			for (uint32_t v = 1; v < W.vertex_count; ++v)
			{
				const V3 p = world(v);
				box.lo = vmin(box.lo, p);
				box.hi = vmax(box.hi, p);
			}
			extend(box, W.radius);
			break;
		}
		case B3G_SHAPE_SDF:
		{
			if (!W.voxels || W.grid[0] < 2 || W.grid[1] < 2 || W.grid[2] < 2)
				return bad(msg, cap, "an SDF needs voxels and at least 2 voxels along each axis", id);
			if (!(W.grid_upper[0] > W.grid_lower[0] && W.grid_upper[1] > W.grid_lower[1] && W.grid_upper[2] > W.grid_lower[2]))
				return bad(msg, cap, "the SDF grid AABB is empty", id);
			const size_t nv = (size_t)W.grid[0] * W.grid[1] * W.grid[2];
			if (nv > (size_t)1 << 28) return bad(msg, cap, "the SDF grid is too large", id);
			for (int c = 0; c < 3; ++c)
			{
				S.dims[c] = (int)W.grid[c];
				S.glo[c] = W.grid_lower[c];
				S.ghi[c] = W.grid_upper[c];
			}
			S.invert = W.invert ? 1 : 0;
			data_at[k] = data.size();
			data.insert(data.end(), W.voxels, W.voxels + nv);
			// sdf_shape.cpp:40-46: the grid AABB transformed (aabb.h:321-336), extended
			box = transform_box(Box{v3(W.grid_lower), v3(W.grid_upper)}, W.rotation, W.translation);
			extend(box, W.radius);
			break;
		}
		default: return bad(msg, cap, "unknown shape type", id);
		}
		put(S.lo, box.lo);
		put(S.hi, box.hi);
		shapes.push_back(S);
	}
	// data offsets, resolved to device pointers by bind_shape_data
	for (uint32_t k = 0; k < d->world_shape_count; ++k)
		shapes[d->world_sphere_count + k].data = (const float*)(uintptr_t)data_at[k];
	return 0;
}

void bind_shape_data(std::vector<DevShape>& shapes, const float* device_data)
{
	for (DevShape& S : shapes)
		if (S.type == B3G_SHAPE_MESH || S.type == B3G_SHAPE_SDF) S.data = device_data + (uintptr_t)S.data;
		else S.data = nullptr;
}

} // namespace b3g
