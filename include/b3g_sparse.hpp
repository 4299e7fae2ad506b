// b3g_sparse.hpp — the reference's sparse value types and solvers over include/b3g_sparse.h
// (header-only C++ façade).
//
// A program written against Bounce Softbody's sparse layer
// (include/bounce_softbody/sparse/{dense_vec3,diag_mat33,sparse_mat33,sparse_solver,
// sparse_force_solver}.h) builds against this header and links libb3g.so: the same type names
// (b3DenseVec3, b3DiagMat33, b3SparseMat33, b3SolveCGInput / Output, b3SolveBEInput / Output,
// b3SparseForceModel, b3SparseForceSolverData), the same free functions and operators (b3Add,
// b3Sub, b3Mul, b3Negate, b3Transpose, b3Dot, b3LengthSquared, b3Length, +, -, *) and the same
// solver calls (b3SparseSolveCG, b3SparseSolveBE). The values live on the GPU and every
// operator runs there; element access (operator[] and operator()(i, j)) works on a host copy
// that is fetched on first access and sent back before the next device operation, so a force
// model can keep writing "(*data->dfdx)(i, j) += K" and "(*data->f)[i] += g".
//
// Containers are made on one context per process (device 0 unless b3SetSparseContext names
// another before the first container). Not thread-safe, like the reference.
#pragma once

#include "b3g_body.hpp"
#include "b3g_sparse.h"

#include <map>
#include <utility>

#ifndef B3G_HAVE_MAT33
#define B3G_HAVE_MAT33
// b3Mat33 (include/bounce_softbody/common/math/mat33.h:25): column-major, columns x, y, z.
struct b3Mat33
{
	b3Mat33() {}
	b3Mat33(const b3Vec3& _x, const b3Vec3& _y, const b3Vec3& _z) : x(_x), y(_y), z(_z) {}
	void SetZero() { x.SetZero(); y.SetZero(); z.SetZero(); }
	void SetIdentity() { x.Set(1, 0, 0); y.Set(0, 1, 0); z.Set(0, 0, 1); }
	scalar operator()(uint32 i, uint32 j) const { return (&(&x)[j].x)[i]; }
	scalar& operator()(uint32 i, uint32 j) { return (&(&x)[j].x)[i]; }
	b3Mat33& operator+=(const b3Mat33& b) { x += b.x; y += b.y; z += b.z; return *this; }
	b3Mat33& operator-=(const b3Mat33& b) { x = x - b.x; y = y - b.y; z = z - b.z; return *this; }
	b3Vec3 x, y, z;
};
inline b3Mat33 operator+(const b3Mat33& a, const b3Mat33& b) { return b3Mat33(a.x + b.x, a.y + b.y, a.z + b.z); }
inline b3Mat33 operator-(const b3Mat33& a, const b3Mat33& b) { return b3Mat33(a.x - b.x, a.y - b.y, a.z - b.z); }
inline b3Mat33 operator*(scalar s, const b3Mat33& a) { return b3Mat33(s * a.x, s * a.y, s * a.z); }
inline b3Vec3 operator*(const b3Mat33& a, const b3Vec3& v) { return v.x * a.x + v.y * a.y + v.z * a.z; }
inline b3Mat33 operator*(const b3Mat33& a, const b3Mat33& b) { return b3Mat33(a * b.x, a * b.y, a * b.z); }
inline b3Mat33 b3Mat33Diagonal(scalar s) { return b3Mat33(b3Vec3(s, 0, 0), b3Vec3(0, s, 0), b3Vec3(0, 0, s)); }
inline b3Mat33 b3Mat33Diagonal(scalar a, scalar b, scalar c)
{
	return b3Mat33(b3Vec3(a, 0, 0), b3Vec3(0, b, 0), b3Vec3(0, 0, c));
}
#endif

namespace b3g_sparse_detail {

inline b3g_context*& context_slot()
{
	static b3g_context* ctx = nullptr;
	return ctx;
}

inline b3g_context* context()
{
	b3g_context*& c = context_slot();
	if (!c && b3g_context_create(0, &c) != B3G_OK) throw std::runtime_error(b3g_last_error());
	return c;
}

inline void check(int rc)
{
	if (rc != B3G_OK) throw std::runtime_error(b3g_last_error());
}

} // namespace b3g_sparse_detail

// The context the sparse containers are made on (before the first container).
inline void b3SetSparseContext(b3g_context* ctx) { b3g_sparse_detail::context_slot() = ctx; }

// ---------------------------------------------------------------- b3DenseVec3 (dense_vec3.h:24)
struct b3DenseVec3
{
	explicit b3DenseVec3(uint32 _n = 0) : n(_n) { b3g_sparse_detail::check(b3g_dense_vec3_create(b3g_sparse_detail::context(), n, &h)); }
	b3DenseVec3(const b3DenseVec3& v) : b3DenseVec3(v.n) { Copy(v); }
	b3DenseVec3(b3DenseVec3&& v) noexcept
	    : n(v.n), h(v.h), own(v.own), host(std::move(v.host)), host_valid(v.host_valid), host_dirty(v.host_dirty)
	{
		v.h = nullptr;
	}
	~b3DenseVec3()
	{
		if (h && own) b3g_dense_vec3_destroy(h);
	}
	b3DenseVec3& operator=(const b3DenseVec3& v)
	{
		if (this != &v) Copy(v);
		return *this;
	}
	void Copy(const b3DenseVec3& v)
	{
		v.Sync();
		Sync();
		b3g_sparse_detail::check(b3g_dense_vec3_copy(h, v.h));
		host_valid = false;
	}
	void SetZero()
	{
		b3g_sparse_detail::check(b3g_dense_vec3_set_zero(h));
		host_valid = false;
		host_dirty = false;
	}
	const b3Vec3& operator[](uint32 i) const
	{
		Fetch();
		return host[i];
	}
	b3Vec3& operator[](uint32 i)
	{
		Fetch();
		host_dirty = true;
		return host[i];
	}
	// the device copy up to date (host writes sent)
	void Sync() const
	{
		if (!host_dirty) return;
		b3g_sparse_detail::check(b3g_dense_vec3_set(h, &host[0].x));
		host_dirty = false;
	}
	// the host copy up to date
	void Fetch() const
	{
		if (host_valid) return;
		host.resize(n);
		if (n) b3g_sparse_detail::check(b3g_dense_vec3_get(h, &host[0].x));
		host_valid = true;
	}
	void Touched() { host_valid = false; host_dirty = false; }
	b3g_dense_vec3* handle() const { Sync(); return h; }

	uint32 n;
	b3g_dense_vec3* h = nullptr;
	bool own = true;
	mutable std::vector<b3Vec3> host;
	mutable bool host_valid = false, host_dirty = false;

	// a view of a container owned by the library (a force model's f, x, v)
	static b3DenseVec3* Borrow(b3g_dense_vec3* handle, uint32 n, std::vector<b3DenseVec3*>& keep)
	{
		b3DenseVec3* v = new b3DenseVec3(Tag(), handle, n);
		keep.push_back(v);
		return v;
	}

private:
	struct Tag {};
	b3DenseVec3(Tag, b3g_dense_vec3* handle, uint32 _n) : n(_n), h(handle), own(false) {}
};

static_assert(sizeof(b3Vec3) == 3 * sizeof(float), "b3Vec3 must be three packed floats");

inline void b3Add(b3DenseVec3& out, const b3DenseVec3& a, const b3DenseVec3& b)
{
	b3g_sparse_detail::check(b3g_dense_vec3_add(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Sub(b3DenseVec3& out, const b3DenseVec3& a, const b3DenseVec3& b)
{
	b3g_sparse_detail::check(b3g_dense_vec3_sub(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Mul(b3DenseVec3& out, scalar a, const b3DenseVec3& b)
{
	b3g_sparse_detail::check(b3g_dense_vec3_scale(out.handle(), a, b.handle()));
	out.Touched();
}
inline void b3Negate(b3DenseVec3& out, const b3DenseVec3& v)
{
	b3g_sparse_detail::check(b3g_dense_vec3_negate(out.handle(), v.handle()));
	out.Touched();
}
inline scalar b3Dot(const b3DenseVec3& a, const b3DenseVec3& b)
{
	double d = 0.0;
	b3g_sparse_detail::check(b3g_dense_vec3_dot(a.handle(), b.handle(), &d));
	return (scalar)d;
}
inline scalar b3LengthSquared(const b3DenseVec3& v) { return b3Dot(v, v); }
inline scalar b3Length(const b3DenseVec3& v) { return std::sqrt(b3LengthSquared(v)); }
inline b3DenseVec3 operator+(const b3DenseVec3& a, const b3DenseVec3& b)
{
	b3DenseVec3 r(a.n);
	b3Add(r, a, b);
	return r;
}
inline b3DenseVec3 operator-(const b3DenseVec3& a, const b3DenseVec3& b)
{
	b3DenseVec3 r(a.n);
	b3Sub(r, a, b);
	return r;
}
inline b3DenseVec3 operator*(scalar a, const b3DenseVec3& b)
{
	b3DenseVec3 r(b.n);
	b3Mul(r, a, b);
	return r;
}
inline b3DenseVec3 operator-(const b3DenseVec3& v)
{
	b3DenseVec3 r(v.n);
	b3Negate(r, v);
	return r;
}

// ---------------------------------------------------------------- b3DiagMat33 (diag_mat33.h:27)
struct b3DiagMat33
{
	explicit b3DiagMat33(uint32 _n = 0) : n(_n) { b3g_sparse_detail::check(b3g_diag_mat33_create(b3g_sparse_detail::context(), n, &h)); }
	b3DiagMat33(const b3DiagMat33& m) : b3DiagMat33(m.n) { Copy(m); }
	b3DiagMat33(b3DiagMat33&& m) noexcept
	    : n(m.n), h(m.h), host(std::move(m.host)), host_valid(m.host_valid), host_dirty(m.host_dirty)
	{
		m.h = nullptr;
	}
	~b3DiagMat33()
	{
		if (h) b3g_diag_mat33_destroy(h);
	}
	b3DiagMat33& operator=(const b3DiagMat33& m)
	{
		if (this != &m) Copy(m);
		return *this;
	}
	void Copy(const b3DiagMat33& m)
	{
		b3g_sparse_detail::check(b3g_diag_mat33_copy(handle(), m.handle()));
		Touched();
	}
	void SetZero()
	{
		b3g_sparse_detail::check(b3g_diag_mat33_set_zero(h));
		Touched();
	}
	void SetIdentity()
	{
		b3g_sparse_detail::check(b3g_diag_mat33_set_identity(h));
		Touched();
	}
	const b3Mat33& operator[](uint32 i) const
	{
		Fetch();
		return host[i];
	}
	b3Mat33& operator[](uint32 i)
	{
		Fetch();
		host_dirty = true;
		return host[i];
	}
	void Sync() const
	{
		if (!host_dirty) return;
		b3g_sparse_detail::check(b3g_diag_mat33_set(h, &host[0].x.x));
		host_dirty = false;
	}
	void Fetch() const
	{
		if (host_valid) return;
		host.resize(n);
		if (n) b3g_sparse_detail::check(b3g_diag_mat33_get(h, &host[0].x.x));
		host_valid = true;
	}
	void Touched() { host_valid = false; host_dirty = false; }
	b3g_diag_mat33* handle() const { Sync(); return h; }

	uint32 n;
	b3g_diag_mat33* h = nullptr;
	mutable std::vector<b3Mat33> host;
	mutable bool host_valid = false, host_dirty = false;
};

static_assert(sizeof(b3Mat33) == 9 * sizeof(float), "b3Mat33 must be nine packed floats");

inline void b3Transpose(b3DiagMat33& out, const b3DiagMat33& a)
{
	b3g_sparse_detail::check(b3g_diag_mat33_transpose(out.handle(), a.handle()));
	out.Touched();
}
inline void b3Add(b3DiagMat33& out, const b3DiagMat33& a, const b3DiagMat33& b)
{
	b3g_sparse_detail::check(b3g_diag_mat33_add(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Sub(b3DiagMat33& out, const b3DiagMat33& a, const b3DiagMat33& b)
{
	b3g_sparse_detail::check(b3g_diag_mat33_sub(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Mul(b3DiagMat33& out, scalar a, const b3DiagMat33& b)
{
	b3g_sparse_detail::check(b3g_diag_mat33_scale(out.handle(), a, b.handle()));
	out.Touched();
}
inline void b3Mul(b3DenseVec3& out, const b3DiagMat33& a, const b3DenseVec3& b)
{
	b3g_sparse_detail::check(b3g_diag_mat33_mul_vec(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Negate(b3DiagMat33& out, const b3DiagMat33& v)
{
	b3g_sparse_detail::check(b3g_diag_mat33_negate(out.handle(), v.handle()));
	out.Touched();
}
inline b3DiagMat33 operator+(const b3DiagMat33& a, const b3DiagMat33& b)
{
	b3DiagMat33 r(a.n);
	b3Add(r, a, b);
	return r;
}
inline b3DiagMat33 operator-(const b3DiagMat33& a, const b3DiagMat33& b)
{
	b3DiagMat33 r(a.n);
	b3Sub(r, a, b);
	return r;
}
inline b3DiagMat33 operator*(scalar a, const b3DiagMat33& b)
{
	b3DiagMat33 r(b.n);
	b3Mul(r, a, b);
	return r;
}
inline b3DenseVec3 operator*(const b3DiagMat33& a, const b3DenseVec3& b)
{
	b3DenseVec3 r(b.n);
	b3Mul(r, a, b);
	return r;
}

// ---------------------------------------------------------------- b3SparseMat33 (sparse_mat33.h:94)
// Element access keeps a host copy of the touched blocks; the device matrix is brought up to date
// (its values zeroed, its blocks kept, then the host blocks added) before the next operation.
struct b3SparseMat33
{
	explicit b3SparseMat33(uint32 m = 0) : rowCount(m) { b3g_sparse_detail::check(b3g_sparse_mat33_create(b3g_sparse_detail::context(), m, &h)); }
	b3SparseMat33(const b3SparseMat33& m) : b3SparseMat33(m.rowCount) { Copy(m); }
	b3SparseMat33(b3SparseMat33&& m) noexcept
	    : rowCount(m.rowCount), h(m.h), own(m.own), host(std::move(m.host)), host_valid(m.host_valid),
	      host_dirty(m.host_dirty)
	{
		m.h = nullptr;
	}
	~b3SparseMat33()
	{
		if (h && own) b3g_sparse_mat33_destroy(h);
	}
	b3SparseMat33& operator=(const b3SparseMat33& m)
	{
		if (this != &m) Copy(m);
		return *this;
	}
	void Copy(const b3SparseMat33& m)
	{
		b3g_sparse_detail::check(b3g_sparse_mat33_copy(handle(), m.handle()));
		Touched();
	}
	void Destroy()
	{
		b3g_sparse_detail::check(b3g_sparse_mat33_clear(h));
		Touched();
	}
	// operator()(i, j): the block, created (zero) when absent
	b3Mat33& operator()(uint32 i, uint32 j)
	{
		Fetch();
		host_dirty = true;
		return host[std::make_pair(i, j)];
	}
	b3Mat33 operator()(uint32 i, uint32 j) const
	{
		Fetch();
		auto it = host.find(std::make_pair(i, j));
		b3Mat33 z;
		z.SetZero();
		return it == host.end() ? z : it->second;
	}
	void operator+=(const b3SparseMat33& m);
	void operator-=(const b3SparseMat33& m);
	void operator+=(const b3DiagMat33& m);
	void operator-=(const b3DiagMat33& m);
	// CreateMatrix (sparse_mat33.h:418): dense, column-major (3 rowCount)^2
	void CreateMatrix(scalar* out) const { b3g_sparse_detail::check(b3g_sparse_mat33_to_dense(handle(), out)); }

	void Sync() const
	{
		if (!host_dirty) return;
		std::vector<uint32_t> rows, cols;
		std::vector<float> blocks;
		rows.reserve(host.size());
		cols.reserve(host.size());
		blocks.reserve(9 * host.size());
		for (const auto& e : host)
		{
			rows.push_back(e.first.first);
			cols.push_back(e.first.second);
			const float* b = &e.second.x.x;
			blocks.insert(blocks.end(), b, b + 9);
		}
		b3g_sparse_detail::check(b3g_sparse_mat33_zero_values(h));
		b3g_sparse_detail::check(b3g_sparse_mat33_add_blocks(h, (uint32_t)rows.size(), rows.data(), cols.data(), blocks.data()));
		host_dirty = false;
	}
	void Fetch() const
	{
		if (host_valid) return;
		host.clear();
		uint32_t n = 0;
		uint64_t nb = 0;
		b3g_sparse_detail::check(b3g_sparse_mat33_size(h, &n, &nb));
		if (nb)
		{
			std::vector<uint32_t> rp(n + 1), cols(nb);
			std::vector<float> blocks(9 * nb);
			uint64_t c = 0;
			b3g_sparse_detail::check(b3g_sparse_mat33_export(h, rp.data(), cols.data(), blocks.data(), nb, &c));
			for (uint32_t i = 0; i < n; ++i)
				for (uint32_t k = rp[i]; k < rp[i + 1]; ++k)
				{
					b3Mat33 m;
					std::copy(&blocks[9 * (size_t)k], &blocks[9 * (size_t)k] + 9, &m.x.x);
					host[std::make_pair(i, cols[k])] = m;
				}
		}
		host_valid = true;
	}
	void Touched() { host_valid = false; host_dirty = false; host.clear(); }
	b3g_sparse_mat33* handle() const { Sync(); return h; }

	uint32 rowCount;
	b3g_sparse_mat33* h = nullptr;
	bool own = true;
	mutable std::map<std::pair<uint32, uint32>, b3Mat33> host;
	mutable bool host_valid = false, host_dirty = false;

	static b3SparseMat33* Borrow(b3g_sparse_mat33* handle, uint32 n, std::vector<b3SparseMat33*>& keep)
	{
		b3SparseMat33* m = new b3SparseMat33(Tag(), handle, n);
		// a force model's matrices start empty in every Newton iteration
		m->host_valid = true;
		keep.push_back(m);
		return m;
	}

private:
	struct Tag {};
	b3SparseMat33(Tag, b3g_sparse_mat33* handle, uint32 n) : rowCount(n), h(handle), own(false) {}
};

inline void b3Add(b3SparseMat33& out, const b3SparseMat33& a, const b3SparseMat33& b)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_add(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Sub(b3SparseMat33& out, const b3SparseMat33& a, const b3SparseMat33& b)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_sub(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Add(b3SparseMat33& out, const b3SparseMat33& a, const b3DiagMat33& b)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_add_diag(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Sub(b3SparseMat33& out, const b3SparseMat33& a, const b3DiagMat33& b)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_sub_diag(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Add(b3SparseMat33& out, const b3DiagMat33& a, const b3SparseMat33& b)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_diag_add(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Sub(b3SparseMat33& out, const b3DiagMat33& a, const b3SparseMat33& b)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_diag_sub(out.handle(), a.handle(), b.handle()));
	out.Touched();
}
inline void b3Mul(b3DenseVec3& out, const b3SparseMat33& A, const b3DenseVec3& v)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_mul_vec(out.handle(), A.handle(), v.handle()));
	out.Touched();
}
inline void b3Mul(b3SparseMat33& out, scalar s, const b3SparseMat33& B)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_scale(out.handle(), s, B.handle()));
	out.Touched();
}
inline void b3Mul(b3SparseMat33& out, const b3DiagMat33& A, const b3SparseMat33& B)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_diag_mul(out.handle(), A.handle(), B.handle()));
	out.Touched();
}
inline void b3Mul(b3SparseMat33& out, const b3SparseMat33& A, const b3DiagMat33& B)
{
	b3g_sparse_detail::check(b3g_sparse_mat33_mul_diag(out.handle(), A.handle(), B.handle()));
	out.Touched();
}
inline void b3SparseMat33::operator+=(const b3SparseMat33& m) { b3Add(*this, *this, m); }
inline void b3SparseMat33::operator-=(const b3SparseMat33& m) { b3Sub(*this, *this, m); }
inline void b3SparseMat33::operator+=(const b3DiagMat33& m) { b3Add(*this, *this, m); }
inline void b3SparseMat33::operator-=(const b3DiagMat33& m) { b3Sub(*this, *this, m); }
inline b3SparseMat33 operator+(const b3SparseMat33& A, const b3SparseMat33& B)
{
	b3SparseMat33 r(A.rowCount);
	b3Add(r, A, B);
	return r;
}
inline b3SparseMat33 operator-(const b3SparseMat33& A, const b3SparseMat33& B)
{
	b3SparseMat33 r(A.rowCount);
	b3Sub(r, A, B);
	return r;
}
inline b3SparseMat33 operator+(const b3SparseMat33& A, const b3DiagMat33& B)
{
	b3SparseMat33 r(A.rowCount);
	b3Add(r, A, B);
	return r;
}
inline b3SparseMat33 operator-(const b3SparseMat33& A, const b3DiagMat33& B)
{
	b3SparseMat33 r(A.rowCount);
	b3Sub(r, A, B);
	return r;
}
inline b3SparseMat33 operator+(const b3DiagMat33& A, const b3SparseMat33& B)
{
	b3SparseMat33 r(B.rowCount);
	b3Add(r, A, B);
	return r;
}
inline b3SparseMat33 operator-(const b3DiagMat33& A, const b3SparseMat33& B)
{
	b3SparseMat33 r(B.rowCount);
	b3Sub(r, A, B);
	return r;
}
inline b3SparseMat33 operator*(scalar A, const b3SparseMat33& B)
{
	b3SparseMat33 r(B.rowCount);
	b3Mul(r, A, B);
	return r;
}
inline b3DenseVec3 operator*(const b3SparseMat33& A, const b3DenseVec3& v)
{
	b3DenseVec3 r(v.n);
	b3Mul(r, A, v);
	return r;
}
inline b3SparseMat33 operator*(const b3DiagMat33& A, const b3SparseMat33& B)
{
	b3SparseMat33 r(B.rowCount);
	b3Mul(r, A, B);
	return r;
}
inline b3SparseMat33 operator*(const b3SparseMat33& A, const b3DiagMat33& B)
{
	b3SparseMat33 r(A.rowCount);
	b3Mul(r, A, B);
	return r;
}

// ---------------------------------------------------------------- b3SparseSolveCG (sparse_solver.h)
struct b3SolveCGInput
{
	const b3SparseMat33* A;
	const b3DenseVec3* b;
	uint32 maxIterations;
	scalar tolerance;
};

struct b3SolveCGOutput
{
	b3DenseVec3* x;   // initial guess on entry
	uint32 iterations;
	scalar error;
};

inline bool b3SparseSolveCG(b3SolveCGOutput* output, const b3SolveCGInput* input)
{
	b3g_solve_cg_input in;
	in.A = input->A->handle();
	in.b = input->b->handle();
	in.max_iterations = input->maxIterations;
	in.tolerance = input->tolerance;
	b3g_solve_cg_output out;
	out.x = output->x->handle();
	b3g_sparse_detail::check(b3g_sparse_solve_cg(&out, &in));
	output->x->Touched();
	output->iterations = out.iterations;
	output->error = (scalar)out.error;
	return true;
}

// ---------------------------------------------------------------- b3SparseSolveBE (sparse_force_solver.h)
struct b3SparseForceSolverData
{
	scalar h, inv_h;
	b3DenseVec3* x;
	b3DenseVec3* v;
	b3DenseVec3* f;
	b3SparseMat33* dfdx;
	b3SparseMat33* dfdv;
};

class b3SparseForceModel
{
public:
	virtual ~b3SparseForceModel() {}
	virtual void ApplyForces(const b3SparseForceSolverData* data) = 0;
};

struct b3SolveBEInput
{
	b3SolveBEInput()
	{
		maxIterations = 1;
		tolerance = FLT_EPSILON;
		maxSubIterations = 20;
		subTolerance = FLT_EPSILON;
	}
	scalar h, inv_h;
	b3SparseForceModel* forceModel;
	uint32 dofCount;
	const b3DenseVec3* x0;
	const b3DenseVec3* v0;
	const b3DenseVec3* fe;
	const b3DiagMat33* M;
	const b3DenseVec3* y;
	const b3DiagMat33* S;
	const b3DenseVec3* z;
	uint32 maxIterations;
	scalar tolerance;
	uint32 maxSubIterations;
	scalar subTolerance;
};

struct b3SolveBEOutput
{
	b3DenseVec3* x;
	b3DenseVec3* v;
	uint32 iterations;
	scalar error;
	uint32 minSubIterations;
	uint32 maxSubIterations;
};

namespace b3g_sparse_detail {

struct ModelAdapter
{
	b3SparseForceModel* model;
	uint32 n;
	static void call(void* user, const b3g_sparse_force_solver_data* d)
	{
		ModelAdapter* a = (ModelAdapter*)user;
		std::vector<b3DenseVec3*> vecs;
		std::vector<b3SparseMat33*> mats;
		b3SparseForceSolverData data;
		data.h = d->h;
		data.inv_h = d->inv_h;
		data.x = b3DenseVec3::Borrow(d->x, a->n, vecs);
		data.v = b3DenseVec3::Borrow(d->v, a->n, vecs);
		data.f = b3DenseVec3::Borrow(d->f, a->n, vecs);
		data.dfdx = b3SparseMat33::Borrow(d->dfdx, a->n, mats);
		data.dfdv = b3SparseMat33::Borrow(d->dfdv, a->n, mats);
		a->model->ApplyForces(&data);
		// the model's host writes go back to the solver's containers
		for (b3DenseVec3* v : vecs)
		{
			v->Sync();
			delete v;
		}
		for (b3SparseMat33* m : mats)
		{
			m->Sync();
			delete m;
		}
	}
};

} // namespace b3g_sparse_detail

inline void b3SparseSolveBE(b3SolveBEOutput* output, const b3SolveBEInput* input)
{
	b3g_sparse_detail::ModelAdapter adapter{input->forceModel, input->dofCount};
	b3g_solve_be_input in;
	in.h = input->h;
	in.inv_h = input->inv_h;
	in.force_model.apply_forces = &b3g_sparse_detail::ModelAdapter::call;
	in.force_model.user = &adapter;
	in.dof_count = input->dofCount;
	in.x0 = input->x0->handle();
	in.v0 = input->v0->handle();
	in.fe = input->fe->handle();
	in.M = input->M->handle();
	in.y = input->y->handle();
	in.S = input->S->handle();
	in.z = input->z->handle();
	in.max_iterations = input->maxIterations;
	in.tolerance = input->tolerance;
	in.max_sub_iterations = input->maxSubIterations;
	in.sub_tolerance = input->subTolerance;
	b3g_solve_be_output out;
	out.x = output->x->handle();
	out.v = output->v->handle();
	out.min_sub_iterations = output->minSubIterations;
	out.max_sub_iterations = output->maxSubIterations;
	b3g_sparse_detail::check(b3g_sparse_solve_be(&out, &in));
	output->x->Touched();
	output->v->Touched();
	output->iterations = out.iterations;
	output->error = (scalar)out.error;
	output->minSubIterations = out.min_sub_iterations;
	output->maxSubIterations = out.max_sub_iterations;
}
