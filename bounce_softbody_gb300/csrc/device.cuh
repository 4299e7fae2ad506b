// Device building blocks of the implicit step, shared by the per-op kernels (kernels.cu) and
// the persistent batch kernel (persistent.cu). Matrices in registers are row-major float[9].
#pragma once

#include "internal.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace b3g {

// settings.h:83-95 of the reference
constexpr float kContactStiffness = 1000.0f;
constexpr float kMaxContactCorrection = 0.2f;
constexpr float kBaumgarte = 0.2f;
constexpr float kFltEps = 1.1920928955078125e-7f;

// ------------------------------------------------------------------ load policies
// LdPlain: ordinary loads, for kernels that only read what earlier launches wrote.
// LdCG: L2-coherent loads (ld.global.cg) for the persistent kernel, which reads data that other
// threads of its team wrote earlier in the same launch; it never uses the read-only path.
struct LdPlain
{
	template <class T> static __device__ __forceinline__ T ld(const T* p) { return *p; }
};
struct LdCG
{
	template <class T> static __device__ __forceinline__ T ld(const T* p) { return __ldcg(p); }
};

// Matrix streams of the SpMV. MatNC: for a large body stepped by the per-op kernels, whose
// matrix (larger than L2) is read once per product: read-only path with an L2 evict-first policy,
// so the vector the SpMV gathers from stays in L2 while the matrix streams past it. MatCG: the
// same policy through L2-coherent loads (for a kernel that assembles the matrix earlier in the
// same launch). MatVia<L>: the loads of policy L without a cache hint, for the persistent batch
// kernel, where a small body's matrix is re-read from L2 by every PCG iteration (evict-first
// measured 6% slower on the 512-body batch).
struct MatNC
{
};
struct MatCG
{
};
template <class L>
struct MatVia
{
};

__device__ __forceinline__ unsigned long long evict_first_policy()
{
	unsigned long long pol;
	asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
	return pol;
}

template <class M>
__device__ __forceinline__ uint4 mat_ld16(const void* p, unsigned long long pol);
template <>
__device__ __forceinline__ uint4 mat_ld16<MatNC>(const void* p, unsigned long long pol)
{
	uint4 r;
	asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
	    : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
	    : "l"(p), "l"(pol));
	return r;
}
template <>
__device__ __forceinline__ uint4 mat_ld16<MatCG>(const void* p, unsigned long long pol)
{
	uint4 r;
	asm volatile("ld.global.cg.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
	             : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
	             : "l"(p), "l"(pol));
	return r;
}
template <class M>
__device__ __forceinline__ uint2 mat_ld8(const void* p, unsigned long long pol);
template <>
__device__ __forceinline__ uint2 mat_ld8<MatNC>(const void* p, unsigned long long pol)
{
	uint2 r;
	asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(r.x), "=r"(r.y) : "l"(p), "l"(pol));
	return r;
}
template <>
__device__ __forceinline__ uint2 mat_ld8<MatCG>(const void* p, unsigned long long pol)
{
	uint2 r;
	asm volatile("ld.global.cg.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(r.x), "=r"(r.y) : "l"(p), "l"(pol));
	return r;
}

// ------------------------------------------------------------------ 4-wide solver vectors
// Component c of vertex i at 4 i + c (the fourth component is padding, kept zero).
template <class TV, class L>
__device__ __forceinline__ void vld(const TV* v, int i, TV o[3]);
template <>
__device__ __forceinline__ void vld<float, LdPlain>(const float* v, int i, float o[3])
{
	const float4 t = *(const float4*)(v + 4 * (size_t)i);
	o[0] = t.x;
	o[1] = t.y;
	o[2] = t.z;
}
template <>
__device__ __forceinline__ void vld<float, LdCG>(const float* v, int i, float o[3])
{
	const float4 t = __ldcg((const float4*)(v + 4 * (size_t)i));
	o[0] = t.x;
	o[1] = t.y;
	o[2] = t.z;
}
template <>
__device__ __forceinline__ void vld<double, LdPlain>(const double* v, int i, double o[3])
{
	const double2 a = *(const double2*)(v + 4 * (size_t)i), b = *(const double2*)(v + 4 * (size_t)i + 2);
	o[0] = a.x;
	o[1] = a.y;
	o[2] = b.x;
}
template <>
__device__ __forceinline__ void vld<double, LdCG>(const double* v, int i, double o[3])
{
	const double2 a = __ldcg((const double2*)(v + 4 * (size_t)i)), b = __ldcg((const double2*)(v + 4 * (size_t)i + 2));
	o[0] = a.x;
	o[1] = a.y;
	o[2] = b.x;
}
__device__ __forceinline__ void vst(float* v, int i, const float o[3])
{
	*(float4*)(v + 4 * (size_t)i) = make_float4(o[0], o[1], o[2], 0.0f);
}
__device__ __forceinline__ void vst(double* v, int i, const double o[3])
{
	*(double2*)(v + 4 * (size_t)i) = make_double2(o[0], o[1]);
	*(double2*)(v + 4 * (size_t)i + 2) = make_double2(o[2], 0.0);
}

// One vertex's term of a PCG dot product: the three products summed in the vector type (FP32
// in the FP32 and BF16 modes, as the reference computes them), then widened, so that the sums
// over vertices, warps and CTAs run in FP64 while the FP64 pipe (a small fraction of the FP32
// rate on this GPU) sees one conversion and one add per vertex.
template <class TV>
__device__ __forceinline__ double dot3(const TV a[3], const TV b[3])
{
	return (double)(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
}

// ------------------------------------------------------------------ float-float arithmetic
// The refined PCG solution is kept as an unevaluated sum hi + lo of two floats (about 48
// significant bits) and updated with error-free transformations: Knuth's TwoSum, and the
// product error fma(a, b, -a*b). This runs on the FP32 pipes; this GPU's FP64 rate is a small
// fraction of its FP32 rate.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
	// explicit round-to-nearest operations: the compiler never contracts them into FMAs, which
	// would break the exactness of the transformation
	s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (hi, lo) += p + pe, where pe is a small correction (a product's rounding error)
__device__ __forceinline__ void ff_add(float& hi, float& lo, float p, float pe)
{
	float s, e;
	two_sum(hi, p, s, e);
	e = __fadd_rn(e, __fadd_rn(lo, pe));
	hi = __fadd_rn(s, e);
	lo = __fsub_rn(e, __fsub_rn(hi, s));
}
__device__ __forceinline__ void ff_ld(const float* x, int i, float hi[3], float lo[3])
{
	const float4 h = *(const float4*)(x + 8 * (size_t)i), l = *(const float4*)(x + 8 * (size_t)i + 4);
	hi[0] = h.x; hi[1] = h.y; hi[2] = h.z;
	lo[0] = l.x; lo[1] = l.y; lo[2] = l.z;
}
__device__ __forceinline__ void ff_st(float* x, int i, const float hi[3], const float lo[3])
{
	*(float4*)(x + 8 * (size_t)i) = make_float4(hi[0], hi[1], hi[2], 0.0f);
	*(float4*)(x + 8 * (size_t)i + 4) = make_float4(lo[0], lo[1], lo[2], 0.0f);
}

// ------------------------------------------------------------------ storage conversions
template <class T> __device__ __forceinline__ float to_f(T v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<double>(double v) { return (float)v; }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <class T> __device__ __forceinline__ T from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ double from_f<double>(float v) { return (double)v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// arithmetic type of a SpMV over storage T: blocks are widened before the multiply
template <class T> struct Acc { typedef float type; };
template <> struct Acc<double> { typedef double type; };

template <class T> __device__ __forceinline__ typename Acc<T>::type widen(T v) { return (typename Acc<T>::type)to_f(v); }
template <> __device__ __forceinline__ double widen<double>(double v) { return v; }

// ------------------------------------------------------------------ small vector math
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
	return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
// vec3.h:93 Normalize: multiply by the reciprocal when longer than FLT_EPSILON
__device__ __forceinline__ float3 normalize3(float3 a)
{
	float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
	if (l > kFltEps)
	{
		float s = 1.0f / l;
		a = f3(a.x * s, a.y * s, a.z * s);
	}
	return a;
}
__device__ __forceinline__ float3 ld3(const float* p, int i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
template <class L>
__device__ __forceinline__ float3 ldl3(const float* p, int i)
{
	return f3(L::ld(p + 3 * i), L::ld(p + 3 * i + 1), L::ld(p + 3 * i + 2));
}
__device__ __forceinline__ void st3(float* p, int i, float3 v)
{
	p[3 * i] = v.x;
	p[3 * i + 1] = v.y;
	p[3 * i + 2] = v.z;
}
// rows r of a row-major 3x3 times v
__device__ __forceinline__ float3 mv9(const float* M, float3 v)
{
	return f3(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z,
	          M[6] * v.x + M[7] * v.y + M[8] * v.z);
}
__device__ __forceinline__ float3 mtv9(const float* M, float3 v)
{
	return f3(M[0] * v.x + M[3] * v.y + M[6] * v.z, M[1] * v.x + M[4] * v.y + M[7] * v.z,
	          M[2] * v.x + M[5] * v.y + M[8] * v.z);
}

// quat.h:133 GetRotationMatrix, row-major
__device__ __forceinline__ void quat_to_mat(float4 q, float R[9])
{
	float x = q.x, y = q.y, z = q.z, w = q.w;
	float x2 = x + x, y2 = y + y, z2 = z + z;
	float xx = x * x2, xy = x * y2, xz = x * z2;
	float yy = y * y2, yz = y * z2, zz = z * z2;
	float wx = w * x2, wy = w * y2, wz = w * z2;
	R[0] = 1.0f - (yy + zz); R[1] = xy - wz;          R[2] = xz + wy;
	R[3] = xy + wz;          R[4] = 1.0f - (xx + zz); R[5] = yz - wx;
	R[6] = xz - wy;          R[7] = yz + wx;          R[8] = 1.0f - (xx + yy);
}

// Rotation of the deformation gradient F (row-major) by the iterative method of
// Mueller et al., "A Robust Method to Extract the Rotational Part of Deformations", warm
// started from q0, with the stopping rules of tetrahedron_element_force.cpp:273-311
// (den == 0, |omega| < 1e-9, inverse denominator + 1e-9, at most 32 iterations).
// In float the |omega| < 1e-9 rule sits at the rounding floor of the torque, so most
// tetrahedra run all 32 iterations (as the reference's float build does); each iteration is
// therefore written without divisions or sincosf for the usual small angles:
//  * the update quaternion (sin(w/2) omega / w, cos(w/2)) from Taylor series in w^2 of
//    sin(x) / x and cos(x), x = w / 2: two terms for w < 1e-3 (the next ones below 1e-14),
//    five for w < 1 (truncation below 3e-10), sincosf otherwise;
//  * the test |omega| < 1e-9 as |omega|^2 < 1e-18;
//  * the normalisation 1 / |q| of a product of unit quaternions, |q|^2 = 1 + d with
//    |d| < 1e-4, as 1 - d / 2 (error 3 d^2 / 8 < 4e-9), else a square root and one reciprocal.
__device__ __forceinline__ float4 extract_rotation(const float F[9], float4 q)
{
	const float kTol = 1.0e-9f;
	const float3 a0 = f3(F[0], F[3], F[6]), a1 = f3(F[1], F[4], F[7]), a2 = f3(F[2], F[5], F[8]);
#pragma unroll 1
	for (int it = 0; it < 32; ++it)
	{
		float R[9];
		quat_to_mat(q, R);
		// columns: R(:, c) . F(:, c) and R(:, c) x F(:, c)
		const float3 r0 = f3(R[0], R[3], R[6]), r1 = f3(R[1], R[4], R[7]), r2 = f3(R[2], R[5], R[8]);
		const float den = fabsf(dot3(r0, a0) + dot3(r1, a1) + dot3(r2, a2));
		if (den == 0.0f) break;
		const float3 torque = cross3(r0, a0) + cross3(r1, a1) + cross3(r2, a2);
		const float inv_den = 1.0f / den + kTol;
		const float3 omega = inv_den * torque;
		const float w2 = dot3(omega, omega);
		if (w2 < kTol * kTol) break;
		float half_sinc, cw;  // sin(w / 2) / w and cos(w / 2)
		if (w2 < 1.0e-6f)
		{
			const float y = 0.25f * w2;  // x^2
			half_sinc = 0.5f - y * (1.0f / 12.0f);
			cw = 1.0f - 0.5f * y;
		}
		else if (w2 < 1.0f)
		{
			const float y = 0.25f * w2;  // x^2
			half_sinc = 0.5f * (1.0f - y * (1.0f / 6.0f) * (1.0f - y * (1.0f / 20.0f) * (1.0f - y * (1.0f / 42.0f) * (1.0f - y * (1.0f / 72.0f)))));
			cw = 1.0f - y * 0.5f * (1.0f - y * (1.0f / 12.0f) * (1.0f - y * (1.0f / 30.0f) * (1.0f - y * (1.0f / 56.0f))));
		}
		else
		{
			const float w = sqrtf(w2);
			float sn;
			sincosf(0.5f * w, &sn, &cw);
			half_sinc = sn / w;
		}
		const float3 av = half_sinc * omega, bv = f3(q.x, q.y, q.z);
		// quat.h:204 b3Mul(qw, q)
		float3 rv = cross3(av, bv) + cw * bv + q.w * av;
		float rs = cw * q.w - dot3(av, bv);
		const float l2 = dot3(rv, rv) + rs * rs;
		const float d = l2 - 1.0f;
		float inv_l;
		if (fabsf(d) < 1.0e-4f) inv_l = 1.0f - 0.5f * d;
		else
		{
			const float l = sqrtf(l2);
			inv_l = l > kFltEps ? 1.0f / l : 1.0f;
		}
		q = make_float4(inv_l * rv.x, inv_l * rv.y, inv_l * rv.z, inv_l * rs);
	}
	return q;
}

// X = [e1 e2 e3] * invE with invE column-major (ie[3 j + r] = invE(r, j)); result row-major.
__device__ __forceinline__ void edge_times_invE(float3 e1, float3 e2, float3 e3, const float ie[9], float X[9])
{
#pragma unroll
	for (int j = 0; j < 3; ++j)
	{
		float c0 = ie[3 * j], c1 = ie[3 * j + 1], c2 = ie[3 * j + 2];
		X[0 + j] = c0 * e1.x + c1 * e2.x + c2 * e3.x;
		X[3 + j] = c0 * e1.y + c1 * e2.y + c2 * e3.y;
		X[6 + j] = c0 * e1.z + c1 * e2.z + c2 * e3.z;
	}
}

// ------------------------------------------------------------------ element kernels (one element)
struct StepParams
{
	float h;
	int first_newton;   // iterate == state (x, v)
};

// Corotational tetrahedron (tetrahedron_element_force.cpp:313-464), in stress form.
// With U = R^T (F + W + kd Vg) - I, where F, W and Vg are the gradients of the positions, of
// w = x0 - x + h v + y and of the velocities, the reference's
//   h (f + f_damping + dfdx w)_a = -h R K0_a* (R^T (p + w + kd v) - rest)
// equals -h V R sigma(sym U) g_a with sigma(e) = lambda tr(e) I + 2 mu e, because
// K0 = V B^T D B is that isotropic operator. The A contribution (h^2 + h kd) R K0_ab R^T is
// kept in factored form: rows of R times the shape gradients, scaled (tet_rec).
template <class L = LdPlain>
__device__ __forceinline__ void tet_element(const DevBody& B, int e, const StepParams& P)
{
	const float h = P.h;
	uint4 id = B.tet[e];
	const float* X = P.first_newton ? B.x : B.xi;
	const float* Vv = P.first_newton ? B.v : B.vi;
	const size_t nt = (size_t)B.nt;
	float ie[9];
#pragma unroll
	for (int k = 0; k < 9; ++k) ie[k] = B.tet_invE[k * nt + e];
	float4 mat = B.tet_mat[e];  // volume, lambda, mu, kd
	float3 p1 = ldl3<L>(X, id.x), p2 = ldl3<L>(X, id.y), p3 = ldl3<L>(X, id.z), p4 = ldl3<L>(X, id.w);
	float F[9];
	edge_times_invE(p2 - p1, p3 - p1, p4 - p1, ie, F);
	float4 q = extract_rotation(F, L::ld(B.tet_q + e));
	B.tet_q[e] = q;
	float R[9];
	quat_to_mat(q, R);

	// w = x0 - x + h v + y
	float3 v1 = ldl3<L>(Vv, id.x), v2 = ldl3<L>(Vv, id.y), v3 = ldl3<L>(Vv, id.z), v4 = ldl3<L>(Vv, id.w);
	float3 y1 = ldl3<L>(B.trans, id.x), y2 = ldl3<L>(B.trans, id.y), y3 = ldl3<L>(B.trans, id.z), y4 = ldl3<L>(B.trans, id.w);
	float3 w1 = h * v1 + y1, w2 = h * v2 + y2, w3 = h * v3 + y3, w4 = h * v4 + y4;
	if (!P.first_newton)
	{
		w1 = w1 + (ldl3<L>(B.x, id.x) - p1);
		w2 = w2 + (ldl3<L>(B.x, id.y) - p2);
		w3 = w3 + (ldl3<L>(B.x, id.z) - p3);
		w4 = w4 + (ldl3<L>(B.x, id.w) - p4);
	}
	float G[9];
	edge_times_invE(w2 - w1, w3 - w1, w4 - w1, ie, G);
	const float kd = mat.w;
	if (kd > 0.0f)
	{
		float Vg[9];
		edge_times_invE(v2 - v1, v3 - v1, v4 - v1, ie, Vg);
#pragma unroll
		for (int k = 0; k < 9; ++k) G[k] += kd * Vg[k];
	}
#pragma unroll
	for (int k = 0; k < 9; ++k) G[k] += F[k];
	// U = R^T G - I
	float U[9];
#pragma unroll
	for (int r = 0; r < 3; ++r)
#pragma unroll
		for (int c = 0; c < 3; ++c)
			U[3 * r + c] = R[r] * G[c] + R[3 + r] * G[3 + c] + R[6 + r] * G[6 + c] - (r == c ? 1.0f : 0.0f);
	const float vol = mat.x, lam = mat.y, mu = mat.z;
	float tr = U[0] + U[4] + U[8];
	float S[9];
#pragma unroll
	for (int r = 0; r < 3; ++r)
#pragma unroll
		for (int c = 0; c < 3; ++c) S[3 * r + c] = mu * (U[3 * r + c] + U[3 * c + r]) + (r == c ? lam * tr : 0.0f);

	float3 g2 = f3(ie[0], ie[3], ie[6]), g3 = f3(ie[1], ie[4], ie[7]), g4 = f3(ie[2], ie[5], ie[8]);
	float3 g1 = -(g2 + g3 + g4);
	float3 g[4] = {g1, g2, g3, g4};
	const float c = (h * h + h * kd) * vol;
	const float su = sqrtf(c * mu);
	const float ratio = mu > 0.0f ? lam / mu : 0.0f;
	float* bc = B.tet_bc + e;
	float4* rec = B.tet_rec + e;
#pragma unroll
	for (int a = 0; a < 4; ++a)
	{
		float3 t = mv9(S, g[a]);
		float3 f = mv9(R, t);
		float s = -h * vol;
		bc[(3 * a + 0) * nt] = s * f.x;
		bc[(3 * a + 1) * nt] = s * f.y;
		bc[(3 * a + 2) * nt] = s * f.z;
		float3 rg = mv9(R, g[a]);
		rec[a * nt] = make_float4(su * rg.x, su * rg.y, su * rg.z, ratio);
	}
}

// mat33.h:310 b3ComputeBasis
__device__ __forceinline__ void compute_basis(float3 a, float3& b, float3& c)
{
	const float sqrt_inv3 = sqrtf(1.0f / 3.0f);
	if (fabsf(a.x) >= sqrt_inv3) b = f3(a.y, -a.x, 0.0f);
	else b = f3(0.0f, a.z, -a.y);
	b = normalize3(b);
	c = cross3(a, b);
}

// Corotational orthotropic membrane triangle (triangle_element_force.cpp:285-468). Writes the
// 9 blocks (h^2 + h kd) K_ab of A and the 3 right-hand-side vectors
// h (f_a - kd (K v)_a - (K w)_a).
template <class L = LdPlain>
__device__ __forceinline__ void tri_element(const DevBody& B, int e, const StepParams& P)
{
	const float h = P.h;
	uint4 id = B.tri[e];
	const float* X = P.first_newton ? B.x : B.xi;
	const float* Vv = P.first_newton ? B.v : B.vi;
	float3 p[3] = {ldl3<L>(X, id.x), ldl3<L>(X, id.y), ldl3<L>(X, id.z)};
	int ids[3] = {(int)id.x, (int)id.y, (int)id.z};
	float3 n = normalize3(cross3(p[1] - p[0], p[2] - p[0]));
	float3 px, py;
	compute_basis(n, px, py);
	float2 x2[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
		x2[k] = make_float2(px.x * p[k].x + px.y * p[k].y + px.z * p[k].z, py.x * p[k].x + py.y * p[k].y + py.z * p[k].z);
	const float* iS = B.tri_invS + 4 * (size_t)e;  // column-major 2x2
	float2 t0 = make_float2(x2[1].x - x2[0].x, x2[1].y - x2[0].y);
	float2 t1 = make_float2(x2[2].x - x2[0].x, x2[2].y - x2[0].y);
	// F = T invS, column-major
	float F00 = t0.x * iS[0] + t1.x * iS[1], F10 = t0.y * iS[0] + t1.y * iS[1];
	float F01 = t0.x * iS[2] + t1.x * iS[3], F11 = t0.y * iS[2] + t1.y * iS[3];
	// triangle_element_force.cpp:131-150 polar decomposition
	float det = F00 * F11 - F01 * F10;
	float sg = (float)(0.0f < det) - (float)(det < 0.0f);
	float q00 = F00 + sg * F11, q10 = F10 - sg * F01;
	float q01 = F01 - sg * F10, q11 = F11 + sg * F00;
	float l0 = sqrtf(q00 * q00 + q10 * q10), l1 = sqrtf(q01 * q01 + q11 * q11);
	if (l0 > kFltEps) { q00 /= l0; q10 /= l0; }
	if (l1 > kFltEps) { q01 /= l1; q11 /= l1; }
	// R = [q00 q01; q10 q11]; us_k = R^T x_k - rest_k
	const float* rest = B.tri_x + 6 * (size_t)e;
	float2 us[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
		us[k] = make_float2(q00 * x2[k].x + q10 * x2[k].y - rest[2 * k], q01 * x2[k].x + q11 * x2[k].y - rest[2 * k + 1]);
	const float* K0 = B.tri_K + 36 * (size_t)e;
	const float kd = B.tri_kd ? B.tri_kd[e] : 0.0f;
	const float cA = h * h + h * kd;
	float3 fa[3];
#pragma unroll
	for (int a = 0; a < 3; ++a)
	{
		float fx = 0.0f, fy = 0.0f;
#pragma unroll
		for (int b = 0; b < 3; ++b)
		{
			const float* k = K0 + 4 * (a + 3 * b);
			fx += k[0] * us[b].x + k[2] * us[b].y;
			fy += k[1] * us[b].x + k[3] * us[b].y;
		}
		float rx = q00 * fx + q01 * fy, ry = q10 * fx + q11 * fy;
		fa[a] = -(rx * px + ry * py);
	}
	// 3-D blocks K_ab = P^T (R K0_ab R^T) P, P = [px^T; py^T]
	float3 vv[3] = {ldl3<L>(Vv, ids[0]), ldl3<L>(Vv, ids[1]), ldl3<L>(Vv, ids[2])};
	float3 ww[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
	{
		ww[k] = h * vv[k] + ldl3<L>(B.trans, ids[k]);
		if (!P.first_newton) ww[k] = ww[k] + (ldl3<L>(B.x, ids[k]) - p[k]);
	}
	float3 acc[3] = {fa[0], fa[1], fa[2]};
	float* blk = B.blocks + 81 * (size_t)e;
#pragma unroll
	for (int a = 0; a < 3; ++a)
#pragma unroll
		for (int b = 0; b < 3; ++b)
		{
			const float* k = K0 + 4 * (a + 3 * b);
			// RK = R k R^T (2x2, column-major k)
			float m00 = q00 * k[0] + q01 * k[1], m10 = q10 * k[0] + q11 * k[1];
			float m01 = q00 * k[2] + q01 * k[3], m11 = q10 * k[2] + q11 * k[3];
			float r00 = m00 * q00 + m01 * q01, r01 = m00 * q10 + m01 * q11;
			float r10 = m10 * q00 + m11 * q01, r11 = m10 * q10 + m11 * q11;
			// K = P^T RK P: K[r][c] = sum_{i,j} P[i][r] RK[i][j] P[j][c]
			float3 c0 = r00 * px + r10 * py;  // P^T * RK column 0
			float3 c1 = r01 * px + r11 * py;  // column 1
			float Kb[9];
			Kb[0] = c0.x * px.x + c1.x * py.x; Kb[1] = c0.x * px.y + c1.x * py.y; Kb[2] = c0.x * px.z + c1.x * py.z;
			Kb[3] = c0.y * px.x + c1.y * py.x; Kb[4] = c0.y * px.y + c1.y * py.y; Kb[5] = c0.y * px.z + c1.y * py.z;
			Kb[6] = c0.z * px.x + c1.z * py.x; Kb[7] = c0.z * px.y + c1.z * py.y; Kb[8] = c0.z * px.z + c1.z * py.z;
			float3 kw = mv9(Kb, ww[b]);
			acc[a] = acc[a] - kw;
			if (kd > 0.0f) acc[a] = acc[a] - kd * mv9(Kb, vv[b]);
			float* o = blk + 9 * (3 * a + b);
#pragma unroll
			for (int t = 0; t < 9; ++t) o[t] = cA * Kb[t];
		}
	float* bv = B.bvec + 9 * (size_t)e;
#pragma unroll
	for (int a = 0; a < 3; ++a)
	{
		bv[3 * a + 0] = h * acc[a].x;
		bv[3 * a + 1] = h * acc[a].y;
		bv[3 * a + 2] = h * acc[a].z;
	}
}

// Tension-only spring (spring_force.cpp:61-143). The stiffness Jacobian keeps the reference's
// unnormalised outer product dx dx^T. Writes one block h^2 Ks + h Kd (+ on the diagonal,
// - off it) and one vector h (f1 - Ks (w1 - w2)) (+ for vertex 1, - for vertex 2).
template <class LP = LdPlain>
__device__ __forceinline__ void spring_element(const DevBody& B, int s, const StepParams& P)
{
	const float h = P.h;
	uint2 id = B.spr[s];
	const float* X = P.first_newton ? B.x : B.xi;
	const float* Vv = P.first_newton ? B.v : B.vi;
	float3 x1 = ldl3<LP>(X, id.x), x2 = ldl3<LP>(X, id.y);
	float3 v1 = ldl3<LP>(Vv, id.x), v2 = ldl3<LP>(Vv, id.y);
	float3 dx = x1 - x2;
	float L = len3(dx);
	float blk[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	float3 f = f3(0, 0, 0);
	float3 kw = f3(0, 0, 0);
	if (L > 0.0f)
	{
		float3 n = f3(dx.x / L, dx.y / L, dx.z / L);
		float ks = B.spr_ks[s], kd = B.spr_kd[s], L0 = B.spr_L0[s];
		float3 w1 = h * v1 + ldl3<LP>(B.trans, id.x), w2 = h * v2 + ldl3<LP>(B.trans, id.y);
		if (!P.first_newton)
		{
			w1 = w1 + (ldl3<LP>(B.x, id.x) - x1);
			w2 = w2 + (ldl3<LP>(B.x, id.y) - x2);
		}
		float3 dw = w1 - w2;
		if (ks > 0.0f && L > L0)
		{
			float C = L - L0;
			f = -(ks * C) * n;
			float t = 1.0f - L0 / L;
			float d[3] = {dx.x, dx.y, dx.z};
			float Ks[9];
#pragma unroll
			for (int r = 0; r < 3; ++r)
#pragma unroll
				for (int c = 0; c < 3; ++c)
				{
					float o = d[r] * d[c];
					Ks[3 * r + c] = ks * (o + t * ((r == c ? 1.0f : 0.0f) - o));
				}
			kw = mv9(Ks, dw);
#pragma unroll
			for (int k = 0; k < 9; ++k) blk[k] += h * h * Ks[k];
		}
		if (kd > 0.0f)
		{
			float dCdt = dot3(n, v1 - v2);
			f = f + (-(kd * dCdt)) * n;
			float nn[3] = {n.x, n.y, n.z};
#pragma unroll
			for (int r = 0; r < 3; ++r)
#pragma unroll
				for (int c = 0; c < 3; ++c) blk[3 * r + c] += h * kd * nn[r] * nn[c];
		}
	}
	float* o = B.blocks + 9 * ((size_t)9 * B.ntr + s);
#pragma unroll
	for (int k = 0; k < 9; ++k) o[k] = blk[k];
	float3 bvv = h * (f - kw);
	st3(B.bvec, 3 * B.ntr + s, bvv);
}

// ------------------------------------------------------------------ cloth forces
// Velocity-level displacement w_k = h v_k + y_k (+ x_k - iterate on later Newton iterates) of an
// element's vertex, the vector the implicit right-hand side h (f + dfdx w) multiplies dfdx by.
template <class LP>
__device__ __forceinline__ float3 element_w(const DevBody& B, const StepParams& P, int id, float3 xk, float3 vk)
{
	float3 w = P.h * vk + ldl3<LP>(B.trans, id);
	if (!P.first_newton) w = w + (ldl3<LP>(B.x, id) - xk);
	return w;
}

// Symmetric 3x3 (xx, xy, xz, yy, yz, zz): s nn^T + t I.
__device__ __forceinline__ void sym_nn(float3 n, float s, float t, float M[6])
{
	M[0] = s * n.x * n.x + t; M[1] = s * n.x * n.y; M[2] = s * n.x * n.z;
	M[3] = s * n.y * n.y + t; M[4] = s * n.y * n.z; M[5] = s * n.z * n.z + t;
}
__device__ __forceinline__ float3 sym_mv(const float M[6], float3 v)
{
	return f3(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[1] * v.x + M[3] * v.y + M[4] * v.z,
	          M[2] * v.x + M[4] * v.y + M[5] * v.z);
}
// o (9 floats, row-major) = s M
__device__ __forceinline__ void sym_store(float* o, const float M[6], float s)
{
	o[0] = s * M[0]; o[1] = s * M[1]; o[2] = s * M[2];
	o[3] = s * M[1]; o[4] = s * M[3]; o[5] = s * M[4];
	o[6] = s * M[2]; o[7] = s * M[4]; o[8] = s * M[5];
}

// One direction (u or v) of the Baraff-Witkin stretch condition
// (stretch_force.cpp:142-270 for u, 272-387 for v): C = alpha (|w_dir| - b), dC_a = alpha g_a n
// with n = w_dir / |w_dir|. Every Jacobian block of the direction is g_a g_b times one symmetric
// matrix, so the direction yields
//   M   = h^2 Ks + h kd alpha^2 nn^T   (the A blocks are g_a g_b M),
//   Ks  = ks (alpha^2 nn^T + [|w_dir| > b] C alpha / |w_dir| (I - nn^T))   (dfdx_ab = -g_a g_b Ks),
// and adds to f_a the stiffness and damping forces and -g_a Ks sum_b g_b w_b.
__device__ __forceinline__ void stretch_direction(float3 wd, const float g[3], float alpha, float ks, float kd,
                                                  float b, const float3 v[3], const float3 w[3], float h,
                                                  float3 f[3], float M[6])
{
#pragma unroll
	for (int q = 0; q < 6; ++q) M[q] = 0.0f;
	const float len = len3(wd);
	if (!(len > 0.0f)) return;
	const float inv_len = 1.0f / len;
	const float3 n = inv_len * wd;
	if (ks > 0.0f)
	{
		const float C = alpha * (len - b);
		const float t = len > b ? C * alpha * inv_len : 0.0f;
		float Ks[6];
		sym_nn(n, ks * (alpha * alpha - t), ks * t, Ks);
		const float3 W = g[0] * w[0] + g[1] * w[1] + g[2] * w[2];
		const float3 KW = sym_mv(Ks, W);
#pragma unroll
		for (int a = 0; a < 3; ++a) f[a] = f[a] - (ks * C * alpha * g[a]) * n - g[a] * KW;
#pragma unroll
		for (int q = 0; q < 6; ++q) M[q] = h * h * Ks[q];
	}
	if (kd > 0.0f)
	{
		const float dCdt = alpha * dot3(g[0] * v[0] + g[1] * v[1] + g[2] * v[2], n);
#pragma unroll
		for (int a = 0; a < 3; ++a) f[a] = f[a] - (kd * dCdt * alpha * g[a]) * n;
		float Md[6];
		sym_nn(n, h * kd * alpha * alpha, 0.0f, Md);
#pragma unroll
		for (int q = 0; q < 6; ++q) M[q] += Md[q];
	}
}

// Baraff-Witkin stretch (stretch_force.cpp:121-388) or shear (shear_force.cpp:106-244) triangle.
// With dx1 = x2 - x1, dx2 = x3 - x1: w_u = (dv2 dx1 - dv1 dx2) / det, w_v = (du1 dx2 - du2 dx1) / det.
// Writes the 9 blocks -h^2 dfdx_ab - h dfdv_ab of A and the 3 vectors h (f_a + sum_b dfdx_ab w_b).
// Shear: C = alpha w_u . w_v, dC_a = alpha (dwu_a w_v + dwv_a w_u), dfdx_ab = -ks dC_a dC_b^T
// (the reference drops the second-derivative term), dfdv_ab = -kd dC_a dC_b^T.
template <class LP = LdPlain>
__device__ __forceinline__ void bw_element(const DevBody& B, int e, const StepParams& P)
{
	const float h = P.h;
	const uint4 id = B.bw[e];
	const int ids[3] = {(int)id.x, (int)id.y, (int)id.z};
	const float* c = B.bw_c + (size_t)kBwFloats * e;
	const float* X = P.first_newton ? B.x : B.xi;
	const float* Vv = P.first_newton ? B.v : B.vi;
	float3 x[3], v[3], w[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
	{
		x[k] = ldl3<LP>(X, ids[k]);
		v[k] = ldl3<LP>(Vv, ids[k]);
		w[k] = element_w<LP>(B, P, ids[k], x[k], v[k]);
	}
	const float alpha = c[0], inv_det = c[1], du1 = c[2], dv1 = c[3], du2 = c[4], dv2 = c[5];
	const float gu[3] = {c[6], c[7], c[8]}, gv[3] = {c[9], c[10], c[11]};
	const float3 dx1 = x[1] - x[0], dx2 = x[2] - x[0];
	const float3 wu = inv_det * (dv2 * dx1 - dv1 * dx2);
	const float3 wv = inv_det * (-du2 * dx1 + du1 * dx2);
	float3 f[3] = {f3(0, 0, 0), f3(0, 0, 0), f3(0, 0, 0)};
	float* blk = B.blocks + 9 * ((size_t)9 * B.ntr + B.ns + 9 * (size_t)e);
	if (id.w == kForceStretch)
	{
		float Mu[6], Mv[6];
		stretch_direction(wu, gu, alpha, c[12], c[13], c[14], v, w, h, f, Mu);
		stretch_direction(wv, gv, alpha, c[15], c[16], c[17], v, w, h, f, Mv);
#pragma unroll
		for (int a = 0; a < 3; ++a)
#pragma unroll
			for (int b = 0; b < 3; ++b)
			{
				const float su = gu[a] * gu[b], sv = gv[a] * gv[b];
				float M[6];
#pragma unroll
				for (int q = 0; q < 6; ++q) M[q] = su * Mu[q] + sv * Mv[q];
				sym_store(blk + 9 * (3 * a + b), M, 1.0f);
			}
	}
	else
	{
		const float ks = c[12], kd = c[13];
		float3 dC[3];
#pragma unroll
		for (int a = 0; a < 3; ++a) dC[a] = alpha * (gu[a] * wv + gv[a] * wu);
		float sA = 0.0f;
		if (ks > 0.0f)
		{
			const float C = alpha * dot3(wu, wv);
			const float S = dot3(dC[0], w[0]) + dot3(dC[1], w[1]) + dot3(dC[2], w[2]);
#pragma unroll
			for (int a = 0; a < 3; ++a) f[a] = f[a] - (ks * (C + S)) * dC[a];
			sA += h * h * ks;
		}
		if (kd > 0.0f)
		{
			const float dCdt = dot3(dC[0], v[0]) + dot3(dC[1], v[1]) + dot3(dC[2], v[2]);
#pragma unroll
			for (int a = 0; a < 3; ++a) f[a] = f[a] - (kd * dCdt) * dC[a];
			sA += h * kd;
		}
#pragma unroll
		for (int a = 0; a < 3; ++a)
#pragma unroll
			for (int b = 0; b < 3; ++b)
			{
				float* o = blk + 9 * (3 * a + b);
				const float ra[3] = {dC[a].x, dC[a].y, dC[a].z}, rb[3] = {dC[b].x, dC[b].y, dC[b].z};
#pragma unroll
				for (int r = 0; r < 3; ++r)
#pragma unroll
					for (int q = 0; q < 3; ++q) o[3 * r + q] = sA * ra[r] * rb[q];
			}
	}
	const size_t v0 = (size_t)3 * B.ntr + B.ns + 3 * (size_t)e;
#pragma unroll
	for (int a = 0; a < 3; ++a) st3(B.bvec, (int)(v0 + a), h * f[a]);
}

// Mouse spring between particle 1 and the point w2 x2 + w3 x3 + w4 x4 of a triangle
// (mouse_force.cpp:58-245): d = x1 - c2, C = |d| - L0, dC_a = c_a n with c = (1, -w2, -w3, -w4).
// Every block is c_a c_b times one symmetric matrix:
//   dfdx_ab = -c_a c_b ks (nn^T + C (I / |d| - dd^T / |d|^3))   (only while |d| > L0),
//   dfdv_ab = -c_a c_b kd nn^T.
template <class LP = LdPlain>
__device__ __forceinline__ void mouse_element(const DevBody& B, int e, const StepParams& P)
{
	const float h = P.h;
	const uint4 id = B.ms[e];
	const int ids[4] = {(int)id.x, (int)id.y, (int)id.z, (int)id.w};
	const float* c = B.ms_c + (size_t)kMouseFloats * e;
	const float* X = P.first_newton ? B.x : B.xi;
	const float* Vv = P.first_newton ? B.v : B.vi;
	const float cw[4] = {1.0f, -c[0], -c[1], -c[2]};
	const float ks = c[3], kd = c[4], L0 = c[5];
	float3 x[4], v[4];
#pragma unroll
	for (int k = 0; k < 4; ++k)
	{
		x[k] = ldl3<LP>(X, ids[k]);
		v[k] = ldl3<LP>(Vv, ids[k]);
	}
	const float3 d = x[0] - (c[0] * x[1] + c[1] * x[2] + c[2] * x[3]);
	const float L = len3(d);
	float M[6] = {0, 0, 0, 0, 0, 0};
	float3 fd = f3(0, 0, 0);  // f_a = c_a fd
	if (L > 0.0f)
	{
		const float inv_L = 1.0f / L;
		const float3 n = inv_L * d;
		if (ks > 0.0f && L > L0)
		{
			const float C = L - L0;
			// nn^T + C (I / L - dd^T / L^3) = (1 - C / L) nn^T + (C / L) I
			float Ks[6];
			sym_nn(n, ks * (1.0f - C * inv_L), ks * C * inv_L, Ks);
			float3 W = f3(0, 0, 0);
#pragma unroll
			for (int k = 0; k < 4; ++k) W = W + cw[k] * element_w<LP>(B, P, ids[k], x[k], v[k]);
			fd = fd - (ks * C) * n - sym_mv(Ks, W);
#pragma unroll
			for (int q = 0; q < 6; ++q) M[q] = h * h * Ks[q];
		}
		if (kd > 0.0f)
		{
			const float dCdt = dot3(v[0] - (c[0] * v[1] + c[1] * v[2] + c[2] * v[3]), n);
			fd = fd - (kd * dCdt) * n;
			float Md[6];
			sym_nn(n, h * kd, 0.0f, Md);
#pragma unroll
			for (int q = 0; q < 6; ++q) M[q] += Md[q];
		}
	}
	float* blk = B.blocks + 9 * ((size_t)9 * B.ntr + B.ns + 9 * (size_t)B.nbw + 16 * (size_t)e);
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int b = 0; b < 4; ++b) sym_store(blk + 9 * (4 * a + b), M, cw[a] * cw[b]);
	const size_t v0 = (size_t)3 * B.ntr + B.ns + 3 * (size_t)B.nbw + 4 * (size_t)e;
#pragma unroll
	for (int a = 0; a < 4; ++a) st3(B.bvec, (int)(v0 + a), (h * cw[a]) * fd);
}

// ------------------------------------------------------------------ row assembly
// ------------------------------------------------------------------ world shapes
// The closest point of each static world shape to a vertex sphere (b3Shape::Collide): the
// manifold point on the shape's core and the normal from the shape to the sphere, or no contact.
__device__ __forceinline__ float3 f3p(const float* p) { return f3(p[0], p[1], p[2]); }

// quat.h:75-79 b3Quat::Rotate, and the rotation by the conjugate (b3MulC)
__device__ __forceinline__ float3 qrot(const float q[4], float3 v, float sign = 1.0f)
{
	const float3 u = f3(sign * q[0], sign * q[1], sign * q[2]);
	const float3 t = 2.0f * cross3(u, v);
	return v + q[3] * t + cross3(u, t);
}

// sphere_shape.cpp:50-77
__device__ __forceinline__ bool collide_sphere(const DevShape& S, float3 Q, float r1, float3& P, float3& n)
{
	const float radius = S.radius + r1;
	const float3 c = f3p(S.a);
	const float3 d = Q - c;
	const float dd = dot3(d, d);
	if (!(dd <= radius * radius)) return false;
	P = c;
	if (dd > kFltEps * kFltEps)
	{
		const float dist = sqrtf(dd);
		n = f3(d.x / dist, d.y / dist, d.z / dist);
	}
	else n = f3(0.0f, 1.0f, 0.0f);
	return true;
}

// closest point P of a feature, normal from it to Q unless Q is on it (then `fallback`)
__device__ __forceinline__ bool point_feature(float3 Q, float3 Pf, float radius, float3 fallback, float3& P, float3& n)
{
	const float3 d = Q - Pf;
	const float dd = dot3(d, d);
	if (dd > radius * radius) return false;
	n = fallback;
	const float l = sqrtf(dd);
	if (l > kFltEps) n = f3(d.x / l, d.y / l, d.z / l);
	P = Pf;
	return true;
}

// capsule_shape.cpp:52-136
__device__ __forceinline__ bool collide_capsule(const DevShape& S, float3 Q, float r1, float3& P, float3& n)
{
	const float3 A = f3p(S.a), B = f3p(S.b);
	const float3 AB = B - A;
	const float u = dot3(B - Q, AB), v = dot3(Q - A, AB);
	const float radius = S.radius + r1;
	if (v <= 0.0f) return point_feature(Q, A, radius, f3(0.0f, 1.0f, 0.0f), P, n);
	if (u <= 0.0f) return point_feature(Q, B, radius, f3(0.0f, 1.0f, 0.0f), P, n);
	const float ss = dot3(AB, AB);
	const float3 Pm = (u * A + v * B);
	const float3 Pc = f3(Pm.x / ss, Pm.y / ss, Pm.z / ss);
	const float3 d = Q - Pc;
	if (dot3(d, d) > radius * radius) return false;
	const float3 AQ = Q - A;
	float3 nn = cross3(cross3(AB, AQ), AB);
	if (dot3(nn, AQ) < 0.0f) nn = -nn;
	n = normalize3(nn);
	P = Pc;
	return true;
}

// box_shape.cpp:63-140: planes (+-x, +-y, +-z) at the extents in the box frame
__device__ __forceinline__ bool collide_box(const DevShape& S, float3 Q, float r1, float3& P, float3& n)
{
	const float3 e = f3p(S.a);
	const float radius = S.radius + r1;
	const float3 cl = qrot(S.q, Q - f3p(S.t), -1.0f);  // b3MulT(xf, Q)
	const float3 normals[6] = {f3(1, 0, 0), f3(-1, 0, 0), f3(0, 1, 0), f3(0, -1, 0), f3(0, 0, 1), f3(0, 0, -1)};
	const float offsets[6] = {e.x, e.x, e.y, e.y, e.z, e.z};
	int face = 0;
	float sep = -3.402823466e+38f;
	for (int k = 0; k < 6; ++k)
	{
		const float sk = dot3(normals[k], cl) - offsets[k];
		if (sk > radius) return false;
		if (sk > sep)
		{
			face = k;
			sep = sk;
		}
	}
	if (sep < 0.0f)
	{
		// the sphere center is inside the box: the closest face
		const float3 cb = cl - sep * normals[face];
		P = qrot(S.q, cb) + f3p(S.t);
		n = qrot(S.q, normals[face]);
		return true;
	}
	const float3 cb = f3(fmaxf(-e.x, fminf(cl.x, e.x)), fmaxf(-e.y, fminf(cl.y, e.y)), fmaxf(-e.z, fminf(cl.z, e.z)));
	const float3 d = cl - cb;
	const float dd = dot3(d, d);
	if (dd > radius * radius) return false;
	if (!(dd > kFltEps * kFltEps)) return false;
	const float dist = sqrtf(dd);
	P = qrot(S.q, cb) + f3p(S.t);
	n = qrot(S.q, f3(d.x / dist, d.y / dist, d.z / dist));
	return true;
}

// geometry.h:27-70 b3BarycentricCoordinates of Q on segment AB (u, v, divisor) and on
// triangle ABC (u, v, w, divisor)
__device__ __forceinline__ void bary2(float out[3], float3 A, float3 B, float3 Q)
{
	const float3 AB = B - A, QA = A - Q, QB = B - Q;
	out[0] = dot3(QB, AB);
	out[1] = -dot3(QA, AB);
	out[2] = dot3(AB, AB);
}
__device__ __forceinline__ void bary3(float out[4], float3 A, float3 B, float3 C, float3 Q)
{
	const float3 AB = B - A, AC = C - A, QA = A - Q, QB = B - Q, QC = C - Q;
	const float3 ABxAC = cross3(AB, AC);
	out[0] = dot3(cross3(QB, QC), ABxAC);
	out[1] = dot3(cross3(QC, QA), ABxAC);
	out[2] = dot3(cross3(QA, QB), ABxAC);
	out[3] = dot3(ABxAC, ABxAC);
}

// triangle_shape.cpp:65-311 with optional wing vertices (mesh children)
__device__ __forceinline__ bool collide_triangle(float3 A, float3 B, float3 C, const float3* wing, const bool* has_wing,
                                                 float shape_radius, float3 Q, float r1, float3& P, float3& n)
{
	const float radius = shape_radius + r1;
	const float3 tn = normalize3(cross3(B - A, C - A));
	float wAB[3], wBC[3], wCA[3];
	bary2(wAB, A, B, Q);
	bary2(wBC, B, C, Q);
	bary2(wCA, C, A, Q);
	if (wAB[1] <= 0.0f && wCA[0] <= 0.0f) return point_feature(Q, A, radius, tn, P, n);
	if (wAB[0] <= 0.0f && wBC[1] <= 0.0f) return point_feature(Q, B, radius, tn, P, n);
	if (wBC[0] <= 0.0f && wCA[1] <= 0.0f) return point_feature(Q, C, radius, tn, P, n);
	float wABC[4];
	bary3(wABC, A, B, C, Q);
	// edge regions: AB (wing 0: face wing, B, A), BC (wing 1: wing, C, B), CA (wing 2: wing, A, C)
	const float* wedge[3] = {wAB, wBC, wCA};
	const float3 E0[3] = {A, B, C}, E1[3] = {B, C, A};
	const float opp[3] = {wABC[2], wABC[0], wABC[1]};
	for (int e = 0; e < 3; ++e)
	{
		const float* w = wedge[e];
		if (w[0] > 0.0f && w[1] > 0.0f && wABC[3] * opp[e] <= 0.0f)
		{
			const float3 Pm = w[0] * E0[e] + w[1] * E1[e];
			const float3 Pe = f3(Pm.x / w[2], Pm.y / w[2], Pm.z / w[2]);
			const float3 d = Q - Pe;
			if (dot3(d, d) > radius * radius) return false;
			if (wing && has_wing[e])
			{
				// is the sphere in the face region of the adjacent triangle (wing, E1, E0)?
				float w1[4];
				bary3(w1, wing[e], E1[e], E0[e], Q);
				if (w1[0] > 0.0f && w1[1] > 0.0f && w1[2] > 0.0f) return false;
			}
			n = tn;
			const float l = len3(d);
			if (l > kFltEps) n = f3(d.x / l, d.y / l, d.z / l);
			P = Pe;
			return true;
		}
	}
	// face region
	const float3 Pm = wABC[0] * A + wABC[1] * B + wABC[2] * C;
	const float3 Pf = f3(Pm.x / wABC[3], Pm.y / wABC[3], Pm.z / wABC[3]);
	return point_feature(Q, Pf, radius, tn, P, n);
}

// mesh_shape.cpp:87-124: the closest child-triangle manifold among the triangles whose mesh-frame
// AABB overlaps the sphere's query box (center in the unscaled mesh frame, radius unscaled)
__device__ __forceinline__ bool collide_mesh(const DevShape& S, float3 Q, float r1, float3& P, float3& n)
{
	const float3 cl0 = qrot(S.q, Q - f3p(S.t), -1.0f);
	const float3 c = f3(S.inv_scale[0] * cl0.x, S.inv_scale[1] * cl0.y, S.inv_scale[2] * cl0.z);
	const float qr = r1 + S.radius;
	float dd0 = 3.402823466e+38f;
	bool found = false;
	for (int k = 0; k < S.count; ++k)
	{
		const float* T = S.data + (size_t)kMeshTriFloats * k;
		if (c.x + qr < T[21] || c.x - qr > T[24] || c.y + qr < T[22] || c.y - qr > T[25] || c.z + qr < T[23] ||
		    c.z - qr > T[26])
			continue;
		const float3 wing[3] = {f3p(T + 9), f3p(T + 12), f3p(T + 15)};
		const bool has[3] = {T[18] != 0.0f, T[19] != 0.0f, T[20] != 0.0f};
		float3 Pk, nk;
		if (!collide_triangle(f3p(T), f3p(T + 3), f3p(T + 6), wing, has, S.radius, Q, r1, Pk, nk)) continue;
		const float3 d = Q - Pk;
		const float dd = dot3(d, d);
		if (dd < dd0)
		{
			dd0 = dd;
			P = Pk;
			n = nk;
			found = true;
		}
	}
	return found;
}

// voxel_grid.h:166-206 trilinear sample of the grid cell around point p (shape frame); grad
// also returns the interpolated gradient (differences across the cell)
__device__ __forceinline__ bool sdf_sample(const DevShape& S, float3 p, float& value, float3& grad)
{
	const float3 lo = f3p(S.glo), hi = f3p(S.ghi);
	const float3 dims = f3((float)(S.dims[0] - 1), (float)(S.dims[1] - 1), (float)(S.dims[2] - 1));
	const float3 ext = hi - lo;
	const float3 cs = f3(ext.x / dims.x, ext.y / dims.y, ext.z / dims.z);
	const float3 lp = p - lo;
	const int i = (int)floorf(lp.x / cs.x), j = (int)floorf(lp.y / cs.y), k = (int)floorf(lp.z / cs.z);
	if (i < 0 || i >= S.dims[0] - 1 || j < 0 || j >= S.dims[1] - 1 || k < 0 || k >= S.dims[2] - 1) return false;
	// regular_grid_indexer.h: the cell AABB from its center and half size
	const float3 half = 0.5f * cs;
	const float3 center = lo + f3(i * cs.x, j * cs.y, k * cs.z) + half;
	const float3 clo = center - half, chi = center + half;
	const float3 cd = chi - clo;
	const float3 rel = f3((p.x - clo.x) / cd.x, (p.y - clo.y) / cd.y, (p.z - clo.z) / cd.z);
	const int W = S.dims[0], H = S.dims[1];
	const float* V = S.data;
	auto vox = [&](int a, int b, int c) { return V[(size_t)a + (size_t)W * ((size_t)b + (size_t)H * (size_t)c)]; };
	const float v[8] = {vox(i, j, k),         vox(i, j, k + 1),     vox(i, j + 1, k),     vox(i, j + 1, k + 1),
	                    vox(i + 1, j, k),     vox(i + 1, j, k + 1), vox(i + 1, j + 1, k), vox(i + 1, j + 1, k + 1)};
	auto lerp = [](float x, float a, float b) { return (1.0f - x) * a + x * b; };
	auto interp = [&](float x, float y, float z) {
		x = fminf(fmaxf(x, 0.0f), 1.0f);
		y = fminf(fmaxf(y, 0.0f), 1.0f);
		z = fminf(fmaxf(z, 0.0f), 1.0f);
		const float c00 = lerp(x, v[0], v[4]), c10 = lerp(x, v[2], v[6]), c01 = lerp(x, v[1], v[5]),
		            c11 = lerp(x, v[3], v[7]);
		return lerp(z, lerp(y, c00, c10), lerp(y, c01, c11));
	};
	value = interp(rel.x, rel.y, rel.z);
	grad = f3(interp(1.0f, rel.y, rel.z) - interp(0.0f, rel.y, rel.z), interp(rel.x, 1.0f, rel.z) - interp(rel.x, 0.0f, rel.z),
	          interp(rel.x, rel.y, 1.0f) - interp(rel.x, rel.y, 0.0f));
	return true;
}

// sdf_shape.cpp:50-84
__device__ __forceinline__ bool collide_sdf(const DevShape& S, float3 Q, float r1, float3& P, float3& n)
{
	const float3 pl = qrot(S.q, Q - f3p(S.t), -1.0f);
	const float radius = r1 + S.radius;
	float dist;
	float3 g;
	if (!sdf_sample(S, pl, dist, g)) return false;
	if (S.invert) dist = -dist;
	if (dist > radius) return false;
	float3 nl = normalize3(g);
	if (S.invert) nl = -nl;
	n = qrot(S.q, nl);
	P = Q - dist * n;
	return true;
}

__device__ __forceinline__ bool world_collide(const DevShape& S, float3 Q, float r1, float3& P, float3& n)
{
	switch (S.type)
	{
	case B3G_SHAPE_SPHERE: return collide_sphere(S, Q, r1, P, n);
	case B3G_SHAPE_CAPSULE: return collide_capsule(S, Q, r1, P, n);
	case B3G_SHAPE_BOX: return collide_box(S, Q, r1, P, n);
	case B3G_SHAPE_TRIANGLE: return collide_triangle(f3p(S.a), f3p(S.b), f3p(S.c), nullptr, nullptr, S.radius, Q, r1, P, n);
	case B3G_SHAPE_MESH: return collide_mesh(S, Q, r1, P, n);
	case B3G_SHAPE_SDF: return collide_sdf(S, Q, r1, P, n);
	default: return false;
	}
}

// aabb.h:371 b3TestOverlap of the vertex sphere's AABB and the world fixture's AABB
__device__ __forceinline__ bool aabb_overlap(float3 p, float r, const DevShape& S)
{
	if (p.x + r < S.lo[0] || p.x - r > S.hi[0]) return false;
	if (p.y + r < S.lo[1] || p.y - r > S.hi[1]) return false;
	if (p.z + r < S.lo[2] || p.z - r > S.hi[2]) return false;
	return true;
}

template <class TV>
__device__ __forceinline__ TV* vp(void* p) { return (TV*)p; }

// p += u_a u_b^T: the outer-product sum of a slot whose tetrahedra share one ratio lambda / mu,
// which add_tet_blocks_uniform turns into that slot's block
__device__ __forceinline__ void add_outer(float p[9], float4 ua, float4 ub)
{
	const float A3[3] = {ua.x, ua.y, ua.z}, B3[3] = {ub.x, ub.y, ub.z};
#pragma unroll
	for (int r = 0; r < 3; ++r)
#pragma unroll
		for (int c = 0; c < 3; ++c) p[3 * r + c] += A3[r] * B3[c];
}

// The sum over a slot's tetrahedra of add_tet_block's blocks with one ratio for all, from their
// outer-product sum P = sum u_a u_b^T: ratio P + P^T + tr(P) I (the same sum, reassociated).
__device__ __forceinline__ void add_tet_blocks_uniform(float a[9], const float p[9], float ratio)
{
	const float tr = p[0] + p[4] + p[8];
#pragma unroll
	for (int r = 0; r < 3; ++r)
#pragma unroll
		for (int c = 0; c < 3; ++c) a[3 * r + c] += ratio * p[3 * r + c] + p[3 * c + r] + (r == c ? tr : 0.0f);
}

// Right-hand-side part of local vertex (code & 3) of the tetrahedron at position code >> 2.
template <class L>
__device__ __forceinline__ float3 tet_bc_part(const float* bc, size_t nt, uint32_t code)
{
	const float* p = bc + (code >> 2) + 3 * (code & 3u) * nt;
	return f3(L::ld(p), L::ld(p + nt), L::ld(p + 2 * nt));
}

// a += (h^2 + h kd) R K0_ab R^T of one tetrahedron from its factored record:
// ratio u_a u_b^T + u_b u_a^T + (u_a . u_b) I with u = sqrt(c mu) R g and ratio = lambda / mu
__device__ __forceinline__ void add_tet_block(float a[9], float4 ua, float4 ub)
{
	const float ratio = ua.w;
	const float uab = ua.x * ub.x + ua.y * ub.y + ua.z * ub.z;
	const float A3[3] = {ua.x, ua.y, ua.z}, B3[3] = {ub.x, ub.y, ub.z};
#pragma unroll
	for (int r = 0; r < 3; ++r)
#pragma unroll
		for (int c = 0; c < 3; ++c) a[3 * r + c] += ratio * A3[r] * B3[c] + B3[r] * A3[c] + (r == c ? uab : 0.0f);
}

// Filtered contacts (B3G_CONTACT_FILTER) of vertex i at the start of a step: the contact update
// of contact_manager.cpp:108-146, then the constraint of the first world shape (shape order) the
// vertex overlaps: n the shape's normal towards the vertex, zn = vt - v.n with vt the Baumgarte
// velocity min(0.2 C, 0.2) / h of the penalty force's depth C (sphere_shape_contact.cpp:98-126).
// The assembly then uses S_i = I - n n^T and z_i = zn n in pA = S A S^T + I - S,
// pb = S (b - A z), and the final update dv = y + z (sparse_force_solver.cpp:170-190, which the
// reference only ever calls with S = I or 0 and z = 0).
__device__ __forceinline__ void contact_filter_vertex(const DevBody& B, int i, float h)
{
	float4 f = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	const bool dyn = B.type[i] == B3G_DYNAMIC;
	const float3 x = ld3(B.x, i);
	const float r1 = B.srad[i];
	bool found = false;
	for (int k = 0; k < B.nw; ++k)
	{
		const int c = i * B.nw + k;
		const DevShape& sh = B.shapes[k];
		if (B.c_exists[c])
		{
			if (!dyn || !aabb_overlap(x, r1, sh)) B.c_exists[c] = 0;
			else
			{
				B.c_nf[c] = 0.0f;
				B.c_apply[c] = 0;
			}
		}
		if (found || !B.c_exists[c]) continue;
		float3 p2, n2;
		if (!world_collide(sh, x, r1, p2, n2)) continue;
		const float3 c1 = x - r1 * n2;
		const float3 c2 = p2 + sh.radius * n2;
		const float C = fminf(kBaumgarte * len3(c2 - c1), kMaxContactCorrection);
		f = make_float4(n2.x, n2.y, n2.z, C / h - dot3(ld3(B.v, i), n2));
		found = true;
	}
	B.filt[i] = f;
}

__device__ __forceinline__ bool filt_on(float4 f) { return f.x != 0.0f || f.y != 0.0f || f.z != 0.0f; }

// The end of row i's assembly once its right-hand side bi and diagonal block are final: pb,
// the Jacobi preconditioner and, when init_pcg is set, r = pb, s = d = M^-1 r and the zero
// initial guess; returns r.s (0 without init_pcg).
template <class TV>
__device__ __forceinline__ double row_finish(const DevBody& B, int i, float3 bi, const float diag[9], bool init_pcg)
{
	TV* pb = vp<TV>(B.pb);
	const TV bv[3] = {(TV)bi.x, (TV)bi.y, (TV)bi.z};
	vst(pb, i, bv);

	// preconditioner: scalar Jacobi (sparse_solver.cpp:38-55) as one 4-wide value, or the rows of
	// the inverted 3x3 diagonal block as three
	TV* Mv = vp<TV>(B.Minv);
	TV m3[9];
	if (B.precond == B3G_PRECOND_BLOCK_JACOBI)
	{
		double d0 = diag[0], d1 = diag[1], d2 = diag[2], d3 = diag[3], d4 = diag[4], d5 = diag[5], d6 = diag[6],
		       d7 = diag[7], d8 = diag[8];
		double c00 = d4 * d8 - d5 * d7, c01 = d2 * d7 - d1 * d8, c02 = d1 * d5 - d2 * d4;
		double c10 = d5 * d6 - d3 * d8, c11 = d0 * d8 - d2 * d6, c12 = d2 * d3 - d0 * d5;
		double c20 = d3 * d7 - d4 * d6, c21 = d1 * d6 - d0 * d7, c22 = d0 * d4 - d1 * d3;
		double det = d0 * c00 + d1 * c10 + d2 * c20;
		double id = 1.0 / det;
		double inv[9] = {c00 * id, c01 * id, c02 * id, c10 * id, c11 * id, c12 * id, c20 * id, c21 * id, c22 * id};
#pragma unroll
		for (int q = 0; q < 9; ++q) m3[q] = (TV)inv[q];
		vst(Mv, 3 * i, m3);
		vst(Mv, 3 * i + 1, m3 + 3);
		vst(Mv, 3 * i + 2, m3 + 6);
	}
	else
	{
		m3[0] = (TV)(1.0f / diag[0]);
		m3[4] = (TV)(1.0f / diag[4]);
		m3[8] = (TV)(1.0f / diag[8]);
		const TV md[3] = {m3[0], m3[4], m3[8]};
		vst(Mv, i, md);
	}
	if (!init_pcg) return 0.0;
	const TV r0 = bv[0], r1 = bv[1], r2 = bv[2];
	TV sv[3];
	if (B.precond == B3G_PRECOND_BLOCK_JACOBI)
	{
		sv[0] = m3[0] * r0 + m3[1] * r1 + m3[2] * r2;
		sv[1] = m3[3] * r0 + m3[4] * r1 + m3[5] * r2;
		sv[2] = m3[6] * r0 + m3[7] * r1 + m3[8] * r2;
	}
	else
	{
		sv[0] = m3[0] * r0;
		sv[1] = m3[4] * r1;
		sv[2] = m3[8] * r2;
	}
	const TV zero[3] = {0, 0, 0};
	vst(vp<TV>(B.r), i, bv);
	vst(vp<TV>(B.s), i, sv);
	vst(vp<TV>(B.d), i, sv);
	vst(vp<TV>(B.py), i, zero);
	if (B.xff)
	{
		const float z[3] = {0.0f, 0.0f, 0.0f};
		ff_st(B.xff, i, z, z);
	}
	return dot3<TV>(bv, sv);
}

// Assembles row i of the pre-filtered system: pA = S A S^T + I - S and pb = S b with
//   A = M - h dfdv - h^2 dfdx,  b = M (v0 - v) + h (fe + fi) + h dfdx (x0 - x + h v + y)
// (sparse_force_solver.cpp:165-174), S = I for dynamic vertices and 0 otherwise
// (force_solver.cpp:110-129). Also forms the Jacobi preconditioner and, when init_pcg is set
// (initial guess zero), r = pb, s = M^-1 r, d = s; returns this row's r.s. FILTER: filtered
// contacts (B.filt) replace the penalty contacts: S_i = I - n n^T for a constrained vertex and
// pb = S (b - A z), z nonzero in the first Newton iteration only.
// TETS: the body has tetrahedra only and no contact spheres (no explicit blocks or vectors, no
// contact terms), so those parts are compiled out: fewer registers, the same arithmetic.
template <class TA, class TV, class L = LdPlain, bool FILTER = false, bool TETS = false>
__device__ __forceinline__ double assemble_row(const DevBody& B, int slice, int lane, const StepParams& P,
                                               bool init_pcg)
{
	const int i = slice * kSlice + lane;
	if (i >= B.n) return 0.0;
	const float h = P.h;
	const int w = B.rowlen[i];
	const int base = B.slice_ptr[slice];
	const bool Si = B.type[i] == B3G_DYNAMIC;
	const float* X = P.first_newton ? B.x : B.xi;
	const float* Vv = P.first_newton ? B.v : B.vi;
	const float m = B.mass[i];
	const float Mi = Si ? m : 1.0f;
	const float damp = B.damping[i];
	float3 xi = ldl3<L>(X, i), vi = ldl3<L>(Vv, i), x0 = ldl3<L>(B.x, i), v0 = ldl3<L>(B.v, i), yi = ldl3<L>(B.trans, i);
	float3 wi = (x0 - xi) + h * vi + yi;

	// vertex terms of b: M (v0 - v) + h (fe + m g + damping force)
	float3 fe = ldl3<L>(B.fext, i);
	if (Si) fe = fe + m * f3(B.gravity[0], B.gravity[1], B.gravity[2]);
	float3 fi = f3(0, 0, 0);
	float diagExtra = Mi;
	if (damp > 0.0f)
	{
		fi = fi + (-damp * m) * vi;
		diagExtra += h * damp * m;
	}
	float Kc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	if (!FILTER && !TETS && B.contacts)
	{
		const float r1 = B.srad[i];
		for (int k = 0; k < B.nw; ++k)
		{
			const int c = i * B.nw + k;
			const DevShape& sh = B.shapes[k];
			if (P.first_newton)
			{
				// contact_manager.cpp:108-146 UpdateContacts at the start of the step
				if (B.c_exists[c])
				{
					if (!Si || !aabb_overlap(x0, r1, sh)) B.c_exists[c] = 0;
					else
					{
						B.c_nf[c] = 0.0f;
						B.c_apply[c] = 0;
					}
				}
			}
			if (!B.c_exists[c]) continue;
			float3 p2, n2;
			if (!world_collide(sh, xi, r1, p2, n2)) continue;
			if (!B.c_apply[c])
			{
				st3(B.c_normal, c, n2);
				B.c_apply[c] = 1;
			}
			// sphere_shape_contact.cpp:98-126
			float3 n1 = -n2;
			float3 c1 = xi + r1 * n1;
			float3 c2 = p2 + sh.radius * n2;
			float C = len3(c2 - c1);
			C = fminf(kBaumgarte * C, kMaxContactCorrection);
			float3 f1 = (-kContactStiffness * C) * n1;
			fi = fi + f1;
			float nn[3] = {n1.x, n1.y, n1.z};
#pragma unroll
			for (int r = 0; r < 3; ++r)
#pragma unroll
				for (int cc = 0; cc < 3; ++cc)
				{
					float o = nn[r] * nn[cc];
					// positive form of -K11 = 1000 (n n^T + C (I - n n^T))
					Kc[3 * r + cc] += kContactStiffness * (o + C * ((r == cc ? 1.0f : 0.0f) - o));
				}
			B.c_nf[c] += len3(f1);
		}
	}
	float3 bi = Mi * (v0 - vi) + h * (fe + fi);
	// contact dfdx w term: h dfdx w = -h Kc w
	if (!TETS) bi = bi - h * mv9(Kc, wi);
	const size_t nt = (size_t)B.nt;
	{
		// tetrahedra's right-hand-side parts of this vertex (code: position << 2 | local vertex),
		// four in flight at a time
		const uint32_t st = __ldg(B.vt_start + i);
		const int cnt = __ldg(B.vt_cnt + i);
		int t = 0;
		for (; t + 4 <= cnt; t += 4)
		{
			uint32_t e[4];
			float3 c[4];
#pragma unroll
			for (int u = 0; u < 4; ++u) e[u] = __ldg(B.vt_list + st + kSlice * (t + u));
#pragma unroll
			for (int u = 0; u < 4; ++u) c[u] = tet_bc_part<L>(B.tet_bc, nt, e[u]);
#pragma unroll
			for (int u = 0; u < 4; ++u) bi = bi + c[u];
		}
		for (; t < cnt; ++t) bi = bi + tet_bc_part<L>(B.tet_bc, nt, __ldg(B.vt_list + st + kSlice * t));
	}
	if (!TETS)
	{
		const uint32_t st = __ldg(B.vb_start + i);
		const int cnt = __ldg(B.vb_cnt + i);
		for (int t = 0; t < cnt; ++t)
		{
			uint32_t e = __ldg(B.vb_list + st + kSlice * t);
			float3 c = ldl3<L>(B.bvec, e >> 1);
			bi = (e & 1) ? bi - c : bi + c;
		}
	}

	float4 fi4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	if (FILTER) fi4 = B.filt[i];
	const bool ci = FILTER && Si && filt_on(fi4);
	float3 bz = f3(0.0f, 0.0f, 0.0f);  // (A z)_i

	float diag[9];
	// Slot pipeline: the next slot's list header and its first four tetrahedron codes load while
	// this slot's records are gathered, so a slot waits on one gather instead of three dependent
	// loads. Contributions are added in list order.
	uint32_t st_n = __ldg(B.tet_cstart + base + lane);
	int cnt_n = __ldg(B.tet_ccnt + base + lane);
	uint32_t cd_n[4];
#pragma unroll
	for (int u = 0; u < 4; ++u) cd_n[u] = u < cnt_n ? __ldg(B.tet_clist + st_n + kSlice * u) : 0u;
	for (int k = 0; k < w; ++k)
	{
		const int slot = base + k * kSlice + lane;           // contribution-list item
		const size_t bs = block_slot((size_t)base, k, lane); // block storage
		const int j = B.col[bs];
		const uint32_t st = st_n;
		const int cnt = cnt_n;
		uint32_t cd[4];
#pragma unroll
		for (int u = 0; u < 4; ++u) cd[u] = cd_n[u];
		if (k + 1 < w)
		{
			st_n = __ldg(B.tet_cstart + slot + kSlice);
			cnt_n = __ldg(B.tet_ccnt + slot + kSlice);
		}
		float a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
		{
			// uniform: every tetrahedron of the body has the same ratio, so the slot sums the
			// outer products u_a u_b^T (in a) and forms its block once at the end
			const bool uniform = B.tet_ratio >= 0.0f;
			float4 ua[4], ub[4];
#pragma unroll
			for (int u = 0; u < 4; ++u)
				if (u < cnt)
				{
					const float4* r0 = B.tet_rec + (cd[u] >> 4);
					ua[u] = L::ld(r0 + ((cd[u] >> 2) & 3u) * nt);
					ub[u] = L::ld(r0 + (cd[u] & 3u) * nt);
				}
			// the codes of the slot's next four contributions, while these records load
			uint32_t nx[4];
#pragma unroll
			for (int u = 0; u < 4; ++u) nx[u] = 4 + u < cnt ? __ldg(B.tet_clist + st + kSlice * (4 + u)) : 0u;
			if (k + 1 < w)
			{
#pragma unroll
				for (int u = 0; u < 4; ++u) cd_n[u] = u < cnt_n ? __ldg(B.tet_clist + st_n + kSlice * u) : 0u;
			}
			if (uniform)
			{
#pragma unroll
				for (int u = 0; u < 4; ++u)
					if (u < cnt) add_outer(a, ua[u], ub[u]);
			}
			else
			{
#pragma unroll
				for (int u = 0; u < 4; ++u)
					if (u < cnt) add_tet_block(a, ua[u], ub[u]);
			}
			// the rest of the slot's contributions, four in flight at a time (the last group
			// partial), each group's codes loaded with the group before
			for (int t = 4; t < cnt; t += 4)
			{
#pragma unroll
				for (int u = 0; u < 4; ++u)
					if (t + u < cnt)
					{
						const float4* r0 = B.tet_rec + (nx[u] >> 4);
						ua[u] = L::ld(r0 + ((nx[u] >> 2) & 3u) * nt);
						ub[u] = L::ld(r0 + (nx[u] & 3u) * nt);
					}
#pragma unroll
				for (int u = 0; u < 4; ++u) nx[u] = t + 4 + u < cnt ? __ldg(B.tet_clist + st + kSlice * (t + 4 + u)) : 0u;
				if (uniform)
				{
#pragma unroll
					for (int u = 0; u < 4; ++u)
						if (t + u < cnt) add_outer(a, ua[u], ub[u]);
				}
				else
				{
#pragma unroll
					for (int u = 0; u < 4; ++u)
						if (t + u < cnt) add_tet_block(a, ua[u], ub[u]);
				}
			}
			if (uniform)
			{
				float p[9];
#pragma unroll
				for (int q = 0; q < 9; ++q)
				{
					p[q] = a[q];
					a[q] = 0.0f;
				}
				add_tet_blocks_uniform(a, p, B.tet_ratio);
			}
		}
		const uint32_t bst = TETS ? 0u : __ldg(B.blk_cstart + slot);
		const int bcnt = TETS ? 0 : __ldg(B.blk_ccnt + slot);
		for (int t = 0; t < bcnt; ++t)
		{
			uint32_t code = __ldg(B.blk_clist + bst + kSlice * t);
			const float* blk = B.blocks + 9 * (size_t)(code >> 1);
			const float sgn = (code & 1) ? -1.0f : 1.0f;
#pragma unroll
			for (int q = 0; q < 9; ++q) a[q] += sgn * L::ld(blk + q);
		}
		const bool Sj = B.type[j] == B3G_DYNAMIC;
		if (FILTER)
		{
			if (k == 0)
			{
				a[0] += diagExtra;
				a[4] += diagExtra;
				a[8] += diagExtra;
			}
			const float4 fj = k == 0 ? fi4 : B.filt[j];
			const bool cj = filt_on(fj);
			// b - A z on the unfiltered block, then S_i A_ij S_j (+ n n^T = I - S_i on the diagonal)
			if (cj && P.first_newton) bz = bz + mv9(a, f3(fj.w * fj.x, fj.w * fj.y, fj.w * fj.z));
			if (Si && Sj)
			{
				const float nj[3] = {fj.x, fj.y, fj.z}, ni[3] = {fi4.x, fi4.y, fi4.z};
				if (cj)
#pragma unroll
					for (int r = 0; r < 3; ++r)
					{
						const float an = a[3 * r] * nj[0] + a[3 * r + 1] * nj[1] + a[3 * r + 2] * nj[2];
#pragma unroll
						for (int c = 0; c < 3; ++c) a[3 * r + c] -= an * nj[c];
					}
				if (ci)
				{
#pragma unroll
					for (int c = 0; c < 3; ++c)
					{
						const float na = ni[0] * a[c] + ni[1] * a[3 + c] + ni[2] * a[6 + c];
#pragma unroll
						for (int r = 0; r < 3; ++r) a[3 * r + c] -= ni[r] * na;
					}
					if (k == 0)
#pragma unroll
						for (int r = 0; r < 3; ++r)
#pragma unroll
							for (int c = 0; c < 3; ++c) a[3 * r + c] += ni[r] * ni[c];
				}
			}
		}
		if (k == 0)
		{
			if (!FILTER)
			{
				if (!TETS)
#pragma unroll
					for (int q = 0; q < 9; ++q) a[q] += h * h * Kc[q];
				a[0] += diagExtra;
				a[4] += diagExtra;
				a[8] += diagExtra;
			}
			if (!Si)
			{
#pragma unroll
				for (int q = 0; q < 9; ++q) a[q] = (q == 0 || q == 4 || q == 8) ? 1.0f : 0.0f;
			}
#pragma unroll
			for (int q = 0; q < 9; ++q) diag[q] = a[q];
		}
		else if (!(Si && Sj))
		{
#pragma unroll
			for (int q = 0; q < 9; ++q) a[q] = 0.0f;
		}
#pragma unroll
		for (int q = 0; q < 9; ++q) B.A32[(size_t)q * B.nslots + bs] = a[q];
		if (B.Alo)
		{
#pragma unroll
			for (int q = 0; q < 9; ++q) ((TA*)B.Alo)[(size_t)q * B.nslots + bs] = from_f<TA>(a[q]);
		}
	}
	if (!Si) bi = f3(0, 0, 0);
	else if (FILTER)
	{
		bi = bi - bz;
		if (ci) bi = bi - dot3(f3(fi4.x, fi4.y, fi4.z), bi) * f3(fi4.x, fi4.y, fi4.z);
	}
	return row_finish<TV>(B, i, bi, diag, init_pcg);
}

// Four consecutive blocks of one lane in one plane, widened to the arithmetic type.
template <class TA, class L>
__device__ __forceinline__ void load4(const TA* p, typename Acc<TA>::type o[4]);
template <>
__device__ __forceinline__ void load4<float, LdPlain>(const float* p, float o[4])
{
	const float4 t = *(const float4*)p;
	o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
}
template <>
__device__ __forceinline__ void load4<float, LdCG>(const float* p, float o[4])
{
	const float4 t = __ldcg((const float4*)p);
	o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
}
template <>
__device__ __forceinline__ void load4<double, LdPlain>(const double* p, double o[4])
{
	const double2 a = *(const double2*)p, b = *(const double2*)(p + 2);
	o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
template <>
__device__ __forceinline__ void load4<double, LdCG>(const double* p, double o[4])
{
	const double2 a = __ldcg((const double2*)p), b = __ldcg((const double2*)(p + 2));
	o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
__device__ __forceinline__ void unpack_bf16x4(uint2 t, float o[4])
{
	o[0] = __uint_as_float(t.x << 16);
	o[1] = __uint_as_float(t.x & 0xffff0000u);
	o[2] = __uint_as_float(t.y << 16);
	o[3] = __uint_as_float(t.y & 0xffff0000u);
}
template <>
__device__ __forceinline__ void load4<__nv_bfloat16, LdPlain>(const __nv_bfloat16* p, float o[4])
{
	unpack_bf16x4(*(const uint2*)p, o);
}
template <>
__device__ __forceinline__ void load4<__nv_bfloat16, LdCG>(const __nv_bfloat16* p, float o[4])
{
	unpack_bf16x4(__ldcg((const uint2*)p), o);
}

// four consecutive blocks' entries of one value plane (or their column ids) with a cache hint
template <class M>
__device__ __forceinline__ void hinted_load4(const float* p, float o[4], unsigned long long pol)
{
	const uint4 t = mat_ld16<M>(p, pol);
	o[0] = __uint_as_float(t.x); o[1] = __uint_as_float(t.y); o[2] = __uint_as_float(t.z); o[3] = __uint_as_float(t.w);
}
template <class M>
__device__ __forceinline__ void hinted_load4(const double* p, double o[4], unsigned long long pol)
{
	const uint4 a = mat_ld16<M>(p, pol), b = mat_ld16<M>(p + 2, pol);
	o[0] = __hiloint2double((int)a.y, (int)a.x); o[1] = __hiloint2double((int)a.w, (int)a.z);
	o[2] = __hiloint2double((int)b.y, (int)b.x); o[3] = __hiloint2double((int)b.w, (int)b.z);
}
template <class M>
__device__ __forceinline__ void hinted_load4(const __nv_bfloat16* p, float o[4], unsigned long long pol)
{
	unpack_bf16x4(mat_ld8<M>(p, pol), o);
}
template <class M>
__device__ __forceinline__ int4 hinted_cols(const int* p, unsigned long long pol)
{
	const uint4 v = mat_ld16<M>(p, pol);
	return make_int4((int)v.x, (int)v.y, (int)v.z, (int)v.w);
}

// dispatch on the matrix stream
template <class L, class TA, class AT>
__device__ __forceinline__ void mat_load4(const TA* p, AT o[4], unsigned long long, MatVia<L>*)
{
	load4<TA, L>(p, o);
}
template <class TA, class AT>
__device__ __forceinline__ void mat_load4(const TA* p, AT o[4], unsigned long long pol, MatNC*)
{
	hinted_load4<MatNC>(p, o, pol);
}
template <class TA, class AT>
__device__ __forceinline__ void mat_load4(const TA* p, AT o[4], unsigned long long pol, MatCG*)
{
	hinted_load4<MatCG>(p, o, pol);
}
template <class L>
__device__ __forceinline__ int4 mat_cols(const int* p, unsigned long long, MatVia<L>*)
{
	return __ldg((const int4*)p);  // column ids never change after creation
}
__device__ __forceinline__ int4 mat_cols(const int* p, unsigned long long pol, MatNC*) { return hinted_cols<MatNC>(p, pol); }
__device__ __forceinline__ int4 mat_cols(const int* p, unsigned long long pol, MatCG*) { return hinted_cols<MatCG>(p, pol); }

// q_i = (A x)_i for row i = 32 s + lane of a slice of width w (a multiple of 4). Per group of
// four blocks a lane issues one 16-byte load of column ids, one vector load per value plane and
// four 16-byte gathers of x, all before the first FMA. Padding blocks are zero.
template <class TA, class TV, class L = LdPlain, class M = MatNC>
__device__ __forceinline__ void spmv_row(const TA* A, const int* __restrict__ col, int nslots, int base, int w,
                                         int lane, const TV* x, TV out[3])
{
	typedef typename Acc<TA>::type AT;
	AT o0 = 0, o1 = 0, o2 = 0;
	const size_t ns = (size_t)nslots;
	const unsigned long long pol = evict_first_policy();
	for (int k = 0; k < w; k += kGroup)
	{
		const size_t off = block_slot((size_t)base, k, lane);
		const int4 jj = mat_cols(col + off, pol, (M*)nullptr);
		AT a[9][4];
#pragma unroll
		for (int p = 0; p < 9; ++p) mat_load4(A + p * ns + off, a[p], pol, (M*)nullptr);
		TV xv[4][3];
		vld<TV, L>(x, jj.x, xv[0]);
		vld<TV, L>(x, jj.y, xv[1]);
		vld<TV, L>(x, jj.z, xv[2]);
		vld<TV, L>(x, jj.w, xv[3]);
#pragma unroll
		for (int u = 0; u < 4; ++u)
		{
			const AT x0 = (AT)xv[u][0], x1 = (AT)xv[u][1], x2 = (AT)xv[u][2];
			o0 += a[0][u] * x0 + a[1][u] * x1 + a[2][u] * x2;
			o1 += a[3][u] * x0 + a[4][u] * x1 + a[5][u] * x2;
			o2 += a[6][u] * x0 + a[7][u] * x1 + a[8][u] * x2;
		}
	}
	out[0] = (TV)o0;
	out[1] = (TV)o1;
	out[2] = (TV)o2;
}

// (A x)_i in float-float for the refinement residual: FP32 blocks times the float-float
// solution, every product split into its float value and rounding error, summed in
// float-float. Returns hi + lo per component.
__device__ __forceinline__ void spmv_row_ff(const float* A, const int* __restrict__ col, int nslots, int base, int w,
                                            int lane, const float* xff, float ohi[3], float olo[3])
{
	float h0 = 0, h1 = 0, h2 = 0, l0 = 0, l1 = 0, l2 = 0;
	const size_t ns = (size_t)nslots;
	const unsigned long long pol = evict_first_policy();
	for (int k = 0; k < w; k += kGroup)
	{
		const size_t off = block_slot((size_t)base, k, lane);
		const int4 jj = mat_cols(col + off, pol, (MatNC*)nullptr);
		float a[9][4];
#pragma unroll
		for (int p = 0; p < 9; ++p) mat_load4(A + p * ns + off, a[p], pol, (MatNC*)nullptr);
		const int js[4] = {jj.x, jj.y, jj.z, jj.w};
#pragma unroll
		for (int u = 0; u < 4; ++u)
		{
			float xh[3], xl[3];
			ff_ld(xff, js[u], xh, xl);
#pragma unroll
			for (int c = 0; c < 3; ++c)
			{
				const float a0 = a[3 * 0 + c][u], a1 = a[3 * 1 + c][u], a2 = a[3 * 2 + c][u];
				// row 0, 1, 2 of the block times component c of x_j
				float p = __fmul_rn(a0, xh[c]);
				ff_add(h0, l0, p, fmaf(a0, xh[c], -p) + a0 * xl[c]);
				p = __fmul_rn(a1, xh[c]);
				ff_add(h1, l1, p, fmaf(a1, xh[c], -p) + a1 * xl[c]);
				p = __fmul_rn(a2, xh[c]);
				ff_add(h2, l2, p, fmaf(a2, xh[c], -p) + a2 * xl[c]);
			}
		}
	}
	ohi[0] = h0; ohi[1] = h1; ohi[2] = h2;
	olo[0] = l0; olo[1] = l1; olo[2] = l2;
}

// b - (hi + lo), rounded once to float
__device__ __forceinline__ float ff_residual(float b, float hi, float lo)
{
	float t, e;
	two_sum(b, -hi, t, e);
	return __fadd_rn(t, __fsub_rn(e, lo));
}

// The SpMV of a PCG iteration with the direction update folded in: q_i = (A d')_i with
// d' = s + beta d, the new direction, formed from the gathered s and d of every column
// (first iteration of a solve: d' = s). The diagonal block leads every row, so the first gathered
// column is the row itself and its d'_i is returned in dn. Every lane forms d'_j with the same
// expression as the owner of row j, so all copies of a value agree bitwise.
template <class TV, class L = LdPlain>
__device__ __forceinline__ void gather_dir(const TV* s, const TV* d, TV beta, bool first, int j, TV o[3])
{
	vld<TV, L>(s, j, o);
	if (first) return;
	TV dj[3];
	vld<TV, L>(d, j, dj);
#pragma unroll
	for (int c = 0; c < 3; ++c) o[c] = o[c] + beta * dj[c];
}

template <class TA, class TV, class L = LdPlain, class M = MatNC>
__device__ __forceinline__ void spmv_row_dir(const TA* A, const int* __restrict__ col, int nslots, int base, int w,
                                             int lane, const TV* s, const TV* d, TV beta, bool first, TV out[3],
                                             TV dn[3])
{
	typedef typename Acc<TA>::type AT;
	AT o0 = 0, o1 = 0, o2 = 0;
	const size_t ns = (size_t)nslots;
	const unsigned long long pol = evict_first_policy();
	for (int k = 0; k < w; k += kGroup)
	{
		const size_t off = block_slot((size_t)base, k, lane);
		const int4 jj = mat_cols(col + off, pol, (M*)nullptr);
		AT a[9][4];
#pragma unroll
		for (int p = 0; p < 9; ++p) mat_load4(A + p * ns + off, a[p], pol, (M*)nullptr);
		TV xv[4][3];
		gather_dir<TV, L>(s, d, beta, first, jj.x, xv[0]);
		gather_dir<TV, L>(s, d, beta, first, jj.y, xv[1]);
		gather_dir<TV, L>(s, d, beta, first, jj.z, xv[2]);
		gather_dir<TV, L>(s, d, beta, first, jj.w, xv[3]);
		if (k == 0)
		{
#pragma unroll
			for (int c = 0; c < 3; ++c) dn[c] = xv[0][c];
		}
#pragma unroll
		for (int u = 0; u < 4; ++u)
		{
			const AT x0 = (AT)xv[u][0], x1 = (AT)xv[u][1], x2 = (AT)xv[u][2];
			o0 += a[0][u] * x0 + a[1][u] * x1 + a[2][u] * x2;
			o1 += a[3][u] * x0 + a[4][u] * x1 + a[5][u] * x2;
			o2 += a[6][u] * x0 + a[7][u] * x1 + a[8][u] * x2;
		}
	}
	out[0] = (TV)o0;
	out[1] = (TV)o1;
	out[2] = (TV)o2;
}

// M^-1 r for one row (scalar or block Jacobi)
template <class TV, class L = LdPlain>
__device__ __forceinline__ void precond_row(const DevBody& B, int i, const TV r[3], TV s[3])
{
	const TV* M = (const TV*)B.Minv;
	if (B.precond == B3G_PRECOND_BLOCK_JACOBI)
	{
		TV m0[3], m1[3], m2[3];
		vld<TV, L>(M, 3 * i, m0);
		vld<TV, L>(M, 3 * i + 1, m1);
		vld<TV, L>(M, 3 * i + 2, m2);
		s[0] = m0[0] * r[0] + m0[1] * r[1] + m0[2] * r[2];
		s[1] = m1[0] * r[0] + m1[1] * r[1] + m1[2] * r[2];
		s[2] = m2[0] * r[0] + m2[1] * r[1] + m2[2] * r[2];
	}
	else
	{
		TV m[3];
		vld<TV, L>(M, i, m);
		s[0] = m[0] * r[0];
		s[1] = m[1] * r[1];
		s[2] = m[2] * r[2];
	}
}

// sphere_shape_contact.cpp:145-189 ApplyFriction for vertex i (velocity only)
__device__ __forceinline__ void apply_friction(const DevBody& B, int i, float h, float3& v)
{
	for (int k = 0; k < B.nw; ++k)
	{
		const int c = i * B.nw + k;
		if (!B.c_exists[c] || !B.c_apply[c]) continue;
		float3 normal = ld3(B.c_normal, c);
		float nf = B.c_nf[c];
		// vec3.h:255 b3Perp
		const float sqrt_inv3 = sqrtf(1.0f / 3.0f);
		float3 t1 = fabsf(normal.x) >= sqrt_inv3 ? f3(normal.y, -normal.x, 0.0f) : f3(0.0f, normal.z, -normal.y);
		t1 = normalize3(t1);
		float3 t2 = cross3(t1, normal);
		float im1 = B.invmass[i];
		float fr = sqrtf(B.sfric[i] * B.shapes[k].friction);
		float tm = im1 > 0.0f ? 1.0f / im1 : 0.0f;
		float cx = dot3(v, t1), cy = dot3(v, t2);
		float ix = tm * -cx, iy = tm * -cy;
		float maxImp = fr * (h * nf);
		if (ix * ix + iy * iy > maxImp * maxImp)
		{
			float l = sqrtf(ix * ix + iy * iy);
			if (l > kFltEps)
			{
				ix /= l;
				iy /= l;
			}
			ix *= maxImp;
			iy *= maxImp;
		}
		float3 Pimp = ix * t1 + iy * t2;
		v = v + im1 * Pimp;
	}
}

// contact_manager.cpp:65-82 FindNewContacts for vertex i at its new position
__device__ __forceinline__ void find_new_contacts(const DevBody& B, int i, float3 x)
{
	if (B.type[i] != B3G_DYNAMIC) return;
	for (int k = 0; k < B.nw; ++k)
	{
		const int c = i * B.nw + k;
		if (B.c_exists[c]) continue;
		if (aabb_overlap(x, B.srad[i], B.shapes[k]))
		{
			B.c_exists[c] = 1;
			B.c_nf[c] = 0.0f;
			B.c_apply[c] = 0;
		}
	}
}

// v = v + dv, x = x0 + h v + y (sparse_force_solver.cpp:194-200); returns |dv|^2 of the vertex.
// finish != 0 also ends the step: friction, clearing of external forces and translations, new
// contacts (body.cpp:572-603), and writes the state instead of the Newton iterate.
template <class TV, class L = LdPlain, bool FILTER = false>
__device__ __forceinline__ double final_vertex(const DevBody& B, int i, float h, bool first_newton, bool finish)
{
	float3 dv;
	if (B.xff)
	{
		float yh[3], yl[3];
		ff_ld(B.xff, i, yh, yl);
		dv = f3(yh[0] + yl[0], yh[1] + yl[1], yh[2] + yl[2]);
	}
	else
	{
		TV y3[3];
		vld<TV, L>((const TV*)B.py, i, y3);
		dv = f3((float)y3[0], (float)y3[1], (float)y3[2]);
	}
	if (FILTER && first_newton)
	{
		// dv = y + z (sparse_force_solver.cpp:187)
		const float4 f = B.filt[i];
		if (filt_on(f)) dv = dv + f.w * f3(f.x, f.y, f.z);
	}
	float3 v = ldl3<L>(first_newton ? B.v : B.vi, i) + dv;
	float3 x = ldl3<L>(B.x, i) + h * v + ldl3<L>(B.trans, i);
	if (finish)
	{
		if (B.contacts) apply_friction(B, i, h, v);
		st3(B.fext, i, f3(0, 0, 0));
		st3(B.trans, i, f3(0, 0, 0));
		if (B.contacts) find_new_contacts(B, i, x);
	}
	st3(finish ? B.x : B.xi, i, x);
	st3(finish ? B.v : B.vi, i, v);
	return (double)dv.x * dv.x + (double)dv.y * dv.y + (double)dv.z * dv.z;
}

// finish a multi-Newton step for vertex i: iterate -> state, friction, clearing, new contacts
template <class L = LdPlain>
__device__ __forceinline__ void post_vertex(const DevBody& B, int i, float h)
{
	float3 v = ldl3<L>(B.vi, i);
	float3 x = ldl3<L>(B.xi, i);
	if (B.contacts) apply_friction(B, i, h, v);
	st3(B.fext, i, f3(0, 0, 0));
	st3(B.trans, i, f3(0, 0, 0));
	if (B.contacts) find_new_contacts(B, i, x);
	st3(B.x, i, x);
	st3(B.v, i, v);
}

// ------------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

} // namespace b3g
