/*
 * ORACLE — test infrastructure only. Never linked into, loaded by or called from the product.
 *
 * A plain-C restatement of the reference's implicit body step, compiled for float
 * (-DB3O_DOUBLE absent: the reference's own `scalar`) and for double (the FP64 oracle).
 * Parity is pinned: tests compare this restatement with the reference library compiled from
 * its own sources (oracle/ref_harness.cpp) on the committed golden inputs.
 *
 * What it restates, with the reference file:line it follows:
 *   - b3Body::Step / Solve order                 src/bounce_softbody/dynamics/body.cpp:552-604
 *   - b3Body::ResetMass (lumped mass)            src/bounce_softbody/dynamics/body.cpp:394-466
 *   - pack / unpack, M, S, fe += m g             src/bounce_softbody/dynamics/force_solver.cpp:88-180
 *   - force model order particles/forces/contacts src/bounce_softbody/dynamics/force_solver.cpp:70-86
 *   - mass damping                               src/bounce_softbody/dynamics/particle.cpp:182-199
 *   - tetrahedron element (K0, rotation, forces) src/bounce_softbody/dynamics/forces/tetrahedron_element_force.cpp:37-464
 *   - triangle element                           src/bounce_softbody/dynamics/forces/triangle_element_force.cpp:30-468
 *   - spring                                     src/bounce_softbody/dynamics/forces/spring_force.cpp:61-143
 *   - stretch (Baraff-Witkin), (u, v) Initialize src/bounce_softbody/dynamics/forces/stretch_force.cpp:36-388
 *   - shear (Baraff-Witkin)                      src/bounce_softbody/dynamics/forces/shear_force.cpp:25-244
 *   - mouse spring                               src/bounce_softbody/dynamics/forces/mouse_force.cpp:25-245
 *   - body ray cast over triangle fixtures       src/bounce_softbody/dynamics/body.cpp:468-521,
 *                                                src/bounce_softbody/collision/shapes/triangle_shape.cpp:314-387
 *   - sphere contact force and friction          src/bounce_softbody/dynamics/contacts/sphere_shape_contact.cpp:53-189
 *   - sphere shape collide                       src/bounce_softbody/collision/shapes/sphere_shape.cpp:50-77
 *   - contact creation / destruction             src/bounce_softbody/dynamics/contact_manager.cpp:65-146
 *   - backward Euler with pre-filter             src/bounce_softbody/sparse/sparse_force_solver.cpp:104-232
 *   - Jacobi PCG, residual refresh every 50      src/bounce_softbody/sparse/sparse_solver.cpp:28-109
 *   - math (quaternion, basis, perp, adjugate)   include/bounce_softbody/common/math/{quat.h:63-146,mat33.h:276-327,vec3.h:255-270}
 *
 * One extension has no reference counterpart and so no reference pin: filtered contacts
 * (b3o_run.contact_mode 1, contact_filter below), which fills the pre-filter's general S and z
 * (sparse_force_solver.cpp:170-190) from the contacts instead of adding penalty springs; its tests
 * check its physics and hold the CUDA path to it.
 *
 * The reference keeps sparse matrices as linked lists; here they are CSR rows of 3x3 blocks
 * with a fixed pattern. Element order follows the reference's head-inserted force and fixture
 * lists (newest first). Sums over a row run in column order, so float results differ from the
 * reference only by summation order.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef B3O_DOUBLE
typedef double real;
#define B3O_EPS DBL_EPSILON
#else
typedef float real;
#define B3O_EPS FLT_EPSILON
#endif

/* settings.h:83-95 */
#define B3O_CONTACT_STIFFNESS ((real)1000.0)
#define B3O_MAX_CONTACT_LINEAR_CORRECTION ((real)0.2)
#define B3O_BAUMGARTE ((real)0.2)

typedef struct { real x, y, z; } v3;
typedef struct { v3 c[3]; } m33;   /* column-major, like b3Mat33 */
typedef struct { real x, y; } v2;
typedef struct { v2 c[2]; } m22;
typedef struct { v3 v; real s; } quat;

/* ------------------------------------------------------------------ small math */
static v3 V(real x, real y, real z) { v3 r = {x, y, z}; return r; }
static v3 add(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(real s, v3 a) { return V(s * a.x, s * a.y, s * a.z); }
static v3 neg(v3 a) { return V(-a.x, -a.y, -a.z); }
static real dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 cross(v3 a, v3 b) { return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static real len(v3 a) { return (real)sqrt((double)dot(a, a)); }
static real rsqrt_(real x) { return (real)sqrt((double)x); }
static v3 normalize(v3 a)
{
	real l = rsqrt_(a.x * a.x + a.y * a.y + a.z * a.z);
	if (l > B3O_EPS) { real s = (real)1 / l; a.x *= s; a.y *= s; a.z *= s; }
	return a;
}
static m33 M3(v3 a, v3 b, v3 c) { m33 m; m.c[0] = a; m.c[1] = b; m.c[2] = c; return m; }
static m33 mzero(void) { return M3(V(0, 0, 0), V(0, 0, 0), V(0, 0, 0)); }
static m33 mdiag(real s) { return M3(V(s, 0, 0), V(0, s, 0), V(0, 0, s)); }
static v3 mv(m33 A, v3 v) { return add(add(scl(v.x, A.c[0]), scl(v.y, A.c[1])), scl(v.z, A.c[2])); }
static m33 mm(m33 A, m33 B) { return M3(mv(A, B.c[0]), mv(A, B.c[1]), mv(A, B.c[2])); }
static m33 madd(m33 A, m33 B) { return M3(add(A.c[0], B.c[0]), add(A.c[1], B.c[1]), add(A.c[2], B.c[2])); }
static m33 msub(m33 A, m33 B) { return M3(sub(A.c[0], B.c[0]), sub(A.c[1], B.c[1]), sub(A.c[2], B.c[2])); }
static m33 mscl(real s, m33 A) { return M3(scl(s, A.c[0]), scl(s, A.c[1]), scl(s, A.c[2])); }
static m33 mtr(m33 A)
{
	return M3(V(A.c[0].x, A.c[1].x, A.c[2].x), V(A.c[0].y, A.c[1].y, A.c[2].y), V(A.c[0].z, A.c[1].z, A.c[2].z));
}
static m33 outer(v3 a, v3 b) { return M3(scl(b.x, a), scl(b.y, a), scl(b.z, a)); }
static real mget(const m33* A, int r, int c) { const real* p = &A->c[c].x; return p[r]; }
static void mset(m33* A, int r, int c, real s) { real* p = &A->c[c].x; p[r] = s; }
/* mat33.h:276 b3Adjugate = transpose(cofactor matrix) */
static m33 adjugate(m33 A) { return mtr(M3(cross(A.c[1], A.c[2]), cross(A.c[2], A.c[0]), cross(A.c[0], A.c[1]))); }
static real det3(v3 a, v3 b, v3 c) { return dot(a, cross(b, c)); }

static v2 V2(real x, real y) { v2 r = {x, y}; return r; }
static v2 add2(v2 a, v2 b) { return V2(a.x + b.x, a.y + b.y); }
static v2 sub2(v2 a, v2 b) { return V2(a.x - b.x, a.y - b.y); }
static v2 scl2(real s, v2 a) { return V2(s * a.x, s * a.y); }
static v2 mv2(m22 A, v2 v) { return add2(scl2(v.x, A.c[0]), scl2(v.y, A.c[1])); }
static m22 M2(v2 a, v2 b) { m22 m; m.c[0] = a; m.c[1] = b; return m; }
static m22 mm2(m22 A, m22 B) { return M2(mv2(A, B.c[0]), mv2(A, B.c[1])); }
static m22 mtr2(m22 A) { return M2(V2(A.c[0].x, A.c[1].x), V2(A.c[0].y, A.c[1].y)); }
static v2 normalize2(v2 a)
{
	real l = rsqrt_(a.x * a.x + a.y * a.y);
	if (l > B3O_EPS) { a.x /= l; a.y /= l; }
	return a;
}
static real sign_(real x) { return (real)((real)0 < x) - (real)(x < (real)0); }

/* quat.h:133 GetRotationMatrix */
static m33 qmat(quat q)
{
	real x = q.v.x, y = q.v.y, z = q.v.z, w = q.s;
	real x2 = x + x, y2 = y + y, z2 = z + z;
	real xx = x * x2, xy = x * y2, xz = x * z2;
	real yy = y * y2, yz = y * z2, zz = z * z2;
	real wx = w * x2, wy = w * y2, wz = w * z2;
	return M3(V((real)1 - (yy + zz), xy + wz, xz - wy),
	          V(xy - wz, (real)1 - (xx + zz), yz + wx),
	          V(xz + wy, yz - wx, (real)1 - (xx + yy)));
}
/* quat.h:204 b3Mul */
static quat qmul(quat a, quat b)
{
	quat r;
	r.v = add(add(cross(a.v, b.v), scl(a.s, b.v)), scl(b.s, a.v));
	r.s = a.s * b.s - dot(a.v, b.v);
	return r;
}
/* quat.h:63 Normalize */
static quat qnormalize(quat q)
{
	real l = rsqrt_(dot(q.v, q.v) + q.s * q.s);
	if (l > B3O_EPS) { q.v = V(q.v.x / l, q.v.y / l, q.v.z / l); q.s /= l; }
	return q;
}
/* quat.h:83 SetAxisAngle: sin/cos of the half angle (evaluated in double, like ::sin) */
static quat qaxisangle(v3 axis, real angle)
{
	real th = (real)0.5 * angle;
	quat q;
	q.v = scl((real)sin((double)th), axis);
	q.s = (real)cos((double)th);
	return q;
}
/* mat33.h:310 b3ComputeBasis */
static void compute_basis(v3 a, v3* b, v3* c)
{
	const real sqrt_inv3 = rsqrt_((real)1 / (real)3);
	if (fabs((double)a.x) >= sqrt_inv3) *b = V(a.y, -a.x, 0);
	else *b = V(0, a.z, -a.y);
	*b = normalize(*b);
	*c = cross(a, *b);
}
/* vec3.h:255 b3Perp */
static v3 perp(v3 v)
{
	const real sqrt_inv3 = rsqrt_((real)1 / (real)3);
	v3 u;
	if (fabs((double)v.x) >= sqrt_inv3) u = V(v.y, -v.x, 0);
	else u = V(0, v.z, -v.y);
	return normalize(u);
}

/* dense column-major products, math.h b3Mul / b3Transpose */
static void dmul(real* out, const real* A, int m, int n, const real* B, int n2, int p)
{
	(void)n2;
	for (int i = 0; i < m; ++i)
		for (int j = 0; j < p; ++j)
		{
			real s = 0;
			for (int k = 0; k < n; ++k) s += A[i + m * k] * B[k + n * j];
			out[i + m * j] = s;
		}
}
static void dtr(real* out, const real* A, int m, int n)
{
	for (int i = 0; i < m; ++i)
		for (int j = 0; j < n; ++j) out[j + n * i] = A[i + m * j];
}

/* ------------------------------------------------------------------ body */
/* A static world fixture's shape (the b3Shape types of collision/shapes/): p per type: sphere
 * center; capsule center1, center2; box half extents; triangle vertex1..3. */
typedef struct b3o_shape
{
	int32_t type; /* 0 sphere, 1 capsule, 2 box, 3 triangle, 4 mesh, 5 sdf */
	double radius, friction;
	double p[9];
	double rotation[4], translation[3], scale[3];
	uint32_t vertex_count;
	const double* vertices;
	uint32_t triangle_count;
	const uint32_t* triangles;
	const uint32_t* wings; /* null = all edges open */
	uint32_t grid[3];
	const double* voxels;
	double grid_lower[3], grid_upper[3];
	int32_t invert;
} b3o_shape;

typedef struct
{
	uint32_t n;
	const double *x, *v;
	const int32_t* type;
	const double* damping;
	uint32_t tet_count;
	const uint32_t* tets;
	const double *tet_rest, *tet_E, *tet_nu, *tet_kdamp, *tet_density;
	uint32_t tri_count;
	const uint32_t* tris;
	const double *tri_rest, *tri_Ex, *tri_Ey, *tri_Es, *tri_nuxy, *tri_nuyx, *tri_kdamp, *tri_density;
	uint32_t spring_count;
	const uint32_t* springs;
	const double *spring_L0, *spring_ks, *spring_kd;
	const double *sphere_radius, *sphere_friction;
	uint32_t world_sphere_count;
	const double* world_spheres;
	double gravity[3];
	uint32_t world_shape_count;
	const struct b3o_shape* world_shapes;
	/* cloth forces; uv null = Initialize from the initial positions */
	uint32_t stretch_count;
	const uint32_t* stretch_tris;
	const double *stretch_uv, *stretch_params; /* 6, 6 per force: ks_u, kd_u, b_u, ks_v, kd_v, b_v */
	uint32_t shear_count;
	const uint32_t* shear_tris;
	const double *shear_uv, *shear_params;     /* 6, 2 per force: ks, kd */
	uint32_t mouse_count;
	const uint32_t* mouse_ids;                 /* 4 per force */
	const double* mouse_params;                /* 6 per force: w2, w3, w4, ks, kd, length */
} b3o_desc;

/* a world shape in the restatement's precision; lo / hi is the fixture AABB */
typedef struct oshape
{
	int type;
	real radius, friction;
	v3 a, b, c;
	quat q;
	v3 t;
	v3 lo, hi;
	v3 inv_scale;
	int dims[3];
	int invert;
	v3 glo, ghi;
	uint32_t count;
	real* tri; /* mesh: 28 per triangle (vertices, wing vertices, wing flags, mesh-frame AABB) */
	real* vox; /* sdf */
} oshape;

static void shape_setup(oshape* S, const b3o_shape* W);

typedef struct
{
	uint32_t steps;
	double dt;
	uint32_t newton_iters;
	uint32_t max_sub;
	double sub_tol;
	int32_t use_body_step; /* unused here: the restatement always takes sub_tol */
	double* x_out;
	double* v_out;
	uint32_t* sub_iters_out;
	double* seconds_out;
	int32_t contact_mode; /* 0 penalty contacts (the reference), 1 filtered contacts */
} b3o_run;

enum { STATIC = 0, KINEMATIC = 1, DYNAMIC = 2 };

/* b3StretchForce / b3ShearForce members (stretch_force.h, shear_force.h) */
typedef struct bwforce
{
	uint32_t p[3];
	int shear;
	real alpha, inv_det, du1, dv1, du2, dv2;
	real dwudx[3], dwvdx[3];
	real ks_u, kd_u, b_u, ks_v, kd_v, b_v; /* shear: ks_u, kd_u */
	uint32_t slot[9];                      /* (row i, column j) at i + 3 j */
} bwforce;

/* b3MouseForce members (mouse_force.h) */
typedef struct mforce
{
	uint32_t p[4];
	real w2, w3, w4, ks, kd, L0;
	uint32_t slot[16];                     /* (row i, column j) at i + 4 j */
} mforce;

typedef struct
{
	uint32_t n;
	v3 *x, *v, *fext, *trans;
	int32_t* type;
	real *mass, *invmass, *damping;
	v3 gravity;

	uint32_t nt;
	uint32_t* tet;
	v3* tet_rest; /* 4 per tet */
	m33* invE;
	m33* K;       /* 16 per tet, K[i + 4j] */
	quat* q;
	real* tkd;

	uint32_t ntr;
	uint32_t* tri;
	v2* tri_x;    /* 3 per tri */
	m22* invS;
	m22* K2;      /* 9 per tri, K[i + 3j] */
	real* trkd;

	uint32_t ns;
	uint32_t* spr;
	real *L0, *ks, *kd;

	int tri_elements; /* 0: triangles are mass fixtures only */
	uint32_t nbw;     /* stretch forces first, then shear forces */
	uint32_t nst;
	struct bwforce* bw;
	uint32_t nms;
	struct mforce* ms;

	real *srad, *sfric;
	uint32_t nw;
	struct oshape* ws;
	/* contacts: one slot per (vertex, world fixture), index i*nw + k */
	uint8_t* c_exists;
	uint8_t* c_apply;
	real* c_normalForce;
	v3* c_normal;

	/* block pattern */
	uint32_t* rowptr;
	uint32_t* col;
	uint32_t nnzb;
	uint32_t* tet_slot; /* 16 per tet */
	uint32_t* tri_slot; /* 9 per tri */
	uint32_t* spr_slot; /* 4 per spring: 11, 12, 21, 22 */
	uint32_t* diag;

	m33 *dfdx, *dfdv, *A;
	v3 *x0, *v0, *fe, *y, *xx, *vv, *fi, *b, *pb, *py, *w, *tmp, *r, *d, *qv, *s, *Minv;
	real* Mval;  /* mass-matrix scalar per row */
	uint8_t* S;  /* 1 = free, 0 = constrained */
	uint32_t contacts_found;
	/* filtered contacts (contact_mode 1): per vertex a flag, the constrained normal n and the
	   normal velocity change zn of z = zn n */
	int contact_mode;
	uint8_t* fcons;
	v3* fn;
	real* fzn;
} body_t;

static void* xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s ? s : 1); }
static v3 D3(const double* p) { return V((real)p[0], (real)p[1], (real)p[2]); }

static int cmp_u64(const void* a, const void* b)
{
	uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
	return x < y ? -1 : (x > y ? 1 : 0);
}

static uint32_t find_slot(const body_t* B, uint32_t i, uint32_t j)
{
	uint32_t lo = B->rowptr[i], hi = B->rowptr[i + 1];
	while (lo < hi)
	{
		uint32_t mid = (lo + hi) >> 1;
		if (B->col[mid] < j) lo = mid + 1;
		else hi = mid;
	}
	return lo;
}

/* tetrahedron_element_force.cpp:219-265 ResetElementData */
static void tet_reset(body_t* B, uint32_t e, real E, real nu)
{
	v3 x1 = B->tet_rest[4 * e + 0], x2 = B->tet_rest[4 * e + 1];
	v3 x3 = B->tet_rest[4 * e + 2], x4 = B->tet_rest[4 * e + 3];
	v3 e1 = sub(x2, x1), e2 = sub(x3, x1), e3 = sub(x4, x1);
	m33 Em = M3(e1, e2, e3);
	real det = det3(e1, e2, e3);
	real Vol = (real)fabs((double)det) / (real)6;
	det = (real)1 / det;
	m33 invE = mscl(det, adjugate(Em));
	B->invE[e] = invE;

	real lambda = (nu * E) / (((real)1 + nu) * ((real)1 - (real)2 * nu));
	real mu = E / ((real)2 * ((real)1 + nu));
	real D[36] = {
		lambda + 2 * mu, lambda, lambda, 0, 0, 0,
		lambda, lambda + 2 * mu, lambda, 0, 0, 0,
		lambda, lambda, lambda + 2 * mu, 0, 0, 0,
		0, 0, 0, mu, 0, 0,
		0, 0, 0, 0, mu, 0,
		0, 0, 0, 0, 0, mu};
	real n2x = invE.c[0].x, n3x = invE.c[0].y, n4x = invE.c[0].z, n1x = -n2x - n3x - n4x;
	real n2y = invE.c[1].x, n3y = invE.c[1].y, n4y = invE.c[1].z, n1y = -n2y - n3y - n4y;
	real n2z = invE.c[2].x, n3z = invE.c[2].y, n4z = invE.c[2].z, n1z = -n2z - n3z - n4z;
	real Bm[72] = {
		n1x, 0, 0, n1y, 0, n1z,  0, n1y, 0, n1x, n1z, 0,  0, 0, n1z, 0, n1y, n1x,
		n2x, 0, 0, n2y, 0, n2z,  0, n2y, 0, n2x, n2z, 0,  0, 0, n2z, 0, n2y, n2x,
		n3x, 0, 0, n3y, 0, n3z,  0, n3y, 0, n3x, n3z, 0,  0, 0, n3z, 0, n3y, n3x,
		n4x, 0, 0, n4y, 0, n4z,  0, n4y, 0, n4x, n4z, 0,  0, 0, n4z, 0, n4y, n4x};
	real BT[72], BTD[72], K[144];
	dtr(BT, Bm, 6, 12);
	dmul(BTD, BT, 12, 6, D, 6, 6);
	dmul(K, BTD, 12, 6, Bm, 6, 12);
	for (int i = 0; i < 144; ++i) K[i] *= Vol;
	m33* Kb = B->K + 16 * e;
	for (int i = 0; i < 12; ++i)
		for (int j = 0; j < 12; ++j)
			mset(&Kb[(i / 3) + 4 * (j / 3)], i % 3, j % 3, K[i + 12 * j]);
}

/* triangle_element_force.cpp:208-279 ResetElementData */
static void tri_reset(body_t* B, uint32_t e, v3 p1, v3 p2, v3 p3, real Ex, real Ey, real Es, real nxy, real nyx)
{
	v3 n = normalize(cross(sub(p2, p1), sub(p3, p1)));
	v3 px, py;
	compute_basis(n, &px, &py);
	v2 x1 = V2(px.x * p1.x + px.y * p1.y + px.z * p1.z, py.x * p1.x + py.y * p1.y + py.z * p1.z);
	v2 x2 = V2(px.x * p2.x + px.y * p2.y + px.z * p2.z, py.x * p2.x + py.y * p2.y + py.z * p2.z);
	v2 x3 = V2(px.x * p3.x + px.y * p3.y + px.z * p3.z, py.x * p3.x + py.y * p3.y + py.z * p3.z);
	B->tri_x[3 * e + 0] = x1;
	B->tri_x[3 * e + 1] = x2;
	B->tri_x[3 * e + 2] = x3;
	v2 e1 = sub2(x2, x1), e2 = sub2(x3, x1);
	real det = e1.x * e2.y - e1.y * e2.x;
	real A = (real)0.5 * (real)fabs((double)det);
	/* triangle_element_force.cpp:260-265: the reference scales the adjugate by det itself (it
	 * does not divide by it, unlike the tetrahedron's invE), so its "invS" is det^2 S^-1. This is
	 * restated as written: the element's stiffness follows that matrix. mat22.h:194 adjugate. */
	m22 invS = M2(V2(det * e2.y, det * -e1.y), V2(det * -e2.x, det * e1.x));
	B->invS[e] = invS;
	real s = (real)1 - nxy * nyx;
	real C[9] = {Ex / s, Ey * nxy / s, 0, Ex * nyx / s, Ey / s, 0, 0, 0, Es};
	real n2x = invS.c[0].x, n3x = invS.c[0].y, n1x = -n2x - n3x;
	real n2y = invS.c[1].x, n3y = invS.c[1].y, n1y = -n2y - n3y;
	real Bm[18] = {n1x, 0, n1y, 0, n1y, n1x, n2x, 0, n2y, 0, n2y, n2x, n3x, 0, n3y, 0, n3y, n3x};
	real BT[18], BTC[18], K[36];
	dtr(BT, Bm, 3, 6);
	dmul(BTC, BT, 6, 3, C, 3, 3);
	dmul(K, BTC, 6, 3, Bm, 3, 6);
	for (int i = 0; i < 36; ++i) K[i] *= A;
	m22* Kb = B->K2 + 9 * e;
	for (int i = 0; i < 6; ++i)
		for (int j = 0; j < 6; ++j)
		{
			real* p = &Kb[(i / 2) + 3 * (j / 2)].c[j % 2].x;
			p[i % 2] = K[i + 6 * j];
		}
}

/* stretch_force.cpp:36-60 / shear_force.cpp:25-49 Initialize, then the constructors
 * (stretch_force.cpp:62-107, shear_force.cpp:51-92) */
static void bw_setup(bwforce* F, const uint32_t* ids, const double* uvin, const double* x, int shear, const double* par)
{
	real uv[6];
	for (int k = 0; k < 3; ++k) F->p[k] = ids[k];
	F->shear = shear;
	if (uvin)
		for (int k = 0; k < 6; ++k) uv[k] = (real)uvin[k];
	else
	{
		v3 A = D3(x + 3 * ids[0]), Bv = D3(x + 3 * ids[1]), C = D3(x + 3 * ids[2]);
		v3 AB = sub(Bv, A), AC = sub(C, A);
		uv[0] = 0;
		uv[1] = 0;
		uv[2] = len(AB);
		uv[3] = 0;
		v3 n_AB = V(AB.x / uv[2], AB.y / uv[2], AB.z / uv[2]); /* vec3.h:152-155: per component */
		real a2 = len(cross(AB, AC));
		uv[4] = dot(AC, n_AB);
		uv[5] = a2 / uv[2];
	}
	F->du1 = uv[2] - uv[0];
	F->dv1 = uv[3] - uv[1];
	F->du2 = uv[4] - uv[0];
	F->dv2 = uv[5] - uv[1];
	real det = F->du1 * F->dv2 - F->du2 * F->dv1;
	F->inv_det = (real)1 / det;
	F->dwudx[0] = F->inv_det * (F->dv1 - F->dv2);
	F->dwudx[1] = F->inv_det * F->dv2;
	F->dwudx[2] = -F->inv_det * F->dv1;
	F->dwvdx[0] = F->inv_det * (F->du2 - F->du1);
	F->dwvdx[1] = -F->inv_det * F->du2;
	F->dwvdx[2] = F->inv_det * F->du1;
	F->alpha = (real)0.5 * (det < 0 ? -det : det);
	F->ks_u = (real)par[0];
	F->kd_u = (real)par[1];
	if (!shear)
	{
		F->b_u = (real)par[2];
		F->ks_v = (real)par[3];
		F->kd_v = (real)par[4];
		F->b_v = (real)par[5];
	}
}

static void body_free(body_t* B);

static body_t* body_create(const b3o_desc* d)
{
	body_t* B = (body_t*)xcalloc(1, sizeof(body_t));
	uint32_t n = d->n;
	B->n = n;
	B->x = xcalloc(n, sizeof(v3));
	B->v = xcalloc(n, sizeof(v3));
	B->fext = xcalloc(n, sizeof(v3));
	B->trans = xcalloc(n, sizeof(v3));
	B->type = xcalloc(n, sizeof(int32_t));
	B->mass = xcalloc(n, sizeof(real));
	B->invmass = xcalloc(n, sizeof(real));
	B->damping = xcalloc(n, sizeof(real));
	B->gravity = D3(d->gravity);
	for (uint32_t i = 0; i < n; ++i)
	{
		B->x[i] = D3(d->x + 3 * i);
		B->v[i] = D3(d->v + 3 * i);
		B->type[i] = d->type[i];
		B->damping[i] = d->damping ? (real)d->damping[i] : 0;
		/* particle.cpp:40-49 constructor: dynamic particles start with unit mass */
		B->mass[i] = B->type[i] == DYNAMIC ? 1 : 0;
		B->invmass[i] = B->mass[i];
	}

	B->nt = d->tet_count;
	B->tet = xcalloc(4 * (size_t)B->nt, sizeof(uint32_t));
	B->tet_rest = xcalloc(4 * (size_t)B->nt, sizeof(v3));
	B->invE = xcalloc(B->nt, sizeof(m33));
	B->K = xcalloc(16 * (size_t)B->nt, sizeof(m33));
	B->q = xcalloc(B->nt, sizeof(quat));
	B->tkd = xcalloc(B->nt, sizeof(real));
	real* tvol = xcalloc(B->nt, sizeof(real));
	for (uint32_t e = 0; e < B->nt; ++e)
	{
		for (int k = 0; k < 4; ++k)
		{
			B->tet[4 * e + k] = d->tets[4 * e + k];
			B->tet_rest[4 * e + k] = d->tet_rest ? D3(d->tet_rest + 12 * e + 3 * k) : D3(d->x + 3 * d->tets[4 * e + k]);
		}
		B->q[e].v = V(0, 0, 0);
		B->q[e].s = 1;
		B->tkd[e] = d->tet_kdamp ? (real)d->tet_kdamp[e] : 0;
		tet_reset(B, e, (real)d->tet_E[e], (real)d->tet_nu[e]);
		/* tetrahedron_fixture.cpp:34-45 volume = sign(det) det / 6 */
		v3 a = B->tet_rest[4 * e], bb = B->tet_rest[4 * e + 1], c = B->tet_rest[4 * e + 2], dd = B->tet_rest[4 * e + 3];
		real det = det3(sub(bb, a), sub(c, a), sub(dd, a));
		tvol[e] = ((real)1 / (real)6) * sign_(det) * det;
	}

	B->ntr = d->tri_count;
	B->tri_elements = d->tri_Ex != NULL;
	B->tri = xcalloc(3 * (size_t)B->ntr, sizeof(uint32_t));
	B->tri_x = xcalloc(3 * (size_t)B->ntr, sizeof(v2));
	B->invS = xcalloc(B->ntr, sizeof(m22));
	B->K2 = xcalloc(9 * (size_t)B->ntr, sizeof(m22));
	B->trkd = xcalloc(B->ntr, sizeof(real));
	real* tarea = xcalloc(B->ntr, sizeof(real));
	for (uint32_t e = 0; e < B->ntr; ++e)
	{
		v3 p[3];
		for (int k = 0; k < 3; ++k)
		{
			B->tri[3 * e + k] = d->tris[3 * e + k];
			p[k] = d->tri_rest ? D3(d->tri_rest + 9 * e + 3 * k) : D3(d->x + 3 * d->tris[3 * e + k]);
		}
		B->trkd[e] = d->tri_kdamp ? (real)d->tri_kdamp[e] : 0;
		if (B->tri_elements)
			tri_reset(B, e, p[0], p[1], p[2], (real)d->tri_Ex[e], (real)d->tri_Ey[e], (real)d->tri_Es[e],
			          (real)d->tri_nuxy[e], (real)d->tri_nuyx[e]);
		/* triangle_fixture.cpp:33-36 area = |cross| / 2 */
		tarea[e] = (real)0.5 * len(cross(sub(p[1], p[0]), sub(p[2], p[0])));
	}

	B->ns = d->spring_count;
	B->spr = xcalloc(2 * (size_t)B->ns, sizeof(uint32_t));
	B->L0 = xcalloc(B->ns, sizeof(real));
	B->ks = xcalloc(B->ns, sizeof(real));
	B->kd = xcalloc(B->ns, sizeof(real));
	for (uint32_t e = 0; e < B->ns; ++e)
	{
		B->spr[2 * e] = d->springs[2 * e];
		B->spr[2 * e + 1] = d->springs[2 * e + 1];
		B->L0[e] = (real)d->spring_L0[e];
		B->ks[e] = (real)d->spring_ks[e];
		B->kd[e] = (real)d->spring_kd[e];
	}

	B->nst = d->stretch_count;
	B->nbw = d->stretch_count + d->shear_count;
	B->bw = xcalloc(B->nbw, sizeof(bwforce));
	for (uint32_t e = 0; e < B->nbw; ++e)
	{
		int shear = e >= B->nst;
		uint32_t k = shear ? e - B->nst : e;
		const uint32_t* ids = (shear ? d->shear_tris : d->stretch_tris) + 3 * k;
		const double* uv = shear ? d->shear_uv : d->stretch_uv;
		bw_setup(&B->bw[e], ids, uv ? uv + 6 * k : NULL, d->x, shear,
		         shear ? d->shear_params + 2 * k : d->stretch_params + 6 * k);
	}
	B->nms = d->mouse_count;
	B->ms = xcalloc(B->nms, sizeof(mforce));
	for (uint32_t e = 0; e < B->nms; ++e)
	{
		mforce* F = &B->ms[e];
		const double* c = d->mouse_params + 6 * e;
		for (int k = 0; k < 4; ++k) F->p[k] = d->mouse_ids[4 * e + k];
		F->w2 = (real)c[0];
		F->w3 = (real)c[1];
		F->w4 = (real)c[2];
		F->ks = (real)c[3];
		F->kd = (real)c[4];
		F->L0 = (real)c[5];
	}

	/* body.cpp:394-466 ResetMass, fixture lists walked newest first */
	for (uint32_t e = 0; e < B->ntr; ++e)
		for (int k = 0; k < 3; ++k) B->mass[B->tri[3 * e + k]] = 0;
	for (uint32_t e = 0; e < B->nt; ++e)
		for (int k = 0; k < 4; ++k) B->mass[B->tet[4 * e + k]] = 0;
	const real inv3 = (real)1 / (real)3, inv4 = (real)1 / (real)4;
	for (uint32_t e = B->ntr; e-- > 0;)
	{
		real m = (real)d->tri_density[e] * tarea[e];
		for (int k = 0; k < 3; ++k) B->mass[B->tri[3 * e + k]] += inv3 * m;
	}
	for (uint32_t e = B->nt; e-- > 0;)
	{
		real m = (real)d->tet_density[e] * tvol[e];
		for (int k = 0; k < 4; ++k) B->mass[B->tet[4 * e + k]] += inv4 * m;
	}
	for (uint32_t i = 0; i < n; ++i)
	{
		if (B->type[i] != DYNAMIC) { B->mass[i] = 0; B->invmass[i] = 0; continue; }
		if (B->mass[i] > 0) B->invmass[i] = (real)1 / B->mass[i];
		else { B->mass[i] = 1; B->invmass[i] = 1; }
	}
	free(tvol);
	free(tarea);

	if (d->sphere_radius)
	{
		B->srad = xcalloc(n, sizeof(real));
		B->sfric = xcalloc(n, sizeof(real));
		for (uint32_t i = 0; i < n; ++i)
		{
			B->srad[i] = (real)d->sphere_radius[i];
			B->sfric[i] = (real)d->sphere_friction[i];
		}
	}
	B->nw = d->world_sphere_count + d->world_shape_count;
	B->ws = xcalloc(B->nw ? B->nw : 1, sizeof(oshape));
	for (uint32_t k = 0; k < d->world_sphere_count; ++k)
	{
		b3o_shape sh;
		memset(&sh, 0, sizeof(sh));
		sh.type = 0;
		memcpy(sh.p, d->world_spheres + 5 * k, 3 * sizeof(double));
		sh.radius = d->world_spheres[5 * k + 3];
		sh.friction = d->world_spheres[5 * k + 4];
		sh.rotation[3] = 1;
		shape_setup(&B->ws[k], &sh);
	}
	for (uint32_t k = 0; k < d->world_shape_count; ++k) shape_setup(&B->ws[d->world_sphere_count + k], d->world_shapes + k);
	size_t nc = (size_t)n * (B->nw ? B->nw : 1);
	B->c_exists = xcalloc(nc, 1);
	B->c_apply = xcalloc(nc, 1);
	B->c_normalForce = xcalloc(nc, sizeof(real));
	B->c_normal = xcalloc(nc, sizeof(v3));

	/* block pattern: diagonal + every element pair */
	size_t npairs = (size_t)n + 16 * (size_t)B->nt + 9 * (size_t)B->ntr + 4 * (size_t)B->ns + 9 * (size_t)B->nbw +
	                16 * (size_t)B->nms;
	uint64_t* keys = xcalloc(npairs, sizeof(uint64_t));
	size_t kk = 0;
	for (uint32_t i = 0; i < n; ++i) keys[kk++] = ((uint64_t)i << 32) | i;
	for (uint32_t e = 0; e < B->nt; ++e)
		for (int a = 0; a < 4; ++a)
			for (int b = 0; b < 4; ++b) keys[kk++] = ((uint64_t)B->tet[4 * e + a] << 32) | B->tet[4 * e + b];
	for (uint32_t e = 0; e < B->ntr; ++e)
		for (int a = 0; a < 3; ++a)
			for (int b = 0; b < 3; ++b) keys[kk++] = ((uint64_t)B->tri[3 * e + a] << 32) | B->tri[3 * e + b];
	for (uint32_t e = 0; e < B->ns; ++e)
		for (int a = 0; a < 2; ++a)
			for (int b = 0; b < 2; ++b) keys[kk++] = ((uint64_t)B->spr[2 * e + a] << 32) | B->spr[2 * e + b];
	for (uint32_t e = 0; e < B->nbw; ++e)
		for (int a = 0; a < 3; ++a)
			for (int b = 0; b < 3; ++b) keys[kk++] = ((uint64_t)B->bw[e].p[a] << 32) | B->bw[e].p[b];
	for (uint32_t e = 0; e < B->nms; ++e)
		for (int a = 0; a < 4; ++a)
			for (int b = 0; b < 4; ++b) keys[kk++] = ((uint64_t)B->ms[e].p[a] << 32) | B->ms[e].p[b];
	qsort(keys, kk, sizeof(uint64_t), cmp_u64);
	size_t u = 0;
	for (size_t k = 0; k < kk; ++k)
		if (k == 0 || keys[k] != keys[u - 1]) keys[u++] = keys[k];
	B->nnzb = (uint32_t)u;
	B->rowptr = xcalloc(n + 1, sizeof(uint32_t));
	B->col = xcalloc(u, sizeof(uint32_t));
	for (size_t k = 0; k < u; ++k)
	{
		B->rowptr[(keys[k] >> 32) + 1]++;
		B->col[k] = (uint32_t)(keys[k] & 0xffffffffu);
	}
	for (uint32_t i = 0; i < n; ++i) B->rowptr[i + 1] += B->rowptr[i];
	free(keys);
	B->diag = xcalloc(n, sizeof(uint32_t));
	for (uint32_t i = 0; i < n; ++i) B->diag[i] = find_slot(B, i, i);
	B->tet_slot = xcalloc(16 * (size_t)B->nt, sizeof(uint32_t));
	for (uint32_t e = 0; e < B->nt; ++e)
		for (int a = 0; a < 4; ++a)
			for (int b = 0; b < 4; ++b)
				B->tet_slot[16 * e + a + 4 * b] = find_slot(B, B->tet[4 * e + a], B->tet[4 * e + b]);
	B->tri_slot = xcalloc(9 * (size_t)B->ntr, sizeof(uint32_t));
	for (uint32_t e = 0; e < B->ntr; ++e)
		for (int a = 0; a < 3; ++a)
			for (int b = 0; b < 3; ++b)
				B->tri_slot[9 * e + a + 3 * b] = find_slot(B, B->tri[3 * e + a], B->tri[3 * e + b]);
	B->spr_slot = xcalloc(4 * (size_t)B->ns, sizeof(uint32_t));
	for (uint32_t e = 0; e < B->ns; ++e)
	{
		uint32_t i1 = B->spr[2 * e], i2 = B->spr[2 * e + 1];
		B->spr_slot[4 * e + 0] = find_slot(B, i1, i1);
		B->spr_slot[4 * e + 1] = find_slot(B, i1, i2);
		B->spr_slot[4 * e + 2] = find_slot(B, i2, i1);
		B->spr_slot[4 * e + 3] = find_slot(B, i2, i2);
	}
	for (uint32_t e = 0; e < B->nbw; ++e)
		for (int a = 0; a < 3; ++a)
			for (int b = 0; b < 3; ++b) B->bw[e].slot[a + 3 * b] = find_slot(B, B->bw[e].p[a], B->bw[e].p[b]);
	for (uint32_t e = 0; e < B->nms; ++e)
		for (int a = 0; a < 4; ++a)
			for (int b = 0; b < 4; ++b) B->ms[e].slot[a + 4 * b] = find_slot(B, B->ms[e].p[a], B->ms[e].p[b]);

	B->dfdx = xcalloc(B->nnzb, sizeof(m33));
	B->dfdv = xcalloc(B->nnzb, sizeof(m33));
	B->A = xcalloc(B->nnzb, sizeof(m33));
	v3** vecs[] = {&B->x0, &B->v0, &B->fe, &B->y, &B->xx, &B->vv, &B->fi, &B->b, &B->pb, &B->py,
	               &B->w, &B->tmp, &B->r, &B->d, &B->qv, &B->s, &B->Minv};
	for (size_t k = 0; k < sizeof(vecs) / sizeof(vecs[0]); ++k) *vecs[k] = xcalloc(n, sizeof(v3));
	B->Mval = xcalloc(n, sizeof(real));
	B->S = xcalloc(n, 1);
	B->fcons = xcalloc(n, 1);
	B->fn = xcalloc(n, sizeof(v3));
	B->fzn = xcalloc(n, sizeof(real));
	return B;
}

static void body_free(body_t* B)
{
	if (!B) return;
	for (uint32_t k = 0; k < B->nw; ++k)
	{
		free(B->ws[k].tri);
		free(B->ws[k].vox);
	}
	free(B->ws);
	void* ptrs[] = {B->x, B->v, B->fext, B->trans, B->type, B->mass, B->invmass, B->damping, B->tet,
	                B->tet_rest, B->invE, B->K, B->q, B->tkd, B->tri, B->tri_x, B->invS, B->K2, B->trkd,
	                B->spr, B->L0, B->ks, B->kd, B->bw, B->ms, B->srad, B->sfric, B->c_exists,
	                B->c_apply, B->c_normalForce, B->c_normal, B->rowptr, B->col, B->tet_slot, B->tri_slot,
	                B->spr_slot, B->diag, B->dfdx, B->dfdv, B->A, B->x0, B->v0, B->fe, B->y, B->xx, B->vv,
	                B->fi, B->b, B->pb, B->py, B->w, B->tmp, B->r, B->d, B->qv, B->s, B->Minv, B->Mval, B->S,
	                B->fcons, B->fn, B->fzn};
	for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); ++k) free(ptrs[k]);
	free(B);
}

/* ------------------------------------------------------------------ force model */
/* tetrahedron_element_force.cpp:273-311 b3ExtractRotation */
static quat extract_rotation(m33 A, quat q0)
{
	quat q = q0;
	for (uint32_t it = 0; it < 32; ++it)
	{
		m33 R = qmat(q);
		real den = (real)fabs((double)(dot(R.c[0], A.c[0]) + dot(R.c[1], A.c[1]) + dot(R.c[2], A.c[2])));
		if (den == 0) break;
		v3 torque = add(add(cross(R.c[0], A.c[0]), cross(R.c[1], A.c[1])), cross(R.c[2], A.c[2]));
		const real kTol = (real)1.0e-9;
		real inv_den = (real)1 / den + kTol;
		v3 omega = scl(inv_den, torque);
		real w = len(omega);
		if (w < kTol) break;
		quat qw = qaxisangle(V(omega.x / w, omega.y / w, omega.z / w), w);
		q = qnormalize(qmul(qw, q));
	}
	return q;
}

/* tetrahedron_element_force.cpp:313-464 */
static void tet_apply(body_t* B, uint32_t e)
{
	const uint32_t* is = B->tet + 4 * e;
	v3 p[4], vel[4];
	for (int k = 0; k < 4; ++k) { p[k] = B->xx[is[k]]; vel[k] = B->vv[is[k]]; }
	m33 Em = M3(sub(p[1], p[0]), sub(p[2], p[0]), sub(p[3], p[0]));
	m33 F = mm(Em, B->invE[e]);
	quat q = extract_rotation(F, B->q[e]);
	B->q[e] = q;
	m33 R = qmat(q), RT = mtr(R);
	const m33* K0 = B->K + 16 * e;
	m33 K[16];
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j) K[i + 4 * j] = mm(mm(R, K0[i + 4 * j]), RT);
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j)
		{
			uint32_t s = B->tet_slot[16 * e + i + 4 * j];
			B->dfdx[s] = msub(B->dfdx[s], K[i + 4 * j]);
		}
	v3 us[4], fs[4];
	for (int k = 0; k < 4; ++k) us[k] = sub(mv(RT, p[k]), B->tet_rest[4 * e + k]);
	for (int i = 0; i < 4; ++i)
	{
		fs[i] = V(0, 0, 0);
		for (int j = 0; j < 4; ++j) fs[i] = add(fs[i], mv(K0[i + 4 * j], us[j]));
	}
	for (int i = 0; i < 4; ++i) B->fi[is[i]] = sub(B->fi[is[i]], mv(R, fs[i]));
	real kd = B->tkd[e];
	if (kd > 0)
	{
		v3 fds[4];
		for (int i = 0; i < 4; ++i)
		{
			fds[i] = V(0, 0, 0);
			for (int j = 0; j < 4; ++j) fds[i] = add(fds[i], mv(mscl(kd, K[i + 4 * j]), vel[j]));
		}
		for (int i = 0; i < 4; ++i) B->fi[is[i]] = sub(B->fi[is[i]], fds[i]);
		for (int i = 0; i < 4; ++i)
			for (int j = 0; j < 4; ++j)
			{
				uint32_t s = B->tet_slot[16 * e + i + 4 * j];
				B->dfdv[s] = msub(B->dfdv[s], mscl(kd, K[i + 4 * j]));
			}
	}
}

/* triangle_element_force.cpp:131-150 polar decomposition (Shoemake-Duff) */
static m22 polar2(m22 M)
{
	real m11 = M.c[0].x, m12 = M.c[1].x, m21 = M.c[0].y, m22v = M.c[1].y;
	real det = m11 * m22v - m12 * m21;
	m22 A = M2(V2(M.c[1].y, -M.c[1].x), V2(-M.c[0].y, M.c[0].x));
	real sg = sign_(det);
	m22 Q = M2(add2(M.c[0], scl2(sg, A.c[0])), add2(M.c[1], scl2(sg, A.c[1])));
	Q.c[0] = normalize2(Q.c[0]);
	Q.c[1] = normalize2(Q.c[1]);
	return Q;
}

/* triangle_element_force.cpp:285-468 */
static void tri_apply(body_t* B, uint32_t e)
{
	const uint32_t* is = B->tri + 3 * e;
	v3 p1 = B->xx[is[0]], p2 = B->xx[is[1]], p3 = B->xx[is[2]];
	v3 vel[3] = {B->vv[is[0]], B->vv[is[1]], B->vv[is[2]]};
	v3 n = normalize(cross(sub(p2, p1), sub(p3, p1)));
	v3 px, py;
	compute_basis(n, &px, &py);
	real P[6] = {px.x, py.x, px.y, py.y, px.z, py.z};   /* 2x3 */
	real PT[6] = {px.x, px.y, px.z, py.x, py.y, py.z};  /* 3x2 */
	v2 x1, x2, x3;
	dmul(&x1.x, P, 2, 3, &p1.x, 3, 1);
	dmul(&x2.x, P, 2, 3, &p2.x, 3, 1);
	dmul(&x3.x, P, 2, 3, &p3.x, 3, 1);
	m22 T = M2(sub2(x2, x1), sub2(x3, x1));
	m22 F = mm2(T, B->invS[e]);
	m22 R = polar2(F), RT = mtr2(R);
	v2 us[3];
	us[0] = sub2(mv2(RT, x1), B->tri_x[3 * e + 0]);
	us[1] = sub2(mv2(RT, x2), B->tri_x[3 * e + 1]);
	us[2] = sub2(mv2(RT, x3), B->tri_x[3 * e + 2]);
	const m22* K0 = B->K2 + 9 * e;
	v2 fs[3];
	for (int i = 0; i < 3; ++i)
	{
		fs[i] = V2(0, 0);
		for (int j = 0; j < 3; ++j) fs[i] = add2(fs[i], mv2(K0[i + 3 * j], us[j]));
	}
	for (int i = 0; i < 3; ++i) fs[i] = mv2(R, fs[i]);
	for (int i = 0; i < 3; ++i)
	{
		v3 f;
		dmul(&f.x, PT, 3, 2, &fs[i].x, 2, 1);
		B->fi[is[i]] = sub(B->fi[is[i]], f);
	}
	m33 K[9];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
		{
			m22 k = mm2(mm2(R, K0[i + 3 * j]), RT);
			real PTk[6];
			dmul(PTk, PT, 3, 2, &k.c[0].x, 2, 2);
			m33 Ke;
			dmul(&Ke.c[0].x, PTk, 3, 2, P, 2, 3);
			K[i + 3 * j] = Ke;
		}
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
		{
			uint32_t s = B->tri_slot[9 * e + i + 3 * j];
			B->dfdx[s] = msub(B->dfdx[s], K[i + 3 * j]);
		}
	real kd = B->trkd[e];
	if (kd > 0)
	{
		v3 fds[3];
		for (int i = 0; i < 3; ++i)
		{
			fds[i] = V(0, 0, 0);
			for (int j = 0; j < 3; ++j) fds[i] = add(fds[i], mv(mscl(kd, K[i + 3 * j]), vel[j]));
		}
		for (int i = 0; i < 3; ++i) B->fi[is[i]] = sub(B->fi[is[i]], fds[i]);
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j)
			{
				uint32_t s = B->tri_slot[9 * e + i + 3 * j];
				B->dfdv[s] = msub(B->dfdv[s], mscl(kd, K[i + 3 * j]));
			}
	}
}

/* spring_force.cpp:61-143 (the stiffness Jacobian uses the unnormalised dx, as there) */
static void spring_apply(body_t* B, uint32_t e)
{
	uint32_t i1 = B->spr[2 * e], i2 = B->spr[2 * e + 1];
	v3 x1 = B->xx[i1], v1 = B->vv[i1], x2 = B->xx[i2], v2v = B->vv[i2];
	m33 I = mdiag(1);
	v3 dx = sub(x1, x2);
	real L = len(dx);
	if (!(L > 0)) return;
	v3 n = V(dx.x / L, dx.y / L, dx.z / L);
	real ks = B->ks[e], kd = B->kd[e], L0 = B->L0[e];
	const uint32_t* sl = B->spr_slot + 4 * e;
	if (ks > 0 && L > L0)
	{
		real Cc = L - L0;
		v3 f1 = scl(-ks * Cc, n);
		B->fi[i1] = add(B->fi[i1], f1);
		B->fi[i2] = add(B->fi[i2], neg(f1));
		m33 K11 = mscl(-ks, madd(outer(dx, dx), mscl((real)1 - L0 / L, msub(I, outer(dx, dx)))));
		m33 K12 = mscl(-1, K11);
		B->dfdx[sl[0]] = madd(B->dfdx[sl[0]], K11);
		B->dfdx[sl[1]] = madd(B->dfdx[sl[1]], K12);
		B->dfdx[sl[2]] = madd(B->dfdx[sl[2]], K12);
		B->dfdx[sl[3]] = madd(B->dfdx[sl[3]], K11);
	}
	if (kd > 0)
	{
		real dCdt = dot(n, sub(v1, v2v));
		v3 f1 = scl(-kd * dCdt, n);
		B->fi[i1] = add(B->fi[i1], f1);
		B->fi[i2] = add(B->fi[i2], neg(f1));
		m33 K11 = mscl(-kd, outer(n, n));
		m33 K12 = mscl(-1, K11);
		B->dfdv[sl[0]] = madd(B->dfdv[sl[0]], K11);
		B->dfdv[sl[1]] = madd(B->dfdv[sl[1]], K12);
		B->dfdv[sl[2]] = madd(B->dfdv[sl[2]], K12);
		B->dfdv[sl[3]] = madd(B->dfdv[sl[3]], K11);
	}
}

/* one direction of stretch_force.cpp:121-388: the u part (142-270) with g = dwu/dx, or the v part */
static void stretch_dir(body_t* B, const bwforce* F, v3 w, const real* g, real ks, real kd, real b, const v3* vs)
{
	real L = len(w);
	if (!(L > 0)) return;
	real inv_len = (real)1 / L;
	v3 n = scl(inv_len, w);
	m33 I = mdiag(1);
	v3 dC[3];
	for (int i = 0; i < 3; ++i) dC[i] = scl(F->alpha * g[i], n);
	if (ks > 0)
	{
		real C = F->alpha * (L - b);
		for (int i = 0; i < 3; ++i) B->fi[F->p[i]] = add(B->fi[F->p[i]], scl(-ks * C, dC[i]));
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j)
			{
				m33 K = outer(dC[i], dC[j]);
				if (L > b) /* only while the eigenvalues stay positive */
					K = madd(K, mscl(C, mscl(F->alpha * inv_len * g[i] * g[j], msub(I, outer(n, n)))));
				uint32_t s = F->slot[i + 3 * j];
				B->dfdx[s] = madd(B->dfdx[s], mscl(-ks, K));
			}
	}
	if (kd > 0)
	{
		real dCdt = 0;
		for (int i = 0; i < 3; ++i) dCdt += dot(dC[i], vs[i]);
		for (int i = 0; i < 3; ++i) B->fi[F->p[i]] = add(B->fi[F->p[i]], scl(-kd * dCdt, dC[i]));
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j)
			{
				uint32_t s = F->slot[i + 3 * j];
				B->dfdv[s] = madd(B->dfdv[s], mscl(-kd, outer(dC[i], dC[j])));
			}
	}
}

/* w_u and w_v of a (u, v) triangle: the deformation's columns (stretch_force.cpp:157-161) */
static void bw_frame(const body_t* B, const bwforce* F, v3* wu, v3* wv, v3* vs)
{
	v3 x1 = B->xx[F->p[0]], x2 = B->xx[F->p[1]], x3 = B->xx[F->p[2]];
	for (int k = 0; k < 3; ++k) vs[k] = B->vv[F->p[k]];
	v3 dx1 = sub(x2, x1), dx2 = sub(x3, x1);
	*wu = scl(F->inv_det, sub(scl(F->dv2, dx1), scl(F->dv1, dx2)));
	*wv = scl(F->inv_det, add(scl(-F->du2, dx1), scl(F->du1, dx2)));
}

/* stretch_force.cpp:121-388 */
static void stretch_apply(body_t* B, const bwforce* F)
{
	v3 wu, wv, vs[3];
	bw_frame(B, F, &wu, &wv, vs);
	stretch_dir(B, F, wu, F->dwudx, F->ks_u, F->kd_u, F->b_u, vs);
	stretch_dir(B, F, wv, F->dwvdx, F->ks_v, F->kd_v, F->b_v, vs);
}

/* shear_force.cpp:106-244: C = alpha w_u . w_v, Jacobian without the second-derivative term */
static void shear_apply(body_t* B, const bwforce* F)
{
	v3 wu, wv, vs[3], dC[3];
	bw_frame(B, F, &wu, &wv, vs);
	for (int i = 0; i < 3; ++i) dC[i] = scl(F->alpha, add(scl(F->dwudx[i], wv), scl(F->dwvdx[i], wu)));
	real ks = F->ks_u, kd = F->kd_u;
	if (ks > 0)
	{
		real C = F->alpha * dot(wu, wv);
		for (int i = 0; i < 3; ++i) B->fi[F->p[i]] = add(B->fi[F->p[i]], scl(-ks * C, dC[i]));
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j)
			{
				uint32_t s = F->slot[i + 3 * j];
				B->dfdx[s] = madd(B->dfdx[s], mscl(-ks, outer(dC[i], dC[j])));
			}
	}
	if (kd > 0)
	{
		real dCdt = 0;
		for (int i = 0; i < 3; ++i) dCdt += dot(dC[i], vs[i]);
		for (int i = 0; i < 3; ++i) B->fi[F->p[i]] = add(B->fi[F->p[i]], scl(-kd * dCdt, dC[i]));
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j)
			{
				uint32_t s = F->slot[i + 3 * j];
				B->dfdv[s] = madd(B->dfdv[s], mscl(-kd, outer(dC[i], dC[j])));
			}
	}
}

/* mouse_force.cpp:58-245. The second derivatives d2C/dx_i dx_j are c_i c_j (I / L - d d^T / L^3)
 * with c = (1, -w2, -w3, -w4); the reference's table of +-w products times A and B = -A is that
 * matrix entry for entry. */
static void mouse_apply(body_t* B, const mforce* F)
{
	v3 x[4], v[4];
	for (int k = 0; k < 4; ++k)
	{
		x[k] = B->xx[F->p[k]];
		v[k] = B->vv[F->p[k]];
	}
	v3 c2 = add(add(scl(F->w2, x[1]), scl(F->w3, x[2])), scl(F->w4, x[3]));
	v3 d = sub(x[0], c2);
	real L = len(d);
	if (!(L > 0)) return;
	real inv_L = (real)1 / L;
	v3 n = scl(inv_L, d);
	const real cw[4] = {1, -F->w2, -F->w3, -F->w4};
	v3 dC[4];
	dC[0] = n;
	for (int i = 1; i < 4; ++i) dC[i] = scl(cw[i], n);
	if (F->ks > 0 && L > F->L0)
	{
		real C = L - F->L0;
		for (int i = 0; i < 4; ++i) B->fi[F->p[i]] = add(B->fi[F->p[i]], scl(-F->ks * C, dC[i]));
		real L3 = L * L * L;
		real inv_L3 = L3 > 0 ? (real)1 / L3 : 0;
		m33 A = msub(mdiag(inv_L), mscl(inv_L3, outer(d, d)));
		for (int i = 0; i < 4; ++i)
			for (int j = 0; j < 4; ++j)
			{
				m33 K = mscl(-F->ks, madd(outer(dC[i], dC[j]), mscl(C, mscl(cw[i] * cw[j], A))));
				uint32_t s = F->slot[i + 4 * j];
				B->dfdx[s] = madd(B->dfdx[s], K);
			}
	}
	if (F->kd > 0)
	{
		v3 vc2 = add(add(scl(F->w2, v[1]), scl(F->w3, v[2])), scl(F->w4, v[3]));
		real dCdt = dot(sub(v[0], vc2), n);
		for (int i = 0; i < 4; ++i) B->fi[F->p[i]] = add(B->fi[F->p[i]], scl(-F->kd * dCdt, dC[i]));
		for (int i = 0; i < 4; ++i)
			for (int j = 0; j < 4; ++j)
			{
				uint32_t s = F->slot[i + 4 * j];
				B->dfdv[s] = madd(B->dfdv[s], mscl(-F->kd, outer(dC[i], dC[j])));
			}
	}
}

/* ------------------------------------------------------------------ world shapes */
/* quat.h:75-79 b3Quat::Rotate; sign -1 rotates by the conjugate (b3MulC) */
static v3 qrot(quat q, v3 v, real sign)
{
	v3 u = scl(sign, q.v);
	v3 t = scl(2, cross(u, v));
	return add(add(v, scl(q.s, t)), cross(u, t));
}
static v3 vmin3(v3 a, v3 b) { return V(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z); }
static v3 vmax3(v3 a, v3 b) { return V(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z); }
static v3 vdiv(v3 a, real s) { return V(a.x / s, a.y / s, a.z / s); }
static v3 P3(const double* p) { return V((real)p[0], (real)p[1], (real)p[2]); }
static v3 xform(const oshape* S, v3 v) { return add(qrot(S->q, v, 1), S->t); }

/* settings.h:70 B3_LINEAR_SLOP */
#define B3O_LINEAR_SLOP ((real)0.005)
#define B3O_NULL_VERTEX 0xFFFFFFFFu

/* the fixture AABBs of the shapes' ComputeAABB, mesh triangles in world space with their wing
 * vertices and mesh-frame AABBs (mesh.h:102-117), SDF voxels */
static void shape_setup(oshape* S, const b3o_shape* W)
{
	memset(S, 0, sizeof(*S));
	S->type = W->type;
	S->radius = (real)W->radius;
	S->friction = (real)W->friction;
	S->a = P3(W->p);
	S->b = P3(W->p + 3);
	S->c = P3(W->p + 6);
	S->q.v = P3(W->rotation);
	S->q.s = (real)W->rotation[3];
	S->t = P3(W->translation);
	v3 r = V(S->radius, S->radius, S->radius);
	v3 lo = V(0, 0, 0), hi = V(0, 0, 0);
	switch (W->type)
	{
	case 0: lo = sub(S->a, r); hi = add(S->a, r); break;                                    /* sphere_shape.cpp:42-48 */
	case 1: lo = sub(vmin3(S->a, S->b), r); hi = add(vmax3(S->a, S->b), r); break;           /* capsule_shape.cpp:40-50 */
	case 2:                                                                                   /* box_shape.cpp:40-61 */
	{
		v3 e = S->a;
		for (int c = 0; c < 8; ++c)
		{
			v3 v = V((c & 4) ? e.x : -e.x, (c & 2) ? e.y : -e.y, (c & 1) ? e.z : -e.z);
			v3 w = xform(S, v);
			lo = c ? vmin3(lo, w) : w;
			hi = c ? vmax3(hi, w) : w;
		}
		lo = sub(lo, r);
		hi = add(hi, r);
		break;
	}
	case 3: lo = sub(vmin3(S->a, vmin3(S->b, S->c)), r); hi = add(vmax3(S->a, vmax3(S->b, S->c)), r); break; /* triangle_shape.cpp:51-63 */
	case 4:                                                                                   /* mesh_shape.cpp:46-52, 129-162 */
	{
		v3 sc = P3(W->scale);
		S->inv_scale = V(1 / sc.x, 1 / sc.y, 1 / sc.z);
		S->count = W->triangle_count;
		S->tri = xcalloc((size_t)28 * W->triangle_count, sizeof(real));
		for (uint32_t t = 0; t < W->triangle_count; ++t)
		{
			real* R = S->tri + (size_t)28 * t;
			const uint32_t* tv = W->triangles + 3 * t;
			v3 loc[3];
			for (int c = 0; c < 3; ++c)
			{
				loc[c] = P3(W->vertices + 3 * tv[c]);
				v3 w = xform(S, V(sc.x * loc[c].x, sc.y * loc[c].y, sc.z * loc[c].z));
				R[3 * c] = w.x; R[3 * c + 1] = w.y; R[3 * c + 2] = w.z;
				uint32_t u = W->wings ? W->wings[3 * t + c] : B3O_NULL_VERTEX;
				if (u != B3O_NULL_VERTEX)
				{
					v3 lu = P3(W->vertices + 3 * u);
					v3 wu = xform(S, V(sc.x * lu.x, sc.y * lu.y, sc.z * lu.z));
					R[9 + 3 * c] = wu.x; R[10 + 3 * c] = wu.y; R[11 + 3 * c] = wu.z;
					R[18 + c] = 1;
				}
			}
			v3 tl = sub(vmin3(loc[0], vmin3(loc[1], loc[2])), V(B3O_LINEAR_SLOP, B3O_LINEAR_SLOP, B3O_LINEAR_SLOP));
			v3 th = add(vmax3(loc[0], vmax3(loc[1], loc[2])), V(B3O_LINEAR_SLOP, B3O_LINEAR_SLOP, B3O_LINEAR_SLOP));
			R[21] = tl.x; R[22] = tl.y; R[23] = tl.z; R[24] = th.x; R[25] = th.y; R[26] = th.z;
		}
		for (uint32_t v = 0; v < W->vertex_count; ++v)
		{
			v3 lv = P3(W->vertices + 3 * v);
			v3 w = xform(S, V(sc.x * lv.x, sc.y * lv.y, sc.z * lv.z));
			lo = v ? vmin3(lo, w) : w;
			hi = v ? vmax3(hi, w) : w;
		}
		lo = sub(lo, r);
		hi = add(hi, r);
		break;
	}
	case 5:                                                                                   /* sdf_shape.cpp:40-46, aabb.h:321-336 */
	{
		for (int c = 0; c < 3; ++c) S->dims[c] = (int)W->grid[c];
		S->invert = W->invert ? 1 : 0;
		S->glo = P3(W->grid_lower);
		S->ghi = P3(W->grid_upper);
		size_t nv = (size_t)W->grid[0] * W->grid[1] * W->grid[2];
		S->vox = xcalloc(nv, sizeof(real));
		for (size_t k = 0; k < nv; ++k) S->vox[k] = (real)W->voxels[k];
		v3 lc = scl((real)0.5, add(S->glo, S->ghi)), lr = scl((real)0.5, sub(S->ghi, S->glo));
		v3 cc = xform(S, lc);
		m33 R = qmat(S->q);
		v3 ax = V(fabs((double)R.c[0].x), fabs((double)R.c[0].y), fabs((double)R.c[0].z));
		v3 ay = V(fabs((double)R.c[1].x), fabs((double)R.c[1].y), fabs((double)R.c[1].z));
		v3 az = V(fabs((double)R.c[2].x), fabs((double)R.c[2].y), fabs((double)R.c[2].z));
		v3 rr = V(dot(lr, ax), dot(lr, ay), dot(lr, az));
		lo = sub(sub(cc, rr), r);
		hi = add(add(cc, rr), r);
		break;
	}
	default: break;
	}
	S->lo = lo;
	S->hi = hi;
}

/* the closest feature point Pf: contact if within radius; normal toward Q unless Q is on it */
static int point_feature(v3 Q, v3 Pf, real radius, v3 fallback, v3* P, v3* n)
{
	v3 d = sub(Q, Pf);
	real dd = dot(d, d);
	if (dd > radius * radius) return 0;
	*n = fallback;
	real l = rsqrt_(dd);
	if (l > B3O_EPS) *n = vdiv(d, l);
	*P = Pf;
	return 1;
}

/* sphere_shape.cpp:50-77 */
static int collide_sphere(const oshape* S, v3 Q, real r1, v3* P, v3* n)
{
	real radius = S->radius + r1;
	v3 d = sub(Q, S->a);
	real dd = dot(d, d);
	if (!(dd <= radius * radius)) return 0;
	*P = S->a;
	if (dd > B3O_EPS * B3O_EPS) *n = vdiv(d, rsqrt_(dd));
	else *n = V(0, 1, 0);
	return 1;
}

/* capsule_shape.cpp:52-136 */
static int collide_capsule(const oshape* S, v3 Q, real r1, v3* P, v3* n)
{
	v3 A = S->a, B = S->b, AB = sub(B, A);
	real u = dot(sub(B, Q), AB), v = dot(sub(Q, A), AB);
	real radius = S->radius + r1;
	if (v <= 0) return point_feature(Q, A, radius, V(0, 1, 0), P, n);
	if (u <= 0) return point_feature(Q, B, radius, V(0, 1, 0), P, n);
	real ss = dot(AB, AB);
	v3 Pc = vdiv(add(scl(u, A), scl(v, B)), ss);
	v3 d = sub(Q, Pc);
	if (dot(d, d) > radius * radius) return 0;
	v3 AQ = sub(Q, A);
	v3 nn = cross(cross(AB, AQ), AB);
	if (dot(nn, AQ) < 0) nn = neg(nn);
	*n = normalize(nn);
	*P = Pc;
	return 1;
}

/* box_shape.cpp:63-140 */
static int collide_box(const oshape* S, v3 Q, real r1, v3* P, v3* n)
{
	v3 e = S->a;
	real radius = S->radius + r1;
	v3 cl = qrot(S->q, sub(Q, S->t), -1);
	v3 normals[6] = {V(1, 0, 0), V(-1, 0, 0), V(0, 1, 0), V(0, -1, 0), V(0, 0, 1), V(0, 0, -1)};
	real offsets[6] = {e.x, e.x, e.y, e.y, e.z, e.z};
	int face = 0;
	real sep = -(real)3.402823466e+38;
	for (int k = 0; k < 6; ++k)
	{
		real sk = dot(normals[k], cl) - offsets[k];
		if (sk > radius) return 0;
		if (sk > sep) { face = k; sep = sk; }
	}
	if (sep < 0)
	{
		v3 cb = sub(cl, scl(sep, normals[face]));
		*P = xform(S, cb);
		*n = qrot(S->q, normals[face], 1);
		return 1;
	}
	v3 cb = vmax3(neg(e), vmin3(cl, e));
	v3 d = sub(cl, cb);
	real dd = dot(d, d);
	if (dd > radius * radius) return 0;
	if (!(dd > B3O_EPS * B3O_EPS)) return 0;
	*P = xform(S, cb);
	*n = qrot(S->q, vdiv(d, rsqrt_(dd)), 1);
	return 1;
}

/* geometry.h:27-70 b3BarycentricCoordinates */
static void bary2(real out[3], v3 A, v3 B, v3 Q)
{
	v3 AB = sub(B, A), QA = sub(A, Q), QB = sub(B, Q);
	out[0] = dot(QB, AB);
	out[1] = -dot(QA, AB);
	out[2] = dot(AB, AB);
}
static void bary3(real out[4], v3 A, v3 B, v3 C, v3 Q)
{
	v3 AB = sub(B, A), AC = sub(C, A), QA = sub(A, Q), QB = sub(B, Q), QC = sub(C, Q);
	v3 ABxAC = cross(AB, AC);
	out[0] = dot(cross(QB, QC), ABxAC);
	out[1] = dot(cross(QC, QA), ABxAC);
	out[2] = dot(cross(QA, QB), ABxAC);
	out[3] = dot(ABxAC, ABxAC);
}

/* triangle_shape.cpp:65-311 with optional wing vertices (mesh children) */
static int collide_triangle(v3 A, v3 B, v3 C, const v3* wing, const int* has, real rshape, v3 Q, real r1, v3* P, v3* n)
{
	real radius = rshape + r1;
	v3 tn = normalize(cross(sub(B, A), sub(C, A)));
	real wAB[3], wBC[3], wCA[3], wABC[4];
	bary2(wAB, A, B, Q);
	bary2(wBC, B, C, Q);
	bary2(wCA, C, A, Q);
	if (wAB[1] <= 0 && wCA[0] <= 0) return point_feature(Q, A, radius, tn, P, n);
	if (wAB[0] <= 0 && wBC[1] <= 0) return point_feature(Q, B, radius, tn, P, n);
	if (wBC[0] <= 0 && wCA[1] <= 0) return point_feature(Q, C, radius, tn, P, n);
	bary3(wABC, A, B, C, Q);
	const real* wedge[3] = {wAB, wBC, wCA};
	v3 E0[3] = {A, B, C}, E1[3] = {B, C, A};
	real opp[3] = {wABC[2], wABC[0], wABC[1]};
	for (int e = 0; e < 3; ++e)
	{
		const real* w = wedge[e];
		if (w[0] > 0 && w[1] > 0 && wABC[3] * opp[e] <= 0)
		{
			v3 Pe = vdiv(add(scl(w[0], E0[e]), scl(w[1], E1[e])), w[2]);
			v3 d = sub(Q, Pe);
			if (dot(d, d) > radius * radius) return 0;
			if (wing && has[e])
			{
				real w1[4];
				bary3(w1, wing[e], E1[e], E0[e], Q);
				if (w1[0] > 0 && w1[1] > 0 && w1[2] > 0) return 0;
			}
			*n = tn;
			real l = len(d);
			if (l > B3O_EPS) *n = vdiv(d, l);
			*P = Pe;
			return 1;
		}
	}
	v3 Pf = vdiv(add(add(scl(wABC[0], A), scl(wABC[1], B)), scl(wABC[2], C)), wABC[3]);
	return point_feature(Q, Pf, radius, tn, P, n);
}

/* mesh_shape.cpp:87-124 */
static int collide_mesh(const oshape* S, v3 Q, real r1, v3* P, v3* n)
{
	v3 cl0 = qrot(S->q, sub(Q, S->t), -1);
	v3 c = V(S->inv_scale.x * cl0.x, S->inv_scale.y * cl0.y, S->inv_scale.z * cl0.z);
	real qr = r1 + S->radius;
	real dd0 = (real)3.402823466e+38;
	int found = 0;
	for (uint32_t k = 0; k < S->count; ++k)
	{
		const real* T = S->tri + (size_t)28 * k;
		if (c.x + qr < T[21] || c.x - qr > T[24] || c.y + qr < T[22] || c.y - qr > T[25] || c.z + qr < T[23] || c.z - qr > T[26]) continue;
		v3 wing[3] = {V(T[9], T[10], T[11]), V(T[12], T[13], T[14]), V(T[15], T[16], T[17])};
		int has[3] = {T[18] != 0, T[19] != 0, T[20] != 0};
		v3 Pk, nk;
		if (!collide_triangle(V(T[0], T[1], T[2]), V(T[3], T[4], T[5]), V(T[6], T[7], T[8]), wing, has, S->radius, Q, r1, &Pk, &nk)) continue;
		v3 d = sub(Q, Pk);
		real dd = dot(d, d);
		if (dd < dd0) { dd0 = dd; *P = Pk; *n = nk; found = 1; }
	}
	return found;
}

/* voxel_grid.h:166-206, regular_grid_indexer.h */
static real lerp_(real x, real a, real b) { return (1 - x) * a + x * b; }
static real interp(const real v[8], real x, real y, real z)
{
	x = x < 0 ? 0 : (x > 1 ? 1 : x);
	y = y < 0 ? 0 : (y > 1 ? 1 : y);
	z = z < 0 ? 0 : (z > 1 ? 1 : z);
	real c00 = lerp_(x, v[0], v[4]), c10 = lerp_(x, v[2], v[6]), c01 = lerp_(x, v[1], v[5]), c11 = lerp_(x, v[3], v[7]);
	return lerp_(z, lerp_(y, c00, c10), lerp_(y, c01, c11));
}
static int sdf_sample(const oshape* S, v3 p, real* value, v3* grad)
{
	v3 ext = sub(S->ghi, S->glo);
	v3 cs = V(ext.x / (real)(S->dims[0] - 1), ext.y / (real)(S->dims[1] - 1), ext.z / (real)(S->dims[2] - 1));
	v3 lp = sub(p, S->glo);
	long i = (long)floor((double)(lp.x / cs.x)), j = (long)floor((double)(lp.y / cs.y)), k = (long)floor((double)(lp.z / cs.z));
	if (i < 0 || i >= S->dims[0] - 1 || j < 0 || j >= S->dims[1] - 1 || k < 0 || k >= S->dims[2] - 1) return 0;
	v3 half = vdiv(cs, 2);
	v3 center = add(add(S->glo, V((real)i * cs.x, (real)j * cs.y, (real)k * cs.z)), half);
	v3 clo = sub(center, half), chi = add(center, half), cd = sub(chi, clo);
	v3 rel = V((p.x - clo.x) / cd.x, (p.y - clo.y) / cd.y, (p.z - clo.z) / cd.z);
	size_t W = (size_t)S->dims[0], H = (size_t)S->dims[1];
#define VOX(a, b, c) S->vox[(size_t)(a) + W * ((size_t)(b) + H * (size_t)(c))]
	real v[8] = {VOX(i, j, k), VOX(i, j, k + 1), VOX(i, j + 1, k), VOX(i, j + 1, k + 1),
	             VOX(i + 1, j, k), VOX(i + 1, j, k + 1), VOX(i + 1, j + 1, k), VOX(i + 1, j + 1, k + 1)};
#undef VOX
	*value = interp(v, rel.x, rel.y, rel.z);
	*grad = V(interp(v, 1, rel.y, rel.z) - interp(v, 0, rel.y, rel.z), interp(v, rel.x, 1, rel.z) - interp(v, rel.x, 0, rel.z),
	          interp(v, rel.x, rel.y, 1) - interp(v, rel.x, rel.y, 0));
	return 1;
}

/* sdf_shape.cpp:50-84 */
static int collide_sdf(const oshape* S, v3 Q, real r1, v3* P, v3* n)
{
	v3 pl = qrot(S->q, sub(Q, S->t), -1);
	real radius = r1 + S->radius;
	real dist;
	v3 g;
	if (!sdf_sample(S, pl, &dist, &g)) return 0;
	if (S->invert) dist = -dist;
	if (dist > radius) return 0;
	v3 nl = normalize(g);
	if (S->invert) nl = neg(nl);
	*n = qrot(S->q, nl, 1);
	*P = sub(Q, scl(dist, *n));
	return 1;
}

static int world_collide(const oshape* S, v3 Q, real r1, v3* P, v3* n)
{
	switch (S->type)
	{
	case 0: return collide_sphere(S, Q, r1, P, n);
	case 1: return collide_capsule(S, Q, r1, P, n);
	case 2: return collide_box(S, Q, r1, P, n);
	case 3: return collide_triangle(S->a, S->b, S->c, NULL, NULL, S->radius, Q, r1, P, n);
	case 4: return collide_mesh(S, Q, r1, P, n);
	case 5: return collide_sdf(S, Q, r1, P, n);
	default: return 0;
	}
}

/* sphere_shape_contact.cpp:53-143 (contact damping stiffness is 0 in settings.h) */
static void contact_apply(body_t* B, uint32_t i, uint32_t k)
{
	size_t c = (size_t)i * B->nw + k;
	v3 x1 = B->xx[i];
	real r1 = B->srad[i], r2 = B->ws[k].radius;
	v3 x2, n2;
	if (!world_collide(&B->ws[k], x1, r1, &x2, &n2)) return;
	if (!B->c_apply[c]) { B->c_normal[c] = n2; B->c_apply[c] = 1; }
	v3 n1 = neg(n2);
	v3 c1 = add(x1, scl(r1, n1));
	v3 c2 = add(x2, scl(r2, n2));
	real C = len(sub(c2, c1));
	C = B3O_BAUMGARTE * C < B3O_MAX_CONTACT_LINEAR_CORRECTION ? B3O_BAUMGARTE * C : B3O_MAX_CONTACT_LINEAR_CORRECTION;
	v3 f1 = scl(-B3O_CONTACT_STIFFNESS * C, n1);
	m33 I = mdiag(1);
	m33 K11 = mscl(-B3O_CONTACT_STIFFNESS, madd(outer(n1, n1), mscl(C, msub(I, outer(n1, n1)))));
	B->fi[i] = add(B->fi[i], f1);
	uint32_t s = B->diag[i];
	B->dfdx[s] = madd(B->dfdx[s], K11);
	B->c_normalForce[c] += len(f1);
}

static void apply_forces(body_t* B)
{
	uint32_t n = B->n;
	for (uint32_t i = 0; i < n; ++i) B->fi[i] = V(0, 0, 0);
	memset(B->dfdx, 0, sizeof(m33) * B->nnzb);
	memset(B->dfdv, 0, sizeof(m33) * B->nnzb);
	/* particle.cpp:182-199 mass damping */
	for (uint32_t i = 0; i < n; ++i)
	{
		real c = B->damping[i];
		if (c > 0)
		{
			v3 fd = scl(-c * B->mass[i], B->vv[i]);
			B->fi[i] = add(B->fi[i], fd);
			uint32_t s = B->diag[i];
			B->dfdv[s] = madd(B->dfdv[s], mdiag(-c * B->mass[i]));
		}
	}
	/* forces, newest first; creation order: tetrahedra, triangles, springs, stretch, shear, mouse */
	for (uint32_t e = B->nms; e-- > 0;) mouse_apply(B, &B->ms[e]);
	for (uint32_t e = B->nbw; e-- > 0;)
	{
		if (B->bw[e].shear) shear_apply(B, &B->bw[e]);
		else stretch_apply(B, &B->bw[e]);
	}
	for (uint32_t e = B->ns; e-- > 0;) spring_apply(B, e);
	if (B->tri_elements)
		for (uint32_t e = B->ntr; e-- > 0;) tri_apply(B, e);
	for (uint32_t e = B->nt; e-- > 0;) tet_apply(B, e);
	if (B->srad && B->contact_mode == 0)
		for (uint32_t i = 0; i < n; ++i)
			for (uint32_t k = 0; k < B->nw; ++k)
				if (B->c_exists[(size_t)i * B->nw + k]) contact_apply(B, i, k);
}

/* Filtered contacts (contact_mode 1), an opt-in extension that uses the general pre-filter of
   sparse_force_solver.cpp:170-178 (any S and z; force_solver.cpp:110-129 itself only passes
   S = I or 0 and z = 0) instead of penalty springs. At the start of a step a dynamic vertex that
   overlaps a world fixture it has a contact with (the first in fixture order; n its normal, from
   the fixture to the vertex) is constrained to the Baumgarte target vt = min(0.2 C, 0.2) / h
   along n (C: distance of the two contact points, as the penalty force measures it):
   S = I - n n^T and z = (vt - v.n) n, so that the step ends with v.n = vt, which falls to zero
   as the overlap closes; a vertex that no longer overlaps is free. The contact is inelastic and
   frictionless (the constraint reports no normal force for the friction impulse). */
static void contact_filter(body_t* B, real h)
{
	for (uint32_t i = 0; i < B->n; ++i)
	{
		B->fcons[i] = 0;
		B->fn[i] = V(0, 0, 0);
		B->fzn[i] = 0;
		if (B->type[i] != DYNAMIC) continue;
		for (uint32_t k = 0; k < B->nw; ++k)
		{
			size_t c = (size_t)i * B->nw + k;
			if (!B->c_exists[c]) continue;
			v3 x1 = B->x[i];
			real r1 = B->srad[i], r2 = B->ws[k].radius;
			v3 x2, n2;
			if (!world_collide(&B->ws[k], x1, r1, &x2, &n2)) continue;
			v3 c1 = sub(x1, scl(r1, n2));
			v3 c2 = add(x2, scl(r2, n2));
			real C = len(sub(c2, c1));
			C = B3O_BAUMGARTE * C < B3O_MAX_CONTACT_LINEAR_CORRECTION ? B3O_BAUMGARTE * C : B3O_MAX_CONTACT_LINEAR_CORRECTION;
			real vt = C / h;
			B->fcons[i] = 1;
			B->fn[i] = n2;
			B->fzn[i] = vt - dot(B->v[i], n2);
			break;
		}
	}
}

/* S_i M for a vertex's filter: M - n (n^T M) when constrained */
static m33 filt_left(v3 n, int cons, m33 M)
{
	if (!cons) return M;
	return msub(M, outer(n, V(dot(n, M.c[0]), dot(n, M.c[1]), dot(n, M.c[2]))));
}
/* M S_j: M - (M n) n^T when constrained */
static m33 filt_right(m33 M, v3 n, int cons)
{
	if (!cons) return M;
	return msub(M, outer(mv(M, n), n));
}

/* ------------------------------------------------------------------ sparse helpers */
static void spmv(const body_t* B, const m33* M, const v3* x, v3* out)
{
	for (uint32_t i = 0; i < B->n; ++i)
	{
		v3 acc = V(0, 0, 0);
		for (uint32_t k = B->rowptr[i]; k < B->rowptr[i + 1]; ++k) acc = add(acc, mv(M[k], x[B->col[k]]));
		out[i] = acc;
	}
}
static real vdot(const v3* a, const v3* b, uint32_t n)
{
	real r = 0;
	for (uint32_t i = 0; i < n; ++i) r += dot(a[i], b[i]);
	return r;
}

/* sparse_solver.cpp:28-109 */
static uint32_t pcg(body_t* B, const m33* A, const v3* b, v3* x, uint32_t maxIt, real eps)
{
	uint32_t n = B->n;
	v3 *r = B->r, *d = B->d, *q = B->qv, *s = B->s, *Minv = B->Minv;
	for (uint32_t i = 0; i < n; ++i)
	{
		m33 a = A[B->diag[i]];
		Minv[i] = V((real)1 / a.c[0].x, (real)1 / a.c[1].y, (real)1 / a.c[2].z);
	}
	spmv(B, A, x, q);
	for (uint32_t i = 0; i < n; ++i) r[i] = sub(b[i], q[i]);
	for (uint32_t i = 0; i < n; ++i) d[i] = V(Minv[i].x * r[i].x, Minv[i].y * r[i].y, Minv[i].z * r[i].z);
	real delta_new = vdot(r, d, n);
	real delta_0 = delta_new;
	uint32_t it = 0;
	for (;;)
	{
		if (it == maxIt) break;
		if (delta_new <= eps * eps * delta_0) break;
		spmv(B, A, d, q);
		real alpha = delta_new / vdot(d, q, n);
		for (uint32_t i = 0; i < n; ++i) x[i] = add(x[i], scl(alpha, d[i]));
		if (it % 50 == 0)
		{
			spmv(B, A, x, q);
			for (uint32_t i = 0; i < n; ++i) r[i] = sub(b[i], q[i]);
		}
		else
			for (uint32_t i = 0; i < n; ++i) r[i] = sub(r[i], scl(alpha, q[i]));
		for (uint32_t i = 0; i < n; ++i) s[i] = V(Minv[i].x * r[i].x, Minv[i].y * r[i].y, Minv[i].z * r[i].z);
		real delta_old = delta_new;
		delta_new = vdot(r, s, n);
		real beta = delta_new / delta_old;
		for (uint32_t i = 0; i < n; ++i) d[i] = add(s[i], scl(beta, d[i]));
		++it;
	}
	return it;
}

/* sparse_force_solver.cpp:104-232 (z = 0) */
static uint32_t solve_be(body_t* B, real h, uint32_t maxIt, uint32_t maxSub, real subEps)
{
	uint32_t n = B->n;
	real eps = B3O_EPS;
	for (uint32_t i = 0; i < n; ++i)
	{
		B->py[i] = V(0, 0, 0);
		B->xx[i] = B->x0[i];
		B->vv[i] = B->v0[i];
	}
	real error0 = 0, error = 0;
	uint32_t maxSubIt = 0;
	for (uint32_t iteration = 0; iteration < maxIt;)
	{
		apply_forces(B);
		/* A = M - h dfdv - h^2 dfdx */
		for (uint32_t i = 0; i < n; ++i)
			for (uint32_t k = B->rowptr[i]; k < B->rowptr[i + 1]; ++k)
			{
				m33 a = mscl(-h, B->dfdv[k]);
				if (k == B->diag[i]) a = madd(mdiag(B->Mval[i]), a);
				B->A[k] = msub(a, mscl(h * h, B->dfdx[k]));
			}
		/* b = M (v0 - v) + h (fe + fi) + (h dfdx)(x0 - x + h v + y) */
		for (uint32_t i = 0; i < n; ++i)
			B->w[i] = add(add(sub(B->x0[i], B->xx[i]), scl(h, B->vv[i])), B->y[i]);
		for (uint32_t i = 0; i < n; ++i)
		{
			v3 acc = V(0, 0, 0);
			for (uint32_t k = B->rowptr[i]; k < B->rowptr[i + 1]; ++k)
				acc = add(acc, mv(mscl(h, B->dfdx[k]), B->w[B->col[k]]));
			v3 Mdv = scl(B->Mval[i], sub(B->v0[i], B->vv[i]));
			B->b[i] = add(add(Mdv, scl(h, add(B->fe[i], B->fi[i]))), acc);
		}
		/* pA = S A S^T + I - S ; pb = S (b - A z); z = 0 after the first Newton iteration */
		const int filt = B->contact_mode == 1;
		for (uint32_t i = 0; i < n; ++i)
		{
			v3 bz = V(0, 0, 0);
			const int ci = filt && B->fcons[i];
			for (uint32_t k = B->rowptr[i]; k < B->rowptr[i + 1]; ++k)
			{
				uint32_t j = B->col[k];
				const int cj = filt && B->fcons[j];
				if (cj && iteration == 0) bz = add(bz, mv(B->A[k], scl(B->fzn[j], B->fn[j])));
				if (!(B->S[i] && B->S[j])) B->A[k] = mzero();
				else if (filt) B->A[k] = filt_left(B->fn[i], ci, filt_right(B->A[k], B->fn[j], cj));
			}
			if (!B->S[i]) B->A[B->diag[i]] = mdiag(1);
			else if (ci) B->A[B->diag[i]] = madd(B->A[B->diag[i]], outer(B->fn[i], B->fn[i]));
			v3 rb = sub(B->b[i], bz);
			if (ci) rb = sub(rb, scl(dot(B->fn[i], rb), B->fn[i]));
			B->pb[i] = B->S[i] ? rb : V(0, 0, 0);
		}
		uint32_t sub_it = pcg(B, B->A, B->pb, B->py, maxSub, subEps);
		if (sub_it > maxSubIt) maxSubIt = sub_it;
		/* dv = py + z */
		for (uint32_t i = 0; i < n; ++i)
		{
			v3 dv = B->py[i];
			if (filt && iteration == 0 && B->fcons[i]) dv = add(dv, scl(B->fzn[i], B->fn[i]));
			B->tmp[i] = dv;
			B->vv[i] = add(B->vv[i], dv);
			B->xx[i] = add(add(B->x0[i], scl(h, B->vv[i])), B->y[i]);
		}
		error = vdot(B->tmp, B->tmp, n);
		if (iteration == 0)
		{
			error0 = error;
			if (error <= eps * eps) break;
		}
		else if (error <= eps * eps * error0) break;
		++iteration;
	}
	return maxSubIt;
}

static int aabb_overlap_shape(v3 p, real r, const oshape* S)
{
	/* aabb.h:371 b3TestOverlap of AABB(p, r) and the fixture's AABB */
	if (p.x + r < S->lo.x || p.x - r > S->hi.x) return 0;
	if (p.y + r < S->lo.y || p.y - r > S->hi.y) return 0;
	if (p.z + r < S->lo.z || p.z - r > S->hi.z) return 0;
	return 1;
}

/* body.cpp:552-604 */
static uint32_t body_step(body_t* B, real dt, uint32_t newtonIt, uint32_t maxSub, real subEps)
{
	uint32_t n = B->n;
	/* contact_manager.cpp:108-146 UpdateContacts */
	if (B->srad)
		for (uint32_t i = 0; i < n; ++i)
			for (uint32_t k = 0; k < B->nw; ++k)
			{
				size_t c = (size_t)i * B->nw + k;
				if (!B->c_exists[c]) continue;
				if (B->type[i] != DYNAMIC || !aabb_overlap_shape(B->x[i], B->srad[i], &B->ws[k]))
				{
					B->c_exists[c] = 0;
					continue;
				}
				B->c_normalForce[c] = 0;
				B->c_apply[c] = 0;
			}
	uint32_t it = 0;
	if (dt > 0)
	{
		for (uint32_t i = 0; i < n; ++i)
		{
			B->x0[i] = B->x[i];
			B->v0[i] = B->v[i];
			B->fe[i] = B->fext[i];
			B->y[i] = B->trans[i];
			if (B->type[i] == DYNAMIC)
			{
				B->Mval[i] = B->mass[i];
				B->fe[i] = add(B->fe[i], scl(B->mass[i], B->gravity));
				B->S[i] = 1;
			}
			else
			{
				B->Mval[i] = 1;
				B->S[i] = 0;
			}
		}
		if (B->srad && B->contact_mode == 1) contact_filter(B, dt);
		it = solve_be(B, dt, newtonIt, maxSub, subEps);
		for (uint32_t i = 0; i < n; ++i)
		{
			B->x[i] = B->xx[i];
			B->v[i] = B->vv[i];
		}
		/* sphere_shape_contact.cpp:145-189 ApplyFriction */
		if (B->srad)
			for (uint32_t i = 0; i < n; ++i)
				for (uint32_t k = 0; k < B->nw; ++k)
				{
					size_t c = (size_t)i * B->nw + k;
					if (!B->c_exists[c] || !B->c_apply[c]) continue;
					v3 normal = B->c_normal[c];
					real nf = B->c_normalForce[c];
					v3 t1 = perp(normal);
					v3 t2 = cross(t1, normal);
					v3 v1 = B->v[i];
					real im1 = B->invmass[i];
					real fr = rsqrt_(B->sfric[i] * B->ws[k].friction);
					real tm = im1 > 0 ? (real)1 / im1 : 0;
					v2 Cdot = V2(dot(v1, t1), dot(v1, t2));
					v2 imp = scl2(tm, V2(-Cdot.x, -Cdot.y));
					real maxImp = fr * (dt * nf);
					if (imp.x * imp.x + imp.y * imp.y > maxImp * maxImp)
					{
						imp = normalize2(imp);
						imp = scl2(maxImp, imp);
					}
					v3 P = add(scl(imp.x, t1), scl(imp.y, t2));
					B->v[i] = add(v1, scl(im1, P));
				}
	}
	for (uint32_t i = 0; i < n; ++i)
	{
		B->fext[i] = V(0, 0, 0);
		B->trans[i] = V(0, 0, 0);
	}
	/* contact_manager.cpp:65-82 FindNewContacts (only dynamic particles collide) */
	if (B->srad)
		for (uint32_t i = 0; i < n; ++i)
			for (uint32_t k = 0; k < B->nw; ++k)
			{
				size_t c = (size_t)i * B->nw + k;
				if (B->c_exists[c]) continue;
				if (B->type[i] != DYNAMIC) continue;
				if (aabb_overlap_shape(B->x[i], B->srad[i], &B->ws[k]))
				{
					B->c_exists[c] = 1;
					B->c_normalForce[c] = 0;
					B->c_apply[c] = 0;
				}
			}
	return it;
}

static double now_sec(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int b3o_simulate(const b3o_desc* d, b3o_run* run)
{
	body_t* B = body_create(d);
	if (!B) return 1;
	B->contact_mode = run->contact_mode;
	double t0 = now_sec();
	for (uint32_t s = 0; s < run->steps; ++s)
	{
		uint32_t it = body_step(B, (real)run->dt, run->newton_iters, run->max_sub, (real)run->sub_tol);
		if (run->sub_iters_out) run->sub_iters_out[s] = it;
	}
	double t1 = now_sec();
	if (run->seconds_out) *run->seconds_out = t1 - t0;
	for (uint32_t i = 0; i < B->n; ++i)
	{
		run->x_out[3 * i + 0] = B->x[i].x; run->x_out[3 * i + 1] = B->x[i].y; run->x_out[3 * i + 2] = B->x[i].z;
		run->v_out[3 * i + 0] = B->v[i].x; run->v_out[3 * i + 1] = B->v[i].y; run->v_out[3 * i + 2] = B->v[i].z;
	}
	body_free(B);
	return 0;
}

/* ------------------------------------------------------------------ ray casts */
typedef struct
{
	int32_t hit;
	uint32_t triangle;
	double fraction;
	double normal[3];
} b3o_hit;

/* triangle_shape.cpp:314-387 b3TriangleShape::RayCast */
static int ray_triangle(v3 p1, v3 p2, v3 A, v3 Bv, v3 C, real maxFraction, real* fraction, v3* normal)
{
	v3 d = sub(p2, p1);
	if (dot(d, d) < B3O_EPS * B3O_EPS) return 0;
	v3 n = normalize(cross(sub(Bv, A), sub(C, A)));
	real num = dot(n, sub(A, p1));
	real den = dot(n, d);
	if (den == 0) return 0;
	real t = num / den;
	if (t < 0 || maxFraction < t) return 0;
	v3 Q = add(p1, scl(t, d));
	v3 AB = sub(Bv, A), AC = sub(C, A);
	v3 QA = sub(A, Q), QB = sub(Bv, Q), QC = sub(C, Q);
	v3 N = cross(AB, AC);
	real u = dot(cross(QB, QC), N);
	real v = dot(cross(QC, QA), N);
	real w = dot(cross(QA, QB), N);
	if (u >= 0 && v >= 0 && w >= 0)
	{
		*fraction = t;
		*normal = num > 0 ? neg(n) : n;
		return 1;
	}
	return 0;
}

/* body.cpp:468-521 b3Body::RayCastSingle after run->steps steps. The reference's tree only prunes
 * (its callback keeps the full max fraction), so every triangle fixture whose ray cast succeeds
 * is a candidate and the smallest fraction wins; ties go to the lowest triangle index. */
int b3o_ray_cast(const b3o_desc* d, b3o_run* run, uint32_t count, const double* segs, b3o_hit* out)
{
	body_t* B = body_create(d);
	if (!B) return 1;
	B->contact_mode = run->contact_mode;
	for (uint32_t s = 0; s < run->steps; ++s)
	{
		uint32_t it = body_step(B, (real)run->dt, run->newton_iters, run->max_sub, (real)run->sub_tol);
		if (run->sub_iters_out) run->sub_iters_out[s] = it;
	}
	for (uint32_t r = 0; r < count; ++r)
	{
		v3 p1 = D3(segs + 6 * r), p2 = D3(segs + 6 * r + 3);
		b3o_hit h;
		memset(&h, 0, sizeof(h));
		real best = 0;
		for (uint32_t e = 0; e < B->ntr; ++e)
		{
			real t;
			v3 n;
			const uint32_t* t3 = B->tri + 3 * e;
			if (ray_triangle(p1, p2, B->x[t3[0]], B->x[t3[1]], B->x[t3[2]], 1, &t, &n) && (!h.hit || t < best))
			{
				best = t;
				h.hit = 1;
				h.triangle = e;
				h.fraction = t;
				h.normal[0] = n.x;
				h.normal[1] = n.y;
				h.normal[2] = n.z;
			}
		}
		out[r] = h;
	}
	if (run->x_out)
		for (uint32_t i = 0; i < B->n; ++i)
		{
			run->x_out[3 * i + 0] = B->x[i].x; run->x_out[3 * i + 1] = B->x[i].y; run->x_out[3 * i + 2] = B->x[i].z;
		}
	body_free(B);
	return 0;
}

/* ------------------------------------------------------------------ many bodies on many threads */
typedef struct
{
	const b3o_desc* descs;
	b3o_run* runs;
	body_t** bodies;
	uint32_t count;
	uint32_t next;
	int phase; /* 0 create, 1 step, 2 write out and free */
	pthread_mutex_t lock;
} batch_job;

static void* batch_worker(void* arg)
{
	batch_job* J = (batch_job*)arg;
	for (;;)
	{
		pthread_mutex_lock(&J->lock);
		uint32_t k = J->next++;
		pthread_mutex_unlock(&J->lock);
		if (k >= J->count) break;
		b3o_run* run = J->runs + k;
		if (J->phase == 0)
		{
			J->bodies[k] = body_create(J->descs + k);
			if (J->bodies[k]) J->bodies[k]->contact_mode = run->contact_mode;
		}
		else if (J->phase == 1)
		{
			body_t* B = J->bodies[k];
			for (uint32_t s = 0; s < run->steps; ++s)
			{
				uint32_t it = body_step(B, (real)run->dt, run->newton_iters, run->max_sub, (real)run->sub_tol);
				if (run->sub_iters_out) run->sub_iters_out[s] = it;
			}
		}
		else
		{
			body_t* B = J->bodies[k];
			for (uint32_t i = 0; i < B->n; ++i)
			{
				run->x_out[3 * i + 0] = B->x[i].x; run->x_out[3 * i + 1] = B->x[i].y; run->x_out[3 * i + 2] = B->x[i].z;
				run->v_out[3 * i + 0] = B->v[i].x; run->v_out[3 * i + 1] = B->v[i].y; run->v_out[3 * i + 2] = B->v[i].z;
			}
			body_free(B);
			J->bodies[k] = NULL;
		}
	}
	return NULL;
}

static void batch_phase(batch_job* J, int phase, uint32_t threads)
{
	pthread_t th[256];
	J->phase = phase;
	J->next = 0;
	for (uint32_t t = 0; t < threads; ++t) pthread_create(&th[t], NULL, batch_worker, J);
	for (uint32_t t = 0; t < threads; ++t) pthread_join(th[t], NULL);
}

/* Independent bodies share nothing, so they run on `threads` host threads: all bodies are built
 * first, then stepped (the timed phase, wall time in *step_seconds), then written out. */
int b3o_simulate_batch(const b3o_desc* descs, b3o_run* runs, uint32_t count, uint32_t threads, double* step_seconds)
{
	batch_job J;
	J.descs = descs;
	J.runs = runs;
	J.count = count;
	J.bodies = (body_t**)xcalloc(count, sizeof(body_t*));
	pthread_mutex_init(&J.lock, NULL);
	if (threads < 1) threads = 1;
	if (threads > 256) threads = 256;
	batch_phase(&J, 0, threads);
	for (uint32_t k = 0; k < count; ++k)
		if (!J.bodies[k]) return 1;
	double t0 = now_sec();
	batch_phase(&J, 1, threads);
	if (step_seconds) *step_seconds = now_sec() - t0;
	batch_phase(&J, 2, threads);
	pthread_mutex_destroy(&J.lock);
	free(J.bodies);
	return 0;
}
