// Device helpers shared by the forward substep kernels (xfem_kernels.cu) and
// the adjoint kernels (xfem_adjoint.cu): the bounded grid barrier, the
// per-vertex advance (finalize + predict), the element solve and the
// bulk-copy staging of chunk blocks. Internal linkage: each translation
// unit gets its own copy.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "xfem_internal.h"

namespace xfem {

namespace {

// Sets the grid-barrier arrival counter to ctx.bar_base (0 or 0xffffffff)
// before a persistent launch.
inline cudaError_t reset_barrier(const DevCtx& ctx, cudaStream_t st) {
	return cudaMemsetAsync(ctx.bar_count, ctx.bar_base ? 0xff : 0, sizeof(uint32_t), st);
}

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
	uint32_t v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

// A relaxed load for polls; one fence.acquire.gpu after the last poll orders
// what follows (an acquire load per poll cost 0.9% of the persistent frame
// and 1.7% of the brick frame).
__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t* p) {
	uint32_t v;
	asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ uint64_t global_ns() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Grid-wide barrier for the co-resident persistent grid. Monotonic arrival
// counter, set to C.bar_base before each launch; every block's target starts
// there too. The counter may wrap past 2^32 within a launch: arrival and
// target are compared through their signed 32-bit difference, which stays
// within +-gridDim.x (no block can be more than one barrier ahead of another).
// Every wait is bounded by C.timeout_ns: on timeout the block records
// kErrBarrierTimeout and all blocks leave at their next barrier.
// C.wait_miss (a test hook, normally 0) adds arrivals that no block makes,
// so the wait runs out on purpose.
__device__ bool grid_sync(const DevCtx& C, uint32_t& target) {
	__shared__ int s_ok;
	__syncthreads();
	target += gridDim.x + C.wait_miss;
	if (threadIdx.x == 0) {
		int ok = 1;
		__threadfence();
		atomicAdd(C.bar_count, 1u);
		uint32_t spins = 0;
		uint64_t t0 = 0;
		while ((int32_t)(ld_relaxed_gpu(C.bar_count) - target) < 0) {
			if (++spins == 256) {
				spins = 0;
				if (*(volatile int*)C.err) {
					ok = 0;
					break;
				}
				const uint64_t t = global_ns();
				if (t0 == 0) {
					t0 = t;
				} else if (t - t0 > C.timeout_ns) {
					atomicCAS(C.err, 0, kErrBarrierTimeout);
					ok = 0;
					break;
				}
			}
		}
		asm volatile("fence.acquire.gpu;" ::: "memory");  // the acquire pattern: relaxed polls, one fence
		s_ok = ok;
	}
	__syncthreads();
	return s_ok != 0;
}

// One vertex's 32-byte state (vert[2v], vert[2v + 1]: one sector, 32-byte
// aligned) in a single 256-bit access (sm_100 and later), L1 bypassed as
// __ldcg / __stcg: half the load and store instructions, and L1 wavefronts,
// of two 128-bit accesses. The memory clobbers keep them ordered with the
// grid barrier and the staging copies like any other global access.
__device__ __forceinline__ void ld_vertex(const float4* p, float4& a, float4& b) {
	asm volatile("ld.global.cg.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
	             : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
	             : "l"(p)
	             : "memory");
}

__device__ __forceinline__ void st_vertex(float4* p, const float4& a, const float4& b) {
	asm volatile("st.global.cg.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z),
	             "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
	             : "memory");
}

struct Vec3 {
	float x, y, z;
};

__device__ __forceinline__ Vec3 v3(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ float dot(Vec3 a, Vec3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }

// Ground plane with Coulomb friction on the substep displacement D
// (extension; no reference counterpart). Returns true on contact.
__device__ __forceinline__ bool ground_contact(const BodyParams& bp, const float4& O, float4& D) {
	const float nx = bp.ground_n[0], ny = bp.ground_n[1], nz = bp.ground_n[2];
	const float h = (nx * O.x + ny * O.y + nz * O.z) - bp.ground_d;
	const float depth = -(h + (nx * D.x + ny * D.y + nz * D.z));
	if (!(depth > 0.0f)) return false;
	D.x += depth * nx;
	D.y += depth * ny;
	D.z += depth * nz;
	const float dn = nx * D.x + ny * D.y + nz * D.z;
	const float tx = D.x - dn * nx, ty = D.y - dn * ny, tz = D.z - dn * nz;
	const float lt = sqrtf(tx * tx + ty * ty + tz * tz);
	const float lim = bp.friction * depth;
	const float s = lt <= lim ? 1.0f : lim / lt;
	D.x -= s * tx;
	D.y -= s * ty;
	D.z -= s * tz;
	return true;
}

// End of a substep for one vertex: locks (XPBDFEM/Geo.cpp:318-331), ground,
// then the velocity V = D / dt (XPBDFEM/Geo.cpp:342-344) is returned. A Left
// vertex stays where the substep started (X = O); a Right vertex goes to its
// target origin + lockedRightTransform3d X0 (X = O = target, so V = 0), read
// from right_target[v] (device vertex v); both keep a zero inverse mass.
__device__ __forceinline__ Vec3 finish_vertex(const BodyParams& bp, float4& O, float4& D, uint32_t& bits, float inv_dt,
                                              const float4* right_target, uint32_t v) {
	if (bp.lock_active && (bits & kFlagLocked)) {
		D.x = D.y = D.z = 0.0f;
		O.w = 0.0f;
	}
	if (bp.lock_right && (bits & kFlagRight)) {
		const float4 t = __ldg(right_target + v);
		O = make_float4(t.x, t.y, t.z, 0.0f);
		D.x = D.y = D.z = 0.0f;
	}
	bits &= ~kFlagContact;
	if (bp.ground && O.w > 0.0f && ground_contact(bp, O, D)) bits |= kFlagContact;
	return {D.x * inv_dt, D.y * inv_dt, D.z * inv_dt};
}

// Finalize the previous substep (unless `first`: (O, D) then hold the
// canonical (X, V)) and predict the next (XPBDFEM/Geo.cpp:307-312) for
// device vertex v. bodies: C.bodies, or a copy of them in shared memory.
__device__ __forceinline__ void advance_vertex_bp(const DevCtx& C, const BodyParams& bp, uint32_t v, float4& O,
                                                  float4& D, bool first, float dt, float inv_dt) {
	uint32_t bits = __float_as_uint(D.w);
	Vec3 V;
	if (first) {
		V = v3(D);
	} else {
		V = finish_vertex(bp, O, D, bits, inv_dt, C.right_target, v);
		O.x += D.x;
		O.y += D.y;
		O.z += D.z;
	}
	V.x = (V.x + bp.gravity[0] * dt) * bp.drag_mul;
	V.y = (V.y + bp.gravity[1] * dt) * bp.drag_mul;
	V.z = (V.z + bp.gravity[2] * dt) * bp.drag_mul;
	D = make_float4(V.x * dt, V.y * dt, V.z * dt, __uint_as_float(bits));
}

__device__ __forceinline__ void advance_vertex(const DevCtx& C, uint32_t v, float4& O, float4& D, bool first, float dt,
                                               float inv_dt, const BodyParams* bodies = nullptr) {
	advance_vertex_bp(C, (bodies ? bodies : C.bodies)[__float_as_uint(D.w) >> 8], v, O, D, first, dt, inv_dt);
}

// Finalize the last substep of a launch: (O, D) -> canonical (X, V) for
// device vertex v. A position or velocity that is no longer finite (a
// diverged solve, or a NaN the caller set) is recorded in the error word as
// kErrNonFinite, which the next synchronising call reports.
__device__ __forceinline__ void finalize_vertex_bp(const DevCtx& C, const BodyParams& bp, uint32_t v, float4& O,
                                                   float4& D, float inv_dt) {
	uint32_t bits = __float_as_uint(D.w);
	const Vec3 V = finish_vertex(bp, O, D, bits, inv_dt, C.right_target, v);
	O.x += D.x;
	O.y += D.y;
	O.z += D.z;
	D = make_float4(V.x, V.y, V.z, __uint_as_float(bits));
	// inf - inf and NaN - NaN are NaN: one compare for all six values
	const float z = (O.x - O.x) + (O.y - O.y) + (O.z - O.z) + (V.x - V.x) + (V.y - V.y) + (V.z - V.z);
	if (z != 0.0f) atomicCAS(C.err, 0, kErrNonFinite);
}

__device__ __forceinline__ void finalize_vertex(const DevCtx& C, uint32_t v, float4& O, float4& D, float inv_dt,
                                                const BodyParams* bodies = nullptr) {
	finalize_vertex_bp(C, (bodies ? bodies : C.bodies)[__float_as_uint(D.w) >> 8], v, O, D, inv_dt);
}

// Rest state of one tet: Qi column-major q[c][r], QQ, QR and c0 = (1/mu)/vol.
struct TetRec {
	float4 a, b, c, d;
};

// The material scalars a solve needs, copied to registers once per cluster.
// Fields that a kernel instantiation does not read are never loaded.
struct Mat {
	float a, ratio, y0, y1, y2;
	uint32_t model, simultaneous;
	float damp;        // in-solve Rayleigh ratio: damping for types 0, 1, else 0
	uint32_t limit;    // 1 = Rayleigh_Limit, 0 = Rayleigh_Paper
	float hw;          // Pixar models: lambda / 2
	float compliance;  // volume passes
	uint32_t nvol;     // volume passes of the body
};

// The same from a copy of the bodies in shared memory (plain loads).
__device__ __forceinline__ Mat load_mat_shared(const BodyParams* bodies, uint32_t body) {
	const BodyParams& b = bodies[body];
	const uint32_t type = b.rayleigh_type;
	return {b.a,  b.ratio, b.yeoh[0], b.yeoh[1], b.yeoh[2], b.model, b.simultaneous, type < 2u ? b.damping : 0.0f,
	        type == 1u ? 1u : 0u, b.hw, b.compliance, b.volume_passes};
}

__device__ __forceinline__ Mat load_mat(const BodyParams* bodies, uint32_t body) {
	const BodyParams* b = bodies + body;
	const uint32_t type = __ldg(&b->rayleigh_type);
	return {__ldg(&b->a),          __ldg(&b->ratio),        __ldg(&b->yeoh[0]),
	        __ldg(&b->yeoh[1]),    __ldg(&b->yeoh[2]),      __ldg(&b->model),
	        __ldg(&b->simultaneous), type < 2u ? __ldg(&b->damping) : 0.0f, type == 1u ? 1u : 0u,
	        __ldg(&b->hw),         __ldg(&b->compliance),   __ldg(&b->volume_passes)};
}

// Hydrostatic term at the single point (XPBDFEM/Fem.cpp:539-549 with the
// adjugate :284-300, F :311-323 and the gradient :338-354). J is formed as
// the reference forms it, det(F) of F = Qi Ds (rows of Ds: P0, P1, P2) through
// the first adjugate column: with an incompressible material the multiplier
// goes as 1 / (J - a), so J's rounding decides the result and must follow the
// reference's path. The gradient (2 (J - a) adj(F) Qi) e_n equals
// 2 (J - a) det(Qi) times the cofactor row of Ds (P1 x P2, P2 x P0, P0 x P1):
// same quantity, a third of the arithmetic. Returns U1 = (J - a)^2.
__device__ __forceinline__ Vec3 cross(Vec3 a, Vec3 b) {
	return {fmaf(a.y, b.z, -b.y * a.z), fmaf(a.z, b.x, -b.z * a.x), fmaf(a.x, b.y, -b.x * a.y)};
}

// ja, detq (optional): J - a and det(Qi), for the adjoint.
__device__ __forceinline__ float hydrostatic(const float q[3][3], const Vec3 P[3], float a, Vec3 g[4],
                                             float* ja = nullptr, float* detq = nullptr) {
	const float detQ = fmaf(q[0][0], fmaf(q[1][1], q[2][2], -q[2][1] * q[1][2]),
	                        fmaf(-q[1][0], fmaf(q[0][1], q[2][2], -q[2][1] * q[0][2]),
	                             q[2][0] * fmaf(q[0][1], q[1][2], -q[1][1] * q[0][2])));
	const Vec3 c0 = cross(P[1], P[2]), c1 = cross(P[2], P[0]), c2 = cross(P[0], P[1]);
	// F[j][r] = sum_n Qi[n][r] P_n[j] (column j, row r)
	const float Pc[3][3] = {{P[0].x, P[1].x, P[2].x}, {P[0].y, P[1].y, P[2].y}, {P[0].z, P[1].z, P[2].z}};
	float F[3][3];
#pragma unroll
	for (int j = 0; j < 3; j++)
#pragma unroll
		for (int r = 0; r < 3; r++) F[j][r] = fmaf(q[0][r], Pc[j][0], fmaf(q[1][r], Pc[j][1], q[2][r] * Pc[j][2]));
	const float a00 = fmaf(F[1][1], F[2][2], -F[1][2] * F[2][1]);
	const float a10 = -fmaf(F[1][0], F[2][2], -F[1][2] * F[2][0]);
	const float a20 = fmaf(F[1][0], F[2][1], -F[1][1] * F[2][0]);
	const float J = fmaf(F[0][0], a00, fmaf(F[0][1], a10, F[0][2] * a20));
	const float Ja = J - a;
	const float s = 2.0f * Ja * detQ;
	g[0] = {s * c0.x, s * c0.y, s * c0.z};
	g[1] = {s * c1.x, s * c1.y, s * c1.z};
	g[2] = {s * c2.x, s * c2.y, s * c2.z};
	g[3] = {-(g[0].x + g[1].x + g[2].x), -(g[0].y + g[1].y + g[2].y), -(g[0].z + g[1].z + g[2].z)};
	if (ja) *ja = Ja;
	if (detq) *detq = detQ;
	return Ja * Ja;
}

// 1/x by the hardware approximation (within about one ulp). The arguments
// are sums of squares plus 1e-22 (or a clamp at 1e-8), never zero, denormal
// or infinite. A Newton step after it rounds to about half an ulp; it lay on
// the solve's dependency chain three times per solve and cost 1.6% of the
// throughput frame, for an error far below the 1e-5 parity bound.
__device__ __forceinline__ float rcp(float x) {
	float r;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return r;
}

// I1 and its gradient, prefactored (XPBDFEM/Fem.cpp:163-192). I1 is a
// quadratic form of the edge vectors, so I1 = (1/2) sum_i g_i . P_i (Euler's
// identity for homogeneous functions): one chain of nine fused multiply-adds
// on the gradient already formed, in place of the reference's six dot
// products (the same value up to rounding; 4% of the throughput frame).
__device__ __forceinline__ float prefactored_i1(const float QQ[3], const float QR[3], const Vec3 P[3], Vec3 g[4]) {
	const float d0 = 2.0f * QQ[0], d1 = 2.0f * QQ[1], d2 = 2.0f * QQ[2];
	g[0] = {fmaf(d0, P[0].x, fmaf(QR[0], P[1].x, QR[1] * P[2].x)), fmaf(d0, P[0].y, fmaf(QR[0], P[1].y, QR[1] * P[2].y)),
	        fmaf(d0, P[0].z, fmaf(QR[0], P[1].z, QR[1] * P[2].z))};
	g[1] = {fmaf(d1, P[1].x, fmaf(QR[0], P[0].x, QR[2] * P[2].x)), fmaf(d1, P[1].y, fmaf(QR[0], P[0].y, QR[2] * P[2].y)),
	        fmaf(d1, P[1].z, fmaf(QR[0], P[0].z, QR[2] * P[2].z))};
	g[2] = {fmaf(d2, P[2].x, fmaf(QR[1], P[0].x, QR[2] * P[1].x)), fmaf(d2, P[2].y, fmaf(QR[1], P[0].y, QR[2] * P[1].y)),
	        fmaf(d2, P[2].z, fmaf(QR[1], P[0].z, QR[2] * P[1].z))};
	g[3] = {-(g[0].x + g[1].x + g[2].x), -(g[0].y + g[1].y + g[2].y), -(g[0].z + g[1].z + g[2].z)};
	return 0.5f * fmaf(g[0].x, P[0].x, fmaf(g[0].y, P[0].y, fmaf(g[0].z, P[0].z, fmaf(g[1].x, P[1].x,
	       fmaf(g[1].y, P[1].y, fmaf(g[1].z, P[1].z, fmaf(g[2].x, P[2].x, fmaf(g[2].y, P[2].y, g[2].z * P[2].z))))))));
}

// Deviatoric term of SolveElementMixed: I1 (MixedSel; Mixed with the clamp
// of XPBDFEM/Fem.cpp:489) or the Yeoh polynomial of I1 - 3 with its clamp
// (YeohSkin, YeohSkinSel: XPBDFEM/Fem.cpp:467-476, 489; YeohSkinFast:
// XPBDFEM/Fem.cpp:525-531). Mixed runs in the extended kernels only (EXT).
template <bool EXT = false>
__device__ __forceinline__ float deviatoric(const Mat& bp, const float QQ[3], const float QR[3], const Vec3 P[3],
                                            Vec3 g[4]) {
	float U = prefactored_i1(QQ, QR, P, g);
	if (EXT && bp.model == kModelNeoClamp) U = fmaxf(0.0001f, U);
	if (bp.model == kModelYeoh) {
		const float IM = U - 3.0f;
		const float C0 = bp.y0, C1 = bp.y1, C2 = bp.y2;
		U = fmaxf(0.0001f, IM * fmaf(IM, fmaf(IM, C2, C1), C0));
		const float gs = fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
#pragma unroll
		for (int n = 0; n < 4; n++) g[n] = {g[n].x * gs, g[n].y * gs, g[n].z * gs};
	}
	return U;
}

__device__ __forceinline__ float wdot(const float w[4], const Vec3 a[4], const Vec3 b[4]) {
	float s = 1.0e-22f;
#pragma unroll
	for (int n = 0; n < 4; n++) s = fmaf(w[n], dot(a[n], b[n]), s);
	return s;
}

// Cramer's rule for M = [A0 A1; A1 A2], b as in XPBDFEM/Xpbd.h:172-180.
__device__ __forceinline__ void cramer(float A0, float A1, float A2, float b0, float b1, float& l0, float& l1) {
	const float i00 = rcp(A0), i11 = rcp(A2);
	const float r0 = A1 * i00, r1 = A1 * i11;
	const float inv_det = rcp(fmaxf(0.00000001f, fmaf(-r0, r1, 1.0f)));
	const float c0 = b0 * i00, c1 = b1 * i11;
	l0 = inv_det * fmaf(-r0, c1, c0);
	l1 = inv_det * fmaf(-c0, r1, c1);
}

// One scalar constraint of the serial solve (XPBDFEM/Xpbd.h:87-121), with the
// in-solve Rayleigh damping when DAMP and bp.damp > 0; D: displacements so far
// (X - O).
template <bool DAMP>
__device__ __forceinline__ float serial_lambda(const Mat& bp, float U, const Vec3 g[4], const float w[4],
                                               const float4 D[4], float alpha, float comp, float inv_dt) {
	const float wgg = wdot(w, g, g);
	if (!DAMP || !(bp.damp > 0.0f)) return (-2.0f * U) * rcp(fmaf(2.0f * U, alpha, wgg));
	float gV = 0.0f;
#pragma unroll
	for (int n = 0; n < 4; n++) gV = fmaf(g[n].x, D[n].x, fmaf(g[n].y, D[n].y, fmaf(g[n].z, D[n].z, gV)));
	const float gamma = bp.damp * inv_dt;
	if (!bp.limit) return (-2.0f * U - gamma * gV) / fmaf(wgg, 1.0f + gamma, 2.0f * U * alpha);
	float l = (-2.0f * U) / fmaf(2.0f * U, alpha, wgg);
	const float A = fmaf(2.0f * U, comp * inv_dt / bp.damp, wgg);
	const float b = (-gV - wgg * l) * (A / fmaxf(A, 4.0f * wgg));
	return l + b / A;
}

// The Pixar models' energy and gradient (XPBDFEM/Fem.cpp:361-427), mu = 2:
// U = I1 + hw (J - a)^2, g = dI1 + hw d(J - a)^2 in g; scratch: h.
__device__ __forceinline__ float pixar_energy(const Mat& bp, const float q[3][3], const float QQ[3], const float QR[3],
                                              const Vec3 P[3], Vec3 g[4], Vec3 h[4]) {
	const float U1 = hydrostatic(q, P, bp.a, h);
	const float U = fmaf(bp.hw, U1, prefactored_i1(QQ, QR, P, g));
#pragma unroll
	for (int n = 0; n < 4; n++) g[n] = {fmaf(bp.hw, h[n].x, g[n].x), fmaf(bp.hw, h[n].y, g[n].y), fmaf(bp.hw, h[n].z, g[n].z)};
	return U;
}

// One volume-pass solve, SolveVolumeOnly (XPBDFEM/Fem.cpp:840-867): U =
// (J - 1)^2, one constraint of compliance Settings::compliance times the
// rest volume 1 / (6 det Qi), no damping.
__device__ __forceinline__ void volume_tet(const Mat& bp, const TetRec& r, float inv_dt2, const float4 O[4], float4 D[4]) {
	const float q[3][3] = {{r.a.x, r.a.y, r.a.z}, {r.a.w, r.b.x, r.b.y}, {r.b.z, r.b.w, r.c.x}};
	const float w[4] = {O[0].w, O[1].w, O[2].w, O[3].w};
	Vec3 P[3], g[4];
#pragma unroll
	for (int i = 0; i < 3; i++)
		P[i] = {(O[i].x - O[3].x) + (D[i].x - D[3].x), (O[i].y - O[3].y) + (D[i].y - D[3].y),
		        (O[i].z - O[3].z) + (D[i].z - D[3].z)};
	float detq;
	const float U = hydrostatic(q, P, 1.0f, g, nullptr, &detq);
	const float alpha = bp.compliance * inv_dt2 / (6.0f * detq);
	const float l = (-2.0f * U) / fmaf(2.0f * U, alpha, wdot(w, g, g));
#pragma unroll
	for (int n = 0; n < 4; n++) {
		const float s = w[n] * l;
		D[n].x = fmaf(s, g[n].x, D[n].x);
		D[n].y = fmaf(s, g[n].y, D[n].y);
		D[n].z = fmaf(s, g[n].z, D[n].z);
	}
}

// DampElement (XPBDFEM/Fem.cpp:908-931): energies and gradients of the tet at
// its current positions, then RayleighDamp (XPBDFEM/Xpbd.h:217-263) on its
// velocities: one constraint for the Pixar models, the pair for the others,
// nothing for the cube models. damp: the Rayleigh ratio (x 8 when amortized).
__device__ __forceinline__ void rayleigh_tet(const Mat& bp, const TetRec& r, const float4 X[4], float4 V[4],
                                             float inv_dt, float damp) {
	if (bp.model == kModelNone) return;  // SolveElementCube damps quads and hexes only
	const float q[3][3] = {{r.a.x, r.a.y, r.a.z}, {r.a.w, r.b.x, r.b.y}, {r.b.z, r.b.w, r.c.x}};
	const float QQ[3] = {r.c.y, r.c.z, r.c.w};
	const float QR[3] = {r.d.x, r.d.y, r.d.z};
	const float w[4] = {X[0].w, X[1].w, X[2].w, X[3].w};
	Vec3 P[3];
#pragma unroll
	for (int i = 0; i < 3; i++) P[i] = {X[i].x - X[3].x, X[i].y - X[3].y, X[i].z - X[3].z};
	Vec3 g0[4], g1[4];
	const float ib0 = r.d.w * inv_dt / damp, ib1 = ib0 * bp.ratio;  // comp / (dt damping)
	if (bp.model == kModelPixar) {
		// SolveElementPixar with DampingMode::On (XPBDFEM/Fem.cpp:429-430): one constraint
		const float U = pixar_energy(bp, q, QQ, QR, P, g0, g1);
		float gV = 0.0f;
#pragma unroll
		for (int n = 0; n < 4; n++) gV = fmaf(g0[n].x, V[n].x, fmaf(g0[n].y, V[n].y, fmaf(g0[n].z, V[n].z, gV)));
		const float l = -gV / fmaf(2.0f * U, ib0, wdot(w, g0, g0));
#pragma unroll
		for (int n = 0; n < 4; n++) {
			const float s = w[n] * l;
			V[n].x = fmaf(s, g0[n].x, V[n].x);
			V[n].y = fmaf(s, g0[n].y, V[n].y);
			V[n].z = fmaf(s, g0[n].z, V[n].z);
		}
		return;
	}
	const float U0 = deviatoric<true>(bp, QQ, QR, P, g0);
	const float U1 = hydrostatic(q, P, bp.a, g1);
	if (bp.simultaneous) {
		float b0 = 0.0f, b1 = 0.0f;
#pragma unroll
		for (int n = 0; n < 4; n++) {
			b0 -= fmaf(g0[n].x, V[n].x, fmaf(g0[n].y, V[n].y, g0[n].z * V[n].z));
			b1 -= fmaf(g1[n].x, V[n].x, fmaf(g1[n].y, V[n].y, g1[n].z * V[n].z));
		}
		float l0, l1;
		cramer(fmaf(2.0f * U0, ib0, wdot(w, g0, g0)), wdot(w, g0, g1), fmaf(2.0f * U1, ib1, wdot(w, g1, g1)), b0, b1, l0,
		       l1);
#pragma unroll
		for (int n = 0; n < 4; n++) {
			V[n].x = fmaf(w[n], fmaf(l1, g1[n].x, l0 * g0[n].x), V[n].x);
			V[n].y = fmaf(w[n], fmaf(l1, g1[n].y, l0 * g0[n].y), V[n].y);
			V[n].z = fmaf(w[n], fmaf(l1, g1[n].z, l0 * g0[n].z), V[n].z);
		}
	} else {
		const Vec3* gs[2] = {g0, g1};
		const float Us[2] = {U0, U1}, ibs[2] = {ib0, ib1};
#pragma unroll
		for (int k = 0; k < 2; k++) {
			const Vec3* g = gs[k];
			float gV = 0.0f;
#pragma unroll
			for (int n = 0; n < 4; n++) gV = fmaf(g[n].x, V[n].x, fmaf(g[n].y, V[n].y, fmaf(g[n].z, V[n].z, gV)));
			const float l = -gV / fmaf(2.0f * Us[k], ibs[k], wdot(w, g, g));
#pragma unroll
			for (int n = 0; n < 4; n++) {
				const float s = w[n] * l;
				V[n].x = fmaf(s, g[n].x, V[n].x);
				V[n].y = fmaf(s, g[n].y, V[n].y);
				V[n].z = fmaf(s, g[n].z, V[n].z);
			}
		}
	}
}

// One element solve: SolveElementMixed's tet path (XPBDFEM/Fem.cpp:437-564)
// with EnergyXpbdConstrainSimultaneous<2> (XPBDFEM/Xpbd.h:123-215) or the
// serial EnergyXpbdConstrain pair (XPBDFEM/Xpbd.h:87-121). EXT (the extended
// kernels) adds the in-solve Rayleigh damping (Paper, Limit), Mixed's clamp,
// the Pixar models (one constraint) and the cube models (no constraint on a
// tet). O[]: start positions + w, D[]: displacements (updated). alpha0 = c0 / dt^2 with c0 = (1/mu)/volume stored per tet;
// alpha1 = alpha0 * (mu / lambda), i.e. (1/lambda)/volume/dt^2.
template <bool EXT = false>
__device__ __forceinline__ float2 solve_tet(const Mat& bp, const TetRec& r, float inv_dt, float inv_dt2,
                                            const float4 O[4], float4 D[4]) {
	constexpr bool DAMP = EXT;
	const float q[3][3] = {{r.a.x, r.a.y, r.a.z}, {r.a.w, r.b.x, r.b.y}, {r.b.z, r.b.w, r.c.x}};
	const float QQ[3] = {r.c.y, r.c.z, r.c.w};
	const float QR[3] = {r.d.x, r.d.y, r.d.z};
	const float alpha0 = r.d.w * inv_dt2;
	const float alpha1 = alpha0 * bp.ratio;
	const float w[4] = {O[0].w, O[1].w, O[2].w, O[3].w};
	if (EXT && bp.model == kModelNone) return make_float2(0.0f, 0.0f);
	Vec3 P[3];
#pragma unroll
	for (int i = 0; i < 3; i++)
		P[i] = {(O[i].x - O[3].x) + (D[i].x - D[3].x), (O[i].y - O[3].y) + (D[i].y - D[3].y),
		        (O[i].z - O[3].z) + (D[i].z - D[3].z)};
	Vec3 g0[4], g1[4];
	if (EXT && bp.model == kModelPixar) {
		// SolveElementPixar (XPBDFEM/Fem.cpp:361-433): U = I1 + (lambda/2)
		// (J - a)^2 (mu / 2 = 1) as one EnergyXpbdConstrain with the
		// compliance per volume c0
		const float U = pixar_energy(bp, q, QQ, QR, P, g0, g1);
		const float l = serial_lambda<true>(bp, U, g0, w, D, alpha0, r.d.w, inv_dt);
#pragma unroll
		for (int n = 0; n < 4; n++) {
			const float s = w[n] * l;
			D[n].x = fmaf(s, g0[n].x, D[n].x);
			D[n].y = fmaf(s, g0[n].y, D[n].y);
			D[n].z = fmaf(s, g0[n].z, D[n].z);
		}
		return make_float2(l, 0.0f);
	}
	const float U0 = deviatoric<EXT>(bp, QQ, QR, P, g0);
	float l0, l1;
	if (bp.simultaneous) {
		const float U1 = hydrostatic(q, P, bp.a, g1);
		if (!DAMP || !(bp.damp > 0.0f)) {
			const float A0 = fmaf(2.0f * U0, alpha0, wdot(w, g0, g0));
			const float A1 = wdot(w, g1, g0);
			const float A2 = fmaf(2.0f * U1, alpha1, wdot(w, g1, g1));
			// Cramer's rule as in XPBDFEM/Xpbd.h:172-180
			cramer(A0, A1, A2, -2.0f * U0, -2.0f * U1, l0, l1);
		} else {
			// XPBDFEM/Xpbd.h:133-205: gV = g . (X - O), Paper scales the
			// diagonal and right-hand side by 1 / (1 + gamma), Limit adds a
			// second solve towards the Rayleigh target
			const float wgg0 = wdot(w, g0, g0), wgg1 = wdot(w, g1, g0), wgg2 = wdot(w, g1, g1);
			float gV0 = 0.0f, gV1 = 0.0f;
#pragma unroll
			for (int n = 0; n < 4; n++) {
				gV0 = fmaf(g0[n].x, D[n].x, fmaf(g0[n].y, D[n].y, fmaf(g0[n].z, D[n].z, gV0)));
				gV1 = fmaf(g1[n].x, D[n].x, fmaf(g1[n].y, D[n].y, fmaf(g1[n].z, D[n].z, gV1)));
			}
			const float gamma = bp.damp * inv_dt;
			float A0, A2, b0 = -2.0f * U0, b1 = -2.0f * U1;
			if (!bp.limit) {
				const float s = 1.0f / (1.0f + gamma);
				A0 = wgg0 + (2.0f * U0 * alpha0) * s;
				A2 = wgg2 + (2.0f * U1 * alpha1) * s;
				b0 = (b0 - gamma * gV0) * s;
				b1 = (b1 - gamma * gV1) * s;
			} else {
				A0 = fmaf(2.0f * U0, alpha0, wgg0);
				A2 = fmaf(2.0f * U1, alpha1, wgg2);
			}
			cramer(A0, wgg1, A2, b0, b1, l0, l1);
			if (bp.limit) {
				const float ib = r.d.w * inv_dt / bp.damp;  // comp0 / (dt damping)
				const float B0 = fmaf(2.0f * U0, ib, wgg0), B2 = fmaf(2.0f * U1, ib * bp.ratio, wgg2);
				float e0 = fmaf(b0, -1.0f - alpha0 * l0, -gV0), e1 = fmaf(b1, -1.0f - alpha1 * l1, -gV1);
				e0 *= B0 / fmaxf(B0, 8.0f * wgg0);
				e1 *= B2 / fmaxf(B2, 8.0f * wgg2);
				float d0, d1;
				cramer(B0, wgg1, B2, e0, e1, d0, d1);
				l0 += d0;
				l1 += d1;
			}
		}
#pragma unroll
		for (int n = 0; n < 4; n++) {
			D[n].x = fmaf(w[n], fmaf(l1, g1[n].x, l0 * g0[n].x), D[n].x);
			D[n].y = fmaf(w[n], fmaf(l1, g1[n].y, l0 * g0[n].y), D[n].y);
			D[n].z = fmaf(w[n], fmaf(l1, g1[n].z, l0 * g0[n].z), D[n].z);
		}
	} else {
		l0 = serial_lambda<DAMP>(bp, U0, g0, w, D, alpha0, r.d.w, inv_dt);
#pragma unroll
		for (int n = 0; n < 4; n++) {
			const float s = w[n] * l0;
			D[n].x = fmaf(s, g0[n].x, D[n].x);
			D[n].y = fmaf(s, g0[n].y, D[n].y);
			D[n].z = fmaf(s, g0[n].z, D[n].z);
		}
#pragma unroll
		for (int i = 0; i < 3; i++)
			P[i] = {(O[i].x - O[3].x) + (D[i].x - D[3].x), (O[i].y - O[3].y) + (D[i].y - D[3].y),
			        (O[i].z - O[3].z) + (D[i].z - D[3].z)};
		const float U1 = hydrostatic(q, P, bp.a, g1);
		l1 = serial_lambda<DAMP>(bp, U1, g1, w, D, alpha1, r.d.w * bp.ratio, inv_dt);
#pragma unroll
		for (int n = 0; n < 4; n++) {
			const float s = w[n] * l1;
			D[n].x = fmaf(s, g1[n].x, D[n].x);
			D[n].y = fmaf(s, g1[n].y, D[n].y);
			D[n].z = fmaf(s, g1[n].z, D[n].z);
		}
	}
	return make_float2(l0, l1);
}

// PbdDamp (XPBDFEM/Xpbd.h:307-346): moves the tet's velocities towards its
// rigid motion (mass-weighted centre velocity plus the rotation that carries
// its angular momentum) by the fraction `damping`.
__device__ __forceinline__ void pbd_tet(const float4 X[4], float4 V[4], float damping) {
	float Wsum = 1.0e-8f;
#pragma unroll
	for (int i = 0; i < 4; i++) Wsum += X[i].w;
	const float Wavg = Wsum * 0.25f, Wmin = 0.0001f * Wavg;
	Vec3 x[4], xcm = {0.0f, 0.0f, 0.0f}, vcm = {0.0f, 0.0f, 0.0f};
	float M[4], Msum = 0.0f;
#pragma unroll
	for (int i = 0; i < 4; i++) {
		x[i] = {X[i].x - X[3].x, X[i].y - X[3].y, X[i].z - X[3].z};
		M[i] = Wavg / fmaxf(Wmin, X[i].w);
		xcm = {fmaf(x[i].x, M[i], xcm.x), fmaf(x[i].y, M[i], xcm.y), fmaf(x[i].z, M[i], xcm.z)};
		vcm = {fmaf(V[i].x, M[i], vcm.x), fmaf(V[i].y, M[i], vcm.y), fmaf(V[i].z, M[i], vcm.z)};
		Msum += M[i];
	}
	const float im = 1.0f / Msum;
	xcm = {xcm.x * im, xcm.y * im, xcm.z * im};
	vcm = {vcm.x * im, vcm.y * im, vcm.z * im};
	Vec3 r[4], L = {0.0f, 0.0f, 0.0f};
	float I00 = 0.0f, I11 = 0.0f, I22 = 0.0f, I01 = 0.0f, I12 = 0.0f, I02 = 0.0f;
#pragma unroll
	for (int i = 0; i < 4; i++) {
		r[i] = {x[i].x - xcm.x, x[i].y - xcm.y, x[i].z - xcm.z};
		const Vec3 c = cross(r[i], v3(V[i]));
		L = {fmaf(M[i], c.x, L.x), fmaf(M[i], c.y, L.y), fmaf(M[i], c.z, L.z)};
		const float xx = r[i].x * r[i].x, yy = r[i].y * r[i].y, zz = r[i].z * r[i].z;
		I00 = fmaf(M[i], yy + zz, I00);
		I11 = fmaf(M[i], xx + zz, I11);
		I22 = fmaf(M[i], xx + yy, I22);
		I01 = fmaf(-M[i], r[i].x * r[i].y, I01);
		I12 = fmaf(-M[i], r[i].y * r[i].z, I12);
		I02 = fmaf(-M[i], r[i].z * r[i].x, I02);
	}
	// omega = I^-1 L (I symmetric): adjugate over determinant
	const float a00 = fmaf(I11, I22, -I12 * I12), a01 = fmaf(I02, I12, -I01 * I22), a02 = fmaf(I01, I12, -I02 * I11);
	const float a11 = fmaf(I00, I22, -I02 * I02), a12 = fmaf(I01, I02, -I00 * I12), a22 = fmaf(I00, I11, -I01 * I01);
	const float idet = 1.0f / fmaf(I00, a00, fmaf(I01, a01, I02 * a02));
	const Vec3 om = {fmaf(a00, L.x, fmaf(a01, L.y, a02 * L.z)) * idet, fmaf(a01, L.x, fmaf(a11, L.y, a12 * L.z)) * idet,
	                 fmaf(a02, L.x, fmaf(a12, L.y, a22 * L.z)) * idet};
#pragma unroll
	for (int i = 0; i < 4; i++) {
		const Vec3 c = cross(om, r[i]);
		V[i].x = fmaf(damping, (vcm.x + c.x) - V[i].x, V[i].x);
		V[i].y = fmaf(damping, (vcm.y + c.y) - V[i].y, V[i].y);
		V[i].z = fmaf(damping, (vcm.z + c.z) - V[i].z, V[i].z);
	}
}

// ---- chunk staging: one TMA bulk copy per chunk into the warp's buffer ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* m) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(m)) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Issued by one lane: expect `bytes` on the barrier and start the copy.
// The chunk records stream through L2 once per substep (about as large as
// L2); they are fetched with an evict-first policy so that they do not push
// the small, hot vertex state out of L2.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
	uint64_t policy;
	asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
	asm volatile(
	    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
	        smem_u32(dst)),
	    "l"(src), "r"(bytes), "r"(smem_u32(mbar)), "l"(policy)
	    : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* m, uint32_t parity) {
	uint32_t ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(smem_u32(m)), "r"(parity)
	    : "memory");
	return ok != 0;
}

// Bounded wait for the copy of the current phase. On timeout the error word
// is set and the wait continues for one more bounded period so that no copy
// is left in flight when the block leaves.
__device__ bool mbar_wait(const DevCtx& C, uint64_t* m, uint32_t parity) {
	uint64_t t0 = 0;
	for (uint32_t spins = 0;; spins++) {
		if (mbar_test(m, parity)) return true;
		if ((spins & 1023u) == 1023u) {
			const uint64_t t = global_ns();
			if (t0 == 0) {
				t0 = t;
			} else if (t - t0 > C.timeout_ns) {
				atomicCAS(C.err, 0, kErrCopyTimeout);
				for (uint32_t k = 0;; k++) {
					if (mbar_test(m, parity)) break;
					if ((k & 1023u) == 1023u && global_ns() - t > C.timeout_ns) break;
				}
				return false;
			}
		}
	}
}

// Per-warp staging state: the chunk buffer, the vertex slots, the barrier.
struct Stage {
	uint8_t* buf;     // chunk block (records, header, vertex ids, slots)
	float4* vs;       // vertex slots: O at [s * 32 + lane], D at [(nvmax + s) * 32 + lane]
	uint64_t* mbar;
	uint32_t parity;
	int inflight;     // chunk whose copy is in flight or resident, -1 = none
	uint4 meta;       // that chunk's descriptor (DevCtx::chunks)
};

// Starts the copy of `chunk`, whose descriptor m the caller has loaded.
__device__ __forceinline__ void stage_issue_m(const DevCtx& C, Stage& st, uint32_t chunk, const uint4& m, uint32_t lane) {
	__syncwarp();
	if (lane == 0) bulk_copy_g2s(st.buf, C.cblk + m.x, m.y, st.mbar);
	st.inflight = (int)chunk;
	st.meta = m;
}

__device__ __forceinline__ void stage_issue(const DevCtx& C, Stage& st, uint32_t chunk, uint32_t lane) {
	stage_issue_m(C, st, chunk, __ldg(reinterpret_cast<const uint4*>(C.chunks) + chunk), lane);
}

// Starts the copy of `chunk` when the buffer is idle (dataflow mode issues it
// before waiting on neighbours: records never depend on them).
__device__ __forceinline__ void stage_issue_or_wait(const DevCtx& C, Stage& st, uint32_t chunk, uint32_t lane) {
	if (st.inflight < 0) stage_issue(C, st, chunk, lane);
}

// Makes `chunk` resident in the warp's buffer. Returns false on timeout.
__device__ __forceinline__ bool stage_acquire(const DevCtx& C, Stage& st, uint32_t chunk, uint32_t lane) {
	if (st.inflight != (int)chunk) {
		if (st.inflight >= 0) {  // a different copy is in flight: let it land first
			if (!mbar_wait(C, st.mbar, st.parity)) return false;
			st.parity ^= 1u;
		}
		stage_issue(C, st, chunk, lane);
	}
	const bool ok = mbar_wait(C, st.mbar, st.parity);
	st.parity ^= 1u;
	st.inflight = -1;
	return ok;
}

// Chunks whose clusters are all whole cubes of the 6-tet split in the
// generator's corner order (every configuration mesh) share one local
// topology, so the 8 vertices stay in registers and the 6 solves unroll with
// compile-time slots: no shared-memory round trip inside the sequential chain.
// Local slot k of tet t: {0123, 0341, 0543, 0365, 0763, 0327}, packed four bits per slot.
__host__ __device__ constexpr int cube_slot(int t, int k) {
	return (int)(((t == 0   ? 0x3210u
	               : t == 1 ? 0x1430u
	               : t == 2 ? 0x3450u
	               : t == 3 ? 0x5630u
	               : t == 4 ? 0x3670u
	                        : 0x7230u) >>
	              (4 * k)) &
	             15u);
}

// The calling warp's chunk buffer, vertex slots and mbarrier.
__device__ __forceinline__ Stage stage_init(const DevCtx& C, uint32_t lane) {
	extern __shared__ __align__(128) uint8_t smem[];
	__shared__ uint64_t mbars[32];
	const uint32_t w = threadIdx.x >> 5;
	uint8_t* base = smem + (size_t)w * C.warp_smem;
	Stage st = {base, reinterpret_cast<float4*>(base + C.vs_off), &mbars[w], 0u, -1, make_uint4(0u, 0u, 0u, 0u)};
	if (lane == 0) mbar_init(st.mbar);
	__syncwarp();
	return st;
}

}  // namespace

}  // namespace xfem
