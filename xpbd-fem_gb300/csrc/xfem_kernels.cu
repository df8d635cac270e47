// CUDA kernels of libxfem.so (sm_103a): the coloured Gauss-Seidel XPBD substep.
//
// Data layout in HBM (all device-order, see xfem_internal.h):
//   vert[2v]   = (O.x, O.y, O.z, w)   position at the start of the substep and
//                                     inverse mass; between calls: X
//   vert[2v+1] = (D.x, D.y, D.z, bits) displacement within the substep; between
//                                     calls: V. bits = lock | contact | body<<8
// One 32-byte sector per vertex, so a gather touches one sector.
//
// Work unit: a cluster = up to 8 tets sharing vertices, solved in sequence by
// one thread with its (<= 8) vertices staged in shared memory. Clusters of one
// colour share no vertex, so there is no atomic and no race. 32 clusters of a
// colour form a chunk (one warp); chunk data is stored lane-minor so every
// per-lane load of a warp is one contiguous 128- or 512-byte run.
//
// Substep schedule (Geo3d::Substep, XPBDFEM/Geo.cpp:305-356, restated):
//   each colour pass: every cluster first advances the vertices it owns (it is
//              the lowest-colour cluster touching them): finalize the
//              previous substep (locks, ground, V = D/dt, O += D) and predict
//              this one (V += g dt, V *= 1 - drag, D = V dt); then it solves
//              its tets in sequence
//   end      : finalize the last substep back to (X, V)
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "xfem_internal.h"

namespace xfem {

namespace {

constexpr uint64_t kBarrierTimeoutNs = 2000000000ull;  // 2 s: far above any legal wait

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
	uint32_t v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ uint64_t global_ns() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Grid-wide barrier for the co-resident persistent grid. Monotonic arrival
// counter (zeroed before each launch); every wait is bounded: on timeout the
// block records kErrBarrierTimeout and all blocks leave at their next barrier.
__device__ bool grid_sync(const DevCtx& C, uint32_t& target) {
	__shared__ int s_ok;
	__syncthreads();
	target += gridDim.x;
	if (threadIdx.x == 0) {
		int ok = 1;
		__threadfence();
		atomicAdd(C.bar_count, 1u);
		uint32_t spins = 0;
		uint64_t t0 = 0;
		while (ld_acquire_gpu(C.bar_count) < target) {
			if (++spins == 256) {
				spins = 0;
				if (*(volatile int*)C.err) {
					ok = 0;
					break;
				}
				const uint64_t t = global_ns();
				if (t0 == 0) {
					t0 = t;
				} else if (t - t0 > kBarrierTimeoutNs) {
					atomicCAS(C.err, 0, kErrBarrierTimeout);
					ok = 0;
					break;
				}
			}
		}
		s_ok = ok;
	}
	__syncthreads();
	return s_ok != 0;
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

// End of a substep for one vertex: locks (XPBDFEM/Geo.cpp:318-322), ground,
// then the velocity V = D / dt (XPBDFEM/Geo.cpp:342-344) is returned.
__device__ __forceinline__ Vec3 finish_vertex(const BodyParams& bp, float4& O, float4& D, uint32_t& bits, float inv_dt) {
	if (bp.lock_active && (bits & kFlagLocked)) {
		D.x = D.y = D.z = 0.0f;
		O.w = 0.0f;
	}
	bits &= ~kFlagContact;
	if (bp.ground && O.w > 0.0f && ground_contact(bp, O, D)) bits |= kFlagContact;
	return {D.x * inv_dt, D.y * inv_dt, D.z * inv_dt};
}

// Finalize the previous substep (unless `first`: (O, D) then hold the
// canonical (X, V)) and predict the next (XPBDFEM/Geo.cpp:307-312).
__device__ __forceinline__ void advance_vertex(const BodyParams* bodies, float4& O, float4& D, bool first, float dt,
                                               float inv_dt) {
	uint32_t bits = __float_as_uint(D.w);
	const BodyParams& bp = bodies[bits >> 8];
	Vec3 V;
	if (first) {
		V = v3(D);
	} else {
		V = finish_vertex(bp, O, D, bits, inv_dt);
		O.x += D.x;
		O.y += D.y;
		O.z += D.z;
	}
	V.x = (V.x + bp.gravity[0] * dt) * bp.drag_mul;
	V.y = (V.y + bp.gravity[1] * dt) * bp.drag_mul;
	V.z = (V.z + bp.gravity[2] * dt) * bp.drag_mul;
	D = make_float4(V.x * dt, V.y * dt, V.z * dt, __uint_as_float(bits));
}

// Finalize the last substep of a launch: (O, D) -> canonical (X, V).
__device__ __forceinline__ void finalize_vertex(const BodyParams* bodies, float4& O, float4& D, float inv_dt) {
	uint32_t bits = __float_as_uint(D.w);
	const BodyParams& bp = bodies[bits >> 8];
	const Vec3 V = finish_vertex(bp, O, D, bits, inv_dt);
	O.x += D.x;
	O.y += D.y;
	O.z += D.z;
	D = make_float4(V.x, V.y, V.z, __uint_as_float(bits));
}

// Rest state of one tet: Qi column-major q[c][r], QQ, QR and c0 = (1/mu)/vol.
struct TetRec {
	float4 a, b, c, d;
};

// The material scalars a solve needs, copied to registers once per cluster.
struct Mat {
	float a, ratio, y0, y1, y2;
	uint32_t energy, simultaneous;
};

__device__ __forceinline__ Mat load_mat(const BodyParams* bodies, uint32_t body) {
	const BodyParams* b = bodies + body;
	return {__ldg(&b->a), __ldg(&b->ratio), __ldg(&b->yeoh[0]), __ldg(&b->yeoh[1]), __ldg(&b->yeoh[2]),
	        __ldg(&b->energy), __ldg(&b->simultaneous)};
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

__device__ __forceinline__ float hydrostatic(const float q[3][3], const Vec3 P[3], float a, Vec3 g[4]) {
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
	return Ja * Ja;
}

// 1/x to about one ulp: hardware approximation plus one Newton step. The
// arguments are sums of squares plus 1e-22 (or a clamp at 1e-8), never zero,
// denormal or infinite.
__device__ __forceinline__ float rcp(float x) {
	float r;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
	return fmaf(r, fmaf(-x, r, 1.0f), r);
}

// Deviatoric term, prefactored (XPBDFEM/Fem.cpp:163-192), with the Yeoh
// transform of XPBDFEM/Fem.cpp:525-531 when energy == 7.
__device__ __forceinline__ float deviatoric(const Mat& bp, const float QQ[3], const float QR[3], const Vec3 P[3],
                                            Vec3 g[4]) {
	float U = QQ[0] * dot(P[0], P[0]);
	U = fmaf(QQ[1], dot(P[1], P[1]), U);
	U = fmaf(QQ[2], dot(P[2], P[2]), U);
	U = fmaf(QR[0], dot(P[0], P[1]), U);
	U = fmaf(QR[1], dot(P[0], P[2]), U);
	U = fmaf(QR[2], dot(P[1], P[2]), U);
	const float d0 = 2.0f * QQ[0], d1 = 2.0f * QQ[1], d2 = 2.0f * QQ[2];
	g[0] = {fmaf(d0, P[0].x, fmaf(QR[0], P[1].x, QR[1] * P[2].x)), fmaf(d0, P[0].y, fmaf(QR[0], P[1].y, QR[1] * P[2].y)),
	        fmaf(d0, P[0].z, fmaf(QR[0], P[1].z, QR[1] * P[2].z))};
	g[1] = {fmaf(d1, P[1].x, fmaf(QR[0], P[0].x, QR[2] * P[2].x)), fmaf(d1, P[1].y, fmaf(QR[0], P[0].y, QR[2] * P[2].y)),
	        fmaf(d1, P[1].z, fmaf(QR[0], P[0].z, QR[2] * P[2].z))};
	g[2] = {fmaf(d2, P[2].x, fmaf(QR[1], P[0].x, QR[2] * P[1].x)), fmaf(d2, P[2].y, fmaf(QR[1], P[0].y, QR[2] * P[1].y)),
	        fmaf(d2, P[2].z, fmaf(QR[1], P[0].z, QR[2] * P[1].z))};
	g[3] = {-(g[0].x + g[1].x + g[2].x), -(g[0].y + g[1].y + g[2].y), -(g[0].z + g[1].z + g[2].z)};
	if (bp.energy == 7u) {
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

// One element solve: SolveElementMixed<MixedSelective | YeohSkinFast> tet path
// (XPBDFEM/Fem.cpp:437-564) with EnergyXpbdConstrainSimultaneous<2>
// (XPBDFEM/Xpbd.h:123-215) or the serial EnergyXpbdConstrain pair
// (XPBDFEM/Xpbd.h:87-121). O[]: start positions + w, D[]: displacements
// (updated). alpha0 = c0 / dt^2 with c0 = (1/mu)/volume stored per tet;
// alpha1 = alpha0 * (mu / lambda), i.e. (1/lambda)/volume/dt^2.
__device__ __forceinline__ float2 solve_tet(const Mat& bp, const TetRec& r, float inv_dt2, const float4 O[4],
                                            float4 D[4]) {
	const float q[3][3] = {{r.a.x, r.a.y, r.a.z}, {r.a.w, r.b.x, r.b.y}, {r.b.z, r.b.w, r.c.x}};
	const float QQ[3] = {r.c.y, r.c.z, r.c.w};
	const float QR[3] = {r.d.x, r.d.y, r.d.z};
	const float alpha0 = r.d.w * inv_dt2;
	const float alpha1 = alpha0 * bp.ratio;
	const float w[4] = {O[0].w, O[1].w, O[2].w, O[3].w};
	Vec3 P[3];
#pragma unroll
	for (int i = 0; i < 3; i++)
		P[i] = {(O[i].x - O[3].x) + (D[i].x - D[3].x), (O[i].y - O[3].y) + (D[i].y - D[3].y),
		        (O[i].z - O[3].z) + (D[i].z - D[3].z)};
	Vec3 g0[4], g1[4];
	const float U0 = deviatoric(bp, QQ, QR, P, g0);
	float l0, l1;
	if (bp.simultaneous) {
		const float U1 = hydrostatic(q, P, bp.a, g1);
		const float A0 = fmaf(2.0f * U0, alpha0, wdot(w, g0, g0));
		const float A1 = wdot(w, g1, g0);
		const float A2 = fmaf(2.0f * U1, alpha1, wdot(w, g1, g1));
		const float b0 = -2.0f * U0, b1 = -2.0f * U1;
		// Cramer's rule as in XPBDFEM/Xpbd.h:172-180
		const float i00 = rcp(A0), i11 = rcp(A2);
		const float r0 = A1 * i00, r1 = A1 * i11;
		const float inv_det = rcp(fmaxf(0.00000001f, fmaf(-r0, r1, 1.0f)));
		const float c0 = b0 * i00, c1 = b1 * i11;
		l0 = inv_det * fmaf(-r0, c1, c0);
		l1 = inv_det * fmaf(-c0, r1, c1);
#pragma unroll
		for (int n = 0; n < 4; n++) {
			D[n].x = fmaf(w[n], fmaf(l1, g1[n].x, l0 * g0[n].x), D[n].x);
			D[n].y = fmaf(w[n], fmaf(l1, g1[n].y, l0 * g0[n].y), D[n].y);
			D[n].z = fmaf(w[n], fmaf(l1, g1[n].z, l0 * g0[n].z), D[n].z);
		}
	} else {
		l0 = (-2.0f * U0) * rcp(fmaf(2.0f * U0, alpha0, wdot(w, g0, g0)));
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
		l1 = (-2.0f * U1) * rcp(fmaf(2.0f * U1, alpha1, wdot(w, g1, g1)));
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
			} else if (t - t0 > kBarrierTimeoutNs) {
				atomicCAS(C.err, 0, kErrCopyTimeout);
				for (uint32_t k = 0;; k++) {
					if (mbar_test(m, parity)) break;
					if ((k & 1023u) == 1023u && global_ns() - t > kBarrierTimeoutNs) break;
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
};

__device__ __forceinline__ void stage_issue(const DevCtx& C, Stage& st, uint32_t chunk, uint32_t lane) {
	const uint4 m = __ldg(reinterpret_cast<const uint4*>(C.chunks) + chunk);
	__syncwarp();
	if (lane == 0) bulk_copy_g2s(st.buf, C.cblk + m.x, m.y, st.mbar);
	st.inflight = (int)chunk;
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

// Header word of a cluster lane: nv | nt << 4 | advance mask << 8 | body << 16.
// A vertex is advanced (previous substep finalized, next one predicted) by
// the lowest-colour cluster touching it, just before that cluster's solve.

template <bool LAMBDAS>
__device__ __forceinline__ void run_chunk_cube(const DevCtx& C, Stage& st, int next, uint32_t lane, bool first, float dt,
                                               float inv_dt, float inv_dt2, uint32_t trow) {
	const float4* rec = reinterpret_cast<const float4*>(st.buf);
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(st.buf + 2048u * 6u);
	const uint32_t* vids = hdrs + kLanes;
	const uint32_t hdr = hdrs[lane];
	const bool live = (hdr & 15u) != 0;
	const uint32_t mask = (hdr >> 8) & 0xffu;
	uint32_t vid[8];
	float4 O[8], D[8];
	if (live) {
		const Mat mat = load_mat(C.bodies, hdr >> 16);
#pragma unroll
		for (int s = 0; s < 8; s++) vid[s] = vids[s * kLanes + lane];
#pragma unroll
		for (int s = 0; s < 8; s++) {
			O[s] = __ldcg(C.vert + 2 * (size_t)vid[s]);
			D[s] = __ldcg(C.vert + 2 * (size_t)vid[s] + 1);
		}
#pragma unroll
		for (int s = 0; s < 8; s++)
			if (mask & (1u << s)) advance_vertex(C.bodies, O[s], D[s], first, dt, inv_dt);
#pragma unroll
		for (int t = 0; t < 6; t++) {
			const float4* r = rec + t * 4 * kLanes + lane;
			const TetRec tr = {r[0], r[kLanes], r[2 * kLanes], r[3 * kLanes]};
			const float4 Ot[4] = {O[cube_slot(t, 0)], O[cube_slot(t, 1)], O[cube_slot(t, 2)], O[cube_slot(t, 3)]};
			float4 Dt[4] = {D[cube_slot(t, 0)], D[cube_slot(t, 1)], D[cube_slot(t, 2)], D[cube_slot(t, 3)]};
			const float2 lam = solve_tet(mat, tr, inv_dt2, Ot, Dt);
#pragma unroll
			for (int k = 0; k < 4; k++) D[cube_slot(t, k)] = Dt[k];
			if (LAMBDAS) C.tlam[(size_t)(trow + t) * kLanes + lane] = lam;
		}
	}
	if (next >= 0) stage_issue(C, st, (uint32_t)next, lane);  // buffer consumed: prefetch
	if (live) {
#pragma unroll
		for (int s = 0; s < 8; s++) {
			if (mask & (1u << s)) __stcg(C.vert + 2 * (size_t)vid[s], O[s]);
			__stcg(C.vert + 2 * (size_t)vid[s] + 1, D[s]);
		}
	}
}

// One warp processes one resident chunk; lane = cluster. `next` >= 0 is the
// warp's next chunk: its copy is issued as soon as this chunk's records have
// been consumed, so it overlaps the write-back and what follows.
template <bool LAMBDAS>
__device__ __forceinline__ void run_chunk(const DevCtx& C, Stage& st, uint32_t chunk, int next, uint32_t lane, bool first,
                                          float dt, float inv_dt, float inv_dt2) {
	const uint4 m = __ldg(reinterpret_cast<const uint4*>(C.chunks) + chunk);
	const uint32_t ntmax = m.z & 0xffu, nvmax = (m.z >> 8) & 0xffu, trow = m.w;
	if (m.z & kShapeCube) {
		run_chunk_cube<LAMBDAS>(C, st, next, lane, first, dt, inv_dt, inv_dt2, trow);
		return;
	}
	const float4* rec = reinterpret_cast<const float4*>(st.buf);
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(st.buf + 2048u * ntmax);
	const uint32_t* vids = hdrs + kLanes;
	const uint32_t* slots = vids + kLanes * nvmax;
	const uint32_t hdr = hdrs[lane];
	const uint32_t nv = hdr & 15u, nt = (hdr >> 4) & 15u, mask = (hdr >> 8) & 0xffu;
	float4* sO = st.vs + lane;
	float4* sD = st.vs + kLanes * nvmax + lane;
	uint32_t vid[kMaxClusterVerts];
	if (nv) {
		const Mat mat = load_mat(C.bodies, hdr >> 16);
#pragma unroll
		for (uint32_t s = 0; s < kMaxClusterVerts; s++)
			if (s < nv) vid[s] = vids[s * kLanes + lane];
#pragma unroll
		for (uint32_t s = 0; s < kMaxClusterVerts; s++) {
			if (s < nv) {
				float4 O = __ldcg(C.vert + 2 * (size_t)vid[s]);
				float4 D = __ldcg(C.vert + 2 * (size_t)vid[s] + 1);
				if (mask & (1u << s)) advance_vertex(C.bodies, O, D, first, dt, inv_dt);
				sO[s * kLanes] = O;
				sD[s * kLanes] = D;
			}
		}
		for (uint32_t t = 0; t < nt; t++) {
			const float4* r = rec + t * 4 * kLanes + lane;
			const TetRec tr = {r[0], r[kLanes], r[2 * kLanes], r[3 * kLanes]};
			const uint32_t sl = slots[t * kLanes + lane];
			const uint32_t s0 = sl & 15u, s1 = (sl >> 4) & 15u, s2 = (sl >> 8) & 15u, s3 = (sl >> 12) & 15u;
			const float4 O[4] = {sO[s0 * kLanes], sO[s1 * kLanes], sO[s2 * kLanes], sO[s3 * kLanes]};
			float4 D[4] = {sD[s0 * kLanes], sD[s1 * kLanes], sD[s2 * kLanes], sD[s3 * kLanes]};
			const float2 lam = solve_tet(mat, tr, inv_dt2, O, D);
			sD[s0 * kLanes] = D[0];
			sD[s1 * kLanes] = D[1];
			sD[s2 * kLanes] = D[2];
			sD[s3 * kLanes] = D[3];
			if (LAMBDAS) C.tlam[(size_t)(trow + t) * kLanes + lane] = lam;
		}
	}
	if (next >= 0) stage_issue(C, st, (uint32_t)next, lane);  // buffer consumed: prefetch
	if (nv) {
#pragma unroll
		for (uint32_t s = 0; s < kMaxClusterVerts; s++) {
			if (s < nv) {
				if (mask & (1u << s)) __stcg(C.vert + 2 * (size_t)vid[s], sO[s * kLanes]);
				__stcg(C.vert + 2 * (size_t)vid[s] + 1, sD[s * kLanes]);
			}
		}
	}
}

// Vertices in no tet: nothing else touches them, so one thread takes each
// through all nsub substeps at once (predict, then finalize + predict); the
// final finalize pass closes the last one.
__device__ __forceinline__ void run_isolated(const DevCtx& C, uint32_t begin, uint32_t step, uint32_t nsub, float dt,
                                             float inv_dt) {
	for (uint32_t i = begin; i < C.nisolated; i += step) {
		const uint32_t v = __ldg(C.isolated + i);
		float4 O = __ldcg(C.vert + 2 * (size_t)v), D = __ldcg(C.vert + 2 * (size_t)v + 1);
		for (uint32_t s = 0; s < nsub; s++) advance_vertex(C.bodies, O, D, s == 0, dt, inv_dt);
		__stcg(C.vert + 2 * (size_t)v, O);
		__stcg(C.vert + 2 * (size_t)v + 1, D);
	}
}

__device__ __forceinline__ void run_finalize(const DevCtx& C, uint32_t begin, uint32_t step, float inv_dt) {
	for (uint32_t v = begin; v < C.nverts; v += step) {
		float4 O = __ldcg(C.vert + 2 * (size_t)v), D = __ldcg(C.vert + 2 * (size_t)v + 1);
		finalize_vertex(C.bodies, O, D, inv_dt);
		__stcg(C.vert + 2 * (size_t)v, O);
		__stcg(C.vert + 2 * (size_t)v + 1, D);
	}
}

__device__ __forceinline__ Stage stage_init(const DevCtx& C, uint32_t lane) {
	extern __shared__ __align__(128) uint8_t smem[];
	__shared__ uint64_t mbars[32];
	const uint32_t w = threadIdx.x >> 5;
	uint8_t* base = smem + (size_t)w * C.warp_smem;
	Stage st = {base, reinterpret_cast<float4*>(base + C.chunk_smem), &mbars[w], 0u, -1};
	if (lane == 0) mbar_init(st.mbar);
	__syncwarp();
	return st;
}

// The warp's next chunk after `ch` (colour c of substep s): the next chunk of
// the same colour, else its first chunk of the following colours (wrapping
// into the next substep); -1 when the launch has no more work for it.
__device__ __forceinline__ int next_chunk(const DevCtx& C, uint32_t s, uint32_t nsub, uint32_t c, uint32_t ch,
                                          uint32_t gwarp, uint32_t nwarps) {
	if (ch + nwarps < __ldg(C.colour_chunk_begin + c + 1)) return (int)(ch + nwarps);
	for (uint32_t k = 1; k <= C.ncolours; k++) {
		uint32_t c2 = c + k, s2 = s;
		if (c2 >= C.ncolours) {
			c2 -= C.ncolours;
			s2++;
		}
		if (s2 >= nsub) return -1;
		const uint32_t first = __ldg(C.colour_chunk_begin + c2) + gwarp;
		if (first < __ldg(C.colour_chunk_begin + c2 + 1)) return (int)first;
	}
	return -1;
}

// Persistent kernel: nsub substeps x ncolours colour passes separated by the
// bounded grid barrier. Must be launched cooperatively (co-resident grid).
template <bool LAMBDAS>
__global__ void __launch_bounds__(256) k_persistent(DevCtx C, uint32_t nsub, float dt) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
	// chunk i of a colour goes to block i % grid, so chunks spread over all SMs
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = wpb * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	Stage st = stage_init(C, lane);
	run_isolated(C, gtid, nthreads, nsub, dt, inv_dt);
	uint32_t target = 0;
	bool ok = true;
	for (uint32_t s = 0; s < nsub && ok; s++) {
		for (uint32_t c = 0; c < C.ncolours && ok; c++) {
			const uint32_t cb = __ldg(C.colour_chunk_begin + c), ce = __ldg(C.colour_chunk_begin + c + 1);
			for (uint32_t ch = cb + gwarp; ch < ce; ch += nwarps) {
				if (!stage_acquire(C, st, ch, lane)) {
					ok = false;
					break;
				}
				run_chunk<LAMBDAS>(C, st, ch, next_chunk(C, s, nsub, c, ch, gwarp, nwarps), lane, s == 0, dt, inv_dt,
				                   inv_dt2);
			}
			if (!grid_sync(C, target)) ok = false;
		}
	}
	if (!ok) {
		// leave no copy in flight
		if (st.inflight >= 0) mbar_wait(C, st.mbar, st.parity);
		return;
	}
	run_finalize(C, gtid, nthreads, inv_dt);
}

__device__ __forceinline__ void st_release_gpu(uint32_t* p, uint32_t v) {
	asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Bounded wait until every neighbour chunk of `ch` has done its share of
// substep s: chunks of a lower colour must have completed s + 1 substeps,
// chunks of a higher colour s substeps (the previous one). One lane per
// neighbour; false (and the error word set) on timeout.
__device__ bool wait_deps(const DevCtx& C, uint32_t ch, uint32_t s, uint32_t lane) {
	const uint32_t b = __ldg(C.dep_begin + ch), e = __ldg(C.dep_begin + ch + 1);
	bool ok = true;
	for (uint32_t i = b + lane; i < e && ok; i += kLanes) {
		const uint32_t d = __ldg(C.deps + i);
		const uint32_t need = s + (d >> 31);
		if (need == 0) continue;
		const uint32_t* f = C.done + (d & 0x7fffffffu);
		uint32_t spins = 0;
		uint64_t t0 = 0;
		while (ld_acquire_gpu(f) < need) {
			if (++spins == 64) {
				spins = 0;
				if (*(volatile int*)C.err) {
					ok = false;
					break;
				}
				const uint64_t t = global_ns();
				if (t0 == 0) {
					t0 = t;
				} else if (t - t0 > kBarrierTimeoutNs) {
					atomicCAS(C.err, 0, kErrDepTimeout);
					ok = false;
					break;
				}
			}
		}
	}
	return __all_sync(0xffffffffu, ok);
}

// Persistent dataflow kernel: the same chunk sequence per warp as
// k_persistent, but a chunk waits only for the neighbouring chunks it shares
// vertices with (per-chunk completion counters) instead of a grid barrier per
// colour. Every dependency points to an earlier (substep, colour) item and each
// warp walks its items in that order, so with a co-resident grid the earliest
// unfinished item can always run: no deadlock. One grid barrier ends the
// launch before the final finalize pass.
template <bool LAMBDAS>
__global__ void __launch_bounds__(256) k_dataflow(DevCtx C, uint32_t nsub, float dt) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = wpb * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	Stage st = stage_init(C, lane);
	run_isolated(C, gtid, nthreads, nsub, dt, inv_dt);
	bool ok = true;
	for (uint32_t s = 0; s < nsub && ok; s++) {
		for (uint32_t c = 0; c < C.ncolours && ok; c++) {
			const uint32_t cb = __ldg(C.colour_chunk_begin + c), ce = __ldg(C.colour_chunk_begin + c + 1);
			for (uint32_t ch = cb + gwarp; ch < ce; ch += nwarps) {
				const int next = next_chunk(C, s, nsub, c, ch, gwarp, nwarps);
				if (st.inflight != (int)ch) stage_issue_or_wait(C, st, ch, lane);  // records do not depend on neighbours
				if (!wait_deps(C, ch, s, lane) || !stage_acquire(C, st, ch, lane)) {
					ok = false;
					break;
				}
				run_chunk<LAMBDAS>(C, st, ch, next, lane, s == 0, dt, inv_dt, inv_dt2);
				__syncwarp();
				if (lane == 0) {
					__threadfence();
					st_release_gpu(C.done + ch, s + 1);
				}
			}
		}
	}
	if (!ok && st.inflight >= 0) {
		mbar_wait(C, st.mbar, st.parity);  // leave no copy in flight
		st.inflight = -1;
	}
	uint32_t target = 0;
	if (!grid_sync(C, target) || !ok) return;
	run_finalize(C, gtid, nthreads, inv_dt);
}

// One colour pass as its own launch (CUDA-graph mode): one chunk per warp.
// In the first launch of a call, blocks past the colour's chunks step the
// isolated vertices through all nsub substeps.
template <bool LAMBDAS>
__global__ void __launch_bounds__(256, 1) k_colour(DevCtx C, uint32_t colour, int first, float dt, uint32_t solve_blocks,
                                                uint32_t nsub) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	if (blockIdx.x >= solve_blocks) {
		const uint32_t b = blockIdx.x - solve_blocks, nb = gridDim.x - solve_blocks;
		run_isolated(C, b * blockDim.x + threadIdx.x, nb * blockDim.x, nsub, dt, inv_dt);
		return;
	}
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t ch = __ldg(C.colour_chunk_begin + colour) + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
	if (ch >= __ldg(C.colour_chunk_begin + colour + 1)) return;
	Stage st = stage_init(C, lane);
	if (!stage_acquire(C, st, ch, lane)) return;
	run_chunk<LAMBDAS>(C, st, ch, -1, lane, first != 0, dt, inv_dt, inv_dt2);
}

__global__ void k_finalize(DevCtx C, float dt) {
	run_finalize(C, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, 1.0f / dt);
}

// ---- transfers ----------------------------------------------------------------
__global__ void k_gather_xyz(const float4* __restrict__ vert, int which, const uint32_t* __restrict__ dev_of,
                             uint32_t n, float* __restrict__ out) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float4 a = vert[2 * (size_t)dev_of[i] + (which & 1)];
	const float wv = a.w;
	if (which == 2) {  // inverse mass
		out[i] = wv;
		return;
	}
	if (which == 3) {  // contact bit
		out[i] = (__float_as_uint(wv) & kFlagContact) ? 1.0f : 0.0f;
		return;
	}
	out[3 * (size_t)i] = a.x;
	out[3 * (size_t)i + 1] = a.y;
	out[3 * (size_t)i + 2] = a.z;
}

__global__ void k_scatter_xyz(float4* __restrict__ vert, int which, const uint32_t* __restrict__ dev_of, uint32_t n,
                              const float* __restrict__ in) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	float4* p = vert + 2 * (size_t)dev_of[i] + which;
	float4 a = *p;
	a.x = in[3 * (size_t)i];
	a.y = in[3 * (size_t)i + 1];
	a.z = in[3 * (size_t)i + 2];
	*p = a;
}

// CalculateElementVolume for T4 (XPBDFEM/Fem.cpp:1066) summed in double.
__global__ void k_volume(const float4* __restrict__ vert, const uint32_t* __restrict__ tets, uint32_t nt,
                         double* __restrict__ out) {
	__shared__ double red[32];
	double acc = 0.0;
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
		const float4 x0 = vert[2 * (size_t)tets[4 * (size_t)t]], x1 = vert[2 * (size_t)tets[4 * (size_t)t + 1]];
		const float4 x2 = vert[2 * (size_t)tets[4 * (size_t)t + 2]], x3 = vert[2 * (size_t)tets[4 * (size_t)t + 3]];
		const double a = (double)x0.x - x3.x, b = (double)x1.x - x3.x, c = (double)x2.x - x3.x;
		const double d = (double)x0.y - x3.y, e = (double)x1.y - x3.y, f = (double)x2.y - x3.y;
		const double g = (double)x0.z - x3.z, h = (double)x1.z - x3.z, i = (double)x2.z - x3.z;
		acc += (a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g)) / 6.0;
	}
	for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
	__syncthreads();
	if (threadIdx.x < 32) {
		acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
		for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
		if (threadIdx.x == 0) atomicAdd(out, acc);
	}
}

}  // namespace

size_t solve_smem_bytes(int block, uint32_t warp_smem) { return (size_t)(block / 32) * warp_smem; }

static void set_smem_attr(const void* f, size_t bytes) {
	cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int configure_kernels(const LaunchCfg& cfg) {
	const size_t smem = solve_smem_bytes(cfg.block, cfg.warp_smem);
	set_smem_attr(cfg.lambdas ? (const void*)k_persistent<true> : (const void*)k_persistent<false>, smem);
	set_smem_attr(cfg.lambdas ? (const void*)k_colour<true> : (const void*)k_colour<false>, smem);
	set_smem_attr(cfg.lambdas ? (const void*)k_dataflow<true> : (const void*)k_dataflow<false>, smem);
	return (int)cudaGetLastError();
}

int persistent_grid(const LaunchCfg& cfg, int* blocks_out) {
	const void* f = cfg.sync_mode == 3
	                    ? (cfg.lambdas ? (const void*)k_dataflow<true> : (const void*)k_dataflow<false>)
	                    : (cfg.lambdas ? (const void*)k_persistent<true> : (const void*)k_persistent<false>);
	const size_t smem = solve_smem_bytes(cfg.block, cfg.warp_smem);
	int dev = 0, sms = 0, per_sm = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, cfg.block, smem);
	if (e != cudaSuccess) return (int)e;
	*blocks_out = per_sm * sms;
	return per_sm > 0 ? 0 : (int)cudaErrorInvalidConfiguration;
}

int launch_substeps(const DevCtx& ctx, const LaunchCfg& cfg, uint32_t nsub, float dt, void* stream) {
	cudaStream_t st = (cudaStream_t)stream;
	const size_t smem = solve_smem_bytes(cfg.block, cfg.warp_smem);
	cudaError_t e = cudaSuccess;
	if (nsub == 0) return 0;
	if (cfg.sync_mode == 1 || cfg.sync_mode == 3) {
		e = cudaMemsetAsync(ctx.bar_count, 0, sizeof(uint32_t), st);
		if (e == cudaSuccess && cfg.sync_mode == 3) e = cudaMemsetAsync(ctx.done, 0, sizeof(uint32_t) * ctx.nchunks, st);
		if (e != cudaSuccess) return (int)e;
		DevCtx c = ctx;
		void* args[] = {&c, &nsub, &dt};
		const void* f = cfg.sync_mode == 1
		                    ? (cfg.lambdas ? (const void*)k_persistent<true> : (const void*)k_persistent<false>)
		                    : (cfg.lambdas ? (const void*)k_dataflow<true> : (const void*)k_dataflow<false>);
		e = cudaLaunchCooperativeKernel(f, dim3(cfg.blocks), dim3(cfg.block), args, smem, st);
		return (int)e;
	}
	// per-colour launches (captured into a CUDA graph by the caller when wanted)
	const void* fc = cfg.lambdas ? (const void*)k_colour<true> : (const void*)k_colour<false>;
	const uint32_t warps_per_block = cfg.block / 32;
	for (uint32_t s = 0; s < nsub; s++) {
		for (uint32_t c = 0; c < ctx.ncolours; c++) {
			const uint32_t nch = cfg.colour_chunk_begin_host[c + 1] - cfg.colour_chunk_begin_host[c];
			uint32_t sb = (nch + warps_per_block - 1) / warps_per_block;
			uint32_t extra = 0;
			if (s == 0 && c == 0 && ctx.nisolated) extra = (ctx.nisolated + cfg.block - 1) / cfg.block;
			const uint32_t grid = sb + extra;
			if (grid == 0) continue;
			DevCtx cc = ctx;
			uint32_t colour = c, ns = nsub;
			int first = s == 0 ? 1 : 0;
			float dtv = dt;
			void* args[] = {&cc, &colour, &first, &dtv, &sb, &ns};
			e = cudaLaunchKernel(fc, dim3(grid), dim3(cfg.block), args, smem, st);
			if (e != cudaSuccess) return (int)e;
		}
	}
	const uint32_t fb = (ctx.nverts + 255) / 256;
	if (fb) {
		k_finalize<<<fb, 256, 0, st>>>(ctx, dt);
		e = cudaGetLastError();
	}
	return (int)e;
}

int launch_gather_xyz(const float4* vert, int which, const uint32_t* dev_of_caller, uint32_t n, float* out,
                      void* stream) {
	if (!n) return 0;
	k_gather_xyz<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(vert, which, dev_of_caller, n, out);
	return (int)cudaGetLastError();
}

int launch_scatter_xyz(float4* vert, int which, const uint32_t* dev_of_caller, uint32_t n, const float* in,
                       void* stream) {
	if (!n) return 0;
	k_scatter_xyz<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(vert, which, dev_of_caller, n, in);
	return (int)cudaGetLastError();
}

int launch_volume(const float4* vert, const uint32_t* tets_dev, uint32_t nt, double* out, void* stream) {
	cudaStream_t st = (cudaStream_t)stream;
	cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
	if (e != cudaSuccess || !nt) return (int)e;
	uint32_t grid = (nt + 255) / 256;
	grid = grid > 1024 ? 1024 : grid;
	k_volume<<<grid, 256, 0, st>>>(vert, tets_dev, nt, out);
	return (int)cudaGetLastError();
}


// ---- allocation-free stepping ---------------------------------------------------
// Some callers cannot allocate device memory at the moment they step: a
// process whose device memory is fully reserved by another allocator (a
// framework's caching pool), a real-time loop that must not take cudaMalloc's
// implicit device-wide synchronisation, or code running while a stream is
// being captured, where cudaMalloc is not permitted. For them the persistent
// substep kernel is launched with its scratch words (the grid-barrier arrival
// counter and the device error word) taken from this fixed array instead of
// buffers of the handle, and without the autotuner or CUDA-graph builder,
// which may allocate.
//
// The array lives in every device that loads the library until the process
// exits. All calls share it and it keeps the last call's contents, so each
// call zeroes the words it uses first; calls whose kernels overlap on one GPU
// would race on it and must not be issued.
namespace {
constexpr uint32_t kNoAllocScratchWords = 64;  // 256 bytes; words 0 and 1 are used
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

int launch_substeps_noalloc(const DevCtx& ctx, int block, uint32_t warp_smem, bool lambdas, uint32_t nsub, float dt,
                            void* stream, int device, int* device_error) {
	if (device < 0 || device >= kNoAllocMaxDevices) return (int)cudaErrorInvalidDevice;
	uint32_t* p = nullptr;
	{
		// Set-up, once per device, with that device current: the array's name
		// in host code is a host-side stand-in, so its device address is
		// looked up and passed to the kernel.
		std::lock_guard<std::mutex> lk(g_noalloc_mu);
		if (!g_noalloc_ptr[device]) {
			const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
			if (e != cudaSuccess) return (int)e;
			g_noalloc_ptr[device] = p;
		}
		p = g_noalloc_ptr[device];
	}
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = lambdas ? (const void*)k_persistent<true> : (const void*)k_persistent<false>;
	const size_t smem = solve_smem_bytes(block, warp_smem);
	int sms = 0, per_sm = 0;
	cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, block, smem);
	if (e != cudaSuccess) return (int)e;
	if (per_sm <= 0) return (int)cudaErrorInvalidConfiguration;
	const uint32_t blocks = (uint32_t)(per_sm * sms);
	// the 32-bit arrival counter must not wrap within one call
	if ((uint64_t)nsub * ctx.ncolours * blocks >= (1ull << 31)) return (int)cudaErrorInvalidValue;
	e = cudaMemsetAsync(p, 0, 2 * sizeof(uint32_t), st);
	if (e != cudaSuccess) return (int)e;
	DevCtx c = ctx;
	c.bar_count = p;
	c.err = reinterpret_cast<int*>(p + 1);
	void* args[] = {&c, &nsub, &dt};
	e = cudaLaunchCooperativeKernel(f, dim3(blocks), dim3(block), args, smem, st);
	if (e != cudaSuccess) return (int)e;
	e = cudaMemcpyAsync(device_error, p + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	return (int)e;
}

}  // namespace xfem
