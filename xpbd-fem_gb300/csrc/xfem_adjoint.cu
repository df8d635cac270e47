// Reverse-mode adjoint of the substep (sm_103a). No reference counterpart:
// the reference (jak-xyz/xpbd-fem) only steps forward. The derivative is that
// of the forward kernels' own method: predict and the velocity update
// (XPBDFEM/Geo.cpp:307-312, 342-344), the coloured Gauss-Seidel sweep of the
// coupled Neo-Hookean solve (XPBDFEM/Fem.cpp:523-553 with
// EnergyXpbdConstrainSimultaneous<2>, XPBDFEM/Xpbd.h:123-215), locks
// (XPBDFEM/Geo.cpp:318-322) and the ground projection with Coulomb friction.
//
// Tape (written by the recording forward, xfem_kernels.cu):
//   tape_v[s][v]          one 32-byte sector per vertex and substep, written
//                         by its owner: O after the advance (the substep's
//                         start position and the w its solves use) and D
//                         before it (the previous substep's swept D)
//   tape_t[s][row][lane]  each solve's input displacement (12 floats)
//   tape_fin[v]           D before the closing finalize
// Reverse order: the closing finalize, then substeps last to first, colours
// last to first; clusters of a colour share no vertex, so each updates the
// adjoint of its vertices in place (no atomics), exactly mirroring the
// forward. A cluster (one thread) walks its tets backwards from their taped
// inputs, with its vertices' adjoints in registers; the vertex owner then
// reverses the advance, as the forward did it right before its solves.
//
// Per-vertex adjoint state (AdjCtx::abar, two float4 per vertex):
//   during the run     Xb = dL/d(position O + D), Ob = dL/dO from the finish
//                      of the substep and the later ones (also across
//                      checkpoint segments, so that segmenting changes no bit)
//   end / start        dL/dX and dL/dV of the canonical state
// Per tet row: cbar += alpha0 * dL/dalpha0 + alpha1 * dL/dalpha1, which is
// -mu dL/dmu since both compliances scale as 1/mu (the host divides by -mu).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "xfem_device.cuh"
#include "xfem_internal.h"

namespace xfem {

namespace {

__device__ __forceinline__ Vec3 vadd(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ Vec3 vsub(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ Vec3 vmul(Vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
// a + b * s
__device__ __forceinline__ Vec3 vfma(Vec3 b, float s, Vec3 a) { return {fmaf(b.x, s, a.x), fmaf(b.y, s, a.y), fmaf(b.z, s, a.z)}; }

// What one coupled solve computes, recomputed for its reverse pass from the
// tet's pre-solve state. g1_i = 2 (J - a) detQ cof_i with cof the cofactor
// rows of Ds (P1 x P2, P2 x P0, P0 x P1), so dJ/dP_i = detQ cof_i.
struct TetFw {
	Vec3 P[3], g0[4], g1[4], cof[3];
	float U0, U1, Ja, detQ, A1, l0, l1, alpha0, alpha1;
	float i00, i11, r0, r1, inv_det;  // the Cramer factors of M = [A0 A1; A1 A2]
};

__device__ __forceinline__ void tet_internals(const Mat& bp, const TetRec& r, float inv_dt2, const float4 O[4],
                                              const Vec3 D[4], TetFw& f) {
	const float q[3][3] = {{r.a.x, r.a.y, r.a.z}, {r.a.w, r.b.x, r.b.y}, {r.b.z, r.b.w, r.c.x}};
	const float QQ[3] = {r.c.y, r.c.z, r.c.w};
	const float QR[3] = {r.d.x, r.d.y, r.d.z};
	f.alpha0 = r.d.w * inv_dt2;
	f.alpha1 = f.alpha0 * bp.ratio;
#pragma unroll
	for (int i = 0; i < 3; i++)
		f.P[i] = {(O[i].x - O[3].x) + (D[i].x - D[3].x), (O[i].y - O[3].y) + (D[i].y - D[3].y),
		          (O[i].z - O[3].z) + (D[i].z - D[3].z)};
	f.U0 = deviatoric(bp, QQ, QR, f.P, f.g0);
	f.U1 = hydrostatic(q, f.P, bp.a, f.g1, &f.Ja, &f.detQ);
	f.cof[0] = cross(f.P[1], f.P[2]);
	f.cof[1] = cross(f.P[2], f.P[0]);
	f.cof[2] = cross(f.P[0], f.P[1]);
	const float w[4] = {O[0].w, O[1].w, O[2].w, O[3].w};
	const float A0 = fmaf(2.0f * f.U0, f.alpha0, wdot(w, f.g0, f.g0));
	f.A1 = wdot(w, f.g1, f.g0);
	const float A2 = fmaf(2.0f * f.U1, f.alpha1, wdot(w, f.g1, f.g1));
	f.i00 = rcp(A0);
	f.i11 = rcp(A2);
	f.r0 = f.A1 * f.i00;
	f.r1 = f.A1 * f.i11;
	f.inv_det = rcp(fmaxf(0.00000001f, fmaf(-f.r0, f.r1, 1.0f)));
	const float c0 = (-2.0f * f.U0) * f.i00, c1 = (-2.0f * f.U1) * f.i11;
	f.l0 = f.inv_det * fmaf(-f.r0, c1, c0);
	f.l1 = f.inv_det * fmaf(-c0, f.r1, c1);
}

// Reverse of one coupled solve. xb[4]: adjoint of the tet's four positions
// after the solve on entry, before it on exit. Returns
// alpha0 dL/dalpha0 + alpha1 dL/dalpha1 of this solve.
__device__ __forceinline__ float tet_reverse(const TetRec& r, const TetFw& f, const float w[4], Vec3 xb[4]) {
	const float QQ[3] = {r.c.y, r.c.z, r.c.w};
	const float QR[3] = {r.d.x, r.d.y, r.d.z};
	Vec3 gb0[4], gb1[4];
	float lb0 = 0.0f, lb1 = 0.0f;
#pragma unroll
	for (int n = 0; n < 4; n++) {
		const Vec3 y = vmul(xb[n], w[n]);
		lb0 += dot(y, f.g0[n]);
		lb1 += dot(y, f.g1[n]);
		gb0[n] = vmul(y, f.l0);
		gb1[n] = vmul(y, f.l1);
	}
	// lambda = M^-1 b with M = [A0 A1; A1 A2] symmetric: m = M^-1 lambda_bar,
	// b_bar = m, M_bar = -m lambda^T (same Cramer form as the forward)
	const float c0 = lb0 * f.i00, c1 = lb1 * f.i11;
	const float m0 = f.inv_det * fmaf(-f.r0, c1, c0);
	const float m1 = f.inv_det * fmaf(-c0, f.r1, c1);
	const float Ab0 = -m0 * f.l0, Ab2 = -m1 * f.l1, Ab1 = -fmaf(m0, f.l1, m1 * f.l0);
	// b = (-2 U0, -2 U1); A0 = sum w |g0|^2 + 2 U0 alpha0; A1 = sum w g1.g0; A2 = sum w |g1|^2 + 2 U1 alpha1
	const float Ub0 = fmaf(2.0f * f.alpha0, Ab0, -2.0f * m0);
	const float Ub1 = fmaf(2.0f * f.alpha1, Ab2, -2.0f * m1);
	const float dalpha = fmaf(f.alpha0, 2.0f * f.U0 * Ab0, f.alpha1 * (2.0f * f.U1 * Ab2));
#pragma unroll
	for (int n = 0; n < 4; n++) {
		gb0[n] = vfma(f.g0[n], 2.0f * w[n] * Ab0, vfma(f.g1[n], w[n] * Ab1, gb0[n]));
		gb1[n] = vfma(f.g1[n], 2.0f * w[n] * Ab2, vfma(f.g0[n], w[n] * Ab1, gb1[n]));
	}
	// g_3 = -(g_0 + g_1 + g_2)
#pragma unroll
	for (int i = 0; i < 3; i++) {
		gb0[i] = vsub(gb0[i], gb0[3]);
		gb1[i] = vsub(gb1[i], gb1[3]);
	}
	// deviatoric: U0 = sum QQ_i |P_i|^2 + QR . (P0.P1, P0.P2, P1.P2), g0_i = dU0/dP_i
	Vec3 Pb[3];
	Pb[0] = vfma(gb0[0], 2.0f * QQ[0], vfma(gb0[1], QR[0], vfma(gb0[2], QR[1], vmul(f.g0[0], Ub0))));
	Pb[1] = vfma(gb0[0], QR[0], vfma(gb0[1], 2.0f * QQ[1], vfma(gb0[2], QR[2], vmul(f.g0[1], Ub0))));
	Pb[2] = vfma(gb0[0], QR[1], vfma(gb0[1], QR[2], vfma(gb0[2], 2.0f * QQ[2], vmul(f.g0[2], Ub0))));
	// hydrostatic: U1 = (J - a)^2, g1_i = 2 (J - a) h_i, h_i = detQ cof_i = dJ/dP_i
	float Jb = 2.0f * f.Ja * Ub1;
	const float s2 = 2.0f * f.Ja * f.detQ;
	Vec3 cb[3];
#pragma unroll
	for (int i = 0; i < 3; i++) {
		Jb = fmaf(2.0f * f.detQ, dot(f.cof[i], gb1[i]), Jb);
		cb[i] = vmul(gb1[i], s2);
	}
#pragma unroll
	for (int i = 0; i < 3; i++) Pb[i] = vfma(f.cof[i], Jb * f.detQ, Pb[i]);
	// c = a x b: a_bar += b x c_bar, b_bar += c_bar x a
	Pb[1] = vadd(Pb[1], cross(f.P[2], cb[0]));
	Pb[2] = vadd(Pb[2], cross(cb[0], f.P[1]));
	Pb[2] = vadd(Pb[2], cross(f.P[0], cb[1]));
	Pb[0] = vadd(Pb[0], cross(cb[1], f.P[2]));
	Pb[0] = vadd(Pb[0], cross(f.P[1], cb[2]));
	Pb[1] = vadd(Pb[1], cross(cb[2], f.P[0]));
	// P_i = x_i - x_3; the identity part of x_out = x_in + w (l0 g0 + l1 g1) stays in xb
#pragma unroll
	for (int i = 0; i < 3; i++) {
		xb[i] = vadd(xb[i], Pb[i]);
		xb[3] = vsub(xb[3], Pb[i]);
	}
	return dalpha;
}

// Reverse of the finish of a substep for one vertex (finish_vertex: locks,
// then the ground projection with friction) in displacement form. Op: O of
// the substep (w before the lock), Ds: D after the sweep (flag bits in .w),
// db: dL/dD' of the finished displacement. Returns dL/dDs; adds the O part
// to ob.
__device__ __forceinline__ Vec3 finish_reverse(const BodyParams& bp, const float4& Op, const float4& Ds, Vec3 db, Vec3& ob) {
	const uint32_t bits = __float_as_uint(Ds.w);
	if (bp.lock_active && (bits & kFlagLocked)) return {0.0f, 0.0f, 0.0f};
	if (!(bp.ground && Op.w > 0.0f)) return db;
	// the forward's ground_contact, recomputed
	const Vec3 n = {bp.ground_n[0], bp.ground_n[1], bp.ground_n[2]};
	const float h = (n.x * Op.x + n.y * Op.y + n.z * Op.z) - bp.ground_d;
	const float depth = -(h + (n.x * Ds.x + n.y * Ds.y + n.z * Ds.z));
	if (!(depth > 0.0f)) return db;
	const Vec3 D1 = {Ds.x + depth * n.x, Ds.y + depth * n.y, Ds.z + depth * n.z};
	const float dn = n.x * D1.x + n.y * D1.y + n.z * D1.z;
	const Vec3 t = {D1.x - dn * n.x, D1.y - dn * n.y, D1.z - dn * n.z};
	const float lt = sqrtf(t.x * t.x + t.y * t.y + t.z * t.z);
	const float lim = bp.friction * depth;
	const bool kinetic = !(lt <= lim);
	const float sc = kinetic ? lim / lt : 1.0f;
	// D' = D1 - sc t, t = D1 - n (n . D1), D1 = Ds + depth n, depth = -(n . Op - d + n . Ds)
	Vec3 tb = vmul(db, -sc);
	float depthb = 0.0f;
	if (kinetic) {  // sc = friction depth / |t|
		const float sb = -dot(t, db);
		const float inv_lt = 1.0f / lt;
		depthb = sb * bp.friction * inv_lt;
		tb = vfma(t, -sb * sc * inv_lt * inv_lt, tb);
	}
	Vec3 D1b = vadd(db, vfma(n, -dot(n, tb), tb));
	depthb += dot(n, D1b);
	ob = vfma(n, -depthb, ob);
	return vfma(n, -depthb, D1b);
}

__device__ __forceinline__ Vec3 tip_grad(const DevCtx& C, const AdjCtx& A, uint32_t v, uint32_t run_sub) {
	const int q = __ldg(C.tip_of + v);
	if (q < 0) return {0.0f, 0.0f, 0.0f};
	return v3(__ldg(A.G + (size_t)run_sub * C.ntips + q));
}

// Tape record of vertex v at launch substep s: O after the advance, D before.
__device__ __forceinline__ const float4* tape_at(const DevCtx& C, uint32_t s, uint32_t v) {
	return C.tape_v + 2 * ((size_t)s * C.nverts + v);
}

// Reverse of the boundary between two substeps for one vertex: the finish
// of the earlier one (its start O = Op, its swept D = Ds) and the predict of
// the later one. xb: dL/d(predicted position of the later substep) with its
// solves already reversed; run_sub: the run substep whose end position is the
// later substep's O (the loss term). Leaves the earlier substep's state.
__device__ __forceinline__ void boundary_reverse(const DevCtx& C, const AdjCtx& A, uint32_t v, const float4& Op,
                                                 const float4& Ds, Vec3 xb, uint32_t run_sub) {
	const BodyParams& bp = C.bodies[__float_as_uint(Ds.w) >> 8];
	// O of the later substep is read by its solves (through O + D), by the
	// substeps after it and by the loss
	const Vec3 os = vadd(vadd(v3(__ldcg(A.abar + 2 * (size_t)v + 1)), xb), tip_grad(C, A, v, run_sub));
	// O = Op + D', D_pred = (D' / dt + g dt) drag dt
	const Vec3 dfin = vfma(xb, bp.drag_mul, os);
	Vec3 ob = os;
	const Vec3 dsb = finish_reverse(bp, Op, Ds, dfin, ob);
	// the earlier substep's swept position is Op + Ds
	ob = vsub(ob, dsb);
	__stcg(A.abar + 2 * (size_t)v, make_float4(dsb.x, dsb.y, dsb.z, 0.0f));
	__stcg(A.abar + 2 * (size_t)v + 1, make_float4(ob.x, ob.y, ob.z, 0.0f));
}

// Reverse of advance_vertex at launch substep s for one owned vertex (xb as
// for boundary_reverse). The first substep of the run ends in the canonical
// dL/dX, dL/dV. The first substep of a later segment keeps the in-segment
// state: the previous segment's finalize reverse continues from it with the
// same arithmetic as a boundary inside a launch, so checkpointed runs give
// the full tape's results bit for bit.
__device__ __forceinline__ void advance_reverse(const DevCtx& C, const AdjCtx& A, uint32_t v, uint32_t s, bool first,
                                                float dt, Vec3 xb) {
	if (first) {
		if (C.sub_base > 0) {
			__stcg(A.abar + 2 * (size_t)v, make_float4(xb.x, xb.y, xb.z, 0.0f));
			return;
		}
		// O = X, D = ((V + g dt) drag) dt
		const float4 Dl = __ldcs(tape_at(C, s, v) + 1);
		const BodyParams& bp = C.bodies[__float_as_uint(Dl.w) >> 8];
		const Vec3 os = vadd(v3(__ldcg(A.abar + 2 * (size_t)v + 1)), xb);
		const Vec3 vb = vmul(xb, bp.drag_mul * dt);
		__stcg(A.abar + 2 * (size_t)v, make_float4(os.x, os.y, os.z, 0.0f));
		__stcg(A.abar + 2 * (size_t)v + 1, make_float4(vb.x, vb.y, vb.z, 0.0f));
		return;
	}
	boundary_reverse(C, A, v, __ldcg(tape_at(C, s - 1, v)), __ldcs(tape_at(C, s, v) + 1), xb, C.sub_base + s - 1);
}

// Reverse of finalize_vertex, the launch's closing finish. For the run's last
// segment abar holds the canonical dL/dX, dL/dV at the end (plus the loss on
// the final position); for an earlier segment it holds the next segment's
// in-segment state, and the closing finish is reversed as a substep boundary.
__device__ __forceinline__ void finalize_reverse(const DevCtx& C, const AdjCtx& A, uint32_t v, uint32_t nsub,
                                                 float inv_dt, bool last) {
	const float4 Ds = __ldcg(C.tape_fin + v);
	const float4 Op = __ldcg(tape_at(C, nsub - 1, v));
	const uint32_t run_sub = C.sub_base + nsub - 1;
	if (!last) {
		boundary_reverse(C, A, v, Op, Ds, v3(__ldcg(A.abar + 2 * (size_t)v)), run_sub);
		return;
	}
	const BodyParams& bp = C.bodies[__float_as_uint(Ds.w) >> 8];
	const Vec3 xcb = v3(__ldcg(A.abar + 2 * (size_t)v));
	const Vec3 vcb = v3(__ldcg(A.abar + 2 * (size_t)v + 1));
	const Vec3 on = vadd(xcb, tip_grad(C, A, v, run_sub));
	// X = O + D', V = D' / dt
	const Vec3 dfin = vfma(vcb, inv_dt, on);
	Vec3 ob = on;
	const Vec3 dsb = finish_reverse(bp, Op, Ds, dfin, ob);
	ob = vsub(ob, dsb);
	__stcg(A.abar + 2 * (size_t)v, make_float4(dsb.x, dsb.y, dsb.z, 0.0f));
	__stcg(A.abar + 2 * (size_t)v + 1, make_float4(ob.x, ob.y, ob.z, 0.0f));
}

// Isolated vertices: no solve touches them; one thread reverses all the
// segment's substeps of one vertex.
__device__ __forceinline__ void isolated_reverse(const DevCtx& C, const AdjCtx& A, uint32_t begin, uint32_t step,
                                                 uint32_t nsub, float dt) {
	for (uint32_t i = begin; i < C.nisolated; i += step) {
		const uint32_t v = __ldg(C.isolated + i);
		for (int s = (int)nsub - 1; s >= 0; s--)
			advance_reverse(C, A, v, (uint32_t)s, s == 0, dt, v3(__ldcg(A.abar + 2 * (size_t)v)));
	}
}

// The tape's input displacement of one solve (12 floats in three float4).
__device__ __forceinline__ void load_tet_input(const DevCtx& C, uint32_t s, uint32_t row, uint32_t lane, Vec3 D[4]) {
	const float4* p = C.tape_t + ((size_t)s * C.ntrows + row) * 3 * kLanes + lane;
	const float4 a = __ldcs(p), b = __ldcs(p + kLanes), c = __ldcs(p + 2 * kLanes);
	D[0] = {a.x, a.y, a.z};
	D[1] = {a.w, b.x, b.y};
	D[2] = {b.z, b.w, c.x};
	D[3] = {c.y, c.z, c.w};
}

// One cluster (lane) of chunk block `blk`, launch substep s: reverse its
// solves last to first from their taped inputs, then the owned vertices'
// advance. CUBE: the canonical 6-tet cube with compile-time slots, all in
// registers. Records, header and vertex ids are read straight from the chunk
// block: lane-minor, so every warp load is one contiguous run.
template <bool CUBE>
__device__ __forceinline__ void cluster_reverse(const DevCtx& C, const AdjCtx& A, const float4* blk, uint32_t ntmax,
                                                uint32_t nvmax, uint32_t trow, uint32_t lane, uint32_t s, bool first,
                                                float dt, float inv_dt2) {
	constexpr uint32_t NV = CUBE ? 8u : kMaxClusterVerts;
	constexpr uint32_t NT = CUBE ? 6u : kMaxClusterTets;
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(blk + 4 * kLanes * ntmax);
	const uint32_t* vids = hdrs + kLanes;
	const uint32_t* slots = vids + kLanes * nvmax;
	const uint32_t hdr = __ldg(hdrs + lane);
	if ((hdr & 15u) == 0u) return;
	const uint32_t nv = CUBE ? 8u : (hdr & 15u), nt = CUBE ? 6u : ((hdr >> 4) & 15u), mask = (hdr >> 8) & 0xffu;
	const Mat mat = load_mat(C.bodies, hdr >> 16);
	uint32_t vid[NV];
	float4 O[NV];
	Vec3 xb[NV];
#pragma unroll
	for (uint32_t k = 0; k < NV; k++) {
		if (k < nv) {
			vid[k] = __ldg(vids + k * kLanes + lane);
			O[k] = __ldcg(tape_at(C, s, vid[k]));
			xb[k] = v3(__ldcg(A.abar + 2 * (size_t)vid[k]));
		}
	}
#pragma unroll
	for (int t = (int)NT - 1; t >= 0; t--) {
		if ((uint32_t)t < nt) {
			const uint32_t sl =
			    CUBE ? (uint32_t)(cube_slot(t, 0) | cube_slot(t, 1) << 4 | cube_slot(t, 2) << 8 | cube_slot(t, 3) << 12)
			         : __ldg(slots + t * kLanes + lane);
			const float4* r = blk + t * 4 * kLanes + lane;
			const TetRec tr = {__ldg(r), __ldg(r + kLanes), __ldg(r + 2 * kLanes), __ldg(r + 3 * kLanes)};
			Vec3 Din[4];
			load_tet_input(C, s, trow + t, lane, Din);
			float4 Ot[4];
			Vec3 xt[4];
			float w[4];
#pragma unroll
			for (int k = 0; k < 4; k++) {
				const uint32_t q = (sl >> (4 * k)) & 15u;
				Ot[k] = O[q];
				w[k] = O[q].w;
				xt[k] = xb[q];
			}
			TetFw f;
			tet_internals(mat, tr, inv_dt2, Ot, Din, f);
			const float dal = tet_reverse(tr, f, w, xt);
#pragma unroll
			for (int k = 0; k < 4; k++) xb[(sl >> (4 * k)) & 15u] = xt[k];
			float* cb = A.cbar + (size_t)(trow + t) * kLanes + lane;
			*cb += dal;
		}
	}
#pragma unroll
	for (uint32_t k = 0; k < NV; k++) {
		if (k < nv) {
			if (mask & (1u << k))
				advance_reverse(C, A, vid[k], s, first, dt, xb[k]);
			else
				__stcg(A.abar + 2 * (size_t)vid[k], make_float4(xb[k].x, xb[k].y, xb[k].z, 0.0f));
		}
	}
}

// The cube reverse with a group of 8 lanes per cluster (meshes whose colour
// passes leave most warps idle). The six solves' forward internals do not
// depend on the reverse chain, only on the tape: lanes 0-5 of the group
// recompute tet j's into shared memory side by side, then lane 0 runs the
// chain of six reverses as cluster_reverse<true> does, in the same order
// with the same arithmetic (the same results bit for bit), with one solve's
// recompute instead of six ahead of it. sh: this group's six slots; cl: the
// cluster's lane in its chunk; j: the lane's index in the group.
// One solve's slot: its forward internals and the record words its reverse
// reads (QQ in c.yzw, QR in d.xyz).
struct TetSlot {
	TetFw f;
	float4 c, d;
};

__device__ __forceinline__ void cluster_reverse_grouped(const DevCtx& C, const AdjCtx& A, const float4* blk,
                                                        uint32_t trow, uint32_t cl, uint32_t j, TetSlot* sh, uint32_t s,
                                                        bool first, float dt, float inv_dt2) {
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(blk + 4 * kLanes * 6);
	const uint32_t* vids = hdrs + kLanes;
	const uint32_t hdr = __ldg(hdrs + cl);
	const bool live = (hdr & 15u) != 0;
	if (live && j < 6u) {
		const Mat mat = load_mat(C.bodies, hdr >> 16);
		const float4* r = blk + j * 4 * kLanes + cl;
		const TetRec tr = {__ldg(r), __ldg(r + kLanes), __ldg(r + 2 * kLanes), __ldg(r + 3 * kLanes)};
		const uint32_t sl = (uint32_t)(cube_slot((int)j, 0) | cube_slot((int)j, 1) << 4 | cube_slot((int)j, 2) << 8 |
		                               cube_slot((int)j, 3) << 12);
		float4 Ot[4];
#pragma unroll
		for (int k = 0; k < 4; k++) Ot[k] = __ldcg(tape_at(C, s, __ldg(vids + ((sl >> (4 * k)) & 15u) * kLanes + cl)));
		Vec3 Din[4];
		load_tet_input(C, s, trow + j, cl, Din);
		tet_internals(mat, tr, inv_dt2, Ot, Din, sh[j].f);
		sh[j].c = tr.c;
		sh[j].d = tr.d;
	}
	__syncwarp();
	Vec3* xs = reinterpret_cast<Vec3*>(sh);  // after the chain: the 8 vertices' adjoints
	if (live && j == 0u) {
		float4 O[8];
		Vec3 xb[8];
#pragma unroll
		for (int k = 0; k < 8; k++) {
			const uint32_t v = __ldg(vids + k * kLanes + cl);
			O[k] = __ldcg(tape_at(C, s, v));
			xb[k] = v3(__ldcg(A.abar + 2 * (size_t)v));
		}
#pragma unroll
		for (int t = 5; t >= 0; t--) {
			const TetRec tr = {make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f), sh[t].c, sh[t].d};
			float w[4];
			Vec3 xt[4];
#pragma unroll
			for (int k = 0; k < 4; k++) {
				w[k] = O[cube_slot(t, k)].w;
				xt[k] = xb[cube_slot(t, k)];
			}
			const TetFw f = sh[t].f;
			const float dal = tet_reverse(tr, f, w, xt);
#pragma unroll
			for (int k = 0; k < 4; k++) xb[cube_slot(t, k)] = xt[k];
			float* cb = A.cbar + (size_t)(trow + t) * kLanes + cl;
			*cb += dal;
		}
		// the slots' reads above come first in this lane's program order
#pragma unroll
		for (int k = 0; k < 8; k++) xs[k] = xb[k];
	}
	__syncwarp();
	// lane j finishes vertex j of the cluster: its advance reverse if the
	// cluster owns it, else its adjoint
	if (live) {
		const uint32_t v = __ldg(vids + j * kLanes + cl);
		const Vec3 x = xs[j];
		if ((hdr >> (8 + j)) & 1u)
			advance_reverse(C, A, v, s, first, dt, x);
		else
			__stcg(A.abar + 2 * (size_t)v, make_float4(x.x, x.y, x.z, 0.0f));
	}
	__syncwarp();  // the group's slots are free for the next cluster
}

// Reverse of one recorded launch of nsub substeps (one checkpoint segment).
// Cooperative persistent grid, one warp per chunk of a colour pass; every
// colour pass ends at the bounded grid barrier, as in the forward. grouped:
// every colour pass's chunks, split in 8 parts of 4 clusters, fit the grid's
// warps at once: a warp takes one part, a group of 8 lanes per cluster
// (cluster_reverse_grouped; other chunks one lane per cluster).
__global__ void __launch_bounds__(256) k_reverse(DevCtx C, AdjCtx A, uint32_t nsub, float dt, int last, int grouped) {
	extern __shared__ __align__(16) unsigned char rsmem[];
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = wpb * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	uint32_t target = C.bar_base;
	for (uint32_t v = gtid; v < C.nverts; v += nthreads) finalize_reverse(C, A, v, nsub, inv_dt, last != 0);
	bool ok = grid_sync(C, target);
	if (ok) isolated_reverse(C, A, gtid, nthreads, nsub, dt);
	TetSlot* gsh = reinterpret_cast<TetSlot*>(rsmem) + (size_t)wib * 24 + (lane >> 3) * 6;
	for (int s = (int)nsub - 1; s >= 0 && ok; s--) {
		for (int c = (int)C.ncolours - 1; c >= 0 && ok; c--) {
			const uint32_t cb = __ldg(C.colour_chunk_begin + c), ce = __ldg(C.colour_chunk_begin + c + 1);
			if (grouped) {
				for (uint32_t it = gwarp; it < 8u * (ce - cb); it += nwarps) {
					const uint32_t ch = cb + it / 8u, cl = (it % 8u) * 4u + (lane >> 3);
					const uint4 m = __ldg(reinterpret_cast<const uint4*>(C.chunks) + ch);
					const float4* blk = C.cblk + m.x;
					if (m.z & kShapeCube) {
						cluster_reverse_grouped(C, A, blk, m.w, cl, lane & 7u, gsh, (uint32_t)s, s == 0, dt, inv_dt2);
					} else if ((lane & 7u) == 0u) {
						cluster_reverse<false>(C, A, blk, m.z & 0xffu, (m.z >> 8) & 0xffu, m.w, cl, (uint32_t)s, s == 0,
						                       dt, inv_dt2);
					}
				}
				if (!grid_sync(C, target)) ok = false;
				continue;
			}
			for (uint32_t ch = cb + gwarp; ch < ce; ch += nwarps) {
				const uint4 m = __ldg(reinterpret_cast<const uint4*>(C.chunks) + ch);
				const float4* blk = C.cblk + m.x;
				const uint32_t ntmax = m.z & 0xffu, nvmax = (m.z >> 8) & 0xffu;
				if (m.z & kShapeCube)
					cluster_reverse<true>(C, A, blk, ntmax, nvmax, m.w, lane, (uint32_t)s, s == 0, dt, inv_dt2);
				else
					cluster_reverse<false>(C, A, blk, ntmax, nvmax, m.w, lane, (uint32_t)s, s == 0, dt, inv_dt2);
			}
			if (!grid_sync(C, target)) ok = false;
		}
	}
}

}  // namespace

int configure_adjoint_kernels(int, uint32_t) { return 0; }

int launch_reverse(const DevCtx& ctx, const AdjCtx& adj, int block, uint32_t, uint32_t max_colour_chunks, uint32_t nsub,
                   float dt, bool last, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	int dev = 0, sms = 0, per_sm = 0;
	// six forward-internal slots per 8-lane group, 4 groups per warp
	const size_t smem = (size_t)(block / 32) * 24 * sizeof(TetSlot);
	cudaError_t e = cudaFuncSetAttribute((const void*)k_reverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess) e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_reverse, block, smem);
	if (e != cudaSuccess) return (int)e;
	if (per_sm <= 0) return (int)cudaErrorInvalidConfiguration;
	// the whole co-resident grid, as the forward: chunk i of a colour goes to
	// block i % grid, so a colour pass with fewer chunks than warps still
	// spreads one chunk per SM (a pass lasts as long as its slowest chunk)
	const uint32_t blocks = (uint32_t)(per_sm * sms);
	e = reset_barrier(ctx, st);
	if (e != cudaSuccess) return (int)e;
	DevCtx c = ctx;
	AdjCtx a = adj;
	int lastv = last ? 1 : 0;
	// the grouped form when one round of the grid's warps takes every part of
	// the largest colour pass
	int grouped = (uint64_t)max_colour_chunks * 8u <= (uint64_t)blocks * (uint32_t)(block / 32) ? 1 : 0;
	if (const char* f = getenv("XFEM_REVERSE_FORM")) grouped = f[0] == 'g' ? 1 : f[0] == 'l' ? 0 : grouped;
	void* args[] = {&c, &a, &nsub, &dt, &lastv, &grouped};
	return (int)cudaLaunchCooperativeKernel((const void*)k_reverse, dim3(blocks), dim3(block), args, smem, st);
}

}  // namespace xfem
