// Quadratic-tet element code of libxfem.so (sm_103a), shared by the T10
// mode (xfem_t10.cu) and meshes mixing T10s and H27s (xfem_qmixed.cu): GeoQuadratic3d on a tet mesh
// (XPBDFEM/Geo.cpp:836-1053). Every tet gets a node on each edge
// (Connectivity3d's edge numbering); SolveElement on ElementParamsQuadraticTet
// (XPBDFEM/Fem.cpp:871-893: SolveElementPixar :361-433 and SolveElementMixed
// :437-564 with Nodes = 10 and the 4-point rule, PointsLo = PointsHi = 4; the
// cube models leave a tet alone), SolveVolumeOnly (:840-867), DampElement
// (:910-928) and PbdDamp (XPBDFEM/Xpbd.h:306-346), in the element kernel of
// xfem_elements.cuh with one thread per T10.
//
// Records: 15 float4 per T10 as a structure of arrays (float4 k of element i
// at el_rec[k * nel + i]): Qi column-major, volume, surface area, the
// prefactored QQ[9] and QR[36]. The map from the corners is linear, so one
// Qi serves all four points; their shape-function gradients come from a
// 120-float table (el_tab) that every thread reads at the same addresses.
#pragma once

#include "xfem_elements.cuh"

namespace xfem {

namespace {

namespace t10e {

constexpr int kQQi = 0, kQVol = 9, kQArea = 10, kQQQ = 11, kQQR = 20;

struct QRec {
	const float4* base;
	uint32_t n, i;
	__device__ __forceinline__ float operator()(int j) const {
		return __ldg(reinterpret_cast<const float*>(base + (size_t)(j >> 2) * n + i) + (j & 3));
	}
};

__device__ __forceinline__ float g4(const DevCtx& C, int p, int n, int k) { return __ldg(C.el_tab + (p * 10 + n) * 3 + k); }

// F = Qi MatMul(dN[0..8], P) at point p (XPBDFEM/Fem.cpp:311-316)
__device__ __forceinline__ void q_def_grad(const DevCtx& C, const float Qi[3][3], int p, const Vec3 P[9], float F[3][3]) {
	float Dm[3][3];
#pragma unroll
	for (int r = 0; r < 3; r++) {
		float x = 0.0f, y = 0.0f, z = 0.0f;
#pragma unroll
		for (int n = 0; n < 9; n++) {
			const float d = g4(C, p, n, r);
			x = fmaf(d, P[n].x, x);
			y = fmaf(d, P[n].y, y);
			z = fmaf(d, P[n].z, z);
		}
		Dm[0][r] = x;
		Dm[1][r] = y;
		Dm[2][r] = z;
	}
#pragma unroll
	for (int c = 0; c < 3; c++)
#pragma unroll
		for (int r = 0; r < 3; r++) F[c][r] = fmaf(Qi[0][r], Dm[c][0], fmaf(Qi[1][r], Dm[c][1], Qi[2][r] * Dm[c][2]));
}

// ApplyEnergyGradient with the constant Qi: g[n] += (G Qi) dN[n], n < 9
__device__ __forceinline__ void q_apply(const DevCtx& C, const float G[3][3], const float Qi[3][3], int p, Vec3 g[10]) {
	float M[3][3];
#pragma unroll
	for (int j = 0; j < 3; j++)
#pragma unroll
		for (int r = 0; r < 3; r++) M[j][r] = fmaf(G[0][r], Qi[j][0], fmaf(G[1][r], Qi[j][1], G[2][r] * Qi[j][2]));
#pragma unroll
	for (int n = 0; n < 9; n++) {
		const float d0 = g4(C, p, n, 0), d1 = g4(C, p, n, 1), d2 = g4(C, p, n, 2);
		g[n].x += fmaf(M[0][0], d0, fmaf(M[1][0], d1, M[2][0] * d2));
		g[n].y += fmaf(M[0][1], d0, fmaf(M[1][1], d1, M[2][1] * d2));
		g[n].z += fmaf(M[0][2], d0, fmaf(M[1][2], d1, M[2][2] * d2));
	}
}

__device__ __forceinline__ float trace_xtx(const float F[3][3]) {
	return fmaf(F[0][0], F[0][0], fmaf(F[0][1], F[0][1], F[0][2] * F[0][2])) +
	       fmaf(F[1][0], F[1][0], fmaf(F[1][1], F[1][1], F[1][2] * F[1][2])) +
	       fmaf(F[2][0], F[2][0], fmaf(F[2][1], F[2][1], F[2][2] * F[2][2]));
}

// (J - a)^2 over the 4 points (weight 1/4 each) into U, g
__device__ __forceinline__ void q_hydro(const DevCtx& C, const float Qi[3][3], const Vec3 P[9], float a, float& U,
                                        Vec3 g[10]) {
#pragma unroll 1
	for (int p = 0; p < 4; p++) {
		float F[3][3], A[3][3], G[3][3];
		q_def_grad(C, Qi, p, P, F);
		const float Ja = adj_det(F, A) - a;
		U = fmaf(0.25f * Ja, Ja, U);
		const float s = 0.5f * Ja;
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) G[c][r] = A[c][r] * s;
		q_apply(C, G, Qi, p, g);
	}
}

// I1 prefactored over the nine edge vectors (XPBDFEM/Fem.cpp:163-192),
// root gradient included
__device__ __forceinline__ float q_pref_i1(const QRec& R, const Vec3 P[9], Vec3 g[10]) {
	float U = 0.0f;
#pragma unroll
	for (int i = 0; i < 9; i++) {
		const float qq = R(kQQQ + i);
		U = fmaf(qq, dot(P[i], P[i]), U);
		const float d = 2.0f * qq;
		g[i] = {d * P[i].x, d * P[i].y, d * P[i].z};
	}
	int k = 0;
#pragma unroll
	for (int i = 0; i < 9; i++)
#pragma unroll
		for (int j = i + 1; j < 9; j++, k++) {
			const float qr = R(kQQR + k);
			U = fmaf(qr, dot(P[i], P[j]), U);
			g[i] = {fmaf(qr, P[j].x, g[i].x), fmaf(qr, P[j].y, g[i].y), fmaf(qr, P[j].z, g[i].z)};
			g[j] = {fmaf(qr, P[i].x, g[j].x), fmaf(qr, P[i].y, g[j].y), fmaf(qr, P[i].z, g[j].z)};
		}
	g[9] = {0.0f, 0.0f, 0.0f};
	rootn<10>(g);
	return U;
}

// The Pixar models (mu / 2 = 1): Full and Reduced on the 4 points, Selective
// the hydrostatic term on them and I1 prefactored
__device__ __forceinline__ float q_pixar(const DevCtx& C, const QRec& R, const BodyParams& bp, uint32_t e,
                                         const float Qi[3][3], const Vec3 P[9], Vec3 g[10]) {
	const float a = __ldg(&bp.a), hw = __ldg(&bp.hw);
	float U = 0.0f;
	zeron<10>(g);
	if (e != 2u) {
#pragma unroll 1
		for (int p = 0; p < 4; p++) {
			float F[3][3], A[3][3], G[3][3];
			q_def_grad(C, Qi, p, P, F);
			const float Ja = adj_det(F, A) - a;
			U = fmaf(0.25f, fmaf(hw * Ja, Ja, trace_xtx(F)), U);
			const float s2 = 0.5f * hw * Ja;
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G[c][r] = fmaf(F[r][c], 0.5f, A[c][r] * s2);
			q_apply(C, G, Qi, p, g);
		}
		rootn<10>(g);
		return U;
	}
	q_hydro(C, Qi, P, a, U, g);
	U *= hw;
#pragma unroll
	for (int n = 0; n < 9; n++) g[n] = {g[n].x * hw, g[n].y * hw, g[n].z * hw};
	rootn<10>(g);
	Vec3 gi[10];
	U += q_pref_i1(R, P, gi);
#pragma unroll
	for (int n = 0; n < 10; n++) g[n] = {g[n].x + gi[n].x, g[n].y + gi[n].y, g[n].z + gi[n].z};
	return U;
}

// The deviatoric term on the 4 points (Mixed, YeohSkin, YeohSkinSel) with
// the hydrostatic term in the same loop when `coupled`; returns U0 before
// the clamp
__device__ __forceinline__ float q_dev_full(const DevCtx& C, const BodyParams& bp, uint32_t e, const float Qi[3][3],
                                            const Vec3 P[9], bool coupled, Vec3 g0[10], float& U1, Vec3 g1[10]) {
	const float a = __ldg(&bp.a);
	const float C0 = __ldg(&bp.yeoh[0]), C1 = __ldg(&bp.yeoh[1]), C2 = __ldg(&bp.yeoh[2]);
	float U0 = 0.0f;
#pragma unroll 1
	for (int p = 0; p < 4; p++) {
		float F[3][3], A[3][3], G[3][3];
		q_def_grad(C, Qi, p, P, F);
		const float J = adj_det(F, A);
		const float I1 = trace_xtx(F);
		float s;
		if (e == 3u) {
			U0 = fmaf(0.25f, I1, U0);
			s = 0.5f;
		} else {
			const float IM = I1 - 3.0f;
			U0 = fmaf(0.25f, IM * fmaf(IM, fmaf(IM, C2, C1), C0), U0);
			s = 0.5f * fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
		}
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) G[c][r] = F[r][c] * s;
		q_apply(C, G, Qi, p, g0);
		if (coupled) {
			const float Ja = J - a;
			U1 = fmaf(0.25f * Ja, Ja, U1);
			const float s1 = 0.5f * Ja;
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G[c][r] = A[c][r] * s1;
			q_apply(C, G, Qi, p, g1);
		}
	}
	return U0;
}

__device__ __forceinline__ void q_load(const DevCtx& C, uint32_t i, uint32_t dv[10]) {
	const uint4 a = __ldg(C.el_vid + 3 * (size_t)i), b = __ldg(C.el_vid + 3 * (size_t)i + 1),
	            c = __ldg(C.el_vid + 3 * (size_t)i + 2);
	dv[0] = a.x, dv[1] = a.y, dv[2] = a.z, dv[3] = a.w, dv[4] = b.x, dv[5] = b.y, dv[6] = b.z, dv[7] = b.w;
	dv[8] = c.x, dv[9] = c.y;
}

__device__ __forceinline__ void q_rel(const float4 O[10], const float4 D[10], bool vmode, Vec3 P[9]) {
#pragma unroll
	for (int i = 0; i < 9; i++)
		P[i] = vmode ? Vec3{O[i].x - O[9].x, O[i].y - O[9].y, O[i].z - O[9].z}
		             : Vec3{(O[i].x - O[9].x) + (D[i].x - D[9].x), (O[i].y - O[9].y) + (D[i].y - D[9].y),
		                    (O[i].z - O[9].z) + (D[i].z - D[9].z)};
}

// One T10 of a pass (the kinds of ElemPass; kRayleigh with the Rayleigh
// ratio rd).
template <int KIND>
__device__ __noinline__ void q_pass(const DevCtx& C, uint32_t i, float inv_dt, float inv_dt2, float rd) {
	uint32_t dv[10];
	q_load(C, i, dv);
	float4 O[10], D[10];
#pragma unroll
	for (int n = 0; n < 10; n++) ld_vertex(C.vert + 2 * (size_t)dv[n], O[n], D[n]);
	const BodyParams& bp = C.bodies[__float_as_uint(D[0].w) >> 8];
	const uint32_t e = __ldg(&bp.energy);
	if (KIND != kVolume && (e == 11u || e == 12u)) return;  // SolveElementCube acts on quads and hexes only
	const QRec R{C.el_rec, C.nel, i};
	float w[10];
#pragma unroll
	for (int n = 0; n < 10; n++) w[n] = O[n].w;
	float Qi[3][3];
#pragma unroll
	for (int c = 0; c < 3; c++)
#pragma unroll
		for (int r = 0; r < 3; r++) Qi[c][r] = R(kQQi + 3 * c + r);
	const float vol = R(kQVol);
	const uint32_t type = __ldg(&bp.rayleigh_type);
	const float damp = KIND == kSolve && type < 2u ? __ldg(&bp.damping) : 0.0f;
	const bool limit = type == 1u;
	const bool sim = __ldg(&bp.simultaneous) != 0u;
	Vec3 P[9], g0[10], g1[10];
	q_rel(O, D, KIND == kRayleigh, P);
	if (KIND == kVolume) {
		float U = 0.0f;
		zeron<10>(g0);
		q_hydro(C, Qi, P, 1.0f, U, g0);
		rootn<10>(g0);
		const float alpha = __ldg(&bp.compliance) * vol * inv_dt2;
		moven<10>(w, (-2.0f * U) / fmaf(2.0f * U, alpha, wdotn<10>(w, g0, g0)), g0, D);
	} else if (e <= 2u) {
		const float U = q_pixar(C, R, bp, e, Qi, P, g0);
		const float comp = __ldg(&bp.compliance) / vol;
		if (KIND == kRayleigh)
			moven<10>(w, -gdotn<10>(g0, D) / fmaf(2.0f * U, comp * inv_dt / rd, wdotn<10>(w, g0, g0)), g0, D);
		else
			moven<10>(w, lambda1n<10>(U, g0, w, D, comp * inv_dt2, comp, damp, limit, inv_dt), g0, D);
	} else {
		const float a = __ldg(&bp.a);
		const float comp0 = __ldg(&bp.inv_mu) / vol, comp1 = __ldg(&bp.inv_lambda) / vol;
		const float alpha0 = comp0 * inv_dt2, alpha1 = comp1 * inv_dt2;
		const bool coupled = KIND == kRayleigh || sim;
		const bool full = full_quadrature(e);
		float U0, U1 = 0.0f;
		zeron<10>(g0);
		zeron<10>(g1);
		if (full) {
			U0 = fmaxf(0.0001f, q_dev_full(C, bp, e, Qi, P, coupled && e != 6u, g0, U1, g1));
			rootn<10>(g0);
		} else {
			U0 = q_pref_i1(R, P, g0);
			if (e == 7u) {
				const float C0 = __ldg(&bp.yeoh[0]), C1 = __ldg(&bp.yeoh[1]), C2 = __ldg(&bp.yeoh[2]);
				const float IM = U0 - 3.0f;
				U0 = fmaxf(0.0001f, IM * fmaf(IM, fmaf(IM, C2, C1), C0));
				const float gs = fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
#pragma unroll
				for (int n = 0; n < 10; n++) g0[n] = {g0[n].x * gs, g0[n].y * gs, g0[n].z * gs};
			}
		}
		if (coupled) {
			if (!full || e == 6u) q_hydro(C, Qi, P, a, U1, g1);
			rootn<10>(g1);
			if (KIND == kRayleigh) {
				if (sim) {
					const float b0 = -gdotn<10>(g0, D), b1 = -gdotn<10>(g1, D);
					float l0, l1;
					cramer(fmaf(2.0f * U0, comp0 * inv_dt / rd, wdotn<10>(w, g0, g0)), wdotn<10>(w, g0, g1),
					       fmaf(2.0f * U1, comp1 * inv_dt / rd, wdotn<10>(w, g1, g1)), b0, b1, l0, l1);
#pragma unroll
					for (int n = 0; n < 10; n++) {
						const float s0 = w[n] * l0, s1 = w[n] * l1;
						D[n].x = fmaf(s1, g1[n].x, fmaf(s0, g0[n].x, D[n].x));
						D[n].y = fmaf(s1, g1[n].y, fmaf(s0, g0[n].y, D[n].y));
						D[n].z = fmaf(s1, g1[n].z, fmaf(s0, g0[n].z, D[n].z));
					}
				} else {
					moven<10>(w, -gdotn<10>(g0, D) / fmaf(2.0f * U0, comp0 * inv_dt / rd, wdotn<10>(w, g0, g0)), g0, D);
					moven<10>(w, -gdotn<10>(g1, D) / fmaf(2.0f * U1, comp1 * inv_dt / rd, wdotn<10>(w, g1, g1)), g1, D);
				}
			} else {
				float l0, l1;
				lambda2n<10>(U0, U1, g0, g1, w, D, alpha0, alpha1, comp0, comp1, damp, limit, inv_dt, l0, l1);
#pragma unroll
				for (int n = 0; n < 10; n++) {
					const float s0 = w[n] * l0, s1 = w[n] * l1;
					D[n].x = fmaf(s1, g1[n].x, fmaf(s0, g0[n].x, D[n].x));
					D[n].y = fmaf(s1, g1[n].y, fmaf(s0, g0[n].y, D[n].y));
					D[n].z = fmaf(s1, g1[n].z, fmaf(s0, g0[n].z, D[n].z));
				}
			}
		} else {
			// serial: deviatoric, refresh P, hydrostatic
			moven<10>(w, lambda1n<10>(U0, g0, w, D, alpha0, comp0, damp, limit, inv_dt), g0, D);
			q_rel(O, D, false, P);
			q_hydro(C, Qi, P, a, U1, g1);
			rootn<10>(g1);
			moven<10>(w, lambda1n<10>(U1, g1, w, D, alpha1, comp1, damp, limit, inv_dt), g1, D);
		}
	}
#pragma unroll
	for (int n = 0; n < 10; n++) st_vertex(C.vert + 2 * (size_t)dv[n], O[n], D[n]);
}

__device__ __noinline__ void q_pbd(const DevCtx& C, uint32_t i, float coeff) {
	uint32_t dv[10];
	q_load(C, i, dv);
	pbd_nodes<10>(C, dv, fminf(1.0f, coeff / QRec{C.el_rec, C.nel, i}(kQArea)));
}

struct T10Elem {
	static constexpr bool kWarp = false;
	static constexpr int kMinBlocks = 1;
	static constexpr uint32_t kVid4 = 3;
	template <int KIND>
	__device__ static void pass(const DevCtx& C, uint32_t i, float inv_dt, float inv_dt2, float rd) {
		q_pass<KIND>(C, i, inv_dt, inv_dt2, rd);
	}
	__device__ static void pbd(const DevCtx& C, uint32_t i, float coeff) { q_pbd(C, i, coeff); }
};

}  // namespace t10e

}  // namespace

}  // namespace xfem
