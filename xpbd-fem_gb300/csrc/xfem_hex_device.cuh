// Device code of the linear hexahedra (H8), shared by the hex mode
// (xfem_hexes.cu) and the mixed tet + hex mode (xfem_mixed.cu): the record
// reader, the element solves (SolveElement on ElementParamsLinearHex,
// XPBDFEM/Fem.cpp:871-896), SolveVolumeOnly, DampElement and PbdDamp over a
// hex. Internal linkage: each translation unit gets its own copy (ptxas 13.0
// crashed on one out-of-line hex solve called from two kernels of one file).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "xfem_elements.cuh"

namespace xfem {

namespace {

// float offsets in the device record
constexpr int kRJL = 0, kRWL = 9, kRVol = 10, kRArea = 11, kRQQ = 12, kRQR = 19, kRJH = 40, kRWH = 112;

struct HexRec {
	const float4* base;
	uint32_t n, i;
	__device__ __forceinline__ float operator()(int j) const {
		return __ldg(reinterpret_cast<const float*>(base + (size_t)(j >> 2) * n + i) + (j & 3));
	}
};

__device__ __forceinline__ float dn(int hi, int p, int n, int k) { return hi ? rest::hex_g8(p, n, k) : rest::hex_g1(n, k); }

// F = Ji MatMul(dN[0..6], P) at a point (XPBDFEM/Fem.cpp:311-323); F and Ji
// column-major ([column][row]).
__device__ __forceinline__ void def_grad(const float Ji[3][3], int hi, int p, const Vec3 P[7], float F[3][3]) {
	float Dm[3][3];  // Dm[c][r] = sum_n dN[n][r] P[n][c]
#pragma unroll
	for (int r = 0; r < 3; r++) {
		float x = 0.0f, y = 0.0f, z = 0.0f;
#pragma unroll
		for (int n = 0; n < 7; n++) {
			const float d = dn(hi, p, n, r);
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
		for (int r = 0; r < 3; r++) F[c][r] = fmaf(Ji[0][r], Dm[c][0], fmaf(Ji[1][r], Dm[c][1], Ji[2][r] * Dm[c][2]));
}

// ApplyEnergyGradient (XPBDFEM/Fem.cpp:338-354): g[n] += (G Ji) dN[n], n < 7.
__device__ __forceinline__ void apply(const float G[3][3], const float Ji[3][3], int hi, int p, Vec3 g[8]) {
	float M[3][3];  // M[j][r] = sum_k G[k][r] Ji[j][k]
#pragma unroll
	for (int j = 0; j < 3; j++)
#pragma unroll
		for (int r = 0; r < 3; r++) M[j][r] = fmaf(G[0][r], Ji[j][0], fmaf(G[1][r], Ji[j][1], G[2][r] * Ji[j][2]));
#pragma unroll
	for (int n = 0; n < 7; n++) {
		const float d0 = dn(hi, p, n, 0), d1 = dn(hi, p, n, 1), d2 = dn(hi, p, n, 2);
		g[n].x += fmaf(M[0][0], d0, fmaf(M[1][0], d1, M[2][0] * d2));
		g[n].y += fmaf(M[0][1], d0, fmaf(M[1][1], d1, M[2][1] * d2));
		g[n].z += fmaf(M[0][2], d0, fmaf(M[1][2], d1, M[2][2] * d2));
	}
}

__device__ __forceinline__ void load_ji(const HexRec& R, int hi, int p, float Ji[3][3]) {
	const int b = hi ? kRJH + 9 * p : kRJL;
#pragma unroll
	for (int c = 0; c < 3; c++)
#pragma unroll
		for (int r = 0; r < 3; r++) Ji[c][r] = R(b + 3 * c + r);
}

// Point p of the centre (hi 0) or 2x2x2 (hi 1) rule: F, adj F, J.
struct Point {
	float Ji[3][3], F[3][3], A[3][3], J, w;
};

__device__ __forceinline__ void point(const HexRec& R, int hi, int p, const Vec3 P[7], Point& q) {
	load_ji(R, hi, p, q.Ji);
	def_grad(q.Ji, hi, p, P, q.F);
	q.J = adj_det(q.F, q.A);
	q.w = R(hi ? kRWH + p : kRWL);
}

// (J - a)^2 over the rule's points into U, g (XPBDFEM/Fem.cpp:539-549).
__device__ __forceinline__ void hydro(const HexRec& R, int hi, const Vec3 P[7], float a, float& U, Vec3 g[8]) {
#pragma unroll 1
	for (int p = 0; p < (hi ? 8 : 1); p++) {
		Point q;
		point(R, hi, p, P, q);
		const float Ja = q.J - a;
		U = fmaf(q.w * Ja, Ja, U);
		const float s = 2.0f * q.w * Ja;
		float G[3][3];
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) G[c][r] = q.A[c][r] * s;
		apply(G, q.Ji, hi, p, g);
	}
}

// I1 prefactored over the seven edge vectors (XPBDFEM/Fem.cpp:163-192),
// root gradient included.
__device__ __forceinline__ float pref_i1(const HexRec& R, const Vec3 P[7], Vec3 g[8]) {
	float U = 0.0f;
#pragma unroll
	for (int i = 0; i < 7; i++) {
		const float qq = R(kRQQ + i);
		U = fmaf(qq, dot(P[i], P[i]), U);
		const float d = 2.0f * qq;
		g[i] = {d * P[i].x, d * P[i].y, d * P[i].z};
	}
	int k = 0;
#pragma unroll
	for (int i = 0; i < 7; i++)
#pragma unroll
		for (int j = i + 1; j < 7; j++, k++) {
			const float qr = R(kRQR + k);
			U = fmaf(qr, dot(P[i], P[j]), U);
			g[i] = {fmaf(qr, P[j].x, g[i].x), fmaf(qr, P[j].y, g[i].y), fmaf(qr, P[j].z, g[i].z)};
			g[j] = {fmaf(qr, P[i].x, g[j].x), fmaf(qr, P[i].y, g[j].y), fmaf(qr, P[i].z, g[j].z)};
		}
	g[7] = {0.0f, 0.0f, 0.0f};
	rootn<8>(g);
	return U;
}

// The Pixar models' U and g (SolveElementPixar, XPBDFEM/Fem.cpp:379-427), mu =
// 2 so mu / 2 = 1: Full on the 2x2x2 points, Reduced on the centre, Selective
// the hydrostatic term on the centre and I1 prefactored.
__device__ __forceinline__ float pixar(const HexRec& R, const BodyParams& bp, uint32_t e, const Vec3 P[7], Vec3 g[8]) {
	const float a = __ldg(&bp.a), hw = __ldg(&bp.hw);
	float U = 0.0f;
	zeron<8>(g);
	if (e != 2u) {
		const int hi = e == 0u;
#pragma unroll 1
		for (int p = 0; p < (hi ? 8 : 1); p++) {
			Point q;
			point(R, hi, p, P, q);
			const float I1 = fmaf(q.F[0][0], q.F[0][0], fmaf(q.F[0][1], q.F[0][1], q.F[0][2] * q.F[0][2])) +
			                 fmaf(q.F[1][0], q.F[1][0], fmaf(q.F[1][1], q.F[1][1], q.F[1][2] * q.F[1][2])) +
			                 fmaf(q.F[2][0], q.F[2][0], fmaf(q.F[2][1], q.F[2][1], q.F[2][2] * q.F[2][2]));
			const float Ja = q.J - a;
			U = fmaf(q.w, fmaf(hw * Ja, Ja, I1), U);
			const float s1 = 2.0f * q.w, s2 = 2.0f * q.w * hw * Ja;
			float G[3][3];
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G[c][r] = fmaf(q.F[r][c], s1, q.A[c][r] * s2);
			apply(G, q.Ji, hi, p, g);
		}
		rootn<8>(g);
		return U;
	}
	hydro(R, 0, P, a, U, g);
	U *= hw;
#pragma unroll
	for (int n = 0; n < 7; n++) g[n] = {g[n].x * hw, g[n].y * hw, g[n].z * hw};
	rootn<8>(g);
	Vec3 gi[8];
	U += pref_i1(R, P, gi);
#pragma unroll
	for (int n = 0; n < 8; n++) g[n] = {g[n].x + gi[n].x, g[n].y + gi[n].y, g[n].z + gi[n].z};
	return U;
}

// The deviatoric term by quadrature on the 2x2x2 points (Mixed: I1;
// YeohSkin, YeohSkinSel: the Yeoh polynomial of I1 - 3; XPBDFEM/Fem.cpp:
// 459-477), with the hydrostatic term in the same loop when `coupled`;
// returns U0 before the clamp of :489.
__device__ __forceinline__ float dev_full(const HexRec& R, const BodyParams& bp, uint32_t e, const Vec3 P[7], bool coupled,
                                          Vec3 g0[8], float& U1, Vec3 g1[8]) {
	const float a = __ldg(&bp.a);
	const float C0 = __ldg(&bp.yeoh[0]), C1 = __ldg(&bp.yeoh[1]), C2 = __ldg(&bp.yeoh[2]);
	float U0 = 0.0f;
#pragma unroll 1
	for (int p = 0; p < 8; p++) {
		Point q;
		point(R, 1, p, P, q);
		const float I1 = fmaf(q.F[0][0], q.F[0][0], fmaf(q.F[0][1], q.F[0][1], q.F[0][2] * q.F[0][2])) +
		                 fmaf(q.F[1][0], q.F[1][0], fmaf(q.F[1][1], q.F[1][1], q.F[1][2] * q.F[1][2])) +
		                 fmaf(q.F[2][0], q.F[2][0], fmaf(q.F[2][1], q.F[2][1], q.F[2][2] * q.F[2][2]));
		float s;
		if (e == 3u) {
			U0 = fmaf(q.w, I1, U0);
			s = 2.0f * q.w;
		} else {
			const float IM = I1 - 3.0f;
			U0 = fmaf(q.w, IM * fmaf(IM, fmaf(IM, C2, C1), C0), U0);
			s = 2.0f * q.w * fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
		}
		float G[3][3];
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) G[c][r] = q.F[r][c] * s;
		apply(G, q.Ji, 1, p, g0);
		if (coupled) {
			const float Ja = q.J - a;
			U1 = fmaf(q.w * Ja, Ja, U1);
			const float s1 = 2.0f * q.w * Ja;
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G[c][r] = q.A[c][r] * s1;
			apply(G, q.Ji, 1, p, g1);
		}
	}
	return U0;
}

__device__ __forceinline__ void rel(const float4 O[8], const float4 D[8], bool vmode, Vec3 P[7]) {
#pragma unroll
	for (int i = 0; i < 7; i++)
		P[i] = vmode ? Vec3{O[i].x - O[7].x, O[i].y - O[7].y, O[i].z - O[7].z}
		             : Vec3{(O[i].x - O[7].x) + (D[i].x - D[7].x), (O[i].y - O[7].y) + (D[i].y - D[7].y),
		                    (O[i].z - O[7].z) + (D[i].z - D[7].z)};
}

// det(F) / 64 of F with rows (sA[i], sB[i], sC[i]) and its adjugate columns
// scaled by 1 / 64 (XPBDFEM/Fem.cpp:613-617, 782-786).
__device__ __forceinline__ float cube_adj(const Vec3& sA, const Vec3& sB, const Vec3& sC, Vec3 A[3]) {
	const float F[3][3] = {{sA.x, sB.x, sC.x}, {sA.y, sB.y, sC.y}, {sA.z, sB.z, sC.z}};
	float M[3][3];
	const float J = adj_det(F, M) * (1.0f / 64.0f);
#pragma unroll
	for (int c = 0; c < 3; c++) A[c] = {M[c][0] * (1.0f / 64.0f), M[c][1] * (1.0f / 64.0f), M[c][2] * (1.0f / 64.0f)};
	return J;
}

// sA, sB, sC: the corner sums weighted by each corner's sign on x, y, z.
__device__ __forceinline__ void corner_sums(const Vec3 R[8], Vec3& sA, Vec3& sB, Vec3& sC) {
	sA = sB = sC = {0.0f, 0.0f, 0.0f};
#pragma unroll
	for (int n = 0; n < 8; n++) {
		const float a = (n & 1) ? 1.0f : -1.0f, b = (n & 2) ? 1.0f : -1.0f, c = (n & 4) ? 1.0f : -1.0f;
		sA = {fmaf(a, R[n].x, sA.x), fmaf(a, R[n].y, sA.y), fmaf(a, R[n].z, sA.z)};
		sB = {fmaf(b, R[n].x, sB.x), fmaf(b, R[n].y, sB.y), fmaf(b, R[n].z, sB.z)};
		sC = {fmaf(c, R[n].x, sC.x), fmaf(c, R[n].y, sC.y), fmaf(c, R[n].z, sC.z)};
	}
}

// SolveElementCube on a hex (XPBDFEM/Fem.cpp:566-838). Positions relative
// to node 7's substep start O7: R[n] = (O[n] - O7) + D[n] (solve mode), or
// O[n] - O7 with V = D (VMODE, the post-step Rayleigh form on the canonical
// state, ratio rd). CubeNeo with nu >= 0.5 and no damping takes the short
// path of :599-640: a uniform pull towards the centroid, then one volume
// projection. Otherwise the I1 term of the corners about the centroid
// (Yeoh for CubeSkin) scales them, and one constraint on det(F) / 64 over the
// four body diagonals restores the volume.
template <bool VMODE>
__device__ __forceinline__ void cube(const BodyParams& bp, const HexRec& R, uint32_t e, const float w[8],
                                     const float4 O[8], float4 D[8], float dt, float inv_dt, float inv_dt2, float rd) {
	const float vol = R(kRVol), area = R(kRArea);
	Vec3 S[8], X[8];
#pragma unroll
	for (int n = 0; n < 8; n++) {
		S[n] = {O[n].x - O[7].x, O[n].y - O[7].y, O[n].z - O[7].z};
		X[n] = VMODE ? S[n] : Vec3{S[n].x + D[n].x, S[n].y + D[n].y, S[n].z + D[n].z};
	}
	Vec3 c = {0.0f, 0.0f, 0.0f};
#pragma unroll
	for (int n = 0; n < 8; n++) c = {c.x + X[n].x, c.y + X[n].y, c.z + X[n].z};
	c = {c.x * 0.125f, c.y * 0.125f, c.z * 0.125f};
	const float damping = VMODE ? rd : __ldg(&bp.damping);
	const uint32_t type = __ldg(&bp.rayleigh_type);
	if (!VMODE && __ldg(&bp.cube_fast)) {
		float wsum = 0.0f;
#pragma unroll
		for (int n = 0; n < 8; n++) wsum += w[n];
		const float ctm = __ldg(&bp.compliance) / (0.125f * wsum);
		const float side = vol / (area * (1.0f / 6.0f));
		const float cs = -2.0f * dt * dt / ctm * (0.5f * side);
		// the moves are added to D as increments: D is small next to the
		// positions, and rebuilding it as X' - S would round it at the
		// positions' ulp (the reference keeps positions in double here)
		Vec3 dX[8];
#pragma unroll
		for (int n = 0; n < 8; n++) {
			dX[n] = {cs * (X[n].x - c.x), cs * (X[n].y - c.y), cs * (X[n].z - c.z)};
			X[n] = {X[n].x + dX[n].x, X[n].y + dX[n].y, X[n].z + dX[n].z};
		}
		Vec3 sA, sB, sC, A[3];
		corner_sums(X, sA, sB, sC);
		const float J = cube_adj(sA, sB, sC, A);
		const float vs = (J - vol) / (8.0f * (dot(A[0], A[0]) + dot(A[1], A[1]) + dot(A[2], A[2])));
#pragma unroll
		for (int n = 0; n < 8; n++) {
			const float a = (n & 1) ? 1.0f : -1.0f, b = (n & 2) ? 1.0f : -1.0f, cc = (n & 4) ? 1.0f : -1.0f;
			const Vec3 g = {fmaf(a, A[0].x, fmaf(b, A[1].x, cc * A[2].x)), fmaf(a, A[0].y, fmaf(b, A[1].y, cc * A[2].y)),
			                fmaf(a, A[0].z, fmaf(b, A[1].z, cc * A[2].z))};
			D[n].x += fmaf(-vs, g.x, dX[n].x);
			D[n].y += fmaf(-vs, g.y, dX[n].y);
			D[n].z += fmaf(-vs, g.z, dX[n].z);
		}
		return;
	}
	Vec3 P[8], dP[8];  // corners about the centroid; their moves (added to D at the end)
#pragma unroll
	for (int n = 0; n < 8; n++) {
		P[n] = {X[n].x - c.x, X[n].y - c.y, X[n].z - c.z};
		dP[n] = {0.0f, 0.0f, 0.0f};
	}
	// the I1 term (Yeoh of it for CubeSkin), XPBDFEM/Fem.cpp:659-712
	{
		float UI = 0.0f, PPw = 0.0f;
#pragma unroll
		for (int n = 0; n < 8; n++) {
			const float PP = dot(P[n], P[n]);
			UI += PP;
			PPw = fmaf(w[n], PP, PPw);
		}
		const float US = 0.5f / ((1.0f / 6.0f) * area);
		UI *= US;
		float gS = 2.0f * US;
		if (e == 12u) {
			const float C0 = __ldg(&bp.yeoh[0]), C1 = __ldg(&bp.yeoh[1]), C2 = __ldg(&bp.yeoh[2]);
			const float IM = UI - 3.0f;
			UI = fmaxf(0.0001f, IM * fmaf(IM, fmaf(IM, C2, C1), C0));
			gS *= fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
		}
		const float alpha = __ldg(&bp.compliance) / vol * inv_dt2;
		float wgg = PPw * gS * gS;
		float lam = (-2.0f * UI) / fmaf(2.0f * UI, alpha, wgg);
		if (!VMODE) {
			if (damping > 0.0f && type < 2u) {
				float gV = 0.0f;
#pragma unroll
				for (int n = 0; n < 8; n++) gV = fmaf(P[n].x, D[n].x, fmaf(P[n].y, D[n].y, fmaf(P[n].z, D[n].z, gV)));
				gV *= gS;
				if (type == 0u) {
					const float gamma = damping * inv_dt;
					lam = (-2.0f * UI - gamma * gV) / fmaf(wgg, 1.0f + gamma, 2.0f * UI * alpha);
				} else {
					const float A = fmaf(2.0f * UI, dt * alpha / damping, wgg);
					const float b = (-gV - wgg * lam) * (A / fmaxf(A, 4.0f * wgg));
					lam += b / A;
				}
			}
			const float PS = lam * gS;
#pragma unroll
			for (int n = 0; n < 8; n++) {
				const float sc = w[n] * PS;
				dP[n] = {P[n].x * sc, P[n].y * sc, P[n].z * sc};
				P[n] = {P[n].x + dP[n].x, P[n].y + dP[n].y, P[n].z + dP[n].z};
			}
		} else if (type >= 2u) {
			wgg += 1.0e-22f;
			float gV = 0.0f;
#pragma unroll
			for (int n = 0; n < 8; n++) gV = fmaf(P[n].x, D[n].x, fmaf(P[n].y, D[n].y, fmaf(P[n].z, D[n].z, gV)));
			const float l2 = -(gS * gV) / fmaf(2.0f * UI, dt * alpha / damping, wgg);
#pragma unroll
			for (int n = 0; n < 8; n++) {
				const float sc = w[n] * l2 * gS;
				D[n].x = fmaf(sc, P[n].x, D[n].x);
				D[n].y = fmaf(sc, P[n].y, D[n].y);
				D[n].z = fmaf(sc, P[n].z, D[n].z);
			}
		}
	}
	// the volume, XPBDFEM/Fem.cpp:779-830: corners q and 7 - q move along
	// +g_q and -g_q
	{
		Vec3 sA, sB, sC, A[3];
		corner_sums(P, sA, sB, sC);
		const float J = cube_adj(sA, sB, sC, A);
		Vec3 g[4];
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const float a = (q & 1) ? 1.0f : -1.0f, b = (q & 2) ? 1.0f : -1.0f;
			g[q] = {fmaf(a, A[0].x, fmaf(b, A[1].x, -A[2].x)), fmaf(a, A[0].y, fmaf(b, A[1].y, -A[2].y)),
			        fmaf(a, A[0].z, fmaf(b, A[1].z, -A[2].z))};
		}
		float wgg = 0.0f;
#pragma unroll
		for (int q = 0; q < 4; q++) wgg = fmaf(w[q] + w[7 - q], dot(g[q], g[q]), wgg);
		const float alpha = vol * __ldg(&bp.inv_lambda) * inv_dt2;
		const float C = J - __ldg(&bp.a) * vol;
		if (VMODE) {
			float gV = 0.0f;
#pragma unroll
			for (int q = 0; q < 4; q++)
				gV += dot({D[q].x - D[7 - q].x, D[q].y - D[7 - q].y, D[q].z - D[7 - q].z}, g[q]);
			const float l2 = -gV / (dt * alpha / damping + (wgg + 1.0e-22f));
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const float s0 = w[q] * l2, s1 = w[7 - q] * l2;
				D[q] = {fmaf(s0, g[q].x, D[q].x), fmaf(s0, g[q].y, D[q].y), fmaf(s0, g[q].z, D[q].z), D[q].w};
				D[7 - q] = {fmaf(-s1, g[q].x, D[7 - q].x), fmaf(-s1, g[q].y, D[7 - q].y), fmaf(-s1, g[q].z, D[7 - q].z),
				            D[7 - q].w};
			}
			return;
		}
		float lam = -C / (wgg + alpha);
		if (damping > 0.0f && type < 2u) {
			// X - O of the corners, with the I1 step's move: D + dP
			float gV = 0.0f;
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const Vec3 d = {(D[q].x + dP[q].x) - (D[7 - q].x + dP[7 - q].x),
				                (D[q].y + dP[q].y) - (D[7 - q].y + dP[7 - q].y),
				                (D[q].z + dP[q].z) - (D[7 - q].z + dP[7 - q].z)};
				gV += dot(d, g[q]);
			}
			if (type == 0u) {
				const float gamma = damping * inv_dt;
				lam = (-C - gamma * gV) / fmaf(wgg, 1.0f + gamma, alpha);
			} else {
				const float Am = wgg + dt * alpha / damping;
				const float b = (-gV - wgg * lam) * (Am / fmaxf(Am, 4.0f * wgg));
				lam += b / Am;
			}
		}
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const float s0 = w[q] * lam, s1 = w[7 - q] * lam;
			dP[q] = {fmaf(s0, g[q].x, dP[q].x), fmaf(s0, g[q].y, dP[q].y), fmaf(s0, g[q].z, dP[q].z)};
			dP[7 - q] = {fmaf(-s1, g[q].x, dP[7 - q].x), fmaf(-s1, g[q].y, dP[7 - q].y), fmaf(-s1, g[q].z, dP[7 - q].z)};
		}
	}
#pragma unroll
	for (int n = 0; n < 8; n++) {
		D[n].x += dP[n].x;
		D[n].y += dP[n].y;
		D[n].z += dP[n].z;
	}
}

// One hex of a pass. kSolve: SolveElement; kVolume: SolveVolumeOnly;
// kRayleigh: DampElement on the canonical state (O = X, D = V) with the
// Rayleigh ratio rd (x 8 when amortized).
template <int KIND>
__device__ __noinline__ void hex_pass(const DevCtx& C, uint32_t i, float inv_dt, float inv_dt2, float rd) {
	const uint4 va = __ldg(C.el_vid + 2 * (size_t)i), vb = __ldg(C.el_vid + 2 * (size_t)i + 1);
	const uint32_t dv[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
	float4 O[8], D[8];
#pragma unroll
	for (int n = 0; n < 8; n++) ld_vertex(C.vert + 2 * (size_t)dv[n], O[n], D[n]);
	const BodyParams& bp = C.bodies[__float_as_uint(D[0].w) >> 8];
	const HexRec R{C.el_rec, C.nel, i};
	const float w[8] = {O[0].w, O[1].w, O[2].w, O[3].w, O[4].w, O[5].w, O[6].w, O[7].w};
	const float vol = R(kRVol);
	const uint32_t e = __ldg(&bp.energy);
	const uint32_t type = __ldg(&bp.rayleigh_type);
	const float damp = KIND == kSolve && type < 2u ? __ldg(&bp.damping) : 0.0f;
	const bool limit = type == 1u;
	const bool sim = __ldg(&bp.simultaneous) != 0u;
	if (KIND != kVolume && (e == 11u || e == 12u)) {
		cube<KIND == kRayleigh>(bp, R, e, w, O, D, 1.0f / inv_dt, inv_dt, inv_dt2, rd);
#pragma unroll
		for (int n = 0; n < 8; n++) st_vertex(C.vert + 2 * (size_t)dv[n], O[n], D[n]);
		return;
	}
	Vec3 P[7], g0[8], g1[8];
	rel(O, D, KIND == kRayleigh, P);
	if (KIND == kVolume) {
		float U = 0.0f;
		zeron<8>(g0);
		hydro(R, 0, P, 1.0f, U, g0);
		rootn<8>(g0);
		const float alpha = __ldg(&bp.compliance) * vol * inv_dt2;
		moven<8>(w, (-2.0f * U) / fmaf(2.0f * U, alpha, wdotn<8>(w, g0, g0)), g0, D);
	} else if (e <= 2u) {
		const float U = pixar(R, bp, e, P, g0);
		const float comp = __ldg(&bp.compliance) / vol;
		if (KIND == kRayleigh) {
			const float gV = gdotn<8>(g0, D);
			moven<8>(w, -gV / fmaf(2.0f * U, comp * inv_dt / rd, wdotn<8>(w, g0, g0)), g0, D);
		} else {
			moven<8>(w, lambda1n<8>(U, g0, w, D, comp * inv_dt2, comp, damp, limit, inv_dt), g0, D);
		}
	} else {
		const float a = __ldg(&bp.a);
		const float comp0 = __ldg(&bp.inv_mu) / vol, comp1 = __ldg(&bp.inv_lambda) / vol;
		const float alpha0 = comp0 * inv_dt2, alpha1 = comp1 * inv_dt2;
		const bool coupled = KIND == kRayleigh || sim;
		const bool full = full_quadrature(e);
		float U0, U1 = 0.0f;
		zeron<8>(g0);
		zeron<8>(g1);
		if (full) {
			U0 = fmaxf(0.0001f, dev_full(R, bp, e, P, coupled && e != 6u, g0, U1, g1));
			rootn<8>(g0);
		} else {
			U0 = pref_i1(R, P, g0);
			if (e == 7u) {
				const float C0 = __ldg(&bp.yeoh[0]), C1 = __ldg(&bp.yeoh[1]), C2 = __ldg(&bp.yeoh[2]);
				const float IM = U0 - 3.0f;
				U0 = fmaxf(0.0001f, IM * fmaf(IM, fmaf(IM, C2, C1), C0));
				const float gs = fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
#pragma unroll
				for (int n = 0; n < 8; n++) g0[n] = {g0[n].x * gs, g0[n].y * gs, g0[n].z * gs};
			}
		}
		if (coupled) {
			if (!full || e == 6u) hydro(R, 0, P, a, U1, g1);
			rootn<8>(g1);
			if (KIND == kRayleigh) {
				// RayleighDamp (XPBDFEM/Xpbd.h:217-263) on V = D
				if (sim) {
					const float b0 = -gdotn<8>(g0, D), b1 = -gdotn<8>(g1, D);
					float l0, l1;
					cramer(fmaf(2.0f * U0, comp0 * inv_dt / rd, wdotn<8>(w, g0, g0)), wdotn<8>(w, g0, g1),
					       fmaf(2.0f * U1, comp1 * inv_dt / rd, wdotn<8>(w, g1, g1)), b0, b1, l0, l1);
#pragma unroll
					for (int n = 0; n < 8; n++) {
						const float s0 = w[n] * l0, s1 = w[n] * l1;
						D[n].x = fmaf(s1, g1[n].x, fmaf(s0, g0[n].x, D[n].x));
						D[n].y = fmaf(s1, g1[n].y, fmaf(s0, g0[n].y, D[n].y));
						D[n].z = fmaf(s1, g1[n].z, fmaf(s0, g0[n].z, D[n].z));
					}
				} else {
					moven<8>(w, -gdotn<8>(g0, D) / fmaf(2.0f * U0, comp0 * inv_dt / rd, wdotn<8>(w, g0, g0)), g0, D);
					moven<8>(w, -gdotn<8>(g1, D) / fmaf(2.0f * U1, comp1 * inv_dt / rd, wdotn<8>(w, g1, g1)), g1, D);
				}
			} else {
				float l0, l1;
				lambda2n<8>(U0, U1, g0, g1, w, D, alpha0, alpha1, comp0, comp1, damp, limit, inv_dt, l0, l1);
#pragma unroll
				for (int n = 0; n < 8; n++) {
					const float s0 = w[n] * l0, s1 = w[n] * l1;
					D[n].x = fmaf(s1, g1[n].x, fmaf(s0, g0[n].x, D[n].x));
					D[n].y = fmaf(s1, g1[n].y, fmaf(s0, g0[n].y, D[n].y));
					D[n].z = fmaf(s1, g1[n].z, fmaf(s0, g0[n].z, D[n].z));
				}
			}
		} else {
			// serial: deviatoric, refresh P, hydrostatic (XPBDFEM/Fem.cpp:490-521, 532-551)
			moven<8>(w, lambda1n<8>(U0, g0, w, D, alpha0, comp0, damp, limit, inv_dt), g0, D);
			rel(O, D, false, P);
			hydro(R, full && e != 6u, P, a, U1, g1);
			rootn<8>(g1);
			moven<8>(w, lambda1n<8>(U1, g1, w, D, alpha1, comp1, damp, limit, inv_dt), g1, D);
		}
	}
#pragma unroll
	for (int n = 0; n < 8; n++) st_vertex(C.vert + 2 * (size_t)dv[n], O[n], D[n]);
}

// PbdDamp over a hex's 8 nodes with coeff / surfaceArea capped at 1.
__device__ __forceinline__ void hex_pbd_inl(const DevCtx& C, uint32_t i, float coeff) {
	const uint4 va = __ldg(C.el_vid + 2 * (size_t)i), vb = __ldg(C.el_vid + 2 * (size_t)i + 1);
	const uint32_t dv[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
	pbd_nodes<8>(C, dv, fminf(1.0f, coeff / HexRec{C.el_rec, C.nel, i}(kRArea)));
}
__device__ __noinline__ void hex_pbd(const DevCtx& C, uint32_t i, float coeff) { hex_pbd_inl(C, i, coeff); }

struct HexElem {
	static constexpr bool kWarp = false;
	static constexpr int kMinBlocks = 1;
	static constexpr uint32_t kVid4 = 2;
	template <int KIND>
	__device__ static void pass(const DevCtx& C, uint32_t i, float inv_dt, float inv_dt2, float rd) {
		hex_pass<KIND>(C, i, inv_dt, inv_dt2, rd);
	}
	__device__ static void pbd(const DevCtx& C, uint32_t i, float coeff) { hex_pbd(C, i, coeff); }
};

}  // namespace

}  // namespace xfem
