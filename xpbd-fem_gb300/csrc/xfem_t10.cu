// Quadratic-tet mode of libxfem.so (sm_103a): GeoQuadratic3d on a tet mesh
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
#include "xfem_elements.cuh"
#include "xfem_ring_update.cuh"

namespace xfem {

namespace {

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

// ---- the continuous-pressure models on T10s -----------------------------------
//
// SolveRing of a mesh vertex's one-ring over the T10s around it
// (XPBDFEM/Geo.cpp:147-225; GeoQuadratic3d::Init rings the mesh's own
// vertices only, :944-953): every ring T10 adds the full-energy branch of
// CalculateElementEnergyAndGradients (XPBDFEM/Fem.cpp:983-1036) weighted by
// elemWeight = (volume / PointsLo) / ring volume, PointsLo = PointsHi = 4,
// the ring volume being a quarter of each T10's volume: the deviatoric term
// (I1 prefactored over the 10 nodes, or for ContinuousSkin the Yeoh
// polynomial of I1 - 3 on the 4 points with the model's own constants) and
// (J - a)^2 on the 4 points. Then one constraint (ContinuousPixar, mu = 2:
// U0 + (lambda / 2) U1) or the coupled pair over the ring's nodes.
//
// One warp per ring: lane j takes the ring's T10s j and j + 32 and leaves
// their ten nodes' gradient contributions in shared memory; lane n takes ring
// nodes n, n + 32, n + 64 and n + 96, sums each one's contributions in T10
// order and takes its update.

struct QRingScratch {
	float4 O[kMaxQRingNodes], D[kMaxQRingNodes];  // ring nodes: (O, w), (D, bits)
	float g0[kMaxQRingElems][10][3];              // per T10 node: deviatoric gradient contribution
	float g1[kMaxQRingElems][10][3];              // per T10 node: (J - a)^2 gradient contribution
};

// Ring T10 `j` of a one-ring (element ei, its nodes at ring slots loc[]):
// its nodes' gradient contributions into the scratch, its weighted
// deviatoric and (J - a)^2 energies returned.
template <bool VMODE>
__device__ __forceinline__ float2 q_ring_elem(const DevCtx& C, QRingScratch& S, const BodyParams& bp, uint32_t j,
                                           uint32_t ei, const uint32_t loc[10], float volume) {
	float4 O[10], D[10];
#pragma unroll
	for (int k = 0; k < 10; k++) {
		O[k] = S.O[loc[k]];
		D[k] = S.D[loc[k]];
	}
	Vec3 P[9], g[10];
	q_rel(O, D, VMODE, P);
	const QRec R{C.el_rec, C.nel, ei};
	float Qi[3][3];
#pragma unroll
	for (int c = 0; c < 3; c++)
#pragma unroll
		for (int r = 0; r < 3; r++) Qi[c][r] = R(kQQi + 3 * c + r);
	const float ew = (R(kQVol) * 0.25f) / volume;  // the T10's share of the ring volume
	float U0 = 0.0f;
	if (__ldg(&bp.energy) == 10u) {
		// ContinuousSkin: the Yeoh polynomial of I1 - 3 on the 4 points
		const float C0 = 0.1095f, C1 = 14.95f, C2 = 4.595f;
		zeron<10>(g);
#pragma unroll 1
		for (int p = 0; p < 4; p++) {
			float F[3][3], G[3][3];
			q_def_grad(C, Qi, p, P, F);
			const float IM = trace_xtx(F) - 3.0f, wt = ew * 0.25f;
			U0 = fmaf(wt, IM * fmaf(IM, fmaf(IM, C2, C1), C0), U0);
			const float sg = wt * fmaf(IM, fmaf(IM, 6.0f * C2, 4.0f * C1), 2.0f * C0);
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G[c][r] = F[r][c] * sg;
			q_apply(C, G, Qi, p, g);
		}
		rootn<10>(g);
	} else {
		U0 = ew * q_pref_i1(R, P, g);
#pragma unroll
		for (int n = 0; n < 10; n++) g[n] = {ew * g[n].x, ew * g[n].y, ew * g[n].z};
	}
#pragma unroll
	for (int n = 0; n < 10; n++) {
		S.g0[j][n][0] = g[n].x;
		S.g0[j][n][1] = g[n].y;
		S.g0[j][n][2] = g[n].z;
	}
	// (J - a)^2 on the 4 points
	const float a = __ldg(&bp.a_ring);
	float U1 = 0.0f;
	zeron<10>(g);
#pragma unroll 1
	for (int p = 0; p < 4; p++) {
		float F[3][3], A[3][3], G[3][3];
		q_def_grad(C, Qi, p, P, F);
		const float Ja = adj_det(F, A) - a, wt = ew * 0.25f;
		U1 = fmaf(wt * Ja, Ja, U1);
		const float sg = wt * 2.0f * Ja;
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) G[c][r] = A[c][r] * sg;
		q_apply(C, G, Qi, p, g);
	}
	rootn<10>(g);
#pragma unroll
	for (int n = 0; n < 10; n++) {
		S.g1[j][n][0] = g[n].x;
		S.g1[j][n][1] = g[n].y;
		S.g1[j][n][2] = g[n].z;
	}
	return make_float2(U0, U1);
}

// Ring entry j of the ring whose entries start at e0: the T10's device index,
// and (when loc is given) its 10 nodes' ring slots.
__device__ __forceinline__ uint32_t ring_t10(const DevCtx& C, uint32_t e0, uint32_t j, uint32_t loc[10]) {
	const float4 e = __ldg(C.ring_ent + 2 * ((size_t)e0 + j));
	if (loc) {
		const uint32_t wd[3] = {__float_as_uint(e.y), __float_as_uint(e.z), __float_as_uint(e.w)};
#pragma unroll
		for (int k = 0; k < 10; k++) loc[k] = (wd[k >> 2] >> (8 * (k & 3))) & 0xffu;
	}
	return __float_as_uint(e.x);
}

// SolveRing of ring r over T10s by the calling warp (every lane takes part).
// VMODE: the post-step Rayleigh form on the canonical state (X, V) for the
// rings of this tick's slice.
template <bool DAMP, bool VMODE>
__device__ __forceinline__ void q_ring_solve(const DevCtx& C, QRingScratch& S, uint32_t r, uint32_t lane, float inv_dt,
                                          float inv_dt2, uint32_t tick) {
	__syncwarp();  // every lane is done with the previous ring's scratch
	const uint4 h = __ldg(C.ring_hdr + r);
	const uint32_t nn = h.z & 0xffu, ne = (h.z >> 8) & 0xffu;
	const BodyParams& bp = C.bodies[h.z >> 16];
	float rd = 0.0f;
	if (VMODE) {
		const uint32_t type = __ldg(&bp.rayleigh_type);
		rd = __ldg(&bp.damping) * (type == 3u ? 8.0f : 1.0f);
		if (!(type >= 2u && rd > 0.0f)) return;
		if (type == 3u) {
			const uint32_t nv = __ldg(&bp.nverts), m = tick % 8u;
			if (h.w < nv * m / 8u || h.w >= nv * (m + 1u) / 8u) return;
		}
	}
	uint32_t dv[kQNodesPerLane];
#pragma unroll
	for (uint32_t k = 0; k < kQNodesPerLane; k++) {
		const uint32_t n = lane + 32u * k;
		dv[k] = 0;
		if (n < nn) {
			dv[k] = __ldg(C.ring_node + h.x + n);
			ld_vertex(C.vert + 2 * (size_t)dv[k], S.O[n], S.D[n]);
		}
	}
	// entry j: the T10's device index and its nodes' ring slots
	float volq = 0.0f;
	for (uint32_t j = lane; j < ne; j += 32u) volq += 0.25f * QRec{C.el_rec, C.nel, ring_t10(C, h.y, j, nullptr)}(kQVol);
	const float volume = warp_sum(volq);  // the ring's volume
	__syncwarp();
	float2 Uc = make_float2(0.0f, 0.0f);
	for (uint32_t j = lane; j < ne; j += 32u) {
		uint32_t loc[10];
		const uint32_t ei = ring_t10(C, h.y, j, loc);
		const float2 u = q_ring_elem<VMODE>(C, S, bp, j, ei, loc, volume);
		Uc.x += u.x;
		Uc.y += u.y;
	}
	const float U0 = warp_sum(Uc.x), U1 = warp_sum(Uc.y);
	__syncwarp();
	// each node's gradients: its contributions summed in T10 order
	Vec3 g0[kQNodesPerLane], g1[kQNodesPerLane];
	const uint16_t* cl = C.ring_cwords + __ldg(C.ring_clist + r);
#pragma unroll
	for (uint32_t k = 0; k < kQNodesPerLane; k++) {
		const uint32_t n = lane + 32u * k;
		g0[k] = {0.0f, 0.0f, 0.0f};
		g1[k] = {0.0f, 0.0f, 0.0f};
		if (n >= nn) continue;
		const uint32_t cb = __ldg(cl + n), ce = __ldg(cl + n + 1);
		for (uint32_t i = cb; i < ce; i++) {
			const uint32_t q = __ldg(cl + nn + 1 + i), j = q >> 4, m = q & 15u;
			g0[k] = {g0[k].x + S.g0[j][m][0], g0[k].y + S.g0[j][m][1], g0[k].z + S.g0[j][m][2]};
			g1[k] = {g1[k].x + S.g1[j][m][0], g1[k].y + S.g1[j][m][1], g1[k].z + S.g1[j][m][2]};
		}
	}
	if (__ldg(&bp.energy) == 8u) {
		// ContinuousPixar: mu = 2, one constraint U0 + (lambda / 2) U1 with
		// compliance per the ring volume
		const float hw = __ldg(&bp.hw);
#pragma unroll
		for (uint32_t k = 0; k < kQNodesPerLane; k++)
			g0[k] = {fmaf(hw, g1[k].x, g0[k].x), fmaf(hw, g1[k].y, g0[k].y), fmaf(hw, g1[k].z, g0[k].z)};
		q_ring_update<DAMP, VMODE>(C, S, bp, lane, nn, dv, g0, g1, false, fmaxf(0.000001f, fmaf(hw, U1, U0)), 0.0f,
		                           __ldg(&bp.compliance) / volume, 0.0f, inv_dt, inv_dt2, rd);
		return;
	}
	// ContinuousMixed / ContinuousSkin: the deviatoric and hydrostatic pair
	const float mu = __ldg(&bp.mu), lambda = __ldg(&bp.lambda);
	q_ring_update<DAMP, VMODE>(C, S, bp, lane, nn, dv, g0, g1, true, fmaxf(0.0001f, U0), U1, 1.0f / (mu * volume),
	                           1.0f / (lambda * volume), inv_dt, inv_dt2, rd);
}

// The persistent T10 ring kernel (cooperative launch, co-resident grid): per
// substep the advance pass, one pass per ring colour, and with post-step
// damping a finalize pass, the rings' Rayleigh passes and the PBD passes
// over the T10 colours (GeoQuadratic3d::Damp, XPBDFEM/Geo.cpp:987-1008).
template <bool DAMP>
__global__ void __launch_bounds__(128) k_t10_rings(DevCtx C, uint32_t nsub, float dt) {
	extern __shared__ __align__(128) unsigned char smem[];
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = (blockDim.x >> 5) * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	QRingScratch& S = reinterpret_cast<QRingScratch*>(smem)[wib];
	const uint32_t tick0 = __ldcg(C.tick);
	const bool dmode = DAMP && C.damp_kinds != 0u;
	uint32_t target = C.bar_base;
	for (uint32_t s = 0; s < nsub; s++) {
		for (uint32_t v = gtid; v < C.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(C.vert + 2 * (size_t)v, O, D);
			advance_vertex(C, v, O, D, s == 0 || dmode, dt, inv_dt);
			st_vertex(C.vert + 2 * (size_t)v, O, D);
		}
		if (!grid_sync(C, target)) return;
		for (uint32_t c = 0; c < C.ring_colours; c++) {
			const uint32_t rb = __ldg(C.colour_ring_begin + c), re = __ldg(C.colour_ring_begin + c + 1);
			for (uint32_t r = rb + gwarp; r < re; r += nwarps) q_ring_solve<DAMP, false>(C, S, r, lane, inv_dt, inv_dt2, 0);
			if (!grid_sync(C, target)) return;
		}
		if (!dmode) continue;
		if constexpr (DAMP) {
			for (uint32_t v = gtid; v < C.nverts; v += nthreads) {
				float4 O, D;
				ld_vertex(C.vert + 2 * (size_t)v, O, D);
				finalize_vertex(C, v, O, D, inv_dt);
				st_vertex(C.vert + 2 * (size_t)v, O, D);
			}
			if (!grid_sync(C, target)) return;
			const uint32_t tick = tick0 + s;
			if (C.damp_kinds & 1u)
				for (uint32_t c = 0; c < C.ring_colours; c++) {
					const uint32_t rb = __ldg(C.colour_ring_begin + c), re = __ldg(C.colour_ring_begin + c + 1);
					for (uint32_t r = rb + gwarp; r < re; r += nwarps)
						q_ring_solve<true, true>(C, S, r, lane, inv_dt, inv_dt2, tick);
					if (!grid_sync(C, target)) return;
				}
			if (C.damp_kinds & 2u)
				for (uint32_t c = 0; c < C.el_colours; c++) {
					const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
					for (uint32_t i = b + gtid; i < e; i += nthreads) {
						const BodyParams& bp = body_of_el<T10Elem>(C, i);
						if (__ldg(&bp.pbd_on) && in_slice(C, bp, i, tick)) {
							// inlined: an out-of-line device function called from two kernels of one
							// file made ptxas 13.0 crash
							const float coeff =
							    __ldg(&bp.rayleigh_type) == 3u ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff);
							uint32_t dvp[10];
							q_load(C, i, dvp);
							pbd_nodes<10>(C, dvp, fminf(1.0f, coeff / QRec{C.el_rec, C.nel, i}(kQArea)));
						}
					}
					if (!grid_sync(C, target)) return;
				}
		}
	}
	if (!dmode) {
		for (uint32_t v = gtid; v < C.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(C.vert + 2 * (size_t)v, O, D);
			finalize_vertex(C, v, O, D, inv_dt);
			st_vertex(C.vert + 2 * (size_t)v, O, D);
		}
	}
	if (gtid == 0) *C.tick = tick0 + nsub;
}

}  // namespace

int launch_t10_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = ctx.ext ? (const void*)k_t10_rings<true> : (const void*)k_t10_rings<false>;
	const size_t smem = (size_t)(block / 32) * sizeof(QRingScratch);
	int dev = 0, sms = 0, per_sm = 0;
	cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess) e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, block, smem);
	if (e != cudaSuccess) return (int)e;
	if (per_sm <= 0) return (int)cudaErrorInvalidConfiguration;
	e = reset_barrier(ctx, st);
	if (e != cudaSuccess) return (int)e;
	DevCtx c = ctx;
	void* args[] = {&c, &nsub, &dt};
	return (int)cudaLaunchCooperativeKernel(f, dim3(per_sm * sms), dim3(block), args, smem, st);
}

int launch_t10(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	return launch_elements<T10Elem>(ctx, block, nsub, dt, stream);
}

}  // namespace xfem
