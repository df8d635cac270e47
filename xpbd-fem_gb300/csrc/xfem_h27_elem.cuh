// Quadratic-hex element code of libxfem.so (sm_103a), shared by the H27
// mode (xfem_h27.cu) and meshes mixing T10s and H27s (xfem_qmixed.cu): GeoQuadratic3d on a hex mesh
// (XPBDFEM/Geo.cpp:836-1053). Every hex gets a node on each edge and face and
// one at its centre, numbered i + 3j + 9k on its 3x3x3 grid; SolveElement on
// ElementParamsQuadraticHex (XPBDFEM/Fem.cpp:871-897: SolveElementPixar
// :361-433 and SolveElementMixed :437-564 with Nodes = 27, PointsLo = 8 and
// PointsHi = 27; the cube models leave an H27 alone), SolveVolumeOnly on the
// 2x2x2 rule (:840-867), DampElement (:910-937) and PbdDamp
// (XPBDFEM/Xpbd.h:306-346), in the element kernel of xfem_elements.cuh.
//
// One warp per H27: an element's 27 nodes, its 703-value record and its 27
// quadrature points do not fit one thread. Lane n < 27 owns node n (its load,
// its share of the prefactored I1, its gradient rows, its update); lane p
// owns quadrature point p when the deformation gradients are formed. The
// node offsets P and each point's G Ji (the energy gradient mapped back to
// the reference frame) pass between the two through 2.2 KB of shared memory
// per warp, next to the warp's copy of the element's record. Sums over lanes
// are xor butterflies, so every lane holds the same bits and every lane takes
// the same branch.
//
// Records: 704 floats per H27 (the 703 of the reference's flattening, one
// pad), element-major, read by every lane of the element's warp. The
// gradient tables (the 2x2x2 rule's 648 floats, then the 3x3x3 rule's 2187)
// sit in el_tab.
#pragma once

#include "xfem_elements.cuh"

namespace xfem {

namespace {

namespace h27e {

constexpr int kJL = 0, kWL = 72, kJH = 80, kWH = 323, kQQ = 350, kQR = 376, kVol = 701, kArea = 702, kRec = 704;
constexpr int kTab8 = 0, kTab27 = 8 * 27 * 3;
constexpr unsigned kAll = 0xffffffffu;

__device__ __forceinline__ float wsum(float v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kAll, v, o);
	return v;
}

// per-warp scratch: the element's record (copied in once per element, so
// the lanes' scattered reads of it wait on shared memory, not on L2), node
// offsets from node 26, and each point's G Ji for the first and the second
// constraint
struct Scratch {
	float4 rec[kRec / 4];
	float P[26][3];
	float M0[27][9], M1[27][9];
};

struct Elem {
	const float* R;  // the record (this warp's shared copy)
	uint32_t lane;
	float4 O, D;  // this lane's node (lanes >= 27: zero)
	float w;
	uint32_t dv;
};

__device__ __forceinline__ float rec(const Elem& E, int j) { return E.R[j]; }

// P_n = (O_n - O_26) + (D_n - D_26) (solve), or O_n - O_26 (vmode)
__device__ __forceinline__ void share_rel(Scratch& s, const Elem& E, bool vmode) {
	const float ox = __shfl_sync(kAll, E.O.x, 26), oy = __shfl_sync(kAll, E.O.y, 26), oz = __shfl_sync(kAll, E.O.z, 26);
	const float dx = __shfl_sync(kAll, E.D.x, 26), dy = __shfl_sync(kAll, E.D.y, 26), dz = __shfl_sync(kAll, E.D.z, 26);
	__syncwarp();
	if (E.lane < 26) {
		s.P[E.lane][0] = vmode ? E.O.x - ox : (E.O.x - ox) + (E.D.x - dx);
		s.P[E.lane][1] = vmode ? E.O.y - oy : (E.O.y - oy) + (E.D.y - dy);
		s.P[E.lane][2] = vmode ? E.O.z - oz : (E.O.z - oz) + (E.D.z - dz);
	}
	__syncwarp();
}

__device__ __forceinline__ float tab(const DevCtx& C, int hi, int p, int n, int k) {
	return __ldg(C.el_tab + (hi ? kTab27 : kTab8) + (p * 27 + n) * 3 + k);
}

__device__ __forceinline__ float trace_xtx(const float F[3][3]) {
	return fmaf(F[0][0], F[0][0], fmaf(F[0][1], F[0][1], F[0][2] * F[0][2])) +
	       fmaf(F[1][0], F[1][0], fmaf(F[1][1], F[1][1], F[1][2] * F[1][2])) +
	       fmaf(F[2][0], F[2][0], fmaf(F[2][1], F[2][1], F[2][2] * F[2][2]));
}

// What a point computes (the per-point terms of SolveElementPixar and
// SolveElementMixed, XPBDFEM/Fem.cpp:379-427, 459-489, 532-549).
enum PointTerm {
	kHydro = 0,      // (J - a)^2 into slot 1
	kPixarFull = 1,  // I1 + hw (J - a)^2 (mu / 2 = 1) into slot 0
	kDev = 2,        // the deviatoric I1 (Mixed) or its Yeoh polynomial into slot 0
	kDevHydro = 3,   // kDev, and (J - a)^2 into slot 1
};

// The point terms over a rule (hi: the 27 points, else the 8) into M0 / M1;
// returns this lane's U contributions (summed by the caller). wscale scales
// every point's weight (a ring element's share of its ring volume); skin: the
// Yeoh constants of ContinuousSkin (XPBDFEM/Fem.cpp:994) instead of the
// body's.
template <int TERM>
__device__ __forceinline__ void points(const DevCtx& C, Scratch& s, const Elem& E, int hi, const BodyParams& bp,
                                       uint32_t e, float a, float& u0, float& u1, float wscale = 1.0f,
                                       bool skin = false) {
	const int np = hi ? 27 : 8;
	u0 = u1 = 0.0f;
	const int p = (int)E.lane;
	if (p < np) {
		float Ji[3][3];
		const int jb = (hi ? kJH : kJL) + 9 * p;
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) Ji[c][r] = rec(E, jb + 3 * c + r);
		const float wt = wscale * rec(E, (hi ? kWH : kWL) + p);
		float Dm[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
#pragma unroll 2
		for (int n = 0; n < 26; n++) {
			const float px = s.P[n][0], py = s.P[n][1], pz = s.P[n][2];
#pragma unroll
			for (int r = 0; r < 3; r++) {
				const float d = tab(C, hi, p, n, r);
				Dm[0][r] = fmaf(d, px, Dm[0][r]);
				Dm[1][r] = fmaf(d, py, Dm[1][r]);
				Dm[2][r] = fmaf(d, pz, Dm[2][r]);
			}
		}
		float F[3][3], A[3][3], G0[3][3], G1[3][3];
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) F[c][r] = fmaf(Ji[0][r], Dm[c][0], fmaf(Ji[1][r], Dm[c][1], Ji[2][r] * Dm[c][2]));
		const float J = adj_det(F, A);
		const float Ja = J - a;
		if (TERM == kHydro || TERM == kDevHydro) {
			u1 = wt * Ja * Ja;
			const float s1 = 2.0f * wt * Ja;
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G1[c][r] = A[c][r] * s1;
		}
		if (TERM == kPixarFull) {
			const float hw = __ldg(&bp.hw);
			u0 = wt * fmaf(hw * Ja, Ja, trace_xtx(F));
			const float s1 = 2.0f * wt, s2 = 2.0f * wt * hw * Ja;
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G0[c][r] = fmaf(F[r][c], s1, A[c][r] * s2);
		}
		if (TERM == kDev || TERM == kDevHydro) {
			const float I1 = trace_xtx(F);
			float sc;
			if (e == 3u) {
				u0 = wt * I1;
				sc = 2.0f * wt;
			} else {
				const float C0 = skin ? 0.1095f : __ldg(&bp.yeoh[0]), C1 = skin ? 14.95f : __ldg(&bp.yeoh[1]),
				            C2 = skin ? 4.595f : __ldg(&bp.yeoh[2]);
				const float IM = I1 - 3.0f;
				u0 = wt * (IM * fmaf(IM, fmaf(IM, C2, C1), C0));
				sc = 2.0f * wt * fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
			}
#pragma unroll
			for (int c = 0; c < 3; c++)
#pragma unroll
				for (int r = 0; r < 3; r++) G0[c][r] = F[r][c] * sc;
		}
		// M[j][r] = sum_k G[k][r] Ji[j][k]
		if (TERM != kHydro)
#pragma unroll
			for (int j = 0; j < 3; j++)
#pragma unroll
				for (int r = 0; r < 3; r++)
					s.M0[p][3 * j + r] = fmaf(G0[0][r], Ji[j][0], fmaf(G0[1][r], Ji[j][1], G0[2][r] * Ji[j][2]));
		if (TERM == kHydro || TERM == kDevHydro)
#pragma unroll
			for (int j = 0; j < 3; j++)
#pragma unroll
				for (int r = 0; r < 3; r++)
					s.M1[p][3 * j + r] = fmaf(G1[0][r], Ji[j][0], fmaf(G1[1][r], Ji[j][1], G1[2][r] * Ji[j][2]));
	}
	__syncwarp();
}

// g_n += sum_p M_p dN_p[n] for this lane's node (n < 26) from slot M
__device__ __forceinline__ Vec3 gather(const DevCtx& C, const float (*M)[9], const Elem& E, int hi) {
	Vec3 g = {0.0f, 0.0f, 0.0f};
	const int np = hi ? 27 : 8, n = (int)E.lane;
	if (n < 26)
#pragma unroll 1
		for (int p = 0; p < np; p++) {
			const float d0 = tab(C, hi, p, n, 0), d1 = tab(C, hi, p, n, 1), d2 = tab(C, hi, p, n, 2);
			g.x += fmaf(M[p][0], d0, fmaf(M[p][3], d1, M[p][6] * d2));
			g.y += fmaf(M[p][1], d0, fmaf(M[p][4], d1, M[p][7] * d2));
			g.z += fmaf(M[p][2], d0, fmaf(M[p][5], d1, M[p][8] * d2));
		}
	return g;
}

// node 26 takes minus the others' sum
__device__ __forceinline__ Vec3 root(const Elem& E, Vec3 g) {
	const float sx = wsum(E.lane < 26 ? g.x : 0.0f), sy = wsum(E.lane < 26 ? g.y : 0.0f),
	            sz = wsum(E.lane < 26 ? g.z : 0.0f);
	return E.lane == 26 ? Vec3{g.x - sx, g.y - sy, g.z - sz} : E.lane < 26 ? g : Vec3{0.0f, 0.0f, 0.0f};
}

// The prefactored I1 over the 26 offsets (XPBDFEM/Fem.cpp:163-192): this
// lane's gradient row (root included) and U.
__device__ __forceinline__ float pref_i1(const Scratch& s, const Elem& E, Vec3& g) {
	float u = 0.0f;
	g = {0.0f, 0.0f, 0.0f};
	const int i = (int)E.lane;
	if (i < 26) {
		const float qq = rec(E, kQQ + i);
		const Vec3 Pi = {s.P[i][0], s.P[i][1], s.P[i][2]};
		u = qq * dot(Pi, Pi);
		g = {2.0f * qq * Pi.x, 2.0f * qq * Pi.y, 2.0f * qq * Pi.z};
		// QR of the pair (lo, hi), lo < hi: row lo starts at lo (51 - lo) / 2
#pragma unroll 2
		for (int j = 0; j < 26; j++) {
			if (j == i) continue;
			const int lo = i < j ? i : j, hi = i < j ? j : i;
			const float qr = rec(E, kQR + lo * (51 - lo) / 2 + (hi - lo - 1));
			const Vec3 Pj = {s.P[j][0], s.P[j][1], s.P[j][2]};
			g = {fmaf(qr, Pj.x, g.x), fmaf(qr, Pj.y, g.y), fmaf(qr, Pj.z, g.z)};
			if (j > i) u = fmaf(qr, dot(Pi, Pj), u);
		}
	}
	g = root(E, g);
	return wsum(u);
}

__device__ __forceinline__ float wgg_of(const Elem& E, const Vec3& a, const Vec3& b) {
	return 1.0e-22f + wsum(E.lane < 27 ? E.w * dot(a, b) : 0.0f);
}
__device__ __forceinline__ float gD_of(const Elem& E, const Vec3& g) {
	return wsum(E.lane < 27 ? fmaf(g.x, E.D.x, fmaf(g.y, E.D.y, g.z * E.D.z)) : 0.0f);
}
__device__ __forceinline__ void move(Elem& E, float l, const Vec3& g) {
	const float s = E.w * l;
	E.D.x = fmaf(s, g.x, E.D.x);
	E.D.y = fmaf(s, g.y, E.D.y);
	E.D.z = fmaf(s, g.z, E.D.z);
}
__device__ __forceinline__ void move2(Elem& E, float l0, const Vec3& g0, float l1, const Vec3& g1) {
	const float s0 = E.w * l0, s1 = E.w * l1;
	E.D.x = fmaf(s1, g1.x, fmaf(s0, g0.x, E.D.x));
	E.D.y = fmaf(s1, g1.y, fmaf(s0, g0.y, E.D.y));
	E.D.z = fmaf(s1, g1.z, fmaf(s0, g0.z, E.D.z));
}

__device__ __forceinline__ Scratch& scratch() {
	__shared__ Scratch s[8];  // 256-thread blocks: 8 warps
	return s[threadIdx.x >> 5];
}

__device__ __forceinline__ void load(const DevCtx& C, uint32_t i, Scratch& s, Elem& E) {
	E.lane = threadIdx.x & 31u;
	// the record, 176 float4, coalesced across the warp, once every lane is
	// done with the previous element's copy
	__syncwarp();
	const float4* src = C.el_rec + (size_t)i * (kRec / 4);
	for (uint32_t k = E.lane; k < kRec / 4; k += 32) s.rec[k] = __ldg(src + k);
	__syncwarp();
	E.R = reinterpret_cast<const float*>(s.rec);
	E.O = E.D = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	E.w = 0.0f;
	E.dv = 0;
	if (E.lane < 27) {
		E.dv = __ldg(reinterpret_cast<const uint32_t*>(C.el_vid + 7 * (size_t)i) + E.lane);
		ld_vertex(C.vert + 2 * (size_t)E.dv, E.O, E.D);
		E.w = E.O.w;
	}
}

// One H27 of a pass (the kinds of ElemPass), every lane of the warp.
template <int KIND>
__device__ __noinline__ void h27_pass(const DevCtx& C, uint32_t i, float inv_dt, float inv_dt2, float rd) {
	Scratch& s = scratch();
	Elem E;
	load(C, i, s, E);
	const BodyParams& bp = C.bodies[__float_as_uint(__shfl_sync(kAll, E.D.w, 0)) >> 8];
	const uint32_t e = __ldg(&bp.energy);
	if (KIND != kVolume && (e == 11u || e == 12u)) return;  // SolveElementCube acts on 8-node hexes only
	const float vol = rec(E, kVol);
	const uint32_t type = __ldg(&bp.rayleigh_type);
	const float damp = KIND == kSolve && type < 2u ? __ldg(&bp.damping) : 0.0f;
	const bool limit = type == 1u;
	const bool sim = __ldg(&bp.simultaneous) != 0u;
	share_rel(s, E, KIND == kRayleigh);
	float u0, u1;
	if (KIND == kVolume) {
		points<kHydro>(C, s, E, 0, bp, e, 1.0f, u0, u1);
		const Vec3 g = root(E, gather(C, s.M1, E, 0));
		const float U = wsum(u1);
		const float alpha = __ldg(&bp.compliance) * vol * inv_dt2;
		move(E, (-2.0f * U) / fmaf(2.0f * U, alpha, wgg_of(E, g, g)), g);
	} else if (e <= 2u) {
		float U;
		Vec3 g;
		if (e != 2u) {
			const int hi = e == 0u;
			points<kPixarFull>(C, s, E, hi, bp, e, __ldg(&bp.a), u0, u1);
			g = root(E, gather(C, s.M0, E, hi));
			U = wsum(u0);
		} else {
			const float hw = __ldg(&bp.hw);
			points<kHydro>(C, s, E, 0, bp, e, __ldg(&bp.a), u0, u1);
			Vec3 gh = root(E, gather(C, s.M1, E, 0));
			Vec3 gi;
			const float UI = pref_i1(s, E, gi);
			U = fmaf(hw, wsum(u1), UI);
			g = {fmaf(hw, gh.x, gi.x), fmaf(hw, gh.y, gi.y), fmaf(hw, gh.z, gi.z)};
		}
		const float comp = __ldg(&bp.compliance) / vol;
		const float wgg = wgg_of(E, g, g);
		if (KIND == kRayleigh)
			move(E, -gD_of(E, g) / fmaf(2.0f * U, comp * inv_dt / rd, wgg), g);
		else
			move(E, lambda1_of(U, wgg, damp > 0.0f ? gD_of(E, g) : 0.0f, comp * inv_dt2, comp, damp, limit, inv_dt), g);
	} else {
		const float a = __ldg(&bp.a);
		const float comp0 = __ldg(&bp.inv_mu) / vol, comp1 = __ldg(&bp.inv_lambda) / vol;
		const float alpha0 = comp0 * inv_dt2, alpha1 = comp1 * inv_dt2;
		const bool coupled = KIND == kRayleigh || sim;
		const bool full = full_quadrature(e);
		float U0, U1 = 0.0f;
		Vec3 g0, g1 = {0.0f, 0.0f, 0.0f};
		if (full) {
			if (coupled && e != 6u) {
				points<kDevHydro>(C, s, E, 1, bp, e, a, u0, u1);
				g1 = root(E, gather(C, s.M1, E, 1));
				U1 = wsum(u1);
			} else {
				points<kDev>(C, s, E, 1, bp, e, a, u0, u1);
			}
			g0 = root(E, gather(C, s.M0, E, 1));
			U0 = fmaxf(0.0001f, wsum(u0));
		} else {
			U0 = pref_i1(s, E, g0);
			if (e == 7u) {
				const float C0 = __ldg(&bp.yeoh[0]), C1 = __ldg(&bp.yeoh[1]), C2 = __ldg(&bp.yeoh[2]);
				const float IM = U0 - 3.0f;
				U0 = fmaxf(0.0001f, IM * fmaf(IM, fmaf(IM, C2, C1), C0));
				const float gs = fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
				g0 = {g0.x * gs, g0.y * gs, g0.z * gs};
			}
		}
		if (coupled) {
			if (!full || e == 6u) {
				__syncwarp();
				points<kHydro>(C, s, E, 0, bp, e, a, u0, u1);
				g1 = root(E, gather(C, s.M1, E, 0));
				U1 = wsum(u1);
			}
			const float wgg0 = wgg_of(E, g0, g0), wgg1 = wgg_of(E, g1, g0), wgg2 = wgg_of(E, g1, g1);
			float l0, l1;
			if (KIND == kRayleigh) {
				if (sim) {
					cramer(fmaf(2.0f * U0, comp0 * inv_dt / rd, wgg0), wgg1, fmaf(2.0f * U1, comp1 * inv_dt / rd, wgg2),
					       -gD_of(E, g0), -gD_of(E, g1), l0, l1);
					move2(E, l0, g0, l1, g1);
				} else {
					move(E, -gD_of(E, g0) / fmaf(2.0f * U0, comp0 * inv_dt / rd, wgg0), g0);
					move(E, -gD_of(E, g1) / fmaf(2.0f * U1, comp1 * inv_dt / rd, wgg2), g1);
				}
			} else {
				const bool dm = damp > 0.0f;
				lambda2_of(U0, U1, wgg0, wgg1, wgg2, dm ? gD_of(E, g0) : 0.0f, dm ? gD_of(E, g1) : 0.0f, alpha0, alpha1,
				           comp0, comp1, damp, limit, inv_dt, l0, l1);
				move2(E, l0, g0, l1, g1);
			}
		} else {
			// serial: deviatoric, refresh P, hydrostatic (XPBDFEM/Fem.cpp:490-521, 532-551)
			const float wgg0 = wgg_of(E, g0, g0);
			move(E, lambda1_of(U0, wgg0, damp > 0.0f ? gD_of(E, g0) : 0.0f, alpha0, comp0, damp, limit, inv_dt), g0);
			share_rel(s, E, false);
			const int hi = full && e != 6u;
			points<kHydro>(C, s, E, hi, bp, e, a, u0, u1);
			g1 = root(E, gather(C, s.M1, E, hi));
			U1 = wsum(u1);
			const float wgg2 = wgg_of(E, g1, g1);
			move(E, lambda1_of(U1, wgg2, damp > 0.0f ? gD_of(E, g1) : 0.0f, alpha1, comp1, damp, limit, inv_dt), g1);
		}
	}
	__syncwarp();
	if (E.lane < 27) st_vertex(C.vert + 2 * (size_t)E.dv, E.O, E.D);
}

// PbdDamp over the 27 nodes (XPBDFEM/Xpbd.h:306-346) on the canonical state
// (O = X, D = V), the coefficient coeff / surfaceArea capped at 1.
__device__ __forceinline__ void h27_pbd_in(const DevCtx& C, Scratch& s, uint32_t i, float coeff) {
	Elem E;
	load(C, i, s, E);
	const bool node = E.lane < 27;
	const float damping = fminf(1.0f, coeff / rec(E, kArea));
	const float Wavg = (1.0e-8f + wsum(E.w)) * (1.0f / 27.0f), Wmin = 0.0001f * Wavg;
	const float rx = __shfl_sync(kAll, E.O.x, 26), ry = __shfl_sync(kAll, E.O.y, 26), rz = __shfl_sync(kAll, E.O.z, 26);
	const Vec3 x = {E.O.x - rx, E.O.y - ry, E.O.z - rz};
	const float M = node ? Wavg / fmaxf(Wmin, E.w) : 0.0f;
	const float im = 1.0f / wsum(M);
	const Vec3 xcm = {wsum(x.x * M) * im, wsum(x.y * M) * im, wsum(x.z * M) * im};
	const Vec3 vcm = {wsum(E.D.x * M) * im, wsum(E.D.y * M) * im, wsum(E.D.z * M) * im};
	const Vec3 r = {x.x - xcm.x, x.y - xcm.y, x.z - xcm.z};
	const Vec3 c = cross(r, v3(E.D));
	const Vec3 L = {wsum(M * c.x), wsum(M * c.y), wsum(M * c.z)};
	const float xx = r.x * r.x, yy = r.y * r.y, zz = r.z * r.z;
	const float I00 = wsum(M * (yy + zz)), I11 = wsum(M * (xx + zz)), I22 = wsum(M * (xx + yy));
	const float I01 = -wsum(M * (r.x * r.y)), I12 = -wsum(M * (r.y * r.z)), I02 = -wsum(M * (r.z * r.x));
	const float a00 = fmaf(I11, I22, -I12 * I12), a01 = fmaf(I02, I12, -I01 * I22), a02 = fmaf(I01, I12, -I02 * I11);
	const float a11 = fmaf(I00, I22, -I02 * I02), a12 = fmaf(I01, I02, -I00 * I12), a22 = fmaf(I00, I11, -I01 * I01);
	const float idet = 1.0f / fmaf(I00, a00, fmaf(I01, a01, I02 * a02));
	const Vec3 om = {fmaf(a00, L.x, fmaf(a01, L.y, a02 * L.z)) * idet, fmaf(a01, L.x, fmaf(a11, L.y, a12 * L.z)) * idet,
	                 fmaf(a02, L.x, fmaf(a12, L.y, a22 * L.z)) * idet};
	const Vec3 cr = cross(om, r);
	E.D.x = fmaf(damping, (vcm.x + cr.x) - E.D.x, E.D.x);
	E.D.y = fmaf(damping, (vcm.y + cr.y) - E.D.y, E.D.y);
	E.D.z = fmaf(damping, (vcm.z + cr.z) - E.D.z, E.D.z);
	if (node) st_vertex(C.vert + 2 * (size_t)E.dv, E.O, E.D);
}

__device__ __noinline__ void h27_pbd(const DevCtx& C, uint32_t i, float coeff) { h27_pbd_in(C, scratch(), i, coeff); }

struct H27Elem {
	static constexpr bool kWarp = true;
	static constexpr int kMinBlocks = 3;  // at most 85 registers: three 256-thread blocks per SM
	static constexpr uint32_t kVid4 = 7;
	template <int KIND>
	__device__ static void pass(const DevCtx& C, uint32_t i, float inv_dt, float inv_dt2, float rd) {
		h27_pass<KIND>(C, i, inv_dt, inv_dt2, rd);
	}
	__device__ static void pbd(const DevCtx& C, uint32_t i, float coeff) { h27_pbd(C, i, coeff); }
};

}  // namespace h27e

}  // namespace

}  // namespace xfem
