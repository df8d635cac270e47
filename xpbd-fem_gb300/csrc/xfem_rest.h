// Set-up arithmetic shared by the host (xfem_host.cpp) and the GPU set-up
// kernels (xfem_setup.cu), so that both run the same operations in the same
// order. The reference's rest-state precompute of one linear tet:
// InitTriTetFiniteElement (XPBDFEM/Fem.cpp:196-224) with
// GeneratePrefactoredCoefficients (XPBDFEM/Fem.cpp:131-161) and
// inverse(mat3) (XPBDFEM/vectormath.cpp:40-58).
// Bit-exact with the reference as long as nothing is fused: the host compiles
// with -ffp-contract=off, the device with -fmad=false, and float division and
// square root are correctly rounded on both (IEEE).
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define XFEM_HD __host__ __device__ __forceinline__
#else
#define XFEM_HD inline
#endif

namespace xfem {
namespace rest {

// Column-major 3x3 as the reference's GLSL-style mat3 (XPBDFEM/vectormath.h:190-197).
struct M3 {
	float c[3][3];  // c[column][row]
};

XFEM_HD float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// determinant(mat3), XPBDFEM/vectormath.cpp:34-39
XFEM_HD float det3(const M3& m) {
	float a = m.c[0][0], b = m.c[1][0], c = m.c[2][0];
	float d = m.c[0][1], e = m.c[1][1], f = m.c[2][1];
	float g = m.c[0][2], h = m.c[1][2], i = m.c[2][2];
	return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

// inverse(mat3): adjugate in double rounded to float, determinant and 1/det
// scaling in float.
XFEM_HD M3 inverse3(const M3& m) {
	const double m00 = m.c[0][0], m01 = m.c[0][1], m02 = m.c[0][2];
	const double m10 = m.c[1][0], m11 = m.c[1][1], m12 = m.c[1][2];
	const double m20 = m.c[2][0], m21 = m.c[2][1], m22 = m.c[2][2];
	M3 adj;
	adj.c[0][0] = (float)(m11 * m22 - m12 * m21);
	adj.c[0][1] = (float)-(m01 * m22 - m02 * m21);
	adj.c[0][2] = (float)(m01 * m12 - m02 * m11);
	adj.c[1][0] = (float)-(m10 * m22 - m12 * m20);
	adj.c[1][1] = (float)(m00 * m22 - m02 * m20);
	adj.c[1][2] = (float)-(m00 * m12 - m02 * m10);
	adj.c[2][0] = (float)(m10 * m21 - m11 * m20);
	adj.c[2][1] = (float)-(m00 * m21 - m01 * m20);
	adj.c[2][2] = (float)(m00 * m11 - m01 * m10);
	const float det = m.c[0][0] * adj.c[0][0] + m.c[0][1] * adj.c[1][0] + m.c[0][2] * adj.c[2][0];
	const float s = 1.0f / det;
	M3 out;
	for (int c = 0; c < 3; c++)
		for (int r = 0; r < 3; r++) out.c[c][r] = adj.c[c][r] * s;
	return out;
}

// Map jacobian sum_n dN_n (x) P_n of the linear tet: column j, row n = P_n[j];
// accumulating from a zero matrix normalises -0 to +0 (the "0.0f +").
XFEM_HD M3 map_jacobian(const float P[4][3]) {
	M3 J;
	for (int c = 0; c < 3; c++)
		for (int r = 0; r < 3; r++) J.c[c][r] = 0.0f + P[r][c];
	return J;
}

// column k of m as (m * e_k), the reference's mat3 * vec3 with a unit vector
XFEM_HD void column_of(const M3& m, int k, float out[3]) {
	const float e[3] = {k == 0 ? 1.0f : 0.0f, k == 1 ? 1.0f : 0.0f, k == 2 ? 1.0f : 0.0f};
	for (int r = 0; r < 3; r++) {
		const float row[3] = {m.c[0][r], m.c[1][r], m.c[2][r]};
		out[r] = dot3(row, e);
	}
}

// FaceArea of InitTriTetFiniteElement (XPBDFEM/Fem.cpp:211-213)
XFEM_HD float face_area(const float P[4][3], int i0, int i1, int i2) {
	float a[3], b[3];
	for (int k = 0; k < 3; k++) {
		a[k] = P[i0][k] - P[i2][k];
		b[k] = P[i1][k] - P[i2][k];
	}
	const float c[3] = {a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]};
	return 0.5f * sqrtf(dot3(c, c));
}

// One tet: o[17] = Qi column-major, QQ, QR, volume, surfaceArea; returns the
// mass (1/4) density volume that each of its nodes receives (LumpsTet4,
// XPBDFEM/Fem.cpp:217-223). `nodes` is the float node array, `is` the tet's
// four vertex ids.
XFEM_HD float tet(const float* nodes, const uint32_t* is, float density, float* o) {
	const float sixth = 1.0f / 6.0f;
	// P[n] = vec3(X[n] - X[root]) with X the node data widened to double
	float P[4][3];
	for (int n = 0; n < 4; n++)
		for (int k = 0; k < 3; k++)
			P[n][k] = (float)((double)nodes[3 * (size_t)is[n] + k] - (double)nodes[3 * (size_t)is[3] + k]);
	const M3 J = map_jacobian(P);
	const M3 Qi = inverse3(J);
	// GeneratePrefactoredCoefficients<Tet>: four quadrature points with the
	// same gradients, so the same inverse and weight (det J / 6) / 4 at each;
	// the four additions stay four additions
	const float wq = det3(J) * sixth * 0.25f;
	float q[3][3];
	for (int i = 0; i < 3; i++) column_of(Qi, i, q[i]);
	float QQ[3] = {0, 0, 0}, QR[3] = {0, 0, 0}, vsum = 0.0f;
	for (int p = 0; p < 4; p++) {
		vsum += wq;
		for (int i = 0; i < 3; i++) QQ[i] += wq * dot3(q[i], q[i]);
		int head = 0;
		for (int i = 0; i < 3; i++)
			for (int j = i + 1; j < 3; j++) QR[head++] += wq * 2.0f * dot3(q[i], q[j]);
	}
	for (int i = 0; i < 3; i++) QQ[i] /= vsum;
	for (int i = 0; i < 3; i++) QR[i] /= vsum;
	const float vol = sixth * det3(J);
	const float area = face_area(P, 0, 1, 2) + face_area(P, 1, 3, 2) + face_area(P, 0, 2, 3) + face_area(P, 3, 1, 0);
	for (int c = 0; c < 3; c++)
		for (int r = 0; r < 3; r++) o[c * 3 + r] = Qi.c[c][r];
	for (int i = 0; i < 3; i++) {
		o[9 + i] = QQ[i];
		o[12 + i] = QR[i];
	}
	o[15] = vol;
	o[16] = area;
	return (1.0f / 4.0f) * density * vol;
}

// ---- linear hexahedra (H8) ----
// Nodes and quadrature points are numbered i + 2j + 4k (sign 2 bit - 1 per
// axis). The reference tabulates the shape functions and their gradients at
// the 2x2x2 Gauss points and the gradients at the centre to six decimals
// (XPBDFEM/Fem.cpp:40, :68-69); each entry is one of these printed magnitudes,
// picked by how many axes node and point agree on. The printed values, not
// the exact Gauss values, are what every rest state is built from.
XFEM_HD float hex_n8(int p, int n) {  // ShapeFunctions<Hex, 8, 8>[p][n]
	const int agree = !((p ^ n) & 1) + !((p ^ n) & 2) + !((p ^ n) & 4);
	return agree == 3 ? 0.490562f : agree == 2 ? 0.131446f : agree == 1 ? 0.035221f : 0.009437f;
}

XFEM_HD float hex_g8(int p, int n, int k) {  // ShapeFunctionGradients<Hex, 8, 8>[p][n][k]
	int agree = 0;
	for (int a = 0; a < 3; a++)
		if (a != k) agree += !(((p ^ n) >> a) & 1);
	const float m = agree == 2 ? 0.311004f : agree == 1 ? 0.083333f : 0.022329f;
	return ((n >> k) & 1) ? m : -m;
}

XFEM_HD float hex_g1(int n, int k) { return ((n >> k) & 1) ? 0.125f : -0.125f; }  // <Hex, 8, 1>[0][n][k]

// Offsets in the 120-value hex record (ElementParamsLinearHex,
// XPBDFEM/Fem.h:90-100, flattened): qcLo.Ji[0] column-major, qcLo.w[0],
// qcHi.Ji[p], qcHi.w[p], ic.QQ[7], ic.QR[21], volume, surfaceArea.
constexpr int kHexJL = 0, kHexWL = 9, kHexJH = 10, kHexWH = 82, kHexQQ = 90, kHexQR = 97, kHexVol = 118,
              kHexArea = 119, kHexRec = 120;

// MatMul(dN, P) over the 8 map nodes (XPBDFEM/Fem.cpp:86-94): from zero,
// element [c][r] accumulates dN[n][r] P[n][c] in node order.
XFEM_HD M3 hex_map_jacobian(const float P[8][3], int hi, int p) {
	M3 J;
	for (int c = 0; c < 3; c++)
		for (int r = 0; r < 3; r++) J.c[c][r] = 0.0f;
	for (int n = 0; n < 8; n++)
		for (int c = 0; c < 3; c++)
			for (int r = 0; r < 3; r++) J.c[c][r] = J.c[c][r] + (hi ? hex_g8(p, n, r) : hex_g1(n, r)) * P[n][c];
	return J;
}

// One hex: InitQuadHexFiniteElement (XPBDFEM/Fem.cpp:225-265) with
// GenerateMappedQuadratureCoefficients (:110-125) for the centre and the
// 2x2x2 points and GeneratePrefactoredCoefficients (:131-161) on the 2x2x2
// points. o: the 120-value record; m[8]: the lumped mass of each node (the
// normalised diagonal of the mass matrix times density and volume).
XFEM_HD void hex(const float* nodes, const uint32_t* is, float density, float* o, float m[8]) {
	float P[8][3];
	for (int n = 0; n < 8; n++)
		for (int k = 0; k < 3; k++)
			P[n][k] = (float)((double)nodes[3 * (size_t)is[n] + k] - (double)nodes[3 * (size_t)is[7] + k]);
	for (int hi = 0; hi < 2; hi++) {
		const int np = hi ? 8 : 1;
		float vsum = 0.0f;
		for (int p = 0; p < np; p++) {
			const M3 J = hex_map_jacobian(P, hi, p);
			const float detJ = det3(J);
			const M3 Ji = inverse3(J);
			float* j = o + (hi ? kHexJH + 9 * p : kHexJL);
			for (int c = 0; c < 3; c++)
				for (int r = 0; r < 3; r++) j[c * 3 + r] = Ji.c[c][r];
			float& w = o[hi ? kHexWH + p : kHexWL];
			w = detJ * (hi ? 1.0f : 8.0f);
			vsum += w;
		}
		for (int p = 0; p < np; p++) o[hi ? kHexWH + p : kHexWL] /= vsum;
	}
	float* QQ = o + kHexQQ;
	float* QR = o + kHexQR;
	for (int i = 0; i < 7; i++) QQ[i] = 0.0f;
	for (int i = 0; i < 21; i++) QR[i] = 0.0f;
	float vsum = 0.0f, vol = 0.0f;
	for (int p = 0; p < 8; p++) {
		const M3 J = hex_map_jacobian(P, 1, p);
		const M3 Ji = inverse3(J);
		const float w = det3(J) * 1.0f * 1.0f;
		float q[7][3];
		for (int i = 0; i < 7; i++) {
			const float dn[3] = {hex_g8(p, i, 0), hex_g8(p, i, 1), hex_g8(p, i, 2)};
			for (int r = 0; r < 3; r++) {
				const float row[3] = {Ji.c[0][r], Ji.c[1][r], Ji.c[2][r]};
				q[i][r] = dot3(row, dn);
			}
		}
		vsum += w;
		for (int i = 0; i < 7; i++) QQ[i] += w * dot3(q[i], q[i]);
		int head = 0;
		for (int i = 0; i < 7; i++)
			for (int j = i + 1; j < 7; j++) QR[head++] += w * 2.0f * dot3(q[i], q[j]);
	}
	for (int i = 0; i < 7; i++) QQ[i] /= vsum;
	for (int i = 0; i < 21; i++) QR[i] /= vsum;
	for (int p = 0; p < 8; p++) vol += det3(hex_map_jacobian(P, 1, p)) * 1.0f;
	o[kHexVol] = vol;
	const int faces[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 2, 4, 6}, {1, 3, 5, 7}};
	float area = 0.0f;
	for (int f = 0; f < 6; f++) {
		float a[3], b[3];
		for (int k = 0; k < 3; k++) {
			a[k] = P[faces[f][0]][k] - P[faces[f][3]][k];
			b[k] = P[faces[f][1]][k] - P[faces[f][2]][k];
		}
		const float c[3] = {a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]};
		area += 0.5f * sqrtf(dot3(c, c));
	}
	o[kHexArea] = area;
	float mmd[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, msum = 0.0f;
	for (int p = 0; p < 8; p++) {
		const float w = o[kHexWH + p];
		for (int n = 0; n < 8; n++) {
			const float Nn = hex_n8(p, n);
			mmd[n] += w * Nn * Nn;
			msum += w * Nn * Nn;
		}
	}
	for (int n = 0; n < 8; n++) m[n] = (mmd[n] / msum) * density * vol;
}

// ---- quadratic tetrahedra (T10), host only ----
// Nodes: the corners 0-3 with barycentric coordinates L0 = x, L1 = y, L2 = z,
// L3 = 1 - x - y - z, then one node per edge (0,1) (0,2) (0,3) (1,2) (1,3)
// (2,3). The gradient of corner c is (4 L_c - 1) grad L_c; of edge node
// (a, b) 4 (L_b grad L_a + L_a grad L_b). The reference prints its tables at
// the 4-point rule (the solve, XPBDFEM/Fem.cpp:60) and the 10-point rule (the
// prefactored coefficients, :61) to six decimals, with the weights (:11-12);
// every entry is the printed magnitude nearest its value, so the tables are
// built from those literals. The rule's coordinates come from the same
// printed numbers: 4-point rule point p has L_p = a4, the others b4; the
// 10-point rule's points 0-3 have L_p = a10 (others b10), and points 4-9,
// one per edge in node order, c10 on the edge's two corners and d10 on the
// other two.
constexpr int kT10EdgeNodes[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

inline double t10_bary(int np, int p, int c) {
	if (np == 4) return p == c ? (1.341641 + 1.0) / 4.0 : (1.0 - 0.447214) / 4.0;
	if (p < 4) return p == c ? (2.113981 + 1.0) / 4.0 : (1.0 - 0.704660) / 4.0;
	const bool on = c == kT10EdgeNodes[p - 4][0] || c == kT10EdgeNodes[p - 4][1];
	return on ? (0.624977 + 1.0) / 4.0 : (1.0 - 0.624977) / 4.0;
}

// ShapeFunctionGradients<Tet, 10, np>[p][n][k] for np = 4 or 10
inline float t10_grad(int np, int p, int n, int k) {
	static const double printed4[] = {0.447214, 0.552786, 1.341641, 1.788854, 2.341641};
	static const double printed10[] = {0.295340, 0.375023, 0.624977, 0.704660, 1.249955,
	                                   1.624977, 2.113981, 2.818642, 3.113981};
	// grad L_c: e_c for c < 3, (-1, -1, -1) for c = 3
	auto gl = [](int c, int axis) { return c == 3 ? -1.0 : (c == axis ? 1.0 : 0.0); };
	double v;
	if (n < 4) {
		v = (4.0 * t10_bary(np, p, n) - 1.0) * gl(n, k);
	} else {
		const int a = kT10EdgeNodes[n - 4][0], b = kT10EdgeNodes[n - 4][1];
		v = 4.0 * (t10_bary(np, p, b) * gl(a, k) + t10_bary(np, p, a) * gl(b, k));
	}
	const double* mag = np == 4 ? printed4 : printed10;
	const int nm = np == 4 ? 5 : 9;
	if (fabs(v) < 1e-3) return 0.0f;
	int best = 0;
	for (int i = 1; i < nm; i++)
		if (fabs(fabs(v) - mag[i]) < fabs(fabs(v) - mag[best])) best = i;
	return v < 0.0 ? -(float)mag[best] : (float)mag[best];
}

// QuadratureWeights<Tet, np>[p]
inline float t10_weight(int np, int p) { return np == 4 ? 0.250000f : p < 4 ? 0.047633f : 0.134911f; }

// The tables built once: g4[p][n][k] at the 4-point rule, g10 at the 10-point
// rule, w10 its weights.
struct T10Tables {
	float g4[4][10][3], g10[10][10][3], w10[10];
};
inline const T10Tables& t10_tables() {
	static const T10Tables t = [] {
		T10Tables r;
		for (int p = 0; p < 10; p++) {
			r.w10[p] = t10_weight(10, p);
			for (int n = 0; n < 10; n++)
				for (int k = 0; k < 3; k++) {
					if (p < 4) r.g4[p][n][k] = t10_grad(4, p, n, k);
					r.g10[p][n][k] = t10_grad(10, p, n, k);
				}
		}
		return r;
	}();
	return t;
}

// Offsets in the 56-value T10 record (ElementParamsQuadraticTet,
// XPBDFEM/Fem.h:61-69, flattened): Qi column-major (one inverse for the whole
// element: the map from the corners is linear), ic.QQ[9], ic.QR[36], volume,
// surfaceArea.
constexpr int kT10Qi = 0, kT10QQ = 9, kT10QR = 18, kT10Vol = 54, kT10Area = 55, kT10Rec = 56;

// One T10: InitTriTetFiniteElement (XPBDFEM/Fem.cpp:196-224) with the corner
// map and GeneratePrefactoredCoefficients on the 10-point rule (:131-161). X:
// the vertex positions in double; is: the T10's 10 indices; o: the 56-value
// record; m[10]: each node's lumped mass (LumpsTet10: 13/472 of density x
// volume per corner, 70/472 per edge node).
inline void t10(const double* X, const uint32_t* is, float density, float* o, float m[10]) {
	const float sixth = 1.0f / 6.0f;
	float P[4][3];
	for (int n = 0; n < 4; n++)
		for (int k = 0; k < 3; k++) P[n][k] = (float)(X[3 * (size_t)is[n] + k] - X[3 * (size_t)is[3] + k]);
	const M3 J = map_jacobian(P);
	const M3 Qi = inverse3(J);
	// every point of the 10-point rule has the map's jacobian J
	const float detJ = det3(J);
	const T10Tables& tb = t10_tables();
	float* QQ = o + kT10QQ;
	float* QR = o + kT10QR;
	for (int i = 0; i < 9; i++) QQ[i] = 0.0f;
	for (int i = 0; i < 36; i++) QR[i] = 0.0f;
	float vsum = 0.0f;
	for (int p = 0; p < 10; p++) {
		const float w = detJ * sixth * tb.w10[p];
		float q[9][3];
		for (int i = 0; i < 9; i++) {
			const float* dn = tb.g10[p][i];
			for (int r = 0; r < 3; r++) {
				const float row[3] = {Qi.c[0][r], Qi.c[1][r], Qi.c[2][r]};
				q[i][r] = dot3(row, dn);
			}
		}
		vsum += w;
		for (int i = 0; i < 9; i++) QQ[i] += w * dot3(q[i], q[i]);
		int head = 0;
		for (int i = 0; i < 9; i++)
			for (int j = i + 1; j < 9; j++) QR[head++] += w * 2.0f * dot3(q[i], q[j]);
	}
	for (int i = 0; i < 9; i++) QQ[i] /= vsum;
	for (int i = 0; i < 36; i++) QR[i] /= vsum;
	const float vol = sixth * det3(J);
	const float area = face_area(P, 0, 1, 2) + face_area(P, 1, 3, 2) + face_area(P, 0, 2, 3) + face_area(P, 3, 1, 0);
	for (int c = 0; c < 3; c++)
		for (int r = 0; r < 3; r++) o[kT10Qi + c * 3 + r] = Qi.c[c][r];
	o[kT10Vol] = vol;
	o[kT10Area] = area;
	for (int n = 0; n < 10; n++) m[n] = ((n < 4 ? 13.0f : 70.0f) / 472.0f) * density * vol;
}

// ---- quadratic hexahedra (H27), host only ----
// Nodes and quadrature points are numbered i + 3j + 9k on each element's
// 3x3x3 grid (i + 2j + 4k on the 2x2x2 rule), with the 1-D nodes -1, 0, 1 and
// the 1-D shape functions x (x - 1) / 2, 1 - x^2, x (x + 1) / 2. The
// reference's tables (XPBDFEM/Fem.cpp:16-18, 41-44, 70-73) are those
// functions evaluated in double at the 1-D Gauss points and weights as
// printed to six decimals (0.774597, 0 and 0.577350; weights 0.555556 and
// 0.888889), each entry then printed to six decimals; that method gives
// every entry, so the tables are built with it.
struct H27Tables {
	float g8[8][27][3], g27[27][27][3], n27[27][27], map27[27][8][3], w27[27];
};
inline const H27Tables& h27_tables() {
	static const H27Tables t = [] {
		const double x3[3] = {-0.774597, 0.0, 0.774597}, x2[2] = {-0.577350, 0.577350};
		const double w3[3] = {0.555556, 0.888889, 0.555556};
		auto q = [](int i, double x) { return i == 0 ? x * (x - 1) / 2 : i == 1 ? (1 - x) * (1 + x) : x * (x + 1) / 2; };
		auto dq = [](int i, double x) { return i == 0 ? x - 0.5 : i == 1 ? -2 * x : x + 0.5; };
		auto r6 = [](double v) { return (float)(nearbyint(v * 1e6) / 1e6); };
		H27Tables r;
		for (int p = 0; p < 27; p++) {
			const double x[3] = {x3[p % 3], x3[(p / 3) % 3], x3[p / 9]};
			r.w27[p] = r6(w3[p % 3] * w3[(p / 3) % 3] * w3[p / 9]);
			for (int n = 0; n < 27; n++) {
				const int ix[3] = {n % 3, (n / 3) % 3, n / 9};
				r.n27[p][n] = r6(q(ix[0], x[0]) * q(ix[1], x[1]) * q(ix[2], x[2]));
				for (int k = 0; k < 3; k++) {
					double v = 1.0;
					for (int a = 0; a < 3; a++) v *= a == k ? dq(ix[a], x[a]) : q(ix[a], x[a]);
					r.g27[p][n][k] = r6(v);
					if (p < 8) {
						const double y[3] = {x2[p & 1], x2[(p >> 1) & 1], x2[p >> 2]};
						double u = 1.0;
						for (int a = 0; a < 3; a++) u *= a == k ? dq(ix[a], y[a]) : q(ix[a], y[a]);
						r.g8[p][n][k] = r6(u);
					}
				}
			}
			for (int n = 0; n < 8; n++)
				for (int k = 0; k < 3; k++) {
					double v = 1.0;
					for (int a = 0; a < 3; a++) {
						const int b = (n >> a) & 1;
						v *= a == k ? (b ? 0.5 : -0.5) : (b ? (1 + x[a]) / 2 : (1 - x[a]) / 2);
					}
					r.map27[p][n][k] = r6(v);
				}
		}
		return r;
	}();
	return t;
}

// Offsets in the 703-value H27 record (ElementParamsQuadraticHex,
// XPBDFEM/Fem.h:101-111, flattened): qcLo.Ji[p] column-major, qcLo.w[p],
// qcHi.Ji[p], qcHi.w[p], ic.QQ[26], ic.QR[325], volume, surfaceArea.
constexpr int kH27JL = 0, kH27WL = 72, kH27JH = 80, kH27WH = 323, kH27QQ = 350, kH27QR = 376, kH27Vol = 701,
              kH27Area = 702, kH27Rec = 703;

// The corner map's jacobian at point p of the 2x2x2 (np 8) or 3x3x3 rule.
inline M3 h27_map_jacobian(const float P[8][3], int np, int p) {
	const H27Tables& tb = h27_tables();
	M3 J;
	for (int c = 0; c < 3; c++)
		for (int r = 0; r < 3; r++) J.c[c][r] = 0.0f;
	for (int n = 0; n < 8; n++)
		for (int c = 0; c < 3; c++)
			for (int r = 0; r < 3; r++) J.c[c][r] = J.c[c][r] + (np == 8 ? hex_g8(p, n, r) : tb.map27[p][n][r]) * P[n][c];
	return J;
}

// One H27: InitQuadHexFiniteElement (XPBDFEM/Fem.cpp:225-265) with the map
// over the corners is[0, 2, 6, 8, 18, 20, 24, 26] (:274): the mapped
// quadrature on the 2x2x2 and 3x3x3 rules, the prefactored I1 on the 3x3x3
// rule, the volume on the 2x2x2 rule, the surface area, and the masses from
// the normalised mass-matrix diagonal. X: the vertex positions in double.
inline void h27(const double* X, const uint32_t* is, float density, float* o, float m[27]) {
	static const int corner[8] = {0, 2, 6, 8, 18, 20, 24, 26};
	const H27Tables& tb = h27_tables();
	float P[8][3];
	for (int n = 0; n < 8; n++)
		for (int k = 0; k < 3; k++)
			P[n][k] = (float)(X[3 * (size_t)is[corner[n]] + k] - X[3 * (size_t)is[corner[7]] + k]);
	for (int hi = 0; hi < 2; hi++) {
		const int np = hi ? 27 : 8;
		float vsum = 0.0f;
		for (int p = 0; p < np; p++) {
			const M3 J = h27_map_jacobian(P, np, p);
			const float detJ = det3(J);
			const M3 Ji = inverse3(J);
			float* j = o + (hi ? kH27JH : kH27JL) + 9 * p;
			for (int c = 0; c < 3; c++)
				for (int r = 0; r < 3; r++) j[c * 3 + r] = Ji.c[c][r];
			float& w = o[(hi ? kH27WH : kH27WL) + p];
			w = detJ * (hi ? tb.w27[p] : 1.0f);
			vsum += w;
		}
		for (int p = 0; p < np; p++) o[(hi ? kH27WH : kH27WL) + p] /= vsum;
	}
	float* QQ = o + kH27QQ;
	float* QR = o + kH27QR;
	for (int i = 0; i < 26; i++) QQ[i] = 0.0f;
	for (int i = 0; i < 325; i++) QR[i] = 0.0f;
	float vsum = 0.0f;
	for (int p = 0; p < 27; p++) {
		const M3 J = h27_map_jacobian(P, 27, p);
		const M3 Ji = inverse3(J);
		const float w = det3(J) * 1.0f * tb.w27[p];
		float q[26][3];
		for (int i = 0; i < 26; i++)
			for (int r = 0; r < 3; r++) {
				const float row[3] = {Ji.c[0][r], Ji.c[1][r], Ji.c[2][r]};
				q[i][r] = dot3(row, tb.g27[p][i]);
			}
		vsum += w;
		for (int i = 0; i < 26; i++) QQ[i] += w * dot3(q[i], q[i]);
		int head = 0;
		for (int i = 0; i < 26; i++)
			for (int j = i + 1; j < 26; j++) QR[head++] += w * 2.0f * dot3(q[i], q[j]);
	}
	for (int i = 0; i < 26; i++) QQ[i] /= vsum;
	for (int i = 0; i < 325; i++) QR[i] /= vsum;
	float vol = 0.0f;
	for (int p = 0; p < 8; p++) vol += det3(h27_map_jacobian(P, 8, p)) * 1.0f;
	o[kH27Vol] = vol;
	const int faces[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 2, 4, 6}, {1, 3, 5, 7}};
	float area = 0.0f;
	for (int f = 0; f < 6; f++) {
		float a[3], b[3];
		for (int k = 0; k < 3; k++) {
			a[k] = P[faces[f][0]][k] - P[faces[f][3]][k];
			b[k] = P[faces[f][1]][k] - P[faces[f][2]][k];
		}
		const float c[3] = {a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]};
		area += 0.5f * sqrtf(dot3(c, c));
	}
	o[kH27Area] = area;
	float mmd[27], msum = 0.0f;
	for (int n = 0; n < 27; n++) mmd[n] = 0.0f;
	for (int p = 0; p < 27; p++) {
		const float w = o[kH27WH + p];
		for (int n = 0; n < 27; n++) {
			const float Nn = tb.n27[p][n];
			mmd[n] += w * Nn * Nn;
			msum += w * Nn * Nn;
		}
	}
	for (int n = 0; n < 27; n++) m[n] = (mmd[n] / msum) * density * vol;
}

// The Left / Right flags of a vertex (XPBDFEM/Geo.cpp:713-727) from the AABB
// of the node data along x: bit 0 Left, bit 1 Right, bit 4 Pickable.
XFEM_HD uint8_t vertex_flags(float x, float mn, float mx) {
	uint8_t f = 1u << 4;
	const float rel = (x - mn) / (mx - mn);
	if (rel < 0.02f) f |= 1u;
	if (rel > 0.98f) f |= 2u;
	return f;
}

}  // namespace rest

// Morton order of the schedule (vertex ranks and cluster order inside a
// colour), shared by the host and the GPU set-up: integer and float steps
// that give the same result on both and on x86-64 and AArch64.
XFEM_HD uint32_t morton_code(uint32_t x, uint32_t y, uint32_t z) {
	uint32_t c = 0;
	for (int b = 0; b < 10; b++)
		c |= (((x >> b) & 1u) << (3 * b)) | (((y >> b) & 1u) << (3 * b + 1)) | (((z >> b) & 1u) << (3 * b + 2));
	return c;
}

// The curve's frame: the AABB of the node data and one scale for all axes
// (the largest extent, 10 bits per axis).
struct MortonFrame {
	float mn[3] = {0.0f, 0.0f, 0.0f}, mx[3] = {0.0f, 0.0f, 0.0f}, sc[3] = {0.0f, 0.0f, 0.0f};

	XFEM_HD void set_scale() {
		float ext = 0.0f;
		for (int k = 0; k < 3; k++) ext = (mx[k] - mn[k]) > ext ? (mx[k] - mn[k]) : ext;
		for (int k = 0; k < 3; k++) sc[k] = ext > 0.0f ? 1023.0f / ext : 0.0f;
	}

	XFEM_HD uint32_t code(const float* p3) const {
		uint32_t q[3];
		for (int k = 0; k < 3; k++) {
			const float f = (p3[k] - mn[k]) * sc[k];
			const uint32_t u = f > 0.0f ? (uint32_t)f : 0u;
			q[k] = u > 1023u ? 1023u : u;
		}
		return morton_code(q[0], q[1], q[2]);
	}
};

// Sort key of a cluster inside its colour: the Morton code of its centroid
// (the mean of its tets' vertex positions, summed tet by tet in float; it
// sits inside a curve cell, where a corner would sit on a cell boundary and
// flip bits with rounding), or without Morton order its smallest vertex id.
XFEM_HD uint32_t cluster_key(const float* nodes, const uint32_t* tets, const uint32_t* cl_tets, uint32_t nt,
                             uint32_t morton, const MortonFrame& f) {
	if (morton) {
		float c[3] = {0.0f, 0.0f, 0.0f};
		for (uint32_t q = 0; q < nt; q++)
			for (int n = 0; n < 4; n++)
				for (int j = 0; j < 3; j++) c[j] += nodes[3 * (size_t)tets[4 * (size_t)cl_tets[q] + n] + j];
		const float cnt = (float)(4u * nt);
		for (int j = 0; j < 3; j++) c[j] = c[j] / cnt;
		return f.code(c);
	}
	uint32_t key = 0xffffffffu;
	for (uint32_t q = 0; q < nt; q++)
		for (int n = 0; n < 4; n++) {
			const uint32_t v = tets[4 * (size_t)cl_tets[q] + n];
			key = v < key ? v : key;
		}
	return key;
}

}  // namespace xfem
