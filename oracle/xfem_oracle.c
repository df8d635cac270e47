/*
 * xfem_oracle.c — CPU restatement of the reference's small-step XPBD tet
 * substep and of this project's schedule (clusters, colours, Morton order).
 * TEST INFRASTRUCTURE ONLY (see oracle/xfem_oracle.h). Build with
 * -ffp-contract=off (oracle/Makefile) so that float results reproduce the
 * reference bit for bit on x86-64 and on AArch64.
 */
#include "xfem_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- one-rings (integer; shared by both instantiations) ------------------ */
/* The one-ring of every vertex as OneRingConstructor builds it
 * (XPBDFEM/Connectivity.h:114-160), filled as GeoLinear3d::Init fills it
 * (XPBDFEM/Geo.cpp:747-757): the vertex's elements (tets, or on a hex mesh
 * hexes) in increasing id (the order Connectivity3d::Init lists them,
 * XPBDFEM/Connectivity.cpp:437-439); the ring's nodes, the vertex first,
 * then each element's vertices in order of first appearance; and for each
 * element corner its node index. */
typedef struct {
	uint32_t* tet_off;  /* nv + 1, into tet_list */
	uint32_t* tet_list; /* element ids */
	uint32_t* node_off; /* nv + 1, into nodes */
	uint32_t* nodes;
	uint16_t* corner;   /* npe per tet_list entry */
} orc_rings;

static void rings_free(orc_rings* r) {
	free(r->tet_off);
	free(r->tet_list);
	free(r->node_off);
	free(r->nodes);
	free(r->corner);
}

/* elems: npe vertex ids per element (4 for tets, 8 for hexes), ne elements. */
static int rings_build(const uint32_t* elems, uint32_t npe, uint32_t ne, uint32_t nv, orc_rings* r) {
	memset(r, 0, sizeof(*r));
	const size_t ninc = (size_t)npe * ne;
	r->tet_off = (uint32_t*)calloc((size_t)nv + 1, 4);
	r->node_off = (uint32_t*)calloc((size_t)nv + 1, 4);
	r->tet_list = (uint32_t*)malloc(4 * (ninc ? ninc : 1));
	r->corner = (uint16_t*)malloc(2 * (ninc ? npe * ninc : 1));
	r->nodes = (uint32_t*)malloc(4 * (npe * ninc + nv + 1));
	if (!r->tet_off || !r->node_off || !r->tet_list || !r->corner || !r->nodes) return -1;
	for (size_t i = 0; i < ninc; i++) r->tet_off[elems[i] + 1]++;
	for (uint32_t v = 0; v < nv; v++) r->tet_off[v + 1] += r->tet_off[v];
	uint32_t* fill = (uint32_t*)malloc(4 * ((size_t)nv + 1));
	if (!fill) return -1;
	memcpy(fill, r->tet_off, 4 * (size_t)nv);
	for (uint32_t t = 0; t < ne; t++)
		for (uint32_t n = 0; n < npe; n++) r->tet_list[fill[elems[(size_t)npe * t + n]]++] = t;
	free(fill);
	uint32_t head = 0;
	for (uint32_t v = 0; v < nv; v++) {
		r->node_off[v] = head;
		uint32_t* nodes = r->nodes + head;
		uint32_t cnt = 1;
		nodes[0] = v;
		for (uint32_t j = r->tet_off[v]; j < r->tet_off[v + 1]; j++) {
			const uint32_t* tv = elems + (size_t)npe * r->tet_list[j];
			for (uint32_t n = 0; n < npe; n++) {
				uint32_t k = cnt;
				for (uint32_t q = 0; q < cnt; q++)
					if (nodes[q] == tv[n]) {
						k = q;
						break;
					}
				if (k == cnt) nodes[cnt++] = tv[n];
				r->corner[(size_t)npe * j + n] = (uint16_t)k;
			}
		}
		head += cnt;
	}
	r->node_off[nv] = head;
	return 0;
}

/* ---- linear-hex tables ------------------------------------------------------ */
/* The reference tabulates the 8-node hex's shape functions and their
 * gradients at the 2x2x2 Gauss points (XPBDFEM/Fem.cpp:40, :69) and the
 * gradients at the centre (:68), printed to six decimals. Nodes and points
 * are numbered i + 2j + 4k, with the sign 2 bit - 1 on each axis. Every
 * entry is one of a few printed magnitudes, fixed by how many axes the node
 * and the point agree on, so the tables are built here from those literals.
 * The literals must be the reference's own, not the exact Gauss values: the
 * rounding shows in every rest state. */
static const float hex_n_lit[4] = {0.009437f, 0.035221f, 0.131446f, 0.490562f}; /* by axes agreeing */
static const float hex_g_lit[3] = {0.022329f, 0.083333f, 0.311004f};           /* by other axes agreeing */

/* ShapeFunctions<Hex, 8, 8>[p][n] */
static float hex_n8(int p, int n) {
	int agree = 0;
	for (int a = 0; a < 3; a++) agree += !(((p ^ n) >> a) & 1);
	return hex_n_lit[agree];
}

/* ShapeFunctionGradients<Hex, 8, 8>[p][n][k]: the sign of node n on axis k */
static float hex_g8(int p, int n, int k) {
	int agree = 0;
	for (int a = 0; a < 3; a++)
		if (a != k) agree += !(((p ^ n) >> a) & 1);
	return ((n >> k) & 1) ? hex_g_lit[agree] : -hex_g_lit[agree];
}

/* ShapeFunctionGradients<Hex, 8, 1>[0][n][k] */
static float hex_g1(int n, int k) { return ((n >> k) & 1) ? 0.125f : -0.125f; }

void orc_hex_tables(float* n8, float* g8, float* g1) {
	for (int p = 0; p < 8; p++)
		for (int n = 0; n < 8; n++) {
			n8[8 * p + n] = hex_n8(p, n);
			for (int k = 0; k < 3; k++) g8[24 * p + 3 * n + k] = hex_g8(p, n, k);
		}
	for (int n = 0; n < 8; n++)
		for (int k = 0; k < 3; k++) g1[3 * n + k] = hex_g1(n, k);
}

/* ---- quadratic-tet (T10) tables -------------------------------------------- */
/* The 10-node tet's shape-function gradients at the 4-point rule (the solve,
 * XPBDFEM/Fem.cpp:60) and the 10-point rule (the prefactored coefficients,
 * :61), and the weights (:11-12), printed by the reference to six decimals.
 * Nodes: corners 0-3 with barycentric L0 = x, L1 = y, L2 = z, L3 = 1 - x - y
 * - z, then the edges (0,1), (0,2), (0,3), (1,2), (1,3), (2,3). A corner's
 * gradient is (4 L_c - 1) grad L_c, an edge's 4 (L_b grad L_a + L_a grad
 * L_b). Point p of the 4-point rule has L_p = a4 and the others b4; the
 * 10-point rule's points 0-3 have L_p = a10 (others b10) and points 4-9, one
 * per edge in node order, L = c10 on the edge's two corners (d10 on the
 * others). Each entry is the signed printed magnitude nearest to its value,
 * so the tables are built from those literals. */
static const double t10_mag4[5] = {0.447214, 0.552786, 1.341641, 1.788854, 2.341641};
static const double t10_mag10[9] = {0.295340, 0.375023, 0.624977, 0.704660, 1.249955,
                                    1.624977, 2.113981, 2.818642, 3.113981};
static const int t10_edge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

/* barycentric coordinate c of point p (rule of np points) */
static double t10_L(int np, int p, int c) {
	if (np == 4) return p == c ? (1.341641 + 1.0) / 4.0 : (1.0 - 0.447214) / 4.0;
	if (p < 4) return p == c ? (2.113981 + 1.0) / 4.0 : (1.0 - 0.704660) / 4.0;
	const int* e = t10_edge[p - 4];
	return (c == e[0] || c == e[1]) ? (0.624977 + 1.0) / 4.0 : (1.0 - 0.624977) / 4.0;
}

static float t10_snap(double v, const double* mag, int nm) {
	if (fabs(v) < 1e-3) return 0.0f;
	int best = 0;
	for (int i = 1; i < nm; i++)
		if (fabs(fabs(v) - mag[i]) < fabs(fabs(v) - mag[best])) best = i;
	return v < 0 ? -(float)mag[best] : (float)mag[best];
}

/* ShapeFunctionGradients<Tet, 10, np>[p][n][k], np = 4 or 10 */
static float t10_g(int np, int p, int n, int k) {
	static const double gl[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, -1, -1}};
	double v;
	if (n < 4) {
		v = (4.0 * t10_L(np, p, n) - 1.0) * gl[n][k];
	} else {
		const int a = t10_edge[n - 4][0], b = t10_edge[n - 4][1];
		v = 4.0 * (t10_L(np, p, b) * gl[a][k] + t10_L(np, p, a) * gl[b][k]);
	}
	return np == 4 ? t10_snap(v, t10_mag4, 5) : t10_snap(v, t10_mag10, 9);
}

/* QuadratureWeights<Tet, np>[p] */
static float t10_w(int np, int p) { return np == 4 ? 0.250000f : p < 4 ? 0.047633f : 0.134911f; }

void orc_t10_tables(float* g4, float* g10, float* w10) {
	for (int p = 0; p < 4; p++)
		for (int n = 0; n < 10; n++)
			for (int k = 0; k < 3; k++) g4[30 * p + 3 * n + k] = t10_g(4, p, n, k);
	for (int p = 0; p < 10; p++) {
		w10[p] = t10_w(10, p);
		for (int n = 0; n < 10; n++)
			for (int k = 0; k < 3; k++) g10[30 * p + 3 * n + k] = t10_g(10, p, n, k);
	}
}

/* The 27-node hex's tables (XPBDFEM/Fem.cpp:16-18, 41-44, 70-73). Nodes and
 * points are numbered i + 3j + 9k (i + 2j + 4k on the 2x2x2 rule) on the
 * 1-D nodes -1, 0, 1; the 1-D shape functions are x (x - 1) / 2, 1 - x^2 and
 * x (x + 1) / 2. The reference's generator evaluated them in double at the
 * 1-D Gauss points and weights as printed to six decimals (0.774597 and 0
 * on the 3-point rule with weights 0.555556 and 0.888889; 0.577350 on the
 * 2-point rule) and printed each entry to six decimals: that method gives
 * every printed entry, where the exact Gauss values miss some. */
static const double h27_x3[3] = {-0.774597, 0.0, 0.774597};
static const double h27_x2[2] = {-0.577350, 0.577350};
static const double h27_w3[3] = {0.555556, 0.888889, 0.555556};

static float h27_round6(double v) { return (float)(nearbyint(v * 1e6) / 1e6); }

static double h27_q(int i, double x) { return i == 0 ? x * (x - 1) / 2 : i == 1 ? (1 - x) * (1 + x) : x * (x + 1) / 2; }
static double h27_dq(int i, double x) { return i == 0 ? x - 0.5 : i == 1 ? -2 * x : x + 0.5; }

/* the coordinates of point p of the np-point rule (np = 8 or 27) */
static void h27_point(int np, int p, double x[3]) {
	if (np == 27) {
		x[0] = h27_x3[p % 3], x[1] = h27_x3[(p / 3) % 3], x[2] = h27_x3[p / 9];
	} else {
		x[0] = h27_x2[p & 1], x[1] = h27_x2[(p >> 1) & 1], x[2] = h27_x2[p >> 2];
	}
}

/* ShapeFunctionGradients<Hex, 27, np>[p][n][k] */
static float h27_g(int np, int p, int n, int k) {
	double x[3];
	h27_point(np, p, x);
	const int ix[3] = {n % 3, (n / 3) % 3, n / 9};
	double v = 1.0;
	for (int a = 0; a < 3; a++) v *= a == k ? h27_dq(ix[a], x[a]) : h27_q(ix[a], x[a]);
	return h27_round6(v);
}

/* ShapeFunctions<Hex, 27, 27>[p][n] */
static float h27_n(int p, int n) {
	double x[3];
	h27_point(27, p, x);
	return h27_round6(h27_q(n % 3, x[0]) * h27_q((n / 3) % 3, x[1]) * h27_q(n / 9, x[2]));
}

/* ShapeFunctionGradients<Hex, 8, 27>[p][n][k]: the corner map at the 3x3x3 points */
static float h27_map_g(int p, int n, int k) {
	double x[3];
	h27_point(27, p, x);
	double v = 1.0;
	for (int a = 0; a < 3; a++) {
		const int b = (n >> a) & 1;
		v *= a == k ? (b ? 0.5 : -0.5) : (b ? (1 + x[a]) / 2 : (1 - x[a]) / 2);
	}
	return h27_round6(v);
}

/* QuadratureWeights<Hex, 27>[p] */
static float h27_w(int p) { return h27_round6(h27_w3[p % 3] * h27_w3[(p / 3) % 3] * h27_w3[p / 9]); }

void orc_h27_tables(float* g8, float* g27, float* n27, float* map27, float* w27) {
	for (int p = 0; p < 27; p++) {
		w27[p] = h27_w(p);
		for (int n = 0; n < 27; n++) {
			n27[27 * p + n] = h27_n(p, n);
			for (int k = 0; k < 3; k++) {
				g27[81 * p + 3 * n + k] = h27_g(27, p, n, k);
				if (p < 8) g8[81 * p + 3 * n + k] = h27_g(8, p, n, k);
			}
		}
		for (int n = 0; n < 8; n++)
			for (int k = 0; k < 3; k++) map27[24 * p + 3 * n + k] = h27_map_g(p, n, k);
	}
}

/* ---- float instantiation (reference semantics) ---------------------------- */
#define R float
#define SFX _f
#define SQRT sqrtf
#define FMAX fmaxf
#define FMIN fminf
#define EPS22 1.0e-22f
#define EPS8 0.00000001f
#define EPS4 0.0001f
#include "xfem_oracle_real.inc"
#include "xfem_oracle_hex.inc"
#include "xfem_oracle_t10.inc"
#include "xfem_oracle_h27.inc"
#include "xfem_oracle_mixed.inc"
#undef R
#undef SFX
#undef SQRT
#undef FMAX
#undef FMIN
#undef EPS22
#undef EPS8
#undef EPS4

/* ---- double instantiation (FP64 run of the same method) ------------------- */
#define R double
#define SFX _d
#define SQRT sqrt
#define FMAX fmax
#define FMIN fmin
#define EPS22 1.0e-22
#define EPS8 1.0e-8
#define EPS4 1.0e-4
#include "xfem_oracle_real.inc"
#include "xfem_oracle_hex.inc"
#include "xfem_oracle_t10.inc"
#include "xfem_oracle_h27.inc"
#include "xfem_oracle_mixed.inc"
#undef R
#undef SFX
#undef SQRT
#undef FMAX
#undef FMIN
#undef EPS22
#undef EPS8
#undef EPS4

/* ---- mesh ------------------------------------------------------------------ */
/* The vertices of GenerateHexBlock (XPBDFEM/MeshGen.cpp:156-186). */
static void block_nodes(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, float wonkiness,
                        float* nodes) {
	float sc[3] = {sx, sy, sz};
	float mn[3] = {sx * (-0.5f * (float)W), sy * (-0.5f * (float)H), sz * (-0.5f * (float)D)};
	uint32_t rs = 1;
	for (uint32_t z = 0; z < D + 1; z++) {
		uint32_t ze = (z == 0 || z == D);
		for (uint32_t y = 0; y < H + 1; y++) {
			uint32_t ye = (y == 0 || y == H);
			for (uint32_t x = 0; x < W + 1; x++) {
				uint32_t xe = (x == 0 || x == W);
				uint32_t i = x + y * (W + 1) + z * (W + 1) * (H + 1);
				/* RandF is drawn for interior coordinates only. The reference draws
				 * inside one vec3(...) argument list, whose evaluation order C++
				 * leaves unspecified; g++ (and MSVC) evaluate right to left, so z
				 * is drawn first. The golden vectors come from g++. */
				float r[3] = {0.0f, 0.0f, 0.0f};
				uint32_t edge[3] = {xe, ye, ze};
				for (int k = 2; k >= 0; k--) {
					if (!edge[k]) {
						rs = (uint32_t)(((uint64_t)rs * 48271u) % 0x7fffffffu);
						r[k] = (float)rs * 9.3132258e-10f - 1.0f;
					}
				}
				float c[3] = {(float)x, (float)y, (float)z};
				for (int k = 0; k < 3; k++) {
					float wig = wonkiness * r[k];
					nodes[3 * i + k] = mn[k] + sc[k] * (c[k] + 0.5f * wig);
				}
			}
		}
	}
}

/* The 8 vertices of the block's cell (x, y, z), uniform (pattern 0) or
 * mirrored in every other cell (XPBDFEM/MeshGen.cpp:189-214). */
static void block_cell(uint32_t W, uint32_t H, uint32_t pattern, uint32_t x, uint32_t y, uint32_t z, uint32_t ih[8]) {
	for (uint32_t k = 0; k < 2; k++)
		for (uint32_t j = 0; j < 2; j++)
			for (uint32_t i = 0; i < 2; i++) {
				if (pattern == 0) {
					ih[i + j * 2 + k * 4] = (x + i) + (y + j) * (W + 1) + (z + k) * (W + 1) * (H + 1);
				} else {
					uint32_t xx = x % 2 == 0 ? i : (1 - i);
					uint32_t yy = y % 2 == 0 ? j : (1 - j);
					uint32_t zz = z % 2 == 0 ? k : (1 - k);
					uint32_t hi = i + j * 2 + k * 4;
					if ((x + y + z) % 2 == 1) hi = 7 - hi;
					ih[hi] = (x + xx) + (y + yy) * (W + 1) + (z + zz) * (W + 1) * (H + 1);
				}
			}
}

/* GenerateHexBlock (XPBDFEM/MeshGen.cpp:156-221). */
void orc_gen_hex_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                       float wonkiness, float* nodes, uint32_t* idx) {
	block_nodes(W, H, D, sx, sy, sz, wonkiness, nodes);
	uint32_t ie = 0;
	for (uint32_t z = 0; z < D; z++)
		for (uint32_t y = 0; y < H; y++)
			for (uint32_t x = 0; x < W; x++) {
				uint32_t* o = idx + 9 * (size_t)ie++;
				o[0] = 8;
				block_cell(W, H, pattern, x, y, z, o + 1);
			}
}

/* The Right lock's targets (XPBDFEM/Geo.cpp:327): origin + m * vec3(X0),
 * m column-major, each row dotted left to right in float. */
void orc_right_targets(uint32_t nv, const float* nodes, const float m[9], const float origin[3], double* out) {
	for (uint32_t i = 0; i < nv; i++) {
		const float x = nodes[3 * (size_t)i], y = nodes[3 * (size_t)i + 1], z = nodes[3 * (size_t)i + 2];
		for (int k = 0; k < 3; k++) {
			const float r = m[k] * x + m[3 + k] * y + m[6 + k] * z;
			out[3 * (size_t)i + k] = (double)(origin[k] + r);
		}
	}
}

/* GenerateHexBlock + GenerateTetBlock (XPBDFEM/MeshGen.cpp:156-244). */
void orc_gen_tet_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                       float wonkiness, float* nodes, uint32_t* idx) {
	block_nodes(W, H, D, sx, sy, sz, wonkiness, nodes);
	uint32_t ie = 0;
	static const uint32_t split[6][4] = {{0, 1, 5, 7}, {0, 7, 3, 1}, {0, 2, 3, 7}, {0, 7, 6, 2}, {0, 4, 6, 7}, {0, 7, 5, 4}};
	for (uint32_t z = 0; z < D; z++)
		for (uint32_t y = 0; y < H; y++)
			for (uint32_t x = 0; x < W; x++) {
				uint32_t ih[8];
				block_cell(W, H, pattern, x, y, z, ih);
				for (int t = 0; t < 6; t++) {
					uint32_t* o = idx + 30 * (size_t)ie + 5 * t;
					o[0] = 4;
					for (int n = 0; n < 4; n++) o[1 + n] = ih[split[t][n]];
				}
				++ie;
			}
}

/* Hex-only tagged stream (XPBDFEM/Connectivity.cpp:251-265): tag 8 = hex;
 * anything else is an error here. With hexes == NULL only counts. */
int orc_parse_hexes(const uint32_t* idx, uint32_t idx_count, uint32_t* hexes, uint32_t* hex_count,
                    uint32_t* vert_count) {
	uint32_t nh = 0, mx = 0;
	for (uint32_t i = 0; i < idx_count; i++) {
		if (idx[i] != 8u || (uint64_t)i + 8u >= (uint64_t)idx_count) return -1;
		for (int n = 0; n < 8; n++) {
			uint32_t v = idx[i + 1 + n];
			if (v > mx) mx = v;
			if (hexes) hexes[8 * (size_t)nh + n] = v;
		}
		nh++;
		i += 8;
	}
	*hex_count = nh;
	*vert_count = nh ? mx + 1 : 0;
	return 0;
}

/* A tagged stream of tets (tag 4) and hexes (tag 8) in any mix
 * (Connectivity3d::Init, XPBDFEM/Connectivity.cpp:251-265): each kind in
 * stream order; another tag or a truncated record is an error. With
 * tets == NULL or hexes == NULL only counts. */
int orc_parse_mixed(const uint32_t* idx, uint32_t idx_count, uint32_t* tets, uint32_t* tet_count, uint32_t* hexes,
                    uint32_t* hex_count, uint32_t* vert_count) {
	uint32_t nt = 0, nh = 0, mx = 0, any = 0;
	for (uint32_t i = 0; i < idx_count; i++) {
		const uint32_t tag = idx[i];
		if ((tag != 4u && tag != 8u) || (uint64_t)i + tag >= (uint64_t)idx_count) return -1;
		for (uint32_t n = 0; n < tag; n++) {
			uint32_t v = idx[i + 1 + n];
			if (v > mx) mx = v;
			if (tag == 4u && tets) tets[4 * (size_t)nt + n] = v;
			if (tag == 8u && hexes) hexes[8 * (size_t)nh + n] = v;
		}
		if (tag == 4u) nt++;
		else nh++;
		any = 1;
		i += tag;
	}
	*tet_count = nt;
	*hex_count = nh;
	*vert_count = any ? mx + 1 : 0;
	return 0;
}

int orc_parse_tets(const uint32_t* idx, uint32_t idx_count, uint32_t* tets, uint32_t* tet_count, uint32_t* vert_count) {
	/* Connectivity3d::Init (XPBDFEM/Connectivity.cpp:251-265): tag 4 = tet,
	 * 8 = hex (not handled by this path), anything else is an error. */
	uint32_t nt = 0, mx = 0;
	for (uint32_t i = 0; i < idx_count; i++) {
		if (idx[i] != 4u || (uint64_t)i + 4u >= (uint64_t)idx_count) return -1;
		for (int n = 0; n < 4; n++) {
			uint32_t v = idx[i + 1 + n];
			if (v > mx) mx = v;
			if (tets) tets[4 * (size_t)nt + n] = v;
		}
		nt++;
		i += 4;
	}
	*tet_count = nt;
	*vert_count = nt ? mx + 1 : 0;
	return 0;
}

void orc_minstd_order(uint32_t nt, uint32_t* order) {
	for (uint32_t i = 0; i < nt; i++) order[i] = i;
	uint32_t rs = 1;
	for (uint32_t i = 0; i < nt; i++) {
		rs = (uint32_t)(((uint64_t)rs * 48271u) % 0x7fffffffu);
		uint32_t j = rs % nt;
		uint32_t c = order[i];
		order[i] = order[j];
		order[j] = c;
	}
}

float orc_volume_f(const double* X, uint32_t nt, const uint32_t* tets) {
	float v = 0.0f;
	for (uint32_t t = 0; t < nt; t++) v += tet_volume_f(X, tets + 4 * (size_t)t);
	return v;
}

double orc_volume_d(const double* X, uint32_t nt, const uint32_t* tets) {
	double v = 0.0;
	for (uint32_t t = 0; t < nt; t++) v += tet_volume_d(X, tets + 4 * (size_t)t);
	return v;
}

/* ---- threaded coloured run (CPU baseline) --------------------------------- */
typedef struct {
	orc_run_f* r;
	const uint32_t* order;
	const uint32_t* cb;
	uint32_t ncol, nsub, tid, nth;
	pthread_barrier_t* bar;
	int rc;
} orc_worker;

static void* orc_worker_main(void* arg) {
	orc_worker* k = (orc_worker*)arg;
	orc_run_f* r = k->r;
	uint32_t vb = (uint32_t)((uint64_t)r->nv * k->tid / k->nth), ve = (uint32_t)((uint64_t)r->nv * (k->tid + 1) / k->nth);
	for (uint32_t s = 0; s < k->nsub; s++) {
		predict_f(r, vb, ve);
		pthread_barrier_wait(k->bar);
		for (uint32_t c = 0; c < k->ncol; c++) {
			uint32_t b = k->cb[c], e = k->cb[c + 1], n = e - b;
			uint32_t tb = b + (uint32_t)((uint64_t)n * k->tid / k->nth), te = b + (uint32_t)((uint64_t)n * (k->tid + 1) / k->nth);
			for (uint32_t i = tb; i < te; i++)
				if (solve_one_f(r, k->order[i])) k->rc = -1;
			pthread_barrier_wait(k->bar);
		}
		finalize_f(r, vb, ve);
		pthread_barrier_wait(k->bar);
	}
	return NULL;
}

int orc_substeps_threaded_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nt,
                            const uint32_t* tets, const float* ep, const float* tet_mu, const uint32_t* order,
                            const uint32_t* colour_begin, uint32_t ncolours, uint32_t nsub, const orc_params* p,
                            uint32_t threads) {
	/* the undamped method without volume passes only: those run in orc_substeps_f */
	if (p->damping > 0.0f || p->pbd_damping > 0.0f || p->volume_passes) return -1;
	if (threads < 1) threads = 1;
	if (threads > 256) threads = 256;
	double* O = (double*)malloc(sizeof(double) * 3 * (size_t)(nv ? nv : 1));
	if (!O) return -1;
	orc_run_f r = {nv, nt, X, V, O, w, lock_mask, tets, ep, tet_mu, p, NULL, NULL};
	pthread_barrier_t bar;
	pthread_barrier_init(&bar, NULL, threads);
	orc_worker wk[256];
	pthread_t th[256];
	for (uint32_t t = 0; t < threads; t++) {
		wk[t] = (orc_worker){&r, order, colour_begin, ncolours, nsub, t, threads, &bar, 0};
		if (t) pthread_create(&th[t], NULL, orc_worker_main, &wk[t]);
	}
	orc_worker_main(&wk[0]);
	int rc = wk[0].rc;
	for (uint32_t t = 1; t < threads; t++) {
		pthread_join(th[t], NULL);
		if (wk[t].rc) rc = wk[t].rc;
	}
	pthread_barrier_destroy(&bar);
	free(O);
	return rc;
}

/* ---- schedule restatement --------------------------------------------------- */
#define ORC_MAXV 8u
#define ORC_MAXT 8u
#define ORC_MAXCOL 4096u

typedef struct {
	uint32_t* off; /* nv + 1 */
	uint32_t* lst; /* 4 nt */
} orc_csr;

static int csr_build(const uint32_t* tets, uint32_t nt, uint32_t nv, orc_csr* c) {
	c->off = (uint32_t*)calloc((size_t)nv + 1, 4);
	c->lst = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)(nt ? nt : 1));
	if (!c->off || !c->lst) return -1;
	for (size_t i = 0; i < 4 * (size_t)nt; i++) c->off[tets[i] + 1]++;
	for (uint32_t v = 0; v < nv; v++) c->off[v + 1] += c->off[v];
	uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)nv + 1));
	if (!fill) return -1;
	memcpy(fill, c->off, sizeof(uint32_t) * ((size_t)nv + 1));
	for (uint32_t t = 0; t < nt; t++)
		for (int n = 0; n < 4; n++) c->lst[fill[tets[4 * (size_t)t + n]]++] = t;
	free(fill);
	return 0;
}

static int tet_has(const uint32_t* tv, uint32_t v) { return tv[0] == v || tv[1] == v || tv[2] == v || tv[3] == v; }

static uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
	uint32_t c = 0;
	for (int b = 0; b < 10; b++)
		c |= (((x >> b) & 1u) << (3 * b)) | (((y >> b) & 1u) << (3 * b + 1)) | (((z >> b) & 1u) << (3 * b + 2));
	return c;
}

static uint32_t orc_quantise(const float* p, const float* mn, const float* sc) {
	uint32_t q[3];
	for (int k = 0; k < 3; k++) {
		float f = (p[k] - mn[k]) * sc[k];
		uint32_t u = f > 0.0f ? (uint32_t)f : 0u;
		q[k] = u > 1023u ? 1023u : u;
	}
	return morton3(q[0], q[1], q[2]);
}

typedef struct { uint64_t key; uint32_t id; } orc_kv;
static int kv_cmp(const void* a, const void* b) {
	const orc_kv* x = (const orc_kv*)a;
	const orc_kv* y = (const orc_kv*)b;
	if (x->key != y->key) return x->key < y->key ? -1 : 1;
	return x->id < y->id ? -1 : (x->id > y->id);
}

/* Vertex ranks: (Morton code of the rest position over the AABB with one
 * scale, the largest extent; vertex id), or the identity. mn, sc: the frame. */
static int orc_vertex_ranks(const float* nodes, uint32_t nv, uint32_t morton, uint32_t* vert_rank, float mn[3],
                            float sc[3]) {
	float mx[3] = {-INFINITY, -INFINITY, -INFINITY};
	if (!morton) {
		for (uint32_t v = 0; v < nv; v++) vert_rank[v] = v;
		return 0;
	}
	for (uint32_t v = 0; v < nv; v++)
		for (int k = 0; k < 3; k++) {
			float x = nodes[3 * (size_t)v + k];
			if (x < mn[k]) mn[k] = x;
			if (x > mx[k]) mx[k] = x;
		}
	float ext = 0.0f;
	for (int k = 0; k < 3; k++) ext = (mx[k] - mn[k]) > ext ? (mx[k] - mn[k]) : ext;
	for (int k = 0; k < 3; k++) sc[k] = ext > 0.0f ? 1023.0f / ext : 0.0f;
	orc_kv* kv = (orc_kv*)malloc(sizeof(orc_kv) * (nv ? nv : 1));
	if (!kv) return -1;
	for (uint32_t v = 0; v < nv; v++) {
		kv[v].key = orc_quantise(nodes + 3 * (size_t)v, mn, sc);
		kv[v].id = v;
	}
	qsort(kv, nv, sizeof(orc_kv), kv_cmp);
	for (uint32_t i = 0; i < nv; i++) vert_rank[kv[i].id] = i;
	free(kv);
	return 0;
}

int orc_ring_schedule(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, uint32_t morton,
                      uint32_t* vorder, uint32_t* colour_begin, uint32_t* ncolours) {
	return orc_ring_schedule_elems(nodes, nv, tets, 4, nt, morton, vorder, colour_begin, ncolours);
}

int orc_ring_schedule_elems(const float* nodes, uint32_t nv, const uint32_t* elems, uint32_t npe, uint32_t ne,
                            uint32_t morton, uint32_t* vorder, uint32_t* colour_begin, uint32_t* ncolours) {
	return orc_ring_schedule_centres(nodes, nv, elems, npe, ne, nv, morton, vorder, colour_begin, ncolours);
}

/* The rings of the first `ncentre` vertices only (GeoQuadratic3d builds
 * rings for the mesh's own vertices, not for the added nodes): colouring in
 * id order over those rings, then (colour, Morton rank among all nv
 * vertices); vorder holds ncentre ids. */
int orc_ring_schedule_centres(const float* nodes, uint32_t nv, const uint32_t* elems, uint32_t npe, uint32_t ne,
                              uint32_t ncentre, uint32_t morton, uint32_t* vorder, uint32_t* colour_begin,
                              uint32_t* ncolours) {
	orc_rings rg;
	if (rings_build(elems, npe, ne, nv, &rg)) {
		rings_free(&rg);
		return -1;
	}
	/* the vertices whose ring holds each node */
	const uint32_t nent = rg.node_off[ncentre];
	uint32_t* ho = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* hl = (uint32_t*)malloc(4 * (size_t)(nent ? nent : 1));
	uint32_t* colour = (uint32_t*)malloc(4 * (size_t)(nv ? nv : 1));
	uint32_t* mark = (uint32_t*)malloc(4 * (size_t)ORC_MAXCOL);
	uint32_t* rank = (uint32_t*)malloc(4 * (size_t)(nv ? nv : 1));
	orc_kv* kv = (orc_kv*)malloc(sizeof(orc_kv) * (nv ? nv : 1));
	int rc = -1;
	if (!ho || !hl || !colour || !mark || !rank || !kv) goto done;
	for (uint32_t i = 0; i < nent; i++) ho[rg.nodes[i] + 1]++;
	for (uint32_t v = 0; v < nv; v++) ho[v + 1] += ho[v];
	{
		uint32_t* f = (uint32_t*)malloc(4 * ((size_t)nv + 1));
		if (!f) goto done;
		memcpy(f, ho, 4 * (size_t)nv);
		for (uint32_t v = 0; v < ncentre; v++)
			for (uint32_t i = rg.node_off[v]; i < rg.node_off[v + 1]; i++) hl[f[rg.nodes[i]]++] = v;
		free(f);
	}
	/* greedy colouring in id order: rings of one colour share no node */
	uint32_t ncol = 0;
	for (uint32_t c = 0; c < ORC_MAXCOL; c++) mark[c] = 0xffffffffu;
	for (uint32_t u = 0; u < ncentre; u++) {
		for (uint32_t i = rg.node_off[u]; i < rg.node_off[u + 1]; i++) {
			const uint32_t x = rg.nodes[i];
			for (uint32_t j = ho[x]; j < ho[x + 1]; j++)
				if (hl[j] < u) mark[colour[hl[j]]] = u;
		}
		uint32_t c = 0;
		while (c < ORC_MAXCOL && mark[c] == u) c++;
		if (c == ORC_MAXCOL) goto done;
		colour[u] = c;
		if (c + 1 > ncol) ncol = c + 1;
	}
	{
		float mn[3] = {INFINITY, INFINITY, INFINITY}, sc[3] = {0.0f, 0.0f, 0.0f};
		if (orc_vertex_ranks(nodes, nv, morton, rank, mn, sc)) goto done;
	}
	for (uint32_t v = 0; v < ncentre; v++) {
		kv[v].key = ((uint64_t)colour[v] << 32) | rank[v];
		kv[v].id = v;
	}
	qsort(kv, ncentre, sizeof(orc_kv), kv_cmp);
	for (uint32_t c = 0; c <= ncol; c++) colour_begin[c] = 0;
	for (uint32_t i = 0; i < ncentre; i++) {
		vorder[i] = kv[i].id;
		colour_begin[colour[kv[i].id] + 1]++;
	}
	for (uint32_t c = 0; c < ncol; c++) colour_begin[c + 1] += colour_begin[c];
	*ncolours = ncol;
	rc = 0;
done:
	free(ho);
	free(hl);
	free(colour);
	free(mark);
	free(rank);
	free(kv);
	rings_free(&rg);
	return rc;
}

/* Elements of `per` vertices coloured greedily in id order (each takes the
 * smallest colour, of ORC_MAXCOL, that no earlier element sharing one of its
 * vertices holds), then ordered inside a colour by (Morton code of the
 * centroid of their vertices, id). */
static int elem_schedule(const float* nodes, uint32_t nv, const uint32_t* elems, uint32_t nh, uint32_t per,
                         uint32_t morton, uint32_t* vert_rank, uint32_t* hex_order, uint32_t* colour_begin,
                         uint32_t* ncolours) {
	uint32_t* off = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* lst = (uint32_t*)malloc(4 * (size_t)(nh ? per * nh : 1));
	uint32_t* mark = (uint32_t*)malloc(4 * (size_t)ORC_MAXCOL);
	uint32_t* colour = (uint32_t*)malloc(4 * (size_t)(nh ? nh : 1));
	orc_kv* kv = (orc_kv*)malloc(sizeof(orc_kv) * (nh ? nh : 1));
	int rc = -1;
	uint32_t ncol = 0;
	float mn[3] = {INFINITY, INFINITY, INFINITY}, sc[3] = {0.0f, 0.0f, 0.0f};
	if (!off || !lst || !mark || !colour || !kv) goto done;
	for (size_t i = 0; i < (size_t)per * nh; i++) off[elems[i] + 1]++;
	for (uint32_t v = 0; v < nv; v++) off[v + 1] += off[v];
	{
		uint32_t* fill = (uint32_t*)malloc(4 * ((size_t)nv + 1));
		if (!fill) goto done;
		memcpy(fill, off, 4 * (size_t)nv);
		for (uint32_t h = 0; h < nh; h++)
			for (uint32_t n = 0; n < per; n++) lst[fill[elems[per * (size_t)h + n]]++] = h;
		free(fill);
	}
	for (uint32_t c = 0; c < ORC_MAXCOL; c++) mark[c] = 0xffffffffu;
	for (uint32_t h = 0; h < nh; h++) {
		for (uint32_t n = 0; n < per; n++) {
			const uint32_t v = elems[per * (size_t)h + n];
			for (uint32_t i = off[v]; i < off[v + 1]; i++)
				if (lst[i] < h) mark[colour[lst[i]]] = h;
		}
		uint32_t c = 0;
		while (c < ORC_MAXCOL && mark[c] == h) c++;
		if (c == ORC_MAXCOL) goto done;
		colour[h] = c;
		if (c + 1 > ncol) ncol = c + 1;
	}
	if (orc_vertex_ranks(nodes, nv, morton, vert_rank, mn, sc)) goto done;
	for (uint32_t h = 0; h < nh; h++) {
		uint32_t key = h;
		if (morton) {
			float c[3] = {0.0f, 0.0f, 0.0f};
			for (uint32_t n = 0; n < per; n++)
				for (int j = 0; j < 3; j++) c[j] += nodes[3 * (size_t)elems[per * (size_t)h + n] + j];
			for (int j = 0; j < 3; j++) c[j] = c[j] / (float)per;
			key = orc_quantise(c, mn, sc);
		}
		kv[h].key = ((uint64_t)colour[h] << 32) | key;
		kv[h].id = h;
	}
	qsort(kv, nh, sizeof(orc_kv), kv_cmp);
	for (uint32_t c = 0; c <= ncol; c++) colour_begin[c] = 0;
	for (uint32_t i = 0; i < nh; i++) {
		hex_order[i] = kv[i].id;
		colour_begin[colour[kv[i].id] + 1]++;
	}
	for (uint32_t c = 0; c < ncol; c++) colour_begin[c + 1] += colour_begin[c];
	*ncolours = ncol;
	rc = 0;
done:
	free(off);
	free(lst);
	free(mark);
	free(colour);
	free(kv);
	return rc;
}

int orc_hex_schedule(const float* nodes, uint32_t nv, const uint32_t* hexes, uint32_t nh, uint32_t morton,
                     uint32_t* vert_rank, uint32_t* hex_order, uint32_t* colour_begin, uint32_t* ncolours) {
	return elem_schedule(nodes, nv, hexes, nh, 8, morton, vert_rank, hex_order, colour_begin, ncolours);
}

int orc_elem_schedule(const float* nodes, uint32_t nv, const uint32_t* elems, uint32_t ne, uint32_t per, uint32_t morton,
                      uint32_t* vert_rank, uint32_t* order, uint32_t* colour_begin, uint32_t* ncolours) {
	return elem_schedule(nodes, nv, elems, ne, per, morton, vert_rank, order, colour_begin, ncolours);
}

int orc_t10_schedule(const float* nodes, uint32_t nv, const uint32_t* t10, uint32_t nt, uint32_t morton,
                     uint32_t* vert_rank, uint32_t* order, uint32_t* colour_begin, uint32_t* ncolours) {
	return elem_schedule(nodes, nv, t10, nt, 10, morton, vert_rank, order, colour_begin, ncolours);
}

int orc_tet_edges(const uint32_t* tets, uint32_t nt, uint32_t nv, uint32_t* edges, uint32_t* nedges, uint32_t* t10) {
	/* per lower vertex, its edge instances in stream order */
	uint32_t* off = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* cnt = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* hi = (uint32_t*)malloc(4 * (size_t)(nt ? 6 * nt : 1));
	uint32_t* lst = (uint32_t*)malloc(4 * (size_t)(nt ? 6 * nt : 1));
	uint32_t* base = (uint32_t*)calloc((size_t)nv + 1, 4);
	static const int te[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
	int rc = -1;
	if (!off || !cnt || !hi || !lst || !base) goto done;
	for (uint32_t t = 0; t < nt; t++)
		for (int k = 0; k < 6; k++) {
			const uint32_t a = tets[4 * (size_t)t + te[k][0]], b = tets[4 * (size_t)t + te[k][1]];
			off[(a < b ? a : b) + 1]++;
		}
	for (uint32_t v = 0; v < nv; v++) off[v + 1] += off[v];
	for (uint32_t t = 0; t < nt; t++)
		for (int k = 0; k < 6; k++) {
			const uint32_t a = tets[4 * (size_t)t + te[k][0]], b = tets[4 * (size_t)t + te[k][1]];
			const uint32_t lo = a < b ? a : b, id = 6 * t + (uint32_t)k;
			hi[id] = a < b ? b : a;
			lst[off[lo] + cnt[lo]++] = id;
		}
	/* duplicates (same upper vertex) replaced by the list's last entry */
	for (uint32_t v = 0; v < nv; v++) {
		uint32_t* L = lst + off[v];
		for (uint32_t j = 0; j < cnt[v]; j++)
			for (uint32_t k = j + 1; k < cnt[v]; k++)
				if (hi[L[j]] == hi[L[k]]) {
					L[k] = L[cnt[v] - 1];
					--cnt[v];
					--k;
				}
	}
	{
		uint32_t ne = 0;
		for (uint32_t v = 0; v < nv; v++) {
			base[v] = ne;
			for (uint32_t j = 0; j < cnt[v]; j++) {
				edges[2 * (size_t)ne] = v;
				edges[2 * (size_t)ne + 1] = hi[lst[off[v] + j]];
				ne++;
			}
		}
		*nedges = ne;
	}
	/* the T10 indices: corners, then nv + the edges (0,1) (0,2) (0,3) (1,2)
	 * (1,3) (2,3) by EdgeFromVerts */
	if (t10)
		for (uint32_t t = 0; t < nt; t++) {
			for (int c = 0; c < 4; c++) t10[10 * (size_t)t + c] = tets[4 * (size_t)t + c];
			for (int k = 0; k < 6; k++) {
				const uint32_t a = tets[4 * (size_t)t + te[k][0]], b = tets[4 * (size_t)t + te[k][1]];
				const uint32_t lo = a < b ? a : b, h = a < b ? b : a;
				uint32_t e = 0xffffffffu;
				for (uint32_t j = 0; j < cnt[lo]; j++)
					if (edges[2 * (size_t)(base[lo] + j) + 1] == h) {
						e = base[lo] + j;
						break;
					}
				t10[10 * (size_t)t + 4 + k] = nv + e;
			}
		}
	rc = 0;
done:
	free(off);
	free(cnt);
	free(hi);
	free(lst);
	free(base);
	return rc;
}

int orc_h27_mesh(const uint32_t* hexes, uint32_t nh, uint32_t nv, uint32_t* edges, uint32_t* nedges, uint32_t* quads,
                 uint32_t* nquads, uint32_t* h27) {
	static const int he[12][2] = {{0, 1}, {0, 2}, {0, 4}, {1, 3}, {1, 5}, {2, 3}, {2, 6}, {3, 7}, {4, 5}, {4, 6}, {5, 7}, {6, 7}};
	static const int hq[6][4] = {{0, 1, 3, 2}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 2, 6, 4}, {1, 3, 7, 5}};
	const size_t ni = 12 * (size_t)nh, nqi = 6 * (size_t)nh;
	uint32_t* eoff = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* ecnt = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* eup = (uint32_t*)malloc(4 * (ni ? ni : 1));
	uint32_t* elst = (uint32_t*)malloc(4 * (ni ? ni : 1));
	uint32_t* ebase = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* qoff = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* qcnt = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* qv = (uint32_t*)malloc(16 * (nqi ? nqi : 1));
	uint32_t* qlst = (uint32_t*)malloc(4 * (nqi ? nqi : 1));
	uint32_t* qbase = (uint32_t*)calloc((size_t)nv + 1, 4);
	int rc = -1;
	if (!eoff || !ecnt || !eup || !elst || !ebase || !qoff || !qcnt || !qv || !qlst || !qbase) goto done;
	/* edge instances under their lower vertex, in stream order
	 * (XPBDFEM/Connectivity.cpp:384-394, 448-459) */
	for (uint32_t h = 0; h < nh; h++)
		for (int k = 0; k < 12; k++) {
			const uint32_t a = hexes[8 * (size_t)h + he[k][0]], b = hexes[8 * (size_t)h + he[k][1]];
			eoff[(a < b ? a : b) + 1]++;
		}
	for (uint32_t v = 0; v < nv; v++) eoff[v + 1] += eoff[v];
	for (uint32_t h = 0; h < nh; h++)
		for (int k = 0; k < 12; k++) {
			const uint32_t a = hexes[8 * (size_t)h + he[k][0]], b = hexes[8 * (size_t)h + he[k][1]];
			const uint32_t lo = a < b ? a : b, id = 12 * h + (uint32_t)k;
			eup[id] = a < b ? b : a;
			elst[eoff[lo] + ecnt[lo]++] = id;
		}
	/* quad instances rotated to their smallest vertex, filed under it
	 * (:410-422, 460-465) */
	for (uint32_t h = 0; h < nh; h++)
		for (int f = 0; f < 6; f++) {
			uint32_t vs[4], best = 0;
			for (int j = 0; j < 4; j++) vs[j] = hexes[8 * (size_t)h + hq[f][j]];
			for (int j = 1; j < 4; j++)
				if (vs[j] < vs[best]) best = (uint32_t)j;
			qoff[vs[best] + 1]++;
		}
	for (uint32_t v = 0; v < nv; v++) qoff[v + 1] += qoff[v];
	for (uint32_t h = 0; h < nh; h++)
		for (int f = 0; f < 6; f++) {
			uint32_t vs[4], best = 0;
			for (int j = 0; j < 4; j++) vs[j] = hexes[8 * (size_t)h + hq[f][j]];
			for (int j = 1; j < 4; j++)
				if (vs[j] < vs[best]) best = (uint32_t)j;
			const uint32_t id = 6 * h + (uint32_t)f;
			for (int j = 0; j < 4; j++) qv[4 * (size_t)id + j] = vs[(best + (uint32_t)j) % 4];
			qlst[qoff[vs[best]] + qcnt[vs[best]]++] = id;
		}
	/* duplicates replaced by the list's last entry (:486-530); a quad is a
	 * duplicate in either winding */
	for (uint32_t v = 0; v < nv; v++) {
		uint32_t* L = elst + eoff[v];
		for (uint32_t j = 0; j < ecnt[v]; j++)
			for (uint32_t k = j + 1; k < ecnt[v]; k++)
				if (eup[L[j]] == eup[L[k]]) {
					L[k] = L[ecnt[v] - 1];
					--ecnt[v];
					--k;
				}
		uint32_t* Q = qlst + qoff[v];
		for (uint32_t j = 0; j < qcnt[v]; j++)
			for (uint32_t k = j + 1; k < qcnt[v]; k++) {
				const uint32_t* a = qv + 4 * (size_t)Q[j];
				const uint32_t* b = qv + 4 * (size_t)Q[k];
				if ((a[1] == b[1] && a[2] == b[2] && a[3] == b[3]) || (a[1] == b[3] && a[2] == b[2] && a[3] == b[1])) {
					Q[k] = Q[qcnt[v] - 1];
					--qcnt[v];
					--k;
				}
			}
	}
	{
		uint32_t ne = 0, nq = 0;
		for (uint32_t v = 0; v < nv; v++) {
			ebase[v] = ne;
			for (uint32_t j = 0; j < ecnt[v]; j++) {
				edges[2 * (size_t)ne] = v;
				edges[2 * (size_t)ne + 1] = eup[elst[eoff[v] + j]];
				ne++;
			}
			qbase[v] = nq;
			for (uint32_t j = 0; j < qcnt[v]; j++) {
				for (int k = 0; k < 4; k++) quads[4 * (size_t)nq + k] = qv[4 * (size_t)qlst[qoff[v] + j] + k];
				nq++;
			}
		}
		*nedges = ne;
		*nquads = nq;
		/* GeoQuadratic3d's H27 indices (XPBDFEM/Geo.cpp:904-931): node
		 * i + 3j + 9k of the 3x3x3 grid; EdgeFromVerts / QuadFromVerts
		 * (XPBDFEM/Connectivity.cpp:587-611) */
		if (h27)
			for (uint32_t h = 0; h < nh; h++) {
				const uint32_t* c = hexes + 8 * (size_t)h;
				uint32_t* o = h27 + 27 * (size_t)h;
				for (int n = 0; n < 27; n++) {
					const int ix[3] = {n % 3, (n / 3) % 3, n / 9};
					int mid = 0, lo = 0, hi = 0;
					for (int a = 0; a < 3; a++) {
						mid += ix[a] == 1;
						lo |= (ix[a] == 2) << a; /* corner bits of the fixed axes */
						hi |= (ix[a] == 1) << a; /* the free axes */
					}
					if (mid == 0) {
						o[n] = c[lo];
					} else if (mid == 1) {
						const int f = hi == 1 ? 1 : hi == 2 ? 2 : 4;
						const uint32_t a = c[lo], b = c[lo | f];
						const uint32_t l = a < b ? a : b, u = a < b ? b : a;
						uint32_t e = 0;
						while (edges[2 * (size_t)(ebase[l] + e) + 1] != u) e++;
						o[n] = nv + ebase[l] + e;
					} else if (mid == 2) {
						const int f1 = hi & 1 ? 1 : 2, f2 = hi & 4 ? 4 : 2;
						const uint32_t vs[4] = {c[lo], c[lo | f1], c[lo | f1 | f2], c[lo | f2]};
						uint32_t best = 0;
						for (int j = 1; j < 4; j++)
							if (vs[j] < vs[best]) best = (uint32_t)j;
						const uint32_t v0 = vs[best], v1 = vs[(best + 1) % 4], v2 = vs[(best + 2) % 4], v3 = vs[(best + 3) % 4];
						uint32_t q = 0;
						for (;; q++) {
							const uint32_t* Q = quads + 4 * (size_t)(qbase[v0] + q);
							if ((Q[1] == v1 && Q[2] == v2 && Q[3] == v3) || (Q[1] == v3 && Q[2] == v2 && Q[3] == v1)) break;
						}
						o[n] = nv + ne + qbase[v0] + q;
					} else {
						o[n] = nv + ne + nq + h;
					}
				}
			}
	}
	rc = 0;
done:
	free(eoff);
	free(ecnt);
	free(eup);
	free(elst);
	free(ebase);
	free(qoff);
	free(qcnt);
	free(qv);
	free(qlst);
	free(qbase);
	return rc;
}

/* Connectivity3d's edges and quads of a tagged stream that may mix tets and
 * hexes (XPBDFEM/Connectivity.cpp:371-530): every element files its edge
 * instances (a tet's 6, a hex's 12) under their lower vertex, and a hex its 6
 * quad instances under their smallest vertex, in stream order; duplicates
 * take the list's last entry in their place; edges and quads are numbered
 * vertex by vertex. Then GeoQuadratic3d's element indices (XPBDFEM/Geo.cpp:
 * 893-931): per tet (tet order) its corners and nv + the edges (0,1) (0,2)
 * (0,3) (1,2) (1,3) (2,3); per hex (hex order) the 27 nodes of its 3x3x3
 * grid, the centre nv + ne + nq + its hex index. t10 / h27 may be NULL. */
int orc_quad_mesh(const uint32_t* idx, uint32_t count, uint32_t nv, uint32_t* edges, uint32_t* nedges, uint32_t* quads,
                  uint32_t* nquads, uint32_t* t10, uint32_t* h27) {
	static const int te[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
	static const int he[12][2] = {{0, 1}, {0, 2}, {0, 4}, {1, 3}, {1, 5}, {2, 3}, {2, 6}, {3, 7}, {4, 5}, {4, 6}, {5, 7}, {6, 7}};
	static const int hq[6][4] = {{0, 1, 3, 2}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 2, 6, 4}, {1, 3, 7, 5}};
	uint32_t nt = 0, nh = 0, nvs = 0;
	if (orc_parse_mixed(idx, count, NULL, &nt, NULL, &nh, &nvs) || nvs > nv) return -1;
	const size_t ni = 6 * (size_t)nt + 12 * (size_t)nh, nqi = 6 * (size_t)nh;
	uint32_t* eoff = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* ecnt = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* eup = (uint32_t*)malloc(4 * (ni ? ni : 1));
	uint32_t* elst = (uint32_t*)malloc(4 * (ni ? ni : 1));
	uint32_t* ebase = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* qoff = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* qcnt = (uint32_t*)calloc((size_t)nv + 1, 4);
	uint32_t* qv = (uint32_t*)malloc(16 * (nqi ? nqi : 1));
	uint32_t* qlst = (uint32_t*)malloc(4 * (nqi ? nqi : 1));
	uint32_t* qbase = (uint32_t*)calloc((size_t)nv + 1, 4);
	int rc = -1;
	if (!eoff || !ecnt || !eup || !elst || !ebase || !qoff || !qcnt || !qv || !qlst || !qbase) goto done;
	/* two walks over the stream: count the instances per vertex, then file them */
	for (int pass = 0; pass < 2; pass++) {
		uint32_t eid = 0, qid = 0;
		for (uint32_t i = 0; i < count; i += 1 + idx[i]) {
			const uint32_t* c = idx + i + 1;
			const int tet = idx[i] == 4u;
			const int ne_el = tet ? 6 : 12;
			for (int k = 0; k < ne_el; k++, eid++) {
				const uint32_t a = c[tet ? te[k][0] : he[k][0]], b = c[tet ? te[k][1] : he[k][1]];
				const uint32_t lo = a < b ? a : b;
				if (pass == 0) {
					eoff[lo + 1]++;
				} else {
					eup[eid] = a < b ? b : a;
					elst[eoff[lo] + ecnt[lo]++] = eid;
				}
			}
			if (tet) continue;
			for (int f = 0; f < 6; f++, qid++) {
				uint32_t vs[4], best = 0;
				for (int j = 0; j < 4; j++) vs[j] = c[hq[f][j]];
				for (int j = 1; j < 4; j++)
					if (vs[j] < vs[best]) best = (uint32_t)j;
				if (pass == 0) {
					qoff[vs[best] + 1]++;
				} else {
					for (int j = 0; j < 4; j++) qv[4 * (size_t)qid + j] = vs[(best + (uint32_t)j) % 4];
					qlst[qoff[vs[best]] + qcnt[vs[best]]++] = qid;
				}
			}
		}
		if (pass == 0)
			for (uint32_t v = 0; v < nv; v++) {
				eoff[v + 1] += eoff[v];
				qoff[v + 1] += qoff[v];
			}
	}
	for (uint32_t v = 0; v < nv; v++) {
		uint32_t* L = elst + eoff[v];
		for (uint32_t j = 0; j < ecnt[v]; j++)
			for (uint32_t k = j + 1; k < ecnt[v]; k++)
				if (eup[L[j]] == eup[L[k]]) {
					L[k] = L[ecnt[v] - 1];
					--ecnt[v];
					--k;
				}
		uint32_t* Q = qlst + qoff[v];
		for (uint32_t j = 0; j < qcnt[v]; j++)
			for (uint32_t k = j + 1; k < qcnt[v]; k++) {
				const uint32_t* a = qv + 4 * (size_t)Q[j];
				const uint32_t* b = qv + 4 * (size_t)Q[k];
				if ((a[1] == b[1] && a[2] == b[2] && a[3] == b[3]) || (a[1] == b[3] && a[2] == b[2] && a[3] == b[1])) {
					Q[k] = Q[qcnt[v] - 1];
					--qcnt[v];
					--k;
				}
			}
	}
	{
		uint32_t ne = 0, nq = 0;
		for (uint32_t v = 0; v < nv; v++) {
			ebase[v] = ne;
			for (uint32_t j = 0; j < ecnt[v]; j++) {
				edges[2 * (size_t)ne] = v;
				edges[2 * (size_t)ne + 1] = eup[elst[eoff[v] + j]];
				ne++;
			}
			qbase[v] = nq;
			for (uint32_t j = 0; j < qcnt[v]; j++) {
				for (int k = 0; k < 4; k++) quads[4 * (size_t)nq + k] = qv[4 * (size_t)qlst[qoff[v] + j] + k];
				nq++;
			}
		}
		*nedges = ne;
		*nquads = nq;
		uint32_t t = 0, h = 0;
		for (uint32_t i = 0; i < count; i += 1 + idx[i]) {
			const uint32_t* c = idx + i + 1;
			if (idx[i] == 4u) {
				if (t10) {
					uint32_t* o = t10 + 10 * (size_t)t;
					for (int k = 0; k < 4; k++) o[k] = c[k];
					for (int k = 0; k < 6; k++) {
						const uint32_t a = c[te[k][0]], b = c[te[k][1]];
						const uint32_t l = a < b ? a : b, u = a < b ? b : a;
						uint32_t e = 0;
						while (edges[2 * (size_t)(ebase[l] + e) + 1] != u) e++;
						o[4 + k] = nv + ebase[l] + e;
					}
				}
				t++;
				continue;
			}
			if (h27) {
				uint32_t* o = h27 + 27 * (size_t)h;
				for (int n = 0; n < 27; n++) {
					const int ix[3] = {n % 3, (n / 3) % 3, n / 9};
					int mid = 0, lo = 0, hi = 0;
					for (int a = 0; a < 3; a++) {
						mid += ix[a] == 1;
						lo |= (ix[a] == 2) << a;
						hi |= (ix[a] == 1) << a;
					}
					if (mid == 0) {
						o[n] = c[lo];
					} else if (mid == 1) {
						const int f = hi == 1 ? 1 : hi == 2 ? 2 : 4;
						const uint32_t a = c[lo], b = c[lo | f];
						const uint32_t l = a < b ? a : b, u = a < b ? b : a;
						uint32_t e = 0;
						while (edges[2 * (size_t)(ebase[l] + e) + 1] != u) e++;
						o[n] = nv + ebase[l] + e;
					} else if (mid == 2) {
						const int f1 = hi & 1 ? 1 : 2, f2 = hi & 4 ? 4 : 2;
						const uint32_t vs[4] = {c[lo], c[lo | f1], c[lo | f1 | f2], c[lo | f2]};
						uint32_t best = 0;
						for (int j = 1; j < 4; j++)
							if (vs[j] < vs[best]) best = (uint32_t)j;
						const uint32_t v0 = vs[best], v1 = vs[(best + 1) % 4], v2 = vs[(best + 2) % 4], v3 = vs[(best + 3) % 4];
						uint32_t q = 0;
						for (;; q++) {
							const uint32_t* Q = quads + 4 * (size_t)(qbase[v0] + q);
							if ((Q[1] == v1 && Q[2] == v2 && Q[3] == v3) || (Q[1] == v3 && Q[2] == v2 && Q[3] == v1)) break;
						}
						o[n] = nv + ne + qbase[v0] + q;
					} else {
						o[n] = nv + ne + nq + h;
					}
				}
			}
			h++;
		}
	}
	rc = 0;
done:
	free(eoff);
	free(ecnt);
	free(eup);
	free(elst);
	free(ebase);
	free(qoff);
	free(qcnt);
	free(qv);
	free(qlst);
	free(qbase);
	return rc;
}

int orc_h27_schedule(const float* nodes, uint32_t nv, const uint32_t* h27, uint32_t nh, uint32_t morton,
                     uint32_t* vert_rank, uint32_t* order, uint32_t* colour_begin, uint32_t* ncolours) {
	return elem_schedule(nodes, nv, h27, nh, 27, morton, vert_rank, order, colour_begin, ncolours);
}

int orc_schedule(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, uint32_t mode, uint32_t morton,
                 uint32_t* cluster_of, uint32_t* cluster_count, uint32_t* colour_of_cluster, uint32_t* ncolours,
                 uint32_t* vert_rank, uint32_t* tet_order, uint32_t* colour_tet_begin) {
	orc_csr csr;
	if (csr_build(tets, nt, nv, &csr)) return -1;
	static const int E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
	/* 1. clusters */
	uint32_t nc = 0;
	uint32_t* cl_begin = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)nt + 1));
	uint32_t* cl_tets = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)nt + 1));
	if (!cl_begin || !cl_tets) return -1;
	for (uint32_t t = 0; t < nt; t++) cluster_of[t] = 0xffffffffu;
	uint32_t fill = 0;
	for (uint32_t t = 0; t < nt; t++) {
		if (cluster_of[t] != 0xffffffffu) continue;
		cl_begin[nc] = fill;
		if (mode == 0) {
			cluster_of[t] = nc;
			cl_tets[fill++] = t;
			nc++;
			continue;
		}
		const uint32_t* tv = tets + 4 * (size_t)t;
		int best = 0;
		uint32_t bestc = 0;
		for (int e = 0; e < 6; e++) {
			uint32_t a = tv[E[e][0]], b = tv[E[e][1]], cnt = 0;
			for (uint32_t k = csr.off[a]; k < csr.off[a + 1]; k++) {
				uint32_t s = csr.lst[k];
				if (cluster_of[s] == 0xffffffffu && tet_has(tets + 4 * (size_t)s, b)) cnt++;
			}
			if (cnt > bestc) { bestc = cnt; best = e; }
		}
		uint32_t a = tv[E[best][0]], b = tv[E[best][1]];
		uint32_t verts[ORC_MAXV], nvv = 0, ntt = 0;
		for (uint32_t k = csr.off[a]; k < csr.off[a + 1]; k++) {
			uint32_t s = csr.lst[k];
			const uint32_t* sv = tets + 4 * (size_t)s;
			if (cluster_of[s] != 0xffffffffu || !tet_has(sv, b)) continue;
			if (ntt == ORC_MAXT) break;
			uint32_t nv2 = nvv, tmp[ORC_MAXV + 4];
			memcpy(tmp, verts, sizeof(uint32_t) * nvv);
			for (int n = 0; n < 4; n++) {
				int found = 0;
				for (uint32_t q = 0; q < nv2; q++)
					if (tmp[q] == sv[n]) { found = 1; break; }
				if (!found) tmp[nv2++] = sv[n];
			}
			if (nv2 > ORC_MAXV) continue;
			memcpy(verts, tmp, sizeof(uint32_t) * nv2);
			nvv = nv2;
			cluster_of[s] = nc;
			cl_tets[fill++] = s;
			ntt++;
		}
		nc++;
	}
	cl_begin[nc] = fill;
	*cluster_count = nc;
	/* 2. greedy colouring in cluster order */
	uint32_t ncol = 0;
	uint32_t* mark = (uint32_t*)malloc(sizeof(uint32_t) * ORC_MAXCOL);
	if (!mark) return -1;
	for (uint32_t c = 0; c < ORC_MAXCOL; c++) mark[c] = 0xffffffffu;
	for (uint32_t k = 0; k < nc; k++) {
		for (uint32_t q = cl_begin[k]; q < cl_begin[k + 1]; q++) {
			const uint32_t* tv = tets + 4 * (size_t)cl_tets[q];
			for (int n = 0; n < 4; n++)
				for (uint32_t j = csr.off[tv[n]]; j < csr.off[tv[n] + 1]; j++) {
					uint32_t o = cluster_of[csr.lst[j]];
					if (o < k) mark[colour_of_cluster[o]] = k;
				}
		}
		uint32_t c = 0;
		while (c < ORC_MAXCOL && mark[c] == k) c++;
		if (c == ORC_MAXCOL) return -1;
		colour_of_cluster[k] = c;
		if (c + 1 > ncol) ncol = c + 1;
	}
	*ncolours = ncol;
	/* 3. vertex order */
	float mn[3] = {INFINITY, INFINITY, INFINITY};
	float sc[3] = {0.0f, 0.0f, 0.0f};
	if (orc_vertex_ranks(nodes, nv, morton, vert_rank, mn, sc)) return -1;
	/* 4. cluster order inside each colour: (colour, Morton code of the
	 * centroid of the cluster's tet vertices, id); without Morton order,
	 * (colour, smallest vertex id, id) */
	orc_kv* ck = (orc_kv*)malloc(sizeof(orc_kv) * (nc ? nc : 1));
	if (!ck) return -1;
	for (uint32_t k = 0; k < nc; k++) {
		uint32_t key = 0xffffffffu;
		if (morton) {
			float c[3] = {0.0f, 0.0f, 0.0f};
			for (uint32_t q = cl_begin[k]; q < cl_begin[k + 1]; q++)
				for (int n = 0; n < 4; n++)
					for (int j = 0; j < 3; j++) c[j] += nodes[3 * (size_t)tets[4 * (size_t)cl_tets[q] + n] + j];
			float cnt = (float)(4u * (cl_begin[k + 1] - cl_begin[k]));
			for (int j = 0; j < 3; j++) c[j] = c[j] / cnt;
			key = orc_quantise(c, mn, sc);
		} else {
			for (uint32_t q = cl_begin[k]; q < cl_begin[k + 1]; q++)
				for (int n = 0; n < 4; n++) {
					uint32_t v = tets[4 * (size_t)cl_tets[q] + n];
					if (v < key) key = v;
				}
		}
		ck[k].key = ((uint64_t)colour_of_cluster[k] << 32) | key;
		ck[k].id = k;
	}
	qsort(ck, nc, sizeof(orc_kv), kv_cmp);
	uint32_t o = 0, col = 0;
	colour_tet_begin[0] = 0;
	for (uint32_t i = 0; i < nc; i++) {
		uint32_t k = ck[i].id;
		while (col < colour_of_cluster[k]) colour_tet_begin[++col] = o;
		for (uint32_t q = cl_begin[k]; q < cl_begin[k + 1]; q++) tet_order[o++] = cl_tets[q];
	}
	while (col < ncol) colour_tet_begin[++col] = o;
	free(ck);
	free(mark);
	free(cl_begin);
	free(cl_tets);
	free(csr.off);
	free(csr.lst);
	return 0;
}
