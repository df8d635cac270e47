// Host-side set-up of libxfem.so: mesh ingestion, the reference's rest-state
// precompute and the colour schedule. Compiled with -ffp-contract=off: the
// rest state must match the reference (compiled without fused multiply-add)
// bit for bit, and the Morton quantisation must give the same integers on
// x86-64 and AArch64.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "xfem_internal.h"

namespace xfem {

namespace {

// Small column-major 3x3 helpers in the reference's evaluation order
// (GLSL-style mat3, XPBDFEM/vectormath.h:190-197, 501-526).
struct M3 {
	float c[3][3];  // c[column][row]
};

inline float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// determinant(mat3), XPBDFEM/vectormath.cpp:34-39
float det3(const M3& m) {
	float a = m.c[0][0], b = m.c[1][0], c = m.c[2][0];
	float d = m.c[0][1], e = m.c[1][1], f = m.c[2][1];
	float g = m.c[0][2], h = m.c[1][2], i = m.c[2][2];
	return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

// inverse(mat3), XPBDFEM/vectormath.cpp:40-58: adjugate in double rounded to
// float, determinant and 1/det scaling in float.
M3 inverse3(const M3& m) {
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
M3 map_jacobian(const float P[4][3]) {
	M3 J;
	for (int c = 0; c < 3; c++)
		for (int r = 0; r < 3; r++) J.c[c][r] = 0.0f + P[r][c];
	return J;
}

// column k of m as (m * e_k), the reference's mat3 * vec3 with a unit vector
void column_of(const M3& m, int k, float out[3]) {
	const float e[3] = {k == 0 ? 1.0f : 0.0f, k == 1 ? 1.0f : 0.0f, k == 2 ? 1.0f : 0.0f};
	for (int r = 0; r < 3; r++) {
		const float row[3] = {m.c[0][r], m.c[1][r], m.c[2][r]};
		out[r] = dot3(row, e);
	}
}

float face_area(const float P[4][3], int i0, int i1, int i2) {
	float a[3], b[3];
	for (int k = 0; k < 3; k++) {
		a[k] = P[i0][k] - P[i2][k];
		b[k] = P[i1][k] - P[i2][k];
	}
	const float c[3] = {a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]};
	return 0.5f * sqrtf(dot3(c, c));
}

}  // namespace

int parse_tets(const uint32_t* idx, uint32_t idx_count, std::vector<uint32_t>& tets, uint32_t& nverts) {
	tets.clear();
	uint32_t mx = 0;
	for (uint64_t i = 0; i < idx_count; i += 5) {
		if (idx[i] != 4u || i + 4 >= idx_count) return -1;
		for (int n = 0; n < 4; n++) {
			const uint32_t v = idx[i + 1 + n];
			mx = v > mx ? v : mx;
			tets.push_back(v);
		}
	}
	nverts = tets.empty() ? 0 : mx + 1;
	return 0;
}

void init_rest(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, float density,
               float* ep, float* w, uint8_t* vflags) {
	// AABB and Left / Right flags (XPBDFEM/Geo.cpp:713-727)
	float mn[3] = {1.0e24f, 1.0e24f, 1.0e24f}, mx[3] = {-1.0e24f, -1.0e24f, -1.0e24f};
	for (uint32_t i = 0; i < nverts; i++) {
		w[i] = 0.0f;
		for (int k = 0; k < 3; k++) {
			mn[k] = fminf(mn[k], nodes[3 * (size_t)i + k]);
			mx[k] = fmaxf(mx[k], nodes[3 * (size_t)i + k]);
		}
	}
	for (uint32_t i = 0; i < nverts; i++) {
		uint8_t f = 1u << 4;
		const float rel = (nodes[3 * (size_t)i] - mn[0]) / (mx[0] - mn[0]);
		if (rel < 0.02f) f |= 1u;
		if (rel > 0.98f) f |= 2u;
		vflags[i] = f;
	}
	const float sixth = 1.0f / 6.0f;
	for (uint32_t t = 0; t < ntets; t++) {
		const uint32_t* is = tets + 4 * (size_t)t;
		// P[n] = vec3(X[n] - X[root]) with X the node data widened to double
		float P[4][3];
		for (int n = 0; n < 4; n++)
			for (int k = 0; k < 3; k++)
				P[n][k] = (float)((double)nodes[3 * (size_t)is[n] + k] - (double)nodes[3 * (size_t)is[3] + k]);
		const M3 J = map_jacobian(P);
		const M3 Qi = inverse3(J);
		// GeneratePrefactoredCoefficients<Tet> (XPBDFEM/Fem.cpp:131-161): four
		// identical quadrature points of weight 0.25
		float QQ[3] = {0, 0, 0}, QR[3] = {0, 0, 0}, vsum = 0.0f;
		for (int p = 0; p < 4; p++) {
			const M3 Ji = inverse3(J);
			const float wq = det3(J) * sixth * 0.25f;
			float q[3][3];
			for (int i = 0; i < 3; i++) column_of(Ji, i, q[i]);
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
		float* o = ep + 17 * (size_t)t;
		for (int c = 0; c < 3; c++)
			for (int r = 0; r < 3; r++) o[c * 3 + r] = Qi.c[c][r];
		for (int i = 0; i < 3; i++) {
			o[9 + i] = QQ[i];
			o[12 + i] = QR[i];
		}
		o[15] = vol;
		o[16] = area;
		// lumped mass, LumpsTet4 (XPBDFEM/Fem.cpp:217-223), accumulated per node
		const float dm = (1.0f / 4.0f) * density * vol;
		for (int n = 0; n < 4; n++) w[is[n]] += dm;
	}
	for (uint32_t i = 0; i < nverts; i++) w[i] = 1.0f / w[i];  // XPBDFEM/Geo.cpp:744
}

void gen_tet_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                   float wonkiness, float* nodes, uint32_t* idx) {
	const float sc[3] = {sx, sy, sz};
	const float mn[3] = {sx * (-0.5f * (float)W), sy * (-0.5f * (float)H), sz * (-0.5f * (float)D)};
	uint32_t state = 1;
	auto randf = [&]() {
		state = (uint32_t)(((uint64_t)state * 48271u) % 0x7fffffffu);
		return (float)state * 9.3132258e-10f - 1.0f;
	};
	for (uint32_t z = 0; z <= D; z++)
		for (uint32_t y = 0; y <= H; y++)
			for (uint32_t x = 0; x <= W; x++) {
				const bool edge[3] = {x == 0 || x == W, y == 0 || y == H, z == 0 || z == D};
				// The reference draws z, y, x in that order (right-to-left evaluation
				// of one constructor's arguments, as g++ and MSVC compile it).
				float r[3] = {0.0f, 0.0f, 0.0f};
				for (int k = 2; k >= 0; k--)
					if (!edge[k]) r[k] = randf();
				const float c[3] = {(float)x, (float)y, (float)z};
				const size_t i = x + (size_t)y * (W + 1) + (size_t)z * (W + 1) * (H + 1);
				for (int k = 0; k < 3; k++) nodes[3 * i + k] = mn[k] + sc[k] * (c[k] + 0.5f * (wonkiness * r[k]));
			}
	static const int split[6][4] = {{0, 1, 5, 7}, {0, 7, 3, 1}, {0, 2, 3, 7}, {0, 7, 6, 2}, {0, 4, 6, 7}, {0, 7, 5, 4}};
	size_t ie = 0;
	for (uint32_t z = 0; z < D; z++)
		for (uint32_t y = 0; y < H; y++)
			for (uint32_t x = 0; x < W; x++, ie++) {
				uint32_t ih[8];
				for (uint32_t k = 0; k < 2; k++)
					for (uint32_t j = 0; j < 2; j++)
						for (uint32_t i = 0; i < 2; i++) {
							uint32_t hi = i + 2 * j + 4 * k, xx = i, yy = j, zz = k;
							if (pattern != 0) {
								xx = x % 2 == 0 ? i : 1 - i;
								yy = y % 2 == 0 ? j : 1 - j;
								zz = z % 2 == 0 ? k : 1 - k;
								if ((x + y + z) % 2 == 1) hi = 7 - hi;
							}
							ih[hi] = (x + xx) + (y + yy) * (W + 1) + (z + zz) * (W + 1) * (H + 1);
						}
				for (int t = 0; t < 6; t++) {
					uint32_t* o = idx + 30 * ie + 5 * t;
					o[0] = 4;
					for (int n = 0; n < 4; n++) o[1 + n] = ih[split[t][n]];
				}
			}
}

namespace {

uint32_t morton_code(uint32_t x, uint32_t y, uint32_t z) {
	uint32_t c = 0;
	for (int b = 0; b < 10; b++)
		c |= (((x >> b) & 1u) << (3 * b)) | (((y >> b) & 1u) << (3 * b + 1)) | (((z >> b) & 1u) << (3 * b + 2));
	return c;
}

bool tet_has(const uint32_t* tv, uint32_t v) { return tv[0] == v || tv[1] == v || tv[2] == v || tv[3] == v; }

}  // namespace

// The schedule. Every rule here is fixed (no hash order, no floating-point
// ties) so the result is deterministic and reproducible by an independent
// implementation:
//  1. vertex -> tet incidence lists in increasing tet id;
//  2. clusters, visiting tets in id order; an unassigned tet t opens a
//     cluster around the first of its six edges (local pairs 01,02,03,12,13,23)
//     with the most unassigned incident tets, and takes those tets in id
//     order while the cluster stays within 8 tets and 8 vertices (mode 0:
//     every tet is its own cluster);
//  3. greedy colouring of clusters in id order: the smallest colour not used
//     by an earlier cluster sharing a vertex;
//  4. vertex rank: Morton code of the rest position (10 bits per axis,
//     quantised over the AABB with one scale, its largest extent) then
//     vertex id; or the identity;
//  5. inside a colour, clusters by (Morton code of their centroid, id), or
//     (smallest vertex id, id) without Morton order.
int build_schedule(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, uint32_t mode,
                   uint32_t morton, Schedule& s) {
	std::vector<uint32_t> off(nverts + 1, 0), lst(4 * (size_t)ntets);
	for (size_t i = 0; i < 4 * (size_t)ntets; i++) off[tets[i] + 1]++;
	for (uint32_t v = 0; v < nverts; v++) off[v + 1] += off[v];
	{
		std::vector<uint32_t> fill(off.begin(), off.end() - 1);
		for (uint32_t t = 0; t < ntets; t++)
			for (int n = 0; n < 4; n++) lst[fill[tets[4 * (size_t)t + n]]++] = t;
	}
	const uint32_t kNone = 0xffffffffu;
	std::vector<uint32_t> cluster_of(ntets, kNone);
	s.cl_begin.clear();
	s.cl_tets.clear();
	s.cl_tets.reserve(ntets);
	static const int E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
	uint32_t nc = 0;
	for (uint32_t t = 0; t < ntets; t++) {
		if (cluster_of[t] != kNone) continue;
		s.cl_begin.push_back((uint32_t)s.cl_tets.size());
		if (mode == 0) {
			cluster_of[t] = nc++;
			s.cl_tets.push_back(t);
			continue;
		}
		const uint32_t* tv = tets + 4 * (size_t)t;
		int best = 0;
		uint32_t best_count = 0;
		for (int e = 0; e < 6; e++) {
			const uint32_t a = tv[E[e][0]], b = tv[E[e][1]];
			uint32_t cnt = 0;
			for (uint32_t k = off[a]; k < off[a + 1]; k++)
				if (cluster_of[lst[k]] == kNone && tet_has(tets + 4 * (size_t)lst[k], b)) cnt++;
			if (cnt > best_count) {
				best_count = cnt;
				best = e;
			}
		}
		const uint32_t a = tv[E[best][0]], b = tv[E[best][1]];
		uint32_t verts[kMaxClusterVerts];
		uint32_t nvv = 0, ntt = 0;
		for (uint32_t k = off[a]; k < off[a + 1]; k++) {
			const uint32_t q = lst[k];
			const uint32_t* qv = tets + 4 * (size_t)q;
			if (cluster_of[q] != kNone || !tet_has(qv, b)) continue;
			if (ntt == kMaxClusterTets) break;
			uint32_t tmp[kMaxClusterVerts + 4];
			uint32_t n2 = nvv;
			std::copy(verts, verts + nvv, tmp);
			for (int n = 0; n < 4; n++)
				if (std::find(tmp, tmp + n2, qv[n]) == tmp + n2) tmp[n2++] = qv[n];
			if (n2 > kMaxClusterVerts) continue;
			std::copy(tmp, tmp + n2, verts);
			nvv = n2;
			cluster_of[q] = nc;
			s.cl_tets.push_back(q);
			ntt++;
		}
		nc++;
	}
	s.cl_begin.push_back((uint32_t)s.cl_tets.size());
	s.nclusters = nc;

	// greedy colouring
	s.cl_colour.assign(nc, 0);
	std::vector<uint32_t> mark(kMaxColours, kNone);
	uint32_t ncol = 0;
	for (uint32_t k = 0; k < nc; k++) {
		for (uint32_t q = s.cl_begin[k]; q < s.cl_begin[k + 1]; q++) {
			const uint32_t* tv = tets + 4 * (size_t)s.cl_tets[q];
			for (int n = 0; n < 4; n++)
				for (uint32_t j = off[tv[n]]; j < off[tv[n] + 1]; j++) {
					const uint32_t o = cluster_of[lst[j]];
					if (o < k) mark[s.cl_colour[o]] = k;
				}
		}
		uint32_t c = 0;
		while (c < kMaxColours && mark[c] == k) c++;
		if (c == kMaxColours) return -1;
		s.cl_colour[k] = c;
		ncol = std::max(ncol, c + 1);
	}
	s.ncolours = ncol;

	// vertex rank
	s.vert_rank.resize(nverts);
	float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
	float sc[3] = {0.0f, 0.0f, 0.0f};
	auto quantise = [&](const float* p3) {
		uint32_t q[3];
		for (int k = 0; k < 3; k++) {
			const float f = (p3[k] - mn[k]) * sc[k];
			const uint32_t u = f > 0.0f ? (uint32_t)f : 0u;
			q[k] = u > 1023u ? 1023u : u;
		}
		return morton_code(q[0], q[1], q[2]);
	};
	if (morton) {
		for (uint32_t v = 0; v < nverts; v++)
			for (int k = 0; k < 3; k++) {
				const float x = nodes[3 * (size_t)v + k];
				mn[k] = x < mn[k] ? x : mn[k];
				mx[k] = x > mx[k] ? x : mx[k];
			}
		// one scale for all axes (the largest extent), so the curve's cells are
		// cubes and consecutive clusters form compact blocks on any box shape
		float ext = 0.0f;
		for (int k = 0; k < 3; k++) ext = (mx[k] - mn[k]) > ext ? (mx[k] - mn[k]) : ext;
		for (int k = 0; k < 3; k++) sc[k] = ext > 0.0f ? 1023.0f / ext : 0.0f;
		std::vector<uint64_t> key(nverts);
		for (uint32_t v = 0; v < nverts; v++) key[v] = ((uint64_t)quantise(nodes + 3 * (size_t)v) << 32) | v;
		std::sort(key.begin(), key.end());
		for (uint32_t i = 0; i < nverts; i++) s.vert_rank[(uint32_t)key[i]] = i;
	} else {
		for (uint32_t v = 0; v < nverts; v++) s.vert_rank[v] = v;
	}

	// cluster order inside each colour: Morton code of the cluster's centroid
	// (the mean of its tets' vertex positions, summed tet by tet in float); it
	// sits inside a curve cell, where a corner would sit on a cell boundary
	// and flip bits with rounding. Without Morton order: smallest vertex id.
	std::vector<std::pair<uint64_t, uint32_t>> ck(nc);
	for (uint32_t k = 0; k < nc; k++) {
		uint32_t key = kNone;
		if (morton) {
			float c[3] = {0.0f, 0.0f, 0.0f};
			for (uint32_t q = s.cl_begin[k]; q < s.cl_begin[k + 1]; q++)
				for (int n = 0; n < 4; n++)
					for (int j = 0; j < 3; j++) c[j] += nodes[3 * (size_t)tets[4 * (size_t)s.cl_tets[q] + n] + j];
			const float cnt = (float)(4u * (s.cl_begin[k + 1] - s.cl_begin[k]));
			for (int j = 0; j < 3; j++) c[j] = c[j] / cnt;
			key = quantise(c);
		} else {
			for (uint32_t q = s.cl_begin[k]; q < s.cl_begin[k + 1]; q++)
				for (int n = 0; n < 4; n++) key = std::min(key, tets[4 * (size_t)s.cl_tets[q] + n]);
		}
		ck[k] = {((uint64_t)s.cl_colour[k] << 32) | key, k};
	}
	std::sort(ck.begin(), ck.end());
	s.colour_cl.resize(nc);
	s.colour_cl_begin.assign(ncol + 1, 0);
	for (uint32_t i = 0; i < nc; i++) {
		s.colour_cl[i] = ck[i].second;
		s.colour_cl_begin[s.cl_colour[ck[i].second] + 1]++;
	}
	for (uint32_t c = 0; c < ncol; c++) s.colour_cl_begin[c + 1] += s.colour_cl_begin[c];
	return 0;
}

}  // namespace xfem
