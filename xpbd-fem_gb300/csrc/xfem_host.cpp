// Host-side set-up of libxfem.so: mesh ingestion, the reference's rest-state
// precompute and the colour schedule. Compiled with -ffp-contract=off: the
// rest state must match the reference (compiled without fused multiply-add)
// bit for bit, and the Morton quantisation must give the same integers on
// x86-64 and AArch64.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "xfem_internal.h"
#include "xfem_rest.h"

namespace xfem {

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
	for (uint32_t i = 0; i < nverts; i++) vflags[i] = rest::vertex_flags(nodes[3 * (size_t)i], mn[0], mx[0]);
	for (uint32_t t = 0; t < ntets; t++) {
		const uint32_t* is = tets + 4 * (size_t)t;
		// lumped mass accumulated per node in tet order
		const float dm = rest::tet(nodes, is, density, ep + 17 * (size_t)t);
		for (int n = 0; n < 4; n++) w[is[n]] += dm;
	}
	for (uint32_t i = 0; i < nverts; i++) w[i] = 1.0f / w[i];  // XPBDFEM/Geo.cpp:744
}

void gen_hex_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
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
	size_t ie = 0;
	for (uint32_t z = 0; z < D; z++)
		for (uint32_t y = 0; y < H; y++)
			for (uint32_t x = 0; x < W; x++, ie++) {
				uint32_t* ih = idx + 9 * ie + 1;
				idx[9 * ie] = 8;
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
			}
}

void gen_tet_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                   float wonkiness, float* nodes, uint32_t* idx) {
	const size_t ncell = (size_t)W * H * D;
	std::vector<uint32_t> hex(9 * ncell);
	gen_hex_block(W, H, D, sx, sy, sz, pattern, wonkiness, nodes, hex.data());
	// six tets per cell (XPBDFEM/MeshGen.cpp:235-240)
	static const int split[6][4] = {{0, 1, 5, 7}, {0, 7, 3, 1}, {0, 2, 3, 7}, {0, 7, 6, 2}, {0, 4, 6, 7}, {0, 7, 5, 4}};
	for (size_t ie = 0; ie < ncell; ie++)
		for (int t = 0; t < 6; t++) {
			uint32_t* o = idx + 30 * ie + 5 * t;
			o[0] = 4;
			for (int n = 0; n < 4; n++) o[1 + n] = hex[9 * ie + 1 + split[t][n]];
		}
}

int parse_hexes(const uint32_t* idx, uint32_t idx_count, std::vector<uint32_t>& hexes, uint32_t& nverts) {
	hexes.clear();
	uint32_t mx = 0;
	for (uint64_t i = 0; i < idx_count; i += 9) {
		if (idx[i] != 8u || i + 8 >= idx_count) return -1;
		for (int n = 0; n < 8; n++) {
			const uint32_t v = idx[i + 1 + n];
			mx = v > mx ? v : mx;
			hexes.push_back(v);
		}
	}
	nverts = hexes.empty() ? 0 : mx + 1;
	return 0;
}

int parse_mixed(const uint32_t* idx, uint32_t idx_count, std::vector<uint32_t>& tets, std::vector<uint32_t>& hexes,
                uint32_t& nverts) {
	tets.clear();
	hexes.clear();
	uint32_t mx = 0;
	bool any = false;
	for (uint64_t i = 0; i < idx_count;) {
		const uint32_t tag = idx[i];
		if ((tag != 4u && tag != 8u) || i + tag >= idx_count) return -1;
		std::vector<uint32_t>& out = tag == 4u ? tets : hexes;
		for (uint32_t n = 0; n < tag; n++) {
			const uint32_t v = idx[i + 1 + n];
			mx = v > mx ? v : mx;
			out.push_back(v);
		}
		any = true;
		i += tag + 1;
	}
	nverts = any ? mx + 1 : 0;
	return 0;
}

void mixed_init_rest(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, const uint32_t* hexes,
                     uint32_t nhexes, float density, float* ep, float* hep, float* w, uint8_t* vflags) {
	float mn[3] = {1.0e24f, 1.0e24f, 1.0e24f}, mx[3] = {-1.0e24f, -1.0e24f, -1.0e24f};
	for (uint32_t i = 0; i < nverts; i++) {
		w[i] = 0.0f;
		for (int k = 0; k < 3; k++) {
			mn[k] = fminf(mn[k], nodes[3 * (size_t)i + k]);
			mx[k] = fmaxf(mx[k], nodes[3 * (size_t)i + k]);
		}
	}
	for (uint32_t i = 0; i < nverts; i++) vflags[i] = rest::vertex_flags(nodes[3 * (size_t)i], mn[0], mx[0]);
	// the tets' lumped masses first, then the hexes' (XPBDFEM/Geo.cpp:733-742)
	for (uint32_t t = 0; t < ntets; t++) {
		const uint32_t* is = tets + 4 * (size_t)t;
		const float dm = rest::tet(nodes, is, density, ep + 17 * (size_t)t);
		for (int n = 0; n < 4; n++) w[is[n]] += dm;
	}
	for (uint32_t h = 0; h < nhexes; h++) {
		const uint32_t* is = hexes + 8 * (size_t)h;
		float m[8];
		rest::hex(nodes, is, density, hep + (size_t)rest::kHexRec * h, m);
		for (int n = 0; n < 8; n++) w[is[n]] += m[n];
	}
	for (uint32_t i = 0; i < nverts; i++) w[i] = 1.0f / w[i];
}

void hex_init_rest(const float* nodes, uint32_t nverts, const uint32_t* hexes, uint32_t nhexes, float density,
                   float* hep, float* w, uint8_t* vflags) {
	float mn[3] = {1.0e24f, 1.0e24f, 1.0e24f}, mx[3] = {-1.0e24f, -1.0e24f, -1.0e24f};
	for (uint32_t i = 0; i < nverts; i++) {
		w[i] = 0.0f;
		for (int k = 0; k < 3; k++) {
			mn[k] = fminf(mn[k], nodes[3 * (size_t)i + k]);
			mx[k] = fmaxf(mx[k], nodes[3 * (size_t)i + k]);
		}
	}
	for (uint32_t i = 0; i < nverts; i++) vflags[i] = rest::vertex_flags(nodes[3 * (size_t)i], mn[0], mx[0]);
	for (uint32_t h = 0; h < nhexes; h++) {
		const uint32_t* is = hexes + 8 * (size_t)h;
		float m[8];
		rest::hex(nodes, is, density, hep + (size_t)rest::kHexRec * h, m);
		for (int n = 0; n < 8; n++) w[is[n]] += m[n];
	}
	for (uint32_t i = 0; i < nverts; i++) w[i] = 1.0f / w[i];
}

namespace {

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
void incidence(const uint32_t* tets, uint32_t nverts, uint32_t ntets, std::vector<uint32_t>& off,
               std::vector<uint32_t>& lst, uint32_t npe) {
	off.assign(nverts + 1, 0);
	lst.resize(npe * (size_t)ntets);
	for (size_t i = 0; i < npe * (size_t)ntets; i++) off[tets[i] + 1]++;
	for (uint32_t v = 0; v < nverts; v++) off[v + 1] += off[v];
	std::vector<uint32_t> fill(off.begin(), off.end() - 1);
	for (uint32_t t = 0; t < ntets; t++)
		for (uint32_t n = 0; n < npe; n++) lst[fill[tets[npe * (size_t)t + n]]++] = t;
}

int cluster_and_colour(const uint32_t* tets, uint32_t ntets, const uint32_t* off, const uint32_t* lst, uint32_t mode,
                       Schedule& s) {
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

	// greedy colouring, over each cluster's distinct vertices
	s.cl_colour.assign(nc, 0);
	std::vector<uint32_t> mark(kMaxColours, kNone);
	uint32_t ncol = 0;
	for (uint32_t k = 0; k < nc; k++) {
		uint32_t vs[4 * kMaxClusterTets], nvs = 0;
		for (uint32_t q = s.cl_begin[k]; q < s.cl_begin[k + 1]; q++) {
			const uint32_t* tv = tets + 4 * (size_t)s.cl_tets[q];
			for (int n = 0; n < 4; n++)
				if (std::find(vs, vs + nvs, tv[n]) == vs + nvs) vs[nvs++] = tv[n];
		}
		for (uint32_t i = 0; i < nvs; i++)
			for (uint32_t j = off[vs[i]]; j < off[vs[i] + 1]; j++) {
				const uint32_t o = cluster_of[lst[j]];
				if (o < k) mark[s.cl_colour[o]] = k;
			}
		uint32_t c = 0;
		while (c < kMaxColours && mark[c] == k) c++;
		if (c == kMaxColours) return -1;
		s.cl_colour[k] = c;
		ncol = std::max(ncol, c + 1);
	}
	s.ncolours = ncol;
	return 0;
}

MortonFrame morton_frame(const float* nodes, uint32_t nverts) {
	MortonFrame f;
	for (int k = 0; k < 3; k++) {
		f.mn[k] = INFINITY;
		f.mx[k] = -INFINITY;
	}
	for (uint32_t v = 0; v < nverts; v++)
		for (int k = 0; k < 3; k++) {
			const float x = nodes[3 * (size_t)v + k];
			f.mn[k] = x < f.mn[k] ? x : f.mn[k];
			f.mx[k] = x > f.mx[k] ? x : f.mx[k];
		}
	// one scale for all axes (the largest extent), so the curve's cells are
	// cubes and consecutive clusters form compact blocks on any box shape
	f.set_scale();
	return f;
}

void vertex_ranks(const float* nodes, uint32_t nverts, uint32_t morton, Schedule& s) {
	s.vert_rank.resize(nverts);
	if (!morton) {
		for (uint32_t v = 0; v < nverts; v++) s.vert_rank[v] = v;
		return;
	}
	const MortonFrame f = morton_frame(nodes, nverts);
	std::vector<uint64_t> key(nverts);
	for (uint32_t v = 0; v < nverts; v++) key[v] = ((uint64_t)f.code(nodes + 3 * (size_t)v) << 32) | v;
	std::sort(key.begin(), key.end());
	for (uint32_t i = 0; i < nverts; i++) s.vert_rank[(uint32_t)key[i]] = i;
}

void cluster_order(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t morton, Schedule& s) {
	const uint32_t nc = s.nclusters, ncol = s.ncolours;
	const MortonFrame f = morton ? morton_frame(nodes, nverts) : MortonFrame{};
	std::vector<std::pair<uint64_t, uint32_t>> ck(nc);
	for (uint32_t k = 0; k < nc; k++)
		ck[k] = {((uint64_t)s.cl_colour[k] << 32) | cluster_key(nodes, tets, s.cl_tets.data() + s.cl_begin[k],
		                                                         s.cl_begin[k + 1] - s.cl_begin[k], morton, f),
		         k};
	std::sort(ck.begin(), ck.end());
	s.colour_cl.resize(nc);
	s.colour_cl_begin.assign(ncol + 1, 0);
	for (uint32_t i = 0; i < nc; i++) {
		s.colour_cl[i] = ck[i].second;
		s.colour_cl_begin[s.cl_colour[ck[i].second] + 1]++;
	}
	for (uint32_t c = 0; c < ncol; c++) s.colour_cl_begin[c + 1] += s.colour_cl_begin[c];
}

int build_ring_schedule(const uint32_t* tets, uint32_t nverts, const uint32_t* off, const uint32_t* lst,
                        const uint32_t* vert_rank, RingSchedule& rs, uint32_t npe, uint32_t ncentre) {
	const uint32_t kNone = 0xffffffffu;
	if (ncentre > nverts) ncentre = nverts;
	const uint32_t max_elems = npe == 27   ? kMaxH27RingElems
	                           : npe == 10 ? kMaxQRingElems
	                           : npe == 8  ? kMaxRingHexes
	                                       : kMaxRingTets;
	const uint32_t max_nodes = npe >= 10 ? kMaxQRingNodes : kMaxRingNodes;
	rs.npe = npe;
	rs.nrings = ncentre;
	rs.tet_off.assign(off, off + nverts + 1);
	rs.tets.assign(lst, lst + off[nverts]);
	rs.node_off.assign(ncentre + 1, 0);
	rs.nodes.clear();
	rs.corner.assign(off[nverts] * npe, 0);
	std::vector<uint32_t> nodes(npe * (size_t)max_elems + 1);
	for (uint32_t v = 0; v < ncentre; v++) {
		rs.node_off[v] = (uint32_t)rs.nodes.size();
		if (off[v + 1] - off[v] > max_elems) return -2;
		uint32_t cnt = 1;
		nodes[0] = v;
		for (uint32_t j = off[v]; j < off[v + 1]; j++) {
			const uint32_t* tv = tets + npe * (size_t)lst[j];
			for (uint32_t n = 0; n < npe; n++) {
				const uint32_t k = (uint32_t)(std::find(nodes.begin(), nodes.begin() + cnt, tv[n]) - nodes.begin());
				if (k == cnt) nodes[cnt++] = tv[n];
				rs.corner[npe * (size_t)j + n] = (uint8_t)k;
			}
		}
		if (cnt > max_nodes) return -2;
		rs.nodes.insert(rs.nodes.end(), nodes.begin(), nodes.begin() + cnt);
	}
	rs.node_off[ncentre] = (uint32_t)rs.nodes.size();
	// the rings holding each node
	std::vector<uint32_t> hoff(nverts + 1, 0), hl(rs.nodes.size());
	for (uint32_t x : rs.nodes) hoff[x + 1]++;
	for (uint32_t v = 0; v < nverts; v++) hoff[v + 1] += hoff[v];
	{
		std::vector<uint32_t> fill(hoff.begin(), hoff.end() - 1);
		for (uint32_t v = 0; v < ncentre; v++)
			for (uint32_t i = rs.node_off[v]; i < rs.node_off[v + 1]; i++) hl[fill[rs.nodes[i]]++] = v;
	}
	// greedy colouring in vertex id order: the smallest colour not used by an
	// earlier ring sharing a node
	std::vector<uint32_t> colour(ncentre, 0), mark(kMaxColours, kNone);
	uint32_t ncol = 0;
	for (uint32_t u = 0; u < ncentre; u++) {
		for (uint32_t i = rs.node_off[u]; i < rs.node_off[u + 1]; i++) {
			const uint32_t x = rs.nodes[i];
			for (uint32_t j = hoff[x]; j < hoff[x + 1]; j++)
				if (hl[j] < u) mark[colour[hl[j]]] = u;
		}
		uint32_t c = 0;
		while (c < kMaxColours && mark[c] == u) c++;
		if (c == kMaxColours) return -1;
		colour[u] = c;
		ncol = std::max(ncol, c + 1);
	}
	rs.ncolours = ncol;
	std::vector<uint64_t> key(ncentre);
	for (uint32_t v = 0; v < ncentre; v++) key[v] = ((uint64_t)colour[v] << 32) | vert_rank[v];
	std::vector<uint32_t> idx(ncentre);
	for (uint32_t v = 0; v < ncentre; v++) idx[v] = v;
	std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
	rs.order = idx;
	rs.colour_begin.assign(ncol + 1, 0);
	for (uint32_t v = 0; v < ncentre; v++) rs.colour_begin[colour[v] + 1]++;
	for (uint32_t c = 0; c < ncol; c++) rs.colour_begin[c + 1] += rs.colour_begin[c];
	return 0;
}

int build_schedule(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, uint32_t mode,
                   uint32_t morton, Schedule& s) {
	std::vector<uint32_t> off, lst;
	incidence(tets, nverts, ntets, off, lst);
	if (cluster_and_colour(tets, ntets, off.data(), lst.data(), mode, s)) return -1;
	vertex_ranks(nodes, nverts, morton, s);
	cluster_order(nodes, nverts, tets, morton, s);
	return 0;
}

// Element schedule (hexes, T10s). The colouring runs over vertex ->
// element incidence lists: element e marks the colours of the earlier
// elements on its vertices with e and takes the smallest unmarked one.
int elem_schedule(const float* nodes, uint32_t nverts, const uint32_t* elems, uint32_t nel, uint32_t per,
                  uint32_t morton, ElemSchedule& es) {
	std::vector<uint32_t> off(nverts + 1, 0), lst((size_t)per * nel);
	for (size_t i = 0; i < (size_t)per * nel; i++) off[elems[i] + 1]++;
	for (uint32_t v = 0; v < nverts; v++) off[v + 1] += off[v];
	{
		std::vector<uint32_t> fill(off.begin(), off.end() - 1);
		for (uint32_t e = 0; e < nel; e++)
			for (uint32_t n = 0; n < per; n++) lst[fill[elems[per * (size_t)e + n]]++] = e;
	}
	std::vector<uint32_t> mark(kMaxElemColours, 0xffffffffu), colour(nel);
	uint32_t ncol = 0;
	for (uint32_t e = 0; e < nel; e++) {
		for (uint32_t n = 0; n < per; n++) {
			const uint32_t v = elems[per * (size_t)e + n];
			for (uint32_t i = off[v]; i < off[v + 1] && lst[i] < e; i++) mark[colour[lst[i]]] = e;
		}
		uint32_t c = 0;
		while (c < kMaxElemColours && mark[c] == e) c++;
		if (c == kMaxElemColours) return -1;
		colour[e] = c;
		ncol = std::max(ncol, c + 1);
	}
	const MortonFrame f = morton ? morton_frame(nodes, nverts) : MortonFrame{};
	std::vector<std::pair<uint64_t, uint32_t>> key(nel);
	for (uint32_t e = 0; e < nel; e++) {
		uint32_t k = e;
		if (morton) {
			float c[3] = {0.0f, 0.0f, 0.0f};
			for (uint32_t n = 0; n < per; n++)
				for (int j = 0; j < 3; j++) c[j] += nodes[3 * (size_t)elems[per * (size_t)e + n] + j];
			for (int j = 0; j < 3; j++) c[j] = c[j] / (float)per;
			k = f.code(c);
		}
		key[e] = {((uint64_t)colour[e] << 32) | k, e};
	}
	std::sort(key.begin(), key.end());
	es.ncolours = ncol;
	es.order.resize(nel);
	es.colour_begin.assign(ncol + 1, 0);
	for (uint32_t i = 0; i < nel; i++) {
		es.order[i] = key[i].second;
		es.colour_begin[colour[key[i].second] + 1]++;
	}
	for (uint32_t c = 0; c < ncol; c++) es.colour_begin[c + 1] += es.colour_begin[c];
	return 0;
}

void tet_edges(const uint32_t* tets, uint32_t ntets, uint32_t nverts, std::vector<uint32_t>& edges,
               std::vector<uint32_t>& t10) {
	// every tet edge instance, listed under its lower vertex in stream order
	std::vector<uint32_t> off(nverts + 1, 0), upper(6 * (size_t)ntets), inst(6 * (size_t)ntets);
	auto lo_hi = [&](uint32_t t, int k, uint32_t& lo, uint32_t& hi) {
		const uint32_t a = tets[4 * (size_t)t + rest::kT10EdgeNodes[k][0]], b = tets[4 * (size_t)t + rest::kT10EdgeNodes[k][1]];
		lo = std::min(a, b);
		hi = std::max(a, b);
	};
	for (uint32_t t = 0; t < ntets; t++)
		for (int k = 0; k < 6; k++) {
			uint32_t lo, hi;
			lo_hi(t, k, lo, hi);
			off[lo + 1]++;
		}
	for (uint32_t v = 0; v < nverts; v++) off[v + 1] += off[v];
	std::vector<uint32_t> cnt(nverts, 0);
	for (uint32_t t = 0; t < ntets; t++)
		for (int k = 0; k < 6; k++) {
			uint32_t lo, hi;
			lo_hi(t, k, lo, hi);
			const uint32_t id = 6 * t + (uint32_t)k;
			upper[id] = hi;
			inst[off[lo] + cnt[lo]++] = id;
		}
	// a later duplicate takes the list's last entry in its place
	for (uint32_t v = 0; v < nverts; v++) {
		uint32_t* L = inst.data() + off[v];
		for (uint32_t j = 0; j < cnt[v]; j++)
			for (uint32_t k = j + 1; k < cnt[v]; k++)
				if (upper[L[j]] == upper[L[k]]) L[k--] = L[--cnt[v]];
	}
	std::vector<uint32_t> first(nverts, 0);
	edges.clear();
	for (uint32_t v = 0; v < nverts; v++) {
		first[v] = (uint32_t)(edges.size() / 2);
		for (uint32_t j = 0; j < cnt[v]; j++) {
			edges.push_back(v);
			edges.push_back(upper[inst[off[v] + j]]);
		}
	}
	t10.resize(10 * (size_t)ntets);
	for (uint32_t t = 0; t < ntets; t++) {
		uint32_t* o = t10.data() + 10 * (size_t)t;
		for (int c = 0; c < 4; c++) o[c] = tets[4 * (size_t)t + c];
		for (int k = 0; k < 6; k++) {
			uint32_t lo, hi;
			lo_hi(t, k, lo, hi);
			uint32_t e = 0;
			while (edges[2 * (size_t)(first[lo] + e) + 1] != hi) e++;
			o[4 + k] = nverts + first[lo] + e;
		}
	}
}

void t10_init_rest(const float* nodes, uint32_t nverts, uint32_t ntets, const uint32_t* edges,
                   uint32_t nedges, const uint32_t* t10, float density, double* X, float* qep, float* w,
                   uint8_t* vflags) {
	const uint32_t n = nverts + nedges;
	for (size_t i = 0; i < 3 * (size_t)nverts; i++) X[i] = (double)nodes[i];
	for (uint32_t e = 0; e < nedges; e++)
		for (int k = 0; k < 3; k++)
			X[3 * (size_t)(nverts + e) + k] = 0.5 * (X[3 * (size_t)edges[2 * e] + k] + X[3 * (size_t)edges[2 * e + 1] + k]);
	// AABB and Left / Right flags over every node (XPBDFEM/Geo.cpp:870-890)
	float mn[3] = {1.0e24f, 1.0e24f, 1.0e24f}, mx[3] = {-1.0e24f, -1.0e24f, -1.0e24f};
	for (uint32_t i = 0; i < n; i++) {
		w[i] = 0.0f;
		for (int k = 0; k < 3; k++) {
			mn[k] = fminf(mn[k], (float)X[3 * (size_t)i + k]);
			mx[k] = fmaxf(mx[k], (float)X[3 * (size_t)i + k]);
		}
	}
	for (uint32_t i = 0; i < n; i++) vflags[i] = rest::vertex_flags((float)X[3 * (size_t)i], mn[0], mx[0]);
	for (uint32_t t = 0; t < ntets; t++) {
		const uint32_t* is = t10 + 10 * (size_t)t;
		float m[10];
		rest::t10(X, is, density, qep + (size_t)rest::kT10Rec * t, m);
		for (int c = 0; c < 10; c++) w[is[c]] += m[c];
	}
	for (uint32_t i = 0; i < n; i++) w[i] = 1.0f / w[i];
}

// GeoQuadratic3d's 27 indices of hex h with corners c (XPBDFEM/Geo.cpp:
// 904-931): node i + 3j + 9k of its 3x3x3 grid is a corner, nverts + an
// edge (EdgeFromVerts), nverts + ne + a quad (QuadFromVerts, either winding)
// or nverts + ne + nq + h; efirst / qfirst: each vertex's first edge / quad.
static void h27_node_ids(const uint32_t* c, uint32_t h, uint32_t nverts, const std::vector<uint32_t>& edges,
                         const std::vector<uint32_t>& efirst, const std::vector<uint32_t>& quads,
                         const std::vector<uint32_t>& qfirst, uint32_t ne, uint32_t nq, uint32_t* out) {
	for (int n = 0; n < 27; n++) {
		const int ix[3] = {n % 3, (n / 3) % 3, n / 9};
		int mid = 0, lo = 0, free = 0;
		for (int a = 0; a < 3; a++) {
			mid += ix[a] == 1;
			lo |= (ix[a] == 2) << a;
			free |= (ix[a] == 1) << a;
		}
		uint32_t id;
		if (mid == 0) {
			id = c[lo];
		} else if (mid == 1) {
			const uint32_t a = c[lo], b = c[lo | free];
			const uint32_t l = std::min(a, b), u = std::max(a, b);
			uint32_t e = 0;
			while (edges[2 * (size_t)(efirst[l] + e) + 1] != u) e++;
			id = nverts + efirst[l] + e;
		} else if (mid == 2) {
			const int f1 = free & 1 ? 1 : 2, f2 = free & 4 ? 4 : 2;
			const uint32_t vs[4] = {c[lo], c[lo | f1], c[lo | f1 | f2], c[lo | f2]};
			uint32_t best = 0;
			for (uint32_t j = 1; j < 4; j++)
				if (vs[j] < vs[best]) best = j;
			const uint32_t v0 = vs[best], v1 = vs[(best + 1) % 4], v2 = vs[(best + 2) % 4], v3 = vs[(best + 3) % 4];
			uint32_t q = 0;
			for (;; q++) {
				const uint32_t* Q = &quads[4 * (size_t)(qfirst[v0] + q)];
				if ((Q[1] == v1 && Q[2] == v2 && Q[3] == v3) || (Q[1] == v3 && Q[2] == v2 && Q[3] == v1)) break;
			}
			id = nverts + ne + qfirst[v0] + q;
		} else {
			id = nverts + ne + nq + h;
		}
		out[n] = id;
	}
}

void hex_edges_quads(const uint32_t* hexes, uint32_t nhexes, uint32_t nverts, std::vector<uint32_t>& edges,
                     std::vector<uint32_t>& quads, std::vector<uint32_t>& h27) {
	static const int he[12][2] = {{0, 1}, {0, 2}, {0, 4}, {1, 3}, {1, 5}, {2, 3}, {2, 6}, {3, 7}, {4, 5}, {4, 6}, {5, 7}, {6, 7}};
	static const int hq[6][4] = {{0, 1, 3, 2}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 2, 6, 4}, {1, 3, 7, 5}};
	// edge and quad instances, each under the vertex it is filed under
	std::vector<uint32_t> eoff(nverts + 1, 0), qoff(nverts + 1, 0);
	std::vector<uint32_t> eup(12 * (size_t)nhexes), einst(12 * (size_t)nhexes), qv(24 * (size_t)nhexes),
	    qinst(6 * (size_t)nhexes);
	auto face = [&](uint32_t h, int f, uint32_t out[4]) {  // rotated to start at its smallest vertex
		uint32_t vs[4], best = 0;
		for (int j = 0; j < 4; j++) vs[j] = hexes[8 * (size_t)h + hq[f][j]];
		for (uint32_t j = 1; j < 4; j++)
			if (vs[j] < vs[best]) best = j;
		for (uint32_t j = 0; j < 4; j++) out[j] = vs[(best + j) % 4];
	};
	for (uint32_t h = 0; h < nhexes; h++) {
		for (int k = 0; k < 12; k++)
			eoff[std::min(hexes[8 * (size_t)h + he[k][0]], hexes[8 * (size_t)h + he[k][1]]) + 1]++;
		for (int f = 0; f < 6; f++) {
			uint32_t v[4];
			face(h, f, v);
			qoff[v[0] + 1]++;
		}
	}
	for (uint32_t v = 0; v < nverts; v++) {
		eoff[v + 1] += eoff[v];
		qoff[v + 1] += qoff[v];
	}
	std::vector<uint32_t> ecnt(nverts, 0), qcnt(nverts, 0);
	for (uint32_t h = 0; h < nhexes; h++) {
		for (int k = 0; k < 12; k++) {
			const uint32_t a = hexes[8 * (size_t)h + he[k][0]], b = hexes[8 * (size_t)h + he[k][1]];
			const uint32_t lo = std::min(a, b), id = 12 * h + (uint32_t)k;
			eup[id] = std::max(a, b);
			einst[eoff[lo] + ecnt[lo]++] = id;
		}
		for (int f = 0; f < 6; f++) {
			const uint32_t id = 6 * h + (uint32_t)f;
			face(h, f, &qv[4 * (size_t)id]);
			qinst[qoff[qv[4 * (size_t)id]] + qcnt[qv[4 * (size_t)id]]++] = id;
		}
	}
	// a later duplicate takes the list's last entry in its place; a quad is a
	// duplicate in either winding
	for (uint32_t v = 0; v < nverts; v++) {
		uint32_t* L = einst.data() + eoff[v];
		for (uint32_t j = 0; j < ecnt[v]; j++)
			for (uint32_t k = j + 1; k < ecnt[v]; k++)
				if (eup[L[j]] == eup[L[k]]) L[k--] = L[--ecnt[v]];
		uint32_t* Q = qinst.data() + qoff[v];
		for (uint32_t j = 0; j < qcnt[v]; j++)
			for (uint32_t k = j + 1; k < qcnt[v]; k++) {
				const uint32_t* a = &qv[4 * (size_t)Q[j]];
				const uint32_t* b = &qv[4 * (size_t)Q[k]];
				if ((a[1] == b[1] && a[2] == b[2] && a[3] == b[3]) || (a[1] == b[3] && a[2] == b[2] && a[3] == b[1]))
					Q[k--] = Q[--qcnt[v]];
			}
	}
	std::vector<uint32_t> efirst(nverts), qfirst(nverts);
	edges.clear();
	quads.clear();
	for (uint32_t v = 0; v < nverts; v++) {
		efirst[v] = (uint32_t)(edges.size() / 2);
		for (uint32_t j = 0; j < ecnt[v]; j++) {
			edges.push_back(v);
			edges.push_back(eup[einst[eoff[v] + j]]);
		}
		qfirst[v] = (uint32_t)(quads.size() / 4);
		for (uint32_t j = 0; j < qcnt[v]; j++)
			for (int k = 0; k < 4; k++) quads.push_back(qv[4 * (size_t)qinst[qoff[v] + j] + k]);
	}
	const uint32_t ne = (uint32_t)(edges.size() / 2), nq = (uint32_t)(quads.size() / 4);
	h27.resize(27 * (size_t)nhexes);
	for (uint32_t h = 0; h < nhexes; h++)
		h27_node_ids(hexes + 8 * (size_t)h, h, nverts, edges, efirst, quads, qfirst, ne, nq, &h27[27 * (size_t)h]);
}

void quad_mesh(const uint32_t* idx, uint32_t count, uint32_t nverts, std::vector<uint32_t>& edges,
               std::vector<uint32_t>& quads, std::vector<uint32_t>& t10, std::vector<uint32_t>& h27) {
	static const int te[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
	static const int he[12][2] = {{0, 1}, {0, 2}, {0, 4}, {1, 3}, {1, 5}, {2, 3}, {2, 6}, {3, 7}, {4, 5}, {4, 6}, {5, 7}, {6, 7}};
	static const int hq[6][4] = {{0, 1, 3, 2}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 2, 6, 4}, {1, 3, 7, 5}};
	// instances in stream order, each element filing its edges (and a hex
	// its faces) as it comes; two walks: count per vertex, then file
	std::vector<uint32_t> eoff(nverts + 1, 0), qoff(nverts + 1, 0), ecnt(nverts, 0), qcnt(nverts, 0);
	std::vector<uint32_t> eup, einst, qv, qinst;
	uint32_t ntets = 0, nhexes = 0;
	for (int pass = 0; pass < 2; pass++) {
		uint32_t eid = 0, qid = 0;
		for (uint32_t i = 0; i < count; i += 1 + idx[i]) {
			const uint32_t* c = idx + i + 1;
			const bool tet = idx[i] == 4u;
			if (pass == 0) (tet ? ntets : nhexes)++;
			for (int k = 0; k < (tet ? 6 : 12); k++, eid++) {
				const uint32_t a = c[tet ? te[k][0] : he[k][0]], b = c[tet ? te[k][1] : he[k][1]];
				const uint32_t lo = std::min(a, b);
				if (pass == 0) {
					eoff[lo + 1]++;
				} else {
					eup[eid] = std::max(a, b);
					einst[eoff[lo] + ecnt[lo]++] = eid;
				}
			}
			if (tet) continue;
			for (int f = 0; f < 6; f++, qid++) {
				uint32_t vs[4], best = 0;
				for (int j = 0; j < 4; j++) vs[j] = c[hq[f][j]];
				for (uint32_t j = 1; j < 4; j++)
					if (vs[j] < vs[best]) best = j;
				if (pass == 0) {
					qoff[vs[best] + 1]++;
				} else {
					for (uint32_t j = 0; j < 4; j++) qv[4 * (size_t)qid + j] = vs[(best + j) % 4];
					qinst[qoff[vs[best]] + qcnt[vs[best]]++] = qid;
				}
			}
		}
		if (pass == 0) {
			for (uint32_t v = 0; v < nverts; v++) {
				eoff[v + 1] += eoff[v];
				qoff[v + 1] += qoff[v];
			}
			eup.resize(eoff[nverts]);
			einst.resize(eoff[nverts]);
			qv.resize(4 * (size_t)qoff[nverts]);
			qinst.resize(qoff[nverts]);
		}
	}
	for (uint32_t v = 0; v < nverts; v++) {
		uint32_t* L = einst.data() + eoff[v];
		for (uint32_t j = 0; j < ecnt[v]; j++)
			for (uint32_t k = j + 1; k < ecnt[v]; k++)
				if (eup[L[j]] == eup[L[k]]) L[k--] = L[--ecnt[v]];
		uint32_t* Q = qinst.data() + qoff[v];
		for (uint32_t j = 0; j < qcnt[v]; j++)
			for (uint32_t k = j + 1; k < qcnt[v]; k++) {
				const uint32_t* a = &qv[4 * (size_t)Q[j]];
				const uint32_t* b = &qv[4 * (size_t)Q[k]];
				if ((a[1] == b[1] && a[2] == b[2] && a[3] == b[3]) || (a[1] == b[3] && a[2] == b[2] && a[3] == b[1]))
					Q[k--] = Q[--qcnt[v]];
			}
	}
	std::vector<uint32_t> efirst(nverts), qfirst(nverts);
	edges.clear();
	quads.clear();
	for (uint32_t v = 0; v < nverts; v++) {
		efirst[v] = (uint32_t)(edges.size() / 2);
		for (uint32_t j = 0; j < ecnt[v]; j++) {
			edges.push_back(v);
			edges.push_back(eup[einst[eoff[v] + j]]);
		}
		qfirst[v] = (uint32_t)(quads.size() / 4);
		for (uint32_t j = 0; j < qcnt[v]; j++)
			for (int k = 0; k < 4; k++) quads.push_back(qv[4 * (size_t)qinst[qoff[v] + j] + k]);
	}
	const uint32_t ne = (uint32_t)(edges.size() / 2), nq = (uint32_t)(quads.size() / 4);
	t10.resize(10 * (size_t)ntets);
	h27.resize(27 * (size_t)nhexes);
	uint32_t t = 0, h = 0;
	for (uint32_t i = 0; i < count; i += 1 + idx[i]) {
		const uint32_t* c = idx + i + 1;
		if (idx[i] != 4u) {
			h27_node_ids(c, h, nverts, edges, efirst, quads, qfirst, ne, nq, &h27[27 * (size_t)h]);
			h++;
			continue;
		}
		uint32_t* o = &t10[10 * (size_t)t++];
		for (int k = 0; k < 4; k++) o[k] = c[k];
		for (int k = 0; k < 6; k++) {
			const uint32_t a = c[te[k][0]], b = c[te[k][1]];
			const uint32_t l = std::min(a, b), u = std::max(a, b);
			uint32_t e = 0;
			while (edges[2 * (size_t)(efirst[l] + e) + 1] != u) e++;
			o[4 + k] = nverts + efirst[l] + e;
		}
	}
}

void qmixed_init_rest(const float* nodes, uint32_t nverts, uint32_t ntets, const uint32_t* hexes, uint32_t nhexes,
                      const uint32_t* edges, uint32_t nedges, const uint32_t* quads, uint32_t nquads, const uint32_t* t10,
                      const uint32_t* h27, float density, double* X, float* qep, float* hep, float* w, uint8_t* vflags) {
	const uint32_t n = nverts + nedges + nquads + nhexes;
	for (size_t i = 0; i < 3 * (size_t)nverts; i++) X[i] = (double)nodes[i];
	for (uint32_t e = 0; e < nedges; e++)
		for (int k = 0; k < 3; k++)
			X[3 * (size_t)(nverts + e) + k] = 0.5 * (X[3 * (size_t)edges[2 * e] + k] + X[3 * (size_t)edges[2 * e + 1] + k]);
	for (uint32_t q = 0; q < nquads; q++) {
		const uint32_t* v = quads + 4 * (size_t)q;
		for (int k = 0; k < 3; k++)
			X[3 * (size_t)(nverts + nedges + q) + k] =
			    0.25 * (X[3 * (size_t)v[0] + k] + X[3 * (size_t)v[1] + k] + X[3 * (size_t)v[2] + k] + X[3 * (size_t)v[3] + k]);
	}
	for (uint32_t h = 0; h < nhexes; h++)
		for (int k = 0; k < 3; k++) {
			double s = X[3 * (size_t)hexes[8 * (size_t)h] + k];
			for (int c = 1; c < 8; c++) s = s + X[3 * (size_t)hexes[8 * (size_t)h + c] + k];
			X[3 * (size_t)(nverts + nedges + nquads + h) + k] = 0.125 * s;
		}
	float mn[3] = {1.0e24f, 1.0e24f, 1.0e24f}, mx[3] = {-1.0e24f, -1.0e24f, -1.0e24f};
	for (uint32_t i = 0; i < n; i++) {
		w[i] = 0.0f;
		for (int k = 0; k < 3; k++) {
			mn[k] = fminf(mn[k], (float)X[3 * (size_t)i + k]);
			mx[k] = fmaxf(mx[k], (float)X[3 * (size_t)i + k]);
		}
	}
	for (uint32_t i = 0; i < n; i++) vflags[i] = rest::vertex_flags((float)X[3 * (size_t)i], mn[0], mx[0]);
	// the masses of every T10, then of every H27, in element order
	for (uint32_t t = 0; t < ntets; t++) {
		const uint32_t* is = t10 + 10 * (size_t)t;
		float m[10];
		rest::t10(X, is, density, qep + (size_t)rest::kT10Rec * t, m);
		for (int c = 0; c < 10; c++) w[is[c]] += m[c];
	}
	(void)rest::h27_tables();
	for (uint32_t h = 0; h < nhexes; h++) {
		float m[27];
		rest::h27(X, h27 + 27 * (size_t)h, density, hep + (size_t)rest::kH27Rec * h, m);
		for (int c = 0; c < 27; c++) w[h27[27 * (size_t)h + c]] += m[c];
	}
	for (uint32_t i = 0; i < n; i++) w[i] = 1.0f / w[i];
}

void h27_init_rest(const float* nodes, uint32_t nverts, const uint32_t* hexes, uint32_t nhexes, const uint32_t* edges,
                   uint32_t nedges, const uint32_t* quads, uint32_t nquads, const uint32_t* h27, float density,
                   double* X, float* ep, float* w, uint8_t* vflags) {
	const uint32_t n = nverts + nedges + nquads + nhexes;
	for (size_t i = 0; i < 3 * (size_t)nverts; i++) X[i] = (double)nodes[i];
	for (uint32_t e = 0; e < nedges; e++)
		for (int k = 0; k < 3; k++)
			X[3 * (size_t)(nverts + e) + k] = 0.5 * (X[3 * (size_t)edges[2 * e] + k] + X[3 * (size_t)edges[2 * e + 1] + k]);
	for (uint32_t q = 0; q < nquads; q++) {
		const uint32_t* v = quads + 4 * (size_t)q;
		for (int k = 0; k < 3; k++)
			X[3 * (size_t)(nverts + nedges + q) + k] =
			    0.25 * (X[3 * (size_t)v[0] + k] + X[3 * (size_t)v[1] + k] + X[3 * (size_t)v[2] + k] + X[3 * (size_t)v[3] + k]);
	}
	for (uint32_t h = 0; h < nhexes; h++)
		for (int k = 0; k < 3; k++) {
			double s = X[3 * (size_t)hexes[8 * (size_t)h] + k];
			for (int c = 1; c < 8; c++) s = s + X[3 * (size_t)hexes[8 * (size_t)h + c] + k];
			X[3 * (size_t)(nverts + nedges + nquads + h) + k] = 0.125 * s;
		}
	float mn[3] = {1.0e24f, 1.0e24f, 1.0e24f}, mx[3] = {-1.0e24f, -1.0e24f, -1.0e24f};
	for (uint32_t i = 0; i < n; i++) {
		w[i] = 0.0f;
		for (int k = 0; k < 3; k++) {
			mn[k] = fminf(mn[k], (float)X[3 * (size_t)i + k]);
			mx[k] = fmaxf(mx[k], (float)X[3 * (size_t)i + k]);
		}
	}
	for (uint32_t i = 0; i < n; i++) vflags[i] = rest::vertex_flags((float)X[3 * (size_t)i], mn[0], mx[0]);
	// the records on all host threads (each H27's own), then the masses
	// accumulated in element order
	std::vector<float> m(27 * (size_t)nhexes);
	(void)rest::h27_tables();  // built once, before the threads read it
	const uint32_t nth = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
	auto work = [&](uint32_t t) {
		for (uint32_t h = t; h < nhexes; h += nth)
			rest::h27(X, h27 + 27 * (size_t)h, density, ep + (size_t)rest::kH27Rec * h, &m[27 * (size_t)h]);
	};
	if (nhexes < 256 || nth == 1) {
		work(0);
		for (uint32_t t = 1; t < nth; t++) work(t);
	} else {
		std::vector<std::thread> pool;
		for (uint32_t t = 0; t < nth; t++) pool.emplace_back(work, t);
		for (std::thread& th : pool) th.join();
	}
	for (uint32_t h = 0; h < nhexes; h++)
		for (int c = 0; c < 27; c++) w[h27[27 * (size_t)h + c]] += m[27 * (size_t)h + c];
	for (uint32_t i = 0; i < n; i++) w[i] = 1.0f / w[i];
}

}  // namespace xfem
