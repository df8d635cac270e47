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

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "xfem_device.cuh"
#include "xfem_internal.h"

namespace xfem {

namespace {

// Adjoint tape: the owner of a vertex records O right after the advance
// (the position the substep starts from, with the inverse mass the solves
// use) and D right before it, in one 32-byte sector, and, from the second
// substep of a launch on, the tip trajectory (O is then the position after
// the previous substep).
__device__ __forceinline__ void tape_vertex(const DevCtx& C, uint32_t v, const float4& O, const float4& Dbefore,
                                            uint32_t s, bool first) {
	float4* p = C.tape_v + 2 * ((size_t)s * C.nverts + v);
	__stcs(p, O);
	__stcs(p + 1, Dbefore);
	if (!first) {
		const int q = __ldg(C.tip_of + v);
		if (q >= 0) C.traj[(size_t)(C.sub_base + s - 1) * C.ntips + q] = O;
	}
}

// Adjoint tape: the input displacement of one solve's four vertices.
__device__ __forceinline__ void tape_tet(const DevCtx& C, uint32_t s, uint32_t row, uint32_t lane, const float4 D[4]) {
	float4* p = C.tape_t + ((size_t)s * C.ntrows + row) * 3 * kLanes + lane;
	__stcs(p, make_float4(D[0].x, D[0].y, D[0].z, D[1].x));
	__stcs(p + kLanes, make_float4(D[1].y, D[1].z, D[2].x, D[2].y));
	__stcs(p + 2 * kLanes, make_float4(D[2].z, D[3].x, D[3].y, D[3].z));
}

// ---- damping after the velocity update (GeoLinear3d::Damp) ------------------
// State during the damping sweeps: vert[2v] = (X, w), vert[2v+1] = (V, bits).

// Whether tet row `row` (lane `lane`) of body bp is damped at this tick, and
// with which Rayleigh ratio and PBD fraction (XPBDFEM/Geo.cpp:346-352,
// 792-798): the amortized type damps one eighth of the body's order per
// tick, x 8.
struct DampTet {
	bool on;
	float rayleigh, pbd;
};

__device__ __forceinline__ DampTet damp_of(const DevCtx& C, const BodyParams& bp, uint32_t row, uint32_t lane,
                                           uint32_t tick, int kind) {
	const uint32_t type = __ldg(&bp.rayleigh_type);
	const bool amort = type == 3u;
	DampTet d = {false, 0.0f, 0.0f};
	if (kind == 0) {
		d.rayleigh = __ldg(&bp.damping) * (amort ? 8.0f : 1.0f);
		d.on = type >= 2u && d.rayleigh > 0.0f;
	} else {
		d.on = __ldg(&bp.pbd_on) != 0u;
	}
	if (!d.on) return d;
	const size_t k = (size_t)row * kLanes + lane;
	if (amort) {
		const uint32_t nt = __ldg(&bp.ntets), f = __ldg(C.tflat + k), m = tick % 8u;
		d.on = f >= nt * m / 8u && f < nt * (m + 1u) / 8u;
	}
	if (kind == 1) d.pbd = fminf(1.0f, (amort ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff)) / __ldg(C.tarea + k));
	return d;
}

// Header word of a cluster lane: nv | nt << 4 | advance mask << 8 | body << 16.
// A vertex is advanced (previous substep finalized, next one predicted) by
// the lowest-colour cluster touching it, just before that cluster's solve.

template <bool LAMBDAS, bool TAPE, bool EXT>
__device__ __forceinline__ void run_chunk_cube(const DevCtx& C, Stage& st, int next, const uint4& mnext, uint32_t lane,
                                               bool first, float dt, float inv_dt, float inv_dt2, uint32_t trow,
                                               uint32_t s_launch, uint32_t chunk, bool finish_last) {
	const float4* rec = reinterpret_cast<const float4*>(st.buf);
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(st.buf + 2048u * 6u);
	const uint32_t* vids = hdrs + kLanes;
	const uint32_t hdr = hdrs[lane];
	const bool live = (hdr & 15u) != 0;
	const uint32_t mask = (hdr >> 8) & 0xffu;
	uint32_t vid[8];
	float4 O[8], D[8];
	bool fin = false;  // this pass is the lane's last of the substep (its body runs no volume passes)
	if (live) {
		const Mat mat = load_mat(C.bodies, hdr >> 16);
		fin = EXT && finish_last && mat.nvol == 0u;
#pragma unroll
		for (int s = 0; s < 8; s++) vid[s] = vids[s * kLanes + lane];
#pragma unroll
		for (int s = 0; s < 8; s++) ld_vertex(C.vert + 2 * (size_t)vid[s], O[s], D[s]);
#pragma unroll
		for (int s = 0; s < 8; s++)
			if (mask & (1u << s)) {
				const float4 Dbefore = D[s];
				advance_vertex(C, vid[s], O[s], D[s], first, dt, inv_dt);
				if (TAPE) tape_vertex(C, vid[s], O[s], Dbefore, s_launch, first);
			}
#pragma unroll
		for (int t = 0; t < 6; t++) {
			const float4* r = rec + t * 4 * kLanes + lane;
			const TetRec tr = {r[0], r[kLanes], r[2 * kLanes], r[3 * kLanes]};
			const float4 Ot[4] = {O[cube_slot(t, 0)], O[cube_slot(t, 1)], O[cube_slot(t, 2)], O[cube_slot(t, 3)]};
			float4 Dt[4] = {D[cube_slot(t, 0)], D[cube_slot(t, 1)], D[cube_slot(t, 2)], D[cube_slot(t, 3)]};
			if (TAPE) tape_tet(C, s_launch, trow + t, lane, Dt);
			const float2 lam = solve_tet<EXT>(mat, tr, inv_dt, inv_dt2, Ot, Dt);
#pragma unroll
			for (int k = 0; k < 4; k++) D[cube_slot(t, k)] = Dt[k];
			if (LAMBDAS) C.tlam[(size_t)(trow + t) * kLanes + lane] = lam;
		}
	}
	if (next >= 0) stage_issue_m(C, st, (uint32_t)next, mnext, lane);  // buffer consumed: prefetch
	if (live) {
		// with damping sweeps, the vertex's last solve of the substep finishes
		// it (to the canonical X, V that the sweeps work on)
		const uint32_t last = fin ? __ldg(C.lastmask + (size_t)chunk * kLanes + lane) : 0u;
		// O changes only where this cluster advanced or finished the vertex
		// (then the whole 32-byte state is stored); no other cluster of the
		// pass touches these vertices
#pragma unroll
		for (int s = 0; s < 8; s++) {
			if (EXT && (last & (1u << s))) finalize_vertex(C, vid[s], O[s], D[s], inv_dt);
			if ((mask | last) & (1u << s))
				st_vertex(C.vert + 2 * (size_t)vid[s], O[s], D[s]);
			else  // only D moved: a 16-byte store
				__stcg(C.vert + 2 * (size_t)vid[s] + 1, D[s]);
		}
	}
}

// One warp processes one resident chunk; lane = cluster. `next` >= 0 is the
// warp's next chunk: its copy is issued as soon as this chunk's records have
// been consumed, so it overlaps the write-back and what follows.
template <bool LAMBDAS, bool TAPE = false, bool EXT = false>
__device__ __forceinline__ void run_chunk(const DevCtx& C, Stage& st, uint32_t chunk, int next, uint32_t lane, bool first,
                                          float dt, float inv_dt, float inv_dt2, uint32_t s_launch = 0,
                                          bool finish_last = false) {
	// the staged chunk's descriptor came with its copy; the next one's is
	// loaded now, off the critical path of the prefetch
	const uint4 m = st.meta;
	const uint4 mnext = next >= 0 ? __ldg(reinterpret_cast<const uint4*>(C.chunks) + next) : make_uint4(0u, 0u, 0u, 0u);
	const uint32_t ntmax = m.z & 0xffu, nvmax = (m.z >> 8) & 0xffu, trow = m.w;
	if (m.z & kShapeCube) {
		run_chunk_cube<LAMBDAS, TAPE, EXT>(C, st, next, mnext, lane, first, dt, inv_dt, inv_dt2, trow, s_launch, chunk,
		                                    finish_last);
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
	bool fin = false;
	if (nv) {
		const Mat mat = load_mat(C.bodies, hdr >> 16);
		fin = EXT && finish_last && mat.nvol == 0u;
#pragma unroll
		for (uint32_t s = 0; s < kMaxClusterVerts; s++)
			if (s < nv) vid[s] = vids[s * kLanes + lane];
#pragma unroll
		for (uint32_t s = 0; s < kMaxClusterVerts; s++) {
			if (s < nv) {
				float4 O, D;
				ld_vertex(C.vert + 2 * (size_t)vid[s], O, D);
				if (mask & (1u << s)) {
					const float4 Dbefore = D;
					advance_vertex(C, vid[s], O, D, first, dt, inv_dt);
					if (TAPE) tape_vertex(C, vid[s], O, Dbefore, s_launch, first);
				}
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
			if (TAPE) tape_tet(C, s_launch, trow + t, lane, D);
			const float2 lam = solve_tet<EXT>(mat, tr, inv_dt, inv_dt2, O, D);
			sD[s0 * kLanes] = D[0];
			sD[s1 * kLanes] = D[1];
			sD[s2 * kLanes] = D[2];
			sD[s3 * kLanes] = D[3];
			if (LAMBDAS) C.tlam[(size_t)(trow + t) * kLanes + lane] = lam;
		}
	}
	if (next >= 0) stage_issue_m(C, st, (uint32_t)next, mnext, lane);  // buffer consumed: prefetch
	if (nv) {
		const uint32_t last = fin ? __ldg(C.lastmask + (size_t)chunk * kLanes + lane) : 0u;
#pragma unroll
		for (uint32_t s = 0; s < kMaxClusterVerts; s++) {
			if (s < nv) {
				float4 O = sO[s * kLanes], D = sD[s * kLanes];
				if (EXT && (last & (1u << s))) finalize_vertex(C, vid[s], O, D, inv_dt);
				st_vertex(C.vert + 2 * (size_t)vid[s], O, D);
			}
		}
	}
}

// The damping and volume sweeps keep two 128-bit vertex accesses: with the
// 256-bit form in both of them, ptxas (CUDA 13.0) fails on this file.

// Volume sweep k (1-based) over a resident chunk: SolveElementVolume on each
// tet of the cluster in order (GeoLinear3d::Constrain, XPBDFEM/Geo.cpp:
// 780-783), for lanes whose body runs at least k volume passes. The state is
// (O, D), as in the solve sweep; only D changes, except that with damping
// sweeps (finish) the body's last volume sweep finishes the vertices whose
// last solve this cluster makes. CUBE: canonical cube chunks, all in
// registers. Not inlined, like the damping passes.
template <bool CUBE>
__device__ __noinline__ void vol_chunk(const DevCtx& C, Stage& st, uint32_t chunk, uint32_t ntmax, uint32_t nvmax,
                                       int next, uint32_t lane, float inv_dt, float inv_dt2, uint32_t k, bool finish) {
	constexpr uint32_t NV = CUBE ? 8u : kMaxClusterVerts;
	constexpr uint32_t NT = CUBE ? 6u : kMaxClusterTets;
	const float4* rec = reinterpret_cast<const float4*>(st.buf);
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(st.buf + 2048u * ntmax);
	const uint32_t* vids = hdrs + kLanes;
	const uint32_t* slots = vids + kLanes * nvmax;
	const uint32_t hdr = hdrs[lane];
	const uint32_t nv = CUBE ? 8u : (hdr & 15u), nt = CUBE ? 6u : ((hdr >> 4) & 15u);
	bool live = (hdr & 15u) != 0;
	uint32_t vid[NV], last = 0;
	float4 O[NV], D[NV];
	if (live) {
		const Mat mat = load_mat(C.bodies, hdr >> 16);
		live = mat.nvol >= k;
		if (finish && mat.nvol == k) last = __ldg(C.lastmask + (size_t)chunk * kLanes + lane);
		if (live) {
#pragma unroll
			for (uint32_t s = 0; s < NV; s++) {
				if (s < nv) {
					vid[s] = vids[s * kLanes + lane];
					O[s] = __ldcg(C.vert + 2 * (size_t)vid[s]);
					D[s] = __ldcg(C.vert + 2 * (size_t)vid[s] + 1);
				}
			}
#pragma unroll
			for (uint32_t t = 0; t < NT; t++) {
				if (t < nt) {
					const uint32_t sl = CUBE ? (uint32_t)(cube_slot(t, 0) | cube_slot(t, 1) << 4 | cube_slot(t, 2) << 8 |
					                                      cube_slot(t, 3) << 12)
					                         : slots[t * kLanes + lane];
					const float4* r = rec + t * 4 * kLanes + lane;
					const TetRec tr = {r[0], r[kLanes], r[2 * kLanes], r[3 * kLanes]};
					float4 Ot[4], Dt[4];
#pragma unroll
					for (int j = 0; j < 4; j++) {
						Ot[j] = O[(sl >> (4 * j)) & 15u];
						Dt[j] = D[(sl >> (4 * j)) & 15u];
					}
					volume_tet(mat, tr, inv_dt2, Ot, Dt);
#pragma unroll
					for (int j = 0; j < 4; j++) D[(sl >> (4 * j)) & 15u] = Dt[j];
				}
			}
		}
	}
	if (next >= 0) stage_issue(C, st, (uint32_t)next, lane);  // records consumed: prefetch
	if (live) {
#pragma unroll
		for (uint32_t s = 0; s < NV; s++) {
			if (s < nv) {
				if (last & (1u << s)) {
					finalize_vertex(C, vid[s], O[s], D[s], inv_dt);
					__stcg(C.vert + 2 * (size_t)vid[s], O[s]);
				}
				__stcg(C.vert + 2 * (size_t)vid[s] + 1, D[s]);
			}
		}
	}
}

__device__ __forceinline__ void run_vol_chunk(const DevCtx& C, Stage& st, uint32_t chunk, int next, uint32_t lane,
                                              float inv_dt, float inv_dt2, uint32_t k, bool finish) {
	const uint4 m = __ldg(reinterpret_cast<const uint4*>(C.chunks) + chunk);
	const uint32_t ntmax = m.z & 0xffu, nvmax = (m.z >> 8) & 0xffu;
	if (m.z & kShapeCube)
		vol_chunk<true>(C, st, chunk, ntmax, nvmax, next, lane, inv_dt, inv_dt2, k, finish);
	else
		vol_chunk<false>(C, st, chunk, ntmax, nvmax, next, lane, inv_dt, inv_dt2, k, finish);
}

// One damping pass over a resident chunk (KIND 0: element Rayleigh damping,
// 1: PBD damping); lane = cluster, tets in the cluster's order. The state is
// the canonical (X, V): each vertex's last solve of the substep finished it.
// Only velocities change. CUBE: canonical cube chunks, all in registers. Not
// inlined: the damping passes then cost the solve path no registers.
template <bool CUBE, int KIND>
__device__ __noinline__ void damp_chunk(const DevCtx& C, Stage& st, uint32_t ntmax, uint32_t nvmax, uint32_t trow,
                                        int next, uint32_t lane, float inv_dt, uint32_t tick) {
	constexpr uint32_t NV = CUBE ? 8u : kMaxClusterVerts;
	constexpr uint32_t NT = CUBE ? 6u : kMaxClusterTets;
	const float4* rec = reinterpret_cast<const float4*>(st.buf);
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(st.buf + 2048u * ntmax);
	const uint32_t* vids = hdrs + kLanes;
	const uint32_t* slots = vids + kLanes * nvmax;
	const uint32_t hdr = hdrs[lane];
	const bool live = (hdr & 15u) != 0;
	const uint32_t nv = CUBE ? 8u : (hdr & 15u), nt = CUBE ? 6u : ((hdr >> 4) & 15u);
	uint32_t vid[NV];
	float4 X[NV], V[NV];
	if (live) {
		const BodyParams& bp = C.bodies[hdr >> 16];
		const Mat mat = load_mat(C.bodies, hdr >> 16);
#pragma unroll
		for (uint32_t k = 0; k < NV; k++) {
			if (k < nv) {
				vid[k] = vids[k * kLanes + lane];
				X[k] = __ldcg(C.vert + 2 * (size_t)vid[k]);
				V[k] = __ldcg(C.vert + 2 * (size_t)vid[k] + 1);
			}
		}
#pragma unroll
		for (uint32_t t = 0; t < NT; t++) {
			if (t < nt) {
				const DampTet d = damp_of(C, bp, trow + t, lane, tick, KIND);
				if (d.on) {
					const uint32_t sl = CUBE ? (uint32_t)(cube_slot(t, 0) | cube_slot(t, 1) << 4 | cube_slot(t, 2) << 8 |
					                                      cube_slot(t, 3) << 12)
					                         : slots[t * kLanes + lane];
					float4 Xt[4], Vt[4];
#pragma unroll
					for (int k = 0; k < 4; k++) {
						Xt[k] = X[(sl >> (4 * k)) & 15u];
						Vt[k] = V[(sl >> (4 * k)) & 15u];
					}
					if (KIND == 0) {
						const float4* r = rec + t * 4 * kLanes + lane;
						const TetRec tr = {r[0], r[kLanes], r[2 * kLanes], r[3 * kLanes]};
						rayleigh_tet(mat, tr, Xt, Vt, inv_dt, d.rayleigh);
					} else {
						pbd_tet(Xt, Vt, d.pbd);
					}
#pragma unroll
					for (int k = 0; k < 4; k++) V[(sl >> (4 * k)) & 15u] = Vt[k];
				}
			}
		}
	}
	if (next >= 0) stage_issue(C, st, (uint32_t)next, lane);  // records consumed: prefetch
	if (live) {
#pragma unroll
		for (uint32_t k = 0; k < NV; k++) {
			if (k < nv) __stcg(C.vert + 2 * (size_t)vid[k] + 1, V[k]);
		}
	}
}

// kind 0: element Rayleigh damping, 1: PBD damping.
__device__ __forceinline__ void run_damp_chunk(const DevCtx& C, Stage& st, uint32_t chunk, int next, uint32_t lane,
                                               int kind, float inv_dt, uint32_t tick) {
	const uint4 m = __ldg(reinterpret_cast<const uint4*>(C.chunks) + chunk);
	const uint32_t ntmax = m.z & 0xffu, nvmax = (m.z >> 8) & 0xffu, trow = m.w;
	if (m.z & kShapeCube) {
		if (kind == 0)
			damp_chunk<true, 0>(C, st, ntmax, nvmax, trow, next, lane, inv_dt, tick);
		else
			damp_chunk<true, 1>(C, st, ntmax, nvmax, trow, next, lane, inv_dt, tick);
	} else {
		if (kind == 0)
			damp_chunk<false, 0>(C, st, ntmax, nvmax, trow, next, lane, inv_dt, tick);
		else
			damp_chunk<false, 1>(C, st, ntmax, nvmax, trow, next, lane, inv_dt, tick);
	}
}

// Whether damping pass (kind index k >= 1, colour c) has work at this tick.
__device__ __forceinline__ bool pass_on(const DevCtx& C, int dk, uint32_t c, uint32_t tick) {
	return __ldg(C.pass_on + ((size_t)dk * 8u + tick % 8u) * C.ncolours + c) != 0;
}

// Vertices in no tet: nothing else touches them, so one thread takes each
// through all nsub substeps at once (predict, then finalize + predict); the
// final finalize pass closes the last one.
// With damping sweeps the launch ends in the canonical state without a
// closing finalize pass, so these vertices are finalized here (finalize_end).
template <bool TAPE = false>
__device__ __forceinline__ void run_isolated(const DevCtx& C, uint32_t begin, uint32_t step, uint32_t nsub, float dt,
                                             float inv_dt, bool finalize_end = false) {
	for (uint32_t i = begin; i < C.nisolated; i += step) {
		const uint32_t v = __ldg(C.isolated + i);
		float4 O, D;
		ld_vertex(C.vert + 2 * (size_t)v, O, D);
		for (uint32_t s = 0; s < nsub; s++) {
			const float4 Dbefore = D;
			advance_vertex(C, v, O, D, s == 0, dt, inv_dt);
			if (TAPE) tape_vertex(C, v, O, Dbefore, s, s == 0);
		}
		if (finalize_end) finalize_vertex(C, v, O, D, inv_dt);
		st_vertex(C.vert + 2 * (size_t)v, O, D);
	}
}

template <bool TAPE = false>
__device__ __forceinline__ void run_finalize(const DevCtx& C, uint32_t begin, uint32_t step, float inv_dt,
                                             uint32_t nsub = 0) {
	for (uint32_t v = begin; v < C.nverts; v += step) {
		float4 O, D;
		ld_vertex(C.vert + 2 * (size_t)v, O, D);
		if (TAPE) __stcs(C.tape_fin + v, D);
		finalize_vertex(C, v, O, D, inv_dt);
		if (TAPE) {
			const int q = __ldg(C.tip_of + v);
			if (q >= 0) C.traj[(size_t)(C.sub_base + nsub - 1) * C.ntips + q] = O;
		}
		st_vertex(C.vert + 2 * (size_t)v, O, D);
	}
}

// A substep is P = kinds x ncolours passes: the solve sweep over the colours,
// the volume sweeps (DevCtx::nvol), then each damping sweep
// (DevCtx::damp_kinds) over them again; pass q works on colour q % ncolours.
__device__ __forceinline__ uint32_t pass_kinds(const DevCtx& C) {
	return 1u + C.nvol + (uint32_t)__popc(C.damp_kinds);
}

// Damping kind of pass-kind index k > nvol: 0 element Rayleigh, 1 PBD.
__device__ __forceinline__ int damp_kind(const DevCtx& C, uint32_t k) {
	return (k == C.nvol + 1u && (C.damp_kinds & 1u)) ? 0 : 1;
}

// Whether pass q (P passes per substep) runs at `tick`: the solve and volume
// passes always, a damping pass only if some tet of its colour is damped then.
__device__ __forceinline__ bool pass_runs(const DevCtx& C, uint32_t q, uint32_t tick) {
	const uint32_t kind = q / C.ncolours;
	return kind <= C.nvol || pass_on(C, damp_kind(C, kind), q - kind * C.ncolours, tick);
}

// The warp's next chunk after `ch` (pass q of substep s, P passes per
// substep, tick0 the launch's first tick): the next chunk of the same colour,
// else its first chunk of the following passes that run (wrapping into the
// next substep); -1 when the launch has no more work for it.
__device__ __forceinline__ int next_chunk(const DevCtx& C, uint32_t s, uint32_t nsub, uint32_t q, uint32_t P,
                                          uint32_t ch, uint32_t gwarp, uint32_t nwarps, uint32_t tick0 = 0,
                                          const uint32_t* ccb = nullptr) {
	if (!ccb) ccb = C.colour_chunk_begin;
	if (ch + nwarps < ccb[q % C.ncolours + 1]) return (int)(ch + nwarps);
	for (uint32_t k = 1; k <= P; k++) {
		uint32_t q2 = q + k, s2 = s;
		if (q2 >= P) {
			q2 -= P;
			s2++;
		}
		if (s2 >= nsub) return -1;
		if (P > C.ncolours && !pass_runs(C, q2, tick0 + s2)) continue;
		const uint32_t c2 = q2 % C.ncolours;
		const uint32_t first = ccb[c2] + gwarp;
		if (first < ccb[c2 + 1]) return (int)first;
	}
	return -1;
}

// Persistent kernel: nsub substeps x P passes separated by the bounded grid
// barrier. Must be launched cooperatively (co-resident grid). Without damping
// the substep state stays (O, D) between substeps and the closing pass
// finalizes it; with damping sweeps they finish every substep and the state
// between substeps is canonical (X, V).
// EXT: the extended kernel, with the damping sweeps, the in-solve damping,
// the Pixar and cube models and the volume sweeps compiled in (handles that
// use any of them); without it they cost the kernel nothing.
template <bool LAMBDAS, bool TAPE = false, bool EXT = false>
__global__ void __launch_bounds__(256) k_persistent(DevCtx C, uint32_t nsub, float dt) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
	// chunk i of a colour goes to block i % grid, so chunks spread over all SMs
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = wpb * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	const bool dmode = EXT && C.damp_kinds != 0u;
	const uint32_t P = (EXT ? pass_kinds(C) : 1u) * C.ncolours;
	const uint32_t tick0 = __ldcg(C.tick);  // read before the first barrier; block 0 advances it at the end
	Stage st = stage_init(C, lane);
	// the colour table in shared memory (up to 64 colours): read after every
	// barrier, a global load there would sit on each pass's critical path
	__shared__ uint32_t s_ccb[65];
	const bool ccb_sh = C.ncolours <= 64u;
	if (ccb_sh)
		for (uint32_t i = threadIdx.x; i <= C.ncolours; i += blockDim.x) s_ccb[i] = __ldg(C.colour_chunk_begin + i);
	__syncthreads();
	const uint32_t* ccb = ccb_sh ? s_ccb : C.colour_chunk_begin;
	run_isolated<TAPE>(C, gtid, nthreads, nsub, dt, inv_dt, dmode);
	uint32_t target = C.bar_base;
	bool ok = true;
	for (uint32_t s = 0; s < nsub && ok; s++) {
		for (uint32_t q = 0; q < P && ok; q++) {
			const uint32_t kind = q / C.ncolours, c = q - kind * C.ncolours;
			// a damping pass with nothing to damp at this tick is skipped by
			// every block alike (same table, same tick): no work, no barrier
			if (EXT && kind > 0 && !pass_runs(C, q, tick0 + s)) continue;
			const uint32_t cb = ccb[c], ce = ccb[c + 1];
			for (uint32_t ch = cb + gwarp; ch < ce; ch += nwarps) {
				if (!stage_acquire(C, st, ch, lane)) {
					ok = false;
					break;
				}
				const int next = next_chunk(C, s, nsub, q, P, ch, gwarp, nwarps, tick0, ccb);
				if (!EXT || kind == 0)
					run_chunk<LAMBDAS, TAPE, EXT>(C, st, ch, next, lane, dmode || s == 0, dt, inv_dt, inv_dt2, s,
					                               dmode);
				else if (kind <= C.nvol)
					run_vol_chunk(C, st, ch, next, lane, inv_dt, inv_dt2, kind, dmode);
				else
					run_damp_chunk(C, st, ch, next, lane, damp_kind(C, kind), inv_dt, tick0 + s);
			}
			if (!grid_sync(C, target)) ok = false;
		}
	}
	if (!ok) {
		// leave no copy in flight
		if (st.inflight >= 0) mbar_wait(C, st.mbar, st.parity);
		return;
	}
	if (!dmode) run_finalize<TAPE>(C, gtid, nthreads, inv_dt, nsub);
	if (gtid == 0) *C.tick = tick0 + nsub;
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
		const uint32_t need = s + (d >> 31) + C.wait_miss;
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
				} else if (t - t0 > C.timeout_ns) {
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
	const uint32_t tick0 = __ldcg(C.tick);
	Stage st = stage_init(C, lane);
	run_isolated(C, gtid, nthreads, nsub, dt, inv_dt);
	bool ok = true;
	for (uint32_t s = 0; s < nsub && ok; s++) {
		for (uint32_t c = 0; c < C.ncolours && ok; c++) {
			const uint32_t cb = __ldg(C.colour_chunk_begin + c), ce = __ldg(C.colour_chunk_begin + c + 1);
			for (uint32_t ch = cb + gwarp; ch < ce; ch += nwarps) {
				const int next = next_chunk(C, s, nsub, c, C.ncolours, ch, gwarp, nwarps);
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
	uint32_t target = C.bar_base;
	if (!grid_sync(C, target) || !ok) return;
	run_finalize(C, gtid, nthreads, inv_dt);
	if (gtid == 0) *C.tick = tick0 + nsub;
}

// ---- brick launch form (sync_mode 4) ------------------------------------------
//
// The clusters are split into spatially compact bricks, one per block. A
// vertex that only one brick's clusters touch stays in that block's shared
// memory for the whole launch; the others stay in vert (L2). A pass is the
// brick's chunks of one colour; instead of a grid barrier the block then
// publishes its pass count and waits for the bricks it shares vertices with.
// Any vertex a pass reads was last written by a brick that shares it, which
// has finished the previous pass; no brick can be more than one pass ahead of
// a brick it shares vertices with. The colour order, the clusters and the
// arithmetic are those of k_persistent, so the results are bit-identical.

// The calling warp's brick chunk buffer and mbarrier.
__device__ __forceinline__ Stage brick_stage_init(uint32_t lane) {
	extern __shared__ __align__(128) uint8_t smem[];
	__shared__ uint64_t bmbars[32];
	const uint32_t w = threadIdx.x >> 5;
	Stage st = {smem + (size_t)w * kBrickChunkBytes, nullptr, &bmbars[w], 0u, -1, make_uint4(0u, 0u, 0u, 0u)};
	if (lane == 0) mbar_init(st.mbar);
	__syncwarp();
	return st;
}

__device__ __forceinline__ void brick_issue(const DevCtx& C, Stage& st, uint32_t chunk, uint32_t lane) {
	__syncwarp();
	if (lane == 0)
		bulk_copy_g2s(st.buf, C.bcblk + (size_t)chunk * (kBrickChunkBytes / 16u), kBrickChunkBytes, st.mbar);
	st.inflight = (int)chunk;
}

// Makes brick chunk `chunk` resident in the warp's buffer; false on timeout.
__device__ __forceinline__ bool brick_acquire(const DevCtx& C, Stage& st, uint32_t chunk, uint32_t lane) {
	if (st.inflight != (int)chunk) {
		if (st.inflight >= 0) {
			if (!mbar_wait(C, st.mbar, st.parity)) return false;
			st.parity ^= 1u;
		}
		brick_issue(C, st, chunk, lane);
	}
	const bool ok = mbar_wait(C, st.mbar, st.parity);
	st.parity ^= 1u;
	st.inflight = -1;
	return ok;
}

// The warp's next brick chunk after `ch` (colour c of substep s; bcb: the
// brick's colour chunk offsets), -1 when the launch has no more for it.
__device__ __forceinline__ int next_brick_chunk(const uint32_t* bcb, uint32_t ncol, uint32_t s, uint32_t nsub,
                                                uint32_t c, uint32_t ch, uint32_t wib, uint32_t wpb) {
	if (ch + wpb < bcb[c + 1]) return (int)(ch + wpb);
	for (uint32_t k = 1; k <= ncol; k++) {
		uint32_t c2 = c + k, s2 = s;
		if (c2 >= ncol) {
			c2 -= ncol;
			s2++;
		}
		if (s2 >= nsub) return -1;
		const uint32_t f = bcb[c2] + wib;
		if (f < bcb[c2 + 1]) return (int)f;
	}
	return -1;
}

// One resident brick chunk (every lane a whole cube, as run_chunk_cube).
// Vertex word w of a lane: a device vertex in vert, or kPrivate | p for the
// brick's shared-memory slot p (O at sv[p], D at sv[bpriv_max + p], device id
// spid[p]; O and D in two arrays so that the 16-byte accesses of a warp, whose
// lanes hold nearby slots, fall in different bank groups).
// bodies: the body parameters (a shared-memory copy when the handle has few).
// ONE: a single body, whose parameters bp1 and material mat1 the kernel holds
// in registers.
template <bool ONE>
__device__ __forceinline__ void run_chunk_brick(const DevCtx& C, Stage& st, int next, uint32_t lane, bool first,
                                                float dt, float inv_dt, float inv_dt2, float4* sv,
                                                const uint32_t* spid, const BodyParams* bodies, bool bshared,
                                                const BodyParams& bp1, const Mat& mat1) {
	const float4* rec = reinterpret_cast<const float4*>(st.buf);
	const uint32_t* hdrs = reinterpret_cast<const uint32_t*>(st.buf + 2048u * 6u);
	const uint32_t* vws = hdrs + kLanes;
	const uint32_t hdr = hdrs[lane];
	const bool live = (hdr & 15u) != 0;
	const uint32_t mask = (hdr >> 8) & 0xffu;
	uint32_t vw[8];
	float4 O[8], D[8];
	if (live) {
		const Mat mat = ONE ? mat1 : bshared ? load_mat_shared(bodies, hdr >> 16) : load_mat(bodies, hdr >> 16);
#pragma unroll
		for (int s = 0; s < 8; s++) vw[s] = vws[s * kLanes + lane];
#pragma unroll
		for (int s = 0; s < 8; s++) {
			if (vw[s] & kPrivate) {
				const uint32_t p = vw[s] & ~kPrivate;
				O[s] = sv[p];
				D[s] = sv[C.bpriv_max + p];
			} else {
				ld_vertex(C.vert + 2 * (size_t)vw[s], O[s], D[s]);
			}
		}
#pragma unroll
		for (int s = 0; s < 8; s++)
			if (mask & (1u << s)) {
				const uint32_t v = (vw[s] & kPrivate) ? spid[vw[s] & ~kPrivate] : vw[s];
				if (ONE)
					advance_vertex_bp(C, bp1, v, O[s], D[s], first, dt, inv_dt);
				else
					advance_vertex(C, v, O[s], D[s], first, dt, inv_dt, bodies);
			}
#pragma unroll
		for (int t = 0; t < 6; t++) {
			const float4* r = rec + t * 4 * kLanes + lane;
			const TetRec tr = {r[0], r[kLanes], r[2 * kLanes], r[3 * kLanes]};
			const float4 Ot[4] = {O[cube_slot(t, 0)], O[cube_slot(t, 1)], O[cube_slot(t, 2)], O[cube_slot(t, 3)]};
			float4 Dt[4] = {D[cube_slot(t, 0)], D[cube_slot(t, 1)], D[cube_slot(t, 2)], D[cube_slot(t, 3)]};
			solve_tet<false>(mat, tr, inv_dt, inv_dt2, Ot, Dt);
#pragma unroll
			for (int k = 0; k < 4; k++) D[cube_slot(t, k)] = Dt[k];
		}
	}
	if (next >= 0) brick_issue(C, st, (uint32_t)next, lane);  // buffer consumed: prefetch
	if (live) {
#pragma unroll
		for (int s = 0; s < 8; s++) {
			if (vw[s] & kPrivate) {
				const uint32_t p = vw[s] & ~kPrivate;
				if (mask & (1u << s)) sv[p] = O[s];
				sv[C.bpriv_max + p] = D[s];
			} else if (mask & (1u << s)) {
				st_vertex(C.vert + 2 * (size_t)vw[s], O[s], D[s]);
			} else {
				__stcg(C.vert + 2 * (size_t)vw[s] + 1, D[s]);
			}
		}
	}
}

// Bounded wait, by the calling threads (`first` of them striding by
// `stride`), until every brick of list[nb0, nb1) has published at least
// `target` passes. Returns false when a wait ran out or another
// block reported an error. The polls are relaxed loads and one acquire
// fence follows them (the acquire pattern of the PTX memory model): an
// acquire load on every poll, or an acquire-release fence, made the
// throughput frame 1.7% and 11% slower.
__device__ bool brick_wait(const DevCtx& C, const uint32_t* list, uint32_t nb0, uint32_t nb1, uint32_t target,
                           uint32_t first, uint32_t stride) {
	target += C.wait_miss;
	bool bad = false;
	for (uint32_t i = nb0 + first; i < nb1 && !bad; i += stride) {
		const uint32_t* f = C.bflag + (size_t)__ldg(list + i) * kBrickFlagStride;
		uint32_t spins = 0;
		uint64_t t0 = 0;
		while ((int32_t)(ld_relaxed_gpu(f) - target) < 0) {
			if (++spins == 256) {
				spins = 0;
				if (*(volatile int*)C.err) {
					bad = true;
					break;
				}
				const uint64_t t = global_ns();
				if (t0 == 0) {
					t0 = t;
				} else if (t - t0 > C.timeout_ns) {
					atomicCAS(C.err, 0, kErrBarrierTimeout);
					bad = true;
					break;
				}
			}
		}
	}
	asm volatile("fence.acquire.gpu;" ::: "memory");
	return !bad;
}

// Persistent brick kernel: one block per brick (grid = nbricks, cooperative
// launch so that every brick is resident), the plain solve only (no damping,
// volume passes or multiplier output). The state between substeps stays
// (O, D), and each brick finalizes its own vertices at the end.
template <bool ONE>
__global__ void __launch_bounds__(256) k_bricks(DevCtx C, uint32_t nsub, float dt) {
	extern __shared__ __align__(128) uint8_t smem[];
	__shared__ uint32_t s_bcb[65], s_bwait[64];
	__shared__ BodyParams s_bodies[kBrickBodies];
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
	const uint32_t b = blockIdx.x, ncol = C.ncolours;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	const uint32_t tick0 = __ldcg(C.tick);  // read before any brick publishes; block 0 advances it at the end
	Stage st = brick_stage_init(lane);
	float4* sv = reinterpret_cast<float4*>(smem + (size_t)wpb * kBrickChunkBytes);
	uint32_t* spid = reinterpret_cast<uint32_t*>(sv + 2 * (size_t)C.bpriv_max);
	for (uint32_t i = threadIdx.x; i <= ncol; i += blockDim.x) {
		s_bcb[i] = __ldg(C.bchunk_begin + (size_t)b * ncol + i);
		if (i < ncol) s_bwait[i] = __ldg(C.bchunk_wait_end + (size_t)b * ncol + i);
	}
	// few bodies: their parameters in shared memory (the advance reads them per vertex)
	const bool bshared = C.nbodies <= kBrickBodies;
	if (bshared) {
		const uint32_t words = C.nbodies * (uint32_t)(sizeof(BodyParams) / 4);
		for (uint32_t i = threadIdx.x; i < words; i += blockDim.x)
			reinterpret_cast<uint32_t*>(s_bodies)[i] = __ldg(reinterpret_cast<const uint32_t*>(C.bodies) + i);
	}
	const BodyParams* bodies = bshared ? s_bodies : C.bodies;
	// a single body: its parameters and material in registers
	BodyParams bp1;
	Mat mat1;
	if (ONE) {
		bp1 = C.bodies[0];
		mat1 = load_mat(C.bodies, 0);
	}
	// the brick's own vertices into shared memory, for the whole launch
	const uint32_t pb = __ldg(C.bpriv_begin + b), pe = __ldg(C.bpriv_begin + b + 1);
	for (uint32_t i = pb + threadIdx.x; i < pe; i += blockDim.x) {
		const uint32_t v = __ldg(C.bpriv_vid + i);
		float4 O, D;
		ld_vertex(C.vert + 2 * (size_t)v, O, D);
		sv[i - pb] = O;
		sv[C.bpriv_max + (i - pb)] = D;
		spid[i - pb] = v;
	}
	__syncthreads();
	// vertices in no tet, finalized here too (no closing pass over all vertices)
	run_isolated(C, gtid, nthreads, nsub, dt, inv_dt, true);
	const uint32_t nb0 = __ldg(C.bnb_begin + b), nb1 = __ldg(C.bnb_begin + b + 1);
	// A pass: the warps whose chunk holds only interior clusters (every vertex
	// private) start at once; a warp with a boundary cluster first waits
	// until the neighbouring bricks have finished the previous pass (their
	// writes to the shared vertices are visible). The block's barrier then
	// ends the pass, and it publishes the pass count.
	uint32_t epoch = 0;
	bool ok = true;
	for (uint32_t s = 0; s < nsub && ok; s++) {
		for (uint32_t c = 0; c < ncol && ok; c++) {
			const uint32_t wend = s_bwait[c];
			bool bad = false, waited = false;
			for (uint32_t ch = s_bcb[c] + wib; ch < s_bcb[c + 1] && !bad; ch += wpb) {
				if (ch < wend && !waited) {
					const uint32_t q = b * ncol + c;
					bad = __any_sync(0xffffffffu, !brick_wait(C, C.bcnb, __ldg(C.bcnb_begin + q),
					                                             __ldg(C.bcnb_begin + q + 1), epoch, lane, 32u));
					__syncwarp();  // orders every lane's loads after the lanes' acquires
					waited = true;
					if (bad) break;
				}
				if (!brick_acquire(C, st, ch, lane)) {
					bad = true;
					break;
				}
				const int next = next_brick_chunk(s_bcb, ncol, s, nsub, c, ch, wib, wpb);
				run_chunk_brick<ONE>(C, st, next, lane, s == 0, dt, inv_dt, inv_dt2, sv, spid, bodies, bshared, bp1,
				                     mat1);
			}
			if (__syncthreads_or(bad ? 1 : 0)) {
				ok = false;
				break;
			}
			++epoch;
			// the release store orders every write of the pass that the
			// barrier made visible to this thread before the count
			if (threadIdx.x == 0) st_release_gpu(C.bflag + (size_t)b * kBrickFlagStride, epoch);
		}
	}
	// every brick sharing a vertex with this one has finished the last pass
	if (ok) ok = !__syncthreads_or(brick_wait(C, C.bnb, nb0, nb1, epoch, threadIdx.x, blockDim.x) ? 0 : 1);
	if (!ok) {
		if (st.inflight >= 0) mbar_wait(C, st.mbar, st.parity);  // leave no copy in flight
		return;
	}
	for (uint32_t i = pb + threadIdx.x; i < pe; i += blockDim.x) {
		const uint32_t v = __ldg(C.bpriv_vid + i);
		float4 O = sv[i - pb], D = sv[C.bpriv_max + (i - pb)];
		if (ONE)
			finalize_vertex_bp(C, bp1, v, O, D, inv_dt);
		else
			finalize_vertex(C, v, O, D, inv_dt, bodies);
		st_vertex(C.vert + 2 * (size_t)v, O, D);
	}
	const uint32_t fb = __ldg(C.bfin_begin + b), fe = __ldg(C.bfin_begin + b + 1);
	for (uint32_t i = fb + threadIdx.x; i < fe; i += blockDim.x) {
		const uint32_t v = __ldg(C.bfin_vid + i);
		float4 O, D;
		ld_vertex(C.vert + 2 * (size_t)v, O, D);
		if (ONE)
			finalize_vertex_bp(C, bp1, v, O, D, inv_dt);
		else
			finalize_vertex(C, v, O, D, inv_dt, bodies);
		st_vertex(C.vert + 2 * (size_t)v, O, D);
	}
	if (gtid == 0) *C.tick = tick0 + nsub;
}

// One colour pass as its own launch (CUDA-graph mode): one chunk per warp.
// kind 0 is the solve pass (first: the state is canonical), 1..nvol the
// volume passes, the rest the damping passes (damp_kind); sub: the substep's
// index in the call (its tick is *C.tick + sub). In the first launch of a
// call, blocks past the colour's chunks step the isolated vertices through
// all nsub substeps.
template <bool LAMBDAS, bool EXT = false>
__global__ void __launch_bounds__(256, 1) k_colour(DevCtx C, uint32_t colour, int first, float dt, uint32_t solve_blocks,
                                                uint32_t nsub, uint32_t kind, uint32_t sub) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	if (blockIdx.x >= solve_blocks) {
		const uint32_t b = blockIdx.x - solve_blocks, nb = gridDim.x - solve_blocks;
		run_isolated(C, b * blockDim.x + threadIdx.x, nb * blockDim.x, nsub, dt, inv_dt, EXT && C.damp_kinds != 0u);
		return;
	}
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t ch = __ldg(C.colour_chunk_begin + colour) + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
	if (ch >= __ldg(C.colour_chunk_begin + colour + 1)) return;
	const uint32_t tick = __ldcg(C.tick) + sub;
	const bool damp_pass = EXT && kind > C.nvol;
	const int dk = damp_pass ? damp_kind(C, kind) : 0;
	// a graph replays its launches at every tick: a damping pass with nothing
	// to damp at this one returns at once
	if (damp_pass && !pass_on(C, dk, colour, tick)) return;
	Stage st = stage_init(C, lane);
	if (!stage_acquire(C, st, ch, lane)) return;
	const bool dmode = EXT && C.damp_kinds != 0u;
	if (!EXT || kind == 0)
		run_chunk<LAMBDAS, false, EXT>(C, st, ch, -1, lane, first != 0, dt, inv_dt, inv_dt2, 0, dmode);
	else if (!damp_pass)
		run_vol_chunk(C, st, ch, -1, lane, inv_dt, inv_dt2, kind, dmode);
	else
		run_damp_chunk(C, st, ch, -1, lane, dk, inv_dt, tick);
}

__global__ void k_finalize(DevCtx C, float dt) {
	run_finalize(C, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, 1.0f / dt);
}

// Advances the tick word by a call's substeps (CUDA-graph mode).
__global__ void k_advance_tick(DevCtx C, uint32_t nsub) { *C.tick += nsub; }

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

// Per-tet material change without re-uploading the chunk blocks: the
// record's c0 = (1/mu)/volume, formed with the same two correctly rounded
// divisions as the host (XPBDFEM/Fem.cpp:449), and 1/mu for the adjoint.
__global__ void k_set_c0(float4* __restrict__ cblk, const uint32_t* __restrict__ rec, const float* __restrict__ vol,
                         const float* __restrict__ mu, float mu_uniform, uint32_t n, float* __restrict__ inv_mu) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float im = 1.0f / (mu ? mu[i] : mu_uniform);
	cblk[rec[i]].w = im / vol[i];
	inv_mu[i] = im;
}

// dL/dmu in caller tet order from the per-row accumulator (-mu dL/dmu).
__global__ void k_gather_dmu(const float* __restrict__ cbar, const uint32_t* __restrict__ slot,
                             const float* __restrict__ inv_mu, uint32_t n, float* __restrict__ out) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	out[i] = -cbar[slot[i]] * inv_mu[i];
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

// The dynamic shared-memory limit is a property of the kernel on one device
// (cudaFuncSetAttribute acts in the current device's context), shared by
// every handle on that device: it only ever grows to the largest size any
// handle launches with (a larger limit does not restrict smaller launches),
// so one handle's configuration cannot lower another's below what it needs.
// Kept per (device, kernel); a failed raise is returned and not recorded.
static cudaError_t set_smem_attr(const void* f, size_t bytes) {
	struct Entry {
		int dev;
		const void* f;
		size_t bytes;
	};
	static std::mutex mu;
	static std::vector<Entry> done;
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	std::lock_guard<std::mutex> lk(mu);
	for (auto& d : done)
		if (d.dev == dev && d.f == f) {
			if (bytes > d.bytes) {
				e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
				if (e == cudaSuccess) d.bytes = bytes;
			}
			return e;
		}
	e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
	if (e == cudaSuccess) done.push_back({dev, f, bytes});
	return e;
}

static const void* persistent_fn(bool lambdas, bool ext) {
	if (ext) return lambdas ? (const void*)k_persistent<true, false, true> : (const void*)k_persistent<false, false, true>;
	return lambdas ? (const void*)k_persistent<true> : (const void*)k_persistent<false>;
}

static const void* colour_fn(bool lambdas, bool ext) {
	if (ext) return lambdas ? (const void*)k_colour<true, true> : (const void*)k_colour<false, true>;
	return lambdas ? (const void*)k_colour<true> : (const void*)k_colour<false>;
}

int configure_kernels(const LaunchCfg& cfg) {
	const size_t smem = solve_smem_bytes(cfg.block, cfg.warp_smem);
	cudaError_t e = cudaSuccess;
	for (bool ext : {false, true}) {
		if (e == cudaSuccess) e = set_smem_attr(persistent_fn(cfg.lambdas, ext), smem);
		if (e == cudaSuccess) e = set_smem_attr(colour_fn(cfg.lambdas, ext), smem);
	}
	if (e == cudaSuccess)
		e = set_smem_attr(cfg.lambdas ? (const void*)k_dataflow<true> : (const void*)k_dataflow<false>, smem);
	return (int)e;
}

size_t brick_smem_bytes(int block, uint32_t bpriv_max) {
	return (size_t)(block / 32) * kBrickChunkBytes + (size_t)bpriv_max * kBrickVertexBytes;
}

int brick_grid_fits(int block, uint32_t bpriv_max, uint32_t nbricks, bool* fits) {
	const size_t smem = brick_smem_bytes(block, bpriv_max);
	cudaError_t e = set_smem_attr((const void*)k_bricks<true>, smem);
	if (e == cudaSuccess) e = set_smem_attr((const void*)k_bricks<false>, smem);
	int dev = 0, sms = 0, per_sm = 0;
	if (e == cudaSuccess) e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	int per_sm1 = 0;
	if (e == cudaSuccess)
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_bricks<false>, block, smem);
	if (e == cudaSuccess)
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm1, (const void*)k_bricks<true>, block, smem);
	if (e != cudaSuccess) return (int)e;
	*fits = (uint64_t)std::min(per_sm, per_sm1) * (uint64_t)sms >= nbricks && nbricks > 0;
	return 0;
}

int persistent_grid(const LaunchCfg& cfg, int* blocks_out) {
	const void* f = cfg.sync_mode == 3
	                    ? (cfg.lambdas ? (const void*)k_dataflow<true> : (const void*)k_dataflow<false>)
	                    : persistent_fn(cfg.lambdas, cfg.ext);
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
	if (cfg.sync_mode == 4) {
		// pass counters start at 0; one launch counts at most 2^30 passes
		const size_t smem_b = brick_smem_bytes(cfg.block, ctx.bpriv_max);
		const uint32_t per = std::max(1u, (1u << 30) / std::max(1u, ctx.ncolours));
		for (uint32_t done = 0; done < nsub;) {
			uint32_t n = std::min(per, nsub - done);
			e = cudaMemsetAsync(ctx.bflag, 0, sizeof(uint32_t) * kBrickFlagStride * ctx.nbricks, st);
			if (e != cudaSuccess) return (int)e;
			DevCtx c = ctx;
			float dtv = dt;
			void* args[] = {&c, &n, &dtv};
			const void* f = ctx.nbodies == 1 ? (const void*)k_bricks<true> : (const void*)k_bricks<false>;
			e = cudaLaunchCooperativeKernel(f, dim3(ctx.nbricks), dim3(cfg.block), args, smem_b, st);
			if (e != cudaSuccess) return (int)e;
			done += n;
		}
		return 0;
	}
	if (cfg.sync_mode == 1 || cfg.sync_mode == 3) {
		e = reset_barrier(ctx, st);
		if (e == cudaSuccess && cfg.sync_mode == 3) e = cudaMemsetAsync(ctx.done, 0, sizeof(uint32_t) * ctx.nchunks, st);
		if (e != cudaSuccess) return (int)e;
		DevCtx c = ctx;
		void* args[] = {&c, &nsub, &dt};
		const void* f = cfg.sync_mode == 1
		                    ? persistent_fn(cfg.lambdas, cfg.ext)
		                    : (cfg.lambdas ? (const void*)k_dataflow<true> : (const void*)k_dataflow<false>);
		e = cudaLaunchCooperativeKernel(f, dim3(cfg.blocks), dim3(cfg.block), args, smem, st);
		return (int)e;
	}
	// per-colour launches (captured into a CUDA graph by the caller when wanted):
	// per substep the solve sweep, the volume sweeps, then each damping sweep
	const void* fc = colour_fn(cfg.lambdas, cfg.ext);
	const uint32_t warps_per_block = cfg.block / 32;
	const bool dmode = cfg.ext && ctx.damp_kinds != 0u;
	const uint32_t kinds = cfg.ext ? 1u + ctx.nvol + (uint32_t)__builtin_popcount(ctx.damp_kinds) : 1u;
	for (uint32_t s = 0; s < nsub; s++) {
		for (uint32_t kind = 0; kind < kinds; kind++) {
			for (uint32_t c = 0; c < ctx.ncolours; c++) {
				const uint32_t nch = cfg.colour_chunk_begin_host[c + 1] - cfg.colour_chunk_begin_host[c];
				uint32_t sb = (nch + warps_per_block - 1) / warps_per_block;
				uint32_t extra = 0;
				if (s == 0 && kind == 0 && c == 0 && ctx.nisolated) extra = (ctx.nisolated + cfg.block - 1) / cfg.block;
				const uint32_t grid = sb + extra;
				if (grid == 0) continue;
				DevCtx cc = ctx;
				uint32_t colour = c, ns = nsub, kd = kind, sub = s;
				int first = (dmode || s == 0) ? 1 : 0;
				float dtv = dt;
				void* args[] = {&cc, &colour, &first, &dtv, &sb, &ns, &kd, &sub};
				e = cudaLaunchKernel(fc, dim3(grid), dim3(cfg.block), args, smem, st);
				if (e != cudaSuccess) return (int)e;
			}
		}
	}
	const uint32_t fb = (ctx.nverts + 255) / 256;
	if (fb && !dmode) {
		k_finalize<<<fb, 256, 0, st>>>(ctx, dt);
		e = cudaGetLastError();
		if (e != cudaSuccess) return (int)e;
	}
	k_advance_tick<<<1, 1, 0, st>>>(ctx, nsub);
	return (int)cudaGetLastError();
}

// The recording forward: k_persistent with the tape writes compiled in. The
// arithmetic is the same inlined code as the plain launch, so the trajectory
// is the plain launch's bit for bit.
int launch_substeps_tape(const DevCtx& ctx, int block, uint32_t warp_smem, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = (const void*)k_persistent<false, true>;
	const size_t smem = solve_smem_bytes(block, warp_smem);
	cudaError_t e = set_smem_attr(f, smem);
	int dev = 0, sms = 0, per_sm = 0;
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

int launch_set_c0(float4* cblk, const uint32_t* rec, const float* vol, const float* mu, float mu_uniform, uint32_t n,
                  float* inv_mu, void* stream) {
	if (!n) return 0;
	k_set_c0<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(cblk, rec, vol, mu, mu_uniform, n, inv_mu);
	return (int)cudaGetLastError();
}

int launch_gather_dmu(const float* cbar, const uint32_t* slot, const float* inv_mu, uint32_t n, float* out,
                      void* stream) {
	if (!n) return 0;
	k_gather_dmu<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(cbar, slot, inv_mu, n, out);
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
// framework's caching pool), or a real-time loop that must not take
// cudaMalloc's implicit device-wide synchronisation. For them the persistent
// substep kernel is launched with its scratch words (the grid-barrier arrival
// counter and the device error word) taken from this fixed array instead of
// buffers of the handle, and without the autotuner or CUDA-graph builder,
// which may allocate.
//
// The array lives in every device that loads the library until the process
// exits. All calls share it and it keeps the last call's contents, so each
// call sets the words it uses first; calls whose kernels overlap on one GPU
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
	const void* f = persistent_fn(lambdas, ctx.ext != 0u);
	const size_t smem = solve_smem_bytes(block, warp_smem);
	cudaError_t e = set_smem_attr(f, smem);  // no allocation: the kernel's shared-memory limit on this device
	int sms = 0, per_sm = 0;
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, block, smem);
	if (e != cudaSuccess) return (int)e;
	if (per_sm <= 0) return (int)cudaErrorInvalidConfiguration;
	const uint32_t blocks = (uint32_t)(per_sm * sms);
	// One call's grid-barrier arrivals stay below 2^31: every block arrives
	// once per pass, and a substep runs (1 + volume sweeps + damping kinds) x
	// colours passes in the extended kernel, one per colour otherwise.
	const uint64_t kinds = ctx.ext ? 1ull + ctx.nvol + (uint64_t)__builtin_popcount(ctx.damp_kinds) : 1ull;
	if ((uint64_t)nsub * kinds * ctx.ncolours * blocks >= (1ull << 31)) return kNoAllocTooLong;
	e = cudaMemsetAsync(p, ctx.bar_base ? 0xff : 0, sizeof(uint32_t), st);
	if (e == cudaSuccess) e = cudaMemsetAsync(p + 1, 0, sizeof(uint32_t), st);
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
