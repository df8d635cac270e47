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
#include "xfem_ring_update.cuh"
#include "xfem_t10_elem.cuh"

namespace xfem {

namespace {

using namespace t10e;

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
	return launch_elements<t10e::T10Elem>(ctx, block, nsub, dt, stream);
}

}  // namespace xfem
