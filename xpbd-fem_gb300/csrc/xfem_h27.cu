// Quadratic-hex mode of libxfem.so (sm_103a): GeoQuadratic3d on a hex mesh
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
#include "xfem_ring_update.cuh"
#include "xfem_h27_elem.cuh"

namespace xfem {

namespace {

using namespace h27e;

// ---- continuous-pressure models: one-rings over the H27s ---------------------
// GeoQuadratic3d builds a ring for every mesh vertex over the H27s around it
// (XPBDFEM/Geo.cpp:944-953) and SolveRing solves one constraint (pair) per
// ring (XPBDFEM/Geo.cpp:147-225) with the full-energy branch of
// CalculateElementEnergyAndGradients on each H27 (XPBDFEM/Fem.cpp:983-1036:
// elemWeight = (volume / 8) / ring volume; prefactored I1 over the 27 nodes,
// or for ContinuousSkin the Yeoh polynomial on the 27 points; (J - a)^2 on
// the 8 points).
//
// One warp per ring, taking the ring's H27s one after another in ring order:
// each in the element kernel's lane layout (lane n < 27 owns node n, lane p
// point p), its nodes read from the warp's copy of the ring's nodes, and
// each node's two gradient contributions added into the ring node's sums,
// so that every node sums its terms in H27 order. Then lane n takes ring
// nodes n, n + 32, n + 64 and n + 96 for the multiplier update.
struct H27RingScratch {
	Scratch el;                                          // the current H27: record, offsets, point terms
	float4 O[kMaxQRingNodes], D[kMaxQRingNodes];         // ring nodes: (O, w), (D, bits)
	float g0[kMaxQRingNodes][3], g1[kMaxQRingNodes][3];  // per ring node: the gradient sums
};

template <bool DAMP, bool VMODE>
__device__ __forceinline__ void h27_ring_solve(const DevCtx& C, H27RingScratch& S, uint32_t r, uint32_t lane,
                                               float inv_dt, float inv_dt2, uint32_t tick) {
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
#pragma unroll
			for (int q = 0; q < 3; q++) S.g0[n][q] = S.g1[n][q] = 0.0f;
		}
	}
	// entry j: two float4, the H27's device index, then its 27 nodes' ring
	// slots one byte each
	const uint32_t* ent = reinterpret_cast<const uint32_t*>(C.ring_ent) + 8 * (size_t)h.y;
	float volq = 0.0f;
	if (lane < ne) {
		const uint32_t ei = __ldg(ent + 8 * lane);
		volq = 0.125f * __ldg(reinterpret_cast<const float*>(C.el_rec + (size_t)ei * (kRec / 4)) + kVol);
	}
	const float volume = warp_sum(volq);  // the ring's volume
	const uint32_t e = __ldg(&bp.energy);
	const float a = __ldg(&bp.a_ring);
	float U0 = 0.0f, U1 = 0.0f;
#pragma unroll 1
	for (uint32_t j = 0; j < ne; j++) {
		const uint32_t ei = __ldg(ent + 8 * j);
		const uint32_t slot = lane < 27 ? (__ldg(ent + 8 * j + 1 + (lane >> 2)) >> (8 * (lane & 3))) & 0xffu : 0u;
		__syncwarp();  // the previous H27's record and point terms are consumed
		const float4* src = C.el_rec + (size_t)ei * (kRec / 4);
		for (uint32_t k = lane; k < kRec / 4; k += 32) S.el.rec[k] = __ldg(src + k);
		__syncwarp();
		Elem E;
		E.lane = lane;
		E.R = reinterpret_cast<const float*>(S.el.rec);
		E.O = E.D = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		E.w = 0.0f;
		E.dv = 0;
		if (lane < 27) {
			E.O = S.O[slot];
			E.D = S.D[slot];
			E.w = E.O.w;
		}
		share_rel(S.el, E, VMODE);
		const float ew = (rec(E, kVol) * 0.125f) / volume;  // the H27's share of the ring volume
		float u0, u1;
		Vec3 g0, g1;
		if (e == 10u) {
			points<kDev>(C, S.el, E, 1, bp, e, a, u0, u1, ew, true);
			g0 = root(E, gather(C, S.el.M0, E, 1));
			U0 += wsum(u0);
		} else {
			U0 = fmaf(ew, pref_i1(S.el, E, g0), U0);
			g0 = {ew * g0.x, ew * g0.y, ew * g0.z};
		}
		points<kHydro>(C, S.el, E, 0, bp, e, a, u0, u1, ew, false);
		g1 = root(E, gather(C, S.el.M1, E, 0));
		U1 += wsum(u1);
		if (lane < 27) {
			S.g0[slot][0] += g0.x;
			S.g0[slot][1] += g0.y;
			S.g0[slot][2] += g0.z;
			S.g1[slot][0] += g1.x;
			S.g1[slot][1] += g1.y;
			S.g1[slot][2] += g1.z;
		}
	}
	__syncwarp();
	Vec3 g0[kQNodesPerLane], g1[kQNodesPerLane];
#pragma unroll
	for (uint32_t k = 0; k < kQNodesPerLane; k++) {
		const uint32_t n = lane + 32u * k;
		g0[k] = g1[k] = {0.0f, 0.0f, 0.0f};
		if (n < nn) {
			g0[k] = {S.g0[n][0], S.g0[n][1], S.g0[n][2]};
			g1[k] = {S.g1[n][0], S.g1[n][1], S.g1[n][2]};
		}
	}
	if (e == 8u) {
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

// The persistent H27 ring kernel (cooperative launch, co-resident grid): per
// substep the advance pass, one pass per ring colour, and with post-step
// damping a finalize pass, the rings' Rayleigh passes and the PBD passes
// over the H27 colours (GeoQuadratic3d::Damp, XPBDFEM/Geo.cpp:987-1008).
template <bool DAMP>
__global__ void __launch_bounds__(128) k_h27_rings(DevCtx C, uint32_t nsub, float dt) {
	extern __shared__ __align__(128) unsigned char smem[];
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = (blockDim.x >> 5) * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	H27RingScratch& S = reinterpret_cast<H27RingScratch*>(smem)[wib];
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
			for (uint32_t r = rb + gwarp; r < re; r += nwarps) h27_ring_solve<DAMP, false>(C, S, r, lane, inv_dt, inv_dt2, 0);
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
						h27_ring_solve<true, true>(C, S, r, lane, inv_dt, inv_dt2, tick);
					if (!grid_sync(C, target)) return;
				}
			if (C.damp_kinds & 2u)
				for (uint32_t c = 0; c < C.el_colours; c++) {
					const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
					for (uint32_t i = b + gwarp; i < e; i += nwarps) {
						const BodyParams& bp = body_of_el<H27Elem>(C, i);
						if (__ldg(&bp.pbd_on) && in_slice(C, bp, i, tick)) {
							const float coeff =
							    __ldg(&bp.rayleigh_type) == 3u ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff);
							__syncwarp();  // the scratch's last readers are done
							h27_pbd_in(C, S.el, i, coeff);
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

int launch_h27_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = ctx.ext ? (const void*)k_h27_rings<true> : (const void*)k_h27_rings<false>;
	const size_t smem = (size_t)(block / 32) * sizeof(H27RingScratch);
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

int launch_h27(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	if (block != 256) return (int)cudaErrorInvalidConfiguration;  // the per-warp scratch is sized for 8 warps
	return launch_elements<h27e::H27Elem>(ctx, block, nsub, dt, stream);
}

}  // namespace xfem
