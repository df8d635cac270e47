// Hex mode of libxfem.so (sm_103a): linear hexahedra (H8). GeoLinear3d's hex
// loops (XPBDFEM/Geo.cpp:774-811) with SolveElement on ElementParamsLinearHex
// (XPBDFEM/Fem.cpp:871-896: SolveElementPixar :361-433 and SolveElementMixed
// :437-564 with Nodes = 8, PointsLo = 1 (the centre), PointsHi = 8 (2x2x2)),
// SolveVolumeOnly (:840-867), DampElement (:910-928) and PbdDamp
// (XPBDFEM/Xpbd.h:306-346).
//
// Schedule: hexes coloured so that the hexes of one colour share no vertex.
// A substep is one pass that advances every vertex (finishes the previous
// substep, predicts this one), one pass per colour with one thread per hex,
// the volume sweeps, and with post-step damping a finalize pass and the
// damping passes; each pass ends at the grid barrier.
//
// Records: 30 float4 per hex, stored as a structure of arrays (float4 k of
// hex i at el_rec[k * nel + i]) so that the threads of a pass read them
// coalesced. The first ten hold what every model reads (the centre's inverse
// map jacobian and weight, volume, surface area, the prefactored QQ and QR);
// the other twenty the 2x2x2 points' inverse jacobians and weights, which only
// the quadrature models read.
#include <cuda_runtime.h>
#include <stdint.h>

#include "xfem_hex_device.cuh"
#include "xfem_ring_update.cuh"

namespace xfem {

namespace {

// ---- the continuous-pressure models on hexes --------------------------------
//
// SolveRing of a vertex one-ring over hexes (XPBDFEM/Geo.cpp:147-225): every
// ring hex adds the full-energy branch of CalculateElementEnergyAndGradients
// (XPBDFEM/Fem.cpp:983-1036) weighted by an eighth of its volume over the
// ring volume: the deviatoric term (I1 prefactored, or for ContinuousSkin the
// Yeoh polynomial of I1 - 3 on the 2x2x2 points with the model's own
// constants) and (J - a)^2 at the centre. Then one constraint
// (ContinuousPixar, mu = 2: U0 + (lambda / 2) U1) or the coupled pair.
//
// One warp per ring: lane j (< 16) takes the ring's hex j and leaves its
// eight corners' gradient contributions in shared memory; lane n sums node
// n's contributions in hex order and takes its update.

struct HexRingScratch {
	float4 O[kMaxRingNodes], D[kMaxRingNodes];  // ring nodes: (O, w), (D, bits)
	float g0[kMaxRingHexes][8][3];              // per hex corner: deviatoric gradient contribution
	float g1[kMaxRingHexes][8][3];              // per hex corner: (J - a)^2 gradient contribution
};

// ContinuousSkin's deviatoric term of one hex: sum over the 2x2x2 points of
// ew w_p Yeoh(I1 - 3) with the constants of XPBDFEM/Fem.cpp:992, root
// gradient included.
__device__ __forceinline__ float ring_skin(const HexRec& R, const Vec3 P[7], float ew, Vec3 g[8]) {
	const float C0 = 0.1095f, C1 = 14.95f, C2 = 4.595f;
	float U = 0.0f;
	zeron<8>(g);
#pragma unroll 1
	for (int p = 0; p < 8; p++) {
		Point q;
		point(R, 1, p, P, q);
		const float I1 = fmaf(q.F[0][0], q.F[0][0], fmaf(q.F[0][1], q.F[0][1], q.F[0][2] * q.F[0][2])) +
		                 fmaf(q.F[1][0], q.F[1][0], fmaf(q.F[1][1], q.F[1][1], q.F[1][2] * q.F[1][2])) +
		                 fmaf(q.F[2][0], q.F[2][0], fmaf(q.F[2][1], q.F[2][1], q.F[2][2] * q.F[2][2]));
		const float IM = I1 - 3.0f, wt = ew * q.w;
		U = fmaf(wt, IM * fmaf(IM, fmaf(IM, C2, C1), C0), U);
		const float s = wt * fmaf(IM, fmaf(IM, 6.0f * C2, 4.0f * C1), 2.0f * C0);
		float G[3][3];
#pragma unroll
		for (int c = 0; c < 3; c++)
#pragma unroll
			for (int r = 0; r < 3; r++) G[c][r] = q.F[r][c] * s;
		apply(G, q.Ji, 1, p, g);
	}
	rootn<8>(g);
	return U;
}

// Ring hex `lane` of a one-ring: its corners' gradient contributions into
// the scratch, its weighted deviatoric and (J - a)^2 energies returned.
template <bool VMODE>
__device__ __noinline__ float2 hex_ring_elem(const DevCtx& C, HexRingScratch& S, const BodyParams& bp, uint32_t lane,
                                             uint32_t ei, uint32_t clo, uint32_t chi, float volume) {
	float4 O[8], D[8];
#pragma unroll
	for (int k = 0; k < 8; k++) {
		const uint32_t q = ((k < 4 ? clo : chi) >> (8 * (k & 3))) & 0xffu;
		O[k] = S.O[q];
		D[k] = S.D[q];
	}
	Vec3 P[7], g[8];
	rel(O, D, VMODE, P);
	const HexRec R{C.el_rec, C.nel, ei};
	const float ew = (R(kRVol) * 0.125f) / volume;  // the hex's share of the ring volume
	float U0;
	if (__ldg(&bp.energy) == 10u) {
		U0 = ring_skin(R, P, ew, g);
	} else {
		U0 = ew * pref_i1(R, P, g);
#pragma unroll
		for (int n = 0; n < 8; n++) g[n] = {ew * g[n].x, ew * g[n].y, ew * g[n].z};
	}
#pragma unroll
	for (int n = 0; n < 8; n++) {
		S.g0[lane][n][0] = g[n].x;
		S.g0[lane][n][1] = g[n].y;
		S.g0[lane][n][2] = g[n].z;
	}
	// (J - a)^2 at the centre
	Point q;
	point(R, 0, 0, P, q);
	const float wt = ew * q.w, Ja = q.J - __ldg(&bp.a_ring);
	const float U1 = wt * Ja * Ja;
	const float sg = wt * 2.0f * Ja;
	float G[3][3];
#pragma unroll
	for (int c = 0; c < 3; c++)
#pragma unroll
		for (int rr = 0; rr < 3; rr++) G[c][rr] = q.A[c][rr] * sg;
	zeron<8>(g);
	apply(G, q.Ji, 0, 0, g);
	rootn<8>(g);
#pragma unroll
	for (int n = 0; n < 8; n++) {
		S.g1[lane][n][0] = g[n].x;
		S.g1[lane][n][1] = g[n].y;
		S.g1[lane][n][2] = g[n].z;
	}
	return make_float2(U0, U1);
}

// SolveRing of ring r over hexes by the calling warp (every lane takes part).
// VMODE: the post-step Rayleigh form on the canonical state (X, V) for the
// rings of this tick's slice, as the tet rings.
template <bool DAMP, bool VMODE>
__device__ __noinline__ void hex_ring_solve(const DevCtx& C, HexRingScratch& S, uint32_t r, uint32_t lane, float inv_dt,
                                            float inv_dt2, uint32_t tick) {
	__syncwarp();  // every lane is done with the previous ring's scratch
	const uint4 h = __ldg(C.ring_hdr + r);
	const uint32_t nn = h.z & 0xffu, nh = (h.z >> 8) & 0xffu;
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
	uint32_t dv = 0;
	if (lane < nn) {
		dv = __ldg(C.ring_node + h.x + lane);
		ld_vertex(C.vert + 2 * (size_t)dv, S.O[lane], S.D[lane]);
	}
	// entry j: the hex's device index and its corners' ring node indices
	uint32_t ei = 0, clo = 0, chi = 0;
	float volq = 0.0f;
	if (lane < nh) {
		const float4 e = __ldg(C.ring_ent + 2 * ((size_t)h.y + lane));
		ei = __float_as_uint(e.x);
		clo = __float_as_uint(e.y);
		chi = __float_as_uint(e.z);
		volq = 0.125f * HexRec{C.el_rec, C.nel, ei}(kRVol);
	}
	const float volume = warp_sum(volq);  // the ring's volume
	__syncwarp();
	float2 Uc = make_float2(0.0f, 0.0f);
	if (lane < nh) Uc = hex_ring_elem<VMODE>(C, S, bp, lane, ei, clo, chi, volume);
	const float U0 = warp_sum(Uc.x), U1 = warp_sum(Uc.y);
	__syncwarp();
	// each node's gradients: its contributions summed in hex order
	Vec3 g0 = {0.0f, 0.0f, 0.0f}, g1 = {0.0f, 0.0f, 0.0f};
	float w = 0.0f;
	float4 Dn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	if (lane < nn) {
		const uint16_t* cl = C.ring_cwords + __ldg(C.ring_clist + r);
		const uint32_t cb = __ldg(cl + lane), ce = __ldg(cl + lane + 1);
		for (uint32_t i = cb; i < ce; i++) {
			const uint32_t q = __ldg(cl + nn + 1 + i), j = q >> 3, k = q & 7u;
			g0 = {g0.x + S.g0[j][k][0], g0.y + S.g0[j][k][1], g0.z + S.g0[j][k][2]};
			g1 = {g1.x + S.g1[j][k][0], g1.y + S.g1[j][k][1], g1.z + S.g1[j][k][2]};
		}
		w = S.O[lane].w;
		Dn = S.D[lane];
	}
	if (__ldg(&bp.energy) == 8u) {
		// ContinuousPixar: mu = 2, one constraint U0 + (lambda / 2) U1 with
		// compliance per the ring volume
		const float hw = __ldg(&bp.hw);
		const float U = fmaxf(0.000001f, fmaf(hw, U1, U0));
		const Vec3 g = {fmaf(hw, g1.x, g0.x), fmaf(hw, g1.y, g0.y), fmaf(hw, g1.z, g0.z)};
		ring_update1<DAMP, VMODE>(C, bp, lane, nn, dv, S.O[lane], Dn, w, g, U, __ldg(&bp.compliance) / volume, inv_dt,
		                          inv_dt2, rd);
		return;
	}
	// ContinuousMixed / ContinuousSkin: the deviatoric and hydrostatic pair
	const float mu = __ldg(&bp.mu), lambda = __ldg(&bp.lambda);
	ring_update2<DAMP, VMODE>(C, bp, lane, nn, dv, S.O[lane], Dn, w, g0, g1, fmaxf(0.0001f, U0), U1,
	                          1.0f / (mu * volume), 1.0f / (lambda * volume), inv_dt, inv_dt2, rd);
}

// The persistent hex ring kernel (cooperative launch, co-resident grid):
// per substep the advance pass, one pass per ring colour, and with post-step
// damping a finalize pass, the rings' Rayleigh passes and the PBD passes
// over the hex colours (GeoLinear3d::Damp, XPBDFEM/Geo.cpp:800-811).
template <bool DAMP>
__global__ void __launch_bounds__(256) k_hex_rings(DevCtx C, uint32_t nsub, float dt) {
	extern __shared__ __align__(128) unsigned char smem[];
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = (blockDim.x >> 5) * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	HexRingScratch& S = reinterpret_cast<HexRingScratch*>(smem)[wib];
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
			for (uint32_t r = rb + gwarp; r < re; r += nwarps)
				hex_ring_solve<DAMP, false>(C, S, r, lane, inv_dt, inv_dt2, 0);
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
						hex_ring_solve<true, true>(C, S, r, lane, inv_dt, inv_dt2, tick);
					if (!grid_sync(C, target)) return;
				}
			if (C.damp_kinds & 2u)
				for (uint32_t c = 0; c < C.el_colours; c++) {
					const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
					for (uint32_t i = b + gtid; i < e; i += nthreads) {
						const BodyParams& bp = body_of_el<HexElem>(C, i);
						if (__ldg(&bp.pbd_on) && in_slice(C, bp, i, tick))
							// inlined: ptxas 13.0 crashed on the out-of-line call from this kernel
							hex_pbd_inl(C, i, __ldg(&bp.rayleigh_type) == 3u ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff));
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

int launch_hexes(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	return launch_elements<HexElem>(ctx, block, nsub, dt, stream);
}

int launch_hex_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = ctx.ext != 0u ? (const void*)k_hex_rings<true> : (const void*)k_hex_rings<false>;
	const size_t smem = (size_t)(block / 32) * sizeof(HexRingScratch);
	cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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

}  // namespace xfem
