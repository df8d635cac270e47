// One-ring mode of libxfem.so (sm_103a): the continuous-pressure models
// (energy ids 8-10), where GeoLinear3d::Constrain solves one constraint (or
// a coupled pair) per vertex over the tets around it instead of one per tet
// (SolveRing, XPBDFEM/Geo.cpp:147-193; the first-order branch of
// CalculateElementEnergyAndGradients, XPBDFEM/Fem.cpp:942-979; SolveSimplex,
// XPBDFEM/Geo.cpp:12-64).
//
// Schedule: vertices coloured so that the rings of one colour share no node;
// a substep is one pass that advances every vertex (finishes the previous
// substep, predicts this one), then one pass per colour, each ended by the
// grid barrier; the launch ends with a finalize pass.
//
// One warp per ring: lane j takes the ring's tet j (its I1 and volume ratio J
// with their gradients, weighted by the tet's share of the ring volume),
// lane n the ring's node n (the sum of its gradient contributions in tet
// order, from a per-node list of its tet corners, then its update). Sums over lanes run in a fixed butterfly order,
// so every launch gives the same bits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "xfem_device.cuh"
#include "xfem_internal.h"
#include "xfem_ring_update.cuh"

namespace xfem {

namespace {

// Per-warp scratch in shared memory.
struct RingScratch {
	float4 O[kMaxRingNodes], D[kMaxRingNodes];  // ring nodes: (O, w), (D, bits)
	float g0[kMaxRingTets][4][3];               // per tet corner: I1 gradient contribution
	float g1[kMaxRingTets][4][3];               // per tet corner: J gradient contribution
};

// SolveRing of ring r by the calling warp (every lane takes part). VMODE:
// the post-step Rayleigh damping form (SolveRing with V, XPBDFEM/Geo.cpp:
// 147-193, called by GeoLinear3d::Damp, XPBDFEM/Geo.cpp:800-806) on the
// canonical state (X, V): energies and gradients at X, RayleighDamp
// (XPBDFEM/Xpbd.h:217-263) on V, for the rings of this tick's slice.
template <bool DAMP, bool VMODE>
__device__ __noinline__ void ring_solve(const DevCtx& C, RingScratch& S, uint32_t r, uint32_t lane, float inv_dt,
                                        float inv_dt2, uint32_t tick) {
	__syncwarp();  // every lane is done with the previous ring's scratch
	const uint4 h = __ldg(C.ring_hdr + r);
	const uint32_t nn = h.z & 0xffu, nt = (h.z >> 8) & 0xffu;
	const BodyParams& bp = C.bodies[h.z >> 16];
	float rd = 0.0f;  // VMODE: the Rayleigh ratio (x 8 when amortized)
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
	// lane j takes the ring's tets j and j + 32
	float volq = 0.0f;
	for (uint32_t j = lane; j < nt; j += 32) {
		volq += 0.25f * __ldg(&C.ring_ent[2 * ((size_t)h.y + j) + 1].z);
	}
	const float volume = warp_sum(volq);  // the ring's volume
	__syncwarp();
	float U0c = 0.0f, U1c = 0.0f;
	for (uint32_t j = lane; j < nt; j += 32) {
		const float4 e0 = __ldg(C.ring_ent + 2 * ((size_t)h.y + j)), e1 = __ldg(C.ring_ent + 2 * ((size_t)h.y + j) + 1);
		const float QQ[3] = {e0.x, e0.y, e0.z}, QR[3] = {e0.w, e1.x, e1.y};
		const float vol = e1.z;
		const uint32_t cn = __float_as_uint(e1.w);
		float4 O[4], D[4];
#pragma unroll
		for (int k = 0; k < 4; k++) {
			const uint32_t q = (cn >> (8 * k)) & 0xffu;
			O[k] = S.O[q];
			D[k] = S.D[q];
		}
		Vec3 P[3];
#pragma unroll
		for (int i = 0; i < 3; i++)
			P[i] = VMODE ? Vec3{O[i].x - O[3].x, O[i].y - O[3].y, O[i].z - O[3].z}
			             : Vec3{(O[i].x - O[3].x) + (D[i].x - D[3].x), (O[i].y - O[3].y) + (D[i].y - D[3].y),
			                    (O[i].z - O[3].z) + (D[i].z - D[3].z)};
		const float ew = (vol * 0.25f) / volume;  // the tet's share of the ring volume
		Vec3 gI[4];
		const float I1 = prefactored_i1(QQ, QR, P, gI);
		// J = det[P0 P1 P2] / (6 vol); dJ/dP_i: the cofactor rows P1 x P2, P2 x P0, P0 x P1
		const Vec3 c0 = cross(P[1], P[2]), c1 = cross(P[2], P[0]), c2 = cross(P[0], P[1]);
		const float det = dot(P[0], c0);
		const float s6 = 1.0f / (6.0f * vol);
		U0c += ew * I1;
		U1c += ew * (det * s6);
		const float sj = ew * s6;
		const Vec3 cs[4] = {c0, c1, c2, {-(c0.x + c1.x + c2.x), -(c0.y + c1.y + c2.y), -(c0.z + c1.z + c2.z)}};
#pragma unroll
		for (int k = 0; k < 4; k++) {
			S.g0[j][k][0] = ew * gI[k].x;
			S.g0[j][k][1] = ew * gI[k].y;
			S.g0[j][k][2] = ew * gI[k].z;
			S.g1[j][k][0] = sj * cs[k].x;
			S.g1[j][k][1] = sj * cs[k].y;
			S.g1[j][k][2] = sj * cs[k].z;
		}
	}
	const float I1 = warp_sum(U0c), J = warp_sum(U1c);
	__syncwarp();
	// each node's gradients: its contributions summed in tet order
	Vec3 g0 = {0.0f, 0.0f, 0.0f}, g1 = {0.0f, 0.0f, 0.0f};
	float w = 0.0f;
	float4 Dn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	if (lane < nn) {
		const uint16_t* cl = C.ring_cwords + __ldg(C.ring_clist + r);
		const uint32_t cb = __ldg(cl + lane), ce = __ldg(cl + lane + 1);
		for (uint32_t i = cb; i < ce; i++) {
			const uint32_t q = __ldg(cl + nn + 1 + i), j = q >> 2, k = q & 3u;
			g0 = {g0.x + S.g0[j][k][0], g0.y + S.g0[j][k][1], g0.z + S.g0[j][k][2]};
			g1 = {g1.x + S.g1[j][k][0], g1.y + S.g1[j][k][1], g1.z + S.g1[j][k][2]};
		}
		w = S.O[lane].w;
		Dn = S.D[lane];
	}
	if (__ldg(&bp.energy) == 8u) {
		// ContinuousPixar: mu = 2, one constraint U = I1 + (lambda/2)(J - a)^2
		// with compliance per the ring volume
		const float a = __ldg(&bp.a), hw = __ldg(&bp.hw);
		const float U = fmaxf(0.0000001f, fmaf(hw * (J - a), J - a, I1));
		const float s1 = 2.0f * hw * (J - a);
		const Vec3 g = {fmaf(s1, g1.x, g0.x), fmaf(s1, g1.y, g0.y), fmaf(s1, g1.z, g0.z)};
		ring_update1<DAMP, VMODE>(C, bp, lane, nn, dv, S.O[lane], Dn, w, g, U, __ldg(&bp.compliance) / volume, inv_dt,
		                          inv_dt2, rd);
		return;
	}
	// ContinuousMixed / ContinuousSkin: the deviatoric and hydrostatic pair
	const float mu = __ldg(&bp.mu), lambda = __ldg(&bp.lambda), a = __ldg(&bp.a);
	float U0 = I1;
	if (__ldg(&bp.energy) == 10u) {
		const float C0 = __ldg(&bp.yeoh[0]), C1 = __ldg(&bp.yeoh[1]), C2 = __ldg(&bp.yeoh[2]);
		const float IM = I1 - 3.0f;
		U0 = fmaxf(0.0001f, IM * fmaf(IM, fmaf(IM, C2, C1), C0));
		const float gs = fmaf(IM, fmaf(IM, 3.0f * C2, 2.0f * C1), C0);
		g0 = {g0.x * gs, g0.y * gs, g0.z * gs};
	}
	const float U1 = (J - a) * (J - a);
	const float gs1 = 2.0f * (J - a);
	g1 = {g1.x * gs1, g1.y * gs1, g1.z * gs1};
	ring_update2<DAMP, VMODE>(C, bp, lane, nn, dv, S.O[lane], Dn, w, g0, g1, U0, U1, 1.0f / (mu * volume),
	                          1.0f / (lambda * volume), inv_dt, inv_dt2, rd);
}

// PBD damping of one tet cluster (its tets in sequence; clusters of one
// colour share no vertex) on the canonical state, for the tets of this
// tick's slice (GeoLinear3d::Damp, XPBDFEM/Geo.cpp:807-810).
__device__ void pbd_cluster(const DevCtx& C, uint32_t k, uint32_t tick) {
	const uint2 cl = __ldg(C.pbd_cl + k);
	for (uint32_t i = cl.x; i < cl.x + cl.y; i++) {
		const uint4 e = __ldg(C.pbd_ent + i);  // tet, index in its body's order, area bits, body
		const BodyParams& bp = C.bodies[e.w];
		if (!__ldg(&bp.pbd_on)) continue;
		const bool amort = __ldg(&bp.rayleigh_type) == 3u;
		if (amort) {
			const uint32_t nt = __ldg(&bp.ntets), m = tick % 8u;
			if (e.y < nt * m / 8u || e.y >= nt * (m + 1u) / 8u) continue;
		}
		const float coeff = amort ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff);
		uint32_t v[4];
		float4 X[4], V[4];
#pragma unroll
		for (int n = 0; n < 4; n++) {
			v[n] = __ldg(C.tet_verts + 4 * (size_t)e.x + n);
			ld_vertex(C.vert + 2 * (size_t)v[n], X[n], V[n]);
		}
		pbd_tet(X, V, fminf(1.0f, coeff / __uint_as_float(e.z)));
#pragma unroll
		for (int n = 0; n < 4; n++) st_vertex(C.vert + 2 * (size_t)v[n], X[n], V[n]);
	}
}

// The persistent ring kernel (cooperative launch, co-resident grid). DAMP:
// damping compiled in, in the solve and after it; with post-step damping
// (damp_kinds) every substep ends in the canonical state and runs the ring
// Rayleigh passes, then the PBD passes.
template <bool DAMP>
__global__ void __launch_bounds__(256) k_rings(DevCtx C, uint32_t nsub, float dt) {
	extern __shared__ __align__(128) unsigned char smem[];
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
	const uint32_t gwarp = wib * gridDim.x + blockIdx.x, nwarps = (blockDim.x >> 5) * gridDim.x;
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	RingScratch& S = reinterpret_cast<RingScratch*>(smem)[wib];
	const uint32_t tick0 = __ldcg(C.tick);
	const bool dmode = DAMP && C.damp_kinds != 0u;
	uint32_t target = C.bar_base;
	for (uint32_t s = 0; s < nsub; s++) {
		// finish the previous substep (unless the damping passes left the
		// canonical state) and predict this one, every vertex
		for (uint32_t v = gtid; v < C.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(C.vert + 2 * (size_t)v, O, D);
			advance_vertex(C, v, O, D, s == 0 || dmode, dt, inv_dt);
			st_vertex(C.vert + 2 * (size_t)v, O, D);
		}
		if (!grid_sync(C, target)) return;
		for (uint32_t c = 0; c < C.ring_colours; c++) {
			const uint32_t rb = __ldg(C.colour_ring_begin + c), re = __ldg(C.colour_ring_begin + c + 1);
			for (uint32_t r = rb + gwarp; r < re; r += nwarps) ring_solve<DAMP, false>(C, S, r, lane, inv_dt, inv_dt2, 0);
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
						ring_solve<true, true>(C, S, r, lane, inv_dt, inv_dt2, tick);
					if (!grid_sync(C, target)) return;
				}
			if (C.damp_kinds & 2u)
				for (uint32_t c = 0; c < C.pbd_colours; c++) {
					const uint32_t kb = __ldg(C.pbd_cl_begin + c), ke = __ldg(C.pbd_cl_begin + c + 1);
					for (uint32_t k = kb + gtid; k < ke; k += nthreads) pbd_cluster(C, k, tick);
					if (!grid_sync(C, target)) return;
				}
		}
	}
	if (!dmode) {
		// finish the last substep: (O, D) -> canonical (X, V)
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

int launch_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	const bool damp = ctx.ext != 0u;
	const void* f = damp ? (const void*)k_rings<true> : (const void*)k_rings<false>;
	const size_t smem = (size_t)(block / 32) * sizeof(RingScratch);
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
