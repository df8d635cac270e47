// Mixed mode of libxfem.so (sm_103a): one mesh holding linear tets and
// linear hexahedra, as GeoLinear3d holds them (XPBDFEM/Geo.cpp:697-811).
#include <cuda_runtime.h>
#include <stdint.h>

#include "xfem_hex_device.cuh"

namespace xfem {

namespace {

// ---- meshes mixing tets and hexes ------------------------------------------
//
// GeoLinear3d on a stream of tets and hexes (XPBDFEM/Geo.cpp:777-811): each
// sweep solves every tet, then every hex (the solve, each volume pass), and
// GeoLinear3d::Damp runs the Rayleigh damping over the tets then the hexes,
// then the PBD damping over the tets then the hexes. Here the tets have a
// colouring of their own (one thread per tet, as the hexes), so a sweep is
// the tet colours followed by the hex colours, each behind the grid barrier.

// Whether the element with flattened index f of n is in this tick's
// damping slice (PostAmortized: one eighth of the order per substep).
__device__ __forceinline__ bool in_slice_of(const BodyParams& bp, uint32_t f, uint32_t n, uint32_t tick) {
	if (__ldg(&bp.rayleigh_type) != 3u) return true;
	const uint32_t m = tick % 8u;
	return f >= n * m / 8u && f < n * (m + 1u) / 8u;
}

// One tet of a mixed mesh: SolveElement (kSolve), SolveVolumeOnly (kVolume)
// or DampElement on the canonical state with ratio rd (kRayleigh), the same
// tet code as the tet mode's; the compliance per volume (1 / mu) / volume
// is formed from the body's material as the tet mode's records hold it.
template <int KIND>
__device__ __noinline__ void mixed_tet_pass(const DevCtx& C, uint32_t i, float inv_dt, float inv_dt2, float rd) {
	const uint4 va = __ldg(C.mt_vid + i);
	const uint32_t dv[4] = {va.x, va.y, va.z, va.w};
	float4 O[4], D[4];
#pragma unroll
	for (int n = 0; n < 4; n++) ld_vertex(C.vert + 2 * (size_t)dv[n], O[n], D[n]);
	const uint32_t body = __float_as_uint(D[0].w) >> 8;
	const Mat mat = load_mat(C.bodies, body);
	const size_t n4 = C.nmt;
	const float4 r3 = __ldg(C.mt_rec + 3 * n4 + i);
	const TetRec tr = {__ldg(C.mt_rec + i), __ldg(C.mt_rec + n4 + i), __ldg(C.mt_rec + 2 * n4 + i),
	                   make_float4(r3.x, r3.y, r3.z, __ldg(&C.bodies[body].inv_mu) / r3.w)};
	if (KIND == kSolve)
		solve_tet<true>(mat, tr, inv_dt, inv_dt2, O, D);
	else if (KIND == kVolume)
		volume_tet(mat, tr, inv_dt2, O, D);
	else
		rayleigh_tet(mat, tr, O, D, inv_dt, rd);
#pragma unroll
	for (int n = 0; n < 4; n++) st_vertex(C.vert + 2 * (size_t)dv[n], O[n], D[n]);
}

__device__ __forceinline__ const BodyParams& body_of_mt(const DevCtx& C, uint32_t i) {
	const uint32_t v0 = __ldg(&C.mt_vid[i].x);
	return C.bodies[__float_as_uint(__ldcg(&C.vert[2 * (size_t)v0 + 1].w)) >> 8];
}

// The persistent mixed-mesh kernel (cooperative launch, co-resident grid).
__global__ void __launch_bounds__(256) k_mixed(DevCtx C, uint32_t nsub, float dt) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	const uint32_t tick0 = __ldcg(C.tick);
	const bool dmode = C.damp_kinds != 0u;
	uint32_t target = C.bar_base;
	for (uint32_t s = 0; s < nsub; s++) {
		for (uint32_t v = gtid; v < C.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(C.vert + 2 * (size_t)v, O, D);
			advance_vertex(C, v, O, D, s == 0 || dmode, dt, inv_dt);
			st_vertex(C.vert + 2 * (size_t)v, O, D);
		}
		if (!grid_sync(C, target)) return;
		// the solve, then each volume pass: every tet colour, then every hex colour
		for (uint32_t it = 0; it <= C.nvol; it++) {
			for (uint32_t c = 0; c < C.mt_colours; c++) {
				const uint32_t b = __ldg(C.colour_mt_begin + c), e = __ldg(C.colour_mt_begin + c + 1);
				for (uint32_t i = b + gtid; i < e; i += nthreads) {
					if (it == 0)
						mixed_tet_pass<kSolve>(C, i, inv_dt, inv_dt2, 0.0f);
					else if (it <= __ldg(&body_of_mt(C, i).volume_passes))
						mixed_tet_pass<kVolume>(C, i, inv_dt, inv_dt2, 0.0f);
				}
				if (!grid_sync(C, target)) return;
			}
			for (uint32_t c = 0; c < C.el_colours; c++) {
				const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
				for (uint32_t i = b + gtid; i < e; i += nthreads) {
					if (it == 0)
						hex_pass<kSolve>(C, i, inv_dt, inv_dt2, 0.0f);
					else if (it <= __ldg(&body_of_el<HexElem>(C, i).volume_passes))
						hex_pass<kVolume>(C, i, inv_dt, inv_dt2, 0.0f);
				}
				if (!grid_sync(C, target)) return;
			}
		}
		if (!dmode) continue;
		for (uint32_t v = gtid; v < C.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(C.vert + 2 * (size_t)v, O, D);
			finalize_vertex(C, v, O, D, inv_dt);
			st_vertex(C.vert + 2 * (size_t)v, O, D);
		}
		if (!grid_sync(C, target)) return;
		const uint32_t tick = tick0 + s;
		if (C.damp_kinds & 1u) {
			for (uint32_t c = 0; c < C.mt_colours; c++) {
				const uint32_t b = __ldg(C.colour_mt_begin + c), e = __ldg(C.colour_mt_begin + c + 1);
				for (uint32_t i = b + gtid; i < e; i += nthreads) {
					const BodyParams& bp = body_of_mt(C, i);
					const uint32_t type = __ldg(&bp.rayleigh_type);
					const float rd = __ldg(&bp.damping) * (type == 3u ? 8.0f : 1.0f);
					if (type >= 2u && rd > 0.0f && in_slice_of(bp, __ldg(C.mt_flat + i), __ldg(&bp.ntets), tick))
						mixed_tet_pass<kRayleigh>(C, i, inv_dt, inv_dt2, rd);
				}
				if (!grid_sync(C, target)) return;
			}
			for (uint32_t c = 0; c < C.el_colours; c++) {
				const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
				for (uint32_t i = b + gtid; i < e; i += nthreads) {
					const BodyParams& bp = body_of_el<HexElem>(C, i);
					const uint32_t type = __ldg(&bp.rayleigh_type);
					const float rd = __ldg(&bp.damping) * (type == 3u ? 8.0f : 1.0f);
					if (type >= 2u && rd > 0.0f && in_slice_of(bp, __ldg(C.el_flat + i), __ldg(&bp.nhexes), tick))
						hex_pass<kRayleigh>(C, i, inv_dt, inv_dt2, rd);
				}
				if (!grid_sync(C, target)) return;
			}
		}
		if (C.damp_kinds & 2u) {
			for (uint32_t c = 0; c < C.mt_colours; c++) {
				const uint32_t b = __ldg(C.colour_mt_begin + c), e = __ldg(C.colour_mt_begin + c + 1);
				for (uint32_t i = b + gtid; i < e; i += nthreads) {
					const BodyParams& bp = body_of_mt(C, i);
					if (!__ldg(&bp.pbd_on) || !in_slice_of(bp, __ldg(C.mt_flat + i), __ldg(&bp.ntets), tick)) continue;
					const float coeff = __ldg(&bp.rayleigh_type) == 3u ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff);
					const uint4 va = __ldg(C.mt_vid + i);
					const uint32_t dv[4] = {va.x, va.y, va.z, va.w};
					pbd_nodes<4>(C, dv, fminf(1.0f, coeff / __ldg(&C.mt_rec[4 * (size_t)C.nmt + i].x)));
				}
				if (!grid_sync(C, target)) return;
			}
			for (uint32_t c = 0; c < C.el_colours; c++) {
				const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
				for (uint32_t i = b + gtid; i < e; i += nthreads) {
					const BodyParams& bp = body_of_el<HexElem>(C, i);
					if (__ldg(&bp.pbd_on) && in_slice_of(bp, __ldg(C.el_flat + i), __ldg(&bp.nhexes), tick))
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

int launch_mixed(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = (const void*)k_mixed;
	int dev = 0, sms = 0, per_sm = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, block, 0);
	if (e != cudaSuccess) return (int)e;
	if (per_sm <= 0) return (int)cudaErrorInvalidConfiguration;
	e = reset_barrier(ctx, st);
	if (e != cudaSuccess) return (int)e;
	DevCtx c = ctx;
	void* args[] = {&c, &nsub, &dt};
	return (int)cudaLaunchCooperativeKernel(f, dim3(per_sm * sms), dim3(block), args, 0, st);
}

}  // namespace xfem
