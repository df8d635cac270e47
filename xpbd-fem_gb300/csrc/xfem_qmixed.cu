// Quadratic mixed mode of libxfem.so (sm_103a): GeoQuadratic3d on a mesh
// mixing tets and hexes (XPBDFEM/Geo.cpp:836-1008), T10s and H27s in one
// body. GeoQuadratic3d::Constrain solves every T10 in tOrder, then every H27
// in hOrder, and each volume pass the same way; Damp runs the Rayleigh
// damping over the T10s then the H27s, then the PBD damping over the T10s
// then the H27s, each over the amortized slice of its own order. Here each
// kind keeps its own colouring and its own element arrays, so a sweep is the
// T10 colours (one thread per T10, the T10 mode's code) followed by the H27
// colours (one warp per H27, the H27 mode's code), each behind the grid
// barrier. The kernel takes two contexts that differ only in their element
// arrays: Ct holds the T10s, Ch the H27s.
#include "xfem_h27_elem.cuh"
#include "xfem_t10_elem.cuh"

namespace xfem {

namespace {

using T10 = t10e::T10Elem;
using H27 = h27e::H27Elem;

// Whether element i (its index f = el_flat[i] in its body's order of n) is
// in this tick's damping slice (PostAmortized: one eighth per substep).
__device__ __forceinline__ bool in_slice_n(const DevCtx& C, const BodyParams& bp, uint32_t i, uint32_t n,
                                           uint32_t tick) {
	if (__ldg(&bp.rayleigh_type) != 3u) return true;
	const uint32_t m = tick % 8u, f = __ldg(C.el_flat + i);
	return f >= n * m / 8u && f < n * (m + 1u) / 8u;
}

// One pass kind over the colours of one element kind (units: threads for
// T10s, warps for H27s); false when a barrier gave up.
template <class E, int KIND>
__device__ __forceinline__ bool sweep(const DevCtx& C, const DevCtx& B, uint32_t gtid, uint32_t nthreads, float inv_dt,
                                      float inv_dt2, uint32_t it, uint32_t tick, uint32_t& target) {
	const uint32_t unit = E::kWarp ? gtid >> 5 : gtid, nunits = E::kWarp ? nthreads >> 5 : nthreads;
	for (uint32_t c = 0; c < C.el_colours; c++) {
		const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
		for (uint32_t i = b + unit; i < e; i += nunits) {
			if (KIND == kSolve) {
				E::template pass<kSolve>(C, i, inv_dt, inv_dt2, 0.0f);
				continue;
			}
			const BodyParams& bp = body_of_el<E>(C, i);
			const uint32_t n = E::kWarp ? __ldg(&bp.nhexes) : __ldg(&bp.ntets);
			if (KIND == kVolume) {
				if (it < __ldg(&bp.volume_passes)) E::template pass<kVolume>(C, i, inv_dt, inv_dt2, 0.0f);
			} else if (KIND == kRayleigh) {
				const uint32_t type = __ldg(&bp.rayleigh_type);
				const float rd = __ldg(&bp.damping) * (type == 3u ? 8.0f : 1.0f);
				if (type >= 2u && rd > 0.0f && in_slice_n(C, bp, i, n, tick))
					E::template pass<kRayleigh>(C, i, inv_dt, inv_dt2, rd);
			} else if (__ldg(&bp.pbd_on) && in_slice_n(C, bp, i, n, tick)) {
				E::pbd(C, i, __ldg(&bp.rayleigh_type) == 3u ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff));
			}
		}
		if (!grid_sync(B, target)) return false;
	}
	return true;
}

constexpr int kPbd = 100;  // the PBD damping sweep (not a pass kind of the elements)

__global__ void __launch_bounds__(256, 1) k_qmixed(DevCtx Ch, DevCtx Ct, uint32_t nsub, float dt) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	const uint32_t tick0 = __ldcg(Ch.tick);
	const bool dmode = Ch.damp_kinds != 0u;
	uint32_t target = Ch.bar_base;
	for (uint32_t s = 0; s < nsub; s++) {
		for (uint32_t v = gtid; v < Ch.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(Ch.vert + 2 * (size_t)v, O, D);
			advance_vertex(Ch, v, O, D, s == 0 || dmode, dt, inv_dt);
			st_vertex(Ch.vert + 2 * (size_t)v, O, D);
		}
		if (!grid_sync(Ch, target)) return;
		const uint32_t tick = tick0 + s;
		if (!sweep<T10, kSolve>(Ct, Ch, gtid, nthreads, inv_dt, inv_dt2, 0, tick, target)) return;
		if (!sweep<H27, kSolve>(Ch, Ch, gtid, nthreads, inv_dt, inv_dt2, 0, tick, target)) return;
		for (uint32_t it = 0; it < Ch.nvol; it++) {
			if (!sweep<T10, kVolume>(Ct, Ch, gtid, nthreads, inv_dt, inv_dt2, it, tick, target)) return;
			if (!sweep<H27, kVolume>(Ch, Ch, gtid, nthreads, inv_dt, inv_dt2, it, tick, target)) return;
		}
		if (!dmode) continue;
		for (uint32_t v = gtid; v < Ch.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(Ch.vert + 2 * (size_t)v, O, D);
			finalize_vertex(Ch, v, O, D, inv_dt);
			st_vertex(Ch.vert + 2 * (size_t)v, O, D);
		}
		if (!grid_sync(Ch, target)) return;
		if (Ch.damp_kinds & 1u) {
			if (!sweep<T10, kRayleigh>(Ct, Ch, gtid, nthreads, inv_dt, inv_dt2, 0, tick, target)) return;
			if (!sweep<H27, kRayleigh>(Ch, Ch, gtid, nthreads, inv_dt, inv_dt2, 0, tick, target)) return;
		}
		if (Ch.damp_kinds & 2u) {
			if (!sweep<T10, kPbd>(Ct, Ch, gtid, nthreads, inv_dt, inv_dt2, 0, tick, target)) return;
			if (!sweep<H27, kPbd>(Ch, Ch, gtid, nthreads, inv_dt, inv_dt2, 0, tick, target)) return;
		}
	}
	if (!dmode) {
		for (uint32_t v = gtid; v < Ch.nverts; v += nthreads) {
			float4 O, D;
			ld_vertex(Ch.vert + 2 * (size_t)v, O, D);
			finalize_vertex(Ch, v, O, D, inv_dt);
			st_vertex(Ch.vert + 2 * (size_t)v, O, D);
		}
	}
	if (gtid == 0) *Ch.tick = tick0 + nsub;
}

}  // namespace

int launch_qmixed(const DevCtx& ch27, const DevCtx& ct10, int block, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	if (block != 256) return (int)cudaErrorInvalidConfiguration;  // the H27 scratch is sized for 8 warps
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = (const void*)k_qmixed;
	int dev = 0, sms = 0, per_sm = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, block, 0);
	if (e != cudaSuccess) return (int)e;
	if (per_sm <= 0) return (int)cudaErrorInvalidConfiguration;
	e = reset_barrier(ch27, st);
	if (e != cudaSuccess) return (int)e;
	DevCtx a = ch27, b = ct10;
	void* args[] = {&a, &b, &nsub, &dt};
	return (int)cudaLaunchCooperativeKernel(f, dim3(per_sm * sms), dim3(block), args, 0, st);
}

}  // namespace xfem
