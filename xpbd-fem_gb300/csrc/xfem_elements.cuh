// Element modes of libxfem.so (sm_103a): the pieces shared by the hex mode
// (xfem_hexes.cu) and the quadratic-tet mode (xfem_t10.cu). The constraint
// solves over N nodes (XPBDFEM/Xpbd.h:87-215), PbdDamp over N nodes
// (XPBDFEM/Xpbd.h:306-346), and the persistent kernel that runs a substep as
// GeoLinear3d / GeoQuadratic3d do: one pass that advances every vertex, one
// pass per colour with one thread per element, the volume sweeps, and with
// post-step damping a finalize pass and the damping passes, each pass ended
// by the bounded grid barrier. Internal linkage: each translation unit gets
// its own copy.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "xfem_device.cuh"
#include "xfem_internal.h"

namespace xfem {

namespace {

// Pass kinds of one element. kSolve: SolveElement; kVolume: SolveVolumeOnly;
// kRayleigh: DampElement on the canonical state (O = X, D = V).
enum ElemPass { kSolve = 0, kVolume = 1, kRayleigh = 2 };

// adjugate and J through the first adjugate column (XPBDFEM/Fem.cpp:284-306)
__device__ __forceinline__ float adj_det(const float F[3][3], float A[3][3]) {
	A[0][0] = fmaf(F[1][1], F[2][2], -F[1][2] * F[2][1]);
	A[0][1] = -fmaf(F[0][1], F[2][2], -F[0][2] * F[2][1]);
	A[0][2] = fmaf(F[0][1], F[1][2], -F[0][2] * F[1][1]);
	A[1][0] = -fmaf(F[1][0], F[2][2], -F[1][2] * F[2][0]);
	A[1][1] = fmaf(F[0][0], F[2][2], -F[0][2] * F[2][0]);
	A[1][2] = -fmaf(F[0][0], F[1][2], -F[0][2] * F[1][0]);
	A[2][0] = fmaf(F[1][0], F[2][1], -F[1][1] * F[2][0]);
	A[2][1] = -fmaf(F[0][0], F[2][1], -F[0][1] * F[2][0]);
	A[2][2] = fmaf(F[0][0], F[1][1], -F[0][1] * F[1][0]);
	return fmaf(F[0][0], A[0][0], fmaf(F[0][1], A[1][0], F[0][2] * A[2][0]));
}

template <int N>
__device__ __forceinline__ void rootn(Vec3 g[N]) {  // g[N - 1] -= the others
	Vec3 s = {0.0f, 0.0f, 0.0f};
#pragma unroll
	for (int n = 0; n < N - 1; n++) s = {s.x + g[n].x, s.y + g[n].y, s.z + g[n].z};
	g[N - 1] = {g[N - 1].x - s.x, g[N - 1].y - s.y, g[N - 1].z - s.z};
}

template <int N>
__device__ __forceinline__ void zeron(Vec3 g[N]) {
#pragma unroll
	for (int n = 0; n < N; n++) g[n] = {0.0f, 0.0f, 0.0f};
}

template <int N>
__device__ __forceinline__ float wdotn(const float w[N], const Vec3 a[N], const Vec3 b[N]) {
	float s = 1.0e-22f;
#pragma unroll
	for (int n = 0; n < N; n++) s = fmaf(w[n], dot(a[n], b[n]), s);
	return s;
}

template <int N>
__device__ __forceinline__ float gdotn(const Vec3 g[N], const float4 D[N]) {
	float s = 0.0f;
#pragma unroll
	for (int n = 0; n < N; n++) s = fmaf(g[n].x, D[n].x, fmaf(g[n].y, D[n].y, fmaf(g[n].z, D[n].z, s)));
	return s;
}

template <int N>
__device__ __forceinline__ void moven(const float w[N], float l, const Vec3 g[N], float4 D[N]) {
#pragma unroll
	for (int n = 0; n < N; n++) {
		const float s = w[n] * l;
		D[n].x = fmaf(s, g[n].x, D[n].x);
		D[n].y = fmaf(s, g[n].y, D[n].y);
		D[n].z = fmaf(s, g[n].z, D[n].z);
	}
}

// One constraint (XPBDFEM/Xpbd.h:87-121) with the in-solve Rayleigh damping
// (types 0 Paper, 1 Limit) when `damp` > 0, from wgg = sum w g.g and gV =
// sum g.(X - O) (read only with damping).
__device__ __forceinline__ float lambda1_of(float U, float wgg, float gV, float alpha, float comp, float damp, bool limit,
                                           float inv_dt) {
	if (!(damp > 0.0f)) return (-2.0f * U) / fmaf(2.0f * U, alpha, wgg);
	const float gamma = damp * inv_dt;
	if (!limit) return (-2.0f * U - gamma * gV) / fmaf(wgg, 1.0f + gamma, 2.0f * U * alpha);
	const float l = (-2.0f * U) / fmaf(2.0f * U, alpha, wgg);
	const float A = fmaf(2.0f * U, comp * inv_dt / damp, wgg);
	const float b = (-gV - wgg * l) * (A / fmaxf(A, 4.0f * wgg));
	return l + b / A;
}

template <int N>
__device__ __forceinline__ float lambda1n(float U, const Vec3 g[N], const float w[N], const float4 D[N], float alpha,
                                         float comp, float damp, bool limit, float inv_dt) {
	const float wgg = wdotn<N>(w, g, g);
	return lambda1_of(U, wgg, damp > 0.0f ? gdotn<N>(g, D) : 0.0f, alpha, comp, damp, limit, inv_dt);
}

// The coupled pair (XPBDFEM/Xpbd.h:123-215): Cramer's rule, the damping forms
// of :133-205, from the weighted gradient products and (with damping) the
// gradients' products with X - O.
__device__ __forceinline__ void lambda2_of(float U0, float U1, float wgg0, float wgg1, float wgg2, float gV0, float gV1,
                                           float alpha0, float alpha1, float comp0, float comp1, float damp, bool limit,
                                           float inv_dt, float& l0, float& l1) {
	if (!(damp > 0.0f)) {
		cramer(fmaf(2.0f * U0, alpha0, wgg0), wgg1, fmaf(2.0f * U1, alpha1, wgg2), -2.0f * U0, -2.0f * U1, l0, l1);
		return;
	}
	const float gamma = damp * inv_dt;
	float A0, A2, b0 = -2.0f * U0, b1 = -2.0f * U1;
	if (!limit) {
		const float s = 1.0f / (1.0f + gamma);
		A0 = wgg0 + (2.0f * U0 * alpha0) * s;
		A2 = wgg2 + (2.0f * U1 * alpha1) * s;
		b0 = (b0 - gamma * gV0) * s;
		b1 = (b1 - gamma * gV1) * s;
	} else {
		A0 = fmaf(2.0f * U0, alpha0, wgg0);
		A2 = fmaf(2.0f * U1, alpha1, wgg2);
	}
	cramer(A0, wgg1, A2, b0, b1, l0, l1);
	if (limit) {
		const float B0 = fmaf(2.0f * U0, comp0 * inv_dt / damp, wgg0), B2 = fmaf(2.0f * U1, comp1 * inv_dt / damp, wgg2);
		float e0 = fmaf(b0, -1.0f - alpha0 * l0, -gV0), e1 = fmaf(b1, -1.0f - alpha1 * l1, -gV1);
		e0 *= B0 / fmaxf(B0, 8.0f * wgg0);
		e1 *= B2 / fmaxf(B2, 8.0f * wgg2);
		float d0, d1;
		cramer(B0, wgg1, B2, e0, e1, d0, d1);
		l0 += d0;
		l1 += d1;
	}
}

template <int N>
__device__ __forceinline__ void lambda2n(float U0, float U1, const Vec3 g0[N], const Vec3 g1[N], const float w[N],
                                        const float4 D[N], float alpha0, float alpha1, float comp0, float comp1,
                                        float damp, bool limit, float inv_dt, float& l0, float& l1) {
	const float wgg0 = wdotn<N>(w, g0, g0), wgg1 = wdotn<N>(w, g1, g0), wgg2 = wdotn<N>(w, g1, g1);
	const bool dm = damp > 0.0f;
	lambda2_of(U0, U1, wgg0, wgg1, wgg2, dm ? gdotn<N>(g0, D) : 0.0f, dm ? gdotn<N>(g1, D) : 0.0f, alpha0, alpha1,
	           comp0, comp1, damp, limit, inv_dt, l0, l1);
}

__device__ __forceinline__ bool full_quadrature(uint32_t e) { return e == 3u || e == 5u || e == 6u; }


// PbdDamp over an element's N nodes (XPBDFEM/Xpbd.h:306-346) on the
// canonical state: towards the rigid motion (centre-of-mass velocity plus
// rotation); dv: the device vertex ids, coeff / area capped at 1.
template <int N>
__device__ __forceinline__ void pbd_nodes(const DevCtx& C, const uint32_t dv[N], float damping) {
	float4 X[N], V[N];
#pragma unroll
	for (int n = 0; n < N; n++) ld_vertex(C.vert + 2 * (size_t)dv[n], X[n], V[n]);
	float Wsum = 1.0e-8f;
#pragma unroll
	for (int n = 0; n < N; n++) Wsum += X[n].w;
	const float Wavg = Wsum * (1.0f / (float)N), Wmin = 0.0001f * Wavg;
	Vec3 x[N], xcm = {0.0f, 0.0f, 0.0f}, vcm = {0.0f, 0.0f, 0.0f};
	float M[N], Msum = 0.0f;
#pragma unroll
	for (int n = 0; n < N; n++) {
		x[n] = {X[n].x - X[N - 1].x, X[n].y - X[N - 1].y, X[n].z - X[N - 1].z};
		M[n] = Wavg / fmaxf(Wmin, X[n].w);
		xcm = {fmaf(x[n].x, M[n], xcm.x), fmaf(x[n].y, M[n], xcm.y), fmaf(x[n].z, M[n], xcm.z)};
		vcm = {fmaf(V[n].x, M[n], vcm.x), fmaf(V[n].y, M[n], vcm.y), fmaf(V[n].z, M[n], vcm.z)};
		Msum += M[n];
	}
	const float im = 1.0f / Msum;
	xcm = {xcm.x * im, xcm.y * im, xcm.z * im};
	vcm = {vcm.x * im, vcm.y * im, vcm.z * im};
	Vec3 r[N], L = {0.0f, 0.0f, 0.0f};
	float I00 = 0.0f, I11 = 0.0f, I22 = 0.0f, I01 = 0.0f, I12 = 0.0f, I02 = 0.0f;
#pragma unroll
	for (int n = 0; n < N; n++) {
		r[n] = {x[n].x - xcm.x, x[n].y - xcm.y, x[n].z - xcm.z};
		const Vec3 c = cross(r[n], v3(V[n]));
		L = {fmaf(M[n], c.x, L.x), fmaf(M[n], c.y, L.y), fmaf(M[n], c.z, L.z)};
		const float xx = r[n].x * r[n].x, yy = r[n].y * r[n].y, zz = r[n].z * r[n].z;
		I00 = fmaf(M[n], yy + zz, I00);
		I11 = fmaf(M[n], xx + zz, I11);
		I22 = fmaf(M[n], xx + yy, I22);
		I01 = fmaf(-M[n], r[n].x * r[n].y, I01);
		I12 = fmaf(-M[n], r[n].y * r[n].z, I12);
		I02 = fmaf(-M[n], r[n].z * r[n].x, I02);
	}
	const float a00 = fmaf(I11, I22, -I12 * I12), a01 = fmaf(I02, I12, -I01 * I22), a02 = fmaf(I01, I12, -I02 * I11);
	const float a11 = fmaf(I00, I22, -I02 * I02), a12 = fmaf(I01, I02, -I00 * I12), a22 = fmaf(I00, I11, -I01 * I01);
	const float idet = 1.0f / fmaf(I00, a00, fmaf(I01, a01, I02 * a02));
	const Vec3 om = {fmaf(a00, L.x, fmaf(a01, L.y, a02 * L.z)) * idet, fmaf(a01, L.x, fmaf(a11, L.y, a12 * L.z)) * idet,
	                 fmaf(a02, L.x, fmaf(a12, L.y, a22 * L.z)) * idet};
#pragma unroll
	for (int n = 0; n < N; n++) {
		const Vec3 c = cross(om, r[n]);
		V[n].x = fmaf(damping, (vcm.x + c.x) - V[n].x, V[n].x);
		V[n].y = fmaf(damping, (vcm.y + c.y) - V[n].y, V[n].y);
		V[n].z = fmaf(damping, (vcm.z + c.z) - V[n].z, V[n].z);
		st_vertex(C.vert + 2 * (size_t)dv[n], X[n], V[n]);
	}
}

// Whether element i is in this tick's damping slice (PostAmortized: one
// eighth of its body's element order per substep, XPBDFEM/Geo.cpp:793-797).
__device__ __forceinline__ bool in_slice(const DevCtx& C, const BodyParams& bp, uint32_t i, uint32_t tick) {
	if (__ldg(&bp.rayleigh_type) != 3u) return true;
	const uint32_t nh = __ldg(&bp.ntets), m = tick % 8u, f = __ldg(C.el_flat + i);
	return f >= nh * m / 8u && f < nh * (m + 1u) / 8u;
}

template <class E>
__device__ __forceinline__ const BodyParams& body_of_el(const DevCtx& C, uint32_t i) {
	const uint32_t v0 = __ldg(&C.el_vid[E::kVid4 * (size_t)i].x);
	return C.bodies[__float_as_uint(__ldcg(&C.vert[2 * (size_t)v0 + 1].w)) >> 8];
}

// The persistent element kernel (cooperative launch, co-resident grid). E:
// the element type (kVid4 uint4 of vertex ids per element; pass<KIND>, pbd;
// kWarp: one warp per element, every lane of the warp calling with the same
// element, else one thread per element; kMinBlocks: the blocks per SM the
// register budget is sized for).
template <class E>
__global__ void __launch_bounds__(256, E::kMinBlocks) k_elements(DevCtx C, uint32_t nsub, float dt) {
	const float inv_dt = 1.0f / dt, inv_dt2 = 1.0f / (dt * dt);
	const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
	// the element loops run over units: threads, or warps (warp-uniform i)
	const uint32_t unit = E::kWarp ? gtid >> 5 : gtid, nunits = E::kWarp ? nthreads >> 5 : nthreads;
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
		for (uint32_t c = 0; c < C.el_colours; c++) {
			const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
			for (uint32_t i = b + unit; i < e; i += nunits) E::template pass<kSolve>(C, i, inv_dt, inv_dt2, 0.0f);
			if (!grid_sync(C, target)) return;
		}
		for (uint32_t it = 0; it < C.nvol; it++)
			for (uint32_t c = 0; c < C.el_colours; c++) {
				const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
				for (uint32_t i = b + unit; i < e; i += nunits)
					if (it < __ldg(&body_of_el<E>(C, i).volume_passes)) E::template pass<kVolume>(C, i, inv_dt, inv_dt2, 0.0f);
				if (!grid_sync(C, target)) return;
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
		if (C.damp_kinds & 1u)
			for (uint32_t c = 0; c < C.el_colours; c++) {
				const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
				for (uint32_t i = b + unit; i < e; i += nunits) {
					const BodyParams& bp = body_of_el<E>(C, i);
					const uint32_t type = __ldg(&bp.rayleigh_type);
					const float rd = __ldg(&bp.damping) * (type == 3u ? 8.0f : 1.0f);
					if (type >= 2u && rd > 0.0f && in_slice(C, bp, i, tick)) E::template pass<kRayleigh>(C, i, inv_dt, inv_dt2, rd);
				}
				if (!grid_sync(C, target)) return;
			}
		if (C.damp_kinds & 2u)
			for (uint32_t c = 0; c < C.el_colours; c++) {
				const uint32_t b = __ldg(C.colour_el_begin + c), e = __ldg(C.colour_el_begin + c + 1);
				for (uint32_t i = b + unit; i < e; i += nunits) {
					const BodyParams& bp = body_of_el<E>(C, i);
					if (__ldg(&bp.pbd_on) && in_slice(C, bp, i, tick))
						E::pbd(C, i, __ldg(&bp.rayleigh_type) == 3u ? __ldg(&bp.pbd_coeff_amortized) : __ldg(&bp.pbd_coeff));
				}
				if (!grid_sync(C, target)) return;
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

template <class E>
int launch_elements(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream) {
	if (nsub == 0) return 0;
	cudaStream_t st = (cudaStream_t)stream;
	const void* f = (const void*)k_elements<E>;
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


}  // namespace

}  // namespace xfem
