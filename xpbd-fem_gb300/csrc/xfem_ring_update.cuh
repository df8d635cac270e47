// The multiplier update of one vertex one-ring (SolveRing's last step,
// XPBDFEM/Geo.cpp:186-225): EnergyXpbdConstrain for ContinuousPixar's single
// constraint, EnergyXpbdConstrainSimultaneous<2> for the coupled pair
// (XPBDFEM/Xpbd.h:87-215), or RayleighDamp in the post-step damping form
// (XPBDFEM/Xpbd.h:217-263). Shared by the tet rings (xfem_rings.cu), the
// hex rings (xfem_hexes.cu) and, with up to four nodes per lane
// (q_ring_update), the T10 and H27 rings (xfem_t10.cu, xfem_h27.cu). One
// warp per ring: lane n holds ring node n
// (its gradients g0, g1, inverse mass w, state On, Dn, device id dv); the
// sums over nodes run in a fixed butterfly order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "xfem_device.cuh"

namespace xfem {

namespace {

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
	return x;
}

// One constraint U with gradient g and compliance `comp` (per the ring
// volume). VMODE: RayleighDamp of the velocities (Dn holds V) with ratio rd.
template <bool DAMP, bool VMODE>
__device__ __forceinline__ void ring_update1(const DevCtx& C, const BodyParams& bp, uint32_t lane, uint32_t nn,
                                             uint32_t dv, const float4& On, float4 Dn, float w, Vec3 g, float U,
                                             float comp, float inv_dt, float inv_dt2, float rd) {
	const float damp = DAMP && __ldg(&bp.rayleigh_type) < 2u ? __ldg(&bp.damping) : 0.0f;
	const bool limit = __ldg(&bp.rayleigh_type) == 1u;
	const float alpha = comp * inv_dt2;
	const float wgg = 1.0e-22f + warp_sum(w * dot(g, g));
	if constexpr (VMODE) {
		const float gV = warp_sum(lane < nn ? dot(g, v3(Dn)) : 0.0f);
		const float l = -gV / fmaf(2.0f * U, comp * inv_dt / rd, wgg);
		if (lane < nn) {
			const float sc = w * l;
			Dn.x = fmaf(sc, g.x, Dn.x);
			Dn.y = fmaf(sc, g.y, Dn.y);
			Dn.z = fmaf(sc, g.z, Dn.z);
			st_vertex(C.vert + 2 * (size_t)dv, On, Dn);
		}
		return;
	}
	float l = (-2.0f * U) / fmaf(2.0f * U, alpha, wgg);
	if constexpr (DAMP) {
		const float gV = warp_sum(lane < nn ? dot(g, v3(Dn)) : 0.0f);
		const float gamma = damp * inv_dt;
		if (!(damp > 0.0f)) {
		} else if (!limit) {
			l = (-2.0f * U - gamma * gV) / fmaf(wgg, 1.0f + gamma, 2.0f * U * alpha);
		} else {
			const float A = fmaf(2.0f * U, comp * inv_dt / damp, wgg);
			const float b = (-gV - wgg * l) * (A / fmaxf(A, 4.0f * wgg));
			l += b / A;
		}
	}
	if (lane < nn) {
		const float sc = w * l;
		Dn.x = fmaf(sc, g.x, Dn.x);
		Dn.y = fmaf(sc, g.y, Dn.y);
		Dn.z = fmaf(sc, g.z, Dn.z);
		st_vertex(C.vert + 2 * (size_t)dv, On, Dn);
	}
}

// The deviatoric and hydrostatic pair (U0, g0), (U1, g1) with compliances
// comp0, comp1 (per the ring volume).
template <bool DAMP, bool VMODE>
__device__ __forceinline__ void ring_update2(const DevCtx& C, const BodyParams& bp, uint32_t lane, uint32_t nn,
                                             uint32_t dv, const float4& On, float4 Dn, float w, Vec3 g0, Vec3 g1,
                                             float U0, float U1, float comp0, float comp1, float inv_dt, float inv_dt2,
                                             float rd) {
	const float damp = DAMP && __ldg(&bp.rayleigh_type) < 2u ? __ldg(&bp.damping) : 0.0f;
	const bool limit = __ldg(&bp.rayleigh_type) == 1u;
	const float alpha0 = comp0 * inv_dt2, alpha1 = comp1 * inv_dt2;
	const float wgg0 = 1.0e-22f + warp_sum(w * dot(g0, g0));
	const float wgg1 = 1.0e-22f + warp_sum(w * dot(g1, g0));
	const float wgg2 = 1.0e-22f + warp_sum(w * dot(g1, g1));
	float l0, l1;
	if constexpr (VMODE) {
		const float b0 = -warp_sum(lane < nn ? dot(g0, v3(Dn)) : 0.0f);
		const float b1 = -warp_sum(lane < nn ? dot(g1, v3(Dn)) : 0.0f);
		cramer(fmaf(2.0f * U0, comp0 * inv_dt / rd, wgg0), wgg1, fmaf(2.0f * U1, comp1 * inv_dt / rd, wgg2), b0, b1, l0,
		       l1);
		if (lane < nn) {
			Dn.x = fmaf(w, fmaf(l1, g1.x, l0 * g0.x), Dn.x);
			Dn.y = fmaf(w, fmaf(l1, g1.y, l0 * g0.y), Dn.y);
			Dn.z = fmaf(w, fmaf(l1, g1.z, l0 * g0.z), Dn.z);
			st_vertex(C.vert + 2 * (size_t)dv, On, Dn);
		}
		return;
	}
	cramer(fmaf(2.0f * U0, alpha0, wgg0), wgg1, fmaf(2.0f * U1, alpha1, wgg2), -2.0f * U0, -2.0f * U1, l0, l1);
	if constexpr (DAMP) {
		// warp-uniform: one body per ring
		if (damp > 0.0f) {
			const float gV0 = warp_sum(lane < nn ? dot(g0, v3(Dn)) : 0.0f);
			const float gV1 = warp_sum(lane < nn ? dot(g1, v3(Dn)) : 0.0f);
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
	}
	if (lane < nn) {
		Dn.x = fmaf(w, fmaf(l1, g1.x, l0 * g0.x), Dn.x);
		Dn.y = fmaf(w, fmaf(l1, g1.y, l0 * g0.y), Dn.y);
		Dn.z = fmaf(w, fmaf(l1, g1.z, l0 * g0.z), Dn.z);
		st_vertex(C.vert + 2 * (size_t)dv, On, Dn);
	}
}

constexpr uint32_t kQNodesPerLane = kMaxQRingNodes / 32u;

// The multiplier update of a quadratic-element ring (SolveRing's last step,
// as ring_update1 / ring_update2 with up to kQNodesPerLane nodes per lane:
// lane n holds ring nodes n, n + 32, n + 64 and n + 96, their states in the
// scratch's O and D arrays):
// EnergyXpbdConstrain, EnergyXpbdConstrainSimultaneous<2> with the in-solve
// Rayleigh damping (XPBDFEM/Xpbd.h:87-215), or RayleighDamp on V (VMODE).
template <bool DAMP, bool VMODE, class Scratch>
__device__ __forceinline__ void q_ring_update(const DevCtx& C, Scratch& S, const BodyParams& bp, uint32_t lane,
                                              uint32_t nn, const uint32_t dv[kQNodesPerLane],
                                              const Vec3 g0[kQNodesPerLane], const Vec3 g1[kQNodesPerLane], bool pair,
                                              float U0, float U1, float comp0, float comp1, float inv_dt,
                                              float inv_dt2, float rd) {
	const float damp = DAMP && __ldg(&bp.rayleigh_type) < 2u ? __ldg(&bp.damping) : 0.0f;
	const bool limit = __ldg(&bp.rayleigh_type) == 1u;
	float s00 = 0.0f, s01 = 0.0f, s11 = 0.0f, v0 = 0.0f, v1 = 0.0f;
#pragma unroll
	for (uint32_t k = 0; k < kQNodesPerLane; k++) {
		const uint32_t n = lane + 32u * k;
		if (n >= nn) continue;
		const float w = S.O[n].w;
		const Vec3 d = v3(S.D[n]);
		s00 = fmaf(w, dot(g0[k], g0[k]), s00);
		s01 = fmaf(w, dot(g1[k], g0[k]), s01);
		s11 = fmaf(w, dot(g1[k], g1[k]), s11);
		v0 += dot(g0[k], d);
		v1 += dot(g1[k], d);
	}
	const float wgg0 = 1.0e-22f + warp_sum(s00);
	float l0 = 0.0f, l1 = 0.0f;
	if (!pair) {
		// one constraint (ContinuousPixar): U0 with gradient g0
		const float alpha = comp0 * inv_dt2;
		if (VMODE) {
			l0 = -warp_sum(v0) / fmaf(2.0f * U0, comp0 * inv_dt / rd, wgg0);
		} else {
			l0 = (-2.0f * U0) / fmaf(2.0f * U0, alpha, wgg0);
			if (DAMP && damp > 0.0f) {
				const float gV = warp_sum(v0), gamma = damp * inv_dt;
				if (!limit) {
					l0 = (-2.0f * U0 - gamma * gV) / fmaf(wgg0, 1.0f + gamma, 2.0f * U0 * alpha);
				} else {
					const float A = fmaf(2.0f * U0, comp0 * inv_dt / damp, wgg0);
					const float b = (-gV - wgg0 * l0) * (A / fmaxf(A, 4.0f * wgg0));
					l0 += b / A;
				}
			}
		}
	} else {
		const float wgg1 = 1.0e-22f + warp_sum(s01), wgg2 = 1.0e-22f + warp_sum(s11);
		const float alpha0 = comp0 * inv_dt2, alpha1 = comp1 * inv_dt2;
		if (VMODE) {
			cramer(fmaf(2.0f * U0, comp0 * inv_dt / rd, wgg0), wgg1, fmaf(2.0f * U1, comp1 * inv_dt / rd, wgg2),
			       -warp_sum(v0), -warp_sum(v1), l0, l1);
		} else {
			cramer(fmaf(2.0f * U0, alpha0, wgg0), wgg1, fmaf(2.0f * U1, alpha1, wgg2), -2.0f * U0, -2.0f * U1, l0, l1);
			if (DAMP && damp > 0.0f) {
				const float gV0 = warp_sum(v0), gV1 = warp_sum(v1), gamma = damp * inv_dt;
				float A0, A2, b0 = -2.0f * U0, b1 = -2.0f * U1;
				if (!limit) {
					const float sc = 1.0f / (1.0f + gamma);
					A0 = wgg0 + (2.0f * U0 * alpha0) * sc;
					A2 = wgg2 + (2.0f * U1 * alpha1) * sc;
					b0 = (b0 - gamma * gV0) * sc;
					b1 = (b1 - gamma * gV1) * sc;
				} else {
					A0 = fmaf(2.0f * U0, alpha0, wgg0);
					A2 = fmaf(2.0f * U1, alpha1, wgg2);
				}
				cramer(A0, wgg1, A2, b0, b1, l0, l1);
				if (limit) {
					const float B0 = fmaf(2.0f * U0, comp0 * inv_dt / damp, wgg0);
					const float B2 = fmaf(2.0f * U1, comp1 * inv_dt / damp, wgg2);
					float e0 = fmaf(b0, -1.0f - alpha0 * l0, -gV0), e1 = fmaf(b1, -1.0f - alpha1 * l1, -gV1);
					e0 *= B0 / fmaxf(B0, 8.0f * wgg0);
					e1 *= B2 / fmaxf(B2, 8.0f * wgg2);
					float d0, d1;
					cramer(B0, wgg1, B2, e0, e1, d0, d1);
					l0 += d0;
					l1 += d1;
				}
			}
		}
	}
#pragma unroll
	for (uint32_t k = 0; k < kQNodesPerLane; k++) {
		const uint32_t n = lane + 32u * k;
		if (n >= nn) continue;
		const float w = S.O[n].w;
		float4 Dn = S.D[n];
		if (pair) {
			Dn.x = fmaf(w, fmaf(l1, g1[k].x, l0 * g0[k].x), Dn.x);
			Dn.y = fmaf(w, fmaf(l1, g1[k].y, l0 * g0[k].y), Dn.y);
			Dn.z = fmaf(w, fmaf(l1, g1[k].z, l0 * g0[k].z), Dn.z);
		} else {
			const float sc = w * l0;
			Dn.x = fmaf(sc, g0[k].x, Dn.x);
			Dn.y = fmaf(sc, g0[k].y, Dn.y);
			Dn.z = fmaf(sc, g0[k].z, Dn.z);
		}
		st_vertex(C.vert + 2 * (size_t)dv[k], S.O[n], Dn);
	}
}

}  // namespace

}  // namespace xfem
