// C ABI of libxfem.so (include/xfem.h): handle management, packing of the
// schedule into the device layout, stepping and transfers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/xfem.h"
#include "xfem_internal.h"

using namespace xfem;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
	g_err = msg;
	return code;
}

#define XCUDA(call)                                                                                    \
	do {                                                                                               \
		cudaError_t e_ = (call);                                                                       \
		if (e_ != cudaSuccess)                                                                         \
			return fail(e_ == cudaErrorMemoryAllocation ? XFEM_ENOMEM : XFEM_ECUDA,                    \
			            std::string(#call) + ": " + cudaGetErrorString(e_));                           \
	} while (0)

// Test hook XFEM_HOOK_FAIL_ALLOC: the n-th device allocation from the
// handles' buffers fails as if the device were full (0 = off).
std::atomic<uint32_t> g_fail_alloc_in{0};

cudaError_t injected_alloc_failure() {
	uint32_t n = g_fail_alloc_in.load();
	while (n != 0) {
		if (g_fail_alloc_in.compare_exchange_weak(n, n - 1)) return n == 1 ? cudaErrorMemoryAllocation : cudaSuccess;
	}
	return cudaSuccess;
}

// Element kinds of a body: linear tets (the chunked tet path, the one-ring
// mode), linear hexahedra (H8), quadratic tets (T10) and quadratic hexahedra
// (H27), the last three in the element kernel.
constexpr uint32_t kElTets = 0, kElHexes = 1, kElT10 = 2, kElH27 = 3, kElMixed = 4, kElQMixed = 5;

struct BodyHost {
	uint32_t nv = 0, nt = 0, vbase = 0, tbase = 0;
	std::vector<float> nodes;         // rest positions, caller order
	std::vector<uint32_t> tets;       // caller order
	std::vector<float> ep;            // 17 per tet
	std::vector<float> w0;            // rest inverse masses
	std::vector<uint8_t> vflags;
	std::vector<float> tet_mu;        // empty = uniform material
	xfem_settings settings;
	Schedule sched;
	RingSchedule rings;               // continuous-pressure models only
	std::vector<uint32_t> tet_slot;   // caller tet -> global row * 32 + lane (multiplier output)
	std::vector<uint64_t> tet_rec;    // caller tet -> float4 index of its plane-3 record in the chunk blocks
	// element bodies (linear hexahedra or quadratic tets; no linear tets)
	uint32_t el = 0;                  // kElTets, kElHexes, kElT10, kElH27, kElMixed (tets and hexes),
	                                  // kElQMixed (T10s and H27s: the H27s in elems, the T10s in qt)
	uint32_t nh = 0;                  // elements
	uint32_t ncorner = 0;             // T10, H27: the mesh's own vertices; the added nodes follow
	std::vector<uint32_t> elems;      // 8 per hex, 10 per T10 or 27 per H27, caller order
	std::vector<uint32_t> edges;      // T10, H27: the two corners of each edge node
	std::vector<uint32_t> quads;      // H27: the four corners of each face node
	std::vector<float> eep;           // rest::kHexRec per hex, rest::kT10Rec per T10, rest::kH27Rec per H27
	ElemSchedule esched;
	std::vector<uint32_t> el_dev;     // hexes, T10s, H27s: each element's device index (build_elements)
	ElemSchedule tsched;              // kElMixed: the tets' own colouring (elements of 4 vertices); kElQMixed: the T10s'
	uint32_t nqt = 0;                 // kElQMixed: T10s (nt stays 0, as for T10 bodies)
	std::vector<uint32_t> qt;         // kElQMixed: 10 per T10 (caller tet order)
	std::vector<float> qtep;          // kElQMixed: rest::kT10Rec per T10
	std::vector<uint32_t> qt_dev;     // kElQMixed: each T10's device index
};

template <typename T>
struct DevBuf {
	T* p = nullptr;
	size_t n = 0;
	~DevBuf() {
		if (p) cudaFree(p);
	}
	cudaError_t alloc(size_t count) {
		if (p) {
			cudaFree(p);
			p = nullptr;
		}
		n = count;
		if (injected_alloc_failure() != cudaSuccess) {
			n = 0;
			return cudaErrorMemoryAllocation;
		}
		return cudaMalloc((void**)&p, sizeof(T) * (count ? count : 1));
	}
	// keeps the buffer when it is already large enough
	cudaError_t reserve(size_t count) { return p && n >= count ? cudaSuccess : alloc(count); }
};

// The recorded run of the last xfem_adjoint_forward.
struct AdjointRun {
	bool valid = false;
	uint32_t nsub = 0, seg = 0, nseg = 0, ntips = 0;
	float dt = 0.0f;
	DevBuf<float4> tape_v, tape_t, tape_fin, traj, ckpt, abar, grad;
	DevBuf<int32_t> tip_of;
	DevBuf<float> cbar;
	std::vector<uint32_t> tips;  // the tips tip_of holds
	bool tips_uploaded = false;
};

}  // namespace

struct xfem_body {
	int device = 0;
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	xfem_options opt{};
	std::vector<BodyHost> bodies;
	uint32_t nverts = 0, ntets = 0, nchunks = 0, nrows = 0, nvrows = 0, ncolours = 0;
	// device buffers
	DevBuf<float4> vert, cblk;
	DevBuf<uint32_t> ccb, isolated, dev_of_vert, tets_dev, bar, dep_begin, deps, done;
	DevBuf<ChunkMeta> chunks;
	uint32_t max_colour_chunks = 0;
	AdjointRun adj;
	DevBuf<BodyParams> params;
	DevBuf<float2> tlam;
	DevBuf<int> err;
	int* err_host = nullptr;  // pinned: the error word's read-back at every synchronising call
	DevBuf<float> stage;
	DevBuf<double> vol;
	// per tet, caller order (all bodies): record index of c0, volume, output
	// row (row * 32 + lane), 1/mu; staging for transfers
	DevBuf<uint32_t> tet_rec_dev, tet_slot_dev;
	DevBuf<uint32_t> tflat, tick;   // per tet row: index in the body's order; the tick word
	DevBuf<float> tarea;            // per tet row: surface area
	DevBuf<float4> right_target;    // per device vertex: the Right lock's target (LockRight bodies)
	DevBuf<uint32_t> lastmask;      // per chunk lane: slots whose last solve it makes
	DevBuf<uint8_t> pass_on;        // [damping kind][tick % 8][colour]
	DevBuf<float> tet_vol_dev, tet_inv_mu, io;
	// one-ring mode (continuous-pressure models)
	bool ring_mode = false;
	DevBuf<uint4> ring_hdr;
	DevBuf<uint32_t> ring_node, ring_cb, pbd_cb, ring_clist;
	DevBuf<uint16_t> ring_cwords;
	DevBuf<float4> ring_ent;
	DevBuf<uint2> pbd_cl;
	DevBuf<uint4> pbd_ent;
	// element mode (kElHexes, kElT10 or kElH27; kElTets: the tet path)
	uint32_t el_mode = kElTets;
	DevBuf<uint4> el_vid;
	DevBuf<float4> el_rec;
	DevBuf<uint32_t> el_cb, el_flat;
	DevBuf<float> el_tab;
	// brick launch form (sync_mode 4; built when every chunk is a cube chunk)
	DevBuf<float4> bcblk;
	DevBuf<uint32_t> tet_brec_dev;  // per tet (all bodies): its c0 word in the brick chunks
	DevBuf<uint32_t> bcb, bwait, bcnb_begin, bcnb, bpriv_begin, bpriv_vid, bfin_begin, bfin_vid, bnb_begin, bnb, bflag;
	// meshes mixing tets and hexes (kElMixed): the tets as elements of their own colouring
	DevBuf<uint4> mt_vid;
	DevBuf<float4> mt_rec;
	DevBuf<uint32_t> mt_cb, mt_flat;
	// meshes mixing T10s and H27s (kElQMixed): the T10s' element arrays (the H27s use el_*)
	DevBuf<uint4> q_vid;
	DevBuf<float4> q_rec;
	DevBuf<uint32_t> q_cb, q_flat;
	DevBuf<float> q_tab;
	uint32_t q_colours = 0, q_nel = 0;
	uint32_t nisolated = 0, max_deps = 0;
	LaunchCfg cfg;
	DevCtx ctx{};
	uint32_t hook_wait_miss = 0;  // XFEM_HOOK_MISSING_ARRIVAL for the next stepping call
	bool tuned = false;
	int brick_block = 256;  // the brick form's default block size (192 with two bricks per SM)
	float tune_ms = 0.0f;  // the autotuner's best trial time (3 calls), when it timed any
	// cached CUDA graph (graph mode)
	cudaGraphExec_t graph = nullptr;
	uint32_t graph_nsub = 0;
	float graph_dt = 0.0f;
	uint64_t device_bytes = 0;

	~xfem_body() {
		if (err_host) cudaFreeHost(err_host);
		if (graph) cudaGraphExecDestroy(graph);
		if (own_stream && stream) cudaStreamDestroy(stream);
	}
};

namespace {

// How the solve treats an energy id on linear tets (TSolveElement's
// dispatch, XPBDFEM/Fem.cpp:872-888; the continuous-pressure ids 8-10 run a
// per-vertex ring solve, GeoLinear3d::Constrain, XPBDFEM/Geo.cpp:784-787).
uint32_t model_of(uint32_t energy) {
	switch (energy) {
	case XFEM_ENERGY_PIXAR:
	case XFEM_ENERGY_PIXAR_REDUCED:
	case XFEM_ENERGY_PIXAR_SEL: return kModelPixar;
	case XFEM_ENERGY_MIXED: return kModelNeoClamp;
	case XFEM_ENERGY_YEOH_SKIN:
	case XFEM_ENERGY_YEOH_SKIN_SEL:
	case XFEM_ENERGY_YEOH_SKIN_FAST: return kModelYeoh;
	case XFEM_ENERGY_CUBE_NEO:
	case XFEM_ENERGY_CUBE_SKIN: return kModelNone;
	case 8u:
	case 9u:
	case 10u: return kModelRing;
	default: return kModelNeo;  // MixedSel, and every id above 12
	}
}

int validate_settings(const xfem_settings& s) {
	const uint32_t energy = (s.flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK;
	const uint32_t model = model_of(energy);
	if (energy == 8u && !(s.poissons_ratio < 0.5f))
		return fail(XFEM_EINVAL, "ContinuousPixar needs poissons_ratio < 0.5 (lambda = 2 / (1 - 2 nu))");
	if (s.volume_passes > XFEM_MAX_VOLUME_PASSES)
		return fail(XFEM_EINVAL, "volume_passes must be at most " + std::to_string(XFEM_MAX_VOLUME_PASSES));
	if (model == kModelPixar && !(s.poissons_ratio < 0.5f))
		return fail(XFEM_EINVAL, "the Pixar models need poissons_ratio < 0.5 (lambda = 2 / (1 - 2 nu))");
	if (!(s.damping >= 0.0f) || !(s.pbd_damping >= 0.0f)) return fail(XFEM_EINVAL, "damping and pbd_damping must be >= 0");
	for (int k = 0; k < 9; k++)
		if (!isfinite(s.locked_right_transform[k])) return fail(XFEM_EINVAL, "locked_right_transform must be finite");
	for (int k = 0; k < 3; k++)
		if (!isfinite(s.origin[k])) return fail(XFEM_EINVAL, "origin must be finite");
	if (!(s.compliance > 0.0f)) return fail(XFEM_EINVAL, "compliance must be > 0");
	if (!(s.poissons_ratio > 0.0f && s.poissons_ratio <= 0.5f))
		return fail(XFEM_EINVAL, "poissons_ratio must be in (0, 0.5]");
	if (s.ground && !(s.friction >= 0.0f)) return fail(XFEM_EINVAL, "friction must be >= 0");
	return XFEM_OK;
}

// The reference's material scalars (XPBDFEM/Fem.cpp:445-449) in float.
BodyParams make_params(const xfem_settings& s) {
	BodyParams p{};
	const float mu = 1.0f / s.compliance;
	const float nu = s.poissons_ratio;
	const float lambda = (2.0f * mu * nu) / (1.0f - 2.0f * nu);
	p.mu = mu;
	p.inv_mu = 1.0f / mu;
	p.inv_lambda = 1.0f / lambda;
	p.a = 1.0f + mu / lambda;
	p.ratio = mu * p.inv_lambda;
	for (int k = 0; k < 3; k++) p.yeoh[k] = s.yeoh[k];
	p.energy = (s.flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK;
	p.model = model_of(p.energy);
	p.lambda = lambda;
	if (p.model == kModelPixar || p.energy == 8u) {
		// SolveElementPixar's own material (XPBDFEM/Fem.cpp:367-368): mu = 2
		const float lp = 2.0f / (1.0f - 2.0f * nu);
		p.a = 1.0f + 2.0f / lp;
		p.hw = lp / 2.0f;
		p.ratio = 0.0f;
	}
	p.volume_passes = s.volume_passes;
	p.compliance = s.compliance;
	p.cube_fast = p.energy == XFEM_ENERGY_CUBE_NEO && nu >= 0.5f && !(s.damping > 0.0f) ? 1u : 0u;
	p.simultaneous = (s.flags >> XFEM_XPBD_SOLVE_BIT) & 1u;
	for (int k = 0; k < 3; k++) p.gravity[k] = s.gravity[k];
	p.drag_mul = 1.0f - s.time_corrected_drag;
	p.lock_active = (s.flags & XFEM_LOCK_LEFT) ? 1u : 0u;
	p.lock_right = (s.flags & XFEM_LOCK_RIGHT) ? 1u : 0u;
	p.a_ring = p.energy == 8u ? 1.0f + (1.0f - 2.0f * nu) : 1.0f / (2.0f * nu);
	p.ground = s.ground ? 1u : 0u;
	p.friction = s.friction;
	for (int k = 0; k < 3; k++) p.ground_n[k] = s.ground_normal[k];
	p.ground_d = s.ground_offset;
	p.damping = s.damping;
	p.rayleigh_type = (s.flags >> XFEM_RAYLEIGH_TYPE_BIT) & 3u;
	p.pbd_on = s.pbd_damping > 0.0f ? 1u : 0u;
	p.pbd_coeff = s.volume_and_time_corrected_pbd_damping;
	p.pbd_coeff_amortized = s.amortized_volume_and_time_corrected_pbd_damping;
	return p;
}

// The element counts a body's damping slices divide: its tets (tet bodies),
// its elements (hex, T10 and H27 bodies), or its tets and its hexes (a mesh
// mixing the two, XPBDFEM/Geo.cpp:792-811).
void set_counts(BodyParams& p, const BodyHost& b) {
	p.ntets = b.el == kElQMixed ? b.nqt : b.el == kElTets || b.el == kElMixed ? b.nt : b.nh;
	p.nhexes = b.el == kElMixed || b.el == kElQMixed ? b.nh : 0u;
	// the rings a body damps in amortized slices: one per vertex, or on a T10
	// or H27 mesh one per mesh vertex (the added nodes have none)
	p.nverts = b.el == kElT10 || b.el == kElH27 ? b.ncorner : b.nv;
}

// Whether any body needs the extended kernels: it damps (in the solve or
// after it), runs Mixed (its clamp), a Pixar or a cube model, or runs volume
// passes.
bool ext_any_of(const std::vector<BodyHost>& bodies) {
	for (const BodyHost& b : bodies) {
		const uint32_t model = model_of((b.settings.flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK);
		if (b.settings.damping > 0.0f || b.settings.pbd_damping > 0.0f || model == kModelNeoClamp ||
		    model >= kModelPixar || b.settings.volume_passes)
			return true;
	}
	return false;
}

// Volume sweeps per substep: the most that any body runs.
uint32_t nvol_of(const std::vector<BodyHost>& bodies) {
	uint32_t n = 0;
	for (const BodyHost& b : bodies) n = std::max(n, b.settings.volume_passes);
	return n;
}

// Damping sweeps the handle runs after each solve sweep: bit 0 element
// Rayleigh damping (any body with a Post type and damping > 0), bit 1 PBD
// damping (any body with pbd_damping > 0).
uint32_t damp_kinds_of(const std::vector<BodyHost>& bodies) {
	uint32_t k = 0;
	for (const BodyHost& b : bodies) {
		const uint32_t type = (b.settings.flags >> XFEM_RAYLEIGH_TYPE_BIT) & 3u;
		if (type >= XFEM_RAYLEIGH_POST && b.settings.damping > 0.0f) k |= 1u;
		if (b.settings.pbd_damping > 0.0f) k |= 2u;
	}
	return k;
}

// [damping kind][tick % 8][colour]: whether some body damps a tet of that
// colour at that tick (kind 0 element Rayleigh for the Post types, 1 PBD);
// the amortized type damps the eighth [nt m / 8, nt (m + 1) / 8) of the
// body's flattened order, which is colour-major.
std::vector<uint8_t> pass_table(const std::vector<BodyHost>& bodies, uint32_t ncol) {
	std::vector<uint8_t> on(16 * (size_t)ncol, 0);
	for (const BodyHost& b : bodies) {
		const uint32_t type = (b.settings.flags >> XFEM_RAYLEIGH_TYPE_BIT) & 3u;
		const bool kind_on[2] = {type >= XFEM_RAYLEIGH_POST && b.settings.damping > 0.0f, b.settings.pbd_damping > 0.0f};
		const Schedule& sc = b.sched;
		std::vector<uint32_t> ct(sc.ncolours + 1, 0);
		for (uint32_t c = 0; c < sc.ncolours; c++) {
			uint32_t n = 0;
			for (uint32_t i = sc.colour_cl_begin[c]; i < sc.colour_cl_begin[c + 1]; i++)
				n += sc.cl_begin[sc.colour_cl[i] + 1] - sc.cl_begin[sc.colour_cl[i]];
			ct[c + 1] = ct[c] + n;
		}
		for (int k = 0; k < 2; k++) {
			if (!kind_on[k]) continue;
			for (uint32_t m = 0; m < 8; m++) {
				const uint32_t lo = type == XFEM_RAYLEIGH_POST_AMORTIZED ? b.nt * m / 8u : 0u;
				const uint32_t hi = type == XFEM_RAYLEIGH_POST_AMORTIZED ? b.nt * (m + 1u) / 8u : b.nt;
				for (uint32_t c = 0; c < sc.ncolours; c++)
					if (ct[c] < hi && lo < ct[c + 1]) on[((size_t)k * 8 + m) * ncol + c] = 1;
			}
		}
	}
	return on;
}

// c0 = (1/mu)/volume exactly as the reference forms comp[0] (XPBDFEM/Fem.cpp:449).
float tet_c0(const BodyHost& b, uint32_t t) {
	const float mu = b.tet_mu.empty() ? 1.0f / b.settings.compliance : b.tet_mu[t];
	return 1.0f / mu / b.ep[17 * (size_t)t + 15];
}

// The Right lock's target of every Right vertex of the bodies that lock them,
// origin + lockedRightTransform3d * vec3(X0) in float with the reference's
// mat3 * vec3 (rows dotted with X0, XPBDFEM/vectormath.h:508-513, and dot's
// left-to-right sum) and the vec3 addition (XPBDFEM/Geo.cpp:327), in device
// vertex order; the buffer exists only while some body locks its Right side.
int update_right_targets(xfem_body* h) {
	bool any = false;
	for (const BodyHost& b : h->bodies) any = any || (b.settings.flags & XFEM_LOCK_RIGHT);
	if (!any) {
		h->ctx.right_target = nullptr;
		return XFEM_OK;
	}
	std::vector<float4> t(h->nverts, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
	for (const BodyHost& b : h->bodies) {
		if (!(b.settings.flags & XFEM_LOCK_RIGHT)) continue;
		const float* T = b.settings.locked_right_transform;
		const float* o = b.settings.origin;
		for (uint32_t v = 0; v < b.nv; v++) {
			if (!(b.vflags[v] & 2u)) continue;
			const float x = b.nodes[3 * (size_t)v], y = b.nodes[3 * (size_t)v + 1], z = b.nodes[3 * (size_t)v + 2];
			float r[3];
			for (int k = 0; k < 3; k++) r[k] = T[k] * x + T[3 + k] * y + T[6 + k] * z;
			t[b.vbase + b.sched.vert_rank[v]] = make_float4(o[0] + r[0], o[1] + r[1], o[2] + r[2], 0.0f);
		}
	}
	XCUDA(h->right_target.reserve(t.size()));
	XCUDA(cudaMemcpyAsync(h->right_target.p, t.data(), t.size() * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
	XCUDA(cudaStreamSynchronize(h->stream));
	h->ctx.right_target = h->right_target.p;
	return XFEM_OK;
}

// Status and message of a device error word (kErr*).
int device_error(int e) {
	switch (e) {
	case kErrBarrierTimeout: return fail(XFEM_EDEVICE_TIMEOUT, "device grid barrier timed out");
	case kErrCopyTimeout: return fail(XFEM_EDEVICE_TIMEOUT, "device wait for a chunk copy timed out");
	case kErrDepTimeout: return fail(XFEM_EDEVICE_TIMEOUT, "device wait for a neighbouring chunk timed out");
	case kErrNonFinite: return fail(XFEM_ENONFINITE, "a position or velocity became NaN or infinite");
	default: return fail(XFEM_ECUDA, "device error " + std::to_string(e));
	}
}

int check_device_error(xfem_body* h) {
	int e = 0;
	if (h->err_host) {  // pinned: an asynchronous copy, no staging
		XCUDA(cudaMemcpyAsync(h->err_host, h->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
		XCUDA(cudaStreamSynchronize(h->stream));
		e = *h->err_host;
	} else {
		XCUDA(cudaMemcpyAsync(&e, h->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
		XCUDA(cudaStreamSynchronize(h->stream));
	}
	if (e != 0) {
		XCUDA(cudaMemsetAsync(h->err.p, 0, sizeof(int), h->stream));
		XCUDA(cudaStreamSynchronize(h->stream));
		return device_error(e);
	}
	return XFEM_OK;
}

int prepare_mesh(const xfem_mesh& m, BodyHost& b) {
	if (!m.node_data || !m.idx_data) return fail(XFEM_EINVAL, "null mesh array");
	if (m.node_data_count % 3) return fail(XFEM_EINVAL, "node_data_count must be a multiple of 3");
	uint32_t ntag[2] = {0, 0};
	for (uint32_t i = 0; i < m.idx_data_count;) {
		const uint32_t tag = m.idx_data[i];
		if (tag != 4u && tag != 8u)
			return fail(XFEM_EINVAL, "unknown element tag " + std::to_string(tag) + " at " + std::to_string(i));
		ntag[tag == 8u]++;
		i += tag + 1;
	}
	b.el = ntag[0] && ntag[1] ? kElMixed : ntag[1] > 0 ? kElHexes : kElTets;
	uint32_t nv = 0;
	if (b.el == kElMixed ? parse_mixed(m.idx_data, m.idx_data_count, b.tets, b.elems, nv)
	    : b.el == kElHexes ? parse_hexes(m.idx_data, m.idx_data_count, b.elems, nv)
	                       : parse_tets(m.idx_data, m.idx_data_count, b.tets, nv))
		return fail(XFEM_EINVAL, "truncated index stream");
	// GeoLinear3d::Init asserts vertCount == nodeDataCount / 3 (XPBDFEM/Geo.cpp:700)
	if (nv != m.node_data_count / 3)
		return fail(XFEM_EINVAL, "vertex count " + std::to_string(nv) + " implied by the index stream != node_data_count/3 = " +
		                             std::to_string(m.node_data_count / 3));
	if (!(m.density > 0.0f)) return fail(XFEM_EINVAL, "density must be > 0");
	b.nv = nv;
	b.nt = (uint32_t)(b.tets.size() / 4);
	b.nh = (uint32_t)(b.elems.size() / 8);
	b.nodes.assign(m.node_data, m.node_data + m.node_data_count);
	return XFEM_OK;
}

// Whether the settings ask for quadratic elements (GeoQuadratic3d: element
// type T10 or H27 in flags bits 0-3, XPBDFEM/Demo.cpp:145-150).
bool quadratic_type(uint32_t flags) {
	const uint32_t t = flags & XFEM_ELEMENT_TYPE_MASK;
	return t == XFEM_ELEMENT_T10 || t == XFEM_ELEMENT_H27;
}

// The argument checks of prepare_mesh and validate_settings for every body,
// made before any device is touched: a bad tag, a truncated stream, a vertex
// count that does not match the node array or invalid settings fail the same
// way with or without a GPU.
int precheck_inputs(uint32_t nb, const xfem_mesh* meshes, const xfem_settings* settings) {
	for (uint32_t k = 0; k < nb; k++) {
		const xfem_mesh& m = meshes[k];
		const std::string who = nb > 1 ? "body " + std::to_string(k) + ": " : std::string();
		if (!m.node_data || !m.idx_data) return fail(XFEM_EINVAL, who + "null mesh array");
		if (m.node_data_count % 3) return fail(XFEM_EINVAL, who + "node_data_count must be a multiple of 3");
		// the reference's empty Geo steps nothing; a handle with nothing to
		// step is refused instead of launching empty grids
		if (m.idx_data_count == 0) return fail(XFEM_EINVAL, who + "the mesh has no elements");
		uint64_t nv = 0;
		uint32_t ntag[2] = {0, 0};
		for (uint32_t i = 0; i < m.idx_data_count;) {
			const uint32_t tag = m.idx_data[i];
			if (tag != 4u && tag != 8u)
				return fail(XFEM_EINVAL, who + "unknown element tag " + std::to_string(tag) + " at " + std::to_string(i));
			if ((uint64_t)i + tag >= m.idx_data_count) return fail(XFEM_EINVAL, who + "truncated index stream");
			for (uint32_t j = 1; j <= tag; j++) nv = std::max<uint64_t>(nv, (uint64_t)m.idx_data[i + j] + 1u);
			ntag[tag == 8u]++;
			i += tag + 1;
		}
		if (ntag[0] && ntag[1] && settings) {
			const uint32_t energy = (settings[k].flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK;
			if (model_of(energy) == kModelRing)
				return fail(XFEM_EUNSUPPORTED, who + "the continuous-pressure models (energy 8-10) run on meshes of one "
				                                     "element kind");
		}
		if (nv != m.node_data_count / 3)
			return fail(XFEM_EINVAL, who + "vertex count " + std::to_string(nv) +
			                             " implied by the index stream != node_data_count/3 = " +
			                             std::to_string(m.node_data_count / 3));
		if (!(m.density > 0.0f)) return fail(XFEM_EINVAL, who + "density must be > 0");
		if (settings) {
			const int rc = validate_settings(settings[k]);
			if (rc) return fail(rc, who + g_err);
		}
	}
	return XFEM_OK;
}

// The rest state on the host (GeoLinear3d::Init's precompute).
void host_rest(const xfem_mesh& m, BodyHost& b) {
	b.ep.resize(17 * (size_t)b.nt);
	b.w0.resize(b.nv);
	b.vflags.resize(b.nv);
	if (b.el == kElHexes) {
		b.eep.resize((size_t)rest::kHexRec * b.nh);
		hex_init_rest(b.nodes.data(), b.nv, b.elems.data(), b.nh, m.density, b.eep.data(), b.w0.data(), b.vflags.data());
		return;
	}
	if (b.el == kElMixed) {
		b.eep.resize((size_t)rest::kHexRec * b.nh);
		mixed_init_rest(b.nodes.data(), b.nv, b.tets.data(), b.nt, b.elems.data(), b.nh, m.density, b.ep.data(),
		                b.eep.data(), b.w0.data(), b.vflags.data());
		return;
	}
	init_rest(b.nodes.data(), b.nv, b.tets.data(), b.nt, m.density, b.ep.data(), b.w0.data(), b.vflags.data());
}

// GeoQuadratic3d::Init on a tet mesh (XPBDFEM/Geo.cpp:836-941): the edge
// nodes at the edges' midpoints and the T10 rest state. The body's vertices
// become the corners followed by the edge nodes (their rest positions
// rounded to float; the rest state is built from the double positions, as
// the reference does). X: the double positions out (3 per vertex), or null.
void prepare_t10(const xfem_mesh& m, BodyHost& b, std::vector<double>* X = nullptr) {
	std::vector<uint32_t> t10;
	tet_edges(b.tets.data(), b.nt, b.nv, b.edges, t10);
	const uint32_t ne = (uint32_t)(b.edges.size() / 2), n = b.nv + ne;
	std::vector<double> x(3 * (size_t)n);
	b.eep.resize((size_t)rest::kT10Rec * b.nt);
	b.w0.resize(n);
	b.vflags.resize(n);
	t10_init_rest(b.nodes.data(), b.nv, b.nt, b.edges.data(), ne, t10.data(), m.density, x.data(), b.eep.data(),
	              b.w0.data(), b.vflags.data());
	b.nodes.resize(3 * (size_t)n);
	for (size_t i = 0; i < 3 * (size_t)n; i++) b.nodes[i] = (float)x[i];
	b.el = kElT10;
	b.ncorner = b.nv;
	b.nv = n;
	b.nh = b.nt;
	b.elems = std::move(t10);
	b.tets.clear();
	b.nt = 0;
	if (X) *X = std::move(x);
}

// GeoQuadratic3d::Init on a hex mesh (XPBDFEM/Geo.cpp:836-933): nodes on the
// edges, the faces and the hex centres, and the H27 rest state; the body's
// vertices become the corners followed by those nodes. X as for prepare_t10.
void prepare_h27(const xfem_mesh& m, BodyHost& b, std::vector<double>* X = nullptr) {
	std::vector<uint32_t> h27;
	hex_edges_quads(b.elems.data(), b.nh, b.nv, b.edges, b.quads, h27);
	const uint32_t ne = (uint32_t)(b.edges.size() / 2), nq = (uint32_t)(b.quads.size() / 4);
	const uint32_t n = b.nv + ne + nq + b.nh;
	std::vector<double> x(3 * (size_t)n);
	std::vector<float> eep((size_t)rest::kH27Rec * b.nh);
	b.w0.resize(n);
	b.vflags.resize(n);
	h27_init_rest(b.nodes.data(), b.nv, b.elems.data(), b.nh, b.edges.data(), ne, b.quads.data(), nq, h27.data(),
	              m.density, x.data(), eep.data(), b.w0.data(), b.vflags.data());
	b.eep = std::move(eep);
	b.nodes.resize(3 * (size_t)n);
	for (size_t i = 0; i < 3 * (size_t)n; i++) b.nodes[i] = (float)x[i];
	b.el = kElH27;
	b.ncorner = b.nv;
	b.nv = n;
	b.elems = std::move(h27);
	if (X) *X = std::move(x);
}

// GeoQuadratic3d::Init on a mesh mixing tets and hexes (XPBDFEM/Geo.cpp:
// 836-953): Connectivity3d's edges and quads over the interleaved stream,
// nodes on the edges, the faces and the hex centres, the T10 and H27 rest
// state and one mass sum. The body's vertices become the corners followed by
// those nodes; its H27s take the element arrays (elems, eep), its T10s qt
// and qtep, and b.nqt / b.nh count them (b.nt becomes 0: no linear tets).
void prepare_qmixed(const xfem_mesh& m, BodyHost& b) {
	std::vector<uint32_t> t10, h27;
	quad_mesh(m.idx_data, m.idx_data_count, b.nv, b.edges, b.quads, t10, h27);
	const uint32_t ne = (uint32_t)(b.edges.size() / 2), nq = (uint32_t)(b.quads.size() / 4), n = b.nv + ne + nq + b.nh;
	std::vector<double> x(3 * (size_t)n);
	b.qtep.resize((size_t)rest::kT10Rec * b.nt);
	b.eep.resize((size_t)rest::kH27Rec * b.nh);
	b.w0.resize(n);
	b.vflags.resize(n);
	qmixed_init_rest(b.nodes.data(), b.nv, b.nt, b.elems.data(), b.nh, b.edges.data(), ne, b.quads.data(), nq,
	                 t10.data(), h27.data(), m.density, x.data(), b.qtep.data(), b.eep.data(), b.w0.data(),
	                 b.vflags.data());
	b.nodes.resize(3 * (size_t)n);
	for (size_t i = 0; i < 3 * (size_t)n; i++) b.nodes[i] = (float)x[i];
	b.el = kElQMixed;
	b.ncorner = b.nv;
	b.nv = n;
	b.elems = std::move(h27);
	b.qt = std::move(t10);
	b.nqt = b.nt;
	b.tets.clear();
	b.nt = 0;
}

// Elements of an element body, and vertices per element.
uint32_t nodes_per_element(uint32_t el) {  // kElMixed: its hexes; kElQMixed: its H27s
	return el == kElH27 || el == kElQMixed ? 27u : el == kElT10 ? 10u : 8u;
}

// Rest state and schedule of one body: on the host (gpu false), or with the
// parallel phases on the GPU (rest state, incidence, vertex ranks, cluster
// order) around the host's greedy clustering and colouring. Both give the
// same result bit for bit.
int prepare_body(const xfem_mesh& m, const xfem_settings* s, uint32_t mode, uint32_t morton, bool gpu, void* stream,
                 BodyHost& b) {
	int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (s) {
		b.settings = *s;
	} else {
		xfem_settings_default(&b.settings);
	}
	rc = validate_settings(b.settings);
	if (rc) return rc;
	const uint32_t energy = (b.settings.flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK;
	const bool ring = model_of(energy) == kModelRing;
	const bool quad = quadratic_type(b.settings.flags);
	if (b.el == kElMixed) {
		// tets and hexes in one mesh: set-up on the host, each kind with a
		// colouring of its own
		if (ring)
			return fail(XFEM_EUNSUPPORTED, "the continuous-pressure models (energy 8-10) run on meshes of one element kind: "
			                               "on a mixed mesh the reference indexes a ring's hexes two different ways");
		if (quad) {
			// T10s and H27s in one body, each kind with a colouring of its own
			prepare_qmixed(m, b);
			vertex_ranks(b.nodes.data(), b.nv, morton, b.sched);
			if (elem_schedule(b.nodes.data(), b.nv, b.elems.data(), b.nh, 27, morton, b.esched) ||
			    elem_schedule(b.nodes.data(), b.nv, b.qt.data(), b.nqt, 10, morton, b.tsched))
				return fail(XFEM_ELIMIT,
				            "the element colouring needs more than " + std::to_string(kMaxElemColours) + " colours");
			return XFEM_OK;
		}
		host_rest(m, b);
		vertex_ranks(b.nodes.data(), b.nv, morton, b.sched);
		if (elem_schedule(b.nodes.data(), b.nv, b.elems.data(), b.nh, 8, morton, b.esched) ||
		    elem_schedule(b.nodes.data(), b.nv, b.tets.data(), b.nt, 4, morton, b.tsched))
			return fail(XFEM_ELIMIT, "the element colouring needs more than " + std::to_string(kMaxElemColours) + " colours");
		return XFEM_OK;
	}
	if (b.el == kElHexes || quad) {
		// hexes, T10s and H27s: set-up on the host (rest state, Morton vertex
		// ranks, the element colouring)
		if (quad && b.el == kElHexes)
			prepare_h27(m, b);
		else if (quad)
			prepare_t10(m, b);
		else
			host_rest(m, b);
		vertex_ranks(b.nodes.data(), b.nv, morton, b.sched);
		if (elem_schedule(b.nodes.data(), b.nv, b.elems.data(), b.nh, nodes_per_element(b.el), morton, b.esched))
			return fail(XFEM_ELIMIT, "the element colouring needs more than " + std::to_string(kMaxElemColours) + " colours");
		if (ring && (b.el == kElT10 || b.el == kElH27)) {
			// the continuous-pressure models on T10s or H27s: one-rings over the
			// elements around the mesh's own vertices (GeoQuadratic3d::Init
			// builds no rings for the added nodes, XPBDFEM/Geo.cpp:944-953)
			const uint32_t per = nodes_per_element(b.el);
			std::vector<uint32_t> off, lst;
			incidence(b.elems.data(), b.nv, b.nh, off, lst, per);
			const int rc2 = build_ring_schedule(b.elems.data(), b.nv, off.data(), lst.data(), b.sched.vert_rank.data(),
			                                    b.rings, per, b.ncorner);
			if (rc2 == -2)
				return fail(XFEM_ELIMIT, "a vertex one-ring has more than " +
				                             std::to_string(b.el == kElH27 ? kMaxH27RingElems : kMaxQRingElems) +
				                             (b.el == kElH27 ? " H27s or " : " T10s or ") +
				                             std::to_string(kMaxQRingNodes) + " nodes");
			if (rc2) return fail(XFEM_ELIMIT, "ring colour limit exceeded");
		} else if (ring) {
			// the continuous-pressure models on hexes: one-rings over the hexes
			std::vector<uint32_t> off, lst;
			incidence(b.elems.data(), b.nv, b.nh, off, lst, 8);
			const int rc2 =
			    build_ring_schedule(b.elems.data(), b.nv, off.data(), lst.data(), b.sched.vert_rank.data(), b.rings, 8);
			if (rc2 == -2) return fail(XFEM_ELIMIT, "a vertex one-ring has more than 16 hexes or 32 vertices");
			if (rc2) return fail(XFEM_ELIMIT, "ring colour limit exceeded");
		}
		return XFEM_OK;
	}
	std::vector<uint32_t> off, lst;
	if (!gpu) {
		host_rest(m, b);
		incidence(b.tets.data(), b.nv, b.nt, off, lst);
		if (cluster_and_colour(b.tets.data(), b.nt, off.data(), lst.data(), mode, b.sched))
			return fail(XFEM_ELIMIT, "colour schedule limit exceeded");
		vertex_ranks(b.nodes.data(), b.nv, morton, b.sched);
		cluster_order(b.nodes.data(), b.nv, b.tets.data(), morton, b.sched);
	} else {
		GpuSetupMesh g;
		int e = gpu_setup_mesh(b.nodes.data(), b.nv, b.tets.data(), b.nt, m.density, morton, g, stream);
		if (e) return fail(XFEM_ECUDA, std::string("GPU set-up: ") + cudaGetErrorString((cudaError_t)e));
		b.ep = std::move(g.ep);
		b.w0 = std::move(g.w0);
		b.vflags = std::move(g.vflags);
		if (cluster_and_colour(b.tets.data(), b.nt, g.off.data(), g.lst.data(), mode, b.sched))
			return fail(XFEM_ELIMIT, "colour schedule limit exceeded");
		b.sched.vert_rank = std::move(g.vert_rank);
		e = gpu_cluster_order(b.nodes.data(), b.nv, b.tets.data(), b.nt, morton, g.frame, b.sched, stream);
		if (e) return fail(XFEM_ECUDA, std::string("GPU set-up: ") + cudaGetErrorString((cudaError_t)e));
		off = std::move(g.off);
		lst = std::move(g.lst);
	}
	if (ring) {
		const int rc2 = build_ring_schedule(b.tets.data(), b.nv, off.data(), lst.data(), b.sched.vert_rank.data(), b.rings);
		if (rc2 == -2) return fail(XFEM_ELIMIT, "a vertex one-ring has more than 64 tets or 32 vertices");
		if (rc2) return fail(XFEM_ELIMIT, "ring colour limit exceeded");
	}
	return XFEM_OK;
}

// fn(i) for i in [0, n) on the host's threads (static split; fn must only
// write what index i owns).
template <typename F>
void parallel_for(uint32_t n, const F& fn) {
	const uint32_t nt = std::min<uint32_t>(std::max(1u, std::thread::hardware_concurrency()), 64u);
	if (n < 64 || nt == 1) {
		for (uint32_t i = 0; i < n; i++) fn(i);
		return;
	}
	std::vector<std::thread> pool;
	for (uint32_t t = 0; t < nt; t++)
		pool.emplace_back([&, t] {
			const uint32_t b = (uint32_t)((uint64_t)n * t / nt), e = (uint32_t)((uint64_t)n * (t + 1) / nt);
			for (uint32_t i = b; i < e; i++) fn(i);
		});
	for (std::thread& th : pool) th.join();
}

// Set-up phase timings, printed to stderr when the environment variable
// XFEM_SETUP_TIMING is set (diagnostics for the handle set-up).
struct SetupClock {
	const bool on = getenv("XFEM_SETUP_TIMING") != nullptr;
	std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
	void lap(const char* what) {
		if (!on) return;
		const auto n = std::chrono::steady_clock::now();
		fprintf(stderr, "xfem set-up: %-22s %8.1f ms\n", what, std::chrono::duration<double, std::milli>(n - t).count());
		t = n;
	}
};

// Bodies of at least this many tets take the GPU set-up path; below it a GPU
// round trip costs more than it saves.
constexpr uint32_t kGpuSetupMinTets = 1u << 16;

// Rest state and schedule of every body of a handle. Bodies are independent
// and each one's result does not depend on where it is computed, so the large
// ones run one after another with their parallel phases on the GPU (the
// handle's stream, this thread) while host threads take the others.
int prepare_bodies(xfem_body* h, uint32_t nb, const xfem_mesh* meshes, const xfem_settings* settings, uint32_t mode,
                   uint32_t morton) {
	std::vector<int> rcs(nb, XFEM_OK);
	std::vector<std::string> errs(nb);
	std::vector<uint32_t> on_host, on_gpu;
	for (uint32_t i = 0; i < nb; i++)
		(h->opt.host_setup == 0 && meshes[i].idx_data_count / 5u >= kGpuSetupMinTets ? on_gpu : on_host).push_back(i);
	auto one = [&](uint32_t i, bool gpu) {
		rcs[i] = prepare_body(meshes[i], settings ? &settings[i] : nullptr, mode, morton, gpu, h->stream, h->bodies[i]);
		if (rcs[i]) errs[i] = g_err;
	};
	std::atomic<uint32_t> next{0};
	const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
	const uint32_t nthreads = (uint32_t)std::min<size_t>(on_host.size() > 1 ? on_host.size() : 0, std::min(hw, 64u));
	std::vector<std::thread> pool;
	for (uint32_t t = 0; t < nthreads; t++)
		pool.emplace_back([&] {
			for (uint32_t k; (k = next.fetch_add(1)) < on_host.size();) one(on_host[k], false);
		});
	if (nthreads == 0)
		for (uint32_t i : on_host) one(i, false);
	for (uint32_t i : on_gpu) one(i, true);
	for (std::thread& t : pool) t.join();
	for (uint32_t i = 0; i < nb; i++)
		if (rcs[i]) return fail(rcs[i], nb > 1 ? "body " + std::to_string(i) + ": " + errs[i] : errs[i]);
	return XFEM_OK;
}

struct Lane {
	uint32_t body, cluster;
};

// Whether a body of a one-ring handle damps (in the solve or after it): the
// ring kernel with damping compiled in is launched.
bool ring_damp_of(const std::vector<BodyHost>& bodies) {
	for (const BodyHost& b : bodies)
		if (b.settings.damping > 0.0f || b.settings.pbd_damping > 0.0f) return true;
	return false;
}

// The rings of every body in device order (colour-major, bodies in order):
// per ring a header, its nodes (device vertex ids) and per ring tet its
// prefactored I1 coefficients, volume and corner node indices.
int build_rings(xfem_body* h) {
	uint32_t ncol = 0;
	for (const BodyHost& b : h->bodies) ncol = std::max(ncol, b.rings.ncolours);
	std::vector<uint4> hdr;
	std::vector<uint32_t> node, cb(ncol + 1, 0), clist;
	std::vector<uint16_t> cwords;
	std::vector<float4> ent;
	for (uint32_t c = 0; c < ncol; c++) {
		cb[c] = (uint32_t)hdr.size();
		for (uint32_t bi = 0; bi < (uint32_t)h->bodies.size(); bi++) {
			const BodyHost& b = h->bodies[bi];
			const RingSchedule& rs = b.rings;
			if (c >= rs.ncolours) continue;
			for (uint32_t i = rs.colour_begin[c]; i < rs.colour_begin[c + 1]; i++) {
				const uint32_t v = rs.order[i];
				const uint32_t nn = rs.node_off[v + 1] - rs.node_off[v], nt = rs.tet_off[v + 1] - rs.tet_off[v];
				const uint32_t npe = rs.npe, sh = npe == 27 ? 5u : npe == 10 ? 4u : npe == 8 ? 3u : 2u;
				hdr.push_back(make_uint4((uint32_t)node.size(), (uint32_t)(ent.size() / 2), nn | (nt << 8) | (bi << 16), i));
				for (uint32_t n = rs.node_off[v]; n < rs.node_off[v + 1]; n++)
					node.push_back(b.vbase + b.sched.vert_rank[rs.nodes[n]]);
				for (uint32_t j = rs.tet_off[v]; j < rs.tet_off[v + 1]; j++) {
					if (npe == 27) {
						// an H27: its device element index and its 27 nodes' ring node indices
						uint32_t wd[7] = {0, 0, 0, 0, 0, 0, 0};
						for (int k = 0; k < 27; k++) wd[k >> 2] |= (uint32_t)rs.corner[27 * (size_t)j + k] << (8 * (k & 3));
						ent.push_back(make_float4(__builtin_bit_cast(float, b.el_dev[rs.tets[j]]),
						                          __builtin_bit_cast(float, wd[0]), __builtin_bit_cast(float, wd[1]),
						                          __builtin_bit_cast(float, wd[2])));
						ent.push_back(make_float4(__builtin_bit_cast(float, wd[3]), __builtin_bit_cast(float, wd[4]),
						                          __builtin_bit_cast(float, wd[5]), __builtin_bit_cast(float, wd[6])));
						continue;
					}
					if (npe == 10) {
						// a T10: its device element index and its 10 nodes' ring node indices
						uint32_t wd[3] = {0, 0, 0};
						for (int k = 0; k < 10; k++) wd[k >> 2] |= (uint32_t)rs.corner[10 * (size_t)j + k] << (8 * (k & 3));
						const float4 f = make_float4(__builtin_bit_cast(float, b.el_dev[rs.tets[j]]),
						                             __builtin_bit_cast(float, wd[0]), __builtin_bit_cast(float, wd[1]),
						                             __builtin_bit_cast(float, wd[2]));
						ent.push_back(f);
						ent.push_back(f);
						continue;
					}
					if (npe == 8) {
						// a hex: its device element index and its 8 corners' node indices
						uint32_t lo = 0, hi = 0;
						for (int k = 0; k < 4; k++) lo |= (uint32_t)rs.corner[8 * (size_t)j + k] << (8 * k);
						for (int k = 0; k < 4; k++) hi |= (uint32_t)rs.corner[8 * (size_t)j + 4 + k] << (8 * k);
						const float4 f = make_float4(__builtin_bit_cast(float, b.el_dev[rs.tets[j]]),
						                             __builtin_bit_cast(float, lo), __builtin_bit_cast(float, hi), 0.0f);
						ent.push_back(f);
						ent.push_back(f);
						continue;
					}
					const float* e = &b.ep[17 * (size_t)rs.tets[j]];
					uint32_t cn = 0;
					for (int k = 0; k < 4; k++) cn |= (uint32_t)rs.corner[4 * (size_t)j + k] << (8 * k);
					ent.push_back(make_float4(e[9], e[10], e[11], e[12]));
					ent.push_back(make_float4(e[13], e[14], e[15], __builtin_bit_cast(float, cn)));
				}
				// each node's corners (local element << 2 (tets), << 3 (hexes), << 4 (T10s) or << 5 (H27s) | corner), in
				// element order
				clist.push_back((uint32_t)cwords.size());
				const size_t ob = cwords.size();
				cwords.resize(ob + nn + 1);
				for (uint32_t n = 0; n < nn; n++) {
					cwords[ob + n] = (uint16_t)(cwords.size() - ob - (nn + 1));
					for (uint32_t j = rs.tet_off[v]; j < rs.tet_off[v + 1]; j++)
						for (uint32_t k = 0; k < npe; k++)
							if (rs.corner[npe * (size_t)j + k] == n)
								cwords.push_back((uint16_t)(((j - rs.tet_off[v]) << sh) | k));
				}
				cwords[ob + nn] = (uint16_t)(cwords.size() - ob - (nn + 1));
			}
		}
	}
	cb[ncol] = (uint32_t)hdr.size();
	// PBD damping: per tet colour the clusters of every body, their tets in
	// sequence, each with its index in its body's flattened (colour-major)
	// tet order
	uint32_t pcol = 0;
	for (const BodyHost& b : h->bodies) pcol = std::max(pcol, b.sched.ncolours);
	std::vector<uint32_t> pcb(pcol + 1, 0);
	std::vector<uint2> pcl;
	std::vector<uint4> pent;
	std::vector<uint32_t> flat_pos(h->bodies.size(), 0);
	for (uint32_t c = 0; c < pcol; c++) {
		pcb[c] = (uint32_t)pcl.size();
		for (uint32_t bi = 0; bi < (uint32_t)h->bodies.size(); bi++) {
			const BodyHost& b = h->bodies[bi];
			const Schedule& sc = b.sched;
			if (c >= sc.ncolours) continue;
			for (uint32_t i = sc.colour_cl_begin[c]; i < sc.colour_cl_begin[c + 1]; i++) {
				const uint32_t k = sc.colour_cl[i];
				pcl.push_back(make_uint2((uint32_t)pent.size(), sc.cl_begin[k + 1] - sc.cl_begin[k]));
				for (uint32_t q = sc.cl_begin[k]; q < sc.cl_begin[k + 1]; q++) {
					const uint32_t t = sc.cl_tets[q];
					pent.push_back(make_uint4(b.tbase + t, flat_pos[bi]++, __builtin_bit_cast(uint32_t, b.ep[17 * (size_t)t + 16]), bi));
				}
			}
		}
	}
	pcb[pcol] = (uint32_t)pcl.size();
	XCUDA(h->pbd_cb.alloc(pcb.size()));
	XCUDA(h->pbd_cl.alloc(pcl.size()));
	XCUDA(h->pbd_ent.alloc(pent.size()));
	XCUDA(h->ring_clist.alloc(clist.size()));
	XCUDA(h->ring_cwords.alloc(cwords.size()));
	XCUDA(h->ring_hdr.alloc(hdr.size()));
	XCUDA(h->ring_node.alloc(node.size()));
	XCUDA(h->ring_ent.alloc(ent.size()));
	XCUDA(h->ring_cb.alloc(cb.size()));
	auto up = [&](void* dst, const void* src, size_t bytes) {
		return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
	};
	XCUDA(up(h->ring_hdr.p, hdr.data(), hdr.size() * sizeof(uint4)));
	XCUDA(up(h->ring_node.p, node.data(), node.size() * 4));
	XCUDA(up(h->ring_ent.p, ent.data(), ent.size() * sizeof(float4)));
	XCUDA(up(h->ring_cb.p, cb.data(), cb.size() * 4));
	XCUDA(up(h->ring_clist.p, clist.data(), clist.size() * 4));
	XCUDA(up(h->ring_cwords.p, cwords.data(), cwords.size() * 2));
	XCUDA(up(h->pbd_cb.p, pcb.data(), pcb.size() * 4));
	XCUDA(up(h->pbd_cl.p, pcl.data(), pcl.size() * sizeof(uint2)));
	XCUDA(up(h->pbd_ent.p, pent.data(), pent.size() * sizeof(uint4)));
	XCUDA(cudaStreamSynchronize(h->stream));
	h->ctx.ring_colours = ncol;
	h->ctx.rings = (uint32_t)hdr.size();
	h->ctx.pbd_colours = pcol;
	h->device_bytes += pcb.size() * 4 + pcl.size() * 8 + pent.size() * 16;
	h->device_bytes += hdr.size() * 16 + node.size() * 4 + ent.size() * 16 + cb.size() * 4;
	return XFEM_OK;
}

// The elements of every body in device order (colour-major, bodies in
// order inside a colour): vertex ids (hex: two uint4; T10: three, the last
// two words zero), records as a structure of arrays (hex 30 float4: the
// centre's inverse jacobian and weight, volume, surface area, QQ, QR, then
// the 2x2x2 points' inverse jacobians and weights; T10 14 float4: Qi,
// volume, surface area, QQ, QR), each element's index in its body's order,
// and for T10s the shape-function gradients at the 4-point rule.
// kind: the element type of the set (kElHexes or kElMixed: hexes; kElT10;
// kElH27); qt: the T10s of meshes mixing T10s and H27s (their qt, tsched and
// qtep, into the q_* arrays) instead of the bodies' element arrays.
static int build_element_set(xfem_body* h, uint32_t kind, bool qt) {
	const bool t10 = kind == kElT10, h27 = kind == kElH27;
	const uint32_t per = nodes_per_element(kind), nvid4 = (per + 3) / 4, nrec4 = h27 ? 176u : t10 ? 14u : 30u;
	const size_t rsz = h27 ? rest::kH27Rec : t10 ? rest::kT10Rec : rest::kHexRec;
	uint32_t ncol = 0, nel = 0;
	for (const BodyHost& b : h->bodies) {
		ncol = std::max(ncol, (qt ? b.tsched : b.esched).ncolours);
		nel += qt ? b.nqt : b.nh;
	}
	std::vector<uint4> vid(nvid4 * (size_t)nel);
	std::vector<uint32_t> cb(ncol + 1, 0), flat(nel);
	std::vector<float4> rec(nrec4 * (size_t)nel);
	uint32_t o = 0;
	for (BodyHost& b : h->bodies) (qt ? b.qt_dev : b.el_dev).assign(qt ? b.nqt : b.nh, 0);
	for (uint32_t c = 0; c < ncol; c++) {
		cb[c] = o;
		for (BodyHost& b : h->bodies) {
			const ElemSchedule& es = qt ? b.tsched : b.esched;
			const std::vector<uint32_t>& els = qt ? b.qt : b.elems;
			std::vector<uint32_t>& dev = qt ? b.qt_dev : b.el_dev;
			if (c >= es.ncolours) continue;
			for (uint32_t k = es.colour_begin[c]; k < es.colour_begin[c + 1]; k++, o++) {
				const uint32_t el = es.order[k];
				dev[el] = o;
				uint32_t d[28] = {0};
				for (uint32_t n = 0; n < per; n++) d[n] = b.vbase + b.sched.vert_rank[els[per * (size_t)el + n]];
				for (uint32_t j = 0; j < nvid4; j++)
					vid[nvid4 * (size_t)o + j] = make_uint4(d[4 * j], d[4 * j + 1], d[4 * j + 2], d[4 * j + 3]);
				flat[o] = k;
				const float* e = &(qt ? b.qtep : b.eep)[rsz * el];
				if (h27) {  // element-major, the 703 values and a pad
					float* dst = reinterpret_cast<float*>(&rec[(size_t)o * nrec4]);
					for (size_t j = 0; j < rsz; j++) dst[j] = e[j];
					dst[rsz] = 0.0f;
					continue;
				}
				float r[120];
				if (t10) {
					for (int j = 0; j < 9; j++) r[j] = e[rest::kT10Qi + j];
					r[9] = e[rest::kT10Vol];
					r[10] = e[rest::kT10Area];
					for (int j = 0; j < 9; j++) r[11 + j] = e[rest::kT10QQ + j];
					for (int j = 0; j < 36; j++) r[20 + j] = e[rest::kT10QR + j];
				} else {
					for (int j = 0; j < 9; j++) r[j] = e[rest::kHexJL + j];
					r[9] = e[rest::kHexWL];
					r[10] = e[rest::kHexVol];
					r[11] = e[rest::kHexArea];
					for (int j = 0; j < 7; j++) r[12 + j] = e[rest::kHexQQ + j];
					for (int j = 0; j < 21; j++) r[19 + j] = e[rest::kHexQR + j];
					for (int j = 0; j < 72; j++) r[40 + j] = e[rest::kHexJH + j];
					for (int j = 0; j < 8; j++) r[112 + j] = e[rest::kHexWH + j];
				}
				for (uint32_t k4 = 0; k4 < nrec4; k4++)
					rec[(size_t)k4 * nel + o] = make_float4(r[4 * k4], r[4 * k4 + 1], r[4 * k4 + 2], r[4 * k4 + 3]);
			}
		}
	}
	cb[ncol] = o;
	std::vector<float> g4(t10 ? 120 : h27 ? 8 * 81 + 27 * 81 : 1, 0.0f);
	if (t10)
		for (int p = 0; p < 4; p++)
			for (int n = 0; n < 10; n++)
				for (int k = 0; k < 3; k++) g4[(p * 10 + n) * 3 + k] = rest::t10_tables().g4[p][n][k];
	if (h27) {
		const rest::H27Tables& tb = rest::h27_tables();
		for (int p = 0; p < 8; p++)
			for (int n = 0; n < 27; n++)
				for (int k = 0; k < 3; k++) g4[(p * 27 + n) * 3 + k] = tb.g8[p][n][k];
		for (int p = 0; p < 27; p++)
			for (int n = 0; n < 27; n++)
				for (int k = 0; k < 3; k++) g4[8 * 81 + (p * 27 + n) * 3 + k] = tb.g27[p][n][k];
	}
	DevBuf<uint4>& vidb = qt ? h->q_vid : h->el_vid;
	DevBuf<float4>& recb = qt ? h->q_rec : h->el_rec;
	DevBuf<uint32_t>& cbb = qt ? h->q_cb : h->el_cb;
	DevBuf<uint32_t>& flatb = qt ? h->q_flat : h->el_flat;
	DevBuf<float>& tabb = qt ? h->q_tab : h->el_tab;
	XCUDA(vidb.alloc(vid.size()));
	XCUDA(recb.alloc(rec.size()));
	XCUDA(cbb.alloc(cb.size()));
	XCUDA(flatb.alloc(flat.size()));
	XCUDA(tabb.alloc(g4.size()));
	auto up = [&](void* dst, const void* src, size_t bytes) {
		return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
	};
	XCUDA(up(vidb.p, vid.data(), vid.size() * sizeof(uint4)));
	XCUDA(up(recb.p, rec.data(), rec.size() * sizeof(float4)));
	XCUDA(up(cbb.p, cb.data(), cb.size() * 4));
	XCUDA(up(flatb.p, flat.data(), flat.size() * 4));
	XCUDA(up(tabb.p, g4.data(), g4.size() * 4));
	XCUDA(cudaStreamSynchronize(h->stream));
	if (qt) {
		h->q_colours = ncol;
		h->q_nel = nel;
	} else {
		h->ctx.el_colours = ncol;
		h->ctx.nel = nel;
	}
	h->device_bytes += vid.size() * 16 + rec.size() * 16 + cb.size() * 4 + flat.size() * 4 + g4.size() * 4;
	return XFEM_OK;
}

int build_elements(xfem_body* h) {
	if (h->el_mode != kElQMixed) return build_element_set(h, h->el_mode, false);
	const int rc = build_element_set(h, kElH27, false);  // the H27s in el_*
	return rc ? rc : build_element_set(h, kElT10, true);  // the T10s in q_*
}

// The tets of every mixed body in device order (colour-major over the tets'
// own colouring, bodies in order inside a colour): four device vertex ids,
// the record as five float4 planes (plane k of tet i at rec[k * n + i]: the
// 17 floats of ElementParamsLinearTet, XPBDFEM/Fem.h:52-60, then three pads)
// and each tet's index in its body's tet order (the amortized damping slices).
int build_mixed_tets(xfem_body* h) {
	uint32_t ncol = 0, n = 0;
	for (const BodyHost& b : h->bodies) {
		ncol = std::max(ncol, b.tsched.ncolours);
		n += b.nt;
	}
	std::vector<uint4> vid(n);
	std::vector<uint32_t> cb(ncol + 1, 0), flat(n);
	std::vector<float4> rec(5 * (size_t)n);
	uint32_t o = 0;
	for (uint32_t c = 0; c < ncol; c++) {
		cb[c] = o;
		for (const BodyHost& b : h->bodies) {
			const ElemSchedule& es = b.tsched;
			if (c >= es.ncolours) continue;
			for (uint32_t k = es.colour_begin[c]; k < es.colour_begin[c + 1]; k++, o++) {
				const uint32_t t = es.order[k];
				const uint32_t* is = &b.tets[4 * (size_t)t];
				vid[o] = make_uint4(b.vbase + b.sched.vert_rank[is[0]], b.vbase + b.sched.vert_rank[is[1]],
				                    b.vbase + b.sched.vert_rank[is[2]], b.vbase + b.sched.vert_rank[is[3]]);
				flat[o] = k;
				const float* e = &b.ep[17 * (size_t)t];
				for (uint32_t k4 = 0; k4 < 4; k4++)
					rec[(size_t)k4 * n + o] = make_float4(e[4 * k4], e[4 * k4 + 1], e[4 * k4 + 2], e[4 * k4 + 3]);
				rec[4 * (size_t)n + o] = make_float4(e[16], 0.0f, 0.0f, 0.0f);
			}
		}
	}
	cb[ncol] = o;
	XCUDA(h->mt_vid.alloc(vid.size()));
	XCUDA(h->mt_rec.alloc(rec.size()));
	XCUDA(h->mt_cb.alloc(cb.size()));
	XCUDA(h->mt_flat.alloc(flat.size()));
	auto up = [&](void* dst, const void* src, size_t bytes) {
		return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
	};
	XCUDA(up(h->mt_vid.p, vid.data(), vid.size() * sizeof(uint4)));
	XCUDA(up(h->mt_rec.p, rec.data(), rec.size() * sizeof(float4)));
	XCUDA(up(h->mt_cb.p, cb.data(), cb.size() * 4));
	XCUDA(up(h->mt_flat.p, flat.data(), flat.size() * 4));
	XCUDA(cudaStreamSynchronize(h->stream));
	h->ctx.mt_colours = ncol;
	h->ctx.nmt = n;
	h->device_bytes += vid.size() * 16 + rec.size() * 16 + cb.size() * 4 + flat.size() * 4;
	return XFEM_OK;
}

// The brick layout of the launch form sync_mode 4 (k_bricks), built from the
// packed cube chunks. Clusters are sorted by their lowest device vertex (a
// Morton rank, so nearby clusters sort together) and cut into `nbricks`
// runs of equal length: the bricks. A brick's clusters of one colour form its
// chunks of that colour, in the colour's own order. A vertex whose clusters
// all lie in one brick gets a slot in that brick's shared memory (up to
// `slot_cap` per brick; the rest stay in vert). Bricks are neighbours when
// they share a vertex. The results do not depend on the split: the colours
// and the clusters are those of the other launch forms.
int build_bricks(xfem_body* h, const std::vector<uint32_t>& ccb, const std::vector<float4>& cblk,
                 const std::vector<ChunkMeta>& meta, const std::vector<uint32_t>& lane_dv,
                 const std::vector<uint8_t>& lane_nv) {
	const uint32_t ncol = h->ncolours, nch = (uint32_t)meta.size();
	int sms = 0, optin = 0, per_sm_smem = 0;
	XCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
	XCUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
	XCUDA(cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device));
	int64_t cap = ((int64_t)optin - 8 * (int64_t)kBrickChunkBytes - 4096) / kBrickVertexBytes;
	if (cap <= 0 || ncol > 64) return XFEM_OK;
	// populated lanes, keyed by their lowest device vertex
	std::vector<uint64_t> lanes;
	std::vector<uint32_t> chunk_colour(nch);
	for (uint32_t c = 0; c < ncol; c++)
		for (uint32_t k = ccb[c]; k < ccb[c + 1]; k++) chunk_colour[k] = c;
	for (size_t i = 0; i < (size_t)nch * kLanes; i++) {
		if (!lane_nv[i]) continue;
		uint32_t key = 0xffffffffu;
		for (uint32_t sl = 0; sl < lane_nv[i]; sl++) key = std::min(key, lane_dv[i * kMaxClusterVerts + sl]);
		lanes.push_back((uint64_t)key << 32 | (uint64_t)i);
	}
	if (lanes.empty()) return XFEM_OK;
	std::sort(lanes.begin(), lanes.end());
	const uint64_t L = lanes.size();
	// one brick per SM (or xfem_options.bricks), about one chunk per brick and colour at least.
	// Two bricks per SM, each with blocks of 192 threads, when each still gets three chunks
	// per colour or more: one brick's neighbour waits and barrier then overlap the other's
	// solves (the throughput mesh, 3.4 chunks per brick and colour: 0.979 ms per frame
	// against 0.990 with one brick of 256 threads). Their private vertices are capped so
	// that two blocks of six chunk buffers fit one SM.
	const bool pairs = !h->opt.bricks && L >= 3ull * 2 * (uint64_t)sms * kLanes * ncol;
	if (pairs) {
		const int64_t cap2 = ((int64_t)per_sm_smem / 2 - 1024 - 6 * (int64_t)kBrickChunkBytes - 4096) / kBrickVertexBytes;
		cap = std::min(cap, cap2);
		if (cap <= 0) return XFEM_OK;
	}
	h->brick_block = pairs ? 192 : 256;
	const uint64_t want = h->opt.bricks ? (uint64_t)h->opt.bricks : (uint64_t)sms * (pairs ? 2u : 1u);
	const uint32_t nb = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, L / ((uint64_t)kLanes * ncol)));
	std::vector<uint32_t> brick_of((size_t)nch * kLanes, 0xffffffffu);
	for (uint64_t j = 0; j < L; j++) brick_of[(uint32_t)lanes[j]] = (uint32_t)(j * nb / L);
	// (vertex, brick) incidences
	// every cluster touching each vertex, as colour << 16 | brick; chunks are
	// colour-major, so each vertex's touches come in ascending colour order
	const uint32_t nvv = h->nverts;
	std::vector<uint32_t> toff((size_t)nvv + 1, 0);
	for (uint32_t k = 0; k < nch; k++)
		for (uint32_t lane = 0; lane < kLanes; lane++) {
			const uint32_t i = k * kLanes + lane;
			if (brick_of[i] != 0xffffffffu)
				for (uint32_t sl = 0; sl < lane_nv[i]; sl++) toff[lane_dv[(size_t)i * kMaxClusterVerts + sl] + 1]++;
		}
	for (uint32_t v = 0; v < nvv; v++) toff[v + 1] += toff[v];
	std::vector<uint32_t> touch(toff[nvv]);
	{
		std::vector<uint32_t> fill(toff.begin(), toff.end() - 1);
		for (uint32_t k = 0; k < nch; k++)
			for (uint32_t lane = 0; lane < kLanes; lane++) {
				const uint32_t i = k * kLanes + lane;
				if (brick_of[i] != 0xffffffffu)
					for (uint32_t sl = 0; sl < lane_nv[i]; sl++)
						touch[fill[lane_dv[(size_t)i * kMaxClusterVerts + sl]]++] = chunk_colour[k] << 16 | brick_of[i];
			}
	}
	std::vector<uint32_t> slot(nvv, 0xffffffffu), npriv(nb, 0);
	std::vector<std::vector<uint32_t>> priv(nb), fin(nb);
	std::vector<std::vector<uint32_t>> nbl(nb);
	for (uint32_t v = 0; v < nvv; v++) {
		const uint32_t t0 = toff[v], t1 = toff[v + 1];
		if (t0 == t1) continue;  // in no cluster
		uint32_t bmin = 0xffffu;
		bool one = true;
		for (uint32_t t = t0; t < t1; t++) {
			bmin = std::min(bmin, touch[t] & 0xffffu);
			one = one && (touch[t] & 0xffffu) == (touch[t0] & 0xffffu);
		}
		if (one && npriv[bmin] < (uint64_t)cap) {
			slot[v] = npriv[bmin]++;
			priv[bmin].push_back(v);
		} else {
			fin[bmin].push_back(v);  // the lowest brick touching it finalizes it
			for (uint32_t x = t0; x < t1; x++)
				for (uint32_t y = t0; y < t1; y++)
					if ((touch[x] & 0xffffu) != (touch[y] & 0xffffu)) nbl[touch[x] & 0xffffu].push_back(touch[y] & 0xffffu);
		}
	}
	std::vector<uint32_t> pbeg(nb + 1, 0), pvid, fbeg(nb + 1, 0), fvid, nbeg(nb + 1, 0), nbv;
	uint32_t pmax = 0;
	for (uint32_t b = 0; b < nb; b++) {
		pbeg[b] = (uint32_t)pvid.size();
		pvid.insert(pvid.end(), priv[b].begin(), priv[b].end());
		pmax = std::max(pmax, (uint32_t)priv[b].size());
		fbeg[b] = (uint32_t)fvid.size();
		fvid.insert(fvid.end(), fin[b].begin(), fin[b].end());
		std::sort(nbl[b].begin(), nbl[b].end());
		nbl[b].erase(std::unique(nbl[b].begin(), nbl[b].end()), nbl[b].end());
		nbeg[b] = (uint32_t)nbv.size();
		nbv.insert(nbv.end(), nbl[b].begin(), nbl[b].end());
	}
	pbeg[nb] = (uint32_t)pvid.size();
	fbeg[nb] = (uint32_t)fvid.size();
	nbeg[nb] = (uint32_t)nbv.size();
	// brick chunks: brick-major, colour-major inside a brick. Inside a brick
	// and colour the clusters touching a vertex of another brick (boundary)
	// come first, in the colour's own order, then the others (interior); the
	// chunks up to the one holding the last boundary cluster wait for the
	// neighbouring bricks, the rest run at once.
	std::vector<std::vector<uint32_t>> bc((size_t)nb * ncol), bi((size_t)nb * ncol);
	for (uint32_t k = 0; k < nch; k++)
		for (uint32_t lane = 0; lane < kLanes; lane++) {
			const uint32_t i = k * kLanes + lane;
			if (brick_of[i] == 0xffffffffu) continue;
			bool bnd = false;
			for (uint32_t sl = 0; sl < lane_nv[i]; sl++) bnd = bnd || slot[lane_dv[(size_t)i * kMaxClusterVerts + sl]] == 0xffffffffu;
			(bnd ? bc : bi)[(size_t)brick_of[i] * ncol + chunk_colour[k]].push_back(i);
		}
	// per brick and colour, the bricks its boundary clusters wait for: for
	// each vertex of such a cluster, the brick of the cluster that touched it
	// last before (the highest lower colour touching it, else the highest
	// colour, in the previous substep), when that is another brick
	std::vector<std::vector<uint32_t>> nbc_l((size_t)nb * ncol);
	for (uint32_t v = 0; v < nvv; v++)
		for (uint32_t x = toff[v]; x < toff[v + 1]; x++) {
			const uint32_t prev = x > toff[v] ? x - 1 : toff[v + 1] - 1;  // the previous touch, wrapping
			const uint32_t bx = touch[x] & 0xffffu, bp = touch[prev] & 0xffffu;
			if (bp != bx) nbc_l[(size_t)bx * ncol + (touch[x] >> 16)].push_back(bp);
		}
	std::vector<uint32_t> cnb_begin((size_t)nb * ncol + 1, 0), cnb;
	for (size_t q = 0; q < nbc_l.size(); q++) {
		std::sort(nbc_l[q].begin(), nbc_l[q].end());
		nbc_l[q].erase(std::unique(nbc_l[q].begin(), nbc_l[q].end()), nbc_l[q].end());
		cnb_begin[q] = (uint32_t)cnb.size();
		cnb.insert(cnb.end(), nbc_l[q].begin(), nbc_l[q].end());
	}
	cnb_begin[nbc_l.size()] = (uint32_t)cnb.size();
	std::vector<uint32_t> bcb((size_t)nb * ncol + 1, 0), bwait((size_t)nb * ncol, 0);
	uint32_t nbc = 0;
	size_t nbnd = 0;
	for (size_t q = 0; q < bc.size(); q++) {
		bcb[q] = nbc;
		bwait[q] = nbc + (uint32_t)((bc[q].size() + kLanes - 1) / kLanes);
		nbnd += bc[q].size();
		bc[q].insert(bc[q].end(), bi[q].begin(), bi[q].end());
		nbc += (uint32_t)((bc[q].size() + kLanes - 1) / kLanes);
	}
	bcb[bc.size()] = nbc;
	const uint32_t per16 = kBrickChunkBytes / 16u;
	std::vector<float4> blk((size_t)nbc * per16, make_float4(0, 0, 0, 0));
	// per tet row and lane of the persistent layout: where the tet's c0 word
	// (plane 3 of its record) sits in the brick chunks, so that material
	// changes reach both layouts
	std::vector<uint32_t> brec_of_slot((size_t)h->nrows * kLanes, 0);
	parallel_for((uint32_t)bc.size(), [&](uint32_t q) {
		for (size_t j = 0; j < bc[q].size(); j++) {
			const uint32_t i = bc[q][j], k = i / kLanes, a = i % kLanes;
			const uint32_t dch = bcb[q] + (uint32_t)(j / kLanes), dl = (uint32_t)(j % kLanes);
			const float4* src = &cblk[meta[k].off16];
			float4* dst = &blk[(size_t)dch * per16];
			for (uint32_t t = 0; t < 6; t++)
				brec_of_slot[((size_t)meta[k].trow + t) * kLanes + a] = dch * per16 + (t * 4u + 3u) * kLanes + dl;
			for (uint32_t r = 0; r < 24; r++) dst[r * kLanes + dl] = src[r * kLanes + a];
			const uint32_t* sw = reinterpret_cast<const uint32_t*>(src + 24 * kLanes);
			uint32_t* dw = reinterpret_cast<uint32_t*>(dst + 24 * kLanes);
			dw[dl] = sw[a];  // header
			for (uint32_t sl = 0; sl < 8; sl++) {
				const uint32_t v = sw[kLanes + sl * kLanes + a];
				dw[kLanes + sl * kLanes + dl] = slot[v] != 0xffffffffu ? (kPrivate | slot[v]) : v;
			}
		}
	});
	std::vector<uint32_t> brec(h->ntets, 0);
	for (const BodyHost& bh : h->bodies)
		for (uint32_t t = 0; t < bh.nt; t++) brec[bh.tbase + t] = brec_of_slot[bh.tet_slot[t]];
	if ((uint64_t)nbc * per16 > 0xffffffffull) return fail(XFEM_ELIMIT, "brick chunks exceed 64 GiB");
	XCUDA(h->tet_brec_dev.alloc(brec.size()));
	XCUDA(h->bcblk.alloc(blk.size()));
	XCUDA(h->bcb.alloc(bcb.size()));
	XCUDA(h->bwait.alloc(bwait.size()));
	XCUDA(h->bcnb_begin.alloc(cnb_begin.size()));
	XCUDA(h->bcnb.alloc(std::max<size_t>(1, cnb.size())));
	XCUDA(h->bpriv_begin.alloc(pbeg.size()));
	XCUDA(h->bpriv_vid.alloc(std::max<size_t>(1, pvid.size())));
	XCUDA(h->bfin_begin.alloc(fbeg.size()));
	XCUDA(h->bfin_vid.alloc(std::max<size_t>(1, fvid.size())));
	XCUDA(h->bnb_begin.alloc(nbeg.size()));
	XCUDA(h->bnb.alloc(std::max<size_t>(1, nbv.size())));
	XCUDA(h->bflag.alloc((size_t)nb * kBrickFlagStride));
	auto up = [&](void* dst, const void* src, size_t bytes) {
		return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
	};
	XCUDA(up(h->bcblk.p, blk.data(), blk.size() * sizeof(float4)));
	XCUDA(up(h->tet_brec_dev.p, brec.data(), brec.size() * 4));
	XCUDA(up(h->bcb.p, bcb.data(), bcb.size() * 4));
	XCUDA(up(h->bwait.p, bwait.data(), bwait.size() * 4));
	XCUDA(up(h->bcnb_begin.p, cnb_begin.data(), cnb_begin.size() * 4));
	XCUDA(up(h->bcnb.p, cnb.data(), cnb.size() * 4));
	XCUDA(up(h->bpriv_begin.p, pbeg.data(), pbeg.size() * 4));
	XCUDA(up(h->bpriv_vid.p, pvid.data(), pvid.size() * 4));
	XCUDA(up(h->bfin_begin.p, fbeg.data(), fbeg.size() * 4));
	XCUDA(up(h->bfin_vid.p, fvid.data(), fvid.size() * 4));
	XCUDA(up(h->bnb_begin.p, nbeg.data(), nbeg.size() * 4));
	XCUDA(up(h->bnb.p, nbv.data(), nbv.size() * 4));
	XCUDA(cudaStreamSynchronize(h->stream));
	DevCtx& c = h->ctx;
	c.bcblk = h->bcblk.p;
	c.bchunk_begin = h->bcb.p;
	c.bchunk_wait_end = h->bwait.p;
	c.bcnb_begin = h->bcnb_begin.p;
	c.bcnb = h->bcnb.p;
	c.bpriv_begin = h->bpriv_begin.p;
	c.bpriv_vid = h->bpriv_vid.p;
	c.bfin_begin = h->bfin_begin.p;
	c.bfin_vid = h->bfin_vid.p;
	c.bnb_begin = h->bnb_begin.p;
	c.bnb = h->bnb.p;
	c.bflag = h->bflag.p;
	c.nbricks = nb;
	c.bpriv_max = pmax;
	h->device_bytes += blk.size() * 16 + (brec.size() + bcb.size() + bwait.size() + cnb_begin.size() + cnb.size() + pbeg.size() + pvid.size() + fbeg.size() + fvid.size() +
	                                      nbeg.size() + nbv.size() + (size_t)nb * kBrickFlagStride) * 4;
	if (getenv("XFEM_SETUP_TIMING"))
		fprintf(stderr, "xfem bricks: %u bricks, %u chunks, %zu private and %zu shared vertices, at most %u private "
		                "per brick, %zu neighbour links (%zu waits per substep over the colours), %zu of %zu clusters "
		                "on a brick boundary\n",
		        nb, nbc, pvid.size(), fvid.size(), pmax, nbv.size(), cnb.size(), nbnd, (size_t)L);
	return XFEM_OK;
}

// Packs every body's schedule into the merged device layout and uploads it.
int build_device(xfem_body* h) {
	SetupClock clk;
	const uint32_t nb = (uint32_t)h->bodies.size();
	uint32_t nverts = 0, ntets = 0, ncol = 1;
	for (auto& b : h->bodies) {
		b.vbase = nverts;
		b.tbase = ntets;
		nverts += b.nv;
		ntets += b.nt;
		ncol = std::max(ncol, b.sched.ncolours);
	}
	if (nb >= (1u << 16)) return fail(XFEM_ELIMIT, "too many bodies (at most 65535 per handle)");
	h->nverts = nverts;
	h->ntets = ntets;
	h->ncolours = ncol;
	// chunks: colour-major, bodies in order, 32 clusters per chunk
	std::vector<uint32_t> ccb(ncol + 1, 0);
	std::vector<std::vector<Lane>> chunk_lanes;
	for (uint32_t c = 0; c < ncol; c++) {
		ccb[c] = (uint32_t)chunk_lanes.size();
		std::vector<Lane> lanes;
		for (uint32_t bi = 0; bi < nb; bi++) {
			const Schedule& s = h->bodies[bi].sched;
			if (c >= s.ncolours) continue;
			for (uint32_t i = s.colour_cl_begin[c]; i < s.colour_cl_begin[c + 1]; i++) lanes.push_back({bi, s.colour_cl[i]});
		}
		for (size_t i = 0; i < lanes.size(); i += kLanes)
			chunk_lanes.emplace_back(lanes.begin() + i, lanes.begin() + std::min(lanes.size(), i + kLanes));
	}
	ccb[ncol] = (uint32_t)chunk_lanes.size();
	const uint32_t nch = (uint32_t)chunk_lanes.size();
	// each lane's distinct vertices in first-touch order (device ids) and tet
	// count; every later pass reads these
	const size_t nlanes = (size_t)nch * kLanes;
	std::vector<uint32_t> lane_dv(nlanes * kMaxClusterVerts);
	std::vector<uint8_t> lane_nv(nlanes, 0), lane_nt(nlanes, 0);
	parallel_for(nch, [&](uint32_t k) {
		for (uint32_t lane = 0; lane < chunk_lanes[k].size(); lane++) {
			const Lane& L = chunk_lanes[k][lane];
			const BodyHost& b = h->bodies[L.body];
			uint32_t vs[kMaxClusterVerts], nvv = 0;
			for (uint32_t q = b.sched.cl_begin[L.cluster]; q < b.sched.cl_begin[L.cluster + 1]; q++)
				for (int n = 0; n < 4; n++) {
					const uint32_t v = b.tets[4 * (size_t)b.sched.cl_tets[q] + n];
					if (std::find(vs, vs + nvv, v) == vs + nvv) vs[nvv++] = v;
				}
			const size_t i = (size_t)k * kLanes + lane;
			for (uint32_t sl = 0; sl < nvv; sl++) lane_dv[i * kMaxClusterVerts + sl] = b.vbase + b.sched.vert_rank[vs[sl]];
			lane_nv[i] = (uint8_t)nvv;
			lane_nt[i] = (uint8_t)(b.sched.cl_begin[L.cluster + 1] - b.sched.cl_begin[L.cluster]);
		}
	});
	std::vector<ChunkMeta> meta(nch);
	std::vector<uint32_t> shape_nt(nch), shape_nv(nch);
	uint64_t total16 = 0;
	uint32_t trows = 0, max_bytes = 128, max_nv = 4;
	for (uint32_t k = 0; k < nch; k++) {
		uint32_t ntm = 0, nvm = 0;
		for (size_t i = (size_t)k * kLanes; i < (size_t)(k + 1) * kLanes; i++) {
			ntm = std::max<uint32_t>(ntm, lane_nt[i]);
			nvm = std::max<uint32_t>(nvm, lane_nv[i]);
		}
		const uint32_t bytes = chunk_block_bytes(ntm, nvm);
		if (total16 + bytes / 16 > 0xffffffffull) return fail(XFEM_ELIMIT, "chunk blocks exceed 64 GiB");
		meta[k] = {(uint32_t)total16, bytes, ntm | (nvm << 8), trows};
		shape_nt[k] = ntm;
		shape_nv[k] = nvm;
		total16 += bytes / 16;
		trows += ntm;
		max_bytes = std::max(max_bytes, bytes);
		max_nv = std::max(max_nv, nvm);
	}
	h->nchunks = nch;
	h->nrows = trows;
	{
		uint32_t mc = 0;
		for (uint32_t c = 0; c < ncol; c++) mc = std::max(mc, ccb[c + 1] - ccb[c]);
		h->max_colour_chunks = mc;
	}
	// The first (lowest-colour) and the last (highest-colour) lane touching
	// each vertex: the first advances it (its owner), the last finishes it
	// when damping sweeps run; chunks are colour-major. Also the chunks
	// touching each vertex (vertex -> chunk lists in increasing chunk order;
	// one vertex appears at most once per chunk, since clusters of one colour
	// share no vertex).
	std::vector<uint32_t> owner(nverts, 0xffffffffu), last(nverts, 0xffffffffu), vc_off(nverts + 1, 0), vc;
	for (size_t i = 0; i < nlanes; i++)
		for (uint32_t sl = 0; sl < lane_nv[i]; sl++) {
			const uint32_t dv = lane_dv[i * kMaxClusterVerts + sl];
			if (owner[dv] == 0xffffffffu) owner[dv] = (uint32_t)i;
			last[dv] = (uint32_t)i;
			vc_off[dv + 1]++;
		}
	for (uint32_t v = 0; v < nverts; v++) vc_off[v + 1] += vc_off[v];
	vc.resize(vc_off[nverts]);
	{
		std::vector<uint32_t> fill(vc_off.begin(), vc_off.end() - 1);
		for (size_t i = 0; i < nlanes; i++)
			for (uint32_t sl = 0; sl < lane_nv[i]; sl++) vc[fill[lane_dv[i * kMaxClusterVerts + sl]]++] = (uint32_t)(i / kLanes);
	}
	clk.lap("chunk shapes");
	std::vector<float4> cblk((size_t)total16, make_float4(0, 0, 0, 0));
	std::vector<uint32_t> lastmask(nlanes, 0);
	for (auto& b : h->bodies) {
		b.tet_slot.assign(b.nt, 0xffffffffu);
		b.tet_rec.assign(b.nt, 0);
	}
	// packing: every chunk writes its own block and its own tets' entries
	parallel_for(nch, [&](uint32_t k) {
		const uint32_t ntm = shape_nt[k], nvm = shape_nv[k];
		float4* rec = &cblk[meta[k].off16];
		uint32_t* hdr = reinterpret_cast<uint32_t*>(rec + 128 * (size_t)ntm);
		uint32_t* vid = hdr + kLanes;
		uint32_t* slot = vid + kLanes * (size_t)nvm;
		for (uint32_t lane = 0; lane < chunk_lanes[k].size(); lane++) {
			const Lane& L = chunk_lanes[k][lane];
			BodyHost& b = h->bodies[L.body];
			const size_t i = (size_t)k * kLanes + lane;
			const uint32_t* dvs = &lane_dv[i * kMaxClusterVerts];
			const uint32_t nvv = lane_nv[i];
			uint32_t ntt = 0;
			for (uint32_t q = b.sched.cl_begin[L.cluster]; q < b.sched.cl_begin[L.cluster + 1]; q++, ntt++) {
				const uint32_t t = b.sched.cl_tets[q];
				uint32_t slots = 0;
				for (int n = 0; n < 4; n++) {
					const uint32_t dv = b.vbase + b.sched.vert_rank[b.tets[4 * (size_t)t + n]];
					slots |= (uint32_t)(std::find(dvs, dvs + nvv, dv) - dvs) << (4 * n);
				}
				slot[(size_t)ntt * kLanes + lane] = slots;
				b.tet_slot[t] = (meta[k].trow + ntt) * kLanes + lane;
				const float* e = &b.ep[17 * (size_t)t];
				float4* r = rec + (size_t)ntt * 4 * kLanes + lane;
				r[0] = make_float4(e[0], e[1], e[2], e[3]);
				r[kLanes] = make_float4(e[4], e[5], e[6], e[7]);
				r[2 * kLanes] = make_float4(e[8], e[9], e[10], e[11]);
				r[3 * kLanes] = make_float4(e[12], e[13], e[14], tet_c0(b, t));
				b.tet_rec[t] = meta[k].off16 + ((size_t)ntt * 4 + 3) * kLanes + lane;
			}
			uint32_t mask = 0, lm = 0;
			for (uint32_t sl = 0; sl < nvv; sl++) {
				vid[(size_t)sl * kLanes + lane] = dvs[sl];
				if (owner[dvs[sl]] == i) mask |= 1u << sl;
				if (last[dvs[sl]] == i) lm |= 1u << sl;
			}
			lastmask[i] = lm;
			hdr[lane] = nvv | (ntt << 4) | (mask << 8) | (L.body << 16);
		}
		// the register-resident cube path needs every lane to be a canonical cube
		static const uint32_t kCube[6] = {0x3210u, 0x1430u, 0x3450u, 0x5630u, 0x3670u, 0x7230u};
		bool cube = ntm == 6 && nvm == 8;
		for (uint32_t lane = 0; cube && lane < chunk_lanes[k].size(); lane++) {
			if ((hdr[lane] & 0xffu) != (8u | (6u << 4))) cube = false;
			for (uint32_t t = 0; cube && t < 6; t++)
				if (slot[(size_t)t * kLanes + lane] != kCube[t]) cube = false;
		}
		if (cube) meta[k].shape |= kShapeCube;
	});
	clk.lap("chunk packing");
	// The cube path takes its slots from a table: its bulk copy stops before
	// the slot words at the end of the block.
	max_bytes = 128;
	for (ChunkMeta& m : meta) {
		if (m.shape & kShapeCube) m.bytes = chunk_block_bytes(6, 8) - 128u * 6u;
		max_bytes = std::max(max_bytes, m.bytes);
	}
	std::vector<uint32_t> isolated;
	for (uint32_t v = 0; v < nverts; v++)
		if (owner[v] == 0xffffffffu) isolated.push_back(v);
	h->nisolated = (uint32_t)isolated.size();
	clk.lap("last masks");
	// dataflow dependencies: the other chunks sharing a vertex, each marked
	// when its colour is lower
	std::vector<uint32_t> chunk_colour(nch), dep_begin(nch + 1, 0), deps;
	for (uint32_t c = 0; c < ncol; c++)
		for (uint32_t k = ccb[c]; k < ccb[c + 1]; k++) chunk_colour[k] = c;
	{
		std::vector<std::vector<uint32_t>> dl(nch);
		parallel_for(nch, [&](uint32_t k) {
			std::vector<uint32_t>& d = dl[k];
			for (size_t i = (size_t)k * kLanes; i < (size_t)(k + 1) * kLanes; i++)
				for (uint32_t sl = 0; sl < lane_nv[i]; sl++) {
					const uint32_t dv = lane_dv[i * kMaxClusterVerts + sl];
					for (uint32_t j = vc_off[dv]; j < vc_off[dv + 1]; j++)
						if (vc[j] != k) d.push_back(vc[j]);
				}
			std::sort(d.begin(), d.end());
			d.erase(std::unique(d.begin(), d.end()), d.end());
			for (uint32_t& j : d) j |= chunk_colour[j] < chunk_colour[k] ? 0x80000000u : 0u;
		});
		uint32_t maxd = 0;
		for (uint32_t k = 0; k < nch; k++) {
			dep_begin[k] = (uint32_t)deps.size();
			deps.insert(deps.end(), dl[k].begin(), dl[k].end());
			maxd = std::max(maxd, (uint32_t)dl[k].size());
		}
		dep_begin[nch] = (uint32_t)deps.size();
		h->max_deps = maxd;
	}
	clk.lap("dataflow deps");
	// vertex state: canonical (X, V) = (rest, 0); bits = lock | body << 8
	std::vector<float4> vert(2 * (size_t)nverts);
	std::vector<uint32_t> dev_of(nverts), tets_dev(4 * (size_t)ntets);
	std::vector<BodyParams> params(nb);
	size_t tbase = 0;
	for (uint32_t bi = 0; bi < nb; bi++) {
		const BodyHost& b = h->bodies[bi];
		for (uint32_t v = 0; v < b.nv; v++) {
			const uint32_t dv = b.vbase + b.sched.vert_rank[v];
			dev_of[b.vbase + v] = dv;
			const uint32_t bits = (b.vflags[v] & 1u ? kFlagLocked : 0u) | (b.vflags[v] & 2u ? kFlagRight : 0u) | (bi << 8);
			vert[2 * (size_t)dv] = make_float4(b.nodes[3 * (size_t)v], b.nodes[3 * (size_t)v + 1], b.nodes[3 * (size_t)v + 2], b.w0[v]);
			vert[2 * (size_t)dv + 1] = make_float4(0.0f, 0.0f, 0.0f, __builtin_bit_cast(float, bits));
		}
		for (size_t i = 0; i < 4 * (size_t)b.nt; i++) tets_dev[tbase + i] = b.vbase + b.sched.vert_rank[b.tets[i]];
		tbase += 4 * (size_t)b.nt;
		params[bi] = make_params(b.settings);
		set_counts(params[bi], b);
	}
	clk.lap("vertex state");
	// upload
	XCUDA(h->vert.alloc(vert.size()));
	XCUDA(h->cblk.alloc(cblk.size()));
	XCUDA(h->ccb.alloc(ccb.size()));
	XCUDA(h->isolated.alloc(isolated.size()));
	XCUDA(h->dep_begin.alloc(dep_begin.size()));
	XCUDA(h->deps.alloc(deps.size()));
	XCUDA(h->done.alloc(nch));
	XCUDA(h->dev_of_vert.alloc(dev_of.size()));
	XCUDA(h->tets_dev.alloc(tets_dev.size()));
	XCUDA(h->chunks.alloc(meta.size()));
	XCUDA(h->params.alloc(params.size()));
	XCUDA(h->bar.alloc(1));
	XCUDA(h->err.alloc(1));
	if (!h->err_host) XCUDA(cudaHostAlloc((void**)&h->err_host, sizeof(int), cudaHostAllocDefault));
	*h->err_host = 0;
	uint32_t maxnv = 1;
	for (auto& b : h->bodies) maxnv = std::max(maxnv, b.nv);
	XCUDA(h->stage.alloc(3 * (size_t)maxnv));
	XCUDA(h->vol.alloc(1));
	if (h->opt.keep_lambdas) XCUDA(h->tlam.alloc((size_t)trows * kLanes));
	auto up = [&](void* dst, const void* src, size_t bytes) {
		return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
	};
	XCUDA(up(h->vert.p, vert.data(), vert.size() * sizeof(float4)));
	XCUDA(up(h->cblk.p, cblk.data(), cblk.size() * sizeof(float4)));
	XCUDA(up(h->ccb.p, ccb.data(), ccb.size() * 4));
	XCUDA(up(h->isolated.p, isolated.data(), isolated.size() * 4));
	XCUDA(up(h->dep_begin.p, dep_begin.data(), dep_begin.size() * 4));
	XCUDA(up(h->deps.p, deps.data(), deps.size() * 4));
	XCUDA(up(h->dev_of_vert.p, dev_of.data(), dev_of.size() * 4));
	XCUDA(up(h->tets_dev.p, tets_dev.data(), tets_dev.size() * 4));
	XCUDA(up(h->chunks.p, meta.data(), meta.size() * sizeof(ChunkMeta)));
	XCUDA(up(h->params.p, params.data(), params.size() * sizeof(BodyParams)));
	XCUDA(cudaMemsetAsync(h->err.p, 0, sizeof(int), h->stream));
	if (h->tlam.p) XCUDA(cudaMemsetAsync(h->tlam.p, 0, h->tlam.n * sizeof(float2), h->stream));
	XCUDA(cudaStreamSynchronize(h->stream));
	clk.lap("upload");
	h->device_bytes = vert.size() * 16 + cblk.size() * 16 + (ccb.size() + isolated.size() + dev_of.size() +
	                  tets_dev.size() + dep_begin.size() + deps.size() + nch) * 4 + meta.size() * 16 + params.size() * sizeof(BodyParams) + h->stage.n * 4 + h->tlam.n * 8;
	{
		std::vector<uint32_t> rec(ntets), slot(ntets);
		std::vector<float> vol(ntets), inv_mu(ntets);
		for (const BodyHost& b : h->bodies)
			for (uint32_t t = 0; t < b.nt; t++) {
				rec[b.tbase + t] = (uint32_t)b.tet_rec[t];
				slot[b.tbase + t] = b.tet_slot[t];
				vol[b.tbase + t] = b.ep[17 * (size_t)t + 15];
				inv_mu[b.tbase + t] = 1.0f / (b.tet_mu.empty() ? 1.0f / b.settings.compliance : b.tet_mu[t]);
			}
		XCUDA(h->tet_rec_dev.alloc(ntets));
		XCUDA(h->tet_slot_dev.alloc(ntets));
		XCUDA(h->tet_vol_dev.alloc(ntets));
		XCUDA(h->tet_inv_mu.alloc(ntets));
		XCUDA(h->io.alloc(6 * (size_t)nverts + ntets));
		XCUDA(up(h->tet_rec_dev.p, rec.data(), rec.size() * 4));
		XCUDA(up(h->tet_slot_dev.p, slot.data(), slot.size() * 4));
		XCUDA(up(h->tet_vol_dev.p, vol.data(), vol.size() * 4));
		XCUDA(up(h->tet_inv_mu.p, inv_mu.data(), inv_mu.size() * 4));
		// per tet row: the index in the body's flattened order (the amortized
		// damping slices) and the surface area (PBD damping)
		std::vector<uint32_t> flat((size_t)trows * kLanes, 0);
		std::vector<float> area((size_t)trows * kLanes, 1.0f);
		for (const BodyHost& b : h->bodies) {
			const Schedule& sc = b.sched;
			uint32_t o = 0;
			for (uint32_t c = 0; c < sc.ncolours; c++)
				for (uint32_t i = sc.colour_cl_begin[c]; i < sc.colour_cl_begin[c + 1]; i++)
					for (uint32_t q = sc.cl_begin[sc.colour_cl[i]]; q < sc.cl_begin[sc.colour_cl[i] + 1]; q++) {
						const uint32_t t = sc.cl_tets[q];
						flat[b.tet_slot[t]] = o++;
						area[b.tet_slot[t]] = b.ep[17 * (size_t)t + 16];
					}
		}
		XCUDA(h->tflat.alloc(flat.size()));
		XCUDA(h->tarea.alloc(area.size()));
		XCUDA(h->tick.alloc(1));
		XCUDA(h->lastmask.alloc(lastmask.size()));
		XCUDA(up(h->lastmask.p, lastmask.data(), lastmask.size() * 4));
		XCUDA(h->pass_on.alloc(16 * (size_t)ncol));
		const std::vector<uint8_t> pt = pass_table(h->bodies, ncol);
		XCUDA(up(h->pass_on.p, pt.data(), pt.size()));
		XCUDA(up(h->tflat.p, flat.data(), flat.size() * 4));
		XCUDA(up(h->tarea.p, area.data(), area.size() * 4));
		const uint32_t tick0 = h->bodies.empty() ? 0u : h->bodies[0].settings.tick_id;
		XCUDA(up(h->tick.p, &tick0, 4));
		XCUDA(cudaStreamSynchronize(h->stream));
		h->device_bytes += (uint64_t)trows * kLanes * 8 + 4;
		h->device_bytes += (uint64_t)ntets * 16 + h->io.n * 4;
	}
	if (h->el_mode) {  // before the rings: a hex ring addresses its hexes by device index
		int rr = build_elements(h);
		if (!rr && h->el_mode == kElMixed) rr = build_mixed_tets(h);
		if (rr) return rr;
	}
	if (h->ring_mode) {
		int rr = build_rings(h);
		if (rr) return rr;
	}
	DevCtx& c = h->ctx;
	c.vert = h->vert.p;
	c.cblk = h->cblk.p;
	c.chunk_smem = max_bytes;
	// When every chunk takes the register-resident cube path the vertex slots
	// are not needed. Leaving them out is not only smaller: the kernel runs
	// faster the less shared memory a block takes (throughput mesh, 256-thread
	// blocks: 1.37 ms per frame at 14.2 KB per warp, 1.49 ms at 22.4 KB,
	// 1.85 ms at 28.4 KB), so the chunk is the only staged data.
	bool all_cube = true;
	for (const ChunkMeta& m : meta) all_cube = all_cube && (m.shape & kShapeCube);
	c.vs_off = max_bytes;
	c.warp_smem = max_bytes + (all_cube ? 0u : 2u * max_nv * kLanes * 16u);
	c.tlam = h->tlam.p;
	c.chunks = h->chunks.p;
	c.ntrows = trows;
	c.damp_kinds = damp_kinds_of(h->bodies);
	c.ext = ext_any_of(h->bodies) ? 1u : 0u;
	c.nvol = nvol_of(h->bodies);
	c.lastmask = h->lastmask.p;
	c.pass_on = h->pass_on.p;
	c.tick = h->tick.p;
	c.tflat = h->tflat.p;
	c.tarea = h->tarea.p;
	c.colour_chunk_begin = h->ccb.p;
	c.isolated = h->isolated.p;
	c.dep_begin = h->dep_begin.p;
	c.deps = h->deps.p;
	c.done = h->done.p;
	c.nchunks = nch;
	c.bodies = h->params.p;
	c.nverts = nverts;
	c.nbodies = nb;
	c.nisolated = h->nisolated;
	c.ncolours = ncol;
	c.bar_count = h->bar.p;
	c.err = h->err.p;
	c.timeout_ns = h->opt.wait_timeout_ms ? (uint64_t)h->opt.wait_timeout_ms * 1000000ull : kDefaultTimeoutNs;
	h->cfg.lambdas = h->opt.keep_lambdas != 0;
	h->cfg.ext = c.ext != 0u;
	c.ring_hdr = h->ring_hdr.p;
	c.ring_node = h->ring_node.p;
	c.ring_ent = h->ring_ent.p;
	c.colour_ring_begin = h->ring_cb.p;
	c.ring_clist = h->ring_clist.p;
	c.ring_cwords = h->ring_cwords.p;
	c.pbd_cl_begin = h->pbd_cb.p;
	c.pbd_cl = h->pbd_cl.p;
	c.pbd_ent = h->pbd_ent.p;
	c.tet_verts = h->tets_dev.p;
	if (h->ring_mode) c.ext = ring_damp_of(h->bodies) ? 1u : 0u;
	c.el_vid = h->el_vid.p;
	c.el_rec = h->el_rec.p;
	c.colour_el_begin = h->el_cb.p;
	c.el_tab = h->el_tab.p;
	c.el_flat = h->el_flat.p;
	c.mt_vid = h->mt_vid.p;
	c.mt_rec = h->mt_rec.p;
	c.colour_mt_begin = h->mt_cb.p;
	c.mt_flat = h->mt_flat.p;
	h->cfg.warp_smem = c.warp_smem;
	h->cfg.total_chunks = nch;
	h->cfg.colour_chunk_begin_host = ccb;
	if (all_cube && !h->ring_mode && !h->el_mode && nch && (h->opt.sync_mode == 0 || h->opt.sync_mode == 4)) {
		const int rb = build_bricks(h, ccb, cblk, meta, lane_dv, lane_nv);
		if (rb) return rb;
		clk.lap("bricks");
	}
	return update_right_targets(h);
}

int set_config(xfem_body* h, int sync_mode, int block) {
	int optin = 0;
	XCUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
	if (sync_mode == 4) {
		// the brick form: the plain solve on an all-cube handle, every brick resident
		if (!h->ctx.nbricks)
			return fail(XFEM_EUNSUPPORTED, "sync_mode 4 (bricks) needs a mesh whose clusters are all whole cubes "
			                               "(the generator's blocks) and one-ring and element modes off");
		if (h->ctx.ext || h->cfg.lambdas)
			return fail(XFEM_EUNSUPPORTED, "sync_mode 4 (bricks) runs no damping, Pixar or cube models, volume passes "
			                               "or multiplier output");
		if (block != 128 && block != 192 && block != 224 && block != 256)
			return fail(XFEM_EINVAL, "sync_mode 4 (bricks) takes blocks of 128, 192, 224 or 256 threads");
		if (brick_smem_bytes(block, h->ctx.bpriv_max) > (size_t)optin)
			return fail(XFEM_EINVAL, "the bricks need more shared memory than the device allows");
		bool fits = false;
		if (const int e = brick_grid_fits(block, h->ctx.bpriv_max, h->ctx.nbricks, &fits))
			return fail(XFEM_ECUDA, std::string("brick kernel configuration: ") + cudaGetErrorString((cudaError_t)e));
		if (!fits) return fail(XFEM_EUNSUPPORTED, "the bricks do not fit on the device at once");
		h->cfg.sync_mode = 4;
		h->cfg.block = block;
		h->cfg.blocks = (int)h->ctx.nbricks;
		if (h->graph) {
			cudaGraphExecDestroy(h->graph);
			h->graph = nullptr;
		}
		return XFEM_OK;
	}
	if (solve_smem_bytes(block, h->cfg.warp_smem) > (size_t)optin)
		return fail(XFEM_EINVAL, "block size " + std::to_string(block) + " needs " +
		                             std::to_string(solve_smem_bytes(block, h->cfg.warp_smem)) +
		                             " bytes of shared memory; the device allows " + std::to_string(optin));
	h->cfg.sync_mode = sync_mode;
	h->cfg.block = block;
	if (const int ek = configure_kernels(h->cfg))
		return fail(XFEM_ECUDA, std::string("kernel configuration: ") + cudaGetErrorString((cudaError_t)ek));
	if (sync_mode == 1 || sync_mode == 3) {
		int blocks = 0;
		const int e = persistent_grid(h->cfg, &blocks);
		if (e) return fail(XFEM_ECUDA, std::string("occupancy query failed: ") + cudaGetErrorString((cudaError_t)e));
		h->cfg.blocks = blocks;
	}
	if (h->graph) {
		cudaGraphExecDestroy(h->graph);
		h->graph = nullptr;
	}
	return XFEM_OK;
}

int run(xfem_body* h, uint32_t nsub, float dt) {
	if (h->cfg.sync_mode == 1 || h->cfg.sync_mode == 3 || h->cfg.sync_mode == 4) {
		const int e = launch_substeps(h->ctx, h->cfg, nsub, dt, h->stream);
		if (e) return fail(XFEM_ECUDA, std::string("persistent launch: ") + cudaGetErrorString((cudaError_t)e));
		return XFEM_OK;
	}
	if (!h->graph || h->graph_nsub != nsub || h->graph_dt != dt) {
		if (h->graph) {
			cudaGraphExecDestroy(h->graph);
			h->graph = nullptr;
		}
		cudaGraph_t g = nullptr;
		XCUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
		const int e = launch_substeps(h->ctx, h->cfg, nsub, dt, h->stream);
		const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
		if (e) return fail(XFEM_ECUDA, std::string("graph capture: ") + cudaGetErrorString((cudaError_t)e));
		if (ec != cudaSuccess) return fail(XFEM_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
		const cudaError_t ei = cudaGraphInstantiate(&h->graph, g, 0);
		cudaGraphDestroy(g);
		if (ei != cudaSuccess) return fail(XFEM_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
		h->graph_nsub = nsub;
		h->graph_dt = dt;
	}
	XCUDA(cudaGraphLaunch(h->graph, h->stream));
	return XFEM_OK;
}

// Times the candidate launch configurations on a saved copy of the state and
// keeps the fastest. The state is restored afterwards.
// force_time: time the pick even when it is the only candidate (the cluster
// layout trial compares two handles by their best time).
int autotune(xfem_body* h, uint32_t nsub, float dt, bool force_time = false) {
	if (h->tuned) return XFEM_OK;
	h->tuned = true;
	const int fixed_sync = (int)h->opt.sync_mode, fixed_block = (int)h->opt.block_size;
	std::vector<std::pair<int, int>> cand;
	// 192 and 224 as well: a colour pass of the throughput mesh has 1,024
	// chunks (6.7 per SM), and fewer warps per block means less shared memory
	const int blocks[] = {64, 128, 192, 224, 256};
	for (int sm : {1, 2, 3, 4}) {
		if (fixed_sync && sm != fixed_sync) continue;
		if (sm == 3 && h->ctx.ext) continue;  // the dataflow kernel runs only the plain solve
		// the brick kernel too, on all-cube handles, without multiplier output
		if (sm == 4 && (h->ctx.ext || !h->ctx.nbricks || h->cfg.lambdas)) continue;
		for (int bs : blocks) {
			if (fixed_block && bs != fixed_block) continue;
			if (sm == 4 && bs == 64) continue;
			cand.push_back({sm, bs});
		}
	}
	if (fixed_sync == 3 && h->ctx.ext) {
		h->tuned = false;
		return fail(XFEM_EUNSUPPORTED, "sync_mode 3 (dataflow) runs no damping, Pixar or cube models or volume passes");
	}
	if (fixed_block && cand.empty()) cand.push_back({fixed_sync ? fixed_sync : 1, fixed_block});
	if (cand.empty()) {
		h->tuned = false;
		return fail(XFEM_EINVAL, "no launch configuration for these options");
	}
	if (cand.size() == 1 && !force_time) return set_config(h, cand[0].first, cand[0].second);
	DevBuf<float4> save;
	XCUDA(save.alloc(h->vert.n));
	XCUDA(cudaMemcpyAsync(save.p, h->vert.p, h->vert.n * sizeof(float4), cudaMemcpyDeviceToDevice, h->stream));
	uint32_t tick_saved = 0;  // the trial launches advance the tick too
	XCUDA(cudaMemcpyAsync(&tick_saved, h->tick.p, 4, cudaMemcpyDeviceToHost, h->stream));
	cudaEvent_t e0, e1;
	XCUDA(cudaEventCreate(&e0));
	XCUDA(cudaEventCreate(&e1));
	const uint32_t ns = std::max(1u, std::min(nsub, 20u));
	float best = 1e30f;
	std::pair<int, int> pick = cand[0];
	for (auto& c : cand) {
		if (set_config(h, c.first, c.second)) continue;
		if (run(h, ns, dt)) continue;  // warm-up (and graph build)
		cudaEventRecord(e0, h->stream);
		int rc = XFEM_OK;
		for (int r = 0; r < 3 && !rc; r++) rc = run(h, ns, dt);
		cudaEventRecord(e1, h->stream);
		if (cudaEventSynchronize(e1) != cudaSuccess || rc) continue;
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (ms < best) {
			best = ms;
			pick = c;
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	XCUDA(cudaMemcpyAsync(h->vert.p, save.p, h->vert.n * sizeof(float4), cudaMemcpyDeviceToDevice, h->stream));
	XCUDA(cudaMemcpyAsync(h->tick.p, &tick_saved, 4, cudaMemcpyHostToDevice, h->stream));
	XCUDA(cudaStreamSynchronize(h->stream));
	int rc = check_device_error(h);
	if (rc) return rc;
	h->tune_ms = best;
	return set_config(h, pick.first, pick.second);
}

int create_common(uint32_t nbodies, const xfem_mesh* meshes, const xfem_settings* settings, const xfem_options* options,
                  xfem_body** out) {
	if (!out) return fail(XFEM_EINVAL, "null output handle");
	*out = nullptr;
	if (nbodies == 0 || !meshes) return fail(XFEM_EINVAL, "no meshes");
	std::unique_ptr<xfem_body> h(new (std::nothrow) xfem_body());
	if (!h) return fail(XFEM_ENOMEM, "host allocation failed");
	if (options) h->opt = *options;
	if (h->opt.block_size && (h->opt.block_size < 64 || h->opt.block_size > 1024 || h->opt.block_size % 32))
		return fail(XFEM_EINVAL, "block_size must be a multiple of 32 in [64, 1024]");
	if (h->opt.sync_mode > 4) return fail(XFEM_EINVAL, "sync_mode must be 0, 1, 2, 3 or 4");
	if (h->opt.cluster_mode > 2) return fail(XFEM_EINVAL, "cluster_mode must be 0, 1, 2 or 3");
	const uint32_t mode = h->opt.cluster_mode == 1 ? 0u : 1u;
	const uint32_t morton = h->opt.no_morton ? 0u : 1u;
	if (const int prc = precheck_inputs(nbodies, meshes, settings)) return prc;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(XFEM_ECUDA, "no CUDA device");
	h->device = h->opt.device > 0 ? h->opt.device : 0;
	if (h->device >= ndev) return fail(XFEM_EINVAL, "device ordinal out of range");
	XCUDA(cudaSetDevice(h->device));
	if (h->opt.stream) {
		h->stream = (cudaStream_t)h->opt.stream;
	} else {
		XCUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
		h->own_stream = true;
	}
	h->bodies.resize(nbodies);
	SetupClock clk;
	int rc = prepare_bodies(h.get(), nbodies, meshes, settings, mode, morton);
	if (rc) return rc;
	uint32_t nring = 0;
	for (const BodyHost& b : h->bodies)
		nring += model_of((b.settings.flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK) == kModelRing ? 1u : 0u;
	if (nring && nring != nbodies)
		return fail(XFEM_EUNSUPPORTED, "continuous-pressure models (energy 8-10) and element models cannot share a handle");
	h->ring_mode = nring > 0;
	for (const BodyHost& b : h->bodies)
		if (b.el != h->bodies[0].el)
			return fail(XFEM_EUNSUPPORTED, "linear tets, hexes and quadratic tets cannot share a handle");
	h->el_mode = h->bodies.empty() ? kElTets : h->bodies[0].el;
	clk.lap("rest state + schedule");
	rc = build_device(h.get());
	clk.lap("device layout");
	if (rc) return rc;
	// default configuration until the first step tunes it
	rc = set_config(h.get(), h->opt.sync_mode ? (int)h->opt.sync_mode : 1,
	                h->opt.block_size ? (int)h->opt.block_size : h->opt.sync_mode == 4 ? h->brick_block : 128);
	if (rc) return rc;
	if (h->opt.sync_mode && h->opt.block_size) h->tuned = true;
	*out = h.release();
	return XFEM_OK;
}

BodyHost* body_of(xfem_body* h, uint32_t body) {
	if (!h || body >= h->bodies.size()) {
		fail(XFEM_EINVAL, "bad handle or body index");
		return nullptr;
	}
	return &h->bodies[body];
}

// The element and one-ring launches (no autotuner, no CUDA graph).
int launch_mode(xfem_body* h, const DevCtx& ctx, uint32_t nsub, float dt) {
	if (h->ring_mode) {
		const int e = h->el_mode == kElHexes ? launch_hex_rings(ctx, 256, nsub, dt, h->stream)
		              : h->el_mode == kElT10 ? launch_t10_rings(ctx, 128, nsub, dt, h->stream)
		              : h->el_mode == kElH27 ? launch_h27_rings(ctx, 128, nsub, dt, h->stream)
		                                     : launch_rings(ctx, 256, nsub, dt, h->stream);
		if (e) return fail(XFEM_ECUDA, std::string("ring launch: ") + cudaGetErrorString((cudaError_t)e));
		return XFEM_OK;
	}
	if (h->el_mode == kElQMixed) {
		// the T10s' context: the same state with the T10 element arrays
		DevCtx ct = ctx;
		ct.el_vid = h->q_vid.p;
		ct.el_rec = h->q_rec.p;
		ct.colour_el_begin = h->q_cb.p;
		ct.el_tab = h->q_tab.p;
		ct.el_flat = h->q_flat.p;
		ct.el_colours = h->q_colours;
		ct.nel = h->q_nel;
		const int e = launch_qmixed(ctx, ct, 256, nsub, dt, h->stream);
		if (e) return fail(XFEM_ECUDA, std::string("element launch: ") + cudaGetErrorString((cudaError_t)e));
		return XFEM_OK;
	}
	const int e = h->el_mode == kElH27     ? launch_h27(ctx, 256, nsub, dt, h->stream)
	              : h->el_mode == kElT10   ? launch_t10(ctx, 256, nsub, dt, h->stream)
	              : h->el_mode == kElMixed ? launch_mixed(ctx, 256, nsub, dt, h->stream)
	                                       : launch_hexes(ctx, 256, nsub, dt, h->stream);
	if (e) return fail(XFEM_ECUDA, std::string("element launch: ") + cudaGetErrorString((cudaError_t)e));
	return XFEM_OK;
}

// Takes the pending XFEM_HOOK_MISSING_ARRIVAL into the context for one
// launch; the destructor clears it again.
struct WaitMissScope {
	xfem_body* h;
	explicit WaitMissScope(xfem_body* hh) : h(hh) {
		h->ctx.wait_miss = h->hook_wait_miss;
		h->hook_wait_miss = 0;
	}
	~WaitMissScope() { h->ctx.wait_miss = 0; }
};

int step(xfem_body* h, uint32_t nsub, float dt) {
	if (!h) return fail(XFEM_EINVAL, "null handle");
	if (!(dt > 0.0f) || !isfinite(dt)) return fail(XFEM_EINVAL, "dt must be > 0");
	if (nsub == 0) return XFEM_OK;
	XCUDA(cudaSetDevice(h->device));
	if (h->ring_mode || h->el_mode) {
		WaitMissScope miss(h);
		return launch_mode(h, h->ctx, nsub, dt);
	}
	int rc = autotune(h, nsub, dt);
	if (rc) return rc;
	if (h->ctx.ext && (h->cfg.sync_mode == 3 || h->cfg.sync_mode == 4)) {
		// damping, a Pixar or cube model or volume passes switched on after
		// the dataflow or the brick kernel was chosen
		if (h->opt.sync_mode == 3)
			return fail(XFEM_EUNSUPPORTED, "sync_mode 3 (dataflow) runs no damping, Pixar or cube models or volume passes");
		if (h->opt.sync_mode == 4)
			return fail(XFEM_EUNSUPPORTED, "sync_mode 4 (bricks) runs no damping, Pixar or cube models or volume passes");
		rc = set_config(h, 1, h->cfg.block);
		if (rc) return rc;
	}
	WaitMissScope miss(h);
	return run(h, nsub, dt);
}

// which: 0 positions, 1 velocities
// A page-locked host buffer that the device addresses directly (memory from
// xfem_alloc_host / cudaMallocHost): its device address, else null.
static void* mapped_host(const void* p) {
	cudaPointerAttributes a{};
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		(void)cudaGetLastError();
		return nullptr;
	}
	return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int get_xyz(xfem_body* h, uint32_t body, int which, float* out) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!out) return fail(XFEM_EINVAL, "null output");
	XCUDA(cudaSetDevice(h->device));
	if (which <= 1) {
		// positions or velocities into page-locked memory: the gather writes
		// them there itself (no staging copy)
		if (float* direct = static_cast<float*>(mapped_host(out))) {
			const int e = launch_gather_xyz(h->vert.p, which, h->dev_of_vert.p + b->vbase, b->nv, direct, h->stream);
			if (e) return fail(XFEM_ECUDA, "gather launch failed");
			return check_device_error(h);
		}
	}
	const int e = launch_gather_xyz(h->vert.p, which, h->dev_of_vert.p + b->vbase, b->nv, h->stage.p, h->stream);
	if (e) return fail(XFEM_ECUDA, "gather launch failed");
	const size_t n = which >= 2 ? b->nv : 3 * (size_t)b->nv;
	XCUDA(cudaMemcpyAsync(out, h->stage.p, n * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
	return check_device_error(h);
}

// Queues the upload of one body's positions (which 0) or velocities (1) on
// the handle's stream, without waiting for it.
static int scatter_xyz(xfem_body* h, const BodyHost* b, int which, const float* in) {
	// page-locked input: the scatter reads it itself (no staging copy)
	const float* src = static_cast<const float*>(mapped_host(in));
	if (!src) {
		XCUDA(cudaMemcpyAsync(h->stage.p, in, 3 * (size_t)b->nv * sizeof(float), cudaMemcpyHostToDevice, h->stream));
		src = h->stage.p;
	}
	const int e = launch_scatter_xyz(h->vert.p, which, h->dev_of_vert.p + b->vbase, b->nv, src, h->stream);
	if (e) return fail(XFEM_ECUDA, "scatter launch failed");
	return XFEM_OK;
}

int set_xyz(xfem_body* h, uint32_t body, int which, const float* in) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!in) return fail(XFEM_EINVAL, "null input");
	XCUDA(cudaSetDevice(h->device));
	const int rc = scatter_xyz(h, b, which, in);
	return rc ? rc : check_device_error(h);
}

// Rewrites c0 = (1/mu)/volume in one body's records on the device (and 1/mu
// for the adjoint) after a material change.
int update_material(xfem_body* h, const BodyHost& b) {
	const float* mu_dev = nullptr;
	if (!b.tet_mu.empty()) {
		XCUDA(cudaMemcpyAsync(h->io.p, b.tet_mu.data(), b.nt * sizeof(float), cudaMemcpyHostToDevice, h->stream));
		mu_dev = h->io.p;
	}
	int e = launch_set_c0(h->cblk.p, h->tet_rec_dev.p + b.tbase, h->tet_vol_dev.p + b.tbase, mu_dev,
	                      1.0f / b.settings.compliance, b.nt, h->tet_inv_mu.p + b.tbase, h->stream);
	if (!e && h->bcblk.p)  // the brick chunks hold their own copy of each record
		e = launch_set_c0(h->bcblk.p, h->tet_brec_dev.p + b.tbase, h->tet_vol_dev.p + b.tbase, mu_dev,
		                  1.0f / b.settings.compliance, b.nt, h->tet_inv_mu.p + b.tbase, h->stream);
	if (e) return fail(XFEM_ECUDA, "material update launch failed");
	XCUDA(cudaStreamSynchronize(h->stream));
	return XFEM_OK;
}

}  // namespace

extern "C" {

int xfem_settings_default(xfem_settings* s) {
	if (!s) return fail(XFEM_EINVAL, "null settings");
	memset(s, 0, sizeof(*s));
	// struct Settings defaults, XPBDFEM/Settings.h:80-91
	s->time_scale = 1.0f;
	s->substeps_per_second = 1800.0f;
	s->volume_passes = 0;
	s->gravity[0] = 0.0f;
	s->gravity[1] = -9.81f;
	s->gravity[2] = 0.0f;
	s->compliance = 0.01f;
	s->damping = 0.0f;
	s->pbd_damping = 0.0f;
	s->drag = 0.0f;
	s->poissons_ratio = 0.45f;
	s->wonkiness = 0.0f;
	s->left_right_separation = 1.0f;
	// flags = 0 in the reference selects Energy_Pixar; this path's default is
	// the Neo-Hookean MixedSel energy with the coupled solve.
	s->flags = (XFEM_ENERGY_MIXED_SEL << XFEM_ENERGY_BIT) | (1u << XFEM_XPBD_SOLVE_BIT);
	s->time_corrected_drag = 0.0f;
	s->yeoh[0] = 0.1095f;
	s->yeoh[1] = 14.95f;
	s->yeoh[2] = 4.595f;
	s->ground = 0;
	s->ground_normal[2] = 1.0f;
	s->ground_offset = 0.0f;
	s->friction = 0.0f;
	// Settings::lockedRightTransform3d = mat3(1) and Geo3d::origin = 0 until
	// the demo sets them (XPBDFEM/Demo.cpp:79, XPBDFEM/Geo.h:69)
	s->locked_right_transform[0] = s->locked_right_transform[4] = s->locked_right_transform[8] = 1.0f;
	return XFEM_OK;
}

int xfem_create(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data, uint32_t idx_data_count,
                float density, const xfem_settings* settings, xfem_body** out) {
	return xfem_create_ex(node_data, node_data_count, idx_data, idx_data_count, density, settings, nullptr, out);
}

// cluster_mode 3, the tets-per-lane axis of the launch configuration: edge-star
// clusters (up to 6 tets per lane, 192 per warp) or one tet per lane (32 per
// warp). The cluster layout fixes the colour order, so it cannot change under
// a handle: both layouts are built, each is tuned over block size and launch
// form and timed on a saved copy of its state (20 substeps of 1/1200 s, the
// state restored afterwards), and the faster handle is kept. Meshes without
// linear-tet clusters (rings, hexes, quadratic or mixed meshes) keep the
// first.
static int create_tuned_layout(uint32_t nbodies, const xfem_mesh* meshes, const xfem_settings* settings,
                               const xfem_options* options, xfem_body** out) {
	if (!out) return fail(XFEM_EINVAL, "null output handle");
	*out = nullptr;
	xfem_options o = *options;
	std::unique_ptr<xfem_body> best;
	for (uint32_t m : {2u, 1u}) {
		o.cluster_mode = m;
		xfem_body* raw = nullptr;
		int rc = create_common(nbodies, meshes, settings, &o, &raw);
		if (rc) {
			if (best) break;  // e.g. the brick form forced: one tet per lane has no cube chunks
			return rc;
		}
		std::unique_ptr<xfem_body> h(raw);
		if (h->ring_mode || h->el_mode) {
			*out = h.release();
			return XFEM_OK;
		}
		h->tuned = false;  // a fixed sync_mode and block_size are still timed
		rc = autotune(h.get(), 20, 1.0f / 1200.0f, true);
		if (rc) return rc;
		if (!best || h->tune_ms < best->tune_ms) best = std::move(h);
	}
	*out = best.release();
	return XFEM_OK;
}

static int create_any(uint32_t nbodies, const xfem_mesh* meshes, const xfem_settings* settings,
                      const xfem_options* options, xfem_body** out) {
	if (options && options->cluster_mode == 3) return create_tuned_layout(nbodies, meshes, settings, options, out);
	return create_common(nbodies, meshes, settings, options, out);
}

int xfem_create_ex(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data, uint32_t idx_data_count,
                   float density, const xfem_settings* settings, const xfem_options* options, xfem_body** out) {
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, density};
	return create_any(1, &m, settings, options, out);
}

int xfem_batch_create(uint32_t nbodies, const xfem_mesh* meshes, const xfem_settings* settings,
                      const xfem_options* options, xfem_body** out) {
	return create_any(nbodies, meshes, settings, options, out);
}

int xfem_destroy(xfem_body* b) {
	if (!b) return XFEM_OK;
	cudaSetDevice(b->device);
	if (b->stream) cudaStreamSynchronize(b->stream);
	delete b;
	return XFEM_OK;
}

int xfem_get_info(const xfem_body* b, xfem_info* out) {
	if (!b || !out) return fail(XFEM_EINVAL, "null argument");
	uint32_t ncl = 0;
	for (auto& x : b->bodies) ncl += x.sched.nclusters;
	*out = {(uint32_t)b->bodies.size(), b->nverts, b->ntets, ncl, b->ncolours, b->nisolated,
	        b->nchunks, b->nrows, (uint32_t)b->cfg.block, (uint32_t)b->cfg.blocks, (uint32_t)b->cfg.sync_mode,
	        b->opt.cluster_mode == 1 ? 1u : 2u, b->max_deps, b->ctx.nbricks, b->device_bytes};
	return XFEM_OK;
}

int xfem_set_settings(xfem_body* h, uint32_t body, const xfem_settings* s) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!s) return fail(XFEM_EINVAL, "null settings");
	int rc = validate_settings(*s);
	if (rc) return rc;
	const uint32_t energy = (s->flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK;
	if (quadratic_type(s->flags) != (b->el == kElT10 || b->el == kElH27 || b->el == kElQMixed))
		return fail(XFEM_EUNSUPPORTED, "switching between linear and quadratic elements (flags bits 0-3) needs a new handle");
	if ((model_of(energy) == kModelRing) != h->ring_mode)
		return fail(XFEM_EUNSUPPORTED, "switching between the continuous-pressure models (energy 8-10) and the "
		                               "element models needs a new handle (their schedules differ)");
	const bool material = s->compliance != b->settings.compliance;
	b->settings = *s;
	XCUDA(cudaSetDevice(h->device));
	BodyParams p = make_params(*s);
	set_counts(p, *b);
	XCUDA(cudaMemcpyAsync(h->params.p + body, &p, sizeof(p), cudaMemcpyHostToDevice, h->stream));
	// Settings::tickId: the handle's substep counter continues from here
	XCUDA(cudaMemcpyAsync(h->tick.p, &s->tick_id, 4, cudaMemcpyHostToDevice, h->stream));
	const std::vector<uint8_t> pt = pass_table(h->bodies, h->ncolours);
	XCUDA(cudaMemcpyAsync(h->pass_on.p, pt.data(), pt.size(), cudaMemcpyHostToDevice, h->stream));
	XCUDA(cudaStreamSynchronize(h->stream));
	const uint32_t kinds = damp_kinds_of(h->bodies);
	const bool ext = ext_any_of(h->bodies);
	const uint32_t nvol = nvol_of(h->bodies);
	if (kinds != h->ctx.damp_kinds || ext != h->cfg.ext || nvol != h->ctx.nvol) {
		h->ctx.damp_kinds = kinds;
		h->ctx.ext = ext ? 1u : 0u;
		h->ctx.nvol = nvol;
		h->cfg.ext = ext;
		if (h->graph) {  // the captured launches follow the old sweeps
			cudaGraphExecDestroy(h->graph);
			h->graph = nullptr;
		}
		if (h->tuned && (h->cfg.sync_mode == 1 || h->cfg.sync_mode == 3)) {
			// the other instantiation may fit another grid
			int blocks = 0;
			if (persistent_grid(h->cfg, &blocks) == 0) h->cfg.blocks = blocks;
		}
	}
	if (h->ring_mode) h->ctx.ext = ring_damp_of(h->bodies) ? 1u : 0u;
	const float4* rt_before = h->ctx.right_target;
	if (const int rr = update_right_targets(h)) return rr;
	if (h->graph && h->ctx.right_target != rt_before) {  // the captured launches hold the old pointer
		cudaGraphExecDestroy(h->graph);
		h->graph = nullptr;
	}
	if (material && b->tet_mu.empty() && !h->el_mode) return update_material(h, *b);
	return XFEM_OK;
}

int xfem_set_lock_mask(xfem_body* h, uint32_t body, const uint8_t* mask) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!mask) return fail(XFEM_EINVAL, "null mask");
	XCUDA(cudaSetDevice(h->device));
	std::vector<float4> vv(2 * (size_t)b->nv);
	XCUDA(cudaMemcpyAsync(vv.data(), h->vert.p + 2 * (size_t)b->vbase, vv.size() * sizeof(float4), cudaMemcpyDeviceToHost,
	                      h->stream));
	XCUDA(cudaStreamSynchronize(h->stream));
	for (uint32_t v = 0; v < b->nv; v++) {
		const uint32_t dv = b->sched.vert_rank[v];
		uint32_t bits = __builtin_bit_cast(uint32_t, vv[2 * (size_t)dv + 1].w);
		bits = mask[v] ? (bits | kFlagLocked) : (bits & ~kFlagLocked);
		vv[2 * (size_t)dv + 1].w = __builtin_bit_cast(float, bits);
	}
	XCUDA(cudaMemcpyAsync(h->vert.p + 2 * (size_t)b->vbase, vv.data(), vv.size() * sizeof(float4), cudaMemcpyHostToDevice,
	                      h->stream));
	XCUDA(cudaStreamSynchronize(h->stream));
	return XFEM_OK;
}

int xfem_set_tet_mu(xfem_body* h, uint32_t body, const float* mu) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (h->ring_mode && mu)
		return fail(XFEM_EUNSUPPORTED, "the continuous-pressure models (energy 8-10) take the body's material only");
	if (h->el_mode) return fail(XFEM_EUNSUPPORTED, "hex, T10 and H27 meshes take the body's material only");
	if (mu) {
		for (uint32_t t = 0; t < b->nt; t++)
			if (!(mu[t] > 0.0f) || !isfinite(mu[t])) return fail(XFEM_EINVAL, "tet mu must be finite and > 0");
		b->tet_mu.assign(mu, mu + b->nt);
	} else {
		b->tet_mu.clear();
	}
	XCUDA(cudaSetDevice(h->device));
	return update_material(h, *b);
}

int xfem_substep(xfem_body* b, float dt) { return step(b, 1, dt); }

int xfem_step_frames(xfem_body* b, uint32_t frames, uint32_t substeps, float dt) {
	const uint64_t n = (uint64_t)frames * substeps;
	if (n > 0xffffffffull) return fail(XFEM_EINVAL, "too many substeps in one call");
	return step(b, (uint32_t)n, dt);
}

int xfem_step_frames_noalloc(xfem_body* h, uint32_t frames, uint32_t substeps, float dt) {
	if (!h) return fail(XFEM_EINVAL, "null handle");
	if (!(dt > 0.0f) || !isfinite(dt)) return fail(XFEM_EINVAL, "dt must be > 0");
	const uint64_t n = (uint64_t)frames * substeps;
	if (n == 0) return XFEM_OK;
	if (n > 0xffffffffull) return fail(XFEM_EINVAL, "too many substeps in one call");
	if (h->ring_mode)
		return fail(XFEM_EUNSUPPORTED, "the continuous-pressure models (energy 8-10) have no allocation-free launch");
	XCUDA(cudaSetDevice(h->device));
	WaitMissScope miss(h);
	if (h->el_mode) {
		// the element launches use the handle's own scratch and allocate nothing
		const int rc = launch_mode(h, h->ctx, (uint32_t)n, dt);
		return rc ? rc : check_device_error(h);
	}
	int dev_err = 0;
	const int e = launch_substeps_noalloc(h->ctx, h->cfg.block, h->cfg.warp_smem, h->cfg.lambdas, (uint32_t)n, dt,
	                                      h->stream, h->device, &dev_err);
	if (e == kNoAllocTooLong)
		return fail(XFEM_ELIMIT, "one call's grid-barrier arrivals (substeps x passes per substep x persistent "
		                         "blocks) must stay below 2^31; split the call");
	if (e) return fail(XFEM_ECUDA, std::string("allocation-free launch: ") + cudaGetErrorString((cudaError_t)e));
	if (dev_err) return device_error(dev_err);
	return XFEM_OK;
}

int xfem_test_hook(xfem_body* b, uint32_t hook, uint32_t value) {
	if (hook == XFEM_HOOK_FAIL_ALLOC) {
		g_fail_alloc_in.store(value);
		return XFEM_OK;
	}
	if (!b) return fail(XFEM_EINVAL, "null handle");
	switch (hook) {
	case XFEM_HOOK_MISSING_ARRIVAL: b->hook_wait_miss = value; return XFEM_OK;
	case XFEM_HOOK_BARRIER_BASE:
		if (value > 1u) return fail(XFEM_EINVAL, "XFEM_HOOK_BARRIER_BASE takes 0 or 1");
		b->ctx.bar_base = value ? 0xffffffffu : 0u;
		if (b->graph) {  // no grid barrier there, but keep the captured context current
			cudaGraphExecDestroy(b->graph);
			b->graph = nullptr;
		}
		return XFEM_OK;
	default: return fail(XFEM_EINVAL, "unknown test hook " + std::to_string(hook));
	}
}

int xfem_synchronize(xfem_body* b) {
	if (!b) return fail(XFEM_EINVAL, "null handle");
	XCUDA(cudaSetDevice(b->device));
	return check_device_error(b);
}

int xfem_get_positions(xfem_body* b, uint32_t body, float* out) { return get_xyz(b, body, 0, out); }
int xfem_set_positions(xfem_body* b, uint32_t body, const float* in) { return set_xyz(b, body, 0, in); }
int xfem_get_velocities(xfem_body* b, uint32_t body, float* out) { return get_xyz(b, body, 1, out); }
int xfem_set_velocities(xfem_body* b, uint32_t body, const float* in) { return set_xyz(b, body, 1, in); }
int xfem_set_state(xfem_body* h, uint32_t body, const float* xyz, const float* vel) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!xyz || !vel) return fail(XFEM_EINVAL, "null input");
	XCUDA(cudaSetDevice(h->device));
	int rc = scatter_xyz(h, b, 0, xyz);
	if (!rc) rc = scatter_xyz(h, b, 1, vel);
	return rc ? rc : check_device_error(h);  // one synchronisation for both
}
int xfem_get_inverse_masses(xfem_body* b, uint32_t body, float* out) { return get_xyz(b, body, 2, out); }

int xfem_get_contacts(xfem_body* h, uint32_t body, uint8_t* out) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!out) return fail(XFEM_EINVAL, "null output");
	std::vector<float> f(b->nv);
	const int rc = get_xyz(h, body, 3, f.data());
	if (rc) return rc;
	for (uint32_t v = 0; v < b->nv; v++) out[v] = f[v] != 0.0f;
	return XFEM_OK;
}

int xfem_get_lambdas(xfem_body* h, uint32_t body, float* out) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!out) return fail(XFEM_EINVAL, "null output");
	if (h->el_mode) return fail(XFEM_EUNSUPPORTED, "hex, T10 and H27 meshes keep no multipliers");
	if (!h->tlam.p) return fail(XFEM_EINVAL, "create the handle with keep_lambdas = 1");
	XCUDA(cudaSetDevice(h->device));
	std::vector<float2> all(h->tlam.n);
	XCUDA(cudaMemcpyAsync(all.data(), h->tlam.p, all.size() * sizeof(float2), cudaMemcpyDeviceToHost, h->stream));
	const int rc = check_device_error(h);
	if (rc) return rc;
	for (uint32_t t = 0; t < b->nt; t++) {
		out[2 * (size_t)t] = all[b->tet_slot[t]].x;
		out[2 * (size_t)t + 1] = all[b->tet_slot[t]].y;
	}
	return XFEM_OK;
}

// TCalculateElementVolume (XPBDFEM/Fem.cpp:1046-1064) summed over a body's
// linear hexes at positions x (caller order): rest volume times the weighted
// det F over the 2x2x2 points, in double.
static double hex_volume(const BodyHost& b, const float* x) {
	double v = 0.0;
	for (uint32_t hx = 0; hx < b.nh; hx++) {
		const uint32_t* is = &b.elems[8 * (size_t)hx];
		const float* e = &b.eep[(size_t)rest::kHexRec * hx];
		double P[7][3];
		for (int i = 0; i < 7; i++)
			for (int k = 0; k < 3; k++) P[i][k] = (double)x[3 * (size_t)is[i] + k] - (double)x[3 * (size_t)is[7] + k];
		double scale = 0.0;
		for (int p = 0; p < 8; p++) {
			double Dm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, F[3][3];
			for (int n = 0; n < 7; n++)
				for (int c = 0; c < 3; c++)
					for (int r = 0; r < 3; r++) Dm[c][r] += (double)rest::hex_g8(p, n, r) * P[n][c];
			const float* ji = e + rest::kHexJH + 9 * p;
			for (int c = 0; c < 3; c++)
				for (int r = 0; r < 3; r++) F[c][r] = ji[r] * Dm[c][0] + ji[3 + r] * Dm[c][1] + ji[6 + r] * Dm[c][2];
			const double det = F[0][0] * (F[1][1] * F[2][2] - F[2][1] * F[1][2]) -
			                   F[1][0] * (F[0][1] * F[2][2] - F[2][1] * F[0][2]) +
			                   F[2][0] * (F[0][1] * F[1][2] - F[1][1] * F[0][2]);
			scale += (double)e[rest::kHexWH + p] * det;
		}
		v += (double)e[rest::kHexVol] * scale;
	}
	return v;
}

static int tet_volume(xfem_body* h, uint32_t body, double* out);

// TCalculateElementVolume (XPBDFEM/Fem.cpp:1046-1064) summed over n H27s:
// rest volume times the weighted det F over the 3x3x3 points, in double.
static double h27_volume(const float* x, const uint32_t* elems, const float* eep, uint32_t n) {
	const rest::H27Tables& tb = rest::h27_tables();
	double v = 0.0;
	for (uint32_t q = 0; q < n; q++) {
		const uint32_t* is = elems + 27 * (size_t)q;
		const float* e = eep + (size_t)rest::kH27Rec * q;
		double P[26][3];
		for (int i = 0; i < 26; i++)
			for (int k = 0; k < 3; k++) P[i][k] = (double)x[3 * (size_t)is[i] + k] - (double)x[3 * (size_t)is[26] + k];
		double scale = 0.0;
		for (int p = 0; p < 27; p++) {
			double Dm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, F[3][3];
			for (int nn = 0; nn < 26; nn++)
				for (int c = 0; c < 3; c++)
					for (int r = 0; r < 3; r++) Dm[c][r] += (double)tb.g27[p][nn][r] * P[nn][c];
			const float* ji = e + rest::kH27JH + 9 * p;
			for (int c = 0; c < 3; c++)
				for (int r = 0; r < 3; r++) F[c][r] = ji[r] * Dm[c][0] + ji[3 + r] * Dm[c][1] + ji[6 + r] * Dm[c][2];
			const double det = F[0][0] * (F[1][1] * F[2][2] - F[2][1] * F[1][2]) -
			                   F[1][0] * (F[0][1] * F[2][2] - F[2][1] * F[0][2]) +
			                   F[2][0] * (F[0][1] * F[1][2] - F[1][1] * F[0][2]);
			scale += (double)e[rest::kH27WH + p] * det;
		}
		v += (double)e[rest::kH27Vol] * scale;
	}
	return v;
}

// The same over n T10s: rest volume times the mean det F over the 4 points.
static double t10_volume(const float* x, const uint32_t* elems, const float* eep, uint32_t n) {
	double v = 0.0;
	for (uint32_t q = 0; q < n; q++) {
		const uint32_t* is = elems + 10 * (size_t)q;
		const float* e = eep + (size_t)rest::kT10Rec * q;
		double P[9][3];
		for (int i = 0; i < 9; i++)
			for (int k = 0; k < 3; k++) P[i][k] = (double)x[3 * (size_t)is[i] + k] - (double)x[3 * (size_t)is[9] + k];
		double scale = 0.0;
		for (int p = 0; p < 4; p++) {
			double Dm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, F[3][3];
			for (int nn = 0; nn < 9; nn++)
				for (int c = 0; c < 3; c++)
					for (int r = 0; r < 3; r++) Dm[c][r] += (double)rest::t10_tables().g4[p][nn][r] * P[nn][c];
			const float* qi = e + rest::kT10Qi;
			for (int c = 0; c < 3; c++)
				for (int r = 0; r < 3; r++) F[c][r] = qi[r] * Dm[c][0] + qi[3 + r] * Dm[c][1] + qi[6 + r] * Dm[c][2];
			const double det = F[0][0] * (F[1][1] * F[2][2] - F[2][1] * F[1][2]) -
			                   F[1][0] * (F[0][1] * F[2][2] - F[2][1] * F[0][2]) +
			                   F[2][0] * (F[0][1] * F[1][2] - F[1][1] * F[0][2]);
			scale += 0.25 * det;
		}
		v += (double)e[rest::kT10Vol] * scale;
	}
	return v;
}

int xfem_calculate_volume(xfem_body* h, uint32_t body, double* out) {
	BodyHost* b = body_of(h, body);
	if (!b) return XFEM_EINVAL;
	if (!out) return fail(XFEM_EINVAL, "null output");
	XCUDA(cudaSetDevice(h->device));
	if (b->el == kElH27 || b->el == kElT10 || b->el == kElQMixed) {
		std::vector<float> x(3 * (size_t)b->nv);
		const int rc = get_xyz(h, body, 0, x.data());
		if (rc) return rc;
		// a mixed quadratic mesh: its T10s, then its H27s (XPBDFEM/Geo.cpp:1048-1053)
		*out = b->el == kElH27   ? h27_volume(x.data(), b->elems.data(), b->eep.data(), b->nh)
		       : b->el == kElT10 ? t10_volume(x.data(), b->elems.data(), b->eep.data(), b->nh)
		                         : t10_volume(x.data(), b->qt.data(), b->qtep.data(), b->nqt) +
		                               h27_volume(x.data(), b->elems.data(), b->eep.data(), b->nh);
		return XFEM_OK;
	}
	if (b->el == kElHexes || b->el == kElMixed) {
		std::vector<float> x(3 * (size_t)b->nv);
		const int rc = get_xyz(h, body, 0, x.data());
		if (rc) return rc;
		const double vh = hex_volume(*b, x.data());
		if (b->el == kElHexes) {
			*out = vh;
			return XFEM_OK;
		}
		// a mixed mesh: the tets' volumes (below) plus the hexes'
		// (XPBDFEM/Geo.cpp:827-832 sums every element of the stream)
		double vt = 0.0;
		const int rt = tet_volume(h, body, &vt);
		if (rt) return rt;
		*out = vt + vh;
		return XFEM_OK;
	}
	return tet_volume(h, body, out);
}

// The tets' part of xfem_calculate_volume, summed on the device in double.
static int tet_volume(xfem_body* h, uint32_t body, double* out) {
	const BodyHost* b = &h->bodies[body];
	size_t tb = 0;
	for (uint32_t i = 0; i < body; i++) tb += 4 * (size_t)h->bodies[i].nt;
	const int e = launch_volume(h->vert.p, h->tets_dev.p + tb, b->nt, h->vol.p, h->stream);
	if (e) return fail(XFEM_ECUDA, "volume launch failed");
	XCUDA(cudaMemcpyAsync(out, h->vol.p, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
	return check_device_error(h);
}

int xfem_get_rest_state(const xfem_body* h, uint32_t body, float* out_ep17, float* out_w) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el && b.el != kElMixed)
		return fail(XFEM_EUNSUPPORTED, "an element body: use xfem_get_hex_rest_state, _t10_ or _h27_");
	if (out_ep17) memcpy(out_ep17, b.ep.data(), b.ep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	return XFEM_OK;
}

int xfem_get_schedule(const xfem_body* h, uint32_t body, uint32_t* vert_rank, uint32_t* tet_order, uint32_t* colour_begin,
                      uint32_t* ncolours) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el) return fail(XFEM_EUNSUPPORTED, "an element body: use xfem_get_hex_schedule, _t10_ or _h27_");
	const Schedule& s = b.sched;
	if (vert_rank) memcpy(vert_rank, s.vert_rank.data(), s.vert_rank.size() * 4);
	if (ncolours) *ncolours = s.ncolours;
	uint32_t o = 0;
	for (uint32_t c = 0; c < s.ncolours; c++) {
		if (colour_begin) colour_begin[c] = o;
		for (uint32_t i = s.colour_cl_begin[c]; i < s.colour_cl_begin[c + 1]; i++) {
			const uint32_t k = s.colour_cl[i];
			for (uint32_t q = s.cl_begin[k]; q < s.cl_begin[k + 1]; q++) {
				if (tet_order) tet_order[o] = s.cl_tets[q];
				o++;
			}
		}
	}
	if (colour_begin) colour_begin[s.ncolours] = o;
	return XFEM_OK;
}

int xfem_body_counts(const xfem_body* h, uint32_t body, uint32_t* nverts, uint32_t* ntets) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	if (nverts) *nverts = h->bodies[body].nv;
	if (ntets) *ntets = h->bodies[body].nt;
	return XFEM_OK;
}

int xfem_compute_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                            uint32_t idx_data_count, float density, float* out_ep17, float* out_w, uint8_t* out_flags) {
	BodyHost b;
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, density};
	const int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el) return fail(XFEM_EUNSUPPORTED, "a hex mesh: use xfem_compute_hex_rest_state");
	host_rest(m, b);
	if (out_ep17) memcpy(out_ep17, b.ep.data(), b.ep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	if (out_flags) memcpy(out_flags, b.vflags.data(), b.vflags.size());
	return XFEM_OK;
}

int xfem_compute_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                          uint32_t idx_data_count, uint32_t cluster_mode, uint32_t no_morton, uint32_t* vert_rank,
                          uint32_t* tet_order, uint32_t* colour_begin, uint32_t* ncolours, uint32_t* nclusters) {
	if (cluster_mode > 2) return fail(XFEM_EINVAL, "cluster_mode must be 0, 1 or 2");
	xfem_body tmp;
	tmp.bodies.resize(1);
	BodyHost& b = tmp.bodies[0];
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, 1.0f};
	int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el) return fail(XFEM_EUNSUPPORTED, "a hex mesh: use xfem_compute_hex_schedule");
	if (build_schedule(b.nodes.data(), b.nv, b.tets.data(), b.nt, cluster_mode == 1 ? 0u : 1u, no_morton ? 0u : 1u, b.sched))
		return fail(XFEM_ELIMIT, "colour schedule limit exceeded");
	if (nclusters) *nclusters = b.sched.nclusters;
	return xfem_get_schedule(&tmp, 0, vert_rank, tet_order, colour_begin, ncolours);
}

static int ring_schedule_out(const RingSchedule& rs, uint32_t* vert_order, uint32_t* colour_begin, uint32_t* ncolours) {
	if (vert_order) memcpy(vert_order, rs.order.data(), rs.order.size() * 4);
	if (colour_begin) memcpy(colour_begin, rs.colour_begin.data(), rs.colour_begin.size() * 4);
	if (ncolours) *ncolours = rs.ncolours;
	return XFEM_OK;
}

int xfem_get_ring_schedule(const xfem_body* h, uint32_t body, uint32_t* vert_order, uint32_t* colour_begin,
                           uint32_t* ncolours) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	if (!h->ring_mode) return fail(XFEM_EUNSUPPORTED, "the handle runs no continuous-pressure model");
	return ring_schedule_out(h->bodies[body].rings, vert_order, colour_begin, ncolours);
}

int xfem_compute_ring_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                               uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_order, uint32_t* colour_begin,
                               uint32_t* ncolours) {
	BodyHost b;
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, 1.0f};
	int rc = prepare_mesh(m, b);
	if (rc) return rc;
	// a tet stream (tag 4) or a hex stream (tag 8): rings over its elements
	const bool hex = b.el == kElHexes;
	const uint32_t* el = hex ? b.elems.data() : b.tets.data();
	std::vector<uint32_t> off, lst;
	incidence(el, b.nv, hex ? b.nh : b.nt, off, lst, hex ? 8u : 4u);
	vertex_ranks(b.nodes.data(), b.nv, no_morton ? 0u : 1u, b.sched);
	rc = build_ring_schedule(el, b.nv, off.data(), lst.data(), b.sched.vert_rank.data(), b.rings, hex ? 8u : 4u);
	if (rc == -2)
		return fail(XFEM_ELIMIT, hex ? "a vertex one-ring has more than 16 hexes or 32 vertices"
		                             : "a vertex one-ring has more than 64 tets or 32 vertices");
	if (rc) return fail(XFEM_ELIMIT, "ring colour limit exceeded");
	return ring_schedule_out(b.rings, vert_order, colour_begin, ncolours);
}

int xfem_body_hex_count(const xfem_body* h, uint32_t body, uint32_t* nhexes) {
	if (!h || body >= h->bodies.size() || !nhexes) return fail(XFEM_EINVAL, "bad handle, body index or output");
	*nhexes = h->bodies[body].nh;
	return XFEM_OK;
}

int xfem_get_hex_rest_state(const xfem_body* h, uint32_t body, float* out_ep120, float* out_w) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElHexes && b.el != kElMixed) return fail(XFEM_EUNSUPPORTED, "not a hex body");
	if (out_ep120) memcpy(out_ep120, b.eep.data(), b.eep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	return XFEM_OK;
}

static int elem_schedule_out(const BodyHost& b, uint32_t* vert_rank, uint32_t* order, uint32_t* colour_begin,
                             uint32_t* ncolours, bool tsched = false) {
	const ElemSchedule& es = tsched ? b.tsched : b.esched;
	if (vert_rank) memcpy(vert_rank, b.sched.vert_rank.data(), b.sched.vert_rank.size() * 4);
	if (order) memcpy(order, es.order.data(), es.order.size() * 4);
	if (colour_begin) memcpy(colour_begin, es.colour_begin.data(), es.colour_begin.size() * 4);
	if (ncolours) *ncolours = es.ncolours;
	return XFEM_OK;
}

int xfem_get_hex_schedule(const xfem_body* h, uint32_t body, uint32_t* vert_rank, uint32_t* hex_order,
                          uint32_t* colour_begin, uint32_t* ncolours) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElHexes && b.el != kElMixed) return fail(XFEM_EUNSUPPORTED, "not a hex body");
	return elem_schedule_out(b, vert_rank, hex_order, colour_begin, ncolours);
}

int xfem_get_mixed_tet_schedule(const xfem_body* h, uint32_t body, uint32_t* tet_order, uint32_t* colour_begin,
                                uint32_t* ncolours) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElMixed) return fail(XFEM_EUNSUPPORTED, "not a mesh mixing tets and hexes");
	if (tet_order) memcpy(tet_order, b.tsched.order.data(), b.tsched.order.size() * 4);
	if (colour_begin) memcpy(colour_begin, b.tsched.colour_begin.data(), b.tsched.colour_begin.size() * 4);
	if (ncolours) *ncolours = b.tsched.ncolours;
	return XFEM_OK;
}

int xfem_compute_mixed_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                  uint32_t idx_data_count, float density, float* out_ep17, float* out_ep120, float* out_w,
                                  uint8_t* out_flags) {
	BodyHost b;
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, density};
	const int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el != kElMixed) return fail(XFEM_EINVAL, "not a mesh mixing tets and hexes");
	host_rest(m, b);
	if (out_ep17) memcpy(out_ep17, b.ep.data(), b.ep.size() * sizeof(float));
	if (out_ep120) memcpy(out_ep120, b.eep.data(), b.eep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	if (out_flags) memcpy(out_flags, b.vflags.data(), b.vflags.size());
	return XFEM_OK;
}

int xfem_compute_mixed_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* tet_order,
                                uint32_t* tet_colour_begin, uint32_t* tet_ncolours, uint32_t* hex_order,
                                uint32_t* hex_colour_begin, uint32_t* hex_ncolours) {
	BodyHost b;
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, 1.0f};
	const int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el != kElMixed) return fail(XFEM_EINVAL, "not a mesh mixing tets and hexes");
	const uint32_t morton = no_morton ? 0u : 1u;
	vertex_ranks(b.nodes.data(), b.nv, morton, b.sched);
	if (elem_schedule(b.nodes.data(), b.nv, b.elems.data(), b.nh, 8, morton, b.esched) ||
	    elem_schedule(b.nodes.data(), b.nv, b.tets.data(), b.nt, 4, morton, b.tsched))
		return fail(XFEM_ELIMIT, "the element colouring needs more than " + std::to_string(kMaxElemColours) + " colours");
	if (tet_order) memcpy(tet_order, b.tsched.order.data(), b.tsched.order.size() * 4);
	if (tet_colour_begin) memcpy(tet_colour_begin, b.tsched.colour_begin.data(), b.tsched.colour_begin.size() * 4);
	if (tet_ncolours) *tet_ncolours = b.tsched.ncolours;
	return elem_schedule_out(b, vert_rank, hex_order, hex_colour_begin, hex_ncolours);
}

int xfem_compute_hex_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, float density, float* out_ep120, float* out_w,
                                uint8_t* out_flags) {
	BodyHost b;
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, density};
	const int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el != kElHexes) return fail(XFEM_EINVAL, "not a hex mesh");
	host_rest(m, b);
	if (out_ep120) memcpy(out_ep120, b.eep.data(), b.eep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	if (out_flags) memcpy(out_flags, b.vflags.data(), b.vflags.size());
	return XFEM_OK;
}

int xfem_compute_hex_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                              uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* hex_order,
                              uint32_t* colour_begin, uint32_t* ncolours) {
	BodyHost b;
	const xfem_mesh m = {node_data, node_data_count, idx_data, idx_data_count, 1.0f};
	const int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el != kElHexes) return fail(XFEM_EINVAL, "not a hex mesh");
	vertex_ranks(b.nodes.data(), b.nv, no_morton ? 0u : 1u, b.sched);
	if (elem_schedule(b.nodes.data(), b.nv, b.elems.data(), b.nh, 8, no_morton ? 0u : 1u, b.esched))
		return fail(XFEM_ELIMIT, "the hex colouring needs more than " + std::to_string(kMaxElemColours) + " colours");
	return elem_schedule_out(b, vert_rank, hex_order, colour_begin, ncolours);
}

int xfem_body_t10_count(const xfem_body* h, uint32_t body, uint32_t* nt10, uint32_t* nedges) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElT10 && b.el != kElQMixed) return fail(XFEM_EUNSUPPORTED, "not a T10 body");
	if (nt10) *nt10 = b.el == kElQMixed ? b.nqt : b.nh;
	if (nedges) *nedges = (uint32_t)(b.edges.size() / 2);
	return XFEM_OK;
}

int xfem_get_t10_rest_state(const xfem_body* h, uint32_t body, float* out_ep56, float* out_w, uint32_t* out_t10,
                            uint32_t* out_edges) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElT10 && b.el != kElQMixed) return fail(XFEM_EUNSUPPORTED, "not a T10 body");
	const std::vector<float>& ep = b.el == kElQMixed ? b.qtep : b.eep;
	const std::vector<uint32_t>& t10 = b.el == kElQMixed ? b.qt : b.elems;
	if (out_ep56) memcpy(out_ep56, ep.data(), ep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	if (out_t10) memcpy(out_t10, t10.data(), t10.size() * 4);
	if (out_edges) memcpy(out_edges, b.edges.data(), b.edges.size() * 4);
	return XFEM_OK;
}

int xfem_get_t10_schedule(const xfem_body* h, uint32_t body, uint32_t* vert_rank, uint32_t* t10_order,
                          uint32_t* colour_begin, uint32_t* ncolours) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElT10 && b.el != kElQMixed) return fail(XFEM_EUNSUPPORTED, "not a T10 body");
	return elem_schedule_out(b, vert_rank, t10_order, colour_begin, ncolours, b.el == kElQMixed);
}

int xfem_compute_t10_edges(const uint32_t* idx_data, uint32_t idx_data_count, uint32_t* out_edges, uint32_t* out_t10,
                           uint32_t* out_nedges) {
	if (!idx_data) return fail(XFEM_EINVAL, "null index stream");
	BodyHost b;
	uint32_t nv = 0;
	if (parse_tets(idx_data, idx_data_count, b.tets, nv)) return fail(XFEM_EINVAL, "not a tet index stream (tag 4)");
	std::vector<uint32_t> edges, t10;
	tet_edges(b.tets.data(), (uint32_t)(b.tets.size() / 4), nv, edges, t10);
	if (out_edges) memcpy(out_edges, edges.data(), edges.size() * 4);
	if (out_t10) memcpy(out_t10, t10.data(), t10.size() * 4);
	if (out_nedges) *out_nedges = (uint32_t)(edges.size() / 2);
	return XFEM_OK;
}

// A tet mesh read as T10s (prepare_mesh then prepare_t10).
static int t10_mesh(const xfem_mesh& m, BodyHost& b, std::vector<double>* X) {
	const int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el != kElTets) return fail(XFEM_EINVAL, "not a tet mesh (tag 4)");
	prepare_t10(m, b, X);
	return XFEM_OK;
}

int xfem_compute_t10_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, float density, double* out_x, float* out_ep56, float* out_w,
                                uint8_t* out_flags) {
	BodyHost b;
	std::vector<double> X;
	const int rc = t10_mesh({node_data, node_data_count, idx_data, idx_data_count, density}, b, &X);
	if (rc) return rc;
	if (out_x) memcpy(out_x, X.data(), X.size() * sizeof(double));
	if (out_ep56) memcpy(out_ep56, b.eep.data(), b.eep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	if (out_flags) memcpy(out_flags, b.vflags.data(), b.vflags.size());
	return XFEM_OK;
}

int xfem_body_h27_count(const xfem_body* h, uint32_t body, uint32_t* nh27, uint32_t* nedges, uint32_t* nquads) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElH27 && b.el != kElQMixed) return fail(XFEM_EUNSUPPORTED, "not an H27 body");
	if (nh27) *nh27 = b.nh;
	if (nedges) *nedges = (uint32_t)(b.edges.size() / 2);
	if (nquads) *nquads = (uint32_t)(b.quads.size() / 4);
	return XFEM_OK;
}

int xfem_get_h27_rest_state(const xfem_body* h, uint32_t body, float* out_ep703, float* out_w, uint32_t* out_h27) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElH27 && b.el != kElQMixed) return fail(XFEM_EUNSUPPORTED, "not an H27 body");
	if (out_ep703) memcpy(out_ep703, b.eep.data(), b.eep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	if (out_h27) memcpy(out_h27, b.elems.data(), b.elems.size() * 4);
	return XFEM_OK;
}

int xfem_get_h27_schedule(const xfem_body* h, uint32_t body, uint32_t* vert_rank, uint32_t* h27_order,
                          uint32_t* colour_begin, uint32_t* ncolours) {
	if (!h || body >= h->bodies.size()) return fail(XFEM_EINVAL, "bad handle or body index");
	const BodyHost& b = h->bodies[body];
	if (b.el != kElH27 && b.el != kElQMixed) return fail(XFEM_EUNSUPPORTED, "not an H27 body");
	return elem_schedule_out(b, vert_rank, h27_order, colour_begin, ncolours);
}

// A hex mesh read as H27s (prepare_mesh then prepare_h27).
static int h27_mesh(const xfem_mesh& m, BodyHost& b, std::vector<double>* X) {
	const int rc = prepare_mesh(m, b);
	if (rc) return rc;
	if (b.el != kElHexes) return fail(XFEM_EINVAL, "not a hex mesh (tag 8)");
	prepare_h27(m, b, X);
	return XFEM_OK;
}

int xfem_compute_h27_mesh(const uint32_t* idx_data, uint32_t idx_data_count, uint32_t* out_edges, uint32_t* out_quads,
                          uint32_t* out_h27, uint32_t* out_nedges, uint32_t* out_nquads) {
	if (!idx_data) return fail(XFEM_EINVAL, "null index stream");
	std::vector<uint32_t> hexes, edges, quads, h27;
	uint32_t nv = 0;
	if (parse_hexes(idx_data, idx_data_count, hexes, nv)) return fail(XFEM_EINVAL, "not a hex index stream (tag 8)");
	hex_edges_quads(hexes.data(), (uint32_t)(hexes.size() / 8), nv, edges, quads, h27);
	if (out_edges) memcpy(out_edges, edges.data(), edges.size() * 4);
	if (out_quads) memcpy(out_quads, quads.data(), quads.size() * 4);
	if (out_h27) memcpy(out_h27, h27.data(), h27.size() * 4);
	if (out_nedges) *out_nedges = (uint32_t)(edges.size() / 2);
	if (out_nquads) *out_nquads = (uint32_t)(quads.size() / 4);
	return XFEM_OK;
}

int xfem_compute_h27_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, float density, double* out_x, float* out_ep703,
                                float* out_w, uint8_t* out_flags) {
	BodyHost b;
	std::vector<double> X;
	const int rc = h27_mesh({node_data, node_data_count, idx_data, idx_data_count, density}, b, &X);
	if (rc) return rc;
	if (out_x) memcpy(out_x, X.data(), X.size() * sizeof(double));
	if (out_ep703) memcpy(out_ep703, b.eep.data(), b.eep.size() * sizeof(float));
	if (out_w) memcpy(out_w, b.w0.data(), b.w0.size() * sizeof(float));
	if (out_flags) memcpy(out_flags, b.vflags.data(), b.vflags.size());
	return XFEM_OK;
}

int xfem_compute_h27_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                              uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* h27_order,
                              uint32_t* colour_begin, uint32_t* ncolours) {
	BodyHost b;
	const int rc = h27_mesh({node_data, node_data_count, idx_data, idx_data_count, 1.0f}, b, nullptr);
	if (rc) return rc;
	vertex_ranks(b.nodes.data(), b.nv, no_morton ? 0u : 1u, b.sched);
	if (elem_schedule(b.nodes.data(), b.nv, b.elems.data(), b.nh, 27, no_morton ? 0u : 1u, b.esched))
		return fail(XFEM_ELIMIT, "the H27 colouring needs more than " + std::to_string(kMaxElemColours) + " colours");
	return elem_schedule_out(b, vert_rank, h27_order, colour_begin, ncolours);
}

int xfem_compute_t10_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                              uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* t10_order,
                              uint32_t* colour_begin, uint32_t* ncolours) {
	BodyHost b;
	const int rc = t10_mesh({node_data, node_data_count, idx_data, idx_data_count, 1.0f}, b, nullptr);
	if (rc) return rc;
	vertex_ranks(b.nodes.data(), b.nv, no_morton ? 0u : 1u, b.sched);
	if (elem_schedule(b.nodes.data(), b.nv, b.elems.data(), b.nh, 10, no_morton ? 0u : 1u, b.esched))
		return fail(XFEM_ELIMIT, "the T10 colouring needs more than " + std::to_string(kMaxElemColours) + " colours");
	return elem_schedule_out(b, vert_rank, t10_order, colour_begin, ncolours);
}

int xfem_generate_hex_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                            float wonkiness, float* out_nodes, uint32_t* out_idx) {
	if (!out_nodes || !out_idx) return fail(XFEM_EINVAL, "null output");
	gen_hex_block(W, H, D, sx, sy, sz, pattern, wonkiness, out_nodes, out_idx);
	return XFEM_OK;
}

int xfem_pbd_damping_coefficients(float pbd_damping, float substep_dt, float spacing, float* out2) {
	if (!out2) return fail(XFEM_EINVAL, "null output");
	// XPBDFEM/Demo.cpp:53-61 (AmortizationPeriod = 8)
	const float tc = 1.0f - powf(1.0f - pbd_damping, 1000.0f * substep_dt);
	const float atc = 1.0f - powf(1.0f - pbd_damping, 1000.0f * 8.0f * substep_dt);
	out2[0] = tc * 6.0f * spacing * spacing;
	out2[1] = atc * 6.0f * spacing * spacing;
	return XFEM_OK;
}

float xfem_time_corrected_drag(float drag, float substep_dt) {
	return 1.0f - powf(1.0f - drag, 1000.0f * substep_dt);
}

int xfem_generate_tet_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                            float wonkiness, float* nodes, uint32_t* idx) {
	if (!nodes || !idx) return fail(XFEM_EINVAL, "null output");
	gen_tet_block(W, H, D, sx, sy, sz, pattern, wonkiness, nodes, idx);
	return XFEM_OK;
}

void* xfem_alloc_host(size_t bytes) {
	void* p = nullptr;
	if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
	return p;
}

void xfem_free_host(void* p) {
	if (p) cudaFreeHost(p);
}

const char* xfem_last_error(void) { return g_err.c_str(); }

}  // extern "C"

// ---- reverse-mode adjoint -------------------------------------------------------
namespace {

// Device vertex of a vertex in the handle's concatenated caller order.
uint32_t dev_vertex(const xfem_body* h, uint32_t i) {
	for (const BodyHost& b : h->bodies)
		if (i < b.vbase + b.nv) return b.vbase + b.sched.vert_rank[i - b.vbase];
	return 0xffffffffu;
}

// Block size of the adjoint kernels: the largest whose staging fits.
int adjoint_block(xfem_body* h, int* block) {
	int optin = 0;
	XCUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
	for (int bs : {256, 128, 64, 32})
		if (solve_smem_bytes(bs, h->cfg.warp_smem) <= (size_t)optin) {
			*block = bs;
			return XFEM_OK;
		}
	return fail(XFEM_ELIMIT, "chunk blocks too large for shared memory");
}

// The handle's DevCtx with the tape of segment j attached.
DevCtx tape_ctx(xfem_body* h, uint32_t j) {
	AdjointRun& a = h->adj;
	DevCtx c = h->ctx;
	c.tape_v = a.tape_v.p;
	c.tape_t = a.tape_t.p;
	c.tape_fin = a.tape_fin.p;
	c.traj = a.traj.p;
	c.tip_of = a.tip_of.p;
	c.sub_base = j * a.seg;
	c.ntips = a.ntips;
	return c;
}

uint32_t seg_len(const AdjointRun& a, uint32_t j) { return std::min(a.seg, a.nsub - j * a.seg); }

}  // namespace

extern "C" {

int xfem_adjoint_forward(xfem_body* h, uint32_t nsub, float dt, uint32_t checkpoint_every, uint32_t ntips,
                         const uint32_t* tips, float* tip_traj) {
	if (!h) return fail(XFEM_EINVAL, "null handle");
	if (!(dt > 0.0f) || !isfinite(dt)) return fail(XFEM_EINVAL, "dt must be > 0");
	if (nsub == 0) return fail(XFEM_EINVAL, "substeps must be > 0");
	if (ntips && !tips) return fail(XFEM_EINVAL, "null tips");
	if (h->el_mode) return fail(XFEM_EUNSUPPORTED, "the adjoint covers linear tet meshes only");
	for (const BodyHost& b : h->bodies) {
		const uint32_t energy = (b.settings.flags >> XFEM_ENERGY_BIT) & XFEM_ENERGY_MASK;
		if (model_of(energy) != kModelNeo || !((b.settings.flags >> XFEM_XPBD_SOLVE_BIT) & 1u))
			return fail(XFEM_EUNSUPPORTED, "the adjoint covers the coupled Neo-Hookean model only (energy 4, XPBD solve bit)");
		if (b.settings.volume_passes)
			return fail(XFEM_EUNSUPPORTED, "the adjoint does not differentiate volume passes (volume_passes must be 0)");
		if (b.settings.damping > 0.0f || b.settings.pbd_damping > 0.0f)
			return fail(XFEM_EUNSUPPORTED, "the adjoint does not differentiate damping (damping, pbd_damping must be 0)");
		if (b.settings.flags & XFEM_LOCK_RIGHT)
			return fail(XFEM_EUNSUPPORTED, "the adjoint does not differentiate the Right lock (XFEM_LOCK_RIGHT)");
	}
	XCUDA(cudaSetDevice(h->device));
	AdjointRun& a = h->adj;
	a.valid = false;
	const bool same_tips = a.tips_uploaded && a.tips.size() == ntips && std::equal(a.tips.begin(), a.tips.end(), tips);
	std::vector<int32_t> tip_of;
	if (!same_tips) {
		tip_of.assign(h->nverts, -1);
		for (uint32_t q = 0; q < ntips; q++) {
			const uint32_t dv = dev_vertex(h, tips[q]);
			if (dv == 0xffffffffu) return fail(XFEM_EINVAL, "tip " + std::to_string(tips[q]) + " out of range");
			if (tip_of[dv] >= 0) return fail(XFEM_EINVAL, "tips must be distinct");
			tip_of[dv] = (int32_t)q;
		}
	}
	const uint32_t seg = checkpoint_every == 0 || checkpoint_every > nsub ? nsub : checkpoint_every;
	const uint32_t nseg = (nsub + seg - 1) / seg;
	const size_t nv = h->nverts;
	XCUDA(a.tape_v.reserve((size_t)seg * 2 * nv));
	XCUDA(a.tape_t.reserve((size_t)seg * h->nrows * 3 * kLanes));
	XCUDA(a.tape_fin.reserve(nv));
	XCUDA(a.traj.reserve((size_t)nsub * std::max(ntips, 1u)));
	XCUDA(a.grad.reserve((size_t)nsub * std::max(ntips, 1u)));
	XCUDA(a.tip_of.reserve(nv));
	XCUDA(a.abar.reserve(2 * nv));
	XCUDA(a.cbar.reserve((size_t)h->nrows * kLanes));
	if (nseg > 1) XCUDA(a.ckpt.reserve((size_t)(nseg + 1) * 2 * nv));
	if (!same_tips) {
		a.tips_uploaded = false;
		XCUDA(cudaMemcpyAsync(a.tip_of.p, tip_of.data(), nv * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
		a.tips.assign(tips, tips + ntips);
		a.tips_uploaded = true;
	}
	a.nsub = nsub;
	a.seg = seg;
	a.nseg = nseg;
	a.ntips = ntips;
	a.dt = dt;
	int block = 0;
	int rc = adjoint_block(h, &block);
	if (rc) return rc;
	for (uint32_t j = 0; j < nseg; j++) {
		if (nseg > 1)
			XCUDA(cudaMemcpyAsync(a.ckpt.p + 2 * nv * j, h->vert.p, 2 * nv * sizeof(float4), cudaMemcpyDeviceToDevice,
			                      h->stream));
		const int e = launch_substeps_tape(tape_ctx(h, j), block, h->cfg.warp_smem, seg_len(a, j), dt, h->stream);
		if (e) return fail(XFEM_ECUDA, std::string("recording launch: ") + cudaGetErrorString((cudaError_t)e));
	}
	if (nseg > 1)
		XCUDA(cudaMemcpyAsync(a.ckpt.p + 2 * nv * nseg, h->vert.p, 2 * nv * sizeof(float4), cudaMemcpyDeviceToDevice,
		                      h->stream));
	std::vector<float4> traj;
	if (tip_traj && ntips) {
		traj.resize((size_t)nsub * ntips);
		XCUDA(cudaMemcpyAsync(traj.data(), a.traj.p, traj.size() * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
	}
	rc = check_device_error(h);
	if (rc) return rc;
	for (size_t i = 0; i < traj.size(); i++) {
		tip_traj[3 * i] = traj[i].x;
		tip_traj[3 * i + 1] = traj[i].y;
		tip_traj[3 * i + 2] = traj[i].z;
	}
	a.valid = true;
	return XFEM_OK;
}

int xfem_adjoint_backward(xfem_body* h, const float* grad_tip_traj, const float* grad_x, const float* grad_v,
                          float* dmu, float* dx0, float* dv0) {
	if (!h) return fail(XFEM_EINVAL, "null handle");
	AdjointRun& a = h->adj;
	if (!a.valid) return fail(XFEM_EINVAL, "no recorded run: call xfem_adjoint_forward first");
	if (a.ntips && !grad_tip_traj) return fail(XFEM_EINVAL, "null grad_tip_traj");
	XCUDA(cudaSetDevice(h->device));
	const size_t nv = h->nverts;
	std::vector<float4> g((size_t)a.nsub * a.ntips);
	for (size_t i = 0; i < g.size(); i++)
		g[i] = make_float4(grad_tip_traj[3 * i], grad_tip_traj[3 * i + 1], grad_tip_traj[3 * i + 2], 0.0f);
	if (!g.empty())
		XCUDA(cudaMemcpyAsync(a.grad.p, g.data(), g.size() * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
	// abar = the canonical dL/dX, dL/dV at the end, scattered to device order
	XCUDA(cudaMemsetAsync(a.abar.p, 0, 2 * nv * sizeof(float4), h->stream));
	for (int which = 0; which < 2; which++) {
		const float* src = which == 0 ? grad_x : grad_v;
		if (!src) continue;
		float* stage = h->io.p + 3 * nv * which;
		XCUDA(cudaMemcpyAsync(stage, src, 3 * nv * sizeof(float), cudaMemcpyHostToDevice, h->stream));
		if (launch_scatter_xyz(a.abar.p, which, h->dev_of_vert.p, (uint32_t)nv, stage, h->stream))
			return fail(XFEM_ECUDA, "scatter launch failed");
	}
	XCUDA(cudaMemsetAsync(a.cbar.p, 0, (size_t)h->nrows * kLanes * sizeof(float), h->stream));
	int block = 0;
	int rc = adjoint_block(h, &block);
	if (rc) return rc;
	if (const int e = configure_adjoint_kernels(block, h->cfg.warp_smem))
		return fail(XFEM_ECUDA, std::string("adjoint kernel configuration: ") + cudaGetErrorString((cudaError_t)e));
	const AdjCtx actx = {a.abar.p, a.cbar.p, a.grad.p};
	for (int j = (int)a.nseg - 1; j >= 0; j--) {
		const DevCtx c = tape_ctx(h, (uint32_t)j);
		if (a.nseg > 1) {  // rebuild this segment's tape from its checkpoint
			XCUDA(cudaMemcpyAsync(h->vert.p, a.ckpt.p + 2 * nv * j, 2 * nv * sizeof(float4), cudaMemcpyDeviceToDevice,
			                      h->stream));
			const int e = launch_substeps_tape(c, block, h->cfg.warp_smem, seg_len(a, j), a.dt, h->stream);
			if (e) return fail(XFEM_ECUDA, std::string("recording launch: ") + cudaGetErrorString((cudaError_t)e));
		}
		const int e = launch_reverse(c, actx, block, h->cfg.warp_smem, h->max_colour_chunks, seg_len(a, j), a.dt,
		                             j == (int)a.nseg - 1, h->stream);
		if (e) return fail(XFEM_ECUDA, std::string("reverse launch: ") + cudaGetErrorString((cudaError_t)e));
	}
	if (a.nseg > 1)
		XCUDA(cudaMemcpyAsync(h->vert.p, a.ckpt.p + 2 * nv * a.nseg, 2 * nv * sizeof(float4), cudaMemcpyDeviceToDevice,
		                      h->stream));
	// outputs in caller order, gathered on the device
	if (dx0 && launch_gather_xyz(a.abar.p, 0, h->dev_of_vert.p, (uint32_t)nv, h->io.p, h->stream))
		return fail(XFEM_ECUDA, "gather launch failed");
	if (dv0 && launch_gather_xyz(a.abar.p, 1, h->dev_of_vert.p, (uint32_t)nv, h->io.p + 3 * nv, h->stream))
		return fail(XFEM_ECUDA, "gather launch failed");
	if (dmu && launch_gather_dmu(a.cbar.p, h->tet_slot_dev.p, h->tet_inv_mu.p, h->ntets, h->io.p + 6 * nv, h->stream))
		return fail(XFEM_ECUDA, "gather launch failed");
	if (dx0) XCUDA(cudaMemcpyAsync(dx0, h->io.p, 3 * nv * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
	if (dv0) XCUDA(cudaMemcpyAsync(dv0, h->io.p + 3 * nv, 3 * nv * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
	if (dmu) XCUDA(cudaMemcpyAsync(dmu, h->io.p + 6 * nv, h->ntets * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
	return check_device_error(h);
}

}  // extern "C"
