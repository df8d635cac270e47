// GPU set-up path of libxfem.so: the parallel phases of a handle's set-up on
// the device, each giving bit for bit what its host counterpart
// (xfem_host.cpp) gives:
//   rest state   per tet, the shared arithmetic of xfem_rest.h
//                (InitTriTetFiniteElement, XPBDFEM/Fem.cpp:196-224)
//   incidence    vertex -> tets in increasing tet id, by one radix sort of
//                (vertex, tet) keys
//   masses       per vertex, the lumped masses of its tets summed in tet
//                order from zero, then inverted (XPBDFEM/Geo.cpp:741-744)
//   flags        the AABB and the Left / Right flags (XPBDFEM/Geo.cpp:713-727)
//   vertex ranks Morton codes of the rest positions, radix-sorted with the
//                vertex id as tie-break
//   cluster order per colour, by (Morton code of the centroid or smallest
//                vertex id, cluster id)
// The greedy clustering and colouring between them stay on the host: each
// decision depends on every earlier one in id order.
//
// Scans and sorts use CUB (part of the CUDA toolkit); every other kernel is
// in this file. All launches go to the caller's stream.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <cub/cub.cuh>

#include "xfem_internal.h"
#include "xfem_rest.h"

namespace xfem {

namespace {

constexpr int kBlock = 256;

inline uint32_t blocks_for(size_t n) { return (uint32_t)((n + kBlock - 1) / kBlock); }

__global__ void k_rest(const float* __restrict__ nodes, const uint32_t* __restrict__ tets, uint32_t nt, float density,
                       float* __restrict__ ep, float* __restrict__ dm) {
	const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nt) return;
	uint32_t is[4];
	for (int n = 0; n < 4; n++) is[n] = tets[4 * (size_t)t + n];
	float o[17];
	dm[t] = rest::tet(nodes, is, density, o);
	for (int k = 0; k < 17; k++) ep[17 * (size_t)t + k] = o[k];
}

// Float order as an integer order (for atomicMin / atomicMax on floats).
__device__ __forceinline__ int ordered(float x) {
	const int b = __float_as_int(x);
	return b >= 0 ? b : b ^ 0x7fffffff;
}
float host_unordered(int b) {
	const int u = b >= 0 ? b : b ^ 0x7fffffff;
	float x;
	memcpy(&x, &u, 4);
	return x;
}

// out[0..2] = min, out[3..5] = max of the node coordinates, as ordered ints
// (initialised to INT_MAX / INT_MIN).
__global__ void k_aabb(const float* __restrict__ nodes, uint32_t nv, int* __restrict__ out) {
	float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
		for (int k = 0; k < 3; k++) {
			const float x = nodes[3 * (size_t)v + k];
			mn[k] = fminf(mn[k], x);
			mx[k] = fmaxf(mx[k], x);
		}
	for (int k = 0; k < 3; k++)
		for (int o = 16; o > 0; o >>= 1) {
			mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
			mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
		}
	if ((threadIdx.x & 31u) == 0)
		for (int k = 0; k < 3; k++) {
			atomicMin(out + k, ordered(mn[k]));
			atomicMax(out + 3 + k, ordered(mx[k]));
		}
}

__global__ void k_flags(const float* __restrict__ nodes, uint32_t nv, float mn, float mx, uint8_t* __restrict__ flags) {
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if (v < nv) flags[v] = rest::vertex_flags(nodes[3 * (size_t)v], mn, mx);
}

// One key per (tet, corner): vertex << 32 | tet; counts per vertex.
__global__ void k_incidence_keys(const uint32_t* __restrict__ tets, uint32_t nt, uint64_t* __restrict__ keys,
                                 uint32_t* __restrict__ count) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= 4u * nt) return;
	const uint32_t v = tets[i];
	keys[i] = ((uint64_t)v << 32) | (i >> 2);
	atomicAdd(count + v, 1u);
}

__global__ void k_low_words(const uint64_t* __restrict__ keys, size_t n, uint32_t* __restrict__ out) {
	const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) out[i] = (uint32_t)keys[i];
}

__global__ void k_masses(const uint32_t* __restrict__ off, const uint32_t* __restrict__ lst,
                         const float* __restrict__ dm, uint32_t nv, float* __restrict__ w) {
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if (v >= nv) return;
	float m = 0.0f;
	for (uint32_t j = off[v]; j < off[v + 1]; j++) m += dm[lst[j]];
	w[v] = 1.0f / m;
}

__global__ void k_vertex_keys(const float* __restrict__ nodes, uint32_t nv, MortonFrame f, uint64_t* __restrict__ keys) {
	const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
	if (v < nv) keys[v] = ((uint64_t)f.code(nodes + 3 * (size_t)v) << 32) | v;
}

__global__ void k_ranks(const uint64_t* __restrict__ sorted, uint32_t nv, uint32_t* __restrict__ rank) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < nv) rank[(uint32_t)sorted[i]] = i;
}

__global__ void k_cluster_keys(const float* __restrict__ nodes, const uint32_t* __restrict__ tets,
                               const uint32_t* __restrict__ cl_begin, const uint32_t* __restrict__ cl_tets,
                               const uint32_t* __restrict__ cl_colour, uint32_t nc, uint32_t morton, MortonFrame f,
                               uint64_t* __restrict__ keys, uint32_t* __restrict__ ids) {
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= nc) return;
	const uint32_t b = cl_begin[k];
	keys[k] = ((uint64_t)cl_colour[k] << 32) | cluster_key(nodes, tets, cl_tets + b, cl_begin[k + 1] - b, morton, f);
	ids[k] = k;
}

// Device buffer owned by the set-up (freed on scope exit).
template <typename T>
struct Buf {
	T* p = nullptr;
	~Buf() {
		if (p) cudaFree(p);
	}
	cudaError_t alloc(size_t n) { return cudaMalloc((void**)&p, sizeof(T) * (n ? n : 1)); }
};

#define XS(call)                                   \
	do {                                           \
		const cudaError_t e_ = (call);             \
		if (e_ != cudaSuccess) return (int)e_;     \
	} while (0)
#define XI(call)                                   \
	do {                                           \
		const int e_ = (call);                     \
		if (e_) return e_;                         \
	} while (0)

int radix_sort_keys(const uint64_t* in, uint64_t* out, size_t n, int end_bit, cudaStream_t st) {
	size_t bytes = 0;
	XS(cub::DeviceRadixSort::SortKeys(nullptr, bytes, in, out, (int64_t)n, 0, end_bit, st));
	Buf<uint8_t> tmp;
	XS(tmp.alloc(bytes));
	XS(cub::DeviceRadixSort::SortKeys(tmp.p, bytes, in, out, (int64_t)n, 0, end_bit, st));
	return (int)cudaStreamSynchronize(st);
}

int bits_for(uint64_t max_value) {
	int b = 1;
	while (b < 64 && (max_value >> b)) b++;
	return b;
}

}  // namespace

int gpu_setup_mesh(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, float density, uint32_t morton,
                   GpuSetupMesh& out, void* stream) {
	cudaStream_t st = (cudaStream_t)stream;
	out.ep.resize(17 * (size_t)nt);
	out.w0.resize(nv);
	out.vflags.resize(nv);
	out.off.assign((size_t)nv + 1, 0);
	out.lst.resize(4 * (size_t)nt);
	out.vert_rank.resize(nv);
	if (nv == 0) return 0;
	const size_t n4 = 4 * (size_t)nt;
	Buf<float> d_nodes, d_ep, d_dm, d_w;
	Buf<uint32_t> d_tets, d_count, d_off, d_lst, d_rank;
	Buf<uint64_t> d_keys, d_sorted;
	Buf<int> d_box;
	Buf<uint8_t> d_flags;
	XS(d_nodes.alloc(3 * (size_t)nv));
	XS(d_tets.alloc(n4));
	XS(d_ep.alloc(17 * (size_t)nt));
	XS(d_dm.alloc(nt));
	XS(d_w.alloc(nv));
	XS(d_count.alloc((size_t)nv + 1));
	XS(d_off.alloc((size_t)nv + 1));
	XS(d_lst.alloc(n4));
	XS(d_keys.alloc(n4 > nv ? n4 : nv));
	XS(d_sorted.alloc(n4 > nv ? n4 : nv));
	XS(d_rank.alloc(nv));
	XS(d_box.alloc(6));
	XS(d_flags.alloc(nv));
	XS(cudaMemcpyAsync(d_nodes.p, nodes, 12 * (size_t)nv, cudaMemcpyHostToDevice, st));
	XS(cudaMemcpyAsync(d_tets.p, tets, 4 * n4, cudaMemcpyHostToDevice, st));
	// rest state and the AABB
	if (nt) k_rest<<<blocks_for(nt), kBlock, 0, st>>>(d_nodes.p, d_tets.p, nt, density, d_ep.p, d_dm.p);
	const int box0[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
	XS(cudaMemcpyAsync(d_box.p, box0, sizeof(box0), cudaMemcpyHostToDevice, st));
	const uint32_t gb = blocks_for(nv) < 1024u ? blocks_for(nv) : 1024u;
	k_aabb<<<gb, kBlock, 0, st>>>(d_nodes.p, nv, d_box.p);
	XS(cudaGetLastError());
	int box[6];
	XS(cudaMemcpyAsync(box, d_box.p, sizeof(box), cudaMemcpyDeviceToHost, st));
	XS(cudaStreamSynchronize(st));
	MortonFrame f;
	for (int k = 0; k < 3; k++) {
		f.mn[k] = host_unordered(box[k]);
		f.mx[k] = host_unordered(box[3 + k]);
	}
	f.set_scale();
	k_flags<<<blocks_for(nv), kBlock, 0, st>>>(d_nodes.p, nv, f.mn[0], f.mx[0], d_flags.p);
	// incidence: (vertex, tet) keys sorted, vertex counts scanned
	XS(cudaMemsetAsync(d_count.p, 0, 4 * ((size_t)nv + 1), st));
	if (nt) {
		k_incidence_keys<<<blocks_for(n4), kBlock, 0, st>>>(d_tets.p, nt, d_keys.p, d_count.p);
		XS(cudaGetLastError());
		XI(radix_sort_keys(d_keys.p, d_sorted.p, n4, 32 + bits_for(nv - 1), st));
		k_low_words<<<blocks_for(n4), kBlock, 0, st>>>(d_sorted.p, n4, d_lst.p);
	}
	{
		size_t bytes = 0;
		XS(cub::DeviceScan::ExclusiveSum(nullptr, bytes, d_count.p, d_off.p, (int64_t)nv + 1, st));
		Buf<uint8_t> tmp;
		XS(tmp.alloc(bytes));
		XS(cub::DeviceScan::ExclusiveSum(tmp.p, bytes, d_count.p, d_off.p, (int64_t)nv + 1, st));
		XS(cudaStreamSynchronize(st));
	}
	k_masses<<<blocks_for(nv), kBlock, 0, st>>>(d_off.p, d_lst.p, d_dm.p, nv, d_w.p);
	// vertex ranks
	if (morton) {
		k_vertex_keys<<<blocks_for(nv), kBlock, 0, st>>>(d_nodes.p, nv, f, d_keys.p);
		XS(cudaGetLastError());
		XI(radix_sort_keys(d_keys.p, d_sorted.p, nv, 64, st));
		k_ranks<<<blocks_for(nv), kBlock, 0, st>>>(d_sorted.p, nv, d_rank.p);
	}
	XS(cudaGetLastError());
	XS(cudaMemcpyAsync(out.ep.data(), d_ep.p, 68 * (size_t)nt, cudaMemcpyDeviceToHost, st));
	XS(cudaMemcpyAsync(out.w0.data(), d_w.p, 4 * (size_t)nv, cudaMemcpyDeviceToHost, st));
	XS(cudaMemcpyAsync(out.vflags.data(), d_flags.p, nv, cudaMemcpyDeviceToHost, st));
	XS(cudaMemcpyAsync(out.off.data(), d_off.p, 4 * ((size_t)nv + 1), cudaMemcpyDeviceToHost, st));
	XS(cudaMemcpyAsync(out.lst.data(), d_lst.p, 4 * n4, cudaMemcpyDeviceToHost, st));
	if (morton) XS(cudaMemcpyAsync(out.vert_rank.data(), d_rank.p, 4 * (size_t)nv, cudaMemcpyDeviceToHost, st));
	XS(cudaStreamSynchronize(st));
	if (!morton)
		for (uint32_t v = 0; v < nv; v++) out.vert_rank[v] = v;
	out.frame = f;
	return 0;
}

int gpu_cluster_order(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, uint32_t morton,
                      const MortonFrame& f, Schedule& s, void* stream) {
	cudaStream_t st = (cudaStream_t)stream;
	const uint32_t nc = s.nclusters, ncol = s.ncolours;
	s.colour_cl.resize(nc);
	s.colour_cl_begin.assign(ncol + 1, 0);
	if (nc == 0) return 0;
	Buf<float> d_nodes;
	Buf<uint32_t> d_tets, d_begin, d_cltets, d_colour, d_ids, d_ids2;
	Buf<uint64_t> d_keys, d_keys2;
	XS(d_nodes.alloc(3 * (size_t)nv));
	XS(d_tets.alloc(4 * (size_t)nt));
	XS(d_begin.alloc((size_t)nc + 1));
	XS(d_cltets.alloc(s.cl_tets.size()));
	XS(d_colour.alloc(nc));
	XS(d_ids.alloc(nc));
	XS(d_ids2.alloc(nc));
	XS(d_keys.alloc(nc));
	XS(d_keys2.alloc(nc));
	XS(cudaMemcpyAsync(d_nodes.p, nodes, 12 * (size_t)nv, cudaMemcpyHostToDevice, st));
	XS(cudaMemcpyAsync(d_tets.p, tets, 16 * (size_t)nt, cudaMemcpyHostToDevice, st));
	XS(cudaMemcpyAsync(d_begin.p, s.cl_begin.data(), 4 * ((size_t)nc + 1), cudaMemcpyHostToDevice, st));
	XS(cudaMemcpyAsync(d_cltets.p, s.cl_tets.data(), 4 * s.cl_tets.size(), cudaMemcpyHostToDevice, st));
	XS(cudaMemcpyAsync(d_colour.p, s.cl_colour.data(), 4 * (size_t)nc, cudaMemcpyHostToDevice, st));
	k_cluster_keys<<<blocks_for(nc), kBlock, 0, st>>>(d_nodes.p, d_tets.p, d_begin.p, d_cltets.p, d_colour.p, nc, morton,
	                                                  f, d_keys.p, d_ids.p);
	XS(cudaGetLastError());
	// stable radix sort: equal keys keep increasing cluster ids, as the host's
	// sort of (key, id) pairs
	size_t bytes = 0;
	const int end_bit = 32 + bits_for(ncol ? ncol - 1 : 0);
	XS(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_keys.p, d_keys2.p, d_ids.p, d_ids2.p, (int64_t)nc, 0, end_bit,
	                                   st));
	Buf<uint8_t> tmp;
	XS(tmp.alloc(bytes));
	XS(cub::DeviceRadixSort::SortPairs(tmp.p, bytes, d_keys.p, d_keys2.p, d_ids.p, d_ids2.p, (int64_t)nc, 0, end_bit,
	                                   st));
	XS(cudaMemcpyAsync(s.colour_cl.data(), d_ids2.p, 4 * (size_t)nc, cudaMemcpyDeviceToHost, st));
	XS(cudaStreamSynchronize(st));
	for (uint32_t k = 0; k < nc; k++) s.colour_cl_begin[s.cl_colour[k] + 1]++;
	for (uint32_t c = 0; c < ncol; c++) s.colour_cl_begin[c + 1] += s.colour_cl_begin[c];
	return 0;
}

}  // namespace xfem
