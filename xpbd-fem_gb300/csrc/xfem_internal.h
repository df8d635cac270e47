// Internal declarations shared by the host code (xfem_host.cpp, xfem_api.cpp)
// and the CUDA kernels (xfem_kernels.cu) of libxfem.so.
#pragma once

#include <stdint.h>
#include <vector_types.h>

#include <vector>

#include "xfem_rest.h"

namespace xfem {

// Limits of one cluster: the tets processed in sequence by one GPU thread.
// An edge star of a 6-tet cube split has 6 tets on 8 vertices.
constexpr uint32_t kMaxClusterVerts = 8;
constexpr uint32_t kMaxClusterTets = 8;
constexpr uint32_t kMaxColours = 4096;
constexpr uint32_t kLanes = 32;  // clusters per chunk (one warp)

// ---- host-side mesh and schedule ------------------------------------------
// Parses the tagged index stream (4 = tet). Returns 0, -1 on a non-tet tag or a
// truncated record.
int parse_tets(const uint32_t* idx, uint32_t idx_count, std::vector<uint32_t>& tets, uint32_t& nverts);

// Rest state of every tet and the inverse masses, bit for bit what
// GeoLinear3d::Init computes (XPBDFEM/Geo.cpp:697-745, XPBDFEM/Fem.cpp:131-224).
// ep: 17 floats per tet (Qi column-major, QQ, QR, volume, surfaceArea).
// vflags: bit 0 Left, bit 1 Right (XPBDFEM/Geo.cpp:724-725), bit 4 Pickable.
void init_rest(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, float density,
               float* ep, float* w, uint8_t* vflags);

// GenerateTetBlock (XPBDFEM/MeshGen.cpp:156-244).
void gen_tet_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                   float wonkiness, float* nodes, uint32_t* idx);

struct Schedule {
	uint32_t nclusters = 0, ncolours = 0;
	std::vector<uint32_t> cl_begin;      // nclusters + 1, into cl_tets
	std::vector<uint32_t> cl_tets;       // member tets in sequence
	std::vector<uint32_t> cl_colour;     // nclusters
	std::vector<uint32_t> vert_rank;     // device rank of each vertex
	std::vector<uint32_t> colour_cl;     // clusters in device order, colour-major
	std::vector<uint32_t> colour_cl_begin;  // ncolours + 1
};

// Clusters (mode 0: one tet each; mode 1: edge stars), greedy colouring,
// Morton vertex order (morton != 0) and cluster order inside each colour.
// Returns 0 or -1 when a limit is exceeded. The phases, which the GPU set-up
// path (xfem_setup.cu) shares or replaces one by one:
int build_schedule(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, uint32_t mode,
                   uint32_t morton, Schedule& s);
// vertex -> tets in increasing tet id (CSR: off[nverts + 1], lst[4 ntets])
void incidence(const uint32_t* tets, uint32_t nverts, uint32_t ntets, std::vector<uint32_t>& off,
               std::vector<uint32_t>& lst, uint32_t npe = 4);
// the greedy clusters and colours in tet / cluster id order (sequential by
// definition); fills nclusters, cl_begin, cl_tets, cl_colour, ncolours
int cluster_and_colour(const uint32_t* tets, uint32_t ntets, const uint32_t* off, const uint32_t* lst, uint32_t mode,
                       Schedule& s);
// vert_rank (Morton rank, or the identity)
void vertex_ranks(const float* nodes, uint32_t nverts, uint32_t morton, Schedule& s);
// colour_cl, colour_cl_begin
void cluster_order(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t morton, Schedule& s);

// One-rings of the continuous-pressure models (OneRingConstructor,
// XPBDFEM/Connectivity.h:114-160): per vertex its tets (the incidence list)
// and its nodes, the vertex first, then each tet's vertices in order of first
// appearance; and the ring schedule: vertices coloured greedily in id order
// so that rings of one colour share no node, ordered inside each colour by
// vertex rank.
struct RingSchedule {
	uint32_t ncolours = 0;
	uint32_t nrings = 0;                    // ring centres: the first nrings vertices
	std::vector<uint32_t> tet_off, tets;    // the incidence: nverts + 1 offsets; tet ids
	std::vector<uint32_t> node_off, nodes;  // nrings + 1 offsets; caller vertex ids
	uint32_t npe = 4;                       // vertices per element: 4 (tets), 8 (hexes) or 10 (T10s)
	std::vector<uint8_t> corner;            // npe per incidence entry: node index of each element corner
	std::vector<uint32_t> order;            // vertices in ring order, colour-major
	std::vector<uint32_t> colour_begin;     // ncolours + 1, into order
};
// off / lst: the incidence (vertex -> tets in increasing id); vert_rank: the
// vertex ranks. Rings are built around the first ncentre vertices (all when
// larger than nverts; a T10 mesh rings its own vertices, not the edge
// nodes). Returns 0, -1 when the colour limit is exceeded, -2 when a ring
// has more than kMaxRingTets tets (kMaxRingHexes hexes, kMaxQRingElems T10s,
// kMaxH27RingElems H27s) or kMaxRingNodes vertices (kMaxQRingNodes on T10s
// and H27s).
int build_ring_schedule(const uint32_t* tets, uint32_t nverts, const uint32_t* off, const uint32_t* lst,
                        const uint32_t* vert_rank, RingSchedule& rs, uint32_t npe = 4, uint32_t ncentre = 0xffffffffu);

// A tagged stream that may mix tets (tag 4) and hexes (tag 8), each kind in
// stream order; -1 on another tag or a truncated record.
int parse_mixed(const uint32_t* idx, uint32_t count, std::vector<uint32_t>& tets, std::vector<uint32_t>& hexes,
                uint32_t& nverts);
// GeoLinear3d::Init on a mixed mesh (XPBDFEM/Geo.cpp:697-745): tet records
// (17 floats), hex records (rest::kHexRec), the masses of all tets then all
// hexes summed per vertex and inverted, the Left / Right flags.
void mixed_init_rest(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, const uint32_t* hexes,
                     uint32_t nhexes, float density, float* ep, float* hep, float* w, uint8_t* vflags);

// Linear hexahedra (H8). The tagged index stream with tag 8 (8 vertex ids
// per hex); -1 on another tag or a truncated record.
int parse_hexes(const uint32_t* idx, uint32_t idx_count, std::vector<uint32_t>& hexes, uint32_t& nverts);
// GeoLinear3d::Init on a hex mesh (XPBDFEM/Geo.cpp:697-745 with
// InitQuadHexFiniteElement, XPBDFEM/Fem.cpp:225-265): 120 floats per hex
// (rest::kHex* offsets), inverse masses and vertex flags, bit for bit.
void hex_init_rest(const float* nodes, uint32_t nverts, const uint32_t* hexes, uint32_t nhexes, float density,
                   float* hep, float* w, uint8_t* vflags);
// GenerateHexBlock (XPBDFEM/MeshGen.cpp:156-221): idx holds 9 words per hex.
void gen_hex_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz, uint32_t pattern,
                   float wonkiness, float* nodes, uint32_t* idx);
// The schedule of an element mode (hexes, T10s): elements coloured greedily
// in id order so that the elements of one colour share no vertex (each takes
// the smallest colour no earlier element on one of its vertices holds; at
// most kMaxElemColours), ordered inside each colour by the Morton code of the
// centroid of their `per` vertices (or by id without Morton order).
constexpr uint32_t kMaxElemColours = 4096;
struct ElemSchedule {
	uint32_t ncolours = 0;
	std::vector<uint32_t> order;         // elements, colour-major
	std::vector<uint32_t> colour_begin;  // ncolours + 1, into order
};
// Returns 0, or -1 when more than kMaxElemColours colours are needed.
int elem_schedule(const float* nodes, uint32_t nverts, const uint32_t* elems, uint32_t nel, uint32_t per,
                  uint32_t morton, ElemSchedule& es);

// Quadratic tetrahedra (T10, GeoQuadratic3d on a tet mesh). Connectivity3d's
// edge numbering (XPBDFEM/Connectivity.cpp:371-393, 478-520, EdgeFromVerts
// :587): for each lower vertex in id
// order, its distinct upper neighbours in the order their first tet edge
// appears in the stream, a later duplicate replacing the entry by the list's
// last one (swap-remove); edges gets 2 words per edge. t10 gets GeoQuadratic3d's
// 10 indices per tet (XPBDFEM/Geo.cpp:893-901): the corners, then nverts +
// the edge ids of the local edges (0,1) (0,2) (0,3) (1,2) (1,3) (2,3).
void tet_edges(const uint32_t* tets, uint32_t ntets, uint32_t nverts, std::vector<uint32_t>& edges,
               std::vector<uint32_t>& t10);
// GeoQuadratic3d::Init's rest state (XPBDFEM/Geo.cpp:836-941): X (3 doubles
// per vertex, nverts corners then one node per edge at the midpoint in
// double), vertex flags over all of them, 56 floats per T10 (rest::kT10*
// offsets) and the inverse lumped masses (LumpsTet10), bit for bit.
void t10_init_rest(const float* nodes, uint32_t nverts, uint32_t ntets, const uint32_t* edges,
                   uint32_t nedges, const uint32_t* t10, float density, double* X, float* qep, float* w,
                   uint8_t* vflags);

// Quadratic hexahedra (H27, GeoQuadratic3d on a hex mesh). Connectivity3d's
// edges (as tet_edges, each hex filing its 12 edges in the order of
// XPBDFEM/Connectivity.cpp:443-454) and quads (each hex face rotated to start
// at its smallest vertex and filed under it, XPBDFEM/Connectivity.cpp:
// 410-422, 456-461; a later duplicate in either winding swap-removed,
// :515-530; numbered vertex by vertex), and GeoQuadratic3d's 27 indices per
// hex (XPBDFEM/Geo.cpp:904-931): node i + 3j + 9k of the hex's 3x3x3 grid is
// a corner, nverts + an edge, nverts + nedges + a quad, or nverts + nedges +
// nquads + the hex.
void hex_edges_quads(const uint32_t* hexes, uint32_t nhexes, uint32_t nverts, std::vector<uint32_t>& edges,
                     std::vector<uint32_t>& quads, std::vector<uint32_t>& h27);
// Connectivity3d's edges and quads of a tagged stream that may mix tets and
// hexes (XPBDFEM/Connectivity.cpp:371-530): each element files its edges (a
// tet's 6, a hex's 12) and a hex its faces in stream order, under the same
// rules as tet_edges and hex_edges_quads, to which it reduces on a stream of
// one kind; t10 gets 10 indices per tet (tet order), h27 27 per hex (hex
// order) as those functions give them.
void quad_mesh(const uint32_t* idx, uint32_t count, uint32_t nverts, std::vector<uint32_t>& edges,
               std::vector<uint32_t>& quads, std::vector<uint32_t>& t10, std::vector<uint32_t>& h27);
// GeoQuadratic3d::Init's rest state on a mesh mixing tets and hexes
// (XPBDFEM/Geo.cpp:836-941): X over every vertex (corners, edge midpoints,
// quad centres, hex centres), flags, the T10 records (56 floats each) and
// the H27 records (703 floats each), the masses of all T10s then all H27s in
// one sum, inverted once; bit for bit.
void qmixed_init_rest(const float* nodes, uint32_t nverts, uint32_t ntets, const uint32_t* hexes, uint32_t nhexes,
                      const uint32_t* edges, uint32_t nedges, const uint32_t* quads, uint32_t nquads, const uint32_t* t10,
                      const uint32_t* h27, float density, double* X, float* qep, float* hep, float* w, uint8_t* vflags);
// GeoQuadratic3d::Init's rest state on a hex mesh (XPBDFEM/Geo.cpp:836-933):
// X (3 doubles per vertex: corners, edge midpoints, face centres, hex
// centres), flags over all of them, 703 floats per H27 (rest::kH27* offsets)
// and the inverse lumped masses, bit for bit.
void h27_init_rest(const float* nodes, uint32_t nverts, const uint32_t* hexes, uint32_t nhexes, const uint32_t* edges,
                   uint32_t nedges, const uint32_t* quads, uint32_t nquads, const uint32_t* h27, float density,
                   double* X, float* ep, float* w, uint8_t* vflags);

// ---- GPU set-up path (xfem_setup.cu) ------------------------------------------
// The parallel phases of the set-up on the device, bit for bit the host's:
// rest state (init_rest), incidence, Morton vertex ranks (vertex_ranks) and
// the cluster order (cluster_order). Return a cudaError_t value (0 = ok).
struct GpuSetupMesh {
	std::vector<float> ep, w0;        // as init_rest
	std::vector<uint8_t> vflags;
	std::vector<uint32_t> off, lst;   // as incidence
	std::vector<uint32_t> vert_rank;  // as vertex_ranks
	MortonFrame frame;                // the curve's frame for the cluster order
};
int gpu_setup_mesh(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, float density,
                   uint32_t morton, GpuSetupMesh& out, void* stream);
// s: clusters and colours from cluster_and_colour; fills colour_cl, colour_cl_begin
int gpu_cluster_order(const float* nodes, uint32_t nverts, const uint32_t* tets, uint32_t ntets, uint32_t morton,
                      const MortonFrame& f, Schedule& s, void* stream);

// ---- device-side structures ------------------------------------------------
// Material and step parameters of one body (uploaded on create / set_settings).
struct BodyParams {
	float mu, inv_mu, inv_lambda, a;  // mu = 1/compliance; inv_* = 1/mu, 1/lambda; a = 1 + mu/lambda
	                                  // (Pixar models: a = 1 + 2/lambda with lambda = 2/(1 - 2 nu))
	float yeoh[3];
	uint32_t energy;        // the reference's energy id (flags bits 6-10)
	float gravity[3];
	float drag_mul;         // 1 - time_corrected_drag
	uint32_t simultaneous;  // 1 = coupled 2x2 solve
	uint32_t lock_active;   // 1 = apply per-vertex lock bits
	uint32_t ground;        // 1 = ground plane
	float friction;
	float ground_n[3];
	float ground_d;
	float ratio;   // mu / lambda (0 when incompressible)
	uint32_t model;  // kModel*: how the solve treats the energy id
	// damping (XPBDFEM/Geo.cpp:346-355, 790-811; XPBDFEM/Xpbd.h:87-346)
	float damping;            // Rayleigh ratio (0 = off)
	uint32_t rayleigh_type;   // 0 Paper, 1 Limit (in the solve), 2 Post, 3 PostAmortized
	uint32_t pbd_on;          // pbd_damping > 0
	float pbd_coeff;          // volume- and time-corrected PBD damping
	float pbd_coeff_amortized;
	uint32_t ntets;           // tets of the body (amortized slices)
	uint32_t volume_passes;   // Settings::volumePasses: SolveElementVolume sweeps after the solve
	float hw;                 // Pixar models: lambda / 2, the weight of (J - a)^2
	float compliance;         // Settings::compliance (the volume passes' compliance per volume)
	float lambda;             // (2 mu nu) / (1 - 2 nu) (continuous-pressure models)
	uint32_t nverts;          // vertices of the body (amortized ring damping slices)
	uint32_t cube_fast;       // SolveElementCube's short path on hexes: CubeNeo, nu >= 0.5, no damping
	uint32_t lock_right;      // Settings_LockRight: hold the Right vertices at DevCtx::right_target
	float a_ring;             // the continuous-pressure models' (J - a)^2 on hexes: a = 1 + (1 - 2 nu)
	                          // (ContinuousPixar) or 1 / (2 nu) (XPBDFEM/Fem.cpp:1016)
	uint32_t nhexes;          // hexes of a body mixing tets and hexes (its hex damping slices)
	uint32_t pad5[3];
};

// Energy models on linear tets, as the solve treats them (BodyParams::model).
// With one quadrature point per tet, the quadrature forms of I1 (Mixed,
// YeohSkin, YeohSkinSel, Pixar, PixarReduced; XPBDFEM/Fem.cpp:379-402,
// 459-489) and the prefactored form (XPBDFEM/Fem.cpp:163-192) are the same
// polynomial of the edge vectors: tr(F^T F) with F = Qi Ds equals
// sum_ij (Qi^T Qi)_ij P_i . P_j, whose coefficients are QQ and QR. The
// solve evaluates the prefactored form for all of them.
constexpr uint32_t kModelNeo = 0;       // MixedSel (4), and ids above 12 (XPBDFEM/Fem.cpp:885-887)
constexpr uint32_t kModelNeoClamp = 1;  // Mixed (3): U0 = I1 clamped at 1e-4 (XPBDFEM/Fem.cpp:489)
constexpr uint32_t kModelYeoh = 2;      // YeohSkin (5), YeohSkinSel (6), YeohSkinFast (7)
constexpr uint32_t kModelPixar = 3;     // Pixar (0), PixarReduced (1), PixarSel (2): one constraint
constexpr uint32_t kModelNone = 4;      // CubeNeo (11), CubeSkin (12): no constraint on tets
constexpr uint32_t kModelRing = 5;      // ContinuousPixar (8), ContinuousMixed (9), ContinuousSkin (10):
                                        // one constraint (pair) per vertex one-ring, not per tet
constexpr uint32_t kMaxRingNodes = 32;  // vertices of a one-ring (one warp lane each)
constexpr uint32_t kMaxRingTets = 64;   // tets of a one-ring (two per warp lane)
constexpr uint32_t kMaxRingHexes = 16;  // hexes of a one-ring on a hex mesh (one per warp lane)
constexpr uint32_t kMaxQRingNodes = 128; // nodes of a one-ring over T10s or H27s (four per warp lane)
constexpr uint32_t kMaxQRingElems = 64;  // T10s of a one-ring (two per warp lane; 48 around a vertex
                                         // on which eight mirrored cubes' diagonals meet)
constexpr uint32_t kMaxH27RingElems = 16; // H27s of a one-ring (taken one after another; 8 on a grid)

// A chunk: 32 clusters of one colour side by side (lane = cluster), stored as
// one contiguous block that a single bulk copy brings into shared memory:
//   records  ntmax rows x 4 planes x 32 lanes x float4 (Qi, QQ, QR, c0)
//   header   32 x u32: nv | nt << 4 | advance mask << 8 | body << 16
//            (mask bit s: this cluster owns vertex slot s, i.e. it is the
//            lowest-colour cluster touching it, and so finalizes the previous
//            substep and predicts the next one for that vertex)
//   vids     nvmax rows x 32 x u32 (device vertex ids)
//   slots    ntmax rows x 32 x u32 (4 x 4-bit local vertex slots per tet)
struct ChunkMeta {
	uint32_t off16;  // block offset in 16-byte units
	uint32_t bytes;  // block size (a multiple of 128)
	uint32_t shape;  // ntmax | nvmax << 8 | kShapeCube
	uint32_t trow;   // first global tet row (multiplier output)
};

// Chunk flag: every populated lane is a whole 6-tet cube in the generator's
// corner order, i.e. local slots {0123, 0341, 0543, 0365, 0763, 0327}.
constexpr uint32_t kShapeCube = 1u << 16;

inline uint32_t chunk_block_bytes(uint32_t ntmax, uint32_t nvmax) { return 2048u * ntmax + 128u * (1u + nvmax + ntmax); }

// Everything a kernel needs, passed by value.
struct DevCtx {
	float4* vert;               // 2 per vertex: (O.xyz, w), (D.xyz, flag bits)
	const float4* cblk;         // chunk blocks
	float2* tlam;               // [trow][lane] multipliers or null
	const ChunkMeta* chunks;
	const uint32_t* colour_chunk_begin;  // ncolours + 1
	const uint32_t* isolated;   // vertices in no tet (stepped on their own)
	const BodyParams* bodies;
	const uint32_t* dep_begin;  // per chunk, into deps (dataflow mode)
	const uint32_t* deps;       // neighbour chunk | 1 << 31 when its colour is lower
	uint32_t* done;             // per chunk: substeps completed in this launch
	uint32_t nverts, nisolated, ncolours, nchunks;
	uint32_t chunk_smem;        // bytes of the largest chunk block
	uint32_t warp_smem;         // chunk_smem + vertex slots (2 x nvmax x 32 x 16 B, none when
	                            // every chunk takes the register-resident cube path)
	uint32_t vs_off;            // byte offset of the vertex slots in a warp's area
	uint32_t* bar_count;        // grid barrier arrival counter
	int* err;                   // device error word (0 = ok)
	const float4* right_target; // per device vertex: origin + lockedRightTransform3d X0 of the
	                            // Right vertices of bodies that lock them (null when none does)
	uint64_t timeout_ns;        // limit of every bounded device wait (barrier, copy, dependency)
	uint32_t bar_base;          // the arrival counter's value at launch: 0, or 0xffffffff
	                            // (a test of the counter's wrap: the first barrier wraps it)
	uint32_t wait_miss;         // test hook, normally 0: arrivals (dependency steps) each
	                            // bounded wait expects beyond those that come, so it runs out
	// Adjoint tape, written only by the recording forward kernel (null otherwise).
	// Substep indices are relative to the launch; `sub_base` is the launch's
	// first substep in the whole run (checkpointed segments).
	float4* tape_v;             // [substep][vertex] x 2 (one 32-byte sector): O after the
	                            // advance (the substep's start, with the w its solves
	                            // use) and D before it (the previous substep's swept D,
	                            // or V on a launch's first substep), written by the owner
	float4* tape_t;             // [substep][tet row][3][lane]: each solve's input D of its
	                            // four vertices, 12 floats in three float4
	float4* tape_fin;           // [vertex]: D before the closing finalize
	float4* traj;               // [run substep][tip]: position after each substep
	const int32_t* tip_of;      // per vertex: tip index or -1
	uint32_t ntrows, sub_base, ntips;
	uint32_t nvol;              // volume sweeps per substep (most of any body's volume_passes)
	// Damping sweeps after each substep's solve and volume sweeps (0 = none:
	// the state between substeps stays (O, D) and the next advance finishes
	// it). Bit 0: element Rayleigh damping (Post types), bit 1: PBD damping.
	uint32_t damp_kinds;
	uint32_t ext;               // some body damps (in the solve or after it), runs a Pixar
	                            // or cube model or volume passes: the extended kernels
	                            // (EXT instantiations) are launched
	uint32_t* tick;             // device word: Settings::tickId of the launch's first substep
	const uint32_t* tflat;      // [tet row][lane]: the tet's index in its body's flattened order
	const float* tarea;         // [tet row][lane]: the tet's surface area (rest state)
	const uint32_t* lastmask;   // [chunk][lane]: slots whose last solve of a substep this
	                            // cluster makes (it finishes them when damping sweeps run)
	const uint8_t* pass_on;     // [damping kind][tick % 8][colour]: some tet is damped
	// One-ring mode (continuous-pressure models; xfem_rings.cu): rings in
	// device order, colour-major. ring_hdr[r] = (first node, first tet entry,
	// nodes | tets << 8 | body << 16, the ring's index in its body's ring
	// order); ring_node: device vertex ids; ring_ent: per ring tet two float4
	// (QQ, QR, volume, corner node indices packed in the last word). The PBD
	// damping passes: per tet colour (pbd_cl_begin) the clusters (pbd_cl:
	// first entry, count), per entry (pbd_ent) the tet, its index in its
	// body's tet order, its surface area bits and its body; tet_verts: the
	// tets' device vertex ids.
	const uint4* ring_hdr;
	const uint32_t* ring_node;
	const float4* ring_ent;
	const uint32_t* colour_ring_begin;  // ring_colours + 1
	uint32_t ring_colours;
	uint32_t rings;
	const uint32_t* ring_clist;    // per ring: offset of its corner lists in ring_cwords
	const uint16_t* ring_cwords;   // per ring: nodes + 1 offsets, then each node's corners
	                               // (tet << 2 | corner) in tet order
	const uint32_t* pbd_cl_begin;  // pbd_colours + 1
	const uint2* pbd_cl;
	const uint4* pbd_ent;
	const uint32_t* tet_verts;
	uint32_t pbd_colours;
	// Element modes (xfem_hexes.cu: linear hexahedra; xfem_t10.cu: quadratic
	// tets; xfem_h27.cu: quadratic hexahedra): elements in device order,
	// colour-major (bodies in order inside a colour). el_vid: the element's
	// device vertex ids (hex: 8 in two uint4; T10: 10 in three uint4; H27: 27
	// in seven); el_rec: the records, as a structure of arrays for the
	// one-thread-per-element modes (float4 k of element i at
	// el_rec[k * nel + i]; hex 30 float4, T10 14) and element-major for H27
	// (704 floats per element, read by its warp); el_flat: each element's
	// index in its body's element order (the amortized damping slices);
	// el_tab: the mode's shape-function gradient tables, [point][node][axis]
	// (T10: the 4-point rule; H27: the 2x2x2 rule, then the 3x3x3 rule).
	uint32_t el_colours;
	const uint4* el_vid;
	const float4* el_rec;
	const uint32_t* colour_el_begin;  // el_colours + 1
	const uint32_t* el_flat;
	uint32_t nel;
	uint32_t mt_colours;
	const float* el_tab;
	// Meshes mixing tets and hexes (xfem_hexes.cu, k_mixed): the hexes as
	// above, the tets as elements of their own colouring: mt_vid the four
	// device vertex ids, mt_rec five float4 per tet as a structure of arrays
	// (float4 k of tet i at mt_rec[k * nmt + i]: Qi column-major, QQ, QR,
	// rest volume, surface area), mt_flat each tet's index in its body's tet
	// order.
	const uint4* mt_vid;
	const float4* mt_rec;
	const uint32_t* colour_mt_begin;  // mt_colours + 1
	const uint32_t* mt_flat;
	uint32_t nmt;
	// Brick launch form (sync_mode 4, k_bricks): the clusters split into
	// nbricks spatially compact bricks, one per block. Brick chunks: 32
	// clusters of one brick and one colour, each block kBrickChunkBytes (the
	// cube chunk's records and header, then the vertex words), brick b's
	// chunks of colour c at [bchunk_begin[b * ncolours + c],
	// bchunk_begin[b * ncolours + c + 1]). A vertex that only one brick's
	// clusters touch lives in that block's shared memory for the whole launch
	// (bpriv_vid: the device vertex of each slot, per brick from
	// bpriv_begin[b]); the others stay in vert. Instead of a grid barrier a
	// block waits after each pass for the bricks it shares vertices with
	// (bnb, from bnb_begin[b]) through their pass counters (bflag). bfin_vid:
	// the shared vertices each brick finalizes at the end of a launch.
	const float4* bcblk;
	const uint32_t* bchunk_begin;
	const uint32_t* bchunk_wait_end;  // per brick and colour: its chunks before this one hold
	                                  // boundary clusters and wait for the neighbours
	const uint32_t* bcnb_begin;       // per brick and colour: the bricks those chunks wait for,
	const uint32_t* bcnb;             // those that touched their shared vertices last before
	const uint32_t* bpriv_begin;
	const uint32_t* bpriv_vid;
	const uint32_t* bfin_begin;
	const uint32_t* bfin_vid;
	const uint32_t* bnb_begin;
	const uint32_t* bnb;
	uint32_t* bflag;
	uint32_t nbricks, bpriv_max;
	uint32_t nbodies;
};

// Brick chunk block: records (6 x 4 x 32 float4), header (32 u32), vertex
// words (8 x 32 u32): the device vertex id, or kPrivate | the vertex's slot
// in the brick's shared memory.
constexpr uint32_t kBrickChunkBytes = 2048u * 6u + 128u * (1u + 8u);
constexpr uint32_t kPrivate = 0x80000000u;
// Bodies whose parameters the brick kernel keeps in shared memory (handles
// with more bodies read them from global memory).
constexpr uint32_t kBrickBodies = 8u;
// Shared-memory bytes per private vertex: its state (32) and device id (4).
constexpr uint32_t kBrickVertexBytes = 36u;
// Words between two bricks' pass counters: each in a 128-byte line of its
// own, so that the polls of one brick's neighbours do not queue behind every
// other brick's on a few shared lines.
constexpr uint32_t kBrickFlagStride = 32u;
// A substep's passes, colour-major within each kind: the solve sweep (kind
// 0), volume sweeps 1..nvol, then one sweep per damping kind.

// Reverse-pass state (xfem_adjoint.cu).
struct AdjCtx {
	float4* abar;        // 2 per vertex: adjoint of the current position X = O + D,
	                     // and of O from the later substeps. At the end of the run
	                     // (in) and at its start (out): dL/dX, dL/dV of the
	                     // canonical state.
	float* cbar;         // [tet row][lane]: sum over substeps of alpha0 * dL/dalpha0 + alpha1 * dL/dalpha1 (= -mu dL/dmu)
	const float4* G;     // [run substep][tip]: dL/d(tip position after the substep)
};

// Vertex flag bits kept in the .w word of the second float4.
constexpr uint32_t kFlagLocked = 1u;
constexpr uint32_t kFlagContact = 2u;
constexpr uint32_t kFlagRight = 4u;  // the reference's Right flag (x above 98% of the extent)

// Device error codes written to DevCtx::err.
constexpr int kErrBarrierTimeout = 1;
constexpr int kErrCopyTimeout = 2;
constexpr int kErrDepTimeout = 3;
constexpr int kErrNonFinite = 4;  // a finished position or velocity is NaN or infinite

// Default limit of a bounded device wait: far above any legal wait.
constexpr uint64_t kDefaultTimeoutNs = 2000000000ull;

// ---- kernel launchers (xfem_kernels.cu) ---------------------------------------
struct LaunchCfg {
	int block = 256;
	int blocks = 0;        // persistent grid size
	int sync_mode = 1;     // 1 persistent + grid barrier, 2 per-colour launches (CUDA graph), 3 persistent dataflow,
	                       // 4 persistent bricks (k_bricks: brick-resident vertices, neighbour waits)
	bool lambdas = false;
	bool ext = false;      // launch the extended instantiations (DevCtx::ext)
	uint32_t warp_smem = 0;
	uint32_t total_chunks = 0;
	std::vector<uint32_t> colour_chunk_begin_host;
};

// Runs nsub substeps (canonical (X, V) in, canonical out) on `stream`.
// Returns a cudaError_t value (0 = success).
int launch_substeps(const DevCtx& ctx, const LaunchCfg& cfg, uint32_t nsub, float dt, void* stream);
// Sets the dynamic shared-memory limit of the solve kernels for cfg.block
// (call before launching or capturing).
int configure_kernels(const LaunchCfg& cfg);
// Largest co-resident grid for the persistent kernel at this block size.
int persistent_grid(const LaunchCfg& cfg, int* blocks_out);
// Dynamic shared memory bytes per block of the brick kernel, and whether
// `nbricks` blocks of `block` threads fit on the device at once (the
// cooperative launch needs the whole grid resident). Returns a cudaError_t
// value; *fits is set on success.
size_t brick_smem_bytes(int block, uint32_t bpriv_max);
int brick_grid_fits(int block, uint32_t bpriv_max, uint32_t nbricks, bool* fits);
// Dynamic shared memory bytes per block of the solve kernels.
size_t solve_smem_bytes(int block, uint32_t warp_smem);

// Allocation-free stepping: the persistent kernel with its scratch words in a
// fixed device array (xfem_kernels.cu). Synchronises `stream` and returns the
// device error word in *device_error. kNoAllocTooLong when the call's
// grid-barrier arrivals (substeps x passes per substep x blocks) would reach
// 2^31; otherwise a cudaError_t value.
constexpr int kNoAllocTooLong = -1;
int launch_substeps_noalloc(const DevCtx& ctx, int block, uint32_t warp_smem, bool lambdas, uint32_t nsub, float dt,
                            void* stream, int device, int* device_error);

// Adjoint (xfem_adjoint.cu, xfem_kernels.cu). The recording forward runs nsub
// substeps exactly as the persistent kernel does (same results bit for bit)
// and writes the tape of ctx. The reverse kernel runs the segment's substeps
// backwards from that tape (`last`: the run's final segment, whose closing
// finish receives the caller's dL/dX, dL/dV). Both are cooperative
// persistent launches.
int launch_substeps_tape(const DevCtx& ctx, int block, uint32_t warp_smem, uint32_t nsub, float dt, void* stream);
int launch_reverse(const DevCtx& ctx, const AdjCtx& adj, int block, uint32_t warp_smem, uint32_t max_colour_chunks,
                   uint32_t nsub, float dt, bool last, void* stream);
int configure_adjoint_kernels(int block, uint32_t warp_smem);

// Transfer helpers (caller order <-> device order), run on `stream`.
int launch_gather_xyz(const float4* vert, int which, const uint32_t* dev_of_caller, uint32_t n, float* out,
                      void* stream);
int launch_scatter_xyz(float4* vert, int which, const uint32_t* dev_of_caller, uint32_t n, const float* in,
                       void* stream);
int launch_volume(const float4* vert, const uint32_t* tets_dev, uint32_t nt, double* out, void* stream);
// One-ring mode (xfem_rings.cu): nsub substeps of the continuous-pressure
// models, a cooperative persistent launch of `block` threads per block
// (canonical (X, V) in and out).
int launch_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
// Hex mode (xfem_hexes.cu): nsub substeps of a hex mesh, a cooperative
// persistent launch (canonical (X, V) in and out).
int launch_hexes(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
// The continuous-pressure models on a hex mesh (xfem_hexes.cu): nsub
// substeps of one-ring solves over the hexes, a cooperative persistent
// launch (canonical (X, V) in and out).
int launch_hex_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
// Meshes mixing tets and hexes (xfem_hexes.cu): nsub substeps, every tet
// colour then every hex colour per sweep, a cooperative persistent launch.
int launch_mixed(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
// Quadratic-tet mode (xfem_t10.cu): nsub substeps of a T10 mesh, likewise.
int launch_t10(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
// The continuous-pressure models on a T10 mesh (xfem_t10.cu): nsub substeps
// of one-ring solves over the T10s around the mesh vertices, a cooperative
// persistent launch (canonical (X, V) in and out).
int launch_t10_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
int launch_h27_rings(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
// A mesh mixing T10s and H27s: ch27 with the H27 element arrays, ct10 the
// same context with the T10 element arrays (blocks of 256 threads).
int launch_qmixed(const DevCtx& ch27, const DevCtx& ct10, int block, uint32_t nsub, float dt, void* stream);
// Quadratic-hex mode (xfem_h27.cu): nsub substeps of an H27 mesh, one warp
// per element (block must be 256).
int launch_h27(const DevCtx& ctx, int block, uint32_t nsub, float dt, void* stream);
// Per-tet material (n tets from the given per-tet tables): c0 of each record
// and 1/mu; mu null = mu_uniform for all.
int launch_set_c0(float4* cblk, const uint32_t* rec, const float* vol, const float* mu, float mu_uniform, uint32_t n,
                  float* inv_mu, void* stream);
// out[t] = -cbar[slot[t]] / mu[t]
int launch_gather_dmu(const float* cbar, const uint32_t* slot, const float* inv_mu, uint32_t n, float* out,
                      void* stream);

}  // namespace xfem
