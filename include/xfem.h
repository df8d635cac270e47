/*
 * xfem.h — C ABI of the GB300 (sm_103a) small-step XPBD tetrahedral solver.
 *
 * A drop-in for the linear-tet path of jak-xyz/xpbd-fem: the same mesh input
 * (tagged index stream + float node array), the same rest-state precompute,
 * material and compliance parameters, the same Neo-Hookean / Yeoh deviatoric
 * plus volumetric constraints and the same one-iteration-per-substep schedule,
 * run as a graph-coloured Gauss-Seidel sweep on the GPU.
 *
 * Conventions
 *   - Every call returns int: XFEM_OK (0) or a negative XFEM_E* code;
 *     xfem_last_error() gives a message for the calling thread.
 *   - The caller owns host arrays; they are copied in or out. The handle owns
 *     all device memory. Arrays are in the caller's vertex and tet order (the
 *     internal Morton / colour permutations never leak out).
 *   - Calls on one handle are serialised on its CUDA stream. Stepping calls
 *     are asynchronous; a device-side error (bounded-wait timeout) is reported
 *     by the next synchronising call (a get_* call or xfem_synchronize).
 *   - One handle per host thread at a time.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   GeoLinear3d::Init            XPBDFEM/Geo.h:147, XPBDFEM/Geo.cpp:697-772
 *   Geo3d::Substep               XPBDFEM/Geo.h:56,  XPBDFEM/Geo.cpp:305-356
 *   GeoLinear3d::Constrain       XPBDFEM/Geo.cpp:774-788
 *   GeoLinear3d::CalculateVolume XPBDFEM/Geo.cpp:827-832
 *   struct Settings              XPBDFEM/Settings.h:79-102
 *   Sim::Update substep loop     XPBDFEM/Demo.cpp:37-103
 *   wasm exports UpdateSettings / AddBlock / FinishAddingBlocks / ResetDemo
 *                                wasm/main.cpp:8-17, 71-95
 *   GenerateTetBlock             XPBDFEM/MeshGen.cpp:223-244
 *   GenerateHexBlock             XPBDFEM/MeshGen.cpp:156-221
 *
 * Meshes of linear hexahedra (tag 8) run in hex mode: GeoLinear3d's hex loops
 * (XPBDFEM/Geo.cpp:736-740, 777-811) with SolveElement on
 * ElementParamsLinearHex (XPBDFEM/Fem.cpp:871-896), every energy model. With
 * the continuous-pressure ones (8-10) a hex mesh solves one constraint (pair)
 * per vertex one-ring over the hexes around it (SolveRing's full-energy
 * branch, XPBDFEM/Geo.cpp:147-225, XPBDFEM/Fem.cpp:980-1036). A mesh that
 * holds both tets and hexes runs in mixed mode (see below).
 *
 * A tet mesh whose settings ask for quadratic elements (element type
 * XFEM_ELEMENT_T10 in flags bits 0-3) runs as GeoQuadratic3d
 * (XPBDFEM/Geo.cpp:836-1053, picked by Sim::AddBlock, XPBDFEM/Demo.cpp:145-150):
 * one node added on every edge (Connectivity3d's edge numbering), T10
 * elements (ElementParamsQuadraticTet, SolveElement with Nodes = 10 on the
 * 4-point rule) and every energy model: with the continuous-pressure ones
 * (8-10) one constraint pair per one-ring of a mesh vertex over the T10s
 * around it (XPBDFEM/Geo.cpp:944-953, 973-982), up to 64 T10s and 128 nodes
 * per ring. The body's vertices are then the mesh's own followed by the edge
 * nodes, and every per-vertex call (positions, velocities, lock mask) covers
 * all of them. A handle holds one element type (linear tets, hexes, mixed,
 * T10s or H27s).
 */
#ifndef XFEM_H
#define XFEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define XFEM_OK 0
#define XFEM_EINVAL (-1)          /* bad argument (null pointer, size mismatch, index out of range) */
#define XFEM_EUNSUPPORTED (-2)    /* meshes, energy models or settings this path does not run */
#define XFEM_ENOMEM (-3)          /* host or device allocation failed */
#define XFEM_ECUDA (-4)           /* CUDA runtime error (no device, launch or copy failure) */
#define XFEM_EDEVICE_TIMEOUT (-5) /* a device-side bounded wait (grid barrier) ran out */
#define XFEM_ELIMIT (-6)          /* a schedule limit was exceeded (colours, cluster size) */
#define XFEM_ENONFINITE (-7)      /* a position or velocity became NaN or infinite (device sentinel) */

/* ---- flags: the reference's Settings::flags layout (XPBDFEM/Settings.h:9-29) - */
#define XFEM_ELEMENT_TYPE_MASK 15u      /* Settings_ElementTypeMask, bits 0-3 (XPBDFEM/Settings.h:9-10, 31-39): */
#define XFEM_ELEMENT_T4 5u              /*   Element_T4: linear tets (as 0) */
#define XFEM_ELEMENT_T10 6u             /*   Element_T10: a tet mesh runs as quadratic tets */
#define XFEM_ELEMENT_H8 7u              /*   Element_H8: linear hexes (as 0) */
#define XFEM_ELEMENT_H27 8u             /*   Element_H27: quadratic (tets: T10s, hexes: H27s; so does T10) */
#define XFEM_ENERGY_BIT 6u
#define XFEM_ENERGY_MASK 31u
/* Energy ids (XPBDFEM/Settings.h:41-53) as SolveElement dispatches them on a
 * linear tet (XPBDFEM/Fem.cpp:872-888); ids above 12 run MixedSel. */
#define XFEM_ENERGY_PIXAR 0u           /* Energy_Pixar: Stable Neo-Hookean, one constraint */
#define XFEM_ENERGY_PIXAR_REDUCED 1u   /* Energy_PixarReduced (= Pixar on a linear tet) */
#define XFEM_ENERGY_PIXAR_SEL 2u       /* Energy_PixarSel */
#define XFEM_ENERGY_MIXED 3u           /* Energy_Mixed: Neo-Hookean, I1 by quadrature */
#define XFEM_ENERGY_MIXED_SEL 4u       /* Energy_MixedSel: Neo-Hookean, prefactored I1 */
#define XFEM_ENERGY_YEOH_SKIN 5u       /* Energy_YeohSkin */
#define XFEM_ENERGY_YEOH_SKIN_SEL 6u   /* Energy_YeohSkinSel (= YeohSkin on a linear tet) */
#define XFEM_ENERGY_YEOH_SKIN_FAST 7u  /* Energy_YeohSkinFast */
#define XFEM_ENERGY_CONTINUOUS_PIXAR 8u /* continuous pressure: one constraint per vertex one-ring */
#define XFEM_ENERGY_CONTINUOUS_MIXED 9u /* likewise, the deviatoric + hydrostatic pair */
#define XFEM_ENERGY_CONTINUOUS_SKIN 10u /* likewise, with the Yeoh deviatoric term */
#define XFEM_ENERGY_CUBE_NEO 11u       /* Energy_CubeNeo: acts on hexes (and quads), on no tet */
#define XFEM_ENERGY_CUBE_SKIN 12u      /* Energy_CubeSkin: likewise */
#define XFEM_MAX_VOLUME_PASSES 64u     /* largest xfem_settings::volume_passes accepted */
#define XFEM_XPBD_SOLVE_BIT 11u        /* set: coupled 2x2 solve; clear: serial */
#define XFEM_RAYLEIGH_TYPE_BIT 20u     /* Settings_RayleighTypeBit, mask 3: */
#define XFEM_RAYLEIGH_PAPER 0u         /*   damping inside the solve (Rayleigh_Paper) */
#define XFEM_RAYLEIGH_LIMIT 1u         /*   damping inside the solve, limited (Rayleigh_Limit) */
#define XFEM_RAYLEIGH_POST 2u          /*   element damping after the velocity update (Rayleigh_Post) */
#define XFEM_RAYLEIGH_POST_AMORTIZED 3u /*  the same on one eighth of the order per substep, x 8 */
#define XFEM_LOCK_LEFT (1u << 26)      /* Settings_LockLeft: apply the lock mask */
#define XFEM_LOCK_RIGHT (1u << 27)     /* Settings_LockRight: hold the Right vertices (x above 98% of
                                          the body's extent) at origin + locked_right_transform X0 */

/* Solver settings. The first block mirrors the reference's Settings field by
 * field (XPBDFEM/Settings.h:79-91) with gravity widened to 3-D; fields this
 * path does not use are kept so a caller can fill the struct the same way. */
typedef struct xfem_settings {
	float time_scale;            /* unused by the solver (the caller picks dt) */
	float substeps_per_second;   /* unused by the solver */
	uint32_t volume_passes;      /* SolveElementVolume sweeps after each solve sweep (<= 64) */
	float gravity[3];            /* reference: vec2 (x, y) */
	float compliance;            /* 1 / mu_ref */
	float damping;               /* Rayleigh damping ratio (type in flags bits 20-21) */
	float pbd_damping;           /* > 0 enables PBD damping (coefficients below) */
	float drag;                  /* informational; the solver uses time_corrected_drag */
	float poissons_ratio;        /* 0.5 = incompressible (zero volumetric compliance) */
	float wonkiness;             /* mesh generation only */
	float left_right_separation; /* unused */
	uint32_t flags;              /* energy bits 6-10, solve bit 11, Rayleigh type bits 20-21, lock bit 26 */
	/* The reference's derived Settings::timeCorrectedDrag
	 * (XPBDFEM/Settings.h:97), filled by Sim::Update (XPBDFEM/Demo.cpp:63);
	 * xfem_time_corrected_drag() computes it. */
	float time_corrected_drag;
	/* Extensions (no reference counterpart). */
	float yeoh[3];               /* Yeoh multipliers; reference constants {0.1095, 14.95, 4.595} */
	uint32_t ground;             /* 1 = ground plane with Coulomb friction */
	float ground_normal[3];      /* unit normal; solid side is dot(n, x) < offset */
	float ground_offset;
	float friction;              /* Coulomb coefficient */
	/* The reference's derived Settings::volumeAndTimeCorrectedPbdDamping and
	 * amortizedVolumeAndTimeCorrectedPbdDamping (XPBDFEM/Settings.h:95-96),
	 * filled by Sim::Update (XPBDFEM/Demo.cpp:53-61);
	 * xfem_pbd_damping_coefficients() computes them. */
	float volume_and_time_corrected_pbd_damping;
	float amortized_volume_and_time_corrected_pbd_damping;
	/* Settings::tickId of the next substep (XPBDFEM/Settings.h:102): selects the
	 * eighth of the order damped by Rayleigh_PostAmortized. The handle counts it
	 * up by one per substep; xfem_set_settings sets it. */
	uint32_t tick_id;
	/* Settings::lockedRightTransform3d (XPBDFEM/Settings.h:100), column-major
	 * like the reference's mat3, and Geo3d::origin (XPBDFEM/Geo.h:69): with
	 * XFEM_LOCK_RIGHT every substep ends with the Right vertices at origin +
	 * transform X0 (X0 the rest position) and a zero inverse mass
	 * (XPBDFEM/Geo.cpp:323-331). The reference's demo animates the transform
	 * per substep (XPBDFEM/Demo.cpp:69-80); here it holds for a stepping call,
	 * so animate it with xfem_set_settings between xfem_substep calls. */
	float locked_right_transform[9];
	float origin[3];
} xfem_settings;

/* Create-time options (all zero = defaults). */
typedef struct xfem_options {
	uint32_t cluster_mode; /* 0 = default (edge-star clusters), 1 = one tet per cluster, 2 = edge-star,
	                          3 = tuned: both layouts built at create, each tuned and timed (20
	                          substeps of 1/1200 s on a saved copy of the state), the faster kept
	                          (xfem_info.cluster_mode tells which). The layout fixes the colour
	                          order, so the choice changes results within rounding */
	uint32_t no_morton;    /* 1 = keep the caller's vertex order on the device */
	uint32_t sync_mode;    /* 0 = auto (autotuned), 1 = persistent kernel + grid barrier, 2 = CUDA graph,
	                          3 = persistent kernel, chunks wait only on neighbouring chunks (dataflow),
	                          4 = persistent kernel over bricks: each block owns a compact brick of cube
	                          clusters whose own vertices stay in shared memory, and waits only on the
	                          bricks it shares vertices with (the plain solve on meshes of whole cubes;
	                          no damping, Pixar or cube models, volume passes or keep_lambdas) */
	uint32_t block_size;   /* 0 = auto; else 64..1024, multiple of 32 */
	uint32_t keep_lambdas; /* 1 = record each tet's two multipliers of the last substep */
	int32_t device;        /* CUDA device ordinal; -1 or 0 = current / 0 */
	void* stream;          /* cudaStream_t to run on; NULL = a stream owned by the handle */
	uint32_t host_setup;   /* 1 = rest state and schedule on the host (default: their parallel
	                          phases on the GPU; the result is the same bit for bit) */
	uint32_t wait_timeout_ms; /* limit of every bounded device wait (grid barrier, chunk copy,
	                             neighbour chunk); 0 = 2000 ms. A wait that runs out makes the
	                             call report XFEM_EDEVICE_TIMEOUT and leaves the context usable */
	uint32_t bricks;       /* sync_mode 4: number of bricks (blocks); 0 = one per SM */
} xfem_options;

/* One mesh for xfem_batch_create, in GeoLinear3d::Init's argument form. */
typedef struct xfem_mesh {
	const float* node_data;   /* 3 floats per vertex */
	uint32_t node_data_count; /* 3 * vertex count */
	const uint32_t* idx_data; /* tagged stream: 4, i0, i1, i2, i3, 4, ... */
	uint32_t idx_data_count;
	float density;
} xfem_mesh;

typedef struct xfem_info {
	uint32_t bodies, vertices, tets, clusters, colours;
	uint32_t isolated;        /* vertices in no tet */
	uint32_t chunks, tet_rows, block_size, blocks;
	uint32_t sync_mode;       /* 1 persistent + grid barrier, 2 CUDA graph, 3 persistent dataflow,
	                             4 persistent bricks */
	uint32_t cluster_mode;    /* 1 one tet per cluster, 2 edge stars */
	uint32_t max_chunk_deps;  /* largest neighbour-chunk list (dataflow mode) */
	uint32_t bricks;          /* bricks of the brick layout (0: none built) */
	uint64_t device_bytes;
} xfem_info;

typedef struct xfem_body xfem_body;

/* ---- lifecycle ------------------------------------------------------------ */
/* Fills s with the reference's Settings defaults (XPBDFEM/Settings.h:80-91)
 * plus gravity z = 0, time_corrected_drag 0, the reference Yeoh constants and
 * no ground. */
int xfem_settings_default(xfem_settings* s);

/* Replaces GeoLinear3d::Init(alloc, density, nodeData, nodeDataCount, idxData,
 * idxDataCount, autoResize = false), XPBDFEM/Geo.cpp:697-772: connectivity,
 * double-precision rest positions, Left/Right flags, rest state per tet,
 * lumped masses and inverse masses — then builds the colour schedule and
 * uploads everything. A mesh of hexes (tag 8) gets the hex rest state
 * (InitQuadHexFiniteElement, XPBDFEM/Fem.cpp:225-265) and the hex colouring;
 * element type T10 or H27 (flags bits 0-3) makes a tet mesh a T10 body and a
 * hex mesh an H27 body (GeoQuadratic3d::Init, XPBDFEM/Geo.cpp:836-941). A
 * mesh mixing tets and hexes is one body holding both (GeoLinear3d on one
 * tagged stream, XPBDFEM/Geo.cpp:697-811): each sweep solves every tet, then
 * every hex, each kind in a colouring of its own; with element type T10 or
 * H27 it is GeoQuadratic3d on that stream: T10s and H27s in one body, every
 * sweep solving every T10, then every H27. Such a mesh with the
 * continuous-pressure models (energy 8-10) is refused (XFEM_EUNSUPPORTED),
 * and so is a T10 or H27 body whose one-rings exceed 64 T10s (16 H27s) or
 * 128 nodes (XFEM_ELIMIT). A mesh without elements returns XFEM_EINVAL (the
 * reference's empty Geo3d steps nothing), as do unknown tags, a truncated
 * stream and a vertex count that the stream does not imply. */
int xfem_create(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                uint32_t idx_data_count, float density, const xfem_settings* settings, xfem_body** out);
int xfem_create_ex(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                   uint32_t idx_data_count, float density, const xfem_settings* settings,
                   const xfem_options* options, xfem_body** out);
/* Many independent bodies in one handle (the batched mode): one merged colour
 * schedule, one launch per frame. settings[i] per body (NULL = defaults). Body
 * b is addressed by index b in the per-body calls below. Replaces the
 * sequential per-body loop of Sim::Update (XPBDFEM/Demo.cpp:86-88). */
int xfem_batch_create(uint32_t nbodies, const xfem_mesh* meshes, const xfem_settings* settings,
                      const xfem_options* options, xfem_body** out);
int xfem_destroy(xfem_body* b);
int xfem_get_info(const xfem_body* b, xfem_info* out);

/* ---- parameters ---------------------------------------------------------- */
/* Replaces the UpdateSettings export (wasm/main.cpp:80-95) for one body. */
int xfem_set_settings(xfem_body* b, uint32_t body, const xfem_settings* s);
/* Per-vertex lock mask in caller order (1 = locked while XFEM_LOCK_LEFT is
 * set). At create time the mask is the reference's Left flag (x within 2% of
 * the minimum, XPBDFEM/Geo.cpp:724). As in the reference, a locked vertex
 * keeps a zero inverse mass from the first substep that locks it on. */
int xfem_set_lock_mask(xfem_body* b, uint32_t body, const uint8_t* mask);
/* Per-tet shear modulus mu_ref (caller tet order) in place of 1/compliance;
 * NULL returns to the uniform material. */
int xfem_set_tet_mu(xfem_body* b, uint32_t body, const float* mu);

/* ---- stepping ------------------------------------------------------------- */
/* One call of Geo3d::Substep (XPBDFEM/Geo.cpp:305-356) for every body:
 * predict, one coloured Gauss-Seidel sweep over all tets, locks, ground,
 * velocity update. */
int xfem_substep(xfem_body* b, float dt);
/* frames * substeps substeps in one launch (persistent kernel or one CUDA
 * graph), the loop of Sim::Update (XPBDFEM/Demo.cpp:67-90) with a fixed dt. */
int xfem_step_frames(xfem_body* b, uint32_t frames, uint32_t substeps, float dt);
/* No counterpart in the reference. The same stepping as xfem_step_frames
 * for callers that cannot allocate device memory when they step: a process
 * whose device memory is fully reserved by another allocator (a framework's
 * caching pool), or a real-time loop that must not take cudaMalloc's
 * device-wide synchronisation. It always runs the persistent kernel at the
 * handle's block size, never the autotuner or the CUDA-graph builder (which
 * may allocate), and calls no cudaMalloc, cudaFree or other allocating
 * routine. The kernel's scratch (the grid-barrier counter and the device
 * error word) lives in one fixed 256-byte device array that every GPU loading
 * the library keeps until exit; all calls share it, so calls whose kernels
 * overlap on one GPU race and must not be issued. The first call on a device
 * looks the array's device address up. Limit: one call's grid-barrier
 * arrivals, substeps x passes per substep (colours, times 1 + volume sweeps +
 * damping kinds when those run) x persistent blocks, must stay below 2^31
 * (else XFEM_ELIMIT; split the call). Hex, T10, H27 and mixed-mesh handles
 * step with their own scratch, allocated at create time. Synchronises the
 * handle's stream and reports device errors, so it is not a call to record
 * into a CUDA graph (no stream of the process may be capturing then). */
int xfem_step_frames_noalloc(xfem_body* b, uint32_t frames, uint32_t substeps, float dt);
/* Waits for queued work; returns XFEM_EDEVICE_TIMEOUT if a bounded device
 * wait ran out since the last check, XFEM_ENONFINITE if a finished position
 * or velocity was NaN or infinite. */
int xfem_synchronize(xfem_body* b);

/* ---- failure-detection test hooks --------------------------------------------- */
/* No counterpart in the reference, whose only checks are asserts
 * (XPBDFEM/Allocator.cpp:5-10, XPBDFEM/Connectivity.cpp:261-263). They make
 * the failures the library detects happen on purpose, without faulting the
 * GPU, so that the detection can be tested.
 *   XFEM_HOOK_MISSING_ARRIVAL (handle): the next stepping call's bounded
 *     device waits (grid barriers; neighbour-chunk waits in dataflow mode)
 *     expect `value` arrivals more than the blocks make, so they run out
 *     after the handle's wait_timeout_ms; the call (or the next synchronising
 *     one) reports XFEM_EDEVICE_TIMEOUT. One call only; the CUDA-graph launch
 *     form has no grid barrier and ignores it.
 *   XFEM_HOOK_BARRIER_BASE (handle): value 1 starts the grid-barrier arrival
 *     counter at 2^32 - 1 in every persistent launch, so the first barrier
 *     wraps it (the results must not change); 0 starts it at 0.
 *   XFEM_HOOK_FAIL_ALLOC (process-wide, b may be NULL): the value-th device
 *     buffer allocation from now on fails as if the device were full
 *     (XFEM_ENOMEM); 0 turns it off. */
#define XFEM_HOOK_MISSING_ARRIVAL 1u
#define XFEM_HOOK_BARRIER_BASE 2u
#define XFEM_HOOK_FAIL_ALLOC 3u
int xfem_test_hook(xfem_body* b, uint32_t hook, uint32_t value);

/* ---- reverse-mode adjoint ---------------------------------------------------- */
/* No counterpart in the reference, which only steps forward: the derivative
 * of Geo3d::Substep (XPBDFEM/Geo.cpp:305-356) as this library runs it, with
 * respect to each tet's shear modulus and the initial state. Only the coupled
 * Neo-Hookean model (energy 4 with the XPBD solve bit) is differentiated;
 * other settings give XFEM_EUNSUPPORTED.
 *
 * xfem_adjoint_forward steps `substeps` substeps of dt (the same results as
 * xfem_step_frames(b, 1, substeps, dt)) and records what the reverse pass
 * needs. Vertices and tets are numbered in the handle's concatenated caller
 * order (body 0's, then body 1's, ...). tip_traj (nullable):
 * substeps x ntips x 3 floats, the position of vertex tips[q] after each
 * substep. checkpoint_every = 0 keeps the tape of every substep on the
 * device; K > 0 keeps the state every K substeps and the tape of K substeps,
 * and the backward pass re-runs each segment forward once. */
int xfem_adjoint_forward(xfem_body* b, uint32_t substeps, float dt, uint32_t checkpoint_every, uint32_t ntips,
                         const uint32_t* tips, float* tip_traj);
/* Reverse pass of the last xfem_adjoint_forward. grad_tip_traj (required):
 * dL/d tip_traj. grad_x, grad_v (nullable = zero, 3 per vertex): dL/d the
 * positions and velocities at the end. Outputs (nullable): dmu (one per tet)
 * dL/dmu, with mu the tet's shear modulus (1/compliance or the value given
 * to xfem_set_tet_mu); dx0, dv0 (3 per vertex): dL/d the positions and
 * velocities at the start. The handle's state stays at the end of the
 * forward run. Synchronising. The reverse kernel takes one of two forms with
 * the same results bit for bit; XFEM_REVERSE_FORM=grouped or =lane in the
 * environment fixes the choice (diagnostics). */
int xfem_adjoint_backward(xfem_body* b, const float* grad_tip_traj, const float* grad_x, const float* grad_v,
                          float* dmu, float* dx0, float* dv0);

/* ---- state transfer (caller vertex order; synchronising) ------------------ */
/* Positions and velocities: 3 floats per vertex. A page-locked buffer
 * (xfem_alloc_host) is read or written by the device directly, with no
 * staging copy; any other buffer goes through the handle's device stage. */
int xfem_get_positions(xfem_body* b, uint32_t body, float* out_xyz);
int xfem_set_positions(xfem_body* b, uint32_t body, const float* xyz);
int xfem_get_velocities(xfem_body* b, uint32_t body, float* out_xyz);
int xfem_set_velocities(xfem_body* b, uint32_t body, const float* xyz);
/* Both at once, as the two calls above with one synchronisation. */
int xfem_set_state(xfem_body* b, uint32_t body, const float* xyz, const float* vel);
int xfem_get_inverse_masses(xfem_body* b, uint32_t body, float* out_w);
/* Ground-contact set of the last substep (1 = in contact). */
int xfem_get_contacts(xfem_body* b, uint32_t body, uint8_t* out);
/* Multipliers (lambda0, lambda1) of each tet in the last substep; needs
 * keep_lambdas at create time. */
int xfem_get_lambdas(xfem_body* b, uint32_t body, float* out_2nt);
/* GeoLinear3d::CalculateVolume (XPBDFEM/Geo.cpp:827-832), summed in double. */
int xfem_calculate_volume(xfem_body* b, uint32_t body, double* out);
/* Rest state per tet (caller order) as 17 floats: Qi column-major, QQ[3],
 * QR[3], volume, surfaceArea (ElementParamsLinearTet, XPBDFEM/Fem.h:52-60),
 * and the rest inverse masses. */
int xfem_get_rest_state(const xfem_body* b, uint32_t body, float* out_ep17, float* out_w);
/* The schedule: device rank of each vertex, the flattened Gauss-Seidel tet
 * order (colour-major, cluster, tet-in-cluster; caller tet ids) and the
 * offsets of each colour in it (ncolours + 1 entries). */
int xfem_get_schedule(const xfem_body* b, uint32_t body, uint32_t* vert_rank, uint32_t* tet_order,
                      uint32_t* colour_begin, uint32_t* ncolours);
/* Counts of one body: vertices, tets. */
int xfem_body_counts(const xfem_body* b, uint32_t body, uint32_t* nverts, uint32_t* ntets);

/* ---- host-only set-up (no GPU needed) --------------------------------------- */
/* The rest state GeoLinear3d::Init would compute for this mesh
 * (XPBDFEM/Geo.cpp:697-745): 17 floats per tet as in xfem_get_rest_state,
 * inverse masses, and vertex flags (bit 0 Left, bit 1 Right, bit 4 Pickable,
 * XPBDFEM/Geo.h:16-20). Any output may be NULL. */
int xfem_compute_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                            uint32_t idx_data_count, float density, float* out_ep17, float* out_w,
                            uint8_t* out_flags);
/* The schedule xfem_create_ex would build (cluster_mode and no_morton as in
 * xfem_options), in the form of xfem_get_schedule; colour_begin needs room
 * for tets + 1 entries. Any output may be NULL. */
int xfem_compute_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                          uint32_t idx_data_count, uint32_t cluster_mode, uint32_t no_morton, uint32_t* vert_rank,
                          uint32_t* tet_order, uint32_t* colour_begin, uint32_t* ncolours, uint32_t* nclusters);
/* The ring schedule of the continuous-pressure models (energy 8-10), whose
 * GeoLinear3d::Constrain solves one constraint pair per vertex over the tets
 * (or hexes) around it (XPBDFEM/Geo.cpp:147-225, 784-787; the vertex order vOrder,
 * XPBDFEM/Geo.cpp:759-771, is replaced by it): vertices coloured so that the
 * one-rings of a colour share no vertex, in caller ids, colour-major;
 * colour_begin needs room for vertices + 1 entries. Any output may be NULL.
 * xfem_get_ring_schedule reads a handle's (XFEM_EUNSUPPORTED for a body that
 * is not in one-ring mode); xfem_compute_ring_schedule computes the one
 * xfem_create_ex would build, without a GPU. A T10 or H27 body rings the
 * mesh's own vertices; two of its rings that share an added node share the
 * vertices of the edge, face or element it belongs to, so its schedule is the
 * one of the linear mesh (vert_order then lists mesh vertices only). */
int xfem_get_ring_schedule(const xfem_body* b, uint32_t body, uint32_t* vert_order, uint32_t* colour_begin,
                           uint32_t* ncolours);
int xfem_compute_ring_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                               uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_order,
                               uint32_t* colour_begin, uint32_t* ncolours);

/* ---- linear hexahedra (hex mode) --------------------------------------------- */
/* Elements of one body: its hexes, or its T10s for a T10 body (0 for a tet body). */
int xfem_body_hex_count(const xfem_body* b, uint32_t body, uint32_t* nhexes);
/* Rest state per hex (caller order) as 120 floats, ElementParamsLinearHex
 * (XPBDFEM/Fem.h:90-100) flattened: qcLo.Ji[0] column-major [0..8],
 * qcLo.w[0] [9], qcHi.Ji[p] [10 + 9p ..], qcHi.w[p] [82 + p], ic.QQ[7]
 * [90..96], ic.QR[21] [97..117], volume [118], surfaceArea [119]; and the
 * rest inverse masses. XFEM_EUNSUPPORTED for a tet body. */
int xfem_get_hex_rest_state(const xfem_body* b, uint32_t body, float* out_ep120, float* out_w);
/* The hex schedule: device rank of each vertex, the hex order (colour-major;
 * the hexes of one colour share no vertex) and the colour offsets in it
 * (ncolours + 1 entries, at most 4097). */
int xfem_get_hex_schedule(const xfem_body* b, uint32_t body, uint32_t* vert_rank, uint32_t* hex_order,
                          uint32_t* colour_begin, uint32_t* ncolours);
/* The same two, computed on the host without a handle or a GPU. */
int xfem_compute_hex_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, float density, float* out_ep120, float* out_w,
                                uint8_t* out_flags);
int xfem_compute_hex_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                              uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* hex_order,
                              uint32_t* colour_begin, uint32_t* ncolours);
/* GenerateHexBlock (XPBDFEM/MeshGen.cpp:156-221): nodes[3 (W+1)(H+1)(D+1)],
 * idx[9 W H D] (tag 8 and 8 vertex ids per hex). */
int xfem_generate_hex_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz,
                            uint32_t pattern, float wonkiness, float* nodes, uint32_t* idx);

/* ---- meshes mixing tets and hexes (mixed mode) --------------------------------
 * A body whose tagged stream holds tets (tag 4) and hexes (tag 8), as
 * GeoLinear3d::Init takes it (XPBDFEM/Geo.cpp:697-745): xfem_body_counts gives
 * its tets, xfem_body_hex_count its hexes, xfem_get_rest_state the tets' 17
 * floats each with the inverse masses of every vertex (the masses of all tets,
 * then all hexes, summed per vertex), xfem_get_hex_rest_state and
 * xfem_get_hex_schedule the hexes' records and colouring. The tets' own
 * colouring (colour-major; the tets of one colour share no vertex; caller tet
 * ids, colour offsets with ncolours + 1 entries, at most 4097), which replaces
 * the stream order of GeoLinear3d::Constrain's tet loop
 * (XPBDFEM/Geo.cpp:777-778): */
int xfem_get_mixed_tet_schedule(const xfem_body* b, uint32_t body, uint32_t* tet_order, uint32_t* colour_begin,
                                uint32_t* ncolours);
/* The same, computed on the host without a handle or a GPU: the rest state
 * (17 floats per tet, 120 per hex, inverse masses, vertex flags) and the
 * schedule (vertex ranks, the tet and the hex colourings). Any output may be
 * NULL; XFEM_EINVAL unless the stream holds both kinds. */
int xfem_compute_mixed_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                  uint32_t idx_data_count, float density, float* out_ep17, float* out_ep120,
                                  float* out_w, uint8_t* out_flags);
int xfem_compute_mixed_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* tet_order,
                                uint32_t* tet_colour_begin, uint32_t* tet_ncolours, uint32_t* hex_order,
                                uint32_t* hex_colour_begin, uint32_t* hex_ncolours);

/* ---- quadratic tets (T10 mode) ----------------------------------------------- */
/* T10s and edge nodes of one body; XFEM_EUNSUPPORTED for another body. The
 * xfem_*_t10_* queries also answer for the T10s of a mesh mixing tets and
 * hexes read as quadratic elements (their records, indices and colouring),
 * and the xfem_*_h27_* queries for its H27s; edge counts are the mesh's. */
int xfem_body_t10_count(const xfem_body* b, uint32_t body, uint32_t* nt10, uint32_t* nedges);
/* Rest state per T10 (caller tet order) as 56 floats, ElementParamsQuadraticTet
 * (XPBDFEM/Fem.h:61-69) flattened: Qi column-major [0..8], ic.QQ[9] [9..17],
 * ic.QR[36] [18..53], volume [54], surfaceArea [55]; the rest inverse masses
 * of all vertices; the 10 indices of each T10 (corners, then the edge nodes
 * of the local edges 01 02 03 12 13 23, XPBDFEM/Geo.cpp:893-901); the two
 * corners of each edge node. Any output may be NULL. */
int xfem_get_t10_rest_state(const xfem_body* b, uint32_t body, float* out_ep56, float* out_w, uint32_t* out_t10,
                            uint32_t* out_edges);
/* The T10 schedule: device rank of each vertex, the T10 order (colour-major;
 * the T10s of one colour share no vertex) and the colour offsets in it. */
int xfem_get_t10_schedule(const xfem_body* b, uint32_t body, uint32_t* vert_rank, uint32_t* t10_order,
                          uint32_t* colour_begin, uint32_t* ncolours);
/* Connectivity3d's edges of a tet index stream (XPBDFEM/Connectivity.cpp:
 * 371-393, 478-497) and the T10 indices: out_edges[2 per edge] (at most 6 per
 * tet), out_t10[10 per tet], *out_nedges. Outputs may be NULL (count first). */
int xfem_compute_t10_edges(const uint32_t* idx_data, uint32_t idx_data_count, uint32_t* out_edges,
                           uint32_t* out_t10, uint32_t* out_nedges);
/* GeoQuadratic3d::Init's rest state on the host: out_x the double rest
 * positions of all vertices (3 each: corners, then edge midpoints), the
 * 56-float records, inverse masses and vertex flags; and its schedule. */
int xfem_compute_t10_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, float density, double* out_x, float* out_ep56,
                                float* out_w, uint8_t* out_flags);
int xfem_compute_t10_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                              uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* t10_order,
                              uint32_t* colour_begin, uint32_t* ncolours);

/* ---- quadratic hexahedra (H27 mode) ----------------------------------------- */
/* A hex mesh whose settings carry element type H27 (or T10) in flags bits
 * 0-3 runs as GeoQuadratic3d on hexes (XPBDFEM/Geo.cpp:836-1053): a node on
 * every edge and face and at every hex centre, 27-node elements
 * (ElementParamsQuadraticHex, SolveElement with PointsLo = 8 and PointsHi =
 * 27). With the continuous-pressure models (8-10) one constraint pair per
 * one-ring of a mesh vertex over the H27s around it (XPBDFEM/Geo.cpp:944-953,
 * 973-982), up to 16 H27s and 128 nodes per ring. The body's vertices are the
 * mesh's own, then the edge, face and centre nodes. */
/* H27s, edge nodes and face nodes of one body; XFEM_EUNSUPPORTED for another body. */
int xfem_body_h27_count(const xfem_body* b, uint32_t body, uint32_t* nh27, uint32_t* nedges, uint32_t* nquads);
/* Rest state per H27 (caller hex order) as 703 floats, ElementParamsQuadraticHex
 * (XPBDFEM/Fem.h:101-111) flattened: qcLo.Ji[p] column-major [9p ..],
 * qcLo.w[p] [72 + p], qcHi.Ji[p] [80 + 9p ..], qcHi.w[p] [323 + p], ic.QQ[26]
 * [350..375], ic.QR[325] [376..700], volume [701], surfaceArea [702]; the
 * rest inverse masses of all vertices; the 27 indices of each H27 (node
 * i + 3j + 9k of its 3x3x3 grid, XPBDFEM/Geo.cpp:904-931). Outputs may be NULL. */
int xfem_get_h27_rest_state(const xfem_body* b, uint32_t body, float* out_ep703, float* out_w, uint32_t* out_h27);
int xfem_get_h27_schedule(const xfem_body* b, uint32_t body, uint32_t* vert_rank, uint32_t* h27_order,
                          uint32_t* colour_begin, uint32_t* ncolours);
/* Connectivity3d's edges (2 each, at most 12 per hex) and quads (4 each,
 * smallest vertex first, at most 6 per hex) of a hex index stream, and the
 * H27 indices (27 per hex). Outputs may be NULL (count first). */
int xfem_compute_h27_mesh(const uint32_t* idx_data, uint32_t idx_data_count, uint32_t* out_edges,
                          uint32_t* out_quads, uint32_t* out_h27, uint32_t* out_nedges, uint32_t* out_nquads);
/* GeoQuadratic3d::Init's rest state on a hex mesh without a GPU: out_x the
 * double rest positions of all vertices, the 703-float records, inverse
 * masses and flags; and its schedule. */
int xfem_compute_h27_rest_state(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                                uint32_t idx_data_count, float density, double* out_x, float* out_ep703,
                                float* out_w, uint8_t* out_flags);
int xfem_compute_h27_schedule(const float* node_data, uint32_t node_data_count, const uint32_t* idx_data,
                              uint32_t idx_data_count, uint32_t no_morton, uint32_t* vert_rank, uint32_t* h27_order,
                              uint32_t* colour_begin, uint32_t* ncolours);

/* ---- helpers --------------------------------------------------------------- */
/* volumeAndTimeCorrectedPbdDamping and its amortized form for a substep of
 * substep_dt and element spacing `spacing` (XPBDFEM/Demo.cpp:53-61, where
 * spacing is the demo's kSpacing): out[0], out[1]. */
int xfem_pbd_damping_coefficients(float pbd_damping, float substep_dt, float spacing, float* out2);
/* timeCorrectedDrag = 1 - (1 - drag)^(1000 sdt), XPBDFEM/Demo.cpp:63. */
float xfem_time_corrected_drag(float drag, float substep_dt);
/* GenerateTetBlock (XPBDFEM/MeshGen.cpp:156-244): a W x H x D block of cubes
 * with edge (sx, sy, sz), 6 tets per cube. nodes needs 3 (W+1)(H+1)(D+1)
 * floats, idx 30 W H D words. */
int xfem_generate_tet_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz,
                            uint32_t pattern, float wonkiness, float* nodes, uint32_t* idx);
/* Pinned host memory for fast transfers (cudaMallocHost / cudaFreeHost). */
void* xfem_alloc_host(size_t bytes);
void xfem_free_host(void* p);
/* Message of the last failing call on this thread ("" if none). */
const char* xfem_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* XFEM_H */
