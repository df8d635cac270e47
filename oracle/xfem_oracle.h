/*
 * xfem_oracle — CPU restatement of the reference's small-step XPBD tetrahedral
 * substep (jak-xyz/xpbd-fem), used ONLY as test infrastructure: by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline / reference arm, and
 * there only as the checker or as the timed CPU baseline. The shipped solver
 * (libxfem.so) never links, loads or calls anything in this directory.
 *
 * Parity status: PINNED. The float instantiation is checked bit-for-bit
 * against golden vectors produced by the unmodified reference code
 * (oracle/build_ref.sh + oracle/refgen.cpp -> tests/golden/), covering mesh
 * generation, rest state, per-element solves and whole substeps, on linear
 * tets and on linear hexahedra (oracle/xfem_oracle_hex.inc).
 *
 * Each routine is instantiated twice from oracle/xfem_oracle_real.inc:
 *   *_f : reference semantics — positions double, element arithmetic float,
 *         exactly the reference's operation order (compile with
 *         -ffp-contract=off so no multiply-add is fused);
 *   *_d : the same method with every quantity in double (the FP64 run that
 *         the FP32 paths are measured against).
 *
 * Extensions that the reference does not have (and whose parity is therefore
 * pinned only by this restatement and hand-derived cases): 3-D gravity,
 * parameterised Yeoh coefficients, per-tet shear modulus, an arbitrary
 * per-vertex lock mask, and a ground plane with Coulomb friction.
 *
 * The schedule routines (clusters, colours, Morton order) restate the
 * product's host algorithms independently so integer/index results can be
 * compared bit-exactly.
 */
#ifndef XFEM_ORACLE_H
#define XFEM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Energy model ids (XPBDFEM/Settings.h:41-53). On linear tets PixarReduced
 * equals Pixar and YeohSkinSel equals YeohSkin (one quadrature point either
 * way); the continuous-pressure ids 8-10 are per-vertex ring solves
 * (unsupported here); the cube ids 11-12 leave tets untouched; any id above
 * 12 runs MixedSel (XPBDFEM/Fem.cpp:885-887). */
#define ORC_ENERGY_PIXAR 0u
#define ORC_ENERGY_PIXAR_REDUCED 1u
#define ORC_ENERGY_PIXAR_SEL 2u
#define ORC_ENERGY_MIXED 3u
#define ORC_ENERGY_MIXED_SEL 4u
#define ORC_ENERGY_YEOH_SKIN 5u
#define ORC_ENERGY_YEOH_SKIN_SEL 6u
#define ORC_ENERGY_YEOH_SKIN_FAST 7u
#define ORC_ENERGY_CONTINUOUS_PIXAR 8u
#define ORC_ENERGY_CONTINUOUS_SKIN 10u
#define ORC_ENERGY_CUBE_NEO 11u
#define ORC_ENERGY_CUBE_SKIN 12u

/* Element parameter record, 17 values per tet, the reference's
 * ElementParamsLinearTet (XPBDFEM/Fem.h:52-60) flattened:
 * Qi column-major [0..8], QQ[9..11], QR[12..14], volume[15], surfaceArea[16]. */
#define ORC_EP 17

typedef struct orc_params {
	float gravity[3];        /* reference: vec2 (x, y) only, XPBDFEM/Settings.h:83 */
	float dt;
	float time_corrected_drag; /* XPBDFEM/Settings.h:97 */
	float compliance;        /* XPBDFEM/Settings.h:84 */
	float poisson;           /* XPBDFEM/Settings.h:88 */
	uint32_t energy;         /* ORC_ENERGY_* */
	uint32_t simultaneous;   /* Settings_XpbdSolveBit, XPBDFEM/Settings.h:15 */
	float yeoh[3];           /* reference hard-codes {0.1095, 14.95, 4.595} */
	uint32_t lock_active;    /* Settings_LockLeft: apply the lock mask */
	uint32_t ground;         /* extension: ground plane enabled */
	float ground_n[3];
	float ground_d;          /* plane dot(n, x) = d, solid where dot(n, x) < d */
	float friction;          /* Coulomb coefficient */
	/* Damping (XPBDFEM/Settings.h:85-86, 94-96, 102; XPBDFEM/Geo.cpp:346-355, 790-811) */
	float damping;             /* Settings::damping, the Rayleigh ratio; 0 = off */
	uint32_t rayleigh_type;    /* (flags >> 20) & 3: 0 Paper, 1 Limit (in the solve), 2 Post, 3 PostAmortized */
	float pbd_damping;         /* Settings::pbdDamping (> 0 enables PBD damping) */
	float pbd_coeff;           /* Settings::volumeAndTimeCorrectedPbdDamping */
	float pbd_coeff_amortized; /* Settings::amortizedVolumeAndTimeCorrectedPbdDamping */
	uint32_t tick;             /* Settings::tickId of the first substep; +1 per substep */
	uint32_t volume_passes;    /* Settings::volumePasses: SolveElementVolume sweeps after the solve */
	/* Settings_LockRight (XPBDFEM/Geo.cpp:323-331): vertices whose lock mask
	 * has bit 1 (the Right flag) end every substep at right_target (3 doubles
	 * per vertex, origin + lockedRightTransform3d X0, see orc_right_targets)
	 * with a zero inverse mass. Left vertices are those with bit 0. */
	uint32_t lock_right;
	const double* right_target;
} orc_params;

/* origin + m * vec3(X0) for every vertex in float, the reference's mat3 *
 * vec3 (rows dotted with the vector, XPBDFEM/vectormath.h:508-513) and vec3
 * addition (XPBDFEM/Geo.cpp:327); m column-major. out: 3 doubles per vertex. */
void orc_right_targets(uint32_t nv, const float* nodes, const float m[9], const float origin[3], double* out);

/* ---- mesh ---------------------------------------------------------------- */
/* GenerateTetBlock (XPBDFEM/MeshGen.cpp:156-244): nodes[3*(W+1)(H+1)(D+1)],
 * idx[5*6*W*H*D] (tagged stream, 4 = tet). */
void orc_gen_tet_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz,
                       uint32_t pattern, float wonkiness, float* nodes, uint32_t* idx);
/* Parse the tagged index stream (XPBDFEM/Connectivity.cpp:251-265). With
 * tets == NULL only counts. Returns 0, or -1 for a non-tet tag (hexes are
 * not supported by this path). */
int orc_parse_tets(const uint32_t* idx, uint32_t idx_count, uint32_t* tets,
                   uint32_t* tet_count, uint32_t* vert_count);
/* MINSTD shuffle of tet indices (XPBDFEM/Geo.cpp:759-771). */
void orc_minstd_order(uint32_t nt, uint32_t* order);

/* ---- rest state (GeoLinear3d::Init, XPBDFEM/Geo.cpp:697-745) -------------- */
void orc_init_rest_f(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt,
                     float density, float* ep, float* w, uint8_t* vflags);
void orc_init_rest_d(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt,
                     double density, double* ep, double* w, uint8_t* vflags);

/* ---- one element (SolveElement, XPBDFEM/Fem.cpp:892) ---------------------- */
/* X: 4x3 doubles, updated in place. O (nullable): the substep's start
 * positions, which the in-solve Rayleigh damping (types 0, 1) reads; without
 * O there is no damping term. mu_override <= 0 uses 1/compliance.
 * lambda_out (nullable) receives the two multipliers (the single-constraint
 * Pixar models: the one multiplier and 0). Returns 0 or -1 for an
 * unsupported energy model (the continuous-pressure ids 8-10). */
int orc_solve_tet_f(double* X, const double* O, const float* w, const float* ep, const orc_params* p,
                    float mu_override, float* lambda_out);
int orc_solve_tet_d(double* X, const double* O, const double* w, const double* ep, const orc_params* p,
                    double mu_override, double* lambda_out);

/* ---- substeps (Geo3d::Substep, XPBDFEM/Geo.cpp:305-356) ------------------- */
/* Runs nsub substeps, damping included (GeoLinear3d::Damp over the same
 * order). order[nt] is the constraint order (the reference's own
 * tOrder, or a coloured schedule flattened). w is updated in place (locks set
 * it to 0, as the reference does). tet_mu (nullable) gives a per-tet shear
 * modulus in place of 1/compliance. contact (nullable, nv) receives the
 * ground-contact set of the last substep. lambdas (nullable, 2*nt) receives
 * each tet's multipliers from the last substep. Returns 0 or -1. */
int orc_substeps_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask,
                   uint32_t nt, const uint32_t* tets, const float* ep, const float* tet_mu,
                   const uint32_t* order, uint32_t nsub, const orc_params* p,
                   uint8_t* contact, float* lambdas);
int orc_substeps_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask,
                   uint32_t nt, const uint32_t* tets, const double* ep, const double* tet_mu,
                   const uint32_t* order, uint32_t nsub, const orc_params* p,
                   uint8_t* contact, double* lambdas);
/* Same schedule, colours run with `threads` POSIX threads (tets of one colour
 * share no vertex, so the result equals the sequential run bit for bit).
 * Undamped settings without volume passes only (returns -1 otherwise).
 * colour_begin[ncolours+1] delimits colours inside `order`. */
int orc_substeps_threaded_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask,
                            uint32_t nt, const uint32_t* tets, const float* ep, const float* tet_mu,
                            const uint32_t* order, const uint32_t* colour_begin, uint32_t ncolours,
                            uint32_t nsub, const orc_params* p, uint32_t threads);

/* Substeps with a continuous-pressure model (energy 8-10; XPBDFEM/Geo.cpp:
 * 147-193, 774-811; XPBDFEM/Fem.cpp:942-979; XPBDFEM/Geo.cpp:12-64): each
 * substep solves every vertex's one-ring in `vorder` (nv), then the rings'
 * post-step Rayleigh damping in `vorder` and the PBD damping over the tets in
 * `torder` (nt). Returns 0, or -1 for another energy model. */
int orc_substeps_rings_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nt,
                         const uint32_t* tets, const float* ep, const uint32_t* torder, const uint32_t* vorder,
                         uint32_t nsub, const orc_params* p, uint8_t* contact);
int orc_substeps_rings_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nt,
                         const uint32_t* tets, const double* ep, const uint32_t* torder, const uint32_t* vorder,
                         uint32_t nsub, const orc_params* p, uint8_t* contact);

/* ---- linear hexahedra (oracle/xfem_oracle_hex.inc) ------------------------ */
/* Hex record, 120 values (the reference's ElementParamsLinearHex,
 * XPBDFEM/Fem.h:90-100, flattened): qcLo.Ji[0] column-major [0..8],
 * qcLo.w[0] [9], qcHi.Ji[p] [10 + 9p ..], qcHi.w[p] [82 + p], ic.QQ[7]
 * [90..96], ic.QR[21] [97..117], volume [118], surfaceArea [119]. */
#define ORC_EPH 120
/* GenerateHexBlock (XPBDFEM/MeshGen.cpp:156-221): nodes[3(W+1)(H+1)(D+1)],
 * idx[9 W H D] (tagged stream, 8 = hex). */
void orc_gen_hex_block(uint32_t W, uint32_t H, uint32_t D, float sx, float sy, float sz,
                       uint32_t pattern, float wonkiness, float* nodes, uint32_t* idx);
/* Hex-only tagged stream; -1 for any other tag. hexes == NULL only counts. */
int orc_parse_hexes(const uint32_t* idx, uint32_t idx_count, uint32_t* hexes,
                    uint32_t* hex_count, uint32_t* vert_count);
/* The hex tables as built: n8[8][8] (point, node), g8[8][8][3], g1[8][3]. */
void orc_hex_tables(float* n8, float* g8, float* g1);
/* The quadratic-tet tables as built: g4[4][10][3] (point, node, axis),
 * g10[10][10][3], w10[10]. */
void orc_t10_tables(float* g4, float* g10, float* w10);
/* GeoLinear3d::Init on a hex mesh (XPBDFEM/Geo.cpp:697-745, 736-740). */
void orc_hex_init_rest_f(const float* nodes, uint32_t nv, const uint32_t* hexes, uint32_t nh,
                         float density, float* ep, float* w, uint8_t* vflags);
void orc_hex_init_rest_d(const float* nodes, uint32_t nv, const uint32_t* hexes, uint32_t nh,
                         double density, double* ep, double* w, uint8_t* vflags);
/* SolveElement on one hex (XPBDFEM/Fem.cpp:896): X 8x3 doubles in place, O
 * (8x3) the substep's start, w[8]. Returns 0, or -1 for the ids the hex path
 * does not cover (8-10: the continuous-pressure models). */
int orc_solve_hex_f(double* X, const double* O, const float* w, const float* ep, const orc_params* p);
int orc_solve_hex_d(double* X, const double* O, const double* w, const double* ep, const orc_params* p);
/* Substeps of a hex mesh in the hex order `order` (GeoLinear3d::Constrain and
 * Damp's hex loops, XPBDFEM/Geo.cpp:774-811): solve, volume passes, locks and
 * velocities, post-step Rayleigh and PBD damping. Returns 0 or -1. */
int orc_hex_substeps_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nh,
                       const uint32_t* hexes, const float* ep, const uint32_t* order, uint32_t nsub,
                       const orc_params* p, uint8_t* contact);
int orc_hex_substeps_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nh,
                       const uint32_t* hexes, const double* ep, const uint32_t* order, uint32_t nsub,
                       const orc_params* p, uint8_t* contact);
/* Substeps of a hex mesh with a continuous-pressure model (energy 8-10):
 * every vertex's one-ring solved in `vorder` (SolveRing's hex branch,
 * XPBDFEM/Geo.cpp:147-225), the rings' post-step Rayleigh damping in
 * `vorder` and the PBD damping over the hexes in `horder`. Returns 0 or -1. */
int orc_hex_substeps_rings_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nh,
                             const uint32_t* hexes, const float* ep, const uint32_t* horder, const uint32_t* vorder,
                             uint32_t nsub, const orc_params* p, uint8_t* contact);
int orc_hex_substeps_rings_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nh,
                             const uint32_t* hexes, const double* ep, const uint32_t* horder, const uint32_t* vorder,
                             uint32_t nsub, const orc_params* p, uint8_t* contact);
/* CalculateVolume of a hex mesh (XPBDFEM/Geo.cpp:830, XPBDFEM/Fem.cpp:1046-1071). */
float orc_hex_volume_f(const double* X, uint32_t nh, const uint32_t* hexes, const float* ep);
double orc_hex_volume_d(const double* X, uint32_t nh, const uint32_t* hexes, const double* ep);

/* ---- meshes mixing tets and hexes (oracle/xfem_oracle_mixed.inc) ---------- */
int orc_parse_mixed(const uint32_t* idx, uint32_t idx_count, uint32_t* tets, uint32_t* tet_count, uint32_t* hexes,
                    uint32_t* hex_count, uint32_t* vert_count);
/* Elements of `per` vertices coloured and ordered as the hexes are
 * (orc_hex_schedule): a mixed mesh's tets take it with per = 4. */
int orc_elem_schedule(const float* nodes, uint32_t nv, const uint32_t* elems, uint32_t ne, uint32_t per, uint32_t morton,
                      uint32_t* vert_rank, uint32_t* order, uint32_t* colour_begin, uint32_t* ncolours);
/* GeoLinear3d::Init on a mixed stream: tet records (ORC_EP), hex records
 * (ORC_EPH), masses summed over the tets then the hexes, then inverted. */
void orc_mixed_init_rest_f(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, const uint32_t* hexes,
                           uint32_t nh, float density, float* ep, float* hep, float* w, uint8_t* vflags);
void orc_mixed_init_rest_d(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, const uint32_t* hexes,
                           uint32_t nh, double density, double* ep, double* hep, double* w, uint8_t* vflags);
/* Substeps of a mixed mesh: the tets in torder, then the hexes in horder, per
 * solve and per volume pass; Rayleigh damping over the tets then the hexes,
 * then PBD damping over both (XPBDFEM/Geo.cpp:777-811). Returns 0 or -1 (a
 * continuous-pressure model). */
int orc_mixed_substeps_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nt,
                         const uint32_t* tets, const float* ep, const uint32_t* torder, uint32_t nh, const uint32_t* hexes,
                         const float* hep, const uint32_t* horder, uint32_t nsub, const orc_params* p, uint8_t* contact);
int orc_mixed_substeps_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nt,
                         const uint32_t* tets, const double* ep, const uint32_t* torder, uint32_t nh,
                         const uint32_t* hexes, const double* hep, const uint32_t* horder, uint32_t nsub,
                         const orc_params* p, uint8_t* contact);
float orc_mixed_volume_f(const double* X, uint32_t nt, const uint32_t* tets, uint32_t nh, const uint32_t* hexes,
                         const float* hep);
double orc_mixed_volume_d(const double* X, uint32_t nt, const uint32_t* tets, uint32_t nh, const uint32_t* hexes,
                          const double* hep);

/* ---- quadratic tetrahedra (oracle/xfem_oracle_t10.inc) -------------------- */
/* T10 record, 56 values (ElementParamsQuadraticTet, XPBDFEM/Fem.h:61-68,
 * flattened): Qi column-major [0..8], ic.QQ[9] [9..17], ic.QR[36] [18..53],
 * volume [54], surfaceArea [55]. */
#define ORC_EPQ 56
/* The unique edges of a tet mesh as Connectivity3d::Init numbers them
 * (XPBDFEM/Connectivity.cpp:387-548): each tet files its edges (0,1) (0,2)
 * (0,3) (1,2) (1,3) (2,3) under their lower vertex in stream order; per
 * vertex, a duplicate is replaced by the list's last entry; edges are
 * numbered vertex by vertex. edges[2 e] = (lower, upper), capacity 12 nt.
 * t10 (nullable, 10 per tet): GeoQuadratic3d's element indices
 * (XPBDFEM/Geo.cpp:892-901): corners, then nv + EdgeFromVerts. */
int orc_tet_edges(const uint32_t* tets, uint32_t nt, uint32_t nv, uint32_t* edges, uint32_t* nedges, uint32_t* t10);
/* GeoQuadratic3d::Init on a tet mesh: X (double, nv + ne vertices), rest
 * state, inverse masses and flags of all vertices. */
void orc_t10_init_rest_f(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, const uint32_t* edges,
                         uint32_t ne, const uint32_t* t10, float density, double* X, float* ep, float* w,
                         uint8_t* vflags);
void orc_t10_init_rest_d(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, const uint32_t* edges,
                         uint32_t ne, const uint32_t* t10, double density, double* X, double* ep, double* w,
                         uint8_t* vflags);
/* SolveElement on one T10 (X 10x3, O the substep start); -1 for 8-10. */
int orc_solve_t10_f(double* X, const double* O, const float* w, const float* ep, const orc_params* p);
int orc_solve_t10_d(double* X, const double* O, const double* w, const double* ep, const orc_params* p);
/* Substeps of a T10 mesh in `order` (GeoQuadratic3d::Constrain and Damp's
 * tet loops, XPBDFEM/Geo.cpp:973-1006). */
/* Substeps of a T10 mesh with a continuous-pressure model (8-10): the rings
 * of the first ncorner nodes (the mesh's own vertices) in vorder, the PBD
 * damping over the T10s in torder (GeoQuadratic3d::Constrain and Damp,
 * XPBDFEM/Geo.cpp:971-1008). */
int orc_t10_substeps_rings_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nt,
                             const uint32_t* t10, const float* ep, const uint32_t* torder, const uint32_t* vorder,
                             uint32_t ncorner, uint32_t nsub, const orc_params* p, uint8_t* contact);
int orc_t10_substeps_rings_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nt,
                             const uint32_t* t10, const double* ep, const uint32_t* torder, const uint32_t* vorder,
                             uint32_t ncorner, uint32_t nsub, const orc_params* p, uint8_t* contact);
/* The same on an H27 mesh: rings over the H27s around each of the first
 * ncorner nodes, PBD damping over the H27s in horder. */
int orc_h27_substeps_rings_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nh,
                             const uint32_t* h27, const float* ep, const uint32_t* horder, const uint32_t* vorder,
                             uint32_t ncorner, uint32_t nsub, const orc_params* p, uint8_t* contact);
int orc_h27_substeps_rings_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nh,
                             const uint32_t* h27, const double* ep, const uint32_t* horder, const uint32_t* vorder,
                             uint32_t ncorner, uint32_t nsub, const orc_params* p, uint8_t* contact);
int orc_t10_substeps_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nt,
                       const uint32_t* t10, const float* ep, const uint32_t* order, uint32_t nsub,
                       const orc_params* p, uint8_t* contact);
int orc_t10_substeps_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nt,
                       const uint32_t* t10, const double* ep, const uint32_t* order, uint32_t nsub,
                       const orc_params* p, uint8_t* contact);
float orc_t10_volume_f(const double* X, uint32_t nt, const uint32_t* t10, const float* ep);
double orc_t10_volume_d(const double* X, uint32_t nt, const uint32_t* t10, const double* ep);
/* The T10 schedule: as orc_hex_schedule over 10-vertex elements; nodes are
 * all nv + ne vertex positions (float). */
int orc_t10_schedule(const float* nodes, uint32_t nv, const uint32_t* t10, uint32_t nt, uint32_t morton,
                     uint32_t* vert_rank, uint32_t* order, uint32_t* colour_begin, uint32_t* ncolours);

/* ---- quadratic hexahedra (H27) ---- */
/* ElementParamsQuadraticHex (XPBDFEM/Fem.h:101-111) flattened: qcLo.Ji[p]
 * [9p ..], qcLo.w[p] [72 + p], qcHi.Ji[p] [80 + 9p ..], qcHi.w[p] [323 + p],
 * ic.QQ[26] [350..375], ic.QR[325] [376..700], volume [701], surfaceArea
 * [702]. */
#define ORC_EPH27 703
/* The H27 tables: g8[8][27][3], g27[27][27][3], n27[27][27], the corner
 * map's gradients at the 27 points map27[27][8][3], w27[27]. */
void orc_h27_tables(float* g8, float* g27, float* n27, float* map27, float* w27);
/* Connectivity3d's edges (2 each, capacity 24 nh) and quads (4 each, the
 * smallest vertex first, capacity 24 nh) of a hex mesh, and GeoQuadratic3d's
 * H27 indices (27 per hex, nullable): corners, then nv + edge, nv + ne +
 * quad, nv + ne + nq + hex. */
/* Connectivity3d's edges and quads of a tagged stream mixing tets and hexes,
 * numbered as the reference numbers them, and GeoQuadratic3d's T10 (per tet)
 * and H27 (per hex) indices; t10 / h27 may be NULL. */
int orc_quad_mesh(const uint32_t* idx, uint32_t count, uint32_t nv, uint32_t* edges, uint32_t* nedges, uint32_t* quads,
                  uint32_t* nquads, uint32_t* t10, uint32_t* h27);
/* GeoQuadratic3d on a mesh mixing tets and hexes: rest state (all vertices'
 * positions X, T10 records ept, H27 records eph, inverse masses, flags),
 * substeps (T10s in torder, then H27s in horder) and CalculateVolume. */
void orc_qmixed_init_rest_f(const float* nodes, uint32_t nv, const uint32_t* edges, uint32_t ne, const uint32_t* quads,
                            uint32_t nq, const uint32_t* hexes, uint32_t nh, const uint32_t* tets, uint32_t nt,
                            const uint32_t* t10, const uint32_t* h27, float density, double* X, float* ept, float* eph,
                            float* w, uint8_t* vflags);
void orc_qmixed_init_rest_d(const float* nodes, uint32_t nv, const uint32_t* edges, uint32_t ne, const uint32_t* quads,
                            uint32_t nq, const uint32_t* hexes, uint32_t nh, const uint32_t* tets, uint32_t nt,
                            const uint32_t* t10, const uint32_t* h27, double density, double* X, double* ept,
                            double* eph, double* w, uint8_t* vflags);
int orc_qmixed_substeps_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nt,
                          const uint32_t* t10, const float* ept, const uint32_t* torder, uint32_t nh, const uint32_t* h27,
                          const float* eph, const uint32_t* horder, uint32_t nsub, const orc_params* p, uint8_t* contact);
int orc_qmixed_substeps_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nt,
                          const uint32_t* t10, const double* ept, const uint32_t* torder, uint32_t nh, const uint32_t* h27,
                          const double* eph, const uint32_t* horder, uint32_t nsub, const orc_params* p, uint8_t* contact);
float orc_qmixed_volume_f(const double* X, uint32_t nt, const uint32_t* t10, const float* ept, uint32_t nh,
                          const uint32_t* h27, const float* eph);
double orc_qmixed_volume_d(const double* X, uint32_t nt, const uint32_t* t10, const double* ept, uint32_t nh,
                           const uint32_t* h27, const double* eph);
int orc_h27_mesh(const uint32_t* hexes, uint32_t nh, uint32_t nv, uint32_t* edges, uint32_t* nedges, uint32_t* quads,
                 uint32_t* nquads, uint32_t* h27);
void orc_h27_init_rest_f(const float* nodes, uint32_t nv, const uint32_t* hexes, uint32_t nh, const uint32_t* edges,
                         uint32_t ne, const uint32_t* quads, uint32_t nq, const uint32_t* h27, float density, double* X,
                         float* ep, float* w, uint8_t* vflags);
void orc_h27_init_rest_d(const float* nodes, uint32_t nv, const uint32_t* hexes, uint32_t nh, const uint32_t* edges,
                         uint32_t ne, const uint32_t* quads, uint32_t nq, const uint32_t* h27, double density,
                         double* X, double* ep, double* w, uint8_t* vflags);
int orc_solve_h27_f(double* X, const double* O, const float* w, const float* ep, const orc_params* p);
int orc_solve_h27_d(double* X, const double* O, const double* w, const double* ep, const orc_params* p);
int orc_h27_substeps_f(uint32_t nv, double* X, double* V, float* w, const uint8_t* lock_mask, uint32_t nh,
                       const uint32_t* h27, const float* ep, const uint32_t* order, uint32_t nsub,
                       const orc_params* p, uint8_t* contact);
int orc_h27_substeps_d(uint32_t nv, double* X, double* V, double* w, const uint8_t* lock_mask, uint32_t nh,
                       const uint32_t* h27, const double* ep, const uint32_t* order, uint32_t nsub,
                       const orc_params* p, uint8_t* contact);
float orc_h27_volume_f(const double* X, uint32_t nh, const uint32_t* h27, const float* ep);
double orc_h27_volume_d(const double* X, uint32_t nh, const uint32_t* h27, const double* ep);
int orc_h27_schedule(const float* nodes, uint32_t nv, const uint32_t* h27, uint32_t nh, uint32_t morton,
                     uint32_t* vert_rank, uint32_t* order, uint32_t* colour_begin, uint32_t* ncolours);

/* CalculateVolume (XPBDFEM/Geo.cpp:827-832, XPBDFEM/Fem.cpp:1066). */
float orc_volume_f(const double* X, uint32_t nt, const uint32_t* tets);
double orc_volume_d(const double* X, uint32_t nt, const uint32_t* tets);

/* ---- FP64 adjoint (oracle/xfem_oracle_adjoint.c) ---------------------------- */
/* Forward nsub substeps in `order` with per-tet shear modulus tet_mu and the
 * loss sum_{s, q} |x_s[tips[q]] - targets[s][q]|^2 (s = state after substep
 * s + 1), then the reverse pass: dL/dmu per tet, dL/dV0 and dL/dX0 (3 nv each,
 * both nullable). With
 * dmu == NULL only the loss is computed. Coupled Neo-Hookean only. */
int orc_adjoint_d(uint32_t nv, const double* X0, const double* V0, const double* w0, const uint8_t* lock_mask,
                  uint32_t nt, const uint32_t* tets, const double* ep, const double* tet_mu, const uint32_t* order,
                  uint32_t nsub, const orc_params* p, uint32_t ntip, const uint32_t* tips, const double* targets,
                  double* loss, double* dmu, double* dV0, double* dX0);

/* ---- schedule restatement -------------------------------------------------- */
/* Edge-star clustering (mode 1) or one tet per cluster (mode 0); greedy
 * colouring of clusters; Morton vertex order (morton != 0) and the cluster
 * order inside each colour. Outputs (caller-allocated, sizes nt / nv / nt+1):
 *   cluster_of[nt], cluster_count, colour_of_cluster[nt], ncolours,
 *   vert_rank[nv] (new index of each vertex), tet_order[nt] (the flattened
 *   Gauss-Seidel order: colour-major, cluster, tet-in-cluster),
 *   colour_tet_begin[ncolours+1] (offsets into tet_order).
 * Returns 0, or -1 if a limit is exceeded. */
int orc_schedule(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt,
                 uint32_t mode, uint32_t morton,
                 uint32_t* cluster_of, uint32_t* cluster_count, uint32_t* colour_of_cluster,
                 uint32_t* ncolours, uint32_t* vert_rank, uint32_t* tet_order,
                 uint32_t* colour_tet_begin);

/* Ring schedule of the continuous-pressure models: vertices coloured greedily
 * in id order so that the rings of one colour share no node (the smallest
 * colour not used by an earlier vertex whose ring shares a node with this
 * one's), then ordered inside each colour by vertex rank (Morton rank of the
 * rest position with morton != 0, else the id). Outputs vorder[nv] (the
 * flattened ring order, colour-major), colour_begin[ncolours + 1] (caller
 * allocates nv + 1). Returns 0, or -1 if a limit is exceeded. */
int orc_ring_schedule(const float* nodes, uint32_t nv, const uint32_t* tets, uint32_t nt, uint32_t morton,
                      uint32_t* vorder, uint32_t* colour_begin, uint32_t* ncolours);
/* The same over elements of npe vertices each (4: tets, 8: hexes). */
int orc_ring_schedule_elems(const float* nodes, uint32_t nv, const uint32_t* elems, uint32_t npe, uint32_t ne,
                            uint32_t morton, uint32_t* vorder, uint32_t* colour_begin, uint32_t* ncolours);
/* The rings of the first ncentre vertices only, in the same form (vorder:
 * ncentre ids). */
int orc_ring_schedule_centres(const float* nodes, uint32_t nv, const uint32_t* elems, uint32_t npe, uint32_t ne,
                              uint32_t ncentre, uint32_t morton, uint32_t* vorder, uint32_t* colour_begin,
                              uint32_t* ncolours);

/* Hex schedule: hexes coloured greedily in id order so that the hexes of one
 * colour share no vertex (each takes the smallest colour not held by an
 * earlier hex sharing a vertex; at most 4096), then ordered inside each
 * colour by (Morton code of the centroid of their 8 vertices, id), or by id
 * with morton == 0. Outputs vert_rank[nv] (as orc_schedule's), hex_order[nh]
 * (colour-major) and colour_begin[ncolours + 1] (caller allocates nh + 1).
 * Returns 0, or -1 if more than 4096 colours are needed. */
int orc_hex_schedule(const float* nodes, uint32_t nv, const uint32_t* hexes, uint32_t nh, uint32_t morton,
                     uint32_t* vert_rank, uint32_t* hex_order, uint32_t* colour_begin, uint32_t* ncolours);

#ifdef __cplusplus
}
#endif
#endif
