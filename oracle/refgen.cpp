/*
 * refgen — golden-vector generator that drives the UNMODIFIED reference solver
 * core (jak-xyz/xpbd-fem, XPBDFEM/{Fem,Geo,Connectivity,Allocator,MeshGen,
 * vectormath,DebugGeo}.cpp) headless.
 *
 * Test infrastructure only. Built by oracle/build_ref.sh into oracle/_ref/ from
 * the reference sources where they lie; the reference is not copied or edited.
 * tests/golden/make_golden.py runs this binary and stores its output as the
 * committed fixtures that pin the oracle restatement (oracle/xfem_oracle.c)
 * and, through it, the GPU path.
 *
 * Output: a stream of named arrays on stdout, each record
 *   u32 name_len | name bytes | u8 dtype ('f','d','I','B') | u64 count | data
 *
 * Commands (argv[1]):
 *   meshgen W H D sx sy sz pattern wonkiness
 *       GenerateTetBlock (XPBDFEM/MeshGen.cpp:223) outputs: nodes, idx.
 *   init W H D sx sy sz pattern wonkiness density
 *       GeoLinear3d::Init (XPBDFEM/Geo.cpp:697): per-tet rest state
 *       (Qi, QQ, QR, volume, surfaceArea; XPBDFEM/Fem.cpp:196-224), inverse
 *       masses w, Left/Right flags, the MINSTD tet order tOrder
 *       (XPBDFEM/Geo.cpp:759-771) and CalculateVolume (XPBDFEM/Geo.cpp:827).
 *   solve seed count energy simultaneous compliance poisson dt
 *       SolveElement (XPBDFEM/Fem.cpp:892) on `count` seeded random tets:
 *       inputs (X, w, rest nodes) and outputs (X after the solve).
 *   substep W H D sx sy sz wonkiness density energy simultaneous compliance
 *           poisson gx gy dt nsub lockleft
 *       Geo3d::Substep (XPBDFEM/Geo.cpp:305) `nsub` times in the reference's
 *       own shuffled order; dumps X and V after 1 substep and after nsub.
 *   ordered W H D sx sy sz wonkiness density energy simultaneous compliance
 *           poisson gx gy dt nsub lockleft < order.u32
 *       Same substep, but the constraint loop runs SolveElement over the tet
 *       order read from stdin (u32 count, then the order) — the replicated
 *       Substep used for same-order parity with the coloured GPU schedule.
 *   damped W H D sx sy sz wonkiness density energy simultaneous compliance
 *          poisson gx gy dt nsub lockleft damping pbdDamping drag rayleighType
 *          spacing [volumePasses] < order.u32
 *       `ordered` with damping: Settings::damping, pbdDamping and drag, the
 *       Rayleigh type in flags bits 20-21, and the derived fields filled as
 *       Sim::Update does (XPBDFEM/Demo.cpp:53-63) with `spacing` in place of
 *       the demo's kSpacing; Geo3d::Substep then runs GeoLinear3d::Damp
 *       (XPBDFEM/Geo.cpp:346-355, 790-811) over the same order. Also dumps
 *       the derived values (volume- and time-corrected PBD damping, its
 *       amortized form, time-corrected drag). volumePasses (default 0) sets
 *       Settings::volumePasses: GeoLinear3d::Constrain then runs that many
 *       SolveElementVolume sweeps over the order after the solve
 *       (XPBDFEM/Geo.cpp:780-783).
 *   locked (arguments as `damped`, volumePasses given) m00 m01 m02 m10 m11 m12
 *          m20 m21 m22 ox oy oz < order.u32
 *       `damped` with Settings_LockRight: Settings::lockedRightTransform3d
 *       (column-major) and Geo3d::origin set as given; Geo3d::Substep then
 *       holds the Right vertices at origin + m X0 (XPBDFEM/Geo.cpp:323-331).
 *   rings  (arguments as `damped`) < torder.u32 vorder.u32
 *       `damped` with a continuous-pressure energy (8-10): stdin holds the
 *       tet order and then the vertex order (each u32 count, then the ids),
 *       which replace tOrder and vOrder; GeoLinear3d::Constrain then solves
 *       the one-rings in that vertex order (XPBDFEM/Geo.cpp:784-787) and
 *       GeoLinear3d::Damp damps them in it (XPBDFEM/Geo.cpp:800-806).
 *
 *   mixed density energy simultaneous compliance poisson gx gy dt nsub lockleft
 *         damping pbdDamping drag rayleighType spacing volumePasses
 *         < mesh order.u32
 *       GeoLinear3d::Init on the tagged stream read from stdin (u32 node
 *       count, the floats, u32 index count, the words), which may mix tets
 *       and hexes; dumps the tet records (as `init`), the hex records (as
 *       `hinit`), w and the flags; then reads the tet order and the hex
 *       order (each u32 count, then the ids) into tOrder and hOrder and runs
 *       Geo3d::Substep as `damped` does: every tet, then every hex
 *       (XPBDFEM/Geo.cpp:777-811).
 *   qmixed (the arguments and stdin of `mixed`)
 *       GeoQuadratic3d::Init on the same stream (XPBDFEM/Geo.cpp:836-953):
 *       every vertex position (corners, edge midpoints, quad centres, hex
 *       centres), the T10 and H27 indices and records, w and the flags;
 *       then the T10 order and the H27 order into tOrder and hOrder and
 *       Geo3d::Substep: every T10, then every H27 (XPBDFEM/Geo.cpp:955-1008).
 *
 * Linear hexahedra: the same commands prefixed with `h` run on a
 * GenerateHexBlock mesh (XPBDFEM/MeshGen.cpp:156-221) and always take the
 * element pattern after the scale:
 *   hmeshgen / hinit W H D sx sy sz pattern wonkiness [density]
 *       hinit dumps the per-hex rest state (qcLo, qcHi, ic, volume,
 *       surfaceArea; InitQuadHexFiniteElement, XPBDFEM/Fem.cpp:225-265),
 *       w, the flags, the MINSTD hex order hOrder and CalculateVolume.
 *   hordered / hdamped W H D sx sy sz pattern wonkiness density ...
 *       (the rest as `ordered` / `damped`) < horder.u32
 *       the order read from stdin replaces hOrder; GeoLinear3d::Constrain
 *       and Damp then run their hex loops (XPBDFEM/Geo.cpp:777-811).
 *   hsolve seed count energy simultaneous compliance poisson dt
 *       SolveElement (XPBDFEM/Fem.cpp:896) on `count` seeded random hexes.
 *
 * Quadratic tets: the same commands prefixed with `q` build GeoQuadratic3d
 * (XPBDFEM/Geo.cpp:836-1053) on a GenerateTetBlock mesh, pattern after the
 * scale:
 *   qinit W H D sx sy sz pattern wonkiness density
 *       all vertex positions (corners, then edge midpoints), the T10 indices,
 *       the per-T10 rest state (Qi, ic.QQ[9], ic.QR[36], volume,
 *       surfaceArea), w, flags, tOrder and CalculateVolume.
 *   qordered / qdamped (as hordered / hdamped) < torder.u32
 *   qrings (as qdamped, with a continuous-pressure energy 8-10) < torder.u32 vorder.u32
 *       the vertex order (the mesh's own vertices) replaces vOrder:
 *       GeoQuadratic3d::Constrain solves their rings over the T10s in it
 *       and Damp damps them in it (XPBDFEM/Geo.cpp:971-1008).
 *   qsolve seed count energy simultaneous compliance poisson dt
 *       SolveElement (XPBDFEM/Fem.cpp:893) on `count` seeded random T10s.
 *
 * Quadratic hexes: the same commands prefixed with `Q` build GeoQuadratic3d
 * on a GenerateHexBlock mesh (H27s, XPBDFEM/Geo.cpp:902-933):
 *   Qinit W H D sx sy sz pattern wonkiness density
 *       all vertex positions (corners, edge midpoints, face centres, hex
 *       centres), the H27 indices, the per-H27 rest state (703 values:
 *       qcLo.Ji[8], qcLo.w[8], qcHi.Ji[27], qcHi.w[27], ic.QQ[26],
 *       ic.QR[325], volume, surfaceArea), w, flags, hOrder and
 *       CalculateVolume.
 *   Qordered / Qdamped (as hordered / hdamped) < horder.u32
 *   Qrings (as Qdamped, energy 8-10) < horder.u32 vorder.u32 (as qrings)
 *   Qsolve seed count energy simultaneous compliance poisson dt
 *       SolveElement (XPBDFEM/Fem.cpp:897) on `count` seeded random H27s.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>

#include "Allocator.h"
#include "Geo.h"
#include "Fem.h"
#include "MeshGen.h"
#include "Manipulator.h"
#include "Settings.h"

// Non-static in XPBDFEM/MeshGen.cpp:223 but not declared in MeshGen.h.
void GenerateTetBlock(Allocator* alloc, uint32_t width, uint32_t height, uint32_t depth, vec3 scale,
                      uint32_t elementPattern, float wonkiness, const float** outNodeData,
                      uint32_t* outNodeDataCount, const uint32_t** outIdxData, uint32_t* outIdxDataCount);
// Non-static in XPBDFEM/MeshGen.cpp:156 but not declared in MeshGen.h.
void GenerateHexBlock(Allocator* alloc, uint32_t width, uint32_t height, uint32_t depth, vec3 scale,
                      uint32_t elementPattern, float wonkiness, const float** outNodeData,
                      uint32_t* outNodeDataCount, const uint32_t** outIdxData, uint32_t* outIdxDataCount);

static void emit(const char* name, char dtype, const void* data, uint64_t count) {
	uint32_t n = (uint32_t)strlen(name);
	fwrite(&n, 4, 1, stdout);
	fwrite(name, 1, n, stdout);
	fwrite(&dtype, 1, 1, stdout);
	fwrite(&count, 8, 1, stdout);
	size_t es = dtype == 'd' ? 8 : dtype == 'B' ? 1 : 4;
	if (count) fwrite(data, es, count, stdout);
}

// splitmix64: the project's seeded generator for harness inputs.
static uint64_t g_rng;
static uint64_t splitmix64() {
	uint64_t z = (g_rng += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}
static double urand() { return (double)(splitmix64() >> 11) * (1.0 / 9007199254740992.0); }

static Allocator* make_alloc(size_t bytes) {
	Allocator* a = new Allocator();
	a->Initialize(malloc(bytes), bytes);
	return a;
}

static Settings make_settings(uint32_t energy, uint32_t simultaneous, float compliance, float poisson,
                              float gx, float gy, uint32_t lockLeft) {
	Settings s;
	s.timeScale = 1.0f;
	s.substepsPerSecond = 1200.0f;
	s.volumePasses = 0;
	s.gravity = vec2(gx, gy);
	s.compliance = compliance;
	s.damping = 0.0f;
	s.pbdDamping = 0.0f;
	s.drag = 0.0f;
	s.poissonsRatio = poisson;
	s.wonkiness = 0.0f;
	s.leftRightSeparation = 1.0f;
	s.flags = (energy << Settings_EnergyBit) | (simultaneous ? (1u << Settings_XpbdSolveBit) : 0u) |
	          (Rayleigh_Post << Settings_RayleighTypeBit) | (lockLeft ? Settings_LockLeft : 0u) |
	          (Element_T4 << Settings_ElementTypeBit);
	// Derived fields (XPBDFEM/Settings.h:93-101) have no initialisers; Sim::Update
	// (XPBDFEM/Demo.cpp:53-63) fills them. With drag = pbdDamping = 0 they are 0.
	s.areaAndTimeCorrectedPbdDamping = 0.0f;
	s.volumeAndTimeCorrectedPbdDamping = 0.0f;
	s.amortizedAreaAndTimeCorrectedPbdDamping = 0.0f;
	s.amortizedVolumeAndTimeCorrectedPbdDamping = 0.0f;
	s.timeCorrectedDrag = 0.0f;
	s.lockedRightTransform = mat2(1.0f);
	s.lockedRightTransform3d = mat3(1.0f);
	s.tickId = 0;
	return s;
}

// Settings::damping, pbdDamping, drag and the Rayleigh type, with the derived
// fields filled as Sim::Update does (XPBDFEM/Demo.cpp:53-63, `spacing` for
// kSpacing); emits the derived values.
static void set_damping(Settings& s, float dt, float damping, float pbd, float drag, uint32_t rtype, float spacing) {
	s.damping = damping;
	s.pbdDamping = pbd;
	s.drag = drag;
	s.flags = (s.flags & ~(Settings_RayleighTypeMask << Settings_RayleighTypeBit)) | (rtype << Settings_RayleighTypeBit);
	const float sdt = dt;
	float tcpd = 1.0f - pow(1.0f - s.pbdDamping, 1000.0f * sdt);
	s.areaAndTimeCorrectedPbdDamping = tcpd * spacing * spacing;
	s.volumeAndTimeCorrectedPbdDamping = tcpd * 6.0f * spacing * spacing;
	float atcpd = 1.0f - pow(1.0f - s.pbdDamping, 1000.0f * (float)AmortizationPeriod * sdt);
	s.amortizedAreaAndTimeCorrectedPbdDamping = atcpd * spacing * spacing;
	s.amortizedVolumeAndTimeCorrectedPbdDamping = atcpd * 6.0f * spacing * spacing;
	s.timeCorrectedDrag = 1.0f - pow(1.0f - s.drag, 1000.0f * sdt);
	const float derived[3] = {s.volumeAndTimeCorrectedPbdDamping, s.amortizedVolumeAndTimeCorrectedPbdDamping,
	                          s.timeCorrectedDrag};
	emit("derived", 'f', derived, 3);
}

static void dump_geo(GeoLinear3d* g) {
	uint32_t nt = g->con.tetCount, nv = g->vertCount;
	std::vector<float> ep(nt * 17);
	std::vector<uint32_t> tidx(nt * 4);
	for (uint32_t i = 0; i < nt; i++) {
		const ElementParamsLinearTet& e = g->t[i].ep;
		float* o = &ep[i * 17];
		for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[c * 3 + r] = e.Qi[c][r];
		for (int k = 0; k < 3; k++) o[9 + k] = e.ic.QQ[k];
		for (int k = 0; k < 3; k++) o[12 + k] = e.ic.QR[k];
		o[15] = e.volume;
		o[16] = e.surfaceArea;
		for (int k = 0; k < 4; k++) tidx[i * 4 + k] = g->t[i].i[k];
	}
	std::vector<uint8_t> flags(g->flags, g->flags + nv);
	emit("tet_idx", 'I', tidx.data(), tidx.size());
	emit("ep", 'f', ep.data(), ep.size());
	emit("w", 'f', g->w, nv);
	emit("vflags", 'B', flags.data(), nv);
	emit("torder", 'I', g->tOrder, nt);
	float vol = g->CalculateVolume();
	emit("volume", 'f', &vol, 1);
}

// ElementParamsLinearHex (XPBDFEM/Fem.h:90-100) flattened, 120 values per hex:
// qcLo.Ji[0] column-major, qcLo.w[0], qcHi.Ji[0..7], qcHi.w[0..7], ic.QQ[7],
// ic.QR[21], volume, surfaceArea.
static void hex_record(const ElementParamsLinearHex& e, float* o) {
	for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[c * 3 + r] = e.qcLo.Ji[0][c][r];
	o[9] = e.qcLo.w[0];
	for (int p = 0; p < 8; p++)
		for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[10 + 9 * p + c * 3 + r] = e.qcHi.Ji[p][c][r];
	for (int p = 0; p < 8; p++) o[82 + p] = e.qcHi.w[p];
	for (int k = 0; k < 7; k++) o[90 + k] = e.ic.QQ[k];
	for (int k = 0; k < 21; k++) o[97 + k] = e.ic.QR[k];
	o[118] = e.volume;
	o[119] = e.surfaceArea;
}

static void dump_hex_geo(GeoLinear3d* g) {
	uint32_t nh = g->con.hexCount, nv = g->vertCount;
	std::vector<float> ep(nh * 120);
	std::vector<uint32_t> hidx(nh * 8);
	for (uint32_t i = 0; i < nh; i++) {
		hex_record(g->h[i].ep, &ep[i * 120]);
		for (int k = 0; k < 8; k++) hidx[i * 8 + k] = g->h[i].i[k];
	}
	std::vector<uint8_t> flags(g->flags, g->flags + nv);
	emit("hex_idx", 'I', hidx.data(), hidx.size());
	emit("hep", 'f', ep.data(), ep.size());
	emit("w", 'f', g->w, nv);
	emit("vflags", 'B', flags.data(), nv);
	emit("horder", 'I', g->hOrder, nh);
	float vol = g->CalculateVolume();
	emit("volume", 'f', &vol, 1);
}

// ElementParamsQuadraticTet (XPBDFEM/Fem.h:61-68) flattened, 56 values.
static void t10_record(const ElementParamsQuadraticTet& e, float* o) {
	for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[c * 3 + r] = e.Qi[c][r];
	for (int k = 0; k < 9; k++) o[9 + k] = e.ic.QQ[k];
	for (int k = 0; k < 36; k++) o[18 + k] = e.ic.QR[k];
	o[54] = e.volume;
	o[55] = e.surfaceArea;
}

// ElementParamsQuadraticHex (XPBDFEM/Fem.h:101-111) flattened, 703 values.
static void h27_record(const ElementParamsQuadraticHex& e, float* o) {
	for (int p = 0; p < 8; p++)
		for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[9 * p + c * 3 + r] = e.qcLo.Ji[p][c][r];
	for (int p = 0; p < 8; p++) o[72 + p] = e.qcLo.w[p];
	for (int p = 0; p < 27; p++)
		for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[80 + 9 * p + c * 3 + r] = e.qcHi.Ji[p][c][r];
	for (int p = 0; p < 27; p++) o[323 + p] = e.qcHi.w[p];
	for (int k = 0; k < 26; k++) o[350 + k] = e.ic.QQ[k];
	for (int k = 0; k < 325; k++) o[376 + k] = e.ic.QR[k];
	o[701] = e.volume;
	o[702] = e.surfaceArea;
}

template <typename G>
static void dump_state(G* g, const char* xname, const char* vname) {
	uint32_t nv = g->vertCount;
	std::vector<double> x(nv * 3), v(nv * 3);
	for (uint32_t i = 0; i < nv; i++)
		for (int k = 0; k < 3; k++) { x[i * 3 + k] = g->X[i][k]; v[i * 3 + k] = g->V[i][k]; }
	emit(xname, 'd', x.data(), x.size());
	emit(vname, 'd', v.data(), v.size());
}

int main(int argc, char** argv) {
	if (argc < 2) { fprintf(stderr, "usage: refgen <cmd> ...\n"); return 2; }
	const bool hex = argv[1][0] == 'h', quad = argv[1][0] == 'q', h27 = argv[1][0] == 'Q';
	const char* cmd = argv[1] + (hex || quad || h27 ? 1 : 0);
	auto U = [&](int i) { return (uint32_t)strtoul(argv[i], 0, 10); };
	auto F = [&](int i) { return (float)strtod(argv[i], 0); };

	if ((quad || h27) &&
	    (!strcmp(cmd, "init") || !strcmp(cmd, "ordered") || !strcmp(cmd, "damped") || !strcmp(cmd, "rings"))) {
		Allocator* alloc = make_alloc((size_t)1 << 31);
		uint32_t W = U(2), H = U(3), D = U(4);
		vec3 scale(F(5), F(6), F(7));
		uint32_t pattern = U(8);
		float wonk = F(9), density = F(10);
		int a = 11;
		const float* nodes; uint32_t nodeCount; const uint32_t* idx; uint32_t idxCount;
		if (h27)
			GenerateHexBlock(alloc, W, H, D, scale, pattern, wonk, &nodes, &nodeCount, &idx, &idxCount);
		else
			GenerateTetBlock(alloc, W, H, D, scale, pattern, wonk, &nodes, &nodeCount, &idx, &idxCount);
		GeoQuadratic3d* g = alloc->New<GeoQuadratic3d>();
		g->Init(alloc, density, nodes, nodeCount, idx, idxCount, false);
		emit("nodes", 'f', nodes, nodeCount);
		emit("idx", 'I', idx, idxCount);
		if (h27 && !strcmp(cmd, "init")) {
			uint32_t nh = g->con.hexCount, nv = g->vertCount;
			std::vector<float> ep(nh * 703);
			std::vector<uint32_t> hi(nh * 27);
			for (uint32_t i = 0; i < nh; i++) {
				h27_record(g->h[i].ep, &ep[i * 703]);
				for (int k = 0; k < 27; k++) hi[i * 27 + k] = g->h[i].i[k];
			}
			std::vector<double> x0(nv * 3);
			for (uint32_t i = 0; i < nv; i++) for (int k = 0; k < 3; k++) x0[i * 3 + k] = g->X[i][k];
			std::vector<uint8_t> flags(g->flags, g->flags + nv);
			emit("x0", 'd', x0.data(), x0.size());
			emit("h27_idx", 'I', hi.data(), hi.size());
			emit("h27ep", 'f', ep.data(), ep.size());
			emit("w", 'f', g->w, nv);
			emit("vflags", 'B', flags.data(), nv);
			emit("horder", 'I', g->hOrder, nh);
			float vol = g->CalculateVolume();
			emit("volume", 'f', &vol, 1);
			return 0;
		}
		if (!strcmp(cmd, "init")) {
			uint32_t nt = g->con.tetCount, nv = g->vertCount;
			std::vector<float> ep(nt * 56);
			std::vector<uint32_t> ti(nt * 10);
			for (uint32_t i = 0; i < nt; i++) {
				t10_record(g->t[i].ep, &ep[i * 56]);
				for (int k = 0; k < 10; k++) ti[i * 10 + k] = g->t[i].i[k];
			}
			std::vector<double> x0(nv * 3);
			for (uint32_t i = 0; i < nv; i++) for (int k = 0; k < 3; k++) x0[i * 3 + k] = g->X[i][k];
			std::vector<uint8_t> flags(g->flags, g->flags + nv);
			emit("x0", 'd', x0.data(), x0.size());
			emit("t10_idx", 'I', ti.data(), ti.size());
			emit("qep", 'f', ep.data(), ep.size());
			emit("w", 'f', g->w, nv);
			emit("vflags", 'B', flags.data(), nv);
			emit("torder", 'I', g->tOrder, nt);
			float vol = g->CalculateVolume();
			emit("volume", 'f', &vol, 1);
			return 0;
		}
		uint32_t energy = U(a++), simul = U(a++);
		float compliance = F(a++), poisson = F(a++), gx = F(a++), gy = F(a++), dt = F(a++);
		uint32_t nsub = U(a++), lockLeft = U(a++);
		Settings s = make_settings(energy, simul, compliance, poisson, gx, gy, lockLeft);
		s.flags = (s.flags & ~(Settings_ElementTypeMask << Settings_ElementTypeBit)) |
		          ((h27 ? Element_H27 : Element_T10) << Settings_ElementTypeBit);
		if (!strcmp(cmd, "damped") || !strcmp(cmd, "rings")) {
			s.damping = F(a++);
			s.pbdDamping = F(a++);
			s.drag = F(a++);
			const uint32_t rtype = U(a++);
			const float spacing = F(a++);
			s.flags = (s.flags & ~(Settings_RayleighTypeMask << Settings_RayleighTypeBit)) | (rtype << Settings_RayleighTypeBit);
			const float sdt = dt;
			float tcpd = 1.0f - pow(1.0f - s.pbdDamping, 1000.0f * sdt);
			s.areaAndTimeCorrectedPbdDamping = tcpd * spacing * spacing;
			s.volumeAndTimeCorrectedPbdDamping = tcpd * 6.0f * spacing * spacing;
			float atcpd = 1.0f - pow(1.0f - s.pbdDamping, 1000.0f * (float)AmortizationPeriod * sdt);
			s.amortizedAreaAndTimeCorrectedPbdDamping = atcpd * spacing * spacing;
			s.amortizedVolumeAndTimeCorrectedPbdDamping = atcpd * 6.0f * spacing * spacing;
			s.timeCorrectedDrag = 1.0f - pow(1.0f - s.drag, 1000.0f * sdt);
			const float derived[3] = {s.volumeAndTimeCorrectedPbdDamping, s.amortizedVolumeAndTimeCorrectedPbdDamping,
			                          s.timeCorrectedDrag};
			emit("derived", 'f', derived, 3);
			if (a < argc) s.volumePasses = U(a++);
		}
		uint32_t n = 0;
		const uint32_t nel = h27 ? g->con.hexCount : g->con.tetCount;
		if (fread(&n, 4, 1, stdin) != 1 || n != nel) { fprintf(stderr, "bad order\n"); return 3; }
		if (fread(h27 ? g->hOrder : g->tOrder, 4, n, stdin) != n) { fprintf(stderr, "short order\n"); return 3; }
		if (!strcmp(cmd, "rings")) {
			// the rings of the mesh's own vertices, in the order read
			if (fread(&n, 4, 1, stdin) != 1 || n != g->con.vertCount) { fprintf(stderr, "bad vertex order\n"); return 3; }
			if (fread(g->vOrder, 4, n, stdin) != n) { fprintf(stderr, "short vertex order\n"); return 3; }
		}
		Manipulator manip;
		manip.pickedGeo = nullptr;
		for (uint32_t k = 0; k < nsub; k++) {
			s.tickId = k;
			g->Substep(s, manip, dt);
			if (k == 0) dump_state(g, "x1", "v1");
		}
		dump_state(g, "xn", "vn");
		float vol = g->CalculateVolume();
		emit("volume", 'f', &vol, 1);
		return 0;
	}

	if (quad && !strcmp(cmd, "solve")) {
		g_rng = strtoull(argv[2], 0, 10);
		uint32_t count = U(3), energy = U(4), simul = U(5);
		float compliance = F(6), poisson = F(7), dt = F(8);
		Settings s = make_settings(energy, simul, compliance, poisson, 0.0f, 0.0f, 0);
		std::vector<double> xin(count * 30), xout(count * 30), rest(count * 30);
		std::vector<float> win(count * 10), epo(count * 56);
		static const int te[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
		for (uint32_t t = 0; t < count; t++) {
			dvec3 X0[10], X[10], O[10];
			float m[10] = {0}, w[10];
			// corners as the linear `solve` command's random tet, midpoints on the edges
			double sc = 0.02 + 0.2 * urand();
			for (int n = 0; n < 4; n++) X0[n] = dvec3(sc * (urand() - 0.5), sc * (urand() - 0.5), sc * (urand() - 0.5));
			X0[0] = X0[3] + dvec3(sc * (0.6 + 0.4 * urand()), 0.1 * sc * (urand() - 0.5), 0.1 * sc * (urand() - 0.5));
			X0[1] = X0[3] + dvec3(0.1 * sc * (urand() - 0.5), sc * (0.6 + 0.4 * urand()), 0.1 * sc * (urand() - 0.5));
			X0[2] = X0[3] + dvec3(0.1 * sc * (urand() - 0.5), 0.1 * sc * (urand() - 0.5), sc * (0.6 + 0.4 * urand()));
			for (int n = 0; n < 4; n++) for (int k = 0; k < 3; k++) X0[n][k] = (double)(float)X0[n][k];
			for (int e = 0; e < 6; e++) X0[4 + e] = 0.5 * (X0[te[e][0]] + X0[te[e][1]]);
			const uint32_t is[10] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9};
			ElementParamsQuadraticTet ep;
			InitFiniteElement(X0, is, 1000.0f, m, &ep);
			uint32_t kind = t % 8;
			double amp = kind < 4 ? 0.05 : kind < 6 ? 0.4 : 1.5;
			for (int n = 0; n < 10; n++) {
				for (int k = 0; k < 3; k++) X[n][k] = X0[n][k] + amp * sc * (urand() - 0.5);
				O[n] = X0[n];
				w[n] = (float)(0.5 + 2.0 * urand());
			}
			if (kind == 6) { dvec3 tmp = X[0]; X[0] = X[1]; X[1] = tmp; }
			if (kind == 7) { w[0] = 0.0f; w[9] = 0.0f; }
			for (int n = 0; n < 10; n++) {
				win[t * 10 + n] = w[n];
				for (int k = 0; k < 3; k++) { xin[t * 30 + n * 3 + k] = X[n][k]; rest[t * 30 + n * 3 + k] = X0[n][k]; }
			}
			SolveElement(dt, X, O, w, is, ep, s);
			for (int n = 0; n < 10; n++) for (int k = 0; k < 3; k++) xout[t * 30 + n * 3 + k] = X[n][k];
			t10_record(ep, &epo[t * 56]);
		}
		emit("rest", 'd', rest.data(), rest.size());
		emit("qep", 'f', epo.data(), epo.size());
		emit("xin", 'd', xin.data(), xin.size());
		emit("w", 'f', win.data(), win.size());
		emit("xout", 'd', xout.data(), xout.size());
		return 0;
	}

	if (!strcmp(cmd, "mixed")) {
		// the mesh, then the tet order and the hex order, from stdin
		Allocator* alloc = make_alloc((size_t)1 << 31);
		auto rd = [&](void* p, size_t bytes) { return fread(p, 1, bytes, stdin) == bytes; };
		uint32_t nodeCount = 0, idxCount = 0;
		if (!rd(&nodeCount, 4)) { fprintf(stderr, "bad mesh\n"); return 3; }
		std::vector<float> nodes(nodeCount);
		if (!rd(nodes.data(), 4 * (size_t)nodeCount) || !rd(&idxCount, 4)) { fprintf(stderr, "bad mesh\n"); return 3; }
		std::vector<uint32_t> idx(idxCount);
		if (!rd(idx.data(), 4 * (size_t)idxCount)) { fprintf(stderr, "bad mesh\n"); return 3; }
		const float density = F(2);
		const uint32_t energy = U(3), simul = U(4);
		const float compliance = F(5), poisson = F(6), gx = F(7), gy = F(8), dt = F(9);
		const uint32_t nsub = U(10), lockLeft = U(11);
		Settings s = make_settings(energy, simul, compliance, poisson, gx, gy, lockLeft);
		set_damping(s, dt, F(12), F(13), F(14), U(15), F(16));
		s.volumePasses = U(17);
		if (quad) {
			// GeoQuadratic3d on the same stream: T10s and H27s in one body
			s.flags = (s.flags & ~(Settings_ElementTypeMask << Settings_ElementTypeBit)) | (Element_T10 << Settings_ElementTypeBit);
			GeoQuadratic3d* q = alloc->New<GeoQuadratic3d>();
			q->Init(alloc, density, nodes.data(), nodeCount, idx.data(), idxCount, false);
			emit("nodes", 'f', nodes.data(), nodeCount);
			emit("idx", 'I', idx.data(), idxCount);
			const uint32_t nt = q->con.tetCount, nh = q->con.hexCount, nv = q->vertCount;
			std::vector<double> x0(nv * 3);
			for (uint32_t i = 0; i < nv; i++)
				for (int k = 0; k < 3; k++) x0[i * 3 + k] = q->X0[i][k];
			std::vector<uint32_t> ti(nt * 10), hi(nh * 27);
			std::vector<float> qep(nt * 56), hep(nh * 703);
			for (uint32_t i = 0; i < nt; i++) {
				for (int c = 0; c < 10; c++) ti[i * 10 + c] = q->t[i].i[c];
				t10_record(q->t[i].ep, &qep[i * 56]);
			}
			for (uint32_t i = 0; i < nh; i++) {
				for (int c = 0; c < 27; c++) hi[i * 27 + c] = q->h[i].i[c];
				h27_record(q->h[i].ep, &hep[i * 703]);
			}
			std::vector<uint8_t> flags(q->flags, q->flags + nv);
			emit("x0", 'd', x0.data(), x0.size());
			emit("t10_idx", 'I', ti.data(), ti.size());
			emit("h27_idx", 'I', hi.data(), hi.size());
			emit("qep", 'f', qep.data(), qep.size());
			emit("h27ep", 'f', hep.data(), hep.size());
			emit("w", 'f', q->w, nv);
			emit("vflags", 'B', flags.data(), nv);
			uint32_t n = 0;
			if (!rd(&n, 4) || n != nt || !rd(q->tOrder, 4 * (size_t)n)) { fprintf(stderr, "bad tet order\n"); return 3; }
			if (!rd(&n, 4) || n != nh || !rd(q->hOrder, 4 * (size_t)n)) { fprintf(stderr, "bad hex order\n"); return 3; }
			Manipulator manip;
			manip.pickedGeo = nullptr;
			for (uint32_t k = 0; k < nsub; k++) {
				s.tickId = k;
				q->Substep(s, manip, dt);
				if (k == 0) dump_state(q, "x1", "v1");
			}
			dump_state(q, "xn", "vn");
			float vol = q->CalculateVolume();
			emit("volume", 'f', &vol, 1);
			return 0;
		}
		GeoLinear3d* g = alloc->New<GeoLinear3d>();
		g->Init(alloc, density, nodes.data(), nodeCount, idx.data(), idxCount, false);
		emit("nodes", 'f', nodes.data(), nodeCount);
		emit("idx", 'I', idx.data(), idxCount);
		const uint32_t nt = g->con.tetCount, nh = g->con.hexCount, nv = g->vertCount;
		std::vector<float> ep(nt * 17), hep(nh * 120);
		for (uint32_t i = 0; i < nt; i++) {
			const ElementParamsLinearTet& e = g->t[i].ep;
			float* o = &ep[i * 17];
			for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[c * 3 + r] = e.Qi[c][r];
			for (int k = 0; k < 3; k++) o[9 + k] = e.ic.QQ[k];
			for (int k = 0; k < 3; k++) o[12 + k] = e.ic.QR[k];
			o[15] = e.volume;
			o[16] = e.surfaceArea;
		}
		for (uint32_t i = 0; i < nh; i++) hex_record(g->h[i].ep, &hep[i * 120]);
		std::vector<uint8_t> flags(g->flags, g->flags + nv);
		emit("ep", 'f', ep.data(), ep.size());
		emit("hep", 'f', hep.data(), hep.size());
		emit("w", 'f', g->w, nv);
		emit("vflags", 'B', flags.data(), nv);
		uint32_t n = 0;
		if (!rd(&n, 4) || n != nt || !rd(g->tOrder, 4 * (size_t)n)) { fprintf(stderr, "bad tet order\n"); return 3; }
		if (!rd(&n, 4) || n != nh || !rd(g->hOrder, 4 * (size_t)n)) { fprintf(stderr, "bad hex order\n"); return 3; }
		Manipulator manip;
		manip.pickedGeo = nullptr;
		for (uint32_t k = 0; k < nsub; k++) {
			s.tickId = k;
			g->Substep(s, manip, dt);
			if (k == 0) dump_state(g, "x1", "v1");
		}
		dump_state(g, "xn", "vn");
		float vol = g->CalculateVolume();
		emit("volume", 'f', &vol, 1);
		return 0;
	}

	if (!strcmp(cmd, "meshgen") || !strcmp(cmd, "init") || !strcmp(cmd, "substep") || !strcmp(cmd, "ordered") ||
	    !strcmp(cmd, "damped") || !strcmp(cmd, "rings") || !strcmp(cmd, "locked")) {
		Allocator* alloc = make_alloc((size_t)1 << 31);
		uint32_t W = U(2), H = U(3), D = U(4);
		vec3 scale(F(5), F(6), F(7));
		int a = 8;
		uint32_t pattern = 0;
		if (hex || !strcmp(cmd, "meshgen") || !strcmp(cmd, "init")) pattern = U(a++);
		float wonk = F(a++);
		const float* nodes; uint32_t nodeCount; const uint32_t* idx; uint32_t idxCount;
		if (hex)
			GenerateHexBlock(alloc, W, H, D, scale, pattern, wonk, &nodes, &nodeCount, &idx, &idxCount);
		else
			GenerateTetBlock(alloc, W, H, D, scale, pattern, wonk, &nodes, &nodeCount, &idx, &idxCount);
		if (!strcmp(cmd, "meshgen")) {
			emit("nodes", 'f', nodes, nodeCount);
			emit("idx", 'I', idx, idxCount);
			return 0;
		}
		float density = F(a++);
		GeoLinear3d* g = alloc->New<GeoLinear3d>();
		g->Init(alloc, density, nodes, nodeCount, idx, idxCount, false);
		if (!strcmp(cmd, "init")) {
			emit("nodes", 'f', nodes, nodeCount);
			emit("idx", 'I', idx, idxCount);
			if (hex)
				dump_hex_geo(g);
			else
				dump_geo(g);
			return 0;
		}
		uint32_t energy = U(a++), simul = U(a++);
		float compliance = F(a++), poisson = F(a++), gx = F(a++), gy = F(a++), dt = F(a++);
		uint32_t nsub = U(a++), lockLeft = U(a++);
		Settings s = make_settings(energy, simul, compliance, poisson, gx, gy, lockLeft);
		const bool rings = !strcmp(cmd, "rings");
		const bool locked = !strcmp(cmd, "locked");
		const bool damped = !strcmp(cmd, "damped") || rings || locked;
		if (damped) {
			set_damping(s, dt, F(a), F(a + 1), F(a + 2), U(a + 3), F(a + 4));
			a += 5;
			if (a < argc) s.volumePasses = U(a++);
		}
		if (locked) {
			float m[9];
			for (int k = 0; k < 9; k++) m[k] = F(a++);
			s.lockedRightTransform3d = mat3(vec3(m[0], m[1], m[2]), vec3(m[3], m[4], m[5]), vec3(m[6], m[7], m[8]));
			g->origin = vec3(F(a), F(a + 1), F(a + 2));
			a += 3;
			s.flags |= Settings_LockRight;
		}
		Manipulator manip;
		manip.pickedGeo = nullptr;
		emit("nodes", 'f', nodes, nodeCount);
		emit("idx", 'I', idx, idxCount);
		if (!strcmp(cmd, "ordered") || damped) {
			// Replace the shuffled tOrder by the order read from stdin; Geo3d::Substep
			// then runs GeoLinear3d::Constrain (XPBDFEM/Geo.cpp:777) over it unchanged.
			uint32_t n = 0;
			const uint32_t want = hex ? g->con.hexCount : g->con.tetCount;
			uint32_t* dst = hex ? g->hOrder : g->tOrder;
			if (fread(&n, 4, 1, stdin) != 1 || n != want) { fprintf(stderr, "bad order\n"); return 3; }
			if (fread(dst, 4, n, stdin) != n) { fprintf(stderr, "short order\n"); return 3; }
		}
		if (rings) {
			uint32_t n = 0;
			if (fread(&n, 4, 1, stdin) != 1 || n != g->con.vertCount) { fprintf(stderr, "bad vertex order\n"); return 3; }
			if (fread(g->vOrder, 4, n, stdin) != n) { fprintf(stderr, "short vertex order\n"); return 3; }
		}
		for (uint32_t k = 0; k < nsub; k++) {
			s.tickId = k;
			g->Substep(s, manip, dt);
			if (k == 0) dump_state(g, "x1", "v1");
		}
		dump_state(g, "xn", "vn");
		float vol = g->CalculateVolume();
		emit("volume", 'f', &vol, 1);
		return 0;
	}

	if (h27 && !strcmp(cmd, "solve")) {
		g_rng = strtoull(argv[2], 0, 10);
		uint32_t count = U(3), energy = U(4), simul = U(5);
		float compliance = F(6), poisson = F(7), dt = F(8);
		Settings s = make_settings(energy, simul, compliance, poisson, 0.0f, 0.0f, 0);
		std::vector<double> xin(count * 81), xout(count * 81), rest(count * 81);
		std::vector<float> win(count * 27), epo(count * 703);
		for (uint32_t t = 0; t < count; t++) {
			dvec3 C[8], X0[27], X[27], O[27];
			float m[27] = {0}, w[27];
			// Rest corners as `hsolve`'s random hex; node (i, j, k) of the
			// 3x3x3 grid at the trilinear point of the corners
			double ext[3];
			for (int k = 0; k < 3; k++) ext[k] = 0.02 + 0.2 * urand();
			for (int n = 0; n < 8; n++)
				for (int k = 0; k < 3; k++) C[n][k] = (double)(float)(ext[k] * (((n >> k) & 1) + 0.1 * (urand() - 0.5)));
			for (int n = 0; n < 27; n++) {
				const double u[3] = {0.5 * (n % 3), 0.5 * ((n / 3) % 3), 0.5 * (n / 9)};
				X0[n] = dvec3(0.0);
				for (int c = 0; c < 8; c++) {
					const double f = (c & 1 ? u[0] : 1.0 - u[0]) * (c & 2 ? u[1] : 1.0 - u[1]) * (c & 4 ? u[2] : 1.0 - u[2]);
					X0[n] += f * C[c];
				}
			}
			uint32_t is[27];
			for (int n = 0; n < 27; n++) is[n] = n;
			ElementParamsQuadraticHex ep;
			InitFiniteElement(X0, is, 1000.0f, m, &ep);
			uint32_t kind = t % 8;
			double amp = kind < 4 ? 0.05 : kind < 6 ? 0.4 : 1.5;
			double sc = (ext[0] + ext[1] + ext[2]) / 3.0;
			for (int n = 0; n < 27; n++) {
				for (int k = 0; k < 3; k++) X[n][k] = X0[n][k] + amp * sc * (urand() - 0.5);
				O[n] = X0[n];
				w[n] = (float)(0.5 + 2.0 * urand());
			}
			if (kind == 6) { dvec3 tmp = X[0]; X[0] = X[26]; X[26] = tmp; }  // inverted
			if (kind == 7) { w[0] = 0.0f; w[26] = 0.0f; }
			for (int n = 0; n < 27; n++) {
				win[t * 27 + n] = w[n];
				for (int k = 0; k < 3; k++) { xin[t * 81 + n * 3 + k] = X[n][k]; rest[t * 81 + n * 3 + k] = X0[n][k]; }
			}
			SolveElement(dt, X, O, w, is, ep, s);
			for (int n = 0; n < 27; n++) for (int k = 0; k < 3; k++) xout[t * 81 + n * 3 + k] = X[n][k];
			h27_record(ep, &epo[t * 703]);
		}
		emit("rest", 'd', rest.data(), rest.size());
		emit("h27ep", 'f', epo.data(), epo.size());
		emit("xin", 'd', xin.data(), xin.size());
		emit("w", 'f', win.data(), win.size());
		emit("xout", 'd', xout.data(), xout.size());
		return 0;
	}

	if (hex && !strcmp(cmd, "solve")) {
		g_rng = strtoull(argv[2], 0, 10);
		uint32_t count = U(3), energy = U(4), simul = U(5);
		float compliance = F(6), poisson = F(7), dt = F(8);
		Settings s = make_settings(energy, simul, compliance, poisson, 0.0f, 0.0f, 0);
		std::vector<double> xin(count * 24), xout(count * 24), rest(count * 24);
		std::vector<float> win(count * 8), epo(count * 120);
		for (uint32_t t = 0; t < count; t++) {
			dvec3 X0[8], X[8], O[8];
			float m[8] = {0, 0, 0, 0, 0, 0, 0, 0}, w[8];
			// Rest hex: a box of random extents, corners jittered by up to
			// 10% of the extent; node n at (i, j, k) = bits of n.
			double ext[3];
			for (int k = 0; k < 3; k++) ext[k] = 0.02 + 0.2 * urand();
			for (int n = 0; n < 8; n++)
				for (int k = 0; k < 3; k++) X0[n][k] = ext[k] * (((n >> k) & 1) + 0.1 * (urand() - 0.5));
			for (int n = 0; n < 8; n++) for (int k = 0; k < 3; k++) X0[n][k] = (double)(float)X0[n][k];
			const uint32_t is[8] = {0, 1, 2, 3, 4, 5, 6, 7};
			ElementParamsLinearHex ep;
			InitFiniteElement(X0, is, 1000.0f, m, &ep);
			// Deformed state: mild, large, inverted, w = 0 on some nodes.
			uint32_t kind = t % 8;
			double amp = kind < 4 ? 0.05 : kind < 6 ? 0.4 : 1.5;
			double sc = (ext[0] + ext[1] + ext[2]) / 3.0;
			for (int n = 0; n < 8; n++) {
				for (int k = 0; k < 3; k++) X[n][k] = X0[n][k] + amp * sc * (urand() - 0.5);
				O[n] = X0[n];
				w[n] = (float)(0.5 + 2.0 * urand());
			}
			if (kind == 6) { dvec3 tmp = X[0]; X[0] = X[7]; X[7] = tmp; }  // inverted
			if (kind == 7) { w[0] = 0.0f; w[7] = 0.0f; }
			for (int n = 0; n < 8; n++) {
				win[t * 8 + n] = w[n];
				for (int k = 0; k < 3; k++) { xin[t * 24 + n * 3 + k] = X[n][k]; rest[t * 24 + n * 3 + k] = X0[n][k]; }
			}
			SolveElement(dt, X, O, w, is, ep, s);
			for (int n = 0; n < 8; n++) for (int k = 0; k < 3; k++) xout[t * 24 + n * 3 + k] = X[n][k];
			hex_record(ep, &epo[t * 120]);
		}
		emit("rest", 'd', rest.data(), rest.size());
		emit("hep", 'f', epo.data(), epo.size());
		emit("xin", 'd', xin.data(), xin.size());
		emit("w", 'f', win.data(), win.size());
		emit("xout", 'd', xout.data(), xout.size());
		return 0;
	}

	if (!hex && !strcmp(cmd, "solve")) {
		g_rng = strtoull(argv[2], 0, 10);
		uint32_t count = U(3), energy = U(4), simul = U(5);
		float compliance = F(6), poisson = F(7), dt = F(8);
		Settings s = make_settings(energy, simul, compliance, poisson, 0.0f, 0.0f, 0);
		std::vector<double> xin(count * 12), xout(count * 12), rest(count * 12);
		std::vector<float> win(count * 4), epo(count * 17);
		for (uint32_t t = 0; t < count; t++) {
			dvec3 X0[4], X[4], O[4];
			float m[4] = {0, 0, 0, 0}, w[4];
			// Rest tet: unit-scale random points, reordered to positive volume.
			double sc = 0.02 + 0.2 * urand();
			for (int n = 0; n < 4; n++) X0[n] = dvec3(sc * (urand() - 0.5), sc * (urand() - 0.5), sc * (urand() - 0.5));
			X0[0] = X0[3] + dvec3(sc * (0.6 + 0.4 * urand()), 0.1 * sc * (urand() - 0.5), 0.1 * sc * (urand() - 0.5));
			X0[1] = X0[3] + dvec3(0.1 * sc * (urand() - 0.5), sc * (0.6 + 0.4 * urand()), 0.1 * sc * (urand() - 0.5));
			X0[2] = X0[3] + dvec3(0.1 * sc * (urand() - 0.5), 0.1 * sc * (urand() - 0.5), sc * (0.6 + 0.4 * urand()));
			// Round rest positions to float, as node data arrives as float.
			for (int n = 0; n < 4; n++) for (int k = 0; k < 3; k++) X0[n][k] = (double)(float)X0[n][k];
			const uint32_t is[4] = {0, 1, 2, 3};
			ElementParamsLinearTet ep;
			InitFiniteElement(X0, is, 1000.0f, m, &ep);
			// Deformed state: case mix = mild, large, inverted, w = 0 on some nodes.
			uint32_t kind = t % 8;
			double amp = kind < 4 ? 0.05 : kind < 6 ? 0.4 : 1.5;
			for (int n = 0; n < 4; n++) {
				for (int k = 0; k < 3; k++) X[n][k] = X0[n][k] + amp * sc * (urand() - 0.5);
				O[n] = X0[n];
				w[n] = (float)(0.5 + 2.0 * urand());
			}
			if (kind == 6) { dvec3 tmp = X[0]; X[0] = X[1]; X[1] = tmp; } // inverted
			if (kind == 7) { w[0] = 0.0f; w[3] = 0.0f; }
			for (int n = 0; n < 4; n++) {
				win[t * 4 + n] = w[n];
				for (int k = 0; k < 3; k++) { xin[t * 12 + n * 3 + k] = X[n][k]; rest[t * 12 + n * 3 + k] = X0[n][k]; }
			}
			SolveElement(dt, X, O, w, is, ep, s);
			for (int n = 0; n < 4; n++) for (int k = 0; k < 3; k++) xout[t * 12 + n * 3 + k] = X[n][k];
			float* o = &epo[t * 17];
			for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) o[c * 3 + r] = ep.Qi[c][r];
			for (int k = 0; k < 3; k++) { o[9 + k] = ep.ic.QQ[k]; o[12 + k] = ep.ic.QR[k]; }
			o[15] = ep.volume; o[16] = ep.surfaceArea;
		}
		emit("rest", 'd', rest.data(), rest.size());
		emit("ep", 'f', epo.data(), epo.size());
		emit("xin", 'd', xin.data(), xin.size());
		emit("w", 'f', win.data(), win.size());
		emit("xout", 'd', xout.data(), xout.size());
		return 0;
	}
	fprintf(stderr, "unknown command %s\n", cmd);
	return 2;
}
