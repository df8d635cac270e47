/*
 * opcount — the exact arithmetic count of one tet-substep, from the oracle's
 * FP64 restatement (oracle/xfem_oracle_real.inc) instantiated on a counting
 * scalar. Test infrastructure only: built and run by
 * tests/test_oracle_opcount.py, which holds the figures the measurement
 * uses.
 *
 * The scalar R is a double that counts each operation it takes part in:
 * add / sub, mul, div, sqrt (one each; the restatement has no fused
 * multiply-add), comparisons (fmax / fmin, < >) separately. Position
 * arithmetic is in plain double in the restatement (X - O, X += ...) and is
 * counted by the caller from the code, per vertex and per tet.
 *
 * Output (stdout, one line per case): name, then the counts per tet solve
 * (orc_solve_tet, one call on a mildly deformed tet) and per vertex
 * (predict + finalize of one free vertex).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xfem_oracle.h"

namespace {

struct Ops {
	uint64_t add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0;
};
Ops g_ops;

struct Cnt {
	double v;
	Cnt() : v(0) {}
	Cnt(double x) : v(x) {}
	operator double() const { return v; }
};
inline Cnt operator+(Cnt a, Cnt b) { g_ops.add++; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { g_ops.add++; return Cnt(a.v - b.v); }
inline Cnt operator*(Cnt a, Cnt b) { g_ops.mul++; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { g_ops.div++; return Cnt(a.v / b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt operator+(Cnt a) { return a; }
inline Cnt& operator+=(Cnt& a, Cnt b) { a = a + b; return a; }
inline Cnt& operator-=(Cnt& a, Cnt b) { a = a - b; return a; }
inline Cnt& operator*=(Cnt& a, Cnt b) { a = a * b; return a; }
inline Cnt& operator/=(Cnt& a, Cnt b) { a = a / b; return a; }
inline bool operator<(Cnt a, Cnt b) { g_ops.cmp++; return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { g_ops.cmp++; return a.v > b.v; }
inline bool operator<=(Cnt a, Cnt b) { g_ops.cmp++; return a.v <= b.v; }
inline bool operator>=(Cnt a, Cnt b) { g_ops.cmp++; return a.v >= b.v; }
// mixed operands count like the scalar ones (exact matches, so no
// conversion to the built-in operators is chosen)
#define CNT_MIXED(T)                                                              \
	inline Cnt operator+(Cnt a, T b) { return a + Cnt(b); }                       \
	inline Cnt operator+(T a, Cnt b) { return Cnt(a) + b; }                       \
	inline Cnt operator-(Cnt a, T b) { return a - Cnt(b); }                       \
	inline Cnt operator-(T a, Cnt b) { return Cnt(a) - b; }                       \
	inline Cnt operator*(Cnt a, T b) { return a * Cnt(b); }                       \
	inline Cnt operator*(T a, Cnt b) { return Cnt(a) * b; }                       \
	inline Cnt operator/(Cnt a, T b) { return a / Cnt(b); }                       \
	inline Cnt operator/(T a, Cnt b) { return Cnt(a) / b; }                       \
	inline bool operator<(Cnt a, T b) { return a < Cnt(b); }                      \
	inline bool operator>(Cnt a, T b) { return a > Cnt(b); }                      \
	inline bool operator<=(Cnt a, T b) { return a <= Cnt(b); }                    \
	inline bool operator>=(Cnt a, T b) { return a >= Cnt(b); }
CNT_MIXED(double)
CNT_MIXED(float)
CNT_MIXED(int)
CNT_MIXED(unsigned)
inline Cnt cnt_sqrt(Cnt a) { g_ops.sqrt++; return Cnt(::sqrt(a.v)); }
inline Cnt cnt_max(Cnt a, Cnt b) { g_ops.cmp++; return a.v > b.v ? a : b; }
inline Cnt cnt_min(Cnt a, Cnt b) { g_ops.cmp++; return a.v < b.v ? a : b; }

}  // namespace

#define ORC_NO_RINGS
#define R Cnt
#define SFX _c
#define SQRT cnt_sqrt
#define FMAX cnt_max
#define FMIN cnt_min
#define EPS22 Cnt(1.0e-22)
#define EPS8 Cnt(1.0e-8)
#define EPS4 Cnt(1.0e-4)
#include "xfem_oracle_real.inc"

static void emit(const char* name, const Ops& o) {
	printf("%s add %llu mul %llu div %llu sqrt %llu cmp %llu flops %llu\n", name, (unsigned long long)o.add,
	       (unsigned long long)o.mul, (unsigned long long)o.div, (unsigned long long)o.sqrt, (unsigned long long)o.cmp,
	       (unsigned long long)(o.add + o.mul + o.div + o.sqrt));
}

int main() {
	// one tet: unit right tet, deformed a little, w = 1
	const float nodes[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
	const uint32_t tet[4] = {0, 1, 2, 3};
	Cnt ep[ORC_EP], w[4];
	uint8_t fl[4];
	orc_init_rest_c(nodes, 4, tet, 1, Cnt(1000.0), ep, w, fl);
	const uint32_t energies[2] = {ORC_ENERGY_MIXED_SEL, ORC_ENERGY_YEOH_SKIN_FAST};
	const char* names[2] = {"tet_solve_nh_coupled", "tet_solve_yeoh_coupled"};
	for (int k = 0; k < 2; k++) {
		orc_params p;
		memset(&p, 0, sizeof(p));
		p.dt = 1.0f / 1200.0f;
		p.compliance = 6e-5f;
		p.poisson = 0.5f;
		p.energy = energies[k];
		p.simultaneous = 1;
		p.yeoh[0] = 0.1095f;
		p.yeoh[1] = 14.95f;
		p.yeoh[2] = 4.595f;
		p.rayleigh_type = 2;
		double X[12], O[12];
		for (int i = 0; i < 12; i++) {
			O[i] = nodes[i];
			X[i] = nodes[i] + 0.01 * ((i * 7) % 5 - 2);
		}
		Cnt lam[2];
		g_ops = Ops();
		orc_solve_tet_c(X, O, w, ep, &p, Cnt(0.0), lam);
		emit(names[k], g_ops);
	}
	// one free vertex: predict and finalize of a substep (no lock, no ground)
	{
		orc_params p;
		memset(&p, 0, sizeof(p));
		p.dt = 1.0f / 1200.0f;
		p.gravity[2] = -9.81f;
		double X[3] = {0, 0, 0}, V[3] = {0, 0, 0}, O[3];
		Cnt wv[1] = {Cnt(1.0)};
		orc_run_c r = {1, 0, X, V, O, wv, 0, 0, 0, 0, &p, 0, 0};
		g_ops = Ops();
		predict_c(&r, 0, 1);
		finalize_c(&r, 0, 1);
		emit("vertex_predict_finalize", g_ops);
	}
	return 0;
}
