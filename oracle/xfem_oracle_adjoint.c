/*
 * FP64 reverse-mode adjoint of the substep — TEST INFRASTRUCTURE ONLY (see
 * oracle/xfem_oracle.h). It differentiates the oracle's double instantiation
 * (orc_substeps_d) exactly: predict (XPBDFEM/Geo.cpp:307-312), the constraint
 * sweep in the given order with the coupled Neo-Hookean solve
 * (XPBDFEM/Fem.cpp:523-553, XPBDFEM/Xpbd.h:123-215), locks
 * (XPBDFEM/Geo.cpp:318-322), the ground projection with Coulomb friction
 * (extension) and the velocity update (XPBDFEM/Geo.cpp:342-344).
 *
 * Loss: sum over substeps s = 1..nsub and tip vertices of |x_s - target_s|^2.
 * Outputs dL/dmu per tet (the per-tet shear modulus mu_ref), dL/dV0 and dL/dX0;
 * with dmu == NULL only the forward runs and the loss is returned.
 * The Cramer clamp max(1e-8, .) and the Yeoh clamp are taken as inactive;
 * only the coupled (bit 11) Neo-Hookean model is differentiated.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xfem_oracle.h"

typedef struct { double x, y, z; } d3;
static inline d3 v(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 add(d3 a, d3 b) { return v(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 sub(d3 a, d3 b) { return v(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 mul(d3 a, double s) { return v(a.x * s, a.y * s, a.z * s); }
static inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 crs(d3 a, d3 b) { return v(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline d3 ld(const double* p) { return v(p[0], p[1], p[2]); }
static inline void st(double* p, d3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }
static inline void acc(double* p, d3 a) { p[0] += a.x; p[1] += a.y; p[2] += a.z; }

/* Everything one tet solve computes, kept for its reverse pass. */
typedef struct {
	d3 P[3], g0[4], g1[4], h[3], cof[3];
	double U0, U1, J, a, detQ, A0, A1, A2, l0, l1, alpha0, alpha1;
	double QQ[3], QR[3];
} tet_fw;

/* Forward of one tet (double), the math of orc_solve_tet_d in the form the
 * reverse pass needs: g1 = 2 (J - a) det(Qi) cof(Ds), equal to the
 * reference's (2 (J - a) adj(F) Qi) e_n. Updates x in place. */
static void tet_forward(double x[4][3], const double w[4], const double* ep, double mu, const orc_params* p,
                        tet_fw* f) {
	const double dt = p->dt, nu = p->poisson;
	const double lambda = (2.0 * mu * nu) / (1.0 - 2.0 * nu);
	f->a = 1.0 + mu / lambda;
	const double vol = ep[15];
	f->alpha0 = (1.0 / mu / vol) / (dt * dt);
	f->alpha1 = (1.0 / lambda / vol) / (dt * dt);
	for (int i = 0; i < 3; i++) f->P[i] = sub(ld(x[i]), ld(x[3]));
	for (int i = 0; i < 3; i++) { f->QQ[i] = ep[9 + i]; f->QR[i] = ep[12 + i]; }
	const d3* P = f->P;
	f->U0 = f->QQ[0] * dot(P[0], P[0]) + f->QQ[1] * dot(P[1], P[1]) + f->QQ[2] * dot(P[2], P[2]) +
	        f->QR[0] * dot(P[0], P[1]) + f->QR[1] * dot(P[0], P[2]) + f->QR[2] * dot(P[1], P[2]);
	f->g0[0] = add(add(mul(P[0], 2 * f->QQ[0]), mul(P[1], f->QR[0])), mul(P[2], f->QR[1]));
	f->g0[1] = add(add(mul(P[1], 2 * f->QQ[1]), mul(P[0], f->QR[0])), mul(P[2], f->QR[2]));
	f->g0[2] = add(add(mul(P[2], 2 * f->QQ[2]), mul(P[0], f->QR[1])), mul(P[1], f->QR[2]));
	f->g0[3] = mul(add(add(f->g0[0], f->g0[1]), f->g0[2]), -1.0);
	const double* q = ep; /* Qi column-major q[c*3+r] */
	f->detQ = q[0] * (q[4] * q[8] - q[7] * q[5]) - q[3] * (q[1] * q[8] - q[7] * q[2]) + q[6] * (q[1] * q[5] - q[4] * q[2]);
	f->cof[0] = crs(P[1], P[2]);
	f->cof[1] = crs(P[2], P[0]);
	f->cof[2] = crs(P[0], P[1]);
	f->J = f->detQ * dot(P[0], f->cof[0]);
	const double s = 2.0 * (f->J - f->a);
	for (int i = 0; i < 3; i++) {
		f->h[i] = mul(f->cof[i], f->detQ);
		f->g1[i] = mul(f->h[i], s);
	}
	f->g1[3] = mul(add(add(f->g1[0], f->g1[1]), f->g1[2]), -1.0);
	f->U1 = (f->J - f->a) * (f->J - f->a);
	double wgg0 = 1e-22, wgg1 = 1e-22, wgg2 = 1e-22;
	for (int n = 0; n < 4; n++) {
		wgg0 += w[n] * dot(f->g0[n], f->g0[n]);
		wgg1 += w[n] * dot(f->g1[n], f->g0[n]);
		wgg2 += w[n] * dot(f->g1[n], f->g1[n]);
	}
	f->A0 = wgg0 + 2.0 * f->U0 * f->alpha0;
	f->A1 = wgg1;
	f->A2 = wgg2 + 2.0 * f->U1 * f->alpha1;
	const double b0 = -2.0 * f->U0, b1 = -2.0 * f->U1, det = f->A0 * f->A2 - f->A1 * f->A1;
	f->l0 = (b0 * f->A2 - f->A1 * b1) / det;
	f->l1 = (f->A0 * b1 - f->A1 * b0) / det;
	for (int n = 0; n < 4; n++) acc(x[n], mul(add(mul(f->g0[n], f->l0), mul(f->g1[n], f->l1)), w[n]));
}

/* Reverse of one tet: xb[4][3] holds the adjoint of the outputs on entry and
 * of the inputs on exit. Returns dL/dmu of this tet. */
static double tet_reverse(const tet_fw* f, const double w[4], double mu, double xb[4][3]) {
	d3 y[4], gb0[4], gb1[4], Pb[3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
	double lb0 = 0, lb1 = 0;
	for (int n = 0; n < 4; n++) {
		y[n] = mul(ld(xb[n]), w[n]);
		lb0 += dot(y[n], f->g0[n]);
		lb1 += dot(y[n], f->g1[n]);
		gb0[n] = mul(y[n], f->l0);
		gb1[n] = mul(y[n], f->l1);
	}
	/* lambda = M^-1 b, M = [A0 A1; A1 A2]: mu = M^-1 lambda_bar, b_bar = mu, M_bar = -mu lambda^T */
	const double det = f->A0 * f->A2 - f->A1 * f->A1;
	const double m0 = (lb0 * f->A2 - f->A1 * lb1) / det, m1 = (f->A0 * lb1 - f->A1 * lb0) / det;
	const double Ab0 = -m0 * f->l0, Ab2 = -m1 * f->l1, Ab1 = -(m0 * f->l1 + m1 * f->l0);
	double Ub0 = -2.0 * m0, Ub1 = -2.0 * m1;
	/* A0 = sum w|g0|^2 + 2 U0 a0; A1 = sum w g1.g0; A2 = sum w|g1|^2 + 2 U1 a1 */
	for (int n = 0; n < 4; n++) {
		gb0[n] = add(gb0[n], add(mul(f->g0[n], 2.0 * w[n] * Ab0), mul(f->g1[n], w[n] * Ab1)));
		gb1[n] = add(gb1[n], add(mul(f->g1[n], 2.0 * w[n] * Ab2), mul(f->g0[n], w[n] * Ab1)));
	}
	Ub0 += 2.0 * f->alpha0 * Ab0;
	Ub1 += 2.0 * f->alpha1 * Ab2;
	const double ab0 = 2.0 * f->U0 * Ab0, ab1 = 2.0 * f->U1 * Ab2;
	/* g_3 = -(g_0 + g_1 + g_2) */
	for (int i = 0; i < 3; i++) {
		gb0[i] = sub(gb0[i], gb0[3]);
		gb1[i] = sub(gb1[i], gb1[3]);
	}
	/* deviatoric: U0 = P^T S P, g0 = 2 S P (S_ii = QQ_i, S_ij = QR/2) */
	const double* QQ = f->QQ;
	const double* QR = f->QR;
	Pb[0] = add(Pb[0], add(add(mul(gb0[0], 2 * QQ[0]), mul(gb0[1], QR[0])), mul(gb0[2], QR[1])));
	Pb[1] = add(Pb[1], add(add(mul(gb0[0], QR[0]), mul(gb0[1], 2 * QQ[1])), mul(gb0[2], QR[2])));
	Pb[2] = add(Pb[2], add(add(mul(gb0[0], QR[1]), mul(gb0[1], QR[2])), mul(gb0[2], 2 * QQ[2])));
	for (int i = 0; i < 3; i++) Pb[i] = add(Pb[i], mul(f->g0[i], Ub0));
	/* hydrostatic: U1 = (J - a)^2, g1_i = 2 (J - a) h_i, h_i = detQ cof_i, dJ/dP_i = h_i */
	double Jb = 2.0 * (f->J - f->a) * Ub1;
	d3 cb[3];
	for (int i = 0; i < 3; i++) {
		Jb += 2.0 * dot(f->h[i], gb1[i]);
		cb[i] = mul(gb1[i], 2.0 * (f->J - f->a) * f->detQ);
	}
	for (int i = 0; i < 3; i++) Pb[i] = add(Pb[i], mul(f->h[i], Jb));
	const d3* P = f->P;
	/* cof0 = P1 x P2, cof1 = P2 x P0, cof2 = P0 x P1; for c = a x b: a_bar = b x c_bar, b_bar = c_bar x a */
	Pb[1] = add(Pb[1], crs(P[2], cb[0]));
	Pb[2] = add(Pb[2], crs(cb[0], P[1]));
	Pb[2] = add(Pb[2], crs(P[0], cb[1]));
	Pb[0] = add(Pb[0], crs(cb[1], P[2]));
	Pb[0] = add(Pb[0], crs(P[1], cb[2]));
	Pb[1] = add(Pb[1], crs(cb[2], P[0]));
	/* P_i = x_i - x_3; the outputs' identity part stays in xb */
	for (int i = 0; i < 3; i++) {
		acc(xb[i], Pb[i]);
		acc(xb[3], mul(Pb[i], -1.0));
	}
	/* alpha0, alpha1 both scale as 1/mu */
	return -(f->alpha0 * ab0 + f->alpha1 * ab1) / mu;
}

/* Ground projection with friction on one vertex (the forward of
 * xfem_oracle_real.inc's ground, in double); returns 1 on contact and fills
 * the quantities its reverse pass needs. */
typedef struct { int contact, kinetic; d3 n, t; double depth, lt, lim, s; } gr_fw;

static int ground_forward(double* X, const double* O, const orc_params* p, gr_fw* g) {
	g->n = v(p->ground_n[0], p->ground_n[1], p->ground_n[2]);
	d3 D = sub(ld(X), ld(O));
	const double h = dot(g->n, ld(O)) - (double)p->ground_d;
	g->depth = -(h + dot(g->n, D));
	g->contact = g->depth > 0.0;
	if (!g->contact) return 0;
	d3 D1 = add(D, mul(g->n, g->depth));
	g->t = sub(D1, mul(g->n, dot(g->n, D1)));
	g->lt = sqrt(dot(g->t, g->t));
	g->lim = (double)p->friction * g->depth;
	g->kinetic = !(g->lt <= g->lim);
	g->s = g->kinetic ? g->lim / g->lt : 1.0;
	st(X, add(ld(O), sub(D1, mul(g->t, g->s))));
	return 1;
}

/* xb: adjoint of the output position (in) -> of the input position (out); ob accumulates. */
static void ground_reverse(const gr_fw* g, double* xb, double* ob) {
	if (!g->contact) return;
	const d3 n = g->n;
	d3 D2b = ld(xb);
	acc(ob, D2b);
	d3 D1b = D2b, tb = mul(D2b, -g->s);
	double depthb = 0.0;
	if (g->kinetic) {
		const double sb = -dot(g->t, D2b);
		const double limb = sb / g->lt, ltb = -sb * g->lim / (g->lt * g->lt);
		depthb += limb * (g->lim / g->depth);
		tb = add(tb, mul(g->t, ltb / g->lt));
	}
	D1b = add(D1b, sub(tb, mul(n, dot(n, tb))));
	d3 Db = D1b;
	depthb += dot(n, D1b);
	/* depth = -(n.O - d + n.D) */
	acc(ob, mul(n, -depthb));
	Db = add(Db, mul(n, -depthb));
	/* D = X - O */
	st(xb, Db);
	acc(ob, mul(Db, -1.0));
}

int orc_adjoint_d(uint32_t nv, const double* X0, const double* V0, const double* w0, const uint8_t* lock_mask,
                  uint32_t nt, const uint32_t* tets, const double* ep, const double* tet_mu, const uint32_t* order,
                  uint32_t nsub, const orc_params* p, uint32_t ntip, const uint32_t* tips, const double* targets,
                  double* loss, double* dmu, double* dV0, double* dX0) {
	if (p->energy != ORC_ENERGY_MIXED_SEL || !p->simultaneous) return -1;
	const size_t n3 = 3 * (size_t)nv;
	const double dt = p->dt, inv_dt = 1.0 / dt, drag = 1.0 - (double)p->time_corrected_drag;
	const double gdt[3] = {p->gravity[0] * dt, p->gravity[1] * dt, p->gravity[2] * dt};
	/* tape: per substep the predicted positions and O; w before each substep */
	double* Xp = (double*)malloc(sizeof(double) * n3 * nsub);
	double* Os = (double*)malloc(sizeof(double) * n3 * nsub);
	double* ws = (double*)malloc(sizeof(double) * nv * nsub);
	double* X = (double*)malloc(sizeof(double) * n3);
	double* V = (double*)malloc(sizeof(double) * n3);
	double* w = (double*)malloc(sizeof(double) * nv);
	double* Xb = (double*)calloc(n3, sizeof(double));
	double* Vb = (double*)calloc(n3, sizeof(double));
	double* Ob = (double*)malloc(sizeof(double) * n3);
	double* Y = (double*)malloc(sizeof(double) * n3);
	tet_fw* tf = (tet_fw*)malloc(sizeof(tet_fw) * (nt ? nt : 1));
	gr_fw* gf = (gr_fw*)malloc(sizeof(gr_fw) * (nv ? nv : 1));
	if (!Xp || !Os || !ws || !X || !V || !w || !Xb || !Vb || !Ob || !Y || !tf || !gf) return -1;
	memcpy(X, X0, sizeof(double) * n3);
	memcpy(V, V0, sizeof(double) * n3);
	memcpy(w, w0, sizeof(double) * nv);
	double L = 0.0;
	/* ---- forward ---- */
	for (uint32_t s = 0; s < nsub; s++) {
		memcpy(ws + (size_t)nv * s, w, sizeof(double) * nv);
		for (size_t j = 0; j < n3; j++) {
			V[j] = (V[j] + gdt[j % 3]) * drag;
			Os[n3 * s + j] = X[j];
			X[j] += V[j] * dt;
		}
		memcpy(Xp + n3 * s, X, sizeof(double) * n3);
		for (uint32_t k = 0; k < nt; k++) {
			const uint32_t t = order[k];
			const uint32_t* is = tets + 4 * (size_t)t;
			double x[4][3], wl[4];
			for (int n = 0; n < 4; n++) { memcpy(x[n], X + 3 * (size_t)is[n], sizeof(double) * 3); wl[n] = w[is[n]]; }
			tet_fw f;
			tet_forward(x, wl, ep + ORC_EP * (size_t)t, tet_mu[t], p, &f);
			for (int n = 0; n < 4; n++) memcpy(X + 3 * (size_t)is[n], x[n], sizeof(double) * 3);
		}
		const double* O = Os + n3 * s;
		for (uint32_t i = 0; i < nv; i++) {
			if (p->lock_active && lock_mask && (lock_mask[i] & 1u)) {
				memcpy(X + 3 * (size_t)i, O + 3 * (size_t)i, sizeof(double) * 3);
				w[i] = 0.0;
			}
			if (p->ground && w[i] > 0.0) {
				gr_fw g;
				ground_forward(X + 3 * (size_t)i, O + 3 * (size_t)i, p, &g);
			}
			for (int k = 0; k < 3; k++) V[3 * (size_t)i + k] = (X[3 * (size_t)i + k] - O[3 * (size_t)i + k]) * inv_dt;
		}
		for (uint32_t q = 0; q < ntip; q++)
			for (int k = 0; k < 3; k++) {
				const double d = X[3 * (size_t)tips[q] + k] - targets[((size_t)s * ntip + q) * 3 + k];
				L += d * d;
			}
	}
	*loss = L;
	if (!dmu) goto done; /* forward only (finite differences) */
	/* ---- reverse ---- */
	for (uint32_t t = 0; t < nt; t++) dmu[t] = 0.0;
	for (int s = (int)nsub - 1; s >= 0; s--) {
		const double* O = Os + n3 * s;
		const double* wsub = ws + (size_t)nv * s;
		/* recompute the sweep of this substep, keeping each tet's forward */
		memcpy(Y, Xp + n3 * s, sizeof(double) * n3);
		for (uint32_t k = 0; k < nt; k++) {
			const uint32_t t = order[k];
			const uint32_t* is = tets + 4 * (size_t)t;
			double x[4][3], wl[4];
			for (int n = 0; n < 4; n++) { memcpy(x[n], Y + 3 * (size_t)is[n], sizeof(double) * 3); wl[n] = wsub[is[n]]; }
			tet_forward(x, wl, ep + ORC_EP * (size_t)t, tet_mu[t], p, &tf[k]);
			for (int n = 0; n < 4; n++) memcpy(Y + 3 * (size_t)is[n], x[n], sizeof(double) * 3);
		}
		/* locks and ground forward again (Y is the post-sweep position) */
		for (uint32_t i = 0; i < nv; i++) {
			const int locked = p->lock_active && lock_mask && (lock_mask[i] & 1u);
			gf[i].contact = 0;
			if (locked) memcpy(Y + 3 * (size_t)i, O + 3 * (size_t)i, sizeof(double) * 3);
			const double wi = locked ? 0.0 : wsub[i];
			if (p->ground && wi > 0.0) ground_forward(Y + 3 * (size_t)i, O + 3 * (size_t)i, p, &gf[i]);
		}
		/* loss at the end of substep s */
		for (uint32_t q = 0; q < ntip; q++)
			for (int k = 0; k < 3; k++) {
				const size_t j = 3 * (size_t)tips[q] + k;
				Xb[j] += 2.0 * (Y[j] - targets[((size_t)s * ntip + q) * 3 + k]);
			}
		/* V = (X - O) / dt, X_out = X */
		for (size_t j = 0; j < n3; j++) {
			Xb[j] += Vb[j] * inv_dt;
			Ob[j] = -Vb[j] * inv_dt;
		}
		/* ground, locks */
		for (uint32_t i = 0; i < nv; i++) {
			ground_reverse(&gf[i], Xb + 3 * (size_t)i, Ob + 3 * (size_t)i);
			if (p->lock_active && lock_mask && (lock_mask[i] & 1u)) {
				acc(Ob + 3 * (size_t)i, ld(Xb + 3 * (size_t)i));
				st(Xb + 3 * (size_t)i, v(0, 0, 0));
			}
		}
		/* the sweep, in reverse */
		for (int k = (int)nt - 1; k >= 0; k--) {
			const uint32_t t = order[k];
			const uint32_t* is = tets + 4 * (size_t)t;
			double xb[4][3], wl[4];
			for (int n = 0; n < 4; n++) { memcpy(xb[n], Xb + 3 * (size_t)is[n], sizeof(double) * 3); wl[n] = wsub[is[n]]; }
			dmu[t] += tet_reverse(&tf[k], wl, tet_mu[t], xb);
			for (int n = 0; n < 4; n++) memcpy(Xb + 3 * (size_t)is[n], xb[n], sizeof(double) * 3);
		}
		/* predict: O = X_in, Xp = X_in + V1 dt, V1 = (V_in + g dt) drag */
		for (size_t j = 0; j < n3; j++) {
			Vb[j] = Xb[j] * dt * drag;  /* V_out's adjoint was consumed above */
			Xb[j] += Ob[j];
		}
	}
	if (dV0) memcpy(dV0, Vb, sizeof(double) * n3);
	if (dX0) memcpy(dX0, Xb, sizeof(double) * n3);
done:
	free(Xp); free(Os); free(ws); free(X); free(V); free(w); free(Xb); free(Vb); free(Ob); free(Y); free(tf); free(gf);
	return 0;
}
