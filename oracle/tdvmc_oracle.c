/*
 * FP64 CPU oracle for the TDVP hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, in plain C, the reference algorithm of mathiasgartner/TDVMC for
 * the periodic pair-spline Bose system (PhysicalSystems::BosonsBulk) and the
 * TDVP driver pieces of src/TDVMC.cpp.  Every routine names the reference
 * lines it follows.  Used by tests/, __graft_entry__.smoke() and the CPU
 * baseline of bench.py only; never by the product library.
 *
 * Parity pin: tests/test_oracle_golden.py checks this file against fixtures
 * produced by the reference itself (oracle/ref/harness.cpp linked against the
 * reference sources; fixtures in tests/golden/).
 */
#include "tdvmc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

struct orc_sys {
	int dim, n, p, ns, nk;
	int np1, np2, np3;
	double L, Lr, L2, rmax, hbar2_2m, time;
	int pot_kind, npot;
	int variant;
	double pot[5];
	double knots[ORC_MAX_KNOTS];
	/* fold[k][s]: parameter k <- spline s (boundary-condition combination) */
	double* fold;
	/* loc[(b*4+q)*4+c]: spline b-q on bin b, coefficient of t^c */
	double* loc;
};

/* ------------------------------------------------------------------ */
/* minimum image: Utils.cpp:266-281 (GetCoordinateNIC), 368-382        */
/* ------------------------------------------------------------------ */
static double nic_coord(double x, double L, double Lr, double L2)
{
	int k = (int)(x * Lr + ((x >= 0.0) ? 0.5 : -0.5));
	double res = x - k * L;
	if (res == L2) res -= 1e-10;
	else if (res == -L2) res += 1e-10;
	return res;
}

double orc_nic_coord(double x, double L)
{
	return nic_coord(x, L, 1.0 / L, L / 2.0);
}

double orc_nic_disp(const double* ri, const double* rj, int dim, double L, double* d)
{
	double Lr = 1.0 / L, L2 = L / 2.0, r2 = 0.0;
	for (int a = 0; a < dim; a++)
	{
		d[a] = nic_coord(ri[a] - rj[a], L, Lr, L2);
		r2 += d[a] * d[a];
	}
	return sqrt(r2);
}

/* ------------------------------------------------------------------ */
/* B-spline pieces by the Cox-de Boor recursion                        */
/* (same polynomials as SplineFactory::GetWeights3, SplineFactory.cpp:54-101) */
/* ------------------------------------------------------------------ */

/* polynomial helpers, degree <= 3, c[0..3] */
static void poly_mul_lin(const double* a, double c0, double c1, double* out)
{
	double o[4] = {0, 0, 0, 0};
	for (int i = 0; i < 4; i++)
	{
		if (a[i] == 0.0) continue;
		o[i] += a[i] * c0;
		if (i + 1 < 4) o[i + 1] += a[i] * c1;
	}
	memcpy(out, o, sizeof(o));
}

/* Polynomial of B-spline N_{s,3} on knot interval b.  local != 0: variable
 * t = (r - k_b)/(k_{b+1} - k_b); otherwise variable r. */
static void bspline_piece(const double* k, int s, int b, int local, double* out)
{
	double N[4][4][4]; /* [degree][i - s][coef] */
	memset(N, 0, sizeof(N));
	double h = k[b + 1] - k[b];
	for (int i = 0; i < 4; i++)
		if (s + i == b) N[0][i][0] = 1.0;
	for (int d = 1; d <= 3; d++)
	{
		for (int i = 0; i + d <= 3; i++)
		{
			int ii = s + i;
			double acc[4] = {0, 0, 0, 0}, tmp[4];
			double den1 = k[ii + d] - k[ii];
			double den2 = k[ii + d + 1] - k[ii + 1];
			if (den1 != 0.0)
			{
				/* (r - k_ii) / den1 */
				double c0 = local ? (k[b] - k[ii]) / den1 : -k[ii] / den1;
				double c1 = local ? h / den1 : 1.0 / den1;
				poly_mul_lin(N[d - 1][i], c0, c1, tmp);
				for (int c = 0; c < 4; c++) acc[c] += tmp[c];
			}
			if (den2 != 0.0)
			{
				/* (k_{ii+d+1} - r) / den2 */
				double c0 = local ? (k[ii + d + 1] - k[b]) / den2 : k[ii + d + 1] / den2;
				double c1 = local ? -h / den2 : -1.0 / den2;
				poly_mul_lin(N[d - 1][i + 1], c0, c1, tmp);
				for (int c = 0; c < 4; c++) acc[c] += tmp[c];
			}
			memcpy(N[d][i], acc, sizeof(acc));
		}
	}
	memcpy(out, N[3][0], 4 * sizeof(double));
}

/* ------------------------------------------------------------------ */
/* system set-up: BosonsBulk.cpp:35-44 (SetNodes), 51-91 (InitSystem),  */
/* SplineFactory.cpp:423-439, 563-579 (uniform BC factors)             */
/* ------------------------------------------------------------------ */
orc_sys* orc_create(int dim, int n, int p, double L, const double* user_knots, int nuser,
                    int pot_kind, const double* pot, int npot, double time, double hbar2_2m)
{
	if (dim < 1 || dim > 3 || n < 2 || p < 4) return NULL;
	int nk = (nuser > 0) ? nuser + 6 : p + 6;
	if (nk > ORC_MAX_KNOTS) return NULL;
	orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
	s->dim = dim;
	s->n = n;
	s->p = p;
	s->L = L;
	s->Lr = 1.0 / L;
	s->L2 = L / 2.0;
	s->hbar2_2m = hbar2_2m;
	s->time = time;
	s->pot_kind = pot_kind;
	s->npot = npot < 5 ? npot : 5;
	for (int i = 0; i < s->npot; i++) s->pot[i] = pot[i];
	if (nuser > 0)
	{
		/* mirror three knots at each end */
		for (int i = 0; i < 3; i++) s->knots[i] = -user_knots[3 - i];
		for (int i = 0; i < nuser; i++) s->knots[3 + i] = user_knots[i];
		for (int i = 0; i < 3; i++) s->knots[3 + nuser + i] = 2.0 * user_knots[nuser - 1] - user_knots[nuser - 2 - i];
	}
	else
	{
		double half = L / 2.0;
		for (int i = -3; i < p + 3; i++) s->knots[i + 3] = ((double)i * half) / ((double)p - 1.0);
	}
	s->nk = nk;
	s->ns = nk - 4;
	s->rmax = s->knots[nk - 4];
	/* two start and two end conditions (uniform factors, as the reference passes uniform=true) */
	s->np1 = 2;
	s->np2 = s->np1 + (p - 4);
	s->np3 = s->np2 + 2;
	if (s->ns - 2 != p)
	{
		free(s);
		return NULL;
	}
	static const double bcs[2][3] = {{0, 1, 0}, {1, 0, 1}};
	static const double bce[2][3] = {{1, 0, 1}, {0, 1, 0}};
	s->fold = (double*)calloc((size_t)p * s->ns, sizeof(double));
	for (int i = 0; i < s->np1; i++)
		for (int j = 0; j < 3; j++) s->fold[i * s->ns + j] = bcs[i][j];
	for (int i = s->np1, sp = 3; i < s->np2; i++, sp++) s->fold[i * s->ns + sp] = 1.0;
	for (int i = s->np2, idx = 0; i < s->np3; i++, idx++)
		for (int j = 0; j < 3; j++) s->fold[i * s->ns + s->ns - 3 + j] = bce[idx][j];
	s->loc = (double*)calloc((size_t)nk * 16, sizeof(double));
	for (int b = 3; b <= nk - 5; b++)
		for (int q = 0; q < 4; q++) bspline_piece(s->knots, b - q, b, 1, s->loc + (b * 4 + q) * 4);
	return s;
}

/* NUBosonsBulkPB::RefreshLocalOperators (NUBosonsBulkPB.cpp:216-226) over the
 * p + 2 splines of the knot vector (the system declares p + 3; the last is never
 * filled) */
void orc_set_variant(orc_sys* s, int variant)
{
	s->variant = variant;
	if (variant != ORC_SYS_NU_PB && variant != ORC_SYS_NU_PB_EXACT) return;
	int P = s->p, ns = s->ns;
	memset(s->fold, 0, (size_t)P * ns * sizeof(double));
	for (int k = 0; k < P; k++) s->fold[k * ns + k + 1] = 1.0;
	s->fold[1 * ns + 0] += 1.0;
	s->fold[(P - 1) * ns + ns - 1] += 1.0;
}

/* The distance a pair enters the spline sums with, and whether it does.
 * BosonsBulk: r, inside r <= r_max (r < r_max for a moved particle's new
 * position, strict).  NUBosonsBulkPB: r' = 2 r_max - r beyond r_max, inside
 * r' < r_max (NUBosonsBulkPB.cpp:249-253, 333-336, 690-693).  rdiv (may be
 * NULL): what the derivative terms divide by, d / rdiv in the gradient and
 * (D-1) / rdiv in the Laplacian -- r' for NUBosonsBulkPB (:381-398), and for
 * its exact form -r at a mirrored pair (d r'/d r = -1 and grad r = d / r). */
static int pair_inside(const orc_sys* s, double r, int strict, double* reff, double* rdiv)
{
	if (s->variant == ORC_SYS_NU_PB || s->variant == ORC_SYS_NU_PB_EXACT)
	{
		int mirrored = !(r < s->rmax);
		double rr = mirrored ? 2.0 * s->rmax - r : r;
		if (rdiv) *rdiv = (mirrored && s->variant == ORC_SYS_NU_PB_EXACT) ? -r : rr;
		*reff = rr;
		return rr < s->rmax;
	}
	if (rdiv) *rdiv = r;
	*reff = r;
	return strict ? (r < s->rmax) : (r <= s->rmax);
}

void orc_free(orc_sys* s)
{
	if (!s) return;
	free(s->fold);
	free(s->loc);
	free(s);
}

int orc_num_knots(const orc_sys* s) { return s->nk; }
int orc_num_splines(const orc_sys* s) { return s->ns; }
double orc_rmax(const orc_sys* s) { return s->rmax; }
void orc_knots(const orc_sys* s, double* out) { memcpy(out, s->knots, (size_t)s->nk * sizeof(double)); }

void orc_abs_weights(const orc_sys* s, double* out)
{
	for (int sp = 0; sp < s->ns; sp++)
		for (int q = 0; q < 4; q++) bspline_piece(s->knots, sp, sp + q, 0, out + (sp * 4 + q) * 4);
}

void orc_local_weights(const orc_sys* s, double* out)
{
	memcpy(out, s->loc, (size_t)s->nk * 16 * sizeof(double));
}

/* interval by lower_bound as at BosonsBulk.cpp:197-198 */
static int find_bin(const orc_sys* s, double r)
{
	int lo = 0, hi = s->nk; /* first index with knots[idx] >= r */
	while (lo < hi)
	{
		int mid = (lo + hi) >> 1;
		if (s->knots[mid] < r) lo = mid + 1;
		else hi = mid;
	}
	int b = lo - 1;
	if (b < 3) b = 3;
	if (b > s->nk - 5) b = s->nk - 5;
	return b;
}

/* value, first and second r-derivative of the 4 splines b-q on bin b */
static void spline_eval(const orc_sys* s, int b, double r, double* v, double* d1, double* d2)
{
	double h = s->knots[b + 1] - s->knots[b];
	double t = (r - s->knots[b]) / h;
	for (int q = 0; q < 4; q++)
	{
		const double* c = s->loc + (b * 4 + q) * 4;
		if (v) v[q] = c[0] + t * (c[1] + t * (c[2] + t * c[3]));
		if (d1) d1[q] = (c[1] + t * (2.0 * c[2] + t * 3.0 * c[3])) / h;
		if (d2) d2[q] = (2.0 * c[2] + 6.0 * c[3] * t) / (h * h);
	}
}

/* pair potential with the quench rule of BosonsBulk.cpp:237-242 */
static double pair_potential(const orc_sys* s, double r)
{
	double a = s->pot[0], b = s->pot[1];
	if (s->npot > 2 && s->time >= s->pot[2])
	{
		a = s->pot[3];
		b = s->pot[4];
	}
	switch (s->pot_kind)
	{
	case ORC_POT_SQUARE:
		return (r < a) ? b : 0.0;
	case ORC_POT_GAUSS:
	{
		double x = r / a;
		return b * exp(-(x * x) / 2.0);
	}
	case ORC_POT_LJ:
	{
		double s2 = (a / r) * (a / r);
		double s6 = s2 * s2 * s2;
		return 4.0 * b * s6 * (s6 - 1.0);
	}
	default:
		return 0.0;
	}
}

static void fold_apply(const orc_sys* s, const double* S, double* O)
{
	for (int k = 0; k < s->p; k++)
	{
		double acc = 0.0;
		for (int j = 0; j < s->ns; j++) acc += s->fold[k * s->ns + j] * S[j];
		O[k] = acc;
	}
}

/* spline sums and outside count: BosonsBulk.cpp:179-218 */
static void spline_sums(const orc_sys* s, const double* R, double* S, double* nout)
{
	int n = s->n, D = s->dim;
	double d[3], v[4];
	memset(S, 0, (size_t)s->ns * sizeof(double));
	*nout = 0.0;
	for (int a = 0; a < n; a++)
		for (int i = 0; i < a; i++)
		{
			double re, r = orc_nic_disp(R + a * D, R + i * D, D, s->L, d);
			if (pair_inside(s, r, 0, &re, NULL))
			{
				int b = find_bin(s, re);
				spline_eval(s, b, re, v, NULL, NULL);
				for (int q = 0; q < 4; q++) S[b - q] += v[q];
			}
			else *nout += 1.0;
		}
}

/* exponent: BosonsBulk.cpp:522-539 */
static double exponent_of(const orc_sys* s, const double* uR, const double* S, double nout)
{
	double* O = (double*)malloc((size_t)s->p * sizeof(double));
	fold_apply(s, S, O);
	double sum = 0.0;
	for (int k = 0; k < s->p; k++) sum += uR[k] * O[k];
	sum += uR[s->p - 1] * nout;
	free(O);
	return sum;
}

void orc_eval(const orc_sys* s, const double* uR, const double* uI, const double* R,
              double* lnpsi, double* O, double* eloc, double* other7, double* dE)
{
	int n = s->n, D = s->dim, ns = s->ns, P = s->p;
	double* S = (double*)calloc((size_t)ns, sizeof(double));
	double* wR = (double*)calloc((size_t)ns, sizeof(double));
	double* wI = (double*)calloc((size_t)ns, sizeof(double));
	double* G = (double*)calloc((size_t)n * 6, sizeof(double)); /* [n][re xyz, im xyz] */
	double* Lsp = (double*)calloc((size_t)ns, sizeof(double));
	double* AR = (double*)calloc((size_t)ns, sizeof(double));
	double* AI = (double*)calloc((size_t)ns, sizeof(double));
	double nout, vint = 0.0, lapR = 0.0, lapI = 0.0;
	double d[3], d1[4], d2[4];

	spline_sums(s, R, S, &nout);
	fold_apply(s, S, O);
	double e = 0.0;
	for (int k = 0; k < P; k++) e += uR[k] * O[k];
	e += uR[P - 1] * nout;
	*lnpsi = e;

	/* per-spline complex weights w_s = sum_k alpha_k fold[k][s] */
	for (int k = 0; k < P; k++)
		for (int j = 0; j < ns; j++)
		{
			wR[j] += uR[k] * s->fold[k * ns + j];
			wI[j] += uI[k] * s->fold[k * ns + j];
		}

	/* ordered pairs: BosonsBulk.cpp:249-331 (sD, sD2, V) folded with alpha as 370-421 */
	for (int a = 0; a < n; a++)
	{
		for (int i = 0; i < n; i++)
		{
			if (i == a) continue;
			double rq, r = orc_nic_disp(R + a * D, R + i * D, D, s->L, d);
			if (!pair_inside(s, r, 0, &r, &rq)) continue; /* r: the distance the pair enters with */
			if (i < a) vint += pair_potential(s, r);
			int b = find_bin(s, r);
			spline_eval(s, b, r, NULL, d1, d2);
			double u1R = 0, u1I = 0, u2R = 0, u2I = 0;
			for (int q = 0; q < 4; q++)
			{
				int sp = b - q;
				u1R += wR[sp] * d1[q];
				u1I += wI[sp] * d1[q];
				u2R += wR[sp] * d2[q];
				u2I += wI[sp] * d2[q];
				Lsp[sp] += d2[q] + (D - 1.0) / rq * d1[q];
			}
			for (int c = 0; c < D; c++)
			{
				double e_c = d[c] / rq;
				G[a * 6 + c] += u1R * e_c;
				G[a * 6 + 3 + c] += u1I * e_c;
			}
			lapR += u2R + (D - 1.0) / rq * u1R;
			lapI += u2I + (D - 1.0) / rq * u1I;
		}
	}
	double sR1 = 0, sI1 = 0, sR1I1 = 0;
	for (int a = 0; a < n; a++)
	{
		double rr = 0, ii = 0, ri = 0;
		for (int c = 0; c < D; c++)
		{
			rr += G[a * 6 + c] * G[a * 6 + c];
			ii += G[a * 6 + 3 + c] * G[a * 6 + 3 + c];
			ri += G[a * 6 + c] * G[a * 6 + 3 + c];
		}
		sR1I1 += 2.0 * ri;
		sR1 += rr;
		sI1 += ii;
	}
	double c = s->hbar2_2m;
	double kinR = -(sR1 - sI1 + lapR) * c;
	double kinI = -(sR1I1 + lapI) * c;
	eloc[0] = kinR + vint;
	eloc[1] = kinI;
	other7[0] = kinR;
	other7[1] = vint;
	other7[2] = sR1;
	other7[3] = sI1;
	other7[4] = lapR;
	other7[5] = lapI;
	other7[6] = sR1I1;

	if (dE)
	{
		/* reverse sweep: A_s = sum over ordered pairs of B'_s(r) (G_a . rhat) */
		for (int a = 0; a < n; a++)
			for (int i = 0; i < n; i++)
			{
				if (i == a) continue;
				double rq, r = orc_nic_disp(R + a * D, R + i * D, D, s->L, d);
				if (!pair_inside(s, r, 0, &r, &rq)) continue;
				int b = find_bin(s, r);
				spline_eval(s, b, r, NULL, d1, NULL);
				double gR = 0, gI = 0;
				for (int cc = 0; cc < D; cc++)
				{
					gR += G[a * 6 + cc] * d[cc] / rq;
					gI += G[a * 6 + 3 + cc] * d[cc] / rq;
				}
				for (int q = 0; q < 4; q++)
				{
					AR[b - q] += d1[q] * gR;
					AI[b - q] += d1[q] * gI;
				}
			}
		for (int k = 0; k < P; k++)
		{
			double re = 0, im = 0;
			for (int j = 0; j < ns; j++)
			{
				double f = s->fold[k * ns + j];
				if (f == 0.0) continue;
				re += f * (2.0 * AR[j] + Lsp[j]);
				im += f * (2.0 * AI[j]);
			}
			dE[2 * k] = -c * re;
			dE[2 * k + 1] = -c * im;
		}
	}
	free(S);
	free(wR);
	free(wI);
	free(G);
	free(Lsp);
	free(AR);
	free(AI);
}

/* ------------------------------------------------------------------ */
/* single-particle move: BosonsBulk.cpp:553-657                         */
/* ------------------------------------------------------------------ */
typedef struct
{
	double* S;
	double* sold;
	double* snew;
	double nout;
	double exponent;
} move_state;

static void move_sums(const orc_sys* s, const double* R, int p, const double* x, int strict, double* acc, double* out)
{
	int D = s->dim;
	double d[3], v[4];
	memset(acc, 0, (size_t)s->ns * sizeof(double));
	*out = 0.0;
	for (int i = 0; i < s->n; i++)
	{
		if (i == p) continue;
		double r = orc_nic_disp(R + i * D, x, D, s->L, d);
		int inside = pair_inside(s, r, strict, &r, NULL);
		if (inside)
		{
			int b = find_bin(s, r);
			spline_eval(s, b, r, v, NULL, NULL);
			for (int q = 0; q < 4; q++) acc[b - q] += v[q];
		}
		else *out += 1.0;
	}
}

/* returns exponentNew; updates nothing */
static double move_exponent(const orc_sys* s, const double* uR, move_state* st, const double* R, int p, const double* xold,
                            const double* xnew, double* Snew, double* noutnew)
{
	double oo, on;
	move_sums(s, R, p, xold, 0, st->sold, &oo);
	move_sums(s, R, p, xnew, 1, st->snew, &on);
	for (int j = 0; j < s->ns; j++)
	{
		double v = st->S[j] - st->sold[j] + st->snew[j];
		Snew[j] = v > 0.0 ? v : 0.0;
	}
	double no = st->nout - oo + on;
	*noutnew = no > 0.0 ? no : 0.0;
	return exponent_of(s, uR, Snew, *noutnew);
}

double orc_move_delta(const orc_sys* s, const double* uR, const double* R, int p, const double* newpos)
{
	move_state st;
	st.S = (double*)calloc((size_t)s->ns, sizeof(double));
	st.sold = (double*)calloc((size_t)s->ns, sizeof(double));
	st.snew = (double*)calloc((size_t)s->ns, sizeof(double));
	double* Snew = (double*)calloc((size_t)s->ns, sizeof(double));
	spline_sums(s, R, st.S, &st.nout);
	st.exponent = exponent_of(s, uR, st.S, st.nout);
	double nn;
	double e1 = move_exponent(s, uR, &st, R, p, R + p * s->dim, newpos, Snew, &nn);
	double res = e1 - st.exponent;
	free(st.S);
	free(st.sold);
	free(st.snew);
	free(Snew);
	return res;
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), restated          */
/* ------------------------------------------------------------------ */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
	uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
	uint32_t k0 = key[0], k1 = key[1];
	for (int r = 0; r < 10; r++)
	{
		uint64_t p0 = (uint64_t)0xD2511F53u * c0;
		uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
		uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
		uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
		c0 = hi1 ^ c1 ^ k0;
		c1 = lo1;
		c2 = hi0 ^ c3 ^ k1;
		c3 = lo0;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
	out[0] = c0;
	out[1] = c1;
	out[2] = c2;
	out[3] = c3;
}

static double u01(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }

/* Random numbers of one move: particle, accept uniform, dim normals. */
static void move_randoms(int n, int dim, uint32_t move, uint32_t walker, uint32_t pass, uint64_t seed,
                         int* part, double* uacc, double* z)
{
	uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
	uint32_t ctr[4] = {move, walker, pass, 0u};
	uint32_t a[4], b[4];
	orc_philox(ctr, key, a);
	*part = (int)(((uint64_t)a[0] * (uint64_t)n) >> 32);
	*uacc = u01(a[1]);
	double rho = sqrt(-2.0 * log(u01(a[2])));
	double th = 2.0 * M_PI * u01(a[3]);
	z[0] = rho * cos(th);
	if (dim > 1) z[1] = rho * sin(th);
	if (dim > 2)
	{
		ctr[3] = 1u;
		orc_philox(ctr, key, b);
		double rho2 = sqrt(-2.0 * log(u01(b[0])));
		double th2 = 2.0 * M_PI * u01(b[1]);
		z[2] = rho2 * cos(th2);
	}
}

/* sampling of one walker held AoS in R (n*dim) */
static int64_t sample_walker(const orc_sys* s, const double* uR, double* R, int moves, double step, uint64_t seed,
                             uint32_t pass, uint32_t walker)
{
	int D = s->dim, ns = s->ns;
	move_state st;
	st.S = (double*)calloc((size_t)ns, sizeof(double));
	st.sold = (double*)calloc((size_t)ns, sizeof(double));
	st.snew = (double*)calloc((size_t)ns, sizeof(double));
	double* Snew = (double*)calloc((size_t)ns, sizeof(double));
	/* CalculateWavefunction at the start of a pass: TDVMC.cpp:1060 */
	spline_sums(s, R, st.S, &st.nout);
	st.exponent = exponent_of(s, uR, st.S, st.nout);
	int64_t acc = 0;
	for (int m = 0; m < moves; m++)
	{
		int p;
		double U, z[3], xnew[3];
		move_randoms(s->n, D, (uint32_t)m, walker, pass, seed, &p, &U, z);
		for (int a = 0; a < D; a++) xnew[a] = nic_coord(R[p * D + a] + step * z[a], s->L, s->Lr, s->L2);
		double nn;
		double enew = move_exponent(s, uR, &st, R, p, R + p * D, xnew, Snew, &nn);
		double delta = enew - st.exponent;
		/* TDVMC.cpp:886-915: exp(2 delta) >= U accepts; a non-finite quotient,
		 * including exp overflow beyond log(DBL_MAX), rejects */
		if (isfinite(delta) && 2.0 * delta >= log(U) && 2.0 * delta < 709.782712893384)
		{
			for (int a = 0; a < D; a++) R[p * D + a] = xnew[a];
			memcpy(st.S, Snew, (size_t)ns * sizeof(double));
			st.nout = nn;
			st.exponent = enew;
			acc++;
		}
	}
	free(st.S);
	free(st.sold);
	free(st.snew);
	free(Snew);
	return acc;
}

static void soa_to_aos(const orc_sys* s, const double* Rsoa, int64_t w, double* R)
{
	int n = s->n, D = s->dim;
	for (int a = 0; a < D; a++)
		for (int i = 0; i < n; i++) R[i * D + a] = Rsoa[((size_t)w * D + a) * n + i];
}

static void aos_to_soa(const orc_sys* s, const double* R, int64_t w, double* Rsoa)
{
	int n = s->n, D = s->dim;
	for (int a = 0; a < D; a++)
		for (int i = 0; i < n; i++) Rsoa[((size_t)w * D + a) * n + i] = R[i * D + a];
}

int64_t orc_sample(const orc_sys* s, const double* uR, double* Rsoa, int64_t nw_total, int64_t w0, int64_t nw,
                   int moves, double step, uint64_t seed, uint32_t pass)
{
	(void)nw_total;
	double* R = (double*)malloc((size_t)s->n * s->dim * sizeof(double));
	int64_t acc = 0;
	for (int64_t w = w0; w < w0 + nw; w++)
	{
		soa_to_aos(s, Rsoa, w, R);
		acc += sample_walker(s, uR, R, moves, step, seed, pass, (uint32_t)w);
		aos_to_soa(s, R, w, Rsoa);
	}
	free(R);
	return acc;
}

typedef struct
{
	const orc_sys* s;
	const double *uR, *uI;
	double* Rsoa;
	int64_t w0, w1;
	int moves;
	double step;
	uint64_t seed;
	uint32_t pass;
	double *lnpsi, *O, *eloc, *other7, *dE;
	int64_t acc;
} stage_job;

static void* stage_worker(void* arg)
{
	stage_job* j = (stage_job*)arg;
	const orc_sys* s = j->s;
	double* R = (double*)malloc((size_t)s->n * s->dim * sizeof(double));
	j->acc = 0;
	for (int64_t w = j->w0; w < j->w1; w++)
	{
		soa_to_aos(s, j->Rsoa, w, R);
		if (j->moves > 0) j->acc += sample_walker(s, j->uR, R, j->moves, j->step, j->seed, j->pass, (uint32_t)w);
		aos_to_soa(s, R, w, j->Rsoa);
		orc_eval(s, j->uR, j->uI, R, j->lnpsi + w, j->O + (size_t)w * s->p, j->eloc + 2 * w, j->other7 + 7 * w,
		         j->dE ? j->dE + (size_t)w * 2 * s->p : NULL);
	}
	free(R);
	return NULL;
}

int64_t orc_stage_threads(const orc_sys* s, const double* uR, const double* uI, double* Rsoa, int64_t nw,
                          int moves, double step, uint64_t seed, uint32_t pass, int threads,
                          double* lnpsi, double* O, double* eloc, double* other7, double* dE)
{
	if (threads < 1) threads = 1;
	if (threads > nw) threads = (int)nw;
	pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
	stage_job* jobs = (stage_job*)calloc((size_t)threads, sizeof(stage_job));
	for (int t = 0; t < threads; t++)
	{
		stage_job* j = &jobs[t];
		j->s = s;
		j->uR = uR;
		j->uI = uI;
		j->Rsoa = Rsoa;
		j->w0 = nw * t / threads;
		j->w1 = nw * (t + 1) / threads;
		j->moves = moves;
		j->step = step;
		j->seed = seed;
		j->pass = pass;
		j->lnpsi = lnpsi;
		j->O = O;
		j->eloc = eloc;
		j->other7 = other7;
		j->dE = dE;
		pthread_create(&th[t], NULL, stage_worker, j);
	}
	int64_t acc = 0;
	for (int t = 0; t < threads; t++)
	{
		pthread_join(th[t], NULL);
		acc += jobs[t].acc;
	}
	free(th);
	free(jobs);
	return acc;
}

/* ------------------------------------------------------------------ */
/* TDVP solve: TDVMC.cpp:1506-1537, 1560-1622, 1658-1682, 1684-1711,    */
/* 1713-1828                                                            */
/* ------------------------------------------------------------------ */
static int cholesky_ref(int P, double* m)
{
	int bad = 0;
	for (int i = 0; i < P; i++)
		for (int j = 0; j <= i; j++)
		{
			double sum = m[i * P + j];
			for (int k = 0; k < j; k++) sum -= m[i * P + k] * m[j * P + k];
			if (i > j) m[i * P + j] = sum / m[j * P + j];
			else if (sum > 0) m[i * P + i] = sqrt(sum);
			else bad = 1;
		}
	return bad;
}

static void cholesky_solve_ref(int P, const double* m, const double* rhs, double* sol)
{
	double* tmp = (double*)calloc((size_t)P, sizeof(double));
	for (int i = 0; i < P; i++)
	{
		double sum = 0;
		for (int j = 0; j < i; j++) sum += m[i * P + j] * tmp[j];
		tmp[i] = 1.0 / m[i * P + i] * (rhs[i] - sum);
	}
	for (int i = P - 1; i >= 0; i--)
	{
		double sum = 0;
		for (int j = P - 1; j > i; j--) sum += m[j * P + i] * sol[j];
		sol[i] = 1.0 / m[i * P + i] * (tmp[i] - sum);
	}
	free(tmp);
}

/* dense solve with partial pivoting (unique solution of a nonsingular system) */
static void lu_solve(int P, const double* A, const double* b, double* x)
{
	double* m = (double*)malloc((size_t)P * (P + 1) * sizeof(double));
	for (int i = 0; i < P; i++)
	{
		for (int j = 0; j < P; j++) m[i * (P + 1) + j] = A[i * P + j];
		m[i * (P + 1) + P] = b[i];
	}
	for (int c = 0; c < P; c++)
	{
		int piv = c;
		for (int r = c + 1; r < P; r++)
			if (fabs(m[r * (P + 1) + c]) > fabs(m[piv * (P + 1) + c])) piv = r;
		if (piv != c)
			for (int j = 0; j <= P; j++)
			{
				double t = m[c * (P + 1) + j];
				m[c * (P + 1) + j] = m[piv * (P + 1) + j];
				m[piv * (P + 1) + j] = t;
			}
		for (int r = c + 1; r < P; r++)
		{
			double f = m[r * (P + 1) + c] / m[c * (P + 1) + c];
			for (int j = c; j <= P; j++) m[r * (P + 1) + j] -= f * m[c * (P + 1) + j];
		}
	}
	for (int i = P - 1; i >= 0; i--)
	{
		double sum = m[i * (P + 1) + P];
		for (int j = i + 1; j < P; j++) sum -= m[i * (P + 1) + j] * x[j];
		x[i] = sum / m[i * (P + 1) + i];
	}
	free(m);
}

static int solve_core(int P, int imag, int precond, int solver, const double* O, double ER, double* m, double* fr,
                      double* fi, double* uDotR, double* uDotI, double* phiDotR, double* phiDotI);

int orc_solve(int P, int imag, int precond, int solver, const double* O, double ER, double EI,
              const double* OO, const double* OER, const double* OEI,
              double* uDotR, double* uDotI, double* phiDotR, double* phiDotI)
{
	double* m = (double*)malloc((size_t)P * P * sizeof(double));
	double* fr = (double*)malloc((size_t)P * sizeof(double));
	double* fi = (double*)malloc((size_t)P * sizeof(double));
	for (int i = 0; i < P; i++)
	{
		if (imag == 0)
		{
			fr[i] = OEI[i] - EI * O[i];
			fi[i] = -OER[i] + ER * O[i];
		}
		else
		{
			fr[i] = -OER[i] + ER * O[i];
			fi[i] = -OEI[i];
		}
		for (int j = 0; j <= i; j++)
		{
			m[i * P + j] = OO[i * P + j] - O[i] * O[j];
			m[j * P + i] = m[i * P + j];
		}
	}
	int bad = solve_core(P, imag, precond, solver, O, ER, m, fr, fi, uDotR, uDotI, phiDotR, phiDotI);
	free(m);
	free(fr);
	free(fi);
	return bad;
}

int orc_solve_centred(int P, int imag, int precond, int solver, const double* O, double ER, double EI,
                      const double* S, const double* covOER, const double* covOEI,
                      double* uDotR, double* uDotI, double* phiDotR, double* phiDotI)
{
	double* m = (double*)malloc((size_t)P * P * sizeof(double));
	double* fr = (double*)malloc((size_t)P * sizeof(double));
	double* fi = (double*)malloc((size_t)P * sizeof(double));
	for (int i = 0; i < P; i++)
	{
		if (imag == 0)
		{
			fr[i] = covOEI[i];
			fi[i] = -covOER[i];
		}
		else
		{
			fr[i] = -covOER[i];
			fi[i] = -(covOEI[i] + O[i] * EI);
		}
		for (int j = 0; j < P; j++) m[i * P + j] = S[i * P + j];
	}
	int bad = solve_core(P, imag, precond, solver, O, ER, m, fr, fi, uDotR, uDotI, phiDotR, phiDotI);
	free(m);
	free(fr);
	free(fi);
	return bad;
}

static int solve_core(int P, int imag, int precond, int solver, const double* O, double ER, double* m, double* fr,
                      double* fi, double* uDotR, double* uDotI, double* phiDotR, double* phiDotI)
{
	double* sc = (double*)malloc((size_t)P * sizeof(double));
	int bad = 0;
	if (precond)
	{
		for (int i = 0; i < P; i++) sc[i] = sqrt(m[i * P + i]);
		for (int i = 0; i < P; i++)
		{
			for (int j = 0; j < P; j++) m[i * P + j] /= (sc[i] * sc[j]);
			fr[i] /= sc[i];
			fi[i] /= sc[i];
		}
	}
	if (solver == 0)
	{
		for (int i = 0; i < P; i++) m[i * P + i] += 0.001;
		bad = cholesky_ref(P, m);
		cholesky_solve_ref(P, m, fr, uDotR);
		cholesky_solve_ref(P, m, fi, uDotI);
	}
	else
	{
		if (precond)
			for (int i = 0; i < P; i++) m[i * P + i] += 0.002;
		lu_solve(P, m, fr, uDotR);
		lu_solve(P, m, fi, uDotI);
		double mr = 0, mi = 0;
		for (int i = 0; i < P; i++)
		{
			mr += uDotR[i];
			mi += uDotI[i];
		}
		mr /= P;
		mi /= P;
		for (int i = 0; i < P; i++)
		{
			uDotR[i] -= mr;
			uDotI[i] -= mi;
		}
	}
	/* CalculatePhiDot (TDVMC.cpp:1658-1682) runs before the preconditioning
	 * scale is undone, as in the reference */
	double pr = 0, pi = 0;
	for (int i = 0; i < P; i++)
	{
		pr -= O[i] * uDotR[i];
		pi -= O[i] * uDotI[i];
	}
	if (imag == 0) pi -= ER;
	else pr -= ER;
	*phiDotR = pr;
	*phiDotI = pi;
	if (precond)
		for (int i = 0; i < P; i++)
		{
			uDotR[i] /= sc[i];
			uDotI[i] /= sc[i];
		}
	free(sc);
	return bad;
}

/* ------------------------------------------------------------------ */
/* g(r) and S(k): BosonsBulk.cpp:474-520                               */
/* ------------------------------------------------------------------ */
int orc_observables(const orc_sys* s, const double* R, int gr_bins, int nshell, const int* shell_off,
                    const double* kvec, double* gr, double* sk)
{
	const int D = s->dim, N = s->n;
	/* grid [0, r_max) with spacing r_max / GR_BIN_COUNT (BosonsBulk.cpp:145,
	 * Grid::Init: count = (max - min) / spacing, truncated) */
	const double spacing = s->rmax / gr_bins;
	const int count = (int)((s->rmax - 0.0) / spacing);
	double* scale = (double*)malloc((size_t)(count > 0 ? count : 1) * sizeof(double));
	/* InitScaling: shell volumes (ObservableVsOnGridWithScaling.cpp:19-44) */
	for (int i = 0; i < count; i++)
	{
		if (D == 1) scale[i] = spacing;
		else if (D == 3) scale[i] = 4.0 * M_PI * pow(spacing * (i + 1), 3.0) / 3.0;
		else scale[i] = M_PI * pow(spacing * (i + 1), 2.0);
	}
	if (D > 1)
		for (int i = count - 1; i > 0; i--) scale[i] = scale[i] - scale[i - 1];
	for (int i = 0; i < count; i++) gr[i] = 0.0;
	const double weight = 1.0 / ((double)(N - 1)) * D;
	double d[3];
	for (int i = 0; i < N; i++)
		for (int j = 0; j < i; j++)
		{
			const double r = orc_nic_disp(R + i * D, R + j * D, D, s->L, d);
			if (r < s->rmax)
			{
				const int bin = (int)floor(r / spacing); /* Grid::GetIndex */
				if (bin < count) gr[bin] += weight / scale[bin];
			}
		}
	free(scale);
	/* structure factor: per shell the squared modulus of the sum over the
	 * shell's vectors and the particles, over N * (vectors in the shell) */
	double* sc = (double*)calloc((size_t)(nshell > 0 ? nshell : 1), sizeof(double));
	double* ss = (double*)calloc((size_t)(nshell > 0 ? nshell : 1), sizeof(double));
	for (int i = 0; i < N; i++)
		for (int k = 0; k < nshell; k++)
			for (int v = shell_off[k]; v < shell_off[k + 1]; v++)
			{
				double dot = 0.0;
				for (int a = 0; a < D; a++) dot += kvec[v * D + a] * R[i * D + a];
				sc[k] += cos(dot);
				ss[k] += sin(dot);
			}
	for (int k = 0; k < nshell; k++)
	{
		const int nv = shell_off[k + 1] - shell_off[k];
		sk[k] = nv > 0 ? (sc[k] * sc[k] + ss[k] * ss[k]) / ((double)(N * nv)) : 0.0;
	}
	free(sc);
	free(ss);
	return count;
}

/* ------------------------------------------------------------------ */
/* Trapped drops: open boundaries, pair spline + one-body Gaussian      */
/* ------------------------------------------------------------------ */
/* No reference system has this form.  The pair spline restates a1-a9 of
 * BosonsBulk (knots, fold, outer-pair term uR[p-1] n_out, B-spline
 * derivatives, BosonsBulk.cpp:61-87, 179-218, 220-336, 349-458, 522-545) with
 * the plain displacement of the open-boundary cluster systems
 * (BosonCluster.cpp:14 USE_NIC = false; VectorDisplacement in its pair loop,
 * BosonCluster.cpp:296).  Added terms, parameter k = p:
 *   ln psi += alpha_p sum_i |r_i|^2,  O_p = sum_i |r_i|^2,
 *   V += kappa sum_i |r_i|^2 with kappa = omega^2 / (4 hbar2_2m) (the trap
 *   (m/2) omega^2 r^2 with hbar = 1), and the Gaussian pair repulsion
 *   v0 exp(-r^2 / (2 sigma^2)) over all pairs.
 * Known answer: v0 = 0, uR[0..p-1] = uI = 0, alpha_p = -omega / (4 hbar2_2m)
 * is the exact ground state, E_loc = (3/2) omega n for every configuration. */
struct orc_drop {
	orc_sys* s; /* pair spline on [0, rmax] (knots of a box of length 2 rmax) */
	int n, p;
	double v0, sigma, kappa;
};

orc_drop* orc_drop_create(int n, int p, double rmax, double v0, double sigma, double omega, double hbar2_2m)
{
	if (n < 2 || p < 4 || !(rmax > 0.0) || !(hbar2_2m > 0.0)) return NULL;
	double none = 0.0;
	orc_sys* s = orc_create(3, n, p, 2.0 * rmax, NULL, 0, ORC_POT_NONE, &none, 0, 0.0, hbar2_2m);
	if (!s) return NULL;
	orc_drop* d = (orc_drop*)calloc(1, sizeof(orc_drop));
	d->s = s;
	d->n = n;
	d->p = p;
	d->v0 = v0;
	d->sigma = sigma;
	d->kappa = omega * omega / (4.0 * hbar2_2m);
	return d;
}

void orc_drop_free(orc_drop* d)
{
	if (!d) return;
	orc_free(d->s);
	free(d);
}

static double drop_disp(const double* a, const double* b, double* d)
{
	double r2 = 0.0;
	for (int c = 0; c < 3; c++)
	{
		d[c] = a[c] - b[c];
		r2 += d[c] * d[c];
	}
	return sqrt(r2);
}

/* pair function u(r) of the spline part (uR only) */
static double drop_u(const orc_sys* s, const double* wR, double r, double uout)
{
	if (r > s->rmax) return uout;
	int b = find_bin(s, r);
	double v[4];
	spline_eval(s, b, r, v, NULL, NULL);
	double u = 0.0;
	for (int q = 0; q < 4; q++) u += wR[b - q] * v[q];
	return u;
}

void orc_drop_eval(const orc_drop* dp, const double* uR, const double* uI, const double* R, double* lnpsi,
                   double* O, double* eloc, double* other7, double* dE)
{
	const orc_sys* s = dp->s;
	const int n = dp->n, P = dp->p, ns = s->ns, D = 3;
	double* S = (double*)calloc((size_t)ns, sizeof(double));
	double* wR = (double*)calloc((size_t)ns, sizeof(double));
	double* wI = (double*)calloc((size_t)ns, sizeof(double));
	double* G = (double*)calloc((size_t)n * 6, sizeof(double));
	double* Lsp = (double*)calloc((size_t)ns, sizeof(double));
	double* AR = (double*)calloc((size_t)ns, sizeof(double));
	double* AI = (double*)calloc((size_t)ns, sizeof(double));
	double nout = 0.0, vint = 0.0, lapR = 0.0, lapI = 0.0, r2sum = 0.0;
	double d[3], v[4], d1[4], d2[4];
	/* spline sums, outer pairs, pair potential over i < a */
	for (int a = 0; a < n; a++)
		for (int i = 0; i < a; i++)
		{
			double r = drop_disp(R + a * D, R + i * D, d);
			vint += dp->v0 * exp(-(r * r) / (2.0 * dp->sigma * dp->sigma));
			if (r <= s->rmax)
			{
				int b = find_bin(s, r);
				spline_eval(s, b, r, v, NULL, NULL);
				for (int q = 0; q < 4; q++) S[b - q] += v[q];
			}
			else nout += 1.0;
		}
	fold_apply(s, S, O);
	for (int a = 0; a < n; a++)
		for (int c = 0; c < D; c++) r2sum += R[a * D + c] * R[a * D + c];
	O[P] = r2sum;
	double e = 0.0;
	for (int k = 0; k < P; k++) e += uR[k] * O[k];
	e += uR[P - 1] * nout + uR[P] * r2sum;
	*lnpsi = e;
	for (int k = 0; k < P; k++)
		for (int j = 0; j < ns; j++)
		{
			wR[j] += uR[k] * s->fold[k * ns + j];
			wI[j] += uI[k] * s->fold[k * ns + j];
		}
	/* ordered pairs within r_max: gradients and Laplacian of the pair part */
	for (int a = 0; a < n; a++)
		for (int i = 0; i < n; i++)
		{
			if (i == a) continue;
			double r = drop_disp(R + a * D, R + i * D, d);
			if (r > s->rmax) continue;
			int b = find_bin(s, r);
			spline_eval(s, b, r, NULL, d1, d2);
			double u1R = 0, u1I = 0, u2R = 0, u2I = 0;
			for (int q = 0; q < 4; q++)
			{
				int sp = b - q;
				u1R += wR[sp] * d1[q];
				u1I += wI[sp] * d1[q];
				u2R += wR[sp] * d2[q];
				u2I += wI[sp] * d2[q];
				Lsp[sp] += d2[q] + (D - 1.0) / r * d1[q];
			}
			for (int c = 0; c < D; c++)
			{
				G[a * 6 + c] += u1R * d[c] / r;
				G[a * 6 + 3 + c] += u1I * d[c] / r;
			}
			lapR += u2R + (D - 1.0) / r * u1R;
			lapI += u2I + (D - 1.0) / r * u1I;
		}
	/* one-body term: gradient 2 alpha_p r, Laplacian 2 D alpha_p per particle */
	for (int a = 0; a < n; a++)
		for (int c = 0; c < D; c++)
		{
			G[a * 6 + c] += 2.0 * uR[P] * R[a * D + c];
			G[a * 6 + 3 + c] += 2.0 * uI[P] * R[a * D + c];
		}
	lapR += 2.0 * D * uR[P] * n;
	lapI += 2.0 * D * uI[P] * n;
	double sR1 = 0, sI1 = 0, sR1I1 = 0, gr = 0, gi = 0;
	for (int a = 0; a < n; a++)
		for (int c = 0; c < D; c++)
		{
			const double x = G[a * 6 + c], y = G[a * 6 + 3 + c];
			sR1 += x * x;
			sI1 += y * y;
			sR1I1 += 2.0 * x * y;
			gr += x * R[a * D + c];
			gi += y * R[a * D + c];
		}
	const double c = s->hbar2_2m;
	const double vtot = vint + dp->kappa * r2sum;
	double kinR = -(sR1 - sI1 + lapR) * c;
	double kinI = -(sR1I1 + lapI) * c;
	eloc[0] = kinR + vtot;
	eloc[1] = kinI;
	other7[0] = kinR;
	other7[1] = vtot;
	other7[2] = sR1;
	other7[3] = sI1;
	other7[4] = lapR;
	other7[5] = lapI;
	other7[6] = sR1I1;
	if (dE)
	{
		/* A_s = sum over ordered pairs of B'_s(r) (G_a . rhat), G the full gradient */
		for (int a = 0; a < n; a++)
			for (int i = 0; i < n; i++)
			{
				if (i == a) continue;
				double r = drop_disp(R + a * D, R + i * D, d);
				if (r > s->rmax) continue;
				int b = find_bin(s, r);
				spline_eval(s, b, r, NULL, d1, NULL);
				double g_r = 0, g_i = 0;
				for (int cc = 0; cc < D; cc++)
				{
					g_r += G[a * 6 + cc] * d[cc] / r;
					g_i += G[a * 6 + 3 + cc] * d[cc] / r;
				}
				for (int q = 0; q < 4; q++)
				{
					AR[b - q] += d1[q] * g_r;
					AI[b - q] += d1[q] * g_i;
				}
			}
		for (int k = 0; k < P; k++)
		{
			double re = 0, im = 0;
			for (int j = 0; j < ns; j++)
			{
				double f = s->fold[k * ns + j];
				if (f == 0.0) continue;
				re += f * (2.0 * AR[j] + Lsp[j]);
				im += f * (2.0 * AI[j]);
			}
			dE[2 * k] = -c * re;
			dE[2 * k + 1] = -c * im;
		}
		/* d/d alpha_p of -c (lap + G.G): -c (2 D n + 4 sum_a G_a . r_a) */
		dE[2 * P] = -c * (2.0 * D * n + 4.0 * gr);
		dE[2 * P + 1] = -c * (4.0 * gi);
	}
	free(S);
	free(wR);
	free(wI);
	free(G);
	free(Lsp);
	free(AR);
	free(AI);
}

/* Metropolis moves of drop walkers stored walker-major SoA (R[w][d][i]):
 * the move rule of DoMetropolisStep (TDVMC.cpp:858-916) with the direct
 * exponent change sum_i u(r_new) - u(r_old) + alpha_p (|x_new|^2 - |x_old|^2)
 * and no wrap (open boundaries).  Random numbers: Philox with counter
 * {move, walker0 + w, pass, call}, as orc_sample.  Returns accepted moves. */
int64_t orc_drop_sample(const orc_drop* dp, const double* uR, double* Rsoa, int64_t nw, int64_t walker0, int moves,
                        double step, uint64_t seed, uint32_t pass)
{
	const orc_sys* s = dp->s;
	const int n = dp->n, P = dp->p, ns = s->ns;
	double* wR = (double*)calloc((size_t)ns, sizeof(double));
	for (int k = 0; k < P; k++)
		for (int j = 0; j < ns; j++) wR[j] += uR[k] * s->fold[k * ns + j];
	double* R = (double*)malloc((size_t)n * 3 * sizeof(double));
	int64_t acc = 0;
	double d[3];
	for (int64_t w = 0; w < nw; w++)
	{
		double* X = Rsoa + (size_t)w * 3 * n;
		for (int a = 0; a < 3; a++)
			for (int i = 0; i < n; i++) R[i * 3 + a] = X[a * n + i];
		for (int m = 0; m < moves; m++)
		{
			int p;
			double U, z[3], xn[3];
			move_randoms(n, 3, (uint32_t)m, (uint32_t)(walker0 + w), pass, seed, &p, &U, z);
			double* xo = R + p * 3;
			double r2n = 0.0, r2o = 0.0;
			for (int a = 0; a < 3; a++)
			{
				xn[a] = xo[a] + step * z[a];
				r2n += xn[a] * xn[a];
				r2o += xo[a] * xo[a];
			}
			double delta = uR[P] * (r2n - r2o);
			for (int i = 0; i < n; i++)
			{
				if (i == p) continue;
				const double rn = drop_disp(xn, R + i * 3, d);
				const double ro = drop_disp(xo, R + i * 3, d);
				delta += drop_u(s, wR, rn, uR[P - 1]) - drop_u(s, wR, ro, uR[P - 1]);
			}
			if (isfinite(delta) && 2.0 * delta >= log(U) && 2.0 * delta < 709.782712893384)
			{
				for (int a = 0; a < 3; a++) xo[a] = xn[a];
				acc++;
			}
		}
		for (int a = 0; a < 3; a++)
			for (int i = 0; i < n; i++) X[a * n + i] = R[i * 3 + a];
	}
	free(R);
	free(wR);
	return acc;
}
