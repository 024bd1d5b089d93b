/*
 * FP64 CPU oracle for the TDVP hot path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference's algorithm for the periodic
 * pair-spline Bose system (mathiasgartner/TDVMC, PhysicalSystems::BosonsBulk
 * and the TDVP driver in src/TDVMC.cpp).  Each function cites the reference
 * lines it follows.  Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * legs of bench.py use this library; the product (tdvmc_gb300/) never links
 * or calls it.
 *
 * Parity of this oracle is pinned against outputs of the reference itself,
 * built from its own sources by oracle/ref/build_ref.sh and captured as
 * fixtures by tests/golden/make_golden.py (see tests/test_oracle_golden.py).
 */
#ifndef TDVMC_ORACLE_H
#define TDVMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_KNOTS 520

/* Pair-potential kinds.  SQUARE follows BosonsBulk.cpp:268-271 (the
 * reference's active choice), GAUSS the commented variant at
 * BosonsBulk.cpp:263-265, LJ follows Potentials/LJ.cpp:16-22.
 * Parameter layout [a, b, t_quench, a', b'] as read at BosonsBulk.cpp:237-242
 * (for LJ: a = sigma, b = epsilon). */
enum { ORC_POT_NONE = 0, ORC_POT_SQUARE = 1, ORC_POT_GAUSS = 2, ORC_POT_LJ = 3 };

typedef struct orc_sys orc_sys;

/* System variants.  BOSONS_BULK: PhysicalSystems::BosonsBulk.  NU_PB:
 * PhysicalSystems::NUBosonsBulkPB (NUBosonsBulkPB.cpp), the same pair spline with
 * a pair beyond r_max entering at the mirrored distance r' = 2 r_max - r
 * (counted outside only at r' = r_max, :240-247, 321-326), its own fold of the
 * p + 2 splines into the p parameters (O_k = S_{k+1}, O_1 += S_0,
 * O_{p-1} += S_{p+1}, :216-226), the gradient, the Laplacian's (D-1)/r and the
 * square-well potential all taken at r' (:321-393: the unit vector is the
 * displacement over r', and the sign flip of the mirrored pairs' derivative is
 * commented out), and r < r_max (strict) for the old and the new position of a
 * move (:622-660). */
/* ORC_SYS_NU_PB_EXACT: NUBosonsBulkPB with the exact derivatives of the
 * mirrored pair term u(2 r_max - r) -- gradient -u'(r') d / r and Laplacian
 * term -(D-1)/r u'(r') at a mirrored pair -- the form the reference's
 * commented-out sign flip (NUBosonsBulkPB.cpp:333-336, 387) points to. */
enum { ORC_SYS_BOSONS_BULK = 0, ORC_SYS_NU_PB = 1, ORC_SYS_NU_PB_EXACT = 2 };

/* Build a system.  user_knots == NULL (nuser = 0) gives the uniform grid of
 * BosonsBulk.cpp:61-67; otherwise the grid is mirrored as in
 * BosonsBulk.cpp:35-44.  Returns NULL on a parameter-count mismatch
 * (BosonsBulk.cpp:85-91). */
orc_sys* orc_create(int dim, int n, int p, double L, const double* user_knots, int nuser,
                    int pot_kind, const double* pot, int npot, double time, double hbar2_2m);
void orc_free(orc_sys* s);
/* Switch an existing system to a variant (rebuilds the fold). */
void orc_set_variant(orc_sys* s, int variant);
int orc_num_knots(const orc_sys* s);
int orc_num_splines(const orc_sys* s);
double orc_rmax(const orc_sys* s);
void orc_knots(const orc_sys* s, double* out);
/* Monomial weights in absolute r, layout [spline][piece][power]
 * (SplineFactory.cpp:54-101). */
void orc_abs_weights(const orc_sys* s, double* out);
/* Local-coordinate piece polynomials, layout [bin][q][power]: spline bin-q on
 * bin in t = (r - k_bin) / (k_bin+1 - k_bin). */
void orc_local_weights(const orc_sys* s, double* out);

/* Minimum-image displacement (Utils.cpp:266-281, 368-382). */
double orc_nic_coord(double x, double L);
double orc_nic_disp(const double* ri, const double* rj, int dim, double L, double* d);

/* Fixed-configuration evaluation of one walker (R: n*dim, particle-major).
 * Follows CalculateWavefunction + CalculateExpectationValues
 * (BosonsBulk.cpp:179-218, 220-336, 349-458, 522-545).
 * Outputs: lnpsi, O[p], eloc[2] (E_R, E_I), other7[7] =
 *   {kineticR, V_int, sumR1, sumI1, sumR2, sumI2, sumR1I1},
 * and, when dE != NULL, the adjoint dE[2p] = (Re, Im) of dE_loc/d uR_k. */
void orc_eval(const orc_sys* s, const double* uR, const double* uI, const double* R,
              double* lnpsi, double* O, double* eloc, double* other7, double* dE);

/* Exponent change of a single-particle move (BosonsBulk.cpp:553-657),
 * incremental with the reference's clamp; returns exponent_new - exponent. */
double orc_move_delta(const orc_sys* s, const double* uR, const double* R, int p, const double* newpos);

/* Philox4x32-10 (Salmon et al., SC'11). */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* One sampling pass for walkers [w0, w0+nw) of an array of walkers stored
 * walker-major SoA: R[w][d][n].  `moves` single-particle moves per walker with
 * the move rule of DoMetropolisStep (TDVMC.cpp:858-916); random numbers from
 * Philox with counter {move, walker, pass, call}.  Returns accepted moves. */
int64_t orc_sample(const orc_sys* s, const double* uR, double* Rsoa, int64_t nw_total, int64_t w0, int64_t nw,
                   int moves, double step, uint64_t seed, uint32_t pass);

/* Same as orc_sample followed by orc_eval of each walker, split over
 * `threads` POSIX threads (CPU baseline).  Per-walker outputs as orc_eval,
 * arrays indexed by walker. */
int64_t orc_stage_threads(const orc_sys* s, const double* uR, const double* uI, double* Rsoa, int64_t nw,
                          int moves, double step, uint64_t seed, uint32_t pass, int threads,
                          double* lnpsi, double* O, double* eloc, double* other7, double* dE);

/* TDVP linear solve from raw sample moments, as SolveForParametersDot
 * (TDVMC.cpp:1506-1537, 1560-1622, 1658-1682, 1684-1711, 1713-1828).
 * solver 0: Cholesky (+1e-3 I); solver 1: the reference solves with Eigen's
 * FullPivHouseholderQR and subtracts the mean of the solution; here a dense
 * elimination with partial pivoting gives the same unique solution of the
 * nonsingular system, then the mean is subtracted.  Returns 1 when the Cholesky met a
 * non-positive pivot (the reference's doNotAcceptStep), else 0. */
int orc_solve(int p, int imag, int precond, int solver, const double* O, double ER, double EI,
              const double* OO, const double* OER, const double* OEI,
              double* uDotR, double* uDotI, double* phiDotR, double* phiDotI);

/* The same solve from centred moments: S (p*p), cov(O, E^R), cov(O, E^I). */
int orc_solve_centred(int p, int imag, int precond, int solver, const double* O, double ER, double EI,
                      const double* S, const double* covOER, const double* covOEI,
                      double* uDotR, double* uDotI, double* phiDotR, double* phiDotI);

/* Pair distribution and static structure factor of one configuration R
 * (n x dim, AoS), BosonsBulk::CalculateAdditionalSystemProperties
 * (BosonsBulk.cpp:474-520) with the grid of BosonsBulk.cpp:142-152 and
 * Observables/Grid.cpp:15-70, ObservableVsOnGridWithScaling.cpp:19-52.
 * gr_bins = GR_BIN_COUNT; returns the number of g(r) bins written to gr.
 * kvec[nvec*dim] are the scaled k vectors, shell s = kvec rows
 * shell_off[s] .. shell_off[s+1]-1; sk[nshell]. */
int orc_observables(const orc_sys* s, const double* R, int gr_bins, int nshell, const int* shell_off,
                    const double* kvec, double* gr, double* sk);

/* Trapped drops (batched systems of uneven particle number): a 3D drop of n bosons
 * with open boundaries, the BosonsBulk pair spline on [0, rmax] (p
 * parameters) plus a one-body parameter alpha_p (ln psi += alpha_p sum |r_i|^2),
 * harmonic trap kappa |r|^2 with kappa = omega^2 / (4 hbar2_2m) and the
 * Gaussian pair repulsion v0 exp(-r^2 / (2 sigma^2)).  Parameter vectors have
 * p + 1 entries; O[p+1], dE[2(p+1)].  R: n*3 particle-major. */
typedef struct orc_drop orc_drop;
orc_drop* orc_drop_create(int n, int p, double rmax, double v0, double sigma, double omega, double hbar2_2m);
void orc_drop_free(orc_drop* d);
void orc_drop_eval(const orc_drop* d, const double* uR, const double* uI, const double* R, double* lnpsi,
                   double* O, double* eloc, double* other7, double* dE);
int64_t orc_drop_sample(const orc_drop* d, const double* uR, double* Rsoa, int64_t nw, int64_t walker0, int moves,
                        double step, uint64_t seed, uint32_t pass);

#ifdef __cplusplus
}
#endif
#endif
